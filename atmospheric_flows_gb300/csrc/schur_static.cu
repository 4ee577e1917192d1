// Schur apply whose intermediate lives in a library-owned static device array.
//
// Who needs this: some callers must not have the library allocate device
// memory when they call it.  A host framework that owns every byte of HBM
// through its own pool or admission budget (for example a serving loop that
// admits members against a fixed memory budget) cannot let a library grab
// memory behind its back, and cudaMalloc/cudaFree synchronise the whole
// device, which a latency-sensitive caller sharing the GPU with other streams
// cannot afford.  This entry point computes the same S p = D p - C A^{-1} B p
// as atm_vmult in NS stage 2, but keeps A^{-1} B p in the file-scope array
// below instead of the context's workspace, and calls no allocating routine.
//
// Limits and sharing rules:
//   * the array holds SCHUR_SCRATCH_DOUBLES doubles (8 MiB); a context whose
//     velocity vector (2 * n_scalar doubles) is longer is rejected with
//     ATM_BAD_ARG.  Every GPU on which this library's device code is loaded
//     keeps the 8 MiB until the process exits.
//   * all calls on a device share the one array and it keeps the last call's
//     contents.  Nothing in it needs to start at zero: the first kernel
//     overwrites every entry it later reads.  Calls whose kernels overlap on
//     the GPU (other streams, other threads, other contexts) race on it; the
//     caller must serialise them.
//   * the device address of the array is looked up by the first call made
//     with a handle, in the CUDA context that handle's memory belongs to
//     (its device, current at the call), and kept in the handle.  A handle
//     is bound to one context, so the address stays valid for the handle's
//     life; after a device reset every old handle is dead and new handles
//     look the address up again.  Make that first call before any stream
//     capture.
//   * kernel timing (atm_timing_enable) must be off, because the timers
//     create CUDA events on demand.
#include "atm_device.cuh"

namespace atm {

constexpr long SCHUR_SCRATCH_DOUBLES = 1L << 20;  // 8 MiB
static __device__ __align__(256) double g_schur_scratch[SCHUR_SCRATCH_DOUBLES];

namespace {
// host-side stand-in -> device address in the current context, once per handle
int scratch_address(atm_ctx &h, double **out) {
  if (!h.static_scratch) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_schur_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_schur_scratch)");
    h.static_scratch = p;
  }
  *out = static_cast<double *>(h.static_scratch);
  return ATM_OK;
}
}  // namespace
}  // namespace atm

extern "C" int atm_schur_vmult_static_scratch(atm_handle h, double *dst, const double *src) {
  using namespace atm;
  if (!h || !dst || !src) {
    set_error("atm_schur_vmult_static_scratch: null handle or pointer");
    return ATM_BAD_ARG;
  }
  if (h->n_vector() > SCHUR_SCRATCH_DOUBLES) {
    set_error("atm_schur_vmult_static_scratch: velocity vector of " +
              std::to_string(h->n_vector()) + " doubles exceeds the static scratch of " +
              std::to_string(SCHUR_SCRATCH_DOUBLES) + " doubles (8 MiB)");
    return ATM_BAD_ARG;
  }
  if (h->timer.on) {
    set_error("atm_schur_vmult_static_scratch: disable kernel timing first");
    return ATM_BAD_ARG;
  }
  int dev = -1;
  ATM_CUDA(cudaGetDevice(&dev));
  if (dev != h->device) {
    set_error("atm_schur_vmult_static_scratch: make the context's device current");
    return ATM_BAD_ARG;
  }
  double *scratch = nullptr;
  int rc = scratch_address(*h, &scratch);
  if (rc) return rc;
  const double co = implicit_coeff(*h);
  // no tile-shape timing here (it would create events): tuned choices made by
  // earlier calls are used, otherwise the default blocks
  const bool tune = h->autotune;
  h->autotune = false;
  rc = launch_B(*h, scratch, src, co * h->dt / (h->Ma * h->Ma), 2);
  if (rc == ATM_OK) rc = launch_CD(*h, dst, scratch, src, co * h->dt, 1);
  h->autotune = tune;
  return rc;
}
