// Hanging-face (2:1 adaptive mesh) instantiations of the energy right-hand
// side, FP64.  One translation unit per equation, apart from the conforming
// instantiations (rhs_kernels.cu), so the families build in parallel; the
// launchers choose by mesh.nhang.
#include "rhs_kernels.cuh"

namespace atm {

int upload_basis_hang_pres(const double *t) { return upload_basis_here(t); }

int rhs_dispatch_hang_pres(const atm_ctx &c, int stage, double *dst, const double *const *src,
                     const StageCoef &co) {
  return rhs_dispatch_kind<true, 2>(c, stage, dst, src, co);
}

}  // namespace atm
