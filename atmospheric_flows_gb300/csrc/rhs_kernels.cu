// Explicit IMEX stage right-hand sides: conforming-mesh instantiations and
// the public launchers (the kernels are in rhs_kernels.cuh).
#include "rhs_kernels.cuh"

namespace atm {

int upload_basis_rhs(const double *t) { return upload_basis_here(t); }

// hanging-face instantiations live in hang_kernels.cu
int rhs_dispatch_hang(const atm_ctx &c, int kind, int stage, double *dst,
                      const double *const *src, const StageCoef &co);

namespace {
int rhs_dispatch(const atm_ctx &c, int kind, int stage, double *dst, const double *const *src,
                 const StageCoef &co) {
  return c.mesh.nhang > 0 ? rhs_dispatch_hang(c, kind, stage, dst, src, co)
                          : rhs_dispatch_t<false>(c, kind, stage, dst, src, co);
}
}  // namespace

int launch_rhs_rho(const atm_ctx &c, int stage, double *dst, const double *const *src,
                   const StageCoef &co) {
  return rhs_dispatch(c, 0, stage, dst, src, co);
}
int launch_rhs_vel(const atm_ctx &c, int stage, double *dst, const double *const *src,
                   const StageCoef &co) {
  return rhs_dispatch(c, 1, stage, dst, src, co);
}
int launch_rhs_pres(const atm_ctx &c, int stage, double *dst, const double *const *src,
                    const StageCoef &co) {
  return rhs_dispatch(c, 2, stage, dst, src, co);
}

}  // namespace atm
