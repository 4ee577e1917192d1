// Explicit IMEX stage right-hand sides: conforming-mesh instantiations and
// the public launchers (the kernels are in rhs_kernels.cuh).
#include "rhs_kernels.cuh"

namespace atm {

int upload_basis_rhs(const double *t) { return upload_basis_here(t); }

// hanging-face instantiations, one translation unit per equation
int rhs_dispatch_hang_rho(const atm_ctx &c, int stage, double *dst, const double *const *src,
                          const StageCoef &co);
int rhs_dispatch_hang_vel(const atm_ctx &c, int stage, double *dst, const double *const *src,
                          const StageCoef &co);
int rhs_dispatch_hang_pres(const atm_ctx &c, int stage, double *dst, const double *const *src,
                           const StageCoef &co);

namespace {
int rhs_dispatch(const atm_ctx &c, int kind, int stage, double *dst, const double *const *src,
                 const StageCoef &co) {
  const bool hg = c.mesh.nhang > 0;
  switch (kind) {
    case 0: return hg ? rhs_dispatch_hang_rho(c, stage, dst, src, co)
                      : rhs_dispatch_kind<false, 0>(c, stage, dst, src, co);
    case 1: return hg ? rhs_dispatch_hang_vel(c, stage, dst, src, co)
                      : rhs_dispatch_kind<false, 1>(c, stage, dst, src, co);
    default: return hg ? rhs_dispatch_hang_pres(c, stage, dst, src, co)
                       : rhs_dispatch_kind<false, 2>(c, stage, dst, src, co);
  }
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
