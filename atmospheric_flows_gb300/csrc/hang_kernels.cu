// Hanging-face (2:1 adaptive mesh) instantiations of every operator with face
// terms: the three explicit right-hand sides and the Schur kernels B and C/D,
// FP64 only.  Compiled separately from the conforming instantiations so the
// two families build in parallel; the launchers choose by mesh.nhang.
#include "rhs_kernels.cuh"
#include "schur_kernels.cuh"

namespace atm {

int upload_basis_hang(const double *t) { return upload_basis_here(t); }

int rhs_dispatch_hang(const atm_ctx &c, int kind, int stage, double *dst,
                      const double *const *src, const StageCoef &co) {
  return rhs_dispatch_t<true>(c, kind, stage, dst, src, co);
}

int launch_B_hang(const atm_ctx &c, double *dst, const double *p, double coeff, int mode) {
  ATM_DISPATCH_K(c.k, (B_launch<K, double, true>(schur_view(c), dst, p, coeff, mode)));
}

int launch_CD_hang(const atm_ctx &c, double *dst, const double *w, const double *p,
                   double coeff, int mode) {
  ATM_DISPATCH_K(c.k, (CD_launch<K, double, true>(schur_view(c), dst, w, p, coeff, mode)));
}

}  // namespace atm
