// Hanging-face (2:1 adaptive mesh) instantiations of the Schur kernels B and
// C/D, FP64.  Compiled apart from the conforming instantiations
// (impl_kernels.cu) so the families build in parallel; the launchers choose by
// mesh.nhang.
#include "schur_kernels.cuh"

namespace atm {

int upload_basis_hang_schur(const double *t) { return upload_basis_here(t); }

int launch_B_hang(const atm_ctx &c, double *dst, const double *p, double coeff, int mode) {
  ATM_DISPATCH_K(c.k, (B_launch<K, double, true>(schur_view(c), dst, p, coeff, mode)));
}

int launch_CD_hang(const atm_ctx &c, double *dst, const double *w, const double *p,
                   double coeff, int mode) {
  ATM_DISPATCH_K(c.k, (CD_launch<K, double, true>(schur_view(c), dst, w, p, coeff, mode)));
}

}  // namespace atm
