// Hanging-face (2:1 adaptive mesh) instantiations of the Schur kernels B and
// C/D in FP64: the operator's own launchers and the FP64 multigrid levels.
// Compiled apart from the conforming instantiations (impl_kernels.cu) so the
// families build in parallel; the launchers choose by mesh.nhang.  The FP32
// level instantiations are in hang_schur_f.cu.
#include "schur_kernels.cuh"

namespace atm {

int upload_basis_hang_schur(const double *t) { return upload_basis_here(t); }

template <typename T>
int level_B_hang(const OpView<T> &o, T *dst, const T *p, T cB, int mode) {
  ATM_DISPATCH_K(o.k, (B_launch<K, T, true>(o, dst, p, cB, mode)));
}
template <typename T>
int level_CD_hang(const OpView<T> &o, T *dst, const T *w, const T *p, T cC, int mode,
                  const ChebArgs<T> *ch) {
  ATM_DISPATCH_K(o.k, (CD_launch<K, T, true>(o, dst, w, p, cC, mode, ch)));
}
template int level_B_hang<double>(const OpView<double> &, double *, const double *, double, int);
template int level_CD_hang<double>(const OpView<double> &, double *, const double *,
                                   const double *, double, int, const ChebArgs<double> *);

int launch_B_hang(const atm_ctx &c, double *dst, const double *p, double coeff, int mode) {
  return level_B_hang<double>(schur_view(c), dst, p, coeff, mode);
}

int launch_CD_hang(const atm_ctx &c, double *dst, const double *w, const double *p,
                   double coeff, int mode) {
  return level_CD_hang<double>(schur_view(c), dst, w, p, coeff, mode, nullptr);
}

}  // namespace atm
