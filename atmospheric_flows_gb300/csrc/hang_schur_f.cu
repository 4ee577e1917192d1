// Hanging-face instantiations of the Schur kernels B and C/D in FP32, for the
// levels of the mixed-precision multigrid on 2:1 adaptive meshes (the FP64
// ones are in hang_schur.cu).  A translation unit of its own so that it
// compiles in parallel with the others.
#include "schur_kernels.cuh"

namespace atm {

int upload_basis_hang_schur_f(const double *t) { return upload_basis_here(t); }

template <typename T>
int level_B_hang(const OpView<T> &o, T *dst, const T *p, T cB, int mode) {
  ATM_DISPATCH_K(o.k, (B_launch<K, T, true>(o, dst, p, cB, mode)));
}
template <typename T>
int level_CD_hang(const OpView<T> &o, T *dst, const T *w, const T *p, T cC, int mode,
                  const ChebArgs<T> *ch) {
  ATM_DISPATCH_K(o.k, (CD_launch<K, T, true>(o, dst, w, p, cC, mode, ch)));
}
template int level_B_hang<float>(const OpView<float> &, float *, const float *, float, int);
template int level_CD_hang<float>(const OpView<float> &, float *, const float *, const float *,
                                  float, int, const ChebArgs<float> *);

}  // namespace atm
