// Implicit-block kernels (FP64):
//   B   pressure gradient, p -> velocity   euler_operator.h:1512-1617
//   C   enthalpy divergence, w -> pressure euler_operator.h:1413-1507
//   D   internal-energy mass               euler_operator.h:1386-1408
//   A   rho_fix-weighted velocity mass     euler_operator.h:2330-2357
//   rho mass                               euler_operator.h:717-740
//   inverse diagonals                      euler_operator.h:2458-2626
// plus the exact cell-wise inverses of the (weighted) DG mass matrices.
// Because every mass-type block of this DG discretisation is cell-local,
// A^{-1}, M^{-1} and D^{-1} are applied exactly with one dense (k+1)^2 block
// per cell instead of the reference's CG iterations (euler_operator.h:2391-2397,
// Atmospheric_Flow.cc:452-536); the Schur apply S p = D p - C A^{-1} B p is
// then two fused kernels: (B, A^{-1}) and (C, D, Jacobi).
#include "schur_kernels.cuh"

namespace atm {

int upload_basis_impl(const double *t) { return upload_basis_here(t); }

// hanging-face instantiations of B and C/D live in hang_schur.cu (FP64) and
// hang_schur_f.cu (FP32 multigrid levels)
int launch_B_hang(const atm_ctx &c, double *dst, const double *p, double coeff, int mode);
int launch_CD_hang(const atm_ctx &c, double *dst, const double *w, const double *p,
                   double coeff, int mode);
template <typename T>
int level_B_hang(const OpView<T> &o, T *dst, const T *p, T cB, int mode);
template <typename T>
int level_CD_hang(const OpView<T> &o, T *dst, const T *w, const T *p, T cC, int mode,
                  const ChebArgs<T> *ch);

// ============================================================ mass apply ===
// dst = M_w src for NCOMP components; weight tile (rho) or constant scale
template <int K, int NCOMP, bool WEIGHTED, typename T>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_mass(T *__restrict__ dst, const T *__restrict__ src,
           const T *__restrict__ weight, T scale, MeshT<T> mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  constexpr int NT = NCOMP + (WEIGHTED ? 1 : 0);
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  T *tiles = sm;
  T *xab = tiles + CPB * NT * NN2;  // [CPB][NCOMP][NN*NQ]
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  load_tiles<K>(tiles, NT, 0, src, NCOMP, c0, cnt);
  if (WEIGHTED) load_tiles<K>(tiles, NT, NCOMP, weight, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  T Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const T *tl = tiles + lc * NT * NN2;
    T wv[NQ];
    if (WEIGHTED) eval_col<K>(tl + NCOMP * NN2, Sx, wv);
    const T *G = mesh.qgeo + (long)c * 5 * NQ2;
#pragma unroll
    for (int comp = 0; comp < NCOMP; ++comp) {
      T v[NQ], V[NQ];
      eval_col<K>(tl + comp * NN2, Sx, v);
#pragma unroll
      for (int qz = 0; qz < NQ; ++qz) {
        const T jxw = G[4 * NQ2 + qz * NQ + col];
        V[qz] = (WEIGHTED ? wv[qz] * v[qz] : scale * v[qz]) * jxw;
      }
      integrate_col_z<K, true, false>(V, V, V, xab + (lc * NCOMP + comp) * NN * NQ, (T *)nullptr,
                                      col);
    }
  }
  __syncthreads();
  if (active && col < NN) {
    T St[NQ], Dt[NQ];
    load_cols<K>(col, St, Dt);
#pragma unroll
    for (int comp = 0; comp < NCOMP; ++comp) {
      T out[NN];
      integrate_out<K, false>(xab + (lc * NCOMP + comp) * NN * NQ, (const T *)nullptr, St, Dt, out);
      T *d = dst + ((long)c * NCOMP + comp) * NN2;
#pragma unroll
      for (int iz = 0; iz < NN; ++iz) d[iz * NN + col] = out[iz];
    }
  }
}

// ===================================================== inverse diagonal ===
template <int K, bool WEIGHTED, typename T>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_invdiag(T *__restrict__ out, int ncomp, const T *__restrict__ weight,
              T scale, MeshT<T> mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  T *tiles = sm;                      // [CPB][NN2] weight
  T *xab = tiles + CPB * NN2;         // [CPB][NN*NQ]
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  if (WEIGHTED) load_tiles<K>(tiles, 1, 0, weight, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  T Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    T wv[NQ];
    if (WEIGHTED) eval_col<K>(tiles + lc * NN2, Sx, wv);
    const T *G = mesh.qgeo + (long)c * 5 * NQ2;
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      T s = T(0.0);
#pragma unroll
      for (int qz = 0; qz < NQ; ++qz) {
        const T b = bS<K, T>(qz, iz);
        const T wj = (WEIGHTED ? wv[qz] : scale) * G[4 * NQ2 + qz * NQ + col];
        s = fma(b * b, wj, s);
      }
      xab[lc * NN * NQ + iz * NQ + col] = s;
    }
  }
  __syncthreads();
  if (active && col < NN) {
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      T s = T(0.0);
#pragma unroll
      for (int qx = 0; qx < NQ; ++qx) {
        const T b = bS<K, T>(qx, col);
        s = fma(b * b, xab[lc * NN * NQ + iz * NQ + qx], s);
      }
      const T inv = T(1.0) / s;
      for (int comp = 0; comp < ncomp; ++comp)
        out[((long)c * ncomp + comp) * NN2 + iz * NN + col] = inv;
    }
  }
}

// ================================================= exact block inverse ===
// One warp per cell.  The (weighted) cell mass matrix
//   M[(iz,ix),(jz,jx)] = sum_q S(qz,iz)S(qz,jz) S(qx,ix)S(qx,jx) w(q) JxW(q)
// is symmetric positive definite: only its lower triangle is assembled, in
// packed storage, by sum factorisation over the symmetric 1D index pairs
// (a <= b) with the products S(q,a)S(q,b) tabulated once per block.  It is
// then inverted in place by the symmetric sweep operator (Gauss-Jordan
// restricted to the lower triangle; SPD, no pivoting), which leaves -M^{-1}.
// The inverse is written out in full, transposed (it is symmetric).
constexpr int BI_WARPS = 2;

template <int K>
struct BlockInvCfg {
  static constexpr int NN = K + 1, NQ = 2 * K + 1, NN2 = NN * NN, NQ2 = NQ * NQ;
  static constexpr int NP = NN * (NN + 1) / 2;        // 1D pairs a <= b
  static constexpr int NTRI = NN2 * (NN2 + 1) / 2;    // packed lower triangle
  static constexpr int PER = NQ2 + NQ * NP + NTRI + 2 * NN2 + NN * NQ;  // per warp
  // block tables: S products [NQ][NP], then byte tables of pair/triangle indices
  static constexpr int TAB_BYTES = ((NQ * NP) * 8 + 2 * NTRI + 7) / 8 * 8;
  template <typename T>
  static size_t smem() { return TAB_BYTES + sizeof(T) * (size_t)BI_WARPS * PER; }
};

__device__ __forceinline__ int tri_index(int i, int j) {  // i >= j
  return i * (i + 1) / 2 + j;
}
__device__ __forceinline__ int sym_index(int i, int j) {
  return i >= j ? tri_index(i, j) : tri_index(j, i);
}

template <int K, typename T>
__global__ void __launch_bounds__(32 * BI_WARPS)
    k_block_inverse(T *__restrict__ out, const T *__restrict__ weight, MeshT<T> mesh) {
  using B = BlockInvCfg<K>;
  constexpr int NN = B::NN, NQ = B::NQ, NN2 = B::NN2, NQ2 = B::NQ2, NP = B::NP;
  constexpr int NTRI = B::NTRI;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *ss = reinterpret_cast<T *>(sm_raw);                              // [NQ][NP]
  unsigned char *ti = sm_raw + (size_t)NQ * NP * sizeof(T);           // [NTRI] row
  unsigned char *tj = ti + NTRI;                                      // [NTRI] column
  T *wsm = reinterpret_cast<T *>(sm_raw + B::TAB_BYTES);
  // block tables
  for (int e = threadIdx.x; e < NQ * NP; e += blockDim.x) {
    const int q = e / NP, p = e - q * NP;
    int b = 0;
    while ((b + 1) * (b + 2) / 2 <= p) ++b;
    const int a = p - b * (b + 1) / 2;
    ss[e] = bS<K, T>(q, a) * bS<K, T>(q, b);
  }
  for (int e = threadIdx.x; e < NTRI; e += blockDim.x) {
    int i = 0;
    while ((i + 1) * (i + 2) / 2 <= e) ++i;
    ti[e] = (unsigned char)i;
    tj[e] = (unsigned char)(e - i * (i + 1) / 2);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * BI_WARPS + warp;
  if (c >= mesh.nc) return;  // warp-uniform; only warp-level barriers below
  T *wq = wsm + warp * B::PER;   // [NQ2] w JxW at the quadrature points
  T *Tb = wq + NQ2;              // [NQ][NP] x-contracted weights
  T *M = Tb + NQ * NP;           // [NTRI] packed lower triangle
  T *colk = M + NTRI;            // [NN2] pivot column
  T *cd = colk + NN2;            // [NN2] pivot column / pivot
  T *tx = cd + NN2;              // [NN][NQ] x-contracted weight field
  const T *G = mesh.qgeo + (long)c * 5 * NQ2;
  if (weight) {
    const T *wt = weight + (long)c * NN2;
    for (int e = lane; e < NN * NQ; e += 32) {
      const int iz = e / NQ, qx = e - iz * NQ;
      T s = T(0.0);
#pragma unroll
      for (int ix = 0; ix < NN; ++ix) s = fma(bS<K, T>(qx, ix), wt[iz * NN + ix], s);
      tx[e] = s;
    }
    __syncwarp();
    for (int q = lane; q < NQ2; q += 32) {
      const int qz = q / NQ, qx = q - qz * NQ;
      T s = T(0.0);
#pragma unroll
      for (int iz = 0; iz < NN; ++iz) s = fma(bS<K, T>(qz, iz), tx[iz * NQ + qx], s);
      wq[q] = s * G[4 * NQ2 + q];
    }
  } else {
    for (int q = lane; q < NQ2; q += 32) wq[q] = G[4 * NQ2 + q];
  }
  __syncwarp();
  for (int e = lane; e < NQ * NP; e += 32) {
    const int qz = e / NP, p = e - qz * NP;
    T s = T(0.0);
#pragma unroll
    for (int qx = 0; qx < NQ; ++qx) s = fma(ss[qx * NP + p], wq[qz * NQ + qx], s);
    Tb[e] = s;
  }
  __syncwarp();
  for (int e = lane; e < NTRI; e += 32) {
    const int I = ti[e], J = tj[e];
    const int iz = I / NN, ix = I - iz * NN, jz = J / NN, jx = J - jz * NN;
    const int pz = sym_index(iz, jz), px = sym_index(ix, jx);
    T s = T(0.0);
#pragma unroll
    for (int qz = 0; qz < NQ; ++qz) s = fma(ss[qz * NP + pz], Tb[qz * NP + px], s);
    M[e] = s;
  }
  __syncwarp();
  // symmetric sweep on pivots k = 0..NN2-1:
  //   a_ij -= a_ik a_kj / a_kk (i, j != k);  a_ik = a_ik / a_kk;  a_kk = -1 / a_kk
  for (int k = 0; k < NN2; ++k) {
    const T d = T(1.0) / M[tri_index(k, k)];
    for (int i = lane; i < NN2; i += 32) {  // NN2 = 36 > 32 for k = 5
      const T a = M[sym_index(i, k)];
      colk[i] = a;
      cd[i] = a * d;
    }
    __syncwarp();
    for (int e = lane; e < NTRI; e += 32) {
      const int i = ti[e], j = tj[e];
      if (i != k && j != k) M[e] = fma(-cd[i], colk[j], M[e]);
    }
    __syncwarp();
    for (int i = lane; i < NN2; i += 32) M[sym_index(i, k)] = i == k ? -d : cd[i];
    __syncwarp();
  }
  T *o = out + (long)c * ainv_stride<K, T>();
  if constexpr (sizeof(T) == 4) {  // packed lower triangle (ainv_stride)
    for (int e = lane; e < NTRI; e += 32) o[e] = -M[e];
  } else {
    for (int e = lane; e < NN2 * NN2; e += 32) {
      const int j = e / NN2, i = e - j * NN2;
      o[e] = -M[sym_index(i, j)];
    }
  }
}

// dst[c][comp][i] = scale * sum_j Binv[c][i][j] src[c][comp][j]  (transposed storage)
template <int K, typename T>
__global__ void k_block_apply(T *__restrict__ dst, const T *__restrict__ src,
                              const T *__restrict__ binvT, int ncomp, T scale,
                              int nc) {
  constexpr int NN2 = (K + 1) * (K + 1);
  static_assert(sizeof(T) == 8, "full A^{-1} blocks are FP64 (FP32 stores a triangle)");
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long)nc * NN2) return;
  const int c = (int)(g / NN2), i = (int)(g - (long)c * NN2);
  const T *B = binvT + (long)c * ainv_stride<K, T>();
  for (int comp = 0; comp < ncomp; ++comp) {
    const T *s = src + ((long)c * ncomp + comp) * NN2;
    T acc = T(0.0);
#pragma unroll 4
    for (int j = 0; j < NN2; ++j) acc = fma(B[j * NN2 + i], s[j], acc);
    dst[((long)c * ncomp + comp) * NN2 + i] = scale * acc;
  }
}

namespace {
template <int K, typename T>
int mass_launch(const OpView<T> &v, T *dst, const T *src, int ncomp, const T *weight,
                T scale) {
  using C = Cfg<K>;
  const int grid = (v.nc + C::CPB - 1) / C::CPB;
  const size_t sm = sizeof(T) * C::CPB * (3 * C::NN2 + 2 * C::NN * C::NQ);
  if (ncomp == 1 && !weight) k_mass<K, 1, false, T><<<grid, C::THREADS, sm, v.st>>>(dst, src, weight, scale, v.mesh);
  else if (ncomp == 1) k_mass<K, 1, true, T><<<grid, C::THREADS, sm, v.st>>>(dst, src, weight, scale, v.mesh);
  else if (!weight) k_mass<K, 2, false, T><<<grid, C::THREADS, sm, v.st>>>(dst, src, weight, scale, v.mesh);
  else k_mass<K, 2, true, T><<<grid, C::THREADS, sm, v.st>>>(dst, src, weight, scale, v.mesh);
  ATM_CHECK_LAUNCH("k_mass");
  return ATM_OK;
}

template <int K, typename T>
int invdiag_launch(const OpView<T> &v, T *out, int ncomp, const T *weight, T scale) {
  using C = Cfg<K>;
  const int grid = (v.nc + C::CPB - 1) / C::CPB;
  const size_t sm = sizeof(T) * C::CPB * (C::NN2 + C::NN * C::NQ);
  if (weight) k_invdiag<K, true, T><<<grid, C::THREADS, sm, v.st>>>(out, ncomp, weight, scale, v.mesh);
  else k_invdiag<K, false, T><<<grid, C::THREADS, sm, v.st>>>(out, ncomp, weight, scale, v.mesh);
  ATM_CHECK_LAUNCH("k_invdiag");
  return ATM_OK;
}

template <int K, typename T>
int block_inverse_launch(const OpView<T> &v, T *out, const T *weight) {
  const size_t sm = BlockInvCfg<K>::template smem<T>();
  ATM_CUDA(allow_smem(k_block_inverse<K, T>, sm));
  const int grid = (v.nc + BI_WARPS - 1) / BI_WARPS;
  k_block_inverse<K, T><<<grid, 32 * BI_WARPS, sm, v.st>>>(out, weight, v.mesh);
  ATM_CHECK_LAUNCH("k_block_inverse");
  return ATM_OK;
}

template <int K, typename T>
int block_apply_launch(const OpView<T> &v, T *dst, const T *src, const T *binv, int ncomp,
                       T scale) {
  constexpr int NN2 = (K + 1) * (K + 1);
  const long n = (long)v.nc * NN2;
  const int threads = 256;
  const int grid = (int)((n + threads - 1) / threads);
  k_block_apply<K, T><<<grid, threads, 0, v.st>>>(dst, src, binv, ncomp, scale, v.nc);
  ATM_CHECK_LAUNCH("k_block_apply");
  return ATM_OK;
}
}  // namespace
int launch_B(const atm_ctx &c, double *dst, const double *p, double coeff, int mode) {
  const double ns = (double)c.nc * c.nn2;
  // p read; B p written (2 comps); mode 1 reads dst too; mode 2 reads A^{-1}
  const double bytes = 8.0 * ns * (1 + 2 + (mode == 1 ? 2 : 0)) +
                       (mode == 2 ? 8.0 * c.nc * c.nn2 * c.nn2 : 0.0);
  const double flops = c.nc * (fl_eval(c.k) + 2 * fl_integrate(c.k, true) +
                               4.0 * (2 * fl_face(c.k) + 2 * fl_face(c.k)) +
                               (mode == 2 ? 4.0 * c.nn2 * c.nn2 : 0.0));
  TimedRegion tr(c, KF_B, bytes, flops);
  if (c.mesh.nhang > 0) return launch_B_hang(c, dst, p, coeff, mode);
  ATM_DISPATCH_K(c.k, (B_launch<K, double, false>(schur_view(c), dst, p, coeff, mode)));
}
int launch_CD(const atm_ctx &c, double *dst, const double *w, const double *p, double coeff,
              int mode) {
  const double ns = (double)c.nc * c.nn2;
  const bool wd = (mode == 1 || mode == 2);
  // w (2 comps) + pfix read, [p], [inverse diagonal], [dst read], dst written
  const double bytes = 8.0 * ns * (3 + (wd ? 1 : 0) + (mode == 2 ? 1 : 0) + (mode == 3 ? 1 : 0) + 1);
  const double flops = c.nc * ((wd ? 4 : 3) * fl_eval(c.k) + fl_integrate(c.k, true) +
                               4.0 * (2 * 3 * fl_face(c.k) + fl_face(c.k)));
  TimedRegion tr(c, KF_CD, bytes, flops);
  if (c.mesh.nhang > 0) return launch_CD_hang(c, dst, w, p, coeff, mode);
  ATM_DISPATCH_K(c.k, (CD_launch<K, double, false>(schur_view(c), dst, w, p, coeff, mode)));
}
int launch_pfix_prep(const atm_ctx &c) {
  // p_fix read; its values at the quadrature points and face traces written
  const double bytes = 8.0 * c.nc * (c.nn2 + c.nq2 + 4.0 * c.nq);
  const double flops = c.nc * (fl_eval(c.k) + 4.0 * fl_face(c.k));
  TimedRegion tr(c, KF_PFIX_PREP, bytes, flops);
  ATM_DISPATCH_K(c.k, (pfix_prep_launch<K, double>(schur_view(c))));
}
int launch_mass(const atm_ctx &c, double *dst, const double *src, int ncomp,
                const double *weight, double scale) {
  const double ns = (double)c.nc * c.nn2;
  const double bytes = 8.0 * ns * (2 * ncomp + (weight ? 1 : 0));
  const double flops = c.nc * ((ncomp + (weight ? 1 : 0)) * fl_eval(c.k) +
                               ncomp * fl_integrate(c.k, false));
  TimedRegion tr(c, KF_MASS, bytes, flops);
  ATM_DISPATCH_K(c.k, (mass_launch<K, double>(schur_view(c), dst, src, ncomp, weight, scale)));
}
int launch_inv_diag(const atm_ctx &c, double *out, int ncomp, const double *weight,
                    double scale) {
  TimedRegion tr(c, KF_DIAG, 8.0 * c.nc * c.nn2 * (ncomp + (weight ? 1 : 0)), 0.0);
  ATM_DISPATCH_K(c.k, (invdiag_launch<K, double>(schur_view(c), out, ncomp, weight, scale)));
}
int launch_block_inverse(const atm_ctx &c, double *out, const double *weight) {
  const double nn = c.nn, nq = c.nq, nn2 = c.nn2;
  // weight read, inverse written; flops: mass assembly + Gauss-Jordan
  const double bytes = 8.0 * c.nc * (nn2 * (weight ? 1 : 0) + nn2 * nn2);
  const double flops = c.nc * (2.0 * (nq * nn * nn * nq + nn2 * nn2 * nq) + 2.0 * nn2 * nn2 * nn2);
  TimedRegion tr(c, KF_BLOCK_INV, bytes, flops);
  ATM_DISPATCH_K(c.k, (block_inverse_launch<K, double>(schur_view(c), out, weight)));
}
int launch_block_apply(const atm_ctx &c, double *dst, const double *src, const double *binv,
                       int ncomp, double scale) {
  const double nn2 = c.nn2;
  const double bytes = 8.0 * c.nc * (nn2 * nn2 + 2.0 * ncomp * nn2);
  const double flops = 2.0 * c.nc * ncomp * nn2 * nn2;
  TimedRegion tr(c, KF_BLOCK_APPLY, bytes, flops);
  ATM_DISPATCH_K(c.k, (block_apply_launch<K, double>(schur_view(c), dst, src, binv, ncomp, scale)));
}

// ---- launchers on a multigrid level (untimed; float or double) -----------
template <typename T>
int level_B(const LevelViewT<T> &v, T *dst, const T *p, T cB, int mode) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st, v.tune, v.pfix, v.pfq, v.pff};
  if (v.mesh.nhang > 0) return level_B_hang<T>(o, dst, p, cB, mode);
  ATM_DISPATCH_K(v.k, (B_launch<K, T, false>(o, dst, p, cB, mode)));
}
template <typename T>
int level_CD(const LevelViewT<T> &v, T *dst, const T *w, const T *p, T cC, int mode) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st, v.tune, v.pfix, v.pfq, v.pff};
  if (v.mesh.nhang > 0) return level_CD_hang<T>(o, dst, w, p, cC, mode, nullptr);
  ATM_DISPATCH_K(v.k, (CD_launch<K, T, false>(o, dst, w, p, cC, mode)));
}
template <typename T>
int level_CD_cheb(const LevelViewT<T> &v, const T *w, T cC, const ChebArgs<T> &ch) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st, v.tune, v.pfix, v.pfq, v.pff};
  if (v.mesh.nhang > 0) return level_CD_hang<T>(o, nullptr, w, ch.x, cC, 4, &ch);
  ATM_DISPATCH_K(v.k, (CD_launch<K, T, false>(o, nullptr, w, ch.x, cC, 4, &ch)));
}
template <typename T>
int level_pfix_prep(const LevelViewT<T> &v) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st, v.tune, v.pfix, v.pfq, v.pff};
  ATM_DISPATCH_K(v.k, (pfix_prep_launch<K, T>(o)));
}
template <typename T>
int level_inv_diag(const LevelViewT<T> &v, T *out, T scale) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st, v.tune, v.pfix, v.pfq, v.pff};
  ATM_DISPATCH_K(v.k, (invdiag_launch<K, T>(o, out, 1, (const T *)nullptr, scale)));
}
template <typename T>
int level_block_inverse(const LevelViewT<T> &v, T *out, const T *weight) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st, v.tune, v.pfix, v.pfq, v.pff};
  ATM_DISPATCH_K(v.k, (block_inverse_launch<K, T>(o, out, weight)));
}
#define ATM_LEVEL_INST(T)                                                                   \
  template int level_B<T>(const LevelViewT<T> &, T *, const T *, T, int);                   \
  template int level_CD<T>(const LevelViewT<T> &, T *, const T *, const T *, T, int);       \
  template int level_pfix_prep<T>(const LevelViewT<T> &);                                   \
  template int level_CD_cheb<T>(const LevelViewT<T> &, const T *, T, const ChebArgs<T> &);   \
  template int level_inv_diag<T>(const LevelViewT<T> &, T *, T);                            \
  template int level_block_inverse<T>(const LevelViewT<T> &, T *, const T *);
ATM_LEVEL_INST(float)
ATM_LEVEL_INST(double)

}  // namespace atm