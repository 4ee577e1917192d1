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
#include "atm_device.cuh"

namespace atm {

int upload_basis_impl(const double *t) { return upload_basis_here(t); }

// ====================================================================== B ===
// MODE 0: dst = B p ; 1: dst -= B p ; 2: dst = A^{-1} B p
template <int K, int MODE, typename T>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_B(T *__restrict__ dst, const T *__restrict__ p, T cB,
        const T *__restrict__ ainv, MeshT<T> mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  constexpr int NT = 1;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  T *tiles = sm;
  T *xab = tiles + CPB * NT * NN2;  // [CPB][2][2][NN*NQ]
  T *fb = xab + CPB * 4 * NN * NQ;  // [CPB][2][4][NQ]
  T *bt = fb + CPB * 8 * NQ;        // [CPB][2][NN2] (MODE 2)
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  load_tiles<K>(tiles, NT, 0, p, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  T Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const T *tl = tiles + lc * NT * NN2;
    T pv[NQ];
    eval_col<K>(tl, Sx, pv);
    const T *G = mesh.qgeo + (long)c * 5 * NQ2;
    T V[NQ], Gxi[NQ], Get[NQ];
    // submit_divergence(-cB p): component d is tested with d(phi)/dx_d
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
#pragma unroll
      for (int qz = 0; qz < NQ; ++qz) {
        const auto g = qgeo<K>(G, qz * NQ + col);
        const T s = -cB * pv[qz];
        Gxi[qz] = (comp == 0 ? g.xx : g.xz) * s;
        Get[qz] = (comp == 0 ? g.ex : g.ez) * s;
        V[qz] = T(0.0);
      }
      T *xa = xab + (lc * 2 + comp) * 2 * NN * NQ;
      integrate_col_z<K, false, true>(V, Gxi, Get, xa, xa + NN * NQ, col);
    }
    for (int f = 0; f < 4; ++f) {
      const int nb = mesh.nbr[c * 4 + f];
      const T *fg = mesh.fgeo + ((long)c * 4 + f) * 3 * NQ;
      const T n0 = fg[col], n1 = fg[NQ + col], jxw = fg[2 * NQ + col];
      const T pp = face_val<K>(tl, f, Sx);
      T avg;
      if (nb >= 0) {
        const T pm = face_val<K>(p + (long)nb * NN2, mesh.nbrf[c * 4 + f], Sx);
        avg = T(0.5) * (pp + pm);
      } else {
        avg = T(0.5) * (pp + pp);  // wall, p_D = p
      }
      fb[((lc * 2 + 0) * 4 + f) * NQ + col] = cB * avg * n0 * jxw;
      fb[((lc * 2 + 1) * 4 + f) * NQ + col] = cB * avg * n1 * jxw;
    }
  }
  __syncthreads();
  if (active && col < NN) {
    T St[NQ], Dt[NQ];
    load_cols<K>(col, St, Dt);
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      T out[NN];
      const T *xa = xab + (lc * 2 + comp) * 2 * NN * NQ;
      integrate_out<K, true>(xa, xa + NN * NQ, St, Dt, out);
      add_face_out<K>(fb + (lc * 2 + comp) * 4 * NQ, col, St, out);
      if (MODE == 2) {
#pragma unroll
        for (int iz = 0; iz < NN; ++iz) bt[(lc * 2 + comp) * NN2 + iz * NN + col] = out[iz];
      } else {
        T *d = dst + ((long)c * 2 + comp) * NN2;
#pragma unroll
        for (int iz = 0; iz < NN; ++iz) {
          if (MODE == 0) d[iz * NN + col] = out[iz];
          else d[iz * NN + col] -= out[iz];
        }
      }
    }
  }
  if (MODE == 2) {
    __syncthreads();
    if (active) {
      const T *Ab = ainv + (long)c * NN2 * NN2;
      const T *b0 = bt + (lc * 2 + 0) * NN2, *b1 = bt + (lc * 2 + 1) * NN2;
      for (int i = col; i < NN2; i += NQ) {
        T s0 = T(0.0), s1 = T(0.0);
#pragma unroll 5
        for (int j = 0; j < NN2; ++j) {
          const T a = Ab[j * NN2 + i];  // transposed storage
          s0 = fma(a, b0[j], s0);
          s1 = fma(a, b1[j], s1);
        }
        dst[((long)c * 2 + 0) * NN2 + i] = s0;
        dst[((long)c * 2 + 1) * NN2 + i] = s1;
      }
    }
  }
}

// ===================================================================== CD ===
// MODE 0: dst = C w ; 1: dst = sD D p - C w ; 2: dst = invd .* (sD D p - C w)
// MODE 3: dst -= C w
template <int K, int MODE, typename T>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_CD(T *__restrict__ dst, const T *__restrict__ w, const T *__restrict__ p,
         const T *__restrict__ pfix, T cC, const T *__restrict__ invd,
         MeshT<T> mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  constexpr bool WITH_D = (MODE == 1 || MODE == 2);
  constexpr int NT = WITH_D ? 4 : 3;  // w(2), pfix, [p]
  constexpr T GM1 = GAS_GAMMA - T(1.0);
  constexpr T HG = GAS_GAMMA / (GAS_GAMMA - T(1.0));
  // sign of the C contribution in dst
  constexpr T SC = WITH_D ? -T(1.0) : T(1.0);
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  T *tiles = sm;
  T *xab = tiles + CPB * NT * NN2;
  T *fb = xab + CPB * 2 * NN * NQ;
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  load_tiles<K>(tiles, NT, 0, w, 2, c0, cnt);
  load_tiles<K>(tiles, NT, 2, pfix, 1, c0, cnt);
  if (WITH_D) load_tiles<K>(tiles, NT, 3, p, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  T Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const T *tl = tiles + lc * NT * NN2;
    T wx[NQ], wz[NQ], pf[NQ], pv[NQ];
    eval_col<K>(tl, Sx, wx);
    eval_col<K>(tl + NN2, Sx, wz);
    eval_col<K>(tl + 2 * NN2, Sx, pf);
    if (WITH_D) eval_col<K>(tl + 3 * NN2, Sx, pv);
    const T *G = mesh.qgeo + (long)c * 5 * NQ2;
    T V[NQ], Gxi[NQ], Get[NQ];
#pragma unroll
    for (int qz = 0; qz < NQ; ++qz) {
      const auto g = qgeo<K>(G, qz * NQ + col);
      // C: submit_gradient(-cC hg pfix w)
      const T gx = SC * (-cC * HG * pf[qz] * wx[qz]);
      const T gz = SC * (-cC * HG * pf[qz] * wz[qz]);
      Gxi[qz] = g.xx * gx + g.xz * gz;
      Get[qz] = g.ex * gx + g.ez * gz;
      V[qz] = WITH_D ? (T(1.0) / GM1) * pv[qz] * g.jxw : T(0.0);
    }
    T *xa = xab + lc * 2 * NN * NQ;
    integrate_col_z<K, WITH_D, true>(V, Gxi, Get, xa, xa + NN * NQ, col);
    for (int f = 0; f < 4; ++f) {
      const int nb = mesh.nbr[c * 4 + f];
      T val = T(0.0);
      if (nb >= 0) {
        const int nf = mesh.nbrf[c * 4 + f];
        const T *fg = mesh.fgeo + ((long)c * 4 + f) * 3 * NQ;
        const T n0 = fg[col], n1 = fg[NQ + col], jxw = fg[2 * NQ + col];
        const T wxp = face_val<K>(tl, f, Sx), wzp = face_val<K>(tl + NN2, f, Sx);
        const T pfp = face_val<K>(tl + 2 * NN2, f, Sx);
        const T wxm = face_val<K>(w + (long)nb * 2 * NN2, nf, Sx);
        const T wzm = face_val<K>(w + ((long)nb * 2 + 1) * NN2, nf, Sx);
        const T pfm = face_val<K>(pfix + (long)nb * NN2, nf, Sx);
        const T av0 = T(0.5) * HG * (pfp * wxp + pfm * wxm);
        const T av1 = T(0.5) * HG * (pfp * wzp + pfm * wzm);
        const T lam = fmax(fabs(wxp * n0 + wzp * n1), fabs(wxm * n0 + wzm * n1));
        const T je = T(1.0) / GM1 * (pfp - pfm);
        val = SC * cC * ((av0 * n0 + av1 * n1) + T(0.5) * lam * je) * jxw;
      }
      fb[(lc * 4 + f) * NQ + col] = val;
    }
  }
  __syncthreads();
  if (active && col < NN) {
    T St[NQ], Dt[NQ], out[NN];
    load_cols<K>(col, St, Dt);
    const T *xa = xab + lc * 2 * NN * NQ;
    integrate_out<K, true>(xa, xa + NN * NQ, St, Dt, out);
    add_face_out<K>(fb + lc * 4 * NQ, col, St, out);
    T *d = dst + (long)c * NN2;
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      const int i = iz * NN + col;
      if (MODE == 2) d[i] = invd[(long)c * NN2 + i] * out[iz];
      else if (MODE == 3) d[i] -= out[iz];
      else d[i] = out[iz];
    }
  }
}

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
// One warp per cell: assemble the (weighted) cell mass matrix by sum
// factorisation, invert it in place by Gauss-Jordan elimination (SPD, no
// pivoting) and store it transposed.
constexpr int BI_WARPS = 2;
template <int K, typename T>
__global__ void __launch_bounds__(32 * BI_WARPS)
    k_block_inverse(T *__restrict__ out, const T *__restrict__ weight, MeshT<T> mesh) {
  constexpr int NN = K + 1, NQ = 2 * K + 1, NN2 = NN * NN, NQ2 = NQ * NQ;
  constexpr int PER = NQ2 + NQ * NN * NN + NN2 * NN2;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * BI_WARPS + warp;
  if (c >= mesh.nc) return;  // warp-uniform; no block-wide barriers below
  T *wq = sm + warp * PER;
  T *Tb = wq + NQ2;
  T *M = Tb + NQ * NN * NN;
  const T *G = mesh.qgeo + (long)c * 5 * NQ2;
  for (int q = lane; q < NQ2; q += 32) {
    const int qz = q / NQ, qx = q - qz * NQ;
    T wv = T(1.0);
    if (weight) {
      const T *wt = weight + (long)c * NN2;
      T s = T(0.0);
      for (int iz = 0; iz < NN; ++iz) {
        T t = T(0.0);
        for (int ix = 0; ix < NN; ++ix) t = fma(bS<K, T>(qx, ix), wt[iz * NN + ix], t);
        s = fma(bS<K, T>(qz, iz), t, s);
      }
      wv = s;
    }
    wq[q] = wv * G[4 * NQ2 + q];
  }
  __syncwarp();
  for (int e = lane; e < NQ * NN * NN; e += 32) {
    const int qz = e / (NN * NN), r = e - qz * NN * NN, ix = r / NN, jx = r - ix * NN;
    T s = T(0.0);
    for (int qx = 0; qx < NQ; ++qx) s = fma(bS<K, T>(qx, ix) * bS<K, T>(qx, jx), wq[qz * NQ + qx], s);
    Tb[e] = s;
  }
  __syncwarp();
  for (int e = lane; e < NN2 * NN2; e += 32) {
    const int i = e / NN2, j = e - i * NN2;
    const int iz = i / NN, ix = i - iz * NN, jz = j / NN, jx = j - jz * NN;
    T s = T(0.0);
    for (int qz = 0; qz < NQ; ++qz)
      s = fma(bS<K, T>(qz, iz) * bS<K, T>(qz, jz), Tb[(qz * NN + ix) * NN + jx], s);
    M[e] = s;
  }
  __syncwarp();
  for (int pv = 0; pv < NN2; ++pv) {
    const T d = T(1.0) / M[pv * NN2 + pv];
    __syncwarp();
    for (int j = lane; j < NN2; j += 32)
      if (j != pv) M[pv * NN2 + j] *= d;
    __syncwarp();
    for (int e = lane; e < NN2 * NN2; e += 32) {
      const int i = e / NN2, j = e - i * NN2;
      if (i != pv && j != pv) M[e] -= M[i * NN2 + pv] * M[pv * NN2 + j];
    }
    __syncwarp();
    for (int i = lane; i < NN2; i += 32)
      if (i != pv) M[i * NN2 + pv] = -M[i * NN2 + pv] * d;
    if (lane == 0) M[pv * NN2 + pv] = d;
    __syncwarp();
  }
  T *o = out + (long)c * NN2 * NN2;
  for (int e = lane; e < NN2 * NN2; e += 32) {
    const int j = e / NN2, i = e - j * NN2;
    o[e] = M[i * NN2 + j];
  }
}

// dst[c][comp][i] = scale * sum_j Binv[c][i][j] src[c][comp][j]  (transposed storage)
template <int K, typename T>
__global__ void k_block_apply(T *__restrict__ dst, const T *__restrict__ src,
                              const T *__restrict__ binvT, int ncomp, T scale,
                              int nc) {
  constexpr int NN2 = (K + 1) * (K + 1);
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long)nc * NN2) return;
  const int c = (int)(g / NN2), i = (int)(g - (long)c * NN2);
  const T *B = binvT + (long)c * NN2 * NN2;
  for (int comp = 0; comp < ncomp; ++comp) {
    const T *s = src + ((long)c * ncomp + comp) * NN2;
    T acc = T(0.0);
#pragma unroll 4
    for (int j = 0; j < NN2; ++j) acc = fma(B[j * NN2 + i], s[j], acc);
    dst[((long)c * ncomp + comp) * NN2 + i] = scale * acc;
  }
}

// ============================================================ launchers ===
namespace {
template <typename T>
struct OpView {
  int k, nc;
  MeshT<T> mesh;
  const T *ainv;
  const T *invd;
  cudaStream_t st;
};

OpView<double> view(const atm_ctx &c) {
  return OpView<double>{c.k, c.nc, c.mesh, c.ainv, c.invdiag_D, c.stream};
}

template <int K, typename T>
int B_launch(const OpView<T> &v, T *dst, const T *p, T cB, int mode) {
  using C = Cfg<K>;
  const int grid = (v.nc + C::CPB - 1) / C::CPB;
  const size_t sm = smem_bytes<K, T>(1, 2) + sizeof(T) * C::CPB * 2 * C::NN2;
  if (mode == 0) k_B<K, 0, T><<<grid, C::THREADS, sm, v.st>>>(dst, p, cB, v.ainv, v.mesh);
  else if (mode == 1) k_B<K, 1, T><<<grid, C::THREADS, sm, v.st>>>(dst, p, cB, v.ainv, v.mesh);
  else k_B<K, 2, T><<<grid, C::THREADS, sm, v.st>>>(dst, p, cB, v.ainv, v.mesh);
  ATM_CHECK_LAUNCH("k_B");
  return ATM_OK;
}

template <int K, typename T>
int CD_launch(const OpView<T> &v, T *dst, const T *w, const T *p, const T *pfix, T cC,
              int mode) {
  using C = Cfg<K>;
  const int grid = (v.nc + C::CPB - 1) / C::CPB;
  const size_t sm = smem_bytes<K, T>(4, 1);
  switch (mode) {
    case 0: k_CD<K, 0, T><<<grid, C::THREADS, sm, v.st>>>(dst, w, p, pfix, cC, v.invd, v.mesh); break;
    case 1: k_CD<K, 1, T><<<grid, C::THREADS, sm, v.st>>>(dst, w, p, pfix, cC, v.invd, v.mesh); break;
    case 2: k_CD<K, 2, T><<<grid, C::THREADS, sm, v.st>>>(dst, w, p, pfix, cC, v.invd, v.mesh); break;
    default: k_CD<K, 3, T><<<grid, C::THREADS, sm, v.st>>>(dst, w, p, pfix, cC, v.invd, v.mesh); break;
  }
  ATM_CHECK_LAUNCH("k_CD");
  return ATM_OK;
}

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
  constexpr int NN = K + 1, NQ = 2 * K + 1, NN2 = NN * NN, NQ2 = NQ * NQ;
  const size_t sm = sizeof(T) * BI_WARPS * (NQ2 + NQ * NN * NN + NN2 * NN2);
  if (sm > 48 * 1024)
    ATM_CUDA(cudaFuncSetAttribute(k_block_inverse<K, T>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
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

#define ATM_DISPATCH_K(kk, call)          \
  switch (kk) {                           \
    case 1: { constexpr int K = 1; return call; } \
    case 2: { constexpr int K = 2; return call; } \
    case 3: { constexpr int K = 3; return call; } \
    case 4: { constexpr int K = 4; return call; } \
    case 5: { constexpr int K = 5; return call; } \
    default: return ATM_BAD_ARG;          \
  }

// ---- FP64 operator launchers (timed) -------------------------------------
int launch_B(const atm_ctx &c, double *dst, const double *p, double coeff, int mode) {
  const double ns = (double)c.nc * c.nn2;
  // p read; B p written (2 comps); mode 1 reads dst too; mode 2 reads A^{-1}
  const double bytes = 8.0 * ns * (1 + 2 + (mode == 1 ? 2 : 0)) +
                       (mode == 2 ? 8.0 * c.nc * c.nn2 * c.nn2 : 0.0);
  const double flops = c.nc * (fl_eval(c.k) + 2 * fl_integrate(c.k, true) +
                               4.0 * (2 * fl_face(c.k) + 2 * fl_face(c.k)) +
                               (mode == 2 ? 4.0 * c.nn2 * c.nn2 : 0.0));
  TimedRegion tr(c, KF_B, bytes, flops);
  ATM_DISPATCH_K(c.k, (B_launch<K, double>(view(c), dst, p, coeff, mode)));
}
int launch_CD(const atm_ctx &c, double *dst, const double *w, const double *p,
              const double *pfix, double coeff, int mode) {
  const double ns = (double)c.nc * c.nn2;
  const bool wd = (mode == 1 || mode == 2);
  // w (2 comps) + pfix read, [p], [inverse diagonal], [dst read], dst written
  const double bytes = 8.0 * ns * (3 + (wd ? 1 : 0) + (mode == 2 ? 1 : 0) + (mode == 3 ? 1 : 0) + 1);
  const double flops = c.nc * ((wd ? 4 : 3) * fl_eval(c.k) + fl_integrate(c.k, true) +
                               4.0 * (2 * 3 * fl_face(c.k) + fl_face(c.k)));
  TimedRegion tr(c, KF_CD, bytes, flops);
  ATM_DISPATCH_K(c.k, (CD_launch<K, double>(view(c), dst, w, p, pfix, coeff, mode)));
}
int launch_mass(const atm_ctx &c, double *dst, const double *src, int ncomp,
                const double *weight, double scale) {
  const double ns = (double)c.nc * c.nn2;
  const double bytes = 8.0 * ns * (2 * ncomp + (weight ? 1 : 0));
  const double flops = c.nc * ((ncomp + (weight ? 1 : 0)) * fl_eval(c.k) +
                               ncomp * fl_integrate(c.k, false));
  TimedRegion tr(c, KF_MASS, bytes, flops);
  ATM_DISPATCH_K(c.k, (mass_launch<K, double>(view(c), dst, src, ncomp, weight, scale)));
}
int launch_inv_diag(const atm_ctx &c, double *out, int ncomp, const double *weight,
                    double scale) {
  TimedRegion tr(c, KF_DIAG, 8.0 * c.nc * c.nn2 * (ncomp + (weight ? 1 : 0)), 0.0);
  ATM_DISPATCH_K(c.k, (invdiag_launch<K, double>(view(c), out, ncomp, weight, scale)));
}
int launch_block_inverse(const atm_ctx &c, double *out, const double *weight) {
  const double nn = c.nn, nq = c.nq, nn2 = c.nn2;
  // weight read, inverse written; flops: mass assembly + Gauss-Jordan
  const double bytes = 8.0 * c.nc * (nn2 * (weight ? 1 : 0) + nn2 * nn2);
  const double flops = c.nc * (2.0 * (nq * nn * nn * nq + nn2 * nn2 * nq) + 2.0 * nn2 * nn2 * nn2);
  TimedRegion tr(c, KF_BLOCK_INV, bytes, flops);
  ATM_DISPATCH_K(c.k, (block_inverse_launch<K, double>(view(c), out, weight)));
}
int launch_block_apply(const atm_ctx &c, double *dst, const double *src, const double *binv,
                       int ncomp, double scale) {
  const double nn2 = c.nn2;
  const double bytes = 8.0 * c.nc * (nn2 * nn2 + 2.0 * ncomp * nn2);
  const double flops = 2.0 * c.nc * ncomp * nn2 * nn2;
  TimedRegion tr(c, KF_BLOCK_APPLY, bytes, flops);
  ATM_DISPATCH_K(c.k, (block_apply_launch<K, double>(view(c), dst, src, binv, ncomp, scale)));
}

// ---- launchers on a multigrid level (untimed; float or double) -----------
template <typename T>
int level_B(const LevelViewT<T> &v, T *dst, const T *p, T cB, int mode) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st};
  ATM_DISPATCH_K(v.k, (B_launch<K, T>(o, dst, p, cB, mode)));
}
template <typename T>
int level_CD(const LevelViewT<T> &v, T *dst, const T *w, const T *p, const T *pfix, T cC,
             int mode) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st};
  ATM_DISPATCH_K(v.k, (CD_launch<K, T>(o, dst, w, p, pfix, cC, mode)));
}
template <typename T>
int level_inv_diag(const LevelViewT<T> &v, T *out, T scale) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st};
  ATM_DISPATCH_K(v.k, (invdiag_launch<K, T>(o, out, 1, (const T *)nullptr, scale)));
}
template <typename T>
int level_block_inverse(const LevelViewT<T> &v, T *out, const T *weight) {
  OpView<T> o{v.k, v.nc, v.mesh, v.ainv, v.invd, v.st};
  ATM_DISPATCH_K(v.k, (block_inverse_launch<K, T>(o, out, weight)));
}
#define ATM_LEVEL_INST(T)                                                                   \
  template int level_B<T>(const LevelViewT<T> &, T *, const T *, T, int);                   \
  template int level_CD<T>(const LevelViewT<T> &, T *, const T *, const T *, const T *, T, int); \
  template int level_inv_diag<T>(const LevelViewT<T> &, T *, T);                            \
  template int level_block_inverse<T>(const LevelViewT<T> &, T *, const T *);
ATM_LEVEL_INST(float)
ATM_LEVEL_INST(double)

}  // namespace atm
