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
template <int K, int MODE>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_B(double *__restrict__ dst, const double *__restrict__ p, double cB,
        const double *__restrict__ ainv, Mesh mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  constexpr int NT = 1;
  extern __shared__ double sm[];
  double *tiles = sm;
  double *xab = tiles + CPB * NT * NN2;  // [CPB][2][2][NN*NQ]
  double *fb = xab + CPB * 4 * NN * NQ;  // [CPB][2][4][NQ]
  double *bt = fb + CPB * 8 * NQ;        // [CPB][2][NN2] (MODE 2)
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  load_tiles<K>(tiles, NT, 0, p, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  double Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const double *T = tiles + lc * NT * NN2;
    double pv[NQ];
    eval_col<K>(T, Sx, pv);
    const double *G = mesh.qgeo + (long)c * 5 * NQ2;
    double V[NQ], Gxi[NQ], Get[NQ];
    // submit_divergence(-cB p): component d is tested with d(phi)/dx_d
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
#pragma unroll
      for (int qz = 0; qz < NQ; ++qz) {
        const QGeo g = qgeo<K>(G, qz * NQ + col);
        const double s = -cB * pv[qz];
        Gxi[qz] = (comp == 0 ? g.xx : g.xz) * s;
        Get[qz] = (comp == 0 ? g.ex : g.ez) * s;
        V[qz] = 0.0;
      }
      double *xa = xab + (lc * 2 + comp) * 2 * NN * NQ;
      integrate_col_z<K, false, true>(V, Gxi, Get, xa, xa + NN * NQ, col);
    }
    for (int f = 0; f < 4; ++f) {
      const int nb = mesh.nbr[c * 4 + f];
      const double *fg = mesh.fgeo + ((long)c * 4 + f) * 3 * NQ;
      const double n0 = fg[col], n1 = fg[NQ + col], jxw = fg[2 * NQ + col];
      const double pp = face_val<K>(T, f, Sx);
      double avg;
      if (nb >= 0) {
        const double pm = face_val<K>(p + (long)nb * NN2, mesh.nbrf[c * 4 + f], Sx);
        avg = 0.5 * (pp + pm);
      } else {
        avg = 0.5 * (pp + pp);  // wall, p_D = p
      }
      fb[((lc * 2 + 0) * 4 + f) * NQ + col] = cB * avg * n0 * jxw;
      fb[((lc * 2 + 1) * 4 + f) * NQ + col] = cB * avg * n1 * jxw;
    }
  }
  __syncthreads();
  if (active && col < NN) {
    double St[NQ], Dt[NQ];
    load_cols<K>(col, St, Dt);
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      double out[NN];
      const double *xa = xab + (lc * 2 + comp) * 2 * NN * NQ;
      integrate_out<K, true>(xa, xa + NN * NQ, St, Dt, out);
      add_face_out<K>(fb + (lc * 2 + comp) * 4 * NQ, col, St, out);
      if (MODE == 2) {
#pragma unroll
        for (int iz = 0; iz < NN; ++iz) bt[(lc * 2 + comp) * NN2 + iz * NN + col] = out[iz];
      } else {
        double *d = dst + ((long)c * 2 + comp) * NN2;
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
      const double *Ab = ainv + (long)c * NN2 * NN2;
      const double *b0 = bt + (lc * 2 + 0) * NN2, *b1 = bt + (lc * 2 + 1) * NN2;
      for (int i = col; i < NN2; i += NQ) {
        double s0 = 0.0, s1 = 0.0;
#pragma unroll 5
        for (int j = 0; j < NN2; ++j) {
          const double a = Ab[j * NN2 + i];  // transposed storage
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
template <int K, int MODE>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_CD(double *__restrict__ dst, const double *__restrict__ w, const double *__restrict__ p,
         const double *__restrict__ pfix, double cC, const double *__restrict__ invd,
         Mesh mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  constexpr bool WITH_D = (MODE == 1 || MODE == 2);
  constexpr int NT = WITH_D ? 4 : 3;  // w(2), pfix, [p]
  constexpr double GM1 = GAS_GAMMA - 1.0;
  constexpr double HG = GAS_GAMMA / (GAS_GAMMA - 1.0);
  // sign of the C contribution in dst
  constexpr double SC = WITH_D ? -1.0 : 1.0;
  extern __shared__ double sm[];
  double *tiles = sm;
  double *xab = tiles + CPB * NT * NN2;
  double *fb = xab + CPB * 2 * NN * NQ;
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  load_tiles<K>(tiles, NT, 0, w, 2, c0, cnt);
  load_tiles<K>(tiles, NT, 2, pfix, 1, c0, cnt);
  if (WITH_D) load_tiles<K>(tiles, NT, 3, p, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  double Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const double *T = tiles + lc * NT * NN2;
    double wx[NQ], wz[NQ], pf[NQ], pv[NQ];
    eval_col<K>(T, Sx, wx);
    eval_col<K>(T + NN2, Sx, wz);
    eval_col<K>(T + 2 * NN2, Sx, pf);
    if (WITH_D) eval_col<K>(T + 3 * NN2, Sx, pv);
    const double *G = mesh.qgeo + (long)c * 5 * NQ2;
    double V[NQ], Gxi[NQ], Get[NQ];
#pragma unroll
    for (int qz = 0; qz < NQ; ++qz) {
      const QGeo g = qgeo<K>(G, qz * NQ + col);
      // C: submit_gradient(-cC hg pfix w)
      const double gx = SC * (-cC * HG * pf[qz] * wx[qz]);
      const double gz = SC * (-cC * HG * pf[qz] * wz[qz]);
      Gxi[qz] = g.xx * gx + g.xz * gz;
      Get[qz] = g.ex * gx + g.ez * gz;
      V[qz] = WITH_D ? (1.0 / GM1) * pv[qz] * g.jxw : 0.0;
    }
    double *xa = xab + lc * 2 * NN * NQ;
    integrate_col_z<K, WITH_D, true>(V, Gxi, Get, xa, xa + NN * NQ, col);
    for (int f = 0; f < 4; ++f) {
      const int nb = mesh.nbr[c * 4 + f];
      double val = 0.0;
      if (nb >= 0) {
        const int nf = mesh.nbrf[c * 4 + f];
        const double *fg = mesh.fgeo + ((long)c * 4 + f) * 3 * NQ;
        const double n0 = fg[col], n1 = fg[NQ + col], jxw = fg[2 * NQ + col];
        const double wxp = face_val<K>(T, f, Sx), wzp = face_val<K>(T + NN2, f, Sx);
        const double pfp = face_val<K>(T + 2 * NN2, f, Sx);
        const double wxm = face_val<K>(w + (long)nb * 2 * NN2, nf, Sx);
        const double wzm = face_val<K>(w + ((long)nb * 2 + 1) * NN2, nf, Sx);
        const double pfm = face_val<K>(pfix + (long)nb * NN2, nf, Sx);
        const double av0 = 0.5 * HG * (pfp * wxp + pfm * wxm);
        const double av1 = 0.5 * HG * (pfp * wzp + pfm * wzm);
        const double lam = fmax(fabs(wxp * n0 + wzp * n1), fabs(wxm * n0 + wzm * n1));
        const double je = 1.0 / GM1 * (pfp - pfm);
        val = SC * cC * ((av0 * n0 + av1 * n1) + 0.5 * lam * je) * jxw;
      }
      fb[(lc * 4 + f) * NQ + col] = val;
    }
  }
  __syncthreads();
  if (active && col < NN) {
    double St[NQ], Dt[NQ], out[NN];
    load_cols<K>(col, St, Dt);
    const double *xa = xab + lc * 2 * NN * NQ;
    integrate_out<K, true>(xa, xa + NN * NQ, St, Dt, out);
    add_face_out<K>(fb + lc * 4 * NQ, col, St, out);
    double *d = dst + (long)c * NN2;
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
template <int K, int NCOMP, bool WEIGHTED>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_mass(double *__restrict__ dst, const double *__restrict__ src,
           const double *__restrict__ weight, double scale, Mesh mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  constexpr int NT = NCOMP + (WEIGHTED ? 1 : 0);
  extern __shared__ double sm[];
  double *tiles = sm;
  double *xab = tiles + CPB * NT * NN2;  // [CPB][NCOMP][NN*NQ]
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  load_tiles<K>(tiles, NT, 0, src, NCOMP, c0, cnt);
  if (WEIGHTED) load_tiles<K>(tiles, NT, NCOMP, weight, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  double Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const double *T = tiles + lc * NT * NN2;
    double wv[NQ];
    if (WEIGHTED) eval_col<K>(T + NCOMP * NN2, Sx, wv);
    const double *G = mesh.qgeo + (long)c * 5 * NQ2;
#pragma unroll
    for (int comp = 0; comp < NCOMP; ++comp) {
      double v[NQ], V[NQ];
      eval_col<K>(T + comp * NN2, Sx, v);
#pragma unroll
      for (int qz = 0; qz < NQ; ++qz) {
        const double jxw = G[4 * NQ2 + qz * NQ + col];
        V[qz] = (WEIGHTED ? wv[qz] * v[qz] : scale * v[qz]) * jxw;
      }
      integrate_col_z<K, true, false>(V, V, V, xab + (lc * NCOMP + comp) * NN * NQ, nullptr,
                                      col);
    }
  }
  __syncthreads();
  if (active && col < NN) {
    double St[NQ], Dt[NQ];
    load_cols<K>(col, St, Dt);
#pragma unroll
    for (int comp = 0; comp < NCOMP; ++comp) {
      double out[NN];
      integrate_out<K, false>(xab + (lc * NCOMP + comp) * NN * NQ, nullptr, St, Dt, out);
      double *d = dst + ((long)c * NCOMP + comp) * NN2;
#pragma unroll
      for (int iz = 0; iz < NN; ++iz) d[iz * NN + col] = out[iz];
    }
  }
}

// ===================================================== inverse diagonal ===
template <int K, bool WEIGHTED>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_invdiag(double *__restrict__ out, int ncomp, const double *__restrict__ weight,
              double scale, Mesh mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  extern __shared__ double sm[];
  double *tiles = sm;                      // [CPB][NN2] weight
  double *xab = tiles + CPB * NN2;         // [CPB][NN*NQ]
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  if (WEIGHTED) load_tiles<K>(tiles, 1, 0, weight, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  double Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    double wv[NQ];
    if (WEIGHTED) eval_col<K>(tiles + lc * NN2, Sx, wv);
    const double *G = mesh.qgeo + (long)c * 5 * NQ2;
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      double s = 0.0;
#pragma unroll
      for (int qz = 0; qz < NQ; ++qz) {
        const double b = bS<K>(qz, iz);
        const double wj = (WEIGHTED ? wv[qz] : scale) * G[4 * NQ2 + qz * NQ + col];
        s = fma(b * b, wj, s);
      }
      xab[lc * NN * NQ + iz * NQ + col] = s;
    }
  }
  __syncthreads();
  if (active && col < NN) {
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      double s = 0.0;
#pragma unroll
      for (int qx = 0; qx < NQ; ++qx) {
        const double b = bS<K>(qx, col);
        s = fma(b * b, xab[lc * NN * NQ + iz * NQ + qx], s);
      }
      const double inv = 1.0 / s;
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
template <int K>
__global__ void __launch_bounds__(32 * BI_WARPS)
    k_block_inverse(double *__restrict__ out, const double *__restrict__ weight, Mesh mesh) {
  constexpr int NN = K + 1, NQ = 2 * K + 1, NN2 = NN * NN, NQ2 = NQ * NQ;
  constexpr int PER = NQ2 + NQ * NN * NN + NN2 * NN2;
  extern __shared__ double sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * BI_WARPS + warp;
  if (c >= mesh.nc) return;  // warp-uniform; no block-wide barriers below
  double *wq = sm + warp * PER;
  double *T = wq + NQ2;
  double *M = T + NQ * NN * NN;
  const double *G = mesh.qgeo + (long)c * 5 * NQ2;
  for (int q = lane; q < NQ2; q += 32) {
    const int qz = q / NQ, qx = q - qz * NQ;
    double wv = 1.0;
    if (weight) {
      const double *wt = weight + (long)c * NN2;
      double s = 0.0;
      for (int iz = 0; iz < NN; ++iz) {
        double t = 0.0;
        for (int ix = 0; ix < NN; ++ix) t = fma(bS<K>(qx, ix), wt[iz * NN + ix], t);
        s = fma(bS<K>(qz, iz), t, s);
      }
      wv = s;
    }
    wq[q] = wv * G[4 * NQ2 + q];
  }
  __syncwarp();
  for (int e = lane; e < NQ * NN * NN; e += 32) {
    const int qz = e / (NN * NN), r = e - qz * NN * NN, ix = r / NN, jx = r - ix * NN;
    double s = 0.0;
    for (int qx = 0; qx < NQ; ++qx) s = fma(bS<K>(qx, ix) * bS<K>(qx, jx), wq[qz * NQ + qx], s);
    T[e] = s;
  }
  __syncwarp();
  for (int e = lane; e < NN2 * NN2; e += 32) {
    const int i = e / NN2, j = e - i * NN2;
    const int iz = i / NN, ix = i - iz * NN, jz = j / NN, jx = j - jz * NN;
    double s = 0.0;
    for (int qz = 0; qz < NQ; ++qz)
      s = fma(bS<K>(qz, iz) * bS<K>(qz, jz), T[(qz * NN + ix) * NN + jx], s);
    M[e] = s;
  }
  __syncwarp();
  for (int pv = 0; pv < NN2; ++pv) {
    const double d = 1.0 / M[pv * NN2 + pv];
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
  double *o = out + (long)c * NN2 * NN2;
  for (int e = lane; e < NN2 * NN2; e += 32) {
    const int j = e / NN2, i = e - j * NN2;
    o[e] = M[i * NN2 + j];
  }
}

// dst[c][comp][i] = scale * sum_j Binv[c][i][j] src[c][comp][j]  (transposed storage)
template <int K>
__global__ void k_block_apply(double *__restrict__ dst, const double *__restrict__ src,
                              const double *__restrict__ binvT, int ncomp, double scale,
                              int nc) {
  constexpr int NN2 = (K + 1) * (K + 1);
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long)nc * NN2) return;
  const int c = (int)(g / NN2), i = (int)(g - (long)c * NN2);
  const double *B = binvT + (long)c * NN2 * NN2;
  for (int comp = 0; comp < ncomp; ++comp) {
    const double *s = src + ((long)c * ncomp + comp) * NN2;
    double acc = 0.0;
#pragma unroll 4
    for (int j = 0; j < NN2; ++j) acc = fma(B[j * NN2 + i], s[j], acc);
    dst[((long)c * ncomp + comp) * NN2 + i] = scale * acc;
  }
}

// ============================================================ launchers ===
namespace {
template <int K>
int B_launch(const atm_ctx &c, double *dst, const double *p, double cB, int mode) {
  using C = Cfg<K>;
  const int grid = (c.nc + C::CPB - 1) / C::CPB;
  const size_t sm = smem_bytes<K>(1, 2) + sizeof(double) * C::CPB * 2 * C::NN2;
  const double ns = (double)c.nc * C::NN2;
  // p read; B p written (2 comps); mode 1 reads dst too; mode 2 reads A^{-1}
  const double bytes = 8.0 * ns * (1 + 2 + (mode == 1 ? 2 : 0)) +
                       (mode == 2 ? 8.0 * c.nc * C::NN2 * C::NN2 : 0.0);
  const double flops = c.nc * (fl_eval(K) + 2 * fl_integrate(K, true) +
                               4.0 * (2 * fl_face(K) + 2 * fl_face(K)) +
                               (mode == 2 ? 4.0 * C::NN2 * C::NN2 : 0.0));
  TimedRegion tr(c, KF_B, bytes, flops);
  if (mode == 0) k_B<K, 0><<<grid, C::THREADS, sm, c.stream>>>(dst, p, cB, c.ainv, c.mesh);
  else if (mode == 1) k_B<K, 1><<<grid, C::THREADS, sm, c.stream>>>(dst, p, cB, c.ainv, c.mesh);
  else k_B<K, 2><<<grid, C::THREADS, sm, c.stream>>>(dst, p, cB, c.ainv, c.mesh);
  ATM_CHECK_LAUNCH("k_B");
  return ATM_OK;
}

template <int K>
int CD_launch(const atm_ctx &c, double *dst, const double *w, const double *p,
              const double *pfix, double cC, int mode) {
  using C = Cfg<K>;
  const int grid = (c.nc + C::CPB - 1) / C::CPB;
  const size_t sm = smem_bytes<K>(4, 1);
  const double ns = (double)c.nc * C::NN2;
  const bool wd = (mode == 1 || mode == 2);
  // w (2 comps) + pfix read, [p], [inverse diagonal], [dst read], dst written
  const double bytes = 8.0 * ns * (3 + (wd ? 1 : 0) + (mode == 2 ? 1 : 0) + (mode == 3 ? 1 : 0) + 1);
  const double flops = c.nc * ((wd ? 4 : 3) * fl_eval(K) + fl_integrate(K, true) +
                               4.0 * (2 * 3 * fl_face(K) + fl_face(K)));
  TimedRegion tr(c, KF_CD, bytes, flops);
  switch (mode) {
    case 0: k_CD<K, 0><<<grid, C::THREADS, sm, c.stream>>>(dst, w, p, pfix, cC, c.invdiag_D, c.mesh); break;
    case 1: k_CD<K, 1><<<grid, C::THREADS, sm, c.stream>>>(dst, w, p, pfix, cC, c.invdiag_D, c.mesh); break;
    case 2: k_CD<K, 2><<<grid, C::THREADS, sm, c.stream>>>(dst, w, p, pfix, cC, c.invdiag_D, c.mesh); break;
    default: k_CD<K, 3><<<grid, C::THREADS, sm, c.stream>>>(dst, w, p, pfix, cC, c.invdiag_D, c.mesh); break;
  }
  ATM_CHECK_LAUNCH("k_CD");
  return ATM_OK;
}

template <int K>
int mass_launch(const atm_ctx &c, double *dst, const double *src, int ncomp,
                const double *weight, double scale) {
  using C = Cfg<K>;
  const int grid = (c.nc + C::CPB - 1) / C::CPB;
  const size_t sm = sizeof(double) * C::CPB * (3 * C::NN2 + 2 * C::NN * C::NQ);
  const double ns = (double)c.nc * C::NN2;
  const double bytes = 8.0 * ns * (2 * ncomp + (weight ? 1 : 0));
  const double flops = c.nc * ((ncomp + (weight ? 1 : 0)) * fl_eval(K) +
                               ncomp * fl_integrate(K, false));
  TimedRegion tr(c, KF_MASS, bytes, flops);
  if (ncomp == 1 && !weight) k_mass<K, 1, false><<<grid, C::THREADS, sm, c.stream>>>(dst, src, weight, scale, c.mesh);
  else if (ncomp == 1) k_mass<K, 1, true><<<grid, C::THREADS, sm, c.stream>>>(dst, src, weight, scale, c.mesh);
  else if (!weight) k_mass<K, 2, false><<<grid, C::THREADS, sm, c.stream>>>(dst, src, weight, scale, c.mesh);
  else k_mass<K, 2, true><<<grid, C::THREADS, sm, c.stream>>>(dst, src, weight, scale, c.mesh);
  ATM_CHECK_LAUNCH("k_mass");
  return ATM_OK;
}

template <int K>
int invdiag_launch(const atm_ctx &c, double *out, int ncomp, const double *weight,
                   double scale) {
  using C = Cfg<K>;
  const int grid = (c.nc + C::CPB - 1) / C::CPB;
  const size_t sm = sizeof(double) * C::CPB * (C::NN2 + C::NN * C::NQ);
  TimedRegion tr(c, KF_DIAG, 8.0 * c.nc * C::NN2 * (ncomp + (weight ? 1 : 0)), 0.0);
  if (weight) k_invdiag<K, true><<<grid, C::THREADS, sm, c.stream>>>(out, ncomp, weight, scale, c.mesh);
  else k_invdiag<K, false><<<grid, C::THREADS, sm, c.stream>>>(out, ncomp, weight, scale, c.mesh);
  ATM_CHECK_LAUNCH("k_invdiag");
  return ATM_OK;
}

template <int K>
int block_inverse_launch(const atm_ctx &c, double *out, const double *weight) {
  constexpr int NN = K + 1, NQ = 2 * K + 1, NN2 = NN * NN, NQ2 = NQ * NQ;
  const size_t sm = sizeof(double) * BI_WARPS * (NQ2 + NQ * NN * NN + NN2 * NN2);
  if (sm > 48 * 1024)
    ATM_CUDA(cudaFuncSetAttribute(k_block_inverse<K>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const int grid = (c.nc + BI_WARPS - 1) / BI_WARPS;
  // weight read, inverse written; flops: mass assembly + Gauss-Jordan
  const double bytes = 8.0 * c.nc * (NN2 * (weight ? 1 : 0) + NN2 * NN2);
  const double flops = c.nc * (2.0 * (NQ * NN * NN * NQ + NN2 * NN2 * NQ) + 2.0 * NN2 * NN2 * NN2);
  TimedRegion tr(c, KF_BLOCK_INV, bytes, flops);
  k_block_inverse<K><<<grid, 32 * BI_WARPS, sm, c.stream>>>(out, weight, c.mesh);
  ATM_CHECK_LAUNCH("k_block_inverse");
  return ATM_OK;
}

template <int K>
int block_apply_launch(const atm_ctx &c, double *dst, const double *src, const double *binv,
                       int ncomp, double scale) {
  constexpr int NN2 = (K + 1) * (K + 1);
  const long n = (long)c.nc * NN2;
  const int threads = 256;
  const int grid = (int)((n + threads - 1) / threads);
  const double bytes = 8.0 * c.nc * (NN2 * NN2 + 2.0 * ncomp * NN2);
  const double flops = 2.0 * c.nc * ncomp * NN2 * NN2;
  TimedRegion tr(c, KF_BLOCK_APPLY, bytes, flops);
  k_block_apply<K><<<grid, threads, 0, c.stream>>>(dst, src, binv, ncomp, scale, c.nc);
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

int launch_B(const atm_ctx &c, double *dst, const double *p, double coeff, int mode) {
  ATM_DISPATCH_K(c.k, B_launch<K>(c, dst, p, coeff, mode));
}
int launch_CD(const atm_ctx &c, double *dst, const double *w, const double *p,
              const double *pfix, double coeff, int mode) {
  ATM_DISPATCH_K(c.k, CD_launch<K>(c, dst, w, p, pfix, coeff, mode));
}
int launch_mass(const atm_ctx &c, double *dst, const double *src, int ncomp,
                const double *weight, double scale) {
  ATM_DISPATCH_K(c.k, mass_launch<K>(c, dst, src, ncomp, weight, scale));
}
int launch_inv_diag(const atm_ctx &c, double *out, int ncomp, const double *weight,
                    double scale) {
  ATM_DISPATCH_K(c.k, invdiag_launch<K>(c, out, ncomp, weight, scale));
}
int launch_block_inverse(const atm_ctx &c, double *out, const double *weight) {
  ATM_DISPATCH_K(c.k, block_inverse_launch<K>(c, out, weight));
}
int launch_block_apply(const atm_ctx &c, double *dst, const double *src, const double *binv,
                       int ncomp, double scale) {
  ATM_DISPATCH_K(c.k, block_apply_launch<K>(c, dst, src, binv, ncomp, scale));
}

}  // namespace atm
