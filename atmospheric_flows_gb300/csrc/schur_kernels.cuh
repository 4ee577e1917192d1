// Schur-complement kernels shared by the conforming and the hanging-face
// builds: B (pressure gradient, then optionally the exact cell-wise A^{-1})
// and C/D (enthalpy divergence, internal-energy mass, Jacobi scale).
//   B   euler_operator.h:1512-1617
//   C   euler_operator.h:1413-1507
//   D   euler_operator.h:1386-1408
// HG selects the face loop with hanging faces (2:1 adaptive meshes).
// Included by impl_kernels.cu (HG = false) and hang_rhs_*.cu / hang_schur.cu (HG = true).
#pragma once
#include "atm_device.cuh"

namespace atm {

// ====================================================================== B ===
// MODE 0: dst = B p ; 1: dst -= B p ; 2: dst = A^{-1} B p
template <int K, int MODE, typename T, bool HG>
__global__ void __launch_bounds__(Cfg<K>::MAX_THREADS)
    k_B(T *__restrict__ dst, const T *__restrict__ p, T cB,
        const T *__restrict__ ainv, MeshT<T> mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2;
  const int CPB = blockDim.x / NQ;  // cells per block, chosen by the autotuner
  constexpr int NT = 1;
  // FP32 (multigrid levels): the A^{-1} blocks of the block's cells are
  // contiguous; they are copied into shared memory asynchronously at the
  // start and arrive while B is computed
  constexpr bool STAGE = MODE == 2 && sizeof(T) == 4;
  constexpr int AS = ainv_stride<K, T>();
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  T *as = sm;                       // [CPB][AS] staged A^{-1} (STAGE)
  T *tiles = sm + (STAGE ? CPB * AS : 0);
  T *xab = tiles + CPB * NT * NN2;  // [CPB][2][2][NN*NQ]
  T *fb = xab + CPB * 4 * NN * NQ;  // [CPB][2][4][NQ]
  T *bt = fb + CPB * 8 * NQ;        // [CPB][2][NN2] (MODE 2)
  T *fh = bt + CPB * 2 * NN2;       // [CPB][2][4][NQ] subface-1 values (HG)
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  if constexpr (STAGE) {
    // cells c0 .. c0+cnt-1: cnt * AS values, 16-byte aligned (AS % 4 == 0)
    const T *src = ainv + (long)c0 * AS;
    const int n16 = cnt * AS / 4;
    for (int e = tid; e < n16; e += blockDim.x) cp_async16(as + 4 * e, src + 4 * e);
    cp_async_commit();
  }
  load_tiles<K>(tiles, NT, 0, p, 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  if (mesh.dts && active) cB *= mesh.dts[c];  // per-member time step
  T Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const T *tl = tiles + lc * NT * NN2;
    T pv[NQ];
    eval_col<K>(tl, Sx, pv);
    const GeoCol<K, T> G(mesh, c, col);
    T V[NQ], Gxi[NQ], Get[NQ];
    // submit_divergence(-cB p): component d is tested with d(phi)/dx_d
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
#pragma unroll
      for (int qz = 0; qz < NQ; ++qz) {
        T gxi, get;
        if (comp == 0) G.dx(qz, gxi, get);
        else G.dz(qz, gxi, get);
        const T s = -cB * pv[qz];
        Gxi[qz] = gxi * s;
        Get[qz] = get * s;
        V[qz] = T(0.0);
      }
      T *xa = xab + (lc * 2 + comp) * 2 * NN * NQ;
      integrate_col_z<K, false, true>(V, Gxi, Get, xa, xa + NN * NQ, col);
    }
    face_terms<K, 2, HG>(mesh, c, col, Sx, fb + lc * 2 * 4 * NQ, fh + lc * 2 * 4 * NQ,
                         [&](int f, int nb, int nf, T n0, T n1, T jxw, const auto &Ro,
                             const auto &Rn, auto &val) {
      const T pp = face_val<K>(tl, f, Ro);
      T avg;
      if (nb >= 0) {
        const T pm = face_val<K>(p + (long)nb * NN2, nf, Rn);
        avg = T(0.5) * (pp + pm);
      } else {
        avg = T(0.5) * (pp + pp);  // wall, p_D = p
      }
      val[0] = cB * avg * n0 * jxw;
      val[1] = cB * avg * n1 * jxw;
    });
  }
  __syncthreads();
  if (active && col < NN) {
    T St[NQ], Dt[NQ];
    load_cols<K>(col, St, Dt);
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      T out[NN];
      const T *xa = xab + (lc * 2 + comp) * 2 * NN * NQ;
      output_phase<K, HG>(mesh, c, xa, xa + NN * NQ, fb + (lc * 2 + comp) * 4 * NQ, fh + (lc * 2 + comp) * 4 * NQ, col, St, Dt,
                          out);
      if (MODE == 2) {
#pragma unroll
        for (int iz = 0; iz < NN; ++iz) bt[(lc * 2 + comp) * NN2 + out_node<K, HG>(col, iz)] = out[iz];
      } else {
        T *d = dst + ((long)c * 2 + comp) * NN2;
#pragma unroll
        for (int iz = 0; iz < NN; ++iz) {
          if (MODE == 0) d[out_node<K, HG>(col, iz)] = out[iz];
          else d[out_node<K, HG>(col, iz)] -= out[iz];
        }
      }
    }
  }
  if (MODE == 2) {
    if constexpr (STAGE) cp_async_wait_all();
    __syncthreads();
    if (active) {
      const T *Ab = STAGE ? as + lc * AS : ainv + (long)c * AS;
      const T *b0 = bt + (lc * 2 + 0) * NN2, *b1 = bt + (lc * 2 + 1) * NN2;
      for (int i = col; i < NN2; i += NQ) {
        T s0 = T(0.0), s1 = T(0.0);
        if constexpr (STAGE) {
          // packed lower triangle: A_ij at i(i+1)/2 + j (j <= i), else
          // j(j+1)/2 + i; the same values in the same order as the full block
          const int ri = i * (i + 1) / 2;
#pragma unroll
          for (int j = 0; j < NN2; ++j) {
            const T a = j <= i ? Ab[ri + j] : Ab[j * (j + 1) / 2 + i];
            s0 = fma(a, b0[j], s0);
            s1 = fma(a, b1[j], s1);
          }
        } else {
#pragma unroll 5
          for (int j = 0; j < NN2; ++j) {
            const T a = Ab[j * NN2 + i];  // transposed storage
            s0 = fma(a, b0[j], s0);
            s1 = fma(a, b1[j], s1);
          }
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
// MODE 4: t = sD D p - C w with p = ch.x, then the Chebyshev update of ch
//         (x and d, with rhs and invd) instead of a store of t
template <int K, int MODE, typename T, bool HG>
__global__ void __launch_bounds__(Cfg<K>::MAX_THREADS, sizeof(T) == 4 ? 4 : 1)
    k_CD(T *__restrict__ dst, const T *__restrict__ w, const T *__restrict__ p,
         const T *__restrict__ pfix, const T *__restrict__ pfq, const T *__restrict__ pff,
         T cC, const T *__restrict__ invd, MeshT<T> mesh, ChebArgs<T> ch) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2;
  const int CPB = blockDim.x / NQ;  // cells per block, chosen by the autotuner
  constexpr bool WITH_D = (MODE == 1 || MODE == 2 || MODE == 4);
  // tiles: w(2), [p]; p_fix enters through its values at the quadrature
  // points (pfq) and its face traces (pff), prepared when p_fix is set.  The
  // hanging-face variant reads the p_fix tile (its traces are needed at
  // subface points): w(2), pfix, [p].
  constexpr bool PT = HG;  // p_fix tile
  constexpr int NT = (PT ? 3 : 2) + (WITH_D ? 1 : 0);
  constexpr int TP = PT ? 3 : 2;  // tile of p
  constexpr T GM1 = GAS_GAMMA - T(1.0);
  constexpr T HG_ = GAS_GAMMA / (GAS_GAMMA - T(1.0));  // enthalpy factor
  // sign of the C contribution in dst
  constexpr T SC = WITH_D ? -T(1.0) : T(1.0);
  // FP32 on conforming levels (latency bound): the block's own face
  // geometry, p_fix traces and quadrature values, and in MODE 4 its rhs,
  // invd and d, are contiguous; they are copied into shared memory with
  // cp.async at the start instead of being loaded thread by thread
  constexpr bool STG = sizeof(T) == 4 && !HG;
  constexpr int FGS = 12 * NQ, PFS = 4 * NQ;  // multiples of 4 values
  constexpr int NV = MODE == 4 ? 3 : 0;
  constexpr int STS = FGS + PFS + NQ2 + NV * NN2;  // staged values per cell
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *sm = reinterpret_cast<T *>(sm_raw);
  T *sfg = sm;                   // [CPB][FGS] (STG)
  T *spf = sfg + CPB * FGS;      // [CPB][PFS]
  T *spq = spf + CPB * PFS;      // [CPB][NQ2]
  T *svec = spq + CPB * NQ2;     // [NV][CPB][NN2]: rhs, invd, d
  T *tiles = sm + (STG ? (CPB * STS + 3) / 4 * 4 : 0);
  T *xab = tiles + CPB * NT * NN2;
  T *fb = xab + CPB * 2 * NN * NQ;
  T *fh = fb + CPB * 4 * NQ;  // subface-1 values (HG)
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  if constexpr (STG) {
    // cells c0 .. c0+cnt-1; fgeo and pff blocks are 16-byte aligned
    const T *gfg = mesh.fgeo + (long)c0 * FGS, *gpf = pff + (long)c0 * PFS;
    for (int e = tid; e < cnt * FGS / 4; e += blockDim.x) cp_async16(sfg + 4 * e, gfg + 4 * e);
    for (int e = tid; e < cnt * PFS / 4; e += blockDim.x) cp_async16(spf + 4 * e, gpf + 4 * e);
    const T *gpq = pfq + (long)c0 * NQ2;
    for (int e = tid; e < cnt * NQ2; e += blockDim.x) cp_async4(spq + e, gpq + e);
    if constexpr (NV > 0) {
      const T *vs[3] = {ch.rhs, invd, ch.d};
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const T *g = vs[v] + (long)c0 * NN2;
        T *d = svec + v * CPB * NN2;
        for (int e = tid; e < cnt * NN2; e += blockDim.x) cp_async4(d + e, g + e);
      }
    }
    cp_async_commit();
  }
  load_tiles<K>(tiles, NT, 0, w, 2, c0, cnt);
  if (PT) load_tiles<K>(tiles, NT, 2, pfix, 1, c0, cnt);
  if (WITH_D) load_tiles<K>(tiles, NT, TP, p, 1, c0, cnt);
  if constexpr (STG) cp_async_wait_all();
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  if (mesh.dts && active) cC *= mesh.dts[c];  // per-member time step
  T Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const T *tl = tiles + lc * NT * NN2;
    T wx[NQ], wz[NQ], pf[NQ], pv[NQ];
    eval_col<K>(tl, Sx, wx);
    eval_col<K>(tl + NN2, Sx, wz);
    if (PT) {
      eval_col<K>(tl + 2 * NN2, Sx, pf);
    } else {
      const T *pq = STG ? spq + lc * NQ2 : pfq + (long)c * NQ2;
#pragma unroll
      for (int qz = 0; qz < NQ; ++qz) pf[qz] = pq[qz * NQ + col];
    }
    if (WITH_D) eval_col<K>(tl + TP * NN2, Sx, pv);
    const GeoCol<K, T> G(mesh, c, col);
    T V[NQ], Gxi[NQ], Get[NQ];
#pragma unroll
    for (int qz = 0; qz < NQ; ++qz) {
      const auto g = G.at(qz);
      // C: submit_gradient(-cC hg pfix w)
      const T gx = SC * (-cC * HG_ * pf[qz] * wx[qz]);
      const T gz = SC * (-cC * HG_ * pf[qz] * wz[qz]);
      Gxi[qz] = g.xx * gx + g.xz * gz;
      Get[qz] = g.ex * gx + g.ez * gz;
      V[qz] = WITH_D ? (T(1.0) / GM1) * pv[qz] * g.jxw : T(0.0);
    }
    T *xa = xab + lc * 2 * NN * NQ;
    integrate_col_z<K, WITH_D, true>(V, Gxi, Get, xa, xa + NN * NQ, col);
    face_terms<K, 1, HG>(mesh, c, col, Sx, fb + lc * 4 * NQ, fh + lc * 4 * NQ,
                         [&](int f, int nb, int nf, T n0, T n1, T jxw, const auto &Ro,
                             const auto &Rn, auto &val) {
      if (nb < 0) {
        val[0] = T(0.0);
        return;
      }
      const T wxp = face_val<K>(tl, f, Ro), wzp = face_val<K>(tl + NN2, f, Ro);
      const T wxm = face_val<K>(w + (long)nb * 2 * NN2, nf, Rn);
      const T wzm = face_val<K>(w + ((long)nb * 2 + 1) * NN2, nf, Rn);
      T pfp, pfm;
      if (HG) {
        pfp = face_val<K>(tl + 2 * NN2, f, Ro);
        pfm = face_val<K>(pfix + (long)nb * NN2, nf, Rn);
      } else {  // conforming: face point col of both sides coincide
        pfp = STG ? spf[lc * PFS + f * NQ + col] : pff[((long)c * 4 + f) * NQ + col];
        pfm = pff[((long)nb * 4 + nf) * NQ + col];
      }
      const T av0 = T(0.5) * HG_ * (pfp * wxp + pfm * wxm);
      const T av1 = T(0.5) * HG_ * (pfp * wzp + pfm * wzm);
      const T lam = fmax(fabs(wxp * n0 + wzp * n1), fabs(wxm * n0 + wzm * n1));
      const T je = T(1.0) / GM1 * (pfp - pfm);
      val[0] = SC * cC * ((av0 * n0 + av1 * n1) + T(0.5) * lam * je) * jxw;
    }, STG ? sfg + lc * FGS : nullptr);
  }
  __syncthreads();
  if (active && col < NN) {
    T St[NQ], Dt[NQ], out[NN];
    load_cols<K>(col, St, Dt);
    const T *xa = xab + lc * 2 * NN * NQ;
    output_phase<K, HG>(mesh, c, xa, xa + NN * NQ, fb + lc * 4 * NQ, fh + lc * 4 * NQ, col, St, Dt,
                        out);
    T *d = MODE == 4 ? nullptr : dst + (long)c * NN2;
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      const int i = out_node<K, HG>(col, iz);
      if (MODE == 2) {
        d[i] = invd[(long)c * NN2 + i] * out[iz];
      } else if (MODE == 3) {
        d[i] -= out[iz];
      } else if (MODE == 4) {
        const long g = (long)c * NN2 + i;
        T rh, dd, iv, xx;
        if constexpr (STG) {  // staged rhs, invd, d; x = p is the tile TP
          rh = svec[lc * NN2 + i];
          iv = svec[(CPB + lc) * NN2 + i];
          dd = svec[(2 * CPB + lc) * NN2 + i];
          xx = tiles[(lc * NT + TP) * NN2 + i];
        } else {
          rh = ch.rhs[g];
          iv = invd[g];
          dd = ch.d[g];
          xx = ch.x[g];
        }
        const T r = rh - out[iz];
        const T dk = (ch.first ? T(0) : ch.a * dd) + ch.b * iv * r;
        ch.d[g] = dk;
        ch.x[g] = xx + dk;
      } else {
        d[i] = out[iz];
      }
    }
  }
}

// ========================================================== p_fix prep ===
// Values of p_fix at the quadrature points, pfq[c][qz][qx], and its traces
// on the four faces, pff[c][f][q]: the C/D kernel's p_fix input, computed
// once per p_fix instead of once per Schur apply.
template <int K, typename T>
__global__ void __launch_bounds__(Cfg<K>::THREADS)
    k_pfix_prep(T *__restrict__ pfq, T *__restrict__ pff, const T *__restrict__ pfix,
                MeshT<T> mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2, CPB = C::CPB;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T *tiles = reinterpret_cast<T *>(sm_raw);
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
  load_tiles<K>(tiles, 1, 0, pfix, 1, c0, cnt);
  __syncthreads();
  if (lc >= cnt) return;
  const int c = c0 + lc;
  const T *tl = tiles + lc * NN2;
  T Sx[NN], Dx[NN], v[NQ];
  load_rows<K>(col, Sx, Dx);
  eval_col<K>(tl, Sx, v);
#pragma unroll
  for (int qz = 0; qz < NQ; ++qz) pfq[(long)c * NQ2 + qz * NQ + col] = v[qz];
#pragma unroll
  for (int f = 0; f < 4; ++f) pff[((long)c * 4 + f) * NQ + col] = face_val<K>(tl, f, Sx);
}

// ============================================================ launchers ===
template <typename T>
struct OpView {
  int k, nc;
  MeshT<T> mesh;
  const T *ainv;
  const T *invd;
  cudaStream_t st;
  bool tune;  // the autotuner may time tile shapes on this stream
  const T *pfix, *pfq, *pff;  // frozen p_fix and its prepared values (C/D)
};

inline OpView<double> schur_view(const atm_ctx &c) {
  return OpView<double>{c.k, c.nc, c.mesh, c.ainv, c.invdiag_D, c.stream,
                        c.autotune && !c.capturing, c.pres_fix, c.pfq, c.pff};
}

template <int K, typename T, bool HG>
int B_launch(const OpView<T> &v, T *dst, const T *p, T cB, int mode) {
  using C = Cfg<K>;
  auto launch = [&](int cpb) -> cudaError_t {
    const int grid = (v.nc + cpb - 1) / cpb, th = cpb * C::NQ;
    const size_t sm = smem_bytes<K, T>(cpb, 1, 2, HG) + sizeof(T) * cpb * 2 * C::NN2 +
                      (mode == 2 && sizeof(T) == 4 ? sizeof(T) * cpb * ainv_stride<K, T>() : 0);
    void (*fn)(T *, const T *, T, const T *, MeshT<T>) =
        mode == 0 ? k_B<K, 0, T, HG> : (mode == 1 ? k_B<K, 1, T, HG> : k_B<K, 2, T, HG>);
    if (cudaError_t e = allow_smem(fn, sm); e != cudaSuccess) return e;
    fn<<<grid, th, sm, v.st>>>(dst, p, cB, v.ainv, v.mesh);
    return cudaGetLastError();
  };
  // mode 1 (dst -= B p) is not idempotent: it uses the choice made for mode 0
  const int cpb = tuned_cpb(v.tune, v.st, TF_B, K, mode == 1 ? 0 : mode, HG, (int)sizeof(T),
                            v.nc, mode != 1 && dst != p, launch);
  ATM_CUDA(launch(cpb));
  g_kernel_launches.fetch_add(1);
  return ATM_OK;
}

template <int K, typename T>
int pfix_prep_launch(const OpView<T> &v) {
  using C = Cfg<K>;
  const int grid = (v.nc + C::CPB - 1) / C::CPB;
  k_pfix_prep<K, T><<<grid, C::THREADS, sizeof(T) * C::CPB * C::NN2, v.st>>>(
      const_cast<T *>(v.pfq), const_cast<T *>(v.pff), v.pfix, v.mesh);
  ATM_CHECK_LAUNCH("k_pfix_prep");
  return ATM_OK;
}

template <int K, typename T, bool HG>
int CD_launch(const OpView<T> &v, T *dst, const T *w, const T *p, T cC, int mode,
              const ChebArgs<T> *cheb = nullptr) {
  const T *pfix = v.pfix;
  const ChebArgs<T> ch = cheb ? *cheb : ChebArgs<T>{};
  using C = Cfg<K>;
  auto launch = [&](int cpb) -> cudaError_t {
    const int grid = (v.nc + cpb - 1) / cpb, th = cpb * C::NQ;
    // plus the FP32 conforming staging buffer (k_CD: STG)
    const size_t stg = (sizeof(T) == 4 && !HG)
                           ? sizeof(T) * (((size_t)cpb * (16 * C::NQ + C::NQ2 +
                                                          (mode == 4 ? 3 * C::NN2 : 0)) + 3) / 4 * 4)
                           : 0;
    const size_t sm = smem_bytes<K, T>(cpb, 4, 1, HG) + stg;
    void (*fn)(T *, const T *, const T *, const T *, const T *, const T *, T, const T *,
               MeshT<T>, ChebArgs<T>) =
        mode == 0 ? k_CD<K, 0, T, HG>
        : mode == 1 ? k_CD<K, 1, T, HG>
        : mode == 2 ? k_CD<K, 2, T, HG>
        : mode == 3 ? k_CD<K, 3, T, HG>
                    : k_CD<K, 4, T, HG>;
    if (cudaError_t e = allow_smem(fn, sm); e != cudaSuccess) return e;
    fn<<<grid, th, sm, v.st>>>(dst, w, p, pfix, v.pfq, v.pff, cC, v.invd, v.mesh, ch);
    return cudaGetLastError();
  };
  // modes 3 (dst -= C w) and 4 (x += d) are not idempotent: they use the
  // choices made for modes 0 and 1
  const bool idem = mode < 3 && dst != w && dst != p && dst != pfix;
  const int key = mode == 3 ? 0 : (mode == 4 ? 1 : mode);
  const int cpb = tuned_cpb(v.tune, v.st, TF_CD, K, key, HG, (int)sizeof(T), v.nc, idem, launch);
  ATM_CUDA(launch(cpb));
  g_kernel_launches.fetch_add(1);
  return ATM_OK;
}

#define ATM_DISPATCH_K(kk, call)          \
  switch (kk) {                           \
    case 1: { constexpr int K = 1; return call; } \
    case 2: { constexpr int K = 2; return call; } \
    case 3: { constexpr int K = 3; return call; } \
    case 4: { constexpr int K = 4; return call; } \
    case 5: { constexpr int K = 5; return call; } \
    default: return ATM_BAD_ARG;          \
  }


}  // namespace atm
