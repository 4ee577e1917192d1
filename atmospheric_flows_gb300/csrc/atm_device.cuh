// Device-side helpers: per-degree launch configuration, constant basis tables
// and the column-wise sum-factorisation primitives shared by every operator
// kernel.
//
// Thread layout of the operator kernels ("column" layout): a block holds CPB
// cells; each cell is served by NQ = 2k+1 threads.  Thread `col` owns the
// quadrature column x = x_col of its cell: it evaluates every field on the
// NQ points of that column in registers (x-contraction from the cell's dof
// tile in shared memory, then the z-contraction in registers), does the
// point-wise physics, and contracts the submitted values back along z.  The
// final x-contraction and the face terms need one exchange through shared
// memory.  The same thread also serves face quadrature point `col` of each
// of the cell's four faces.  Face terms are element-centric: each cell reads
// the neighbour's face trace and adds only its own side, so no atomics are
// needed and results are bitwise reproducible run to run.
#pragma once
#include "atm_internal.h"

namespace atm {

template <int K>
struct Cfg {
  static constexpr int NN = K + 1;
  static constexpr int NQ = 2 * K + 1;
  static constexpr int NN2 = NN * NN;
  static constexpr int NQ2 = NQ * NQ;
  static constexpr int CPB = 128 / NQ;  // default cells per block
  static constexpr int THREADS = CPB * NQ;
  // the face kernels take the cells per block from blockDim (autotuned among
  // 64/NQ, 128/NQ and 256/NQ cells)
  static constexpr int MAX_THREADS = (256 / NQ) * NQ;
};

// [degree][w][q*(k+1)+i]: w = 0 values and 1 derivatives at the 2k+1 Gauss
// points g_q; w = 2, 3 values at the subface points (g_q + s)/2, s = 0, 1, of
// a hanging face; w = 4..7 the even/odd halves of the value and derivative
// tables for q < k, i < (k+1)/2 (E = (S(q,i) + S(q,k-i))/2,
// O = (S(q,i) - S(q,k-i))/2, same for D), used by the even-odd
// contractions.  Each translation unit holds its own copy in its constant
// bank.
constexpr int BASIS_TABLES = 8;
static __constant__ double c_basis[KMAX + 1][BASIS_TABLES][NQ_MAX * NN_MAX];
static __constant__ float c_basis_f[KMAX + 1][BASIS_TABLES][NQ_MAX * NN_MAX];

// [degree][r][q]: the degree-2 Lagrange basis on the reference points
// {0, 1/2, 1} at the 2k+1 Gauss points (r = 0..2 values, 3..5 derivatives)
// and the Gauss weights (r = 6).  The FP32 Schur kernels of the multigrid
// levels form the Jacobian of the degree-2 mapping (MeshT::map2) from it.
constexpr int GEO2_ROWS = 7;
static __constant__ float c_geo2_f[KMAX + 1][GEO2_ROWS][NQ_MAX];

// `table` holds the basis tables ([KMAX+1][BASIS_TABLES][NQ_MAX*NN_MAX])
// followed by the degree-2 mapping tables ([KMAX+1][GEO2_ROWS][NQ_MAX])
static inline int upload_basis_here(const double *table) {
  constexpr int NB = (KMAX + 1) * BASIS_TABLES * NQ_MAX * NN_MAX;
  constexpr int NG = (KMAX + 1) * GEO2_ROWS * NQ_MAX;
  float tf[NB], tg[NG];
  for (int i = 0; i < NB; ++i) tf[i] = (float)table[i];
  for (int i = 0; i < NG; ++i) tg[i] = (float)table[NB + i];
  if (cudaMemcpyToSymbol(c_basis, table, sizeof(c_basis)) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(c_geo2_f, tg, sizeof(c_geo2_f)) != cudaSuccess) return 1;
  return cudaMemcpyToSymbol(c_basis_f, tf, sizeof(c_basis_f)) == cudaSuccess ? 0 : 1;
}

template <typename T>
struct CBasis;
template <>
struct CBasis<double> {
  static __device__ __forceinline__ double get(int k, int w, int idx) { return c_basis[k][w][idx]; }
};
template <>
struct CBasis<float> {
  static __device__ __forceinline__ float get(int k, int w, int idx) { return c_basis_f[k][w][idx]; }
};

template <int K, typename T = double>
__device__ __forceinline__ T bS(int q, int i) { return CBasis<T>::get(K, 0, q * (K + 1) + i); }
template <int K, typename T = double>
__device__ __forceinline__ T bD(int q, int i) { return CBasis<T>::get(K, 1, q * (K + 1) + i); }
// even/odd halves (q < K, i < (K+1)/2): w = 4 E_S, 5 O_S, 6 E_D, 7 O_D
template <int K, typename T = double>
__device__ __forceinline__ T bEO(int w, int q, int i) {
  return CBasis<T>::get(K, w, q * (K + 1) + i);
}
// value of basis function i at point q of subface s of a hanging face
template <int K, typename T = double>
__device__ __forceinline__ T bH(int s, int q, int i) {
  return CBasis<T>::get(K, 2 + s, q * (K + 1) + i);
}

struct SrcPtrs {
  const double *p[12];
};

// local node index of node i (0..k) on face f: 0 x=0, 1 x=1, 2 z=0, 3 z=1
template <int K>
__device__ __forceinline__ int face_node(int f, int i) {
  constexpr int NN = K + 1;
  return f == 0 ? i * NN : (f == 1 ? i * NN + K : (f == 2 ? i : K * NN + i));
}

// thread-dependent basis row (x = x_col) and column (node t) in registers
template <int K, typename T>
__device__ __forceinline__ void load_rows(int col, T (&Sx)[K + 1], T (&Dx)[K + 1]) {
#pragma unroll
  for (int i = 0; i <= K; ++i) {
    Sx[i] = bS<K, T>(col, i);
    Dx[i] = bD<K, T>(col, i);
  }
}
template <int K, typename T>
__device__ __forceinline__ void load_cols(int t, T (&St)[2 * K + 1], T (&Dt)[2 * K + 1]) {
#pragma unroll
  for (int q = 0; q < 2 * K + 1; ++q) {
    St[q] = bS<K, T>(q, t);
    Dt[q] = bD<K, T>(q, t);
  }
}

// values of a nodal tile on the thread's quadrature column.  The
// z-contraction uses the even-odd split of the symmetric point sets
// (S(2k-q, k-i) = S(q, i)): for the pair (q, 2k-q) it forms
//   e = sum_i E(q,i) (t_i + t_{k-i}) [+ S(q,k/2) t_{k/2}],
//   o = sum_i O(q,i) (t_i - t_{k-i}),   v_q = e + o,  v_{2k-q} = e - o.
template <int K, typename T>
__device__ __forceinline__ void eval_col(const T *__restrict__ tile, const T (&Sx)[K + 1],
                                         T (&v)[2 * K + 1]) {
  constexpr int NN = K + 1, NQ = 2 * K + 1, H = NN / 2;
  constexpr bool MID = (NN & 1) != 0;
  T t[NN];
#pragma unroll
  for (int iz = 0; iz < NN; ++iz) {
    T s = 0;
#pragma unroll
    for (int ix = 0; ix < NN; ++ix) s = fma(Sx[ix], tile[iz * NN + ix], s);
    t[iz] = s;
  }
  T te[H > 0 ? H : 1], to[H > 0 ? H : 1];
#pragma unroll
  for (int i = 0; i < H; ++i) {
    te[i] = t[i] + t[K - i];
    to[i] = t[i] - t[K - i];
  }
#pragma unroll
  for (int q = 0; q < K; ++q) {
    T e = MID ? bS<K, T>(q, H) * t[H] : T(0);
    T o = 0;
#pragma unroll
    for (int i = 0; i < H; ++i) {
      e = fma(bEO<K, T>(4, q, i), te[i], e);
      o = fma(bEO<K, T>(5, q, i), to[i], o);
    }
    v[q] = e + o;
    v[NQ - 1 - q] = e - o;
  }
  {
    T e = MID ? bS<K, T>(K, H) * t[H] : T(0);
#pragma unroll
    for (int i = 0; i < H; ++i) e = fma(bS<K, T>(K, i), te[i], e);
    v[K] = e;
  }
}

// z-contraction of the submitted quantities of one column:
//   xa[iz][col] = sum_qz S(qz,iz) V + D(qz,iz) Geta ;  xb[iz][col] = sum_qz S(qz,iz) Gxi
// V, Gxi, Geta already carry JxW and the inverse Jacobian.  Even-odd split
// over the point pairs (q, 2k-q) and the output pairs (i, k-i); D is
// antisymmetric (D(2k-q, k-i) = -D(q, i)):
//   e = sum_q E_S (V_q + V_q') + E_D (G_q - G_q') [+ S(k,i) V_k]
//   o = sum_q O_S (V_q - V_q') + O_D (G_q + G_q') [+ D(k,i) G_k]
//   out_i = e + o,  out_{k-i} = e - o.
template <int K, bool HAS_V, bool HAS_G, typename T>
__device__ __forceinline__ void integrate_col_z(const T (&V)[2 * K + 1], const T (&Gxi)[2 * K + 1],
                                                const T (&Get)[2 * K + 1], T *__restrict__ xa,
                                                T *__restrict__ xb, int col) {
  constexpr int NN = K + 1, NQ = 2 * K + 1, H = NN / 2;
  constexpr bool MID = (NN & 1) != 0;
  T ve[K], vo[K], ge[K], go[K], xe[K], xo[K];
#pragma unroll
  for (int q = 0; q < K; ++q) {
    if (HAS_V) {
      ve[q] = V[q] + V[NQ - 1 - q];
      vo[q] = V[q] - V[NQ - 1 - q];
    }
    if (HAS_G) {
      ge[q] = Get[q] + Get[NQ - 1 - q];
      go[q] = Get[q] - Get[NQ - 1 - q];
      xe[q] = Gxi[q] + Gxi[NQ - 1 - q];
      xo[q] = Gxi[q] - Gxi[NQ - 1 - q];
    }
  }
#pragma unroll
  for (int i = 0; i < H; ++i) {
    T e = 0, o = 0;
    if (HAS_V) e = bS<K, T>(K, i) * V[K];
    if (HAS_G) o = bD<K, T>(K, i) * Get[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
      if (HAS_V) {
        e = fma(bEO<K, T>(4, q, i), ve[q], e);
        o = fma(bEO<K, T>(5, q, i), vo[q], o);
      }
      if (HAS_G) {
        e = fma(bEO<K, T>(6, q, i), go[q], e);
        o = fma(bEO<K, T>(7, q, i), ge[q], o);
      }
    }
    xa[i * NQ + col] = e + o;
    xa[(K - i) * NQ + col] = e - o;
    if (HAS_G) {
      T eb = bS<K, T>(K, i) * Gxi[K], ob = 0;
#pragma unroll
      for (int q = 0; q < K; ++q) {
        eb = fma(bEO<K, T>(4, q, i), xe[q], eb);
        ob = fma(bEO<K, T>(5, q, i), xo[q], ob);
      }
      xb[i * NQ + col] = eb + ob;
      xb[(K - i) * NQ + col] = eb - ob;
    }
  }
  if (MID) {
    // i = k/2: O_S = O_D = 0 and D(k, k/2) = 0
    T e = 0;
    if (HAS_V) e = bS<K, T>(K, H) * V[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
      if (HAS_V) e = fma(bS<K, T>(q, H), ve[q], e);
      if (HAS_G) e = fma(bD<K, T>(q, H), go[q], e);
    }
    xa[H * NQ + col] = e;
    if (HAS_G) {
      T eb = bS<K, T>(K, H) * Gxi[K];
#pragma unroll
      for (int q = 0; q < K; ++q) eb = fma(bS<K, T>(q, H), xe[q], eb);
      xb[H * NQ + col] = eb;
    }
  }
}

// Output phase by rows (conforming meshes), thread t < k+1 owns row iz = t:
//   out[ix] = sum_qx S(qx,ix) r[qx] + D(qx,ix) xb[iz][qx]
//           + [ix = 0] sum_q S(q,iz) F0[q] + [ix = k] sum_q S(q,iz) F1[q]
// with r = xa[iz] plus the z-face values (F2 on row 0, F3 on row k: the face
// points of z-faces are the x quadrature points, so those terms fold into the
// same contraction).  The x-contraction uses the even-odd split over the
// point pairs (qx, 2k-qx), as integrate_col_z.  St holds S(., iz); F is the
// cell's [4][NQ] face values of this component.
template <int K, typename T>
__device__ __forceinline__ void integrate_row(const T *__restrict__ xa, const T *__restrict__ xb,
                                              const T *__restrict__ F, int iz,
                                              const T (&St)[2 * K + 1], T (&out)[K + 1]) {
  constexpr int NQ = 2 * K + 1, H = (K + 1) / 2;
  constexpr bool MID = ((K + 1) & 1) != 0;
  T r[NQ], g[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    T v = xa[iz * NQ + q];
    if (iz == 0) v += F[2 * NQ + q];
    if (iz == K) v += F[3 * NQ + q];
    r[q] = v;
    g[q] = xb[iz * NQ + q];
  }
  T re[K], ro[K], ge[K], go[K];
#pragma unroll
  for (int q = 0; q < K; ++q) {
    re[q] = r[q] + r[NQ - 1 - q];
    ro[q] = r[q] - r[NQ - 1 - q];
    ge[q] = g[q] + g[NQ - 1 - q];
    go[q] = g[q] - g[NQ - 1 - q];
  }
#pragma unroll
  for (int i = 0; i < H; ++i) {
    T e = bS<K, T>(K, i) * r[K], o = bD<K, T>(K, i) * g[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
      e = fma(bEO<K, T>(4, q, i), re[q], e);
      e = fma(bEO<K, T>(6, q, i), go[q], e);
      o = fma(bEO<K, T>(5, q, i), ro[q], o);
      o = fma(bEO<K, T>(7, q, i), ge[q], o);
    }
    out[i] = e + o;
    out[K - i] = e - o;
  }
  if (MID) {
    T e = bS<K, T>(K, H) * r[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
      e = fma(bS<K, T>(q, H), re[q], e);
      e = fma(bD<K, T>(q, H), go[q], e);
    }
    out[H] = e;
  }
  T s0 = 0, s1 = 0;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    s0 = fma(St[q], F[q], s0);
    s1 = fma(St[q], F[NQ + q], s1);
  }
  out[0] += s0;
  out[K] += s1;
}

// local node written by output slot j of thread t: column layout (hanging-
// face kernels: node (iz = j, ix = t)) or row layout (node (iz = t, ix = j))
template <int K, bool HG>
__device__ __forceinline__ int out_node(int t, int j) {
  return HG ? j * (K + 1) + t : t * (K + 1) + j;
}

// output phase of one component: rows (conforming) or columns + face terms
// (hanging faces, add_face_out_hg)
template <int K, bool HG, typename T>
__device__ __forceinline__ void output_phase(const MeshT<T> &mesh, int c, const T *__restrict__ xa,
                                             const T *__restrict__ xb, const T *__restrict__ F,
                                             const T *__restrict__ Fh, int t,
                                             const T (&St)[2 * K + 1], const T (&Dt)[2 * K + 1],
                                             T (&out)[K + 1]);

// x-contraction for output node column ix = t: out[iz] = sum_qx S(qx,t) xa + D(qx,t) xb
template <int K, bool HAS_G, typename T>
__device__ __forceinline__ void integrate_out(const T *__restrict__ xa, const T *__restrict__ xb,
                                              const T (&St)[2 * K + 1], const T (&Dt)[2 * K + 1],
                                              T (&out)[K + 1]) {
  constexpr int NN = K + 1, NQ = 2 * K + 1;
#pragma unroll
  for (int iz = 0; iz < NN; ++iz) {
    T s = 0;
#pragma unroll
    for (int qx = 0; qx < NQ; ++qx) {
      s = fma(St[qx], xa[iz * NQ + qx], s);
      if (HAS_G) s = fma(Dt[qx], xb[iz * NQ + qx], s);
    }
    out[iz] = s;
  }
}

// add the face contributions F[f][q] (JxW included) to output node column t
template <int K, typename T>
__device__ __forceinline__ void add_face_out(const T *__restrict__ F, int t,
                                             const T (&St)[2 * K + 1], T (&out)[K + 1]) {
  constexpr int NN = K + 1, NQ = 2 * K + 1;
  // faces z=0 / z=1: node (iz=0|K, ix=t)
  T s2 = 0, s3 = 0;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    s2 = fma(St[q], F[2 * NQ + q], s2);
    s3 = fma(St[q], F[3 * NQ + q], s3);
  }
  out[0] += s2;
  out[K] += s3;
  // faces x=0 / x=1: whole node column ix = 0 / ix = K
  if (t == 0 || t == K) {
    const T *Ff = F + (t == 0 ? 0 : NQ);
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      T s = 0;
#pragma unroll
      for (int q = 0; q < NQ; ++q) s = fma(bS<K, T>(q, iz), Ff[q], s);
      out[iz] += s;
    }
  }
}

// Face contributions with hanging faces: like add_face_out, but on a face of
// code 3 (this cell is the coarse side, bit f of hmask) the two subface
// fluxes F (s = 0) and Fh (s = 1) are integrated against the shifted basis.
template <int K, typename T>
__device__ __forceinline__ void add_face_out_hg(const T *__restrict__ F, const T *__restrict__ Fh,
                                                int hmask, int t, const T (&St)[2 * K + 1],
                                                T (&out)[K + 1]) {
  if (hmask == 0) {
    add_face_out<K>(F, t, St, out);
    return;
  }
  constexpr int NN = K + 1, NQ = 2 * K + 1;
#pragma unroll
  for (int f = 2; f < 4; ++f) {
    T s = 0;
    if ((hmask >> f) & 1) {
      for (int q = 0; q < NQ; ++q)
        s = fma(bH<K, T>(0, q, t), F[f * NQ + q], fma(bH<K, T>(1, q, t), Fh[f * NQ + q], s));
    } else {
#pragma unroll
      for (int q = 0; q < NQ; ++q) s = fma(St[q], F[f * NQ + q], s);
    }
    out[f == 2 ? 0 : K] += s;
  }
  if (t == 0 || t == K) {
    const int f = t == 0 ? 0 : 1;
    const bool hang = (hmask >> f) & 1;
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      T s = 0;
      if (hang) {
        for (int q = 0; q < NQ; ++q)
          s = fma(bH<K, T>(0, q, iz), F[f * NQ + q], fma(bH<K, T>(1, q, iz), Fh[f * NQ + q], s));
      } else {
#pragma unroll
        for (int q = 0; q < NQ; ++q) s = fma(bS<K, T>(q, iz), F[f * NQ + q], s);
      }
      out[iz] += s;
    }
  }
}

// bit f set when face f of cell c is the coarse side of a hanging face
template <typename T>
__device__ __forceinline__ int hanging_mask(const MeshT<T> &mesh, int c) {
  int m = 0;
#pragma unroll
  for (int f = 0; f < 4; ++f)
    if (mesh.nbr[c * 4 + f] >= 0 && (mesh.nbrf[c * 4 + f] >> 2) == 3) m |= 1 << f;
  return m;
}

// Walks the four faces of cell c for the column thread `col` and calls
//   body(f, nb, nf, n0, n1, jxw, Ro, Rn, val)
// once per face point: nb/nf the neighbour cell and its local face (nb < 0 at a
// wall), (n0, n1, jxw) the outward normal and the face weight, Ro / Rn the
// basis rows giving this cell's and the neighbour's trace at the point.  The
// body returns NC face values in val, stored at fbc[comp*4*NQ + f*NQ + col].
// With HG, a face of code 1/2 reads the neighbour at the shifted points; a face
// of code 3 is integrated on its two subfaces, with the s = 1 values going to
// fhc (same layout).  Without HG the loop is the conforming one.
//
// `fgc` (optional): this cell's conforming face geometry [4][3][NQ] already
// staged in shared memory, read instead of mesh.fgeo.
template <int K, int NC, bool HG, typename T, typename Body>
__device__ __forceinline__ void face_terms(const MeshT<T> &mesh, int c, int col,
                                           const T (&Sx)[K + 1], T *__restrict__ fbc,
                                           T *__restrict__ fhc, Body &&body,
                                           const T *__restrict__ fgc = nullptr) {
  constexpr int NQ = 2 * K + 1;
  // the four neighbours and their faces in two 16-byte loads; FP32 (latency
  // bound) unrolls the faces so that their loads overlap
  const int4 nb4 = *reinterpret_cast<const int4 *>(mesh.nbr + c * 4);
  const int4 nf4 = *reinterpret_cast<const int4 *>(mesh.nbrf + c * 4);
#pragma unroll(sizeof(T) == 4 ? 4 : 1)
  for (int f = 0; f < 4; ++f) {
    const int nb = f == 0 ? nb4.x : f == 1 ? nb4.y : f == 2 ? nb4.z : nb4.w;
    const int nfc = f == 0 ? nf4.x : f == 1 ? nf4.y : f == 2 ? nf4.z : nf4.w;
    const int code = HG && nb >= 0 ? (nfc >> 2) : 0;
    T val[NC];
    if (code == 0) {
      const T *fg = fgc ? fgc + f * 3 * NQ : mesh.fgeo + ((long)c * 4 + f) * 3 * NQ;
      body(f, nb, nfc & 3, fg[col], fg[NQ + col], fg[2 * NQ + col], Sx, Sx, val);
#pragma unroll
      for (int comp = 0; comp < NC; ++comp) fbc[comp * 4 * NQ + f * NQ + col] = val[comp];
    } else if (code < 3) {
      const T *fg = mesh.fgeo + ((long)c * 4 + f) * 3 * NQ;
      T Rn[K + 1];
#pragma unroll
      for (int i = 0; i <= K; ++i) Rn[i] = bH<K, T>(code - 1, col, i);
      body(f, nb, nfc & 3, fg[col], fg[NQ + col], fg[2 * NQ + col], Sx, Rn, val);
#pragma unroll
      for (int comp = 0; comp < NC; ++comp) fbc[comp * 4 * NQ + f * NQ + col] = val[comp];
    } else {
      for (int s = 0; s < 2; ++s) {
        const T *hg = mesh.hgeo + ((long)nb * 2 + s) * 3 * NQ;
        T Ro[K + 1];
#pragma unroll
        for (int i = 0; i <= K; ++i) Ro[i] = bH<K, T>(s, col, i);
        body(f, mesh.hnb[nb * 2 + s], nfc & 3, hg[col], hg[NQ + col], hg[2 * NQ + col], Ro, Sx,
             val);
        T *o = s == 0 ? fbc : fhc;
#pragma unroll
        for (int comp = 0; comp < NC; ++comp) o[comp * 4 * NQ + f * NQ + col] = val[comp];
      }
    }
  }
}

template <int K, bool HG, typename T>
__device__ __forceinline__ void output_phase(const MeshT<T> &mesh, int c, const T *__restrict__ xa,
                                             const T *__restrict__ xb, const T *__restrict__ F,
                                             const T *__restrict__ Fh, int t,
                                             const T (&St)[2 * K + 1], const T (&Dt)[2 * K + 1],
                                             T (&out)[K + 1]) {
  if (HG) {
    integrate_out<K, true>(xa, xb, St, Dt, out);
    add_face_out_hg<K>(F, Fh, hanging_mask(mesh, c), t, St, out);
  } else {
    integrate_row<K>(xa, xb, F, t, St, out);
  }
}

// trace of a nodal tile at face quadrature point `col` (row Sx = S[col][.])
template <int K, typename T>
__device__ __forceinline__ T face_val(const T *__restrict__ tile, int f, const T (&Sx)[K + 1]) {
  T s = 0;
#pragma unroll
  for (int i = 0; i <= K; ++i) s = fma(Sx[i], tile[face_node<K>(f, i)], s);
  return s;
}

// cooperative, coalesced copy of the block's cells of one field into tiles
// dst tile slot = tiles[(lc*NT + t0 + comp)*NN2 + i]
template <int K, typename T>
__device__ __forceinline__ void load_tiles(T *__restrict__ tiles, int NT, int t0,
                                           const T *__restrict__ src, int ncomp, int c0,
                                           int cnt) {
  constexpr int NN2 = (K + 1) * (K + 1);
  const int per = ncomp * NN2;
  const T *s = src + (long)c0 * per;
  for (int e = threadIdx.x; e < cnt * per; e += blockDim.x) {
    const int lc = e / per;
    const int r = e - lc * per;
    const int comp = r / NN2;
    const int i = r - comp * NN2;
    tiles[(lc * NT + t0 + comp) * NN2 + i] = s[e];
  }
}

// physical gradient (gx, gz) at a quadrature point -> reference space * JxW
template <typename T>
struct QGeoT {
  T xx, xz, ex, ez, jxw;
};
using QGeo = QGeoT<double>;
template <int K, typename T>
__device__ __forceinline__ QGeoT<T> qgeo(const T *__restrict__ g, int q) {
  constexpr int NQ2 = (2 * K + 1) * (2 * K + 1);
  QGeoT<T> r;
  r.xx = g[q];
  r.xz = g[NQ2 + q];
  r.ex = g[2 * NQ2 + q];
  r.ez = g[3 * NQ2 + q];
  r.jxw = g[4 * NQ2 + q];
  return r;
}

// Values between two cells' A^{-1} blocks ([nc][stride]).  FP64: the full
// (k+1)^2 x (k+1)^2 block.  FP32 (multigrid levels): A^{-1} is symmetric, so
// only its lower triangle is stored, row by row ((r, c <= r) at
// r (r+1)/2 + c), padded to a multiple of 16 bytes: the B kernel stages the
// blocks of its cells into shared memory with 16-byte cp.async copies, and
// half the bytes leave more room there.
template <int K, typename T>
__host__ __device__ constexpr int ainv_stride() {
  return sizeof(T) == 4
             ? ((K + 1) * (K + 1) * ((K + 1) * (K + 1) + 1) / 2 + 3) / 4 * 4
             : (K + 1) * (K + 1) * (K + 1) * (K + 1);
}
inline long ainv_stride_rt(int k, size_t elem) {
  const long n2 = (long)(k + 1) * (k + 1);
  return elem == 4 ? (n2 * (n2 + 1) / 2 + 3) / 4 * 4 : n2 * n2;
}

// 16-byte asynchronous global -> shared copies (cp.async, bypassing L1) and
// the wait for all of this thread's outstanding copies
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Quadrature-point geometry of cell c along the column of Gauss points
// (g_col, g_qz), qz = 0..NQ-1, as the Schur kernels consume it.  FP64 reads
// the stored table qgeo.  FP32 (multigrid levels) forms it from the cell's
// degree-2 mapping (18 values instead of 5 (2k+1)^2): with
// J = [[x_xi, x_eta], [z_xi, z_eta]] and w = w_col w_qz the entries are
// z_eta w, -x_eta w, -z_xi w, x_xi w and det(J) w (the cofactors of J
// times JxW / det J), contracted first along xi for the column, then along
// eta per point.
template <int K, typename T>
struct GeoCol {
  const T *G;
  int col;
  __device__ __forceinline__ GeoCol(const MeshT<T> &m, int c, int col_)
      : G(m.qgeo + (long)c * 5 * (2 * K + 1) * (2 * K + 1)), col(col_) {}
  __device__ __forceinline__ QGeoT<T> at(int qz) const {
    return qgeo<K>(G, qz * (2 * K + 1) + col);
  }
  // (dxi/dx, deta/dx) JxW and (dxi/dz, deta/dz) JxW alone
  __device__ __forceinline__ void dx(int qz, T &gxi, T &get) const {
    constexpr int NQ2 = (2 * K + 1) * (2 * K + 1);
    gxi = G[qz * (2 * K + 1) + col];
    get = G[2 * NQ2 + qz * (2 * K + 1) + col];
  }
  __device__ __forceinline__ void dz(int qz, T &gxi, T &get) const {
    constexpr int NQ2 = (2 * K + 1) * (2 * K + 1);
    gxi = G[NQ2 + qz * (2 * K + 1) + col];
    get = G[3 * NQ2 + qz * (2 * K + 1) + col];
  }
};
template <int K>
struct GeoCol<K, float> {
  float ax[3], az[3], bx[3], bz[3], wc;  // per eta node: d/dxi and value along xi
  __device__ __forceinline__ GeoCol(const MeshT<float> &m, int c, int col) {
    const float2 *X = reinterpret_cast<const float2 *>(m.map2) + (long)c * 9;
    float La[3], dLa[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      La[a] = c_geo2_f[K][a][col];
      dLa[a] = c_geo2_f[K][3 + a][col];
    }
    wc = c_geo2_f[K][6][col];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      ax[e] = az[e] = bx[e] = bz[e] = 0.0f;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float2 x = __ldg(X + e * 3 + a);
        ax[e] = fmaf(x.x, dLa[a], ax[e]);
        az[e] = fmaf(x.y, dLa[a], az[e]);
        bx[e] = fmaf(x.x, La[a], bx[e]);
        bz[e] = fmaf(x.y, La[a], bz[e]);
      }
    }
  }
  __device__ __forceinline__ QGeoT<float> at(int qz) const {
    float xxi = 0.0f, zxi = 0.0f, xet = 0.0f, zet = 0.0f;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const float L = c_geo2_f[K][e][qz], dL = c_geo2_f[K][3 + e][qz];
      xxi = fmaf(ax[e], L, xxi);
      zxi = fmaf(az[e], L, zxi);
      xet = fmaf(bx[e], dL, xet);
      zet = fmaf(bz[e], dL, zet);
    }
    const float w = wc * c_geo2_f[K][6][qz];
    QGeoT<float> r;
    r.xx = zet * w;
    r.xz = -xet * w;
    r.ex = -zxi * w;
    r.ez = xxi * w;
    r.jxw = (xxi * zet - xet * zxi) * w;
    return r;
  }
  // (dxi/dx, deta/dx) JxW = (z_eta, -z_xi) w: the z coordinate alone
  __device__ __forceinline__ void dx(int qz, float &gxi, float &get) const {
    float zxi = 0.0f, zet = 0.0f;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      zxi = fmaf(az[e], c_geo2_f[K][e][qz], zxi);
      zet = fmaf(bz[e], c_geo2_f[K][3 + e][qz], zet);
    }
    const float w = wc * c_geo2_f[K][6][qz];
    gxi = zet * w;
    get = -zxi * w;
  }
  // (dxi/dz, deta/dz) JxW = (-x_eta, x_xi) w: the x coordinate alone
  __device__ __forceinline__ void dz(int qz, float &gxi, float &get) const {
    float xxi = 0.0f, xet = 0.0f;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      xxi = fmaf(ax[e], c_geo2_f[K][e][qz], xxi);
      xet = fmaf(bx[e], c_geo2_f[K][3 + e][qz], xet);
    }
    const float w = wc * c_geo2_f[K][6][qz];
    gxi = -xet * w;
    get = xxi * w;
  }
};

// Let kernel `fn` use up to the device's opt-in maximum of dynamic shared
// memory when a launch needs more than the default 48 KB.  The limit is set
// to that maximum, always the same value: host threads launching the same
// kernel with different block shapes (serving members, the autotuner) must
// never lower each other's limit between setting it and launching.
template <typename F>
inline cudaError_t allow_smem(F fn, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  static int cap[64] = {0};  // per device; a benign race writes the same value
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int mx = dev >= 0 && dev < 64 ? cap[dev] : 0;
  if (mx == 0) {
    e = cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) cap[dev] = mx;
  }
  if (bytes > (size_t)mx) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

// tiles, x-contraction exchange, face values [, subface-1 face values]
template <int K, typename T = double>
inline size_t smem_bytes(int cpb, int n_tiles, int ncomp_out, bool hg = false) {
  using C = Cfg<K>;
  return sizeof(T) * (size_t)cpb *
         ((size_t)n_tiles * C::NN2 + (size_t)ncomp_out * 2 * C::NN * C::NQ +
          (size_t)ncomp_out * 4 * C::NQ * (hg ? 2 : 1));
}

}  // namespace atm
