// Multigrid-preconditioned Schur solve: FP64 flexible GMRES, right-
// preconditioned by a geometric multigrid V-cycle with Chebyshev smoothing,
// with the V-cycle in FP32 (mixed precision) or FP64.
//
// The reference solves the Schur system with GMRES + Jacobi on the diagonal
// of D (Atmospheric_Flow.cc:656-672) and builds FP64 GMG + Chebyshev(3)
// hierarchies only for its mass-type systems (Atmospheric_Flow.cc:456-522:
// smoothing range 15, degree 3, 10 eigenvalue iterations).  Here the same
// smoother recipe is applied to the Schur/Helmholtz operator itself:
//   * level 0 is the operator mesh; level l+1 merges groups of 2x2 cells of
//     level l (on a 2:1 adaptive mesh, the finest cells first; the other
//     cells stay as they are, so coarse levels may have hanging faces too)
//     and carries a rediscretisation of S = D - C A^{-1} B on that mesh (the
//     FP64 operator kernels instantiated for the level's scalar type), with
//     rho_fix and p_fix injected level by level and A^{-1} rebuilt per level;
//   * transfer is the exact embedding of the coarse polynomial space into the
//     four children (prolongation) and its transpose (restriction); a cell
//     that is not merged is copied;
//   * smoother: Chebyshev of degree 3 preconditioned by the inverse diagonal
//     of D on [1.2 lambda_max / 15, 1.2 lambda_max], lambda_max from 10 power
//     iterations; the coarsest level runs a higher-degree Chebyshev.
// FP64 is kept for the outer residual, the Krylov basis, every inner
// product and the solution update.  The host keeps the level tables; the
// device hierarchy of a precision is built on its first use.
#include <cmath>
#include <cstring>

#include "atm_device.cuh"

namespace atm {

template <typename T>
struct XferTabT {
  T E[2][NN_MAX][NN_MAX];  // E[a][i][j] = l_j((a + x_i)/2): coarse basis at fine node i
  T F[NN_MAX][NN_MAX];     // F[j][i] = l_i(2 x_j - a_j): fine basis at coarse node j
  int fa[NN_MAX];          // child half (0: lower, 1: upper) holding coarse node j
};

template <typename T>
struct MGLevelT {
  int nc = 0;
  MeshT<T> mesh;
  int *parent = nullptr;    // [nc] cell of level+1 containing this cell
  int *ppos = nullptr;      // [nc] position a + 2b of this cell inside its parent (4: same cell)
  int *children = nullptr;  // [nc][4] cells of level-1 (levels >= 1)
  T *ainv = nullptr, *invd = nullptr, *rho = nullptr, *pfix = nullptr;
  T *pfq = nullptr, *pff = nullptr;  // p_fix at quadrature points / face traces
  T *x = nullptr, *b = nullptr, *r = nullptr, *t = nullptr, *d = nullptr, *wv = nullptr;
  double lam = 0.0;
};

template <typename T>
struct MGHier {
  std::vector<MGLevelT<T>> lv;
  XferTabT<T> tab;
  bool built = false;
  bool rho_dirty = true;
  // The V-cycle as a captured CUDA graph.  Its kernel arguments depend on the
  // implicit coefficient, dt, Ma (level operators) and the eigenvalue
  // estimates (Chebyshev), so it is re-captured when any of them changes.
  cudaGraphExec_t graph = nullptr;
  long graph_kernels = 0;   // kernels in one replay
  double graph_key[4] = {0, 0, 0, -1};
  long lam_epoch = 0;       // bumped whenever the eigenvalue estimates change
  bool graph_failed = false;
};

struct MG {
  // level tables on the host; entry 0 is the operator mesh
  std::vector<HostMesh> hm;
  std::vector<std::vector<int>> children;  // per level >= 1: [nc][4]
  std::vector<int> ncells;
  MGHier<float> f;
  MGHier<double> d;
  // degree 4: on the 320x160 Q4 flow over a hill (mixed precision, rtol
  // 1e-11) 97 FGMRES iterations per step instead of 133 at degree 3, and a
  // 14% shorter step; degree 5 saves too few iterations for its cost
  int cheb_deg = 4;
  double range = 15.0;
  int eig_its = 10;
  // coarsest-level Chebyshev degree 6: the FGMRES iteration counts are those
  // of degree 10 (320x160 Q4, 40x20 Q4, 160x80 Q2, 80x40 Q5) and the steps
  // 2-10% shorter
  int coarse_deg = 6;
  double coarse_range = 50.0;
  int restart = 16;
  double *zbasis = nullptr;  // FGMRES preconditioned directions [restart][ns]
  long vcycles = 0;
  bool use_graphs = true;             // replay the V-cycle as a CUDA graph
  cudaStream_t cap_stream = nullptr;  // private stream the V-cycle is captured on
  long graph_replays = 0;
};

namespace {

// ----------------------------------------------------------------- kernels --
template <typename A, typename B>
__global__ void k_convert(A *__restrict__ o, const B *__restrict__ i, long n) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    o[k] = (A)i[k];
}
// Chebyshev update with r = rhs - t (t ignored when `zero_t`):
//   mode 0: d = b invd r, x = d        (start from x = 0)
//   mode 1: d = b invd r, x += d       (first step from a given x)
//   mode 2: d = a d + b invd r, x += d (later steps)
template <typename T>
__global__ void k_cheb(T *__restrict__ x, T *__restrict__ d, const T *__restrict__ rhs,
                       const T *__restrict__ t, const T *__restrict__ invd, T a, T b,
                       int zero_t, int mode, long n) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const T r = zero_t ? rhs[k] : rhs[k] - t[k];
    const T dk = (mode == 2 ? a * d[k] : T(0)) + b * invd[k] * r;
    d[k] = dk;
    x[k] = mode == 0 ? dk : x[k] + dk;
  }
}
template <typename T>
__global__ void k_scale_copy(T *__restrict__ o, const T *__restrict__ i, T s, long n) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    o[k] = s * i[k];
}
template <typename T>
__global__ void k_sub(T *__restrict__ r, const T *__restrict__ b, const T *__restrict__ t,
                      long n) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    r[k] = b[k] - t[k];
}
template <typename T>
__global__ void k_scale_invd(T *__restrict__ w, const T *__restrict__ invd,
                             const T *__restrict__ t, long n) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    w[k] = invd[k] * t[k];
}
// deterministic: fixed grid, per-block partial sums in FP64
constexpr int NB = 304;
template <typename T>
__global__ void k_nrm2_partial(const T *__restrict__ v, long n, double *__restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (long k = (long)blockIdx.x * 256 + threadIdx.x; k < n; k += (long)NB * 256) {
    const double a = v[k];
    s += a * a;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_sum_partial(const double *__restrict__ part, double *__restrict__ out) {
  __shared__ double sh[512];
  double s = 0.0;
  for (int k = threadIdx.x; k < NB; k += 512) s += part[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 256; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}
// deterministic pseudo-random start vector for the power iteration
template <typename T>
__global__ void k_hash_init(T *__restrict__ v, long n) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)k * 2654435761u ^ 0x9e3779b9u;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    v[k] = T(0.5) + T(h & 0xffffu) / T(65536.0);
  }
}

template <int K, typename T>
__global__ void k_prolong_add(T *__restrict__ fine, const T *__restrict__ coarse,
                              const int *__restrict__ parent, const int *__restrict__ ppos,
                              int ncf, XferTabT<T> tb) {
  constexpr int NN = K + 1, NN2 = NN * NN;
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long)ncf * NN2) return;
  const int cf = (int)(g / NN2), i = (int)(g - (long)cf * NN2);
  const int iz = i / NN, ix = i - iz * NN;
  const int pos = ppos[cf], a = pos & 1, b = pos >> 1;
  const T *u = coarse + (long)parent[cf] * NN2;
  if (pos == 4) {  // cell unchanged on the coarser level
    fine[g] += u[i];
    return;
  }
  T s = 0;
#pragma unroll
  for (int jz = 0; jz < NN; ++jz) {
    T t = 0;
#pragma unroll
    for (int jx = 0; jx < NN; ++jx) t = fma(tb.E[a][ix][jx], u[jz * NN + jx], t);
    s = fma(tb.E[b][iz][jz], t, s);
  }
  fine[g] += s;
}

template <int K, typename T>
__global__ void k_restrict(T *__restrict__ coarse, const T *__restrict__ fine,
                           const int *__restrict__ children, int ncc, XferTabT<T> tb) {
  constexpr int NN = K + 1, NN2 = NN * NN;
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long)ncc * NN2) return;
  const int cc = (int)(g / NN2), j = (int)(g - (long)cc * NN2);
  const int jz = j / NN, jx = j - jz * NN;
  if (children[cc * 4 + 1] < 0) {  // cell unchanged on this level
    coarse[g] = fine[(long)children[cc * 4] * NN2 + j];
    return;
  }
  T s = 0;
#pragma unroll
  for (int pos = 0; pos < 4; ++pos) {
    const int a = pos & 1, b = pos >> 1;
    const T *r = fine + (long)children[cc * 4 + pos] * NN2;
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) {
      T t = 0;
#pragma unroll
      for (int ix = 0; ix < NN; ++ix) t = fma(tb.E[a][ix][jx], r[iz * NN + ix], t);
      s = fma(tb.E[b][iz][jz], t, s);
    }
  }
  coarse[g] = s;
}

template <int K, typename T>
__global__ void k_inject(T *__restrict__ coarse, const T *__restrict__ fine,
                         const int *__restrict__ children, int ncc, XferTabT<T> tb) {
  constexpr int NN = K + 1, NN2 = NN * NN;
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long)ncc * NN2) return;
  const int cc = (int)(g / NN2), j = (int)(g - (long)cc * NN2);
  const int jz = j / NN, jx = j - jz * NN;
  if (children[cc * 4 + 1] < 0) {  // cell unchanged on this level
    coarse[g] = fine[(long)children[cc * 4] * NN2 + j];
    return;
  }
  const int child = children[cc * 4 + tb.fa[jx] + 2 * tb.fa[jz]];
  const T *u = fine + (long)child * NN2;
  T s = 0;
#pragma unroll
  for (int iz = 0; iz < NN; ++iz) {
    T t = 0;
#pragma unroll
    for (int ix = 0; ix < NN; ++ix) t = fma(tb.F[jx][ix], u[iz * NN + ix], t);
    s = fma(tb.F[jz][iz], t, s);
  }
  coarse[g] = s;
}

inline int gsz(long n) {
  long g = (n + 255) / 256;
  if (g > 152L * 16) g = 152L * 16;
  return (int)(g < 1 ? 1 : g);
}
#define LAUNCHED()                  \
  do {                              \
    g_kernel_launches.fetch_add(1); \
    ATM_CUDA(cudaGetLastError());   \
  } while (0)

#define MG_DISPATCH(kk, T, kern, grid, ...)                                  \
  switch (kk) {                                                              \
    case 1: kern<1, T><<<grid, 256, 0, c.stream>>>(__VA_ARGS__); break;      \
    case 2: kern<2, T><<<grid, 256, 0, c.stream>>>(__VA_ARGS__); break;      \
    case 3: kern<3, T><<<grid, 256, 0, c.stream>>>(__VA_ARGS__); break;      \
    case 4: kern<4, T><<<grid, 256, 0, c.stream>>>(__VA_ARGS__); break;      \
    default: kern<5, T><<<grid, 256, 0, c.stream>>>(__VA_ARGS__); break;     \
  }

template <typename T>
LevelViewT<T> lview(const atm_ctx &c, const MGLevelT<T> &L) {
  return LevelViewT<T>{c.k, L.nc, L.mesh, L.ainv, L.invd, c.stream, c.autotune && !c.capturing,
                       L.pfix, L.pfq, L.pff};
}

template <typename T>
MGHier<T> &hier(MG &mg);
template <>
MGHier<float> &hier<float>(MG &mg) { return mg.f; }
template <>
MGHier<double> &hier<double>(MG &mg) { return mg.d; }

template <typename T>
void level_free(MGLevelT<T> &L) {
  cudaFree(L.mesh.qgeo); cudaFree(L.mesh.fgeo); cudaFree(L.mesh.nbr); cudaFree(L.mesh.nbrf);
  cudaFree(L.mesh.hnb); cudaFree(L.mesh.hgeo); cudaFree(L.mesh.dts); cudaFree(L.mesh.map2);
  cudaFree(L.parent); cudaFree(L.ppos); cudaFree(L.children);
  cudaFree(L.ainv); cudaFree(L.invd); cudaFree(L.rho); cudaFree(L.pfix);
  cudaFree(L.pfq); cudaFree(L.pff);
  cudaFree(L.x); cudaFree(L.b); cudaFree(L.r); cudaFree(L.t); cudaFree(L.d); cudaFree(L.wv);
  L = MGLevelT<T>();
}

template <typename T>
void hier_drop_graph(MGHier<T> &H) {
  if (H.graph) cudaGraphExecDestroy(H.graph);
  H.graph = nullptr;
  H.graph_kernels = 0;
  H.graph_key[3] = -1;
}

template <typename T>
void hier_free(MGHier<T> &H) {
  hier_drop_graph(H);
  for (auto &L : H.lv) level_free(L);
  H.lv.clear();
  H.built = false;
  H.rho_dirty = true;
  H.graph_failed = false;
}

template <typename T>
void make_xfer(int k, XferTabT<T> &tb) {
  std::memset(&tb, 0, sizeof(tb));
  const std::vector<double> x = gll_nodes(k);
  const int nn = k + 1;
  std::vector<double> v(nn);
  for (int a = 0; a < 2; ++a)
    for (int i = 0; i < nn; ++i) {
      lagrange_eval(x, 0.5 * (a + x[i]), v.data(), nullptr);
      for (int j = 0; j < nn; ++j) tb.E[a][i][j] = (T)v[j];
    }
  for (int j = 0; j < nn; ++j) {
    const int a = x[j] > 0.5 ? 1 : 0;
    tb.fa[j] = a;
    lagrange_eval(x, 2.0 * x[j] - a, v.data(), nullptr);
    for (int i = 0; i < nn; ++i) tb.F[j][i] = (T)v[i];
  }
}

template <typename T>
int level_alloc(atm_ctx &c, MGLevelT<T> &L, const HostMesh &hm) {
  const int nn2 = c.nn2, nq = c.nq, nq2 = nq * nq;
  const long ns = (long)L.nc * nn2;
  L.mesh.nc = L.nc; L.mesh.k = c.k; L.mesh.nn = c.nn; L.mesh.nq = nq;
  L.mesh.nn2 = nn2; L.mesh.nq2 = nq2;
  std::vector<T> qf(hm.qgeo.begin(), hm.qgeo.end()), ff(hm.fgeo.begin(), hm.fgeo.end());
  if (hm.map2.size() != (size_t)L.nc * 18) {
    set_error("multigrid level: missing degree-2 mapping table");
    return ATM_BAD_ARG;
  }
  if (sizeof(T) == 4) {  // the FP32 Schur kernels form their geometry from it
    std::vector<T> m2(hm.map2.begin(), hm.map2.end());
    ATM_CUDA(cudaMalloc(&L.mesh.map2, m2.size() * sizeof(T)));
    ATM_CUDA(cudaMemcpyAsync(L.mesh.map2, m2.data(), m2.size() * sizeof(T), cudaMemcpyHostToDevice, c.stream));
    ATM_CUDA(cudaStreamSynchronize(c.stream));  // pageable source
  }
  ATM_CUDA(cudaMalloc(&L.mesh.qgeo, qf.size() * sizeof(T)));
  ATM_CUDA(cudaMalloc(&L.mesh.fgeo, ff.size() * sizeof(T)));
  ATM_CUDA(cudaMalloc(&L.mesh.nbr, hm.nbr.size() * sizeof(int)));
  ATM_CUDA(cudaMalloc(&L.mesh.nbrf, hm.nbrf.size() * sizeof(int)));
  ATM_CUDA(cudaMemcpyAsync(L.mesh.qgeo, qf.data(), qf.size() * sizeof(T), cudaMemcpyHostToDevice, c.stream));
  ATM_CUDA(cudaMemcpyAsync(L.mesh.fgeo, ff.data(), ff.size() * sizeof(T), cudaMemcpyHostToDevice, c.stream));
  ATM_CUDA(cudaMemcpyAsync(L.mesh.nbr, hm.nbr.data(), hm.nbr.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
  ATM_CUDA(cudaMemcpyAsync(L.mesh.nbrf, hm.nbrf.data(), hm.nbrf.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
  L.mesh.nhang = hm.nhang;
  if (hm.nhang > 0) {
    std::vector<T> hg(hm.hgeo.begin(), hm.hgeo.end());
    ATM_CUDA(cudaMalloc(&L.mesh.hnb, hm.hnb.size() * sizeof(int)));
    ATM_CUDA(cudaMalloc(&L.mesh.hgeo, hg.size() * sizeof(T)));
    ATM_CUDA(cudaMemcpyAsync(L.mesh.hnb, hm.hnb.data(), hm.hnb.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    ATM_CUDA(cudaMemcpyAsync(L.mesh.hgeo, hg.data(), hg.size() * sizeof(T), cudaMemcpyHostToDevice, c.stream));
    // the host copies above are pageable: finish them before `hg` goes away
    ATM_CUDA(cudaStreamSynchronize(c.stream));
  }
  T **vecs[] = {&L.invd, &L.rho, &L.pfix, &L.x, &L.b, &L.r, &L.t, &L.d};
  for (T **v : vecs) {
    ATM_CUDA(cudaMalloc(v, ns * sizeof(T)));
    ATM_CUDA(cudaMemsetAsync(*v, 0, ns * sizeof(T), c.stream));
  }
  ATM_CUDA(cudaMalloc(&L.wv, 2 * ns * sizeof(T)));
  ATM_CUDA(cudaMalloc(&L.ainv, (size_t)L.nc * ainv_stride_rt(c.k, sizeof(T)) * sizeof(T)));
  // the padding after each FP32 triangle is copied but never used
  ATM_CUDA(cudaMemsetAsync(L.ainv, 0, (size_t)L.nc * ainv_stride_rt(c.k, sizeof(T)) * sizeof(T),
                           c.stream));
  ATM_CUDA(cudaMalloc(&L.pfq, (size_t)L.nc * c.nq2 * sizeof(T)));
  ATM_CUDA(cudaMalloc(&L.pff, (size_t)L.nc * 4 * c.nq * sizeof(T)));
  return level_inv_diag<T>(lview(c, L), L.invd, (T)(1.0 / (GAS_GAMMA - 1.0)));
}

template <typename T>
int build_hier(atm_ctx &c, MG &mg) {
  MGHier<T> &H = hier<T>(mg);
  if (H.built) return ATM_OK;
  make_xfer<T>(c.k, H.tab);
  const size_t nl = mg.hm.size();
  H.lv.resize(nl);
  for (size_t l = 0; l < nl; ++l) {
    H.lv[l].nc = mg.ncells[l];
    int rc = level_alloc<T>(c, H.lv[l], mg.hm[l]);
    if (rc) return rc;
    if (l >= 1) {
      const std::vector<int> &ch = mg.children[l];
      MGLevelT<T> &F = H.lv[l - 1];
      std::vector<int> parent(F.nc, -1), ppos(F.nc, -1);
      for (int cc = 0; cc < H.lv[l].nc; ++cc) {
        if (ch[4 * cc + 1] < 0) {  // the cell is unchanged on this level
          parent[ch[4 * cc]] = cc;
          ppos[ch[4 * cc]] = 4;
          continue;
        }
        for (int p = 0; p < 4; ++p) {
          parent[ch[4 * cc + p]] = cc;
          ppos[ch[4 * cc + p]] = p;
        }
      }
      ATM_CUDA(cudaMalloc(&F.parent, F.nc * sizeof(int)));
      ATM_CUDA(cudaMalloc(&F.ppos, F.nc * sizeof(int)));
      ATM_CUDA(cudaMalloc(&H.lv[l].children, ch.size() * sizeof(int)));
      ATM_CUDA(cudaMemcpyAsync(F.parent, parent.data(), F.nc * sizeof(int), cudaMemcpyHostToDevice, c.stream));
      ATM_CUDA(cudaMemcpyAsync(F.ppos, ppos.data(), F.nc * sizeof(int), cudaMemcpyHostToDevice, c.stream));
      ATM_CUDA(cudaMemcpyAsync(H.lv[l].children, ch.data(), ch.size() * sizeof(int),
                               cudaMemcpyHostToDevice, c.stream));
    }
  }
  if (c.mem) {
    // each level cell carries its member's time-step multiplier (a merged
    // cell's children belong to one member)
    std::vector<double> prev(c.mem->dts_host);
    for (size_t l = 0; l < nl; ++l) {
      std::vector<T> cur(H.lv[l].nc);
      if (l == 0) {
        for (int i = 0; i < H.lv[0].nc; ++i) cur[i] = (T)prev[i];
      } else {
        std::vector<double> next(H.lv[l].nc);
        for (int cc = 0; cc < H.lv[l].nc; ++cc) next[cc] = prev[mg.children[l][4 * cc]];
        for (int i = 0; i < H.lv[l].nc; ++i) cur[i] = (T)next[i];
        prev.swap(next);
      }
      ATM_CUDA(cudaMalloc(&H.lv[l].mesh.dts, cur.size() * sizeof(T)));
      ATM_CUDA(cudaMemcpy(H.lv[l].mesh.dts, cur.data(), cur.size() * sizeof(T),
                          cudaMemcpyHostToDevice));
    }
  }
  H.built = true;
  H.rho_dirty = true;
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  return ATM_OK;
}

// S_l x -> out, with L.wv as the velocity intermediate
template <typename T>
int level_apply(atm_ctx &c, MGLevelT<T> &L, T *out, const T *x) {
  const double co = implicit_coeff(c);
  LevelViewT<T> v = lview(c, L);
  // algorithmic bytes: x, pfix, invd-free D/C read + B/A^{-1} intermediate
  // (2 comps written + read) + A^{-1} as stored (FP32: its triangle) + out; flops: the FP64 formulas of
  // launch_B (mode 2) and launch_CD (mode 1)
  const double ns = (double)L.nc * c.nn2, sz = sizeof(T);
  const double bytes = sz * (ns * (1 + 2 + 2 + 1 + 1 + 1) + (double)L.nc * ainv_stride_rt(c.k, sz));
  const double flops = L.nc * (fl_eval(c.k) + 2 * fl_integrate(c.k, true) + 4.0 * 4 * fl_face(c.k) +
                               4.0 * c.nn2 * c.nn2 + 4 * fl_eval(c.k) + fl_integrate(c.k, true) +
                               4.0 * 7 * fl_face(c.k));
  TimedRegion tr(c, KF_MG_APPLY, bytes, flops);
  int rc = level_B<T>(v, L.wv, x, (T)(co * c.dt / (c.Ma * c.Ma)), 2);
  if (rc) return rc;
  return level_CD<T>(v, out, L.wv, x, (T)(co * c.dt), 1);
}

// One Chebyshev step on level L fused with its operator: t = S_l x (B, then
// C/D), r = b - t, d = (first ? 0 : a d) + b_coef invd r, x += d; the C/D
// kernel does the update in its epilogue instead of storing t.
template <typename T>
int level_apply_cheb(atm_ctx &c, MGLevelT<T> &L, double a, double b_coef, bool first) {
  const double co = implicit_coeff(c);
  LevelViewT<T> v = lview(c, L);
  const double ns = (double)L.nc * c.nn2, sz = sizeof(T);
  // as level_apply, plus rhs, invd, d read and d, x written in the update
  const double bytes = sz * (ns * (1 + 2 + 2 + 1 + 1 + 5) + (double)L.nc * ainv_stride_rt(c.k, sz));
  const double flops = L.nc * (fl_eval(c.k) + 2 * fl_integrate(c.k, true) + 4.0 * 4 * fl_face(c.k) +
                               4.0 * c.nn2 * c.nn2 + 4 * fl_eval(c.k) + fl_integrate(c.k, true) +
                               4.0 * 7 * fl_face(c.k));
  TimedRegion tr(c, KF_MG_APPLY, bytes, flops);
  int rc = level_B<T>(v, L.wv, L.x, (T)(co * c.dt / (c.Ma * c.Ma)), 2);
  if (rc) return rc;
  ChebArgs<T> ch;
  ch.x = L.x;
  ch.d = L.d;
  ch.rhs = L.b;
  ch.a = (T)a;
  ch.b = (T)b_coef;
  ch.first = first ? 1 : 0;
  return level_CD_cheb<T>(v, L.wv, (T)(co * c.dt), ch);
}

template <typename T>
int nrm2(atm_ctx &c, const T *v, long n, double *out_host) {
  k_nrm2_partial<T><<<NB, 256, 0, c.stream>>>(v, n, c.red);
  LAUNCHED();
  k_sum_partial<<<1, 512, 0, c.stream>>>(c.red, c.red_out);
  LAUNCHED();
  int rc = read_scalars(c, 1);
  if (rc) return rc;
  *out_host = std::sqrt(c.h_red[0]);
  return ATM_OK;
}

// largest eigenvalue of invd .* S_l by power iteration
template <typename T>
int estimate_lambda(atm_ctx &c, MGLevelT<T> &L, int its) {
  const long n = (long)L.nc * c.nn2;
  k_hash_init<T><<<gsz(n), 256, 0, c.stream>>>(L.x, n);
  LAUNCHED();
  double nv = 0.0, lam = 0.0;
  int rc = nrm2<T>(c, L.x, n, &nv);
  if (rc) return rc;
  for (int it = 0; it < its; ++it) {
    if ((rc = level_apply<T>(c, L, L.t, L.x))) return rc;
    k_scale_invd<T><<<gsz(n), 256, 0, c.stream>>>(L.d, L.invd, L.t, n);
    LAUNCHED();
    double nw = 0.0;
    if ((rc = nrm2<T>(c, L.d, n, &nw))) return rc;
    if (!(nw > 0.0) || !std::isfinite(nw)) {
      set_error("multigrid: eigenvalue estimate failed");
      return ATM_NONFINITE;
    }
    lam = nw / nv;
    k_scale_copy<T><<<gsz(n), 256, 0, c.stream>>>(L.x, L.d, (T)(1.0 / nw), n);
    LAUNCHED();
    nv = 1.0;
  }
  L.lam = lam;
  return ATM_OK;
}

// Chebyshev smoothing of S_l x = b on [1.2 lam / range, 1.2 lam]
template <typename T>
int chebyshev(atm_ctx &c, MGLevelT<T> &L, int degree, double range, bool zero_start) {
  const long n = (long)L.nc * c.nn2;
  const double hi = 1.2 * L.lam, lo = hi / range;
  const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
  double rho = 1.0 / sigma;
  int rc;
  if (zero_start) {
    k_cheb<T><<<gsz(n), 256, 0, c.stream>>>(L.x, L.d, L.b, L.t, L.invd, T(0),
                                             (T)(1.0 / theta), 1, 0, n);
    LAUNCHED();
  } else if ((rc = level_apply_cheb<T>(c, L, 0.0, 1.0 / theta, true))) {
    return rc;
  }
  for (int k = 1; k < degree; ++k) {
    const double rho_new = 1.0 / (2.0 * sigma - rho);
    if ((rc = level_apply_cheb<T>(c, L, rho_new * rho, 2.0 * rho_new / delta, false))) return rc;
    rho = rho_new;
  }
  return ATM_OK;
}

template <typename T>
int vcycle(atm_ctx &c, MG &mg, MGHier<T> &H, int l) {
  MGLevelT<T> &L = H.lv[l];
  const long n = (long)L.nc * c.nn2;
  int rc;
  // the vector work of this level (transfers, Chebyshev updates) is timed
  // as a whole by the caller's KF_MG_OTHER region minus the level applies
  if (l == (int)H.lv.size() - 1) return chebyshev<T>(c, L, mg.coarse_deg, mg.coarse_range, true);
  if ((rc = chebyshev<T>(c, L, mg.cheb_deg, mg.range, true))) return rc;
  if ((rc = level_apply<T>(c, L, L.t, L.x))) return rc;
  k_sub<T><<<gsz(n), 256, 0, c.stream>>>(L.r, L.b, L.t, n);
  LAUNCHED();
  MGLevelT<T> &Cl = H.lv[l + 1];
  const long nc2 = (long)Cl.nc * c.nn2;
  MG_DISPATCH(c.k, T, k_restrict, (int)((nc2 + 255) / 256), Cl.b, L.r, Cl.children, Cl.nc,
              H.tab);
  LAUNCHED();
  if ((rc = vcycle<T>(c, mg, H, l + 1))) return rc;
  MG_DISPATCH(c.k, T, k_prolong_add, (int)((n + 255) / 256), L.x, Cl.x, L.parent, L.ppos, L.nc,
              H.tab);
  LAUNCHED();
  return chebyshev<T>(c, L, mg.cheb_deg, mg.range, false);
}

// bring rho_fix / p_fix down the hierarchy; rebuild A^{-1} and the
// eigenvalue estimates when rho_fix changed
template <typename T>
int prepare(atm_ctx &c, MG &mg) {
  int rc = build_hier<T>(c, mg);
  if (rc) return rc;
  MGHier<T> &H = hier<T>(mg);
  const long n0 = c.n_scalar();
  MGLevelT<T> &L0 = H.lv[0];
  k_convert<T, double><<<gsz(n0), 256, 0, c.stream>>>(L0.pfix, c.pres_fix, n0);
  LAUNCHED();
  if (H.rho_dirty) {
    k_convert<T, double><<<gsz(n0), 256, 0, c.stream>>>(L0.rho, c.rho_fix, n0);
    LAUNCHED();
  }
  for (size_t l = 1; l < H.lv.size(); ++l) {
    MGLevelT<T> &Cl = H.lv[l], &Fl = H.lv[l - 1];
    const long nc2 = (long)Cl.nc * c.nn2;
    const int grid = (int)((nc2 + 255) / 256);
    MG_DISPATCH(c.k, T, k_inject, grid, Cl.pfix, Fl.pfix, Cl.children, Cl.nc, H.tab);
    LAUNCHED();
    if (H.rho_dirty) {
      MG_DISPATCH(c.k, T, k_inject, grid, Cl.rho, Fl.rho, Cl.children, Cl.nc, H.tab);
      LAUNCHED();
    }
  }
  for (auto &L : H.lv)
    if ((rc = level_pfix_prep<T>(lview(c, L)))) return rc;
  if (H.rho_dirty) {
    for (auto &L : H.lv) {
      if ((rc = level_block_inverse<T>(lview(c, L), L.ainv, L.rho))) return rc;
      if ((rc = estimate_lambda<T>(c, L, mg.eig_its))) return rc;
    }
    H.rho_dirty = false;
    ++H.lam_epoch;
  }
  return ATM_OK;
}

// Record one V-cycle (input L0.b, output L0.x) into H.graph.  The capture
// runs on the hierarchy's private non-blocking stream (the legacy default
// stream cannot be captured) in thread-local mode, so members captured or
// running on other threads are not affected; the kernels counted while
// recording did not run and are taken off the launch counter.
template <typename T>
int capture_vcycle(atm_ctx &c, MG &mg, MGHier<T> &H) {
  if (!mg.cap_stream)
    ATM_CUDA(cudaStreamCreateWithFlags(&mg.cap_stream, cudaStreamNonBlocking));
  hier_drop_graph(H);
  // the capture stream must not start before work already queued on c.stream
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  cudaStream_t saved = c.stream;
  c.stream = mg.cap_stream;
  c.capturing = true;
  const long before = g_kernel_launches.load();
  cudaError_t e = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal);
  int rc = e == cudaSuccess ? ATM_OK : cuda_fail(e, "cudaStreamBeginCapture");
  if (rc == ATM_OK) {
    rc = vcycle<T>(c, mg, H, 0);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(c.stream, &g);
    if (rc == ATM_OK && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamEndCapture");
    if (rc == ATM_OK) {
      e = cudaGraphInstantiate(&H.graph, g, 0);
      if (e != cudaSuccess) {
        H.graph = nullptr;
        rc = cuda_fail(e, "cudaGraphInstantiate");
      }
    }
    if (g) cudaGraphDestroy(g);
  }
  const long recorded = g_kernel_launches.load() - before;
  g_kernel_launches.fetch_sub(recorded);
  c.capturing = false;
  c.stream = saved;
  if (rc == ATM_OK) H.graph_kernels = recorded;
  cudaGetLastError();  // a failed capture leaves no sticky error behind
  return rc;
}

template <typename T>
int precondition(atm_ctx &c, MG &mg, double *z, const double *v) {
  MGHier<T> &H = hier<T>(mg);
  MGLevelT<T> &L0 = H.lv[0];
  const long n = c.n_scalar();
  k_convert<T, double><<<gsz(n), 256, 0, c.stream>>>(L0.b, v, n);
  LAUNCHED();
  int rc = ATM_OK;
  bool replayed = false;
  if (mg.use_graphs && !H.graph_failed) {
    const double key[4] = {implicit_coeff(c), c.dt, c.Ma, (double)H.lam_epoch};
    if (!H.graph || std::memcmp(key, H.graph_key, sizeof(key)) != 0) {
      if (capture_vcycle<T>(c, mg, H) == ATM_OK) {
        std::memcpy(H.graph_key, key, sizeof(key));
      } else {
        H.graph_failed = true;  // keep running the V-cycle launch by launch
        hier_drop_graph(H);
      }
    }
    if (H.graph) {
      TimedRegion tr(c, KF_MG_OTHER, 0.0, 0.0);  // whole V-cycle
      ATM_CUDA(cudaGraphLaunch(H.graph, c.stream));
      g_kernel_launches.fetch_add(H.graph_kernels);
      ++mg.graph_replays;
      replayed = true;
    }
  }
  if (!replayed) {
    TimedRegion tr(c, KF_MG_OTHER, 0.0, 0.0);  // whole V-cycle (includes the level applies)
    rc = vcycle<T>(c, mg, H, 0);
  }
  if (rc) return rc;
  ++mg.vcycles;
  k_convert<double, T><<<gsz(n), 256, 0, c.stream>>>(z, L0.x, n);
  LAUNCHED();
  return ATM_OK;
}

int prepare_any(atm_ctx &c, int precision) {
  return precision == 2 ? prepare<double>(c, *c.mg) : prepare<float>(c, *c.mg);
}

}  // namespace

int mg_prepare(atm_ctx &c, int precision) {
  if (!c.mg || c.mg->hm.size() < 2) {
    set_error("no multigrid levels (atm_mg_add_level)");
    return ATM_NOT_READY;
  }
  return prepare_any(c, precision);
}
int mg_vcycle_only(atm_ctx &c, int precision, double *z, const double *v) {
  return precision == 2 ? precondition<double>(c, *c.mg, z, v)
                        : precondition<float>(c, *c.mg, z, v);
}
double *mg_zbasis(atm_ctx &c) { return c.mg ? c.mg->zbasis : nullptr; }
int mg_restart(const atm_ctx &c) { return c.mg ? c.mg->restart : 16; }
void mg_invalidate(atm_ctx &c) {
  if (!c.mg) return;
  hier_free(c.mg->f);
  hier_free(c.mg->d);
}

// ------------------------------------------------------------- set-up --
int mg_free(atm_ctx &c) {
  if (!c.mg) return ATM_OK;
  hier_free(c.mg->f);
  hier_free(c.mg->d);
  cudaFree(c.mg->zbasis);
  if (c.mg->cap_stream) cudaStreamDestroy(c.mg->cap_stream);
  delete c.mg;
  c.mg = nullptr;
  return ATM_OK;
}

// level 0 (the operator mesh) is recorded on the first call
int mg_add_level(atm_ctx &c, int n_cells, int mapdeg, const double *nodes, int n_inner,
                 const int *inner, int n_bdry, const int *bdry, const int *children) {
  if (!children || n_cells < 1) {
    set_error("atm_mg_add_level: need n_cells >= 1 and a children table");
    return ATM_BAD_ARG;
  }
  if (!c.mg) {
    MG *mg = new MG();
    HostMesh hm;
    hm.qgeo.resize((size_t)c.nc * 5 * c.nq2);
    hm.fgeo.resize((size_t)c.nc * 4 * 3 * c.nq);
    hm.nbr.resize((size_t)c.nc * 4);
    hm.nbrf.resize((size_t)c.nc * 4);
    hm.nhang = c.mesh.nhang;
    hm.hnb.resize((size_t)c.mesh.nhang * 2);
    hm.hgeo.resize((size_t)c.mesh.nhang * 2 * 3 * c.nq);
    hm.map2 = c.map2;
    ATM_CUDA(cudaMemcpyAsync(hm.qgeo.data(), c.mesh.qgeo, hm.qgeo.size() * 8, cudaMemcpyDeviceToHost, c.stream));
    ATM_CUDA(cudaMemcpyAsync(hm.fgeo.data(), c.mesh.fgeo, hm.fgeo.size() * 8, cudaMemcpyDeviceToHost, c.stream));
    ATM_CUDA(cudaMemcpyAsync(hm.nbr.data(), c.mesh.nbr, hm.nbr.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    ATM_CUDA(cudaMemcpyAsync(hm.nbrf.data(), c.mesh.nbrf, hm.nbrf.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    if (hm.nhang > 0) {
      ATM_CUDA(cudaMemcpyAsync(hm.hnb.data(), c.mesh.hnb, hm.hnb.size() * 4, cudaMemcpyDeviceToHost, c.stream));
      ATM_CUDA(cudaMemcpyAsync(hm.hgeo.data(), c.mesh.hgeo, hm.hgeo.size() * 8, cudaMemcpyDeviceToHost, c.stream));
    }
    ATM_CUDA(cudaStreamSynchronize(c.stream));
    mg->hm.push_back(std::move(hm));
    mg->ncells.push_back(c.nc);
    mg->children.emplace_back();
    const long zn = (long)mg->restart * c.n_scalar();
    cudaError_t e = cudaMalloc(&mg->zbasis, zn * sizeof(double));
    if (e != cudaSuccess) {
      delete mg;
      return cuda_fail(e, "cudaMalloc FGMRES basis");
    }
    c.mg = mg;
  }
  MG &mg = *c.mg;
  const int nfine = mg.ncells.back();
  // a row is four cells of the finer level (a merged cell) or one cell and
  // three -1 (a cell that stays as it is: adaptive meshes coarsen their
  // finest cells first); every finer cell appears exactly once
  std::vector<int> seen(nfine, 0), ch(children, children + 4L * n_cells);
  long covered = 0;
  for (int cc = 0; cc < n_cells; ++cc) {
    const int *r = &ch[4L * cc];
    const bool same = r[1] < 0 && r[2] < 0 && r[3] < 0;
    for (int q = 0; q < (same ? 1 : 4); ++q) {
      if (r[q] < 0 || r[q] >= nfine || seen[r[q]]) {
        set_error("atm_mg_add_level: children row " + std::to_string(cc) +
                  " has an entry out of range or repeated (rows are 4 finer cells, or one "
                  "finer cell and three -1)");
        return ATM_BAD_ARG;
      }
      seen[r[q]] = 1;
      ++covered;
    }
  }
  if (covered != nfine || n_cells >= nfine) {
    set_error("atm_mg_add_level: the children table must cover every cell of the finer level "
              "exactly once and merge at least one group");
    return ATM_BAD_ARG;
  }
  HostMesh hm;
  int rc = build_mesh_tables(c.k, n_cells, mapdeg, nodes, n_inner, inner, n_bdry, bdry, hm);
  if (rc) return rc;
  mg.hm.push_back(std::move(hm));
  mg.ncells.push_back(n_cells);
  mg.children.push_back(std::move(ch));
  // device hierarchies are rebuilt on next use
  hier_free(mg.f);
  hier_free(mg.d);
  return ATM_OK;
}

int mg_precondition(atm_ctx &c, int precision, double *z, const double *v) {
  if (!c.mg || c.mg->hm.size() < 2) {
    set_error("no multigrid levels (atm_mg_add_level)");
    return ATM_NOT_READY;
  }
  int rc = prepare_any(c, precision);
  if (rc) return rc;
  return precision == 2 ? precondition<double>(c, *c.mg, z, v)
                        : precondition<float>(c, *c.mg, z, v);
}

// FGMRES(m) on S x = b with the V-cycle as right preconditioner; stops when
// the (unpreconditioned) residual estimate <= tol, or, with the true-residual
// check on, when the recomputed residual is.  Same CGS2 (arnoldi_step) and
// Givens machinery as gmres_schur.
int fgmres_mg(atm_ctx &c, int precision, double *x, const double *b, double tol, int maxit,
              int *its, double *res) {
  if (!c.mg || c.mg->hm.size() < 2) {
    set_error("FGMRES: no multigrid levels (atm_mg_add_level)");
    return ATM_NOT_READY;
  }
  if (precision != 1 && precision != 2) {
    set_error("FGMRES: precision must be 1 (FP32 V-cycle) or 2 (FP64 V-cycle)");
    return ATM_BAD_ARG;
  }
  MG &mg = *c.mg;
  int rc = prepare_any(c, precision);
  if (rc) return rc;
  const long n = c.n_scalar();
  const int m = mg.restart;
  double *V = c.krylov, *Z = mg.zbasis;
  double *w = c.ws1, *t = c.ws2;
  double *nsq = c.dsmall + 64, *ydev = c.dsmall + 96;
  std::vector<double> H((m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m), hcol(m + 1);
  *its = 0;
  *res = 0.0;
  for (;;) {
    if ((rc = schur_apply(c, t, x, false))) return rc;
    k_sub<double><<<gsz(n), 256, 0, c.stream>>>(V, b, t, n);
    LAUNCHED();
    if ((rc = vec_dot(c.stream, V, V, n, c.red, nsq))) return rc;
    ATM_CUDA(cudaMemcpyAsync(c.h_red, nsq, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    ATM_CUDA(cudaStreamSynchronize(c.stream));
    const double beta = std::sqrt(c.h_red[0]);
    *res = beta;
    if (!std::isfinite(beta)) { set_error("FGMRES: non-finite residual"); return ATM_NONFINITE; }
    if (beta <= tol) return ATM_OK;
    if (*its >= maxit) return ATM_NOT_CONVERGED;
    if ((rc = vec_scale_by_inv_norm(c.stream, V, V, nsq, n))) return rc;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int jend = 0;
    bool done = false;
    for (int j = 0; j < m; ++j) {
      ++*its;
      rc = precision == 2 ? precondition<double>(c, mg, Z + (long)j * n, V + (long)j * n)
                          : precondition<float>(c, mg, Z + (long)j * n, V + (long)j * n);
      if (rc) return rc;
      if ((rc = schur_apply(c, w, Z + (long)j * n, false))) return rc;
      double hn = 0.0;
      if ((rc = arnoldi_step(c.stream, V, n, j, w, c.red, c.dsmall, c.h_red, hcol.data(), &hn)))
        return rc;
      for (int l = 0; l <= j; ++l) H[l * m + j] = hcol[l];
      if (!std::isfinite(hn)) { set_error("FGMRES: non-finite Arnoldi vector"); return ATM_NONFINITE; }
      H[(j + 1) * m + j] = hn;
      for (int l = 0; l < j; ++l) {
        const double a = H[l * m + j], bb = H[(l + 1) * m + j];
        H[l * m + j] = cs[l] * a + sn[l] * bb;
        H[(l + 1) * m + j] = -sn[l] * a + cs[l] * bb;
      }
      const double a = H[j * m + j], bb = H[(j + 1) * m + j];
      const double r = std::sqrt(a * a + bb * bb);
      cs[j] = a / r;
      sn[j] = bb / r;
      H[j * m + j] = r;
      H[(j + 1) * m + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      jend = j + 1;
      *res = std::fabs(g[j + 1]);
      if (*res <= tol || hn == 0.0 || *its >= maxit) { done = true; break; }
    }
    for (int l = jend - 1; l >= 0; --l) {
      double s = g[l];
      for (int mm = l + 1; mm < jend; ++mm) s -= H[l * m + mm] * y[mm];
      y[l] = s / H[l * m + l];
    }
    ATM_CUDA(cudaMemcpyAsync(ydev, y.data(), jend * sizeof(double), cudaMemcpyHostToDevice,
                             c.stream));
    if ((rc = vec_multiaxpy(c.stream, x, Z, n, jend, ydev, 1.0, n))) return rc;
    ATM_CUDA(cudaStreamSynchronize(c.stream));
    if (done && !c.true_residual_check)
      return (*res <= tol) ? ATM_OK : (*its >= maxit ? ATM_NOT_CONVERGED : ATM_OK);
  }
}

void mg_mark_rho_changed(atm_ctx &c) {
  if (c.mg) {
    c.mg->f.rho_dirty = true;
    c.mg->d.rho_dirty = true;
  }
}

int mg_set_params(atm_ctx &c, int degree, double range, int eig_its, int coarse_degree) {
  if (!c.mg) {
    set_error("atm_mg_set_smoother: add levels first");
    return ATM_NOT_READY;
  }
  if (degree < 1 || !(range > 1.0) || eig_its < 1 || coarse_degree < 1) {
    set_error("atm_mg_set_smoother: bad parameters");
    return ATM_BAD_ARG;
  }
  hier_drop_graph(c.mg->f);
  hier_drop_graph(c.mg->d);
  c.mg->cheb_deg = degree;
  c.mg->range = range;
  c.mg->eig_its = eig_its;
  c.mg->coarse_deg = coarse_degree;
  mg_mark_rho_changed(c);
  return ATM_OK;
}

long mg_vcycles(const atm_ctx &c) { return c.mg ? c.mg->vcycles : 0; }
int mg_set_graphs(atm_ctx &c, bool on) {
  if (!c.mg) {
    set_error("atm_mg_set_graphs: add levels first");
    return ATM_NOT_READY;
  }
  c.mg->use_graphs = on;
  if (!on) {
    hier_drop_graph(c.mg->f);
    hier_drop_graph(c.mg->d);
  }
  return ATM_OK;
}
void mg_stats(const atm_ctx &c, long *out) {
  out[0] = c.mg ? c.mg->vcycles : 0;
  out[1] = c.mg ? c.mg->graph_replays : 0;
}
int mg_levels(const atm_ctx &c) { return c.mg ? (int)c.mg->hm.size() : 0; }

}  // namespace atm
