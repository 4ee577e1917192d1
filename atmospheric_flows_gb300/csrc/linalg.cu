// Krylov vector kernels and diagnostics reductions (FP64).
// Reductions are deterministic: a fixed grid of RED_BLOCKS blocks with a fixed
// element-to-thread map writes per-block partials, and a second pass sums the
// partials in a fixed order, so a result never depends on scheduling.
// They replace the deal.II vector operations used by SolverCG/SolverGMRES and
// the diagnostics of Atmospheric_Flow.cc:991-1087, 1140-1148.
#include <cfloat>
#include <cmath>

#include "atm_device.cuh"

namespace atm {

namespace {
constexpr int RT = 256;  // threads per reduction block
constexpr int MAXM = 32;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
// op: 0 sum, 1 max, 2 min; result valid in thread 0
template <int OP>
__device__ double block_reduce(double v, double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = OP == 0 ? warp_sum(v) : (OP == 1 ? warp_max(v) : warp_min(v));
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  if (wid == 0) {
    v = lane < nw ? sh[lane] : (OP == 0 ? 0.0 : (OP == 1 ? -DBL_MAX : DBL_MAX));
    v = OP == 0 ? warp_sum(v) : (OP == 1 ? warp_max(v) : warp_min(v));
  }
  return v;
}

__global__ void k_copy(double *__restrict__ d, const double *__restrict__ s, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    d[i] = s[i];
}
__global__ void k_fill(double *__restrict__ d, double v, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    d[i] = v;
}
__global__ void k_axpy(double *__restrict__ y, double a, const double *__restrict__ x, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
__global__ void k_xmy_scaled(double *__restrict__ d, const double *__restrict__ dg,
                             const double *__restrict__ b, const double *__restrict__ t, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    d[i] = dg[i] * (b[i] - t[i]);
}
__global__ void k_scale_inv_norm(double *__restrict__ d, const double *__restrict__ s,
                                 const double *__restrict__ nsq, long n) {
  const double inv = 1.0 / sqrt(*nsq);
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    d[i] = s[i] * inv;
}

__global__ void k_dot_partial(const double *__restrict__ x, const double *__restrict__ y, long n,
                              double *__restrict__ red) {
  __shared__ double sh[RT / 32];
  double acc = 0.0;
  for (long i = (long)blockIdx.x * RT + threadIdx.x; i < n; i += (long)RED_BLOCKS * RT)
    acc = fma(x[i], y[i], acc);
  acc = block_reduce<0>(acc, sh);
  if (threadIdx.x == 0) red[blockIdx.x] = acc;
}

// out[row] = sum of red[row*RED_BLOCKS .. +RED_BLOCKS) (OP 0), max (1), min (2)
template <int OP>
__global__ void k_finalize(const double *__restrict__ red, double *__restrict__ out) {
  __shared__ double sh[RT / 32];
  const double *r = red + (long)blockIdx.x * RED_BLOCKS;
  double acc = OP == 0 ? 0.0 : (OP == 1 ? -DBL_MAX : DBL_MAX);
  for (int i = threadIdx.x; i < RED_BLOCKS; i += RT)
    acc = OP == 0 ? acc + r[i] : (OP == 1 ? fmax(acc, r[i]) : fmin(acc, r[i]));
  acc = block_reduce<OP>(acc, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

// M vectors per pass: fixed-size accumulators stay in registers
template <int M>
__global__ void k_multidot_partial(const double *__restrict__ V, long ldv,
                                   const double *__restrict__ w, long n,
                                   double *__restrict__ red) {
  __shared__ double sh[RT / 32];
  double acc[M];
#pragma unroll
  for (int l = 0; l < M; ++l) acc[l] = 0.0;
  for (long i = (long)blockIdx.x * RT + threadIdx.x; i < n; i += (long)RED_BLOCKS * RT) {
    const double wi = w[i];
#pragma unroll
    for (int l = 0; l < M; ++l) acc[l] = fma(V[l * ldv + i], wi, acc[l]);
  }
#pragma unroll
  for (int l = 0; l < M; ++l) {
    const double s = block_reduce<0>(acc[l], sh);
    if (threadIdx.x == 0) red[(long)l * RED_BLOCKS + blockIdx.x] = s;
  }
}

// up to 8 vectors per launch; larger m is split into chunks of 8
void multidot_chunk(cudaStream_t st, const double *V, long ldv, int m, const double *w,
                    long n, double *red) {
  switch (m) {
    case 1: k_multidot_partial<1><<<RED_BLOCKS, RT, 0, st>>>(V, ldv, w, n, red); break;
    case 2: k_multidot_partial<2><<<RED_BLOCKS, RT, 0, st>>>(V, ldv, w, n, red); break;
    case 3: k_multidot_partial<3><<<RED_BLOCKS, RT, 0, st>>>(V, ldv, w, n, red); break;
    case 4: k_multidot_partial<4><<<RED_BLOCKS, RT, 0, st>>>(V, ldv, w, n, red); break;
    case 5: k_multidot_partial<5><<<RED_BLOCKS, RT, 0, st>>>(V, ldv, w, n, red); break;
    case 6: k_multidot_partial<6><<<RED_BLOCKS, RT, 0, st>>>(V, ldv, w, n, red); break;
    case 7: k_multidot_partial<7><<<RED_BLOCKS, RT, 0, st>>>(V, ldv, w, n, red); break;
    default: k_multidot_partial<8><<<RED_BLOCKS, RT, 0, st>>>(V, ldv, w, n, red); break;
  }
  g_kernel_launches.fetch_add(1);
}

__global__ void k_multiaxpy(double *__restrict__ w, const double *__restrict__ V, long ldv,
                            int m, const double *__restrict__ h, double sign, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int l = 0; l < m; ++l) s = fma(h[l], V[l * ldv + i], s);
    w[i] += sign * s;
  }
}

// w <- w - sum_l h[l] V_l over all m vectors, then the first M dot products
// V_l . w with the updated w: "subtract, then project again" of CGS2 in one
// sweep over V.  The per-element sums, the element-to-thread map and the
// summation order are those of k_multiaxpy and k_multidot_partial, so the
// results are the same bits as the two separate kernels.
template <int M>
__global__ void k_axpy_multidot(double *__restrict__ w, const double *__restrict__ V, long ldv,
                                int m, const double *__restrict__ h, long n,
                                double *__restrict__ red) {
  __shared__ double sh[RT / 32];
  double acc[M];
#pragma unroll
  for (int l = 0; l < M; ++l) acc[l] = 0.0;
  for (long i = (long)blockIdx.x * RT + threadIdx.x; i < n; i += (long)RED_BLOCKS * RT) {
    double v[M], s = 0.0;
#pragma unroll
    for (int l = 0; l < M; ++l) {
      v[l] = V[l * ldv + i];
      s = fma(h[l], v[l], s);
    }
    for (int l = M; l < m; ++l) s = fma(h[l], V[l * ldv + i], s);
    const double wi = w[i] + -1.0 * s;
    w[i] = wi;
#pragma unroll
    for (int l = 0; l < M; ++l) acc[l] = fma(v[l], wi, acc[l]);
  }
#pragma unroll
  for (int l = 0; l < M; ++l) {
    const double t = block_reduce<0>(acc[l], sh);
    if (threadIdx.x == 0) red[(long)l * RED_BLOCKS + blockIdx.x] = t;
  }
}

// w <- w - sum_l h[l] V_l, then |w|^2 (k_multiaxpy followed by k_dot_partial
// on w, in one sweep, same bits)
__global__ void k_axpy_dot(double *__restrict__ w, const double *__restrict__ V, long ldv, int m,
                           const double *__restrict__ h, long n, double *__restrict__ red) {
  __shared__ double sh[RT / 32];
  double acc = 0.0;
  for (long i = (long)blockIdx.x * RT + threadIdx.x; i < n; i += (long)RED_BLOCKS * RT) {
    double s = 0.0;
    for (int l = 0; l < m; ++l) s = fma(h[l], V[l * ldv + i], s);
    const double wi = w[i] + -1.0 * s;
    w[i] = wi;
    acc = fma(wi, wi, acc);
  }
  acc = block_reduce<0>(acc, sh);
  if (threadIdx.x == 0) red[blockIdx.x] = acc;
}

__global__ void k_maxdiff_partial(const double *__restrict__ a, const double *__restrict__ b,
                                  long n, double *__restrict__ red) {
  __shared__ double sh[RT / 32];
  double m0 = 0.0, m1 = 0.0;
  for (long i = (long)blockIdx.x * RT + threadIdx.x; i < n; i += (long)RED_BLOCKS * RT) {
    const double ai = a[i];
    m1 = fmax(m1, fabs(ai));
    m0 = fmax(m0, fabs(b ? ai - b[i] : ai));
  }
  m0 = block_reduce<1>(m0, sh);
  if (threadIdx.x == 0) red[blockIdx.x] = m0;
  m1 = block_reduce<1>(m1, sh);
  if (threadIdx.x == 0) red[RED_BLOCKS + blockIdx.x] = m1;
}

__global__ void k_diag_partial(const double *__restrict__ rho, const double *__restrict__ u,
                               const double *__restrict__ p, int nc, int nn2,
                               double *__restrict__ red) {
  __shared__ double sh[RT / 32];
  double rmin = DBL_MAX, rmax = 0.0, cmax = 0.0, umax = 0.0;
  const long n = (long)nc * nn2;
  for (long i = (long)blockIdx.x * RT + threadIdx.x; i < n; i += (long)RED_BLOCKS * RT) {
    const long c = i / nn2, j = i - c * nn2;
    const double r = rho[i];
    rmin = fmin(rmin, r);
    rmax = fmax(rmax, fabs(r));
    cmax = fmax(cmax, sqrt(GAS_GAMMA * p[i] / r));
    const double u0 = u[(c * 2) * nn2 + j], u1 = u[(c * 2 + 1) * nn2 + j];
    umax = fmax(umax, sqrt(u0 * u0 + u1 * u1));
  }
  double v = block_reduce<2>(rmin, sh);
  if (threadIdx.x == 0) red[blockIdx.x] = v;
  v = block_reduce<1>(rmax, sh);
  if (threadIdx.x == 0) red[RED_BLOCKS + blockIdx.x] = v;
  v = block_reduce<1>(cmax, sh);
  if (threadIdx.x == 0) red[2 * RED_BLOCKS + blockIdx.x] = v;
  v = block_reduce<1>(umax, sh);
  if (threadIdx.x == 0) red[3 * RED_BLOCKS + blockIdx.x] = v;
}

// relax u toward (ub0, ub1), or toward the per-node target velocity (same
// layout as u) when one is given
__global__ void k_sponge(double *__restrict__ u, const double *__restrict__ alpha, double dt,
                         double ub0, double ub1, const double *__restrict__ target,
                         const double *__restrict__ dts, int nc, int nn2) {
  const long n = (long)nc * nn2;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long c = i / nn2, j = i - c * nn2;
    const double a = dt * (dts ? dts[c] : 1.0) * alpha[i];
    if (a == 0.0) continue;
    const long i0 = (c * 2) * nn2 + j, i1 = (c * 2 + 1) * nn2 + j;
    const double t0 = target ? target[i0] : ub0, t1 = target ? target[i1] : ub1;
    u[i0] = (u[i0] + a * t0) / (1.0 + a);
    u[i1] = (u[i1] + a * t1) / (1.0 + a);
  }
}

inline int grid_for(long n) {
  long g = (n + 255) / 256;
  if (g > 152L * 16) g = 152L * 16;  // grid-stride beyond 16 blocks per SM
  return (int)(g < 1 ? 1 : g);
}
}  // namespace

int vec_copy(cudaStream_t st, double *dst, const double *src, long n) {
  if (n <= 0 || dst == src) return ATM_OK;
  k_copy<<<grid_for(n), 256, 0, st>>>(dst, src, n);
  ATM_CHECK_LAUNCH("k_copy");
  return ATM_OK;
}
int vec_fill(cudaStream_t st, double *dst, double v, long n) {
  if (n <= 0) return ATM_OK;
  k_fill<<<grid_for(n), 256, 0, st>>>(dst, v, n);
  ATM_CHECK_LAUNCH("k_fill");
  return ATM_OK;
}
int vec_axpy(cudaStream_t st, double *y, double a, const double *x, long n) {
  if (n <= 0) return ATM_OK;
  k_axpy<<<grid_for(n), 256, 0, st>>>(y, a, x, n);
  ATM_CHECK_LAUNCH("k_axpy");
  return ATM_OK;
}
int vec_xmy_scaled(cudaStream_t st, double *dst, const double *d, const double *b,
                   const double *t, long n) {
  k_xmy_scaled<<<grid_for(n), 256, 0, st>>>(dst, d, b, t, n);
  ATM_CHECK_LAUNCH("k_xmy_scaled");
  return ATM_OK;
}
int vec_scale_by_inv_norm(cudaStream_t st, double *dst, const double *src, const double *nsq,
                          long n) {
  k_scale_inv_norm<<<grid_for(n), 256, 0, st>>>(dst, src, nsq, n);
  ATM_CHECK_LAUNCH("k_scale_inv_norm");
  return ATM_OK;
}
int vec_dot(cudaStream_t st, const double *x, const double *y, long n, double *red,
            double *out) {
  k_dot_partial<<<RED_BLOCKS, RT, 0, st>>>(x, y, n, red);
  k_finalize<0><<<1, RT, 0, st>>>(red, out);
  ATM_CHECK_LAUNCH("vec_dot");
  return ATM_OK;
}
int vec_multidot(cudaStream_t st, const double *V, long ldv, int m, const double *w, long n,
                 double *red, double *out) {
  if (m < 1 || m > MAXM) return ATM_BAD_ARG;
  for (int l0 = 0; l0 < m; l0 += 8) {
    const int mm = m - l0 < 8 ? m - l0 : 8;
    multidot_chunk(st, V + (long)l0 * ldv, ldv, mm, w, n, red + (long)l0 * RED_BLOCKS);
  }
  k_finalize<0><<<m, RT, 0, st>>>(red, out);
  ATM_CHECK_LAUNCH("vec_multidot");
  return ATM_OK;
}
int vec_multiaxpy(cudaStream_t st, double *w, const double *V, long ldv, int m,
                  const double *h, double sign, long n) {
  if (m < 1) return ATM_OK;
  k_multiaxpy<<<grid_for(n), 256, 0, st>>>(w, V, ldv, m, h, sign, n);
  ATM_CHECK_LAUNCH("k_multiaxpy");
  return ATM_OK;
}
int arnoldi_step(cudaStream_t st, double *V, long n, int j, double *w, double *red,
                 double *dsmall, double *h_pinned, double *hcol, double *hn) {
  double *h1 = dsmall, *h2 = dsmall + 32, *nsq = dsmall + 64;
  const int m = j + 1;
  if (m > MAXM) {
    set_error("Arnoldi step: more basis vectors than the reduction buffer holds");
    return ATM_BAD_ARG;
  }
  int rc;
  // h1 = V^T w
  if ((rc = vec_multidot(st, V, n, m, w, n, red, h1))) return rc;
  // w -= V h1 and h2 = V^T w, fused over the first 8 vectors
  const int m0 = m < 8 ? m : 8;
  switch (m0) {
    case 1: k_axpy_multidot<1><<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h1, n, red); break;
    case 2: k_axpy_multidot<2><<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h1, n, red); break;
    case 3: k_axpy_multidot<3><<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h1, n, red); break;
    case 4: k_axpy_multidot<4><<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h1, n, red); break;
    case 5: k_axpy_multidot<5><<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h1, n, red); break;
    case 6: k_axpy_multidot<6><<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h1, n, red); break;
    case 7: k_axpy_multidot<7><<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h1, n, red); break;
    default: k_axpy_multidot<8><<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h1, n, red); break;
  }
  g_kernel_launches.fetch_add(1);
  for (int l0 = 8; l0 < m; l0 += 8) {
    const int mm = m - l0 < 8 ? m - l0 : 8;
    multidot_chunk(st, V + (long)l0 * n, n, mm, w, n, red + (long)l0 * RED_BLOCKS);
  }
  k_finalize<0><<<m, RT, 0, st>>>(red, h2);
  ATM_CHECK_LAUNCH("k_axpy_multidot");
  // w -= V h2 and |w|^2
  k_axpy_dot<<<RED_BLOCKS, RT, 0, st>>>(w, V, n, m, h2, n, red);
  g_kernel_launches.fetch_add(1);
  k_finalize<0><<<1, RT, 0, st>>>(red, nsq);
  ATM_CHECK_LAUNCH("k_axpy_dot");
  ATM_CUDA(cudaMemcpyAsync(h_pinned, dsmall, 65 * sizeof(double), cudaMemcpyDeviceToHost, st));
  ATM_CUDA(cudaStreamSynchronize(st));
  for (int l = 0; l <= j; ++l) hcol[l] = h_pinned[l] + h_pinned[32 + l];
  *hn = std::sqrt(h_pinned[64]);
  if (*hn > 0.0 && std::isfinite(*hn))
    if ((rc = vec_scale_by_inv_norm(st, V + (long)(j + 1) * n, w, nsq, n))) return rc;
  return ATM_OK;
}
int vec_maxdiff(cudaStream_t st, const double *a, const double *b, long n, double *red,
                double *out) {
  k_maxdiff_partial<<<RED_BLOCKS, RT, 0, st>>>(a, b, n, red);
  k_finalize<1><<<2, RT, 0, st>>>(red, out);
  ATM_CHECK_LAUNCH("vec_maxdiff");
  return ATM_OK;
}
int vec_diagnostics(cudaStream_t st, const double *rho, const double *u, const double *p,
                    int nc, int nn2, double *red, double *out) {
  k_diag_partial<<<RED_BLOCKS, RT, 0, st>>>(rho, u, p, nc, nn2, red);
  k_finalize<2><<<1, RT, 0, st>>>(red, out);
  k_finalize<1><<<3, RT, 0, st>>>(red + RED_BLOCKS, out + 1);
  ATM_CHECK_LAUNCH("vec_diagnostics");
  return ATM_OK;
}
int vec_sponge(cudaStream_t st, double *u, const double *alpha, double dt, double ub0,
               double ub1, const double *target, const double *dts, int nc, int nn2) {
  const long n = (long)nc * nn2;
  k_sponge<<<grid_for(n), 256, 0, st>>>(u, alpha, dt, ub0, ub1, target, dts, nc, nn2);
  ATM_CHECK_LAUNCH("k_sponge");
  return ATM_OK;
}

}  // namespace atm

// ------------------------------------------------------------------------
// FMA throughput probe: 8 independent FMA chains per thread on a grid of
// 8 blocks per SM; used to measure the FP64 / FP32 denominators of the
// compute roofline on the machine the bench runs on.
namespace atm {
namespace {
template <typename T>
__global__ void k_fma_probe(T *out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
template <typename T>
int probe(int iters, double *gflops) {
  int dev = 0, nsm = 0;
  ATM_CUDA(cudaGetDevice(&dev));
  ATM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = nsm * 8, threads = 256;
  T *out = nullptr;
  ATM_CUDA(cudaMalloc(&out, sizeof(T) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_probe<T><<<blocks, threads>>>(out, 16, (T)0.999, (T)0.001);
  cudaEventRecord(e0);
  k_fma_probe<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  g_kernel_launches.fetch_add(2);
  if (err != cudaSuccess) return cuda_fail(err, "fma probe");
  *gflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e9;
  return ATM_OK;
}
}  // namespace
}  // namespace atm

extern "C" int atm_probe_fma_peak(double *fp64_gflops, double *fp32_gflops) {
  if (!fp64_gflops || !fp32_gflops) return ATM_BAD_ARG;
  int rc = atm::probe<double>(4000, fp64_gflops);
  if (rc) return rc;
  return atm::probe<float>(100000, fp32_gflops);
}
