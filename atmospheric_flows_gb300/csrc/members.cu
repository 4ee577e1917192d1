// Several independent members in one context (a concatenated cell list):
// member tables, member-wise reductions and vector updates, and the Schur
// solve of every member with its own Krylov iteration.
//
// The reference runs one member per process (Atmospheric_Flow.cc:1265-1313);
// this is the serving form of the same solvers.  The operators are block
// diagonal over members (members share no faces), so one kernel launch
// applies every member's operator.  What couples members in a plain
// concatenated solve is the Krylov method's inner products; here every inner
// product, norm and Hessenberg matrix is member-wise, each member stops on its
// own residual, and a member that has stopped (or is frozen by its Picard
// loop) takes no further update.  In exact arithmetic each member's iterates
// are those of its solo run (GMRES + Jacobi: identical; FGMRES + multigrid:
// the V-cycle's Chebyshev interval is the batch's, so the preconditioner, not
// the solution, differs).
#include <cmath>
#include <cstring>

#include "atm_device.cuh"

namespace atm {

namespace {
constexpr int RT = 256;

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
// OP 0 sum, 1 max; result in thread 0
template <int OP>
__device__ double block_red(double v, double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = OP == 0 ? warp_sum(v) : warp_max(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sh[lane] : (OP == 0 ? 0.0 : -1.0);
    v = OP == 0 ? warp_sum(v) : warp_max(v);
  }
  return v;
}

// block (b, m) reduces its share of member m's elements eoff[m]..eoff[m+1];
// partials red[(l * nm + m) * sb + b]
template <int M>
__global__ void k_seg_multidot(const double *__restrict__ V, long ldv,
                               const double *__restrict__ w, const long *__restrict__ eoff,
                               int nm, int sb, double *__restrict__ red) {
  __shared__ double sh[RT / 32];
  const int m = blockIdx.y, b = blockIdx.x;
  const long lo = eoff[m], hi = eoff[m + 1];
  double acc[M];
#pragma unroll
  for (int l = 0; l < M; ++l) acc[l] = 0.0;
  for (long i = lo + (long)b * RT + threadIdx.x; i < hi; i += (long)sb * RT) {
    const double wi = w[i];
#pragma unroll
    for (int l = 0; l < M; ++l) acc[l] = fma(V[l * ldv + i], wi, acc[l]);
  }
#pragma unroll
  for (int l = 0; l < M; ++l) {
    const double s = block_red<0>(acc[l], sh);
    if (threadIdx.x == 0) red[((long)l * nm + m) * sb + b] = s;
  }
}

// rows 0: max |a - b|, 1: max |a| per member
__global__ void k_seg_maxdiff(const double *__restrict__ a, const double *__restrict__ bv,
                              const long *__restrict__ eoff, int nm, int sb,
                              double *__restrict__ red) {
  __shared__ double sh[RT / 32];
  const int m = blockIdx.y, b = blockIdx.x;
  const long lo = eoff[m], hi = eoff[m + 1];
  double m0 = 0.0, m1 = 0.0;
  for (long i = lo + (long)b * RT + threadIdx.x; i < hi; i += (long)sb * RT) {
    const double ai = a[i];
    m1 = fmax(m1, fabs(ai));
    m0 = fmax(m0, fabs(ai - bv[i]));
  }
  // a NaN must survive the max: fmax drops it, so flag it as +inf
  if (m0 != m0) m0 = INFINITY;
  if (m1 != m1) m1 = INFINITY;
  m0 = block_red<1>(m0, sh);
  if (threadIdx.x == 0) red[(long)m * sb + b] = m0;
  m1 = block_red<1>(m1, sh);
  if (threadIdx.x == 0) red[((long)nm + m) * sb + b] = m1;
}

// out[row] = sum (OP 0) or max (OP 1) of red[row * sb .. + sb)
template <int OP>
__global__ void k_seg_finalize(const double *__restrict__ red, int sb, double *__restrict__ out) {
  __shared__ double sh[RT / 32];
  const double *r = red + (long)blockIdx.x * sb;
  double acc = OP == 0 ? 0.0 : -1.0;
  for (int i = threadIdx.x; i < sb; i += blockDim.x) acc = OP == 0 ? acc + r[i] : fmax(acc, r[i]);
  acc = block_red<OP>(acc, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

// w[i] += sign * sum_l coef[l * nm + mem(i)] V_l[i]
__global__ void k_seg_multiaxpy(double *__restrict__ w, const double *__restrict__ V, long ldv,
                                int cols, const double *__restrict__ coef, int nm, double sign,
                                const int *__restrict__ cell_mem, int nn2, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const int m = cell_mem[i / nn2];
    double s = 0.0;
    // a zero coefficient (a member that takes no update) adds exactly nothing,
    // whatever that member's basis vectors hold
    for (int l = 0; l < cols; ++l) {
      const double cf = coef[l * nm + m];
      if (cf != 0.0) s = fma(cf, V[l * ldv + i], s);
    }
    w[i] += sign * s;
  }
}

// d[i] = coef[mem(i)] * s[i]
__global__ void k_seg_scale(double *__restrict__ d, const double *__restrict__ s,
                            const double *__restrict__ coef, const int *__restrict__ cell_mem,
                            int nn2, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
  {
    const double cf = coef[cell_mem[i / nn2]];
    d[i] = cf != 0.0 ? cf * s[i] : 0.0;  // inactive members get exact zeros
  }
}

inline int gs(long n) {
  long g = (n + 255) / 256;
  if (g > 152L * 16) g = 152L * 16;
  return (int)(g < 1 ? 1 : g);
}

void multidot_chunk(cudaStream_t st, dim3 grid, const double *V, long ldv, int m,
                    const double *w, const long *eoff, int nm, int sb, double *red) {
  switch (m) {
    case 1: k_seg_multidot<1><<<grid, RT, 0, st>>>(V, ldv, w, eoff, nm, sb, red); break;
    case 2: k_seg_multidot<2><<<grid, RT, 0, st>>>(V, ldv, w, eoff, nm, sb, red); break;
    case 3: k_seg_multidot<3><<<grid, RT, 0, st>>>(V, ldv, w, eoff, nm, sb, red); break;
    case 4: k_seg_multidot<4><<<grid, RT, 0, st>>>(V, ldv, w, eoff, nm, sb, red); break;
    case 5: k_seg_multidot<5><<<grid, RT, 0, st>>>(V, ldv, w, eoff, nm, sb, red); break;
    case 6: k_seg_multidot<6><<<grid, RT, 0, st>>>(V, ldv, w, eoff, nm, sb, red); break;
    case 7: k_seg_multidot<7><<<grid, RT, 0, st>>>(V, ldv, w, eoff, nm, sb, red); break;
    default: k_seg_multidot<8><<<grid, RT, 0, st>>>(V, ldv, w, eoff, nm, sb, red); break;
  }
  g_kernel_launches.fetch_add(1);
}
}  // namespace

// ------------------------------------------------------------ tables --
void members_free(atm_ctx &c) {
  if (!c.mem) return;
  Members &M = *c.mem;
  cudaFree(M.cell_mem);
  cudaFree(M.eoff);
  cudaFree(M.dts);
  cudaFree(M.red);
  cudaFree(M.out);
  cudaFree(M.coef);
  if (M.h_out) cudaFreeHost(M.h_out);
  if (M.h_coef) cudaFreeHost(M.h_coef);
  c.mesh.dts = nullptr;
  delete c.mem;
  c.mem = nullptr;
  mg_invalidate(c);
}

int members_refresh_dt(atm_ctx &c) {
  if (!c.mem) return ATM_OK;
  Members &M = *c.mem;
  for (int m = 0; m < M.n; ++m)
    for (int cell = M.off[m]; cell < M.off[m + 1]; ++cell) M.dts_host[cell] = M.dt[m] / c.dt;
  ATM_CUDA(cudaMemcpyAsync(M.dts, M.dts_host.data(), c.nc * sizeof(double),
                           cudaMemcpyHostToDevice, c.stream));
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  mg_invalidate(c);  // the levels carry their own copies of the multipliers
  return ATM_OK;
}

int members_set(atm_ctx &c, int n, const int *cell_off, const double *dt) {
  members_free(c);
  if (n <= 0) return ATM_OK;
  if (!cell_off || !dt) {
    set_error("atm_set_members: need the cell offsets and the time steps");
    return ATM_BAD_ARG;
  }
  if (cell_off[0] != 0 || cell_off[n] != c.nc) {
    set_error("atm_set_members: offsets must start at 0 and end at the number of cells");
    return ATM_BAD_ARG;
  }
  for (int m = 0; m < n; ++m) {
    if (cell_off[m + 1] <= cell_off[m] || !(dt[m] > 0.0)) {
      set_error("atm_set_members: member " + std::to_string(m) +
                " needs at least one cell and a positive time step");
      return ATM_BAD_ARG;
    }
  }
  // members may not share faces: every neighbour lies in the same member
  std::vector<int> nbr((size_t)c.nc * 4), mem(c.nc);
  for (int m = 0; m < n; ++m)
    for (int cell = cell_off[m]; cell < cell_off[m + 1]; ++cell) mem[cell] = m;
  ATM_CUDA(cudaMemcpyAsync(nbr.data(), c.mesh.nbr, nbr.size() * sizeof(int),
                           cudaMemcpyDeviceToHost, c.stream));
  std::vector<int> nbrf((size_t)c.nc * 4), hnb((size_t)c.mesh.nhang * 2);
  ATM_CUDA(cudaMemcpyAsync(nbrf.data(), c.mesh.nbrf, nbrf.size() * sizeof(int),
                           cudaMemcpyDeviceToHost, c.stream));
  if (c.mesh.nhang > 0)
    ATM_CUDA(cudaMemcpyAsync(hnb.data(), c.mesh.hnb, hnb.size() * sizeof(int),
                             cudaMemcpyDeviceToHost, c.stream));
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  for (int cell = 0; cell < c.nc; ++cell)
    for (int f = 0; f < 4; ++f) {
      const int nb = nbr[cell * 4 + f];
      if (nb < 0) continue;
      if ((nbrf[cell * 4 + f] >> 2) == 3) {  // coarse side of a hanging face
        for (int s = 0; s < 2; ++s)
          if (mem[hnb[2 * nb + s]] != mem[cell]) goto shared;
      } else if (mem[nb] != mem[cell]) {
        goto shared;
      }
    }
  {
    Members *M = new Members();
    c.mem = M;
    M->n = n;
    M->off.assign(cell_off, cell_off + n + 1);
    M->dt.assign(dt, dt + n);
    M->dts_host.assign(c.nc, 1.0);
    M->sb = std::max(1, std::min(64, RED_BLOCKS / n));
    std::vector<long> eo(n + 1);
    for (int m = 0; m <= n; ++m) eo[m] = (long)cell_off[m] * c.nn2;
    auto fail = [&](cudaError_t e, const char *w) {
      int rc = cuda_fail(e, w);
      members_free(c);
      return rc;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&M->cell_mem, c.nc * sizeof(int)))) return fail(e, "cudaMalloc members");
    if ((e = cudaMalloc(&M->eoff, (n + 1) * sizeof(long)))) return fail(e, "cudaMalloc members");
    if ((e = cudaMalloc(&M->dts, c.nc * sizeof(double)))) return fail(e, "cudaMalloc members");
    if ((e = cudaMalloc(&M->red, (size_t)8 * n * M->sb * sizeof(double))))
      return fail(e, "cudaMalloc members");
    if ((e = cudaMalloc(&M->out, (size_t)MEM_ROWS * n * sizeof(double))))
      return fail(e, "cudaMalloc members");
    if ((e = cudaMalloc(&M->coef, (size_t)32 * n * sizeof(double))))
      return fail(e, "cudaMalloc members");
    if ((e = cudaMallocHost(&M->h_out, (size_t)MEM_ROWS * n * sizeof(double))))
      return fail(e, "cudaMallocHost members");
    if ((e = cudaMallocHost(&M->h_coef, (size_t)32 * n * sizeof(double))))
      return fail(e, "cudaMallocHost members");
    ATM_CUDA(cudaMemcpyAsync(M->cell_mem, mem.data(), c.nc * sizeof(int), cudaMemcpyHostToDevice,
                             c.stream));
    ATM_CUDA(cudaMemcpyAsync(M->eoff, eo.data(), (n + 1) * sizeof(long), cudaMemcpyHostToDevice,
                             c.stream));
    M->status.assign(n, ATM_OK);
    M->picard.assign(n, 0);
    M->krylov.assign(n, 0);
    M->fail_step.assign(n, -1);
    M->active.assign(n, 1);
    M->last_its.assign(n, 0);
    M->last_res.assign(n, 0.0);
    c.mesh.dts = M->dts;
    return members_refresh_dt(c);
  }
shared:
  set_error("atm_set_members: a member shares a face with another member (members must be "
            "disconnected cell ranges)");
  return ATM_BAD_ARG;
}

// -------------------------------------------------- member-wise vectors --
int seg_read(atm_ctx &c, int rows) {
  Members &M = *c.mem;
  ATM_CUDA(cudaMemcpyAsync(M.h_out, M.out, (size_t)rows * M.n * sizeof(double),
                           cudaMemcpyDeviceToHost, c.stream));
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  return ATM_OK;
}

int seg_multidot(atm_ctx &c, const double *V, long ldv, int m, const double *w) {
  Members &M = *c.mem;
  const dim3 grid(M.sb, M.n);
  for (int l0 = 0; l0 < m; l0 += 8) {
    const int cols = std::min(8, m - l0);
    multidot_chunk(c.stream, grid, V + (long)l0 * ldv, ldv, cols, w, M.eoff, M.n, M.sb, M.red);
    ATM_CUDA(cudaGetLastError());
    k_seg_finalize<0><<<cols * M.n, RT, 0, c.stream>>>(M.red, M.sb, M.out + (long)l0 * M.n);
    ATM_CHECK_LAUNCH("k_seg_finalize");
  }
  return ATM_OK;
}

int seg_maxdiff(atm_ctx &c, const double *a, const double *b) {
  Members &M = *c.mem;
  k_seg_maxdiff<<<dim3(M.sb, M.n), RT, 0, c.stream>>>(a, b, M.eoff, M.n, M.sb, M.red);
  ATM_CHECK_LAUNCH("k_seg_maxdiff");
  k_seg_finalize<1><<<2 * M.n, RT, 0, c.stream>>>(M.red, M.sb, M.out);
  ATM_CHECK_LAUNCH("k_seg_finalize");
  return ATM_OK;
}

int seg_multiaxpy(atm_ctx &c, double *w, const double *V, long ldv, int cols, double sign) {
  Members &M = *c.mem;
  if (cols <= 0) return ATM_OK;
  ATM_CUDA(cudaMemcpyAsync(M.coef, M.h_coef, (size_t)cols * M.n * sizeof(double),
                           cudaMemcpyHostToDevice, c.stream));
  const long n = c.n_scalar();
  k_seg_multiaxpy<<<gs(n), 256, 0, c.stream>>>(w, V, ldv, cols, M.coef, M.n, sign, M.cell_mem,
                                               c.nn2, n);
  ATM_CHECK_LAUNCH("k_seg_multiaxpy");
  // h_coef is reused by the next call: the copy must have left it
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  return ATM_OK;
}

int seg_scale(atm_ctx &c, double *d, const double *s) {
  Members &M = *c.mem;
  ATM_CUDA(cudaMemcpyAsync(M.coef, M.h_coef, (size_t)M.n * sizeof(double),
                           cudaMemcpyHostToDevice, c.stream));
  const long n = c.n_scalar();
  k_seg_scale<<<gs(n), 256, 0, c.stream>>>(d, s, M.coef, M.cell_mem, c.nn2, n);
  ATM_CHECK_LAUNCH("k_seg_scale");
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  return ATM_OK;
}

// ------------------------------------------------------ Krylov solve --
// Member-wise restarted GMRES (precision 0: left Jacobi on diag(D), basis of
// c.restart vectors, stop on the Jacobi-scaled residual) or flexible GMRES
// right-preconditioned by the multigrid V-cycle (precision 1/2), with the
// stopping rules of gmres_schur / fgmres_mg applied to each member.
// state[m] on entry: 0 solve this member, -1 skip it; on return: ATM_OK,
// ATM_NOT_CONVERGED, ATM_NONFINITE or -1.
int krylov_members(atm_ctx &c, int precision, double *x, const double *b,
                   const std::vector<double> &tol, int maxit, std::vector<int> &state) {
  Members &M = *c.mem;
  const int nm = M.n;
  const long n = c.n_scalar();
  const bool flex = precision != 0;
  int rc;
  if (flex && (rc = mg_prepare(c, precision))) return rc;
  const int mr = flex ? mg_restart(c) : c.restart;
  double *V = c.krylov, *Z = flex ? mg_zbasis(c) : nullptr;
  double *w = c.ws1, *t = c.ws2;
  const int MR1 = mr + 1;
  std::vector<double> H((size_t)nm * MR1 * mr, 0.0), cs((size_t)nm * mr), sn((size_t)nm * mr);
  std::vector<double> g((size_t)nm * MR1), y(mr);
  std::vector<int> its(nm, 0), jend(nm, 0);
  std::vector<char> pending(nm), run(nm), cyc(nm), hit(nm);
  for (int m = 0; m < nm; ++m) {
    pending[m] = state[m] == 0;
    M.last_its[m] = 0;
  }
  double *hc = M.h_coef;
  for (;;) {
    // residual of every pending member
    if ((rc = schur_apply(c, t, x, false))) return rc;
    if (flex) {
      ATM_CUDA(cudaMemcpyAsync(V, b, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
      if ((rc = vec_axpy(c.stream, V, -1.0, t, n))) return rc;
    } else if ((rc = vec_xmy_scaled(c.stream, V, c.invdiag_D, b, t, n))) {
      return rc;
    }
    if ((rc = seg_multidot(c, V, n, 1, V)) || (rc = seg_read(c, 1))) return rc;
    bool any = false;
    for (int m = 0; m < nm; ++m) {
      run[m] = 0;
      hc[m] = 0.0;
      if (!pending[m]) continue;
      const double beta = std::sqrt(M.h_out[m]);
      M.last_res[m] = beta;
      if (!std::isfinite(beta)) {
        state[m] = ATM_NONFINITE;
        pending[m] = 0;
      } else if (beta <= tol[m]) {
        state[m] = ATM_OK;
        pending[m] = 0;
      } else if (its[m] >= maxit) {
        state[m] = ATM_NOT_CONVERGED;
        pending[m] = 0;
      } else {
        run[m] = 1;
        any = true;
        hc[m] = 1.0 / beta;
        std::fill(&g[(size_t)m * MR1], &g[(size_t)m * MR1] + MR1, 0.0);
        g[(size_t)m * MR1] = beta;
      }
    }
    if (!any) break;
    if ((rc = seg_scale(c, V, V))) return rc;
    for (int m = 0; m < nm; ++m) {
      cyc[m] = run[m];
      jend[m] = 0;
      hit[m] = 0;
    }
    for (int j = 0; j < mr; ++j) {
      double *Vj = V + (long)j * n;
      if (flex) {
        if ((rc = mg_vcycle_only(c, precision, Z + (long)j * n, Vj))) return rc;
        if ((rc = schur_apply(c, w, Z + (long)j * n, false))) return rc;
      } else if ((rc = schur_apply(c, w, Vj, true))) {
        return rc;
      }
      // classical Gram-Schmidt, twice, with member-wise coefficients
      if ((rc = seg_multidot(c, V, n, j + 1, w)) || (rc = seg_read(c, j + 1))) return rc;
      std::vector<double> h1(M.h_out, M.h_out + (size_t)(j + 1) * nm);
      for (size_t q = 0; q < h1.size(); ++q) hc[q] = h1[q];
      if ((rc = seg_multiaxpy(c, w, V, n, j + 1, -1.0))) return rc;
      if ((rc = seg_multidot(c, V, n, j + 1, w)) || (rc = seg_read(c, j + 1))) return rc;
      std::vector<double> h2(M.h_out, M.h_out + (size_t)(j + 1) * nm);
      for (size_t q = 0; q < h2.size(); ++q) hc[q] = h2[q];
      if ((rc = seg_multiaxpy(c, w, V, n, j + 1, -1.0))) return rc;
      if ((rc = seg_multidot(c, w, n, 1, w)) || (rc = seg_read(c, 1))) return rc;
      bool more = false;
      for (int m = 0; m < nm; ++m) {
        hc[m] = 0.0;
        if (!cyc[m]) continue;
        ++its[m];
        double *Hm = &H[(size_t)m * MR1 * mr], *gm = &g[(size_t)m * MR1];
        double *csm = &cs[(size_t)m * mr], *snm = &sn[(size_t)m * mr];
        for (int l = 0; l <= j; ++l) Hm[l * mr + j] = h1[(size_t)l * nm + m] + h2[(size_t)l * nm + m];
        const double hn = std::sqrt(M.h_out[m]);
        if (!std::isfinite(hn)) {  // the member fails; its x is left as it was
          state[m] = ATM_NONFINITE;
          pending[m] = 0;
          cyc[m] = 0;
          run[m] = 0;
          jend[m] = 0;
          continue;
        }
        Hm[(j + 1) * mr + j] = hn;
        for (int l = 0; l < j; ++l) {
          const double a = Hm[l * mr + j], bb = Hm[(l + 1) * mr + j];
          Hm[l * mr + j] = csm[l] * a + snm[l] * bb;
          Hm[(l + 1) * mr + j] = -snm[l] * a + csm[l] * bb;
        }
        const double a = Hm[j * mr + j], bb = Hm[(j + 1) * mr + j];
        const double r = std::sqrt(a * a + bb * bb);
        csm[j] = a / r;
        snm[j] = bb / r;
        Hm[j * mr + j] = r;
        Hm[(j + 1) * mr + j] = 0.0;
        gm[j + 1] = -snm[j] * gm[j];
        gm[j] = csm[j] * gm[j];
        jend[m] = j + 1;
        M.last_res[m] = std::fabs(gm[j + 1]);
        if (M.last_res[m] <= tol[m] || hn == 0.0 || its[m] >= maxit) {
          cyc[m] = 0;
          hit[m] = M.last_res[m] <= tol[m] || hn == 0.0;
        } else {
          hc[m] = 1.0 / hn;
          more = true;
        }
      }
      if (!more) break;
      if ((rc = seg_scale(c, V + (long)(j + 1) * n, w))) return rc;
    }
    // x += sum_l y_l V_l (or Z_l) with each member's own y
    int cols = 0;
    for (int m = 0; m < nm; ++m)
      if (run[m]) cols = std::max(cols, jend[m]);
    std::fill(hc, hc + (size_t)std::max(cols, 1) * nm, 0.0);
    for (int m = 0; m < nm; ++m) {
      if (!run[m] || jend[m] == 0) continue;
      const double *Hm = &H[(size_t)m * MR1 * mr], *gm = &g[(size_t)m * MR1];
      for (int l = jend[m] - 1; l >= 0; --l) {
        double s = gm[l];
        for (int q = l + 1; q < jend[m]; ++q) s -= Hm[l * mr + q] * y[q];
        y[l] = s / Hm[l * mr + l];
      }
      for (int l = 0; l < jend[m]; ++l) hc[(size_t)l * nm + m] = y[l];
    }
    if ((rc = seg_multiaxpy(c, x, flex ? Z : V, n, cols, 1.0))) return rc;
    // without the true-residual check a cycle that met its stop ends the
    // member's solve (as in the solo solvers); with it the restart decides
    if (!c.true_residual_check)
      for (int m = 0; m < nm; ++m)
        if (run[m] && pending[m] && (hit[m] || its[m] >= maxit)) {
          state[m] = hit[m] ? ATM_OK : ATM_NOT_CONVERGED;
          pending[m] = 0;
        }
  }
  for (int m = 0; m < nm; ++m) {
    M.last_its[m] = its[m];
    M.krylov[m] += its[m];
  }
  return ATM_OK;
}

}  // namespace atm
