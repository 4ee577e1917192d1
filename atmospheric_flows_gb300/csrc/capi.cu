// C ABI (include/atm_gb300.h).  Validation, ownership and error mapping;
// the numerical work lives in the kernel and solver translation units.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "atm_internal.h"

namespace atm {
std::atomic<long> g_kernel_launches{0};

TimedRegion::TimedRegion(const atm_ctx &ctx, int family, double bytes, double flops)
    : c(ctx), slot(0), on(ctx.timer.on && !ctx.capturing) {
  if (!on) return;
  KTimer &t = c.timer;
  if (t.used * 2 + 2 > t.ev.size()) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
      on = false;
      return;
    }
    t.ev.push_back(a);
    t.ev.push_back(b);
    t.fam.push_back(family);
    t.bytes.push_back(0.0);
    t.flops.push_back(0.0);
  }
  slot = t.used++;
  t.fam[slot] = family;
  t.bytes[slot] = bytes;
  t.flops[slot] = flops;
  cudaEventRecord(t.ev[2 * slot], c.stream);
}
TimedRegion::~TimedRegion() {
  if (on) cudaEventRecord(c.timer.ev[2 * slot + 1], c.stream);
}

static thread_local std::string g_err = "";
void set_error(const std::string &msg) { g_err = msg; }
int cuda_fail(cudaError_t e, const char *where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? ATM_OOM : ATM_CUDA_ERROR;
}
}  // namespace atm

using namespace atm;

#define CHECK_H(h)                                   \
  do {                                               \
    if (!(h)) {                                      \
      set_error("null handle");                      \
      return ATM_BAD_ARG;                            \
    }                                                \
  } while (0)
#define CHECK_PTR(p, name)                           \
  do {                                               \
    if (!(p)) {                                      \
      set_error(std::string("null pointer: ") + name); \
      return ATM_BAD_ARG;                            \
    }                                                \
  } while (0)

extern "C" {

const char *atm_last_error(void) { return g_err.c_str(); }
const char *atm_version(void) { return "atm_gb300 0.1 (sm_103a, FP64 IMEX-DG, dim 2, k 1-5)"; }

static void ctx_free(atm_ctx *c) {
  if (!c) return;
  if (c->solver) {
    solver_free(*c->solver);
    delete c->solver;
  }
  mesh_free(c->mesh);
  cudaFree(c->rho_fix);
  cudaFree(c->pres_fix);
  cudaFree(c->pfq);
  cudaFree(c->pff);
  cudaFree(c->u_fix);
  cudaFree(c->ainv);
  cudaFree(c->invdiag_D);
  cudaFree(c->wv1);
  cudaFree(c->wv2);
  cudaFree(c->ws1);
  cudaFree(c->ws2);
  cudaFree(c->red);
  cudaFree(c->red_out);
  cudaFree(c->krylov);
  cudaFree(c->dsmall);
  if (c->h_red) cudaFreeHost(c->h_red);
  members_free(*c);
  mg_free(*c);
  for (cudaEvent_t e : c->timer.ev) cudaEventDestroy(e);
  delete c;
}

int atm_check_mesh(int degree, int n_cells, int mapping_degree, const double *mapping_nodes,
                   int n_inner, const int *inner_faces, int n_bdry, const int *bdry_faces,
                   int *n_hanging) {
  if (degree < 1 || degree > KMAX) { set_error("degree must be in 1..5"); return ATM_BAD_ARG; }
  if (n_cells < 1 || n_inner < 0 || n_bdry < 0) { set_error("bad sizes"); return ATM_BAD_ARG; }
  HostMesh hm;
  const int rc = build_mesh_tables(degree, n_cells, mapping_degree, mapping_nodes, n_inner,
                                   inner_faces, n_bdry, bdry_faces, hm);
  if (rc == ATM_OK && n_hanging) *n_hanging = hm.nhang;
  return rc;
}

int atm_ctx_create(int dim, int degree, int n_cells, int mapping_degree,
                   const double *mapping_nodes, int n_inner, const int *inner_faces,
                   int n_bdry, const int *bdry_faces, atm_handle *out) {
  CHECK_PTR(out, "out");
  *out = nullptr;
  if (dim != 2) { set_error("only dim = 2 is supported"); return ATM_BAD_ARG; }
  if (degree < 1 || degree > KMAX) { set_error("degree must be in 1..5"); return ATM_BAD_ARG; }
  if (n_cells < 1 || n_inner < 0 || n_bdry < 0) { set_error("bad sizes"); return ATM_BAD_ARG; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    set_error("no CUDA device: the GB300 operator library has no CPU path");
    return ATM_CUDA_ERROR;
  }
  atm_ctx *c = new (std::nothrow) atm_ctx();
  if (!c) { set_error("host allocation failed"); return ATM_OOM; }
  cudaGetDevice(&c->device);
  c->k = degree; c->nn = degree + 1; c->nq = 2 * degree + 1;
  c->nn2 = c->nn * c->nn; c->nq2 = c->nq * c->nq; c->nc = n_cells;
  c->tab = Tableau::make();
  int rc = upload_basis_all();
  auto fail = [&](int r) { ctx_free(c); return r; };
  if (rc) return fail(rc);
  const long ns = c->n_scalar(), nv = c->n_vector();
  const size_t blk = (size_t)n_cells * c->nn2 * c->nn2;
#define ALLOC(ptr, n)                                                          \
  do {                                                                         \
    cudaError_t e = cudaMalloc(&(ptr), (size_t)(n) * sizeof(double));          \
    if (e != cudaSuccess) return fail(cuda_fail(e, "cudaMalloc " #ptr));       \
    cudaMemsetAsync((ptr), 0, (size_t)(n) * sizeof(double), c->stream);         \
  } while (0)
  ALLOC(c->rho_fix, ns);
  ALLOC(c->pres_fix, ns);
  ALLOC(c->pfq, (long)n_cells * c->nq2);
  ALLOC(c->pff, (long)n_cells * 4 * c->nq);
  ALLOC(c->u_fix, nv);
  ALLOC(c->ainv, blk);
  ALLOC(c->invdiag_D, ns);
  ALLOC(c->wv1, nv);
  ALLOC(c->wv2, nv);
  ALLOC(c->ws1, ns);
  ALLOC(c->ws2, ns);
  ALLOC(c->red, 32 * RED_BLOCKS);
  ALLOC(c->red_out, 64);
  ALLOC(c->krylov, (size_t)(c->restart + 1) * ns);
  ALLOC(c->dsmall, 256);
#undef ALLOC
  if (cudaMallocHost(&c->h_red, 256 * sizeof(double)) != cudaSuccess)
    return fail(cuda_fail(cudaErrorMemoryAllocation, "cudaMallocHost"));
  rc = mesh_upload(*c, mapping_degree, mapping_nodes, n_inner, inner_faces, n_bdry, bdry_faces);
  if (rc) return fail(rc);
  *out = c;
  return ATM_OK;
}

int atm_ctx_destroy(atm_handle h) {
  if (h) {
    cudaStreamSynchronize(h->stream);
    ctx_free(h);
  }
  return ATM_OK;
}

int atm_upload_mesh(atm_handle h, int mapping_degree, const double *mapping_nodes, int n_inner,
                    const int *inner_faces, int n_bdry, const int *bdry_faces) {
  CHECK_H(h);
  // a multigrid hierarchy built on the old mesh no longer matches
  mg_free(*h);
  return mesh_upload(*h, mapping_degree, mapping_nodes, n_inner, inner_faces, n_bdry,
                     bdry_faces);
}

int atm_set_stream(atm_handle h, void *stream) {
  CHECK_H(h);
  h->stream = static_cast<cudaStream_t>(stream);
  return ATM_OK;
}
int atm_stream_create(void **out) {
  CHECK_PTR(out, "out");
  cudaStream_t s = nullptr;
  ATM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *out = s;
  return ATM_OK;
}
int atm_stream_destroy(void *stream) {
  if (stream) ATM_CUDA(cudaStreamDestroy(static_cast<cudaStream_t>(stream)));
  return ATM_OK;
}
int atm_device_memory(double *free_bytes, double *total_bytes) {
  size_t f = 0, t = 0;
  ATM_CUDA(cudaMemGetInfo(&f, &t));
  if (free_bytes) *free_bytes = (double)f;
  if (total_bytes) *total_bytes = (double)t;
  return ATM_OK;
}
int atm_synchronize(atm_handle h) {
  CHECK_H(h);
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  return ATM_OK;
}
long atm_n_scalar(atm_handle h) { return h ? h->n_scalar() : -1; }

long atm_kernel_launches(void) { return g_kernel_launches.load(); }

int atm_timing_enable(atm_handle h, int on) {
  CHECK_H(h);
  h->timer.on = on != 0;
  return ATM_OK;
}

int atm_timing_read(atm_handle h, double *ms, long *launches, double *bytes, double *flops,
                    int n) {
  CHECK_H(h);
  KTimer &t = h->timer;
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  for (size_t i = 0; i < t.used; ++i) {
    float e = 0.0f;
    ATM_CUDA(cudaEventElapsedTime(&e, t.ev[2 * i], t.ev[2 * i + 1]));
    t.ms[t.fam[i]] += e;
    t.n[t.fam[i]] += 1;
    t.tb[t.fam[i]] += t.bytes[i];
    t.tf[t.fam[i]] += t.flops[i];
  }
  t.used = 0;
  for (int i = 0; i < n && i < KF_COUNT; ++i) {
    if (ms) ms[i] = t.ms[i];
    if (launches) launches[i] = t.n[i];
    if (bytes) bytes[i] = t.tb[i];
    if (flops) flops[i] = t.tf[i];
    t.ms[i] = 0.0;
    t.n[i] = 0;
    t.tb[i] = 0.0;
    t.tf[i] = 0.0;
  }
  return ATM_OK;
}

int atm_set_dt(atm_handle h, double dt) {
  CHECK_H(h);
  if (!(dt > 0.0)) { set_error("dt must be positive"); return ATM_BAD_ARG; }
  h->dt = dt;
  return members_refresh_dt(*h);
}
int atm_set_mach(atm_handle h, double v) {
  CHECK_H(h);
  if (!(v > 0.0)) { set_error("Mach must be positive"); return ATM_BAD_ARG; }
  h->Ma = v;
  return ATM_OK;
}
int atm_set_froude(atm_handle h, double v) {
  CHECK_H(h);
  if (!(v > 0.0)) { set_error("Froude must be positive"); return ATM_BAD_ARG; }
  h->Fr = v;
  return ATM_OK;
}
int atm_set_hyperbolic_stage(atm_handle h, int stage) {
  CHECK_H(h);
  if (stage < 1 || stage > 3) { set_error("IMEX stage must be 1..3"); return ATM_BAD_ARG; }
  h->hstage = stage;
  return ATM_OK;
}
int atm_set_ns_stage(atm_handle h, int stage) {
  CHECK_H(h);
  if (stage < 1 || stage > 6) { set_error("NS stage must be 1..6"); return ATM_BAD_ARG; }
  h->nsstage = stage;
  return ATM_OK;
}

int atm_set_rho_for_fixed(atm_handle h, const double *rho) {
  CHECK_H(h);
  CHECK_PTR(rho, "rho");
  int rc = vec_copy(h->stream, h->rho_fix, rho, h->n_scalar());
  if (rc) return rc;
  return rebuild_ainv(*h);
}
int atm_set_pres_fixed(atm_handle h, const double *p) {
  CHECK_H(h);
  CHECK_PTR(p, "pres");
  int rc = vec_copy(h->stream, h->pres_fix, p, h->n_scalar());
  return rc ? rc : launch_pfix_prep(*h);
}
int atm_set_u_fixed(atm_handle h, const double *u) {
  CHECK_H(h);
  CHECK_PTR(u, "u");
  return vec_copy(h->stream, h->u_fix, u, h->n_vector());
}

static int check_src(const double *const *src, int nsrc, int expect) {
  if (!src || nsrc != expect) {
    set_error("source list must have " + std::to_string(expect) + " entries for this stage");
    return ATM_BAD_ARG;
  }
  for (int i = 0; i < nsrc; ++i)
    if (!src[i]) { set_error("null source vector " + std::to_string(i)); return ATM_BAD_ARG; }
  return ATM_OK;
}

int atm_vmult_rhs_rho_update(atm_handle h, double *dst, const double *const *src, int nsrc) {
  CHECK_H(h);
  CHECK_PTR(dst, "dst");
  const int expect[3] = {2, 4, 6};
  if (int rc = check_src(src, nsrc, expect[h->hstage - 1])) return rc;
  return launch_rhs_rho(*h, h->hstage, dst, src, stage_coef_rho(*h, h->hstage));
}
int atm_vmult_rhs_velocity_fixed(atm_handle h, double *dst, const double *const *src, int nsrc) {
  CHECK_H(h);
  CHECK_PTR(dst, "dst");
  const int expect[3] = {4, 7, 9};
  if (int rc = check_src(src, nsrc, expect[h->hstage - 1])) return rc;
  return launch_rhs_vel(*h, h->hstage, dst, src, stage_coef_flux(*h, h->hstage));
}
int atm_vmult_rhs_pressure(atm_handle h, double *dst, const double *const *src, int nsrc) {
  CHECK_H(h);
  CHECK_PTR(dst, "dst");
  const int expect[3] = {5, 8, 11};
  if (int rc = check_src(src, nsrc, expect[h->hstage - 1])) return rc;
  return launch_rhs_pres(*h, h->hstage, dst, src, stage_coef_flux(*h, h->hstage));
}

int atm_vmult_pressure(atm_handle h, double *dst, const double *src) {
  CHECK_H(h);
  CHECK_PTR(dst, "dst");
  CHECK_PTR(src, "src");
  const double co = implicit_coeff(*h);
  return launch_B(*h, dst, src, co * h->dt / (h->Ma * h->Ma), 0);
}
int atm_vmult_enthalpy(atm_handle h, double *dst, const double *src) {
  CHECK_H(h);
  CHECK_PTR(dst, "dst");
  CHECK_PTR(src, "src");
  return launch_CD(*h, dst, src, nullptr, implicit_coeff(*h) * h->dt, 0);
}
int atm_vmult(atm_handle h, double *dst, const double *src) {
  CHECK_H(h);
  CHECK_PTR(dst, "dst");
  CHECK_PTR(src, "src");
  return op_vmult(*h, dst, src);
}
int atm_diagonal_inverse(atm_handle h, double *dst) {
  CHECK_H(h);
  CHECK_PTR(dst, "dst");
  switch (h->nsstage) {
    case 1:
    case 4: return launch_inv_diag(*h, dst, 1, nullptr, 1.0);
    case 2:
    case 6: return launch_inv_diag(*h, dst, 1, nullptr, 1.0 / (GAS_GAMMA - 1.0));
    default: return launch_inv_diag(*h, dst, 2, h->rho_fix, 1.0);
  }
}
int atm_solve(atm_handle h, double *x, const double *b, double tol, int maxit, int *iters,
              double *res) {
  CHECK_H(h);
  CHECK_PTR(x, "x");
  CHECK_PTR(b, "b");
  if (maxit < 0 || !(tol >= 0.0)) { set_error("bad tolerance or maxit"); return ATM_BAD_ARG; }
  return op_solve(*h, x, b, tol, maxit, iters, res);
}

// ------------------------------------------------------------- multigrid --
int atm_mg_add_level(atm_handle h, int n_cells, int mapping_degree, const double *mapping_nodes,
                     int n_inner, const int *inner_faces, int n_bdry, const int *bdry_faces,
                     const int *children) {
  CHECK_H(h);
  return mg_add_level(*h, n_cells, mapping_degree, mapping_nodes, n_inner, inner_faces, n_bdry,
                      bdry_faces, children);
}
int atm_mg_set_smoother(atm_handle h, int degree, double smoothing_range, int eig_iterations,
                        int coarse_degree) {
  CHECK_H(h);
  return mg_set_params(*h, degree, smoothing_range, eig_iterations, coarse_degree);
}
int atm_mg_vcycle(atm_handle h, int precision, double *dst, const double *src) {
  CHECK_H(h);
  CHECK_PTR(dst, "dst");
  CHECK_PTR(src, "src");
  if (precision != 1 && precision != 2) { set_error("precision must be 1 or 2"); return ATM_BAD_ARG; }
  return mg_precondition(*h, precision, dst, src);
}
int atm_set_autotune(atm_handle h, int on) {
  CHECK_H(h);
  h->autotune = on != 0;
  return ATM_OK;
}
int atm_autotune_table(int *out, int max_entries) {
  if (max_entries < 0) {
    set_error("atm_autotune_table: max_entries < 0");
    return ATM_BAD_ARG;
  }
  return tune_table(out, max_entries);
}
int atm_mg_set_graphs(atm_handle h, int on) {
  CHECK_H(h);
  return mg_set_graphs(*h, on != 0);
}
int atm_mg_stats(atm_handle h, long *out) {
  CHECK_H(h);
  CHECK_PTR(out, "out");
  mg_stats(*h, out);
  return ATM_OK;
}
int atm_set_true_residual_check(atm_handle h, int on) {
  CHECK_H(h);
  h->true_residual_check = on != 0;
  return ATM_OK;
}
int atm_solve_fgmres(atm_handle h, int precision, double *x, const double *b, double tol,
                     int maxit, int *iters, double *res) {
  CHECK_H(h);
  CHECK_PTR(x, "x");
  CHECK_PTR(b, "b");
  if (maxit < 0 || !(tol >= 0.0)) { set_error("bad tolerance or maxit"); return ATM_BAD_ARG; }
  int it = 0;
  double r = 0.0;
  int rc = fgmres_mg(*h, precision, x, b, tol, maxit, &it, &r);
  if (iters) *iters = it;
  if (res) *res = r;
  return rc;
}

// ----------------------------------------------------------------- solver --
int atm_solver_init(atm_handle h, double dt, double mach, double froude, double eps,
                    int max_its, int precision) {
  CHECK_H(h);
  if (!(dt > 0.0) || !(mach > 0.0) || !(froude > 0.0) || !(eps > 0.0) || max_its < 1) {
    set_error("atm_solver_init: dt, Mach, Froude, eps must be positive, max_its >= 1");
    return ATM_BAD_ARG;
  }
  if (precision < 0 || precision > 2) {
    set_error("atm_solver_init: precision must be 0 (GMRES + Jacobi), 1 (FGMRES + FP32 "
              "multigrid) or 2 (FGMRES + FP64 multigrid)");
    return ATM_BAD_ARG;
  }
  if (precision > 0 && mg_levels(*h) < 2) {
    set_error("atm_solver_init: precision 1/2 needs multigrid levels (atm_mg_add_level)");
    return ATM_NOT_READY;
  }
  if (h->solver) {
    solver_free(*h->solver);
    delete h->solver;
    h->solver = nullptr;
  }
  Solver *s = new (std::nothrow) Solver();
  if (!s) { set_error("host allocation failed"); return ATM_OOM; }
  int rc = solver_alloc(*h, *s);
  if (rc) { delete s; return rc; }
  h->solver = s;
  s->eps = eps;
  s->max_its = max_its;
  s->precision = precision;
  h->dt = dt; h->Ma = mach; h->Fr = froude;
  return members_refresh_dt(*h);
}

#define CHECK_S(h)                                             \
  do {                                                         \
    CHECK_H(h);                                                \
    if (!(h)->solver) {                                        \
      set_error("solver not initialised (atm_solver_init)");   \
      return ATM_NOT_READY;                                    \
    }                                                          \
  } while (0)

static int state_copy(atm_handle h, double *rho, double *u, double *p, const double *rs,
                      const double *us, const double *ps, cudaMemcpyKind kind) {
  const size_t ns = h->n_scalar() * sizeof(double), nv = h->n_vector() * sizeof(double);
  ATM_CUDA(cudaMemcpyAsync(rho, rs, ns, kind, h->stream));
  ATM_CUDA(cudaMemcpyAsync(u, us, nv, kind, h->stream));
  ATM_CUDA(cudaMemcpyAsync(p, ps, ns, kind, h->stream));
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  return ATM_OK;
}

int atm_solver_set_state(atm_handle h, const double *rho, const double *u, const double *p) {
  CHECK_S(h);
  CHECK_PTR(rho, "rho"); CHECK_PTR(u, "u"); CHECK_PTR(p, "p");
  Solver &v = *h->solver;
  return state_copy(h, v.rho_old, v.u_old, v.pres_old, rho, u, p, cudaMemcpyHostToDevice);
}
int atm_solver_get_state(atm_handle h, double *rho, double *u, double *p) {
  CHECK_S(h);
  CHECK_PTR(rho, "rho"); CHECK_PTR(u, "u"); CHECK_PTR(p, "p");
  Solver &v = *h->solver;
  return state_copy(h, rho, u, p, v.rho_old, v.u_old, v.pres_old, cudaMemcpyDeviceToHost);
}
int atm_solver_set_state_device(atm_handle h, const double *rho, const double *u,
                                const double *p) {
  CHECK_S(h);
  CHECK_PTR(rho, "rho"); CHECK_PTR(u, "u"); CHECK_PTR(p, "p");
  Solver &v = *h->solver;
  return state_copy(h, v.rho_old, v.u_old, v.pres_old, rho, u, p, cudaMemcpyDeviceToDevice);
}
int atm_solver_get_state_device(atm_handle h, double *rho, double *u, double *p) {
  CHECK_S(h);
  CHECK_PTR(rho, "rho"); CHECK_PTR(u, "u"); CHECK_PTR(p, "p");
  Solver &v = *h->solver;
  return state_copy(h, rho, u, p, v.rho_old, v.u_old, v.pres_old, cudaMemcpyDeviceToDevice);
}
int atm_solver_set_sponge(atm_handle h, const double *alpha, double ubg_x, double ubg_z) {
  CHECK_S(h);
  Solver &v = *h->solver;
  if (!alpha) { v.sponge = false; return ATM_OK; }
  ATM_CUDA(cudaMemcpyAsync(v.alpha, alpha, h->n_scalar() * sizeof(double),
                           cudaMemcpyHostToDevice, h->stream));
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  v.sponge = true;
  v.ubg0 = ubg_x;
  v.ubg1 = ubg_z;
  return ATM_OK;
}
int atm_solver_set_sponge_target(atm_handle h, const double *u_target) {
  CHECK_S(h);
  Solver &v = *h->solver;
  if (!u_target) {
    cudaFree(v.sponge_target);
    v.sponge_target = nullptr;
    return ATM_OK;
  }
  const size_t n = h->n_vector() * sizeof(double);
  if (!v.sponge_target) ATM_CUDA(cudaMalloc(&v.sponge_target, n));
  ATM_CUDA(cudaMemcpyAsync(v.sponge_target, u_target, n, cudaMemcpyHostToDevice, h->stream));
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  return ATM_OK;
}
int atm_solver_set_clock(atm_handle h, double time, long steps) {
  CHECK_S(h);
  if (steps < 0 || !(time >= 0.0)) { set_error("time and steps must be >= 0"); return ATM_BAD_ARG; }
  h->solver->time = time;
  h->solver->steps = steps;
  return ATM_OK;
}
int atm_solver_set_continue_on_not_converged(atm_handle h, int on) {
  CHECK_S(h);
  h->solver->continue_on_not_converged = on != 0;
  return ATM_OK;
}
int atm_solver_run(atm_handle h, int n_steps) {
  CHECK_S(h);
  if (n_steps < 0) { set_error("n_steps must be >= 0"); return ATM_BAD_ARG; }
  for (int i = 0; i < n_steps; ++i) {
    int rc = solver_step(*h, *h->solver);
    if (rc) return rc;
  }
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  ATM_CUDA(cudaGetLastError());
  return ATM_OK;
}
int atm_set_members(atm_handle h, int n_members, const int *cell_offsets,
                    const double *member_dt) {
  CHECK_H(h);
  if (n_members < 0 || n_members == 1) {
    set_error("atm_set_members: n_members must be 0 (one member) or >= 2");
    return ATM_BAD_ARG;
  }
  return members_set(*h, n_members, cell_offsets, member_dt);
}
int atm_member_stats(atm_handle h, int n, double *out) {
  CHECK_H(h);
  CHECK_PTR(out, "out");
  if (!h->mem || n != h->mem->n) {
    set_error("atm_member_stats: n must equal the number of members (atm_set_members)");
    return ATM_BAD_ARG;
  }
  const Members &M = *h->mem;
  for (int m = 0; m < n; ++m) {
    double *o = out + 5 * m;
    o[0] = M.status[m];
    o[1] = (double)M.picard[m];
    o[2] = (double)M.krylov[m];
    o[3] = (double)M.fail_step[m];
    o[4] = M.dt[m];
  }
  return ATM_OK;
}
int atm_solver_stats(atm_handle h, double *st) {
  CHECK_S(h);
  CHECK_PTR(st, "stats");
  Solver &v = *h->solver;
  st[0] = (double)v.steps;
  st[1] = (double)v.picard_total;
  st[2] = (double)v.krylov_total;
  st[3] = v.last_picard[0];
  st[4] = v.last_picard[1];
  st[5] = (double)v.failures;
  st[6] = v.time;
  st[7] = h->dt;
  st[8] = (double)mg_vcycles(*h);
  return ATM_OK;
}
int atm_solver_diagnostics(atm_handle h, double *out) {
  CHECK_S(h);
  CHECK_PTR(out, "out");
  return solver_diagnostics(*h, *h->solver, out);
}

}  // extern "C"
