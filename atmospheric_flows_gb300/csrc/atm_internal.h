// Internal declarations shared by the host and device translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <functional>
#include <vector>

#include "../../include/atm_gb300.h"

namespace atm {

constexpr int KMAX = 5;           // highest supported polynomial degree
constexpr int NQ_MAX = 2 * KMAX + 1;
constexpr int NN_MAX = KMAX + 1;
constexpr double GAS_GAMMA = 1.4;  // EquationData::Cp_Cv (equation_data.h:23)

// IMEX ARK2 tableau, euler_operator.h:220-240
struct Tableau {
  double gamma, a21, a22, a31, a32, a33;
  double a21t, a22t, a31t, a32t, a33t, b1, b2, b3;
  static Tableau make();
};

// Per-stage weights handed to the explicit-operator kernels.
struct Solver;
struct MG;
struct Members;

struct StageCoef {
  double ca[3];  // explicit advection weights (a / b)
  double ct[3];  // pressure / enthalpy weights (a~ / b)
  double cg[3];  // gravity weights (a~ / b)
  double dt, Ma, Fr;
};


// Kernel families timed by the optional per-launch CUDA-event timers.
enum KFam {
  KF_RHS_RHO = 0, KF_RHS_VEL, KF_RHS_PRES, KF_B, KF_CD, KF_MASS, KF_DIAG, KF_BLOCK_INV,
  KF_BLOCK_APPLY, KF_MG_APPLY, KF_MG_OTHER, KF_PFIX_PREP, KF_COUNT
};

// CUDA-event timers around operator launches (off unless enabled).
struct KTimer {
  bool on = false;
  std::vector<cudaEvent_t> ev;  // pairs (start, stop)
  std::vector<int> fam;         // family of each pair
  size_t used = 0;              // pairs recorded since the last read
  std::vector<double> bytes, flops;  // algorithmic bytes / FP64 flops per pair
  double ms[KF_COUNT] = {0};
  long n[KF_COUNT] = {0};
  double tb[KF_COUNT] = {0}, tf[KF_COUNT] = {0};
};

// Every kernel launch of the library increments this counter.
extern std::atomic<long> g_kernel_launches;

// Device geometry + connectivity of one mesh (T = double for the operator,
// float for the multigrid levels of the mixed-precision preconditioner).
template <typename T>
struct MeshT {
  int nc = 0, k = 0, nn = 0, nq = 0, nn2 = 0, nq2 = 0;
  T *qgeo = nullptr;   // [nc][5][nq2]: dxi/dx*JxW, dxi/dz*JxW, deta/dx*JxW, deta/dz*JxW, JxW
  T *fgeo = nullptr;   // [nc][4][3][nq]: n_x, n_z, JxW (own-side, outward)
  int *nbr = nullptr;  // [nc][4] neighbour cell, -1 at a wall (hanging index h, code 3)
  int *nbrf = nullptr; // [nc][4] neighbour's local face | code << 2 (see below)
  T *minv = nullptr;   // [nc][nn2*nn2] inverse unit mass, stored transposed
  // Hanging faces of 2:1 adaptive meshes.  Code of a cell face (nbrf >> 2):
  //   0 conforming; 1, 2: this cell is the fine side and its face is subface
  //   code-1 of the neighbour's face; 3: this cell is the coarse side, nbr
  //   holds the hanging-face index h, hnb[2h+s] is the fine neighbour on
  //   subface s and hgeo[2h+s][3][nq] the subface geometry (n_x, n_z, JxW)
  //   seen from this cell at the points (gauss_q + s)/2 of its face.
  int nhang = 0;
  int *hnb = nullptr;
  T *hgeo = nullptr;
  // [nc] per-cell multiplier of the time step (null: 1).  A context that
  // holds several members gives each member's cells dt_member / dt, so
  // every dt-weighted term (stage fluxes, gravity, B, C, sponge) uses the
  // member's own step; members share no faces, so a row scale is exact.
  T *dts = nullptr;
  // [nc][3][3][2] the mapping at degree 2: (x, z) at the reference points
  // (xi, eta) in {0, 1/2, 1}^2, eta slowest.  Exact for mapping degree <= 2,
  // its interpolant otherwise.  The FP32 multigrid levels form their
  // quadrature-point geometry from it in the Schur kernels instead of
  // reading qgeo (null on the FP64 operator mesh).
  T *map2 = nullptr;
};
using Mesh = MeshT<double>;

}  // namespace atm

struct atm_ctx {
  int device = 0;
  int k = 0, nn = 0, nq = 0, nn2 = 0, nq2 = 0, nc = 0, mapdeg = 0;
  cudaStream_t stream = nullptr;
  atm::Mesh mesh;
  double dt = 1.0, Ma = 1.0, Fr = 1.0;
  int hstage = 1, nsstage = 1;
  atm::Tableau tab;
  // frozen fields (owned copies) and derived data
  double *rho_fix = nullptr, *pres_fix = nullptr, *u_fix = nullptr;
  double *pfq = nullptr, *pff = nullptr;  // p_fix at quadrature points / face traces
  double *ainv = nullptr;       // [nc][nn2*nn2] inverse of rho_fix-weighted mass
  double *invdiag_D = nullptr;  // inverse diagonal of D (Schur Jacobi)
  // workspace
  double *wv1 = nullptr, *wv2 = nullptr;  // velocity-sized
  double *ws1 = nullptr, *ws2 = nullptr;  // scalar-sized
  double *red = nullptr;                  // reduction partials (device)
  double *red_out = nullptr;              // reduction results (device)
  double *h_red = nullptr;                // pinned host mirror of red_out
  // GMRES basis (restart+1 scalar vectors) + small device arrays
  int restart = 28;
  double *krylov = nullptr;
  double *dsmall = nullptr;  // device scratch for Hessenberg columns / y
  atm::Solver *solver = nullptr;
  atm::MG *mg = nullptr;  // multigrid hierarchy of the FGMRES Schur solves
  atm::Members *mem = nullptr;  // several independent members in one context
  // GMRES/FGMRES only stop on a recomputed true residual (S is nonlinear)
  bool true_residual_check = false;
  bool autotune = true;  // choose the face kernels' cells per block by timing
  mutable atm::KTimer timer;
  bool capturing = false;  // a CUDA graph is being recorded: timers are off
  // device address of the static Schur scratch array in this handle's
  // context (atm_schur_vmult_static_scratch; looked up on first use)
  void *static_scratch = nullptr;
  // host copy of the operator mesh's mapping at degree 2 (MeshT::map2
  // layout): the geometry of the FP32 multigrid level 0
  std::vector<double> map2;
  long n_scalar() const { return (long)nc * nn2; }
  long n_vector() const { return 2L * nc * nn2; }
};

namespace atm {

// ------------------------------------------------------------------ errors --
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *where);
#define ATM_CUDA(call)                                        \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return atm::cuda_fail(_e, #call);  \
  } while (0)
#define ATM_CHECK_LAUNCH(where)                       \
  do {                                                \
    atm::g_kernel_launches.fetch_add(1);              \
    ATM_CUDA(cudaGetLastError());                     \
  } while (0)

// RAII: records a (start, stop) event pair around the launches in scope
struct TimedRegion {
  const atm_ctx &c;
  size_t slot;
  bool on;
  // bytes: algorithmic HBM bytes of the launch (fields read + written, 8 B
  // per node value); flops: FP64 flops of its sum-factorisation contractions
  TimedRegion(const atm_ctx &ctx, int family, double bytes = 0.0, double flops = 0.0);
  ~TimedRegion();
};

// ------------------------------------------------------------------ basis --
// Host tables: S[q*nn+i] = l_i(x_q), D[q*nn+i] = l_i'(x_q) on Gauss points.
struct HostBasis {
  int k, nn, nq;
  std::vector<double> gll, gauss, weights, S, D;
};
HostBasis make_basis(int k);
std::vector<double> gll_nodes(int k);
void lagrange_eval(const std::vector<double> &nodes, double x, double *val, double *der);
// upload S/D tables of every degree to each translation unit's constant bank
int upload_basis_all();

// --------------------------------------------------------- kernel launches --
// every launcher returns ATM_OK or an error status, and runs on `st`
int launch_rhs_rho(const atm_ctx &c, int stage, double *dst, const double *const *src,
                   const StageCoef &co);
int launch_rhs_vel(const atm_ctx &c, int stage, double *dst, const double *const *src,
                   const StageCoef &co);
int launch_rhs_pres(const atm_ctx &c, int stage, double *dst, const double *const *src,
                    const StageCoef &co);
// B p -> dst (velocity); mode 0: dst = B p; 1: dst -= B p;
// 2: dst = A^{-1} B p (uses c.ainv)
int launch_B(const atm_ctx &c, double *dst, const double *p, double coeff, int mode);
// C/D family on pressure space:
//   mode 0: dst = C w
//   mode 1: dst = sD*D p - C w
//   mode 2: dst = invdiag .* (sD*D p - C w)
//   mode 3: dst -= C w
// (C uses the context's frozen p_fix, prepared by launch_pfix_prep)
int launch_CD(const atm_ctx &c, double *dst, const double *w, const double *p, double coeff,
              int mode);
// values of p_fix at the quadrature points and its face traces (after every
// change of p_fix)
int launch_pfix_prep(const atm_ctx &c);
// matrix-free mass apply: dst = M_w src, weight = tile field or constant scale
int launch_mass(const atm_ctx &c, double *dst, const double *src, int ncomp,
                const double *weight, double scale);
// inverse diagonal of the (weighted) mass: out for ncomp components
int launch_inv_diag(const atm_ctx &c, double *out, int ncomp, const double *weight,
                    double scale);
// build per-cell inverse of the weighted mass (weight null -> unit), transposed
int launch_block_inverse(const atm_ctx &c, double *out, const double *weight);
// dst = scale * Binv src, ncomp components per cell
int launch_block_apply(const atm_ctx &c, double *dst, const double *src, const double *binv,
                       int ncomp, double scale);

// ----------------------------------------------------------- vector ops ---
// All run on `st`, deterministic two-pass reductions.
int vec_copy(cudaStream_t st, double *dst, const double *src, long n);
int vec_fill(cudaStream_t st, double *dst, double v, long n);
int vec_axpy(cudaStream_t st, double *y, double a, const double *x, long n);  // y += a x
int vec_xmy_scaled(cudaStream_t st, double *dst, const double *d, const double *b,
                   const double *t, long n);  // dst = d .* (b - t)
int vec_scale_by_inv_norm(cudaStream_t st, double *dst, const double *src,
                          const double *normsq, long n);  // dst = src/sqrt(*normsq)
// partial-sum buffer `red` must hold 29*RED_BLOCKS doubles
constexpr int RED_BLOCKS = 608;
int vec_dot(cudaStream_t st, const double *x, const double *y, long n, double *red,
            double *out);  // out[0] = x.y (device)
// One Arnoldi orthogonalisation of the new direction w against V_0..V_j,
// all of length n with stride n: classical Gram-Schmidt with one
// re-orthogonalisation pass (CGS2), then V_{j+1} = w / |w| when |w| is
// nonzero (w is overwritten by the unscaled result), in three sweeps over V:
// project; subtract and project again; subtract and take the norm (the
// arithmetic of five separate kernels, the same bits).  hcol[0..j] gets the projection
// coefficients, *hn the remaining norm.  `dsmall` is device scratch of >= 65
// values (dsmall[64] ends as |V_{j+1}|^2 before the scaling), `h_pinned` a
// pinned host mirror of >= 65; one stream synchronisation.  (A second pass
// only when the first cancels, by the criterion of Daniel, Gragg, Kaufman
// and Stewart, saves nothing here: with the Jacobi-scaled Schur operator
// close to the identity the first pass always cancels, and the extra
// synchronisation made the step slower.)
int arnoldi_step(cudaStream_t st, double *V, long n, int j, double *w, double *red,
                 double *dsmall, double *h_pinned, double *hcol, double *hn);
int vec_multidot(cudaStream_t st, const double *V, long ldv, int m, const double *w, long n,
                 double *red, double *out);  // out[l] = V_l . w, l < m
// w += sign * sum_l h[l] V_l  (h device)
int vec_multiaxpy(cudaStream_t st, double *w, const double *V, long ldv, int m,
                  const double *h, double sign, long n);
// out[0] = max|a-b|, out[1] = max|a| (b may be null -> out[0] = out[1])
int vec_maxdiff(cudaStream_t st, const double *a, const double *b, long n, double *red,
                double *out);
// out[0..3] = min rho, max |rho|, max sqrt(g p/rho), max |u|
int vec_diagnostics(cudaStream_t st, const double *rho, const double *u, const double *p,
                    int nc, int nn2, double *red, double *out);
int vec_sponge(cudaStream_t st, double *u, const double *alpha, double dt, double ub0,
               double ub1, const double *target, const double *dts, int nc, int nn2);

// ------------------------------------------------------------- MG levels --
// Operator data of one multigrid level (T = float: mixed precision; double:
// the FP64 multigrid path).
template <typename T>
struct LevelViewT {
  int k, nc;
  MeshT<T> mesh;
  const T *ainv;  // [nc][nn2*nn2] inverse rho_fix-weighted mass (transposed)
  const T *invd;  // inverse diagonal of D
  cudaStream_t st;
  bool tune = false;  // the autotuner may time tile shapes on this stream
  const T *pfix = nullptr, *pfq = nullptr, *pff = nullptr;  // level p_fix (+ prepared)
};
template <typename T>
int level_B(const LevelViewT<T> &v, T *dst, const T *p, T cB, int mode);
template <typename T>
int level_CD(const LevelViewT<T> &v, T *dst, const T *w, const T *p, T cC, int mode);
// Chebyshev update fused into the C/D epilogue (multigrid smoother): with
// t = S x computed by the kernel, r = rhs - t, d = (first ? 0 : a d) + b invd r,
// x += d.  x is also the kernel's D input, read for the cell's own nodes only.
template <typename T>
struct ChebArgs {
  T *x = nullptr, *d = nullptr;
  const T *rhs = nullptr;
  T a = T(0), b = T(0);
  int first = 0;
};
template <typename T>
int level_CD_cheb(const LevelViewT<T> &v, const T *w, T cC, const ChebArgs<T> &ch);
template <typename T>
int level_pfix_prep(const LevelViewT<T> &v);
template <typename T>
int level_inv_diag(const LevelViewT<T> &v, T *out, T scale);
template <typename T>
int level_block_inverse(const LevelViewT<T> &v, T *out, const T *weight);

// multigrid hierarchy (mg.cu)
int mg_add_level(atm_ctx &c, int n_cells, int mapdeg, const double *nodes, int n_inner,
                 const int *inner, int n_bdry, const int *bdry, const int *children);
int mg_free(atm_ctx &c);
int mg_set_params(atm_ctx &c, int degree, double range, int eig_its, int coarse_degree);
int mg_precondition(atm_ctx &c, int precision, double *z, const double *v);
// precision 1: FP32 V-cycle, 2: FP64 V-cycle
int fgmres_mg(atm_ctx &c, int precision, double *x, const double *b, double tol, int maxit,
              int *its, double *res);
void mg_mark_rho_changed(atm_ctx &c);
long mg_vcycles(const atm_ctx &c);

// ------------------------------------------------------------- autotuner --
// Cells per block of the face kernels, among 64/NQ, 128/NQ and 256/NQ, per
// (device, kernel family, degree, mode or stage, hanging faces, value size,
// log2 of the cell count).  On the first idempotent launch of a key with
// tuning allowed, `launch(cpb)` is timed for each candidate (1 warm-up + 3
// timed launches, CUDA events on `st`) and the fastest is kept; until then,
// for meshes below 2048 cells, and when tuning is off the default 128/NQ is
// used.  The choice never changes results: every cell is computed by its own
// threads whatever the block grouping.
enum TuneFamily { TF_RHS_RHO = 0, TF_RHS_VEL, TF_RHS_PRES, TF_B, TF_CD };
int tuned_cpb(bool tune, cudaStream_t st, int family, int k, int mode, bool hg, int tsize,
              int nc, bool idempotent, const std::function<cudaError_t(int)> &launch);
int tune_table(int *out, int max_entries);
int mg_set_graphs(atm_ctx &c, bool on);
void mg_stats(const atm_ctx &c, long *out);
int mg_levels(const atm_ctx &c);

// ------------------------------------------------------------ mesh set-up --
struct HostMesh {
  std::vector<double> qgeo, fgeo;
  std::vector<int> nbr, nbrf;
  std::vector<int> hnb;      // [nhang][2]
  std::vector<double> hgeo;  // [nhang][2][3][nq]
  std::vector<double> map2;  // [nc][3][3][2] the mapping at degree 2 (MeshT::map2)
  int nhang = 0;
};
int build_mesh_tables(int k, int nc, int mapdeg, const double *nodes, int n_inner,
                      const int *inner, int n_bdry, const int *bdry, HostMesh &out);
int mesh_upload(atm_ctx &c, int mapdeg, const double *nodes, int n_inner, const int *inner,
                int n_bdry, const int *bdry);
void mesh_free(Mesh &m);

// ---------------------------------------------------------- operator glue --
// FP64 flops of the sum-factorisation contractions per cell (2 per FMA)
inline double fl_eval(int k) {  // values of one field at the Gauss points
  const double nn = k + 1, nq = 2 * k + 1;
  return 2.0 * (nq * nn * nn + nq * nq * nn);
}
inline double fl_integrate(int k, bool grad) {  // one output component
  const double nn = k + 1, nq = 2 * k + 1;
  return grad ? 2.0 * (3 * nn * nq * nq + 2 * nn * nn * nq) : 2.0 * (nn * nq * nq + nn * nn * nq);
}
inline double fl_face(int k) {  // one field trace at the points of one face
  return 2.0 * (2 * k + 1) * (k + 1);
}
StageCoef stage_coef_rho(const atm_ctx &c, int stage);
StageCoef stage_coef_flux(const atm_ctx &c, int stage);
double implicit_coeff(const atm_ctx &c);
int schur_apply(atm_ctx &c, double *dst, const double *p, bool precondition);
int op_vmult(atm_ctx &c, double *dst, const double *src);
int op_solve(atm_ctx &c, double *x, const double *b, double tol, int maxit, int *its,
             double *res);
int gmres_schur(atm_ctx &c, double *x, const double *b, double tol, int maxit, int *its,
                double *res);
int read_scalars(atm_ctx &c, int n);  // device red_out[0..n) -> h_red (sync)
int rebuild_ainv(atm_ctx &c);

// ------------------------------------------------------------ time loop --
struct Solver {
  double eps = 1e-8;
  int max_its = 30000;
  int precision = 0;
  // false (default): a Schur solve that reaches max_its ends the step with
  // ATM_NOT_CONVERGED, as deal.II's SolverControl throws (caught in main,
  // Atmospheric_Flow.cc:1289-1311); true: count it and carry on
  bool continue_on_not_converged = false;
  double time = 0.0;
  long steps = 0, picard_total = 0, krylov_total = 0, failures = 0;
  int last_picard[2] = {0, 0};
  double ubg0 = 0.0, ubg1 = 0.0;
  bool sponge = false;
  double *sponge_target = nullptr;  // per-node target velocity, or the (ubg0, ubg1)
  // state and stage vectors (device)
  double *rho_old, *rho_tmp_2, *rho_tmp_3, *rho_curr, *rhs_rho;
  double *u_old, *u_tmp_2, *u_tmp_3, *u_curr, *u_fixed, *rhs_u, *tmp_1;
  double *pres_old, *pres_tmp_2, *pres_tmp_3, *pres_fixed, *pres_fixed_old, *rhs_pres;
  double *alpha;
  double *pool = nullptr;
};

// ------------------------------------------------- members of a batch --
// A context may hold several independent members whose cells are
// contiguous ranges and share no faces (a concatenated cell list).  Each
// member then has its own time step (the per-cell dt multiplier), its own
// Krylov solves (member-wise inner products, Hessenberg matrices and stops)
// and its own Picard stop; a member whose solve fails is frozen and reported
// without stopping the others.
struct Members {
  int n = 0;
  std::vector<int> off;        // [n+1] first cell of each member
  std::vector<double> dt;      // [n] each member's time step
  std::vector<double> dts_host;  // [nc] dt multiplier of every cell
  int *cell_mem = nullptr;     // [nc] member of each cell (device)
  long *eoff = nullptr;        // [n+1] first scalar-vector element of each member
  double *dts = nullptr;       // [nc] dt multiplier (device; mesh.dts points here)
  double *red = nullptr;       // partial sums [rows][n][sb] (device)
  double *out = nullptr;       // reduced values [rows][n] (device)
  double *h_out = nullptr;     // pinned host mirror of out
  double *coef = nullptr;      // coefficients [cols][n] (device)
  double *h_coef = nullptr;    // pinned host staging of coef
  int sb = 1;                  // reduction blocks per member
  // per-member solver record
  std::vector<int> status;     // ATM_OK, or the sticky failure of the member
  std::vector<long> picard, krylov, fail_step;
  std::vector<char> active;    // takes part in the current Picard loop / solve
  std::vector<int> last_its;   // Krylov iterations of the last solve
  std::vector<double> last_res;
};
constexpr int MEM_ROWS = 72;  // reduced rows per call (2 x 32 Hessenberg + 8)
int members_set(atm_ctx &c, int n, const int *cell_off, const double *dt);
void members_free(atm_ctx &c);
int members_refresh_dt(atm_ctx &c);  // after a change of c.dt
// member-wise reductions: out[col * n + m] (device, then copied to h_out)
int seg_multidot(atm_ctx &c, const double *V, long ldv, int m, const double *w);
int seg_maxdiff(atm_ctx &c, const double *a, const double *b);  // rows 0, 1
int seg_read(atm_ctx &c, int rows);                             // out -> h_out (sync)
// member-wise vector updates with coefficients coef[col * n + m] (host
// values in h_coef, copied to the device first)
int seg_multiaxpy(atm_ctx &c, double *w, const double *V, long ldv, int cols, double sign);
int seg_scale(atm_ctx &c, double *d, const double *s);  // d = coef[member] * s
// Schur solve of every active member: precision 0 GMRES + Jacobi (left),
// 1/2 FGMRES + multigrid (FP32/FP64 V-cycle).  tol[m] as the solo solvers'.
// Per-member iterations, residuals and outcomes in last_its / last_res and
// `state` (ATM_OK, ATM_NOT_CONVERGED, ATM_NONFINITE; -1 for inactive members).
int krylov_members(atm_ctx &c, int precision, double *x, const double *b,
                   const std::vector<double> &tol, int maxit, std::vector<int> &state);
// multigrid pieces used by krylov_members (mg.cu)
int mg_prepare(atm_ctx &c, int precision);
int mg_vcycle_only(atm_ctx &c, int precision, double *z, const double *v);
double *mg_zbasis(atm_ctx &c);
int mg_restart(const atm_ctx &c);
void mg_invalidate(atm_ctx &c);  // device hierarchies are rebuilt on next use

int solver_alloc(atm_ctx &c, Solver &s);
void solver_free(Solver &s);
int solver_step(atm_ctx &c, Solver &s);
int solver_diagnostics(atm_ctx &c, Solver &s, double *out);

}  // namespace atm
