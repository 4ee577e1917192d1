// Operator glue: IMEX stage weights, Base::vmult dispatch, the Schur apply,
// exact mass-type solves and the restarted GMRES for the Schur system.
#include <cmath>
#include <cstring>

#include "atm_device.cuh"

namespace atm {

Tableau Tableau::make() {
  // euler_operator.h:220-224
  Tableau t;
  t.gamma = 2.0 - std::sqrt(2.0);
  t.a21 = t.gamma; t.a22 = 0.0; t.a31 = 0.5; t.a32 = 0.5; t.a33 = 0.0;
  t.a21t = 0.5 * t.gamma; t.a22t = 0.5 * t.gamma;
  t.a31t = std::sqrt(2.0) / 4.0; t.a32t = std::sqrt(2.0) / 4.0;
  t.a33t = 1.0 - std::sqrt(2.0) / 2.0;
  t.b1 = t.a31t; t.b2 = t.a32t; t.b3 = t.a33t;
  return t;
}

StageCoef stage_coef_rho(const atm_ctx &c, int stage) {
  StageCoef s{};
  const Tableau &t = c.tab;
  if (stage == 1) { s.ca[0] = t.a21; }
  else if (stage == 2) { s.ca[0] = t.a31; s.ca[1] = t.a32; }
  else { s.ca[0] = t.b1; s.ca[1] = t.b2; s.ca[2] = t.b3; }
  s.dt = c.dt; s.Ma = c.Ma; s.Fr = c.Fr;
  return s;
}

StageCoef stage_coef_flux(const atm_ctx &c, int stage) {
  StageCoef s{};
  const Tableau &t = c.tab;
  if (stage == 1) {
    s.ca[0] = t.a21; s.ct[0] = t.a21t;
    s.cg[0] = t.a21t; s.cg[1] = t.a22t;
  } else if (stage == 2) {
    s.ca[0] = t.a31; s.ca[1] = t.a32; s.ct[0] = t.a31t; s.ct[1] = t.a32t;
    s.cg[0] = t.a31t; s.cg[1] = t.a32t; s.cg[2] = t.a33t;
  } else {
    s.ca[0] = t.b1; s.ca[1] = t.b2; s.ca[2] = t.b3;
    s.ct[0] = t.b1; s.ct[1] = t.b2; s.ct[2] = t.b3;
    s.cg[0] = t.b1; s.cg[1] = t.b2; s.cg[2] = t.b3;
  }
  s.dt = c.dt; s.Ma = c.Ma; s.Fr = c.Fr;
  return s;
}

// euler_operator.h:1428,1526: a22~ in IMEX stage 1, a33~ otherwise
double implicit_coeff(const atm_ctx &c) { return c.hstage == 1 ? c.tab.a22t : c.tab.a33t; }

int read_scalars(atm_ctx &c, int n) {
  ATM_CUDA(cudaMemcpyAsync(c.h_red, c.red_out, n * sizeof(double), cudaMemcpyDeviceToHost,
                           c.stream));
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  return ATM_OK;
}

static int read_small(atm_ctx &c, const double *dev, int n) {
  ATM_CUDA(cudaMemcpyAsync(c.h_red, dev, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  return ATM_OK;
}

int rebuild_ainv(atm_ctx &c) {
  mg_mark_rho_changed(c);
  return launch_block_inverse(c, c.ainv, c.rho_fix);
}

// S p = D p - C A^{-1} B p  (euler_operator.h:2374-2408); with `precondition`
// the result is multiplied by the inverse diagonal of D (PreconditionJacobi
// on the diagonal of D only, euler_operator.h:2607-2611).
int schur_apply(atm_ctx &c, double *dst, const double *p, bool precondition) {
  const double co = implicit_coeff(c);
  int rc = launch_B(c, c.wv1, p, co * c.dt / (c.Ma * c.Ma), 2);
  if (rc) return rc;
  return launch_CD(c, dst, c.wv1, p, co * c.dt, precondition ? 2 : 1);
}

// Base::vmult -> apply_add (euler_operator.h:2366-2417)
int op_vmult(atm_ctx &c, double *dst, const double *src) {
  switch (c.nsstage) {
    case 1:
    case 4: return launch_mass(c, dst, src, 1, nullptr, 1.0);
    case 2: return schur_apply(c, dst, src, false);
    case 3:
    case 5: return launch_mass(c, dst, src, 2, c.rho_fix, 1.0);
    case 6: return launch_mass(c, dst, src, 1, nullptr, 1.0 / (GAS_GAMMA - 1.0));
    default: set_error("NS stage out of range"); return ATM_BAD_ARG;
  }
}

int op_solve(atm_ctx &c, double *x, const double *b, double tol, int maxit, int *its,
             double *res) {
  int it = 1;
  int rc = ATM_OK;
  switch (c.nsstage) {
    case 1:
    case 4: rc = launch_block_apply(c, x, b, c.mesh.minv, 1, 1.0); break;
    case 6: rc = launch_block_apply(c, x, b, c.mesh.minv, 1, GAS_GAMMA - 1.0); break;
    case 3:
    case 5: rc = launch_block_apply(c, x, b, c.ainv, 2, 1.0); break;
    case 2: {
      double r = 0.0;
      rc = gmres_schur(c, x, b, tol, maxit, &it, &r);
      if (res) *res = r;
      if (its) *its = it;
      return rc;
    }
    default: set_error("NS stage out of range"); return ATM_BAD_ARG;
  }
  if (its) *its = it;
  if (res) *res = 0.0;
  return rc;
}

// Restarted GMRES with left Jacobi preconditioning (deal.II SolverGMRES with
// right_preconditioning = false, max_n_tmp_vectors = 30 -> 28 basis vectors):
// classical Gram-Schmidt with one re-orthogonalisation pass (CGS2,
// arnoldi_step), Givens rotations, stop when the preconditioned residual
// estimate <= tol.  The same algorithm is restated in the CPU oracle.
int gmres_schur(atm_ctx &c, double *x, const double *b, double tol, int maxit, int *its,
                double *res) {
  const long n = c.n_scalar();
  const int m = c.restart;
  double *V = c.krylov;
  double *w = c.ws1, *t = c.ws2;
  double *nsq = c.dsmall + 64, *ydev = c.dsmall + 96;
  std::vector<double> H((m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m), hcol(m + 1);
  int rc;
  *its = 0;
  *res = 0.0;
  for (;;) {
    if ((rc = schur_apply(c, t, x, false))) return rc;
    if ((rc = vec_xmy_scaled(c.stream, V, c.invdiag_D, b, t, n))) return rc;
    if ((rc = vec_dot(c.stream, V, V, n, c.red, nsq))) return rc;
    if ((rc = read_small(c, nsq, 1))) return rc;
    const double beta = std::sqrt(c.h_red[0]);
    *res = beta;
    if (!std::isfinite(beta)) { set_error("GMRES: non-finite residual"); return ATM_NONFINITE; }
    if (beta <= tol) return ATM_OK;
    if (*its >= maxit) return ATM_NOT_CONVERGED;
    if ((rc = vec_scale_by_inv_norm(c.stream, V, V, nsq, n))) return rc;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int jend = 0;
    bool done = false;
    for (int j = 0; j < m; ++j) {
      ++*its;
      double *Vj = V + (long)j * n;
      if ((rc = schur_apply(c, w, Vj, true))) return rc;
      double hn = 0.0;
      if ((rc = arnoldi_step(c.stream, V, n, j, w, c.red, c.dsmall, c.h_red, hcol.data(), &hn)))
        return rc;
      for (int l = 0; l <= j; ++l) H[l * m + j] = hcol[l];
      if (!std::isfinite(hn)) { set_error("GMRES: non-finite Arnoldi vector"); return ATM_NONFINITE; }
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
    if ((rc = vec_multiaxpy(c.stream, x, V, n, jend, ydev, 1.0, n))) return rc;
    // y lives in pageable host memory: make sure the copy finished before
    // the vector is reused
    ATM_CUDA(cudaStreamSynchronize(c.stream));
    // with the true-residual check a converged estimate only ends the cycle:
    // the restart recomputes b - S(x) and decides
    if (done && !c.true_residual_check)
      return (*res <= tol) ? ATM_OK : (*its >= maxit ? ATM_NOT_CONVERGED : ATM_OK);
  }
}

}  // namespace atm
