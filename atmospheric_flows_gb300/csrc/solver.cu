// IMEX time loop on the device: EulerSolver::run and its stage solvers
// (Atmospheric_Flow.cc:430-871, 1100-1257).
//
// Differences from the reference, by design:
//   * the mass-type systems (rho mass, A, D) are block diagonal in this DG
//     discretisation and are solved exactly with the per-cell inverse instead
//     of CG + geometric multigrid to a tolerance (Atmospheric_Flow.cc:452-536,
//     701-780, 801-870).  The answer is the reference's answer without the
//     solver error.
//   * inside the Schur apply A^{-1} is the exact per-cell inverse instead of
//     CG + Jacobi to 1e-12 (euler_operator.h:2391-2397).
//   * diagnostics and L2 error analysis are not part of the step (they are
//     printouts in the reference, Atmospheric_Flow.cc:1121-1122,1225-1242);
//     atm_solver_diagnostics computes them on demand.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "atm_device.cuh"

namespace atm {

int solver_alloc(atm_ctx &c, Solver &s) {
  const long ns = c.n_scalar(), nv = c.n_vector();
  const long total = 12 * ns + 7 * nv;
  ATM_CUDA(cudaMalloc(&s.pool, total * sizeof(double)));
  ATM_CUDA(cudaMemsetAsync(s.pool, 0, total * sizeof(double), c.stream));
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  double *p = s.pool;
  auto take = [&](long n) { double *r = p; p += n; return r; };
  s.rho_old = take(ns); s.rho_tmp_2 = take(ns); s.rho_tmp_3 = take(ns);
  s.rho_curr = take(ns); s.rhs_rho = take(ns);
  s.pres_old = take(ns); s.pres_tmp_2 = take(ns); s.pres_tmp_3 = take(ns);
  s.pres_fixed = take(ns); s.pres_fixed_old = take(ns); s.rhs_pres = take(ns);
  s.alpha = take(ns);
  s.u_old = take(nv); s.u_tmp_2 = take(nv); s.u_tmp_3 = take(nv); s.u_curr = take(nv);
  s.u_fixed = take(nv); s.rhs_u = take(nv); s.tmp_1 = take(nv);
  return ATM_OK;
}

void solver_free(Solver &s) {
  cudaFree(s.pool);
  cudaFree(s.sponge_target);
  s.pool = nullptr;
  s.sponge_target = nullptr;
}

namespace {

#define TRY(x)              \
  do {                      \
    int _rc = (x);          \
    if (_rc) return _rc;    \
  } while (0)

int set_rho_fixed(atm_ctx &c, const double *rho) {
  TRY(vec_copy(c.stream, c.rho_fix, rho, c.n_scalar()));
  return rebuild_ainv(c);
}

// Atmospheric_Flow.cc:430-537
int update_density(atm_ctx &c, Solver &s) {
  const StageCoef co = stage_coef_rho(c, c.hstage);
  if (c.hstage == 1) {
    const double *src[] = {s.rho_old, s.u_old};
    TRY(launch_rhs_rho(c, 1, s.rhs_rho, src, co));
    return launch_block_apply(c, s.rho_tmp_2, s.rhs_rho, c.mesh.minv, 1, 1.0);
  } else if (c.hstage == 2) {
    const double *src[] = {s.rho_old, s.u_old, s.rho_tmp_2, s.u_tmp_2};
    TRY(launch_rhs_rho(c, 2, s.rhs_rho, src, co));
    return launch_block_apply(c, s.rho_tmp_3, s.rhs_rho, c.mesh.minv, 1, 1.0);
  }
  const double *src[] = {s.rho_old, s.u_old, s.rho_tmp_2, s.u_tmp_2, s.rho_tmp_3, s.u_tmp_3};
  TRY(launch_rhs_rho(c, 3, s.rhs_rho, src, co));
  return launch_block_apply(c, s.rho_curr, s.rhs_rho, c.mesh.minv, 1, 1.0);
}

// ------------------------------------------ several members per context --
// A member whose solve fails is frozen: its fields are set to a uniform rest
// state (rho = 1, u = 0, p = 1) so that nothing non-finite reaches the
// operators or the multigrid set-up shared with the other members, and it
// takes no further Picard or Krylov update.  Its status and the step at which
// it failed are kept for atm_member_stats.
void member_fill(atm_ctx &c, Solver &s, int m) {
  const Members &M = *c.mem;
  const long a = (long)M.off[m] * c.nn2, len = (long)(M.off[m + 1] - M.off[m]) * c.nn2;
  double *ones[] = {s.rho_old, s.rho_tmp_2, s.rho_tmp_3, s.rho_curr, s.pres_old, s.pres_tmp_2,
                    s.pres_tmp_3, s.pres_fixed, s.pres_fixed_old, c.rho_fix, c.pres_fix};
  double *zeros[] = {s.u_old, s.u_tmp_2, s.u_tmp_3, s.u_curr, s.u_fixed, c.u_fix};
  for (double *v : ones) vec_fill(c.stream, v + a, 1.0, len);
  for (double *v : zeros) vec_fill(c.stream, v + 2 * a, 0.0, 2 * len);
}

void member_fail(atm_ctx &c, Solver &s, int m, int code) {
  Members &M = *c.mem;
  if (M.status[m] == ATM_OK) {
    M.status[m] = code;
    M.fail_step[m] = s.steps + 1;
  }
  M.active[m] = 0;
  member_fill(c, s, m);
}

// members whose field `v` holds a non-finite value fail now (each check is
// followed by set_rho_fixed, which rebuilds A^{-1} from the reset fields)
int members_check_finite(atm_ctx &c, Solver &s, const double *v) {
  Members &M = *c.mem;
  TRY(seg_maxdiff(c, v, v));
  TRY(seg_read(c, 2));
  for (int m = 0; m < M.n; ++m)
    if (M.status[m] == ATM_OK && !std::isfinite(M.h_out[M.n + m]))
      member_fail(c, s, m, ATM_NONFINITE);
  return ATM_OK;
}

// the Schur solve of pressure_fixed_point for every active member
int schur_solve_members(atm_ctx &c, Solver &s) {
  Members &M = *c.mem;
  const long ns = c.n_scalar();
  TRY(seg_multidot(c, s.rhs_pres, ns, 1, s.rhs_pres));
  TRY(seg_read(c, 1));
  std::vector<double> tol(M.n);
  std::vector<int> st(M.n);
  for (int m = 0; m < M.n; ++m) {
    tol[m] = s.eps * std::sqrt(M.h_out[m]);
    st[m] = M.active[m] ? 0 : -1;
  }
  TRY(vec_copy(c.stream, s.pres_fixed, s.pres_fixed_old, ns));
  TRY(krylov_members(c, s.precision, s.pres_fixed, s.rhs_pres, tol, s.max_its, st));
  for (int m = 0; m < M.n; ++m) {
    if (st[m] < 0) continue;
    s.krylov_total += M.last_its[m];
    if (st[m] == ATM_NOT_CONVERGED) {
      ++s.failures;
      if (!s.continue_on_not_converged) member_fail(c, s, m, ATM_NOT_CONVERGED);
    } else if (st[m] == ATM_NONFINITE) {
      member_fail(c, s, m, ATM_NONFINITE);
    }
  }
  return ATM_OK;
}

// Atmospheric_Flow.cc:544-673
int pressure_fixed_point(atm_ctx &c, Solver &s) {
  const long ns = c.n_scalar();
  TRY(vec_copy(c.stream, c.pres_fix, s.pres_fixed_old, ns));  // set_pres_fixed
  TRY(launch_pfix_prep(c));
  const StageCoef co = stage_coef_flux(c, c.hstage);
  if (c.hstage == 1) {
    const double *sp[] = {s.rho_old, s.u_old, s.pres_old, s.rho_tmp_2, s.u_fixed};
    TRY(launch_rhs_pres(c, 1, s.rhs_pres, sp, co));
    const double *su[] = {s.rho_old, s.u_old, s.pres_old, s.rho_tmp_2};
    TRY(launch_rhs_vel(c, 1, s.rhs_u, su, co));
  } else {
    const double *sp[] = {s.rho_old, s.u_old, s.pres_old, s.rho_tmp_2, s.u_tmp_2,
                          s.pres_tmp_2, s.rho_tmp_3, s.u_fixed};
    TRY(launch_rhs_pres(c, 2, s.rhs_pres, sp, co));
    const double *su[] = {s.rho_old, s.u_old, s.pres_old, s.rho_tmp_2, s.u_tmp_2,
                          s.pres_tmp_2, s.rho_tmp_3};
    TRY(launch_rhs_vel(c, 2, s.rhs_u, su, co));
  }
  // tmp_1 = A^{-1} rhs_u ; rhs_pres -= C tmp_1
  TRY(launch_block_apply(c, s.tmp_1, s.rhs_u, c.ainv, 2, 1.0));
  const double cc = implicit_coeff(c);
  TRY(launch_CD(c, s.rhs_pres, s.tmp_1, nullptr, cc * c.dt, 3));
  if (c.mem) return schur_solve_members(c, s);
  TRY(vec_dot(c.stream, s.rhs_pres, s.rhs_pres, ns, c.red, c.red_out));
  TRY(read_scalars(c, 1));
  const double tol = s.eps * std::sqrt(c.h_red[0]);
  TRY(vec_copy(c.stream, s.pres_fixed, s.pres_fixed_old, ns));
  int its = 0;
  double res = 0.0;
  int rc = s.precision == 0
               ? gmres_schur(c, s.pres_fixed, s.rhs_pres, tol, s.max_its, &its, &res)
               : fgmres_mg(c, s.precision, s.pres_fixed, s.rhs_pres, tol, s.max_its, &its, &res);
  s.krylov_total += its;
  if (rc == ATM_NOT_CONVERGED) {
    ++s.failures;
    if (s.continue_on_not_converged) return ATM_OK;
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "Schur solve did not converge in IMEX stage %d of step %ld: %d iterations, "
                  "residual %.3e > tolerance %.3e (step abandoned; the state is that of the "
                  "last completed step)",
                  c.hstage, s.steps + 1, its, res, tol);
    set_error(msg);
  }
  return rc;
}

// Atmospheric_Flow.cc:680-781
int update_velocity(atm_ctx &c, Solver &s) {
  if (c.hstage == 1 || c.hstage == 2) {
    const double co = implicit_coeff(c);
    TRY(launch_B(c, s.rhs_u, s.pres_fixed, co * c.dt / (c.Ma * c.Ma), 1));
    return launch_block_apply(c, s.u_fixed, s.rhs_u, c.ainv, 2, 1.0);
  }
  const StageCoef co = stage_coef_flux(c, 3);
  const double *su[] = {s.rho_old, s.u_old, s.pres_old, s.rho_tmp_2, s.u_tmp_2,
                        s.pres_tmp_2, s.rho_tmp_3, s.u_tmp_3, s.pres_tmp_3};
  TRY(launch_rhs_vel(c, 3, s.rhs_u, su, co));
  return launch_block_apply(c, s.u_curr, s.rhs_u, c.ainv, 2, 1.0);
}

// Atmospheric_Flow.cc:788-871
int update_pressure(atm_ctx &c, Solver &s) {
  const StageCoef co = stage_coef_flux(c, 3);
  const double *sp[] = {s.rho_old, s.u_old, s.pres_old, s.rho_tmp_2, s.u_tmp_2,
                        s.pres_tmp_2, s.rho_tmp_3, s.u_tmp_3, s.pres_tmp_3,
                        s.rho_curr, s.u_curr};
  TRY(launch_rhs_pres(c, 3, s.rhs_pres, sp, co));
  return launch_block_apply(c, s.pres_old, s.rhs_pres, c.mesh.minv, 1, GAS_GAMMA - 1.0);
}

// Picard loop of every member, each with its own stop: a member that meets
// the 1e-10 criterion is frozen for the rest of the loop (its Schur solve
// takes no further update, so its pres_fixed and u_fixed keep the values of
// its last iteration, as in its solo run).
int picard_members(atm_ctx &c, Solver &s, int which) {
  Members &M = *c.mem;
  const long ns = c.n_scalar();
  std::vector<int> iters(M.n, 0);
  for (int m = 0; m < M.n; ++m) M.active[m] = M.status[m] == ATM_OK;
  for (int iter = 0; iter < 100; ++iter) {
    TRY(pressure_fixed_point(c, s));
    TRY(update_velocity(c, s));
    TRY(seg_maxdiff(c, s.pres_fixed, s.pres_fixed_old));
    TRY(seg_read(c, 2));
    bool any = false;
    for (int m = 0; m < M.n; ++m) {
      if (!M.active[m]) continue;
      ++iters[m];
      const double error = M.h_out[m] / (M.h_out[M.n + m] + 1e-10);
      if (!std::isfinite(error)) member_fail(c, s, m, ATM_NONFINITE);
      else if (error < 1e-10) M.active[m] = 0;
      else any = true;
    }
    if (!any) break;
    TRY(vec_copy(c.stream, s.pres_fixed_old, s.pres_fixed, ns));
  }
  int most = 0;
  for (int m = 0; m < M.n; ++m) {
    M.picard[m] += iters[m];
    most = std::max(most, iters[m]);
  }
  s.last_picard[which] = most;
  s.picard_total += most;
  return ATM_OK;
}

// Picard loop, Atmospheric_Flow.cc:1135-1153 / 1176-1194
int picard(atm_ctx &c, Solver &s, int which) {
  if (c.mem) return picard_members(c, s, which);
  const long ns = c.n_scalar();
  int iters = 0;
  for (int iter = 0; iter < 100; ++iter) {
    TRY(pressure_fixed_point(c, s));
    TRY(update_velocity(c, s));
    ++iters;
    TRY(vec_maxdiff(c.stream, s.pres_fixed, s.pres_fixed_old, ns, c.red, c.red_out));
    TRY(read_scalars(c, 2));
    const double den = c.h_red[1];
    const double error = c.h_red[0] / (den + 1e-10);
    if (!std::isfinite(error)) { set_error("Picard: non-finite pressure"); return ATM_NONFINITE; }
    if (error < 1e-10) break;
    TRY(vec_copy(c.stream, s.pres_fixed_old, s.pres_fixed, ns));
  }
  s.last_picard[which] = iters;
  s.picard_total += iters;
  return ATM_OK;
}

}  // namespace

// one pass of the while loop of Atmospheric_Flow.cc:1110-1250.  The state
// (rho_old, u_old, pres_old) is written only in stage 3, which has no Krylov
// solve, so a step that fails in stage 1 or 2 leaves the state, the time and
// the step count of the last completed step.
int solver_step(atm_ctx &c, Solver &s) {
  const long ns = c.n_scalar(), nv = c.n_vector();
  if (c.mem) {
    // failed members stay at rest; a member whose pressure is not finite
    // (an uploaded state, say) fails before it reaches a shared reduction
    for (int m = 0; m < c.mem->n; ++m)
      if (c.mem->status[m] != ATM_OK) member_fill(c, s, m);
    TRY(members_check_finite(c, s, s.pres_old));
  }
  // stage 1
  c.hstage = 1;
  TRY(update_density(c, s));
  if (c.mem) TRY(members_check_finite(c, s, s.rho_tmp_2));  // sees rho_old and u_old
  TRY(set_rho_fixed(c, s.rho_tmp_2));
  TRY(vec_copy(c.stream, s.pres_fixed_old, s.pres_old, ns));
  TRY(vec_copy(c.stream, s.u_fixed, s.u_old, nv));
  TRY(picard(c, s, 0));
  TRY(vec_copy(c.stream, s.pres_tmp_2, s.pres_fixed, ns));
  TRY(vec_copy(c.stream, s.u_tmp_2, s.u_fixed, nv));
  // stage 2
  c.hstage = 2;
  TRY(update_density(c, s));
  if (c.mem) TRY(members_check_finite(c, s, s.rho_tmp_3));
  TRY(set_rho_fixed(c, s.rho_tmp_3));
  TRY(vec_copy(c.stream, s.pres_fixed_old, s.pres_tmp_2, ns));
  TRY(vec_copy(c.stream, s.u_fixed, s.u_tmp_2, nv));
  TRY(picard(c, s, 1));
  TRY(vec_copy(c.stream, s.pres_tmp_3, s.pres_fixed, ns));
  TRY(vec_copy(c.stream, s.u_tmp_3, s.u_fixed, nv));
  // stage 3 (final combination)
  c.hstage = 3;
  TRY(update_density(c, s));
  if (c.mem) TRY(members_check_finite(c, s, s.rho_curr));
  TRY(set_rho_fixed(c, s.rho_curr));
  TRY(update_velocity(c, s));
  TRY(update_pressure(c, s));
  TRY(vec_copy(c.stream, s.rho_old, s.rho_curr, ns));
  TRY(vec_copy(c.stream, s.u_old, s.u_curr, nv));
  if (s.sponge)
    TRY(vec_sponge(c.stream, s.u_old, s.alpha, c.dt, s.ubg0, s.ubg1, s.sponge_target,
                   c.mesh.dts, c.nc, c.nn2));
  s.time += c.dt;
  ++s.steps;
  return ATM_OK;
}

int solver_diagnostics(atm_ctx &c, Solver &s, double *out) {
  TRY(vec_diagnostics(c.stream, s.rho_old, s.u_old, s.pres_old, c.nc, c.nn2, c.red,
                      c.red_out));
  TRY(read_scalars(c, 4));
  for (int i = 0; i < 4; ++i) out[i] = c.h_red[i];
  return ATM_OK;
}

}  // namespace atm
