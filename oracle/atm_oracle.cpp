// ============================================================================
// atm_oracle.cpp -- CPU FP64 restatement of the IMEX-DG hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle and the timed
// CPU baseline.  Nothing in the product library links it; only the tests, the
// smoke entry and the bench's cpu_baseline / reference arm load it.
//
// PARITY UNPINNED: the reference (GiuseppeOrlando878776/Atmospheric_Flows)
// needs deal.II >= 9.3 with MPI and p4est, none of which exists on this
// machine, so its own FP64 MatrixFree run cannot be executed here and the
// reference ships no golden vectors.  This restatement is checked against
// analytic properties instead (exact quadrature, conservation, adjointness,
// steady states) in tests/test_oracle.py and tests/test_known_answer.py.
//
// What it restates (file:line refer to the reference project):
//   * EULEROperator<dim=2,...>  euler_operator.h:24-2627
//       - Butcher tableau                          euler_operator.h:220-240
//       - rho rhs cell/face (3 IMEX stages)        euler_operator.h:344-712
//       - rho mass                                 euler_operator.h:717-740
//       - energy (pressure) rhs cell/face          euler_operator.h:745-1381
//       - D internal-energy mass                   euler_operator.h:1386-1408
//       - C enthalpy operator                      euler_operator.h:1413-1507
//       - B pressure-gradient operator             euler_operator.h:1512-1617
//       - momentum rhs cell/face/boundary          euler_operator.h:1622-2325
//       - A rho-weighted velocity mass             euler_operator.h:2330-2357
//       - apply_add dispatch incl. Schur NS 2      euler_operator.h:2366-2417
//       - diagonal / inverse diagonal              euler_operator.h:2458-2626
//   * EulerSolver stage solvers and time loop    Atmospheric_Flow.cc:430-871,1100-1257
//
// Discretisation conventions restated from deal.II (library not vendored):
//   FE_DGQ(k): Lagrange polynomials on Gauss-Lobatto support points of [0,1],
//   lexicographic (x fastest); FESystem(FE_DGQ,dim) stores the components of
//   a cell as consecutive blocks.  All operator integrals use QGauss(2k+1)
//   (n_q_points_1d_u = 2*degree_u+1, Atmospheric_Flow.cc:151-153,345).
//   MappingQ(m): tensor Lagrange interpolation of the geometry on the
//   Gauss-Lobatto points of degree m.  Inner faces: n = outward normal of the
//   "+" (interior) cell, the "-" side receives the negated flux.
//
// Dimension: the reference hard-wires dim=3 on a spherical shell
// (Atmospheric_Flow.cc:283,1277).  This restatement is the dim=2 form on a
// Cartesian domain: the radial unit vector e_r becomes e_z and the factor
// a^2/r^2 becomes 1 (euler_operator.h:790-811).
//
// Vector layouts: scalar fields [cell][node]; velocity [cell][comp][node],
// node = iz*(k+1)+ix.
// ============================================================================
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double GAMMA_GAS = 1.4;  // EquationData::Cp_Cv, equation_data.h:23

// ---------------------------------------------------------------- 1D rules --
void legendre(int n, double x, double &p, double &dp) {
  if (n == 0) { p = 1.0; dp = 0.0; return; }
  double p0 = 1.0, p1 = x;
  for (int j = 2; j <= n; ++j) {
    const double p2 = ((2.0 * j - 1.0) * x * p1 - (j - 1.0) * p0) / j;
    p0 = p1;
    p1 = p2;
  }
  p = p1;
  // derivative from the recurrence n (x P_n - P_{n-1}) / (x^2 - 1)
  dp = n * (x * p1 - p0) / (x * x - 1.0);
}

// Gauss-Legendre points/weights on [0,1], ascending.
void gauss_rule(int n, std::vector<double> &x, std::vector<double> &w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    double t = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre(n, t, p, dp);
      const double dt = p / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    double p, dp;
    legendre(n, t, p, dp);
    x[n - 1 - i] = 0.5 * (t + 1.0);
    w[n - 1 - i] = 1.0 / ((1.0 - t * t) * dp * dp);  // (2/((1-t^2)P'^2)) / 2
  }
}

// Gauss-Lobatto points of degree k on [0,1], ascending.
void gll_points(int k, std::vector<double> &x) {
  x.assign(k + 1, 0.0);
  x[0] = 0.0;
  x[k] = 1.0;
  for (int i = 1; i < k; ++i) {
    double t = -std::cos(M_PI * i / k);
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre(k, t, p, dp);
      const double d2p = (2.0 * t * dp - k * (k + 1.0) * p) / (1.0 - t * t);
      const double dt = dp / d2p;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    x[i] = 0.5 * (t + 1.0);
  }
}

double lagrange(const std::vector<double> &xn, int i, double x) {
  double v = 1.0;
  for (size_t j = 0; j < xn.size(); ++j)
    if ((int)j != i) v *= (x - xn[j]) / (xn[i] - xn[j]);
  return v;
}

double lagrange_d(const std::vector<double> &xn, int i, double x) {
  double s = 0.0;
  for (size_t m = 0; m < xn.size(); ++m) {
    if ((int)m == i) continue;
    double v = 1.0 / (xn[i] - xn[m]);
    for (size_t j = 0; j < xn.size(); ++j)
      if ((int)j != i && j != m) v *= (x - xn[j]) / (xn[i] - xn[j]);
    s += v;
  }
  return s;
}

using Vec = std::vector<double>;

double dot(const Vec &a, const Vec &b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s)
  for (long i = 0; i < (long)a.size(); ++i) s += a[i] * b[i];
  return s;
}
double norm2(const Vec &a) { return std::sqrt(dot(a, a)); }
double linfty(const Vec &a) {
  double m = 0.0;
#pragma omp parallel for reduction(max : m)
  for (long i = 0; i < (long)a.size(); ++i) m = std::max(m, std::fabs(a[i]));
  return m;
}
void axpy(double a, const Vec &x, Vec &y) {
#pragma omp parallel for
  for (long i = 0; i < (long)y.size(); ++i) y[i] += a * x[i];
}

}  // namespace

// ============================================================================
// The operator.  Mirrors EULEROperator's state and entry points.
// ============================================================================
struct Oracle {
  int k = 1, nn = 2, nq = 3, nc = 0, m = 1, mn = 2;
  int nn2 = 4, nq2 = 9;
  Vec S, D, W;  // [q][i] values / derivatives of the node basis at Gauss pts
  Vec Sh[2];    // [q][i] values at the subface points (g_q + s)/2, s = 0, 1
  Vec cJinv, cJxW, cX;  // per cell per qp: dxi_a/dx_b (4), JxW, (x,z)
  // [nf][5] (c+,f+,c-,f-,o), [nb][3].  o = 0 conforming; o = 1, 2: hanging
  // face, c+ is the fine cell and its face is subface o-1 of face f- of the
  // coarse cell c- (deal.II: the fine cell is the interior side, the normal
  // and JxW come from it, and the coarse side is evaluated on the subface).
  std::vector<int> inner, bdry;
  int nf = 0, nb = 0;
  Vec fN, fJxW;  // inner faces, from the "+" side: [nf][nq][2], [nf][nq]
  Vec bN, bJxW;  // boundary faces
  // cell -> face contributions: 2 slots per cell face (a coarse hanging face
  // collects both subfaces): (type, index, side), type -1 none, 0 inner,
  // 1 boundary
  std::vector<int> cface;  // [nc][4][2][3]

  // parameters and tableau (euler_operator.h:220-240)
  double Ma = 1, Fr = 1, dt = 1;
  double gamma = 2.0 - std::sqrt(2.0);
  double a21 = gamma, a22 = 0.0, a31 = 0.5, a32 = 0.5, a33 = 0.0;
  double a21_tilde = 0.5 * gamma, a22_tilde = 0.5 * gamma;
  double a31_tilde = std::sqrt(2.0) / 4.0, a32_tilde = std::sqrt(2.0) / 4.0;
  double a33_tilde = 1.0 - std::sqrt(2.0) / 2.0;
  double b1 = a31_tilde, b2 = a32_tilde, b3 = a33_tilde;
  int hstage = 1, nsstage = 1;
  double inner_cg_tol = 1e-12;  // Schur-internal CG, euler_operator.h:2391
  long inner_cg_iters = 0;
  // When set, GMRES only stops on the true (recomputed) residual: a converged
  // estimate ends the cycle and the restart re-checks b - S(x).  S is not
  // linear, so without this the answer depends on the Krylov algorithm at the
  // level of the nonlinearity.  Off = deal.II SolverGMRES behaviour.
  bool true_residual_check = false;
  // When set, the Schur GMRES tolerance is eps * |D^{-1} b| (relative in the
  // norm GMRES measures) instead of the reference's eps * |b| compared with
  // |D^{-1} r| (Atmospheric_Flow.cc:656), which with D^{-1} ~ 1/(cell area)
  // lets a nominal eps = 1e-12 stop at a true relative residual near 1e-7.
  bool schur_tol_preconditioned = false;

  Vec rho_for_fixed, pres_fixed, u_fixed;
  Vec inv_diag;

  long ns() const { return (long)nc * nn2; }
  long nv() const { return 2L * nc * nn2; }

  // ---------------------------------------------------------------- setup --
  void setup(int degree, int ncells, int map_degree, const double *nodes,
             int n_inner, const int *inner_faces, int n_bdry,
             const int *bdry_faces) {
    k = degree;
    nn = k + 1;
    nq = 2 * k + 1;
    nn2 = nn * nn;
    nq2 = nq * nq;
    nc = ncells;
    m = map_degree;
    mn = m + 1;
    std::vector<double> gx, gw, xn, mx;
    gauss_rule(nq, gx, gw);
    gll_points(k, xn);
    gll_points(m, mx);
    S.assign(nq * nn, 0.0);
    D.assign(nq * nn, 0.0);
    W = gw;
    for (int q = 0; q < nq; ++q)
      for (int i = 0; i < nn; ++i) {
        S[q * nn + i] = lagrange(xn, i, gx[q]);
        D[q * nn + i] = lagrange_d(xn, i, gx[q]);
      }
    for (int s = 0; s < 2; ++s) {
      Sh[s].assign(nq * nn, 0.0);
      for (int q = 0; q < nq; ++q)
        for (int i = 0; i < nn; ++i) Sh[s][q * nn + i] = lagrange(xn, i, 0.5 * (gx[q] + s));
    }
    // mapping derivative tables at the Gauss points and at 0, 1
    auto map_eval = [&](int c, double xi, double eta, double *x, double *J) {
      // J = [[dx/dxi, dx/deta],[dz/dxi, dz/deta]]
      x[0] = x[1] = 0.0;
      J[0] = J[1] = J[2] = J[3] = 0.0;
      for (int b = 0; b < mn; ++b)
        for (int a = 0; a < mn; ++a) {
          const double la = lagrange(mx, a, xi), lb = lagrange(mx, b, eta);
          const double da = lagrange_d(mx, a, xi), db = lagrange_d(mx, b, eta);
          const double *X = nodes + ((long)c * mn * mn + b * mn + a) * 2;
          for (int d = 0; d < 2; ++d) {
            x[d] += X[d] * la * lb;
            J[d * 2 + 0] += X[d] * da * lb;
            J[d * 2 + 1] += X[d] * la * db;
          }
        }
    };
    cJinv.assign((long)nc * nq2 * 4, 0.0);
    cJxW.assign((long)nc * nq2, 0.0);
    cX.assign((long)nc * nq2 * 2, 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c)
      for (int qz = 0; qz < nq; ++qz)
        for (int qx = 0; qx < nq; ++qx) {
          const long q = (long)c * nq2 + qz * nq + qx;
          double x[2], J[4];
          map_eval(c, gx[qx], gx[qz], x, J);
          const double det = J[0] * J[3] - J[1] * J[2];
          cJinv[q * 4 + 0] = J[3] / det;   // dxi/dx
          cJinv[q * 4 + 1] = -J[1] / det;  // dxi/dz
          cJinv[q * 4 + 2] = -J[2] / det;  // deta/dx
          cJinv[q * 4 + 3] = J[0] / det;   // deta/dz
          cJxW[q] = det * gw[qx] * gw[qz];
          cX[q * 2 + 0] = x[0];
          cX[q * 2 + 1] = x[1];
        }
    auto face_geom = [&](int c, int f, int q, double *n, double *jxw) {
      double xi, eta, nr[2];
      const double s = gx[q];
      switch (f) {
        case 0: xi = 0.0; eta = s; nr[0] = -1; nr[1] = 0; break;
        case 1: xi = 1.0; eta = s; nr[0] = 1; nr[1] = 0; break;
        case 2: xi = s; eta = 0.0; nr[0] = 0; nr[1] = -1; break;
        default: xi = s; eta = 1.0; nr[0] = 0; nr[1] = 1; break;
      }
      double x[2], J[4];
      map_eval(c, xi, eta, x, J);
      const double det = J[0] * J[3] - J[1] * J[2];
      const double Ji[4] = {J[3] / det, -J[1] / det, -J[2] / det, J[0] / det};
      // (J^{-T} n_ref)_b = sum_a Jinv[a][b] nr_a
      const double t0 = Ji[0] * nr[0] + Ji[2] * nr[1];
      const double t1 = Ji[1] * nr[0] + Ji[3] * nr[1];
      const double len = std::sqrt(t0 * t0 + t1 * t1);
      n[0] = t0 / len;
      n[1] = t1 / len;
      *jxw = det * len * gw[q];
    };
    nf = n_inner;
    nb = n_bdry;
    inner.assign(inner_faces, inner_faces + 5L * nf);
    bdry.assign(bdry_faces, bdry_faces + 3L * nb);
    fN.assign((long)nf * nq * 2, 0.0);
    fJxW.assign((long)nf * nq, 0.0);
    bN.assign((long)nb * nq * 2, 0.0);
    bJxW.assign((long)nb * nq, 0.0);
#pragma omp parallel for
    for (int f = 0; f < nf; ++f)
      for (int q = 0; q < nq; ++q)
        face_geom(inner[5 * f], inner[5 * f + 1], q, &fN[((long)f * nq + q) * 2],
                  &fJxW[(long)f * nq + q]);
#pragma omp parallel for
    for (int f = 0; f < nb; ++f)
      for (int q = 0; q < nq; ++q)
        face_geom(bdry[3 * f], bdry[3 * f + 1], q, &bN[((long)f * nq + q) * 2],
                  &bJxW[(long)f * nq + q]);
    cface.assign((long)nc * 8 * 3, -1);
    auto slot = [&](int c, int lf) {
      int *e = &cface[((long)c * 4 + lf) * 2 * 3];
      return e[0] < 0 ? e : e + 3;
    };
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[5 * f], fp = inner[5 * f + 1];
      const int cm = inner[5 * f + 2], fm = inner[5 * f + 3];
      int *e = slot(cp, fp);
      e[0] = 0; e[1] = f; e[2] = 0;
      e = slot(cm, fm);
      e[0] = 0; e[1] = f; e[2] = 1;
    }
    for (int f = 0; f < nb; ++f) {
      const int c = bdry[3 * f], lf = bdry[3 * f + 1];
      int *e = slot(c, lf);
      e[0] = 1; e[1] = f; e[2] = 0;
    }
  }

  // ----------------------------------------------------- sum factorisation --
  // nodal values u[nn2] -> values at Gauss points v[nq2]
  void eval(const double *u, double *v) const {
    double t[16 * 16];
    for (int iz = 0; iz < nn; ++iz)
      for (int qx = 0; qx < nq; ++qx) {
        double s = 0.0;
        for (int ix = 0; ix < nn; ++ix) s += S[qx * nn + ix] * u[iz * nn + ix];
        t[iz * nq + qx] = s;
      }
    for (int qz = 0; qz < nq; ++qz)
      for (int qx = 0; qx < nq; ++qx) {
        double s = 0.0;
        for (int iz = 0; iz < nn; ++iz) s += S[qz * nn + iz] * t[iz * nq + qx];
        v[qz * nq + qx] = s;
      }
  }
  // out[nn2] += sum_q V phi_i JxW + (Gx,Gz).grad(phi_i) JxW ; V/G physical,
  // any of V, Gx/Gz may be null.
  void integrate(int c, const double *V, const double *Gx, const double *Gz,
                 double *out) const {
    double Vr[16 * 16], Gxi[16 * 16], Get[16 * 16];
    for (int q = 0; q < nq2; ++q) {
      const long cq = (long)c * nq2 + q;
      const double jxw = cJxW[cq];
      const double *Ji = &cJinv[cq * 4];
      Vr[q] = V ? V[q] * jxw : 0.0;
      if (Gx) {
        Gxi[q] = (Ji[0] * Gx[q] + Ji[1] * Gz[q]) * jxw;
        Get[q] = (Ji[2] * Gx[q] + Ji[3] * Gz[q]) * jxw;
      } else {
        Gxi[q] = Get[q] = 0.0;
      }
    }
    double a[16 * 16], b[16 * 16];
    for (int iz = 0; iz < nn; ++iz)
      for (int qx = 0; qx < nq; ++qx) {
        double sa = 0.0, sb = 0.0;
        for (int qz = 0; qz < nq; ++qz) {
          sa += S[qz * nn + iz] * Vr[qz * nq + qx] + D[qz * nn + iz] * Get[qz * nq + qx];
          sb += S[qz * nn + iz] * Gxi[qz * nq + qx];
        }
        a[iz * nq + qx] = sa;
        b[iz * nq + qx] = sb;
      }
    for (int iz = 0; iz < nn; ++iz)
      for (int ix = 0; ix < nn; ++ix) {
        double s = 0.0;
        for (int qx = 0; qx < nq; ++qx)
          s += S[qx * nn + ix] * a[iz * nq + qx] + D[qx * nn + ix] * b[iz * nq + qx];
        out[iz * nn + ix] += s;
      }
  }
  int face_node(int f, int i) const {
    switch (f) {
      case 0: return i * nn;
      case 1: return i * nn + k;
      case 2: return i;
      default: return k * nn + i;
    }
  }
  // trace at the face points; sub >= 0: at the points of subface `sub`
  void eval_face(const double *u, int f, double *v, int sub = -1) const {
    const double *T = sub < 0 ? S.data() : Sh[sub].data();
    for (int q = 0; q < nq; ++q) {
      double s = 0.0;
      for (int i = 0; i < nn; ++i) s += T[q * nn + i] * u[face_node(f, i)];
      v[q] = s;
    }
  }
  // face contribution buffer entry (nn values) from flux F[q] (JxW included)
  void integrate_face(const double *F, double *out, int sub = -1) const {
    const double *T = sub < 0 ? S.data() : Sh[sub].data();
    for (int i = 0; i < nn; ++i) {
      double s = 0.0;
      for (int q = 0; q < nq; ++q) s += T[q * nn + i] * F[q];
      out[i] = s;
    }
  }

  // ---------------------------------------------------- loop machinery --
  // face buffers: inner [nf][2 sides][ncomp][nn], boundary [nb][ncomp][nn]
  mutable Vec fbuf, bbuf;
  void prep_buffers(int ncomp) const {
    fbuf.assign((long)nf * 2 * ncomp * nn, 0.0);
    bbuf.assign((long)nb * ncomp * nn, 0.0);
  }
  void gather_faces(double *dst, int ncomp) const {
#pragma omp parallel for
    for (int c = 0; c < nc; ++c)
      for (int sl = 0; sl < 8; ++sl) {
        const int lf = sl >> 1;
        const int *e = &cface[((long)c * 8 + sl) * 3];
        if (e[0] < 0) continue;
        for (int comp = 0; comp < ncomp; ++comp) {
          const double *src = e[0] == 0
              ? &fbuf[(((long)e[1] * 2 + e[2]) * ncomp + comp) * nn]
              : &bbuf[((long)e[1] * ncomp + comp) * nn];
          double *d = dst + ((long)c * ncomp + comp) * nn2;
          for (int i = 0; i < nn; ++i) d[face_node(lf, i)] += src[i];
        }
      }
  }
  // helpers to evaluate a source field at the cell / face points
  const double *tile(const double *v, int c, int ncomp, int comp) const {
    return v + ((long)c * ncomp + comp) * nn2;
  }

  // =========================================================================
  // rho rhs: euler_operator.h:344-473 (cell), 478-692 (face), no boundary
  // src: stage1 {rho_old,u_old}; stage2 +{rho_2,u_2}; stage3 +{rho_3,u_3}
  // =========================================================================
  void vmult_rhs_rho_update(double *dst, const double *const *src) const {
    const int nst = hstage;  // number of (rho,u) states used
    double cf[3];
    if (hstage == 1) { cf[0] = a21; }
    else if (hstage == 2) { cf[0] = a31; cf[1] = a32; }
    else { cf[0] = b1; cf[1] = b2; cf[2] = b3; }
    std::fill(dst, dst + ns(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double r[3][256], ux[3][256], uz[3][256];
      for (int j = 0; j < nst; ++j) {
        eval(tile(src[2 * j], c, 1, 0), r[j]);
        eval(tile(src[2 * j + 1], c, 2, 0), ux[j]);
        eval(tile(src[2 * j + 1], c, 2, 1), uz[j]);
      }
      double V[256], Gx[256], Gz[256];
      for (int q = 0; q < nq2; ++q) {
        V[q] = r[0][q];
        double gx = 0.0, gz = 0.0;
        for (int j = 0; j < nst; ++j) {
          gx += cf[j] * dt * r[j][q] * ux[j][q];
          gz += cf[j] * dt * r[j][q] * uz[j][q];
        }
        Gx[q] = gx;
        Gz[q] = gz;
      }
      integrate(c, V, Gx, Gz, dst + (long)c * nn2);
    }
    prep_buffers(1);
#pragma omp parallel for
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[5 * f], fp = inner[5 * f + 1];
      const int cm = inner[5 * f + 2], fm = inner[5 * f + 3];
      const int hs = inner[5 * f + 4] - 1;  // subface of the "-" side, -1 conforming
      double rp[3][16], rm[3][16], uxp[3][16], uxm[3][16], uzp[3][16], uzm[3][16];
      for (int j = 0; j < nst; ++j) {
        eval_face(tile(src[2 * j], cp, 1, 0), fp, rp[j]);
        eval_face(tile(src[2 * j], cm, 1, 0), fm, rm[j], hs);
        eval_face(tile(src[2 * j + 1], cp, 2, 0), fp, uxp[j]);
        eval_face(tile(src[2 * j + 1], cm, 2, 0), fm, uxm[j], hs);
        eval_face(tile(src[2 * j + 1], cp, 2, 1), fp, uzp[j]);
        eval_face(tile(src[2 * j + 1], cm, 2, 1), fm, uzm[j], hs);
      }
      double Fp[16], Fm[16];
      for (int q = 0; q < nq; ++q) {
        const double n0 = fN[((long)f * nq + q) * 2], n1 = fN[((long)f * nq + q) * 2 + 1];
        double flux = 0.0;
        for (int j = 0; j < nst; ++j) {
          const double avg0 = 0.5 * (rp[j][q] * uxp[j][q] + rm[j][q] * uxm[j][q]);
          const double avg1 = 0.5 * (rp[j][q] * uzp[j][q] + rm[j][q] * uzm[j][q]);
          const double lam = std::max(std::fabs(uxp[j][q] * n0 + uzp[j][q] * n1),
                                      std::fabs(uxm[j][q] * n0 + uzm[j][q] * n1));
          const double jump = rp[j][q] - rm[j][q];
          flux += cf[j] * dt * ((avg0 * n0 + avg1 * n1) + 0.5 * lam * jump);
        }
        const double jxw = fJxW[(long)f * nq + q];
        Fp[q] = -flux * jxw;
        Fm[q] = flux * jxw;
      }
      integrate_face(Fp, &fbuf[((long)f * 2 + 0) * nn]);
      integrate_face(Fm, &fbuf[((long)f * 2 + 1) * nn], hs);
    }
    gather_faces(dst, 1);
  }

  // =========================================================================
  // momentum rhs: euler_operator.h:1622-1886 cell, 1891-2184 face,
  // 2189-2305 boundary (wall: p_D = p)
  // src: stage1 {rho_old,u_old,p_old,rho_2}
  //      stage2 {rho_old,u_old,p_old,rho_2,u_2,p_2,rho_3}
  //      stage3 {rho_old,u_old,p_old,rho_2,u_2,p_2,rho_3,u_3,p_3}
  // =========================================================================
  void vmult_rhs_velocity_fixed(double *dst, const double *const *src) const {
    int nst;            // number of full (rho,u,p) states in the flux terms
    double ca[3], ct[3];  // explicit (a) and implicit-explicit (a~) weights
    double cg[3];         // gravity weights
    const double *grho[3];  // densities in the gravity terms (per cell tile)
    int ng;
    if (hstage == 1) {
      nst = 1; ca[0] = a21; ct[0] = a21_tilde;
      ng = 2; cg[0] = a21_tilde; cg[1] = a22_tilde;
      grho[0] = src[0]; grho[1] = src[3];
    } else if (hstage == 2) {
      nst = 2; ca[0] = a31; ca[1] = a32; ct[0] = a31_tilde; ct[1] = a32_tilde;
      ng = 3; cg[0] = a31_tilde; cg[1] = a32_tilde; cg[2] = a33_tilde;
      grho[0] = src[0]; grho[1] = src[3]; grho[2] = src[6];
    } else {
      nst = 3; ca[0] = b1; ca[1] = b2; ca[2] = b3; ct[0] = b1; ct[1] = b2; ct[2] = b3;
      ng = 3; cg[0] = b1; cg[1] = b2; cg[2] = b3;
      grho[0] = src[0]; grho[1] = src[3]; grho[2] = src[6];
    }
    std::fill(dst, dst + nv(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double r[3][256], ux[3][256], uz[3][256], p[3][256], rg[3][256];
      for (int j = 0; j < nst; ++j) {
        eval(tile(src[3 * j], c, 1, 0), r[j]);
        eval(tile(src[3 * j + 1], c, 2, 0), ux[j]);
        eval(tile(src[3 * j + 1], c, 2, 1), uz[j]);
        eval(tile(src[3 * j + 2], c, 1, 0), p[j]);
      }
      for (int j = 0; j < ng; ++j) eval(tile(grho[j], c, 1, 0), rg[j]);
      double V0[256], V1[256], G00[256], G01[256], G10[256], G11[256];
      for (int q = 0; q < nq2; ++q) {
        // submit_value: rho_old u_old - sum cg dt/Fr^2 rho e_z
        double v0 = r[0][q] * ux[0][q], v1 = r[0][q] * uz[0][q];
        for (int j = 0; j < ng; ++j) v1 -= cg[j] * dt / (Fr * Fr) * rg[j][q];
        V0[q] = v0;
        V1[q] = v1;
        // submit_gradient: sum ca dt rho u (x) u + ct dt/Ma^2 p I
        double g00 = 0, g01 = 0, g10 = 0, g11 = 0;
        for (int j = 0; j < nst; ++j) {
          const double ru0 = ca[j] * dt * r[j][q] * ux[j][q];
          const double ru1 = ca[j] * dt * r[j][q] * uz[j][q];
          const double pp = ct[j] * dt / (Ma * Ma) * p[j][q];
          g00 += ru0 * ux[j][q] + pp;
          g01 += ru0 * uz[j][q];
          g10 += ru1 * ux[j][q];
          g11 += ru1 * uz[j][q] + pp;
        }
        G00[q] = g00; G01[q] = g01; G10[q] = g10; G11[q] = g11;
      }
      integrate(c, V0, G00, G01, dst + ((long)c * 2 + 0) * nn2);
      integrate(c, V1, G10, G11, dst + ((long)c * 2 + 1) * nn2);
    }
    prep_buffers(2);
#pragma omp parallel for
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[5 * f], fp = inner[5 * f + 1];
      const int cm = inner[5 * f + 2], fm = inner[5 * f + 3];
      const int hs = inner[5 * f + 4] - 1;  // subface of the "-" side, -1 conforming
      double rp[3][16], rm[3][16], uxp[3][16], uxm[3][16], uzp[3][16], uzm[3][16],
          pp_[3][16], pm[3][16];
      for (int j = 0; j < nst; ++j) {
        eval_face(tile(src[3 * j], cp, 1, 0), fp, rp[j]);
        eval_face(tile(src[3 * j], cm, 1, 0), fm, rm[j], hs);
        eval_face(tile(src[3 * j + 1], cp, 2, 0), fp, uxp[j]);
        eval_face(tile(src[3 * j + 1], cm, 2, 0), fm, uxm[j], hs);
        eval_face(tile(src[3 * j + 1], cp, 2, 1), fp, uzp[j]);
        eval_face(tile(src[3 * j + 1], cm, 2, 1), fm, uzm[j], hs);
        eval_face(tile(src[3 * j + 2], cp, 1, 0), fp, pp_[j]);
        eval_face(tile(src[3 * j + 2], cm, 1, 0), fm, pm[j], hs);
      }
      double Fp0[16], Fp1[16], Fm0[16], Fm1[16];
      for (int q = 0; q < nq; ++q) {
        const double n0 = fN[((long)f * nq + q) * 2], n1 = fN[((long)f * nq + q) * 2 + 1];
        double f0 = 0.0, f1 = 0.0;
        for (int j = 0; j < nst; ++j) {
          // avg of rho u (x) u, contracted with n
          const double unp = uxp[j][q] * n0 + uzp[j][q] * n1;
          const double unm = uxm[j][q] * n0 + uzm[j][q] * n1;
          const double at0 = 0.5 * (rp[j][q] * uxp[j][q] * unp + rm[j][q] * uxm[j][q] * unm);
          const double at1 = 0.5 * (rp[j][q] * uzp[j][q] * unp + rm[j][q] * uzm[j][q] * unm);
          const double avgp = 0.5 * (pp_[j][q] + pm[j][q]);
          const double lam = std::max(std::fabs(unp), std::fabs(unm));
          const double j0 = rp[j][q] * uxp[j][q] - rm[j][q] * uxm[j][q];
          const double j1 = rp[j][q] * uzp[j][q] - rm[j][q] * uzm[j][q];
          f0 += ca[j] * dt * at0 + ct[j] * dt / (Ma * Ma) * avgp * n0 + ca[j] * dt * 0.5 * lam * j0;
          f1 += ca[j] * dt * at1 + ct[j] * dt / (Ma * Ma) * avgp * n1 + ca[j] * dt * 0.5 * lam * j1;
        }
        const double jxw = fJxW[(long)f * nq + q];
        Fp0[q] = -f0 * jxw; Fp1[q] = -f1 * jxw;
        Fm0[q] = f0 * jxw;  Fm1[q] = f1 * jxw;
      }
      integrate_face(Fp0, &fbuf[(((long)f * 2 + 0) * 2 + 0) * nn]);
      integrate_face(Fp1, &fbuf[(((long)f * 2 + 0) * 2 + 1) * nn]);
      integrate_face(Fm0, &fbuf[(((long)f * 2 + 1) * 2 + 0) * nn], hs);
      integrate_face(Fm1, &fbuf[(((long)f * 2 + 1) * 2 + 1) * nn], hs);
    }
#pragma omp parallel for
    for (int f = 0; f < nb; ++f) {
      const int c = bdry[3 * f], lf = bdry[3 * f + 1];
      double pb[3][16];
      for (int j = 0; j < nst; ++j) eval_face(tile(src[3 * j + 2], c, 1, 0), lf, pb[j]);
      double F0[16], F1[16];
      for (int q = 0; q < nq; ++q) {
        const double n0 = bN[((long)f * nq + q) * 2], n1 = bN[((long)f * nq + q) * 2 + 1];
        double f0 = 0.0, f1 = 0.0;
        for (int j = 0; j < nst; ++j) {
          const double avg = 0.5 * (pb[j][q] + pb[j][q]);  // p_D = p
          f0 -= ct[j] * dt / (Ma * Ma) * avg * n0;
          f1 -= ct[j] * dt / (Ma * Ma) * avg * n1;
        }
        const double jxw = bJxW[(long)f * nq + q];
        F0[q] = f0 * jxw;
        F1[q] = f1 * jxw;
      }
      integrate_face(F0, &bbuf[((long)f * 2 + 0) * nn]);
      integrate_face(F1, &bbuf[((long)f * 2 + 1) * nn]);
    }
    gather_faces(dst, 2);
  }

  // =========================================================================
  // energy rhs for p: euler_operator.h:745-1007 cell, 1012-1361 face
  // src: stage1 {rho_old,u_old,p_old,rho_2,u_fix}
  //      stage2 {rho_old,u_old,p_old,rho_2,u_2,p_2,rho_3,u_fix}
  //      stage3 {rho_old,u_old,p_old,rho_2,u_2,p_2,rho_3,u_3,p_3,rho_cur,u_cur}
  // =========================================================================
  void vmult_rhs_pressure(double *dst, const double *const *src) const {
    const double gm1 = GAMMA_GAS - 1.0;
    const double M2 = Ma * Ma;
    int nst;
    double ca[3], ct[3];
    // gravity work terms: weight, density, velocity
    int ng;
    double cg[3];
    const double *grho[3], *gu[3];
    const double *kin_rho, *kin_u;  // -1/2 rho Ma^2 |u_fix|^2
    if (hstage == 1) {
      nst = 1; ca[0] = a21; ct[0] = a21_tilde;
      ng = 2; cg[0] = a21_tilde; cg[1] = a22_tilde;
      grho[0] = src[0]; gu[0] = src[1]; grho[1] = src[3]; gu[1] = src[4];
      kin_rho = src[3]; kin_u = src[4];
    } else if (hstage == 2) {
      nst = 2; ca[0] = a31; ca[1] = a32; ct[0] = a31_tilde; ct[1] = a32_tilde;
      ng = 3; cg[0] = a31_tilde; cg[1] = a32_tilde; cg[2] = a33_tilde;
      grho[0] = src[0]; gu[0] = src[1]; grho[1] = src[3]; gu[1] = src[4];
      grho[2] = src[6]; gu[2] = src[7];
      kin_rho = src[6]; kin_u = src[7];
    } else {
      nst = 3; ca[0] = b1; ca[1] = b2; ca[2] = b3; ct[0] = b1; ct[1] = b2; ct[2] = b3;
      ng = 3; cg[0] = b1; cg[1] = b2; cg[2] = b3;
      grho[0] = src[0]; gu[0] = src[1]; grho[1] = src[3]; gu[1] = src[4];
      grho[2] = src[6]; gu[2] = src[7];
      kin_rho = src[9]; kin_u = src[10];
    }
    std::fill(dst, dst + ns(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double r[3][256], ux[3][256], uz[3][256], p[3][256];
      for (int j = 0; j < nst; ++j) {
        eval(tile(src[3 * j], c, 1, 0), r[j]);
        eval(tile(src[3 * j + 1], c, 2, 0), ux[j]);
        eval(tile(src[3 * j + 1], c, 2, 1), uz[j]);
        eval(tile(src[3 * j + 2], c, 1, 0), p[j]);
      }
      double gr[3][256], guz[3][256], kr[256], kux[256], kuz[256];
      for (int j = 0; j < ng; ++j) {
        eval(tile(grho[j], c, 1, 0), gr[j]);
        eval(tile(gu[j], c, 2, 1), guz[j]);  // only u.e_z is needed
      }
      eval(tile(kin_rho, c, 1, 0), kr);
      eval(tile(kin_u, c, 2, 0), kux);
      eval(tile(kin_u, c, 2, 1), kuz);
      double V[256], Gx[256], Gz[256];
      for (int q = 0; q < nq2; ++q) {
        const double uu0 = ux[0][q] * ux[0][q] + uz[0][q] * uz[0][q];
        const double E0 = 1.0 / gm1 * (p[0][q] / r[0][q]) + 0.5 * M2 * uu0;
        double v = r[0][q] * E0 - 0.5 * kr[q] * M2 * (kux[q] * kux[q] + kuz[q] * kuz[q]);
        for (int j = 0; j < ng; ++j) v -= cg[j] * dt * M2 / (Fr * Fr) * gr[j][q] * guz[j][q];
        V[q] = v;
        double gx = 0.0, gz = 0.0;
        for (int j = 0; j < nst; ++j) {
          const double uu = ux[j][q] * ux[j][q] + uz[j][q] * uz[j][q];
          const double Ej = 1.0 / gm1 * (p[j][q] / r[j][q]) + 0.5 * M2 * uu;
          const double kin = 0.5 * ca[j] * dt * M2 * uu * r[j][q];
          const double ent = ct[j] * dt * (r[j][q] * (Ej - 0.5 * M2 * uu) + p[j][q]);
          gx += kin * ux[j][q] + ent * ux[j][q];
          gz += kin * uz[j][q] + ent * uz[j][q];
        }
        Gx[q] = gx;
        Gz[q] = gz;
      }
      integrate(c, V, Gx, Gz, dst + (long)c * nn2);
    }
    prep_buffers(1);
#pragma omp parallel for
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[5 * f], fp = inner[5 * f + 1];
      const int cm = inner[5 * f + 2], fm = inner[5 * f + 3];
      const int hs = inner[5 * f + 4] - 1;  // subface of the "-" side, -1 conforming
      double rp[3][16], rm[3][16], uxp[3][16], uxm[3][16], uzp[3][16], uzm[3][16],
          pp_[3][16], pm[3][16];
      for (int j = 0; j < nst; ++j) {
        eval_face(tile(src[3 * j], cp, 1, 0), fp, rp[j]);
        eval_face(tile(src[3 * j], cm, 1, 0), fm, rm[j], hs);
        eval_face(tile(src[3 * j + 1], cp, 2, 0), fp, uxp[j]);
        eval_face(tile(src[3 * j + 1], cm, 2, 0), fm, uxm[j], hs);
        eval_face(tile(src[3 * j + 1], cp, 2, 1), fp, uzp[j]);
        eval_face(tile(src[3 * j + 1], cm, 2, 1), fm, uzm[j], hs);
        eval_face(tile(src[3 * j + 2], cp, 1, 0), fp, pp_[j]);
        eval_face(tile(src[3 * j + 2], cm, 1, 0), fm, pm[j], hs);
      }
      double Fp[16], Fm[16];
      for (int q = 0; q < nq; ++q) {
        const double n0 = fN[((long)f * nq + q) * 2], n1 = fN[((long)f * nq + q) * 2 + 1];
        double flux = 0.0;
        for (int j = 0; j < nst; ++j) {
          const double uup = uxp[j][q] * uxp[j][q] + uzp[j][q] * uzp[j][q];
          const double uum = uxm[j][q] * uxm[j][q] + uzm[j][q] * uzm[j][q];
          const double unp = uxp[j][q] * n0 + uzp[j][q] * n1;
          const double unm = uxm[j][q] * n0 + uzm[j][q] * n1;
          // avg kinetic flux . n
          const double akin = 0.5 * (0.5 * uup * rp[j][q] * unp + 0.5 * uum * rm[j][q] * unm);
          const double Ep = 1.0 / gm1 * pp_[j][q] / rp[j][q] + 0.5 * M2 * uup;
          const double Em = 1.0 / gm1 * pm[j][q] / rm[j][q] + 0.5 * M2 * uum;
          const double hp = (Ep - 0.5 * M2 * uup) * rp[j][q] + pp_[j][q];
          const double hm = (Em - 0.5 * M2 * uum) * rm[j][q] + pm[j][q];
          const double aent = 0.5 * (hp * unp + hm * unm);
          const double lam = std::max(std::fabs(unp), std::fabs(unm));
          if (hstage == 3) {
            // stage 3 jumps total rho E (euler_operator.h:1290,1313,1336)
            const double jE = rp[j][q] * Ep - rm[j][q] * Em;
            flux += ca[j] * dt * M2 * akin + ca[j] * dt * aent + ca[j] * dt * 0.5 * lam * jE;
          } else {
            double jkin;
            if (hstage == 2 && j == 1) {
              // quirk kept: the tmp_2 kinetic jump mixes in u_old
              // (euler_operator.h:1182-1183)
              jkin = rp[1][q] * 0.5 * (uxp[1][q] * uxp[0][q] + uzp[1][q] * uzp[0][q]) -
                     rm[1][q] * 0.5 * (uxm[1][q] * uxm[0][q] + uzm[1][q] * uzm[0][q]);
            } else {
              jkin = rp[j][q] * 0.5 * uup - rm[j][q] * 0.5 * uum;
            }
            const double je = rp[j][q] * (Ep - 0.5 * M2 * uup) - rm[j][q] * (Em - 0.5 * M2 * uum);
            flux += ca[j] * dt * M2 * (akin + 0.5 * lam * jkin) + ct[j] * dt * (aent + 0.5 * lam * je);
          }
        }
        const double jxw = fJxW[(long)f * nq + q];
        Fp[q] = -flux * jxw;
        Fm[q] = flux * jxw;
      }
      integrate_face(Fp, &fbuf[((long)f * 2 + 0) * nn]);
      integrate_face(Fm, &fbuf[((long)f * 2 + 1) * nn], hs);
    }
    gather_faces(dst, 1);
  }

  double implicit_coeff() const { return hstage == 1 ? a22_tilde : a33_tilde; }

  // =========================================================================
  // B = vmult_pressure: euler_operator.h:1512-1617, 2422-2435
  // =========================================================================
  void vmult_pressure(double *dst, const double *src) const {
    const double co = implicit_coeff() * dt / (Ma * Ma);
    std::fill(dst, dst + nv(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double p[256], G[256], Z[256];
      eval(tile(src, c, 1, 0), p);
      for (int q = 0; q < nq2; ++q) { G[q] = -co * p[q]; Z[q] = 0.0; }
      // submit_divergence(s): component 0 tested with d/dx, component 1 with d/dz
      integrate(c, nullptr, G, Z, dst + ((long)c * 2 + 0) * nn2);
      integrate(c, nullptr, Z, G, dst + ((long)c * 2 + 1) * nn2);
    }
    prep_buffers(2);
#pragma omp parallel for
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[5 * f], fp = inner[5 * f + 1];
      const int cm = inner[5 * f + 2], fm = inner[5 * f + 3];
      const int hs = inner[5 * f + 4] - 1;  // subface of the "-" side, -1 conforming
      double pp_[16], pm[16];
      eval_face(tile(src, cp, 1, 0), fp, pp_);
      eval_face(tile(src, cm, 1, 0), fm, pm, hs);
      double Fp0[16], Fp1[16], Fm0[16], Fm1[16];
      for (int q = 0; q < nq; ++q) {
        const double n0 = fN[((long)f * nq + q) * 2], n1 = fN[((long)f * nq + q) * 2 + 1];
        const double avg = 0.5 * (pp_[q] + pm[q]);
        const double jxw = fJxW[(long)f * nq + q];
        Fp0[q] = co * avg * n0 * jxw; Fp1[q] = co * avg * n1 * jxw;
        Fm0[q] = -co * avg * n0 * jxw; Fm1[q] = -co * avg * n1 * jxw;
      }
      integrate_face(Fp0, &fbuf[(((long)f * 2 + 0) * 2 + 0) * nn]);
      integrate_face(Fp1, &fbuf[(((long)f * 2 + 0) * 2 + 1) * nn]);
      integrate_face(Fm0, &fbuf[(((long)f * 2 + 1) * 2 + 0) * nn], hs);
      integrate_face(Fm1, &fbuf[(((long)f * 2 + 1) * 2 + 1) * nn], hs);
    }
#pragma omp parallel for
    for (int f = 0; f < nb; ++f) {
      const int c = bdry[3 * f], lf = bdry[3 * f + 1];
      double pb[16], F0[16], F1[16];
      eval_face(tile(src, c, 1, 0), lf, pb);
      for (int q = 0; q < nq; ++q) {
        const double n0 = bN[((long)f * nq + q) * 2], n1 = bN[((long)f * nq + q) * 2 + 1];
        const double jxw = bJxW[(long)f * nq + q];
        const double pD = pb[q];
        F0[q] = co * 0.5 * (pb[q] + pD) * n0 * jxw;
        F1[q] = co * 0.5 * (pb[q] + pD) * n1 * jxw;
      }
      integrate_face(F0, &bbuf[((long)f * 2 + 0) * nn]);
      integrate_face(F1, &bbuf[((long)f * 2 + 1) * nn]);
    }
    gather_faces(dst, 2);
  }

  // =========================================================================
  // C = vmult_enthalpy: euler_operator.h:1413-1507, 2440-2453 (uses pres_fixed)
  // =========================================================================
  void vmult_enthalpy(double *dst, const double *src) const {
    const double co = implicit_coeff();
    const double hg = GAMMA_GAS / (GAMMA_GAS - 1.0);
    std::fill(dst, dst + ns(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double pf[256], wx[256], wz[256], Gx[256], Gz[256];
      eval(tile(pres_fixed.data(), c, 1, 0), pf);
      eval(tile(src, c, 2, 0), wx);
      eval(tile(src, c, 2, 1), wz);
      for (int q = 0; q < nq2; ++q) {
        Gx[q] = -co * dt * hg * pf[q] * wx[q];
        Gz[q] = -co * dt * hg * pf[q] * wz[q];
      }
      integrate(c, nullptr, Gx, Gz, dst + (long)c * nn2);
    }
    prep_buffers(1);
#pragma omp parallel for
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[5 * f], fp = inner[5 * f + 1];
      const int cm = inner[5 * f + 2], fm = inner[5 * f + 3];
      const int hs = inner[5 * f + 4] - 1;  // subface of the "-" side, -1 conforming
      double pfp[16], pfm[16], wxp[16], wxm[16], wzp[16], wzm[16];
      eval_face(tile(pres_fixed.data(), cp, 1, 0), fp, pfp);
      eval_face(tile(pres_fixed.data(), cm, 1, 0), fm, pfm, hs);
      eval_face(tile(src, cp, 2, 0), fp, wxp);
      eval_face(tile(src, cm, 2, 0), fm, wxm, hs);
      eval_face(tile(src, cp, 2, 1), fp, wzp);
      eval_face(tile(src, cm, 2, 1), fm, wzm, hs);
      double Fp[16], Fm[16];
      for (int q = 0; q < nq; ++q) {
        const double n0 = fN[((long)f * nq + q) * 2], n1 = fN[((long)f * nq + q) * 2 + 1];
        const double av0 = 0.5 * hg * (pfp[q] * wxp[q] + pfm[q] * wxm[q]);
        const double av1 = 0.5 * hg * (pfp[q] * wzp[q] + pfm[q] * wzm[q]);
        const double lam = std::max(std::fabs(wxp[q] * n0 + wzp[q] * n1),
                                    std::fabs(wxm[q] * n0 + wzm[q] * n1));
        const double je = 1.0 / (GAMMA_GAS - 1.0) * (pfp[q] - pfm[q]);
        const double flux = co * dt * ((av0 * n0 + av1 * n1) + 0.5 * lam * je);
        const double jxw = fJxW[(long)f * nq + q];
        Fp[q] = flux * jxw;
        Fm[q] = -flux * jxw;
      }
      integrate_face(Fp, &fbuf[((long)f * 2 + 0) * nn]);
      integrate_face(Fm, &fbuf[((long)f * 2 + 1) * nn], hs);
    }
    gather_faces(dst, 1);
  }

  // ----------------------------------------------------- mass operators --
  // dst += sum_q w(q) src phi_i JxW ; w from weight tile or constant
  void mass_add(double *dst, const double *src, int ncomp, const double *weight,
                double scale) const {
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double wq[256], v[256];
      if (weight) eval(tile(weight, c, 1, 0), wq);
      for (int comp = 0; comp < ncomp; ++comp) {
        eval(tile(src, c, ncomp, comp), v);
        for (int q = 0; q < nq2; ++q) v[q] = (weight ? wq[q] * v[q] : scale * v[q]);
        integrate(c, v, nullptr, nullptr, dst + ((long)c * ncomp + comp) * nn2);
      }
    }
  }
  long vsize() const {  // size of the vector the current NS stage acts on
    if (nsstage == 3 || nsstage == 5) return nv();
    return ns();
  }

  // Base::vmult -> apply_add (euler_operator.h:2366-2417), dst overwritten
  void vmult(double *dst, const double *src) {
    std::fill(dst, dst + vsize(), 0.0);
    if (nsstage == 1 || nsstage == 4) {
      mass_add(dst, src, 1, nullptr, 1.0);
    } else if (nsstage == 2) {
      mass_add(dst, src, 1, nullptr, 1.0 / (GAMMA_GAS - 1.0));
      Vec tmp1(nv()), tmp2(nv(), 0.0), tmp3(ns());
      vmult_pressure(tmp1.data(), src);
      nsstage = 3;
      Vec dinv = diagonal_inverse();
      const double tol = inner_cg_tol * norm2(tmp1);
      int its = 0;
      cg(tmp2, tmp1, tol, 10000, dinv, &its);
      inner_cg_iters += its;
      vmult_enthalpy(tmp3.data(), tmp2.data());
      for (long i = 0; i < ns(); ++i) dst[i] -= tmp3[i];
      nsstage = 2;
    } else if (nsstage == 3 || nsstage == 5) {
      mass_add(dst, src, 2, rho_for_fixed.data(), 1.0);
    } else {
      mass_add(dst, src, 1, nullptr, 1.0 / (GAMMA_GAS - 1.0));
    }
  }

  // compute_diagonal (euler_operator.h:2591-2626): inverse of the diagonal
  Vec diagonal_inverse() const {
    const bool vel = !(nsstage == 1 || nsstage == 4 || nsstage == 2 || nsstage == 6);
    const int ncomp = vel ? 2 : 1;
    const double scale = (nsstage == 2 || nsstage == 6) ? 1.0 / (GAMMA_GAS - 1.0) : 1.0;
    Vec d((long)nc * ncomp * nn2, 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double wq[256];
      if (vel) eval(tile(rho_for_fixed.data(), c, 1, 0), wq);
      for (int iz = 0; iz < nn; ++iz)
        for (int ix = 0; ix < nn; ++ix) {
          double s = 0.0;
          for (int qz = 0; qz < nq; ++qz)
            for (int qx = 0; qx < nq; ++qx) {
              const int q = qz * nq + qx;
              const double ph = S[qz * nn + iz] * S[qx * nn + ix];
              const double w = vel ? wq[q] : scale;
              s += w * ph * ph * cJxW[(long)c * nq2 + q];
            }
          for (int comp = 0; comp < ncomp; ++comp)
            d[((long)c * ncomp + comp) * nn2 + iz * nn + ix] = 1.0 / s;
        }
    }
    return d;
  }

  // ------------------------------------------------------------- solvers --
  // preconditioned CG with Jacobi, deal.II SolverCG stopping rule |r| <= tol
  int cg(Vec &x, const Vec &b, double tol, int maxit, const Vec &dinv, int *its) {
    const long n = (long)x.size();
    Vec r(n), z(n), p(n), v(n);
    vmult(v.data(), x.data());
    for (long i = 0; i < n; ++i) r[i] = b[i] - v[i];
    double res = norm2(r);
    *its = 0;
    if (res <= tol) return 0;
    for (long i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
    p = z;
    double rz = dot(r, z);
    for (int it = 1; it <= maxit; ++it) {
      vmult(v.data(), p.data());
      const double alpha = rz / dot(p, v);
      axpy(alpha, p, x);
      axpy(-alpha, v, r);
      res = norm2(r);
      *its = it;
      if (res <= tol) return 0;
      for (long i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
      const double rz2 = dot(r, z);
      const double beta = rz2 / rz;
      rz = rz2;
#pragma omp parallel for
      for (long i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    return 1;
  }

  // restarted GMRES, left Jacobi preconditioning, classical Gram-Schmidt
  // with one re-orthogonalisation pass, Givens rotations; stops when the
  // preconditioned residual estimate <= tol (deal.II SolverGMRES with
  // right_preconditioning=false, restart length max_n_tmp_vectors-2 = 28).
  int gmres(Vec &x, const Vec &b, double tol, int maxit, int restart,
            const Vec &dinv, int *its) {
    const long n = (long)x.size();
    const int mdim = restart;
    std::vector<Vec> V(mdim + 1, Vec(n));
    Vec w(n), t(n);
    std::vector<double> H((mdim + 1) * mdim), cs(mdim), sn(mdim), g(mdim + 1), y(mdim);
    *its = 0;
    for (;;) {
      vmult(t.data(), x.data());
      for (long i = 0; i < n; ++i) V[0][i] = dinv[i] * (b[i] - t[i]);
      const double beta = norm2(V[0]);
      if (beta <= tol) return 0;
      if (*its >= maxit) return 1;
      for (long i = 0; i < n; ++i) V[0][i] /= beta;
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int jend = 0;
      bool done = false;
      for (int j = 0; j < mdim; ++j) {
        ++*its;
        vmult(t.data(), V[j].data());
        for (long i = 0; i < n; ++i) w[i] = dinv[i] * t[i];
        for (int pass = 0; pass < 2; ++pass) {
          std::vector<double> h(j + 1);
          for (int l = 0; l <= j; ++l) h[l] = dot(V[l], w);
          for (int l = 0; l <= j; ++l) axpy(-h[l], V[l], w);
          for (int l = 0; l <= j; ++l) {
            if (pass == 0) H[l * mdim + j] = h[l];
            else H[l * mdim + j] += h[l];
          }
        }
        const double hn = norm2(w);
        H[(j + 1) * mdim + j] = hn;
        for (int l = 0; l < j; ++l) {
          const double a = H[l * mdim + j], bb = H[(l + 1) * mdim + j];
          H[l * mdim + j] = cs[l] * a + sn[l] * bb;
          H[(l + 1) * mdim + j] = -sn[l] * a + cs[l] * bb;
        }
        const double a = H[j * mdim + j], bb = H[(j + 1) * mdim + j];
        const double r = std::sqrt(a * a + bb * bb);
        cs[j] = a / r;
        sn[j] = bb / r;
        H[j * mdim + j] = r;
        H[(j + 1) * mdim + j] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        jend = j + 1;
        const double res = std::fabs(g[j + 1]);
        if (hn > 0.0)
          for (long i = 0; i < n; ++i) V[j + 1][i] = w[i] / hn;
        if (res <= tol || hn == 0.0 || *its >= maxit) { done = true; break; }
      }
      for (int l = jend - 1; l >= 0; --l) {
        double s = g[l];
        for (int mm = l + 1; mm < jend; ++mm) s -= H[l * mdim + mm] * y[mm];
        y[l] = s / H[l * mdim + l];
      }
      for (int l = 0; l < jend; ++l) axpy(y[l], V[l], x);
      if (done && !true_residual_check) {
        // report convergence on the estimate used for stopping
        const double res = std::fabs(g[jend]);
        return res <= tol ? 0 : (*its >= maxit ? 1 : 0);
      }
    }
  }
};

// ============================================================================
// Time loop: EulerSolver::run and stage solvers (Atmospheric_Flow.cc)
// ============================================================================
struct Solver {
  Oracle op;
  double eps = 1e-8;   // parameter-file.prm:23
  int max_its = 30000;  // parameter-file.prm:22
  int restart = 28;
  double time = 0.0;
  int n = 0;
  Vec rho_old, rho_tmp_2, rho_tmp_3, rho_curr, rhs_rho;
  Vec u_old, u_tmp_2, u_tmp_3, u_curr, u_fixed, rhs_u, tmp_1;
  Vec pres_old, pres_tmp_2, pres_tmp_3, pres_fixed, pres_fixed_old, rhs_pres;
  Vec sponge_alpha;  // per scalar node relaxation rate (0 = no sponge)
  double ubg0 = 0.0, ubg1 = 0.0;
  // statistics
  long picard_total = 0, gmres_total = 0, cg_total = 0, solve_fail = 0;
  int last_picard[2] = {0, 0};

  void init_vectors() {
    const long s = op.ns(), v = op.nv();
    for (Vec *x : {&rho_old, &rho_tmp_2, &rho_tmp_3, &rho_curr, &rhs_rho, &pres_old,
                   &pres_tmp_2, &pres_tmp_3, &pres_fixed, &pres_fixed_old, &rhs_pres})
      x->assign(s, 0.0);
    for (Vec *x : {&u_old, &u_tmp_2, &u_tmp_3, &u_curr, &u_fixed, &rhs_u, &tmp_1})
      x->assign(v, 0.0);
    op.rho_for_fixed.assign(s, 0.0);
    op.pres_fixed.assign(s, 0.0);
    op.u_fixed.assign(v, 0.0);
    sponge_alpha.assign(s, 0.0);
  }

  void solve_cg(Vec &x, const Vec &b, double tol) {
    Vec dinv = op.diagonal_inverse();
    int its = 0;
    if (op.cg(x, b, tol, max_its, dinv, &its)) ++solve_fail;
    cg_total += its;
  }

  // Atmospheric_Flow.cc:430-537
  void update_density() {
    op.nsstage = 1;
    if (op.hstage == 1) {
      const double *s[] = {rho_old.data(), u_old.data()};
      op.vmult_rhs_rho_update(rhs_rho.data(), s);
    } else if (op.hstage == 2) {
      const double *s[] = {rho_old.data(), u_old.data(), rho_tmp_2.data(), u_tmp_2.data()};
      op.vmult_rhs_rho_update(rhs_rho.data(), s);
    } else {
      op.nsstage = 4;
      const double *s[] = {rho_old.data(), u_old.data(), rho_tmp_2.data(),
                           u_tmp_2.data(), rho_tmp_3.data(), u_tmp_3.data()};
      op.vmult_rhs_rho_update(rhs_rho.data(), s);
    }
    const double tol = eps * norm2(rhs_rho);
    if (op.hstage == 1) { rho_tmp_2 = rho_old; solve_cg(rho_tmp_2, rhs_rho, tol); }
    else if (op.hstage == 2) { rho_tmp_3 = rho_tmp_2; solve_cg(rho_tmp_3, rhs_rho, tol); }
    else { rho_curr = rho_tmp_3; solve_cg(rho_curr, rhs_rho, tol); }
  }

  // Atmospheric_Flow.cc:544-673
  void pressure_fixed_point() {
    op.nsstage = 2;
    op.pres_fixed = pres_fixed_old;
    op.u_fixed = u_fixed;
    if (op.hstage == 1) {
      const double *sp[] = {rho_old.data(), u_old.data(), pres_old.data(), rho_tmp_2.data(),
                            u_fixed.data()};
      op.vmult_rhs_pressure(rhs_pres.data(), sp);
      const double *su[] = {rho_old.data(), u_old.data(), pres_old.data(), rho_tmp_2.data()};
      op.vmult_rhs_velocity_fixed(rhs_u.data(), su);
    } else {
      const double *sp[] = {rho_old.data(), u_old.data(), pres_old.data(), rho_tmp_2.data(),
                            u_tmp_2.data(), pres_tmp_2.data(), rho_tmp_3.data(),
                            u_fixed.data()};
      op.vmult_rhs_pressure(rhs_pres.data(), sp);
      const double *su[] = {rho_old.data(), u_old.data(), pres_old.data(), rho_tmp_2.data(),
                            u_tmp_2.data(), pres_tmp_2.data(), rho_tmp_3.data()};
      op.vmult_rhs_velocity_fixed(rhs_u.data(), su);
    }
    op.nsstage = 3;
    solve_cg(tmp_1, rhs_u, 1e-12 * norm2(rhs_u));
    Vec tmp_2(op.ns());
    op.vmult_enthalpy(tmp_2.data(), tmp_1.data());
    axpy(-1.0, tmp_2, rhs_pres);
    op.nsstage = 2;
    Vec dinv = op.diagonal_inverse();
    double tol = eps * norm2(rhs_pres);
    if (op.schur_tol_preconditioned) {
      Vec pb(rhs_pres.size());
      for (size_t i = 0; i < pb.size(); ++i) pb[i] = dinv[i] * rhs_pres[i];
      tol = eps * norm2(pb);
    }
    pres_fixed = pres_fixed_old;
    int its = 0;
    if (op.gmres(pres_fixed, rhs_pres, tol, max_its, restart, dinv, &its)) ++solve_fail;
    gmres_total += its;
  }

  // Atmospheric_Flow.cc:680-781
  void update_velocity() {
    if (op.hstage == 1 || op.hstage == 2) {
      op.nsstage = 3;
      Vec tmp_3(op.nv());
      op.vmult_pressure(tmp_3.data(), pres_fixed.data());
      axpy(-1.0, tmp_3, rhs_u);
    } else {
      op.nsstage = 5;
      const double *su[] = {rho_old.data(), u_old.data(), pres_old.data(),
                            rho_tmp_2.data(), u_tmp_2.data(), pres_tmp_2.data(),
                            rho_tmp_3.data(), u_tmp_3.data(), pres_tmp_3.data()};
      op.vmult_rhs_velocity_fixed(rhs_u.data(), su);
    }
    const double tol = eps * norm2(rhs_u);
    if (op.hstage == 1 || op.hstage == 2) solve_cg(u_fixed, rhs_u, tol);
    else { u_curr = u_tmp_3; solve_cg(u_curr, rhs_u, tol); }
  }

  // Atmospheric_Flow.cc:788-871
  void update_pressure() {
    op.nsstage = 6;
    const double *sp[] = {rho_old.data(), u_old.data(), pres_old.data(),
                          rho_tmp_2.data(), u_tmp_2.data(), pres_tmp_2.data(),
                          rho_tmp_3.data(), u_tmp_3.data(), pres_tmp_3.data(),
                          rho_curr.data(), u_curr.data()};
    op.vmult_rhs_pressure(rhs_pres.data(), sp);
    const double tol = eps * norm2(rhs_pres);
    pres_old = pres_tmp_3;
    solve_cg(pres_old, rhs_pres, tol);
  }

  int picard(int which) {
    int iters = 0;
    for (int iter = 0; iter < 100; ++iter) {
      pressure_fixed_point();
      update_velocity();
      ++iters;
      const double den = linfty(pres_fixed);
      Vec d = pres_fixed;
      axpy(-1.0, pres_fixed_old, d);
      const double error = linfty(d) / (den + 1e-10);
      if (error < 1e-10) break;
      pres_fixed_old = pres_fixed;
    }
    last_picard[which] = iters;
    picard_total += iters;
    return iters;
  }

  // Atmospheric_Flow.cc:1110-1250 (one pass of the while loop)
  void step() {
    time += op.dt;
    ++n;
    op.hstage = 1;
    update_density();
    op.rho_for_fixed = rho_tmp_2;
    pres_fixed_old = pres_old;
    u_fixed = u_old;
    picard(0);
    pres_tmp_2 = pres_fixed;
    u_tmp_2 = u_fixed;

    op.hstage = 2;
    update_density();
    op.rho_for_fixed = rho_tmp_3;
    pres_fixed_old = pres_tmp_2;
    u_fixed = u_tmp_2;
    picard(1);
    pres_tmp_3 = pres_fixed;
    u_tmp_3 = u_fixed;

    op.hstage = 3;
    update_density();
    op.rho_for_fixed = rho_curr;
    update_velocity();
    update_pressure();
    rho_old = rho_curr;
    u_old = u_curr;
    apply_sponge();
  }

  // Rayleigh relaxation of u toward the background (not in the reference;
  // hook at Atmospheric_Flow.cc:1220): u <- (u + dt a u_bg)/(1 + dt a)
  void apply_sponge() {
    const int nn2 = op.nn2;
#pragma omp parallel for
    for (int c = 0; c < op.nc; ++c)
      for (int i = 0; i < nn2; ++i) {
        const double a = op.dt * sponge_alpha[(long)c * nn2 + i];
        if (a == 0.0) continue;
        double *u0 = &u_old[((long)c * 2 + 0) * nn2 + i];
        double *u1 = &u_old[((long)c * 2 + 1) * nn2 + i];
        *u0 = (*u0 + a * ubg0) / (1.0 + a);
        *u1 = (*u1 + a * ubg1) / (1.0 + a);
      }
  }
};

// ============================================================================
// C entry points (ctypes)
// ============================================================================
extern "C" {

void *orc_create(int degree, int n_cells, int map_degree, const double *nodes, int n_inner,
                 const int *inner, int n_bdry, const int *bdry) {
  Oracle *o = new Oracle();
  o->setup(degree, n_cells, map_degree, nodes, n_inner, inner, n_bdry, bdry);
  o->rho_for_fixed.assign(o->ns(), 0.0);
  o->pres_fixed.assign(o->ns(), 0.0);
  o->u_fixed.assign(o->nv(), 0.0);
  return o;
}
void orc_destroy(void *h) { delete static_cast<Oracle *>(h); }
void orc_set_params(void *h, double dt, double Ma, double Fr) {
  Oracle *o = static_cast<Oracle *>(h);
  o->dt = dt; o->Ma = Ma; o->Fr = Fr;
}
void orc_set_stage(void *h, int hs, int nss) {
  Oracle *o = static_cast<Oracle *>(h);
  o->hstage = hs; o->nsstage = nss;
}
void orc_set_inner_tol(void *h, double t) { static_cast<Oracle *>(h)->inner_cg_tol = t; }
void orc_set_rho_for_fixed(void *h, const double *v) {
  Oracle *o = static_cast<Oracle *>(h);
  o->rho_for_fixed.assign(v, v + o->ns());
}
void orc_set_pres_fixed(void *h, const double *v) {
  Oracle *o = static_cast<Oracle *>(h);
  o->pres_fixed.assign(v, v + o->ns());
}
void orc_set_u_fixed(void *h, const double *v) {
  Oracle *o = static_cast<Oracle *>(h);
  o->u_fixed.assign(v, v + o->nv());
}
void orc_vmult_rhs_rho_update(void *h, double *dst, const double *const *src) {
  static_cast<Oracle *>(h)->vmult_rhs_rho_update(dst, src);
}
void orc_vmult_rhs_velocity_fixed(void *h, double *dst, const double *const *src) {
  static_cast<Oracle *>(h)->vmult_rhs_velocity_fixed(dst, src);
}
void orc_vmult_rhs_pressure(void *h, double *dst, const double *const *src) {
  static_cast<Oracle *>(h)->vmult_rhs_pressure(dst, src);
}
void orc_vmult_pressure(void *h, double *dst, const double *src) {
  static_cast<Oracle *>(h)->vmult_pressure(dst, src);
}
void orc_vmult_enthalpy(void *h, double *dst, const double *src) {
  static_cast<Oracle *>(h)->vmult_enthalpy(dst, src);
}
void orc_vmult(void *h, double *dst, const double *src) {
  static_cast<Oracle *>(h)->vmult(dst, src);
}
void orc_diagonal_inverse(void *h, double *dst) {
  Oracle *o = static_cast<Oracle *>(h);
  Vec d = o->diagonal_inverse();
  std::memcpy(dst, d.data(), d.size() * sizeof(double));
}
// solve op x = b for the current NS stage: CG for mass-type stages, GMRES for
// NS 2.  x holds the initial guess on entry.
int orc_solve(void *h, double *x, const double *b, double tol, int maxit, int *its) {
  Oracle *o = static_cast<Oracle *>(h);
  const long n = o->vsize();
  Vec xv(x, x + n), bv(b, b + n);
  Vec dinv = o->diagonal_inverse();
  int rc = (o->nsstage == 2) ? o->gmres(xv, bv, tol, maxit, 28, dinv, its)
                             : o->cg(xv, bv, tol, maxit, dinv, its);
  std::memcpy(x, xv.data(), n * sizeof(double));
  return rc;
}
void orc_geometry(void *h, double *jxw, double *qx) {
  Oracle *o = static_cast<Oracle *>(h);
  std::memcpy(jxw, o->cJxW.data(), o->cJxW.size() * sizeof(double));
  std::memcpy(qx, o->cX.data(), o->cX.size() * sizeof(double));
}
void orc_basis(void *h, double *S, double *D, double *W) {
  Oracle *o = static_cast<Oracle *>(h);
  std::memcpy(S, o->S.data(), o->S.size() * sizeof(double));
  std::memcpy(D, o->D.data(), o->D.size() * sizeof(double));
  std::memcpy(W, o->W.data(), o->W.size() * sizeof(double));
}

// ------------------------------------------------------------ time loop --
void *orc_solver_create(int degree, int n_cells, int map_degree, const double *nodes,
                        int n_inner, const int *inner, int n_bdry, const int *bdry,
                        double dt, double Ma, double Fr, double eps, int max_its) {
  Solver *s = new Solver();
  s->op.setup(degree, n_cells, map_degree, nodes, n_inner, inner, n_bdry, bdry);
  s->op.dt = dt; s->op.Ma = Ma; s->op.Fr = Fr;
  s->eps = eps;
  s->max_its = max_its;
  s->init_vectors();
  return s;
}
void orc_solver_destroy(void *h) { delete static_cast<Solver *>(h); }
void orc_solver_set_inner_tol(void *h, double t) { static_cast<Solver *>(h)->op.inner_cg_tol = t; }
void orc_solver_set_true_residual_check(void *h, int on) {
  static_cast<Solver *>(h)->op.true_residual_check = on != 0;
}
void orc_solver_set_schur_tol_preconditioned(void *h, int on) {
  static_cast<Solver *>(h)->op.schur_tol_preconditioned = on != 0;
}
void orc_set_true_residual_check(void *h, int on) {
  static_cast<Oracle *>(h)->true_residual_check = on != 0;
}
void orc_solver_set_state(void *h, const double *rho, const double *u, const double *p) {
  Solver *s = static_cast<Solver *>(h);
  s->rho_old.assign(rho, rho + s->op.ns());
  s->u_old.assign(u, u + s->op.nv());
  s->pres_old.assign(p, p + s->op.ns());
}
void orc_solver_get_state(void *h, double *rho, double *u, double *p) {
  Solver *s = static_cast<Solver *>(h);
  std::memcpy(rho, s->rho_old.data(), s->op.ns() * sizeof(double));
  std::memcpy(u, s->u_old.data(), s->op.nv() * sizeof(double));
  std::memcpy(p, s->pres_old.data(), s->op.ns() * sizeof(double));
}
void orc_solver_set_sponge(void *h, const double *alpha, double ubg0, double ubg1) {
  Solver *s = static_cast<Solver *>(h);
  s->sponge_alpha.assign(alpha, alpha + s->op.ns());
  s->ubg0 = ubg0;
  s->ubg1 = ubg1;
}
void orc_solver_run(void *h, int n_steps) {
  Solver *s = static_cast<Solver *>(h);
  for (int i = 0; i < n_steps; ++i) s->step();
}
// Diagnostics of the state after a completed step, Atmospheric_Flow.cc:991-1087:
// get_min_density / get_max_density (rho_curr == rho_old after the step,
// :1221), compute_max_celerity (sqrt(Cp_Cv p / rho), pres_old and rho_old) and
// get_max_velocity (|u_old|).  The reference evaluates FE_DGQ fields with
// QGaussLobatto(k+1), whose points are the element's own support points, so the
// values are the nodal coefficients.  Its celerity maximum starts from
// numeric_limits<double>::min() and its velocity maximum from 0.
// out[0..3] = min rho, max |rho|, max celerity, max |u|.
void orc_solver_diagnostics(void *h, double *out) {
  Solver *s = static_cast<Solver *>(h);
  const long ns = s->op.ns();
  const int nn2 = s->op.nn2;
  double rmin = std::numeric_limits<double>::max(), rmax = 0.0;
  double cmax = std::numeric_limits<double>::min(), umax = 0.0;
  for (long i = 0; i < ns; ++i) {
    const long c = i / nn2, j = i % nn2;
    const double r = s->rho_old[i];
    rmin = std::min(rmin, r);
    rmax = std::max(rmax, std::fabs(r));
    cmax = std::max(cmax, std::sqrt(GAMMA_GAS * s->pres_old[i] / r));
    const double ux = s->u_old[(2 * c) * nn2 + j], uz = s->u_old[(2 * c + 1) * nn2 + j];
    umax = std::max(umax, std::sqrt(ux * ux + uz * uz));
  }
  out[0] = rmin; out[1] = rmax; out[2] = cmax; out[3] = umax;
}
// stats: picard_total, gmres_total, cg_total, solve_fail, inner_cg, picard1, picard2
void orc_solver_stats(void *h, long *out) {
  Solver *s = static_cast<Solver *>(h);
  out[0] = s->picard_total; out[1] = s->gmres_total; out[2] = s->cg_total;
  out[3] = s->solve_fail; out[4] = s->op.inner_cg_iters;
  out[5] = s->last_picard[0]; out[6] = s->last_picard[1];
}
int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
}
