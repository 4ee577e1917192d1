// ============================================================================
// shell_oracle.cpp -- CPU FP64 restatement of the IMEX-DG hot path in 3D, for
// the reference's own test case: steady solid-body rotation on a spherical
// shell (FE_DGQ(1) for every field, QGauss(3), radial gravity).
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product library links it; only
// the tests load it, as the checker of the GPU's 3D path.
//
// PARITY UNPINNED: the reference (deal.II >= 9.3 with MPI and p4est) cannot
// be built here.  This restatement is pinned by the reference's own known
// answer instead: the exact steady state of equation_data.h:57-176, which the
// reference checks every step (analyze_results, Atmospheric_Flow.cc:925-985).
//
// What it restates (file:line in the reference project), for dim = 3:
//   * Butcher tableau                              euler_operator.h:220-240
//   * rho rhs cell/face (3 IMEX stages)            euler_operator.h:344-712
//   * energy (pressure) rhs cell/face              euler_operator.h:745-1381
//     with the radial gravity work, a^2/r^2 e_r    euler_operator.h:790-811
//     and the stage-2 kinetic jump with u_old      euler_operator.h:1182-1183
//     and the stage-3 total rho E jump             euler_operator.h:1290-1336
//   * momentum rhs cell/face/wall                  euler_operator.h:1622-2305
//   * B, C, D, A, rho mass, Schur S, diagonal      euler_operator.h:717-740,
//                                                  1386-1617, 2330-2626
//   * stage solvers and the IMEX loop with Picard  Atmospheric_Flow.cc:430-871,
//                                                  1100-1257
// Gravity: the reference evaluates e_r and r at one SIMD lane of a cell batch
// (euler_operator.h:792-804); here at every quadrature point.
//
// Written face-centric (one loop over inner faces adding to both sides, one
// over walls), with a dense basis table -- a different structure from the
// GPU's element-centric kernels.
// ============================================================================
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using Vec = std::vector<double>;
constexpr double GAMMA_GAS = 1.4;        // equation_data.h:23
constexpr double EARTH_A = 6.37122e6;    // equation_data.h:26
constexpr int NN = 8, NQ = 27, NF = 9;   // nodes, cell points, face points

double dot(const Vec &a, const Vec &b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}
double norm2(const Vec &a) { return std::sqrt(dot(a, a)); }
void axpy(double a, const Vec &x, Vec &y) {
  for (size_t i = 0; i < y.size(); ++i) y[i] += a * x[i];
}

struct Gauss3 {
  double x[3], w[3];
  Gauss3() {
    const double s = std::sqrt(0.6);
    x[0] = 0.5 * (1.0 - s); x[1] = 0.5; x[2] = 0.5 * (1.0 + s);
    w[0] = 5.0 / 18.0; w[1] = 8.0 / 18.0; w[2] = 5.0 / 18.0;
  }
};

// degree-2 Lagrange basis on {0, 1/2, 1} and its derivative
void lag2(double t, double *v, double *d) {
  v[0] = 2.0 * (t - 0.5) * (t - 1.0);
  v[1] = -4.0 * t * (t - 1.0);
  v[2] = 2.0 * t * (t - 0.5);
  d[0] = 4.0 * t - 3.0;
  d[1] = -8.0 * t + 4.0;
  d[2] = 4.0 * t - 1.0;
}

struct Geo {  // at one point: position, inverse Jacobian, det
  double x[3], Ji[3][3], det;
};

// x(xi) and J from the 27 mapping nodes of a cell (first coordinate fastest)
Geo map_point(const double *nodes, const double xi[3]) {
  double v[3][3], d[3][3];
  for (int e = 0; e < 3; ++e) lag2(xi[e], v[e], d[e]);
  Geo g{};
  double J[3][3] = {{0}};
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) {
        const double *X = nodes + 3 * ((c * 3 + b) * 3 + a);
        const double w = v[0][a] * v[1][b] * v[2][c];
        const double dw[3] = {d[0][a] * v[1][b] * v[2][c], v[0][a] * d[1][b] * v[2][c],
                              v[0][a] * v[1][b] * d[2][c]};
        for (int i = 0; i < 3; ++i) {
          g.x[i] += w * X[i];
          for (int e = 0; e < 3; ++e) J[i][e] += dw[e] * X[i];  // dx_i/dxi_e
        }
      }
  g.det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
          J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  // Ji[e][i] = dxi_e/dx_i
  g.Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / g.det;
  g.Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / g.det;
  g.Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / g.det;
  g.Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / g.det;
  g.Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / g.det;
  g.Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / g.det;
  g.Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / g.det;
  g.Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / g.det;
  g.Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / g.det;
  return g;
}

// Q1 basis: phi_v(xi) = prod_d (bit_d(v) ? xi_d : 1 - xi_d)
void q1(const double xi[3], double *phi, double (*dphi)[3]) {
  for (int v = 0; v < NN; ++v) {
    double f[3], df[3];
    for (int d = 0; d < 3; ++d) {
      const bool hi = (v >> d) & 1;
      f[d] = hi ? xi[d] : 1.0 - xi[d];
      df[d] = hi ? 1.0 : -1.0;
    }
    phi[v] = f[0] * f[1] * f[2];
    if (dphi) {
      dphi[v][0] = df[0] * f[1] * f[2];
      dphi[v][1] = f[0] * df[1] * f[2];
      dphi[v][2] = f[0] * f[1] * df[2];
    }
  }
}

// reference point of face point q of local face f (0/1: xi1 = 0/1, 2/3: xi2,
// 4/5: xi3); tangential coordinates in increasing order, the first fastest
void face_ref(int f, int q, const Gauss3 &g, double xi[3], double *w) {
  const int d = f / 2, t0 = d == 0 ? 1 : 0, t1 = d == 2 ? 1 : 2;
  xi[d] = (double)(f % 2);
  xi[t0] = g.x[q % 3];
  xi[t1] = g.x[q / 3];
  *w = g.w[q % 3] * g.w[q / 3];
}

}  // namespace

struct Shell {
  int nc = 0, nf = 0, nb = 0;
  std::vector<int> inner, perm, bdry;  // [nf][4], [nf][9], [nb][3]
  // cell data at the 27 points: basis values and physical gradients x JxW
  Vec phi;   // [27][8]
  Vec grad;  // [nc][27][8][3]: dphi/dx
  Vec jxw;   // [nc][27]
  Vec er;    // [nc][27][4]: e_r (3), a^2/r^2
  // faces: basis values at the 9 points of each local face [6][9][8]
  Vec fphi;
  Vec fn, fjxw;  // inner faces from the "+" side: [nf][9][3], [nf][9]
  Vec bn, bjxw;  // walls: [nb][9][3], [nb][9]
  double dt = 1.0, Ma = 1.0, Fr = 1.0;
  int hstage = 1, nsstage = 1;
  double inner_tol = 1e-12;
  bool true_residual_check = false;
  long inner_cg_iters = 0;
  Vec rho_fix, pres_fix, u_fix;
  // tableau, euler_operator.h:220-240
  double gam, a21, a31, a32, a21t, a22t, a31t, a32t, a33t, b1, b2, b3;

  long ns() const { return (long)nc * NN; }
  long nv() const { return 3L * nc * NN; }

  void setup(int n_cells, const double *nodes, int n_inner, const int *in, const int *pm,
             int n_bdry, const int *bd) {
    nc = n_cells; nf = n_inner; nb = n_bdry;
    inner.assign(in, in + 4L * nf);
    perm.assign(pm, pm + 9L * nf);
    bdry.assign(bd, bd + 3L * nb);
    gam = 2.0 - std::sqrt(2.0);
    a21 = gam; a31 = 0.5; a32 = 0.5;
    a21t = 0.5 * gam; a22t = 0.5 * gam;
    a31t = std::sqrt(2.0) / 4.0; a32t = std::sqrt(2.0) / 4.0; a33t = 1.0 - std::sqrt(2.0) / 2.0;
    b1 = a31t; b2 = a32t; b3 = a33t;
    Gauss3 g;
    phi.assign(NQ * NN, 0.0);
    grad.assign((size_t)nc * NQ * NN * 3, 0.0);
    jxw.assign((size_t)nc * NQ, 0.0);
    er.assign((size_t)nc * NQ * 4, 0.0);
    for (int q = 0; q < NQ; ++q) {
      const double xi[3] = {g.x[q % 3], g.x[(q / 3) % 3], g.x[q / 9]};
      q1(xi, &phi[q * NN], nullptr);
    }
    for (int c = 0; c < nc; ++c)
      for (int q = 0; q < NQ; ++q) {
        const double xi[3] = {g.x[q % 3], g.x[(q / 3) % 3], g.x[q / 9]};
        const double w = g.w[q % 3] * g.w[(q / 3) % 3] * g.w[q / 9];
        const Geo G = map_point(nodes + 81L * c, xi);
        double ph[NN], dph[NN][3];
        q1(xi, ph, dph);
        for (int v = 0; v < NN; ++v)
          for (int i = 0; i < 3; ++i) {
            double s = 0.0;
            for (int e = 0; e < 3; ++e) s += dph[v][e] * G.Ji[e][i];
            grad[(((size_t)c * NQ + q) * NN + v) * 3 + i] = s;
          }
        jxw[(size_t)c * NQ + q] = G.det * w;
        const double r = std::sqrt(G.x[0] * G.x[0] + G.x[1] * G.x[1] + G.x[2] * G.x[2]);
        for (int i = 0; i < 3; ++i) er[((size_t)c * NQ + q) * 4 + i] = G.x[i] / r;
        er[((size_t)c * NQ + q) * 4 + 3] = EARTH_A * EARTH_A / (r * r);
      }
    fphi.assign(6 * NF * NN, 0.0);
    for (int f = 0; f < 6; ++f)
      for (int q = 0; q < NF; ++q) {
        double xi[3], w;
        face_ref(f, q, g, xi, &w);
        q1(xi, &fphi[(f * NF + q) * NN], nullptr);
      }
    auto face_geo = [&](int c, int f, double *n, double *jw) {
      for (int q = 0; q < NF; ++q) {
        double xi[3], w;
        face_ref(f, q, g, xi, &w);
        const Geo G = map_point(nodes + 81L * c, xi);
        const int d = f / 2;
        const double s = (f % 2) ? 1.0 : -1.0;
        double m[3], len = 0.0;
        for (int i = 0; i < 3; ++i) { m[i] = G.Ji[d][i]; len += m[i] * m[i]; }
        len = std::sqrt(len);
        for (int i = 0; i < 3; ++i) n[q * 3 + i] = s * m[i] / len;
        jw[q] = G.det * len * w;
      }
    };
    fn.assign((size_t)nf * NF * 3, 0.0); fjxw.assign((size_t)nf * NF, 0.0);
    for (int f = 0; f < nf; ++f) face_geo(inner[4 * f], inner[4 * f + 1], &fn[f * 27L], &fjxw[f * 9L]);
    bn.assign((size_t)nb * NF * 3, 0.0); bjxw.assign((size_t)nb * NF, 0.0);
    for (int f = 0; f < nb; ++f) face_geo(bdry[3 * f], bdry[3 * f + 1], &bn[f * 27L], &bjxw[f * 9L]);
    rho_fix.assign(ns(), 0.0); pres_fix.assign(ns(), 0.0); u_fix.assign(nv(), 0.0);
  }

  // ------------------------------------------------------------ evaluation --
  const double *tile(const double *v, int c, int ncomp, int comp) const {
    return v + ((long)c * ncomp + comp) * NN;
  }
  void eval(const double *t, double *out) const {
    for (int q = 0; q < NQ; ++q) {
      double s = 0.0;
      for (int v = 0; v < NN; ++v) s += phi[q * NN + v] * t[v];
      out[q] = s;
    }
  }
  // the trace at face point q of (c, f), q given in that face's own numbering
  double trace(const double *t, int f, int q) const {
    double s = 0.0;
    for (int v = 0; v < NN; ++v) s += fphi[(f * NF + q) * NN + v] * t[v];
    return s;
  }
  // dst[c] += sum_q (V phi + G . grad phi) JxW
  void integrate(int c, const double *V, const double (*G)[3], double *dst) const {
    for (int v = 0; v < NN; ++v) {
      double s = 0.0;
      for (int q = 0; q < NQ; ++q) {
        const double *gr = &grad[(((size_t)c * NQ + q) * NN + v) * 3];
        double t = V ? V[q] * phi[q * NN + v] : 0.0;
        if (G) t += G[q][0] * gr[0] + G[q][1] * gr[1] + G[q][2] * gr[2];
        s += t * jxw[(size_t)c * NQ + q];
      }
      dst[v] += s;
    }
  }
  void face_add(double *dst, int f, const double *F) const {  // F already has JxW
    for (int v = 0; v < NN; ++v) {
      double s = 0.0;
      for (int q = 0; q < NF; ++q) s += F[q] * fphi[(f * NF + q) * NN + v];
      dst[v] += s;
    }
  }

  void stage_weights(double *ca, double *ct, int *nst) const {
    if (hstage == 1) { *nst = 1; ca[0] = a21; ct[0] = a21t; }
    else if (hstage == 2) { *nst = 2; ca[0] = a31; ca[1] = a32; ct[0] = a31t; ct[1] = a32t; }
    else { *nst = 3; ca[0] = b1; ca[1] = b2; ca[2] = b3; ct[0] = b1; ct[1] = b2; ct[2] = b3; }
  }

  // ---------------------------------------------------------------- rho rhs --
  void rhs_rho(double *dst, const double *const *src) const {
    double cf[3], ct[3];
    int nst;
    stage_weights(cf, ct, &nst);
    std::fill(dst, dst + ns(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double r[3][NQ], u[3][3][NQ], V[NQ], G[NQ][3];
      for (int j = 0; j < nst; ++j) {
        eval(tile(src[2 * j], c, 1, 0), r[j]);
        for (int d = 0; d < 3; ++d) eval(tile(src[2 * j + 1], c, 3, d), u[j][d]);
      }
      for (int q = 0; q < NQ; ++q) {
        V[q] = r[0][q];
        for (int d = 0; d < 3; ++d) {
          G[q][d] = 0.0;
          for (int j = 0; j < nst; ++j) G[q][d] += cf[j] * dt * r[j][q] * u[j][d][q];
        }
      }
      integrate(c, V, G, dst + (long)c * NN);
    }
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[4 * f], fp = inner[4 * f + 1], cm = inner[4 * f + 2], fm = inner[4 * f + 3];
      double Fp[NF], Fm[NF] = {0};
      for (int q = 0; q < NF; ++q) {
        const int qm = perm[9 * f + q];
        const double *n = &fn[(f * NF + q) * 3];
        double flux = 0.0;
        for (int j = 0; j < nst; ++j) {
          const double rp = trace(tile(src[2 * j], cp, 1, 0), fp, q);
          const double rm = trace(tile(src[2 * j], cm, 1, 0), fm, qm);
          double avg = 0.0, unp = 0.0, unm = 0.0;
          for (int d = 0; d < 3; ++d) {
            const double up = trace(tile(src[2 * j + 1], cp, 3, d), fp, q);
            const double um = trace(tile(src[2 * j + 1], cm, 3, d), fm, qm);
            avg += 0.5 * (rp * up + rm * um) * n[d];
            unp += up * n[d];
            unm += um * n[d];
          }
          const double lam = std::max(std::fabs(unp), std::fabs(unm));
          flux += cf[j] * dt * (avg + 0.5 * lam * (rp - rm));
        }
        const double w = fjxw[f * NF + q];
        Fp[q] = -flux * w;
        Fm[qm] = flux * w;
      }
      face_add(dst + (long)cp * NN, fp, Fp);
      face_add(dst + (long)cm * NN, fm, Fm);
    }
  }

  // ------------------------------------------------------------ momentum --
  void rhs_vel(double *dst, const double *const *src) const {
    double ca[3], ct[3], cg[3];
    int nst, ng;
    const double *grho[3];
    stage_weights(ca, ct, &nst);
    if (hstage == 1) { ng = 2; cg[0] = a21t; cg[1] = a22t; grho[0] = src[0]; grho[1] = src[3]; }
    else if (hstage == 2) {
      ng = 3; cg[0] = a31t; cg[1] = a32t; cg[2] = a33t;
      grho[0] = src[0]; grho[1] = src[3]; grho[2] = src[6];
    } else {
      ng = 3; cg[0] = b1; cg[1] = b2; cg[2] = b3;
      grho[0] = src[0]; grho[1] = src[3]; grho[2] = src[6];
    }
    std::fill(dst, dst + nv(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double r[3][NQ], u[3][3][NQ], p[3][NQ], rg[3][NQ];
      for (int j = 0; j < nst; ++j) {
        eval(tile(src[3 * j], c, 1, 0), r[j]);
        for (int d = 0; d < 3; ++d) eval(tile(src[3 * j + 1], c, 3, d), u[j][d]);
        eval(tile(src[3 * j + 2], c, 1, 0), p[j]);
      }
      for (int j = 0; j < ng; ++j) eval(tile(grho[j], c, 1, 0), rg[j]);
      for (int d = 0; d < 3; ++d) {
        double V[NQ], G[NQ][3];
        for (int q = 0; q < NQ; ++q) {
          const double *e = &er[((size_t)c * NQ + q) * 4];
          double v = r[0][q] * u[0][d][q];
          for (int j = 0; j < ng; ++j) v -= cg[j] * dt / (Fr * Fr) * rg[j][q] * e[d] * e[3];
          V[q] = v;
          for (int k = 0; k < 3; ++k) {
            double s = 0.0;
            for (int j = 0; j < nst; ++j) {
              s += ca[j] * dt * r[j][q] * u[j][d][q] * u[j][k][q];
              if (k == d) s += ct[j] * dt / (Ma * Ma) * p[j][q];
            }
            G[q][k] = s;
          }
        }
        integrate(c, V, G, dst + ((long)c * 3 + d) * NN);
      }
    }
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[4 * f], fp = inner[4 * f + 1], cm = inner[4 * f + 2], fm = inner[4 * f + 3];
      double Fp[3][NF], Fm[3][NF] = {{0}};
      for (int q = 0; q < NF; ++q) {
        const int qm = perm[9 * f + q];
        const double *n = &fn[(f * NF + q) * 3];
        double fl[3] = {0, 0, 0};
        for (int j = 0; j < nst; ++j) {
          const double rp = trace(tile(src[3 * j], cp, 1, 0), fp, q);
          const double rm = trace(tile(src[3 * j], cm, 1, 0), fm, qm);
          const double pp = trace(tile(src[3 * j + 2], cp, 1, 0), fp, q);
          const double pm = trace(tile(src[3 * j + 2], cm, 1, 0), fm, qm);
          double up[3], um[3], unp = 0.0, unm = 0.0;
          for (int d = 0; d < 3; ++d) {
            up[d] = trace(tile(src[3 * j + 1], cp, 3, d), fp, q);
            um[d] = trace(tile(src[3 * j + 1], cm, 3, d), fm, qm);
            unp += up[d] * n[d];
            unm += um[d] * n[d];
          }
          const double lam = std::max(std::fabs(unp), std::fabs(unm));
          for (int d = 0; d < 3; ++d) {
            const double at = 0.5 * (rp * up[d] * unp + rm * um[d] * unm);
            fl[d] += ca[j] * dt * at + ct[j] * dt / (Ma * Ma) * 0.5 * (pp + pm) * n[d] +
                     ca[j] * dt * 0.5 * lam * (rp * up[d] - rm * um[d]);
          }
        }
        const double w = fjxw[f * NF + q];
        for (int d = 0; d < 3; ++d) { Fp[d][q] = -fl[d] * w; Fm[d][qm] = fl[d] * w; }
      }
      for (int d = 0; d < 3; ++d) {
        face_add(dst + ((long)cp * 3 + d) * NN, fp, Fp[d]);
        face_add(dst + ((long)cm * 3 + d) * NN, fm, Fm[d]);
      }
    }
    for (int f = 0; f < nb; ++f) {  // walls, p_D = p
      const int c = bdry[3 * f], lf = bdry[3 * f + 1];
      double F[3][NF];
      for (int q = 0; q < NF; ++q) {
        const double *n = &bn[(f * NF + q) * 3];
        double s = 0.0;
        for (int j = 0; j < nst; ++j) {
          const double pb = trace(tile(src[3 * j + 2], c, 1, 0), lf, q);
          s += ct[j] * dt / (Ma * Ma) * 0.5 * (pb + pb);
        }
        for (int d = 0; d < 3; ++d) F[d][q] = -s * n[d] * bjxw[f * NF + q];
      }
      for (int d = 0; d < 3; ++d) face_add(dst + ((long)c * 3 + d) * NN, lf, F[d]);
    }
  }

  // -------------------------------------------------------------- energy --
  void rhs_pres(double *dst, const double *const *src) const {
    const double gm1 = GAMMA_GAS - 1.0, M2 = Ma * Ma;
    double ca[3], ct[3], cg[3];
    int nst, ng;
    const double *grho[3], *gu[3], *kin_rho, *kin_u;
    stage_weights(ca, ct, &nst);
    if (hstage == 1) {
      ng = 2; cg[0] = a21t; cg[1] = a22t;
      grho[0] = src[0]; gu[0] = src[1]; grho[1] = src[3]; gu[1] = src[4];
      kin_rho = src[3]; kin_u = src[4];
    } else if (hstage == 2) {
      ng = 3; cg[0] = a31t; cg[1] = a32t; cg[2] = a33t;
      grho[0] = src[0]; gu[0] = src[1]; grho[1] = src[3]; gu[1] = src[4];
      grho[2] = src[6]; gu[2] = src[7];
      kin_rho = src[6]; kin_u = src[7];
    } else {
      ng = 3; cg[0] = b1; cg[1] = b2; cg[2] = b3;
      grho[0] = src[0]; gu[0] = src[1]; grho[1] = src[3]; gu[1] = src[4];
      grho[2] = src[6]; gu[2] = src[7];
      kin_rho = src[9]; kin_u = src[10];
    }
    std::fill(dst, dst + ns(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double r[3][NQ], u[3][3][NQ], p[3][NQ], gr[3][NQ], gv[3][3][NQ], kr[NQ], ku[3][NQ];
      for (int j = 0; j < nst; ++j) {
        eval(tile(src[3 * j], c, 1, 0), r[j]);
        for (int d = 0; d < 3; ++d) eval(tile(src[3 * j + 1], c, 3, d), u[j][d]);
        eval(tile(src[3 * j + 2], c, 1, 0), p[j]);
      }
      for (int j = 0; j < ng; ++j) {
        eval(tile(grho[j], c, 1, 0), gr[j]);
        for (int d = 0; d < 3; ++d) eval(tile(gu[j], c, 3, d), gv[j][d]);
      }
      eval(tile(kin_rho, c, 1, 0), kr);
      for (int d = 0; d < 3; ++d) eval(tile(kin_u, c, 3, d), ku[d]);
      double V[NQ], G[NQ][3];
      for (int q = 0; q < NQ; ++q) {
        const double *e = &er[((size_t)c * NQ + q) * 4];
        const double uu0 = u[0][0][q] * u[0][0][q] + u[0][1][q] * u[0][1][q] + u[0][2][q] * u[0][2][q];
        const double E0 = p[0][q] / (gm1 * r[0][q]) + 0.5 * M2 * uu0;
        const double kk = ku[0][q] * ku[0][q] + ku[1][q] * ku[1][q] + ku[2][q] * ku[2][q];
        double v = r[0][q] * E0 - 0.5 * kr[q] * M2 * kk;
        for (int j = 0; j < ng; ++j) {
          const double ue = gv[j][0][q] * e[0] + gv[j][1][q] * e[1] + gv[j][2][q] * e[2];
          v -= cg[j] * dt * M2 / (Fr * Fr) * gr[j][q] * ue * e[3];
        }
        V[q] = v;
        for (int d = 0; d < 3; ++d) G[q][d] = 0.0;
        for (int j = 0; j < nst; ++j) {
          const double uu = u[j][0][q] * u[j][0][q] + u[j][1][q] * u[j][1][q] + u[j][2][q] * u[j][2][q];
          const double Ej = p[j][q] / (gm1 * r[j][q]) + 0.5 * M2 * uu;
          const double kin = 0.5 * ca[j] * dt * M2 * uu * r[j][q];
          const double ent = ct[j] * dt * (r[j][q] * (Ej - 0.5 * M2 * uu) + p[j][q]);
          for (int d = 0; d < 3; ++d) G[q][d] += (kin + ent) * u[j][d][q];
        }
      }
      integrate(c, V, G, dst + (long)c * NN);
    }
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[4 * f], fp = inner[4 * f + 1], cm = inner[4 * f + 2], fm = inner[4 * f + 3];
      double Fp[NF], Fm[NF] = {0};
      for (int q = 0; q < NF; ++q) {
        const int qm = perm[9 * f + q];
        const double *n = &fn[(f * NF + q) * 3];
        double up[3][3], um[3][3];
        for (int j = 0; j < nst; ++j)
          for (int d = 0; d < 3; ++d) {
            up[j][d] = trace(tile(src[3 * j + 1], cp, 3, d), fp, q);
            um[j][d] = trace(tile(src[3 * j + 1], cm, 3, d), fm, qm);
          }
        double flux = 0.0;
        for (int j = 0; j < nst; ++j) {
          const double rp = trace(tile(src[3 * j], cp, 1, 0), fp, q);
          const double rm = trace(tile(src[3 * j], cm, 1, 0), fm, qm);
          const double pp = trace(tile(src[3 * j + 2], cp, 1, 0), fp, q);
          const double pm = trace(tile(src[3 * j + 2], cm, 1, 0), fm, qm);
          double uup = 0, uum = 0, unp = 0, unm = 0;
          for (int d = 0; d < 3; ++d) {
            uup += up[j][d] * up[j][d]; uum += um[j][d] * um[j][d];
            unp += up[j][d] * n[d]; unm += um[j][d] * n[d];
          }
          const double akin = 0.5 * (0.5 * uup * rp * unp + 0.5 * uum * rm * unm);
          const double Ep = pp / (gm1 * rp) + 0.5 * M2 * uup;
          const double Em = pm / (gm1 * rm) + 0.5 * M2 * uum;
          const double hp = (Ep - 0.5 * M2 * uup) * rp + pp;
          const double hm = (Em - 0.5 * M2 * uum) * rm + pm;
          const double aent = 0.5 * (hp * unp + hm * unm);
          const double lam = std::max(std::fabs(unp), std::fabs(unm));
          if (hstage == 3) {
            flux += ca[j] * dt * M2 * akin + ca[j] * dt * aent +
                    ca[j] * dt * 0.5 * lam * (rp * Ep - rm * Em);
          } else {
            double jkin;
            if (hstage == 2 && j == 1) {  // mixes in u_old, euler_operator.h:1182-1183
              double kp = 0, km = 0;
              for (int d = 0; d < 3; ++d) { kp += up[1][d] * up[0][d]; km += um[1][d] * um[0][d]; }
              jkin = rp * 0.5 * kp - rm * 0.5 * km;
            } else {
              jkin = rp * 0.5 * uup - rm * 0.5 * uum;
            }
            const double je = rp * (Ep - 0.5 * M2 * uup) - rm * (Em - 0.5 * M2 * uum);
            flux += ca[j] * dt * M2 * (akin + 0.5 * lam * jkin) + ct[j] * dt * (aent + 0.5 * lam * je);
          }
        }
        const double w = fjxw[f * NF + q];
        Fp[q] = -flux * w;
        Fm[qm] = flux * w;
      }
      face_add(dst + (long)cp * NN, fp, Fp);
      face_add(dst + (long)cm * NN, fm, Fm);
    }
  }

  double icoef() const { return hstage == 1 ? a22t : a33t; }

  // ------------------------------------------------------------------- B --
  void apply_B(double *dst, const double *src) const {
    const double co = icoef() * dt / (Ma * Ma);
    std::fill(dst, dst + nv(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double p[NQ];
      eval(tile(src, c, 1, 0), p);
      for (int d = 0; d < 3; ++d) {
        double G[NQ][3];
        for (int q = 0; q < NQ; ++q) {
          for (int k = 0; k < 3; ++k) G[q][k] = 0.0;
          G[q][d] = -co * p[q];
        }
        integrate(c, nullptr, G, dst + ((long)c * 3 + d) * NN);
      }
    }
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[4 * f], fp = inner[4 * f + 1], cm = inner[4 * f + 2], fm = inner[4 * f + 3];
      double Fp[3][NF], Fm[3][NF] = {{0}};
      for (int q = 0; q < NF; ++q) {
        const int qm = perm[9 * f + q];
        const double *n = &fn[(f * NF + q) * 3];
        const double avg = 0.5 * (trace(tile(src, cp, 1, 0), fp, q) + trace(tile(src, cm, 1, 0), fm, qm));
        const double w = fjxw[f * NF + q];
        for (int d = 0; d < 3; ++d) { Fp[d][q] = co * avg * n[d] * w; Fm[d][qm] = -co * avg * n[d] * w; }
      }
      for (int d = 0; d < 3; ++d) {
        face_add(dst + ((long)cp * 3 + d) * NN, fp, Fp[d]);
        face_add(dst + ((long)cm * 3 + d) * NN, fm, Fm[d]);
      }
    }
    for (int f = 0; f < nb; ++f) {
      const int c = bdry[3 * f], lf = bdry[3 * f + 1];
      double F[3][NF];
      for (int q = 0; q < NF; ++q) {
        const double *n = &bn[(f * NF + q) * 3];
        const double pb = trace(tile(src, c, 1, 0), lf, q);
        for (int d = 0; d < 3; ++d) F[d][q] = co * 0.5 * (pb + pb) * n[d] * bjxw[f * NF + q];
      }
      for (int d = 0; d < 3; ++d) face_add(dst + ((long)c * 3 + d) * NN, lf, F[d]);
    }
  }

  // ------------------------------------------------------------------- C --
  void apply_C(double *dst, const double *src) const {
    const double co = icoef(), hg = GAMMA_GAS / (GAMMA_GAS - 1.0);
    std::fill(dst, dst + ns(), 0.0);
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double pf[NQ], w[3][NQ], G[NQ][3];
      eval(tile(pres_fix.data(), c, 1, 0), pf);
      for (int d = 0; d < 3; ++d) eval(tile(src, c, 3, d), w[d]);
      for (int q = 0; q < NQ; ++q)
        for (int d = 0; d < 3; ++d) G[q][d] = -co * dt * hg * pf[q] * w[d][q];
      integrate(c, nullptr, G, dst + (long)c * NN);
    }
    for (int f = 0; f < nf; ++f) {
      const int cp = inner[4 * f], fp = inner[4 * f + 1], cm = inner[4 * f + 2], fm = inner[4 * f + 3];
      double Fp[NF], Fm[NF] = {0};
      for (int q = 0; q < NF; ++q) {
        const int qm = perm[9 * f + q];
        const double *n = &fn[(f * NF + q) * 3];
        const double pfp = trace(tile(pres_fix.data(), cp, 1, 0), fp, q);
        const double pfm = trace(tile(pres_fix.data(), cm, 1, 0), fm, qm);
        double av = 0.0, wnp = 0.0, wnm = 0.0;
        for (int d = 0; d < 3; ++d) {
          const double wp = trace(tile(src, cp, 3, d), fp, q);
          const double wm = trace(tile(src, cm, 3, d), fm, qm);
          av += 0.5 * hg * (pfp * wp + pfm * wm) * n[d];
          wnp += wp * n[d];
          wnm += wm * n[d];
        }
        const double lam = std::max(std::fabs(wnp), std::fabs(wnm));
        const double flux = co * dt * (av + 0.5 * lam * (pfp - pfm) / (GAMMA_GAS - 1.0));
        const double w = fjxw[f * NF + q];
        Fp[q] = flux * w;
        Fm[qm] = -flux * w;
      }
      face_add(dst + (long)cp * NN, fp, Fp);
      face_add(dst + (long)cm * NN, fm, Fm);
    }
  }

  // ------------------------------------------------------- mass operators --
  void mass_add(double *dst, const double *src, int ncomp, const double *weight, double scale) const {
#pragma omp parallel for
    for (int c = 0; c < nc; ++c) {
      double wq[NQ], v[NQ];
      if (weight) eval(tile(weight, c, 1, 0), wq);
      for (int k = 0; k < ncomp; ++k) {
        eval(tile(src, c, ncomp, k), v);
        for (int q = 0; q < NQ; ++q) v[q] *= weight ? wq[q] : scale;
        integrate(c, v, nullptr, dst + ((long)c * ncomp + k) * NN);
      }
    }
  }
  long vsize() const { return (nsstage == 3 || nsstage == 5) ? nv() : ns(); }

  void vmult(double *dst, const double *src) {
    std::fill(dst, dst + vsize(), 0.0);
    if (nsstage == 1 || nsstage == 4) {
      mass_add(dst, src, 1, nullptr, 1.0);
    } else if (nsstage == 2) {  // S p = D p - C A^{-1} B p, A^{-1} by CG
      mass_add(dst, src, 1, nullptr, 1.0 / (GAMMA_GAS - 1.0));
      Vec t1(nv()), t2(nv(), 0.0), t3(ns());
      apply_B(t1.data(), src);
      nsstage = 3;
      Vec dinv = diagonal_inverse();
      int its = 0;
      cg(t2, t1, inner_tol * norm2(t1), 10000, dinv, &its);
      inner_cg_iters += its;
      apply_C(t3.data(), t2.data());
      for (long i = 0; i < ns(); ++i) dst[i] -= t3[i];
      nsstage = 2;
    } else if (nsstage == 3 || nsstage == 5) {
      mass_add(dst, src, 3, rho_fix.data(), 1.0);
    } else {
      mass_add(dst, src, 1, nullptr, 1.0 / (GAMMA_GAS - 1.0));
    }
  }

  // inverse diagonal; NS 2 uses diag(D) only (euler_operator.h:2607-2611)
  Vec diagonal_inverse() const {
    const bool vel = nsstage == 3 || nsstage == 5;
    const int ncomp = vel ? 3 : 1;
    const double scale = (nsstage == 2 || nsstage == 6) ? 1.0 / (GAMMA_GAS - 1.0) : 1.0;
    Vec d((long)nc * ncomp * NN);
    for (int c = 0; c < nc; ++c) {
      double wq[NQ];
      if (vel) eval(tile(rho_fix.data(), c, 1, 0), wq);
      for (int v = 0; v < NN; ++v) {
        double s = 0.0;
        for (int q = 0; q < NQ; ++q)
          s += (vel ? wq[q] : scale) * phi[q * NN + v] * phi[q * NN + v] * jxw[(size_t)c * NQ + q];
        for (int k = 0; k < ncomp; ++k) d[((long)c * ncomp + k) * NN + v] = 1.0 / s;
      }
    }
    return d;
  }

  int cg(Vec &x, const Vec &b, double tol, int maxit, const Vec &dinv, int *its) {
    const long n = (long)x.size();
    Vec r(n), z(n), p(n), v(n);
    vmult(v.data(), x.data());
    for (long i = 0; i < n; ++i) r[i] = b[i] - v[i];
    *its = 0;
    if (norm2(r) <= tol) return 0;
    for (long i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
    p = z;
    double rz = dot(r, z);
    for (int it = 1; it <= maxit; ++it) {
      vmult(v.data(), p.data());
      const double alpha = rz / dot(p, v);
      axpy(alpha, p, x);
      axpy(-alpha, v, r);
      *its = it;
      if (norm2(r) <= tol) return 0;
      for (long i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
      const double rz2 = dot(r, z);
      for (long i = 0; i < n; ++i) p[i] = z[i] + rz2 / rz * p[i];
      rz = rz2;
    }
    return 1;
  }

  // GMRES(28), left Jacobi, CGS2, Givens, as deal.II SolverGMRES
  int gmres(Vec &x, const Vec &b, double tol, int maxit, const Vec &dinv, int *its) {
    const long n = (long)x.size();
    const int m = 28;
    std::vector<Vec> V(m + 1, Vec(n));
    Vec w(n), t(n);
    std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
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
      for (int j = 0; j < m; ++j) {
        ++*its;
        vmult(t.data(), V[j].data());
        for (long i = 0; i < n; ++i) w[i] = dinv[i] * t[i];
        for (int pass = 0; pass < 2; ++pass) {
          std::vector<double> h(j + 1);
          for (int l = 0; l <= j; ++l) h[l] = dot(V[l], w);
          for (int l = 0; l <= j; ++l) axpy(-h[l], V[l], w);
          for (int l = 0; l <= j; ++l) H[l * m + j] = (pass ? H[l * m + j] : 0.0) + h[l];
        }
        const double hn = norm2(w);
        H[(j + 1) * m + j] = hn;
        for (int l = 0; l < j; ++l) {
          const double a = H[l * m + j], bb = H[(l + 1) * m + j];
          H[l * m + j] = cs[l] * a + sn[l] * bb;
          H[(l + 1) * m + j] = -sn[l] * a + cs[l] * bb;
        }
        const double a = H[j * m + j], bb = H[(j + 1) * m + j];
        const double r = std::sqrt(a * a + bb * bb);
        cs[j] = a / r; sn[j] = bb / r;
        H[j * m + j] = r; H[(j + 1) * m + j] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        jend = j + 1;
        if (hn > 0.0) for (long i = 0; i < n; ++i) V[j + 1][i] = w[i] / hn;
        if (std::fabs(g[j + 1]) <= tol || hn == 0.0 || *its >= maxit) { done = true; break; }
      }
      for (int l = jend - 1; l >= 0; --l) {
        double s = g[l];
        for (int k = l + 1; k < jend; ++k) s -= H[l * m + k] * y[k];
        y[l] = s / H[l * m + l];
      }
      for (int l = 0; l < jend; ++l) axpy(y[l], V[l], x);
      if (done && !true_residual_check) return std::fabs(g[jend]) <= tol ? 0 : (*its >= maxit ? 1 : 0);
    }
  }
};

// ============================================================================
// Time loop (Atmospheric_Flow.cc:1100-1257), the stage solvers restated as in
// the 2D oracle: CG + Jacobi for the mass-type systems, GMRES + Jacobi for S.
// ============================================================================
struct ShellSolver {
  Shell op;
  double eps = 1e-8;
  int max_its = 30000;
  bool scaled_tol = false;
  long steps = 0, picard_total = 0, gmres_total = 0, solve_fail = 0;
  Vec rho_old, rho_2, rho_3, rho_cur, rhs_rho;
  Vec u_old, u_2, u_3, u_cur, u_fix, rhs_u, tmp_1;
  Vec p_old, p_2, p_3, p_fix, p_fix_old, rhs_p;

  void init() {
    const long s = op.ns(), v = op.nv();
    for (Vec *x : {&rho_old, &rho_2, &rho_3, &rho_cur, &rhs_rho, &p_old, &p_2, &p_3, &p_fix,
                   &p_fix_old, &rhs_p})
      x->assign(s, 0.0);
    for (Vec *x : {&u_old, &u_2, &u_3, &u_cur, &u_fix, &rhs_u, &tmp_1}) x->assign(v, 0.0);
  }
  void solve_cg(Vec &x, const Vec &b, double tol) {
    Vec dinv = op.diagonal_inverse();
    int its = 0;
    if (op.cg(x, b, tol, max_its, dinv, &its)) ++solve_fail;
  }
  void update_density() {
    op.nsstage = 1;
    if (op.hstage == 1) {
      const double *s[] = {rho_old.data(), u_old.data()};
      op.rhs_rho(rhs_rho.data(), s);
      rho_2 = rho_old;
      solve_cg(rho_2, rhs_rho, eps * norm2(rhs_rho));
    } else if (op.hstage == 2) {
      const double *s[] = {rho_old.data(), u_old.data(), rho_2.data(), u_2.data()};
      op.rhs_rho(rhs_rho.data(), s);
      rho_3 = rho_2;
      solve_cg(rho_3, rhs_rho, eps * norm2(rhs_rho));
    } else {
      op.nsstage = 4;
      const double *s[] = {rho_old.data(), u_old.data(), rho_2.data(), u_2.data(),
                           rho_3.data(), u_3.data()};
      op.rhs_rho(rhs_rho.data(), s);
      rho_cur = rho_3;
      solve_cg(rho_cur, rhs_rho, eps * norm2(rhs_rho));
    }
  }
  void pressure_fixed_point() {
    op.nsstage = 2;
    op.pres_fix = p_fix_old;
    op.u_fix = u_fix;
    if (op.hstage == 1) {
      const double *sp[] = {rho_old.data(), u_old.data(), p_old.data(), rho_2.data(), u_fix.data()};
      op.rhs_pres(rhs_p.data(), sp);
      const double *su[] = {rho_old.data(), u_old.data(), p_old.data(), rho_2.data()};
      op.rhs_vel(rhs_u.data(), su);
    } else {
      const double *sp[] = {rho_old.data(), u_old.data(), p_old.data(), rho_2.data(), u_2.data(),
                            p_2.data(), rho_3.data(), u_fix.data()};
      op.rhs_pres(rhs_p.data(), sp);
      const double *su[] = {rho_old.data(), u_old.data(), p_old.data(), rho_2.data(), u_2.data(),
                            p_2.data(), rho_3.data()};
      op.rhs_vel(rhs_u.data(), su);
    }
    op.nsstage = 3;
    solve_cg(tmp_1, rhs_u, 1e-12 * norm2(rhs_u));
    Vec t2(op.ns());
    op.apply_C(t2.data(), tmp_1.data());
    axpy(-1.0, t2, rhs_p);
    op.nsstage = 2;
    Vec dinv = op.diagonal_inverse();
    // SolverControl(max_its, eps |rhs|) against the Jacobi-scaled residual
    // of left-preconditioned GMRES (Atmospheric_Flow.cc:656-672).  On this
    // mesh diag(D)^{-1} ~ 1/|cell| ~ 1e-15, so that rule stops before the
    // first iteration; with `scaled_tol` the bar is eps |diag(D)^{-1} rhs|.
    double tol = eps * norm2(rhs_p);
    if (scaled_tol) {
      double s = 0.0;
      for (long i = 0; i < op.ns(); ++i) s += dinv[i] * rhs_p[i] * dinv[i] * rhs_p[i];
      tol = eps * std::sqrt(s);
    }
    p_fix = p_fix_old;
    int its = 0;
    if (op.gmres(p_fix, rhs_p, tol, max_its, dinv, &its)) ++solve_fail;
    gmres_total += its;
  }
  void update_velocity() {
    if (op.hstage == 1 || op.hstage == 2) {
      op.nsstage = 3;
      Vec t3(op.nv());
      op.apply_B(t3.data(), p_fix.data());
      axpy(-1.0, t3, rhs_u);
      solve_cg(u_fix, rhs_u, eps * norm2(rhs_u));
    } else {
      op.nsstage = 5;
      const double *su[] = {rho_old.data(), u_old.data(), p_old.data(), rho_2.data(), u_2.data(),
                            p_2.data(), rho_3.data(), u_3.data(), p_3.data()};
      op.rhs_vel(rhs_u.data(), su);
      u_cur = u_3;
      solve_cg(u_cur, rhs_u, eps * norm2(rhs_u));
    }
  }
  void update_pressure() {
    op.nsstage = 6;
    const double *sp[] = {rho_old.data(), u_old.data(), p_old.data(), rho_2.data(), u_2.data(),
                          p_2.data(), rho_3.data(), u_3.data(), p_3.data(), rho_cur.data(),
                          u_cur.data()};
    op.rhs_pres(rhs_p.data(), sp);
    p_old = p_3;
    solve_cg(p_old, rhs_p, eps * norm2(rhs_p));
  }
  void picard() {
    for (int it = 0; it < 100; ++it) {
      pressure_fixed_point();
      update_velocity();
      ++picard_total;
      double num = 0.0, den = 0.0;
      for (long i = 0; i < op.ns(); ++i) {
        num = std::max(num, std::fabs(p_fix[i] - p_fix_old[i]));
        den = std::max(den, std::fabs(p_fix[i]));
      }
      if (num / (den + 1e-10) < 1e-10) break;
      p_fix_old = p_fix;
    }
  }
  void step() {
    op.hstage = 1;
    update_density();
    op.rho_fix = rho_2;
    p_fix_old = p_old;
    u_fix = u_old;
    picard();
    p_2 = p_fix;
    u_2 = u_fix;
    op.hstage = 2;
    update_density();
    op.rho_fix = rho_3;
    p_fix_old = p_2;
    u_fix = u_2;
    picard();
    p_3 = p_fix;
    u_3 = u_fix;
    op.hstage = 3;
    update_density();
    op.rho_fix = rho_cur;
    update_velocity();
    update_pressure();
    rho_old = rho_cur;
    u_old = u_cur;
    ++steps;
  }
};

extern "C" {
void *orc3_create(int n_cells, const double *nodes, int n_inner, const int *inner,
                  const int *perm, int n_bdry, const int *bdry, double dt, double Ma, double Fr,
                  double eps) {
  ShellSolver *s = new ShellSolver();
  s->op.setup(n_cells, nodes, n_inner, inner, perm, n_bdry, bdry);
  s->op.dt = dt; s->op.Ma = Ma; s->op.Fr = Fr;
  s->eps = eps;
  s->init();
  return s;
}
void orc3_destroy(void *h) { delete static_cast<ShellSolver *>(h); }
void orc3_set_tolerances(void *h, double inner_tol, int true_residual_check, int max_its,
                         int scaled_tol) {
  ShellSolver *s = static_cast<ShellSolver *>(h);
  s->scaled_tol = scaled_tol != 0;
  s->op.inner_tol = inner_tol;
  s->op.true_residual_check = true_residual_check != 0;
  s->max_its = max_its;
}
void orc3_set_stage(void *h, int hstage, int nsstage) {
  ShellSolver *s = static_cast<ShellSolver *>(h);
  s->op.hstage = hstage;
  s->op.nsstage = nsstage;
}
void orc3_set_frozen(void *h, const double *rho, const double *p, const double *u) {
  ShellSolver *s = static_cast<ShellSolver *>(h);
  if (rho) s->op.rho_fix.assign(rho, rho + s->op.ns());
  if (p) s->op.pres_fix.assign(p, p + s->op.ns());
  if (u) s->op.u_fix.assign(u, u + s->op.nv());
}
// which: 0 rho rhs, 1 momentum rhs, 2 energy rhs
void orc3_rhs(void *h, int which, double *dst, const double *const *src) {
  Shell &o = static_cast<ShellSolver *>(h)->op;
  if (which == 0) o.rhs_rho(dst, src);
  else if (which == 1) o.rhs_vel(dst, src);
  else o.rhs_pres(dst, src);
}
// which: 0 B, 1 C, 2 Base::vmult of the current NS stage
void orc3_apply(void *h, int which, double *dst, const double *src) {
  Shell &o = static_cast<ShellSolver *>(h)->op;
  if (which == 0) o.apply_B(dst, src);
  else if (which == 1) o.apply_C(dst, src);
  else o.vmult(dst, src);
}
void orc3_set_state(void *h, const double *rho, const double *u, const double *p) {
  ShellSolver *s = static_cast<ShellSolver *>(h);
  s->rho_old.assign(rho, rho + s->op.ns());
  s->u_old.assign(u, u + s->op.nv());
  s->p_old.assign(p, p + s->op.ns());
}
void orc3_get_state(void *h, double *rho, double *u, double *p) {
  ShellSolver *s = static_cast<ShellSolver *>(h);
  std::memcpy(rho, s->rho_old.data(), s->op.ns() * sizeof(double));
  std::memcpy(u, s->u_old.data(), s->op.nv() * sizeof(double));
  std::memcpy(p, s->p_old.data(), s->op.ns() * sizeof(double));
}
void orc3_run(void *h, int n) {
  ShellSolver *s = static_cast<ShellSolver *>(h);
  for (int i = 0; i < n; ++i) s->step();
}
// picard_total, gmres_total, solve_fail, steps
void orc3_stats(void *h, long *out) {
  ShellSolver *s = static_cast<ShellSolver *>(h);
  out[0] = s->picard_total; out[1] = s->gmres_total; out[2] = s->solve_fail; out[3] = s->steps;
}
// jxw [nc][27] and quadrature points are not exported: the host recomputes
// them from the mapping (shell.exact_l2_errors)
}
