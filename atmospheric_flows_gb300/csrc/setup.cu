// Host-side set-up: 1D rules and Lagrange tables, mapping geometry, face
// connectivity and the per-cell exact inverse of the unit mass matrix.
//
// This is what deal.II's MatrixFree::reinit produces for the reference
// (Atmospheric_Flow.cc:325-348): FE_DGQ(k) Lagrange basis on Gauss-Lobatto
// points, QGauss(2k+1) (n_q_points_1d_u = 2*degree_u+1, Atmospheric_Flow.cc:345),
// inverse Jacobians and JxW at cell quadrature points, outward normals and
// JxW at face quadrature points, from a degree-m tensor Lagrange mapping
// (MappingQ(m), Atmospheric_Flow.cc:239).  Geometry is stored once per cell
// and re-uploaded after mesh adaptation (atm_upload_mesh).
#include <cmath>
#include <cstring>
#include <mutex>

#include "atm_device.cuh"

namespace atm {

int upload_basis_rhs(const double *t);
int upload_basis_impl(const double *t);
int upload_basis_hang_rho(const double *t);
int upload_basis_hang_vel(const double *t);
int upload_basis_hang_pres(const double *t);
int upload_basis_hang_schur(const double *t);
int upload_basis_hang_schur_f(const double *t);

// Legendre P_n(x) and P_n'(x) by the three-term recurrence
static void legendre_pd(int n, double x, double *p, double *dp) {
  double pm1 = 1.0, pc = x;
  if (n == 0) { *p = 1.0; *dp = 0.0; return; }
  for (int j = 1; j < n; ++j) {
    const double pn = ((2 * j + 1) * x * pc - j * pm1) / (j + 1);
    pm1 = pc;
    pc = pn;
  }
  *p = pc;
  *dp = n * (pm1 - x * pc) / (1.0 - x * x);
}

std::vector<double> gll_nodes(int k) {
  std::vector<double> x(k + 1);
  x[0] = 0.0;
  x[k] = 1.0;
  for (int i = 1; i < k; ++i) {
    // Newton on P_k'(t) with P_k'' from the Legendre equation
    double t = -std::cos(M_PI * i / k);
    for (int it = 0; it < 64; ++it) {
      double p, dp;
      legendre_pd(k, t, &p, &dp);
      const double d2p = (2.0 * t * dp - k * (k + 1.0) * p) / (1.0 - t * t);
      const double step = dp / d2p;
      t -= step;
      if (std::fabs(step) <= 1e-17) break;
    }
    x[i] = 0.5 * (1.0 + t);
  }
  return x;
}

static void gauss_nodes(int n, std::vector<double> &x, std::vector<double> &w) {
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    double t = -std::cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 64; ++it) {
      double p, dp;
      legendre_pd(n, t, &p, &dp);
      const double step = p / dp;
      t -= step;
      if (std::fabs(step) <= 1e-17) break;
    }
    double p, dp;
    legendre_pd(n, t, &p, &dp);
    x[i] = 0.5 * (1.0 + t);
    w[i] = 1.0 / ((1.0 - t * t) * dp * dp);
  }
}

// values and derivatives of all Lagrange polynomials on `nodes` at x
void lagrange_eval(const std::vector<double> &nodes, double x, double *val, double *der) {
  const int n = (int)nodes.size();
  for (int i = 0; i < n; ++i) {
    double v = 1.0, d = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      const double inv = 1.0 / (nodes[i] - nodes[j]);
      d = d * (x - nodes[j]) * inv + v * inv;
      v *= (x - nodes[j]) * inv;
    }
    val[i] = v;
    if (der) der[i] = d;
  }
}

HostBasis make_basis(int k) {
  HostBasis b;
  b.k = k;
  b.nn = k + 1;
  b.nq = 2 * k + 1;
  b.gll = gll_nodes(k);
  gauss_nodes(b.nq, b.gauss, b.weights);
  b.S.assign(b.nq * b.nn, 0.0);
  b.D.assign(b.nq * b.nn, 0.0);
  for (int q = 0; q < b.nq; ++q)
    lagrange_eval(b.gll, b.gauss[q], &b.S[q * b.nn], &b.D[q * b.nn]);
  return b;
}

int upload_basis_all() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  ATM_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (dev >= 0 && dev < 64 && done[dev]) return ATM_OK;
  // [k][w][q*(k+1)+i]: w = 0 values, 1 derivatives at the Gauss points,
  // 2 and 3 values at the subface points (g_q + s)/2 (hanging faces)
  constexpr int NW = 8;
  static_assert(NW == BASIS_TABLES, "basis table count");
  // followed by the degree-2 mapping tables [k][r][q] (r = 0..2 values and
  // 3..5 derivatives of the Lagrange basis on {0, 1/2, 1}, 6 Gauss weights)
  constexpr size_t NB = (size_t)(KMAX + 1) * NW * NQ_MAX * NN_MAX;
  std::vector<double> tab(NB + (size_t)(KMAX + 1) * GEO2_ROWS * NQ_MAX, 0.0);
  const std::vector<double> m2 = gll_nodes(2);
  for (int k = 1; k <= KMAX; ++k) {
    HostBasis b = make_basis(k);
    double *S = &tab[(k * NW + 0) * NQ_MAX * NN_MAX];
    double *D = &tab[(k * NW + 1) * NQ_MAX * NN_MAX];
    std::memcpy(S, b.S.data(), b.S.size() * sizeof(double));
    std::memcpy(D, b.D.data(), b.D.size() * sizeof(double));
    for (int s = 0; s < 2; ++s) {
      double *H = &tab[(k * NW + 2 + s) * NQ_MAX * NN_MAX];
      for (int q = 0; q < b.nq; ++q)
        lagrange_eval(b.gll, 0.5 * (b.gauss[q] + s), &H[q * b.nn], nullptr);
    }
    for (int q = 0; q < b.nq; ++q) {
      double v[3], d[3];
      lagrange_eval(m2, b.gauss[q], v, d);
      for (int a = 0; a < 3; ++a) {
        tab[NB + ((size_t)k * GEO2_ROWS + a) * NQ_MAX + q] = v[a];
        tab[NB + ((size_t)k * GEO2_ROWS + 3 + a) * NQ_MAX + q] = d[a];
      }
      tab[NB + ((size_t)k * GEO2_ROWS + 6) * NQ_MAX + q] = b.weights[q];
    }
    // even/odd halves for q < k, i < (k+1)/2 (same [q*(k+1)+i] indexing)
    for (int w = 0; w < 2; ++w) {
      const std::vector<double> &src = w == 0 ? b.S : b.D;
      double *E = &tab[(k * NW + 4 + 2 * w) * NQ_MAX * NN_MAX];
      double *O = &tab[(k * NW + 5 + 2 * w) * NQ_MAX * NN_MAX];
      for (int q = 0; q < k; ++q)
        for (int i = 0; i < b.nn / 2; ++i) {
          const double a = src[q * b.nn + i], c = src[q * b.nn + k - i];
          E[q * b.nn + i] = 0.5 * (a + c);
          O[q * b.nn + i] = 0.5 * (a - c);
        }
    }
  }
  if (upload_basis_rhs(tab.data()) || upload_basis_impl(tab.data()) ||
      upload_basis_hang_rho(tab.data()) || upload_basis_hang_vel(tab.data()) ||
      upload_basis_hang_pres(tab.data()) || upload_basis_hang_schur(tab.data()) ||
      upload_basis_hang_schur_f(tab.data())) {
    set_error("failed to upload basis tables to constant memory");
    return ATM_CUDA_ERROR;
  }
  if (dev >= 0 && dev < 64) done[dev] = true;
  return ATM_OK;
}

void mesh_free(Mesh &m) {
  cudaFree(m.qgeo);
  cudaFree(m.fgeo);
  cudaFree(m.nbr);
  cudaFree(m.nbrf);
  cudaFree(m.minv);
  cudaFree(m.hnb);
  cudaFree(m.hgeo);
  m.qgeo = m.fgeo = m.minv = m.hgeo = nullptr;
  m.nbr = m.nbrf = m.hnb = nullptr;
  m.nhang = 0;
}

int build_mesh_tables(int k, int nc, int mapdeg, const double *nodes, int n_inner,
                      const int *inner, int n_bdry, const int *bdry, HostMesh &out) {
  const int nq = 2 * k + 1, nq2 = nq * nq;
  if (mapdeg < 1 || mapdeg > 8 || !nodes || (n_inner > 0 && !inner) || (n_bdry > 0 && !bdry)) {
    set_error("mesh tables: bad mapping degree or null table");
    return ATM_BAD_ARG;
  }
  // --- connectivity.  inner face: (c+, f+, c-, f-, o); o = 0 conforming,
  // o = 1, 2: c+ is the fine cell and its face f+ is subface o-1 of face f-
  // of the coarse cell c- (2:1 adaptive meshes, deal.II puts the fine cell
  // on the interior side of a hanging face).
  std::vector<int> &nbr = out.nbr, &nbrf = out.nbrf;
  nbr.assign((size_t)nc * 4, -2);
  nbrf.assign((size_t)nc * 4, -1);
  std::vector<int> hidx((size_t)nc * 4, -1);
  out.hnb.clear();
  for (int f = 0; f < n_inner; ++f) {
    const int *e = inner + 5L * f;
    if (e[0] < 0 || e[0] >= nc || e[2] < 0 || e[2] >= nc || e[1] < 0 || e[1] > 3 ||
        e[3] < 0 || e[3] > 3) {
      set_error("inner face " + std::to_string(f) + ": cell or face index out of range");
      return ATM_BAD_ARG;
    }
    if (e[4] < 0 || e[4] > 2) {
      set_error("inner face " + std::to_string(f) +
                ": the last entry must be 0 (conforming) or 1, 2 (hanging subface)");
      return ATM_BAD_ARG;
    }
    if ((e[1] >> 1) != (e[3] >> 1) || e[1] == e[3]) {
      set_error("inner face " + std::to_string(f) +
                ": the two sides must be opposite faces (0/1 or 2/3)");
      return ATM_BAD_ARG;
    }
    const size_t a = (size_t)e[0] * 4 + e[1], b = (size_t)e[2] * 4 + e[3];
    if (nbr[a] != -2) {
      set_error("inner face " + std::to_string(f) + ": cell face listed twice");
      return ATM_BAD_ARG;
    }
    nbr[a] = e[2];
    nbrf[a] = e[3] | (e[4] << 2);
    if (e[4] == 0) {
      if (nbr[b] != -2) {
        set_error("inner face " + std::to_string(f) + ": cell face listed twice");
        return ATM_BAD_ARG;
      }
      nbr[b] = e[0];
      nbrf[b] = e[1];
    } else {
      if (hidx[b] < 0) {
        if (nbr[b] != -2) {
          set_error("inner face " + std::to_string(f) +
                    ": coarse face is also listed as a conforming or boundary face");
          return ATM_BAD_ARG;
        }
        hidx[b] = (int)(out.hnb.size() / 2);
        out.hnb.push_back(-1);
        out.hnb.push_back(-1);
        nbr[b] = hidx[b];
        nbrf[b] = e[1] | (3 << 2);
      }
      int &slot = out.hnb[(size_t)hidx[b] * 2 + (e[4] - 1)];
      if (slot != -1) {
        set_error("inner face " + std::to_string(f) + ": hanging subface listed twice");
        return ATM_BAD_ARG;
      }
      slot = e[0];
    }
  }
  out.nhang = (int)(out.hnb.size() / 2);
  for (int h = 0; h < out.nhang; ++h)
    if (out.hnb[2 * h] < 0 || out.hnb[2 * h + 1] < 0) {
      set_error("hanging face " + std::to_string(h) + ": only one of its two subfaces is listed");
      return ATM_BAD_ARG;
    }
  for (int f = 0; f < n_bdry; ++f) {
    const int *e = bdry + 3L * f;
    if (e[0] < 0 || e[0] >= nc || e[1] < 0 || e[1] > 3) {
      set_error("boundary face " + std::to_string(f) + ": index out of range");
      return ATM_BAD_ARG;
    }
    const size_t a = (size_t)e[0] * 4 + e[1];
    if (nbr[a] != -2 || hidx[a] >= 0) {
      set_error("boundary face " + std::to_string(f) + ": cell face listed twice");
      return ATM_BAD_ARG;
    }
    nbr[a] = -1; nbrf[a] = -1;
  }
  for (size_t a = 0; a < nbr.size(); ++a)
    if (nbr[a] == -2) {
      set_error("cell " + std::to_string(a / 4) + " face " + std::to_string(a % 4) +
                " is neither an inner nor a boundary face");
      return ATM_BAD_ARG;
    }
  // --- geometry
  HostBasis b = make_basis(k);
  const std::vector<double> mx = gll_nodes(mapdeg);
  const int mn = mapdeg + 1;
  auto tab = [&](double x, std::vector<double> &v, std::vector<double> &d) {
    v.resize(mn);
    d.resize(mn);
    lagrange_eval(mx, x, v.data(), d.data());
  };
  std::vector<std::vector<double>> Lg(nq), dLg(nq);
  for (int q = 0; q < nq; ++q) tab(b.gauss[q], Lg[q], dLg[q]);
  std::vector<double> L0, dL0, L1, dL1;
  tab(0.0, L0, dL0);
  tab(1.0, L1, dL1);
  std::vector<double> &qgeo = out.qgeo, &fgeo = out.fgeo;
  qgeo.assign((size_t)nc * 5 * nq2, 0.0);
  fgeo.assign((size_t)nc * 4 * 3 * nq, 0.0);
  // J = [[dx/dxi, dx/deta],[dz/dxi, dz/deta]] at (La, dLa) x (Lb, dLb)
  auto jac = [&](int cell, const double *La, const double *dLa, const double *Lb,
                 const double *dLb, double J[4]) {
    J[0] = J[1] = J[2] = J[3] = 0.0;
    for (int bb = 0; bb < mn; ++bb)
      for (int aa = 0; aa < mn; ++aa) {
        const double *X = nodes + (((size_t)cell * mn + bb) * mn + aa) * 2;
        for (int d = 0; d < 2; ++d) {
          J[d * 2 + 0] += X[d] * dLa[aa] * Lb[bb];
          J[d * 2 + 1] += X[d] * La[aa] * dLb[bb];
        }
      }
  };
  // outward unit normal and face weight of face f at the face parameter
  // whose mapping-basis values are (Lt, dLt); written to o[0], o[st], o[2 st]
  auto face_geo = [&](int cell, int f, const double *Lt, const double *dLt, double w,
                      double *o, int st) {
    const double *La, *dLa, *Lb, *dLb;
    double nr0, nr1;
    switch (f) {
      case 0: La = L0.data(); dLa = dL0.data(); Lb = Lt; dLb = dLt; nr0 = -1; nr1 = 0; break;
      case 1: La = L1.data(); dLa = dL1.data(); Lb = Lt; dLb = dLt; nr0 = 1; nr1 = 0; break;
      case 2: La = Lt; dLa = dLt; Lb = L0.data(); dLb = dL0.data(); nr0 = 0; nr1 = -1; break;
      default: La = Lt; dLa = dLt; Lb = L1.data(); dLb = dL1.data(); nr0 = 0; nr1 = 1; break;
    }
    double J[4];
    jac(cell, La, dLa, Lb, dLb, J);
    const double det = J[0] * J[3] - J[1] * J[2];
    // physical normal ~ J^{-T} n_ref; |J^{-T} n_ref| det = face metric
    const double t0 = (J[3] * nr0 - J[2] * nr1) / det;
    const double t1 = (-J[1] * nr0 + J[0] * nr1) / det;
    const double len = std::sqrt(t0 * t0 + t1 * t1);
    o[0] = t0 / len;
    o[st] = t1 / len;
    o[2 * st] = det * len * w;
  };
  for (int cell = 0; cell < nc; ++cell) {
    for (int qz = 0; qz < nq; ++qz)
      for (int qx = 0; qx < nq; ++qx) {
        double J[4];
        jac(cell, Lg[qx].data(), dLg[qx].data(), Lg[qz].data(), dLg[qz].data(), J);
        const double det = J[0] * J[3] - J[1] * J[2];
        if (!(det > 0.0)) {
          set_error("cell " + std::to_string(cell) + ": non-positive Jacobian");
          return ATM_BAD_ARG;
        }
        const double jxw = det * b.weights[qx] * b.weights[qz];
        const size_t base = (size_t)cell * 5 * nq2, q = (size_t)qz * nq + qx;
        qgeo[base + 0 * nq2 + q] = J[3] / det * jxw;   // dxi/dx
        qgeo[base + 1 * nq2 + q] = -J[1] / det * jxw;  // dxi/dz
        qgeo[base + 2 * nq2 + q] = -J[2] / det * jxw;  // deta/dx
        qgeo[base + 3 * nq2 + q] = J[0] / det * jxw;   // deta/dz
        qgeo[base + 4 * nq2 + q] = jxw;
      }
    for (int f = 0; f < 4; ++f)
      for (int q = 0; q < nq; ++q) {
        const size_t base = ((size_t)cell * 4 + f) * 3 * nq;
        face_geo(cell, f, Lg[q].data(), dLg[q].data(), b.weights[q], &fgeo[base + q], nq);
      }
  }
  // the mapping at degree 2: its values at (xi, eta) in {0, 1/2, 1}^2
  out.map2.assign((size_t)nc * 18, 0.0);
  {
    std::vector<double> L2[3];
    for (int a = 0; a < 3; ++a) {
      L2[a].resize(mn);
      lagrange_eval(mx, 0.5 * a, L2[a].data(), nullptr);
    }
    for (int cell = 0; cell < nc; ++cell)
      for (int e = 0; e < 3; ++e)
        for (int a = 0; a < 3; ++a)
          for (int bb = 0; bb < mn; ++bb)
            for (int aa = 0; aa < mn; ++aa) {
              const double *X = nodes + (((size_t)cell * mn + bb) * mn + aa) * 2;
              const double w = L2[a][aa] * L2[e][bb];
              for (int d = 0; d < 2; ++d) out.map2[(size_t)cell * 18 + (e * 3 + a) * 2 + d] += w * X[d];
            }
  }
  // subface geometry of the coarse side of every hanging face, at the points
  // (g_q + s)/2 of the coarse face with weights w_q/2
  out.hgeo.assign((size_t)out.nhang * 2 * 3 * nq, 0.0);
  std::vector<double> Ls, dLs;
  for (size_t a = 0; a < hidx.size(); ++a) {
    if (hidx[a] < 0) continue;
    const int cell = (int)(a / 4), f = (int)(a % 4), h = hidx[a];
    for (int s = 0; s < 2; ++s)
      for (int q = 0; q < nq; ++q) {
        tab(0.5 * (b.gauss[q] + s), Ls, dLs);
        face_geo(cell, f, Ls.data(), dLs.data(), 0.5 * b.weights[q],
                 &out.hgeo[((size_t)h * 2 + s) * 3 * nq + q], nq);
      }
  }
  return ATM_OK;
}

int mesh_upload(atm_ctx &c, int mapdeg, const double *nodes, int n_inner, const int *inner,
                int n_bdry, const int *bdry) {
  HostMesh hm;
  int rc = build_mesh_tables(c.k, c.nc, mapdeg, nodes, n_inner, inner, n_bdry, bdry, hm);
  if (rc) return rc;
  const int k = c.k, nn = k + 1, nq = 2 * k + 1, nq2 = nq * nq, nc = c.nc;
  mesh_free(c.mesh);
  Mesh &m = c.mesh;
  m.nc = nc; m.k = k; m.nn = nn; m.nq = nq; m.nn2 = nn * nn; m.nq2 = nq2;
  ATM_CUDA(cudaMalloc(&m.qgeo, hm.qgeo.size() * sizeof(double)));
  ATM_CUDA(cudaMalloc(&m.fgeo, hm.fgeo.size() * sizeof(double)));
  ATM_CUDA(cudaMalloc(&m.nbr, hm.nbr.size() * sizeof(int)));
  ATM_CUDA(cudaMalloc(&m.nbrf, hm.nbrf.size() * sizeof(int)));
  ATM_CUDA(cudaMalloc(&m.minv, (size_t)nc * m.nn2 * m.nn2 * sizeof(double)));
  ATM_CUDA(cudaMemcpyAsync(m.qgeo, hm.qgeo.data(), hm.qgeo.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  ATM_CUDA(cudaMemcpyAsync(m.fgeo, hm.fgeo.data(), hm.fgeo.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  ATM_CUDA(cudaMemcpyAsync(m.nbr, hm.nbr.data(), hm.nbr.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
  ATM_CUDA(cudaMemcpyAsync(m.nbrf, hm.nbrf.data(), hm.nbrf.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
  if (hm.nhang > 0) {
    ATM_CUDA(cudaMalloc(&m.hnb, hm.hnb.size() * sizeof(int)));
    ATM_CUDA(cudaMalloc(&m.hgeo, hm.hgeo.size() * sizeof(double)));
    ATM_CUDA(cudaMemcpyAsync(m.hnb, hm.hnb.data(), hm.hnb.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    ATM_CUDA(cudaMemcpyAsync(m.hgeo, hm.hgeo.data(), hm.hgeo.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  }
  m.nhang = hm.nhang;
  c.mapdeg = mapdeg;
  c.map2 = std::move(hm.map2);
  rc = launch_block_inverse(c, m.minv, nullptr);
  if (rc) return rc;
  rc = launch_inv_diag(c, c.invdiag_D, 1, nullptr, 1.0 / (GAS_GAMMA - 1.0));
  if (rc) return rc;
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  return ATM_OK;
}

}  // namespace atm
