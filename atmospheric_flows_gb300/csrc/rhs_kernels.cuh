// Explicit IMEX stage right-hand sides (FP64), one kernel per equation,
// templated on the polynomial degree K, the IMEX stage ST and HG (mesh with
// hanging faces).  Included by rhs_kernels.cu (HG = false) and
// hang_rhs_*.cu / hang_schur.cu (HG = true), so the two families compile in parallel.
//
//   rho      : euler_operator.h:344-473 (cell), 478-692 (face), no boundary
//   momentum : euler_operator.h:1622-1886 (cell), 1891-2184 (face),
//              2189-2305 (wall, p_D = p)
//   energy   : euler_operator.h:745-1007 (cell), 1012-1361 (face), no boundary
//
// 2D form of the reference's 3D operators: gravity acts along -e_z with the
// factor a^2/r^2 = 1 (euler_operator.h:790-811 on a Cartesian domain).
// The face formulas are evaluated from each cell's own side (element-centric):
// the reference's "+" and "-" contributions are the same expression with
// own/neighbour swapped and n -> -n, so every cell adds
//   -F(own, neighbour, n_own)
// for the explicit operators.
#pragma once
#include "atm_device.cuh"

namespace atm {

// ============================================================== rho rhs ===
template <int K, int ST, bool HG>
__global__ void __launch_bounds__(Cfg<K>::MAX_THREADS)
    k_rhs_rho(double *__restrict__ dst, SrcPtrs src, StageCoef co, Mesh mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2;
  const int CPB = blockDim.x / NQ;  // cells per block, chosen by the autotuner
  constexpr int NT = 3 * ST;
  extern __shared__ double sm[];
  double *tiles = sm;
  double *xab = tiles + CPB * NT * NN2;
  double *fb = xab + CPB * 2 * NN * NQ;
  double *fh = fb + CPB * 4 * NQ;  // subface-1 values (HG)
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
#pragma unroll
  for (int j = 0; j < ST; ++j) {
    load_tiles<K>(tiles, NT, 3 * j, src.p[2 * j], 1, c0, cnt);
    load_tiles<K>(tiles, NT, 3 * j + 1, src.p[2 * j + 1], 2, c0, cnt);
  }
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  if (mesh.dts && active) co.dt *= mesh.dts[c];  // per-member time step
  double Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  if (active) {
    const double *T = tiles + lc * NT * NN2;
    double gx[NQ], gz[NQ], v0[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) gx[q] = gz[q] = 0.0;
#pragma unroll
    for (int j = 0; j < ST; ++j) {
      double r[NQ], ux[NQ], uz[NQ];
      eval_col<K>(T + (3 * j) * NN2, Sx, r);
      eval_col<K>(T + (3 * j + 1) * NN2, Sx, ux);
      eval_col<K>(T + (3 * j + 2) * NN2, Sx, uz);
      const double w = co.ca[j] * co.dt;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        if (j == 0) v0[q] = r[q];
        gx[q] += w * r[q] * ux[q];
        gz[q] += w * r[q] * uz[q];
      }
    }
    const double *G = mesh.qgeo + (long)c * 5 * NQ2;
    double V[NQ], Gxi[NQ], Get[NQ];
#pragma unroll
    for (int qz = 0; qz < NQ; ++qz) {
      const QGeo g = qgeo<K>(G, qz * NQ + col);
      V[qz] = v0[qz] * g.jxw;
      Gxi[qz] = g.xx * gx[qz] + g.xz * gz[qz];
      Get[qz] = g.ex * gx[qz] + g.ez * gz[qz];
    }
    double *xa = xab + lc * 2 * NN * NQ;
    integrate_col_z<K, true, true>(V, Gxi, Get, xa, xa + NN * NQ, col);
    // faces
    face_terms<K, 1, HG>(mesh, c, col, Sx, fb + lc * 4 * NQ, fh + lc * 4 * NQ,
                         [&](int f, int nb, int nf, double n0, double n1, double jxw,
                             const auto &Ro, const auto &Rn, auto &val) {
      double flux = 0.0;
      if (nb >= 0) {
#pragma unroll
        for (int j = 0; j < ST; ++j) {
          const double rp = face_val<K>(T + (3 * j) * NN2, f, Ro);
          const double uxp = face_val<K>(T + (3 * j + 1) * NN2, f, Ro);
          const double uzp = face_val<K>(T + (3 * j + 2) * NN2, f, Ro);
          const double rm = face_val<K>(src.p[2 * j] + (long)nb * NN2, nf, Rn);
          const double uxm = face_val<K>(src.p[2 * j + 1] + (long)nb * 2 * NN2, nf, Rn);
          const double uzm = face_val<K>(src.p[2 * j + 1] + ((long)nb * 2 + 1) * NN2, nf, Rn);
          const double avg0 = 0.5 * (rp * uxp + rm * uxm);
          const double avg1 = 0.5 * (rp * uzp + rm * uzm);
          const double lam = fmax(fabs(uxp * n0 + uzp * n1), fabs(uxm * n0 + uzm * n1));
          flux += co.ca[j] * co.dt * ((avg0 * n0 + avg1 * n1) + 0.5 * lam * (rp - rm));
        }
      }
      val[0] = nb >= 0 ? -flux * jxw : 0.0;
    });
  }
  __syncthreads();
  if (active && col < NN) {
    double St[NQ], Dt[NQ], out[NN];
    load_cols<K>(col, St, Dt);
    const double *xa = xab + lc * 2 * NN * NQ;
    output_phase<K, HG>(mesh, c, xa, xa + NN * NQ, fb + lc * 4 * NQ, fh + lc * 4 * NQ, col, St, Dt,
                        out);
    double *d = dst + (long)c * NN2;
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) d[out_node<K, HG>(col, iz)] = out[iz];
  }
}

// ========================================================= momentum rhs ===
template <int K, int ST, bool HG>
__global__ void __launch_bounds__(Cfg<K>::MAX_THREADS)
    k_rhs_vel(double *__restrict__ dst, SrcPtrs src, StageCoef co, Mesh mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2;
  const int CPB = blockDim.x / NQ;  // cells per block, chosen by the autotuner
  constexpr int NG = (ST == 1) ? 2 : 3;             // gravity terms
  constexpr int NT = 4 * ST + (ST < 3 ? 1 : 0);     // tiles
  extern __shared__ double sm[];
  double *tiles = sm;
  double *xab = tiles + CPB * NT * NN2;             // [CPB][2 comp][2][NN*NQ]
  double *fb = xab + CPB * 4 * NN * NQ;             // [CPB][2 comp][4][NQ]
  double *fh = fb + CPB * 8 * NQ;                   // subface-1 values (HG)
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
#pragma unroll
  for (int j = 0; j < ST; ++j) {
    load_tiles<K>(tiles, NT, 4 * j, src.p[3 * j], 1, c0, cnt);
    load_tiles<K>(tiles, NT, 4 * j + 1, src.p[3 * j + 1], 2, c0, cnt);
    load_tiles<K>(tiles, NT, 4 * j + 3, src.p[3 * j + 2], 1, c0, cnt);
  }
  if (ST < 3) load_tiles<K>(tiles, NT, 4 * ST, src.p[3 * ST], 1, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  if (mesh.dts && active) co.dt *= mesh.dts[c];  // per-member time step
  double Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  const double dtM2 = co.dt / (co.Ma * co.Ma);
  if (active) {
    const double *T = tiles + lc * NT * NN2;
    double v0[NQ], v1[NQ], g00[NQ], g01[NQ], g10[NQ], g11[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) g00[q] = g01[q] = g10[q] = g11[q] = 0.0;
#pragma unroll
    for (int j = 0; j < ST; ++j) {
      double r[NQ], ux[NQ], uz[NQ], p[NQ];
      eval_col<K>(T + (4 * j) * NN2, Sx, r);
      eval_col<K>(T + (4 * j + 1) * NN2, Sx, ux);
      eval_col<K>(T + (4 * j + 2) * NN2, Sx, uz);
      eval_col<K>(T + (4 * j + 3) * NN2, Sx, p);
      const double wa = co.ca[j] * co.dt, wp = co.ct[j] * dtM2;
      const double wg = co.cg[j] * co.dt / (co.Fr * co.Fr);
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        if (j == 0) {
          v0[q] = r[q] * ux[q];
          v1[q] = r[q] * uz[q];
        }
        v1[q] -= wg * r[q];
        const double ru0 = wa * r[q] * ux[q], ru1 = wa * r[q] * uz[q];
        const double pp = wp * p[q];
        g00[q] += ru0 * ux[q] + pp;
        g01[q] += ru0 * uz[q];
        g10[q] += ru1 * ux[q];
        g11[q] += ru1 * uz[q] + pp;
      }
    }
    if (NG > ST) {  // implicit gravity term of the density being solved for
      double r[NQ];
      eval_col<K>(T + (4 * ST) * NN2, Sx, r);
      const double wg = co.cg[ST] * co.dt / (co.Fr * co.Fr);
#pragma unroll
      for (int q = 0; q < NQ; ++q) v1[q] -= wg * r[q];
    }
    const double *G = mesh.qgeo + (long)c * 5 * NQ2;
    double V[NQ], Gxi[NQ], Get[NQ];
    double *xa0 = xab + (lc * 2 + 0) * 2 * NN * NQ;
    double *xa1 = xab + (lc * 2 + 1) * 2 * NN * NQ;
#pragma unroll
    for (int qz = 0; qz < NQ; ++qz) {
      const QGeo g = qgeo<K>(G, qz * NQ + col);
      V[qz] = v0[qz] * g.jxw;
      Gxi[qz] = g.xx * g00[qz] + g.xz * g01[qz];
      Get[qz] = g.ex * g00[qz] + g.ez * g01[qz];
    }
    integrate_col_z<K, true, true>(V, Gxi, Get, xa0, xa0 + NN * NQ, col);
#pragma unroll
    for (int qz = 0; qz < NQ; ++qz) {
      const QGeo g = qgeo<K>(G, qz * NQ + col);
      V[qz] = v1[qz] * g.jxw;
      Gxi[qz] = g.xx * g10[qz] + g.xz * g11[qz];
      Get[qz] = g.ex * g10[qz] + g.ez * g11[qz];
    }
    integrate_col_z<K, true, true>(V, Gxi, Get, xa1, xa1 + NN * NQ, col);
    // faces
    face_terms<K, 2, HG>(mesh, c, col, Sx, fb + lc * 2 * 4 * NQ, fh + lc * 2 * 4 * NQ,
                         [&](int f, int nb, int nf, double n0, double n1, double jxw,
                             const auto &Ro, const auto &Rn, auto &val) {
      double f0 = 0.0, f1 = 0.0;
      if (nb >= 0) {
#pragma unroll
        for (int j = 0; j < ST; ++j) {
          const double rp = face_val<K>(T + (4 * j) * NN2, f, Ro);
          const double uxp = face_val<K>(T + (4 * j + 1) * NN2, f, Ro);
          const double uzp = face_val<K>(T + (4 * j + 2) * NN2, f, Ro);
          const double pp = face_val<K>(T + (4 * j + 3) * NN2, f, Ro);
          const double rm = face_val<K>(src.p[3 * j] + (long)nb * NN2, nf, Rn);
          const double uxm = face_val<K>(src.p[3 * j + 1] + (long)nb * 2 * NN2, nf, Rn);
          const double uzm = face_val<K>(src.p[3 * j + 1] + ((long)nb * 2 + 1) * NN2, nf, Rn);
          const double pm = face_val<K>(src.p[3 * j + 2] + (long)nb * NN2, nf, Rn);
          const double unp = uxp * n0 + uzp * n1, unm = uxm * n0 + uzm * n1;
          const double at0 = 0.5 * (rp * uxp * unp + rm * uxm * unm);
          const double at1 = 0.5 * (rp * uzp * unp + rm * uzm * unm);
          const double avgp = 0.5 * (pp + pm);
          const double lam = fmax(fabs(unp), fabs(unm));
          const double wa = co.ca[j] * co.dt, wp = co.ct[j] * dtM2;
          f0 += wa * at0 + wp * avgp * n0 + wa * 0.5 * lam * (rp * uxp - rm * uxm);
          f1 += wa * at1 + wp * avgp * n1 + wa * 0.5 * lam * (rp * uzp - rm * uzm);
        }
      } else {
        // no-flux wall: only the pressure term with p_D = p
#pragma unroll
        for (int j = 0; j < ST; ++j) {
          const double pp = face_val<K>(T + (4 * j + 3) * NN2, f, Ro);
          const double avg = 0.5 * (pp + pp);
          f0 += co.ct[j] * dtM2 * avg * n0;
          f1 += co.ct[j] * dtM2 * avg * n1;
        }
      }
      val[0] = -f0 * jxw;
      val[1] = -f1 * jxw;
    });
  }
  __syncthreads();
  if (active && col < NN) {
    double St[NQ], Dt[NQ];
    load_cols<K>(col, St, Dt);
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      double out[NN];
      const double *xa = xab + (lc * 2 + comp) * 2 * NN * NQ;
      output_phase<K, HG>(mesh, c, xa, xa + NN * NQ, fb + (lc * 2 + comp) * 4 * NQ, fh + (lc * 2 + comp) * 4 * NQ, col, St, Dt,
                          out);
      double *d = dst + ((long)c * 2 + comp) * NN2;
#pragma unroll
      for (int iz = 0; iz < NN; ++iz) d[out_node<K, HG>(col, iz)] = out[iz];
    }
  }
}

// ======================================================== energy rhs (p) ===
template <int K, int ST, bool HG>
__global__ void __launch_bounds__(Cfg<K>::MAX_THREADS)
    k_rhs_pres(double *__restrict__ dst, SrcPtrs src, StageCoef co, Mesh mesh) {
  using C = Cfg<K>;
  constexpr int NN = C::NN, NQ = C::NQ, NN2 = C::NN2, NQ2 = C::NQ2;
  const int CPB = blockDim.x / NQ;  // cells per block, chosen by the autotuner
  constexpr int NG = (ST == 1) ? 2 : 3;
  constexpr int NT = 4 * ST + 3;
  constexpr double GM1 = GAS_GAMMA - 1.0;
  // The reference forms E = p / ((gamma-1) rho) + Ma^2 |u|^2 / 2 and then
  // only uses rho E and rho (E - Ma^2 |u|^2 / 2) + p.  Those are
  // p / (gamma-1) + rho Ma^2 |u|^2 / 2 and gamma / (gamma-1) p: the division
  // by rho cancels, and the kernel forms the products directly (no FP64
  // division per point; the values agree to rounding).
  constexpr double IG = 1.0 / GM1, HGF = GAS_GAMMA / GM1;
  extern __shared__ double sm[];
  double *tiles = sm;
  double *xab = tiles + CPB * NT * NN2;
  double *fb = xab + CPB * 2 * NN * NQ;
  double *fh = fb + CPB * 4 * NQ;  // subface-1 values (HG)
  const int tid = threadIdx.x, lc = tid / NQ, col = tid - lc * NQ;
  const int c0 = blockIdx.x * CPB;
  const int cnt = min(CPB, mesh.nc - c0);
#pragma unroll
  for (int j = 0; j < ST; ++j) {
    load_tiles<K>(tiles, NT, 4 * j, src.p[3 * j], 1, c0, cnt);
    load_tiles<K>(tiles, NT, 4 * j + 1, src.p[3 * j + 1], 2, c0, cnt);
    load_tiles<K>(tiles, NT, 4 * j + 3, src.p[3 * j + 2], 1, c0, cnt);
  }
  load_tiles<K>(tiles, NT, 4 * ST, src.p[3 * ST], 1, c0, cnt);
  load_tiles<K>(tiles, NT, 4 * ST + 1, src.p[3 * ST + 1], 2, c0, cnt);
  __syncthreads();
  const bool active = lc < cnt;
  const int c = c0 + lc;
  if (mesh.dts && active) co.dt *= mesh.dts[c];  // per-member time step
  double Sx[NN], Dx[NN];
  load_rows<K>(col, Sx, Dx);
  const double M2 = co.Ma * co.Ma;
  if (active) {
    const double *T = tiles + lc * NT * NN2;
    double v[NQ], gx[NQ], gz[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] = gx[q] = gz[q] = 0.0;
#pragma unroll
    for (int j = 0; j < ST; ++j) {
      double r[NQ], ux[NQ], uz[NQ], p[NQ];
      eval_col<K>(T + (4 * j) * NN2, Sx, r);
      eval_col<K>(T + (4 * j + 1) * NN2, Sx, ux);
      eval_col<K>(T + (4 * j + 2) * NN2, Sx, uz);
      eval_col<K>(T + (4 * j + 3) * NN2, Sx, p);
      const double wgrav = co.cg[j] * co.dt * M2 / (co.Fr * co.Fr);
      const double wk = 0.5 * co.ca[j] * co.dt * M2;
      const double we = co.ct[j] * co.dt;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const double uu = ux[q] * ux[q] + uz[q] * uz[q];
        if (j == 0) v[q] += IG * p[q] + 0.5 * M2 * uu * r[q];  // rho E
        v[q] -= wgrav * r[q] * uz[q];
        const double kin = wk * uu * r[q];
        const double ent = we * HGF * p[q];  // rho (E - Ma^2 |u|^2 / 2) + p
        gx[q] += kin * ux[q] + ent * ux[q];
        gz[q] += kin * uz[q] + ent * uz[q];
      }
    }
    {
      // kinetic energy of the fixed-point velocity, and the implicit gravity
      // work of the density being solved for (stages 1, 2)
      double r[NQ], ux[NQ], uz[NQ];
      eval_col<K>(T + (4 * ST) * NN2, Sx, r);
      eval_col<K>(T + (4 * ST + 1) * NN2, Sx, ux);
      eval_col<K>(T + (4 * ST + 2) * NN2, Sx, uz);
      const double wgrav = (NG > ST) ? co.cg[ST] * co.dt * M2 / (co.Fr * co.Fr) : 0.0;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        v[q] -= 0.5 * r[q] * M2 * (ux[q] * ux[q] + uz[q] * uz[q]);
        if (NG > ST) v[q] -= wgrav * r[q] * uz[q];
      }
    }
    const double *G = mesh.qgeo + (long)c * 5 * NQ2;
    double V[NQ], Gxi[NQ], Get[NQ];
#pragma unroll
    for (int qz = 0; qz < NQ; ++qz) {
      const QGeo g = qgeo<K>(G, qz * NQ + col);
      V[qz] = v[qz] * g.jxw;
      Gxi[qz] = g.xx * gx[qz] + g.xz * gz[qz];
      Get[qz] = g.ex * gx[qz] + g.ez * gz[qz];
    }
    double *xa = xab + lc * 2 * NN * NQ;
    integrate_col_z<K, true, true>(V, Gxi, Get, xa, xa + NN * NQ, col);
    // faces
    face_terms<K, 1, HG>(mesh, c, col, Sx, fb + lc * 4 * NQ, fh + lc * 4 * NQ,
                         [&](int f, int nb, int nf, double n0, double n1, double jxw,
                             const auto &Ro, const auto &Rn, auto &val) {
      if (nb < 0) {
        val[0] = 0.0;
        return;
      }
      double flux = 0.0;
      double ux0p = 0.0, uz0p = 0.0, ux0m = 0.0, uz0m = 0.0;  // state-0 velocity traces
#pragma unroll
      for (int j = 0; j < ST; ++j) {
        const double rp = face_val<K>(T + (4 * j) * NN2, f, Ro);
        const double uxp = face_val<K>(T + (4 * j + 1) * NN2, f, Ro);
        const double uzp = face_val<K>(T + (4 * j + 2) * NN2, f, Ro);
        const double pp = face_val<K>(T + (4 * j + 3) * NN2, f, Ro);
        const double rm = face_val<K>(src.p[3 * j] + (long)nb * NN2, nf, Rn);
        const double uxm = face_val<K>(src.p[3 * j + 1] + (long)nb * 2 * NN2, nf, Rn);
        const double uzm = face_val<K>(src.p[3 * j + 1] + ((long)nb * 2 + 1) * NN2, nf, Rn);
        const double pm = face_val<K>(src.p[3 * j + 2] + (long)nb * NN2, nf, Rn);
        if (j == 0) { ux0p = uxp; uz0p = uzp; ux0m = uxm; uz0m = uzm; }
        const double uup = uxp * uxp + uzp * uzp, uum = uxm * uxm + uzm * uzm;
        const double unp = uxp * n0 + uzp * n1, unm = uxm * n0 + uzm * n1;
        const double akin = 0.5 * (0.5 * uup * rp * unp + 0.5 * uum * rm * unm);
        // enthalpy rho (E - Ma^2 |u|^2 / 2) + p of each side
        const double hp = HGF * pp, hm = HGF * pm;
        const double aent = 0.5 * (hp * unp + hm * unm);
        const double lam = fmax(fabs(unp), fabs(unm));
        const double wa = co.ca[j] * co.dt;
        if (ST == 3) {
          // stage 3 jumps the total rho E (euler_operator.h:1290,1313,1336)
          const double jE = IG * (pp - pm) + 0.5 * M2 * (rp * uup - rm * uum);
          flux += wa * M2 * akin + wa * aent + wa * 0.5 * lam * jE;
        } else {
          // stage 2 keeps the reference's mixed kinetic jump for tmp_2
          // (euler_operator.h:1182-1183)
          const double jkin = (ST == 2 && j == 1)
                                  ? rp * 0.5 * (uxp * ux0p + uzp * uz0p) -
                                        rm * 0.5 * (uxm * ux0m + uzm * uz0m)
                                  : rp * 0.5 * uup - rm * 0.5 * uum;
          const double je = IG * (pp - pm);  // jump of rho (E - Ma^2 |u|^2 / 2)
          flux += wa * M2 * (akin + 0.5 * lam * jkin) +
                  co.ct[j] * co.dt * (aent + 0.5 * lam * je);
        }
      }
      val[0] = -flux * jxw;
    });
  }
  __syncthreads();
  if (active && col < NN) {
    double St[NQ], Dt[NQ], out[NN];
    load_cols<K>(col, St, Dt);
    const double *xa = xab + lc * 2 * NN * NQ;
    output_phase<K, HG>(mesh, c, xa, xa + NN * NQ, fb + lc * 4 * NQ, fh + lc * 4 * NQ, col, St, Dt,
                        out);
    double *d = dst + (long)c * NN2;
#pragma unroll
    for (int iz = 0; iz < NN; ++iz) d[out_node<K, HG>(col, iz)] = out[iz];
  }
}

// ============================================================ launchers ===
// KIND 0 density, 1 momentum, 2 energy (a template parameter, so each kind's
// kernels can be instantiated in a translation unit of its own)
template <int K, bool HG, int KIND>
int rhs_launch(const atm_ctx &c, int stage, double *dst, const double *const *src,
               const StageCoef &co) {
  using C = Cfg<K>;
  constexpr int kind = KIND;
  SrcPtrs sp{};
  const int nsrc_tab[3][3] = {{2, 4, 6}, {4, 7, 9}, {5, 8, 11}};
  const int nsrc = nsrc_tab[kind][stage - 1];
  for (int i = 0; i < nsrc; ++i) sp.p[i] = src[i];
  int ntile;
  void (*fn)(double *, SrcPtrs, StageCoef, Mesh) = nullptr;
  if constexpr (KIND == 0) {
    ntile = 3 * stage;
    fn = stage == 1 ? k_rhs_rho<K, 1, HG> : (stage == 2 ? k_rhs_rho<K, 2, HG> : k_rhs_rho<K, 3, HG>);
  } else if constexpr (KIND == 1) {
    ntile = 4 * stage + (stage < 3 ? 1 : 0);
    fn = stage == 1 ? k_rhs_vel<K, 1, HG> : (stage == 2 ? k_rhs_vel<K, 2, HG> : k_rhs_vel<K, 3, HG>);
  } else {
    ntile = 4 * stage + 3;
    fn = stage == 1 ? k_rhs_pres<K, 1, HG> : (stage == 2 ? k_rhs_pres<K, 2, HG> : k_rhs_pres<K, 3, HG>);
  }
  const int ncomp = kind == 1 ? 2 : 1;
  auto launch = [&](int cpb) -> cudaError_t {
    const size_t sm = smem_bytes<K>(cpb, ntile, ncomp, HG);
    if (cudaError_t e = allow_smem(fn, sm); e != cudaSuccess) return e;
    fn<<<(c.nc + cpb - 1) / cpb, cpb * C::NQ, sm, c.stream>>>(dst, sp, co, c.mesh);
    return cudaGetLastError();
  };
  bool idem = true;  // the kernel only writes dst: safe to run repeatedly
  for (int i = 0; i < nsrc; ++i) idem = idem && src[i] != dst;
  const int cpb = tuned_cpb(c.autotune && !c.capturing, c.stream, TF_RHS_RHO + kind, K, stage,
                            HG, 8, c.nc, idem, launch);
  // algorithmic bytes: every source field read once, the result written once
  const double ns = (double)c.nc * C::NN2;
  const int nfields = (kind == 0) ? 3 * stage : (kind == 1 ? 4 * stage + (stage < 3) : 4 * stage + 3);
  const int nout = kind == 1 ? 2 : 1;
  const double bytes = 8.0 * ns * (nfields + nout);
  // contractions: evaluate every source tile, integrate values+gradients per
  // output component, face traces of both sides (4 faces) and face integration
  const int ntrace = (kind == 0) ? 3 * stage : 4 * stage;
  const double flops = c.nc * (nfields * fl_eval(K) + nout * fl_integrate(K, true) +
                               4.0 * (2 * ntrace * fl_face(K) + nout * fl_face(K)));
  TimedRegion tr(c, KF_RHS_RHO + kind, bytes, flops);
  ATM_CUDA(launch(cpb));
  g_kernel_launches.fetch_add(1);
  return ATM_OK;
}

template <bool HG, int KIND>
int rhs_dispatch_kind(const atm_ctx &c, int stage, double *dst, const double *const *src,
                      const StageCoef &co) {
  if (stage < 1 || stage > 3) return ATM_BAD_ARG;
  switch (c.k) {
    case 1: return rhs_launch<1, HG, KIND>(c, stage, dst, src, co);
    case 2: return rhs_launch<2, HG, KIND>(c, stage, dst, src, co);
    case 3: return rhs_launch<3, HG, KIND>(c, stage, dst, src, co);
    case 4: return rhs_launch<4, HG, KIND>(c, stage, dst, src, co);
    case 5: return rhs_launch<5, HG, KIND>(c, stage, dst, src, co);
    default: return ATM_BAD_ARG;
  }
}

}  // namespace atm
