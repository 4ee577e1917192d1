// The reference's own test case in 3D: FE_DGQ(1) hexahedra on a spherical
// shell with radial gravity (Atmospheric_Flow.cc:279-286, euler_operator.h,
// dim = 3, degree 1, QGauss(3)).  One kernel family restates every operator
// of the IMEX step for this case, and a host time loop drives it exactly as
// the 2D path does (Atmospheric_Flow.cc:1100-1257).
//
// Layout: scalar fields [cell][8], velocity [cell][3][8]; node v = ix + 2 iy
// + 4 iz on the cell's vertices (Gauss-Lobatto points of degree 1).  Cell
// geometry at the 27 Gauss points: dxi_e/dx_i * JxW (9 values), JxW, and the
// gravity direction e_r a^2/r^2 (3); face geometry at the 9 points of each
// local face: outward normal (3) and JxW.  Faces are element-centric: every
// cell adds its own side of each of its six faces, reading the neighbour's
// trace at the matching point (the face-point permutation handles the rotated
// and flipped parameterisations where cubed-sphere patches meet), so no
// atomics are needed.
//
// One thread per cell: the shell is the known-answer regression of the
// reference, a few thousand cells, not a throughput path.
#include <cmath>
#include <cstdio>
#include <vector>

#include "atm_device.cuh"

struct atm3_ctx;

namespace atm {
namespace s3 {

constexpr int NN = 8, NQ = 27, NF = 9;
constexpr double EARTH_A = 6.37122e6;  // equation_data.h:26

__constant__ double c_phi[NQ][NN];      // basis values at the cell points
__constant__ double c_dphi[NQ][NN][3];  // reference derivatives at the cell points
__constant__ double c_fphi[6][NF][NN];  // basis values at the face points

struct Geo3 {
  int nc;
  const double *cg;    // [nc][27][13]: G[e][i] (9), JxW, gvec (3)
  const double *fg;    // [nc][6][9][4]: n (3), JxW
  const int *nbr;      // [nc][6]: neighbour or -1 (wall)
  const int *nbf;      // [nc][6]: neighbour's local face
  const int *nperm;    // [nc][6][9]: neighbour's point of each own face point
};

struct Coef3 {
  double ca[3], ct[3], cg[3];
  int nst, ng;
  double dt, Ma, Fr;
};

__device__ __forceinline__ void load8(const double *v, int c, int ncomp, int comp, double *t) {
  const double *s = v + ((long)c * ncomp + comp) * NN;
#pragma unroll
  for (int i = 0; i < NN; ++i) t[i] = s[i];
}
__device__ __forceinline__ double at_q(const double *t, int q) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NN; ++i) s = fma(c_phi[q][i], t[i], s);
  return s;
}
// k-th (k < 4) vertex of local face f, in increasing vertex order: the
// vertices whose bit f/2 equals f%2.  The other four basis functions vanish
// on the face exactly, so the face sums below skip them.
__device__ __forceinline__ int fnode(int f, int k) {
  const int a = f >> 1, lo = k & ((1 << a) - 1);
  return lo | ((f & 1) << a) | ((k >> a) << (a + 1));
}
// the neighbour across face f of cell c at own face point q: its cell, its
// local face and the matching point there (loaded once per face point)
struct NbPt {
  int nb, nf, qn;
};
__device__ __forceinline__ NbPt nb_point(const Geo3 &g, int c, int f, int q) {
  return NbPt{g.nbr[c * 6 + f], g.nbf[c * 6 + f], g.nperm[(c * 6 + f) * NF + q]};
}
// The basis tables staged in a block's shared memory.  The warp-per-cell
// kernels index them by lane (point, face, vertex): from constant memory,
// whose cache serves one address per cycle, those divergent reads would be
// serialised.
constexpr int TAB3 = NQ * NN + NQ * NN * 3 + 6 * NF * NN;
struct Tab3S {
  const double (*phi)[NN];
  const double (*dphi)[NN][3];
  const double (*fphi)[NF][NN];
};
__device__ __forceinline__ Tab3S stage_tab3(double *buf) {
  const double *src[3] = {&c_phi[0][0], &c_dphi[0][0][0], &c_fphi[0][0][0]};
  const int len[3] = {NQ * NN, NQ * NN * 3, 6 * NF * NN};
  double *dst = buf;
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    for (int e = threadIdx.x; e < len[t]; e += blockDim.x) dst[e] = src[t][e];
    dst += len[t];
  }
  return Tab3S{reinterpret_cast<const double (*)[NN]>(buf),
               reinterpret_cast<const double (*)[NN][3]>(buf + NQ * NN),
               reinterpret_cast<const double (*)[NF][NN]>(buf + NQ * NN * 4)};
}
// value of the vertex field t at cell point q
__device__ __forceinline__ double at_qs(const double *t, int q, const Tab3S &T) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NN; ++i) s = fma(T.phi[q][i], t[i], s);
  return s;
}
// trace of t at point q of local face f (the face's four vertices)
__device__ __forceinline__ double at_faces(const double *t, int f, int q, const Tab3S &T) {
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) s = fma(T.fphi[f][q][fnode(f, k)], t[fnode(f, k)], s);
  return s;
}
// the neighbour's trace of component comp of a field with ncomp components
__device__ __forceinline__ double nb_vals(const NbPt &n, const double *v, int ncomp, int comp,
                                          const Tab3S &T) {
  const double *s = v + ((long)n.nb * ncomp + comp) * NN;
  double r = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) r = fma(T.fphi[n.nf][n.qn][fnode(n.nf, k)], s[fnode(n.nf, k)], r);
  return r;
}
// physical vector P (x JxW already) -> reference components Gr[e] = sum_i G[e][i] P_i
__device__ __forceinline__ void to_ref(const double *cgq, const double *P, double *Gr) {
#pragma unroll
  for (int e = 0; e < 3; ++e) Gr[e] = cgq[3 * e] * P[0] + cgq[3 * e + 1] * P[1] + cgq[3 * e + 2] * P[2];
}

// Every face-integral kernel runs one warp per cell (CELLS3 cells per
// block): lanes take the 27 quadrature points and the 54 face points of the
// cell, write their integrands to shared memory, and one lane per output
// node and component sums them against the basis.  One thread per cell
// would leave 6144 cells on a third of the SMs with long serial chains.
constexpr int CELLS3 = 4;

// Copy n values per cell of a field with ncomp components into shared memory:
// dst[comp][i] for the cell's components comp < ncomp (lanes of one warp).
__device__ __forceinline__ void tile3(double *dst, const double *src, int c, int ncomp,
                                      int lane) {
  for (int e = lane; e < ncomp * NN; e += 32) dst[e] = src[(long)c * ncomp * NN + e];
}

// For vertex i = lane % 8: the sum over the cell's points of
// V_q phi_i + Gr_q . grad phi_i and over the points of the three faces that
// hold the vertex of F_fq phi_i.  The four lanes of each vertex take every
// fourth term and the partial sums are combined by shuffles, so that all 32
// lanes work (an FP64 warp instruction costs the same with 8 active lanes as
// with 32).  Every lane of the warp must call it; lanes 0..7 hold the result
// of their vertex (all lanes do).
__device__ __forceinline__ double gather3(const double (*sv)[4], const double (*sf)[NF],
                                          int lane, const Tab3S &T) {
  const int i = lane & 7, part = lane >> 3;
  double o = 0.0;
  for (int q = part; q < NQ; q += 4)
    o += sv[q][0] * T.phi[q][i] + sv[q][1] * T.dphi[q][i][0] + sv[q][2] * T.dphi[q][i][1] +
         sv[q][3] * T.dphi[q][i][2];
  for (int t = part; t < 3 * NF; t += 4) {
    const int a = t / NF, q = t - a * NF, f = 2 * a + ((i >> a) & 1);
    o += sf[f][q] * T.fphi[f][q][i];
  }
  o += __shfl_xor_sync(0xffffffffu, o, 8);
  o += __shfl_xor_sync(0xffffffffu, o, 16);
  return o;
}

// The same sums for vertex i by one lane alone (three components at once
// keep 24 of the 32 lanes busy without the shuffles)
__device__ __forceinline__ double gather3_one(const double (*sv)[4], const double (*sf)[NF],
                                              int i, const Tab3S &T) {
  double o = 0.0;
  for (int q = 0; q < NQ; ++q)
    o += sv[q][0] * T.phi[q][i] + sv[q][1] * T.dphi[q][i][0] + sv[q][2] * T.dphi[q][i][1] +
         sv[q][3] * T.dphi[q][i][2];
  for (int a = 0; a < 3; ++a) {  // the faces holding vertex i, in increasing order
    const int f = 2 * a + ((i >> a) & 1);
#pragma unroll
    for (int q = 0; q < NF; ++q) o += sf[f][q] * T.fphi[f][q][i];
  }
  return o;
}

// ------------------------------------------------------------- rho rhs --
// euler_operator.h:344-712; src = (rho^(j), u^(j)) for j < nst
__global__ void __launch_bounds__(32 * CELLS3)
    k3_rhs_rho(double *__restrict__ dst, SrcPtrs src, Coef3 co, Geo3 g) {
  __shared__ double srt[CELLS3][3][NN], sut[CELLS3][3][3][NN];
  __shared__ double sv[CELLS3][NQ][4], sf[CELLS3][6][NF];
  const int lc = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * CELLS3 + lc;
  const bool active = c < g.nc;
  __shared__ double stab[TAB3];
  const Tab3S T = stage_tab3(stab);  // read after the first barrier
  if (active)
    for (int j = 0; j < co.nst; ++j) {
      tile3(srt[lc][j], src.p[2 * j], c, 1, lane);
      tile3(&sut[lc][j][0][0], src.p[2 * j + 1], c, 3, lane);
    }
  __syncthreads();
  if (active) {
    if (lane < NQ) {
      const int q = lane;
      const double *cq = g.cg + ((long)c * NQ + q) * 13;
      sv[lc][q][0] = at_qs(srt[lc][0], q, T) * cq[9];
      double P[3] = {0, 0, 0};
      for (int j = 0; j < co.nst; ++j) {
        const double r = at_qs(srt[lc][j], q, T), w = co.ca[j] * co.dt * r;
        for (int d = 0; d < 3; ++d) P[d] += w * at_qs(sut[lc][j][d], q, T);
      }
      to_ref(cq, P, &sv[lc][q][1]);
    }
    for (int e = lane; e < 6 * NF; e += 32) {
      const int f = e / NF, q = e - f * NF;
      double F = 0.0;
      if (g.nbr[c * 6 + f] >= 0) {  // no boundary term (euler_operator.h:111-114)
        const double *fq = g.fg + (((long)c * 6 + f) * NF + q) * 4;
        double flux = 0.0;
        const NbPt np = nb_point(g, c, f, q);
        for (int j = 0; j < co.nst; ++j) {
          const double ro = at_faces(srt[lc][j], f, q, T), rn = nb_vals(np, src.p[2 * j], 1, 0, T);
          double avg = 0.0, uno = 0.0, unn = 0.0;
          for (int d = 0; d < 3; ++d) {
            const double uo = at_faces(sut[lc][j][d], f, q, T);
            const double un = nb_vals(np, src.p[2 * j + 1], 3, d, T);
            avg += 0.5 * (ro * uo + rn * un) * fq[d];
            uno += uo * fq[d];
            unn += un * fq[d];
          }
          flux += co.ca[j] * co.dt * (avg + 0.5 * fmax(fabs(uno), fabs(unn)) * (ro - rn));
        }
        F = -flux * fq[3];
      }
      sf[lc][f][q] = F;
    }
  }
  __syncthreads();
  if (active) {  // warp-uniform: every lane of the cell's warp takes part
    const double o = gather3(sv[lc], sf[lc], lane, T);
    if (lane < NN) dst[(long)c * NN + lane] = o;
  }
}

// ------------------------------------------------------------ momentum --
// euler_operator.h:1622-2305; src = (rho, u, p)^(j) for j < nst, then the
// densities of the gravity terms at gsrc[0..ng)
__global__ void __launch_bounds__(32 * CELLS3)
    k3_rhs_vel(double *__restrict__ dst, SrcPtrs src, SrcPtrs gsrc, Coef3 co, Geo3 g) {
  __shared__ double srt[CELLS3][3][NN], sut[CELLS3][3][3][NN], spt[CELLS3][3][NN];
  __shared__ double sgt[CELLS3][3][NN];
  __shared__ double sv[CELLS3][3][NQ][4], sf[CELLS3][3][6][NF];  // per component d
  const int lc = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * CELLS3 + lc;
  const bool active = c < g.nc;
  __shared__ double stab[TAB3];
  const Tab3S T = stage_tab3(stab);  // read after the first barrier
  const double iM2 = 1.0 / (co.Ma * co.Ma), iF2 = 1.0 / (co.Fr * co.Fr);
  if (active) {
    for (int j = 0; j < co.nst; ++j) {
      tile3(srt[lc][j], src.p[3 * j], c, 1, lane);
      tile3(&sut[lc][j][0][0], src.p[3 * j + 1], c, 3, lane);
      tile3(spt[lc][j], src.p[3 * j + 2], c, 1, lane);
    }
    for (int j = 0; j < co.ng; ++j) tile3(sgt[lc][j], gsrc.p[j], c, 1, lane);
  }
  __syncthreads();
  if (active) {
    if (lane < NQ) {
      const int q = lane;
      const double *cq = g.cg + ((long)c * NQ + q) * 13;
      for (int d = 0; d < 3; ++d) {
        double v = at_qs(srt[lc][0], q, T) * at_qs(sut[lc][0][d], q, T);
        for (int j = 0; j < co.ng; ++j)
          v -= co.cg[j] * co.dt * iF2 * at_qs(sgt[lc][j], q, T) * cq[10 + d];
        sv[lc][d][q][0] = v * cq[9];
        double P[3] = {0, 0, 0};
        for (int j = 0; j < co.nst; ++j) {
          const double ru = co.ca[j] * co.dt * at_qs(srt[lc][j], q, T) * at_qs(sut[lc][j][d], q, T);
          for (int k = 0; k < 3; ++k) P[k] += ru * at_qs(sut[lc][j][k], q, T);
          P[d] += co.ct[j] * co.dt * iM2 * at_qs(spt[lc][j], q, T);
        }
        to_ref(cq, P, &sv[lc][d][q][1]);  // the geometry factors carry JxW
      }
    }
    for (int e = lane; e < 6 * NF; e += 32) {
      const int f = e / NF, q = e - f * NF;
      const NbPt np = nb_point(g, c, f, q);
      const bool wall = np.nb < 0;
      const double *fq = g.fg + (((long)c * 6 + f) * NF + q) * 4;
      double fl[3] = {0, 0, 0};
      for (int j = 0; j < co.nst; ++j) {
        const double po = at_faces(spt[lc][j], f, q, T);
        if (wall) {  // p_D = p (euler_operator.h:2189-2305)
          for (int d = 0; d < 3; ++d) fl[d] += co.ct[j] * co.dt * iM2 * 0.5 * (po + po) * fq[d];
          continue;
        }
        const double ro = at_faces(srt[lc][j], f, q, T), rn = nb_vals(np, src.p[3 * j], 1, 0, T);
        const double pn = nb_vals(np, src.p[3 * j + 2], 1, 0, T);
        double uo[3], un[3], uno = 0.0, unn = 0.0;
        for (int k = 0; k < 3; ++k) {
          uo[k] = at_faces(sut[lc][j][k], f, q, T);
          un[k] = nb_vals(np, src.p[3 * j + 1], 3, k, T);
          uno += uo[k] * fq[k];
          unn += un[k] * fq[k];
        }
        const double lam = fmax(fabs(uno), fabs(unn));
        for (int d = 0; d < 3; ++d)
          fl[d] += co.ca[j] * co.dt * 0.5 * (ro * uo[d] * uno + rn * un[d] * unn) +
                   co.ct[j] * co.dt * iM2 * 0.5 * (po + pn) * fq[d] +
                   co.ca[j] * co.dt * 0.5 * lam * (ro * uo[d] - rn * un[d]);
      }
      for (int d = 0; d < 3; ++d) sf[lc][d][f][q] = -fl[d] * fq[3];
    }
  }
  __syncthreads();
  if (active && lane < 3 * NN) {
    const int d = lane / NN, i = lane - d * NN;
    dst[((long)c * 3 + d) * NN + i] = gather3_one(sv[lc][d], sf[lc][d], i, T);
  }
}

// -------------------------------------------------------------- energy --
// euler_operator.h:745-1381 with the radial gravity work (:790-811), the
// stage-2 kinetic jump mixing in u_old (:1182-1183) and the stage-3 total
// rho E jump (:1290-1336).  src = (rho, u, p)^(j); gsrc = gravity densities
// and velocities (rho, u)^(j) for j < ng, then the kinetic (rho, u).  The
// reference's E = p / ((gamma-1) rho) + Ma^2 |u|^2 / 2 only enters as rho E
// and rho (E - Ma^2 |u|^2 / 2) + p, where the division by rho cancels: the
// kernel forms p / (gamma-1) + rho Ma^2 |u|^2 / 2 and gamma p / (gamma-1).
__global__ void __launch_bounds__(32 * CELLS3)
    k3_rhs_pres(double *__restrict__ dst, SrcPtrs src, SrcPtrs gsrc, Coef3 co, int hstage,
                Geo3 g) {
  __shared__ double srt[CELLS3][3][NN], sut[CELLS3][3][3][NN], spt[CELLS3][3][NN];
  __shared__ double sgr[CELLS3][4][NN], sgu[CELLS3][4][3][NN];  // gravity j < ng, kinetic
  __shared__ double sv[CELLS3][NQ][4], sf[CELLS3][6][NF];
  const int lc = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * CELLS3 + lc;
  const bool active = c < g.nc;
  __shared__ double stab[TAB3];
  const Tab3S T = stage_tab3(stab);  // read after the first barrier
  const double ig = 1.0 / (GAS_GAMMA - 1.0), hgf = GAS_GAMMA / (GAS_GAMMA - 1.0);
  const double M2 = co.Ma * co.Ma, iF2 = 1.0 / (co.Fr * co.Fr);
  if (active) {
    for (int j = 0; j < co.nst; ++j) {
      tile3(srt[lc][j], src.p[3 * j], c, 1, lane);
      tile3(&sut[lc][j][0][0], src.p[3 * j + 1], c, 3, lane);
      tile3(spt[lc][j], src.p[3 * j + 2], c, 1, lane);
    }
    for (int j = 0; j <= co.ng; ++j) {  // j = ng: the kinetic (rho, u)
      tile3(sgr[lc][j], gsrc.p[2 * j], c, 1, lane);
      tile3(&sgu[lc][j][0][0], gsrc.p[2 * j + 1], c, 3, lane);
    }
  }
  __syncthreads();
  if (active) {
    if (lane < NQ) {
      const int q = lane;
      const double *cq = g.cg + ((long)c * NQ + q) * 13;
      const double r0 = at_qs(srt[lc][0], q, T), p0 = at_qs(spt[lc][0], q, T);
      double uu0 = 0.0;
      for (int d = 0; d < 3; ++d) {
        const double u = at_qs(sut[lc][0][d], q, T);
        uu0 += u * u;
      }
      const double kr = at_qs(sgr[lc][co.ng], q, T);
      double kk = 0.0;
      for (int d = 0; d < 3; ++d) {
        const double kv = at_qs(sgu[lc][co.ng][d], q, T);
        kk += kv * kv;
      }
      double v = ig * p0 + 0.5 * M2 * uu0 * r0 - 0.5 * kr * M2 * kk;  // rho E - kinetic
      for (int j = 0; j < co.ng; ++j) {
        const double gr = at_qs(sgr[lc][j], q, T);
        double ue = 0.0;
        for (int d = 0; d < 3; ++d) ue += at_qs(sgu[lc][j][d], q, T) * cq[10 + d];  // u . e_r a^2/r^2
        v -= co.cg[j] * co.dt * M2 * iF2 * gr * ue;
      }
      sv[lc][q][0] = v * cq[9];
      double P[3] = {0, 0, 0};
      for (int j = 0; j < co.nst; ++j) {
        const double r = at_qs(srt[lc][j], q, T), p = at_qs(spt[lc][j], q, T);
        double u[3], uu = 0.0;
        for (int d = 0; d < 3; ++d) {
          u[d] = at_qs(sut[lc][j][d], q, T);
          uu += u[d] * u[d];
        }
        const double w = 0.5 * co.ca[j] * co.dt * M2 * uu * r + co.ct[j] * co.dt * hgf * p;
        for (int d = 0; d < 3; ++d) P[d] += w * u[d];
      }
      to_ref(cq, P, &sv[lc][q][1]);
    }
    for (int e = lane; e < 6 * NF; e += 32) {
      const int f = e / NF, q = e - f * NF;
      double F = 0.0;
      if (g.nbr[c * 6 + f] >= 0) {  // no boundary term
        const double *fq = g.fg + (((long)c * 6 + f) * NF + q) * 4;
        const NbPt np = nb_point(g, c, f, q);
        double uo[3][3], un[3][3];
        for (int j = 0; j < co.nst; ++j)
          for (int d = 0; d < 3; ++d) {
            uo[j][d] = at_faces(sut[lc][j][d], f, q, T);
            un[j][d] = nb_vals(np, src.p[3 * j + 1], 3, d, T);
          }
        double flux = 0.0;
        for (int j = 0; j < co.nst; ++j) {
          const double ro = at_faces(srt[lc][j], f, q, T), rn = nb_vals(np, src.p[3 * j], 1, 0, T);
          const double po = at_faces(spt[lc][j], f, q, T), pn = nb_vals(np, src.p[3 * j + 2], 1, 0, T);
          double uuo = 0, uun = 0, uno = 0, unn = 0;
          for (int d = 0; d < 3; ++d) {
            uuo += uo[j][d] * uo[j][d]; uun += un[j][d] * un[j][d];
            uno += uo[j][d] * fq[d]; unn += un[j][d] * fq[d];
          }
          const double akin = 0.5 * (0.5 * uuo * ro * uno + 0.5 * uun * rn * unn);
          const double aent = 0.5 * (hgf * po * uno + hgf * pn * unn);
          const double lam = fmax(fabs(uno), fabs(unn));
          if (hstage == 3) {  // jump of the total rho E
            const double jE = ig * (po - pn) + 0.5 * M2 * (ro * uuo - rn * uun);
            flux += co.ca[j] * co.dt * M2 * akin + co.ca[j] * co.dt * aent +
                    co.ca[j] * co.dt * 0.5 * lam * jE;
          } else {
            double jk;
            if (hstage == 2 && j == 1) {
              double ko = 0, kn = 0;
              for (int d = 0; d < 3; ++d) { ko += uo[1][d] * uo[0][d]; kn += un[1][d] * un[0][d]; }
              jk = ro * 0.5 * ko - rn * 0.5 * kn;
            } else {
              jk = ro * 0.5 * uuo - rn * 0.5 * uun;
            }
            const double je = ig * (po - pn);  // jump of rho (E - Ma^2 |u|^2 / 2)
            flux += co.ca[j] * co.dt * M2 * (akin + 0.5 * lam * jk) +
                    co.ct[j] * co.dt * (aent + 0.5 * lam * je);
          }
        }
        F = -flux * fq[3];
      }
      sf[lc][f][q] = F;
    }
  }
  __syncthreads();
  if (active) {  // warp-uniform: every lane of the cell's warp takes part
    const double o = gather3(sv[lc], sf[lc], lane, T);
    if (lane < NN) dst[(long)c * NN + lane] = o;
  }
}

// ------------------------------------------------------------------- B --
// euler_operator.h:1512-1617; mode 0 dst = B p, 1 dst -= B p, 2 dst = A^{-1} B p
__global__ void __launch_bounds__(32 * CELLS3)
    k3_B(double *__restrict__ dst, const double *__restrict__ p, double cB,
         const double *__restrict__ ainv, int mode, Geo3 g) {
  __shared__ double sp[CELLS3][NN];            // p on the cell's vertices
  __shared__ double sgr[CELLS3][NQ][3][3];     // [q][d][e]: -cB p(q) dxi_e/dx_d JxW
  __shared__ double sfn[CELLS3][6][NF][3];     // [f][q][d]: cB {p} n_d JxW
  __shared__ double sout[CELLS3][3][NN];
  const int lc = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * CELLS3 + lc;
  const bool active = c < g.nc;
  __shared__ double stab[TAB3];
  const Tab3S T = stage_tab3(stab);  // read after the first barrier
  if (active && lane < NN) sp[lc][lane] = p[(long)c * NN + lane];
  __syncthreads();
  if (active) {
    if (lane < NQ) {
      const int q = lane;
      const double *cq = g.cg + ((long)c * NQ + q) * 13;
      const double s = -cB * at_qs(sp[lc], q, T);
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int e = 0; e < 3; ++e) sgr[lc][q][d][e] = s * cq[3 * e + d];
    }
    for (int e = lane; e < 6 * NF; e += 32) {
      const int f = e / NF, q = e - f * NF;
      const double *fq = g.fg + (((long)c * 6 + f) * NF + q) * 4;
      const double po = at_faces(sp[lc], f, q, T);
      const NbPt np = nb_point(g, c, f, q);
      const double pn = np.nb < 0 ? po : nb_vals(np, p, 1, 0, T);
      const double a = cB * 0.5 * (po + pn) * fq[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) sfn[lc][f][q][d] = a * fq[d];
    }
  }
  __syncthreads();
  if (active) {  // warp-uniform; per component, four lanes per vertex (as gather3)
    const int i = lane & 7, part = lane >> 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double o = 0.0;
      for (int q = part; q < NQ; q += 4)
        o += sgr[lc][q][d][0] * T.dphi[q][i][0] + sgr[lc][q][d][1] * T.dphi[q][i][1] +
             sgr[lc][q][d][2] * T.dphi[q][i][2];
      for (int t = part; t < 3 * NF; t += 4) {  // the faces holding vertex i
        const int a = t / NF, q = t - a * NF, f = 2 * a + ((i >> a) & 1);
        o += sfn[lc][f][q][d] * T.fphi[f][q][i];
      }
      o += __shfl_xor_sync(0xffffffffu, o, 8);
      o += __shfl_xor_sync(0xffffffffu, o, 16);
      if (lane < NN) sout[lc][d][i] = o;
    }
  }
  __syncthreads();
  if (active && lane < 3 * NN) {
    const int d = lane / NN, i = lane - d * NN;
    const long gi = ((long)c * 3 + d) * NN + i;
    if (mode == 2) {
      const double *A = ainv + (long)c * NN * NN + i * NN;
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < NN; ++j) s += A[j] * sout[lc][d][j];
      dst[gi] = s;
    } else {
      dst[gi] = mode == 0 ? sout[lc][d][i] : dst[gi] - sout[lc][d][i];
    }
  }
}

// ----------------------------------------------------------------- C/D --
// euler_operator.h:1386-1507.  mode 0 dst = C w; 1 dst = D p - C w;
// 2 dst = invd .* (D p - C w); 3 dst -= C w.  D = mass / (gamma - 1).
__global__ void __launch_bounds__(32 * CELLS3)
    k3_CD(double *__restrict__ dst, const double *__restrict__ w,
          const double *__restrict__ p, const double *__restrict__ pfix, double cC,
          const double *__restrict__ invd, int mode, Geo3 g) {
  __shared__ double swt[CELLS3][3][NN], sft[CELLS3][NN], spt[CELLS3][NN];
  __shared__ double sv[CELLS3][NQ][4];         // [q]: V, Gr (3)
  __shared__ double sfa[CELLS3][6][NF];        // [f][q]: face flux x JxW
  const int lc = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * CELLS3 + lc;
  const bool active = c < g.nc;
  __shared__ double stab[TAB3];
  const Tab3S T = stage_tab3(stab);  // read after the first barrier
  // 1/(gamma-1) as a constant factor: a division by (gamma-1) at every point
  // would cost an FP64 division sequence each (the values agree to rounding)
  const double hg = GAS_GAMMA / (GAS_GAMMA - 1.0), ig = 1.0 / (GAS_GAMMA - 1.0);
  const bool withD = mode == 1 || mode == 2;
  const double sc = withD ? -1.0 : 1.0;  // sign of C in dst
  if (active && lane < 3 * NN) swt[lc][lane / NN][lane % NN] = w[(long)c * 3 * NN + lane];
  if (active && lane < NN) {
    sft[lc][lane] = pfix[(long)c * NN + lane];
    if (withD) spt[lc][lane] = p[(long)c * NN + lane];
  }
  __syncthreads();
  if (active) {
    if (lane < NQ) {
      const int q = lane;
      const double *cq = g.cg + ((long)c * NQ + q) * 13;
      const double pf = at_qs(sft[lc], q, T);
      double P[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) P[d] = sc * (-cC * hg * pf * at_qs(swt[lc][d], q, T));
      double Gr[3];
      to_ref(cq, P, Gr);
      sv[lc][q][0] = withD ? at_qs(spt[lc], q, T) * ig * cq[9] : 0.0;
#pragma unroll
      for (int e = 0; e < 3; ++e) sv[lc][q][1 + e] = Gr[e];
    }
    for (int e = lane; e < 6 * NF; e += 32) {
      const int f = e / NF, q = e - f * NF;
      double a = 0.0;
      const NbPt np = nb_point(g, c, f, q);
      if (np.nb >= 0) {  // no boundary term
        const double *fq = g.fg + (((long)c * 6 + f) * NF + q) * 4;
        const double pfo = at_faces(sft[lc], f, q, T), pfn = nb_vals(np, pfix, 1, 0, T);
        double av = 0.0, wno = 0.0, wnn = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const double wo = at_faces(swt[lc][d], f, q, T), wn = nb_vals(np, w, 3, d, T);
          av += 0.5 * hg * (pfo * wo + pfn * wn) * fq[d];
          wno += wo * fq[d];
          wnn += wn * fq[d];
        }
        const double lam = fmax(fabs(wno), fabs(wnn));
        a = sc * cC * (av + 0.5 * lam * (pfo - pfn) * ig) * fq[3];
      }
      sfa[lc][f][q] = a;
    }
  }
  __syncthreads();
  if (active) {  // warp-uniform: every lane of the cell's warp takes part
    const double o = gather3(sv[lc], sfa[lc], lane, T);
    if (lane >= NN) return;
    const int i = lane;
    const long gi = (long)c * NN + i;
    if (mode == 2) dst[gi] = invd[gi] * o;
    else if (mode == 3) dst[gi] -= o;
    else dst[gi] = o;
  }
}

// ------------------------------------------------ cell-wise mass inverses --
// inv = (sum_q w(q) phi_i phi_j JxW)^{-1} per cell, weight tile or 1;
// Gauss-Jordan with partial pivoting on the 8x8 block
__global__ void k3_block_inverse(double *__restrict__ inv, const double *__restrict__ weight,
                                 Geo3 g) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nc) return;
  double wt[NN];
  if (weight) load8(weight, c, 1, 0, wt);
  double M[NN][2 * NN];
  for (int i = 0; i < NN; ++i)
    for (int j = 0; j < 2 * NN; ++j) M[i][j] = (j - NN == i) ? 1.0 : 0.0;
  for (int q = 0; q < NQ; ++q) {
    const double jw = g.cg[((long)c * NQ + q) * 13 + 9] * (weight ? at_q(wt, q) : 1.0);
    for (int i = 0; i < NN; ++i)
      for (int j = 0; j < NN; ++j) M[i][j] += jw * c_phi[q][i] * c_phi[q][j];
  }
  for (int k = 0; k < NN; ++k) {
    int piv = k;
    for (int i = k + 1; i < NN; ++i)
      if (fabs(M[i][k]) > fabs(M[piv][k])) piv = i;
    if (piv != k)
      for (int j = 0; j < 2 * NN; ++j) { const double t = M[k][j]; M[k][j] = M[piv][j]; M[piv][j] = t; }
    const double d = 1.0 / M[k][k];
    for (int j = 0; j < 2 * NN; ++j) M[k][j] *= d;
    for (int i = 0; i < NN; ++i) {
      if (i == k) continue;
      const double f = M[i][k];
      for (int j = 0; j < 2 * NN; ++j) M[i][j] -= f * M[k][j];
    }
  }
  for (int i = 0; i < NN; ++i)
    for (int j = 0; j < NN; ++j) inv[(long)c * NN * NN + i * NN + j] = M[i][NN + j];
}

// dst = scale * inv src, ncomp components per cell
__global__ void k3_block_apply(double *__restrict__ dst, const double *__restrict__ src,
                               const double *__restrict__ inv, int ncomp, double scale, int nc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double *A = inv + (long)c * NN * NN;
  for (int d = 0; d < ncomp; ++d) {
    double t[NN];
    load8(src, c, ncomp, d, t);
    for (int i = 0; i < NN; ++i) {
      double s = 0.0;
      for (int j = 0; j < NN; ++j) s += A[i * NN + j] * t[j];
      dst[((long)c * ncomp + d) * NN + i] = scale * s;
    }
  }
}

// mass apply dst = M_w src (ncomp components, weight tile or constant)
__global__ void k3_mass(double *__restrict__ dst, const double *__restrict__ src, int ncomp,
                        const double *__restrict__ weight, double scale, Geo3 g) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nc) return;
  double wt[NN];
  if (weight) load8(weight, c, 1, 0, wt);
  for (int d = 0; d < ncomp; ++d) {
    double t[NN], out[NN] = {0};
    load8(src, c, ncomp, d, t);
    for (int q = 0; q < NQ; ++q) {
      const double v = at_q(t, q) * (weight ? at_q(wt, q) : scale) *
                       g.cg[((long)c * NQ + q) * 13 + 9];
#pragma unroll
      for (int i = 0; i < NN; ++i) out[i] += v * c_phi[q][i];
    }
    for (int i = 0; i < NN; ++i) dst[((long)c * ncomp + d) * NN + i] = out[i];
  }
}

// inverse diagonal of D (the Schur Jacobi, euler_operator.h:2607-2611)
__global__ void k3_invdiag_D(double *__restrict__ out, Geo3 g) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nc) return;
  for (int i = 0; i < NN; ++i) {
    double s = 0.0;
    for (int q = 0; q < NQ; ++q)
      s += c_phi[q][i] * c_phi[q][i] * g.cg[((long)c * NQ + q) * 13 + 9];
    out[(long)c * NN + i] = (GAS_GAMMA - 1.0) / s;
  }
}

}  // namespace s3
}  // namespace atm

// ============================================================================
// Host side: context, set-up, operators and the IMEX loop
// ============================================================================
using namespace atm;
using namespace atm::s3;

struct atm3_ctx {
  int device = 0, nc = 0;
  cudaStream_t stream = nullptr;
  Geo3 g{};
  double *cg = nullptr, *fg = nullptr;
  int *nbr = nullptr, *nbf = nullptr, *nperm = nullptr;
  double dt = 1.0, Ma = 1.0, Fr = 1.0;
  int hstage = 1, nsstage = 1;
  Tableau tab;
  double *rho_fix = nullptr, *pres_fix = nullptr, *u_fix = nullptr;
  double *minv = nullptr, *ainv = nullptr, *invd = nullptr;
  double *wv1 = nullptr, *ws1 = nullptr, *ws2 = nullptr;
  double *red = nullptr, *red_out = nullptr, *h_red = nullptr, *dsmall = nullptr;
  double *krylov = nullptr;
  // solver
  bool solver = false;
  double eps = 1e-8;
  int max_its = 30000;
  bool scaled_tol = false, true_check = false;
  long steps = 0, picard_total = 0, krylov_total = 0, failures = 0;
  double *pool = nullptr;
  double *rho_old, *rho_2, *rho_3, *rho_cur, *rhs_rho, *p_old, *p_2, *p_3, *p_fix, *p_fix_old,
      *rhs_p, *u_old, *u_2, *u_3, *u_cur, *u_fixd, *rhs_u, *tmp_1;
  long ns() const { return (long)nc * NN; }
  long nv() const { return 3L * nc * NN; }
};

namespace {

constexpr int RESTART3 = 28;
#define TRY3(x)           \
  do {                    \
    int _rc = (x);        \
    if (_rc) return _rc;  \
  } while (0)

inline int blocks(int n) { return (n + 127) / 128; }

int upload_tables3() {
  // degree-1 basis on the vertices, 3-point Gauss rule on [0, 1]
  const double s = std::sqrt(0.6);
  const double gx[3] = {0.5 * (1.0 - s), 0.5, 0.5 * (1.0 + s)};
  double phi[NQ][NN], dphi[NQ][NN][3], fphi[6][NF][NN];
  auto q1 = [](const double xi[3], double *ph, double (*dp)[3]) {
    for (int v = 0; v < NN; ++v) {
      double f[3], df[3];
      for (int d = 0; d < 3; ++d) {
        const bool hi = (v >> d) & 1;
        f[d] = hi ? xi[d] : 1.0 - xi[d];
        df[d] = hi ? 1.0 : -1.0;
      }
      ph[v] = f[0] * f[1] * f[2];
      if (dp) {
        dp[v][0] = df[0] * f[1] * f[2];
        dp[v][1] = f[0] * df[1] * f[2];
        dp[v][2] = f[0] * f[1] * df[2];
      }
    }
  };
  for (int q = 0; q < NQ; ++q) {
    const double xi[3] = {gx[q % 3], gx[(q / 3) % 3], gx[q / 9]};
    q1(xi, phi[q], dphi[q]);
  }
  for (int f = 0; f < 6; ++f)
    for (int q = 0; q < NF; ++q) {
      const int d = f / 2, t0 = d == 0 ? 1 : 0, t1 = d == 2 ? 1 : 2;
      double xi[3];
      xi[d] = (double)(f % 2);
      xi[t0] = gx[q % 3];
      xi[t1] = gx[q / 3];
      q1(xi, fphi[f][q], nullptr);
    }
  if (cudaMemcpyToSymbol(c_phi, phi, sizeof(phi)) != cudaSuccess ||
      cudaMemcpyToSymbol(c_dphi, dphi, sizeof(dphi)) != cudaSuccess ||
      cudaMemcpyToSymbol(c_fphi, fphi, sizeof(fphi)) != cudaSuccess) {
    set_error("failed to upload the 3D basis tables");
    return ATM_CUDA_ERROR;
  }
  return ATM_OK;
}

// x and dx/dxi of the degree-2 mapping of one cell at xi
void map3(const double *nodes, const double xi[3], double x[3], double J[3][3]) {
  double v[3][3], d[3][3];
  for (int e = 0; e < 3; ++e) {
    const double t = xi[e];
    v[e][0] = 2.0 * (t - 0.5) * (t - 1.0); v[e][1] = -4.0 * t * (t - 1.0); v[e][2] = 2.0 * t * (t - 0.5);
    d[e][0] = 4.0 * t - 3.0; d[e][1] = -8.0 * t + 4.0; d[e][2] = 4.0 * t - 1.0;
  }
  for (int i = 0; i < 3; ++i) {
    x[i] = 0.0;
    for (int e = 0; e < 3; ++e) J[i][e] = 0.0;
  }
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) {
        const double *X = nodes + 3 * ((c * 3 + b) * 3 + a);
        const double w = v[0][a] * v[1][b] * v[2][c];
        const double dw[3] = {d[0][a] * v[1][b] * v[2][c], v[0][a] * d[1][b] * v[2][c],
                              v[0][a] * v[1][b] * d[2][c]};
        for (int i = 0; i < 3; ++i) {
          x[i] += w * X[i];
          for (int e = 0; e < 3; ++e) J[i][e] += dw[e] * X[i];
        }
      }
}

// inverse of J (Ji[e][i] = dxi_e/dx_i) and det
double inv3(const double J[3][3], double Ji[3][3]) {
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  for (int e = 0; e < 3; ++e)
    for (int i = 0; i < 3; ++i) {
      // cofactor of J[i][e]
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, e1 = (e + 1) % 3, e2 = (e + 2) % 3;
      Ji[e][i] = (J[i1][e1] * J[i2][e2] - J[i1][e2] * J[i2][e1]) / det;
    }
  return det;
}

int alloc3(atm3_ctx &c, double **p, size_t n) {
  ATM_CUDA(cudaMalloc(p, n * sizeof(double)));
  ATM_CUDA(cudaMemsetAsync(*p, 0, n * sizeof(double), c.stream));
  return ATM_OK;
}

void free3(atm3_ctx *c) {
  if (!c) return;
  double *ds[] = {c->cg, c->fg, c->rho_fix, c->pres_fix, c->u_fix, c->minv, c->ainv, c->invd,
                  c->wv1, c->ws1, c->ws2, c->red, c->red_out, c->dsmall, c->krylov, c->pool};
  for (double *d : ds) cudaFree(d);
  cudaFree(c->nbr); cudaFree(c->nbf); cudaFree(c->nperm);
  if (c->h_red) cudaFreeHost(c->h_red);
  delete c;
}

int read3(atm3_ctx &c, const double *dev, int n) {
  ATM_CUDA(cudaMemcpyAsync(c.h_red, dev, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  ATM_CUDA(cudaStreamSynchronize(c.stream));
  return ATM_OK;
}

Coef3 coef3(const atm3_ctx &c, int stage, bool rho_only) {
  Coef3 s{};
  const Tableau &t = c.tab;
  s.dt = c.dt; s.Ma = c.Ma; s.Fr = c.Fr;
  if (stage == 1) {
    s.nst = 1; s.ca[0] = t.a21; s.ct[0] = t.a21t;
    s.ng = 2; s.cg[0] = t.a21t; s.cg[1] = t.a22t;
  } else if (stage == 2) {
    s.nst = 2; s.ca[0] = t.a31; s.ca[1] = t.a32; s.ct[0] = t.a31t; s.ct[1] = t.a32t;
    s.ng = 3; s.cg[0] = t.a31t; s.cg[1] = t.a32t; s.cg[2] = t.a33t;
  } else {
    s.nst = 3; s.ca[0] = t.b1; s.ca[1] = t.b2; s.ca[2] = t.b3;
    s.ct[0] = t.b1; s.ct[1] = t.b2; s.ct[2] = t.b3;
    s.ng = 3; s.cg[0] = t.b1; s.cg[1] = t.b2; s.cg[2] = t.b3;
  }
  (void)rho_only;
  return s;
}
double icoef3(const atm3_ctx &c) { return c.hstage == 1 ? c.tab.a22t : c.tab.a33t; }

// ---- operators (positional source lists as the 2D entry points) -------------
int rhs_rho3(atm3_ctx &c, double *dst, const double *const *src) {
  SrcPtrs sp{};
  const Coef3 co = coef3(c, c.hstage, true);
  for (int i = 0; i < 2 * co.nst; ++i) sp.p[i] = src[i];
  k3_rhs_rho<<<(c.nc + CELLS3 - 1) / CELLS3, 32 * CELLS3, 0, c.stream>>>(dst, sp, co, c.g);
  ATM_CHECK_LAUNCH("k3_rhs_rho");
  return ATM_OK;
}
// src: stage 1 {rho_old,u_old,p_old,rho_2}; 2 {.., u_2, p_2, rho_3};
// 3 {.., u_3, p_3}
int rhs_vel3(atm3_ctx &c, double *dst, const double *const *src) {
  const Coef3 co = coef3(c, c.hstage, false);
  SrcPtrs sp{}, gp{};
  for (int i = 0; i < 3 * co.nst; ++i) sp.p[i] = src[i];
  gp.p[0] = src[0];
  gp.p[1] = src[3];
  if (co.ng > 2) gp.p[2] = src[6];
  k3_rhs_vel<<<(c.nc + CELLS3 - 1) / CELLS3, 32 * CELLS3, 0, c.stream>>>(dst, sp, gp, co, c.g);
  ATM_CHECK_LAUNCH("k3_rhs_vel");
  return ATM_OK;
}
// src: stage 1 {rho_old,u_old,p_old,rho_2,u_fix}; 2 {.., u_2, p_2, rho_3,
// u_fix}; 3 {.., u_3, p_3, rho_cur, u_cur}
int rhs_pres3(atm3_ctx &c, double *dst, const double *const *src) {
  const Coef3 co = coef3(c, c.hstage, false);
  SrcPtrs sp{}, gp{};
  for (int i = 0; i < 3 * co.nst; ++i) sp.p[i] = src[i];
  if (c.hstage == 1) {
    const double *g[] = {src[0], src[1], src[3], src[4], src[3], src[4]};
    for (int i = 0; i < 6; ++i) gp.p[i] = g[i];
  } else if (c.hstage == 2) {
    const double *g[] = {src[0], src[1], src[3], src[4], src[6], src[7], src[6], src[7]};
    for (int i = 0; i < 8; ++i) gp.p[i] = g[i];
  } else {
    const double *g[] = {src[0], src[1], src[3], src[4], src[6], src[7], src[9], src[10]};
    for (int i = 0; i < 8; ++i) gp.p[i] = g[i];
  }
  k3_rhs_pres<<<(c.nc + CELLS3 - 1) / CELLS3, 32 * CELLS3, 0, c.stream>>>(dst, sp, gp, co, c.hstage, c.g);
  ATM_CHECK_LAUNCH("k3_rhs_pres");
  return ATM_OK;
}
int B3(atm3_ctx &c, double *dst, const double *p, double cB, int mode) {
  k3_B<<<(c.nc + CELLS3 - 1) / CELLS3, 32 * CELLS3, 0, c.stream>>>(dst, p, cB, c.ainv, mode, c.g);
  ATM_CHECK_LAUNCH("k3_B");
  return ATM_OK;
}
int CD3(atm3_ctx &c, double *dst, const double *w, const double *p, double cC, int mode) {
  k3_CD<<<(c.nc + CELLS3 - 1) / CELLS3, 32 * CELLS3, 0, c.stream>>>(dst, w, p, c.pres_fix, cC, c.invd,
                                                                      mode, c.g);
  ATM_CHECK_LAUNCH("k3_CD");
  return ATM_OK;
}
int block_apply3(atm3_ctx &c, double *dst, const double *src, const double *inv, int ncomp,
                 double scale) {
  k3_block_apply<<<blocks(c.nc), 128, 0, c.stream>>>(dst, src, inv, ncomp, scale, c.nc);
  ATM_CHECK_LAUNCH("k3_block_apply");
  return ATM_OK;
}
int rebuild_ainv3(atm3_ctx &c) {
  k3_block_inverse<<<blocks(c.nc), 128, 0, c.stream>>>(c.ainv, c.rho_fix, c.g);
  ATM_CHECK_LAUNCH("k3_block_inverse");
  return ATM_OK;
}
// S p = D p - C A^{-1} B p (with `precondition`: times diag(D)^{-1})
int schur3(atm3_ctx &c, double *dst, const double *p, bool precondition) {
  const double co = icoef3(c);
  TRY3(B3(c, c.wv1, p, co * c.dt / (c.Ma * c.Ma), 2));
  return CD3(c, dst, c.wv1, p, co * c.dt, precondition ? 2 : 1);
}
int vmult3(atm3_ctx &c, double *dst, const double *src) {
  switch (c.nsstage) {
    case 1:
    case 4: k3_mass<<<blocks(c.nc), 128, 0, c.stream>>>(dst, src, 1, nullptr, 1.0, c.g); break;
    case 2: return schur3(c, dst, src, false);
    case 3:
    case 5: k3_mass<<<blocks(c.nc), 128, 0, c.stream>>>(dst, src, 3, c.rho_fix, 1.0, c.g); break;
    case 6:
      k3_mass<<<blocks(c.nc), 128, 0, c.stream>>>(dst, src, 1, nullptr, 1.0 / (GAS_GAMMA - 1.0), c.g);
      break;
    default: set_error("NS stage out of range"); return ATM_BAD_ARG;
  }
  ATM_CHECK_LAUNCH("k3_mass");
  return ATM_OK;
}

// GMRES(28) + left Jacobi on diag(D), CGS2 (arnoldi_step), Givens; the
// algorithm of the 2D path's gmres_schur on the 3D operator
int gmres3(atm3_ctx &c, double *x, const double *b, double tol, int maxit, int *its, double *res) {
  const long n = c.ns();
  const int m = RESTART3;
  double *V = c.krylov, *w = c.ws1, *t = c.ws2;
  double *nsq = c.dsmall + 64, *ydev = c.dsmall + 96;
  std::vector<double> H((m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m), hcol(m + 1);
  *its = 0;
  *res = 0.0;
  for (;;) {
    TRY3(schur3(c, t, x, false));
    TRY3(vec_xmy_scaled(c.stream, V, c.invd, b, t, n));
    TRY3(vec_dot(c.stream, V, V, n, c.red, nsq));
    TRY3(read3(c, nsq, 1));
    const double beta = std::sqrt(c.h_red[0]);
    *res = beta;
    if (!std::isfinite(beta)) { set_error("GMRES: non-finite residual"); return ATM_NONFINITE; }
    if (beta <= tol) return ATM_OK;
    if (*its >= maxit) return ATM_NOT_CONVERGED;
    TRY3(vec_scale_by_inv_norm(c.stream, V, V, nsq, n));
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int jend = 0;
    bool done = false;
    for (int j = 0; j < m; ++j) {
      ++*its;
      TRY3(schur3(c, w, V + (long)j * n, true));
      double hn = 0.0;
      TRY3(arnoldi_step(c.stream, V, n, j, w, c.red, c.dsmall, c.h_red, hcol.data(), &hn));
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
      for (int k = l + 1; k < jend; ++k) s -= H[l * m + k] * y[k];
      y[l] = s / H[l * m + l];
    }
    ATM_CUDA(cudaMemcpyAsync(ydev, y.data(), jend * sizeof(double), cudaMemcpyHostToDevice,
                             c.stream));
    TRY3(vec_multiaxpy(c.stream, x, V, n, jend, ydev, 1.0, n));
    ATM_CUDA(cudaStreamSynchronize(c.stream));
    if (done && !c.true_check)
      return (*res <= tol) ? ATM_OK : (*its >= maxit ? ATM_NOT_CONVERGED : ATM_OK);
  }
}

// ---- the IMEX step (Atmospheric_Flow.cc:430-871, 1100-1257) ---------------
int update_density3(atm3_ctx &c) {
  if (c.hstage == 1) {
    const double *s[] = {c.rho_old, c.u_old};
    TRY3(rhs_rho3(c, c.rhs_rho, s));
    return block_apply3(c, c.rho_2, c.rhs_rho, c.minv, 1, 1.0);
  }
  if (c.hstage == 2) {
    const double *s[] = {c.rho_old, c.u_old, c.rho_2, c.u_2};
    TRY3(rhs_rho3(c, c.rhs_rho, s));
    return block_apply3(c, c.rho_3, c.rhs_rho, c.minv, 1, 1.0);
  }
  const double *s[] = {c.rho_old, c.u_old, c.rho_2, c.u_2, c.rho_3, c.u_3};
  TRY3(rhs_rho3(c, c.rhs_rho, s));
  return block_apply3(c, c.rho_cur, c.rhs_rho, c.minv, 1, 1.0);
}
int set_rho_fixed3(atm3_ctx &c, const double *rho) {
  TRY3(vec_copy(c.stream, c.rho_fix, rho, c.ns()));
  return rebuild_ainv3(c);
}
int pressure_fixed_point3(atm3_ctx &c) {
  const long ns = c.ns();
  TRY3(vec_copy(c.stream, c.pres_fix, c.p_fix_old, ns));
  if (c.hstage == 1) {
    const double *sp[] = {c.rho_old, c.u_old, c.p_old, c.rho_2, c.u_fixd};
    TRY3(rhs_pres3(c, c.rhs_p, sp));
    const double *su[] = {c.rho_old, c.u_old, c.p_old, c.rho_2};
    TRY3(rhs_vel3(c, c.rhs_u, su));
  } else {
    const double *sp[] = {c.rho_old, c.u_old, c.p_old, c.rho_2, c.u_2, c.p_2, c.rho_3, c.u_fixd};
    TRY3(rhs_pres3(c, c.rhs_p, sp));
    const double *su[] = {c.rho_old, c.u_old, c.p_old, c.rho_2, c.u_2, c.p_2, c.rho_3};
    TRY3(rhs_vel3(c, c.rhs_u, su));
  }
  TRY3(block_apply3(c, c.tmp_1, c.rhs_u, c.ainv, 3, 1.0));
  const double cc = icoef3(c);
  TRY3(CD3(c, c.rhs_p, c.tmp_1, nullptr, cc * c.dt, 3));
  // SolverControl(eps |rhs|) on the Jacobi-scaled residual
  // (Atmospheric_Flow.cc:656-672); with scaled_tol, eps |diag(D)^{-1} rhs|
  double nb2;
  if (c.scaled_tol) {
    TRY3(vec_fill(c.stream, c.ws1, 0.0, ns));
    TRY3(vec_xmy_scaled(c.stream, c.ws2, c.invd, c.rhs_p, c.ws1, ns));
    TRY3(vec_dot(c.stream, c.ws2, c.ws2, ns, c.red, c.red_out));
  } else {
    TRY3(vec_dot(c.stream, c.rhs_p, c.rhs_p, ns, c.red, c.red_out));
  }
  TRY3(read3(c, c.red_out, 1));
  nb2 = c.h_red[0];
  const double tol = c.eps * std::sqrt(nb2);
  TRY3(vec_copy(c.stream, c.p_fix, c.p_fix_old, ns));
  int its = 0;
  double res = 0.0;
  int rc = gmres3(c, c.p_fix, c.rhs_p, tol, c.max_its, &its, &res);
  c.krylov_total += its;
  if (rc == ATM_NOT_CONVERGED) {
    ++c.failures;
    char msg[200];
    std::snprintf(msg, sizeof msg, "shell: Schur solve did not converge in stage %d of step %ld "
                  "(%d iterations, residual %.3e > %.3e)", c.hstage, c.steps + 1, its, res, tol);
    set_error(msg);
  }
  return rc;
}
int update_velocity3(atm3_ctx &c) {
  if (c.hstage == 1 || c.hstage == 2) {
    TRY3(B3(c, c.rhs_u, c.p_fix, icoef3(c) * c.dt / (c.Ma * c.Ma), 1));
    return block_apply3(c, c.u_fixd, c.rhs_u, c.ainv, 3, 1.0);
  }
  const double *su[] = {c.rho_old, c.u_old, c.p_old, c.rho_2, c.u_2, c.p_2, c.rho_3, c.u_3, c.p_3};
  TRY3(rhs_vel3(c, c.rhs_u, su));
  return block_apply3(c, c.u_cur, c.rhs_u, c.ainv, 3, 1.0);
}
int update_pressure3(atm3_ctx &c) {
  const double *sp[] = {c.rho_old, c.u_old, c.p_old, c.rho_2, c.u_2, c.p_2, c.rho_3, c.u_3,
                        c.p_3, c.rho_cur, c.u_cur};
  TRY3(rhs_pres3(c, c.rhs_p, sp));
  return block_apply3(c, c.p_old, c.rhs_p, c.minv, 1, GAS_GAMMA - 1.0);
}
int picard3(atm3_ctx &c) {
  const long ns = c.ns();
  for (int it = 0; it < 100; ++it) {
    TRY3(pressure_fixed_point3(c));
    TRY3(update_velocity3(c));
    ++c.picard_total;
    TRY3(vec_maxdiff(c.stream, c.p_fix, c.p_fix_old, ns, c.red, c.red_out));
    TRY3(read3(c, c.red_out, 2));
    const double err = c.h_red[0] / (c.h_red[1] + 1e-10);
    if (!std::isfinite(err)) { set_error("shell: non-finite Picard update"); return ATM_NONFINITE; }
    if (err < 1e-10) break;
    TRY3(vec_copy(c.stream, c.p_fix_old, c.p_fix, ns));
  }
  return ATM_OK;
}
int step3(atm3_ctx &c) {
  const long ns = c.ns(), nv = c.nv();
  c.hstage = 1;
  TRY3(update_density3(c));
  TRY3(set_rho_fixed3(c, c.rho_2));
  TRY3(vec_copy(c.stream, c.p_fix_old, c.p_old, ns));
  TRY3(vec_copy(c.stream, c.u_fixd, c.u_old, nv));
  TRY3(picard3(c));
  TRY3(vec_copy(c.stream, c.p_2, c.p_fix, ns));
  TRY3(vec_copy(c.stream, c.u_2, c.u_fixd, nv));
  c.hstage = 2;
  TRY3(update_density3(c));
  TRY3(set_rho_fixed3(c, c.rho_3));
  TRY3(vec_copy(c.stream, c.p_fix_old, c.p_2, ns));
  TRY3(vec_copy(c.stream, c.u_fixd, c.u_2, nv));
  TRY3(picard3(c));
  TRY3(vec_copy(c.stream, c.p_3, c.p_fix, ns));
  TRY3(vec_copy(c.stream, c.u_3, c.u_fixd, nv));
  c.hstage = 3;
  TRY3(update_density3(c));
  TRY3(set_rho_fixed3(c, c.rho_cur));
  TRY3(update_velocity3(c));
  TRY3(update_pressure3(c));
  TRY3(vec_copy(c.stream, c.rho_old, c.rho_cur, ns));
  TRY3(vec_copy(c.stream, c.u_old, c.u_cur, nv));
  ++c.steps;
  return ATM_OK;
}

}  // namespace

// ============================================================================
// C ABI (declared in include/atm_gb300.h)
// ============================================================================
extern "C" {

int atm3_ctx_create(int n_cells, const double *nodes, int n_inner, const int *inner,
                    const int *face_perm, int n_bdry, const int *bdry, atm3_ctx **out) {
  if (!out || !nodes || n_cells < 1 || (n_inner > 0 && (!inner || !face_perm)) ||
      (n_bdry > 0 && !bdry)) {
    set_error("atm3_ctx_create: bad arguments");
    return ATM_BAD_ARG;
  }
  *out = nullptr;
  // tables: every cell face listed exactly once (inner faces from both sides)
  std::vector<int> nbr(6L * n_cells, -2), nbf(6L * n_cells, -1), nperm(54L * n_cells, 0);
  auto bad = [&](const std::string &m) { set_error("atm3_ctx_create: " + m); return ATM_BAD_ARG; };
  for (int f = 0; f < n_inner; ++f) {
    const int cp = inner[4 * f], fp = inner[4 * f + 1], cm = inner[4 * f + 2], fm = inner[4 * f + 3];
    if (cp < 0 || cp >= n_cells || cm < 0 || cm >= n_cells || fp < 0 || fp > 5 || fm < 0 || fm > 5)
      return bad("inner face " + std::to_string(f) + " out of range");
    if (nbr[6 * cp + fp] != -2 || nbr[6 * cm + fm] != -2)
      return bad("cell face listed twice (inner face " + std::to_string(f) + ")");
    nbr[6 * cp + fp] = cm; nbf[6 * cp + fp] = fm;
    nbr[6 * cm + fm] = cp; nbf[6 * cm + fm] = fp;
    int seen = 0;
    for (int q = 0; q < 9; ++q) {
      const int qm = face_perm[9 * f + q];
      if (qm < 0 || qm > 8 || (seen >> qm) & 1) return bad("face_perm of face " + std::to_string(f) + " is not a permutation");
      seen |= 1 << qm;
      nperm[(6 * cp + fp) * 9 + q] = qm;
      nperm[(6 * cm + fm) * 9 + qm] = q;
    }
  }
  for (int f = 0; f < n_bdry; ++f) {
    const int c = bdry[3 * f], lf = bdry[3 * f + 1];
    if (c < 0 || c >= n_cells || lf < 0 || lf > 5) return bad("boundary face out of range");
    if (nbr[6 * c + lf] != -2) return bad("cell face listed twice (boundary)");
    nbr[6 * c + lf] = -1;
  }
  for (int i = 0; i < 6 * n_cells; ++i)
    if (nbr[i] == -2) return bad("cell " + std::to_string(i / 6) + " face " + std::to_string(i % 6) + " is not listed");
  // geometry
  const double s = std::sqrt(0.6);
  const double gx[3] = {0.5 * (1.0 - s), 0.5, 0.5 * (1.0 + s)}, gw[3] = {5.0 / 18, 8.0 / 18, 5.0 / 18};
  std::vector<double> cg((size_t)n_cells * NQ * 13), fg((size_t)n_cells * 6 * NF * 4);
  for (int c = 0; c < n_cells; ++c) {
    const double *X = nodes + 81L * c;
    for (int q = 0; q < NQ; ++q) {
      const double xi[3] = {gx[q % 3], gx[(q / 3) % 3], gx[q / 9]};
      double x[3], J[3][3], Ji[3][3];
      map3(X, xi, x, J);
      const double det = inv3(J, Ji);
      if (!(det > 0.0)) return bad("non-positive Jacobian in cell " + std::to_string(c));
      const double jw = det * gw[q % 3] * gw[(q / 3) % 3] * gw[q / 9];
      double *o = &cg[((size_t)c * NQ + q) * 13];
      for (int e = 0; e < 3; ++e)
        for (int i = 0; i < 3; ++i) o[3 * e + i] = Ji[e][i] * jw;
      o[9] = jw;
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      for (int i = 0; i < 3; ++i) o[10 + i] = x[i] / r * EARTH_A * EARTH_A / (r * r);
    }
    for (int f = 0; f < 6; ++f)
      for (int q = 0; q < NF; ++q) {
        const int d = f / 2, t0 = d == 0 ? 1 : 0, t1 = d == 2 ? 1 : 2;
        double xi[3];
        xi[d] = (double)(f % 2);
        xi[t0] = gx[q % 3];
        xi[t1] = gx[q / 3];
        double x[3], J[3][3], Ji[3][3];
        map3(X, xi, x, J);
        const double det = inv3(J, Ji);
        double len = 0.0;
        for (int i = 0; i < 3; ++i) len += Ji[d][i] * Ji[d][i];
        len = std::sqrt(len);
        const double sg = (f % 2) ? 1.0 : -1.0;
        double *o = &fg[(((size_t)c * 6 + f) * NF + q) * 4];
        for (int i = 0; i < 3; ++i) o[i] = sg * Ji[d][i] / len;
        o[3] = det * len * gw[q % 3] * gw[q / 3];
      }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("atm3_ctx_create: no CUDA device (there is no CPU path)");
    return ATM_CUDA_ERROR;
  }
  atm3_ctx *c = new atm3_ctx();
  auto fail = [&](int rc) { free3(c); return rc; };
  cudaGetDevice(&c->device);
  c->nc = n_cells;
  c->tab = Tableau::make();
  int rc = upload_tables3();
  if (rc) return fail(rc);
  if ((rc = alloc3(*c, &c->cg, cg.size())) || (rc = alloc3(*c, &c->fg, fg.size()))) return fail(rc);
  if (cudaMalloc(&c->nbr, nbr.size() * sizeof(int)) || cudaMalloc(&c->nbf, nbf.size() * sizeof(int)) ||
      cudaMalloc(&c->nperm, nperm.size() * sizeof(int)))
    return fail(cuda_fail(cudaErrorMemoryAllocation, "cudaMalloc shell tables"));
  cudaMemcpy(c->cg, cg.data(), cg.size() * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(c->fg, fg.data(), fg.size() * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(c->nbr, nbr.data(), nbr.size() * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(c->nbf, nbf.data(), nbf.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (cudaMemcpy(c->nperm, nperm.data(), nperm.size() * sizeof(int), cudaMemcpyHostToDevice))
    return fail(cuda_fail(cudaGetLastError(), "upload shell tables"));
  c->g = Geo3{n_cells, c->cg, c->fg, c->nbr, c->nbf, c->nperm};
  const long ns = c->ns(), nv = c->nv();
  double **sv[] = {&c->rho_fix, &c->pres_fix, &c->invd, &c->ws1, &c->ws2};
  for (double **p : sv)
    if ((rc = alloc3(*c, p, ns))) return fail(rc);
  if ((rc = alloc3(*c, &c->u_fix, nv)) || (rc = alloc3(*c, &c->wv1, nv)) ||
      (rc = alloc3(*c, &c->minv, (size_t)n_cells * 64)) ||
      (rc = alloc3(*c, &c->ainv, (size_t)n_cells * 64)) ||
      (rc = alloc3(*c, &c->red, 32 * RED_BLOCKS)) || (rc = alloc3(*c, &c->red_out, 64)) ||
      (rc = alloc3(*c, &c->dsmall, 256)) ||
      (rc = alloc3(*c, &c->krylov, (size_t)(RESTART3 + 1) * ns)))
    return fail(rc);
  if (cudaMallocHost(&c->h_red, 256 * sizeof(double)) != cudaSuccess)
    return fail(cuda_fail(cudaErrorMemoryAllocation, "cudaMallocHost"));
  k3_block_inverse<<<blocks(n_cells), 128, 0, c->stream>>>(c->minv, nullptr, c->g);
  k3_invdiag_D<<<blocks(n_cells), 128, 0, c->stream>>>(c->invd, c->g);
  g_kernel_launches.fetch_add(2);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess)
    return fail(cuda_fail(cudaGetLastError(), "shell set-up kernels"));
  *out = c;
  return ATM_OK;
}

int atm3_ctx_destroy(atm3_ctx *h) {
  free3(h);
  return ATM_OK;
}

int atm3_set_params(atm3_ctx *h, double dt, double mach, double froude) {
  if (!h || !(dt > 0) || !(mach > 0) || !(froude > 0)) {
    set_error("atm3_set_params: null handle or non-positive value");
    return ATM_BAD_ARG;
  }
  h->dt = dt; h->Ma = mach; h->Fr = froude;
  return ATM_OK;
}

int atm3_set_stage(atm3_ctx *h, int hyperbolic_stage, int ns_stage) {
  if (!h || hyperbolic_stage < 1 || hyperbolic_stage > 3 || ns_stage < 1 || ns_stage > 6) {
    set_error("atm3_set_stage: null handle or stage out of range");
    return ATM_BAD_ARG;
  }
  h->hstage = hyperbolic_stage;
  h->nsstage = ns_stage;
  return ATM_OK;
}

int atm3_set_frozen(atm3_ctx *h, const double *rho, const double *pres, const double *u) {
  if (!h) { set_error("null handle"); return ATM_BAD_ARG; }
  if (rho) {
    ATM_CUDA(cudaMemcpyAsync(h->rho_fix, rho, h->ns() * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    int rc = rebuild_ainv3(*h);
    if (rc) return rc;
  }
  if (pres) ATM_CUDA(cudaMemcpyAsync(h->pres_fix, pres, h->ns() * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  if (u) ATM_CUDA(cudaMemcpyAsync(h->u_fix, u, h->nv() * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  return ATM_OK;
}

int atm3_rhs(atm3_ctx *h, int which, double *dst, const double *const *src, int nsrc) {
  if (!h || !dst || !src || which < 0 || which > 2) {
    set_error("atm3_rhs: bad arguments");
    return ATM_BAD_ARG;
  }
  static const int need[3][3] = {{2, 4, 6}, {4, 7, 9}, {5, 8, 11}};
  if (nsrc != need[which][h->hstage - 1]) {
    set_error("atm3_rhs: wrong number of sources for this equation and IMEX stage");
    return ATM_BAD_ARG;
  }
  for (int i = 0; i < nsrc; ++i)
    if (!src[i]) { set_error("atm3_rhs: null source"); return ATM_BAD_ARG; }
  int rc = which == 0 ? rhs_rho3(*h, dst, src) : which == 1 ? rhs_vel3(*h, dst, src)
                                                          : rhs_pres3(*h, dst, src);
  if (rc) return rc;
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  return ATM_OK;
}

int atm3_apply(atm3_ctx *h, int which, double *dst, const double *src) {
  if (!h || !dst || !src || which < 0 || which > 2) {
    set_error("atm3_apply: bad arguments");
    return ATM_BAD_ARG;
  }
  int rc;
  if (which == 0) rc = B3(*h, dst, src, icoef3(*h) * h->dt / (h->Ma * h->Ma), 0);
  else if (which == 1) rc = CD3(*h, dst, src, nullptr, icoef3(*h) * h->dt, 0);
  else rc = vmult3(*h, dst, src);
  if (rc) return rc;
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  return ATM_OK;
}

int atm3_solver_init(atm3_ctx *h, double eps, int max_its, int scaled_tol, int true_residual_check) {
  if (!h || !(eps > 0.0) || max_its < 1) {
    set_error("atm3_solver_init: null handle, eps <= 0 or max_its < 1");
    return ATM_BAD_ARG;
  }
  if (!h->pool) {
    const long ns = h->ns(), nv = h->nv();
    int rc = alloc3(*h, &h->pool, 11 * ns + 7 * nv);
    if (rc) return rc;
    double *p = h->pool;
    auto take = [&](long n) { double *r = p; p += n; return r; };
    h->rho_old = take(ns); h->rho_2 = take(ns); h->rho_3 = take(ns); h->rho_cur = take(ns);
    h->rhs_rho = take(ns); h->p_old = take(ns); h->p_2 = take(ns); h->p_3 = take(ns);
    h->p_fix = take(ns); h->p_fix_old = take(ns); h->rhs_p = take(ns);
    h->u_old = take(nv); h->u_2 = take(nv); h->u_3 = take(nv); h->u_cur = take(nv);
    h->u_fixd = take(nv); h->rhs_u = take(nv); h->tmp_1 = take(nv);
  }
  h->solver = true;
  h->eps = eps;
  h->max_its = max_its;
  h->scaled_tol = scaled_tol != 0;
  h->true_check = true_residual_check != 0;
  h->steps = h->picard_total = h->krylov_total = h->failures = 0;
  return ATM_OK;
}

int atm3_solver_set_state(atm3_ctx *h, const double *rho, const double *u, const double *p) {
  if (!h || !h->solver || !rho || !u || !p) {
    set_error("atm3_solver_set_state: solver not initialised or null pointer");
    return ATM_BAD_ARG;
  }
  ATM_CUDA(cudaMemcpy(h->rho_old, rho, h->ns() * sizeof(double), cudaMemcpyHostToDevice));
  ATM_CUDA(cudaMemcpy(h->u_old, u, h->nv() * sizeof(double), cudaMemcpyHostToDevice));
  ATM_CUDA(cudaMemcpy(h->p_old, p, h->ns() * sizeof(double), cudaMemcpyHostToDevice));
  return ATM_OK;
}

int atm3_solver_get_state(atm3_ctx *h, double *rho, double *u, double *p) {
  if (!h || !h->solver || !rho || !u || !p) {
    set_error("atm3_solver_get_state: solver not initialised or null pointer");
    return ATM_BAD_ARG;
  }
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  ATM_CUDA(cudaMemcpy(rho, h->rho_old, h->ns() * sizeof(double), cudaMemcpyDeviceToHost));
  ATM_CUDA(cudaMemcpy(u, h->u_old, h->nv() * sizeof(double), cudaMemcpyDeviceToHost));
  ATM_CUDA(cudaMemcpy(p, h->p_old, h->ns() * sizeof(double), cudaMemcpyDeviceToHost));
  return ATM_OK;
}

int atm3_solver_run(atm3_ctx *h, int n_steps) {
  if (!h || !h->solver || n_steps < 0) {
    set_error("atm3_solver_run: solver not initialised or n_steps < 0");
    return ATM_BAD_ARG;
  }
  for (int i = 0; i < n_steps; ++i) {
    int rc = step3(*h);
    if (rc) return rc;
  }
  ATM_CUDA(cudaStreamSynchronize(h->stream));
  return ATM_OK;
}

int atm3_solver_stats(atm3_ctx *h, double *out) {
  if (!h || !out) { set_error("null handle or pointer"); return ATM_BAD_ARG; }
  out[0] = (double)h->steps;
  out[1] = (double)h->picard_total;
  out[2] = (double)h->krylov_total;
  out[3] = (double)h->failures;
  return ATM_OK;
}

}  // extern "C"
