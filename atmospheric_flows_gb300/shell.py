"""The reference's own test case in 3D: steady solid-body rotation on a
spherical shell, the known answer it checks every step (analyze_results,
Atmospheric_Flow.cc:925-985; exact fields equation_data.h:57-176).

Host-side set-up, as hill.py is for the flow over a hill:
  * mesh: a cubed-sphere shell between 0.9 a and a (a = Earth radius, L_ref =
    1), six patches of n x n columns of nr cells.  The reference builds
    concentric_hyper_shells(0.9, 1.0) and refines it globally
    (Atmospheric_Flow.cc:283-286); n = 16, nr = 4 gives its 6144 cells.  Each
    cell's degree-2 mapping nodes lie on the exact sphere (MappingQ(2),
    equation_data.h:43);
  * faces: inner faces carry the permutation between the two sides' face
    quadrature points (neighbouring patches meet with rotated or flipped face
    parameterisations); the inner and outer spheres are walls;
  * fields: FE_DGQ(1) nodal values (the reference's degree 1,
    equation_data.h:19-21) of the exact rho, u, p, non-dimensionalised as the
    reference does (p_ref = p0, rho_ref = p_ref/(R T_bar), u_ref = L_ref = 1).

Gravity is radial, -e_r a^2/r^2 / Fr^2 (euler_operator.h:790-811, evaluated
at each quadrature point).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .hill import GAMMA, G_GRAV, P0, R_GAS, gll_points, lagrange_matrix

EARTH_A = 6.37122e6          # equation_data.h:26
T_BAR = 273.0                # isothermal temperature, equation_data.h:28
OMEGA_SBR = 2.0 * math.pi / 86400.0  # solid-body rotation rate, equation_data.h:32
RHO_REF = P0 / (R_GAS * T_BAR)
MACH = 0.00357254516         # parameter-file.prm:7
FROUDE = 0.31933793491       # parameter-file.prm:8

# gauss points of the 3-point rule on [0, 1] (2k+1 = 3 for k = 1)
_G3 = 0.5 * (np.polynomial.legendre.leggauss(3)[0] + 1.0)


@dataclasses.dataclass
class ShellParams:
    n: int = 4          # cells along a patch edge
    nr: int = 2         # radial layers
    r_in: float = 0.9 * EARTH_A
    r_out: float = 1.0 * EARTH_A
    dt: float = 8.64    # parameter-file.prm:12
    degree: int = 1
    mapping_degree: int = 2
    # every `rotate_every`-th cell has its reference axes turned by 90 degrees
    # about xi3 (0: none), so that neighbours meet with permuted face points
    rotate_every: int = 0


@dataclasses.dataclass
class ShellCase:
    params: ShellParams
    n_cells: int
    mapping_nodes: np.ndarray   # [nc, 27, 3]
    inner_faces: np.ndarray     # [nf, 4] int32: c+, f+, c-, f-
    face_perm: np.ndarray       # [nf, 9] int32: point q of (c+, f+) is point perm[q] of (c-, f-)
    boundary_faces: np.ndarray  # [nb, 3] int32: cell, face, id (0 inner, 1 outer)
    node_xyz: np.ndarray        # [nc, 8, 3]
    rho: np.ndarray             # [nc*8]
    u: np.ndarray               # [nc*3*8]
    p: np.ndarray               # [nc*8]
    dt: float
    Ma: float = MACH
    Fr: float = FROUDE

    @property
    def n_dofs(self) -> int:
        return 5 * self.n_cells * 8


# ------------------------------------------------------------ exact state --
def exact_fields(xyz: np.ndarray):
    """rho / rho_ref, u (3 components), p / p_ref of the steady solid-body
    rotation at points xyz [..., 3] (equation_data.h:57-176)."""
    x, y, z = xyz[..., 0], xyz[..., 1], xyz[..., 2]
    r = np.sqrt(x * x + y * y + z * z)
    lat = np.arcsin(z / r)
    lon = np.arctan2(y, x)
    s = r * np.cos(lat)  # distance from the polar axis
    q = (0.5 * OMEGA_SBR ** 2 * s * s - EARTH_A * G_GRAV * (1.0 - EARTH_A / r)) / (R_GAS * T_BAR)
    rho = (P0 / (R_GAS * T_BAR) / RHO_REF) * np.exp(q)
    p = np.exp(q)  # p0 / p_ref = 1
    U = r * OMEGA_SBR * np.cos(lat)
    u = np.stack([-U * np.sin(lon), U * np.cos(lon), np.zeros_like(U)], axis=-1)
    return rho, u, p


# ------------------------------------------------------------------- mesh --
# cube face: (outward axis, sign), and the axes of the two patch coordinates
_PATCHES = [(0, 1.0, 1, 2), (0, -1.0, 2, 1), (1, 1.0, 2, 0),
            (1, -1.0, 0, 2), (2, 1.0, 0, 1), (2, -1.0, 1, 0)]


def _patch_point(pi: int, al, be, r):
    """Physical point of patch pi at equiangular coordinates (al, be) in
    [-pi/4, pi/4] and radius r (broadcasting)."""
    ax, sg, a1, a2 = _PATCHES[pi]
    al, be, r = np.broadcast_arrays(np.asarray(al, float), np.asarray(be, float),
                                    np.asarray(r, float))
    v = np.zeros(al.shape + (3,))
    v[..., ax] = sg
    v[..., a1] = np.tan(al)
    v[..., a2] = np.tan(be)
    return v / np.linalg.norm(v, axis=-1, keepdims=True) * r[..., None]


def _cell_map(pi, i, j, k, n, nr, r_in, r_out):
    """x(xi) of one cell: reference [0,1]^3 -> physical (exact geometry)."""
    h = 0.5 * math.pi / n
    dr = (r_out - r_in) / nr

    def f(x1, x2, x3):
        return _patch_point(pi, -0.25 * math.pi + (i + np.asarray(x1)) * h,
                            -0.25 * math.pi + (j + np.asarray(x2)) * h,
                            r_in + (k + np.asarray(x3)) * dr)
    return f


def _tensor_points(pts):
    """[len^3, 3] reference points, first coordinate fastest."""
    m = len(pts)
    out = np.empty((m ** 3, 3))
    for c in range(m):
        for b in range(m):
            for a in range(m):
                out[(c * m + b) * m + a] = (pts[a], pts[b], pts[c])
    return out


def map_q2(nodes27: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """Evaluate the degree-2 mappings [nc, 27, 3] at reference points [np, 3]."""
    g = gll_points(2)
    L = [lagrange_matrix(g, ref[:, d]) for d in range(3)]  # [np, 3] each
    B = np.einsum("pa,pb,pc->pcba", L[0], L[1], L[2]).reshape(len(ref), 27)
    return np.einsum("pn,cnd->cpd", B, nodes27)


def _face_ref_points(f: int) -> np.ndarray:
    """The 9 Gauss points of local face f (0/1: xi1 = 0/1, 2/3: xi2, 4/5: xi3)
    in reference coordinates, the lower tangential index fastest."""
    d, side = f // 2, float(f % 2)
    t = [e for e in range(3) if e != d]
    out = np.empty((9, 3))
    for b in range(3):
        for a in range(3):
            p = np.zeros(3)
            p[d] = side
            p[t[0]] = _G3[a]
            p[t[1]] = _G3[b]
            out[b * 3 + a] = p
    return out


def build_shell(p: ShellParams | None = None, **kw) -> ShellCase:
    p = p or ShellParams(**kw)
    if p.degree != 1 or p.mapping_degree != 2:
        raise ValueError("the shell path is FE_DGQ(1) with a degree-2 mapping, as the reference")
    n, nr = p.n, p.nr
    ref27 = _tensor_points(gll_points(2))
    corners = _tensor_points(np.array([0.0, 1.0]))
    cells = []
    for pi in range(6):
        for k in range(nr):
            for j in range(n):
                for i in range(n):
                    f = _cell_map(pi, i, j, k, n, nr, p.r_in, p.r_out)
                    # right-handed reference axes: reverse xi1 where needed
                    x = f(ref27[:, 0], ref27[:, 1], ref27[:, 2])
                    c = f(0.5, 0.5, 0.5)
                    e = 1e-3
                    J = np.stack([(f(0.5 + e, 0.5, 0.5) - c), (f(0.5, 0.5 + e, 0.5) - c),
                                  (f(0.5, 0.5, 0.5 + e) - c)], axis=1)
                    if np.linalg.det(J) < 0:
                        x = f(1.0 - ref27[:, 0], ref27[:, 1], ref27[:, 2])
                    if p.rotate_every and len(cells) % p.rotate_every == 0:
                        # (xi1, xi2) -> (xi2, 1 - xi1): still right-handed
                        g = x.reshape(3, 3, 3, 3)  # [c][b][a][d]
                        rot = np.empty_like(g)
                        for ic in range(3):
                            for ib in range(3):
                                for ia in range(3):
                                    rot[ic, ib, ia] = g[ic, 2 - ia, ib]
                        x = rot.reshape(27, 3)
                    cells.append(x)
    nodes = np.ascontiguousarray(np.array(cells))
    nc = len(nodes)
    # faces by their four corners
    fref = [_face_ref_points(f) for f in range(6)]
    key_of = {}
    face_pts = {}
    bdry, inner, perm = [], [], []
    cx = map_q2(nodes, corners)  # [nc, 8, 3]
    for c in range(nc):
        for f in range(6):
            d, side = f // 2, f % 2
            sel = [v for v in range(8) if ((v >> d) & 1) == side]
            key = tuple(sorted(tuple(np.round(cx[c, v] / 10.0).astype(np.int64)) for v in sel))
            if key in key_of:
                cp, fp = key_of.pop(key)
                inner.append((cp, fp, c, f))
            else:
                key_of[key] = (c, f)
    for (c, f) in key_of.values():
        r = np.linalg.norm(cx[c, [v for v in range(8) if ((v >> 2) & 1) == f % 2]], axis=1)
        if f // 2 != 2:
            raise RuntimeError("unmatched lateral face")
        bdry.append((c, f, 0 if np.allclose(r, p.r_in, rtol=1e-9) else 1))
    for (cp, fp, cm, fm) in inner:
        xp = map_q2(nodes[cp:cp + 1], fref[fp])[0]
        xm = map_q2(nodes[cm:cm + 1], fref[fm])[0]
        dist = np.linalg.norm(xp[:, None, :] - xm[None, :, :], axis=2)
        pm = np.argmin(dist, axis=1)
        if sorted(pm.tolist()) != list(range(9)) or np.max(np.min(dist, axis=1)) > 1e-3:
            raise RuntimeError("face quadrature points do not match")
        perm.append(pm)
    node_xyz = map_q2(nodes, corners)  # FE_DGQ(1) nodes = cell vertices, xi1 fastest
    rho, u, pres = exact_fields(node_xyz)
    return ShellCase(params=p, n_cells=nc, mapping_nodes=nodes,
                     inner_faces=np.asarray(inner, dtype=np.int32).reshape(-1, 4),
                     face_perm=np.asarray(perm, dtype=np.int32).reshape(-1, 9),
                     boundary_faces=np.asarray(bdry, dtype=np.int32).reshape(-1, 3),
                     node_xyz=node_xyz, rho=np.ascontiguousarray(rho.reshape(-1)),
                     u=np.ascontiguousarray(np.transpose(u, (0, 2, 1)).reshape(-1)),
                     p=np.ascontiguousarray(pres.reshape(-1)), dt=p.dt)


def exact_l2_errors(case: ShellCase, quad_values) -> dict:
    """Relative L2 errors of fields given at the Gauss points of every cell
    (dict name -> [nc, 27] or [nc, 27, 3]) against the exact state, with the
    cells' JxW from the degree-2 mapping (analyze_results,
    Atmospheric_Flow.cc:925-985)."""
    ref = _tensor_points(_G3)
    w1 = 0.5 * np.polynomial.legendre.leggauss(3)[1]
    W = np.einsum("a,b,c->cba", w1, w1, w1).reshape(-1)
    xq = map_q2(case.mapping_nodes, ref)
    e = 1e-6
    J = np.stack([(map_q2(case.mapping_nodes, ref + e * np.eye(3)[d]) -
                   map_q2(case.mapping_nodes, ref - e * np.eye(3)[d])) / (2 * e)
                  for d in range(3)], axis=-1)
    jxw = np.abs(np.linalg.det(J)) * W
    rho, u, p = exact_fields(xq)
    exact = {"rho": rho, "u": u, "p": p}
    out = {}
    for name, v in quad_values.items():
        diff = (v - exact[name]) ** 2
        ref_ = exact[name] ** 2
        if diff.ndim == 3:
            diff, ref_ = diff.sum(-1), ref_.sum(-1)
        out[name] = float(np.sqrt(np.sum(diff * jxw) / np.sum(ref_ * jxw)))
    return out


def nodal_to_quad(case: ShellCase, field: np.ndarray, ncomp: int = 1) -> np.ndarray:
    """Values of an FE_DGQ(1) field at the 27 Gauss points of every cell."""
    ref = _tensor_points(_G3)
    x = np.array([0.0, 1.0])
    L = [lagrange_matrix(x, ref[:, d]) for d in range(3)]
    B = np.einsum("pa,pb,pc->pcba", L[0], L[1], L[2]).reshape(27, 8)
    f = field.reshape(case.n_cells, ncomp, 8)
    v = np.einsum("pn,ckn->cpk", B, f)
    return v[..., 0] if ncomp == 1 else v


def acoustic_cfl(case: ShellCase) -> float:
    """CFL_c of the reference's printout (Atmospheric_Flow.cc:1227-1228) for
    the case's dt and initial state."""
    c = np.sqrt(GAMMA * case.p / case.rho)
    corners = case.node_xyz
    d = np.max(np.linalg.norm(corners[:, [7, 6, 5, 4]] - corners[:, [0, 1, 2, 3]], axis=2), axis=1)
    return case.dt * float(np.max(c)) / case.Ma * case.params.degree * math.sqrt(3) / float(np.min(d))


# ------------------------------------------------------------- device path --
class ShellSolver:
    """The 3D shell case on the GB300 (atm3_* entry points): the operators
    of EULEROperator<3> and the EulerSolver<3> time loop for FE_DGQ(1).

    `scaled_tol`: the reference's Schur stop compares the Jacobi-scaled
    residual with eps |rhs|; on this mesh diag(D)^{-1} ~ 1/|cell| ~ 1e-15 and
    that rule ends GMRES before its first iteration (as it does in the
    reference), so the default compares with eps |diag(D)^{-1} rhs|."""

    def __init__(self, case: ShellCase, eps=1e-8, max_its=30000, scaled_tol=True,
                 true_residual_check=False):
        import ctypes

        from . import _lib

        self._lib = _lib
        self.case = case
        self._keep = [np.ascontiguousarray(case.mapping_nodes, dtype=np.float64),
                      np.ascontiguousarray(case.inner_faces, dtype=np.int32),
                      np.ascontiguousarray(case.face_perm, dtype=np.int32),
                      np.ascontiguousarray(case.boundary_faces, dtype=np.int32)]
        nodes, inner, perm, bdry = self._keep
        dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        h = ctypes.c_void_p()
        _lib.call("atm3_ctx_create", case.n_cells, nodes.ctypes.data_as(dp), len(inner),
                  inner.ctypes.data_as(ip), perm.ctypes.data_as(ip), len(bdry),
                  bdry.ctypes.data_as(ip), ctypes.byref(h))
        self.h = h
        self.ns = case.n_cells * 8
        _lib.call("atm3_set_params", h, case.dt, case.Ma, case.Fr)
        _lib.call("atm3_solver_init", h, float(eps), int(max_its), int(bool(scaled_tol)),
                  int(bool(true_residual_check)))
        self.set_state(case.rho, case.u, case.p)

    def _dp(self, a):
        import ctypes

        assert a.dtype == np.float64 and a.flags.c_contiguous
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    def set_state(self, rho, u, p):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (rho, u, p)]
        self._lib.call("atm3_solver_set_state", self.h, *[self._dp(a) for a in arrs])

    def get_state(self):
        r, u, p = np.empty(self.ns), np.empty(3 * self.ns), np.empty(self.ns)
        self._lib.call("atm3_solver_get_state", self.h, self._dp(r), self._dp(u), self._dp(p))
        return r, u, p

    def run(self, n):
        self._lib.call("atm3_solver_run", self.h, int(n))

    def stats(self):
        out = np.zeros(4)
        self._lib.call("atm3_solver_stats", self.h, self._dp(out))
        return dict(zip(("steps", "picard_total", "krylov_total", "solve_fail"), out.tolist()))

    # ---- single operators on device tensors (torch) ----
    def set_stage(self, hyperbolic_stage, ns_stage):
        self._lib.call("atm3_set_stage", self.h, int(hyperbolic_stage), int(ns_stage))

    def set_frozen(self, rho=None, pres=None, u=None):
        import ctypes

        ptr = (lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None)
        self._lib.call("atm3_set_frozen", self.h, ptr(rho), ptr(pres), ptr(u))

    def rhs(self, which, dst, src):
        import ctypes

        arr = (ctypes.c_void_p * len(src))(*[t.data_ptr() for t in src])
        self._lib.call("atm3_rhs", self.h, int(which), ctypes.c_void_p(dst.data_ptr()), arr,
                       len(src))

    def apply(self, which, dst, src):
        import ctypes

        self._lib.call("atm3_apply", self.h, int(which), ctypes.c_void_p(dst.data_ptr()),
                       ctypes.c_void_p(src.data_ptr()))

    def close(self):
        if getattr(self, "h", None) is not None:
            self._lib.call("atm3_ctx_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
