"""Flow-over-hill case: mesh tables, mapping nodes, background state.

This is host-side set-up, the part the reference leaves to deal.II
(``create_triangulation``/``setup_dofs``/``initialize``,
Atmospheric_Flow.cc:279-423).  It produces the plain arrays that the C-ABI
consumes (``atm_ctx_create``): per-cell mapping nodes, the inner-face and
boundary-face tables, and nodal initial data.

Geometry: a terrain-following mesh of ``nx x nz`` quadrilaterals over
``x in [x0, x1]``, ``z in [h(x), H]`` with the Witch-of-Agnesi hill
``h(x) = h0 / (1 + (x/a)^2)`` and ``z = h(x) + s (H - h(x))``.  Each cell is
described by the Gauss-Lobatto points of a degree-``m`` Lagrange mapping
(``m = 2`` mirrors ``MappingQ(2)``, equation_data.h:43), evaluated on the exact
geometry.  x is periodic by default; the bottom (id 0) and top (id 1) are
no-flux walls as in the reference (euler_operator.h:111-114,2189-2305).

Non-dimensionalisation follows the reference: u_ref = L_ref = 1,
p_ref = p0, rho_ref = p_ref/(R T_ref); Ma = 1/sqrt(R T_ref), Fr = 1/sqrt(g)
(parameter-file.prm:7-8, equation_data.h:24-38).  With T_ref = 273 K these are
the values of the reference parameter file.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# physical constants, equation_data.h:23-33
GAMMA = 1.4
R_GAS = 287.0
G_GRAV = 9.80616
P0 = 100000.0
T_REF = 273.0
CP = GAMMA * R_GAS / (GAMMA - 1.0)
MACH = 1.0 / math.sqrt(R_GAS * T_REF)
FROUDE = 1.0 / math.sqrt(G_GRAV)
RHO_REF = P0 / (R_GAS * T_REF)


def gll_points(k: int) -> np.ndarray:
    """Gauss-Lobatto points of degree k on [0, 1], ascending."""
    if k == 0:
        return np.array([0.5])
    if k == 1:
        return np.array([0.0, 1.0])
    # interior points: roots of P_k' -> eigenvalues of the Jacobi(1,1) matrix
    n = k - 1
    j = np.arange(1, n)
    off = np.sqrt(j * (j + 2) / ((2 * j + 1) * (2 * j + 3)))
    mat = np.diag(off, 1) + np.diag(off, -1)
    inner = np.sort(np.linalg.eigvalsh(mat)) if n > 0 else np.array([])
    return np.concatenate([[0.0], 0.5 * (inner + 1.0), [1.0]])


def lagrange_matrix(nodes: np.ndarray, x: np.ndarray) -> np.ndarray:
    """L[p, i] = l_i(x_p) for the Lagrange basis on ``nodes``."""
    n = len(nodes)
    out = np.ones((len(x), n))
    for i in range(n):
        for j in range(n):
            if j != i:
                out[:, i] *= (x - nodes[j]) / (nodes[i] - nodes[j])
    return out


@dataclasses.dataclass
class HillParams:
    nx: int = 40
    nz: int = 20
    degree: int = 4
    x0: float = -20000.0
    x1: float = 20000.0
    height: float = 20000.0
    h0: float = 400.0
    a: float = 1000.0
    brunt: float = 0.01
    theta0: float = 300.0
    u0: float = 10.0
    sponge_start: float = 12000.0
    sponge_rate: float = 0.05
    cfl: float = 5.0
    periodic: bool = True
    mapping_degree: int = 2
    theta_noise: float = 0.0
    seed: int = 0


@dataclasses.dataclass
class HillCase:
    params: HillParams
    n_cells: int
    mapping_nodes: np.ndarray  # [nc, (m+1)^2, 2]
    inner_faces: np.ndarray  # [nf, 5] int32: c+, f+, c-, f-, orientation
    boundary_faces: np.ndarray  # [nb, 3] int32: c, f, boundary id
    node_xz: np.ndarray  # [nc, (k+1)^2, 2] physical DG node positions
    rho: np.ndarray  # [nc*(k+1)^2]
    u: np.ndarray  # [nc*2*(k+1)^2]
    p: np.ndarray  # [nc*(k+1)^2]
    sponge_alpha: np.ndarray  # [nc*(k+1)^2] relaxation rate per node (1/s)
    dt: float
    Ma: float = MACH
    Fr: float = FROUDE
    tree: object = None  # amr.QuadTree of an adaptive case (None: uniform mesh)

    @property
    def degree(self) -> int:
        return self.params.degree

    @property
    def n_dofs(self) -> int:
        """DoFs = 4 scalar unknowns (rho, u_x, u_z, p) per DG node."""
        return 4 * self.n_cells * (self.params.degree + 1) ** 2


def terrain(p: HillParams, x: np.ndarray) -> np.ndarray:
    return p.h0 / (1.0 + (x / p.a) ** 2)


def background(p: HillParams, z: np.ndarray):
    """Constant-N background: theta, Exner, p, rho (dimensional)."""
    n2 = p.brunt ** 2
    theta = p.theta0 * np.exp(n2 * z / G_GRAV)
    exner = 1.0 + G_GRAV ** 2 / (CP * p.theta0 * n2) * (np.exp(-n2 * z / G_GRAV) - 1.0)
    pres = P0 * exner ** (CP / R_GAS)
    rho = pres / (R_GAS * theta * exner)
    return theta, exner, pres, rho


def build_mesh(p: HillParams):
    """Mapping nodes and face tables for the terrain-following mesh."""
    nx, nz, m = p.nx, p.nz, p.mapping_degree
    ref = gll_points(m)
    dx = (p.x1 - p.x0) / nx
    nc = nx * nz
    nodes = np.empty((nc, (m + 1) ** 2, 2))
    for iz in range(nz):
        for ix in range(nx):
            c = iz * nx + ix
            for b in range(m + 1):
                for a_ in range(m + 1):
                    x = p.x0 + (ix + ref[a_]) * dx
                    s = (iz + ref[b]) / nz
                    h = terrain(p, np.array(x))
                    nodes[c, b * (m + 1) + a_, 0] = x
                    nodes[c, b * (m + 1) + a_, 1] = float(h + s * (p.height - h))
    inner = []
    bdry = []
    for iz in range(nz):
        for ix in range(nx):
            c = iz * nx + ix
            # x-faces: this cell's face 1 against the right neighbour's face 0
            if ix + 1 < nx:
                inner.append((c, 1, c + 1, 0, 0))
            elif p.periodic:
                inner.append((c, 1, iz * nx, 0, 0))
            else:
                bdry.append((c, 1, 3))
            if ix == 0 and not p.periodic:
                bdry.append((c, 0, 2))
            # z-faces
            if iz + 1 < nz:
                inner.append((c, 3, c + nx, 2, 0))
            else:
                bdry.append((c, 3, 1))
            if iz == 0:
                bdry.append((c, 2, 0))
    return (nodes, np.asarray(inner, dtype=np.int32).reshape(-1, 5),
            np.asarray(bdry, dtype=np.int32).reshape(-1, 3))


def map_points(nodes: np.ndarray, m: int, ref_pts: np.ndarray) -> np.ndarray:
    """Physical positions of a tensor grid of reference points, per cell.

    Returns [nc, len(ref)^2, 2] with the x index fastest."""
    L = lagrange_matrix(gll_points(m), ref_pts)  # [n, m+1]
    nodes_r = nodes.reshape(nodes.shape[0], m + 1, m + 1, 2)  # [c, b, a, d]
    out = np.einsum("zb,xa,cbad->czxd", L, L, nodes_r)
    return out.reshape(nodes.shape[0], -1, 2)


def min_cell_diameter(nodes: np.ndarray, m: int) -> float:
    """Smallest cell diameter (longest corner-to-corner distance per cell)."""
    c = nodes.reshape(nodes.shape[0], m + 1, m + 1, 2)
    v00, v10, v01, v11 = c[:, 0, 0], c[:, 0, m], c[:, m, 0], c[:, m, m]
    d1 = np.linalg.norm(v11 - v00, axis=1)
    d2 = np.linalg.norm(v10 - v01, axis=1)
    return float(np.min(np.maximum(d1, d2)))


def build_case(p: HillParams | None = None, **kw) -> HillCase:
    p = p or HillParams(**kw)
    nodes, inner, bdry = build_mesh(p)
    k = p.degree
    nc = p.nx * p.nz
    nn2 = (k + 1) ** 2
    xz = map_points(nodes, p.mapping_degree, gll_points(k))
    z = xz[..., 1]
    theta, exner, pres, rho = background(p, z)
    if p.theta_noise > 0.0:
        rng = np.random.default_rng(p.seed)
        theta = theta + p.theta_noise * rng.standard_normal(theta.shape)
        rho = pres / (R_GAS * theta * exner)
    rho_nd = (rho / RHO_REF).reshape(-1)
    p_nd = (pres / P0).reshape(-1)
    u = np.zeros((nc, 2, nn2))
    u[:, 0, :] = p.u0
    alpha = np.zeros((nc, nn2))
    mask = z > p.sponge_start
    span = max(p.height - p.sponge_start, 1e-30)
    alpha[mask] = p.sponge_rate * np.sin(0.5 * np.pi * (z[mask] - p.sponge_start) / span) ** 2
    # acoustic CFL with the reference formula (Atmospheric_Flow.cc:1227-1228)
    cmax = float(np.max(np.sqrt(GAMMA * p_nd / rho_nd)))
    hmin = min_cell_diameter(nodes, p.mapping_degree)
    dt = p.cfl * hmin / ((1.0 / MACH) * cmax * k * math.sqrt(2.0))
    return HillCase(params=p, n_cells=nc, mapping_nodes=np.ascontiguousarray(nodes),
                    inner_faces=inner, boundary_faces=bdry,
                    node_xz=xz, rho=np.ascontiguousarray(rho_nd),
                    u=np.ascontiguousarray(u.reshape(-1)),
                    p=np.ascontiguousarray(p_nd), sponge_alpha=alpha.reshape(-1),
                    dt=dt)


def mg_hierarchy(p: HillParams, max_levels: int = 8, min_cells_z: int = 1):
    """Coarse levels for the FP32 multigrid preconditioner.

    Returns a list of dicts (fine to coarse, level 1 first) with the mesh
    tables of the (nx/2^l) x (nz/2^l) mesh and ``children[n_cells][4]``: the
    level l-1 cells at positions (x-,z-), (x+,z-), (x-,z+), (x+,z+)."""
    levels = []
    nx, nz = p.nx, p.nz
    while (len(levels) + 1 < max_levels and nx % 2 == 0 and nz % 2 == 0
           and nz // 2 >= min_cells_z and nx // 2 >= 1):
        nxc, nzc = nx // 2, nz // 2
        pc = dataclasses.replace(p, nx=nxc, nz=nzc)
        nodes, inner, bdry = build_mesh(pc)
        ch = np.empty((nxc * nzc, 4), dtype=np.int32)
        for iz in range(nzc):
            for ix in range(nxc):
                c = iz * nxc + ix
                for b in range(2):
                    for a in range(2):
                        ch[c, a + 2 * b] = (2 * iz + b) * nx + 2 * ix + a
        levels.append(dict(n_cells=nxc * nzc, mapping_nodes=np.ascontiguousarray(nodes),
                           inner_faces=inner, boundary_faces=bdry, children=ch,
                           nx=nxc, nz=nzc))
        nx, nz = nxc, nzc
    return levels
