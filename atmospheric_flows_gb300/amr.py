"""Adaptive refinement of the flow-over-hill mesh: a 2:1-balanced quadtree
over the terrain-following base mesh, the leaf mesh tables with hanging
faces, the refinement indicator and the solution transfer.

This is the host side of adaptive meshes, the part the reference leaves to
deal.II/p4est (``parallel::distributed::Triangulation``, the
``refine_global`` call at Atmospheric_Flow.cc:283 and deal.II's
``SolutionTransfer``).  The device side is the hanging-face variant of every
face kernel, which the C ABI selects from the inner-face table
(``atm_ctx_create``: the last entry of an inner face is 0 for a conforming
face and 1 + s when the first cell is the fine side of subface s of the
second cell's face).

Geometry.  A leaf at level l is a 2^-l x 2^-l square of its base cell's
reference square, and its degree-m mapping is the base cell's mapping
restricted to that square (a Q_m polynomial restricted to a sub-square is
again Q_m).  So a fine face coincides exactly with its coarse neighbour's
subface and refinement adds no new terrain information.

Transfer.  Refinement interpolates the parent polynomial into the children
(exact).  Coarsening is the physical L2 projection of the four children onto
the parent, with the Gauss rule of the operators, so the discrete integrals
(mass, energy content) are conserved in both directions.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .hill import (CP, GAMMA, MACH, P0, R_GAS, RHO_REF, HillCase, HillParams, background,
                   build_case, build_mesh, gll_points, lagrange_matrix)

_OPP = (1, 0, 3, 2)


def lagrange_deriv_matrix(nodes: np.ndarray, x: np.ndarray) -> np.ndarray:
    """L'[p, i] = l_i'(x_p) for the Lagrange basis on ``nodes``."""
    n = len(nodes)
    out = np.zeros((len(x), n))
    for i in range(n):
        for j in range(n):
            if j == i:
                continue
            term = np.full(len(x), 1.0 / (nodes[i] - nodes[j]))
            for m in range(n):
                if m != i and m != j:
                    term = term * (x - nodes[m]) / (nodes[i] - nodes[m])
            out[:, i] += term
    return out


def gauss_rule(n: int):
    """Gauss-Legendre points and weights on [0, 1]."""
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


class QuadTree:
    """2:1-balanced refinement of an nx x nz base mesh (x periodic or not).

    A node is (level, ix, iz) in the level's index space (nx 2^l x nz 2^l).
    ``refined`` holds the nodes that are split; every other node reachable
    from a base cell is a leaf.  Leaves are numbered base cell by base cell
    (z-major, as the uniform mesh) and, inside a base cell, depth first with
    the children in the order (x-,z-), (x+,z-), (x-,z+), (x+,z+).  With no
    refinement the numbering is the uniform mesh's."""

    def __init__(self, nx: int, nz: int, periodic: bool = True, max_level: int = 2):
        self.nx, self.nz, self.periodic, self.max_level = nx, nz, periodic, max_level
        self.refined: set[tuple[int, int, int]] = set()
        self._leaves = None

    # ------------------------------------------------------------- leaves --
    def leaves(self) -> list[tuple[int, int, int]]:
        if self._leaves is None:
            out = []

            def walk(node):
                if node in self.refined:
                    l, ix, iz = node
                    for b in range(2):
                        for a in range(2):
                            walk((l + 1, 2 * ix + a, 2 * iz + b))
                else:
                    out.append(node)

            for iz in range(self.nz):
                for ix in range(self.nx):
                    walk((0, ix, iz))
            self._leaves = out
        return self._leaves

    def leaf_index(self) -> dict:
        return {n: i for i, n in enumerate(self.leaves())}

    def _invalidate(self):
        self._leaves = None

    def is_leaf(self, node) -> bool:
        l, ix, iz = node
        if node in self.refined:
            return False
        if l == 0:
            return True
        return (l - 1, ix >> 1, iz >> 1) in self.refined

    # --------------------------------------------------------- neighbours --
    def neighbour_pos(self, node, f):
        """Same-level position across face f, or None at a boundary."""
        l, ix, iz = node
        nxl, nzl = self.nx << l, self.nz << l
        if f == 0:
            ix -= 1
        elif f == 1:
            ix += 1
        elif f == 2:
            iz -= 1
        else:
            iz += 1
        if iz < 0 or iz >= nzl:
            return None
        if ix < 0 or ix >= nxl:
            if not self.periodic:
                return None
            ix %= nxl
        return (l, ix, iz)

    def _deepest_along(self, node, side) -> int:
        """Finest leaf level inside `node` touching its face `side`."""
        if node not in self.refined:
            return node[0]
        l, ix, iz = node
        if side in (0, 1):
            a = 0 if side == 0 else 1
            kids = [(l + 1, 2 * ix + a, 2 * iz + b) for b in range(2)]
        else:
            b = 0 if side == 2 else 1
            kids = [(l + 1, 2 * ix + a, 2 * iz + b) for a in range(2)]
        return max(self._deepest_along(k, side) for k in kids)

    # ------------------------------------------------------------ editing --
    def refine(self, nodes):
        for n in nodes:
            if n[0] < self.max_level and self.is_leaf(n):
                self.refined.add(n)
        self._invalidate()

    def coarsen(self, parents):
        """Merge the four children of each parent whose children are all leaves."""
        for p in parents:
            if p in self.refined:
                l, ix, iz = p
                kids = [(l + 1, 2 * ix + a, 2 * iz + b) for b in range(2) for a in range(2)]
                if all(k not in self.refined for k in kids):
                    self.refined.discard(p)
        self._invalidate()

    def balance(self) -> int:
        """Refine leaves until face neighbours differ by at most one level."""
        added = 0
        while True:
            todo = []
            for leaf in self.leaves():
                for f in range(4):
                    n = self.neighbour_pos(leaf, f)
                    if n is not None and self._deepest_along(n, _OPP[f]) > leaf[0] + 1:
                        todo.append(leaf)
                        break
            if not todo:
                return added
            self.refine(todo)
            added += len(todo)

    def is_balanced(self) -> bool:
        for leaf in self.leaves():
            for f in range(4):
                n = self.neighbour_pos(leaf, f)
                if n is not None and self._deepest_along(n, _OPP[f]) > leaf[0] + 1:
                    return False
        return True

    # --------------------------------------------------------- face tables --
    def face_tables(self):
        """Inner faces [n][5] (c+, f+, c-, f-, o) and boundary faces [n][3].

        Conforming faces are listed once from their x+/z+ side; a hanging face
        is listed from each fine cell with o = 1 + subface."""
        idx = self.leaf_index()
        inner, bdry = [], []
        for i, leaf in enumerate(self.leaves()):
            l, ix, iz = leaf
            for f in range(4):
                n = self.neighbour_pos(leaf, f)
                if n is None:
                    bdry.append((i, f, {0: 2, 1: 3, 2: 0, 3: 1}[f]))
                    continue
                if n in idx:
                    if f in (1, 3):
                        inner.append((i, f, idx[n], _OPP[f], 0))
                    continue
                parent = (l - 1, n[1] >> 1, n[2] >> 1)
                if l > 0 and parent in idx:
                    s = (iz & 1) if f in (0, 1) else (ix & 1)
                    inner.append((i, f, idx[parent], _OPP[f], 1 + s))
                # otherwise the neighbour is refined: its fine cells list the face
        return (np.asarray(inner, dtype=np.int32).reshape(-1, 5),
                np.asarray(bdry, dtype=np.int32).reshape(-1, 3))


# ------------------------------------------------------------------ geometry --
def leaf_mapping_nodes(tree: QuadTree, base_nodes: np.ndarray, m: int) -> np.ndarray:
    """Mapping nodes of every leaf: its base cell's mapping at the leaf's
    sub-square GLL points.  Returns [n_leaves, (m+1)^2, 2]."""
    ref = gll_points(m)
    leaves = np.asarray(tree.leaves(), dtype=np.int64).reshape(-1, 3)
    out = np.empty((len(leaves), (m + 1) ** 2, 2))
    base = base_nodes.reshape(base_nodes.shape[0], m + 1, m + 1, 2)
    l, ix, iz = leaves[:, 0], leaves[:, 1], leaves[:, 2]
    bx, bz = ix >> l, iz >> l
    ox, oz = ix - (bx << l), iz - (bz << l)
    cell = bz * tree.nx + bx
    key = (l * 64 + ox) * 64 + oz
    for kv in np.unique(key):
        sel = np.nonzero(key == kv)[0]
        lv, a, b = int(l[sel[0]]), int(ox[sel[0]]), int(oz[sel[0]])
        h = 1.0 / (1 << lv)
        La = lagrange_matrix(ref, a * h + h * ref)
        Lb = lagrange_matrix(ref, b * h + h * ref)
        out[sel] = np.einsum("zb,xa,cbad->czxd", Lb, La, base[cell[sel]]).reshape(len(sel), -1, 2)
    return out


def jacobians(nodes: np.ndarray, m: int, pts: np.ndarray):
    """Jacobian entries at a tensor grid of reference points for every cell:
    (dx/dxi, dx/deta, dz/dxi, dz/deta), each [nc, len(pts)^2] (x fastest)."""
    ref = gll_points(m)
    L = lagrange_matrix(ref, pts)
    dL = lagrange_deriv_matrix(ref, pts)
    X = nodes.reshape(nodes.shape[0], m + 1, m + 1, 2)  # [c, b, a, d]
    dxi = np.einsum("zb,xa,cbad->czxd", L, dL, X).reshape(nodes.shape[0], -1, 2)
    deta = np.einsum("zb,xa,cbad->czxd", dL, L, X).reshape(nodes.shape[0], -1, 2)
    return dxi[..., 0], deta[..., 0], dxi[..., 1], deta[..., 1]


# ---------------------------------------------------------- solution transfer --
def _prolong_1d(k: int):
    x = gll_points(k)
    return [lagrange_matrix(x, 0.5 * (x + s)) for s in range(2)]


def prolong_cell(u: np.ndarray, k: int) -> list[np.ndarray]:
    """Nodal values [.., (k+1)^2] of a parent -> its four children (a + 2b)."""
    P = _prolong_1d(k)
    nn = k + 1
    U = u.reshape(u.shape[:-1] + (nn, nn))
    out = []
    for b in range(2):
        for a in range(2):
            out.append(np.einsum("zj,xi,...ji->...zx", P[b], P[a], U).reshape(u.shape))
    return out


def _restrict_cell(children, child_nodes, parent_nodes, k, m):
    """Physical L2 projection of four children (fields [..., nn2]) onto the parent."""
    nq = 2 * k + 1
    g, w = gauss_rule(nq)
    x = gll_points(k)
    S = lagrange_matrix(x, g)              # [q, i]
    W2 = np.outer(w, w).reshape(-1)
    # parent mass matrix with |J|
    a, b, c_, d = jacobians(parent_nodes[None], m, g)
    detp = (a * d - b * c_)[0]
    Phi = np.einsum("zj,xi->zxji", S, S).reshape(nq * nq, -1)  # [q, node]
    M = Phi.T @ (Phi * (W2 * detp)[:, None])
    rhs = 0.0
    P = [lagrange_matrix(x, 0.5 * (g + s)) for s in range(2)]  # parent basis at child pts
    for cb in range(2):
        for ca in range(2):
            ch = children[ca + 2 * cb]
            a, b, c_, d = jacobians(child_nodes[ca + 2 * cb][None], m, g)
            detc = (a * d - b * c_)[0]
            Phic = np.einsum("zj,xi->zxji", P[cb], P[ca]).reshape(nq * nq, -1)
            vals = ch.reshape(ch.shape[:-1] + (-1,)) @ Phi.T  # child at its Gauss points
            rhs = rhs + (vals * (W2 * detc)) @ Phic
    return np.linalg.solve(M, rhs.T).T


def transfer_state(old: QuadTree, new: QuadTree, base_nodes, fields, k, m):
    """Move nodal fields ([n_old_leaves, ncomp, nn2] each) from `old` leaves
    to `new` leaves.  Leaves present in both are copied; leaves below an old
    leaf are interpolated from it (one matrix per depth and position, applied
    to all such leaves at once); leaves above old leaves are L2 projections of
    their children (recursively)."""
    oidx = old.leaf_index()
    nn = k + 1
    nn2 = nn * nn
    new_leaves = new.leaves()
    out = [np.empty((len(new_leaves),) + f.shape[1:]) for f in fields]
    P1 = _prolong_1d(k)
    groups = {}  # (depth, ox, oz) -> (new positions, old leaf indices)
    coarser = []
    for j, node in enumerate(new_leaves):
        if node in oidx:
            groups.setdefault((0, 0, 0), ([], []))
            g = groups[(0, 0, 0)]
            g[0].append(j)
            g[1].append(oidx[node])
            continue
        l, ix, iz = node
        found = None
        for d in range(1, l + 1):
            anc = (l - d, ix >> d, iz >> d)
            if anc in oidx:
                found = (d, ix - (anc[1] << d), iz - (anc[2] << d), oidx[anc])
                break
        if found is None:
            coarser.append((j, node))
            continue
        d, ox, oz, oi = found
        g = groups.setdefault((d, ox, oz), ([], []))
        g[0].append(j)
        g[1].append(oi)
    for (d, ox, oz), (js, ois) in groups.items():
        Px, Pz = np.eye(nn), np.eye(nn)
        for t in range(d):  # from the ancestor down: bit d-1-t of the offset
            Px = P1[(ox >> (d - 1 - t)) & 1] @ Px
            Pz = P1[(oz >> (d - 1 - t)) & 1] @ Pz
        js, ois = np.asarray(js), np.asarray(ois)
        for f, arr in enumerate(fields):
            U = arr[ois].reshape(len(ois), -1, nn, nn)
            out[f][js] = np.einsum("zj,xi,cnji->cnzx", Pz, Px, U).reshape(len(ois), -1, nn2)

    geo = {}

    def node_geometry(node):
        if node not in geo:
            t = QuadTree(old.nx, old.nz, old.periodic, old.max_level)
            t._leaves = [node]
            geo[node] = leaf_mapping_nodes(t, base_nodes, m)[0]
        return geo[node]

    def value_of(node, f):
        if node in oidx:
            return fields[f][oidx[node]]
        l, ix, iz = node
        kids = [(l + 1, 2 * ix + a, 2 * iz + b) for b in range(2) for a in range(2)]
        vals = [value_of(kn, f) for kn in kids]
        return _restrict_cell(vals, [node_geometry(kn) for kn in kids], node_geometry(node), k, m)

    for j, node in coarser:
        for f in range(len(fields)):
            out[f][j] = value_of(node, f)
    return out


# ------------------------------------------------------------------ indicator --
def theta_perturbation_gradient(p: HillParams, nodes, rho, pres) -> np.ndarray:
    """max over the nodes of |grad theta'| per cell (K/m), theta' = theta -
    theta_background(z); rho, pres nondimensional nodal fields [nc, nn2]."""
    k, m = p.degree, p.mapping_degree
    x = gll_points(k)
    nn = k + 1
    xz = np.einsum("zb,xa,cbad->czxd", lagrange_matrix(gll_points(m), x),
                   lagrange_matrix(gll_points(m), x),
                   nodes.reshape(nodes.shape[0], m + 1, m + 1, 2)).reshape(nodes.shape[0], -1, 2)
    pd = pres * P0
    rd = rho * RHO_REF
    T = pd / (R_GAS * rd)
    theta = T * (P0 / pd) ** (R_GAS / CP)
    theta_bg = background(p, xz[..., 1])[0]
    tp = (theta - theta_bg).reshape(-1, nn, nn)
    Dm = lagrange_deriv_matrix(x, x)
    dxi = np.einsum("xi,czi->czx", Dm, tp).reshape(tp.shape[0], -1)
    deta = np.einsum("zj,cjx->czx", Dm, tp).reshape(tp.shape[0], -1)
    a, b, c_, d = jacobians(nodes, m, x)
    det = a * d - b * c_
    gx = (d * dxi - c_ * deta) / det
    gz = (-b * dxi + a * deta) / det
    return np.max(np.sqrt(gx * gx + gz * gz), axis=1)


# ----------------------------------------------------------------- the member --
@dataclasses.dataclass
class AdaptParams:
    max_level: int = 2
    refine_fraction: float = 0.10   # refine leaves above this top fraction
    coarsen_fraction: float = 0.50  # coarsen parents whose children are all below
    every: int = 50                 # steps between re-adaptations


def coarser_tree(tree: QuadTree) -> QuadTree | None:
    """The tree with its finest cells merged into their parents, or None when
    nothing is refined.  All children of a deepest refined node are leaves,
    and merging every deepest group keeps the 2:1 balance."""
    if not tree.refined:
        return None
    top = max(n[0] for n in tree.refined)
    out = QuadTree(tree.nx, tree.nz, tree.periodic, tree.max_level)
    out.refined = {n for n in tree.refined if n[0] < top}
    return out


def mg_hierarchy_adaptive(p: HillParams, tree: QuadTree, max_levels: int = 8) -> list:
    """Coarse levels of the multigrid Schur preconditioner on an adaptive mesh
    (fine to coarse, the leaf mesh itself excluded).

    Each level merges the finest 2x2 groups of the level above and keeps
    every other cell, so levels may have hanging faces; once the base mesh is
    reached the uniform 2x2 coarsening of ``hill.mg_hierarchy`` continues.
    ``children[n_cells][4]`` lists the merged cells at positions (x-,z-),
    (x+,z-), (x-,z+), (x+,z+), or (cell, -1, -1, -1) for a cell that stays.
    A merged cell's mapping is its base cell's mapping on the union of the
    four sub-squares, so the children are exact sub-squares of the parent
    and the prolongation is the exact polynomial embedding."""
    from .hill import mg_hierarchy

    base_nodes = build_mesh(p)[0]
    levels = []
    cur = tree
    while len(levels) + 1 < max_levels:
        nxt = coarser_tree(cur)
        if nxt is None:
            break
        cidx = cur.leaf_index()
        ch = []
        for node in nxt.leaves():
            if node in cidx:
                ch.append((cidx[node], -1, -1, -1))
            else:
                l, ix, iz = node
                ch.append(tuple(cidx[(l + 1, 2 * ix + a, 2 * iz + b)]
                                for b in range(2) for a in range(2)))
        inner, bdry = nxt.face_tables()
        levels.append(dict(n_cells=len(ch),
                           mapping_nodes=np.ascontiguousarray(
                               leaf_mapping_nodes(nxt, base_nodes, p.mapping_degree)),
                           inner_faces=inner, boundary_faces=bdry,
                           children=np.asarray(ch, dtype=np.int32).reshape(-1, 4)))
        cur = nxt
    if not cur.refined and len(levels) + 1 < max_levels:
        # the uniform base mesh numbers its cells as the unrefined tree does
        levels.extend(mg_hierarchy(p, max_levels=max_levels - len(levels)))
    return levels


def adaptive_case(p: HillParams, tree: QuadTree, state=None, dt=None) -> HillCase:
    """HillCase on the leaves of `tree`; `state` = (rho, u, p) on those leaves
    or None for the initial condition interpolated from the base mesh."""
    base_nodes, _, _ = build_mesh(p)
    k, m = p.degree, p.mapping_degree
    nodes = leaf_mapping_nodes(tree, base_nodes, m)
    inner, bdry = tree.face_tables()
    nc = nodes.shape[0]
    nn2 = (k + 1) ** 2
    from .hill import map_points, min_cell_diameter

    xz = map_points(nodes, m, gll_points(k))
    if state is None:
        uni = build_case(dataclasses.replace(p))
        flat = QuadTree(p.nx, p.nz, p.periodic, tree.max_level)
        fields = [uni.rho.reshape(-1, 1, nn2), uni.u.reshape(-1, 2, nn2), uni.p.reshape(-1, 1, nn2)]
        fields = transfer_state(flat, tree, base_nodes, fields, k, m)
        rho, u, pres = (f.reshape(-1) for f in fields)
    else:
        rho, u, pres = state
    z = xz[..., 1]
    alpha = np.zeros((nc, nn2))
    mask = z > p.sponge_start
    span = max(p.height - p.sponge_start, 1e-30)
    alpha[mask] = p.sponge_rate * np.sin(0.5 * np.pi * (z[mask] - p.sponge_start) / span) ** 2
    if dt is None:
        cmax = float(np.max(np.sqrt(GAMMA * pres / rho)))
        hmin = min_cell_diameter(nodes, m)
        dt = p.cfl * hmin / ((1.0 / MACH) * cmax * k * math.sqrt(2.0))
    return HillCase(params=p, n_cells=nc, mapping_nodes=np.ascontiguousarray(nodes),
                    inner_faces=inner, boundary_faces=bdry, node_xz=xz,
                    rho=np.ascontiguousarray(rho), u=np.ascontiguousarray(u),
                    p=np.ascontiguousarray(pres), sponge_alpha=alpha.reshape(-1), dt=dt,
                    tree=tree)


def mark(tree: QuadTree, indicator: np.ndarray, ap: AdaptParams):
    """Refine the top `refine_fraction` leaves by indicator and coarsen the
    parents whose four children are leaves below the `coarsen_fraction`
    quantile; then restore the 2:1 balance."""
    leaves = tree.leaves()
    hi = np.quantile(indicator, 1.0 - ap.refine_fraction)
    lo = np.quantile(indicator, ap.coarsen_fraction)
    ref = [leaves[i] for i in np.nonzero(indicator > hi)[0]]
    low = {leaves[i] for i in np.nonzero(indicator < lo)[0]}
    parents = set()
    for (l, ix, iz) in low:
        if l > 0:
            par = (l - 1, ix >> 1, iz >> 1)
            kids = [(l, 2 * par[1] + a, 2 * par[2] + b) for b in range(2) for a in range(2)]
            if all(kk in low for kk in kids):
                parents.add(par)
    new = QuadTree(tree.nx, tree.nz, tree.periodic, tree.max_level)
    new.refined = set(tree.refined)
    new.coarsen(parents)
    new.refine(ref)
    new.balance()
    return new


class AdaptiveMember:
    """One flow-over-hill member on an adaptive mesh: runs the device solver
    and re-adapts every ``ap.every`` steps (indicator |grad theta'|, refine
    the top 10%, up to ``ap.max_level`` levels), moving the state on the host
    between meshes.  dt is fixed from the finest admissible level."""

    def __init__(self, p: HillParams, ap: AdaptParams | None = None, eps=1e-8, precision=0,
                 initial_adaptations=None, stream=None):
        from .euler_solver import EulerSolver

        self.p, self.ap = p, ap or AdaptParams()
        self.eps, self.precision, self.stream = eps, precision, stream
        self._Solver = EulerSolver
        self.base_nodes = build_mesh(p)[0]
        self.tree = QuadTree(p.nx, p.nz, p.periodic, self.ap.max_level)
        uni = build_case(p)
        self.dt = uni.dt / (1 << self.ap.max_level)
        self.case = adaptive_case(p, self.tree, dt=self.dt)
        for _ in range(self.ap.max_level if initial_adaptations is None else initial_adaptations):
            self._adapt_state(self.case.rho, self.case.u, self.case.p)
        self.solver = self._make_solver()
        self.steps = 0
        self.adaptations = 0
        self.time = 0.0

    def _make_solver(self):
        if self.precision == 0:
            return self._Solver(self.case, eps=self.eps, precision=0, dt=self.dt,
                                stream=self.stream)
        # multigrid Schur solve: the hierarchy of this leaf mesh, rebuilt
        # after every adaptation; stop on the true residual (S is nonlinear)
        return self._Solver(self.case, eps=self.eps, precision=self.precision, dt=self.dt,
                            stream=self.stream, true_residual_check=True,
                            levels=mg_hierarchy_adaptive(self.p, self.tree, max_levels=3))

    def _adapt_state(self, rho, u, pres):
        k, m = self.p.degree, self.p.mapping_degree
        nn2 = (k + 1) ** 2
        ind = theta_perturbation_gradient(self.p, self.case.mapping_nodes,
                                          rho.reshape(-1, nn2), pres.reshape(-1, nn2))
        new = mark(self.tree, ind, self.ap)
        fields = [rho.reshape(-1, 1, nn2), u.reshape(-1, 2, nn2), pres.reshape(-1, 1, nn2)]
        fields = transfer_state(self.tree, new, self.base_nodes, fields, k, m)
        self.tree = new
        self.case = adaptive_case(self.p, new, state=tuple(f.reshape(-1) for f in fields),
                                  dt=self.dt)

    def adapt(self):
        rho, u, pres = self.solver.get_state()
        st = self.solver.stats()
        self.solver.close()
        self._adapt_state(rho, u, pres)
        self.solver = self._make_solver()
        _clock(self.solver, st["time"], int(st["steps"]))
        self.adaptations += 1

    def run(self, n_steps: int):
        left = n_steps
        while left > 0:
            n = min(left, self.ap.every - self.steps % self.ap.every)
            self.solver.run(n)
            self.steps += n
            left -= n
            if self.steps % self.ap.every == 0 and left > 0:
                self.adapt()

    @property
    def n_dofs(self) -> int:
        return self.case.n_dofs

    def close(self):
        self.solver.close()


def _clock(solver, time, steps):
    from . import _lib

    _lib.call("atm_solver_set_clock", solver.op.handle, float(time), int(steps))


def example_tree(nx: int, nz: int, periodic: bool = True, max_level: int = 2) -> QuadTree:
    """A fixed 2-level refinement that exercises every hanging-face situation:
    a refined cell on the periodic seam and at the bottom wall, one at the
    top wall, a second level inside the first, and the 2:1 closure around
    them."""
    t = QuadTree(nx, nz, periodic, max_level)
    t.refine([(0, 0, 0), (0, nx - 1, min(1, nz - 1)), (0, nx // 2, nz - 1)])
    if max_level >= 2:
        t.refine([(1, 1, 1), (1, 2 * nx - 1, 0)])
    t.balance()
    return t
