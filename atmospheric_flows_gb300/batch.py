"""Batched members: several flow-over-hill members concatenated into one
device context, so every kernel launch covers the cells of all of them.

Members of one batch share the polynomial degree and the mapping degree;
their meshes, terrain, background, perturbations and time steps may differ.
Their cells are concatenated with disjoint connectivity, so every operator is
block diagonal over the members and one launch advances them all: the
"concatenated cell list" of the serving design.  The library runs the
solvers member-wise (atm_set_members): each member keeps its own dt, and
its inner products, Krylov stops and Picard stops are its own, so a member's
fields match its solo run -- with GMRES + Jacobi to the Krylov round-off,
with FGMRES + multigrid to the Schur tolerance (the V-cycle's Chebyshev
interval is estimated over the batch, so the preconditioner differs).  A
member that fails is frozen and reported without stopping the others.

The multigrid hierarchy is each member's hierarchy concatenated level by
level; a member whose hierarchy is shallower keeps its coarsest level on the
deeper levels (children rows (cell, -1, -1, -1)).  The sponge relaxes each
member toward its own background wind (atm_solver_set_sponge_target).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .hill import HillCase, mg_hierarchy


@dataclasses.dataclass
class Batch:
    case: HillCase            # the concatenated member set
    offsets: list             # first cell of each member, then the total
    levels: list              # concatenated multigrid levels (fine to coarse)
    u_target: np.ndarray      # per-node sponge target velocity [cells][2][node]
    dts: list                 # each member's own time step

    @property
    def members(self) -> int:
        return len(self.offsets) - 1

    def split(self, field: np.ndarray, ncomp: int = 1) -> list:
        """Per-member views of a concatenated nodal field."""
        per = ncomp * (self.case.degree + 1) ** 2
        o = self.offsets
        return [field[o[i] * per:o[i + 1] * per] for i in range(self.members)]

    def split_state(self, state) -> list:
        rho, u, p = state
        return list(zip(self.split(rho), self.split(u, 2), self.split(p)))


def batch_key(params) -> tuple:
    """Members can share a batch when these agree."""
    return (params.degree, params.mapping_degree)


def _offset_faces(inner, bdry, off):
    inner = inner.copy()
    inner[:, 0] += off
    inner[:, 2] += off
    bdry = bdry.copy()
    bdry[:, 0] += off
    return inner, bdry


def concat(cases, mg_levels: int = 3) -> Batch:
    """Concatenate members (same batch_key; any mesh sizes) into one case."""
    if not cases:
        raise ValueError("empty batch")
    key = batch_key(cases[0].params)
    if any(batch_key(c.params) != key for c in cases):
        raise ValueError("batched members need the same degree and mapping degree")
    if any(getattr(c, "tree", None) is not None for c in cases):
        raise ValueError("batched members need uniform meshes")
    nn2 = (cases[0].degree + 1) ** 2
    offsets = [0]
    for c in cases:
        offsets.append(offsets[-1] + c.n_cells)
    inner, bdry = [], []
    for i, c in enumerate(cases):
        a, b = _offset_faces(c.inner_faces, c.boundary_faces, offsets[i])
        inner.append(a)
        bdry.append(b)
    u_target = np.zeros((offsets[-1], 2, nn2))
    for i, c in enumerate(cases):
        u_target[offsets[i]:offsets[i + 1], 0, :] = c.params.u0
    case = dataclasses.replace(
        cases[0], n_cells=offsets[-1],
        mapping_nodes=np.ascontiguousarray(np.concatenate([c.mapping_nodes for c in cases])),
        inner_faces=np.ascontiguousarray(np.concatenate(inner)),
        boundary_faces=np.ascontiguousarray(np.concatenate(bdry)),
        node_xz=np.concatenate([c.node_xz for c in cases]),
        rho=np.ascontiguousarray(np.concatenate([c.rho for c in cases])),
        u=np.ascontiguousarray(np.concatenate([c.u for c in cases])),
        p=np.ascontiguousarray(np.concatenate([c.p for c in cases])),
        sponge_alpha=np.ascontiguousarray(np.concatenate([c.sponge_alpha for c in cases])),
        dt=cases[0].dt)
    per = [mg_hierarchy(c.params, max_levels=mg_levels) for c in cases]
    # each member's current level: (cells, mapping nodes, inner, boundary)
    cur = [(c.n_cells, c.mapping_nodes, c.inner_faces, c.boundary_faces) for c in cases]
    levels = []
    for lv in range(max(len(h) for h in per)):
        prev_off = np.cumsum([0] + [m[0] for m in cur])
        nodes, inner, bdry, ch, nxt = [], [], [], [], []
        off = 0
        for i, hier in enumerate(per):
            if lv < len(hier):
                L = hier[lv]
                nxt.append((L["n_cells"], L["mapping_nodes"], L["inner_faces"],
                            L["boundary_faces"]))
                ch.append(L["children"] + prev_off[i])
            else:  # this member's hierarchy ended: its coarsest level stays
                nxt.append(cur[i])
                rows = np.full((cur[i][0], 4), -1, dtype=np.int64)
                rows[:, 0] = prev_off[i] + np.arange(cur[i][0])
                ch.append(rows)
            n_i, nd, fi, fb = nxt[-1]
            a, b = _offset_faces(fi, fb, off)
            nodes.append(nd)
            inner.append(a)
            bdry.append(b)
            off += n_i
        levels.append(dict(
            n_cells=off, mapping_nodes=np.ascontiguousarray(np.concatenate(nodes)),
            inner_faces=np.ascontiguousarray(np.concatenate(inner)),
            boundary_faces=np.ascontiguousarray(np.concatenate(bdry)),
            children=np.ascontiguousarray(np.concatenate(ch).astype(np.int32))))
        cur = nxt
    return Batch(case=case, offsets=offsets, levels=levels, u_target=u_target.reshape(-1),
                 dts=[c.dt for c in cases])
