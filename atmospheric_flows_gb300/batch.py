"""Batched members: several flow-over-hill members concatenated into one
device context, so every kernel launch covers the cells of all of them.

Members of one batch share the mesh size and polynomial degree (their
terrain, background and perturbations differ).  Their cells are concatenated
with disjoint connectivity, so every operator is block diagonal over the
members and one launch advances them all: the "concatenated cell list" of
the serving design.  The Krylov solves and the Picard loop then run on the
whole batch: a solve stops when the batch's residual meets the tolerance,
and the Picard loop iterates until every member has converged.  Each member's
relative residual is therefore within sqrt(members) of the stated
tolerance, and its fields agree with a solo run at the same dt to the solver
tolerance (1e-8 in u at Schur rtol 1e-10; test_member_same_alone_and_in_batch
bounds it by 1e-7).

The batch advances with the smallest dt of its members (the strictest
acoustic CFL); the sponge relaxes each member toward its own background wind
(atm_solver_set_sponge_target).  The multigrid hierarchy is each member's
hierarchy concatenated level by level.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .hill import HillCase, mg_hierarchy


@dataclasses.dataclass
class Batch:
    case: HillCase            # the concatenated member set
    offsets: list             # first cell of each member
    cells: int                # cells per member
    levels: list              # concatenated multigrid levels (fine to coarse)
    u_target: np.ndarray      # per-node sponge target velocity [cells][2][node]

    @property
    def members(self) -> int:
        return len(self.offsets)

    def split(self, field: np.ndarray, ncomp: int = 1) -> list:
        """Per-member views of a concatenated nodal field."""
        per = self.cells * ncomp * (self.case.degree + 1) ** 2
        return [field[i * per:(i + 1) * per] for i in range(self.members)]

    def split_state(self, state) -> list:
        rho, u, p = state
        return list(zip(self.split(rho), self.split(u, 2), self.split(p)))


def batch_key(params) -> tuple:
    """Members can share a batch when these agree."""
    return (params.nx, params.nz, params.degree, params.mapping_degree, params.periodic)


def _offset_faces(inner, bdry, off):
    inner = inner.copy()
    inner[:, 0] += off
    inner[:, 2] += off
    bdry = bdry.copy()
    bdry[:, 0] += off
    return inner, bdry


def concat(cases, mg_levels: int = 8) -> Batch:
    """Concatenate members (same batch_key) into one case."""
    if not cases:
        raise ValueError("empty batch")
    key = batch_key(cases[0].params)
    if any(batch_key(c.params) != key for c in cases):
        raise ValueError("batched members need the same mesh size, degree and mapping")
    nc = cases[0].n_cells
    nn2 = (cases[0].degree + 1) ** 2
    inner, bdry = [], []
    for i, c in enumerate(cases):
        a, b = _offset_faces(c.inner_faces, c.boundary_faces, i * nc)
        inner.append(a)
        bdry.append(b)
    u_target = np.zeros((len(cases) * nc, 2, nn2))
    for i, c in enumerate(cases):
        u_target[i * nc:(i + 1) * nc, 0, :] = c.params.u0
    case = dataclasses.replace(
        cases[0], n_cells=len(cases) * nc,
        mapping_nodes=np.ascontiguousarray(np.concatenate([c.mapping_nodes for c in cases])),
        inner_faces=np.ascontiguousarray(np.concatenate(inner)),
        boundary_faces=np.ascontiguousarray(np.concatenate(bdry)),
        node_xz=np.concatenate([c.node_xz for c in cases]),
        rho=np.ascontiguousarray(np.concatenate([c.rho for c in cases])),
        u=np.ascontiguousarray(np.concatenate([c.u for c in cases])),
        p=np.ascontiguousarray(np.concatenate([c.p for c in cases])),
        sponge_alpha=np.ascontiguousarray(np.concatenate([c.sponge_alpha for c in cases])),
        dt=min(c.dt for c in cases))
    per = [mg_hierarchy(c.params, max_levels=mg_levels) for c in cases]
    levels = []
    prev_nc = nc
    for lv in range(len(per[0])):
        m = per[0][lv]["n_cells"]
        inner, bdry, ch = [], [], []
        for i, hier in enumerate(per):
            L = hier[lv]
            a, b = _offset_faces(L["inner_faces"], L["boundary_faces"], i * m)
            inner.append(a)
            bdry.append(b)
            ch.append(L["children"] + i * prev_nc)
        levels.append(dict(
            n_cells=len(cases) * m,
            mapping_nodes=np.ascontiguousarray(np.concatenate([h[lv]["mapping_nodes"] for h in per])),
            inner_faces=np.ascontiguousarray(np.concatenate(inner)),
            boundary_faces=np.ascontiguousarray(np.concatenate(bdry)),
            children=np.ascontiguousarray(np.concatenate(ch).astype(np.int32))))
        prev_nc = m
    return Batch(case=case, offsets=[i * nc for i in range(len(cases))], cells=nc,
                 levels=levels, u_target=u_target.reshape(-1))
