"""Element partitions of one DG mesh, with a halo exchange between SSP-RK3 stages.

dgfem's explicit step (time_step_ssp_rk3, src/solver/compressible_solver_base.cpp:106-112,
three stages of time_stepping.hpp:39-55) reads, for each element, only its own state and the
states of its face neighbours (DGMesh::build_precomputed_faces, src/core/mesh.cpp:404-480,
with the pairs set_periodic_boundaries adds, :482-588).  So the elements can be split into
parts, one per rank (one GPU each):

* a part holds its owned elements and a one-element halo: every neighbour of an owned element
  that another part owns;
* before each stage the owners send the halo elements' stage state; every part then runs the
  stage on its elements and keeps the owned results.

``PartitionPlan`` builds, on the host, the parts (contiguous blocks of the global element
order by default: row blocks of the structured meshes), each part's mesh arrays and the
exchange lists.  A part's elements are its owned and halo elements in increasing global index,
so each face keeps the left/right roles it has in the global face list, and an owned element's
residual is computed from the same numbers in the same order as on the whole mesh: a run on
parts equals the run on the whole mesh bit for bit (FP64).  The part's boundary edges are those
of the owned elements' faces and of the faces paired with them across a periodic boundary;
the halo elements' other faces are boundary faces without a condition, which take no part.

``PartitionedRK3`` steps one part (an engine with ``rk3_stage``, e.g. an FP64 ``DGContext``)
through the stages with an exchange: ``TorchExchange`` (torch.distributed point-to-point:
NCCL between GPUs, gloo between host processes) or ``LocalExchange`` (several parts in one
process).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np


@dataclass
class Part:
    rank: int
    elements: np.ndarray              # global ids of the part's elements, increasing
    owned: np.ndarray                 # local indices of the owned elements
    vertices: np.ndarray              # [n][2]
    local_elements: np.ndarray        # [n_elements][nvpe], local vertex ids
    boundary_edges: Dict[int, List[Tuple[int, int]]]   # tag -> local vertex pairs
    send: Dict[int, np.ndarray] = field(default_factory=dict)   # peer -> local ids of owned rows it needs
    recv: Dict[int, np.ndarray] = field(default_factory=dict)   # peer -> local ids of halo rows it owns

    @property
    def n_elements(self) -> int:
        return len(self.elements)


class PartitionPlan:
    """Parts of a mesh and their exchange lists.

    vertices [nv][2], elements [ne][nvpe], boundary_edges {tag: [(v1, v2), ...]} and
    boundary_tags {name: tag}: the arrays a DGMesh is built from.  periodic: the tag-name pairs
    passed to set_periodic_boundaries; bcs: {tag name: BoundaryConditionEuler} (constant
    conditions).  interior_faces [n][5]: the whole mesh's face list (DGMesh.get_interior_faces()
    after its periodic pairing).  owner: the part of each element (default: n_parts contiguous
    blocks of the element order)."""

    def __init__(self, vertices, elements, boundary_edges, boundary_tags, periodic: Sequence[Tuple[str, str]],
                 interior_faces, n_parts: int, owner: Optional[np.ndarray] = None, bcs=None):
        V = np.asarray(vertices, dtype=np.float64).reshape(-1, 2)
        E = np.asarray(elements, dtype=np.int64)
        ne, K = E.shape
        if n_parts < 1 or n_parts > max(ne, 1):
            raise ValueError(f"n_parts must be between 1 and the number of elements ({ne})")
        self.n_parts, self.n_elements, self.nvpe = n_parts, ne, K
        self.boundary_tags = dict(boundary_tags)
        self.periodic = [tuple(p) for p in periodic]
        self.bcs = dict(bcs or {})
        self.owner = (np.arange(ne) * n_parts // ne if owner is None else np.asarray(owner)).astype(np.int64)
        F = np.asarray(interior_faces, dtype=np.int64).reshape(-1, 5)
        # neighbour across each (element, face) slot
        nbr = np.full((ne, K), -1, dtype=np.int64)
        nbr[F[:, 0], F[:, 2]] = F[:, 1]
        nbr[F[:, 1], F[:, 3]] = F[:, 0]
        self.neighbors = nbr
        # global boundary edges keyed by their (unordered) vertex pair, in their given order
        nv = len(V)
        bl = [(tag, int(a), int(b)) for tag in sorted(boundary_edges) for a, b in boundary_edges[tag]]
        B = np.array(bl, dtype=np.int64).reshape(-1, 3)
        bkey = np.minimum(B[:, 1], B[:, 2]) * nv + np.maximum(B[:, 1], B[:, 2])
        # every (element, face) slot's edge key
        va, vb = E, np.roll(E, -1, axis=1)
        slot_key = np.minimum(va, vb) * nv + np.maximum(va, vb)
        slot_is_bdry = np.isin(slot_key, bkey)
        self.parts: List[Part] = []
        lmaps = []
        for r in range(n_parts):
            own = np.flatnonzero(self.owner == r)
            nb = nbr[own].ravel()
            nb = nb[nb >= 0]
            halo = np.unique(nb[self.owner[nb] != r])
            elems = np.union1d(own, halo)
            is_owned = self.owner[elems] == r
            vids = np.unique(E[elems].ravel())
            vmap = np.full(nv, -1, dtype=np.int64)
            vmap[vids] = np.arange(len(vids))
            lmap = np.full(ne, -1, dtype=np.int64)
            lmap[elems] = np.arange(len(elems))
            lmaps.append(lmap)
            # boundary edges kept: faces of owned elements, and faces of halo elements whose
            # neighbour across that face (a periodic partner) is owned
            n_across = nbr[elems]
            partner_owned = (n_across >= 0) & (self.owner[np.maximum(n_across, 0)] == r)
            keep_slot = slot_is_bdry[elems] & (is_owned[:, None] | partner_owned)
            keep = np.isin(bkey, slot_key[elems][keep_slot])
            bedges: Dict[int, List[Tuple[int, int]]] = {}
            for tag, a, b in B[keep]:
                bedges.setdefault(int(tag), []).append((int(vmap[a]), int(vmap[b])))
            self.parts.append(Part(rank=r, elements=elems, owned=np.flatnonzero(is_owned), vertices=V[vids],
                                   local_elements=vmap[E[elems]], boundary_edges=bedges))
        # exchange lists: part s needs from part r the halo elements r owns (increasing global id)
        for s, ps in enumerate(self.parts):
            halo_global = np.setdiff1d(ps.elements, ps.elements[ps.owned])
            for r in np.unique(self.owner[halo_global]):
                g = halo_global[self.owner[halo_global] == r]
                ps.recv[int(r)] = lmaps[s][g]
                self.parts[int(r)].send[s] = lmaps[int(r)][g]

    def mesh(self, dg, r: int):
        """The DGMesh of part r (periodic pairing and boundary conditions applied)."""
        p = self.parts[r]
        m = dg.DGMesh(p.vertices, p.local_elements, None, self.boundary_tags, p.boundary_edges)
        present = {self.boundary_tags[n] for n in self.boundary_tags} & set(p.boundary_edges)
        for t1, t2 in self.periodic:
            h1, h2 = self.boundary_tags[t1] in present, self.boundary_tags[t2] in present
            if h1 and h2:
                m.set_periodic_boundaries(t1, t2)
            elif h1 or h2:
                raise RuntimeError(f"part {r} holds faces of '{t1 if h1 else t2}' without their periodic partners")
        for name, bc in self.bcs.items():
            m.set_boundary_condition_euler(name, bc)
        return m

    def scatter(self, u) -> List[np.ndarray]:
        """The whole-mesh state [ne][np][4] split into the parts' states (owned and halo rows)."""
        return [np.ascontiguousarray(np.asarray(u)[p.elements]) for p in self.parts]

    def gather(self, parts) -> np.ndarray:
        """The whole-mesh state from the parts' owned rows."""
        first = np.asarray(parts[0])
        out = np.empty((self.n_elements,) + first.shape[1:], dtype=first.dtype)
        for p, u in zip(self.parts, parts):
            out[p.elements[p.owned]] = np.asarray(u)[p.owned]
        return out


class LocalExchange:
    """The halo exchange of several parts held by one process (lists of per-part states,
    numpy arrays or torch tensors)."""

    def __init__(self, plan: PartitionPlan):
        self.plan = plan

    def exchange_all(self, states) -> None:
        for s, ps in enumerate(self.plan.parts):
            for r, dst in ps.recv.items():
                src = self.plan.parts[r].send[s]
                states[s][dst] = states[r][src]


class TorchExchange:
    """The halo exchange of one part per process over torch.distributed (NCCL between GPUs,
    gloo between host processes): paired isend / irecv of the listed rows."""

    def __init__(self, plan: PartitionPlan, rank: int, group=None):
        self.plan, self.rank, self.group = plan, rank, group

    def exchange(self, u) -> None:
        import torch
        import torch.distributed as dist
        part = self.plan.parts[self.rank]
        t = u if isinstance(u, torch.Tensor) else torch.from_numpy(u)
        ops, recvs = [], []
        for peer in sorted(set(part.send) | set(part.recv)):
            if peer in part.send:
                idx = torch.as_tensor(part.send[peer], device=t.device)
                ops.append(dist.P2POp(dist.isend, t.index_select(0, idx).contiguous(), peer, self.group))
            if peer in part.recv:
                buf = torch.empty((len(part.recv[peer]),) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
                ops.append(dist.P2POp(dist.irecv, buf, peer, self.group))
                recvs.append((peer, buf))
        if ops:
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        for peer, buf in recvs:
            t[torch.as_tensor(part.recv[peer], device=t.device)] = buf


class PartitionedRK3:
    """SSP-RK3 steps of one part: before each stage the halo rows of the stage state arrive from
    their owners; the engine runs the stage on the part's elements (engine.rk3_stage(u_n, u_s,
    out, dt, stage), e.g. DGContext.rk3_stage on device tensors)."""

    def __init__(self, engine, exchange, work=None):
        self.engine, self.exchange = engine, exchange
        self.work = work  # two states shaped like the part's (allocated on first use)

    def step(self, u, dt: float, n_steps: int = 1):
        if self.work is None:
            self.work = (u.clone(), u.clone()) if hasattr(u, "clone") else (u.copy(), u.copy())
        w1, w2 = self.work
        for _ in range(n_steps):
            self.exchange(u)
            self.engine.rk3_stage(u, u, w1, dt, 1)
            self.exchange(w1)
            self.engine.rk3_stage(u, w1, w2, dt, 2)
            self.exchange(w2)
            self.engine.rk3_stage(u, w2, u, dt, 3)
        return u


def step_local(plan: PartitionPlan, engines, states, dt: float, n_steps: int = 1):
    """Every part of a plan in one process (in-process exchange between the stages)."""
    ex = LocalExchange(plan)
    work = [((u.clone(), u.clone()) if hasattr(u, "clone") else (u.copy(), u.copy())) for u in states]
    for _ in range(n_steps):
        ex.exchange_all(states)
        for e, u, (w1, _) in zip(engines, states, work):
            e.rk3_stage(u, u, w1, dt, 1)
        ex.exchange_all([w[0] for w in work])
        for e, u, (w1, w2) in zip(engines, states, work):
            e.rk3_stage(u, w1, w2, dt, 2)
        ex.exchange_all([w[1] for w in work])
        for e, u, (_, w2) in zip(engines, states, work):
            e.rk3_stage(u, w2, u, dt, 3)
    return states
