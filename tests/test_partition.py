"""Element partitions with a halo exchange between SSP-RK3 stages (dgfem_gb300.partition), on
the host: the plan's parts and exchange lists, and partitioned runs against the whole mesh.

The stage engine here is the FP64 oracle (each part's mesh restated on the CPU; a stage is
out = a u_n + b (u_s + dt M^-1 R(u_s)), the three stages of time_stepping.hpp:39-55), so the
partition, the parts' meshes (periodic pairs across parts, boundary conditions, halo faces that
take no part) and the exchange are checked without a GPU.  A run on parts must equal the run on
the whole mesh bit for bit: every owned element's residual comes from the same numbers in the
same order.  The gloo tests run 2 and 4 ranks as separate processes (torch.distributed point-
to-point exchange, as between GPUs with NCCL).
"""

import os
import socket
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from meshes import BOTTOM, LEFT, RIGHT, TAGS, TOP, isentropic_vortex, periodic_rectangle, primitive_to_conserved

ROOT = Path(__file__).resolve().parent.parent
TAG_IDS = dict(TAGS)
MATCH_Y = {"Left": True, "Right": True, "Bottom": False, "Top": False}
U_INF = primitive_to_conserved([1.0, 0.4, 0.1, 1.0])
WALLS = {"Bottom": (O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]), "Right": (O.FAR_FIELD, U_INF),
         "Top": (O.SLIP_WALL, [0.0, 0.0, 0.0, 0.0]), "Left": (O.FAR_FIELD, U_INF)}


@pytest.fixture(scope="module")
def dg():
    import dgfem_gb300 as d
    return d


def edges_of(b):
    out = {}
    for t, a, c in b:
        out.setdefault(int(t), []).append((int(a), int(c)))
    return out


def case(kind, n=8):
    """(vertices, elements, boundary edges, periodic pairs, boundary conditions, physics, order)"""
    v, e, b = periodic_rectangle(n)
    if kind == "walls":
        rng = np.random.default_rng(5)
        inner = (np.abs(v[:, 0]) < 4.99) & (np.abs(v[:, 1]) < 4.99)
        v = v.copy()
        v[inner] += 0.15 * (10.0 / n) * rng.uniform(-1, 1, (inner.sum(), 2))
        return v, e, b, [], WALLS, O.euler(1.4), 2
    periodic = [("Left", "Right"), ("Bottom", "Top")]
    if kind == "channel":  # periodic in x, walls below and above
        return v, e, b, [("Left", "Right")], {"Bottom": WALLS["Bottom"], "Top": WALLS["Top"]}, O.euler(1.4), 3
    phys = O.navier_stokes(1.4, 0.02, 0.72, 5.0) if kind == "ns" else O.euler(1.4)
    return v, e, b, periodic, {}, phys, 3 if kind == "euler" else 2


def make_plan(dg, v, e, b, periodic, bcs, n_parts):
    from dgfem_gb300.partition import PartitionPlan
    m = dg.DGMesh(v, e, None, TAGS, edges_of(b))
    for t1, t2 in periodic:
        m.set_periodic_boundaries(t1, t2)
    return PartitionPlan(v, e, edges_of(b), TAGS, periodic, m.get_interior_faces(), n_parts,
                         bcs={k: dg.BoundaryConditionEuler(t, val) for k, (t, val) in bcs.items()})


class OracleEngine:
    """One part's FP64 stages on the CPU oracle (test infrastructure)."""

    def __init__(self, plan, r, order, phys, bcs):
        p = plan.parts[r]
        be = np.array([(t, a, c) for t in sorted(p.boundary_edges) for a, c in p.boundary_edges[t]],
                      dtype=np.int32).reshape(-1, 3)
        present = set(p.boundary_edges)
        per = [(TAG_IDS[t1], TAG_IDS[t2], MATCH_Y[t1]) for t1, t2 in plan.periodic
               if TAG_IDS[t1] in present and TAG_IDS[t2] in present]
        self.om = O.OracleMesh(p.vertices, p.local_elements, be, order=order, basis=O.DUBINER, periodic=per)
        for name, (t, val) in bcs.items():
            self.om.set_bc(TAG_IDS[name], t, value=val)
        self.phys = phys

    def rk3_stage(self, u_n, u_s, out, dt, stage):
        un, us, o = (np.asarray(x) for x in (u_n, u_s, out))
        L = self.om.rhs(self.phys, us)
        a, b = ((0.0, 1.0), (0.75, 0.25), (1.0 / 3.0, 2.0 / 3.0))[stage - 1]
        o[...] = (us + dt * L) if stage == 1 else a * un + b * (us + dt * L)


def run_parts(dg, kind, n_parts, steps=5):
    from dgfem_gb300.partition import step_local
    v, e, b, periodic, bcs, phys, order = case(kind)
    plan = make_plan(dg, v, e, b, periodic, bcs, n_parts)
    ref_plan = make_plan(dg, v, e, b, periodic, bcs, 1)
    om = OracleEngine(ref_plan, 0, order, phys, bcs).om
    u0 = om.project(isentropic_vortex(om.quad_points(), beta=4.0, xc=0.4, yc=-0.3, uinf=0.4))
    dt = 0.02 / om.max_cfl(1.4, u0, 1.0)
    states = plan.scatter(u0)
    engines = [OracleEngine(plan, r, order, phys, bcs) for r in range(n_parts)]
    step_local(plan, engines, states, dt, steps)
    return plan.gather(states), u0, dt, ref_plan, order, phys, bcs


@pytest.mark.parametrize("n_parts", [2, 3, 4, 7])
@pytest.mark.parametrize("kind", ["euler", "walls", "channel"])
def test_plan_parts_keep_the_global_faces(dg, kind, n_parts):
    """Every owned element of every part has, in the part's own mesh, the neighbours, face
    numbers, point order and left/right roles it has in the whole mesh; the exchange lists pair
    up and cover every halo element once."""
    v, e, b, periodic, bcs, _, _ = case(kind)
    plan = make_plan(dg, v, e, b, periodic, bcs, n_parts)
    m = dg.DGMesh(v, e, None, TAGS, edges_of(b))
    for t1, t2 in periodic:
        m.set_periodic_boundaries(t1, t2)
    G = m.get_interior_faces()
    gface = {}
    for eL, eR, fL, fR, rev in G:
        gface[(eL, fL)] = (eR, fR, rev, True)
        gface[(eR, fR)] = (eL, fL, rev, False)
    owned_all = np.concatenate([p.elements[p.owned] for p in plan.parts])
    assert np.array_equal(np.sort(owned_all), np.arange(len(e)))
    for r, p in enumerate(plan.parts):
        lm = plan.mesh(dg, r)
        lf = {}
        for eL, eR, fL, fR, rev in lm.get_interior_faces():
            lf[(eL, fL)] = (eR, fR, rev, True)
            lf[(eR, fR)] = (eL, fL, rev, False)
        for li in p.owned:
            ge = p.elements[li]
            for f in range(3):
                if (ge, f) in gface:
                    nb, nf, rev, is_l = gface[(ge, f)]
                    lnb, lnf, lrev, lis_l = lf[(li, f)]
                    assert (p.elements[lnb], lnf, lrev, lis_l) == (nb, nf, rev, is_l), (r, ge, f)
                else:
                    assert (li, f) not in lf
        halo = np.setdiff1d(np.arange(p.n_elements), p.owned)
        got = np.sort(np.concatenate([ix for ix in p.recv.values()])) if p.recv else np.zeros(0, int)
        assert np.array_equal(got, halo)
        for s, ix in p.recv.items():
            src = plan.parts[s]
            assert np.array_equal(src.elements[src.send[r]], p.elements[ix])
            assert np.all(np.isin(src.send[r], src.owned))


@pytest.mark.parametrize("n_parts", [2, 4])
@pytest.mark.parametrize("kind", ["euler", "ns", "walls", "channel"])
def test_partitioned_run_equals_whole_mesh(dg, kind, n_parts):
    """Five steps on parts (in-process exchange) equal five steps on the whole mesh bit for bit."""
    from dgfem_gb300.partition import step_local
    u_parts, u0, dt, ref_plan, order, phys, bcs = run_parts(dg, kind, n_parts)
    whole = [u0.copy()]
    step_local(ref_plan, [OracleEngine(ref_plan, 0, order, phys, bcs)], whole, dt, 5)
    assert np.isfinite(whole[0]).all()
    assert np.linalg.norm(whole[0] - u0) > 1e-6 * np.linalg.norm(u0)  # the state moved
    assert np.array_equal(u_parts, whole[0])
    # and the whole-mesh stage engine agrees with the oracle's own SSP-RK3 step
    om = OracleEngine(ref_plan, 0, order, phys, bcs).om
    ref = om.rk3_step(phys, u0, dt, 5)
    assert np.linalg.norm(whole[0] - ref) <= 1e-13 * np.linalg.norm(ref)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("n_ranks", [2, 4])
@pytest.mark.parametrize("kind", ["euler", "ns"])
def test_partitioned_run_on_gloo_ranks(dg, tmp_path, kind, n_ranks):
    """One part per process, halo rows exchanged over torch.distributed (gloo), five steps: the
    gathered owned rows equal the whole-mesh run bit for bit."""
    script = tmp_path / "worker.py"
    script.write_text(textwrap.dedent(f"""
        import sys
        sys.path[:0] = [{str(ROOT / "tests")!r}, {str(ROOT / "oracle")!r},
                        {str(ROOT / "discontinuous-galerkin-fem_gb300")!r}]
        import numpy as np
        import torch
        import torch.distributed as dist
        import dgfem_gb300 as dg
        from dgfem_gb300.partition import PartitionedRK3, TorchExchange
        import test_partition as T
        dist.init_process_group("gloo")
        rank, ws = dist.get_rank(), dist.get_world_size()
        v, e, b, periodic, bcs, phys, order = T.case({kind!r})
        plan = T.make_plan(dg, v, e, b, periodic, bcs, ws)
        ref_plan = T.make_plan(dg, v, e, b, periodic, bcs, 1)
        om = T.OracleEngine(ref_plan, 0, order, phys, bcs).om
        u0 = om.project(T.isentropic_vortex(om.quad_points(), beta=4.0, xc=0.4, yc=-0.3, uinf=0.4))
        dt = 0.02 / om.max_cfl(1.4, u0, 1.0)
        u = torch.from_numpy(plan.scatter(u0)[rank])
        eng = T.OracleEngine(plan, rank, order, phys, bcs)
        PartitionedRK3(eng, TorchExchange(plan, rank).exchange).step(u, dt, 5)
        np.save({str(tmp_path)!r} + f"/part{{rank}}.npy", u.numpy())
        dist.barrier()
        dist.destroy_process_group()
    """))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", str(n_ranks),
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(script)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    u_gloo = make_plan(dg, *case(kind)[:5], n_ranks).gather([np.load(tmp_path / f"part{k}.npy") for k in range(n_ranks)])
    u_local, *_ = run_parts(dg, kind, 1)
    assert np.array_equal(u_gloo, u_local)
