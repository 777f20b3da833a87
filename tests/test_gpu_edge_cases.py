"""Edge cases through the C ABI: a mesh without elements, meshes of one element (a triangle
and a quadrilateral whose every face is a boundary face), and a ragged last tile, in every
precision mode; each against the oracle where there is something to compare."""

import numpy as np
import pytest

import oracle as O
from meshes import TAGS, isentropic_vortex, periodic_rectangle, primitive_to_conserved, PERIODIC_PAIRS

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

U_INF = primitive_to_conserved([1.0, 0.3, 0.1, 1.0])


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    return d


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("precision", ["fp64", "mixed", "df64"])
@pytest.mark.parametrize("nvpe", [3, 4])
def test_mesh_without_elements(dg, precision, nvpe):
    v = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    m = dg.DGMesh(v, np.zeros((0, nvpe), np.int32), None, dict(TAGS), {})
    space = dg.DGSpace("triangle", 2, "dubiner") if nvpe == 3 else dg.DGSpace("quad", 2)
    ctx = dg.DGContext(m, space, dg.EulerWeakFormulation(1.4), precision)
    assert ctx.n_elements == 0
    u = np.zeros(ctx.shape)
    assert ctx.residual(u).shape == ctx.shape
    assert ctx.rk3_step(u, 0.01, 3).shape == ctx.shape
    ut = torch.zeros(ctx.shape, dtype=torch.float64, device="cuda")
    ctx.rk3_step(ut, 0.01, 2)
    assert ctx.max_cfl(ut, 0.01) == 0.0
    assert not ctx.step_nonfinite()


def one_element(nvpe):
    if nvpe == 3:
        v = np.array([[0.0, 0.0], [1.0, 0.1], [0.2, 0.9]])
        e = np.array([[0, 1, 2]], np.int32)
        b = np.array([(TAGS["Bottom"], 0, 1), (TAGS["Right"], 1, 2), (TAGS["Left"], 2, 0)], np.int32)
    else:
        v = np.array([[0.0, 0.0], [1.0, 0.1], [1.1, 1.0], [-0.1, 0.8]])
        e = np.array([[0, 1, 2, 3]], np.int32)
        b = np.array([(TAGS["Bottom"], 0, 1), (TAGS["Right"], 1, 2), (TAGS["Top"], 2, 3), (TAGS["Left"], 3, 0)],
                     np.int32)
    return v, e, b


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("nvpe", [3, 4])
def test_single_element_all_boundary_faces(dg, nvpe, visc):
    v, e, b = one_element(nvpe)
    basis = O.LEGENDRE if nvpe == 4 else O.DUBINER
    om = O.OracleMesh(v, e, b, order=2, basis=basis)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    spec = [("Bottom", O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]), ("Right", O.FAR_FIELD, U_INF),
            ("Top", O.SLIP_WALL, [0.0] * 4), ("Left", O.FAR_FIELD, U_INF)]
    for name, typ, val in spec:
        if name == "Top" and nvpe == 3:
            continue
        om.set_bc(TAGS[name], typ, value=val)
        pm.set_boundary_condition_euler(name, dg.BoundaryConditionEuler(typ, val))
    if visc:
        ph, wf = O.navier_stokes(1.4, 0.05, 0.72, 5.0), dg.NavierStokesWeakFormulation(1.4, 0.05, 0.72, 5.0)
    else:
        ph, wf = O.euler(1.4), dg.EulerWeakFormulation(1.4)
    u = om.project(np.broadcast_to(U_INF, om.quad_points().shape[:-1] + (4,)).copy())
    u = u + 1e-2 * np.random.default_rng(2).standard_normal(u.shape) * np.abs(u).max()
    space = dg.DGSpace("quad", 2) if nvpe == 4 else dg.DGSpace("triangle", 2, "dubiner")
    R = om.residual(ph, u)
    c64 = dg.DGContext(pm, space, wf, "fp64")
    assert rel(c64.residual(u), R) <= 1e-12
    assert rel(dg.DGContext(pm, space, wf, "df64").residual(u), R) <= 1e-11
    assert rel(dg.DGContext(pm, space, wf, "mixed").residual(u), R) <= 2e-5
    dt = 0.01 / om.max_cfl(1.4, u, 1.0)
    ref = om.rk3_step(ph, u, dt, 3)
    assert rel(c64.rk3_step(u, dt, 3), ref) <= 1e-11
    assert rel(dg.DGContext(pm, space, wf, "mixed").rk3_step(u, dt, 3), ref) <= 1e-6


@pytest.mark.parametrize("n", [5, 9, 13])
def test_ragged_last_tile(dg, n):
    """n x n x 2 elements: 50, 162, 338, so the last 128-element tile is partial."""
    v, e, b = periodic_rectangle(n)
    om = O.OracleMesh(v, e, b, order=3, basis=O.DUBINER, periodic=PERIODIC_PAIRS)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    pm.set_periodic_boundaries("Left", "Right")
    pm.set_periodic_boundaries("Bottom", "Top")
    u0 = om.project(isentropic_vortex(om.quad_points(), beta=4.0, xc=0.5))
    dt = 0.05 / om.max_cfl(1.4, u0, 1.0)
    ref = om.rk3_step(O.euler(1.4), u0, dt, 2)
    space = dg.DGSpace("triangle", 3, "dubiner")
    for precision, tol in (("fp64", 1e-11), ("mixed", 1e-6), ("df64", 1e-11)):
        ctx = dg.DGContext(pm, space, dg.EulerWeakFormulation(1.4), precision)
        ut = torch.tensor(u0, device="cuda")
        ctx.rk3_step(ut, dt, 2)
        assert rel(ut.cpu().numpy(), ref) <= tol, precision
