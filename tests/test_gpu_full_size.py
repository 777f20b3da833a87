"""GPU parity against the CPU oracle at the full sizes of the headline workloads.

The other parity tests run meshes of at most 16 x 16 x 2; these compare the C-ABI path with
the oracle where ragged indexing, the persistent stage grids and the face-trace buffers run
at scale:

* Euler isentropic vortex, periodic [-5,5]^2, 512 x 512 x 2 = 524,288 triangles, Dubiner p=3
  (20,971,520 DOF), vortex centre drawn from seed 0 in [-2,2]^2, dt = 0.05 / max CFL:
    FP64 residual of that state (assemble_euler_residual)   <= max(1e-12, 2 kappa)
    FP64 residual of that state plus 1e-3 noise              <= 1e-12 relative L2
    FP64 SSP-RK3, 3 steps                                    <= 1e-11
    mixed precision SSP-RK3, 3 steps                         <= 1e-6
* Navier-Stokes Taylor-Green-type vortex, periodic [0,2pi]^2, 256 x 256 x 2 = 131,072
  triangles, Dubiner p=4, mu = 1/1600 (Re 1600), Pr 0.71, sigma0 5, velocity noise 1e-3:
    FP64 residual                                 <= max(1e-12, 2 kappa)
    mixed-precision residual (FP32 arithmetic)    <= max(2e-5, 2 kappa32)
    mixed precision SSP-RK3, 3 steps              <= 1e-6

kappa is the conditioning of the residual of that state, measured on the oracle itself: the
relative change of the oracle's residual when every input value is moved by one unit in the
last place (random sign).  The residual of a smooth field on a fine mesh is a small
difference of large flux terms, so kappa grows like 1/h: 6.5e-14 at 16 x 16 x 2, 2.1e-12 at
512 x 512 x 2 for the vortex.  Two FP64 evaluations that round in a different order (FMA
contraction, summation order; dgfem's own Release build uses -ffast-math) cannot agree more
closely than that, so on such states the bar is 2 kappa where that exceeds 1e-12.  kappa32
is the same measurement with a one-ulp change in FP32 (2^-24): the floor of any residual
computed in FP32 arithmetic, 4.9e-4 for the Taylor-Green state (its pressure, 1/(gamma M^2) =
71, dwarfs the velocity terms).  The stepping tests need no such allowance: a step adds
dt times the residual to the state, so the state's own scale sets their error.

The oracle runs on every host core (OpenMP); its results do not depend on the thread count.
"""

import math
import os

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, TAGS, isentropic_vortex, periodic_rectangle, taylor_green

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    O.set_threads(os.cpu_count() or 1)
    yield d
    O.set_threads(1)


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def conditioning(om, ph, u, R, ulp=2.0 ** -53):
    """Relative change of the oracle's residual under a one-ulp (`ulp`), random-sign change
    of every input value (the residual's own rounding floor for this state)."""
    rng = np.random.default_rng(12345)
    up = u * (1.0 + ulp * rng.choice([-1.0, 1.0], size=u.shape))
    return rel(om.residual(ph, up), R)


def make_pair(dg, v, e, b, order):
    om = O.OracleMesh(v, e, b, order=order, basis=O.DUBINER, periodic=PERIODIC_PAIRS)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    pm.set_periodic_boundaries("Left", "Right")
    pm.set_periodic_boundaries("Bottom", "Top")
    return om, pm


@pytest.fixture(scope="module")
def euler_512(dg):
    v, e, b = periodic_rectangle(512)
    om, pm = make_pair(dg, v, e, b, 3)
    xc, yc = np.random.default_rng(0).uniform(-2.0, 2.0, size=2)
    u = om.project(isentropic_vortex(om.quad_points(), beta=5.0, xc=xc, yc=yc))
    dt = 0.05 / om.max_cfl(1.4, u, 1.0)
    return om, pm, u, dt


def test_euler_512_fp64_residual(dg, euler_512):
    om, pm, u, _ = euler_512
    assert om.ne == 524288
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "fp64")
    ph = O.euler(1.4)
    R_ref = om.residual(ph, u)
    kappa = conditioning(om, ph, u, R_ref)
    assert kappa < 1e-11  # a sanity bound on the measured floor itself
    err = rel(ctx.residual(torch.tensor(u, device="cuda")).cpu().numpy(), R_ref)
    assert err <= max(1e-12, 2.0 * kappa), (err, kappa)
    # the same state with noise of 1e-3 of its largest value: the residual is then far from
    # its rounding floor and the plain 1e-12 bar applies
    un = u + 1e-3 * np.random.default_rng(3).standard_normal(u.shape) * np.abs(u).max()
    err = rel(ctx.residual(torch.tensor(un, device="cuda")).cpu().numpy(), om.residual(ph, un))
    assert err <= 1e-12, err


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-6)])
def test_euler_512_rk3(dg, euler_512, precision, tol):
    om, pm, u, dt = euler_512
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), precision)
    ut = torch.tensor(u, device="cuda")
    ctx.rk3_step(ut, dt, 3)
    ref = om.rk3_step(O.euler(1.4), u, dt, 3)
    err = rel(ut.cpu().numpy(), ref)
    assert err <= tol, err
    assert rel(ref, u) > 1e-6  # the state moved by more than the bar


@pytest.fixture(scope="module")
def ns_256(dg):
    v, e, b = periodic_rectangle(256, 0.0, 2 * math.pi, 0.0, 2 * math.pi)
    om, pm = make_pair(dg, v, e, b, 4)
    u = om.project(taylor_green(om.quad_points(), seed=0))
    ph = O.navier_stokes(1.4, 1.0 / 1600.0, 0.71, 5.0)
    wf = dg.NavierStokesWeakFormulation(1.4, 1.0 / 1600.0, 0.71, 5.0)
    dt = 0.025 / om.max_cfl(1.4, u, 1.0)
    return om, pm, u, ph, wf, dt


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ns_256_residual(dg, ns_256, precision):
    om, pm, u, ph, wf, _ = ns_256
    assert om.ne == 131072
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 4, "dubiner"), wf, precision)
    R = ctx.residual(torch.tensor(u, device="cuda")).cpu().numpy()
    R_ref = om.residual(ph, u)
    err = rel(R, R_ref)
    if precision == "fp64":
        kappa = conditioning(om, ph, u, R_ref)
        assert kappa < 1e-11
        assert err <= max(1e-12, 2.0 * kappa), (err, kappa)
    else:
        kappa32 = conditioning(om, ph, u, R_ref, ulp=2.0 ** -24)
        assert err <= max(2e-5, 2.0 * kappa32), (err, kappa32)


def test_ns_256_mixed_rk3(dg, ns_256):
    om, pm, u, ph, wf, dt = ns_256
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 4, "dubiner"), wf, "mixed")
    ut = torch.tensor(u, device="cuda")
    ctx.rk3_step(ut, dt, 3)
    ref = om.rk3_step(ph, u, dt, 3)
    err = rel(ut.cpu().numpy(), ref)
    assert err <= 1e-6, err
