"""CPU tests of the batched-solve entry points' argument checks (dgx_batch_create rejects
what the batched kernel does not cover before it touches a GPU: other precisions, mixed
physics or parameters, NavierStokesWeakFormulation's own checks), through the C ABI."""

import ctypes as C

import pytest

from meshes import TAGS, periodic_rectangle


@pytest.fixture(scope="module")
def dg():
    import dgfem_gb300 as d
    return d


def _mesh(dg, n):
    v, e, b = periodic_rectangle(n)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    m = dg.DGMesh(v, e, None, dict(TAGS), edges)
    m.set_periodic_boundaries("Left", "Right")
    m.set_periodic_boundaries("Bottom", "Top")
    return m


def _create(dg, meshes, params):
    from dgfem_gb300 import _lib as L
    lib = L.load()
    n = len(params)
    prm = (L.Params * max(n, 1))(*params)
    hs = (C.c_void_p * max(n, 1))(*[m._h.value for m in meshes])
    out = C.c_void_p()
    rc = lib.dgx_batch_create(n, hs, C.cast(prm, C.c_void_p), C.byref(out))
    return rc, out, lib.dgx_last_error().decode()


def _p(L, order=2, physics=None, precision=None, gamma=1.4, basis=None, visc=(0.0, 0.0, 0.0)):
    return L.Params(order, L.BASIS_DUBINER if basis is None else basis, L.EULER if physics is None else physics,
                    L.MIXED if precision is None else precision, gamma, *visc)


NS = (0.01, 0.72, 5.0)


@pytest.mark.parametrize("case,needle", [
    ("order", "between 1 and 4"),
    ("physics", "share the basis, gamma and physics"),
    ("precision", "mixed precision"),
    ("gamma", "share the basis, gamma and physics"),
    ("basis", "share the basis, gamma and physics"),
    ("unknown", "unknown physics"),
    ("mu", "share mu, Prandtl and sigma0"),
    ("sigma0", "share mu, Prandtl and sigma0"),
    ("mu_zero", "Dynamic viscosity must be positive"),
])
def test_batch_create_rejects(dg, case, needle):
    from dgfem_gb300 import _lib as L
    ms = [_mesh(dg, 3), _mesh(dg, 4)]
    first = _p(L, physics=L.NAVIER_STOKES, visc=NS) if case in ("mu", "sigma0", "mu_zero") else _p(L)
    if case == "mu_zero":
        first = _p(L, physics=L.NAVIER_STOKES, visc=(0.0, 0.72, 5.0))
    bad = {"order": _p(L, order=5), "physics": _p(L, physics=L.NAVIER_STOKES, visc=NS),
           "precision": _p(L, precision=L.FP64), "gamma": _p(L, gamma=1.3),
           "basis": _p(L, basis=L.BASIS_MONOMIAL), "unknown": _p(L, physics=7),
           "mu": _p(L, physics=L.NAVIER_STOKES, visc=(0.02, 0.72, 5.0)),
           "sigma0": _p(L, physics=L.NAVIER_STOKES, visc=(0.01, 0.72, 4.0)),
           "mu_zero": _p(L, physics=L.NAVIER_STOKES, visc=(0.0, 0.72, 5.0))}[case]
    rc, out, msg = _create(dg, ms, [first, bad])
    assert rc == L.ERR_INVALID and not out.value
    want = "instance 0" if case == "mu_zero" else "instance 1"
    assert needle in msg and want in msg, msg


def test_batch_create_rejects_quadrilateral_meshes(dg):
    from dgfem_gb300 import _lib as L
    q = dg.DGMesh.rectangle(3, 3, 0.0, 1.0, 0.0, 1.0, element_type="quad")
    rc, out, msg = _create(dg, [_mesh(dg, 3), q], [_p(L), _p(L, basis=L.BASIS_DUBINER)])
    assert rc == L.ERR_INVALID and not out.value
    assert "triangle meshes" in msg and "instance 1" in msg


def test_batch_create_rejects_empty_and_null(dg):
    from dgfem_gb300 import _lib as L
    rc, out, _ = _create(dg, [], [])
    assert rc == L.ERR_INVALID
    lib = L.load()
    out = C.c_void_p()
    assert lib.dgx_batch_create(1, None, None, C.byref(out)) == L.ERR_INVALID
    assert lib.dgx_batch_info(None, 0, None, None, None) == L.ERR_INVALID
    assert lib.dgx_batch_launch_shape(None, None, None) == L.ERR_INVALID
    assert lib.dgx_batch_stage_form(None, None) == L.ERR_INVALID
    assert lib.dgx_launch_shape(None, None, None, None) == L.ERR_INVALID
    assert lib.dgx_stage_tile(None, None, None) == L.ERR_INVALID
    assert lib.dgx_batch_rk3_step(None, None, 1, None) == L.ERR_INVALID


def test_python_batch_rejects_mismatched_lists(dg):
    with pytest.raises(ValueError):
        dg.DGBatch([_mesh(dg, 3)], [])
    with pytest.raises(ValueError):
        dg.DGBatch([], [])
