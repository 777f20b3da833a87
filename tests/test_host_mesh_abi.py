"""CPU tests of the product's host side: mesh connectivity against the oracle (dgfem's
DGMesh semantics), the structured generator, error behaviour without a GPU, and that
libdgx.so exports every function include/dgx.h declares."""

import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, TAGS, periodic_rectangle, quad_rectangle, two_triangle_mesh

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def dg():
    import dgfem_gb300 as d
    return d


def _product_mesh(dg, v, e, b, periodic=False):
    tags = dict(TAGS)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    m = dg.DGMesh(v, e, None, tags, edges)
    if periodic:
        m.set_periodic_boundaries("Left", "Right")
        m.set_periodic_boundaries("Bottom", "Top")
    return m


def test_header_symbols_exported():
    hdr = (ROOT / "include" / "dgx.h").read_text()
    declared = set(re.findall(r"\b(dgx_\w+)\s*\(", hdr))
    so = ROOT / "discontinuous-galerkin-fem_gb300" / "libdgx.so"
    if not so.exists():
        import build as b  # noqa
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (dgx_\w+)", out))
    assert declared, "no declarations parsed"
    assert declared <= exported, declared - exported


def test_library_loads_and_binding_matches_header(dg):
    from dgfem_gb300 import _lib
    lib = _lib.load()
    hdr = (ROOT / "include" / "dgx.h").read_text()
    declared = set(re.findall(r"\b(dgx_\w+)\s*\(", hdr))
    assert declared == set(_lib.SIGNATURES)
    assert lib.dgx_version().startswith(b"dgx")


@pytest.mark.parametrize("n", [2, 3, 5, 8])
def test_periodic_faces_match_oracle(dg, n):
    v, e, b = periodic_rectangle(n)
    om = O.OracleMesh(v, e, b, order=1, periodic=PERIODIC_PAIRS)
    pm = _product_mesh(dg, v, e, b, periodic=True)
    assert np.array_equal(pm.get_interior_faces(), om.interior_faces())
    assert np.array_equal(pm.get_boundary_face_data(), om.boundary_faces())


def test_open_mesh_faces_match_oracle(dg):
    v, e, b = periodic_rectangle(4, 0, 1, 0, 2)
    om = O.OracleMesh(v, e, b, order=1)
    pm = _product_mesh(dg, v, e, b)
    assert np.array_equal(pm.get_interior_faces(), om.interior_faces())
    assert np.array_equal(pm.get_boundary_face_data(), om.boundary_faces())


def test_two_triangle_mesh_matches_oracle(dg):
    v, e, b = two_triangle_mesh()
    om = O.OracleMesh(v, e, b, order=1)
    tags = {"bottom": 1, "right": 2, "top": 3, "left": 4}
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, tags, edges)
    assert np.array_equal(pm.get_interior_faces(), om.interior_faces())
    assert np.array_equal(pm.get_boundary_face_data(), om.boundary_faces())


def test_perturbed_unstructured_mesh_matches_oracle(dg):
    rng = np.random.default_rng(3)
    v, e, b = periodic_rectangle(6, 0, 1, 0, 1)
    inner = (v[:, 0] > 0) & (v[:, 0] < 1) & (v[:, 1] > 0) & (v[:, 1] < 1)
    v = v.copy()
    v[inner] += rng.uniform(-0.04, 0.04, size=(inner.sum(), 2))
    perm = rng.permutation(len(e))
    e = e[perm]
    om = O.OracleMesh(v, e, b, order=2)
    pm = _product_mesh(dg, v, e, b)
    assert np.array_equal(pm.get_interior_faces(), om.interior_faces())
    assert np.array_equal(pm.get_boundary_face_data(), om.boundary_faces())


@pytest.mark.parametrize("n,nx", [(4, None), (16, None), (3, 5)])
def test_rectangle_generator_matches_reference_layout(dg, n, nx):
    v, e, b = periodic_rectangle(n, -5, 5, -5, 5, nx=nx)
    pm = dg.DGMesh.rectangle(nx or n, n, -5, 5, -5, 5, periodic=True)
    assert np.array_equal(pm.get_vertices(), v)
    assert np.array_equal(pm.get_elements(), e)
    om = O.OracleMesh(v, e, b, order=1, periodic=PERIODIC_PAIRS)
    assert np.array_equal(pm.get_interior_faces(), om.interior_faces())
    assert len(pm.get_boundary_face_data()) == 0


def test_error_behaviour(dg):
    with pytest.raises(ValueError):
        dg.DGMesh.rectangle(0, 4, 0, 1, 0, 1)
    m = dg.DGMesh.rectangle(2, 2, 0, 1, 0, 1, periodic=False)
    with pytest.raises(ValueError):
        m.set_periodic_boundaries("Nope", "Top")
    with pytest.raises(IndexError):
        dg.DGMesh(np.zeros((3, 2)), np.array([[0, 1, 5]]), None, {}, {})
    with pytest.raises(ValueError):
        dg.NavierStokesWeakFormulation(1.4, -1.0)


def test_no_gpu_fails_loudly(dg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    m = dg.DGMesh.rectangle(2, 2, 0, 1, 0, 1)
    with pytest.raises(dg.DGXError) as ei:
        dg.DGContext(m, dg.DGSpace("triangle", 2), dg.EulerWeakFormulation())
    assert "no CPU fallback" in str(ei.value)


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("n,nx,distort", [(3, None, 0.0), (5, 4, 0.25), (8, None, 0.2)])
def test_quad_mesh_faces_match_oracle(dg, n, nx, distort, periodic):
    """Quadrilateral meshes (4-column element arrays): neighbour pairing, face lists and
    the reversed flags equal the oracle's restatement of DGMesh."""
    v, e, b = quad_rectangle(n, nx=nx, distort=distort, seed=n)
    om = O.OracleMesh(v, e, b, order=2, basis=O.LEGENDRE, periodic=PERIODIC_PAIRS if periodic else ())
    pm = _product_mesh(dg, v, e, b, periodic=periodic)
    assert pm.get_element_type() == "quad" and pm.vertices_per_element() == 4
    assert np.array_equal(pm.get_elements(), e)
    assert np.array_equal(pm.get_interior_faces(), om.interior_faces())
    assert np.array_equal(pm.get_boundary_face_data(), om.boundary_faces())
    if periodic:
        assert len(pm.get_boundary_face_data()) == 0


def test_quad_mesh_permuted_elements_match_oracle(dg):
    rng = np.random.default_rng(7)
    v, e, b = quad_rectangle(6, distort=0.2)
    e = e[rng.permutation(len(e))]
    om = O.OracleMesh(v, e, b, order=1, basis=O.LEGENDRE)
    pm = _product_mesh(dg, v, e, b)
    assert np.array_equal(pm.get_interior_faces(), om.interior_faces())
    assert np.array_equal(pm.get_boundary_face_data(), om.boundary_faces())


def test_element_type_errors(dg):
    with pytest.raises(ValueError):
        dg.DGMesh(np.zeros((5, 2)), np.array([[0, 1, 2, 3, 4]]), None, {}, {})
    with pytest.raises(ValueError):
        dg.DGSpace("hexagon", 2)
    with pytest.raises(ValueError):
        dg.DGSpace("quad", 2, "dubiner")
    with pytest.raises(ValueError):
        dg.DGSpace("triangle", 2, "legendre")
    assert dg.DGSpace("quad", 2).basis == 2


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("n,nx", [(4, None), (3, 5)])
def test_quad_rectangle_generator(dg, n, nx, periodic):
    v, e, b = quad_rectangle(n, -5, 5, -5, 5, nx=nx)
    pm = dg.DGMesh.rectangle(nx or n, n, -5, 5, -5, 5, periodic=periodic, element_type="quad")
    assert np.array_equal(pm.get_vertices(), v)
    assert np.array_equal(pm.get_elements(), e)
    om = O.OracleMesh(v, e, b, order=1, basis=O.LEGENDRE, periodic=PERIODIC_PAIRS if periodic else ())
    assert np.array_equal(pm.get_interior_faces(), om.interior_faces())
    assert np.array_equal(pm.get_boundary_face_data(), om.boundary_faces())
