"""Device-side set-up (dgx_setup.cu) against the host's, through the C ABI.

* connectivity: meshes of at least 65,536 face slots pair their faces on the GPU (a stable radix
  sort of the vertex-pair keys); the face lists (interior faces with their roles, face numbers and
  orientation; boundary faces with their tags) equal the host-built ones entry for entry, before
  and after periodic pairing, for triangles and quadrilaterals;
* geometry: dgx_create computes the element records and the volume points on the GPU; contexts
  built with DGX_SETUP_ON_HOST=1 (the host's records) give the same quadrature points, the same
  residual and the same mixed-precision steps bit for bit;
* a degenerate element is rejected by either path with dgfem's message.
"""

import numpy as np
import pytest

from meshes import TAGS, periodic_rectangle, quad_rectangle, isentropic_vortex, primitive_to_conserved

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    return d


def edges_of(b):
    out = {}
    for t, a, c in b:
        out.setdefault(int(t), []).append((int(a), int(c)))
    return out


def mesh_arrays(kind):
    if kind == "tri":
        v, e, b = periodic_rectangle(200)
        rng = np.random.default_rng(1)
        inner = (np.abs(v[:, 0]) < 4.99) & (np.abs(v[:, 1]) < 4.99)
        v = v.copy()
        v[inner] += 0.1 * (10.0 / 200) * rng.uniform(-1, 1, (inner.sum(), 2))
        return v, e, b
    return quad_rectangle(160, distort=0.2, seed=3)


def both(monkeypatch, make):
    monkeypatch.setenv("DGX_SETUP_ON_HOST", "1")
    host = make()
    monkeypatch.delenv("DGX_SETUP_ON_HOST")
    dev = make()
    return host, dev


@pytest.mark.parametrize("kind", ["tri", "quad"])
def test_device_connectivity_equals_host(dg, monkeypatch, kind):
    v, e, b = mesh_arrays(kind)
    assert len(e) * e.shape[1] >= 1 << 16  # the device pairing's threshold
    host, dev = both(monkeypatch, lambda: dg.DGMesh(v, e, None, dict(TAGS), edges_of(b)))
    assert np.array_equal(host.get_interior_faces(), dev.get_interior_faces())
    assert np.array_equal(host.get_boundary_face_data(), dev.get_boundary_face_data())
    for m in (host, dev):
        m.set_periodic_boundaries("Left", "Right")
        m.set_periodic_boundaries("Bottom", "Top")
    assert np.array_equal(host.get_interior_faces(), dev.get_interior_faces())
    assert len(host.get_boundary_face_data()) == 0 == len(dev.get_boundary_face_data())


def test_device_pairing_of_odd_meshes_equals_host(dg, monkeypatch):
    """Small meshes forced to the device pairing (DGX_SETUP_ON_DEVICE=1): an edge shared by three
    triangles (dgfem pairs the first two faces in element order; the third is a boundary face), a
    duplicated element, a hanging vertex and an element whose two faces meet the same neighbour."""
    V = np.array([[0.0, 0.0], [1.0, 0.0], [0.5, 1.0], [0.5, -1.0], [1.5, 0.5], [0.5, 2.0], [2.0, 2.0]])
    cases = [
        np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4]]),            # non-manifold edge (0, 1)
        np.array([[0, 1, 2], [0, 1, 2], [1, 4, 2]]),            # duplicated element
        np.array([[0, 1, 2], [1, 4, 2], [2, 4, 5], [4, 6, 5]]),  # plain fan with a hanging corner
        np.array([[0, 1, 2], [2, 1, 0]]),                        # two elements sharing all three edges
    ]
    for E in cases:
        E = np.ascontiguousarray(E, dtype=np.int32)
        monkeypatch.setenv("DGX_SETUP_ON_HOST", "1")
        host = dg.DGMesh(V, E, None, {}, {})
        monkeypatch.delenv("DGX_SETUP_ON_HOST")
        monkeypatch.setenv("DGX_SETUP_ON_DEVICE", "1")
        dev = dg.DGMesh(V, E, None, {}, {})
        monkeypatch.delenv("DGX_SETUP_ON_DEVICE")
        assert np.array_equal(host.get_interior_faces(), dev.get_interior_faces()), E
        assert np.array_equal(host.get_boundary_face_data(), dev.get_boundary_face_data()), E


@pytest.mark.parametrize("walls", [False, True])
@pytest.mark.parametrize("kind", ["tri", "quad"])
def test_device_geometry_equals_host(dg, monkeypatch, kind, walls):
    v, e, b = mesh_arrays(kind)
    m = dg.DGMesh(v, e, None, dict(TAGS), edges_of(b))
    U_inf = primitive_to_conserved([1.0, 0.4, 0.1, 1.0])
    if walls:
        for name, typ, val in (("Bottom", dg.BCTypeEuler.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]),
                               ("Right", dg.BCTypeEuler.FAR_FIELD, U_inf),
                               ("Top", dg.BCTypeEuler.SLIP_WALL, [0.0] * 4),
                               ("Left", dg.BCTypeEuler.FAR_FIELD, U_inf)):
            m.set_boundary_condition_euler(name, dg.BoundaryConditionEuler(typ, val))
    else:
        m.set_periodic_boundaries("Left", "Right")
        m.set_periodic_boundaries("Bottom", "Top")
    space = dg.DGSpace("triangle", 3, "dubiner") if kind == "tri" else dg.DGSpace("quad", 3)
    wf = dg.EulerWeakFormulation(1.4)
    h64, d64 = both(monkeypatch, lambda: dg.DGContext(m, space, wf, "fp64"))
    xq = h64.quad_points()
    assert np.array_equal(xq, d64.quad_points())
    assert torch.equal(h64.quad_points_device(), d64.quad_points_device())
    u0 = h64.project(torch.tensor(isentropic_vortex(xq, beta=4.0, xc=0.3, yc=-0.2, uinf=0.4), device="cuda"))
    assert torch.equal(u0, d64.project(torch.tensor(isentropic_vortex(xq, beta=4.0, xc=0.3, yc=-0.2, uinf=0.4),
                                                    device="cuda")))
    assert torch.equal(h64.residual(u0), d64.residual(u0))
    dt = 0.02 / h64.max_cfl(u0, 1.0)
    assert dt == 0.02 / d64.max_cfl(u0, 1.0)
    hmx, dmx = both(monkeypatch, lambda: dg.DGContext(m, space, wf, "mixed"))
    a, c = u0.clone(), u0.clone()
    hmx.rk3_step(a, dt, 3)
    dmx.rk3_step(c, dt, 3)
    torch.cuda.synchronize()
    assert torch.isfinite(a).all() and not torch.equal(a, u0)
    assert torch.equal(a, c)


@pytest.mark.parametrize("host", [True, False])
def test_degenerate_element_rejected(dg, monkeypatch, host):
    if host:
        monkeypatch.setenv("DGX_SETUP_ON_HOST", "1")
    else:
        monkeypatch.delenv("DGX_SETUP_ON_HOST", raising=False)
    v = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0], [0.0, 1.0]])
    e = np.array([[0, 1, 3], [0, 1, 2]], dtype=np.int32)  # the second triangle is flat
    m = dg.DGMesh(v, e, None, {}, {})
    with pytest.raises(dg.DGXError, match="Singular Jacobian matrix"):
        dg.DGContext(m, dg.DGSpace("triangle", 2, "dubiner"), dg.EulerWeakFormulation(1.4), "fp64")
