"""Device-fed VTK output: dgx_eval_points against an exactly represented linear field, and
the Euler file's fields at the lattice points."""

import numpy as np
import pytest

from meshes import TAGS, periodic_rectangle, quad_rectangle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    return d


def linear(xy):
    x, y = xy[..., 0], xy[..., 1]
    return np.stack([1.0 + 0.1 * x, 0.3 - 0.05 * y, 0.02 * x + 0.01 * y, 3.0 + 0.05 * y], -1)


@pytest.mark.parametrize("basis", ["monomial", "dubiner"])
@pytest.mark.parametrize("order", [1, 3])
def test_linear_field_at_lattice_points(dg, tmp_path, order, basis):
    m = dg.DGMesh.rectangle(4, 3, 0.0, 2.0, 0.0, 1.0, periodic=False)
    ctx = dg.DGContext(m, dg.DGSpace("triangle", order, basis), dg.EulerWeakFormulation(1.4), "fp64")
    u = ctx.project(torch.tensor(linear(ctx.quad_points()), device="cuda"))
    dg.VTKWriter.write_euler_solution(ctx, u, str(tmp_path / "sol"), 1.4, 3)
    text = (tmp_path / "sol.vtk").read_text().splitlines()
    npts = int(text[4].split()[1])
    assert npts == ctx.n_elements * 10
    xy = np.array([[float(a) for a in l.split()[:2]] for l in text[5:5 + npts]])
    i = text.index("SCALARS rho double 1")
    rho = np.array([float(l) for l in text[i + 2:i + 2 + npts]])
    # the file carries 11 significant digits (dgfem's scientific, precision 10)
    assert np.allclose(rho, linear(xy)[:, 0], rtol=1e-10, atol=0)
    i = text.index("SCALARS E double 1")
    E = np.array([float(l) for l in text[i + 2:i + 2 + npts]])
    assert np.allclose(E, linear(xy)[:, 3], rtol=1e-10, atol=0)


@pytest.mark.parametrize("basis", ["monomial", "dubiner"])
@pytest.mark.parametrize("order", [2, 4])
def test_eval_points_then_projection_is_identity(dg, order, basis):
    """Values at the volume quadrature points, projected back, return the coefficients:
    the evaluation uses the context's own basis."""
    v, e, b = periodic_rectangle(5)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, basis), dg.EulerWeakFormulation(1.4), "fp64")
    xq = ctx.quad_points()[0]  # physical quadrature points of element 0 -> reference coordinates
    V = pm.get_vertices()[pm.get_elements()[0]]
    J = np.column_stack([V[1] - V[0], V[2] - V[0]])
    ref = np.linalg.solve(J, (xq - V[0]).T).T
    u = torch.tensor(np.random.default_rng(4).standard_normal(ctx.shape), device="cuda")
    uq = dg.VTKWriter.evaluate_at_points(ctx, u, ref)
    back = ctx.project(uq.contiguous())
    tol = 1e-12 if basis == "dubiner" else 1e-9  # cond(M) of the monomial basis amplifies rounding
    assert float(torch.linalg.vector_norm(back - u) / torch.linalg.vector_norm(u)) <= tol


@pytest.mark.parametrize("order", [1, 3])
def test_quad_linear_field_at_lattice_points(dg, tmp_path, order):
    """On bilinear quadrilaterals a linear field lies in the tensor space Q_p (p >= 1), so the
    projection reproduces it and the sub-quad lattice carries its exact values."""
    v, e, b = quad_rectangle(4, 0.0, 2.0, 0.0, 1.0, distort=0.2, seed=order)
    m = dg.DGMesh(v, e, None, dict(TAGS), {})
    ctx = dg.DGContext(m, dg.DGSpace("quad", order), dg.EulerWeakFormulation(1.4), "fp64")
    u = ctx.project(torch.tensor(linear(ctx.quad_points()), device="cuda"))
    dg.VTKWriter.write_euler_solution(ctx, u, str(tmp_path / "qsol"), 1.4, 3)
    text = (tmp_path / "qsol.vtk").read_text().splitlines()
    npts = int(text[4].split()[1])
    assert npts == ctx.n_elements * 16
    xy = np.array([[float(a) for a in l.split()[:2]] for l in text[5:5 + npts]])
    i = text.index("SCALARS rho double 1")
    rho = np.array([float(l) for l in text[i + 2:i + 2 + npts]])
    assert np.allclose(rho, linear(xy)[:, 0], rtol=1e-10, atol=0)
    assert text[text.index(f"CELL_TYPES {ctx.n_elements * 9}") + 1] == "9"
