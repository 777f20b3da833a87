"""The VTK writer's host side: dgfem's reference-triangle lattice and sub-triangles
(src/utils/vtk_writer.cpp:325-409), the legacy-VTK layout and number format, and the
mesh-only file (no GPU)."""

import numpy as np
import pytest

from meshes import TAGS, periodic_rectangle, quad_rectangle


@pytest.fixture(scope="module")
def dg():
    import dgfem_gb300 as d
    return d


def test_reference_lattice_matches_dgfem_order(dg):
    from dgfem_gb300.vtk import reference_subdivision
    pts, tris = reference_subdivision(2)
    assert np.allclose(pts, [(0, 0), (0.5, 0), (1, 0), (0, 0.5), (0.5, 0.5), (0, 1)])
    assert tris.tolist() == [[0, 1, 3], [1, 4, 3], [1, 2, 4], [3, 4, 5]]
    for r in (1, 3, 5):
        pts, tris = reference_subdivision(r)
        assert len(pts) == (r + 1) * (r + 2) // 2 and len(tris) == r * r
        # every sub-triangle counter-clockwise with area 1/(2 r^2)
        a = pts[tris]
        area = 0.5 * ((a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1]) -
                      (a[:, 2, 0] - a[:, 0, 0]) * (a[:, 1, 1] - a[:, 0, 1]))
        assert np.allclose(area, 0.5 / r ** 2)


def test_mesh_file_layout(dg, tmp_path):
    v, e, b = periodic_rectangle(3)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    m = dg.DGMesh(v, e, None, dict(TAGS), edges)
    dg.VTKWriter.write_mesh(m, str(tmp_path / "mesh"))
    lines = (tmp_path / "mesh.vtk").read_text().splitlines()
    assert lines[:4] == ["# vtk DataFile Version 3.0", "DGFEM Mesh", "ASCII", "DATASET UNSTRUCTURED_GRID"]
    assert lines[4] == f"POINTS {len(v)} double"
    assert lines[5] == f"{v[0, 0]:.10e} {v[0, 1]:.10e} 0.0"
    k = 5 + len(v)
    assert lines[k] == f"CELLS {len(e)} {4 * len(e)}"
    assert lines[k + 1] == "3 " + " ".join(str(x) for x in e[0])
    assert lines[k + 1 + len(e)] == f"CELL_TYPES {len(e)}"
    assert set(lines[k + 2 + len(e):]) == {"5"}


def test_euler_fields_order_and_values(dg):
    from dgfem_gb300.vtk import euler_fields
    U = np.array([[2.0, 1.0, -0.5, 5.0]])
    f = dict(euler_fields(U, 1.4))
    assert [n for n, _ in euler_fields(U)] == ["density", "u_velocity", "v_velocity", "velocity_magnitude",
                                               "pressure", "temperature", "mach", "rho", "rho_u", "rho_v", "E"]
    p = 0.4 * (5.0 - 0.5 * 2.0 * (0.25 + 0.0625))
    assert np.isclose(f["pressure"][0], p) and np.isclose(f["temperature"][0], p / 2.0)
    assert np.isclose(f["mach"][0], np.sqrt(0.3125) / np.sqrt(1.4 * p / 2.0))


def test_quad_lattice_and_mesh_file(dg, tmp_path):
    """[-1, 1]^2 lattice with j outer, i inner and counter-clockwise sub-quads
    (vtk_writer.cpp:340-347, 394-405); VTK_QUAD = 9 cells (:475-483)."""
    from dgfem_gb300.vtk import reference_subdivision
    pts, quads = reference_subdivision(2, "quad")
    assert np.allclose(pts, [(x, y) for y in (-1, 0, 1) for x in (-1, 0, 1)])
    assert quads.tolist() == [[0, 1, 4, 3], [1, 2, 5, 4], [3, 4, 7, 6], [4, 5, 8, 7]]
    with pytest.raises(ValueError):
        reference_subdivision(2, "hexagon")
    v, e, b = quad_rectangle(3, distort=0.2)
    m = dg.DGMesh(v, e, None, dict(TAGS), {})
    dg.VTKWriter.write_mesh(m, str(tmp_path / "qmesh"))
    lines = (tmp_path / "qmesh.vtk").read_text().splitlines()
    k = 5 + len(v)
    assert lines[k] == f"CELLS {len(e)} {5 * len(e)}"
    assert lines[k + 1] == "4 " + " ".join(str(x) for x in e[0])
    assert set(lines[k + 2 + len(e):]) == {"9"}
