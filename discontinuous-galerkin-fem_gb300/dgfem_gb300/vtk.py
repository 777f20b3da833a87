"""Legacy-VTK output of DG solutions, fed from the device.

Mirrors dgfem's VTKWriter (include/dgfem/utils/vtk_writer.hpp:29-180,
src/utils/vtk_writer.cpp): each triangle is subdivided into resolution_factor^2 triangles
whose vertices are a uniform lattice of the reference triangle (each quadrilateral into
resolution_factor^2 quadrilaterals over a lattice of [-1, 1]^2); the solution is evaluated
at the lattice points (here on the GPU, dgx_eval_points) and written as an ASCII
UNSTRUCTURED_GRID with one SCALARS block per field.  The lattice order, the sub-triangle
connectivity, the field names and the number format follow dgfem's writer, so files from
either can be compared line by line.
"""

from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

import numpy as np

from . import _lib as L
from ._lib import check


def reference_subdivision(resolution_factor: int, element_type: str = "triangle") -> Tuple[np.ndarray, np.ndarray]:
    """Lattice points (xi, eta) of the reference element and the sub-cells over them
    (get_reference_subdivision_points / _connectivity, vtk_writer.cpp:325-409)."""
    r = int(resolution_factor)
    if r < 1:
        raise ValueError("resolution_factor must be at least 1")
    n1 = r + 1
    if element_type == "quad":
        pts = [(-1.0 + 2.0 * i / r, -1.0 + 2.0 * j / r) for j in range(n1) for i in range(n1)]
        quads = [(j * n1 + i, j * n1 + i + 1, (j + 1) * n1 + i + 1, (j + 1) * n1 + i)
                 for j in range(r) for i in range(r)]
        return np.array(pts, dtype=np.float64), np.array(quads, dtype=np.int64)
    if element_type != "triangle":
        raise ValueError(f"Unknown element type: {element_type}")
    pts = [(i / r, j / r) for j in range(n1) for i in range(n1 - j)]

    def idx(i, j):
        return sum(n1 - jj for jj in range(j)) + i

    tris = []
    for j in range(r):
        for i in range(r - j):
            tris.append((idx(i, j), idx(i + 1, j), idx(i, j + 1)))
            if i < r - j - 1:
                tris.append((idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)))
    return np.array(pts, dtype=np.float64), np.array(tris, dtype=np.int64)


def _points_and_cells(vertices: np.ndarray, elements: np.ndarray, r: int):
    quad = elements.shape[1] == 4
    ref, sub = reference_subdivision(r, "quad" if quad else "triangle")
    V = vertices[elements]  # (E, nv, 2)
    xi, eta = ref[:, 0], ref[:, 1]
    if quad:  # ReferenceQuad's bilinear shape functions
        N = 0.25 * np.stack([(1 - xi) * (1 - eta), (1 + xi) * (1 - eta), (1 + xi) * (1 + eta), (1 - xi) * (1 + eta)], axis=1)
    else:  # the affine map of the triangle
        N = np.stack([1.0 - xi - eta, xi, eta], axis=1)
    xy = np.einsum("pk,ekd->epd", N, V).reshape(-1, 2)
    cells = (sub[None, :, :] + (np.arange(len(elements)) * len(ref))[:, None, None]).reshape(-1, sub.shape[1])
    return ref, xy, cells


def _write(filename: str, title: str, xy: np.ndarray, cells: np.ndarray, fields: Sequence[Tuple[str, np.ndarray]]):
    with open(filename + ".vtk", "w") as f:
        f.write("# vtk DataFile Version 3.0\n" + title + "\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        f.write(f"POINTS {len(xy)} double\n")
        np.savetxt(f, xy, fmt="%.10e %.10e 0.0")
        nvc = cells.shape[1]
        f.write(f"CELLS {len(cells)} {(nvc + 1) * len(cells)}\n")
        np.savetxt(f, np.column_stack([np.full(len(cells), nvc), cells]), fmt="%d")
        f.write(f"CELL_TYPES {len(cells)}\n")
        f.write(("9\n" if nvc == 4 else "5\n") * len(cells))  # VTK_QUAD / VTK_TRIANGLE
        if fields:
            f.write(f"POINT_DATA {len(xy)}\n")
            for name, values in fields:
                f.write(f"SCALARS {name} double 1\nLOOKUP_TABLE default\n")
                np.savetxt(f, np.asarray(values, dtype=np.float64).reshape(-1, 1), fmt="%.10e")


def euler_fields(U: np.ndarray, gamma: float = 1.4):
    """dgfem's Euler output fields from conserved values U (..., 4), in its order
    (write_euler_solution, vtk_writer.cpp:115-160; gas constant 1)."""
    rho, ru, rv, E = U[..., 0], U[..., 1], U[..., 2], U[..., 3]
    u, v = ru / rho, rv / rho
    p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v))
    vel = np.sqrt(u * u + v * v)
    c = np.sqrt(gamma * p / rho)
    return [("density", rho), ("u_velocity", u), ("v_velocity", v), ("velocity_magnitude", vel),
            ("pressure", p), ("temperature", p / rho), ("mach", vel / c),
            ("rho", rho), ("rho_u", ru), ("rho_v", rv), ("E", E)]


class VTKWriter:
    """dgfem's VTKWriter entry points for the Euler path."""

    @staticmethod
    def evaluate_at_points(ctx, solution, ref_xy: np.ndarray):
        """(E, npts, 4) values of the state at reference points, evaluated on the GPU."""
        import torch
        u = solution if isinstance(solution, torch.Tensor) else torch.tensor(
            np.ascontiguousarray(solution, dtype=np.float64).reshape(ctx.shape), device="cuda")
        u = u.reshape(ctx.shape).contiguous()
        ref = np.ascontiguousarray(ref_xy, dtype=np.float64)
        out = torch.empty((ctx.n_elements, len(ref), 4), dtype=torch.float64, device=u.device)
        stream = C.c_void_p(torch.cuda.current_stream(u.device).cuda_stream)
        check(L.load().dgx_eval_points(ctx._h, len(ref), ref.ctypes.data_as(C.POINTER(C.c_double)),
                                       C.c_void_p(u.data_ptr()), C.c_void_p(out.data_ptr()), stream))
        return out

    @staticmethod
    def write_euler_solution(ctx, solution, filename: str, gamma: float = 1.4, resolution_factor: int = 3):
        """Conserved and primitive fields of an Euler state (device tensor, or host array of
        shape (E, Np, 4) / dgfem's flat (E, Np*4) frame) to `filename`.vtk."""
        ctx = getattr(ctx, "ctx", ctx)  # a solver carries its context
        ref, xy, cells = _points_and_cells(ctx.mesh.get_vertices(), ctx.mesh.get_elements(), resolution_factor)
        U = VTKWriter.evaluate_at_points(ctx, solution, ref).cpu().numpy().reshape(-1, 4)
        _write(filename, "DGFEM Euler Solution", xy, cells, euler_fields(U, gamma))

    @staticmethod
    def write_mesh(mesh, filename: str):
        """The mesh's own cells, no data (write_mesh, vtk_writer.cpp:180-192)."""
        _write(filename, "DGFEM Mesh", mesh.get_vertices(), mesh.get_elements().astype(np.int64), [])
