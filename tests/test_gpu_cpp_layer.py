"""The header-only C++ layer (include/dgx_dgfem.hpp) driven like dgfem drives its own
classes, from a compiled C++ program, checked against the oracle."""

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, isentropic_vortex, periodic_rectangle, quad_rectangle

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
LIBDIR = ROOT / "discontinuous-galerkin-fem_gb300"


@pytest.mark.parametrize("element_type", ["triangle", "quad"])
def test_cpp_layer_matches_oracle(tmp_path, element_type):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    exe = tmp_path / "test_dgfem_compat"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "test_dgfem_compat.cpp"), "-o", str(exe),
                    "-L", str(LIBDIR), "-ldgx", f"-Wl,-rpath,{LIBDIR}"], check=True)
    order = 3
    quad = element_type == "quad"
    v, e, b = quad_rectangle(8, distort=0.2) if quad else periodic_rectangle(10)
    basis = O.LEGENDRE if quad else O.DUBINER
    om = O.OracleMesh(v, e, b, order=order, basis=basis, periodic=PERIODIC_PAIRS)
    u = om.project(isentropic_vortex(om.quad_points(), beta=5.0, xc=0.4))
    dt = 0.05 / om.max_cfl(1.4, u, 1.0)
    v.astype(np.float64).tofile(tmp_path / "vertices.bin")
    e.astype(np.int32).tofile(tmp_path / "elements.bin")
    b.astype(np.int32).tofile(tmp_path / "bedges.bin")
    u.astype(np.float64).tofile(tmp_path / "state.bin")
    np.array([order, dt, e.shape[1], basis], dtype=np.float64).tofile(tmp_path / "params.bin")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def load(name):
        return np.fromfile(tmp_path / name, dtype=np.float64).reshape(u.shape)

    def rel(a, ref):
        return np.linalg.norm(a - ref) / np.linalg.norm(ref)

    ph = O.euler(1.4)
    R = om.residual(ph, u)
    assert rel(load("residual.bin"), R) <= 1e-12
    assert rel(load("minv.bin"), om.apply_mass_inv(R)) <= 1e-11
    assert rel(load("rk3.bin"), om.rk3_step(ph, u, dt, 1)) <= 1e-11
    cfl, lo, hi = (float.fromhex(x) for x in (tmp_path / "monitors.txt").read_text().split())
    assert abs(cfl - om.max_cfl(1.4, u, dt)) <= 1e-12 * cfl
    rlo, rhi = om.density_range(u)
    assert abs(lo - rlo) <= 1e-12 and abs(hi - rhi) <= 1e-12
