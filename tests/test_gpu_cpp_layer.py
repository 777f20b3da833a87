"""The header-only C++ layer (include/dgx_dgfem.hpp) driven like dgfem drives its own
classes, from compiled C++ programs, checked against the oracle:
* tests/cpp/test_dgfem_compat.cpp: DGMesh, DGSpace, DGAssembler(mesh, weak_form),
  EulerDGSolver(mesh, gamma) and the host-state methods, triangles and quadrilaterals;
* the integration guide's C++ sample (the block after its `sample: run_vortex` marker), extracted
  verbatim: EulerDGSolver::solve with the state on the GPU, every saved frame against the oracle's
  steps."""

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, isentropic_vortex, periodic_rectangle, quad_rectangle

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
INTEGRATION_GUIDE = "INTEGRATION.md"  # the guide whose C++ sample the test compiles
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
    assert np.array_equal(load("residual_assembler.bin"), load("residual.bin"))
    assert rel(load("minv.bin"), om.apply_mass_inv(R)) <= 1e-11
    assert rel(load("rk3.bin"), om.rk3_step(ph, u, dt, 1)) <= 1e-11
    cfl, lo, hi = (float.fromhex(x) for x in (tmp_path / "monitors.txt").read_text().split())
    assert abs(cfl - om.max_cfl(1.4, u, dt)) <= 1e-12 * cfl
    rlo, rhi = om.density_range(u)
    assert abs(lo - rlo) <= 1e-12 and abs(hi - rhi) <= 1e-12


def test_integration_sample_solve(tmp_path):
    """The sample's run_vortex: 12 x 12 x 2 periodic vortex, p=3, FP64, dt = 0.02 until T_final =
    0.21 (11 steps of dgfem's while (t < T_final) loop), a frame every 4 steps and the last."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    doc = (ROOT / INTEGRATION_GUIDE).read_text()
    block = doc.split("<!-- sample: run_vortex -->", 1)[1]
    code = block.split("```cpp\n", 1)[1].split("```", 1)[0]
    (tmp_path / "integration_sample.inc").write_text(code)
    exe = tmp_path / "run_integration_sample"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(tmp_path), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "run_integration_sample.cpp"), "-o", str(exe),
                    "-L", str(LIBDIR), "-ldgx", f"-Wl,-rpath,{LIBDIR}"], check=True)
    n, order, T_final, dt, save_every = 12, 3, 0.21, 0.02, 4
    r = subprocess.run([str(exe), str(tmp_path), str(n), str(order), repr(T_final), repr(dt), str(save_every)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # dgfem's loop: the steps after which a frame is kept
    saved, t, step = [0], 0.0, 0
    while t < T_final:
        if step % save_every == 0 and step > 0:
            saved.append(step)
        t += dt
        step += 1
    if step % save_every != 0:
        saved.append(step)
    assert int((tmp_path / "frames.txt").read_text()) == len(saved)
    v, e, b = periodic_rectangle(n)
    om = O.OracleMesh(v, e, b, order=order, basis=O.MONOMIAL, periodic=PERIODIC_PAIRS)
    u0 = om.project(isentropic_vortex(om.quad_points(), beta=5.0))
    frames = np.fromfile(tmp_path / "frames.bin", dtype=np.float64).reshape(len(saved), om.ne, om.np * 4)
    for k, s_ in enumerate(saved):
        ref = om.rk3_step(O.euler(1.4), u0, dt, s_) if s_ else u0
        err = np.linalg.norm(frames[k] - ref.reshape(om.ne, -1)) / np.linalg.norm(ref)
        assert err <= 1e-10, (s_, err)
