"""The FP32 reciprocal and square root of the mixed path (hardware approximations,
csrc/dg_physics.cuh) stay within 2 ulp of the exact values over 2^26 random normal inputs
and keep the special values (tests/cpp/test_fast_math.cu, compiled here with nvcc for
sm_103a)."""

import re
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_rcp_sqrt_error_bounds(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "test_fast_math"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I",
                    str(ROOT / "discontinuous-galerkin-fem_gb300" / "csrc"), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "test_fast_math.cu"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"rcp max ulp ([0-9.]+), sqrt max ulp ([0-9.]+), special values wrong (\d+)", r.stdout)
    assert m and float(m.group(1)) <= 2.0 and float(m.group(2)) <= 2.0 and int(m.group(3)) == 0
