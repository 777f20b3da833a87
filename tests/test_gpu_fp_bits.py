"""The integer-pipe FP32 <-> FP64 conversions used by the stage-3 epilogues
(csrc/fp_bits.cuh) agree bit for bit with the hardware conversions on 2^28 values of every
class (tests/cpp/test_fp_bits.cu, compiled here with nvcc for sm_103a)."""

import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_conversions_match_hardware(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "test_fp_bits"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I",
                    str(ROOT / "discontinuous-galerkin-fem_gb300" / "csrc"),
                    str(ROOT / "tests" / "cpp" / "test_fp_bits.cu"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0, binary64->binary32 mismatches 0" in r.stdout
