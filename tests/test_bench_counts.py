"""The unit counts behind bench.py's rooflines: algorithmic bytes and flops per element and RK
stage, against the figures they are defined by (FP64 state read twice and written once plus 92
bytes of geometry and connectivity; the Euler flop count 2.7 / 6.7 / 12.6 kflop at p = 2 / 3 / 4,
and the Navier-Stokes additions).  No GPU needed."""

import math
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def n_basis(p):
    return (p + 1) * (p + 2) // 2


def test_algorithmic_bytes_p3():
    assert bench.ALGO_BYTES_PER_ELEM_STAGE == 3 * n_basis(3) * 4 * 8 + 92 == 1052


def test_euler_flops_per_element_stage():
    # 2.7, 6.7 and 12.6 kflop per element and stage at p = 2, 3, 4
    got = {p: bench.flops_per_element_stage(p, False) for p in (2, 3, 4)}
    assert got == {2: 2718, 3: 6680, 4: 12570}
    for p, k in ((2, 2.7), (3, 6.7), (4, 12.6)):
        assert math.isclose(got[p] / 1000, k, abs_tol=0.05)


def test_navier_stokes_flops_add_the_viscous_terms():
    p, nq, nfq, v = 4, 16, 5, 4
    np_ = n_basis(p)
    extra = 4 * nq * np_ * v + 60 * nq + 4 * nq * np_ * v + 1.5 * 8 * nfq * np_ * v + 1.5 * nfq * 20
    assert bench.flops_per_element_stage(p, True) == bench.flops_per_element_stage(p, False) + extra == 24960


def test_flop_roofline_fraction():
    r = bench.flop_roofline(3, False, 1000, 2.0, 10.0, "fp32")
    achieved = 6680 * 1000 * 3 / 2e-3 / 1e12
    assert math.isclose(r["achieved_tflops"], achieved) and math.isclose(r["frac"], achieved / 10.0)
    assert bench.flop_roofline(3, False, 1000, None, 10.0, "fp32") is None
