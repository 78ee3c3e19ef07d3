"""bench.py's host-side bookkeeping (no GPU): the algorithmic byte counts the
roofline fractions divide by, and the figures it reads from the committed
ncu summaries."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class Dom:
    nx = ny = 512


def test_engine_bytes_per_launch(bench):
    """10 RK4 steps x (6 state + 27 field accesses) per cell: 156 B x 512^2
    in the mixed form."""
    assert bench.algorithmic_bytes("engine", Dom, 1, 1) == 10 * 156 * 512 * 512
    assert bench.algorithmic_bytes("engine", Dom, 0, 1) == 10 * (6 * 8 + 27 * 8) * 512 * 512


def test_stage_stencil_bytes(bench):
    """The mixed true-stage kernel sequence's stencil: the pair of x (8 B),
    the previous stage output at three stages of four (3 B on average), dxw
    (4 B), D, q0, 1/(2 eta) (12 B), the mask (1 B) and f (4 B); the FP64
    state form reads y and w_ref as doubles and the fields in FP64."""
    n = 512 * 512
    assert bench.algorithmic_bytes("flexure", Dom, 1, 1) == 32 * n
    assert bench.algorithmic_bytes("flexure", Dom, 0, 1) == (8 + 8 + 24 + 1 + 8) * n
    assert bench.algorithmic_bytes("flexure", Dom, 1, 0) == (8 + 12 + 1 + 4) * n
    assert bench.algorithmic_bytes("rk_final", Dom, 1, 1) == 68 * n
    assert bench.algorithmic_bytes("rk_stage", Dom, 1, 1) == 28 * n


def test_committed_profile_figures(bench):
    """The engine's DRAM traffic and its L2 view come from the committed
    capture summary; a kernel with no capture gives None."""
    assert bench.ncu_traffic("engine") == pytest.approx(10_770_000)
    l2 = bench.l2_line("engine", 900.0)
    assert l2["bytes_per_launch"] == pytest.approx(1_355_964_032)
    assert l2["achieved_gbs"] == pytest.approx(1_355_964_032 / 900e-6 / 1e9)
    assert 0 < l2["frac_of_l2_peak_ncu"] < 1
    assert bench.ncu_value("traffic_per_launch", "no_such_kernel") is None
    assert bench.l2_line("no_such_kernel", 900.0) is None
