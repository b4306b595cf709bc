"""Host logic of bench.py on the CPU: the parity report that sets the measured GPU result
against the oracle's result on the same inputs (the bench's CPU baseline computes it)."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


@pytest.fixture(scope="module")
def ref():
    """The oracle's OpenMP product of a 2-D Laplacian pattern (24 x 24 grid) carrying
    uniform random values."""
    import oracle
    from opsparse_gb300 import gen

    oracle.build()
    rpt, col, _ = gen.laplacian2d(24)
    val = np.random.default_rng(5).uniform(-1.0, 1.0, col.size)
    return oracle.omp_spgemm(rpt, col, val, rpt, col, val)


def test_identical_result(ref):
    rep = bench.parity_report(ref, ref, "f64")
    assert rep["structure_identical"] and rep["values_bit_identical"] and rep["zeros_exact"]
    assert rep["max_abs_err"] == 0.0 and rep["max_rel_err"] == 0.0 and rep["within_tolerance"]
    assert rep["entries"] == ref[1].size


def test_fp32_result(ref):
    """An FP32 result (here the oracle's rounded to float) is measured against the FP64
    oracle: its error is the rounding's, inside the 1e-5 relative tolerance."""
    g = (ref[0].astype(np.int32), ref[1], ref[2].astype(np.float32))
    rep = bench.parity_report(g, ref, "f32")
    assert rep["structure_identical"] and "values_bit_identical" not in rep
    assert 0.0 < rep["max_rel_err"] <= 2.0 ** -24 and rep["within_tolerance"]


def test_value_and_structure_changes_are_reported(ref):
    v = ref[2].copy()
    v[7] *= 1.0 + 1e-9
    rep = bench.parity_report((ref[0], ref[1], v), ref, "f64")
    assert rep["structure_identical"] and not rep["values_bit_identical"]
    assert rep["max_rel_err"] == pytest.approx(1e-9, rel=1e-3) and not rep["within_tolerance"]
    c = ref[1].copy()
    c[3] += 1
    rep = bench.parity_report((ref[0], c, ref[2]), ref, "f64")
    assert rep["structure_identical"] is False and "max_rel_err" not in rep
    short = (ref[0], ref[1][:-1], ref[2][:-1])
    assert bench.parity_report(short, ref, "f64")["structure_identical"] is False


def test_zero_entries_must_stay_zero(ref):
    o = (ref[0], ref[1], ref[2].copy())
    o[2][0] = 0.0  # an entry the oracle folds to zero
    g = (ref[0], ref[1], o[2].copy())
    g[2][0] = 1e-30
    rep = bench.parity_report(g, o, "f64")
    assert rep["zeros_exact"] is False and not rep["within_tolerance"]


def test_fp32_cancellation_is_judged_against_the_terms(ref):
    """An FP32 entry whose terms cancel may differ from the FP64 oracle by far more than
    1e-5 of its own size; it is judged relative to 2^-24 * sum|a*b| of its terms."""
    o = (ref[0], ref[1], ref[2].copy())
    o[2][5] = 3e-9                       # the oracle's value of a cancelling entry
    scale = np.abs(o[2]) + 1.0           # sum of |a*b| of each entry's terms
    g = (ref[0].astype(np.int32), ref[1], o[2].astype(np.float32))
    g[2][5] = np.float32(3e-9 + 2e-13)  # 7e-5 of the entry, 3e-6 of its terms' resolution
    rep = bench.parity_report(g, o, "f32", scale_fn=lambda: scale)
    assert rep["max_rel_err"] > 1e-5                   # the plain relative bound would fail it
    assert rep["max_rel_err_scaled"] <= 1e-5 and rep["within_tolerance"]
    g[2][5] = np.float32(1.0)                          # a real error stays an error
    rep = bench.parity_report(g, o, "f32", scale_fn=lambda: scale)
    assert not rep["within_tolerance"]
