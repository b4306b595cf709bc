"""Golden fixtures: outputs of OpSparse's own kernels (tests/golden/make_golden.py).

CPU: the oracle reproduces the reference's C structure bit-for-bit and its values to
within rounding of the reference's run-order summation; its flop counts equal the
reference's compute_flop.  When the OpSparse sources are present, the fixtures are also
regenerated and must match.  GPU: the library reproduces the reference's structure
bit-for-bit and its values to the same bound (and the oracle's values exactly).
"""
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLDEN = sorted((Path(__file__).resolve().parent / "golden").glob("*.npz"))
IDS = [p.stem for p in GOLDEN]
# reference values are sums of rounded products in run order; the oracle folds with fma
# in ascending j.  Both are within a few ulps of sum_j |a_ij b_jk|.
VALUE_TOL = 1e-14


def load(p):
    z = np.load(p)
    a = (z["a_rpt"], z["a_col"], z["a_val"])
    b = (z["b_rpt"], z["b_col"], z["b_val"])
    return z, a, b, int(z["ncols"])


def check_against_reference(z, a, b, n, rpt, col, val):
    assert np.array_equal(np.asarray(rpt, np.int64), z["c_rpt"].astype(np.int64))
    assert np.array_equal(col, z["c_col"])
    scale = oracle.abs_sums(*a, *b, n)
    err = np.abs(np.asarray(val, np.float64) - z["c_val"])
    assert np.all(err <= VALUE_TOL * scale), float((err / np.maximum(scale, 1e-300)).max())


@pytest.mark.parametrize("path", GOLDEN, ids=IDS)
def test_oracle_matches_reference_kernels(path):
    z, a, b, n = load(path)
    rpt, col, val = oracle.spgemm(*a, *b, n)
    check_against_reference(z, a, b, n, rpt, col, val)
    tot, rf = oracle.flop(a[0], a[1], b[0])
    assert tot == int(z["total_flop"]) and np.array_equal(rf, z["row_flop"].astype(np.int64))


def test_fixtures_cover_reference_paths():
    """Between them the fixtures reach every symbolic and numeric bin of the reference,
    including its global-hash fallback."""
    sym = np.zeros(8, np.int64)
    num = np.zeros(8, np.int64)
    fallback = 0
    for p in GOLDEN:
        z = np.load(p)
        sym += z["bins_symbolic"]
        num += z["bins_numeric"]
        fallback += int(z["global_fallback_rows"])
    assert fallback > 0
    assert np.all(num > 0), num
    assert np.all(sym > 0), sym


def test_regenerated_fixtures_match():
    ref = pytest.importorskip("oracle.ref")
    if not ref.available():
        pytest.skip("OpSparse sources not present")
    for p in GOLDEN[:4]:
        z, a, b, n = load(p)
        rpt, col, val, info = ref.spgemm(*a, *b, n)
        assert np.array_equal(rpt, z["c_rpt"]) and np.array_equal(col, z["c_col"])
        assert np.array_equal(val, z["c_val"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=IDS)
def test_library_matches_reference_kernels(cuda, path):
    import opsparse_gb300 as ops

    z, a, b, n = load(path)
    A = ops.csr_to_device(*a, len(a[0]) - 1, len(b[0]) - 1)
    B = ops.csr_to_device(*b, len(b[0]) - 1, n)
    with ops.Handle() as h:
        rpt, col, val = h.spgemm(A, B).to_host()
    check_against_reference(z, a, b, n, rpt, col, val)
    orpt, ocol, oval = oracle.spgemm(*a, *b, n)
    assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))
