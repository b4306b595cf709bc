"""CPU tests of the oracle: known sizes of the benchmark configurations, agreement with
an independent implementation (scipy.sparse), FP32/FP64 consistency, the OpenMP
baseline, the backward formulas and edge cases."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from opsparse_gb300 import gen


def scipy_product(rpt, col, val, brpt, bcol, bval, shape_a, shape_b):
    A = sp.csr_matrix((val, col, rpt), shape=shape_a)
    B = sp.csr_matrix((bval, bcol, brpt), shape=shape_b)
    C = (A @ B).tocsr()
    C.sort_indices()
    return C


def test_laplacian_known_sizes():
    rpt, col, val = gen.laplacian2d(128)
    assert len(rpt) - 1 == 16384 and len(col) == 81408
    tot, _ = oracle.flop(rpt, col, rpt)
    assert tot == 405000
    crpt, ccol, cval = oracle.spgemm(rpt, col, val, rpt, col, val, 16384)
    assert len(ccol) == 210436
    assert np.diff(crpt).max() == 13
    C = scipy_product(rpt, col, val, rpt, col, val, (16384, 16384), (16384, 16384))
    assert np.array_equal(C.indptr, crpt) and np.array_equal(C.indices, ccol)
    assert np.array_equal(C.data, cval)  # integer-valued: every summation order is exact


def test_stencil27_known_sizes():
    rpt, col, val = gen.stencil27(80)
    assert len(rpt) - 1 == 512000 and len(col) == 13481272
    tot, _ = oracle.flop(rpt, col, rpt)
    assert tot == 357911000
    crpt, nnz = oracle.symbolic(rpt, col, rpt, col, 512000)
    assert nnz == 61162984
    assert np.diff(crpt).max() == 125


@pytest.mark.parametrize("case", ["stencil27", "web", "er", "powerlaw"])
def test_matches_scipy(case):
    if case == "stencil27":
        a = gen.stencil27(12)
        n = 12 ** 3
    elif case == "web":
        a = gen.web_powerlaw(20000, lmax=800)
        n = 20000
    elif case == "er":
        a = gen.erdos_renyi(3000, 9.0)
        n = 3000
    else:
        a = gen.powerlaw_square(4000, 16, 2.2)
        n = 4000
    rpt, col, val = a
    crpt, ccol, cval = oracle.spgemm(rpt, col, val, rpt, col, val, n)
    C = scipy_product(rpt, col, val, rpt, col, val, (n, n), (n, n))
    # scipy drops entries that cancel to exactly 0.0; random values make that measure-zero
    assert np.array_equal(C.indptr, crpt)
    assert np.array_equal(C.indices, ccol)
    scale = oracle.abs_sums(rpt, col, val, rpt, col, val, n)
    assert np.all(np.abs(C.data - cval) <= 1e-13 * scale)


def test_rectangular_and_empty_rows():
    rng = np.random.default_rng(1)
    A = sp.random(300, 200, density=0.02, random_state=rng, format="csr")
    B = sp.random(200, 500, density=0.03, random_state=rng, format="csr")
    A.sort_indices()
    B.sort_indices()
    crpt, ccol, cval = oracle.spgemm(A.indptr, A.indices, A.data, B.indptr, B.indices, B.data, 500)
    C = (A @ B).tocsr()
    C.sort_indices()
    assert np.array_equal(C.indptr, crpt) and np.array_equal(C.indices, ccol)
    assert np.allclose(C.data, cval, rtol=1e-13, atol=0)
    assert (np.diff(A.indptr) == 0).any()  # the case covers empty rows


def test_empty_matrices():
    rpt = np.zeros(1, dtype=np.int32)
    col = np.zeros(0, dtype=np.int32)
    val = np.zeros(0)
    crpt, ccol, cval = oracle.spgemm(rpt, col, val, rpt, col, val, 0)
    assert len(crpt) == 1 and len(ccol) == 0
    rpt = np.zeros(11, dtype=np.int32)
    crpt, ccol, cval = oracle.spgemm(rpt, col, val, rpt, col, val, 10)
    assert np.all(crpt == 0) and len(ccol) == 0


def test_f32_within_tolerance_of_f64():
    rpt, col, val = gen.stencil27(14)
    n = 14 ** 3
    v32 = val.astype(np.float32)
    r64 = oracle.spgemm(rpt, col, v32.astype(np.float64), rpt, col, v32.astype(np.float64), n)
    r32 = oracle.spgemm(rpt, col, v32, rpt, col, v32, n, dtype=np.float32)
    assert np.array_equal(r64[1], r32[1])
    rel = np.abs(r32[2].astype(np.float64) - r64[2]) / np.maximum(np.abs(r64[2]), 1e-300)
    assert rel.max() <= 1e-5


def test_omp_baseline_bit_identical():
    rpt, col, val = gen.web_powerlaw(30000, lmax=1500)
    ref = oracle.spgemm(rpt, col, val, rpt, col, val, 30000)
    got = oracle.omp_spgemm(rpt, col, val, rpt, col, val)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)


def test_flop_matches_numpy():
    rpt, col, val = gen.powerlaw_square(5000, 16, 2.2)
    tot, rf = oracle.flop(rpt, col, rpt)
    ref = gen.row_flop(rpt, col, rpt)
    assert tot == ref.sum() and np.array_equal(rf, ref)


def test_backward_matches_dense_gradient():
    rng = np.random.default_rng(7)
    A = sp.random(60, 40, density=0.15, random_state=rng, format="csr")
    B = sp.random(40, 50, density=0.15, random_state=rng, format="csr")
    A.sort_indices()
    B.sort_indices()
    crpt, ccol, cval = oracle.spgemm(A.indptr, A.indices, A.data, B.indptr, B.indices, B.data, 50)
    W = rng.standard_normal(len(ccol))
    da, db = oracle.backward(A.indptr, A.indices, A.data, B.indptr, B.indices, B.data, 50, crpt, ccol, W)
    Wd = sp.csr_matrix((W, ccol, crpt), shape=(60, 50)).toarray()
    dA = Wd @ B.toarray().T
    dB = A.toarray().T @ Wd
    rows_a = np.repeat(np.arange(60), np.diff(A.indptr))
    rows_b = np.repeat(np.arange(40), np.diff(B.indptr))
    assert np.allclose(da, dA[rows_a, A.indices], rtol=1e-12, atol=1e-12)
    assert np.allclose(db, dB[rows_b, B.indices], rtol=1e-12, atol=1e-12)


def _long_entry_case(m=5000, seed=31):
    """One A row of m entries, all 1.0, over B rows that each hold column 0 and one other
    column: C[0, 0] has m contributions (folded in blocks), the others one each."""
    rng = np.random.default_rng(seed)
    arpt = np.array([0, m], dtype=np.int32)
    acol = np.arange(m, dtype=np.int32)
    aval = np.ones(m)
    brpt = np.arange(0, 2 * m + 1, 2, dtype=np.int32)
    bcol = np.stack([np.zeros(m, dtype=np.int32), 1 + np.arange(m, dtype=np.int32)], axis=1).ravel()
    bval = rng.standard_normal(2 * m)
    return (arpt, acol, aval), (brpt, bcol, bval), m + 1


def test_oracle_blocked_long_entry_f64():
    """Entries of more than 2,560 contributions fold in 32 consecutive blocks of ceil(m/32),
    each from +0.0 in ascending j, the block sums added in order (with a = 1.0 every fma is
    an exact addition, so Python floats restate it)."""
    a, b, n = _long_entry_case()
    _, col, val = oracle.spgemm(*a, *b, n)
    terms = [float(x) for x in b[2][0::2]]  # B values of column 0, ascending j
    c = (len(terms) + 31) // 32
    parts = []
    for k in range(32):
        s = 0.0
        for t in terms[k * c:(k + 1) * c]:
            s += t
        parts.append(s)
    total = parts[0]
    for p in parts[1:]:
        total += p
    seq = 0.0
    for t in terms:
        seq += t
    assert col[0] == 0
    assert np.float64(val[0]).view(np.uint64) == np.float64(total).view(np.uint64)
    assert total != seq  # the case does tell the two orders apart
    # entries of one contribution are the product itself
    assert np.array_equal(val[1:], b[2][1::2])


def test_oracle_blocked_long_entry_f32():
    """The same rule for FP32 Dot2 states: blocks folded with the Dot2 step, block states
    combined by TwoSum of the sums plus the sum of the compensations."""
    a, b, n = _long_entry_case()
    f = np.float32
    a32 = (a[0], a[1], a[2].astype(f))
    b32 = (b[0], b[1], b[2].astype(f))
    _, col, val = oracle.spgemm(*a32, *b32, n, dtype=np.float32)

    def step(st, h):  # a = 1: TwoProduct is exact (r = 0)
        s0, c0 = st
        s = f(s0 + h)
        z = f(s - s0)
        q = f(f(s0 - f(s - z)) + f(h - z))
        return s, f(c0 + f(q + f(0.0)))

    def merge(u, v):
        s = f(u[0] + v[0])
        z = f(s - u[0])
        q = f(f(u[0] - f(s - z)) + f(v[0] - z))
        return s, f(f(u[1] + v[1]) + q)

    terms = list(b32[2][0::2])
    c = (len(terms) + 31) // 32
    parts = []
    for k in range(32):
        st = (f(0.0), f(0.0))
        for t in terms[k * c:(k + 1) * c]:
            st = step(st, t)
        parts.append(st)
    tot = parts[0]
    for p in parts[1:]:
        tot = merge(tot, p)
    want = f(tot[0] + tot[1])
    assert col[0] == 0
    assert np.float32(val[0]).view(np.uint32) == want.view(np.uint32)
