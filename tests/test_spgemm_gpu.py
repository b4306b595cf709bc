"""GPU parity tests: the CUDA library through its C ABI against the CPU oracle.

FP64: row_ptr, col_idx and values are bit-identical to the oracle (both fold each
entry's contributions in ascending j with one FMA each).  FP32: structure bit-identical;
values bit-identical to the oracle's FP32 (Dot2) evaluation and within 1e-5 relative of
the FP64 oracle on the same (float) inputs.
"""
import numpy as np
import pytest

import oracle
import opsparse_gb300 as ops
from tests.cases import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
IDS = [c[0] for c in CASES]
F32_REL_TOL = 1e-5
F64_REL_TOL = 1e-12


@pytest.fixture(scope="module")
def handle(cuda):
    h = ops.Handle(timing=True)
    yield h
    h.close()


def to_dev(cuda, m, ncols, dtype):
    rpt, col, val = m
    return ops.csr_to_device(rpt, col, val, len(rpt) - 1, ncols, dtype=dtype)


def run_case(cuda, handle, case, dtype, oneshot=False):
    name, a, b, ncols = case
    kcols = len(b[0]) - 1
    A = to_dev(cuda, a, kcols, dtype)
    B = to_dev(cuda, b, ncols, dtype)
    C = handle.spgemm_oneshot(A, B) if oneshot else handle.spgemm(A, B)
    cuda.cuda.synchronize()
    return C.to_host()


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_f64_bit_exact(cuda, handle, case):
    name, a, b, ncols = case
    rpt, col, val = run_case(cuda, handle, case, cuda.float64)
    orpt, ocol, oval = oracle.spgemm(*a, *b, ncols)
    assert np.array_equal(rpt.astype(np.int64), orpt), name
    assert np.array_equal(col, ocol), name
    assert np.array_equal(val.view(np.uint64), oval.view(np.uint64)), name
    t = handle.timings()
    assert t["nnz"] == len(ocol)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_f32(cuda, handle, case):
    name, a, b, ncols = case
    a32 = (a[0], a[1], a[2].astype(np.float32))
    b32 = (b[0], b[1], b[2].astype(np.float32))
    rpt, col, val = run_case(cuda, handle, (name, a32, b32, ncols), cuda.float32)
    orpt, ocol, oval32 = oracle.spgemm(*a32, *b32, ncols, dtype=np.float32)
    assert np.array_equal(rpt.astype(np.int64), orpt) and np.array_equal(col, ocol)
    assert np.array_equal(val.view(np.uint32), oval32.view(np.uint32))
    _, _, oval64 = oracle.spgemm(a[0], a[1], a32[2].astype(np.float64), b[0], b[1], b32[2].astype(np.float64), ncols)
    nz = oval64 != 0
    rel = np.abs(val[nz].astype(np.float64) - oval64[nz]) / np.abs(oval64[nz])
    assert (rel.max() if rel.size else 0.0) <= F32_REL_TOL
    assert np.all(val[~nz] == 0)


@pytest.mark.parametrize("one_pass", [2, 0], ids=["one_pass", "two_pass"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_oneshot_against_oracle(cuda, case, dtype, one_pass):
    """ops_spgemm (values known before counting, so all rows but the heaviest may be
    computed in one pass through the staging area) is bit-identical to the oracle either
    way; mode 2 stages even these small inputs."""
    name, a, b, ncols = case
    npd = np.float64 if dtype == "f64" else np.float32
    a = (a[0], a[1], a[2].astype(npd))
    b = (b[0], b[1], b[2].astype(npd))
    with ops.Handle() as h:
        h.set_one_pass(one_pass)
        for _ in range(2):  # the second call reuses the staging area
            rpt, col, val = run_case(cuda, h, (name, a, b, ncols), getattr(cuda, "float64" if dtype == "f64" else
                                                                           "float32"), oneshot=True)
            orpt, ocol, oval = oracle.spgemm(*a, *b, ncols, dtype=npd)
            assert np.array_equal(rpt.astype(np.int64), orpt), name
            assert np.array_equal(col, ocol), name
            ut = np.uint64 if dtype == "f64" else np.uint32
            assert np.array_equal(val.view(ut), oval.view(ut)), name


@pytest.mark.parametrize("case", CASES[:4] + CASES[6:7], ids=IDS[:4] + IDS[6:7])
def test_oneshot_matches_two_phase(cuda, handle, case):
    r1 = run_case(cuda, handle, case, cuda.float64, oneshot=True)
    r2 = run_case(cuda, handle, case, cuda.float64, oneshot=False)
    for x, y in zip(r1, r2):
        assert np.array_equal(x, y)


def test_class_coverage(cuda, handle):
    """The case set reaches every row class."""
    seen = np.zeros(7, dtype=np.int64)
    for case in CASES:
        run_case(cuda, handle, case, cuda.float64)
        seen += np.array(handle.timings()["class_rows"])
    assert np.all(seen > 0), seen


def test_subclass_coverage(cuda, handle):
    """The case set reaches every sub-kernel of the re-binned classes (E1 numeric: warp
    sort, warp hash, expand/sort/compress; E2: mid and large shape)."""
    seen = {}
    for case in CASES:
        run_case(cuda, handle, case, cuda.float64)
        for k, v in handle.subclass_rows().items():
            seen[k] = seen.get(k, 0) + v
    # the rank-path counters have their own rows (tests/test_rank_gpu.py)
    assert all(v > 0 for k, v in seen.items() if k not in ("d_dense", "rank", "rank_refold", "rank_sorted")), seen


@pytest.mark.parametrize("oneshot", [False, True], ids=["two_phase", "one_pass"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_d_rows_dense_fallback(cuda, dtype, oneshot):
    """With a scratch budget too small for the whole-GPU sort, the D rows take the
    CTA-per-row dense kernel; both give the oracle's bits.  Through ops_spgemm in one-pass
    mode the D rows are computed while counting when the sort fits, and left to two passes
    (the dense kernel) when it does not."""
    case = next(c for c in CASES if c[0] == "dense_row")
    name, a, b, ncols = case
    for budget, path in ((None, "d_sort"), (1 << 20, "d_dense")):
        h = ops.Handle()
        if oneshot:
            h.set_one_pass(2)
        if budget:
            h.set_dense_budget(budget)
        if dtype == "f64":
            rpt, col, val = run_case(cuda, h, case, cuda.float64, oneshot=oneshot)
            orpt, ocol, oval = oracle.spgemm(*a, *b, ncols)
            assert np.array_equal(val.view(np.uint64), oval.view(np.uint64)), path
        else:
            a32 = (a[0], a[1], a[2].astype(np.float32))
            b32 = (b[0], b[1], b[2].astype(np.float32))
            rpt, col, val = run_case(cuda, h, (name, a32, b32, ncols), cuda.float32, oneshot=oneshot)
            orpt, ocol, oval = oracle.spgemm(*a32, *b32, ncols, dtype=np.float32)
            assert np.array_equal(val.view(np.uint32), oval.view(np.uint32)), path
        assert np.array_equal(rpt.astype(np.int64), orpt) and np.array_equal(col, ocol), path
        sub = h.subclass_rows()
        assert sub[path] > 0, (path, sub)
        h.close()


def _stretch_columns(case, factor=600):
    """Same products with B's columns spread over factor*N columns by the strictly
    increasing map c -> factor*c + c % 7; C is the original C under the same map."""
    name, a, b, ncols = case
    f = lambda c: (c.astype(np.int64) * factor + c % 7).astype(np.int32)
    return (name + "_wide", a, (b[0], f(b[1]), b[2]), int(f(np.array([ncols - 1]))[0]) + 1), f


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_wide_columns(cuda, handle, dtype):
    """More than 2^25 columns: the warp-sort kernels switch to 64-bit (column, product)
    keys.  Results are the oracle's under the column map."""
    case, f = _stretch_columns(CASES[2])
    assert case[3] > (1 << 25)
    name, a, b, ncols = case
    orig = CASES[2]
    if dtype == "f64":
        rpt, col, val = run_case(cuda, handle, case, cuda.float64)
        orpt, ocol, oval = oracle.spgemm(*orig[1], *orig[2], orig[3])
        assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))
    else:
        a32 = (a[0], a[1], a[2].astype(np.float32))
        b32 = (b[0], b[1], b[2].astype(np.float32))
        rpt, col, val = run_case(cuda, handle, (name, a32, b32, ncols), cuda.float32)
        orpt, ocol, oval = oracle.spgemm(a[0], a[1], a32[2], orig[2][0], orig[2][1], b32[2], orig[3],
                                         dtype=np.float32)
        assert np.array_equal(val.view(np.uint32), oval.view(np.uint32))
    assert np.array_equal(rpt.astype(np.int64), orpt)
    assert np.array_equal(col, f(ocol))
    assert handle.subclass_rows()["e1_sort"] > 0


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_wide_columns_one_pass(cuda, dtype):
    """The one-pass kernels with 64-bit (column, product) keys: ops_spgemm on more than
    2^25 columns, staged at any size, gives the oracle's bits under the column map."""
    case, f = _stretch_columns(CASES[2])
    name, a, b, ncols = case
    orig = CASES[2]
    npd = np.float64 if dtype == "f64" else np.float32
    a = (a[0], a[1], a[2].astype(npd))
    b = (b[0], b[1], b[2].astype(npd))
    with ops.Handle() as h:
        h.set_one_pass(2)
        rpt, col, val = run_case(cuda, h, (name, a, b, ncols), getattr(cuda, "float64" if dtype == "f64" else
                                                                       "float32"), oneshot=True)
        orpt, ocol, oval = oracle.spgemm(orig[1][0], orig[1][1], a[2], orig[2][0], orig[2][1], b[2], orig[3],
                                         dtype=npd)
        ut = np.uint64 if dtype == "f64" else np.uint32
        assert np.array_equal(rpt.astype(np.int64), orpt)
        assert np.array_equal(col, f(ocol))
        assert np.array_equal(val.view(ut), oval.view(ut))
        assert h.subclass_rows()["e1_sort"] > 0


def test_many_d_rows_wide(cuda, handle):
    """1,100 rows of 20,000 products each (D rows) over 11M columns: the D-row sort key
    (row, column) needs more than 32 bits.  Results are the oracle's under the column map."""
    rng = np.random.default_rng(21)
    import scipy.sparse as sp
    n = 20000
    A = sp.random(1100, n, density=200 / n, random_state=rng, format="csr")
    B = sp.random(n, n, density=100 / n, random_state=rng, format="csr")
    from tests.cases import _csr
    base = ("many_d", _csr(A), _csr(B), n)
    case, f = _stretch_columns(base, factor=550)
    rpt, col, val = run_case(cuda, handle, case, cuda.float64)
    orpt, ocol, oval = oracle.spgemm(*base[1], *base[2], n)
    assert np.array_equal(rpt.astype(np.int64), orpt)
    assert np.array_equal(col, f(ocol))
    assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))
    assert handle.subclass_rows()["d_sort"] > 1024
    with ops.Handle() as h:  # the same D rows computed while counting (one pass)
        h.set_one_pass(2)
        rpt, col, val = run_case(cuda, h, case, cuda.float64, oneshot=True)
        assert np.array_equal(rpt.astype(np.int64), orpt)
        assert np.array_equal(col, f(ocol))
        assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))
        assert h.subclass_rows()["d_sort"] > 1024


def test_repeat_and_resize(cuda, handle):
    """Workspace reuse across calls of different sizes gives identical results."""
    big = CASES[2]
    small = CASES[0]
    first = run_case(cuda, handle, big, cuda.float64)
    run_case(cuda, handle, small, cuda.float64)
    again = run_case(cuda, handle, big, cuda.float64)
    for x, y in zip(first, again):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("budget", [None, 1 << 16], ids=["staged", "over_budget"])
def test_one_pass_resize_and_budget(cuda, budget):
    """One-pass calls on one handle across sizes and value types (the staging area grows
    and is reused), and with a staging budget too small for the inputs (two passes
    instead): the oracle's bits every time."""
    with ops.Handle() as h:
        h.set_one_pass(2)
        if budget:
            h.set_stage_budget(budget)
        for case, dtype in ((CASES[0], "f64"), (CASES[2], "f64"), (CASES[4], "f32"), (CASES[0], "f32"),
                            (CASES[2], "f64")):
            name, a, b, ncols = case
            npd = np.float64 if dtype == "f64" else np.float32
            a = (a[0], a[1], a[2].astype(npd))
            b = (b[0], b[1], b[2].astype(npd))
            rpt, col, val = run_case(cuda, h, (name, a, b, ncols),
                                     cuda.float64 if dtype == "f64" else cuda.float32, oneshot=True)
            orpt, ocol, oval = oracle.spgemm(*a, *b, ncols, dtype=npd)
            ut = np.uint64 if dtype == "f64" else np.uint32
            assert np.array_equal(rpt.astype(np.int64), orpt) and np.array_equal(col, ocol), name
            assert np.array_equal(val.view(ut), oval.view(ut)), name


def test_empty_inputs(cuda, handle):
    z = (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    C = handle.spgemm(ops.csr_to_device(*z, 0, 0), ops.csr_to_device(*z, 0, 0))
    assert C.nnz == 0 and C.rpt.numel() == 1
    e = (np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0))
    A = ops.csr_to_device(*e, 5, 7)
    B = ops.csr_to_device(np.zeros(8, np.int32), np.zeros(0, np.int32), np.zeros(0), 7, 9)
    C = handle.spgemm(A, B)
    assert C.nnz == 0 and np.all(C.rpt.cpu().numpy() == 0)


@pytest.mark.parametrize("case", [CASES[2], CASES[4], CASES[6]], ids=[IDS[2], IDS[4], IDS[6]])
def test_numeric_after_one_pass_call(cuda, case):
    """The plan an ops_spgemm call leaves on the handle (its counting phase computed most
    rows in one pass) serves ops_spgemm_numeric with new values: every class's two-pass
    numeric runs on the lists that call made, and gives the oracle's bits."""
    name, a, b, ncols = case
    kcols = len(b[0]) - 1
    with ops.Handle() as h:
        h.set_one_pass(2)
        A = to_dev(cuda, a, kcols, cuda.float64)
        B = to_dev(cuda, b, ncols, cuda.float64)
        C = h.spgemm_oneshot(A, B)
        a2 = (a[0], a[1], a[2] * 1.5 - 0.25)
        A2 = to_dev(cuda, a2, kcols, cuda.float64)
        A2 = ops.CsrMatrix(A.rows, A.cols, A.rpt, A.col, A2.val)  # same structure arrays as the plan
        c_col, c_val = h.numeric(A2, B, C.rpt, C.nnz)
        cuda.cuda.synchronize()
        orpt, ocol, oval = oracle.spgemm(*a2, *b, ncols)
        assert np.array_equal(C.rpt.cpu().numpy().astype(np.int64), orpt)
        assert np.array_equal(c_col.cpu().numpy(), ocol)
        assert np.array_equal(c_val.cpu().numpy().view(np.uint64), oval.view(np.uint64))


def test_empty_inputs_one_pass(cuda):
    """ops_spgemm on empty and structurally empty inputs with one pass forced on."""
    with ops.Handle() as h:
        h.set_one_pass(2)
        z = (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
        C = h.spgemm_oneshot(ops.csr_to_device(*z, 0, 0), ops.csr_to_device(*z, 0, 0))
        assert C.nnz == 0 and C.rpt.numel() == 1
        A = ops.csr_to_device(np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0), 5, 7)
        B = ops.csr_to_device(np.zeros(8, np.int32), np.zeros(0, np.int32), np.zeros(0), 7, 9)
        C = h.spgemm_oneshot(A, B)
        assert C.nnz == 0 and np.all(C.rpt.cpu().numpy() == 0)


def test_invalid_column_is_reported(cuda, handle):
    rpt = np.array([0, 2, 3], np.int32)
    col = np.array([0, 5, 1], np.int32)  # 5 >= cols (3)
    A = ops.csr_to_device(rpt, col, np.ones(3), 2, 3)
    with pytest.raises(ops.OpsError) as ei:
        handle.symbolic(A, A)
    assert ei.value.status == ops.capi.OPS_INVALID_CSR


@pytest.mark.parametrize("one_pass", [2, 0], ids=["one_pass", "two_pass"])
def test_invalid_b_column_is_reported(cuda, one_pass):
    """A column of B outside [0, cols) under a row of 9-16 products (the R16 class) is
    reported by ops_spgemm as invalid CSR, whether the row is computed while counting or
    in two passes."""
    A = ops.csr_to_device(np.array([0, 3], np.int32), np.array([0, 1, 2], np.int32), np.ones(3), 1, 3)
    brpt = np.array([0, 4, 8, 12], np.int32)
    bcol = np.array([0, 1, 2, 3, 0, 1, 2, 9, 0, 1, 2, 3], np.int32)  # 9 >= cols (4)
    B = ops.csr_to_device(brpt, bcol, np.ones(12), 3, 4)
    with ops.Handle() as h:
        h.set_one_pass(one_pass)
        with pytest.raises(ops.OpsError) as ei:
            h.spgemm_oneshot(A, B)
        assert ei.value.status == ops.capi.OPS_INVALID_CSR


def test_numeric_without_symbolic_is_rejected(cuda):
    h = ops.Handle()
    a = CASES[0][1]
    A = to_dev(cuda, a, 16384, cuda.float64)
    c_rpt = cuda.zeros(16385, dtype=cuda.int32, device="cuda")
    with pytest.raises(ops.OpsError) as ei:
        h.numeric(A, A, c_rpt, 10)
    assert ei.value.status == ops.capi.OPS_NOT_SUPPORTED
    h.close()


def test_device_flop_count(cuda):
    for name, a, b, ncols in CASES[:6]:
        A = to_dev(cuda, a, len(b[0]) - 1, cuda.float64)
        B = to_dev(cuda, b, ncols, cuda.float64)
        assert ops.flop(A, B) == oracle.flop(a[0], a[1], b[0])[0]


def test_timings_reported(cuda, handle):
    run_case(cuda, handle, CASES[2], cuda.float64, oneshot=True)
    t = handle.timings()
    assert t["total"] > 0 and t["symbolic"] > 0 and t["numeric"] > 0
    assert t["flop"] == oracle.flop(CASES[2][1][0], CASES[2][1][1], CASES[2][2][0])[0]


def _long_run_case(seed=31):
    """One row of 20,000 A entries over B rows that all hold the same 12 columns (plus a
    few others): 12 output entries of 20,000 products each, far beyond a warp's batch, and
    a D row (more than 13,312 products) for the whole-GPU sort and its long-run fold."""
    import scipy.sparse as sp
    from tests.cases import _csr
    rng = np.random.default_rng(seed)
    n = 20000
    A = sp.csr_matrix((rng.standard_normal(n), (np.zeros(n, dtype=np.int64), np.arange(n))), shape=(2, n))
    rows = np.repeat(np.arange(n), 12)
    cols = np.tile(np.arange(0, 120, 10), n)
    extra_r = rng.integers(0, n, 3000)
    extra_c = rng.integers(0, 5000, 3000)
    B = sp.csr_matrix((rng.standard_normal(rows.size + extra_r.size),
                       (np.concatenate([rows, extra_r]), np.concatenate([cols, extra_c]))), shape=(n, 5000))
    return "long_runs", _csr(A), _csr(B), 5000


@pytest.mark.parametrize("oneshot", [False, True], ids=["two_phase", "one_pass"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_long_runs(cuda, dtype, oneshot):
    """Output entries folding 20,000 products each (the D rows' long-run fold): the
    oracle's bits, two-phase and in one pass."""
    name, a, b, ncols = _long_run_case()
    npd = np.float64 if dtype == "f64" else np.float32
    a = (a[0], a[1], a[2].astype(npd))
    b = (b[0], b[1], b[2].astype(npd))
    with ops.Handle() as h:
        h.set_one_pass(2)
        rpt, col, val = run_case(cuda, h, (name, a, b, ncols), getattr(cuda, "float64" if dtype == "f64" else
                                                                       "float32"), oneshot=oneshot)
        orpt, ocol, oval = oracle.spgemm(*a, *b, ncols, dtype=npd)
        ut = np.uint64 if dtype == "f64" else np.uint32
        assert np.array_equal(rpt.astype(np.int64), orpt) and np.array_equal(col, ocol)
        assert np.array_equal(val.view(ut), oval.view(ut))
        assert h.subclass_rows()["d_sort"] == 1


def _banded(n, half, seed):
    """n x n banded CSR: row r holds columns r - half .. r + half within [0, n)."""
    rng = np.random.default_rng(seed)
    lens = np.array([min(n, r + half + 1) - max(0, r - half) for r in range(n)])
    rpt = np.zeros(n + 1, np.int32)
    rpt[1:] = np.cumsum(lens)
    col = np.concatenate([np.arange(max(0, r - half), min(n, r + half + 1)) for r in range(n)]).astype(np.int32)
    return rpt, col, rng.uniform(-1.0, 1.0, col.size)


def _window_operands(cuda, shape, n=3001):
    a = _banded(n, 13 if shape == "short" else 19, 11)  # 27 or 39 A entries per row
    b = _banded(n, 12, 12)  # B rows of 25 columns: 675 or 975 products, E1 rows read row-wise
    return a, b


@pytest.mark.parametrize("shape", ["short", "long"])
@pytest.mark.parametrize("misaligned", [False, True], ids=["bcol16", "bcol_offset4"])
@pytest.mark.parametrize("one_pass", [2, 0], ids=["one_pass", "two_pass"])
def test_window_rows(cuda, shape, misaligned, one_pass):
    """Banded A·B: E1 rows with long B rows whose products fall in a window of columns are
    counted over a bitmap.  With at most 32 A entries ("short") a lane per entry reads its
    B row as 16-byte quads, or column by column where B's column array is not 16-byte
    aligned and for the last B rows (nnz(B) is not a multiple of 4); with more ("long") the
    window is read first.  The oracle's bits, two-phase and in one pass."""
    n = 3001
    a, b = _window_operands(cuda, shape, n)
    assert b[1].size % 4 != 0
    A = ops.csr_to_device(*a, n, n, dtype=cuda.float64)
    B = ops.csr_to_device(*b, n, n, dtype=cuda.float64)
    if misaligned:
        buf = cuda.zeros(b[1].size + 1, dtype=cuda.int32, device=B.col.device)
        buf[1:] = B.col
        B = ops.CsrMatrix(B.rows, B.cols, B.rpt, buf[1:], B.val)
        assert B.col.data_ptr() % 16 != 0
    orpt, ocol, oval = oracle.spgemm(*a, *b, n)
    with ops.Handle() as h:
        h.set_one_pass(one_pass)
        rpt, col, val = h.spgemm_oneshot(A, B).to_host()
    assert np.array_equal(rpt.astype(np.int64), orpt) and np.array_equal(col, ocol)
    assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))


@pytest.mark.parametrize("shape", ["short", "long"])
@pytest.mark.parametrize("one_pass", [2, 0], ids=["one_pass", "two_pass"])
def test_invalid_b_column_in_window_row(cuda, shape, one_pass):
    """A column of B at or past cols as the last (largest) column of a B row that window
    rows read: reported as invalid CSR by the counting of those rows."""
    n = 400
    a, b = _window_operands(cuda, shape, n)
    bcol = b[1].copy()
    bcol[b[0][201] - 1] = n + 7  # B row 200 stays sorted
    A = ops.csr_to_device(*a, n, n, dtype=cuda.float64)
    B = ops.csr_to_device(b[0], bcol, b[2], n, n, dtype=cuda.float64)
    with ops.Handle() as h:
        h.set_one_pass(one_pass)
        with pytest.raises(ops.OpsError) as ei:
            h.spgemm_oneshot(A, B)
        assert ei.value.status == ops.capi.OPS_INVALID_CSR
