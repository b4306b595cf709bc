"""The C++ drop-in API (include/opsparse/**, libopsparse.so) run on the GPU.

opsparse_gb300/_build/facade_selftest drives the drop-in the way OpSparse's benchmark
drivers do (benchmarks/opsparse_profile.cu, opsparse_reg.cu): CSR loaded from MatrixMarket
files (CSR::construct, following src/opsparse/core_ds/csr.cu:187-352), H2D, opsparse_spgemm
/ _reg / _safe, SpgemmTimings::print, D2H, C.release() of the cudaMalloc'ed output, and
opsparse_spgemm_backward.  The files are written here from seeded inputs in every format the
reader accepts (general, symmetric and skew-symmetric; real, integer and pattern); the
program writes back the matrices it loaded and the product, which are compared bit for bit
with the expected expansion and with the oracle's product and gradients.
"""
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from opsparse_gb300 import build as B
from opsparse_gb300 import gen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def selftest(cuda):
    B.build()
    oracle.build()
    return B.selftest_path()


def _write_mtx(path, rows, cols, entries, field="real", symmetry="general"):
    """entries: (i, j, v) 0-based; written 1-based with 17 significant digits."""
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {symmetry}\n% written by the drop-in test\n")
        f.write(f"{rows} {cols} {len(entries)}\n")
        for i, j, v in entries:
            if field == "pattern":
                f.write(f"{i + 1} {j + 1}\n")
            elif field == "integer":
                f.write(f"{i + 1} {j + 1} {int(v)}\n")
            else:
                f.write(f"{i + 1} {j + 1} {float(v):.17g}\n")


def _entries(rpt, col, val):
    rows = np.repeat(np.arange(len(rpt) - 1), np.diff(rpt))
    return list(zip(rows.tolist(), np.asarray(col).tolist(), np.asarray(val).tolist()))


def _csr(m):
    m = sp.csr_matrix(m)
    m.sort_indices()
    return m.indptr.astype(np.int32), m.indices.astype(np.int32), m.data.astype(np.float64)


def _read_csr(path):
    raw = open(path, "rb").read()
    M, N, nnz = np.frombuffer(raw[:24], dtype=np.int64)
    o = 24
    rpt = np.frombuffer(raw[o:o + 4 * (M + 1)], dtype=np.int32)
    o += 4 * (M + 1)
    col = np.frombuffer(raw[o:o + 4 * nnz], dtype=np.int32)
    o += 4 * nnz
    val = np.frombuffer(raw[o:o + 8 * nnz], dtype=np.float64)
    return int(M), int(N), rpt, col, val


def _run(selftest, args):
    res = subprocess.run([str(selftest), *map(str, args)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and "FACADE_SELFTEST OK" in res.stdout, res.stdout[-4000:] + res.stderr[-2000:]
    return res.stdout


def _same(x, y):
    return np.array_equal(np.asarray(x).astype(np.int64), np.asarray(y).astype(np.int64))


def _check_loaded(out, name, expect, shape):
    M, N, rpt, col, val = _read_csr(out / name)
    assert (M, N) == shape
    assert _same(rpt, expect[0]) and _same(col, expect[1])
    assert np.array_equal(val.view(np.uint64), np.asarray(expect[2], dtype=np.float64).view(np.uint64))


def _check_product(out, a, b, ncols):
    M, N, rpt, col, val = _read_csr(out / "C.bin")
    orpt, ocol, oval = oracle.spgemm(*a, *b, ncols)
    assert _same(rpt, orpt) and _same(col, ocol)
    assert np.array_equal(val.view(np.uint64), oval.view(np.uint64)), "C values differ from the oracle"
    return orpt, ocol, oval


def _check_log(log):
    for line in ("time(ms):", "sum_total", "perf(Gflops):", "STATUS,ok", "STATUS,nonsquare", "PERF,reg,",
                 "MEMORY,free_before"):
        assert line in log, line


def test_selfcheck(selftest):
    """The program's own check: a symmetric Laplacian file, every entry point, the
    reference's tolerant operator==."""
    log = _run(selftest, [])
    _check_log(log)


def test_general_real_web_graph_with_backward(selftest, tmp_path):
    """A 60,000-row web-like power-law graph in general real format: C = A*A through every
    entry point bit-identical to the oracle, then the C++ backward with seeded dC, its dA and
    dB bit-identical to the oracle's backward (twice, the second on the kept plan)."""
    a = gen.web_powerlaw(60000, lmax=2000)
    n = len(a[0]) - 1
    _write_mtx(tmp_path / "A.mtx", n, n, _entries(*a))
    crpt, ccol, _ = oracle.spgemm(*a, *a, n)
    dc = np.random.default_rng(17).standard_normal(len(ccol))
    dc.tofile(tmp_path / "dC.bin")
    log = _run(selftest, ["run", tmp_path / "A.mtx", "-", tmp_path, tmp_path / "dC.bin"])
    _check_log(log)
    _check_loaded(tmp_path, "A.bin", a, (n, n))
    _check_product(tmp_path, a, a, n)
    da, db = oracle.backward(*a, *a, n, crpt, ccol, dc)
    ga = np.fromfile(tmp_path / "dA.bin", dtype=np.float64)
    gb = np.fromfile(tmp_path / "dB.bin", dtype=np.float64)
    assert np.array_equal(ga.view(np.uint64), da.view(np.uint64)), "dA differs from the oracle"
    assert np.array_equal(gb.view(np.uint64), db.view(np.uint64)), "dB differs from the oracle"


def test_symmetric_lower_triangle(selftest, tmp_path):
    """A symmetric file holding only the lower triangle (the 2-D Laplacian, 64 x 64 grid) is
    expanded to the full matrix."""
    full = gen.laplacian2d(64)
    n = len(full[0]) - 1
    lower = [(i, j, v) for i, j, v in _entries(*full) if j <= i]
    _write_mtx(tmp_path / "A.mtx", n, n, lower, symmetry="symmetric")
    _run(selftest, ["run", tmp_path / "A.mtx", "-", tmp_path])
    _check_loaded(tmp_path, "A.bin", full, (n, n))
    _check_product(tmp_path, full, full, n)


def test_skew_symmetric(selftest, tmp_path):
    """A skew-symmetric file (strict lower triangle) expands to A with A^T = -A."""
    rng = np.random.default_rng(23)
    n = 3000
    low = sp.tril(sp.random(n, n, density=6 / n, random_state=rng, format="csr"), k=-1).tocsr()
    full = _csr(low - low.T)
    _write_mtx(tmp_path / "A.mtx", n, n, _entries(*_csr(low)), symmetry="skew-symmetric")
    _run(selftest, ["run", tmp_path / "A.mtx", "-", tmp_path])
    _check_loaded(tmp_path, "A.bin", full, (n, n))
    _check_product(tmp_path, full, full, n)


def test_pattern_and_integer_rectangular(selftest, tmp_path):
    """A is a pattern file (values 1.0), B an integer file; A is 700 x 300 and B 300 x 900,
    so C = A*B is rectangular."""
    rng = np.random.default_rng(29)
    a = _csr(sp.random(700, 300, density=0.03, random_state=rng, format="csr"))
    b = _csr(sp.random(300, 900, density=0.05, random_state=rng, format="csr"))
    a1 = (a[0], a[1], np.ones_like(a[2]))
    bi = (b[0], b[1], np.floor(b[2] * 20.0) - 7.0)
    _write_mtx(tmp_path / "A.mtx", 700, 300, _entries(*a1), field="pattern")
    _write_mtx(tmp_path / "B.mtx", 300, 900, _entries(*bi), field="integer")
    _run(selftest, ["run", tmp_path / "A.mtx", tmp_path / "B.mtx", tmp_path])
    _check_loaded(tmp_path, "A.bin", a1, (700, 300))
    _check_loaded(tmp_path, "B.bin", bi, (300, 900))
    _check_product(tmp_path, a1, bi, 900)
