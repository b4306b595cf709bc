"""The library against OpSparse's own kernels on the same GPU.

oracle/ref_gpu runs the reference's kernels (compiled from its sources into a cubin) in
its own host sequence.  Structure (row_ptr, col_idx) must be bit-identical; values agree
to within the reference's run-order summation error, ≤ 1e-14·Σ|a·b| (the library's values
equal the oracle's exactly).  Skipped where the reference's cubin was not built.
"""
import numpy as np
import pytest

import oracle
import opsparse_gb300 as ops
from oracle import ref_gpu
from tests.cases import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
IDS = [c[0] for c in CASES]
VALUE_TOL = 1e-14


@pytest.fixture(scope="module")
def refgpu(cuda):
    if not ref_gpu.build() or not ref_gpu.available():
        pytest.skip("the reference's GPU build is not available")
    return ref_gpu.lib()


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_matches_reference_on_gpu(cuda, refgpu, case):
    name, a, b, ncols = case
    kcols = len(b[0]) - 1
    A = ops.csr_to_device(*a, len(a[0]) - 1, kcols, dtype=cuda.float64)
    B = ops.csr_to_device(*b, kcols, ncols, dtype=cuda.float64)
    with ops.Handle() as h:
        rpt, col, val = h.spgemm(A, B).to_host()
    ap, bp = A.ptrs(), B.ptrs()
    r = ref_gpu.spgemm(len(a[0]) - 1, ap[0], ap[1], ap[2], bp[0], bp[1], bp[2])
    m = len(a[0]) - 1

    def fetch(ptr, n, typestr):
        if n == 0:
            return np.zeros(0, np.int32 if typestr == "<i4" else np.float64)
        return cuda.as_tensor(ops._DevArray(ptr, n, typestr), device="cuda").cpu().numpy()

    try:
        rr = fetch(r.rpt, m + 1, "<i4")
        rc = fetch(r.col, r.nnz, "<i4")
        rv = fetch(r.val, r.nnz, "<f8")
    finally:
        r.free()
    assert r.nnz == len(col), name
    assert np.array_equal(rr.astype(np.int64), rpt.astype(np.int64)), name
    assert np.array_equal(rc, col), name
    scale = oracle.abs_sums(*a, *b, ncols)
    err = np.abs(rv - val)
    assert np.all(err <= VALUE_TOL * scale), (name, float((err / np.maximum(scale, 1e-300)).max()))
