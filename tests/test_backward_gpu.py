"""Fixed-pattern backward of C = A*B (loss = sum(W .* C), dC = W).

FP64: dA and dB are bit-identical to the oracle (dA folded over k in B's row order, dB
over ascending i, one FMA per term), with and without the stored product->position map.
They also match the dense reference gradient dA = (W B^T) .* mask(A), dB = (A^T W) .*
mask(B) and FP64 finite differences (torch.autograd.gradcheck on a 2,000-row power-law
instance).  FP32: within 1e-5 relative of the FP64 oracle on the same inputs.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
import opsparse_gb300 as ops
from opsparse_gb300 import gen
from opsparse_gb300.autograd import FixedPatternSpGEMM

pytestmark = pytest.mark.gpu


def make(n, deg, seed):
    a = gen.powerlaw_square(n, deg, 2.2, seed=seed)
    b = gen.transpose_pattern(a[0], a[1], n, seed=seed)
    return a, b


def run(cuda, a, b, n, dtype, map_budget=None):
    A = ops.csr_to_device(*a, n, n, dtype=dtype)
    B = ops.csr_to_device(*b, n, n, dtype=dtype)
    h = ops.Handle()
    if map_budget is not None:
        ops.capi.check(h.lib.ops_handle_set_map_budget(h.h, map_budget))
    op = FixedPatternSpGEMM(A, B, h)
    c_val = op.forward_values(A.val, B.val)
    rng = np.random.default_rng(3)
    w = cuda.as_tensor(rng.standard_normal(op.nnz)).to(dtype).cuda()
    da, db = op.backward_values(A.val, B.val, w)
    info = op.plan_info()
    res = (op.c_rpt.cpu().numpy(), op.c_col.cpu().numpy(), c_val.cpu().numpy(), w.cpu().numpy(),
           da.cpu().numpy(), db.cpu().numpy(), info)
    h.close()
    return res


@pytest.mark.parametrize("map_mode", [True, False], ids=["map", "search"])
def test_f64_bit_exact_vs_oracle(cuda, map_mode):
    n = 3000
    a, b = make(n, 12, 11)
    crpt, ccol, cval, w, da, db, info = run(cuda, a, b, n, cuda.float64, None if map_mode else 0)
    assert info[1] == map_mode
    orpt, ocol, oval = oracle.spgemm(*a, *b, n)
    assert np.array_equal(crpt.astype(np.int64), orpt) and np.array_equal(ccol, ocol)
    oda, odb = oracle.backward(*a, *b, n, orpt, ocol, w)
    assert np.array_equal(da.view(np.uint64), oda.view(np.uint64))
    assert np.array_equal(db.view(np.uint64), odb.view(np.uint64))


def test_dense_reference_gradient(cuda):
    n = 2000
    a, b = make(n, 16, 5)
    crpt, ccol, cval, w, da, db, _ = run(cuda, a, b, n, cuda.float64)
    A = sp.csr_matrix((a[2], a[1], a[0]), shape=(n, n)).toarray()
    B = sp.csr_matrix((b[2], b[1], b[0]), shape=(n, n)).toarray()
    W = sp.csr_matrix((w, ccol, crpt), shape=(n, n)).toarray()
    dA = W @ B.T
    dB = A.T @ W
    ra = np.repeat(np.arange(n), np.diff(a[0]))
    rb = np.repeat(np.arange(n), np.diff(b[0]))
    assert np.allclose(da, dA[ra, a[1]], rtol=1e-10, atol=1e-10)
    assert np.allclose(db, dB[rb, b[1]], rtol=1e-10, atol=1e-10)


def test_f32_within_tolerance(cuda):
    n = 3000
    a, b = make(n, 12, 13)
    a32 = (a[0], a[1], a[2].astype(np.float32))
    b32 = (b[0], b[1], b[2].astype(np.float32))
    crpt, ccol, cval, w, da, db, _ = run(cuda, a32, b32, n, cuda.float32)
    a64 = (a[0], a[1], a32[2].astype(np.float64))
    b64 = (b[0], b[1], b32[2].astype(np.float64))
    orpt, ocol, _ = oracle.spgemm(*a64, *b64, n)
    oda, odb = oracle.backward(*a64, *b64, n, orpt, ocol, w.astype(np.float64))
    for got, ref in ((da, oda), (db, odb)):
        nz = ref != 0
        rel = np.abs(got[nz].astype(np.float64) - ref[nz]) / np.abs(ref[nz])
        assert rel.max() <= 1e-5


def test_gradcheck_finite_differences(cuda):
    torch = cuda
    n = 2000
    a, b = make(n, 4, 17)
    A = ops.csr_to_device(*a, n, n)
    B = ops.csr_to_device(*b, n, n)
    op = FixedPatternSpGEMM(A, B)
    av = A.val.clone().requires_grad_(True)
    bv = B.val.clone().requires_grad_(True)
    rng = np.random.default_rng(9)
    w = torch.as_tensor(rng.standard_normal(op.nnz)).cuda()

    def loss(x, y):
        return (op(x, y) * w).sum()

    assert torch.autograd.gradcheck(loss, (av, bv), eps=1e-6, atol=1e-7, rtol=1e-6, fast_mode=True)
    # explicit central differences on a sample of entries (the loss is bilinear, so the
    # difference quotient is exact up to rounding)
    la = loss(av, bv)
    la.backward()
    for t, g in ((av, av.grad), (bv, bv.grad)):
        idx = rng.choice(t.numel(), 25, replace=False)
        for i in idx:
            with torch.no_grad():
                e = torch.zeros_like(t)
                e[i] = 1e-3
                fd = (loss(av + (e if t is av else 0), bv + (e if t is bv else 0)) -
                      loss(av - (e if t is av else 0), bv - (e if t is bv else 0))) / 2e-3
            assert abs(float(fd) - float(g[i])) <= 1e-8 * max(1.0, abs(float(g[i])))


def test_reuse_plan_new_values(cuda):
    torch = cuda
    n = 2500
    a, b = make(n, 10, 21)
    A = ops.csr_to_device(*a, n, n)
    B = ops.csr_to_device(*b, n, n)
    op = FixedPatternSpGEMM(A, B)
    rng = np.random.default_rng(1)
    for _ in range(2):
        av = torch.as_tensor(rng.standard_normal(len(a[1]))).cuda()
        bv = torch.as_tensor(rng.standard_normal(len(b[1]))).cuda()
        w = torch.as_tensor(rng.standard_normal(op.nnz)).cuda()
        op.forward_values(av, bv)
        da, db = op.backward_values(av, bv, w)
        oda, odb = oracle.backward(a[0], a[1], av.cpu().numpy(), b[0], b[1], bv.cpu().numpy(), n,
                                   op.c_rpt.cpu().numpy().astype(np.int64), op.c_col.cpu().numpy(), w.cpu().numpy())
        assert np.array_equal(da.cpu().numpy().view(np.uint64), oda.view(np.uint64))
        assert np.array_equal(db.cpu().numpy().view(np.uint64), odb.view(np.uint64))
