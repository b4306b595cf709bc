"""Batched SpGEMM: every C_b of a batch of uneven problems equals the single-call result
bit-for-bit (FP64 and FP32) and the oracle; repeated graph replays after changing the
input values give the new products; a segment limit splits big batches."""
import numpy as np
import pytest

import oracle
import opsparse_gb300 as ops
from opsparse_gb300 import gen

pytestmark = pytest.mark.gpu


def make_batch(count, seed, lo=64, hi=4096):
    rng = np.random.default_rng(seed)
    out = []
    for b in range(count):
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        d = rng.uniform(4, 32)
        a = gen.erdos_renyi(n, d, seed=seed * 1000 + 2 * b)
        bb = gen.erdos_renyi(n, d, seed=seed * 1000 + 2 * b + 1)
        out.append((n, a, bb))
    return out


@pytest.mark.parametrize("dtype_name", ["f64", "f32"])
def test_batch_matches_single_calls(cuda, dtype_name):
    torch = cuda
    dt = torch.float64 if dtype_name == "f64" else torch.float32
    probs = make_batch(48, 7)
    h = ops.Handle()
    pairs = [(ops.csr_to_device(*a, n, n, dtype=dt), ops.csr_to_device(*b, n, n, dtype=dt)) for n, a, b in probs]
    batch = ops.Batch(h, pairs)
    for use_graph in (True, True, False):
        batch.execute(use_graph)
        batch.check()
    single = ops.Handle()
    for i, (n, a, b) in enumerate(probs):
        rpt, col, val = batch.result(i)
        s = single.spgemm(*pairs[i]).to_host()
        assert np.array_equal(rpt, s[0]) and np.array_equal(col, s[1])
        assert np.array_equal(val.view(np.uint8), s[2].view(np.uint8))
        if dtype_name == "f64" and i % 8 == 0:
            o = oracle.spgemm(*a, *b, n)
            assert np.array_equal(col, o[1]) and np.array_equal(val.view(np.uint64), o[2].view(np.uint64))
    batch.close()


def test_graph_replay_sees_new_values(cuda):
    torch = cuda
    probs = make_batch(16, 3)
    h = ops.Handle()
    pairs = [(ops.csr_to_device(*a, n, n), ops.csr_to_device(*b, n, n)) for n, a, b in probs]
    batch = ops.Batch(h, pairs)
    batch.execute(True)
    rng = np.random.default_rng(5)
    for A, B in pairs:  # new values in the same arrays
        A.val.copy_(torch.as_tensor(rng.standard_normal(A.nnz)))
        B.val.copy_(torch.as_tensor(rng.standard_normal(B.nnz)))
    batch.execute(True)
    batch.check()
    for i, (n, a, b) in enumerate(probs):
        A, B = pairs[i]
        o = oracle.spgemm(a[0], a[1], A.val.cpu().numpy(), b[0], b[1], B.val.cpu().numpy(), n)
        rpt, col, val = batch.result(i)
        assert np.array_equal(val.view(np.uint64), o[2].view(np.uint64))
    batch.close()


def test_info(cuda):
    probs = make_batch(8, 11)
    h = ops.Handle()
    pairs = [(ops.csr_to_device(*a, n, n), ops.csr_to_device(*b, n, n)) for n, a, b in probs]
    batch = ops.Batch(h, pairs)
    seg, flop, nnz = batch.info()
    assert seg >= 1
    assert flop == sum(oracle.flop(a[0], a[1], b[0])[0] for n, a, b in probs)
    assert nnz == sum(len(oracle.spgemm(*a, *b, n)[1]) for n, a, b in probs)
    batch.close()


def test_repeated_batches_reuse_pool_and_segment_handles(cuda):
    """Batches created one after another on one handle take the released batch's pool
    memory and segment handles, with plain calls on the same handle in between: every C_b
    still equals the single-call result bit-for-bit, whatever the previous batch's sizes."""
    h = ops.Handle()
    single = ops.Handle()
    for k, (seed, count, hi) in enumerate(((21, 24, 4096), (22, 40, 16384), (21, 24, 4096), (23, 6, 256))):
        probs = make_batch(count, seed, hi=hi)
        pairs = [(ops.csr_to_device(*a, n, n), ops.csr_to_device(*b, n, n)) for n, a, b in probs]
        batch = ops.Batch(h, pairs)
        batch.execute(k % 2 == 0)
        batch.check()
        for i in range(count):
            rpt, col, val = batch.result(i)
            s = single.spgemm(*pairs[i]).to_host()
            assert np.array_equal(rpt, s[0]) and np.array_equal(col, s[1])
            assert np.array_equal(val.view(np.uint64), s[2].view(np.uint64))
        batch.close()
        s = single.spgemm(*pairs[0]).to_host()
        c = h.spgemm_oneshot(*pairs[0]).to_host()
        assert np.array_equal(c[1], s[1]) and np.array_equal(c[2].view(np.uint64), s[2].view(np.uint64))
