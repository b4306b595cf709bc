"""Batched SpGEMM: every C_b of a batch of uneven problems equals the single-call result
bit-for-bit (FP64 and FP32) and the oracle, through the persistent kernels (one setup
kernel, then one kernel per row-size queue and phase over every problem's rows) and
through the per-segment pipeline; a batch with a row beyond the persistent kernels' queues
falls back to the per-segment pipeline; repeated graph replays after changing the input
values give the new products."""
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


MODES = {"persistent": dict(batch_persistent=1), "persistent_warp128": dict(batch_persistent=1, batch_warp_max=128),
         "segments": dict(batch_persistent=0)}


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("dtype_name", ["f64", "f32"])
def test_batch_matches_single_calls(cuda, dtype_name, mode):
    torch = cuda
    dt = torch.float64 if dtype_name == "f64" else torch.float32
    probs = make_batch(48, 7)
    h = ops.Handle()
    h.set_tuning(**MODES[mode])
    pairs = [(ops.csr_to_device(*a, n, n, dtype=dt), ops.csr_to_device(*b, n, n, dtype=dt)) for n, a, b in probs]
    batch = ops.Batch(h, pairs)
    persistent, warp_rows, cta_rows = batch.queues()
    assert persistent == (mode != "segments")
    if persistent:
        assert warp_rows > 0 and cta_rows > 0  # this batch uses both kinds of queue
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


@pytest.mark.parametrize("mode", ["persistent", "segments"])
def test_graph_replay_sees_new_values(cuda, mode):
    torch = cuda
    probs = make_batch(16, 3)
    h = ops.Handle()
    h.set_tuning(**MODES[mode])
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


def test_rows_beyond_the_queues_take_the_segment_pipeline(cuda):
    """A problem with a row of more than 4,096 products (beyond the persistent kernels'
    queues) in an otherwise small batch: the batch runs the per-segment pipeline and every
    C_b still equals the single-call result and the oracle."""
    from tests.cases import dense_row_case

    probs = make_batch(6, 13)
    _, a, b, ncols = dense_row_case()
    h = ops.Handle()
    pairs = [(ops.csr_to_device(*x, n, n), ops.csr_to_device(*y, n, n)) for n, x, y in probs]
    pairs.append((ops.csr_to_device(*a, len(a[0]) - 1, len(b[0]) - 1), ops.csr_to_device(*b, len(b[0]) - 1, ncols)))
    batch = ops.Batch(h, pairs)
    assert batch.queues()[0] is False
    batch.execute(True)
    batch.check()
    single = ops.Handle()
    for i in range(len(pairs)):
        rpt, col, val = batch.result(i)
        s = single.spgemm(*pairs[i]).to_host()
        assert np.array_equal(rpt, s[0]) and np.array_equal(col, s[1])
        assert np.array_equal(val.view(np.uint64), s[2].view(np.uint64))
    o = oracle.spgemm(*a, *b, ncols)
    assert np.array_equal(batch.result(len(pairs) - 1)[2].view(np.uint64), o[2].view(np.uint64))
    batch.close()


def test_tuning_record_round_trip(cuda):
    """ops_handle_set_tuning / get_tuning keep every field; out-of-range values are refused."""
    h = ops.Handle()
    t = h.get_tuning()
    assert t["batch_persistent"] == 1 and t["hash_slots"] == 4 and t["batch_warp_max"] == 512
    h.set_tuning(thresholds=[8, 16, 32, 64, 512, 4096], hash_slots=2, batch_persistent=0, batch_warp_max=128)
    assert h.get_tuning() == {"thresholds": [8, 16, 32, 64, 512, 4096], "hash_slots": 2, "batch_persistent": 0,
                              "batch_warp_max": 128}
    for bad in (dict(hash_slots=3), dict(batch_warp_max=1024), dict(batch_warp_max=64), dict(batch_persistent=2)):
        with pytest.raises(ops.OpsError):
            h.set_tuning(**bad)
    h.close()


@pytest.mark.parametrize("slots", [2, 4])
def test_hash_slots_give_the_same_product(cuda, slots):
    """The warp-hash numeric table at 2 or 4 slots per output entry: the same bits."""
    from tests.cases import small_cases

    case = next(c for c in small_cases() if c[0] == "web60k")
    _, a, b, ncols = case
    h = ops.Handle()
    h.set_tuning(hash_slots=slots)
    A = ops.csr_to_device(*a, len(a[0]) - 1, len(b[0]) - 1)
    B = ops.csr_to_device(*b, len(b[0]) - 1, ncols)
    rpt, col, val = h.spgemm(A, B).to_host()
    o = oracle.spgemm(*a, *b, ncols)
    assert np.array_equal(col, o[1]) and np.array_equal(val.view(np.uint64), o[2].view(np.uint64))
    h.close()


def test_persistent_batch_wide_columns_and_empty_problems(cuda):
    """The persistent path with 64-bit sort keys (a problem whose B has more than 2^20
    columns) next to degenerate problems: a 0-row problem, a problem whose A has no
    entries, and one whose B rows are all empty.  Every C_b equals its single call and the
    oracle, bit for bit."""
    import scipy.sparse as sp

    rng = np.random.default_rng(31)

    def csr(m):
        m = sp.csr_matrix(m)
        m.sort_indices()
        return m.indptr.astype(np.int32), m.indices.astype(np.int32), m.data.astype(np.float64)

    probs = []
    # wide: 3,000 x 2,000 times 2,000 x 1,500,000 (about 40 products per row)
    probs.append((csr(sp.random(3000, 2000, density=5 / 2000, random_state=rng)),
                  csr(sp.random(2000, 1_500_000, density=8 / 1_500_000, random_state=rng)), 1_500_000))
    probs.append((csr(sp.csr_matrix((0, 50))), csr(sp.random(50, 60, density=0.1, random_state=rng)), 60))
    probs.append((csr(sp.csr_matrix((40, 30))), csr(sp.random(30, 70, density=0.2, random_state=rng)), 70))
    probs.append((csr(sp.random(40, 30, density=0.2, random_state=rng)), csr(sp.csr_matrix((30, 70))), 70))
    for n, a, b in make_batch(5, 17):
        probs.append((a, b, n))
    pairs = [(ops.csr_to_device(*a, len(a[0]) - 1, len(b[0]) - 1), ops.csr_to_device(*b, len(b[0]) - 1, nc))
             for a, b, nc in probs]
    h = ops.Handle()
    batch = ops.Batch(h, pairs)
    assert batch.queues()[0] is True
    batch.execute(True)
    batch.check()
    single = ops.Handle()
    for i, (a, b, nc) in enumerate(probs):
        rpt, col, val = batch.result(i)
        o = oracle.spgemm(*a, *b, nc)
        assert np.array_equal(rpt.astype(np.int64), o[0]) and np.array_equal(col, o[1])
        assert np.array_equal(val.view(np.uint64), o[2].view(np.uint64))
        if len(a[0]) > 1:
            s = single.spgemm(*pairs[i]).to_host()
            assert np.array_equal(col, s[1]) and np.array_equal(val.view(np.uint64), s[2].view(np.uint64))
    batch.close()
