"""Entries of more than 2,560 products (possible only in D rows, whose A rows may be longer
than that) fold in 32 consecutive blocks, the block states merged in order — the fixed
order the oracle follows for them (oracle/oracle.c, tests/test_oracle.py pins it).

Rows of 3,000 to 9,000 A entries whose B rows share a few hub columns give entries of 2,561
to 9,000 products beside ordinary ones; both D-row paths (the whole-GPU sort, and the
dense-row kernel under a small scratch budget), FP64 and FP32, two passes and one pass:
results bit-identical to the oracle.
"""
import numpy as np
import pytest

import oracle
import opsparse_gb300 as ops

pytestmark = pytest.mark.gpu


def long_entry_case(seed=41):
    """A: 5 rows of 3,000, 4,100, 9,000, 40 and 2,600 entries; each A entry owns a B row of
    2-4 columns: hub columns (0, 1 or 2, chosen so the hubs collect thousands of products;
    in the last row one hub of 2,561 and one of 2,560 products, either side of the rule's
    bound) plus distinct private columns."""
    rng = np.random.default_rng(seed)
    lens = [3000, 4100, 9000, 40, 2600]
    b_rows = []
    nxt = 3
    for i, L in enumerate(lens):
        for e in range(L):
            hubs = [0] if i != 1 else ([0, 1] if e % 3 else [1])
            if i == 2 and e % 2:
                hubs = [0, 2]
            if i == 4:  # column 0: 2,561 products (blocked); column 1: 2,560 (plain)
                hubs = ([0] if e < 2561 else []) + ([1] if e < 2560 else [])
            priv = list(range(nxt, nxt + int(rng.integers(1, 3))))
            nxt += len(priv)
            b_rows.append(sorted(hubs + priv))
    arpt = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    acol = np.arange(arpt[-1], dtype=np.int32)
    aval = rng.standard_normal(len(acol))
    brpt = np.concatenate([[0], np.cumsum([len(r) for r in b_rows])]).astype(np.int32)
    bcol = np.concatenate(b_rows).astype(np.int32)
    bval = rng.standard_normal(len(bcol))
    return (arpt, acol, aval), (brpt, bcol, bval), nxt


@pytest.mark.parametrize("path", ["d_sort", "d_dense"])
@pytest.mark.parametrize("oneshot", [False, True], ids=["two_phase", "one_pass"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_long_entries_fold_in_blocks(cuda, dtype, oneshot, path):
    torch = cuda
    a, b, ncols = long_entry_case()
    npdt = np.float64 if dtype == "f64" else np.float32
    tdt = torch.float64 if dtype == "f64" else torch.float32
    a = (a[0], a[1], a[2].astype(npdt))
    b = (b[0], b[1], b[2].astype(npdt))
    # the case holds entries of more than 2,560 products
    orpt, ocol, oval = oracle.spgemm(*a, *b, ncols, dtype=npdt)
    assert ocol[orpt[0]] == 0 and ocol[orpt[2]:orpt[2] + 2].tolist() == [0, 2]
    A = ops.csr_to_device(*a, len(a[0]) - 1, len(b[0]) - 1, dtype=tdt)
    B = ops.csr_to_device(*b, len(b[0]) - 1, ncols, dtype=tdt)
    with ops.Handle() as h:
        if oneshot:
            h.set_one_pass(2)
        if path == "d_dense":
            h.set_dense_budget(1 << 20)
        C = h.spgemm_oneshot(A, B) if oneshot else h.spgemm(A, B)
        rpt, col, val = C.to_host()
        sub = h.subclass_rows()
    assert np.array_equal(rpt.astype(np.int64), orpt)
    assert np.array_equal(col, ocol)
    bits = np.uint64 if dtype == "f64" else np.uint32
    assert np.array_equal(val.view(bits), oval.view(bits))
    assert sub[path] >= 4, sub  # the four long rows took the path under test
