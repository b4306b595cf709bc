"""The column-window rank path of the CTA expand kernels (numeric rows of 257 to 1,024
outputs whose columns span fewer than 65,536 columns).

Rows are built to reach each branch: products in distinct columns (rank, no late
product), a few products in repeated columns (re-fold of 20, 50 and 100 late products:
the one-, two- and four-key-per-lane sorts of the late list), many repeated columns (more
than 128 late products: the sort), and a B wider than the window (the sort-only kernel,
not counted).  Through the two-pass and the one-pass call, FP64 and FP32: results
bit-identical to the oracle, and the rows counted on each path.
"""
import numpy as np
import pytest

import oracle
import opsparse_gb300 as ops

pytestmark = pytest.mark.gpu

A_LEN = 24  # A entries per row; each points at B rows of its own


def _row_b_rows(rng, kind, span):
    """A_LEN B rows (sorted column lists) for one A row of the given kind."""
    if kind == "distinct":  # 720 products, 720 columns
        cols = rng.choice(span, A_LEN * 30, replace=False)
        return [np.sort(c) for c in np.split(cols, A_LEN)]
    if kind.startswith("late"):  # 720 products, 720 - late columns
        late = int(kind[4:])
        pool = rng.choice(span, A_LEN * 30 - late, replace=False)
        parts = [list(c) for c in np.array_split(pool, A_LEN)]
        for c in rng.choice(pool, late, replace=False):
            while True:  # into a B row that lacks it (B rows are sets)
                i = int(rng.integers(A_LEN))
                if c not in parts[i]:
                    parts[i].append(c)
                    break
        return [np.sort(np.array(p)) for p in parts]
    if kind == "crowded":  # 960 products onto at most 350 columns
        pool = rng.choice(span, 350, replace=False)
        return [np.sort(rng.choice(pool, 40, replace=False)) for _ in range(A_LEN)]
    raise ValueError(kind)


def rank_case(seed=5, wide=False):
    """A: 40 rows per group; row i owns B rows [24 i, 24 i + 24).  Narrow groups (B of
    65,536 columns, so every row fits the window): products in distinct columns (80 rows),
    20, 50, 100, 128 and 129 late products (40 rows each) and crowded columns (40 rows).  wide=True:
    40 rows of distinct columns spread over 200,000 columns (B wider than the window: the
    sort-only shape)."""
    rng = np.random.default_rng(seed)
    if wide:
        kinds, ncols = [("distinct", 200000)], 200000
    else:
        kinds = [("distinct", 60000), ("late20", 60000), ("late50", 50000), ("late100", 65536), ("crowded", 30000),
                 ("distinct", 2000), ("late128", 60000), ("late129", 60000)]
        ncols = 65536
    b_rows = []
    for kind, span in kinds:
        for _ in range(40):
            b_rows.extend(_row_b_rows(rng, kind, span))
    m = len(kinds) * 40
    a_rpt = np.arange(0, m * A_LEN + 1, A_LEN, dtype=np.int32)
    a_col = np.arange(m * A_LEN, dtype=np.int32)
    a_val = rng.standard_normal(m * A_LEN)
    b_rpt = np.concatenate([[0], np.cumsum([len(r) for r in b_rows])]).astype(np.int32)
    b_col = np.concatenate(b_rows).astype(np.int32)
    b_val = rng.standard_normal(len(b_col))
    return (a_rpt, a_col, a_val), (b_rpt, b_col, b_val), ncols


@pytest.mark.parametrize("wide", [False, True], ids=["window", "wide"])
@pytest.mark.parametrize("oneshot", [False, True], ids=["two_phase", "one_pass"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_rank_path_branches(cuda, dtype, oneshot, wide):
    torch = cuda
    a, b, ncols = rank_case(wide=wide)
    tdt = torch.float64 if dtype == "f64" else torch.float32
    npdt = np.float64 if dtype == "f64" else np.float32
    a = (a[0], a[1], a[2].astype(npdt))
    b = (b[0], b[1], b[2].astype(npdt))
    A = ops.csr_to_device(*a, len(a[0]) - 1, len(b[0]) - 1, dtype=tdt)
    B = ops.csr_to_device(*b, len(b[0]) - 1, ncols, dtype=tdt)
    with ops.Handle() as h:
        if oneshot:
            h.set_one_pass(2)  # stage the rows whatever their number
        C = h.spgemm_oneshot(A, B) if oneshot else h.spgemm(A, B)
        rpt, col, val = C.to_host()
        sub = h.subclass_rows()
    orpt, ocol, oval = oracle.spgemm(*a, *b, ncols, dtype=npdt)
    assert np.array_equal(rpt.astype(np.int64), orpt)
    assert np.array_equal(col, ocol)
    bits = np.uint64 if dtype == "f64" else np.uint32
    assert np.array_equal(val.view(bits), oval.view(bits))
    assert sub["e1_esc"] == len(rpt) - 1, sub  # every row is an expand row
    if wide:
        assert sub["rank"] == 0 and sub["rank_refold"] == 0 and sub["rank_sorted"] == 0, sub
    else:
        # 80 rows without late products, 160 re-folded (128 late products is the list's
        # capacity), 80 sorted (crowded columns, and 129 late products)
        assert sub["rank"] == 80 and sub["rank_refold"] == 160 and sub["rank_sorted"] == 80, sub
