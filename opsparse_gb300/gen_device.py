"""Device-side generator of the batched workload (many Erdos-Renyi pairs), using torch on
the GPU: the full batch has ~39M rows and ~0.7G non-zeros per side, too large to build
with numpy on the host in reasonable time.

Problem b: n_b = floor(exp(U(ln lo, ln hi))) rows and columns, mean degree d_b ~ U(4, 32);
row degrees Poisson(d_b), columns uniform in [0, n_b), duplicates removed, values N(0,1).
Returns one concatenated CSR per side (row pointers int64 over all rows) and per-problem
(row_base, n) so each problem is a slice.
"""
from __future__ import annotations

import numpy as np


def er_batch(count: int, lo: int = 64, hi: int = 65536, dmin: float = 4.0, dmax: float = 32.0, seed: int = 20261203,
             dtype=None, device: str = "cuda"):
    import torch

    dtype = dtype or torch.float32
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), size=count))).astype(np.int64)
    degs = rng.uniform(dmin, dmax, size=count)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    row_base = np.concatenate([[0], np.cumsum(sizes)])
    total_rows = int(row_base[-1])
    n_of_row = torch.repeat_interleave(torch.as_tensor(sizes, device=device), torch.as_tensor(sizes, device=device))
    deg_of_row = torch.repeat_interleave(torch.as_tensor(degs, device=device, dtype=torch.float32),
                                         torch.as_tensor(sizes, device=device))

    def one_side():
        cnt = torch.poisson(deg_of_row, generator=gen).to(torch.int64)
        cnt = torch.minimum(cnt, n_of_row)
        rows = torch.repeat_interleave(torch.arange(total_rows, device=device), cnt)
        nrow = n_of_row[rows]
        cols = (torch.rand(rows.numel(), generator=gen, device=device, dtype=torch.float64) * nrow).to(torch.int64)
        keys = torch.unique(rows * 65536 + cols)  # sorted, de-duplicated
        r = keys // 65536
        c = (keys % 65536).to(torch.int32)
        rpt = torch.zeros(total_rows + 1, dtype=torch.int64, device=device)
        rpt[1:] = torch.cumsum(torch.bincount(r, minlength=total_rows), 0)
        val = torch.randn(c.numel(), generator=gen, device=device, dtype=dtype)
        return rpt, c, val

    a = one_side()
    b = one_side()
    return sizes, row_base, a, b


def problem_slices(sizes, row_base, side):
    """[(rpt int32 rebased, col view, val view, nnz)] per problem (device tensors)."""
    import torch

    rpt, col, val = side
    out = []
    rpt_cpu = rpt.cpu().numpy()
    for b, n in enumerate(sizes):
        r0 = int(row_base[b])
        s, e = int(rpt_cpu[r0]), int(rpt_cpu[r0 + n])
        out.append(((rpt[r0:r0 + n + 1] - s).to(torch.int32), col[s:e], val[s:e], e - s))
    return out
