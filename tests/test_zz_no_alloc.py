"""ops_flop_noalloc — the product counter for callers that may not allocate device memory
(serving loops that forbid the CUDA allocator once running, hosts with a fixed memory
budget).

Called through the C ABI twice in a row on the same inputs; each call's per-row counts and
total must equal ops_flop's and the oracle's (integers: exact).  The second call checks
that the shared scratch array is cleared between calls.  This file is collected last so
that a run stopping at the first failure has already run every other test; it also passes
on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from opsparse_gb300 import capi, gen

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.as_tensor(a).cuda()


def test_noalloc_matches_ops_flop_twice(cuda):
    torch = cuda
    lib = capi.load()
    rpt, col, _ = gen.web_powerlaw(200_000, lmax=3000)
    n = len(rpt) - 1
    d_rpt, d_col = _dev(torch, rpt), _dev(torch, col)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    ref_rows = torch.empty(n, dtype=torch.int64, device="cuda")
    ref_total = C.c_int64(0)
    assert lib.ops_flop(n, n, d_rpt.data_ptr(), d_col.data_ptr(), d_rpt.data_ptr(), ref_rows.data_ptr(),
                        C.byref(ref_total), stream) == capi.OPS_OK
    orc_total, orc_rows = oracle.flop(rpt, col, rpt)
    assert ref_total.value == orc_total
    assert np.array_equal(ref_rows.cpu().numpy(), orc_rows)

    for _ in range(2):
        rows = torch.full((n,), -1, dtype=torch.int64, device="cuda")
        total = C.c_int64(-1)
        st = lib.ops_flop_noalloc(n, n, d_rpt.data_ptr(), d_col.data_ptr(), d_rpt.data_ptr(), rows.data_ptr(),
                                  C.byref(total), stream)
        assert st == capi.OPS_OK, capi.status_string(st)
        assert total.value == ref_total.value == orc_total
        assert np.array_equal(rows.cpu().numpy(), orc_rows)


def test_noalloc_refuses_oversized_input(cuda):
    lib = capi.load()
    total = C.c_int64(0)
    one = cuda.zeros(1, dtype=cuda.int32, device="cuda")
    st = lib.ops_flop_noalloc(2_097_153, 1, one.data_ptr(), one.data_ptr(), one.data_ptr(), None, C.byref(total),
                              None)
    assert st == capi.OPS_NOT_SUPPORTED
