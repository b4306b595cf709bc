"""torch.autograd harness for the fixed-pattern SpGEMM (test harness over the C ABI).

FixedPatternSpGEMM runs the symbolic phase once for given A and B patterns; calling it
with A's and B's values runs the numeric phase (C's values on the fixed pattern), and
gradients flow back through ops_spgemm_backward.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import CsrMatrix, Handle, _dtype_code, _stream_ptr
from .capi import check


class FixedPatternSpGEMM:
    def __init__(self, A: CsrMatrix, B: CsrMatrix, handle: Handle | None = None):
        self.h = handle or Handle()
        self.A, self.B = A, B
        self.c_rpt, self.nnz = self.h.symbolic(A, B)
        self.c_col = torch.empty(self.nnz, dtype=torch.int32, device=A.rpt.device)

    def forward_values(self, a_val, b_val):
        A = CsrMatrix(self.A.rows, self.A.cols, self.A.rpt, self.A.col, a_val.contiguous())
        B = CsrMatrix(self.B.rows, self.B.cols, self.B.rpt, self.B.col, b_val.contiguous())
        c_val = torch.empty(self.nnz, dtype=a_val.dtype, device=a_val.device)
        self.h.numeric(A, B, self.c_rpt, self.nnz, c_col=self.c_col, c_val=c_val)
        return c_val

    def backward_values(self, a_val, b_val, dc, need_a=True, need_b=True):
        da = torch.empty_like(a_val) if need_a else None
        db = torch.empty_like(b_val) if need_b else None
        lib = self.h.lib
        A, B = self.A, self.B
        dc = dc.contiguous()
        st = _stream_ptr()
        check(lib.ops_spgemm_backward(self.h.h, _dtype_code(a_val), A.rows, A.cols, B.cols, A.rpt.data_ptr(),
                                      A.col.data_ptr() if A.nnz else None, a_val.data_ptr() if A.nnz else None, A.nnz,
                                      B.rpt.data_ptr(), B.col.data_ptr() if B.nnz else None,
                                      b_val.data_ptr() if B.nnz else None, B.nnz, self.c_rpt.data_ptr(),
                                      self.c_col.data_ptr() if self.nnz else None, dc.data_ptr() if self.nnz else None,
                                      da.data_ptr() if (da is not None and A.nnz) else None,
                                      db.data_ptr() if (db is not None and B.nnz) else None, st), self.h.h)
        check(lib.ops_spgemm_check(self.h.h, st), self.h.h)
        return da, db

    def plan_info(self):
        prod, wm = C.c_int64(0), C.c_int(0)
        check(self.h.lib.ops_backward_plan_info(self.h.h, C.byref(prod), C.byref(wm)))
        return int(prod.value), bool(wm.value)

    def __call__(self, a_val, b_val):
        return _SpGEMMFn.apply(a_val, b_val, self)


class _SpGEMMFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a_val, b_val, op):
        ctx.save_for_backward(a_val, b_val)
        ctx.op = op
        return op.forward_values(a_val, b_val)

    @staticmethod
    def backward(ctx, dc):
        a_val, b_val = ctx.saved_tensors
        da, db = ctx.op.backward_values(a_val, b_val, dc, ctx.needs_input_grad[0], ctx.needs_input_grad[1])
        return da, db, None
