"""opsparse_gb300 — GB300-native CSR SpGEMM (C = A * B), Python harness.

The product is the C ABI in ``include/opsparse_gb300.h`` (and the C++ drop-in facade in
``include/opsparse/``); this module wraps the C ABI with ctypes for tests and benchmarks,
using PyTorch CUDA tensors as device memory.  Nothing here computes on the CPU: when the
CUDA library is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import capi
from .capi import OPS_F32, OPS_F64, OpsError, Timings, check, load

__all__ = ["CsrMatrix", "Handle", "OpsError", "OPS_F32", "OPS_F64", "load", "csr_to_device", "flop"]


def _torch():
    import torch

    return torch


@dataclass
class CsrMatrix:
    """Device CSR matrix held in torch tensors (int32 row_ptr/col_idx)."""

    rows: int
    cols: int
    rpt: "object"
    col: "object"
    val: "object"

    @property
    def nnz(self) -> int:
        return int(self.col.numel())

    def ptrs(self):
        return (self.rpt.data_ptr(), self.col.data_ptr() if self.col.numel() else None,
                self.val.data_ptr() if self.val is not None and self.val.numel() else None)

    def to_host(self):
        return (self.rpt.cpu().numpy(), self.col.cpu().numpy(), None if self.val is None else self.val.cpu().numpy())


def csr_to_device(rpt, col, val, rows: int, cols: int, dtype=None, device: str = "cuda") -> CsrMatrix:
    torch = _torch()
    dtype = dtype or torch.float64
    t_rpt = torch.as_tensor(rpt, dtype=torch.int32).to(device)
    t_col = torch.as_tensor(col, dtype=torch.int32).to(device)
    t_val = None if val is None else torch.as_tensor(val).to(dtype).to(device)
    return CsrMatrix(rows, cols, t_rpt, t_col, t_val)


def _dtype_code(t) -> int:
    torch = _torch()
    if t.dtype == torch.float64:
        return OPS_F64
    if t.dtype == torch.float32:
        return OPS_F32
    raise TypeError(f"unsupported value dtype {t.dtype}")


class _DevArray:
    """Exposes a library-owned device allocation to torch through __cuda_array_interface__."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None}


def _stream_ptr(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class Handle:
    """One library handle (streams, memory pool, workspace); not thread-safe."""

    def __init__(self, timing: int = 0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.ops_handle_create(C.byref(h)))
        self.h = h
        if timing:
            check(self.lib.ops_handle_set_timing(self.h, int(timing)), self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.ops_handle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_timing(self, level: int):
        check(self.lib.ops_handle_set_timing(self.h, int(level)), self.h)

    def set_thresholds(self, th):
        arr = (C.c_int32 * 6)(*[int(x) for x in th])
        check(self.lib.ops_handle_set_thresholds(self.h, arr, 6), self.h)

    def get_thresholds(self):
        arr = (C.c_int32 * 6)()
        check(self.lib.ops_handle_get_thresholds(self.h, arr, 6), self.h)
        return list(arr)

    def set_one_pass(self, mode: int):
        """ops_spgemm in one pass: 0 off, 1 on for large inputs (default), 2 on at any size."""
        check(self.lib.ops_handle_set_one_pass(self.h, int(mode)), self.h)

    def get_tuning(self) -> dict:
        """Every run-time kernel and size choice of the handle (ops_tuning)."""
        t = capi.Tuning()
        check(self.lib.ops_handle_get_tuning(self.h, C.byref(t)), self.h)
        return t.as_dict()

    def set_tuning(self, **kw):
        """Changes the named fields of the handle's ops_tuning (thresholds, hash_slots,
        batch_persistent, batch_warp_max)."""
        cur = self.get_tuning()
        cur.update(kw)
        check(self.lib.ops_handle_set_tuning(self.h, C.byref(capi.Tuning.from_dict(cur))), self.h)

    def set_stage_budget(self, nbytes: int):
        """Largest one-pass staging area; beyond it ops_spgemm runs two passes."""
        check(self.lib.ops_handle_set_stage_budget(self.h, int(nbytes)), self.h)

    def set_dense_budget(self, nbytes: int):
        check(self.lib.ops_handle_set_dense_budget(self.h, int(nbytes)), self.h)

    def timings(self) -> dict:
        t = Timings()
        check(self.lib.ops_handle_get_timings(self.h, C.byref(t)), self.h)
        return t.as_dict()

    def subclass_rows(self) -> dict:
        """Rows per sub-kernel of the last call: E1 numeric (warp sort, warp hash,
        expand/sort/compress), E2 (mid, large shape), D (whole-GPU sort, dense kernel), and
        the expand rows of narrow column span by path (rank, rank with re-fold, sorted)."""
        arr = (C.c_int32 * 10)()
        check(self.lib.ops_handle_subclass_rows(self.h, arr, 10), self.h)
        return dict(zip(("e1_sort", "e1_hash", "e1_esc", "e2_mid", "e2_large", "d_sort", "d_dense", "rank",
                         "rank_refold", "rank_sorted"), list(arr)))

    # -- two-phase ------------------------------------------------------------
    def symbolic(self, A: CsrMatrix, B: CsrMatrix, c_rpt=None, stream=None):
        torch = _torch()
        if c_rpt is None:
            c_rpt = torch.empty(A.rows + 1, dtype=torch.int32, device=A.rpt.device)
        nnz = C.c_int64(0)
        a = A.ptrs()
        b = B.ptrs()
        check(self.lib.ops_spgemm_symbolic(self.h, A.rows, A.cols, B.cols, a[0], a[1], A.nnz, b[0], b[1], B.nnz,
                                           c_rpt.data_ptr(), C.byref(nnz), _stream_ptr(stream)), self.h)
        return c_rpt, int(nnz.value)

    def numeric(self, A: CsrMatrix, B: CsrMatrix, c_rpt, nnz: int, c_col=None, c_val=None, stream=None,
                check_flags: bool = True):
        torch = _torch()
        if c_col is None:
            c_col = torch.empty(nnz, dtype=torch.int32, device=A.rpt.device)
        if c_val is None:
            c_val = torch.empty(nnz, dtype=A.val.dtype, device=A.rpt.device)
        a = A.ptrs()
        b = B.ptrs()
        check(self.lib.ops_spgemm_numeric(self.h, _dtype_code(A.val), A.rows, A.cols, B.cols, a[0], a[1], a[2],
                                          b[0], b[1], b[2], c_rpt.data_ptr(),
                                          c_col.data_ptr() if nnz else None, c_val.data_ptr() if nnz else None,
                                          _stream_ptr(stream)), self.h)
        if check_flags:
            check(self.lib.ops_spgemm_check(self.h, _stream_ptr(stream)), self.h)
        return c_col, c_val

    def spgemm(self, A: CsrMatrix, B: CsrMatrix, stream=None) -> CsrMatrix:
        """C = A * B through the two-phase API with torch-allocated outputs."""
        c_rpt, nnz = self.symbolic(A, B, stream=stream)
        c_col, c_val = self.numeric(A, B, c_rpt, nnz, stream=stream)
        return CsrMatrix(A.rows, B.cols, c_rpt, c_col, c_val)

    # -- one-shot (library-allocated outputs) ----------------------------------
    def spgemm_oneshot(self, A: CsrMatrix, B: CsrMatrix, stream=None) -> CsrMatrix:
        """C = A * B through ops_spgemm; the library's arrays are copied into torch and freed."""
        torch = _torch()
        rp, cp, vp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nnz = C.c_int64(0)
        a = A.ptrs()
        b = B.ptrs()
        st = _stream_ptr(stream)
        check(self.lib.ops_spgemm(self.h, _dtype_code(A.val), A.rows, A.cols, B.cols, a[0], a[1], a[2], A.nnz,
                                  b[0], b[1], b[2], B.nnz, C.byref(rp), C.byref(cp), C.byref(vp), C.byref(nnz), st),
              self.h)
        n = int(nnz.value)
        vstr = "<f8" if A.val.dtype == torch.float64 else "<f4"
        dev = A.rpt.device
        c_rpt = torch.as_tensor(_DevArray(rp.value, A.rows + 1, "<i4"), device=dev).clone()
        c_col = torch.as_tensor(_DevArray(cp.value, n, "<i4"), device=dev).clone() if n else \
            torch.empty(0, dtype=torch.int32, device=dev)
        c_val = torch.as_tensor(_DevArray(vp.value, n, vstr), device=dev).clone() if n else \
            torch.empty(0, dtype=A.val.dtype, device=dev)
        torch.cuda.current_stream().synchronize()
        for p in (rp, cp, vp):
            check(self.lib.ops_free(p, st))
        return CsrMatrix(A.rows, B.cols, c_rpt, c_col, c_val)


def flop(A: CsrMatrix, B: CsrMatrix, stream=None) -> int:
    """Total intermediate products of A * B, computed on the device."""
    lib = load()
    tot = C.c_int64(0)
    check(lib.ops_flop(A.rows, A.cols, A.rpt.data_ptr(), A.col.data_ptr() if A.nnz else None, B.rpt.data_ptr(),
                       None, C.byref(tot), _stream_ptr(stream)))
    return int(tot.value)


class Batch:
    """Many independent products C_b = A_b * B_b planned once (ops_batch_create) and
    executed repeatedly (ops_batch_execute, optionally as one CUDA-graph launch)."""

    def __init__(self, handle: Handle, pairs, stream=None):
        torch = _torch()
        self.h = handle
        self.lib = handle.lib
        self.pairs = pairs  # keep the device arrays alive
        n = len(pairs)
        items = (capi.BatchItem * max(n, 1))()
        self.dtype = pairs[0][0].val.dtype if n else torch.float64
        for i, (A, B) in enumerate(pairs):
            a, b = A.ptrs(), B.ptrs()
            items[i] = capi.BatchItem(A.rows, A.cols, B.cols, A.nnz, B.nnz, a[0], a[1], a[2], b[0], b[1], b[2])
        out = C.c_void_p()
        self.stream = stream or torch.cuda.Stream()
        check(self.lib.ops_batch_create(handle.h, _dtype_code(torch.empty(0, dtype=self.dtype)), n, items,
                                        C.byref(out), C.c_void_p(self.stream.cuda_stream)), handle.h)
        self.b = out
        self.n = n

    def execute(self, use_graph: bool = True):
        check(self.lib.ops_batch_execute(self.b, 1 if use_graph else 0, C.c_void_p(self.stream.cuda_stream)),
              self.h.h)

    def check(self):
        check(self.lib.ops_batch_check(self.b, C.c_void_p(self.stream.cuda_stream)), self.h.h)

    def info(self):
        seg, fl, nz = C.c_int32(0), C.c_int64(0), C.c_int64(0)
        check(self.lib.ops_batch_info(self.b, C.byref(seg), C.byref(fl), C.byref(nz)))
        return int(seg.value), int(fl.value), int(nz.value)

    def queues(self):
        """(persistent, warp-queue rows, CTA-queue rows) of the batch's plan."""
        p, w, c = C.c_int32(0), C.c_int64(0), C.c_int64(0)
        check(self.lib.ops_batch_queues(self.b, C.byref(p), C.byref(w), C.byref(c)))
        return bool(p.value), int(w.value), int(c.value)

    def result(self, i: int):
        """(rpt, col, val) numpy copies of C_i."""
        torch = _torch()
        rp, cp, vp, nnz = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_int64(0)
        check(self.lib.ops_batch_result(self.b, i, C.byref(rp), C.byref(cp), C.byref(vp), C.byref(nnz)), self.h.h)
        A = self.pairs[i][0]
        n = int(nnz.value)
        self.stream.synchronize()
        rpt = torch.as_tensor(_DevArray(rp.value, A.rows + 1, "<i4"), device="cuda").cpu().numpy()
        if n == 0:
            return rpt, np_empty("i4"), np_empty("f8" if self.dtype == torch.float64 else "f4")
        col = torch.as_tensor(_DevArray(cp.value, n, "<i4"), device="cuda").cpu().numpy()
        val = torch.as_tensor(_DevArray(vp.value, n, "<f8" if self.dtype == torch.float64 else "<f4"),
                              device="cuda").cpu().numpy()
        return rpt, col, val

    def result_device(self, i: int):
        """(rpt, col, val, nnz) of C_i as torch views of the batch's device storage (valid
        until close())."""
        torch = _torch()
        rp, cp, vp, nnz = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_int64(0)
        check(self.lib.ops_batch_result(self.b, i, C.byref(rp), C.byref(cp), C.byref(vp), C.byref(nnz)), self.h.h)
        A = self.pairs[i][0]
        n = int(nnz.value)
        dev = A.rpt.device
        vstr = "<f8" if self.dtype == torch.float64 else "<f4"
        rpt = torch.as_tensor(_DevArray(rp.value, A.rows + 1, "<i4"), device=dev)
        if n == 0:
            return rpt, torch.empty(0, dtype=torch.int32, device=dev), torch.empty(0, dtype=self.dtype, device=dev), 0
        col = torch.as_tensor(_DevArray(cp.value, n, "<i4"), device=dev)
        val = torch.as_tensor(_DevArray(vp.value, n, vstr), device=dev)
        return rpt, col, val, n

    def close(self):
        if getattr(self, "b", None):
            self.lib.ops_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def np_empty(kind: str):
    import numpy as np

    return np.zeros(0, dtype=kind)


def batch_items(pairs):
    items = (capi.BatchItem * max(len(pairs), 1))()
    for i, (A, B) in enumerate(pairs):
        a, b = A.ptrs(), B.ptrs()
        items[i] = capi.BatchItem(A.rows, A.cols, B.cols, A.nnz, B.nnz, a[0], a[1], a[2], b[0], b[1], b[2])
    return items


def autotune(handle: Handle, pairs, reps: int = 3, stream=None):
    """Runs the library's autotuner on (a sample of) a workload and installs the best tuning
    on the handle (handle.get_tuning() reads all of it); returns (thresholds, ms)."""
    torch = _torch()
    best = (C.c_int32 * 6)()
    ms = C.c_float(0)
    st = stream or torch.cuda.Stream()
    check(handle.lib.ops_autotune(handle.h, _dtype_code(pairs[0][0].val), len(pairs), batch_items(pairs), reps, best,
                                  C.byref(ms), C.c_void_p(st.cuda_stream)), handle.h)
    return list(best), float(ms.value)


def tuning_store(path: str, key: str, thresholds) -> None:
    arr = (C.c_int32 * 6)(*[int(x) for x in thresholds])
    check(load().ops_tuning_store(str(path).encode(), key.encode(), arr))


def tuning_lookup(path: str, key: str):
    arr = (C.c_int32 * 6)()
    st = load().ops_tuning_lookup(str(path).encode(), key.encode(), arr)
    return list(arr) if st == capi.OPS_OK else None


def tuning_store_record(path: str, key: str, tuning: dict) -> None:
    """Stores a whole ops_tuning (as returned by Handle.get_tuning) under key."""
    check(load().ops_tuning_store_record(str(path).encode(), key.encode(), C.byref(capi.Tuning.from_dict(tuning))))


def tuning_lookup_record(path: str, key: str):
    t = capi.Tuning()
    st = load().ops_tuning_lookup_record(str(path).encode(), key.encode(), C.byref(t))
    return t.as_dict() if st == capi.OPS_OK else None
