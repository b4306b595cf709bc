"""ctypes binding of the C ABI declared in ``include/opsparse_gb300.h``.

The library is loaded from the in-tree build folder.  There is no fallback: if the
shared object is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

from . import build as _build

_LIB = None

OPS_OK = 0
OPS_NONSQUARE = 1
OPS_INT32_OVERFLOW = 2
OPS_OOM = 3
OPS_CUDA_ERROR = 4
OPS_EXCEPTION = 5
OPS_INVALID_ARGUMENT = 6
OPS_INVALID_CSR = 7
OPS_PROBE_LIMIT = 8
OPS_TIMEOUT = 9
OPS_NOT_SUPPORTED = 10
OPS_COUNT_MISMATCH = 11

OPS_F64 = 0
OPS_F32 = 1

P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64


class Timings(C.Structure):
    _fields_ = [
        ("setup", C.c_double),
        ("symbolic_binning", C.c_double),
        ("symbolic", C.c_double),
        ("reduce", C.c_double),
        ("numeric_binning", C.c_double),
        ("prefix", C.c_double),
        ("allocate", C.c_double),
        ("numeric", C.c_double),
        ("cleanup", C.c_double),
        ("total", C.c_double),
        ("flop", I64),
        ("nnz", I64),
        ("class_rows", I32 * 8),
        ("launches", I64),
        ("kernel_ms", (C.c_float * 8) * 2),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("class_rows", "kernel_ms")}
        d["class_rows"] = list(self.class_rows)[:7]
        d["kernel_ms"] = [list(self.kernel_ms[0])[:7], list(self.kernel_ms[1])[:7]]
        return d


class Tuning(C.Structure):
    _fields_ = [("thresholds", I32 * 6), ("hash_slots", I32), ("batch_persistent", I32), ("batch_warp_max", I32)]

    def as_dict(self) -> dict:
        return {"thresholds": list(self.thresholds), "hash_slots": self.hash_slots,
                "batch_persistent": self.batch_persistent, "batch_warp_max": self.batch_warp_max}

    @classmethod
    def from_dict(cls, d):
        return cls((I32 * 6)(*[int(x) for x in d["thresholds"]]), int(d["hash_slots"]), int(d["batch_persistent"]),
                   int(d["batch_warp_max"]))


class BatchItem(C.Structure):
    _fields_ = [("rows", I32), ("cols_a", I32), ("cols_b", I32), ("a_nnz", I64), ("b_nnz", I64),
                ("a_rpt", P), ("a_col", P), ("a_val", P), ("b_rpt", P), ("b_col", P), ("b_val", P)]


_SIGS = {
    "ops_version": (C.c_char_p, []),
    "ops_status_string": (C.c_char_p, [C.c_int]),
    "ops_handle_create": (C.c_int, [C.POINTER(P)]),
    "ops_handle_destroy": (C.c_int, [P]),
    "ops_handle_set_timing": (C.c_int, [P, C.c_int]),
    "ops_handle_get_timings": (C.c_int, [P, C.POINTER(Timings)]),
    "ops_handle_set_dense_budget": (C.c_int, [P, C.c_size_t]),
    "ops_handle_set_output_malloc": (C.c_int, [P, C.c_int]),
    "ops_handle_set_one_pass": (C.c_int, [P, C.c_int]),
    "ops_handle_set_stage_budget": (C.c_int, [P, C.c_size_t]),
    "ops_handle_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "ops_handle_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "ops_handle_set_thresholds": (C.c_int, [P, C.POINTER(I32), C.c_int]),
    "ops_handle_get_thresholds": (C.c_int, [P, C.POINTER(I32), C.c_int]),
    "ops_handle_last_error": (C.c_char_p, [P]),
    "ops_handle_subclass_rows": (C.c_int, [P, C.POINTER(I32), C.c_int]),
    "ops_spgemm": (C.c_int, [P, C.c_int, I32, I32, I32, P, P, P, I64, P, P, P, I64,
                             C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(I64), P]),
    "ops_spgemm_symbolic": (C.c_int, [P, I32, I32, I32, P, P, I64, P, P, I64, P, C.POINTER(I64), P]),
    "ops_spgemm_numeric": (C.c_int, [P, C.c_int, I32, I32, I32, P, P, P, P, P, P, P, P, P, P]),
    "ops_spgemm_check": (C.c_int, [P, P]),
    "ops_flop": (C.c_int, [I32, I32, P, P, P, P, C.POINTER(I64), P]),
    "ops_flop_noalloc": (C.c_int, [I32, I32, P, P, P, P, C.POINTER(I64), P]),
    "ops_free": (C.c_int, [P, P]),
    "ops_spgemm_backward": (C.c_int, [P, C.c_int, I32, I32, I32, P, P, P, I64, P, P, P, I64, P, P, P, P, P, P]),
    "ops_handle_set_map_budget": (C.c_int, [P, C.c_size_t]),
    "ops_backward_plan_info": (C.c_int, [P, C.POINTER(I64), C.POINTER(C.c_int)]),
    "ops_batch_create": (C.c_int, [P, C.c_int, I32, C.POINTER(BatchItem), C.POINTER(P), P]),
    "ops_batch_execute": (C.c_int, [P, C.c_int, P]),
    "ops_batch_check": (C.c_int, [P, P]),
    "ops_batch_result": (C.c_int, [P, I32, C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(I64)]),
    "ops_batch_info": (C.c_int, [P, C.POINTER(I32), C.POINTER(I64), C.POINTER(I64)]),
    "ops_batch_queues": (C.c_int, [P, C.POINTER(I32), C.POINTER(I64), C.POINTER(I64)]),
    "ops_batch_destroy": (C.c_int, [P]),
    "ops_autotune": (C.c_int, [P, C.c_int, I32, C.POINTER(BatchItem), C.c_int, C.POINTER(I32), C.POINTER(C.c_float), P]),
    "ops_tuning_store": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(I32)]),
    "ops_tuning_lookup": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(I32)]),
    "ops_tuning_store_record": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(Tuning)]),
    "ops_tuning_lookup_record": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(Tuning)]),
}


def header_symbols() -> list[str]:
    """Function names declared in include/opsparse_gb300.h (and its siblings)."""
    names: list[str] = []
    for h in sorted((_build.INCLUDE).glob("opsparse_gb300*.h")):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_\s\*]*?\b(ops_[a-z0-9_]+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def load(path: str | Path | None = None):
    """Load (and type) the C-ABI shared library; builds it in-tree if it is absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else _build.lib_path()
    if not p.exists():
        _build.build()
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


class OpsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{status_string(status)} ({status}): {msg}")
        self.status = status


def status_string(s: int) -> str:
    return load().ops_status_string(int(s)).decode()


def check(status: int, handle=None) -> None:
    if status != OPS_OK:
        msg = ""
        if handle is not None:
            msg = load().ops_handle_last_error(handle).decode()
        raise OpsError(status, msg)
