"""CPU oracle for the SpGEMM parity tests — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use this
package; the library never imports it.  It wraps ``oracle/oracle.c`` (see that file's
header for what each function restates and how it is pinned) with ctypes.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SO = HERE / "_build" / "liboracle.so"
_LIB = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_I = C.c_int32


def build(force: bool = False) -> Path:
    src = HERE / "oracle.c"
    if force or not SO.exists() or SO.stat().st_mtime < src.stat().st_mtime:
        SO.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(SO), str(src)],
                       check=True)
    return SO


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = C.CDLL(str(SO))
        L.orc_flop.restype = C.c_int64
        L.orc_flop.argtypes = [_I, _i32p, _i32p, _i32p, C.c_void_p]
        L.orc_symbolic.restype = C.c_int64
        L.orc_symbolic.argtypes = [_I, _I, _i32p, _i32p, _i32p, _i32p, _i64p]
        L.orc_spgemm_f64.restype = None
        L.orc_spgemm_f64.argtypes = [_I, _I, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _i64p, _i32p, _f64p]
        L.orc_spgemm_f32.restype = None
        L.orc_spgemm_f32.argtypes = [_I, _I, _i32p, _i32p, _f32p, _i32p, _i32p, _f32p, _i64p, _i32p, _f32p]
        L.orc_backward_f64.restype = None
        L.orc_backward_f64.argtypes = [_I, _I, _I, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _i64p, _i32p, _f64p,
                                       _f64p, _f64p]
        L.orc_omp_symbolic.restype = C.c_int64
        L.orc_omp_symbolic.argtypes = [_I, _i32p, _i32p, _i32p, _i32p, _i64p]
        L.orc_omp_numeric_f64.restype = None
        L.orc_omp_numeric_f64.argtypes = [_I, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _i64p, _i32p, _f64p]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]
        _LIB = L
    return _LIB


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def set_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


def flop(arpt, acol, brpt):
    """(total, row_flop int64[M]) — per-row intermediate products."""
    M = len(arpt) - 1
    rf = np.zeros(max(M, 1), dtype=np.int64)
    tot = lib().orc_flop(M, _c(arpt, np.int32), _c(acol, np.int32), _c(brpt, np.int32), rf.ctypes.data)
    return int(tot), rf[:M]


def symbolic(arpt, acol, brpt, bcol, ncols: int):
    M = len(arpt) - 1
    crpt = np.zeros(M + 1, dtype=np.int64)
    nnz = lib().orc_symbolic(M, int(ncols), _c(arpt, np.int32), _c(acol, np.int32), _c(brpt, np.int32),
                             _c(bcol, np.int32), crpt)
    return crpt, int(nnz)


def spgemm(arpt, acol, aval, brpt, bcol, bval, ncols: int, dtype=np.float64):
    """C = A*B: (rpt int64[M+1], col int32[nnz], val dtype[nnz]) with the oracle's
    summation order (FP64: fma chain in ascending j; FP32: Dot2)."""
    M = len(arpt) - 1
    crpt, nnz = symbolic(arpt, acol, brpt, bcol, ncols)
    ccol = np.zeros(max(nnz, 1), dtype=np.int32)
    if dtype == np.float64:
        cval = np.zeros(max(nnz, 1), dtype=np.float64)
        lib().orc_spgemm_f64(M, int(ncols), _c(arpt, np.int32), _c(acol, np.int32), _c(aval, np.float64),
                             _c(brpt, np.int32), _c(bcol, np.int32), _c(bval, np.float64), crpt, ccol, cval)
    elif dtype == np.float32:
        cval = np.zeros(max(nnz, 1), dtype=np.float32)
        lib().orc_spgemm_f32(M, int(ncols), _c(arpt, np.int32), _c(acol, np.int32), _c(aval, np.float32),
                             _c(brpt, np.int32), _c(bcol, np.int32), _c(bval, np.float32), crpt, ccol, cval)
    else:
        raise TypeError(dtype)
    return crpt, ccol[:nnz], cval[:nnz]


def backward(arpt, acol, aval, brpt, bcol, bval, ncols: int, crpt, ccol, dcval):
    """(dA values on A's pattern, dB values on B's pattern) for loss = sum(dC .* C)."""
    M = len(arpt) - 1
    K = len(brpt) - 1
    da = np.zeros(max(len(acol), 1), dtype=np.float64)
    db = np.zeros(max(len(bcol), 1), dtype=np.float64)
    lib().orc_backward_f64(M, int(ncols), K, _c(arpt, np.int32), _c(acol, np.int32), _c(aval, np.float64),
                           _c(brpt, np.int32), _c(bcol, np.int32), _c(bval, np.float64), _c(crpt, np.int64),
                           _c(ccol, np.int32), _c(dcval, np.float64), da, db)
    return da[:len(acol)], db[:len(bcol)]


def omp_spgemm(arpt, acol, aval, brpt, bcol, bval):
    """OpenMP row-wise hash Gustavson (the timed CPU baseline); FP64."""
    M = len(arpt) - 1
    arpt, acol, aval = _c(arpt, np.int32), _c(acol, np.int32), _c(aval, np.float64)
    brpt, bcol, bval = _c(brpt, np.int32), _c(bcol, np.int32), _c(bval, np.float64)
    crpt = np.zeros(M + 1, dtype=np.int64)
    nnz = lib().orc_omp_symbolic(M, arpt, acol, brpt, bcol, crpt)
    ccol = np.zeros(max(nnz, 1), dtype=np.int32)
    cval = np.zeros(max(nnz, 1), dtype=np.float64)
    lib().orc_omp_numeric_f64(M, arpt, acol, aval, brpt, bcol, bval, crpt, ccol, cval)
    return crpt, ccol[:nnz], cval[:nnz]


def abs_sums(arpt, acol, aval, brpt, bcol, bval, ncols: int):
    """sum_j |a_ij| |b_jk| per output entry — the scale of each entry's rounding error."""
    return spgemm(arpt, acol, np.abs(np.asarray(aval, dtype=np.float64)), brpt, bcol,
                  np.abs(np.asarray(bval, dtype=np.float64)), ncols)[2]
