"""OpSparse's own SpGEMM kernels run on the CPU (oracle/ref_emul, built into oracle/_ref/)
— TEST INFRASTRUCTURE ONLY, used to pin the oracle and to generate golden fixtures.

Available only on a machine that holds the OpSparse sources; the GPU tests use
the committed fixtures in tests/golden/ instead.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SO = HERE / "_ref" / "libref_opsparse.so"
_LIB = None


def make_vars() -> list[str]:
    """make variables naming the OpSparse source tree: OPSPARSE_SRC from the environment
    when set, else none (the recipe's own default applies)."""
    src = os.environ.get("OPSPARSE_SRC")
    return [f"OPSPARSE_SRC={src}"] if src else []


def has_sources(recipe_dir: Path) -> bool:
    """Whether the recipe in `recipe_dir` finds the OpSparse source tree."""
    try:
        res = subprocess.run(["make", "-s", "-C", str(recipe_dir), *make_vars(), "has-src"],
                             stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    except OSError:  # no make on this machine
        return False
    return res.returncode == 0


def available() -> bool:
    return SO.exists() or has_sources(HERE / "ref_emul")


def build(force: bool = False) -> Path:
    srcs = [HERE / "ref_emul" / f for f in ("ref_driver.cpp", "emul.cpp", "cuda_emul.hpp")]
    if force or not SO.exists() or any(SO.stat().st_mtime < s.stat().st_mtime for s in srcs):
        if not has_sources(HERE / "ref_emul"):
            raise RuntimeError("OpSparse sources not found (set OPSPARSE_SRC to its source tree)")
        subprocess.run(["make", "-s", "-C", str(HERE / "ref_emul"), *make_vars(), f"OUT={SO.parent}"], check=True)
    return SO


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = C.CDLL(str(SO))
        L.ref_spgemm.restype = C.c_int
        L.ref_spgemm.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 6
        L.ref_fetch.restype = None
        L.ref_fetch.argtypes = [C.c_void_p] * 6
        L.ref_compute_flop.restype = C.c_long
        L.ref_compute_flop.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        _LIB = L
    return _LIB


def spgemm(arpt, acol, aval, brpt, bcol, bval, ncols: int):
    """C = A*B by OpSparse's kernels: (rpt, col, val, info) with info holding the symbolic
    and numeric bin histograms and the number of rows that used the global-hash path."""
    a = [np.ascontiguousarray(x, dtype=t) for x, t in ((arpt, np.int32), (acol, np.int32), (aval, np.float64))]
    b = [np.ascontiguousarray(x, dtype=t) for x, t in ((brpt, np.int32), (bcol, np.int32), (bval, np.float64))]
    M = len(a[0]) - 1
    K = len(b[0]) - 1
    nnz = lib().ref_spgemm(M, K, int(ncols), *(x.ctypes.data for x in a + b))
    rpt = np.zeros(M + 1, np.int32)
    col = np.zeros(max(nnz, 1), np.int32)
    val = np.zeros(max(nnz, 1), np.float64)
    bs = np.zeros(8, np.int32)
    bn = np.zeros(8, np.int32)
    fail = np.zeros(1, np.int32)
    lib().ref_fetch(rpt.ctypes.data, col.ctypes.data, val.ctypes.data, bs.ctypes.data, bn.ctypes.data,
                    fail.ctypes.data)
    return rpt, col[:nnz], val[:nnz], {"bins_symbolic": bs.tolist(), "bins_numeric": bn.tolist(),
                                       "global_fallback_rows": int(fail[0])}


def compute_flop(arpt, acol, brpt):
    """OpSparse's host compute_flop: (total, per-row int32)."""
    arpt = np.ascontiguousarray(arpt, np.int32)
    acol = np.ascontiguousarray(acol, np.int32)
    brpt = np.ascontiguousarray(brpt, np.int32)
    M = len(arpt) - 1
    rf = np.zeros(max(M, 1), np.int32)
    tot = lib().ref_compute_flop(arpt.ctypes.data, acol.ctypes.data, brpt.ctypes.data, M, rf.ctypes.data)
    return int(tot), rf[:M]
