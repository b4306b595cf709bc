"""OpSparse's own SpGEMM kernels run on the GPU — TEST AND BENCHMARK INFRASTRUCTURE ONLY.

The kernels are compiled from OpSparse's sources into oracle/_ref/ref_kernels.cubin by
oracle/ref_gpu/Makefile on a machine that holds the sources; the cubin travels
with the repository.  oracle/ref_gpu/ref_gpu.cu, built on the GPU machine, loads it and
replays OpSparse's host sequence (phases, streams, allocations, synchronisations).  The
GPU tests use it to check this library against the reference on the same GPU, and
bench.py to time the reference with its own protocol (1 warm-up, mean of 10 calls).
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

from .ref import has_sources, make_vars

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
CUBIN = OUT / "ref_kernels.cubin"
NAMES = OUT / "ref_kernels.names"
SO = OUT / "libref_gpu.so"
_LIB = None


def _nvcc() -> str | None:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    return None


def build(force: bool = False) -> bool:
    """Builds the cubin (needs the OpSparse sources) and the host driver (needs the cubin).
    Returns whether the driver is available."""
    nvcc = _nvcc()
    if nvcc is None:
        return False
    kern = HERE / "ref_gpu" / "kernels.cu"
    if (force or not CUBIN.exists() or CUBIN.stat().st_mtime < kern.stat().st_mtime) and \
            has_sources(HERE / "ref_gpu"):
        subprocess.run(["make", "-s", "-C", str(HERE / "ref_gpu"), *make_vars(), f"OUT={OUT}", f"NVCC={nvcc}"],
                       check=True)
    if not (CUBIN.exists() and NAMES.exists()):
        return False
    drv = HERE / "ref_gpu" / "ref_gpu.cu"
    if force or not SO.exists() or SO.stat().st_mtime < drv.stat().st_mtime:
        subprocess.run([nvcc, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                        "-gencode", "arch=compute_103a,code=sm_103a", "-o", str(SO), str(drv), "-lcuda"],
                       check=True)
    return True


def available() -> bool:
    return SO.exists() and CUBIN.exists() and NAMES.exists()


def lib():
    global _LIB
    if _LIB is None:
        if not build():
            raise RuntimeError("the reference's GPU build is not available")
        L = C.CDLL(str(SO))
        L.refgpu_init.restype = C.c_int
        L.refgpu_init.argtypes = [C.c_char_p, C.c_char_p]
        L.refgpu_error.restype = C.c_char_p
        L.refgpu_spgemm.restype = C.c_longlong
        L.refgpu_spgemm.argtypes = [C.c_int] + [C.c_void_p] * 6 + [C.POINTER(C.c_void_p)] * 3 + [C.c_void_p] * 3
        L.refgpu_free.argtypes = [C.c_void_p]
        if L.refgpu_init(str(CUBIN).encode(), str(NAMES).encode()) != 0:
            raise RuntimeError("reference GPU init: " + L.refgpu_error().decode())
        _LIB = L
    return _LIB


class RefResult:
    """One reference call: device pointers of C (owned; free() releases them), nnz, the
    reference's SpgemmTimings fields (seconds) and its bin histograms."""
    FIELDS = ("setup", "symbolic_binning", "symbolic", "numeric_binning", "allocate", "prefix", "numeric", "cleanup",
              "total")

    def __init__(self, nnz, rpt, col, val, t, bins, fail_rows):
        self.nnz, self.rpt, self.col, self.val = nnz, rpt, col, val
        self.timings = dict(zip(self.FIELDS, list(t)))
        self.bins_symbolic = list(bins[:8])
        self.bins_numeric = list(bins[8:])
        self.fail_rows = fail_rows

    def free(self):
        L = lib()
        for p in (self.rpt, self.col, self.val):
            if p:
                L.refgpu_free(p)
        self.rpt = self.col = self.val = None


def spgemm(M, arpt, acol, aval, brpt, bcol, bval) -> RefResult:
    """C = A*B with OpSparse's kernels; arguments are device pointers (ints), FP64 values."""
    L = lib()
    rp, cp, vp = C.c_void_p(), C.c_void_p(), C.c_void_p()
    t = (C.c_double * 9)()
    bins = (C.c_int * 16)()
    fail = C.c_int(0)
    nnz = L.refgpu_spgemm(int(M), arpt, acol, aval, brpt, bcol, bval, C.byref(rp), C.byref(cp), C.byref(vp), t,
                          bins, C.byref(fail))
    if nnz < 0:
        raise RuntimeError("reference GPU spgemm: " + L.refgpu_error().decode())
    return RefResult(int(nnz), rp.value, cp.value, vp.value, t, bins, fail.value)
