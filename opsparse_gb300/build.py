"""In-tree build of the GB300 SpGEMM library.

Produces, under ``opsparse_gb300/_build/``:
  * ``libopsparse_gb300.so`` — CUDA kernels + the C ABI of ``include/opsparse_gb300.h``
    (nvcc, ``-gencode arch=compute_103a,code=sm_103a`` only);
  * ``libopsparse.so`` — the C++ drop-in facade (``include/opsparse/...``: CSR,
    SpgemmMeta, SpgemmTimings, SpgemmPerf, opsparse_spgemm*) over the C ABI;
  * ``facade_selftest`` — a small C++ program exercising the facade (run by the GPU tests).

Sources are compiled in parallel; a stamp of the source contents skips unchanged builds.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _sources() -> dict[str, list[Path]]:
    return {
        "cuda": sorted(CSRC.glob("*.cu")),
        "facade": sorted((CSRC / "facade").glob("*.cpp")),
        "headers": sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.rglob("*.h*")),
        "selftest": [CSRC / "facade" / "selftest" / "facade_selftest.cpp"],
    }


def _stamp() -> str:
    h = hashlib.sha256()
    for group in _sources().values():
        for p in group:
            if p.exists():
                h.update(p.name.encode())
                h.update(p.read_bytes())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}")


def lib_path() -> Path:
    return OUT / "libopsparse_gb300.so"


def facade_path() -> Path:
    return OUT / "libopsparse.so"


def selftest_path() -> Path:
    return OUT / "facade_selftest"


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA/C++ artefact of the package; returns the C-ABI library path."""
    OUT.mkdir(parents=True, exist_ok=True)
    stamp = _stamp()
    stamp_file = OUT / "stamp.txt"
    wanted = [lib_path(), facade_path(), selftest_path()]
    if not force and stamp_file.exists() and stamp_file.read_text() == stamp and all(p.exists() for p in wanted):
        return lib_path()
    nvcc = _nvcc()
    cuda = _cuda_home()
    srcs = _sources()
    objs: list[Path] = []
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for src in srcs["cuda"]:
            obj = OUT / (src.stem + ".o")
            objs.append(obj)
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
            jobs.append(ex.submit(_run, cmd))
        fobjs: list[Path] = []
        for src in srcs["facade"]:
            obj = OUT / ("facade_" + src.stem + ".o")
            fobjs.append(obj)
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{INCLUDE}", f"-I{cuda / 'include'}", "-c", str(src),
                   "-o", str(obj)]
            jobs.append(ex.submit(_run, cmd))
        for j in jobs:
            j.result()
    cudart = cuda / "lib64"
    if not (cudart / "libcudart.so").exists():
        cudart = cuda / "targets" / ("sbsa-linux" if os.uname().machine == "aarch64" else "x86_64-linux") / "lib"
    _run([nvcc, *ARCH, "-shared", "-o", str(lib_path()), *map(str, objs), "-lcudart"])
    _run(["g++", "-shared", "-o", str(facade_path()), *map(str, fobjs), f"-L{OUT}", "-lopsparse_gb300",
          f"-L{cudart}", "-lcudart", f"-Wl,-rpath,{OUT}", f"-Wl,-rpath,{cudart}"])
    if srcs["selftest"][0].exists():
        _run(["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", f"-I{cuda / 'include'}", str(srcs["selftest"][0]),
              "-o", str(selftest_path()), f"-L{OUT}", "-lopsparse", "-lopsparse_gb300", f"-L{cudart}", "-lcudart",
              f"-Wl,-rpath,{OUT}", f"-Wl,-rpath,{cudart}"])
    stamp_file.write_text(stamp)
    if verbose:
        print(f"built {lib_path()}")
    return lib_path()


if __name__ == "__main__":
    build(force=True, verbose=True)
