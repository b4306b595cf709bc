"""CPU-only checks of the C ABI boundary: the shared libraries build and load without a
GPU, and export every function that include/opsparse_gb300.h declares."""
import ctypes
import subprocess
from pathlib import Path

import pytest

from opsparse_gb300 import build as B
from opsparse_gb300 import capi


@pytest.fixture(scope="module")
def built():
    B.build()
    return B


def test_header_symbols_exported(built):
    names = capi.header_symbols()
    assert "ops_spgemm" in names and "ops_handle_create" in names
    lib = ctypes.CDLL(str(built.lib_path()))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(built.lib_path())], capture_output=True, text=True).stdout
    for n in names:
        assert f" T {n}" in out, n


def test_every_export_is_declared(built):
    out = subprocess.run(["nm", "-D", "--defined-only", str(built.lib_path())], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T ops_" in line}
    assert exported == set(capi.header_symbols())


def test_typed_binding_loads(built):
    lib = capi.load()
    assert lib.ops_version().decode().startswith("opsparse_gb300")
    assert lib.ops_status_string(0) == b"ok"
    assert lib.ops_status_string(2) == b"int32_overflow"


def test_facade_library_loads(built):
    lib = ctypes.CDLL(str(built.facade_path()))
    out = subprocess.run(["nm", "-D", "-C", "--defined-only", str(built.facade_path())], capture_output=True,
                         text=True).stdout
    for sym in ("opsparse::opsparse_spgemm(", "opsparse::opsparse_spgemm_reg(", "opsparse::opsparse_spgemm_safe(",
                "opsparse::CSR::construct(", "opsparse::SpgemmTimings::print(", "opsparse::compute_flop("):
        assert sym in out, sym
    assert lib is not None


def test_no_device_work_without_gpu(built):
    """Creating a handle needs a device: without one the call fails with a status code
    instead of crashing or falling back to the CPU."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = capi.load()
    h = ctypes.c_void_p()
    assert lib.ops_handle_create(ctypes.byref(h)) == capi.OPS_CUDA_ERROR


def test_reference_benchmark_drivers_compile_against_dropin(built, tmp_path):
    """OpSparse's own benchmark drivers (benchmarks/opsparse_profile.cu, opsparse_reg.cu)
    compile and link unchanged against include/opsparse/ and libopsparse.so (recipe:
    oracle/dropin_check/Makefile)."""
    from oracle.ref import has_sources, make_vars

    recipe = Path(__file__).resolve().parents[1] / "oracle" / "dropin_check"
    if not has_sources(recipe):
        pytest.skip("OpSparse sources not present")
    res = subprocess.run(["make", "-s", "-C", str(recipe), *make_vars(), f"NVCC={built._nvcc()}",
                          f"INCLUDE={built.INCLUDE}", f"LIBDIR={built.OUT}", f"OUT={tmp_path}"],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    for name in ("opsparse_profile", "opsparse_reg"):
        assert (tmp_path / name).exists()
