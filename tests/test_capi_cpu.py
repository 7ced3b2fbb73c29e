"""Host-side checks of the C ABI library that need no GPU."""
import ctypes
import os

import pytest

import ugacc_gb300 as U


@pytest.fixture(scope="module")
def lib():
    from ugacc_gb300.build import build

    build()
    return U.load_library()


def test_library_exports_every_declared_symbol(lib):
    names = U.declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_status_strings_and_defaults(lib):
    assert lib.ucc_status_string(1).decode() == "Computation has not converged."
    o = U._Options()
    lib.ucc_options_default(ctypes.byref(o))
    assert o.maxiter == 100 and abs(o.r_convergence - 1e-7) < 1e-20 and o.diis == 1 and o.precision == 0


def test_null_arguments_are_rejected(lib):
    assert lib.ucc_ctx_destroy(None) == 4
    assert lib.ucc_ccsd(None, None, None) == 4
    assert lib.ucc_ctx_create(None, 0) == 4


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES", None) != "", reason="only meaningful with no GPU visible")
def test_context_creation_fails_cleanly_without_gpu(lib):
    h = ctypes.c_void_p()
    assert lib.ucc_ctx_create(ctypes.byref(h), 0) != 0


def test_no_cpu_fallback_when_library_missing(tmp_path):
    with pytest.raises(U.UccError):
        U._lib = None
        try:
            U.load_library(str(tmp_path / "missing.so"))
        finally:
            U._lib = None


def test_cpp_driver_usage_and_bad_input(tmp_path):
    import subprocess

    from ugacc_gb300.build import DRIVER, build

    build()
    r = subprocess.run([DRIVER], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"NOPE" + b"\0" * 64)
    r = subprocess.run([DRIVER, str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "not a synthetic Hamiltonian file" in r.stderr
