"""The C ABI library builds, loads and exports what include/*.h declares
(CPU only: no kernel is launched)."""
import ctypes as C
import subprocess

import pytest

from relativistic_solver_hllc_gb300 import _native


def test_library_exports_every_header_symbol(native_lib):
    names = _native.header_symbols()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", str(_native.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in names:
        assert hasattr(native_lib, n)


def test_bindings_cover_header(native_lib):
    names = set(_native.header_symbols())
    bound = set(_native._SIGNATURES)
    unbound = {n for n in names if n.startswith("rts_batch") or n.startswith("rts_serve")
               or n.endswith("_noalloc")}
    assert names <= bound | unbound, sorted(names - bound - unbound)


def test_abi_version_and_null_handling(native_lib):
    assert native_lib.rts_abi_version() == 1
    assert native_lib.rts_ctx_destroy(None) == _native.OK
    assert native_lib.rts_last_error(None) == b""
    # calls on a null context are argument errors, never crashes
    assert native_lib.rts_wait(None, 0) == _native.ERR_INVALID_ARGUMENT
    assert native_lib.rts_set_hbm_budget(None, 1) == _native.ERR_INVALID_ARGUMENT
    assert native_lib.rts_scattering(None, None, None) == _native.ERR_INVALID_ARGUMENT


def test_context_without_device_reports_error(native_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present; the no-device path is exercised on CPU hosts only")
    h = C.c_void_p()
    rc = native_lib.rts_ctx_create(0, C.byref(h))
    assert rc == _native.ERR_CUDA
    assert not h.value
    with pytest.raises(_native.RtsError) as ei:
        _native.Context(0)
    assert ei.value.status == _native.ERR_CUDA
