"""The native library builds for sm_103a, loads without a GPU and exports
every function include/tncontract_gb300.h declares (no compute calls)."""
import ctypes
import shutil

import pytest


@pytest.fixture(scope="module")
def lib():
    if shutil.which("nvcc") is None and not __import__("os").path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("CUDA toolkit not available")
    import __graft_entry__
    __graft_entry__.build()
    from tncontract_gb300 import _lib
    return _lib


def test_exports_match_header(lib):
    names = lib.header_symbols()
    assert len(names) >= 20
    L = lib.lib()
    for n in names:
        assert hasattr(L, n), n
        assert n in lib.SIGNATURES, "no ctypes signature for %s" % n
    assert set(lib.SIGNATURES) == set(names)


def test_host_only_entry_points(lib):
    L = lib.lib()
    assert L.tnc_abi_version() == 1
    assert L.tnc_status_string(2).decode().startswith("Jacobi")
    sz = ctypes.c_size_t()
    assert L.tnc_svd_workspace_size(3, 512, 768, ctypes.byref(sz)) == 0 and sz.value > 512 * 768 * 16
    assert L.tnc_qr_workspace_size(1, 10, 4, ctypes.byref(sz)) == 0 and sz.value > 0
    assert L.tnc_qr_workspace_size(9, 10, 4, ctypes.byref(sz)) == lib.ERR_ARG
    assert lib.kernel_launches() >= 0


def test_no_cpu_fallback_without_library(monkeypatch, tmp_path):
    """Device ops fail loudly when the native library is missing."""
    from tncontract_gb300 import _build, _lib
    monkeypatch.setattr(_build, "LIBPATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_lib, "_LIB", None)
    with pytest.raises(RuntimeError, match="native library not built"):
        _lib.lib()
