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


def test_argument_checks_before_any_launch(lib):
    """The entry points added for the sweep's core refuse bad arguments on the
    host, before touching the device (non-null dummy pointers never
    dereferenced): a tall input to the double-float finish, a type it does
    not take, a short workspace, a negative stage-stop tolerance, an aliased
    row sort, a negative row count."""
    L = lib.lib()
    d = ctypes.c_void_p(16)  # never dereferenced: every call below fails its checks first
    ws = ctypes.c_void_p(32)
    sz = ctypes.c_size_t()
    assert L.tnc_svd_rows_workspace_size(lib.C128, 8, 16, ctypes.byref(sz)) == 0
    # double-float finish: m > n, FP64 input, too small a workspace
    assert L.tnc_svd_rows_df(lib.C64, 16, 8, d, d, d, d, 0, 0.0, 0, 16, ws, sz.value, d, None) == lib.ERR_ARG
    assert L.tnc_svd_rows_df(lib.C128, 8, 16, d, d, d, d, 0, 0.0, 0, 8, ws, sz.value, d, None) == lib.ERR_ARG
    assert L.tnc_svd_rows_df(lib.C64, 8, 16, d, d, d, d, 0, 0.0, 0, 8, ws, 16, d, None) == lib.ERR_WORKSPACE
    assert L.tnc_svd_rows_df(lib.C64, 8, 16, d, d, d, d, 0, 0.0, 0, -1, ws, sz.value, d, None) == lib.ERR_ARG
    # staged Jacobi: negative (or NaN) stop tolerance
    assert L.tnc_svd_rows_stage(lib.C64, 8, 16, d, d, d, d, 0, 0.0, -1.0, 0, ws, sz.value, d, None) == lib.ERR_ARG
    assert L.tnc_svd_rows_stage(lib.C64, 8, 16, d, d, d, d, 0, 0.0, float("nan"), 0, ws, sz.value, d,
                                None) == lib.ERR_ARG
    # kept-row Jacobi: negative nkeep
    assert L.tnc_svd_rows_keep(lib.C64, 8, 16, d, d, d, d, 0, 0.0, 0, -1, ws, sz.value, d, None) == lib.ERR_ARG
    # row sort: source and destination the same buffer; permute: negative count, aliasing
    assert L.tnc_sort_rows(lib.C64, 8, 16, d, d, d, d, d, None) == lib.ERR_ARG
    assert L.tnc_sort_rows(lib.C64, (1 << 16) + 1, 16, d, ws, d, d, d, None) == lib.ERR_ARG
    assert L.tnc_permute_rows(lib.C64, -1, 16, d, d, ws, None) == lib.ERR_ARG
    assert L.tnc_permute_rows(lib.C64, 4, 16, d, d, d, None) == lib.ERR_ARG
    assert L.tnc_permute_rows(lib.C64, 0, 16, d, d, ws, None) == lib.OK  # nothing to do
