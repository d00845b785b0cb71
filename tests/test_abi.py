"""The C-ABI library loads without a GPU and exports every entry point that
include/svox2_gb300.h declares (no compute calls here)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "svox2_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(svx_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_operator_surface():
    names = declared_functions()
    for op in ("volume_render_cuvol", "volume_render_cuvol_image", "volume_render_cuvol_backward",
               "volume_render_cuvol_fused", "sample_grid", "sample_grid_backward", "tv_grad", "tv_grad_sparse",
               "rmsprop_step", "sgd_step"):
        assert "svx_" + op in names


def test_library_exports_every_declared_symbol():
    from svox2_gb300 import _build, _lib
    _build.build()
    lib = ctypes.CDLL(str(_lib.library_path()))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    assert lib.svx_abi_version() == _lib.ABI_VERSION
    # every declared function has a ctypes signature in the Python binding
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_errors_are_reported_without_a_gpu():
    from svox2_gb300 import _lib
    lib = _lib.load()
    # invalid arguments are rejected on the host before any CUDA call
    rc = lib.svx_volume_render_cuvol(None, None, None, None, None, None)
    assert rc == _lib.SVX_ERR_INVALID
    assert b"null" in lib.svx_last_error()
    rc = lib.svx_rmsprop_step(None, 0, None, None, 10, 3, 9, None, 0, 0.9, 1.0, 1e-8, -1e9, -1.0, None)
    assert rc == _lib.SVX_ERR_INVALID
