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


def test_new_entry_points_validate_on_the_host():
    """Null or out-of-range arguments of every entry point beyond the reference's first table
    return a status and a message before any CUDA call."""
    import ctypes as C
    from svox2_gb300 import _lib
    lib = _lib.load()
    size = (C.c_int32 * 3)(4, 4, 4)
    cases = [
        (lambda: lib.svx_accel_dist_prop(None, size, None), _lib.SVX_ERR_INVALID, b"null"),
        (lambda: lib.svx_accel_dist_prop(None, None, None), _lib.SVX_ERR_INVALID, b"null"),
        (lambda: lib.svx_dilate(None, None, size, None), _lib.SVX_ERR_INVALID, b"null"),
        (lambda: lib.svx_tv(None, size, None, 0, 1, 1, C.c_float(2.0), 0, C.c_float(-1.0), C.c_float(-1.0), None,
                            None), _lib.SVX_ERR_UNSUPPORTED, b"logalpha"),
        (lambda: lib.svx_tv(None, size, None, 0, 1, 0, C.c_float(2.0), 0, C.c_float(-1.0), C.c_float(-1.0), None,
                            None), _lib.SVX_ERR_INVALID, b"null"),
        (lambda: lib.svx_add_accum(None, 26, 27, 10, None, None, None), _lib.SVX_ERR_INVALID, b"stride"),
        (lambda: lib.svx_ray_order(None, None, None, 0, None, None), _lib.SVX_ERR_INVALID, b"null"),
        (lambda: lib.svx_volume_render_expected_term(None, None, None, None, None), _lib.SVX_ERR_INVALID, b"null"),
        (lambda: lib.svx_volume_render_sigma_thresh(None, None, None, C.c_float(1.0), None, None),
         _lib.SVX_ERR_INVALID, b"null"),
        (lambda: lib.svx_grid_weight_render(None, size, None, C.c_float(0.5), C.c_float(0.0), 0, None, None, None,
                                            None), _lib.SVX_ERR_INVALID, b"null"),
        (lambda: lib.svx_camera_rays(None, None, None, None), _lib.SVX_ERR_INVALID, b"null"),
    ]
    for call, status, word in cases:
        assert call() == status, lib.svx_last_error()
        assert word in lib.svx_last_error()
