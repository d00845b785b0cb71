"""ctypes binding of ``libsvox2_gb300.so`` (the C ABI in ``include/svox2_gb300.h``).

The structures below mirror the header field for field.  ``call`` invokes an
entry point and turns a non-zero status into ``RuntimeError`` carrying the
library's message, the way the reference's TORCH_CHECK failures surfaced.
There is no fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

from . import _build

ABI_VERSION = 3

SVX_OK = 0
SVX_ERR_INVALID = 1
SVX_ERR_UNSUPPORTED = 2
SVX_ERR_CUDA = 3
SVX_ERR_TOO_LARGE = 4

SVX_F32, SVX_BF16, SVX_F16 = 0, 1, 2
SVX_INDEX_ALL, SVX_INDEX_NONE, SVX_INDEX_MASK, SVX_INDEX_LIST = 0, 1, 2, 3


class SvxGrid(C.Structure):
    _fields_ = [
        ("density_data", C.c_void_p),
        ("sh_data", C.c_void_p),
        ("links", C.c_void_p),
        ("n_voxels", C.c_int64),
        ("size", C.c_int32 * 3),
        ("basis_dim", C.c_int32),
        ("sh_data_dim", C.c_int32),
        ("basis_type", C.c_int32),
        ("sh_dtype", C.c_int32),
        ("background_nlayers", C.c_int32),
        ("offset", C.c_float * 3),
        ("scaling", C.c_float * 3),
        ("background_links", C.c_void_p),
        ("background_data", C.c_void_p),
        ("background_capacity", C.c_int64),
        ("background_reso", C.c_int32),
    ]


class SvxRays(C.Structure):
    _fields_ = [("origins", C.c_void_p), ("dirs", C.c_void_p), ("n_rays", C.c_int64)]


class SvxCamera(C.Structure):
    _fields_ = [
        ("c2w", C.c_void_p),
        ("c2w_rows", C.c_int32),
        ("fx", C.c_float),
        ("fy", C.c_float),
        ("cx", C.c_float),
        ("cy", C.c_float),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("ndc_coeffx", C.c_float),
        ("ndc_coeffy", C.c_float),
    ]


class SvxRenderOpts(C.Structure):
    _fields_ = [
        ("background_brightness", C.c_float),
        ("step_size", C.c_float),
        ("sigma_thresh", C.c_float),
        ("stop_thresh", C.c_float),
        ("near_clip", C.c_float),
        ("use_spheric_clip", C.c_int32),
        ("last_sample_opaque", C.c_int32),
    ]


class SvxGridGrads(C.Structure):
    _fields_ = [("grad_density_out", C.c_void_p), ("grad_sh_out", C.c_void_p), ("mask_out", C.c_void_p),
                ("grad_background_out", C.c_void_p), ("mask_background_out", C.c_void_p)]


class SvxRenderStats(C.Structure):
    _fields_ = [("eval_samples", C.c_void_p), ("ray_trace", C.c_void_p), ("march_start", C.c_void_p),
                ("march_stop", C.c_void_p), ("background_samples", C.c_void_p)]


class SvxBatchGrid(C.Structure):
    _fields_ = [("grid", SvxGrid), ("grads", SvxGridGrads), ("accum", C.c_void_p), ("accum_stride", C.c_int32),
                ("norm", C.c_float), ("beta", C.c_float), ("sparsity", C.c_float)]


class SvxTable(C.Structure):
    _fields_ = [("data", C.c_void_p), ("dtype", C.c_int32), ("n_rows", C.c_int64), ("n_cols", C.c_int32)]


P = C.POINTER
_vp, _i32, _i64, _f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float

# name -> argtypes (restype is int for all but the three library queries)
SIGNATURES = {
    "svx_volume_render_cuvol": [P(SvxGrid), P(SvxRays), P(SvxRenderOpts), _vp, P(SvxRenderStats), _vp],
    "svx_volume_render_cuvol_image": [P(SvxGrid), P(SvxCamera), P(SvxRenderOpts), _vp, P(SvxRenderStats), _vp],
    "svx_volume_render_cuvol_backward": [P(SvxGrid), P(SvxRays), P(SvxRenderOpts), _vp, _vp, P(SvxGridGrads),
                                         P(SvxRenderStats), _vp],
    "svx_volume_render_cuvol_fused": [P(SvxGrid), P(SvxRays), P(SvxRenderOpts), _vp, _f32, _f32, _vp,
                                      P(SvxGridGrads), P(SvxRenderStats), _vp],
    "svx_volume_render_cuvol_fused_noalloc": [P(SvxGrid), P(SvxRays), P(SvxRenderOpts), _vp, _f32, _f32, _vp,
                                              P(SvxGridGrads), P(SvxRenderStats), _vp],
    "svx_render_batch": [_i32, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _i64, P(SvxRenderOpts), _vp, _vp,
                         _vp, _vp, _i64, _vp],
    "svx_batch_colour_cache_bytes": [_i32],
    "svx_batch_record_bytes": [_i64, _i32],
    "svx_ray_order": [P(SvxGrid), P(SvxRays), P(SvxRenderOpts), _i32, _vp, _vp],
    "svx_add_accum": [_vp, _i32, _i32, _i64, _vp, _vp, _vp],
    "svx_camera_rays": [P(SvxCamera), _vp, _vp, _vp],
    "svx_sample_grid": [P(SvxGrid), _vp, _i64, _i32, _vp, _vp, _vp],
    "svx_sample_grid_backward": [P(SvxGrid), _vp, _i64, _vp, _vp, _vp, _vp, _i32, _vp],
    "svx_accel_dist_prop": [_vp, P(_i32), _vp],
    "svx_dilate": [_vp, _vp, P(_i32), _vp],
    "svx_grid_weight_render": [_vp, P(_i32), P(SvxCamera), _f32, _f32, _i32, P(_f32), P(_f32), _vp, _vp],
    "svx_volume_render_expected_term": [P(SvxGrid), P(SvxRays), P(SvxRenderOpts), _vp, _vp],
    "svx_volume_render_sigma_thresh": [P(SvxGrid), P(SvxRays), P(SvxRenderOpts), _f32, _vp, _vp],
    "svx_tv": [_vp, P(_i32), P(SvxTable), _i32, _i32, _i32, _f32, _i32, _f32, _f32, _vp, _vp],
    "svx_tv_grad": [_vp, P(_i32), P(SvxTable), _i32, _i32, _f32, _i32, _f32, _i32, _f32, _f32, _vp, _vp],
    "svx_tv_grad_sparse": [_vp, P(_i32), P(SvxTable), _vp, _i64, _vp, _i32, _i32, _f32, _i32, _f32, _i32,
                           _i32, _f32, _f32, _vp, _vp],
    "svx_msi_tv_grad_sparse": [_vp, _i32, _vp, _i64, _i32, _i32, _vp, _i64, _vp, _f32, _f32, _vp, _vp],
    "svx_rmsprop_step": [_vp, _i32, _vp, _vp, _i64, _i32, _i32, _vp, _i64, _f32, _f32, _f32, _f32, _f32, _vp],
    "svx_sgd_step": [_vp, _i32, _vp, _i64, _i32, _i32, _vp, _i64, _f32, _f32, _vp],
    "svx_last_error": [],
    "svx_abi_version": [],
    "svx_color_cache_capacity": [],
}

_lib = None
_lock = threading.Lock()


def library_path() -> Path:
    return Path(os.environ.get("SVOX2_GB300_LIB", str(_build.LIB_PATH)))


def load() -> C.CDLL:
    """Load the CUDA library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not path.exists():
            raise ImportError(
                f"svox2_gb300 CUDA library not found at {path}; build it with "
                "`python -m svox2_gb300._build` (or __graft_entry__.build()). "
                "There is no CPU fallback."
            )
        lib = C.CDLL(str(path))
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = (C.c_char_p if name == "svx_last_error" else
                          C.c_int64 if name in ("svx_batch_colour_cache_bytes", "svx_batch_record_bytes")
                          else C.c_int)
        v = lib.svx_abi_version()
        if v != ABI_VERSION:
            raise ImportError(f"libsvox2_gb300 ABI version {v}, expected {ABI_VERSION}; rebuild the library")
        _lib = lib
        return lib


def call(name: str, *args) -> None:
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != SVX_OK:
        msg = lib.svx_last_error().decode(errors="replace")
        raise RuntimeError(f"{name}: {msg} (status {rc})")
