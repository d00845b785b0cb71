"""numpy front end of the CPU oracle (liboracle.so) — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU arms import this
module; the svox2_gb300 product never does.  Every function takes numpy
arrays (float32 grid tables, int32 links, float32 rays) and returns numpy
results in the requested precision ("f32" = the reference's float arithmetic,
"f64" = the double-precision yardstick).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import build as _build

_lib = None


class OGrid(C.Structure):
    _fields_ = [("links", C.c_void_p), ("density", C.c_void_p), ("sh", C.c_void_p), ("n_voxels", C.c_int64),
                ("size", C.c_int * 3), ("basis_dim", C.c_int), ("offset", C.c_float * 3),
                ("scaling", C.c_float * 3), ("bg_links", C.c_void_p), ("bg_data", C.c_void_p), ("bg_reso", C.c_int),
                ("bg_nlayers", C.c_int)]


class OOpt(C.Structure):
    _fields_ = [("bg", C.c_float), ("step", C.c_float), ("sigma_thresh", C.c_float), ("stop_thresh", C.c_float),
                ("near_clip", C.c_float), ("spheric", C.c_int), ("last_opaque", C.c_int), ("bg_cpu", C.c_int)]


class OCam(C.Structure):
    _fields_ = [("c2w", C.c_void_p), ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("width", C.c_int), ("height", C.c_int), ("ndcx", C.c_float), ("ndcy", C.c_float)]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(_build.build()))
    return _lib


@dataclass
class Grid:
    """Grid tables in the reference layout (numpy, float32 / int32)."""
    links: np.ndarray          # int32 [X, Y, Z]
    density: np.ndarray        # float32 [N, 1] or [N]
    sh: np.ndarray             # float32 [N, 3*bd]
    basis_dim: int
    offset: tuple              # grid = world * scaling + offset (the reference's _to_cpp transform)
    scaling: tuple
    bg_links: Optional[np.ndarray] = None   # int32 [2 * reso, reso]: MSI background (None: none)
    bg_data: Optional[np.ndarray] = None    # float32 [capacity, nlayers, 4]

    def struct(self) -> OGrid:
        self.links = np.ascontiguousarray(self.links, dtype=np.int32)
        self.density = np.ascontiguousarray(self.density, dtype=np.float32)
        self.sh = np.ascontiguousarray(self.sh, dtype=np.float32)
        g = OGrid()
        if self.bg_links is not None and self.bg_links.size > 0:
            self.bg_links = np.ascontiguousarray(self.bg_links, dtype=np.int32)
            self.bg_data = np.ascontiguousarray(self.bg_data, dtype=np.float32)
            assert self.bg_data.ndim == 3 and self.bg_data.shape[2] == 4 and self.bg_data.shape[1] >= 2
            g.bg_links = self.bg_links.ctypes.data
            g.bg_data = self.bg_data.ctypes.data
            g.bg_reso = self.bg_links.shape[1]
            g.bg_nlayers = self.bg_data.shape[1]
        g.links = self.links.ctypes.data
        g.density = self.density.ctypes.data
        g.sh = self.sh.ctypes.data
        g.n_voxels = self.density.shape[0]
        g.size = (C.c_int * 3)(*self.links.shape)
        g.basis_dim = self.basis_dim
        g.offset = (C.c_float * 3)(*[float(v) for v in self.offset])
        g.scaling = (C.c_float * 3)(*[float(v) for v in self.scaling])
        return g


@dataclass
class Opt:
    background_brightness: float = 1.0
    step_size: float = 0.5
    sigma_thresh: float = 1e-10
    stop_thresh: float = 1e-7
    near_clip: float = 0.0
    use_spheric_clip: bool = False
    last_sample_opaque: bool = False
    bg_cpu_semantics: bool = False   # MSI background as the reference's pure-PyTorch path computes it

    def struct(self) -> OOpt:
        return OOpt(self.background_brightness, self.step_size, self.sigma_thresh, self.stop_thresh,
                    self.near_clip, int(self.use_spheric_clip), int(self.last_sample_opaque),
                    int(self.bg_cpu_semantics))


def _real(prec: str):
    if prec not in ("f32", "f64"):
        raise ValueError("prec must be 'f32' or 'f64'")
    return np.float32 if prec == "f32" else np.float64


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def default_threads() -> int:
    return int(os.environ.get("ORACLE_THREADS", os.cpu_count() or 1))


def render(grid: Grid, opt: Opt, origins, dirs, mode: int = 0, rgb_gt=None, grad_out=None, color=None,
           beta_loss: float = 0.0, sparsity_loss: float = 0.0, prec: str = "f32", want_grads: bool = True,
           want_mask: bool = True, trace: bool = False, nthreads: Optional[int] = None,
           stops=None, want_magnitude: bool = False) -> dict:
    """volume_render_cuvol (mode 0), _fused (1), _backward (2, color = forward colour).
    With an MSI background the result also holds grad_background [capacity, nlayers, 4] and,
    in mode 1, mask_background [capacity, nlayers].

    The result's "stops" holds each ray's early-stop count (-1: no early stop).  Passing a
    float run's "stops" back in (stops=...) makes every ray stop where that run stopped, so that
    a "f64" run evaluates exactly the float run's samples (the sampling geometry is float in
    both precisions).  want_magnitude adds "mag_density" / "mag_sh": per gradient entry, the
    sum of the absolute values of the terms that make it up (the scale of float rounding)."""
    R = _real(prec)
    origins = np.ascontiguousarray(origins, dtype=np.float32)
    dirs = np.ascontiguousarray(dirs, dtype=np.float32)
    Q = origins.shape[0]
    N = grid.density.shape[0]
    Cc = 3 * grid.basis_dim
    rgb = np.zeros((Q, 3), dtype=R) if color is None else np.ascontiguousarray(color, dtype=R).copy()
    gd = np.zeros((N, 1), dtype=R) if (mode and want_grads) else None
    gs = np.zeros((N, Cc), dtype=R) if (mode and want_grads) else None
    mask = np.zeros((N,), dtype=np.uint8) if (mode == 1 and want_mask) else None
    tr = np.zeros((Q,), dtype=np.uint64) if trace else None
    ne = np.zeros((1,), dtype=np.uint64)
    nb = np.zeros((1,), dtype=np.uint64)
    has_bg = grid.bg_links is not None and grid.bg_links.size > 0
    gbg = np.zeros(grid.bg_data.shape, dtype=R) if (has_bg and mode and want_grads) else None
    mbg = np.zeros(grid.bg_data.shape[:2], dtype=np.uint8) if (has_bg and mode == 1 and want_mask) else None
    gt = None if rgb_gt is None else np.ascontiguousarray(rgb_gt, dtype=np.float32)
    go = None if grad_out is None else np.ascontiguousarray(grad_out, dtype=np.float32)
    st_out = np.full((Q,), -1, dtype=np.int32) if mode in (0, 1) else None
    st_in = None if stops is None else np.ascontiguousarray(stops, dtype=np.int32)
    if st_in is not None and st_in.shape != (Q,):
        raise ValueError("stops must hold one entry per ray")
    md = np.zeros((N, 1), dtype=R) if (mode and want_magnitude) else None
    ms = np.zeros((N, Cc), dtype=R) if (mode and want_magnitude) else None
    g = grid.struct()
    o = opt.struct()
    fn = getattr(lib(), "oracle_render_" + prec)
    fn.restype = None
    fn(C.byref(g), C.byref(o), C.c_void_p(_p(origins)), C.c_void_p(_p(dirs)), C.c_int64(Q), C.c_int(mode),
       C.c_void_p(_p(gt)), C.c_void_p(_p(go)), C.c_float(beta_loss), C.c_float(sparsity_loss),
       C.c_void_p(_p(rgb)), C.c_void_p(_p(gd)), C.c_void_p(_p(gs)), C.c_void_p(_p(mask)), C.c_void_p(_p(gbg)),
       C.c_void_p(_p(mbg)), C.c_void_p(_p(tr)), C.c_void_p(_p(ne)), C.c_void_p(_p(nb)),
       C.c_int(nthreads or default_threads()), C.c_void_p(_p(st_out)), C.c_void_p(_p(st_in)),
       C.c_void_p(_p(md)), C.c_void_p(_p(ms)))
    return {"rgb": rgb, "grad_density": gd, "grad_sh": gs, "mask": None if mask is None else mask.astype(bool),
            "grad_background": gbg, "mask_background": None if mbg is None else mbg.astype(bool),
            "trace": tr, "n_eval": int(ne[0]), "n_background": int(nb[0]), "stops": st_out,
            "mag_density": md, "mag_sh": ms}


def render_image(grid: Grid, opt: Opt, c2w, fx, fy, cx, cy, width, height, ndc=(-1.0, -1.0), prec="f32",
                 trace=False, nthreads=None) -> dict:
    R = _real(prec)
    c2w = np.ascontiguousarray(np.asarray(c2w, dtype=np.float32)[:3, :4])
    cam = OCam(c2w.ctypes.data, fx, fy, cx, cy, width, height, ndc[0], ndc[1])
    out = np.zeros((height, width, 3), dtype=R)
    tr = np.zeros((height * width,), dtype=np.uint64) if trace else None
    g = grid.struct()
    o = opt.struct()
    fn = getattr(lib(), "oracle_render_image_" + prec)
    fn.restype = None
    fn(C.byref(g), C.byref(o), C.byref(cam), C.c_void_p(out.ctypes.data), C.c_void_p(_p(tr)),
       C.c_int(nthreads or default_threads()))
    return {"rgb": out, "trace": tr}


def sample(grid: Grid, points, want_colors=True, prec="f32"):
    R = _real(prec)
    pts = np.ascontiguousarray(points, dtype=np.float32)
    P = pts.shape[0]
    d = np.zeros((P, 1), dtype=R)
    s = np.zeros((P, 3 * grid.basis_dim), dtype=R)
    g = grid.struct()
    fn = getattr(lib(), "oracle_sample_" + prec)
    fn.restype = None
    fn(C.byref(g), C.c_void_p(pts.ctypes.data), C.c_int64(P), C.c_int(int(want_colors)), C.c_void_p(d.ctypes.data),
       C.c_void_p(s.ctypes.data))
    return d, s


def sample_backward(grid: Grid, points, grad_d, grad_sh, want_colors=True, prec="f32"):
    R = _real(prec)
    pts = np.ascontiguousarray(points, dtype=np.float32)
    P = pts.shape[0]
    gd_in = np.ascontiguousarray(grad_d, dtype=np.float32)
    gs_in = np.ascontiguousarray(grad_sh, dtype=np.float32)
    N = grid.density.shape[0]
    od = np.zeros((N, 1), dtype=R)
    os_ = np.zeros((N, 3 * grid.basis_dim), dtype=R)
    g = grid.struct()
    fn = getattr(lib(), "oracle_sample_backward_" + prec)
    fn.restype = None
    fn(C.byref(g), C.c_void_p(pts.ctypes.data), C.c_int64(P), C.c_int(int(want_colors)),
       C.c_void_p(gd_in.ctypes.data), C.c_void_p(gs_in.ctypes.data), C.c_void_p(od.ctypes.data),
       C.c_void_p(os_.ctypes.data))
    return od, os_


def tv_grad(links, data, start, end, scale, ignore_edge, cells=None, ignore_last_z=False, grad=None, mask=None,
            prec="f32"):
    """tv_grad (cells None) or tv_grad_sparse; accumulates into grad (returned) and mask."""
    R = _real(prec)
    links = np.ascontiguousarray(links, dtype=np.int32)
    data = np.ascontiguousarray(data, dtype=np.float32)
    grad = np.zeros(data.shape, dtype=R) if grad is None else grad
    cl = None if cells is None else np.ascontiguousarray(cells, dtype=np.int32)
    size = (C.c_int * 3)(*links.shape)
    fn = getattr(lib(), "oracle_tv_grad_" + prec)
    fn.restype = None
    fn(C.c_void_p(links.ctypes.data), size, C.c_void_p(data.ctypes.data), C.c_int64(data.shape[0]),
       C.c_int(data.shape[1]), C.c_void_p(_p(cl)), C.c_int64(0 if cl is None else cl.shape[0]), C.c_int(start),
       C.c_int(end), C.c_float(scale), C.c_int(int(ignore_edge)), C.c_int(int(ignore_last_z)),
       C.c_void_p(grad.ctypes.data), C.c_void_p(_p(mask)))
    return grad


def optim(rmsprop: bool, data, rms, grad, kind: int, indexer=None, beta=0.9, lr=1.0, eps=1e-8, minval=-1e9,
          lr_last=-1.0, prec="f32"):
    """rmsprop_step / sgd_step on copies; kind 0 all, 1 none, 2 mask, 3 index list."""
    R = _real(prec)
    data = np.ascontiguousarray(data, dtype=R).copy()
    grad = np.ascontiguousarray(grad, dtype=R).copy()
    rms = None if rms is None else np.ascontiguousarray(rms, dtype=R).copy()
    mask = np.ascontiguousarray(indexer, dtype=np.uint8) if kind == 2 else None
    index = np.ascontiguousarray(indexer, dtype=np.int64) if kind == 3 else None
    fn = getattr(lib(), "oracle_optim_" + prec)
    fn.restype = None
    fn(C.c_int(int(rmsprop)), C.c_void_p(data.ctypes.data), C.c_void_p(_p(rms)), C.c_void_p(grad.ctypes.data),
       C.c_int64(data.shape[0]), C.c_int(data.shape[1]), C.c_int(kind), C.c_void_p(_p(mask)),
       C.c_void_p(_p(index)), C.c_int64(0 if index is None else index.shape[0]), C.c_float(beta), C.c_float(lr),
       C.c_float(eps), C.c_float(minval), C.c_float(lr_last))
    return data, rms, grad


def accel_dist_prop(links: np.ndarray) -> np.ndarray:
    """accel_dist_prop on a copy of an int32 [X, Y, Z] links table; returns the new links."""
    out = np.ascontiguousarray(links, dtype=np.int32).copy()
    size = (C.c_int * 3)(*out.shape)
    fn = lib().oracle_accel_dist_prop
    fn.restype = None
    fn(C.c_void_p(out.ctypes.data), size)
    return out


def render_depth(grid: Grid, opt: Opt, origins, dirs, sigma_thresh=None, prec="f32", nthreads=None):
    """volume_render_expected_term (sigma_thresh None) or volume_render_sigma_thresh: [Q]."""
    R = _real(prec)
    o = np.ascontiguousarray(origins, dtype=np.float32)
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    out = np.zeros((o.shape[0],), dtype=R)
    fn = getattr(lib(), "oracle_render_depth_" + prec)
    fn.restype = None
    gs, os_ = grid.struct(), opt.struct()
    fn(C.byref(gs), C.byref(os_), C.c_void_p(o.ctypes.data), C.c_void_p(d.ctypes.data), C.c_int64(o.shape[0]),
       C.c_int(0 if sigma_thresh is None else 1), C.c_float(0.0 if sigma_thresh is None else sigma_thresh),
       C.c_void_p(out.ctypes.data), C.c_int(nthreads or default_threads()))
    return out


def dilate(mask: np.ndarray) -> np.ndarray:
    """dilate (svox2/csrc/misc_kernel.cu:20-48): OR over the 3x3x3 block around each voxel,
    clamped at the faces (numpy; boolean work, exact)."""
    m = np.ascontiguousarray(mask, dtype=bool)
    p = np.pad(m, 1, mode="edge")
    out = np.zeros_like(m)
    X, Y, Z = m.shape
    for a in range(3):
        for b in range(3):
            for c in range(3):
                out |= p[a:a + X, b:b + Y, c:c + Z]
    return out


def grid_weight_render(data, cam: dict, step_size, stop_thresh, last_opaque, offset, scaling, wmax=None,
                       prec="f32"):
    """grid_weight_render on a dense float32 density grid [X,Y,Z]; cam = dict(c2w [3|4,4], fx, fy,
    cx, cy, width, height).  Returns the raised wmax (a new array unless given)."""
    R = _real(prec)
    d = np.ascontiguousarray(data, dtype=np.float32)
    w = np.zeros(d.shape, dtype=R) if wmax is None else wmax
    c2w = np.ascontiguousarray(cam["c2w"], dtype=np.float32)
    oc = OCam(C.c_void_p(c2w.ctypes.data), cam["fx"], cam["fy"], cam["cx"], cam["cy"], cam["width"], cam["height"],
              -1.0, -1.0)
    fn = getattr(lib(), "oracle_grid_weight_render_" + prec)
    fn.restype = None
    fn(C.c_void_p(d.ctypes.data), (C.c_int * 3)(*d.shape), C.byref(oc), C.c_float(step_size),
       C.c_float(stop_thresh), C.c_int(int(last_opaque)), (C.c_float * 3)(*offset), (C.c_float * 3)(*scaling),
       C.c_void_p(w.ctypes.data))
    return w


def tv_value(links, data, start, end, ignore_edge, prec="f64"):
    """tv: the TV value of channels [start, end) of the float32 table data [N, C]."""
    links = np.ascontiguousarray(links, dtype=np.int32)
    data = np.ascontiguousarray(data, dtype=np.float32)
    fn = getattr(lib(), "oracle_tv_value_" + prec)
    fn.restype = C.c_double if prec == "f64" else C.c_float
    return float(fn(C.c_void_p(links.ctypes.data), (C.c_int * 3)(*links.shape), C.c_void_p(data.ctypes.data),
                    C.c_int(data.shape[1]), C.c_int(start), C.c_int(end), C.c_int(int(ignore_edge))))


def msi_tv_grad(links, msi, cells, scale, scale_last, grad=None, mask=None, prec="f32"):
    """msi_tv_grad_sparse: adds the MSI background's TV gradient over the listed cells to
    grad (float [capacity, nlayers, channels], returned) and sets mask [capacity, nlayers]."""
    R = _real(prec)
    links = np.ascontiguousarray(links, dtype=np.int32)
    msi = np.ascontiguousarray(msi, dtype=np.float32)
    cl = np.ascontiguousarray(cells, dtype=np.int32)
    grad = np.zeros(msi.shape, dtype=R) if grad is None else grad
    fn = getattr(lib(), "oracle_msi_tv_grad_" + prec)
    fn.restype = None
    fn(C.c_void_p(links.ctypes.data), C.c_int(links.shape[0]), C.c_int(links.shape[1]), C.c_void_p(msi.ctypes.data),
       C.c_int(msi.shape[1]), C.c_int(msi.shape[2]), C.c_void_p(cl.ctypes.data), C.c_int64(cl.shape[0]),
       C.c_float(scale), C.c_float(scale_last), C.c_void_p(grad.ctypes.data), C.c_void_p(_p(mask)))
    return grad
