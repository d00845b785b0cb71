"""Operator surface of the reference's ``svox2.csrc`` extension, on the C ABI.

Same function names, argument order and meaning, and the same spec classes
with the same read-write fields as the pybind11 module (svox2/csrc/svox2.cpp:
declarations 11-72, table 74-112, classes 114-171).  Tensors are validated
the way ``SparseGridSpec::check()`` and friends did (svox2/csrc/include/
data_spec.hpp:32-112) and failures raise ``RuntimeError``.  Every op launches
on the current PyTorch stream of the data's device and never synchronises
the host (the reference used the legacy default stream, and ``sample_grid``
created and synchronised two private streams per call).

Operators this library leaves out (the nvol/svox1 backends, lumisphere TV)
are not exported, so ``name in csrc.__dict__`` checks like the reference's
``volume_render_image`` dispatch behave as with a module that lacks them.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import torch

from .. import _lib

__all__ = [
    "SparseGridSpec", "RaysSpec", "CameraSpec", "RenderOptions", "GridOutputGrads",
    "volume_render_cuvol", "volume_render_cuvol_image", "volume_render_cuvol_backward",
    "volume_render_cuvol_fused", "sample_grid", "sample_grid_backward", "tv_grad",
    "tv_grad_sparse", "rmsprop_step", "sgd_step", "accel_dist_prop", "volume_render_expected_term",
    "volume_render_sigma_thresh", "dilate", "grid_weight_render", "tv", "msi_tv_grad_sparse",
]

_DTYPES = {torch.float32: _lib.SVX_F32, torch.bfloat16: _lib.SVX_BF16, torch.float16: _lib.SVX_F16}


# ---------------------------------------------------------------- spec classes

class SparseGridSpec:
    """svox2/csrc/include/data_spec.hpp:18-52."""

    def __init__(self):
        self.density_data: Optional[torch.Tensor] = None
        self.sh_data: Optional[torch.Tensor] = None
        self.links: Optional[torch.Tensor] = None
        self._offset: Optional[torch.Tensor] = None
        self._scaling: Optional[torch.Tensor] = None
        self.background_links: Optional[torch.Tensor] = None
        self.background_data: Optional[torch.Tensor] = None
        self.basis_dim: int = 0
        self.basis_type: int = 1
        self.basis_data: Optional[torch.Tensor] = None


class GridOutputGrads:
    """data_spec.hpp:54-81."""

    def __init__(self):
        self.grad_density_out: Optional[torch.Tensor] = None
        self.grad_sh_out: Optional[torch.Tensor] = None
        self.grad_basis_out: Optional[torch.Tensor] = None
        self.grad_background_out: Optional[torch.Tensor] = None
        self.mask_out: Optional[torch.Tensor] = None
        self.mask_background_out: Optional[torch.Tensor] = None


class CameraSpec:
    """data_spec.hpp:83-102."""

    def __init__(self):
        self.c2w: Optional[torch.Tensor] = None
        self.fx = self.fy = self.cx = self.cy = 0.0
        self.width = self.height = 0
        self.ndc_coeffx = self.ndc_coeffy = -1.0


class RaysSpec:
    """data_spec.hpp:104-113."""

    def __init__(self):
        self.origins: Optional[torch.Tensor] = None
        self.dirs: Optional[torch.Tensor] = None


class RenderOptions:
    """data_spec.hpp:115-135."""

    def __init__(self):
        self.background_brightness = 1.0
        self.step_size = 0.5
        self.sigma_thresh = 1e-10
        self.stop_thresh = 1e-7
        self.near_clip = 0.0
        self.use_spheric_clip = False
        self.last_sample_opaque = False


# ---------------------------------------------------------------- checks

def _check(cond: bool, msg: str) -> None:
    if not cond:
        raise RuntimeError(msg)


def _cuda_input(t: Optional[torch.Tensor], name: str) -> torch.Tensor:
    _check(t is not None, f"{name} must be defined")
    _check(t.is_cuda, f"{name} must be a CUDA tensor")
    _check(t.is_contiguous(), f"{name} must be contiguous")
    return t


def _cpu_input(t: Optional[torch.Tensor], name: str) -> torch.Tensor:
    _check(t is not None, f"{name} must be defined")
    _check(not t.is_cuda, f"{name} must be a CPU tensor")
    _check(t.is_contiguous(), f"{name} must be contiguous")
    return t


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _stream(dev: torch.device) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


def _grid_struct(grid: SparseGridSpec) -> _lib.SvxGrid:
    dens = _cuda_input(grid.density_data, "density_data")
    sh = _cuda_input(grid.sh_data, "sh_data")
    links = _cuda_input(grid.links, "links")
    off = _cpu_input(grid._offset, "_offset")
    scl = _cpu_input(grid._scaling, "_scaling")
    _check(dens.ndim == 2, "density_data must be 2-D")
    _check(sh.ndim == 2, "sh_data must be 2-D")
    _check(links.ndim == 3, "links must be 3-D")
    _check(links.dtype == torch.int32, "links must be int32")
    _check(dens.dtype == torch.float32, "density_data must be float32")
    _check(sh.dtype in _DTYPES, f"sh_data dtype {sh.dtype} not supported (float32, bfloat16, float16)")
    _check(dens.device == sh.device == links.device, "grid tensors must be on one device")
    _check(sh.size(0) == dens.size(0), "density_data and sh_data row counts differ")
    bl = grid.background_links
    has_bg = bl is not None and bl.numel() > 0
    if has_bg:
        # SparseGridSpec::check, data_spec.hpp:36-41, plus the kernel's 4 channels per layer
        bl = _cuda_input(bl, "background_links")
        bd = _cuda_input(grid.background_data, "background_data")
        _check(bl.ndim == 2 and bl.dtype == torch.int32, "background_links must be int32 [2 * reso, reso]")
        _check(bl.size(0) == 2 * bl.size(1), "background_links must be [2 * reso, reso]")
        _check(bd.ndim == 3 and bd.dtype == torch.float32, "background_data must be float32 [N, nlayers, 4]")
        _check(bd.size(2) == 4 and bd.size(1) >= 2, "background_data must have 4 channels and >= 2 layers")
        _check(bl.device == bd.device == links.device, "background tables must be on the grid's device")
    _check(off.numel() == 3 and scl.numel() == 3, "_offset and _scaling must have 3 elements")
    offv = off.to(torch.float32).tolist()
    sclv = scl.to(torch.float32).tolist()
    g = _lib.SvxGrid()
    g.density_data = dens.data_ptr()
    g.sh_data = sh.data_ptr()
    g.links = links.data_ptr()
    g.n_voxels = dens.size(0)
    g.size = (C.c_int32 * 3)(*links.shape)
    g.basis_dim = int(grid.basis_dim)
    g.sh_data_dim = sh.size(1)
    g.basis_type = int(grid.basis_type)
    g.sh_dtype = _DTYPES[sh.dtype]
    g.background_nlayers = 0
    g.offset = (C.c_float * 3)(*offv)
    g.scaling = (C.c_float * 3)(*sclv)
    if has_bg:
        g.background_nlayers = bd.size(1)
        g.background_links = bl.data_ptr()
        g.background_data = bd.data_ptr()
        g.background_capacity = bd.size(0)
        g.background_reso = bl.size(1)
    return g


def _rays_struct(rays: RaysSpec, dev: torch.device) -> _lib.SvxRays:
    o = _cuda_input(rays.origins, "origins")
    d = _cuda_input(rays.dirs, "dirs")
    _check(o.is_floating_point() and d.is_floating_point(), "rays must be floating point")
    _check(o.dtype == torch.float32 and d.dtype == torch.float32, "rays must be float32")
    _check(o.ndim == 2 and o.size(1) == 3 and d.shape == o.shape, "origins and dirs must be [Q, 3]")
    _check(o.device == dev and d.device == dev, "rays must be on the grid's device")
    return _lib.SvxRays(o.data_ptr(), d.data_ptr(), o.size(0))


def _opt_struct(opt: RenderOptions) -> _lib.SvxRenderOpts:
    return _lib.SvxRenderOpts(float(opt.background_brightness), float(opt.step_size), float(opt.sigma_thresh),
                              float(opt.stop_thresh), float(opt.near_clip), int(bool(opt.use_spheric_clip)),
                              int(bool(opt.last_sample_opaque)))


def _bg_shape(grid: SparseGridSpec, g: _lib.SvxGrid) -> Optional[Tuple[int, ...]]:
    return tuple(grid.background_data.shape) if g.background_nlayers > 0 else None


def _grads_struct(grads: GridOutputGrads, n_vox: int, C_: int, dev: torch.device,
                  with_mask: bool, bg_shape: Optional[Tuple[int, ...]] = None) -> _lib.SvxGridGrads:
    g = _lib.SvxGridGrads()
    if grads.grad_density_out is not None:
        t = _cuda_input(grads.grad_density_out, "grad_density_out")
        _check(t.dtype == torch.float32 and t.numel() == n_vox and t.device == dev,
               "grad_density_out must be float32 [N, 1] on the grid's device")
        g.grad_density_out = t.data_ptr()
    if grads.grad_sh_out is not None:
        t = _cuda_input(grads.grad_sh_out, "grad_sh_out")
        _check(t.dtype == torch.float32 and t.numel() == n_vox * C_ and t.device == dev,
               "grad_sh_out must be float32 [N, C] on the grid's device")
        g.grad_sh_out = t.data_ptr()
    if with_mask and grads.mask_out is not None and grads.mask_out.numel() > 0:
        t = _cuda_input(grads.mask_out, "mask_out")
        _check(t.dtype == torch.bool and t.numel() == n_vox and t.device == dev,
               "mask_out must be bool [N] on the grid's device")
        g.mask_out = t.data_ptr()
    if bg_shape is not None:
        if grads.grad_background_out is not None:
            t = _cuda_input(grads.grad_background_out, "grad_background_out")
            _check(t.dtype == torch.float32 and tuple(t.shape) == tuple(bg_shape) and t.device == dev,
                   "grad_background_out must be float32 shaped like background_data on the grid's device")
            g.grad_background_out = t.data_ptr()
        mb = grads.mask_background_out
        if mb is not None and mb.numel() > 0:
            t = _cuda_input(mb, "mask_background_out")
            _check(t.dtype == torch.bool and t.numel() == bg_shape[0] * bg_shape[1] and t.device == dev,
                   "mask_background_out must be bool [N, nlayers] on the grid's device")
            g.mask_background_out = t.data_ptr()
    return g


def _stats_struct(stats) -> Optional[C.POINTER(_lib.SvxRenderStats)]:
    if stats is None:
        return None
    s = _lib.SvxRenderStats()
    s.eval_samples = _ptr(stats.get("eval_samples"))
    s.ray_trace = _ptr(stats.get("ray_trace"))
    s.background_samples = _ptr(stats.get("background_samples"))
    # torch.cuda.Event objects (timing enabled) recorded around the ray-march kernel
    for key in ("march_start", "march_stop"):
        ev = stats.get(key)
        if ev is not None:
            if ev.cuda_event == 0:        # torch creates the event lazily on first record
                ev.record()
            setattr(s, key, ev.cuda_event)
    return C.byref(s)


# ---------------------------------------------------------------- rendering

def volume_render_cuvol(grid: SparseGridSpec, rays: RaysSpec, opt: RenderOptions, *, stats=None) -> torch.Tensor:
    """svox2/csrc/render_lerp_kernel_cuvol.cu:918-958: colours [Q, 3] of the rays."""
    g = _grid_struct(grid)
    dev = grid.sh_data.device
    r = _rays_struct(rays, dev)
    out = torch.empty_like(rays.origins)
    with torch.cuda.device(dev):
        _lib.call("svx_volume_render_cuvol", C.byref(g), C.byref(r), C.byref(_opt_struct(opt)),
                  out.data_ptr(), _stats_struct(stats), _stream(dev))
    return out


def volume_render_expected_term(grid: SparseGridSpec, rays: RaysSpec, opt: RenderOptions) -> torch.Tensor:
    """svox2/csrc/render_lerp_kernel_cuvol.cu:1154-1172: expected termination distance [Q]."""
    g = _grid_struct(grid)
    dev = grid.sh_data.device
    r = _rays_struct(rays, dev)
    out = torch.empty((rays.origins.size(0),), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        _lib.call("svx_volume_render_expected_term", C.byref(g), C.byref(r), C.byref(_opt_struct(opt)),
                  out.data_ptr(), _stream(dev))
    return out


def volume_render_sigma_thresh(grid: SparseGridSpec, rays: RaysSpec, opt: RenderOptions,
                               sigma_thresh: float) -> torch.Tensor:
    """svox2/csrc/render_lerp_kernel_cuvol.cu:1174-1195: distance of the first sample with
    sigma > sigma_thresh [Q] (0 if none)."""
    g = _grid_struct(grid)
    dev = grid.sh_data.device
    r = _rays_struct(rays, dev)
    out = torch.empty((rays.origins.size(0),), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        _lib.call("svx_volume_render_sigma_thresh", C.byref(g), C.byref(r), C.byref(_opt_struct(opt)),
                  float(sigma_thresh), out.data_ptr(), _stream(dev))
    return out


def _camera_struct(cam: CameraSpec) -> _lib.SvxCamera:
    c2w = _cuda_input(cam.c2w, "c2w")
    _check(c2w.is_floating_point() and c2w.ndim == 2 and c2w.size(1) == 4 and c2w.size(0) in (3, 4),
           "c2w must be float [3|4, 4]")
    _check(c2w.dtype == torch.float32, "c2w must be float32")
    return _lib.SvxCamera(c2w.data_ptr(), c2w.size(0), float(cam.fx), float(cam.fy), float(cam.cx), float(cam.cy),
                          int(cam.width), int(cam.height), float(cam.ndc_coeffx), float(cam.ndc_coeffy))


def volume_render_cuvol_image(grid: SparseGridSpec, cam: CameraSpec, opt: RenderOptions, *,
                              stats=None) -> torch.Tensor:
    """render_lerp_kernel_cuvol.cu:960-1008: image [H, W, 3] of a pinhole camera."""
    g = _grid_struct(grid)
    dev = grid.sh_data.device
    c = _camera_struct(cam)
    out = torch.empty((int(cam.height), int(cam.width), 3), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        _lib.call("svx_volume_render_cuvol_image", C.byref(g), C.byref(c), C.byref(_opt_struct(opt)),
                  out.data_ptr(), _stats_struct(stats), _stream(dev))
    return out


def volume_render_cuvol_backward(grid: SparseGridSpec, rays: RaysSpec, opt: RenderOptions,
                                 grad_out: torch.Tensor, color_cache: torch.Tensor,
                                 grads: GridOutputGrads, *, stats=None) -> None:
    """render_lerp_kernel_cuvol.cu:1010-1068: accumulate dL/dgrid for dL/drgb = grad_out."""
    g = _grid_struct(grid)
    dev = grid.sh_data.device
    r = _rays_struct(rays, dev)
    go = _cuda_input(grad_out, "grad_out")
    _check(go.dtype == torch.float32 and go.shape == rays.origins.shape, "grad_out must be float32 [Q, 3]")
    cc = None
    if color_cache is not None:
        cc = _cuda_input(color_cache, "color_cache")
    gg = _grads_struct(grads, g.n_voxels, g.sh_data_dim, dev, with_mask=False, bg_shape=_bg_shape(grid, g))
    with torch.cuda.device(dev):
        _lib.call("svx_volume_render_cuvol_backward", C.byref(g), C.byref(r), C.byref(_opt_struct(opt)),
                  go.data_ptr(), _ptr(cc), C.byref(gg), _stats_struct(stats), _stream(dev))


def volume_render_cuvol_fused(grid: SparseGridSpec, rays: RaysSpec, opt: RenderOptions,
                              rgb_gt: torch.Tensor, beta_loss: float, sparsity_loss: float,
                              rgb_out: torch.Tensor, grads: GridOutputGrads, *, stats=None) -> None:
    """render_lerp_kernel_cuvol.cu:1070-1152: render into rgb_out and accumulate the MSE gradient."""
    g = _grid_struct(grid)
    dev = grid.sh_data.device
    r = _rays_struct(rays, dev)
    gt = _cuda_input(rgb_gt, "rgb_gt")
    out = _cuda_input(rgb_out, "rgb_out")
    _check(gt.dtype == torch.float32 and gt.shape == rays.origins.shape, "rgb_gt must be float32 [Q, 3]")
    _check(out.dtype == torch.float32 and out.shape == rays.origins.shape, "rgb_out must be float32 [Q, 3]")
    gg = _grads_struct(grads, g.n_voxels, g.sh_data_dim, dev, with_mask=True, bg_shape=_bg_shape(grid, g))
    with torch.cuda.device(dev):
        _lib.call("svx_volume_render_cuvol_fused", C.byref(g), C.byref(r), C.byref(_opt_struct(opt)),
                  gt.data_ptr(), float(beta_loss), float(sparsity_loss), out.data_ptr(), C.byref(gg),
                  _stats_struct(stats), _stream(dev))


# ---------------------------------------------------------------- sampling

def sample_grid(grid: SparseGridSpec, points: torch.Tensor, want_colors: bool) -> Tuple[torch.Tensor, torch.Tensor]:
    """svox2/csrc/svox2_kernel.cu:181-217."""
    g = _grid_struct(grid)
    dev = grid.sh_data.device
    pts = _cuda_input(points, "points")
    _check(pts.ndim == 2 and pts.size(1) == 3 and pts.dtype == torch.float32, "points must be float32 [P, 3]")
    P = pts.size(0)
    out_d = torch.empty((P, grid.density_data.size(1)), dtype=pts.dtype, device=dev)
    out_sh = torch.empty((P if want_colors else 0, grid.sh_data.size(1)), dtype=pts.dtype, device=dev)
    with torch.cuda.device(dev):
        _lib.call("svx_sample_grid", C.byref(g), pts.data_ptr(), P, int(bool(want_colors)), out_d.data_ptr(),
                  out_sh.data_ptr() if want_colors and P > 0 else None, _stream(dev))
    return out_d, out_sh


def sample_grid_backward(grid: SparseGridSpec, points: torch.Tensor, grad_out_density: torch.Tensor,
                         grad_out_sh: torch.Tensor, grad_density_out: torch.Tensor,
                         grad_sh_out: torch.Tensor, want_colors: bool) -> None:
    """svox2/csrc/svox2_kernel.cu:219-267."""
    g = _grid_struct(grid)
    dev = grid.sh_data.device
    pts = _cuda_input(points, "points")
    gd = _cuda_input(grad_out_density, "grad_out_density")
    gs = _cuda_input(grad_out_sh, "grad_out_sh")
    od = _cuda_input(grad_density_out, "grad_density_out")
    osh = _cuda_input(grad_sh_out, "grad_sh_out")
    _check(pts.ndim == 2 and gd.ndim == 2 and gs.ndim == 2, "points and output grads must be 2-D")
    P = pts.size(0)
    _check(gd.numel() == P, "grad_out_density must be [P, 1]")
    _check(not want_colors or gs.numel() == P * g.sh_data_dim, "grad_out_sh must be [P, C]")
    _check(od.dtype == torch.float32 and osh.dtype == torch.float32, "gradient outputs must be float32")
    with torch.cuda.device(dev):
        _lib.call("svx_sample_grid_backward", C.byref(g), pts.data_ptr(), P, gd.data_ptr(),
                  gs.data_ptr() if want_colors else None, od.data_ptr(),
                  osh.data_ptr() if want_colors else None, int(bool(want_colors)), _stream(dev))


# ---------------------------------------------------------------- total variation

def _table(data: torch.Tensor, name: str) -> _lib.SvxTable:
    t = _cuda_input(data, name)
    _check(t.is_floating_point(), f"{name} must be floating point")
    _check(t.ndim == 2, f"{name} must be 2-D")
    _check(t.dtype in _DTYPES, f"{name} dtype {t.dtype} not supported")
    return _lib.SvxTable(t.data_ptr(), _DTYPES[t.dtype], t.size(0), t.size(1))


def _links_args(links: torch.Tensor):
    t = _cuda_input(links, "links")
    _check(not t.is_floating_point() and t.dtype == torch.int32, "links must be int32")
    _check(t.ndim == 3, "links must be 3-D")
    return t, (C.c_int32 * 3)(*t.shape)


def accel_dist_prop(grid: torch.Tensor) -> None:
    """svox2/csrc/misc_kernel.cu:356-416: empty-space skip levels written into the links
    table in place (negative entries become -(1 + empty pyramid levels above))."""
    lt, size = _links_args(grid)
    with torch.cuda.device(lt.device):
        _lib.call("svx_accel_dist_prop", lt.data_ptr(), size, _stream(lt.device))


def dilate(grid: torch.Tensor) -> torch.Tensor:
    """svox2/csrc/misc_kernel.cu:335-350: 3x3x3 dilation of a bool [X, Y, Z] CUDA mask."""
    t = _cuda_input(grid, "grid")
    _check(not t.is_floating_point() and t.dtype == torch.bool and t.ndim == 3, "grid must be a 3-D bool tensor")
    out = torch.empty_like(t)
    with torch.cuda.device(t.device):
        _lib.call("svx_dilate", t.data_ptr(), out.data_ptr(), (C.c_int32 * 3)(*t.shape), _stream(t.device))
    return out


def grid_weight_render(data: torch.Tensor, cam: CameraSpec, step_size: float, stop_thresh: float,
                       last_sample_opaque: bool, offset: torch.Tensor, scaling: torch.Tensor,
                       grid_weight: torch.Tensor) -> None:
    """svox2/csrc/misc_kernel.cu:418-448: raise grid_weight [X, Y, Z] to the largest rendering
    weight each voxel gets from the camera's rays through the dense density grid data."""
    d = _cuda_input(data, "data")
    w = _cuda_input(grid_weight, "grid_weight")
    _check(d.dtype == torch.float32 and d.ndim == 3, "data must be float32 [X, Y, Z]")
    _check(w.dtype == torch.float32 and w.shape == d.shape, "grid_weight must be float32 like data")
    off = [float(v) for v in torch.as_tensor(offset).reshape(-1).tolist()]
    scl = [float(v) for v in torch.as_tensor(scaling).reshape(-1).tolist()]
    _check(len(off) == 3 and len(scl) == 3, "offset and scaling must have 3 elements")
    c = _camera_struct(cam)
    with torch.cuda.device(d.device):
        _lib.call("svx_grid_weight_render", d.data_ptr(), (C.c_int32 * 3)(*d.shape), C.byref(c), float(step_size),
                  float(stop_thresh), int(bool(last_sample_opaque)), (C.c_float * 3)(*off), (C.c_float * 3)(*scl),
                  w.data_ptr(), _stream(d.device))


def tv(links: torch.Tensor, data: torch.Tensor, start_dim: int, end_dim: int, use_logalpha: bool,
       logalpha_delta: float, ignore_edge: bool, ndc_coeffx: float, ndc_coeffy: float) -> torch.Tensor:
    """svox2/csrc/loss_kernel.cu:483-515: the TV value (a 0-d float32 tensor on the data's device)."""
    lt, size = _links_args(links)
    tab = _table(data, "data")
    dev = data.device
    out = torch.empty((), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        _lib.call("svx_tv", lt.data_ptr(), size, C.byref(tab), int(start_dim), int(end_dim), int(bool(use_logalpha)),
                  float(logalpha_delta), int(bool(ignore_edge)), float(ndc_coeffx), float(ndc_coeffy),
                  out.data_ptr(), _stream(dev))
    return out


def tv_grad(links: torch.Tensor, data: torch.Tensor, start_dim: int, end_dim: int, scale: float,
            use_logalpha: bool, logalpha_delta: float, ignore_edge: bool, ndc_coeffx: float,
            ndc_coeffy: float, grad_data: torch.Tensor) -> None:
    """svox2/csrc/loss_kernel.cu:522-556."""
    lt, size = _links_args(links)
    tab = _table(data, "data")
    gd = _cuda_input(grad_data, "grad_data")
    _check(gd.is_floating_point() and gd.ndim == 2 and gd.dtype == torch.float32, "grad_data must be float32 2-D")
    _check(gd.shape == data.shape, "grad_data must match data")
    dev = data.device
    with torch.cuda.device(dev):
        _lib.call("svx_tv_grad", lt.data_ptr(), size, C.byref(tab), int(start_dim), int(end_dim), float(scale),
                  int(bool(use_logalpha)), float(logalpha_delta), int(bool(ignore_edge)), float(ndc_coeffx),
                  float(ndc_coeffy), gd.data_ptr(), _stream(dev))


def tv_grad_sparse(links: torch.Tensor, data: torch.Tensor, rand_cells: torch.Tensor, mask_out: torch.Tensor,
                   start_dim: int, end_dim: int, scale: float, use_logalpha: bool, logalpha_delta: float,
                   ignore_edge: bool, ignore_last_z: bool, ndc_coeffx: float, ndc_coeffy: float,
                   grad_data: torch.Tensor) -> None:
    """svox2/csrc/loss_kernel.cu:558-604."""
    lt, size = _links_args(links)
    tab = _table(data, "data")
    gd = _cuda_input(grad_data, "grad_data")
    rc = _cuda_input(rand_cells, "rand_cells")
    mk = _cuda_input(mask_out, "mask_out")
    _check(gd.is_floating_point() and gd.ndim == 2 and gd.dtype == torch.float32, "grad_data must be float32 2-D")
    _check(gd.shape == data.shape, "grad_data must match data")
    _check(rc.dtype == torch.int32 and rc.ndim == 1, "rand_cells must be int32 [n]")
    use_mask = mk.dim() > 0 and mk.numel() > 0
    if use_mask:
        _check(mk.dtype == torch.bool and mk.numel() == data.size(0), "mask_out must be bool [N]")
    dev = data.device
    with torch.cuda.device(dev):
        _lib.call("svx_tv_grad_sparse", lt.data_ptr(), size, C.byref(tab), rc.data_ptr(), rc.size(0),
                  mk.data_ptr() if use_mask else None, int(start_dim), int(end_dim), float(scale),
                  int(bool(use_logalpha)), float(logalpha_delta), int(bool(ignore_edge)),
                  int(bool(ignore_last_z)), float(ndc_coeffx), float(ndc_coeffy), gd.data_ptr(), _stream(dev))


def msi_tv_grad_sparse(links: torch.Tensor, msi: torch.Tensor, rand_cells: torch.Tensor, mask_out: torch.Tensor,
                       scale: float, scale_last: float, grad_msi: torch.Tensor) -> None:
    """svox2/csrc/loss_kernel.cu:606-641: TV gradient of the MSI background on a list of cells."""
    lk = _cuda_input(links, "links")
    m = _cuda_input(msi, "msi")
    rc = _cuda_input(rand_cells, "rand_cells")
    mk = _cuda_input(mask_out, "mask_out")
    gd = _cuda_input(grad_msi, "grad_msi")
    _check(lk.dtype == torch.int32 and lk.ndim == 2 and lk.size(0) == 2 * lk.size(1),
           "links must be int32 [2 * reso, reso]")
    _check(m.dtype == torch.float32 and m.ndim == 3, "msi must be float32 [N, nlayers, channels]")
    _check(gd.dtype == torch.float32 and gd.shape == m.shape, "grad_msi must be float32 shaped like msi")
    _check(rc.dtype == torch.int32 and rc.ndim == 1, "rand_cells must be int32 [n]")
    use_mask = mk.dim() > 0 and mk.size(0) > 0
    if use_mask:
        _check(mk.dtype == torch.bool and mk.numel() == m.size(0) * m.size(1), "mask_out must be bool [N, nlayers]")
    _check(lk.device == m.device == rc.device == gd.device, "tensors must be on one device")
    dev = m.device
    with torch.cuda.device(dev):
        _lib.call("svx_msi_tv_grad_sparse", lk.data_ptr(), lk.size(1), m.data_ptr(), m.size(0), m.size(1), m.size(2),
                  rc.data_ptr(), rc.size(0), mk.data_ptr() if use_mask else None, float(scale), float(scale_last),
                  gd.data_ptr(), _stream(dev))


# ---------------------------------------------------------------- optimisers

def _indexer_args(indexer: torch.Tensor, n_rows: int):
    ix = _cuda_input(indexer, "indexer")
    if ix.dim() == 0:
        return _lib.SVX_INDEX_ALL, None, 0
    if ix.size(0) == 0:
        return _lib.SVX_INDEX_NONE, None, 0
    if ix.dtype == torch.bool:
        _check(ix.numel() == n_rows, "bool indexer must have one entry per row")
        return _lib.SVX_INDEX_MASK, ix.data_ptr(), ix.numel()
    _check(ix.dtype == torch.int64 and ix.ndim == 1, "index indexer must be int64 [n]")
    return _lib.SVX_INDEX_LIST, ix.data_ptr(), ix.size(0)


def rmsprop_step(data: torch.Tensor, rms: torch.Tensor, grad: torch.Tensor, indexer: torch.Tensor, beta: float,
                 lr: float, epsilon: float, minval: float, lr_last: float) -> None:
    """svox2/csrc/optim_kernel.cu:154-218."""
    d = _cuda_input(data, "data")
    r = _cuda_input(rms, "rms")
    g = _cuda_input(grad, "grad")
    _check(d.ndim == 2 and r.shape == d.shape and g.shape == d.shape, "data, rms and grad must be [N, C]")
    _check(d.dtype in _DTYPES and r.dtype == torch.float32 and g.dtype == torch.float32,
           "rms and grad must be float32; data float32, bfloat16 or float16")
    kind, ip, n = _indexer_args(indexer, d.size(0))
    dev = d.device
    with torch.cuda.device(dev):
        _lib.call("svx_rmsprop_step", d.data_ptr(), _DTYPES[d.dtype], r.data_ptr(), g.data_ptr(), d.size(0),
                  d.size(1), kind, ip, n, float(beta), float(lr), float(epsilon), float(minval), float(lr_last),
                  _stream(dev))


def sgd_step(data: torch.Tensor, grad: torch.Tensor, indexer: torch.Tensor, lr: float, lr_last: float) -> None:
    """svox2/csrc/optim_kernel.cu:220-267."""
    d = _cuda_input(data, "data")
    g = _cuda_input(grad, "grad")
    _check(d.ndim == 2 and g.shape == d.shape, "data and grad must be [N, C]")
    _check(d.dtype in _DTYPES and g.dtype == torch.float32, "grad must be float32")
    kind, ip, n = _indexer_args(indexer, d.size(0))
    dev = d.device
    with torch.cuda.device(dev):
        _lib.call("svx_sgd_step", d.data_ptr(), _DTYPES[d.dtype], g.data_ptr(), d.size(0), d.size(1), kind, ip,
                  n, float(lr), float(lr_last), _stream(dev))
