"""Grid API of the reference (``svox2.SparseGrid`` and its companions) on the
GB300 kernels.

Classes and methods keep the reference's names, signatures, defaults and data
layout (svox2/svox2.py): ``links`` int32 [X, Y, Z], ``density_data`` float32
[N, 1], ``sh_data`` [N, 3 * basis_dim] channel-major per voxel, CPU
``radius``/``center``/``_offset``/``_scaling``.  Every operation runs on the
CUDA library; there is no CPU path — ``use_kernel=False`` and CPU grids raise.

Additions: ``sh_dtype`` (store SH coefficients as bfloat16 or float16; all
arithmetic stays float32, gradients and optimiser state are float32).
Left out (raise NotImplementedError): learned/MLP bases and their optimiser,
nvol/svox1 backends, resize, svox1 export and lumisphere TV.
"""
from __future__ import annotations

from dataclasses import dataclass
from functools import reduce
from typing import List, Optional, Tuple, Union

import numpy as np
import torch
from torch import autograd, nn

from . import csrc as _C
from . import utils
from .defs import BASIS_TYPE_3D_TEXTURE, BASIS_TYPE_MLP, BASIS_TYPE_SH


def _no_cpu_path(what: str):
    raise RuntimeError(f"{what}: svox2_gb300 has no CPU path; the grid and rays must be on a CUDA device")


@dataclass
class RenderOptions:
    """Rendering options (svox2/svox2.py:17-80); same fields and defaults."""

    backend: str = "cuvol"
    background_brightness: float = 1.0
    step_size: float = 0.5
    sigma_thresh: float = 1e-10
    stop_thresh: float = 1e-7
    last_sample_opaque: bool = False
    near_clip: float = 0.0
    use_spheric_clip: bool = False
    random_sigma_std: float = 1.0
    random_sigma_std_background: float = 1.0

    def _to_cpp(self, randomize: bool = False):
        if self.backend != "cuvol":
            raise NotImplementedError(f"backend {self.backend!r}: only 'cuvol' is built")
        opt = _C.RenderOptions()
        opt.background_brightness = self.background_brightness
        opt.step_size = self.step_size
        opt.sigma_thresh = self.sigma_thresh
        opt.stop_thresh = self.stop_thresh
        opt.near_clip = self.near_clip
        opt.use_spheric_clip = self.use_spheric_clip
        opt.last_sample_opaque = self.last_sample_opaque
        return opt


@dataclass
class Rays:
    origins: torch.Tensor
    dirs: torch.Tensor

    def _to_cpp(self):
        spec = _C.RaysSpec()
        spec.origins = self.origins
        spec.dirs = self.dirs
        return spec

    def __getitem__(self, key):
        return Rays(self.origins[key], self.dirs[key])

    @property
    def is_cuda(self) -> bool:
        return self.origins.is_cuda and self.dirs.is_cuda


@dataclass
class Camera:
    """Pinhole camera, OpenCV convention (svox2/svox2.py:105-183)."""

    c2w: torch.Tensor
    fx: float = 1111.11
    fy: Optional[float] = None
    cx: Optional[float] = None
    cy: Optional[float] = None
    width: int = 800
    height: int = 800
    ndc_coeffs: Union[Tuple[float, float], List[float]] = (-1.0, -1.0)

    @property
    def fx_val(self):
        return self.fx

    @property
    def fy_val(self):
        return self.fx if self.fy is None else self.fy

    @property
    def cx_val(self):
        return self.width * 0.5 if self.cx is None else self.cx

    @property
    def cy_val(self):
        return self.height * 0.5 if self.cy is None else self.cy

    @property
    def using_ndc(self):
        return self.ndc_coeffs[0] > 0.0

    def _to_cpp(self):
        spec = _C.CameraSpec()
        spec.c2w = self.c2w
        spec.fx = self.fx_val
        spec.fy = self.fy_val
        spec.cx = self.cx_val
        spec.cy = self.cy_val
        spec.width = self.width
        spec.height = self.height
        spec.ndc_coeffx = self.ndc_coeffs[0]
        spec.ndc_coeffy = self.ndc_coeffs[1]
        return spec

    @property
    def is_cuda(self) -> bool:
        return self.c2w.is_cuda

    def gen_rays(self) -> Rays:
        """Per-pixel rays (H*W, 3), pixel centres, directions formed in float64."""
        dev = self.c2w.device
        H, W = self.height, self.width
        ys = torch.arange(H, dtype=torch.float64, device=dev) + 0.5
        xs = torch.arange(W, dtype=torch.float64, device=dev) + 0.5
        yy, xx = torch.meshgrid(ys, xs, indexing="ij")
        d = torch.stack(((xx - self.cx_val) / self.fx_val, (yy - self.cy_val) / self.fy_val,
                         torch.ones_like(xx)), dim=-1)
        d = d / torch.norm(d, dim=-1, keepdim=True)
        d = (self.c2w[None, :3, :3].double() @ d.reshape(-1, 3, 1))[..., 0].reshape(-1, 3).float()
        origins = self.c2w[None, :3, 3].expand(H * W, -1).contiguous()
        if self.using_ndc:
            origins, d = _convert_to_ndc(origins, d, self.ndc_coeffs)
            d = d / torch.norm(d, dim=-1, keepdim=True)
        return Rays(origins, d.contiguous())


def _convert_to_ndc(origins, directions, ndc_coeffs, near: float = 1.0):
    """Shift rays to the near plane and map them to NDC (same map as the image kernel)."""
    t = (near - origins[..., 2]) / directions[..., 2]
    origins = origins + t[..., None] * directions
    dx, dy, dz = directions.unbind(-1)
    ox, oy, oz = origins.unbind(-1)
    o0 = ndc_coeffs[0] * (ox / oz)
    o1 = ndc_coeffs[1] * (oy / oz)
    o2 = 1 - 2 * near / oz
    d0 = ndc_coeffs[0] * (dx / dz - ox / oz)
    d1 = ndc_coeffs[1] * (dy / dz - oy / oz)
    d2 = 2 * near / oz
    return torch.stack([o0, o1, o2], -1), torch.stack([d0, d1, d2], -1)


# ---------------------------------------------------------------- autograd

class _SampleGridAutogradFunction(autograd.Function):
    """svox2/svox2.py:187-223."""

    @staticmethod
    def forward(ctx, data_density, data_sh, grid, points, want_colors):
        assert not points.requires_grad, "Point gradient not supported"
        out_density, out_sh = _C.sample_grid(grid, points, want_colors)
        ctx.save_for_backward(points)
        ctx.grid = grid
        ctx.want_colors = want_colors
        return out_density, out_sh

    @staticmethod
    def backward(ctx, grad_out_density, grad_out_sh):
        (points,) = ctx.saved_tensors
        grad_density_grid = torch.zeros_like(ctx.grid.density_data, dtype=torch.float32)
        grad_sh_grid = torch.zeros_like(ctx.grid.sh_data, dtype=torch.float32)
        if grad_out_sh is None or grad_out_sh.numel() == 0:
            grad_out_sh = torch.zeros((points.size(0), grad_sh_grid.size(1)), device=points.device)
        if grad_out_density is None:
            grad_out_density = torch.zeros((points.size(0), 1), device=points.device)
        _C.sample_grid_backward(ctx.grid, points, grad_out_density.contiguous(), grad_out_sh.contiguous(),
                                grad_density_grid, grad_sh_grid, ctx.want_colors)
        if not ctx.needs_input_grad[0]:
            grad_density_grid = None
        if not ctx.needs_input_grad[1]:
            grad_sh_grid = None
        return grad_density_grid, grad_sh_grid, None, None, None


class _TotalVariationFunction(autograd.Function):
    """TV value of channels [start_dim, end_dim) of a grid table and its gradient
    (svox2/svox2.py:292-329): forward tv, backward tv_grad.  The reference returns the
    gradient of the TV itself whatever the incoming gradient; here it is scaled by it, as
    autograd expects (identical for a TV term used with weight 1)."""

    @staticmethod
    def forward(ctx, data, links, start_dim, end_dim, use_logalpha, logalpha_delta, ignore_edge, ndc_coeffs):
        value = _C.tv(links, data, start_dim, end_dim, use_logalpha, logalpha_delta, ignore_edge,
                      ndc_coeffs[0], ndc_coeffs[1])
        ctx.save_for_backward(links, data)
        ctx.args = (start_dim, end_dim, use_logalpha, logalpha_delta, ignore_edge, ndc_coeffs)
        return value

    @staticmethod
    def backward(ctx, grad_out):
        links, data = ctx.saved_tensors
        start_dim, end_dim, use_logalpha, logalpha_delta, ignore_edge, ndc_coeffs = ctx.args
        grad = None
        if ctx.needs_input_grad[0]:
            grad = torch.zeros(data.shape, dtype=torch.float32, device=data.device)
            _C.tv_grad(links, data, start_dim, end_dim, 1.0, use_logalpha, logalpha_delta, ignore_edge,
                       ndc_coeffs[0], ndc_coeffs[1], grad)
            grad = (grad * grad_out).to(data.dtype)
        return grad, None, None, None, None, None, None, None


class _VolumeRenderFunction(autograd.Function):
    """svox2/svox2.py:226-288.  The backward is the reverse-order adjoint kernel;
    the colour it is handed is not needed by it and is kept for interface parity.
    With the MSI background, its table (data_background) gets a gradient too."""

    @staticmethod
    def forward(ctx, data_density, data_sh, data_basis, data_background, grid, rays, opt, backend):
        if backend != "cuvol":
            raise NotImplementedError(f"backend {backend!r}: only 'cuvol' is built")
        color = _C.volume_render_cuvol(grid, rays, opt)
        ctx.save_for_backward(color)
        ctx.grid = grid
        ctx.rays = rays
        ctx.opt = opt
        return color

    @staticmethod
    def backward(ctx, grad_out):
        (color_cache,) = ctx.saved_tensors
        grad_density_grid = torch.zeros_like(ctx.grid.density_data, dtype=torch.float32)
        grad_sh_grid = torch.zeros_like(ctx.grid.sh_data, dtype=torch.float32)
        holder = _C.GridOutputGrads()
        holder.grad_density_out = grad_density_grid
        holder.grad_sh_out = grad_sh_grid
        grad_background = None
        if ctx.grid.background_data is not None and ctx.needs_input_grad[3]:
            grad_background = torch.zeros_like(ctx.grid.background_data, dtype=torch.float32)
            holder.grad_background_out = grad_background
        _C.volume_render_cuvol_backward(ctx.grid, ctx.rays, ctx.opt, grad_out.contiguous(), color_cache, holder)
        ctx.grid = ctx.rays = ctx.opt = None
        if not ctx.needs_input_grad[0]:
            grad_density_grid = None
        if not ctx.needs_input_grad[1]:
            grad_sh_grid = None
        return grad_density_grid, grad_sh_grid, None, grad_background, None, None, None, None


# ---------------------------------------------------------------- grid

class SparseGrid(nn.Module):
    """Sparse voxel grid of density and SH coefficients (svox2/svox2.py:335-2357).

    :param reso: int or 3 ints, grid resolution
    :param radius: half side length (scalar or per axis)
    :param center: grid centre
    :param basis_type: only BASIS_TYPE_SH is built
    :param basis_dim: 1, 4 or 9 (SH degree 0, 1, 2)
    :param use_z_order: Morton order of the initial links (cubic power-of-2 grids)
    :param use_sphere_bound: allocate only voxels within the unit ball
    :param background_nlayers: 0, or the layer count (>= 2) of the MSI background model
    :param background_reso: MSI background resolution (equirectangular 2 reso x reso cells per layer)
    :param device: torch device
    :param sh_dtype: storage type of sh_data: torch.float32 (default), bfloat16 or float16
    """

    def __init__(
        self,
        reso: Union[int, List[int], Tuple[int, int, int]] = 128,
        radius: Union[float, List[float]] = 1.0,
        center: Union[float, List[float]] = [0.0, 0.0, 0.0],
        basis_type: int = BASIS_TYPE_SH,
        basis_dim: int = 9,
        basis_reso: int = 16,
        use_z_order: bool = False,
        use_sphere_bound: bool = False,
        mlp_posenc_size: int = 0,
        mlp_width: int = 16,
        background_nlayers: int = 0,
        background_reso: int = 256,
        device: Union[torch.device, str] = "cpu",
        sh_dtype: torch.dtype = torch.float32,
    ):
        super().__init__()
        if basis_type != BASIS_TYPE_SH:
            raise NotImplementedError("only the SH basis (BASIS_TYPE_SH) is built")
        if basis_dim not in (1, 4, 9):
            raise NotImplementedError("basis_dim must be 1, 4 or 9 (SH degree <= 2)")
        assert background_nlayers == 0 or background_nlayers > 1, "Please use at least 2 MSI layers (trilerp limitation)"
        if sh_dtype not in (torch.float32, torch.bfloat16, torch.float16):
            raise ValueError("sh_dtype must be float32, bfloat16 or float16")
        self.basis_type = basis_type
        self.basis_dim = basis_dim
        self.mlp_posenc_size = mlp_posenc_size
        self.mlp_width = mlp_width
        self.background_nlayers = background_nlayers
        self.background_reso = background_reso

        if isinstance(reso, int):
            reso = [reso] * 3
        else:
            assert len(reso) == 3, "reso must be an integer or indexable object of 3 ints"
        reso = [int(r) for r in reso]
        if use_z_order and not (reso[0] == reso[1] == reso[2] and utils.is_pow2(reso[0])):
            print("Morton code requires a cube grid of power-of-2 size, ignoring...")
            use_z_order = False

        if isinstance(radius, (float, int)):
            radius = [radius] * 3
        radius = (radius.to(device="cpu", dtype=torch.float32) if isinstance(radius, torch.Tensor)
                  else torch.tensor(radius, dtype=torch.float32))
        center = (center.to(device="cpu", dtype=torch.float32) if isinstance(center, torch.Tensor)
                  else torch.tensor(center, dtype=torch.float32))
        self.radius: torch.Tensor = radius
        self.center: torch.Tensor = center
        self._offset = 0.5 * (1.0 - self.center / self.radius)
        self._scaling = 0.5 / self.radius

        n3 = reduce(lambda a, b: a * b, reso)
        if use_z_order:
            init_links = utils.gen_morton(reso[0], device=device, dtype=torch.int32).flatten()
        else:
            init_links = torch.arange(n3, device=device, dtype=torch.int32)

        if use_sphere_bound:
            gsz = torch.tensor(reso, dtype=torch.float32)
            axes = [torch.arange(r, dtype=torch.float32, device=device) - 0.5 for r in reso]
            X, Y, Z = torch.meshgrid(*axes, indexing="ij")
            pts = torch.stack((X, Y, Z), dim=-1).view(-1, 3)
            pts = torch.addcmul((1.0 / gsz - 1.0).to(device), pts, (2.0 / gsz).to(device))
            inside = pts.norm(dim=-1) <= 1.0 + (3 ** 0.5) / gsz.max()
            self.capacity: int = int(inside.sum())
            slot = torch.zeros(n3, dtype=torch.int32, device=device)
            idxs = init_links[inside].long()
            slot[idxs] = 1
            slot = torch.cumsum(slot, dim=0) - 1
            init_links[inside] = slot[idxs].int()
            init_links[~inside] = -1
        else:
            self.capacity = n3

        self.density_data = nn.Parameter(torch.zeros(self.capacity, 1, dtype=torch.float32, device=device))
        self.sh_data = nn.Parameter(torch.zeros(self.capacity, self.basis_dim * 3, dtype=sh_dtype, device=device))
        self.basis_data = nn.Parameter(torch.empty(0, 0, 0, 0, dtype=torch.float32, device=device),
                                       requires_grad=False)
        if self.use_background:
            # MSI background (svox2/svox2.py:497-512): every cell of every layer allocated
            bg_cap = 2 * self.background_reso ** 2
            self.register_buffer("background_links", torch.arange(bg_cap, dtype=torch.int32, device=device)
                                 .reshape(2 * self.background_reso, self.background_reso))
            self.background_data = nn.Parameter(torch.zeros(bg_cap, self.background_nlayers, 4,
                                                            dtype=torch.float32, device=device))
        else:
            self.background_data = nn.Parameter(torch.empty(0, 0, 0, dtype=torch.float32, device=device),
                                                requires_grad=False)
            self.background_links: Optional[torch.Tensor] = None
        self.register_buffer("links", init_links.view(reso))
        self.links: torch.Tensor
        self.opt = RenderOptions()
        self.sparse_grad_indexer: Optional[torch.Tensor] = None
        self.sparse_sh_grad_indexer: Optional[torch.Tensor] = None
        self.sparse_background_indexer: Optional[torch.Tensor] = None
        self.density_rms: Optional[torch.Tensor] = None
        self.sh_rms: Optional[torch.Tensor] = None
        self.background_rms: Optional[torch.Tensor] = None
        self.basis_rms: Optional[torch.Tensor] = None

        if self.links.is_cuda and use_sphere_bound:
            self.accelerate()

    @classmethod
    def from_tables(cls, links: torch.Tensor, density_data: torch.Tensor, sh_data: torch.Tensor,
                    radius: Union[float, List[float]] = 1.0, center: Union[float, List[float]] = [0.0, 0.0, 0.0],
                    basis_dim: Optional[int] = None) -> "SparseGrid":
        """A grid over existing tables (links int32 [X,Y,Z], density [N,1], sh [N,3*bd]) on their
        device, without allocating a dense grid first (what SparseGrid.load does for a checkpoint)."""
        bd = basis_dim if basis_dim is not None else sh_data.size(1) // 3
        grid = cls(reso=[2, 2, 2], radius=radius, center=center, basis_dim=bd, device=links.device,
                   sh_dtype=sh_data.dtype)
        grid.links = links.to(torch.int32).contiguous()
        grid.density_data = nn.Parameter(density_data.contiguous())
        grid.sh_data = nn.Parameter(sh_data.contiguous())
        grid.capacity = density_data.size(0)
        return grid

    # ---- properties (svox2/svox2.py:537-559)
    @property
    def data_dim(self):
        return self.sh_data.size(1) + 1

    @property
    def basis_reso(self):
        return 0

    @property
    def use_background(self):
        return self.background_nlayers > 0

    @property
    def shape(self):
        return list(self.links.shape) + [self.data_dim]

    def basis_type_name(self):
        """Name of the basis type (svox2/svox2.py:2110-2117)."""
        return {BASIS_TYPE_SH: "SH", BASIS_TYPE_3D_TEXTURE: "3D_TEXTURE", BASIS_TYPE_MLP: "MLP"}.get(
            self.basis_type, "UNKNOWN")

    def __repr__(self):
        return (f"svox2.SparseGrid(basis_type={self.basis_type_name()}, basis_dim={self.basis_dim}, "
                f"reso={list(self.links.shape)}, capacity:{self.sh_data.size(0)})")

    def is_cubic_pow2(self):
        r = self.links.shape
        return r[0] == r[1] == r[2] and utils.is_pow2(r[0])

    # ---- sampling
    def sample(self, points: torch.Tensor, use_kernel: bool = True, grid_coords: bool = False,
               want_colors: bool = True):
        """Trilinear samples (density [P,1], colour coefficients [P,C]) at points (svox2/svox2.py:576-653)."""
        if not use_kernel or not self.links.is_cuda:
            _no_cpu_path("SparseGrid.sample")
        assert points.is_cuda
        return _SampleGridAutogradFunction.apply(self.density_data, self.sh_data,
                                                 self._to_cpp(grid_coords=grid_coords), points, want_colors)

    def forward(self, points: torch.Tensor, use_kernel: bool = True):
        return self.sample(points, use_kernel=use_kernel)

    # ---- rendering
    def volume_render(self, rays: Rays, use_kernel: bool = True, randomize: bool = False,
                      return_raylen: bool = False):
        """Colours (Q, 3) of the rays, differentiable w.r.t. density_data and sh_data (svox2/svox2.py:1036-1069)."""
        if return_raylen:
            raise NotImplementedError("return_raylen belongs to the reference's CPU path, not built here")
        if not use_kernel or not self.links.is_cuda:
            _no_cpu_path("SparseGrid.volume_render")
        assert rays.is_cuda
        return _VolumeRenderFunction.apply(self.density_data, self.sh_data, None,
                                           self.background_data if self.use_background else None,
                                           self._to_cpp(), rays._to_cpp(), self.opt._to_cpp(randomize=randomize),
                                           self.opt.backend)

    def volume_render_fused(self, rays: Rays, rgb_gt: torch.Tensor, randomize: bool = False,
                            beta_loss: float = 0.0, sparsity_loss: float = 0.0):
        """Render and accumulate the MSE gradient into .grad (svox2/svox2.py:1072-1142).

        Sets ``sparse_grad_indexer`` (bool [N]: voxels that received a gradient)
        and ``sparse_sh_grad_indexer`` (a copy), as the reference does; with the MSI
        background also its gradient and ``sparse_background_indexer`` (bool [N_bg, nlayers]).
        """
        if not self.sh_data.is_cuda:
            _no_cpu_path("SparseGrid.volume_render_fused")
        assert rays.is_cuda
        grad_density, grad_sh = self._get_data_grads()
        rgb_out = torch.zeros_like(rgb_gt)
        self.sparse_grad_indexer = torch.zeros((self.density_data.size(0),), dtype=torch.bool,
                                               device=self.density_data.device)
        holder = _C.GridOutputGrads()
        holder.grad_density_out = grad_density
        holder.grad_sh_out = grad_sh
        holder.mask_out = self.sparse_grad_indexer
        if self.use_background:
            holder.grad_background_out = self._grad_buffer(self.background_data)
            self.sparse_background_indexer = torch.zeros(list(self.background_data.shape[:-1]), dtype=torch.bool,
                                                         device=self.background_data.device)
            holder.mask_background_out = self.sparse_background_indexer
        _C.volume_render_cuvol_fused(self._to_cpp(), rays._to_cpp(), self.opt._to_cpp(randomize=randomize),
                                     rgb_gt, beta_loss, sparsity_loss, rgb_out, holder)
        self.sparse_sh_grad_indexer = self.sparse_grad_indexer.clone()
        return rgb_out

    def volume_render_image(self, camera: Camera, use_kernel: bool = True, randomize: bool = False,
                            batch_size: int = 5000, return_raylen: bool = False):
        """Image (H, W, 3) of a camera (svox2/svox2.py:1144-1179)."""
        if return_raylen:
            raise NotImplementedError("return_raylen belongs to the reference's CPU path, not built here")
        if not use_kernel or not self.links.is_cuda:
            _no_cpu_path("SparseGrid.volume_render_image")
        if not torch.is_grad_enabled():
            return _C.volume_render_cuvol_image(self._to_cpp(), camera._to_cpp(), self.opt._to_cpp())
        rays = camera.gen_rays()
        parts = [self.volume_render(rays[s:s + batch_size], randomize=randomize)
                 for s in range(0, camera.height * camera.width, batch_size)]
        return torch.cat(parts, dim=0).view(camera.height, camera.width, -1)

    # ---- coordinates (svox2/svox2.py:1496-1524)
    def world2grid(self, points):
        gsz = self._grid_size()
        offset = self._offset * gsz - 0.5
        scaling = self._scaling * gsz
        return torch.addcmul(offset.to(device=points.device), points, scaling.to(device=points.device))

    def grid2world(self, points):
        gsz = self._grid_size()
        roffset = self.radius * (1.0 / gsz - 1.0) + self.center
        rscaling = 2.0 * self.radius / gsz
        return torch.addcmul(roffset.to(device=points.device), points, rscaling.to(device=points.device))

    # ---- regularisers (svox2/svox2.py:1731-1820)
    def inplace_tv_grad(self, grad: torch.Tensor, scaling: float = 1.0, sparse_frac: float = 0.01,
                        logalpha: bool = False, logalpha_delta: float = 2.0,
                        ndc_coeffs: Tuple[float, float] = (-1.0, -1.0), contiguous: bool = True):
        """Add scaling * d(TV(density))/d(density) into grad (sparse over a random cell window)."""
        if grad is None:
            grad = self._grad_buffer(self.density_data)
        assert self.density_data.is_cuda and grad.is_cuda, "the grid and grad must be on a CUDA device"
        assert not logalpha, "No longer supported"
        rand_cells = self._get_rand_cells(sparse_frac, contiguous=contiguous)
        if rand_cells is not None:
            if rand_cells.size(0) > 0:
                _C.tv_grad_sparse(self.links, self.density_data, rand_cells, self._get_sparse_grad_indexer(),
                                  0, 1, scaling, logalpha, logalpha_delta, False, self.opt.last_sample_opaque,
                                  ndc_coeffs[0], ndc_coeffs[1], grad)
        else:
            _C.tv_grad(self.links, self.density_data, 0, 1, scaling, logalpha, logalpha_delta, False,
                       ndc_coeffs[0], ndc_coeffs[1], grad)
            self.sparse_grad_indexer = None

    def inplace_l2_color_grad(self, grad: torch.Tensor, start_dim: int = 0, end_dim: Optional[int] = None,
                              scaling: float = 1.0):
        """Add the gradient of an L2 penalty on the SH channels [start_dim, end_dim) into grad,
        times scaling / (rows penalised): every row, or the rows of sparse_sh_grad_indexer
        (svox2/svox2.py:1897-1932; plain tensor arithmetic, as in the reference)."""
        with torch.no_grad():
            C = self.sh_data.size(1)
            end_dim = C if end_dim is None else (end_dim + C if end_dim < 0 else end_dim)
            start_dim = start_dim + C if start_dim < 0 else start_dim
            sh = self.sh_data[:, start_dim:end_dim].float()
            if self.sparse_sh_grad_indexer is None:
                grad[:, start_dim:end_dim] += (scaling / self.sh_data.size(0)) * sh
            else:
                idx = self.sparse_sh_grad_indexer
                nz = int(torch.count_nonzero(idx).item()) if idx.dtype == torch.bool else idx.size(0)
                if nz > 0:
                    grad[idx, start_dim:end_dim] += (scaling / nz) * sh[idx]

    def tv(self, logalpha: bool = False, logalpha_delta: float = 2.0,
           ndc_coeffs: Tuple[float, float] = (-1.0, -1.0)):
        """Total variation of the density, a differentiable scalar: the sum over channels of the
        mean over cells (svox2/svox2.py:1678-1693)."""
        if not self.links.is_cuda:
            _no_cpu_path("SparseGrid.tv")
        assert not logalpha, "No longer supported"
        return _TotalVariationFunction.apply(self.density_data, self.links, 0, 1, logalpha, logalpha_delta,
                                             False, ndc_coeffs)

    def tv_color(self, start_dim: int = 0, end_dim: Optional[int] = None, logalpha: bool = False,
                 logalpha_delta: float = 2.0, ndc_coeffs: Tuple[float, float] = (-1.0, -1.0)):
        """Total variation of the SH channels [start_dim, end_dim), a differentiable scalar
        (svox2/svox2.py:1695-1722)."""
        if not self.links.is_cuda:
            _no_cpu_path("SparseGrid.tv_color")
        assert not logalpha, "No longer supported"
        C = self.sh_data.size(1)
        end_dim = C if end_dim is None else (end_dim + C if end_dim < 0 else end_dim)
        start_dim = start_dim + C if start_dim < 0 else start_dim
        return _TotalVariationFunction.apply(self.sh_data, self.links, start_dim, end_dim, logalpha,
                                             logalpha_delta, True, ndc_coeffs)

    def inplace_tv_color_grad(self, grad: torch.Tensor, start_dim: int = 0, end_dim: Optional[int] = None,
                              scaling: float = 1.0, sparse_frac: float = 0.01, logalpha: bool = False,
                              logalpha_delta: float = 2.0, ndc_coeffs: Tuple[float, float] = (-1.0, -1.0),
                              contiguous: bool = True):
        """Add scaling * d(TV(sh[:, start:end]))/d(sh) into grad (None: the grid's own SH gradient)."""
        if grad is None:
            grad = self._grad_buffer(self.sh_data)
        assert self.sh_data.is_cuda and grad.is_cuda, "the grid and grad must be on a CUDA device"
        assert not logalpha, "No longer supported"
        C = self.sh_data.size(1)
        if end_dim is None:
            end_dim = C
        end_dim = end_dim + C if end_dim < 0 else end_dim
        start_dim = start_dim + C if start_dim < 0 else start_dim
        rand_cells = self._get_rand_cells(sparse_frac, contiguous=contiguous)
        if rand_cells is not None:
            if rand_cells.size(0) > 0:
                _C.tv_grad_sparse(self.links, self.sh_data, rand_cells, self._get_sparse_sh_grad_indexer(),
                                  start_dim, end_dim, scaling, logalpha, logalpha_delta, True, False,
                                  ndc_coeffs[0], ndc_coeffs[1], grad)
        else:
            _C.tv_grad(self.links, self.sh_data, start_dim, end_dim, scaling, logalpha, logalpha_delta, True,
                       ndc_coeffs[0], ndc_coeffs[1], grad)
            self.sparse_sh_grad_indexer = None

    def inplace_tv_background_grad(self, grad: torch.Tensor, scaling: float = 1.0,
                                   scaling_density: Optional[float] = None, sparse_frac: float = 0.01,
                                   contiguous: bool = False):
        """Add the MSI background's TV gradient into grad (None: background_data's own gradient):
        colour channels times scaling, sigma times scaling_density (default scaling), over a
        random set of cells (svox2/svox2.py:1930-1955)."""
        if grad is None:
            grad = self._grad_buffer(self.background_data)
        assert self.background_data.is_cuda and grad.is_cuda, "the grid and grad must be on a CUDA device"
        rand_cells_bg = self._get_rand_cells_background(sparse_frac, contiguous)
        indexer = self._get_sparse_background_grad_indexer()
        if scaling_density is None:
            scaling_density = scaling
        _C.msi_tv_grad_sparse(self.background_links, self.background_data, rand_cells_bg, indexer, scaling,
                              scaling_density, grad)

    # ---- optimisers (svox2/svox2.py:1972-2041)
    def optim_density_step(self, lr: float, beta: float = 0.9, epsilon: float = 1e-8, optim: str = "rmsprop"):
        """RMSprop or SGD step on density_data over the voxels the last render touched."""
        assert self.sh_data.is_cuda, "the grid must be on a CUDA device"
        indexer = self._maybe_convert_sparse_grad_indexer()
        if optim == "rmsprop":
            if self.density_rms is None or self.density_rms.shape != self.density_data.shape:
                self.density_rms = torch.zeros_like(self.density_data.data)
            _C.rmsprop_step(self.density_data.data, self.density_rms, self._grad_buffer(self.density_data), indexer,
                            beta, lr, epsilon, -1e9, lr)
        elif optim == "sgd":
            _C.sgd_step(self.density_data.data, self._grad_buffer(self.density_data), indexer, lr, lr)
        else:
            raise NotImplementedError(f"Unsupported optimizer {optim}")

    def optim_sh_step(self, lr: float, beta: float = 0.9, epsilon: float = 1e-8, optim: str = "rmsprop"):
        """RMSprop or SGD step on sh_data."""
        assert self.sh_data.is_cuda, "the grid must be on a CUDA device"
        indexer = self._maybe_convert_sparse_grad_indexer(sh=True)
        if optim == "rmsprop":
            if self.sh_rms is None or self.sh_rms.shape != self.sh_data.shape:
                self.sh_rms = torch.zeros(self.sh_data.shape, dtype=torch.float32, device=self.sh_data.device)
            _C.rmsprop_step(self.sh_data.data, self.sh_rms, self._grad_buffer(self.sh_data), indexer, beta, lr,
                            epsilon, -1e9, lr)
        elif optim == "sgd":
            _C.sgd_step(self.sh_data.data, self._grad_buffer(self.sh_data), indexer, lr, lr)
        else:
            raise NotImplementedError(f"Unsupported optimizer {optim}")

    def optim_background_step(self, lr_sigma: float, lr_color: float, beta: float = 0.9, epsilon: float = 1e-8,
                              optim: str = "rmsprop"):
        """RMSprop or SGD step on the MSI background (svox2/svox2.py:2043-2084): rows are
        (cell, layer) pairs of four channels, the last (sigma) at lr_sigma, the colours at
        lr_color, over the rows the last fused render touched."""
        assert self.background_data.is_cuda, "the grid must be on a CUDA device"
        indexer = self._maybe_convert_sparse_grad_indexer(bg=True)
        n_chnl = self.background_data.size(-1)
        grad = self._grad_buffer(self.background_data)
        if optim == "rmsprop":
            if self.background_rms is None or self.background_rms.shape != self.background_data.shape:
                self.background_rms = torch.zeros_like(self.background_data.data)
            _C.rmsprop_step(self.background_data.data.view(-1, n_chnl), self.background_rms.view(-1, n_chnl),
                            grad.view(-1, n_chnl), indexer, beta, lr_color, epsilon, -1e9, lr_sigma)
        elif optim == "sgd":
            _C.sgd_step(self.background_data.data.view(-1, n_chnl), grad.view(-1, n_chnl), indexer, lr_color,
                        lr_sigma)
        else:
            raise NotImplementedError(f"Unsupported optimizer {optim}")

    # ---- internals (svox2/svox2.py:2135-2241)
    def _to_cpp(self, grid_coords: bool = False, replace_basis_data: Optional[torch.Tensor] = None):
        gspec = _C.SparseGridSpec()
        gspec.density_data = self.density_data
        gspec.sh_data = self.sh_data
        gspec.links = self.links
        if grid_coords:
            gspec._offset = torch.zeros_like(self._offset)
            gspec._scaling = torch.ones_like(self._offset)
        else:
            gsz = self._grid_size()
            gspec._offset = self._offset * gsz - 0.5
            gspec._scaling = self._scaling * gsz
        gspec.basis_dim = self.basis_dim
        gspec.basis_type = self.basis_type
        if self.use_background:
            gspec.background_links = self.background_links
            gspec.background_data = self.background_data
        return gspec

    def _grid_size(self):
        return torch.tensor(self.links.shape, device="cpu", dtype=torch.float32)

    def _grad_buffer(self, p: torch.Tensor) -> torch.Tensor:
        """float32 gradient of a grid table.  For float32 storage this is p.grad;
        for bfloat16/float16 SH storage autograd cannot hold a float32 .grad,
        so the buffer lives beside the parameter as p._svx_grad32."""
        if p.dtype == torch.float32:
            if p.grad is None or p.grad.shape != p.shape:
                p.grad = torch.zeros_like(p.data)
            return p.grad
        g = getattr(p, "_svx_grad32", None)
        if g is None or g.shape != p.shape:
            g = torch.zeros(p.shape, dtype=torch.float32, device=p.device)
            p._svx_grad32 = g
        return g

    def _get_data_grads(self):
        """Gradient buffers of density_data and sh_data, allocated once and reused (svox2/svox2.py:2166-2182)."""
        return [self._grad_buffer(self.density_data), self._grad_buffer(self.sh_data)]

    def _get_sparse_grad_indexer(self):
        indexer = self.sparse_grad_indexer
        if indexer is None:
            indexer = torch.empty((0,), dtype=torch.bool, device=self.density_data.device)
        return indexer

    def _get_sparse_sh_grad_indexer(self):
        indexer = self.sparse_sh_grad_indexer
        if indexer is None:
            indexer = torch.empty((0,), dtype=torch.bool, device=self.density_data.device)
        return indexer

    def _maybe_convert_sparse_grad_indexer(self, sh: bool = False, bg: bool = False):
        """Indexer for the optimiser: the render's bool mask (or all rows if none).

        The reference converted a mask with fewer than N/8 set entries into an
        index list, which costs a device->host synchronisation per step; the
        mask kernel produces identical results, so the mask is passed as is.
        """
        indexer = self.sparse_sh_grad_indexer if sh else self.sparse_grad_indexer
        if bg:
            indexer = self.sparse_background_indexer
            if indexer is not None:
                indexer = indexer.view(-1)
        if indexer is None:
            return torch.empty((), device=self.density_data.device)
        return indexer

    def _get_sparse_background_grad_indexer(self):
        indexer = self.sparse_background_indexer
        if indexer is None:
            indexer = torch.empty((0, 0), dtype=torch.bool, device=self.density_data.device)
        return indexer

    @staticmethod
    def _tv_cells(n_cells: int, sparse_frac: float, contiguous: bool, device) -> torch.Tensor:
        """int32 indices of max(int(sparse_frac * n_cells), 1) cells for a sparse TV term: a
        window of consecutive cells that wraps past the last one, starting at a cell drawn
        from numpy's global RNG, or (contiguous False) cells drawn uniformly by torch on the
        device.  The draws are the reference's (svox2/svox2.py:2224-2260), so a seeded run
        selects the same cells."""
        count = max(int(sparse_frac * n_cells), 1)
        if not contiguous:
            return torch.randint(0, n_cells, (count,), dtype=torch.int32, device=device)
        first = np.random.randint(0, n_cells)
        window = torch.arange(count, dtype=torch.int64, device=device).add_(first).remainder_(n_cells)
        return window.to(torch.int32)

    def _require_mask_state(self, indexer, what: str):
        if indexer is not None and indexer.dtype != torch.bool:
            raise AssertionError(f"{what} must come between the render that marks the touched cells and the "
                                 "optimiser step that consumes the mark")

    def _get_rand_cells_background(self, sparse_frac: float, contiguous: bool = True):
        """Random cells of the MSI background's [2 reso, reso, nlayers] (cell, layer) table for
        its TV term (svox2/svox2.py:2243-2260)."""
        if not self.use_background:
            raise AssertionError("this grid has no MSI background to regularise")
        self._require_mask_state(self.sparse_background_indexer, "the background TV term")
        n_cells = self.background_links.numel() * self.background_data.size(1)
        return self._tv_cells(n_cells, sparse_frac, contiguous, self.links.device)

    def _get_rand_cells(self, sparse_frac: float, force: bool = False, contiguous: bool = True):
        """Random grid cells for a sparse TV term (svox2/svox2.py:2224-2241), or None for the
        dense term (sparse_frac >= 1 and not force)."""
        if sparse_frac >= 1.0 and not force:
            return None
        self._require_mask_state(self.sparse_grad_indexer, "a sparse TV term")
        return self._tv_cells(self.links.numel(), sparse_frac, contiguous, self.links.device)

    # ---- depth renders (svox2/svox2.py:1181-1221)
    def volume_render_depth(self, rays: Rays, sigma_thresh: Optional[float] = None):
        """Per-ray distance along the ray (world units): the expected termination, or with
        sigma_thresh the first point whose density strictly exceeds it.  Returns (N,)."""
        if sigma_thresh is None:
            return _C.volume_render_expected_term(self._to_cpp(), rays._to_cpp(), self.opt._to_cpp())
        return _C.volume_render_sigma_thresh(self._to_cpp(), rays._to_cpp(), self.opt._to_cpp(), sigma_thresh)

    def volume_render_depth_image(self, camera: Camera, sigma_thresh: Optional[float] = None,
                                  batch_size: int = 5000):
        """Depth image (H, W) of a camera, rays in batches of batch_size."""
        rays = camera.gen_rays()
        depths = [self.volume_render_depth(rays[b:b + batch_size], sigma_thresh)
                  for b in range(0, camera.height * camera.width, batch_size)]
        return torch.cat(depths, dim=0).view(camera.height, camera.width)

    # ---- resampling (svox2/svox2.py:1223-1424)
    def resample(self, reso: Union[int, List[int]], sigma_thresh: float = 5.0, weight_thresh: float = 0.01,
                 dilate: int = 2, cameras: Optional[List["Camera"]] = None, use_z_order: bool = False,
                 accelerate: bool = True, weight_render_stop_thresh: float = 0.2, max_elements: int = 0):
        """Resample the grid to reso and sparsify it.  The old grid is sampled at the new voxel
        centres (grid coordinates); a voxel is kept if its density reaches sigma_thresh or, with
        cameras, if its largest rendering weight over the cameras' rays reaches weight_thresh.
        max_elements > 0 raises the threshold so at most that many voxels are kept.  The mask is
        dilated `dilate` times, colours are sampled for the kept voxels only, and links are
        rebuilt in raster (or Morton) order.  Optimiser state and gradients are dropped."""
        if not self.links.is_cuda:
            _no_cpu_path("SparseGrid.resample")
        with torch.no_grad():
            device = self.links.device
            reso = [int(reso)] * 3 if isinstance(reso, int) else [int(r) for r in reso]
            assert len(reso) == 3, "reso must be an integer or indexable object of 3 ints"
            if use_z_order and not (reso[0] == reso[1] == reso[2] and utils.is_pow2(reso[0])):
                print("Morton code requires a cube grid of power-of-2 size, ignoring...")
                use_z_order = False
            # new voxel centres in the current grid's coordinates
            cur = self.links.shape
            axes = []
            for i in range(3):
                f = 0.5 * cur[i] / reso[i]
                axes.append(torch.linspace(f - 0.5, cur[i] - f - 0.5, reso[i], dtype=torch.float32))
            X, Y, Z = torch.meshgrid(*axes, indexing="ij")
            points = torch.stack((X, Y, Z), dim=-1).view(-1, 3)
            morton = None
            if use_z_order:
                morton = utils.gen_morton(reso[0], dtype=torch.long).view(-1)
                points[morton] = points.clone()
            points = points.to(device=device)

            batch = 720720
            dens = torch.cat([self.sample(points[i:i + batch], grid_coords=True, want_colors=False)[0]
                              for i in range(0, points.size(0), batch)], dim=0).view(reso)
            self.density_data.grad = None
            self.sh_data.grad = None
            self.sparse_grad_indexer = None
            self.sparse_sh_grad_indexer = None
            self.density_rms = None
            self.sh_rms = None

            if cameras is not None:
                gsz = torch.tensor(reso, dtype=torch.float32)
                offset = self._offset * gsz - 0.5
                scaling = self._scaling * gsz
                wmax = torch.zeros(reso, dtype=torch.float32, device=device)
                for cam in cameras:
                    _C.grid_weight_render(dens, cam._to_cpp(), 0.5, weight_render_stop_thresh, False,
                                          offset, scaling, wmax)
                score, thresh = wmax, weight_thresh
            else:
                score, thresh = dens, sigma_thresh
            mask = score >= thresh
            if 0 < max_elements < score.numel() and max_elements < int(torch.count_nonzero(mask)):
                bounded = torch.topk(score.view(-1), k=max_elements, sorted=False).values.min().item()
                thresh = max(thresh, bounded)
                mask = score >= thresh
            if cameras is None and self.opt.last_sample_opaque:
                mask[:, :, -1] = True          # keep the last z layer
            del score
            for _ in range(int(dilate)):
                mask = _C.dilate(mask)
            mask = mask.view(-1)
            new_dens = dens.view(-1)[mask]
            kept = points[mask]
            cols = [self.sample(kept[i:i + batch], grid_coords=True, want_colors=True)[1]
                    for i in range(0, kept.size(0), batch)]
            new_sh = torch.cat(cols, dim=0) if cols else torch.empty_like(self.sh_data[:0])

            if morton is not None:
                inv = torch.empty_like(morton)
                inv[morton] = torch.arange(morton.size(0), dtype=morton.dtype)
                order = inv.to(device)[mask]
                links = torch.full((mask.size(0),), -1, dtype=torch.int32, device=device)
                links[order] = torch.arange(order.size(0), dtype=torch.int32, device=device)
            else:
                links = torch.cumsum(mask.to(torch.int32), dim=-1).to(torch.int32) - 1
                links[~mask] = -1
            self.capacity = int(new_dens.size(0))
            self.density_data = nn.Parameter(new_dens.view(-1, 1).contiguous())
            self.sh_data = nn.Parameter(new_sh.to(self.sh_data.dtype).contiguous())
            self.links = links.view(reso).contiguous()
            if accelerate:
                self.accelerate()

    # ---- checkpoints (svox2/svox2.py:1526-1628): the reference's npz format
    def save(self, path: str, compress: bool = False):
        """Write radius, center, links, density_data, sh_data (stored as float16, as the
        reference stores it) and basis_type to an npz file."""
        save_fn = np.savez_compressed if compress else np.savez
        data = {
            "radius": self.radius.numpy(),
            "center": self.center.numpy(),
            "links": self.links.cpu().numpy(),
            "density_data": self.density_data.data.cpu().numpy(),
            # through float32 (exact for bfloat16 / float16) to the file's float16
            "sh_data": self.sh_data.data.float().cpu().numpy().astype(np.float16),
        }
        if self.use_background:
            data["background_links"] = self.background_links.cpu().numpy()
            data["background_data"] = self.background_data.data.cpu().numpy()
        data["basis_type"] = self.basis_type
        save_fn(path, **data)

    @classmethod
    def load(cls, path: str, device: Union[torch.device, str] = "cpu",
             sh_dtype: torch.dtype = torch.float32) -> "SparseGrid":
        """Read a checkpoint written by save (or by the reference).  SH comes back as float32
        like the reference, or kept in sh_dtype (bfloat16 / float16 storage); a grid placed on
        a CUDA device is accelerated, as the reference does."""
        z = np.load(path)
        if "data" in z.keys():           # older single-table layout: [density | sh]
            all_data = z.f.data
            sh_data = all_data[..., 1:]
            density_data = all_data[..., :1]
        else:
            sh_data = z.f.sh_data
            density_data = z.f.density_data
        basis_type = z["basis_type"].item() if "basis_type" in z else BASIS_TYPE_SH
        if basis_type != BASIS_TYPE_SH or "basis_data" in z.keys():
            raise NotImplementedError("only SH-basis checkpoints are supported by svox2_gb300")
        radius = z.f.radius.tolist() if "radius" in z.files else [1.0, 1.0, 1.0]
        center = z.f.center.tolist() if "center" in z.files else [0.0, 0.0, 0.0]
        sh = torch.from_numpy(np.ascontiguousarray(sh_data.astype(np.float32)))
        dens = torch.from_numpy(np.ascontiguousarray(density_data.astype(np.float32)))
        links = torch.from_numpy(np.ascontiguousarray(z.f.links).astype(np.int32))
        grid = cls.from_tables(links.to(device=device), dens.to(device=device),
                               sh.to(device=device, dtype=sh_dtype), radius=radius, center=center)
        if "background_data" in z:
            bd = torch.from_numpy(np.ascontiguousarray(z["background_data"])).to(device=device)
            bl = torch.from_numpy(np.ascontiguousarray(z["background_links"])).to(device=device)
            grid.background_nlayers = bd.shape[1]
            grid.background_reso = bl.shape[1]
            grid.background_data = nn.Parameter(bd)
            grid.background_links = bl
        if grid.links.is_cuda:
            grid.accelerate()
        return grid

    def sparsify_background(self, sigma_thresh: float = 1.0, dilate: int = 1):
        """Drop the MSI background cells whose sigma stays below sigma_thresh in every layer,
        after `dilate` 3x3x3 dilations of the kept (cell, layer) mask, and number the rest in
        raster order (svox2/svox2.py:1426-1448).  Each cell's layers are read through its own
        link."""
        if not self.use_background:
            raise AssertionError("this grid has no MSI background to sparsify")
        if int(dilate) > 0 and not self.background_links.is_cuda:
            raise RuntimeError("sparsify_background dilates with a CUDA kernel: the grid must be on a CUDA device")
        links = self.background_links
        device = links.device
        rows = links.reshape(-1).long()
        present = rows >= 0
        dense = self.background_data[..., -1] >= sigma_thresh          # [rows, nlayers]
        keep = torch.zeros((rows.numel(), dense.size(1)), dtype=torch.bool, device=device)
        keep[present] = dense[rows[present]]
        keep = keep.view(*links.shape, dense.size(1))
        for _ in range(int(dilate)):
            keep = _C.dilate(keep)
        kept_cells = keep.any(-1).reshape(-1) & present
        kept_rows = rows[kept_cells]
        renumbered = torch.full_like(rows, -1)
        renumbered[kept_cells] = torch.arange(kept_rows.numel(), device=device)
        self.background_links = renumbered.to(torch.int32).view(links.shape)
        self.background_data = nn.Parameter(self.background_data.data[kept_rows])

    # ---- empty-space skipping
    def accelerate(self):
        """Empty-space skip levels in the links table (svox2/svox2.py:1487-1494): every
        negative link becomes -(1 + the empty levels of the 2x pyramid above it), which the
        ray march turns into jumps over empty blocks."""
        if not self.links.is_cuda:
            raise RuntimeError("accelerate needs the grid on a CUDA device (there is no CPU path)")
        _C.accel_dist_prop(self.links)

    # ---- not built here
    def _unbuilt(self, *a, **k):
        raise NotImplementedError("this SparseGrid method is not implemented in svox2_gb300")

    resize = to_svox1 = _unbuilt
    inplace_tv_lumisphere_grad = inplace_tv_basis_grad = tv_basis = _unbuilt
    optim_basis_step = reinit_learned_bases = _unbuilt
