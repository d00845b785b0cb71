"""Seeded synthetic workloads with the benchmark configurations' shapes and
value distributions (no datasets are used; the reference's scenes are not
available).

Grid: radius 1, centre 0, so world = [-1, 1]^3; voxel i has world centre
(i + 0.5) * 2 / reso - 1.  Allocated voxels get
    density = max(0, 40 * max(0, 1 - |x| / 0.6) + N(0, 1)),  SH ~ N(0, 0.3).
Sparse grids allocate the union of n_balls balls: centres U[-1,1]^3, base
radii U[0.1, 0.3], all radii scaled by one factor s chosen so that the
allocated fraction hits the target (s is the target quantile of the per-voxel
min over balls of |x - c| / r, so the fraction is exact to one voxel).
Links are cumsum(mask) - 1 in raster order, -1 elsewhere.
Rays: origin = 1.5 * normalize(N(0, I)), direction = normalize(U[-0.5,0.5]^3 -
origin); target colours U[0,1]^3.

Random numbers come from one CPU torch.Generator per call, drawn in the
order: balls (centres, radii), density noise, SH, ray origins, ray targets,
target colours.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

import torch


@dataclass
class GridData:
    links: torch.Tensor      # int32 [X, Y, Z]
    density: torch.Tensor    # float32 [N, 1]
    sh: torch.Tensor         # float32 [N, 3*bd]
    reso: tuple
    scale_factor: float      # ball radius factor s (1.0 for dense)
    occupancy: float


def voxel_centres(reso, device="cpu", dtype=torch.float32):
    axes = [(torch.arange(r, dtype=dtype, device=device) + 0.5) * (2.0 / r) - 1.0 for r in reso]
    X, Y, Z = torch.meshgrid(*axes, indexing="ij")
    return X, Y, Z


def _ball_ratio(reso, centres, radii, device):
    """min over balls of |x - c| / r per voxel (float64), computed in z-slabs."""
    X = reso[0]
    out = torch.empty(reso, dtype=torch.float64, device=device)
    ax = [(torch.arange(r, dtype=torch.float64, device=device) + 0.5) * (2.0 / r) - 1.0 for r in reso]
    c = centres.to(device=device, dtype=torch.float64)
    rr = radii.to(device=device, dtype=torch.float64)
    for x0 in range(0, X, 16):
        xs = ax[0][x0:x0 + 16]
        gx, gy, gz = torch.meshgrid(xs, ax[1], ax[2], indexing="ij")
        best = torch.full(gx.shape, float("inf"), dtype=torch.float64, device=device)
        for b in range(c.shape[0]):
            d = torch.sqrt((gx - c[b, 0]) ** 2 + (gy - c[b, 1]) ** 2 + (gz - c[b, 2]) ** 2) / rr[b]
            best = torch.minimum(best, d)
        out[x0:x0 + 16] = best
    return out


def make_grid(reso, occupancy: Optional[float] = None, n_balls: int = 8, basis_dim: int = 9, seed: int = 0,
              density_mode: str = "ball", device="cpu") -> GridData:
    """Synthetic grid.  occupancy None -> dense (links = arange).

    density_mode "ball": the benchmark density; "normal53": max(0, N(5, 3)) (the
    differentiation-check grid)."""
    if isinstance(reso, int):
        reso = (reso, reso, reso)
    reso = tuple(int(r) for r in reso)
    gen = torch.Generator().manual_seed(seed)
    n3 = reso[0] * reso[1] * reso[2]
    if occupancy is None:
        mask = None
        s = 1.0
        links = torch.arange(n3, dtype=torch.int32).view(reso)
    else:
        centres = torch.rand((n_balls, 3), generator=gen, dtype=torch.float64) * 2 - 1
        radii = torch.rand((n_balls,), generator=gen, dtype=torch.float64) * 0.2 + 0.1
        ratio = _ball_ratio(reso, centres, radii, device).flatten()
        k = max(int(round(occupancy * n3)), 1)
        s = float(torch.kthvalue(ratio, k).values)
        mask = (ratio <= s).view(reso).cpu()
        del ratio
        links = torch.full(reso, -1, dtype=torch.int32)
        links[mask] = torch.arange(int(mask.sum()), dtype=torch.int32)
    N = n3 if mask is None else int(mask.sum())
    noise = torch.randn((N,), generator=gen, dtype=torch.float32)
    sh = torch.randn((N, 3 * basis_dim), generator=gen, dtype=torch.float32) * 0.3
    if density_mode == "ball":
        X, Y, Z = voxel_centres(reso, device=device)
        rad = torch.sqrt(X * X + Y * Y + Z * Z)
        del X, Y, Z
        base = 40.0 * torch.clamp(1.0 - rad / 0.6, min=0.0)
        base = (base.flatten() if mask is None else base[mask.to(base.device)]).cpu()
        density = torch.clamp(base + noise, min=0.0)
    elif density_mode == "normal53":
        density = torch.clamp(noise * 3.0 + 5.0, min=0.0)
    else:
        raise ValueError(density_mode)
    return GridData(links.contiguous(), density.view(N, 1).contiguous(), sh.contiguous(), reso, s, N / n3)


def make_rays(n: int, seed: int = 1, device="cpu"):
    """(origins, dirs, rgb_gt) float32 [n, 3] each."""
    gen = torch.Generator().manual_seed(seed)
    o = torch.randn((n, 3), generator=gen, dtype=torch.float32)
    o = 1.5 * o / torch.norm(o, dim=-1, keepdim=True)
    tgt = torch.rand((n, 3), generator=gen, dtype=torch.float32) - 0.5
    d = tgt - o
    d = d / torch.norm(d, dim=-1, keepdim=True)
    gt = torch.rand((n, 3), generator=gen, dtype=torch.float32)
    return o.to(device).contiguous(), d.to(device).contiguous(), gt.to(device).contiguous()


def look_at_c2w(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)) -> torch.Tensor:
    """OpenCV camera-to-world 4x4 (x right, y down, z forward) looking from eye at target."""
    eye = torch.tensor(eye, dtype=torch.float64)
    fwd = torch.tensor(target, dtype=torch.float64) - eye
    fwd = fwd / fwd.norm()
    upv = torch.tensor(up, dtype=torch.float64)
    right = torch.linalg.cross(fwd, upv)
    if right.norm() < 1e-9:
        right = torch.linalg.cross(fwd, torch.tensor([1.0, 0.0, 0.0], dtype=torch.float64))
    right = right / right.norm()
    down = torch.linalg.cross(fwd, right)
    m = torch.eye(4, dtype=torch.float64)
    m[:3, 0] = right
    m[:3, 1] = down
    m[:3, 2] = fwd
    m[:3, 3] = eye
    return m.float()


def grid_transform(reso):
    """(offset, scaling) of the world->grid map for a radius-1, centre-0 grid
    (the reference's _to_cpp values: offset = 0.5 * gsz - 0.5, scaling = 0.5 * gsz)."""
    off = tuple(0.5 * r - 0.5 for r in reso)
    scl = tuple(0.5 * r for r in reso)
    return off, scl


def max_samples_per_ray(reso, step: float = 0.5) -> int:
    return int(math.sqrt(sum(r * r for r in reso)) / step) + 2
