"""Shared helpers for the parity tests: build the same seeded inputs for the
CUDA operators (svox2_gb300.csrc, the reference-facing API) and for the CPU
oracle, and compare results with stated tolerances."""
from __future__ import annotations

import numpy as np
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S

# Tolerances (float32 results vs the float32 oracle):
#   colours: |k - o| <= RTOL_RGB * |o| + ATOL_RGB
#   gradients: |k - o| <= RTOL_GRAD * |o| + ATOL_GRAD_FRAC * max|o|   (atomics reorder sums)
RTOL_RGB, ATOL_RGB = 1e-5, 1e-6
RTOL_GRAD, ATOL_GRAD_FRAC = 1e-4, 1e-5


def opt_struct(sigma_thresh=1e-8, stop_thresh=1e-7, bg=1.0, step=0.5, near_clip=0.0, spheric=False,
               last_opaque=False):
    from svox2_gb300 import csrc as C
    o = C.RenderOptions()
    o.background_brightness = bg
    o.step_size = step
    o.sigma_thresh = sigma_thresh
    o.stop_thresh = stop_thresh
    o.near_clip = near_clip
    o.use_spheric_clip = spheric
    o.last_sample_opaque = last_opaque
    oo = O.Opt(bg, step, sigma_thresh, stop_thresh, near_clip, spheric, last_opaque)
    return o, oo


def grid_pair(g: S.GridData, basis_dim=9, sh_dtype=torch.float32, device="cuda"):
    """(SparseGridSpec on device, oracle Grid with the same (rounded) values)."""
    from svox2_gb300 import csrc as C
    sh = g.sh[:, : 3 * basis_dim].contiguous()
    sh_dev = sh.to(device=device, dtype=sh_dtype)
    sh_np = sh_dev.float().cpu().numpy()          # the values the kernel actually reads
    off, scl = S.grid_transform(g.reso)
    spec = C.SparseGridSpec()
    spec.density_data = g.density.to(device)
    spec.sh_data = sh_dev
    spec.links = g.links.to(device)
    spec._offset = torch.tensor(off, dtype=torch.float32)
    spec._scaling = torch.tensor(scl, dtype=torch.float32)
    spec.basis_dim = basis_dim
    spec.basis_type = 1
    og = O.Grid(g.links.numpy(), g.density.numpy(), sh_np, basis_dim, off, scl)
    return spec, og


def rays_pair(o, d, device="cuda"):
    from svox2_gb300 import csrc as C
    r = C.RaysSpec()
    r.origins = o.to(device).contiguous()
    r.dirs = d.to(device).contiguous()
    return r


def assert_rgb(k, o, what=""):
    k = np.asarray(k, dtype=np.float64)
    o = np.asarray(o, dtype=np.float64)
    err = np.abs(k - o)
    bad = err > RTOL_RGB * np.abs(o) + ATOL_RGB
    assert not bad.any(), f"{what}: {bad.sum()} colour entries off, max err {err.max():.3e}"


def assert_grad(k, o, what=""):
    k = np.asarray(k, dtype=np.float64)
    o = np.asarray(o, dtype=np.float64)
    scale = max(np.abs(o).max(), 1e-30)
    err = np.abs(k - o)
    bad = err > RTOL_GRAD * np.abs(o) + ATOL_GRAD_FRAC * scale
    assert not bad.any(), (f"{what}: {bad.sum()} of {bad.size} gradient entries off, max err "
                           f"{err.max():.3e} (max |ref| {scale:.3e})")


def rel_err(k, o):
    k = np.asarray(k, dtype=np.float64)
    o = np.asarray(o, dtype=np.float64)
    return float(np.abs(k - o).max() / max(np.abs(o).max(), 1e-30))
