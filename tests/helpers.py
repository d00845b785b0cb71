"""Shared helpers for the parity tests: build the same seeded inputs for the
CUDA operators (svox2_gb300.csrc, the reference-facing API) and for the CPU
oracle, and compare results with stated tolerances."""
from __future__ import annotations

import numpy as np
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S

# Tolerances.
#   colours: |k - o| <= RTOL_RGB * |o| + ATOL_RGB
#   gradients of the render, per entry, against the float64 oracle run along the float32 run's
#   samples (oracle.render(..., prec="f64", stops=...)):
#       |k - o64| <= RTOL_GRAD * |o64|   or   |k - o64| <= FLOOR_K * u * mag
#   with u = 2^-24 and mag the entry's first-order float32 error bound from the float64 oracle
#   (oracle_impl.h bwd_ray): the sum over its terms of |term| times the rounding units that a
#   float32 evaluation of that term can lose (the transmittance chain, the trilinear lerp's
#   cancellation near an empty face, the SH basis's xx - yy differences, the loss residual
#   out - gt, the light behind the sample summed over the ray, the colour clamp's kink).  The
#   second form is the float32 floor: an entry whose terms cancel, or whose terms are small
#   against their rounding, cannot be held to a fraction of its own value.  FLOOR_K allows 4x
#   the bound; the kernel's measured worst case is printed by every check.
#   gradients of other operators (sample, TV, ...): assert_grad, relative to the largest entry.
RTOL_RGB, ATOL_RGB = 1e-5, 1e-6
RTOL_GRAD = 1e-5
FLOOR_K = 4.0
U32 = 2.0 ** -24
RTOL_GRAD_OP, ATOL_GRAD_FRAC = 1e-4, 1e-5


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
    """Gradients of the non-render operators (sample, TV): relative to the largest entry."""
    k = np.asarray(k, dtype=np.float64)
    o = np.asarray(o, dtype=np.float64)
    scale = max(np.abs(o).max(), 1e-30)
    err = np.abs(k - o)
    bad = err > RTOL_GRAD_OP * np.abs(o) + ATOL_GRAD_FRAC * scale
    assert not bad.any(), (f"{what}: {bad.sum()} of {bad.size} gradient entries off, max err "
                           f"{err.max():.3e} (max |ref| {scale:.3e})")


def floor_ratio(k, o64, mag):
    """(worst |k - o64| / (u * mag) over the entries outside RTOL_GRAD of o64, how many such
    entries there are, worst relative error over all nonzero entries)."""
    k = np.asarray(k, dtype=np.float64)
    o64 = np.asarray(o64, dtype=np.float64)
    mag = np.asarray(mag, dtype=np.float64)
    err = np.abs(k - o64)
    out = err > RTOL_GRAD * np.abs(o64)
    r = err[out] / (U32 * np.maximum(mag[out], 1e-300)) if out.any() else np.zeros(1)
    nz = o64 != 0
    rel = float((err[nz] / np.abs(o64[nz])).max()) if nz.any() else 0.0
    return float(r.max()), int(out.sum()), rel


def assert_grad_f64(k, o64, mag, what="", k32=None):
    """Render gradients per entry against the float64 oracle: within RTOL_GRAD relative, or
    within FLOOR_K * u * mag (the float32 summation floor).  Prints the measured floor of the
    kernel and, when given, of the float32 oracle (the reference's algorithm in float)."""
    K, n_out, rel = floor_ratio(k, o64, mag)
    msg = f"{what}: floor {K:.2f} u*mag over {n_out} entries outside {RTOL_GRAD:g} rel (worst rel {rel:.1e})"
    if k32 is not None:
        K32, n32, rel32 = floor_ratio(k32, o64, mag)
        msg += f"; float32 oracle: floor {K32:.2f} over {n32} entries (worst rel {rel32:.1e})"
    print(msg)
    assert K <= FLOOR_K, msg
    return K


def rel_err(k, o):
    k = np.asarray(k, dtype=np.float64)
    o = np.asarray(o, dtype=np.float64)
    return float(np.abs(k - o).max() / max(np.abs(o).max(), 1e-30))


def stats_dict(Q):
    """The stats outputs of a render call: evaluated-sample count and per-ray sample trace."""
    return {"eval_samples": torch.zeros(1, dtype=torch.int64, device="cuda"),
            "ray_trace": torch.zeros(Q, dtype=torch.int64, device="cuda")}


def check_fused(rgb, grads, trace, n_eval, og, oopt, o, d, gt, beta=0.0, sparsity=0.0, long_rays=False,
                label=""):
    """Compare a fused render (colours, gradients, mask, and when given the per-ray trace and
    evaluated-sample count) with the oracle.  long_rays: thousands of samples per ray summed in
    float32; colours are held to the float64 yardstick at twice the float32 oracle's own error
    (the oracle keeps the reference's 1 - exp(-x) weight, which loses digits on such thin
    media).  Returns (float32 result, float64 result)."""
    o_np, d_np, gt_np = (x.numpy() if torch.is_tensor(x) else x for x in (o, d, gt))
    ref = O.render(og, oopt, o_np, d_np, mode=1, rgb_gt=gt_np, beta_loss=beta, sparsity_loss=sparsity,
                   prec="f32", trace=trace is not None)
    if trace is not None:
        mism = int((np.asarray(trace).view(np.uint64) != ref["trace"]).sum())
        assert mism == 0, f"{label}: sample indexing differs on {mism} of {o_np.shape[0]} rays"
    if n_eval is not None:
        assert int(n_eval) == ref["n_eval"], f"{label}: evaluated samples {int(n_eval)} vs {ref['n_eval']}"
    if grads.mask_out is not None:
        np.testing.assert_array_equal(grads.mask_out.cpu().numpy(), ref["mask"])
    r64 = O.render(og, oopt, o_np, d_np, mode=1, rgb_gt=gt_np, beta_loss=beta, sparsity_loss=sparsity,
                   prec="f64", stops=ref["stops"], want_magnitude=True)
    k_rgb = rgb.cpu().numpy()
    if long_rays:
        e_k = np.abs(k_rgb - r64["rgb"]).max()
        e_o = np.abs(ref["rgb"] - r64["rgb"]).max()
        assert e_k <= 2 * e_o + 1e-6, f"{label}: long-ray colour error {e_k:.2e} vs float32 oracle's {e_o:.2e}"
    else:
        assert_rgb(k_rgb, ref["rgb"], f"{label} rgb vs float32 oracle")
        assert_rgb(k_rgb, r64["rgb"], f"{label} rgb vs float64 oracle")
    assert_grad_f64(grads.grad_density_out.cpu().numpy(), r64["grad_density"], r64["mag_density"],
                    f"{label} grad_density", k32=ref["grad_density"])
    assert_grad_f64(grads.grad_sh_out.cpu().numpy(), r64["grad_sh"], r64["mag_sh"], f"{label} grad_sh",
                    k32=ref["grad_sh"])
    print(f"{label} vs f64: kernel rgb {rel_err(k_rgb, r64['rgb']):.2e} "
          f"gsh {rel_err(grads.grad_sh_out.cpu().numpy(), r64['grad_sh']):.2e} "
          f"gd {rel_err(grads.grad_density_out.cpu().numpy(), r64['grad_density']):.2e} | "
          f"oracle32 rgb {rel_err(ref['rgb'], r64['rgb']):.2e} gsh {rel_err(ref['grad_sh'], r64['grad_sh']):.2e} "
          f"gd {rel_err(ref['grad_density'], r64['grad_density']):.2e} (relative to the largest entry); "
          f"n_eval {ref['n_eval']}")
    return ref, r64


def run_fused_kernel(spec, rays, opt, gt, n_voxels, n_sh, beta=0.0, sparsity=0.0, mask=True):
    """volume_render_cuvol_fused through the operator API into fresh zeroed gradients;
    returns (rgb, grads, stats)."""
    from svox2_gb300 import csrc as C
    Q = rays.origins.shape[0]
    rgb = torch.zeros((Q, 3), device="cuda")
    grads = C.GridOutputGrads()
    grads.grad_density_out = torch.zeros((n_voxels, 1), device="cuda")
    grads.grad_sh_out = torch.zeros((n_voxels, n_sh), device="cuda")
    if mask:
        grads.mask_out = torch.zeros((n_voxels,), dtype=torch.bool, device="cuda")
    st = stats_dict(Q)
    C.volume_render_cuvol_fused(spec, rays, opt, gt.cuda(), beta, sparsity, rgb, grads, stats=st)
    torch.cuda.synchronize()
    return rgb, grads, st
