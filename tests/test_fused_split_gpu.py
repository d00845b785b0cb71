"""The fused step and the plain backward as two kernels (a forward with per-ray records, then
the reverse pass from them).

For SH9 grids, svx_volume_render_cuvol_fused (with or without the MSI background) and
svx_volume_render_cuvol_backward (without it) run as two kernels when the per-ray records fit
the budget (SVX_FUSED_SPLIT_BYTES, read at each call), in chunks of rays when they do not all fit
at once, and as one kernel when the budget is 0.  Every GPU test of those entries runs the
two-kernel form at its default budget; this file holds the forms to one another and to the
oracle on the same inputs:
  * colours and the per-ray sample trace bit for bit between the forms (the forward arithmetic is
    the same; only the gradient atomics' order differs);
  * gradients and masks of each form against the oracle (helpers.check_fused, assert_grad_f64);
  * an unsorted small batch, a coherence-sorted batch with the accumulation rows, several chunks,
    BF16 storage, last_sample_opaque and the beta / sparsity terms; the plain backward; the MSI
    background (forms against each other).
"""
import os

import numpy as np
import pytest
import torch

from svox2_gb300 import synthetic as S

from helpers import check_fused, grid_pair, opt_struct, rays_pair, run_fused_kernel

pytestmark = pytest.mark.gpu

ENV = "SVX_FUSED_SPLIT_BYTES"


def _run(budget, spec, rays, opt, gt, N, n_sh, **kw):
    old = os.environ.get(ENV)
    try:
        if budget is None:
            os.environ.pop(ENV, None)
        else:
            os.environ[ENV] = str(budget)
        return run_fused_kernel(spec, rays, opt, gt, N, n_sh, **kw)
    finally:
        if old is None:
            os.environ.pop(ENV, None)
        else:
            os.environ[ENV] = old


def _record_bytes(reso, step=0.5):
    # 2 + cap float4 and cap float2 entries per ray, cap = ceil(max samples / 32) * 32, as the
    # host sizes them
    cap = int(np.ceil((np.sqrt(3.0) * reso / step + 2.0) / 32.0) * 32)
    return 16 * (2 + cap + cap // 2)


CASES = {
    # name: (reso, occupancy, rays, sh dtype, chunks, opt kwargs, beta, sparsity)
    "small_unsorted": (40, 0.3, 3000, torch.float32, 1, {}, 0.0, 0.0),
    "sorted_40960": (48, 0.3, 40960, torch.float32, 1, {}, 0.0, 0.0),
    "sorted_40960_5chunks": (48, 0.3, 40960, torch.float32, 5, {}, 0.0, 0.0),
    "bf16_sorted": (48, 0.3, 40960, torch.bfloat16, 1, {}, 0.0, 0.0),
    "opaque_beta_sparsity": (40, 0.3, 3000, torch.float32, 1, {"last_opaque": True}, 0.3, 0.01),
}


@pytest.mark.parametrize("name", list(CASES))
def test_two_kernel_fused_matches_one_kernel_and_oracle(name):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    reso, occ, Q, dt, chunks, okw, beta, sparsity = CASES[name]
    grid = S.make_grid(reso, occupancy=occ, seed=61)
    spec, og = grid_pair(grid, sh_dtype=dt)
    o, d, gt = S.make_rays(Q, seed=62)
    rays = rays_pair(o, d)
    opt, oopt = opt_struct(**okw)
    N, n_sh = og.density.shape[0], og.sh.shape[1]
    kw = dict(beta=beta, sparsity=sparsity)
    budget = None if chunks == 1 else _record_bytes(reso) * ((Q + chunks - 1) // chunks)
    two = _run(budget, spec, rays, opt, gt, N, n_sh, **kw)
    one = _run(0, spec, rays, opt, gt, N, n_sh, **kw)
    for key in ("ray_trace", "eval_samples"):
        np.testing.assert_array_equal(two[2][key].cpu().numpy(), one[2][key].cpu().numpy())
    np.testing.assert_array_equal(two[0].cpu().numpy(), one[0].cpu().numpy())
    np.testing.assert_array_equal(two[1].mask_out.cpu().numpy(), one[1].mask_out.cpu().numpy())
    for label, (rgb, grads, st) in (("two kernels", two), ("one kernel", one)):
        check_fused(rgb, grads, st["ray_trace"].cpu().numpy(), st["eval_samples"].item(), og, oopt, o, d, gt,
                    beta=beta, sparsity=sparsity, label=f"{name} {label}")


def _bwd(budget, spec, rays, opt, go, N, n_sh):
    from svox2_gb300 import csrc as C
    grads = C.GridOutputGrads()
    grads.grad_density_out = torch.zeros((N, 1), device="cuda")
    grads.grad_sh_out = torch.zeros((N, n_sh), device="cuda")
    old = os.environ.get(ENV)
    try:
        if budget is None:
            os.environ.pop(ENV, None)
        else:
            os.environ[ENV] = str(budget)
        C.volume_render_cuvol_backward(spec, rays, opt, go, None, grads)
        torch.cuda.synchronize()
    finally:
        if old is None:
            os.environ.pop(ENV, None)
        else:
            os.environ[ENV] = old
    return grads


@pytest.mark.parametrize("Q", [1024, 40960])
def test_two_kernel_backward_matches_one_kernel_and_oracle(Q):
    """The plain backward (given dL/dcolour) in both forms against the float64 oracle."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from helpers import assert_grad_f64
    import oracle.oracle as O
    grid = S.make_grid(40, occupancy=0.3, seed=63)
    spec, og = grid_pair(grid)
    o, d, _ = S.make_rays(Q, seed=64)
    rays = rays_pair(o, d)
    opt, oopt = opt_struct()
    go = torch.randn((Q, 3), generator=torch.Generator().manual_seed(65))
    N, n_sh = og.density.shape[0], og.sh.shape[1]
    ref = O.render(og, oopt, o.numpy(), d.numpy(), mode=0, trace=False)
    rb = O.render(og, oopt, o.numpy(), d.numpy(), mode=2, grad_out=go.numpy(), color=ref["rgb"], prec="f64",
                  stops=ref["stops"], want_magnitude=True)
    two = _bwd(None, spec, rays, opt, go.cuda(), N, n_sh)
    one = _bwd(0, spec, rays, opt, go.cuda(), N, n_sh)
    for label, gr in (("two kernels", two), ("one kernel", one)):
        assert_grad_f64(gr.grad_density_out.cpu().numpy(), rb["grad_density"], rb["mag_density"],
                        f"{Q} {label} grad_density")
        assert_grad_f64(gr.grad_sh_out.cpu().numpy(), rb["grad_sh"], rb["mag_sh"], f"{Q} {label} grad_sh")


@pytest.mark.parametrize("Q", [2000, 40960])
def test_two_kernel_background_matches_one_kernel(Q):
    """With the MSI background the forward kernel also runs the background's adjoint; both forms
    on the same inputs: colours bit for bit, masks equal, gradients within 1e-5 of the largest
    entry (only the atomics' order differs).  The background tests hold the default form to
    the oracle and to the reference's kernels."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from svox2_gb300 import csrc as C
    grid = S.make_grid(24, occupancy=0.3, seed=66)
    spec, og = grid_pair(grid)
    gen = torch.Generator().manual_seed(67)
    keep = torch.rand((32, 16), generator=gen) >= 0.2
    links = torch.full(keep.shape, -1, dtype=torch.int32)
    links[keep] = torch.arange(int(keep.sum()), dtype=torch.int32)
    data = torch.randn((int(keep.sum()), 8, 4), generator=gen) * 0.5
    data[..., 3] = torch.rand((int(keep.sum()), 8), generator=gen) * 4.0 - 0.5
    spec.background_links, spec.background_data = links.cuda(), data.cuda()
    o, d, gt = S.make_rays(Q, seed=68)
    dr = torch.randn((Q // 2, 3), generator=gen)
    d[Q // 2:] = dr / dr.norm(dim=-1, keepdim=True)
    rays = rays_pair(o, d.contiguous())
    opt, _ = opt_struct()
    N, n_sh = og.density.shape[0], og.sh.shape[1]
    out = {}
    for budget in (None, 0):
        old = os.environ.get(ENV)
        try:
            if budget is None:
                os.environ.pop(ENV, None)
            else:
                os.environ[ENV] = str(budget)
            rgb = torch.zeros((Q, 3), device="cuda")
            grads = C.GridOutputGrads()
            grads.grad_density_out = torch.zeros((N, 1), device="cuda")
            grads.grad_sh_out = torch.zeros((N, n_sh), device="cuda")
            grads.mask_out = torch.zeros((N,), dtype=torch.bool, device="cuda")
            grads.grad_background_out = torch.zeros(tuple(data.shape), device="cuda")
            grads.mask_background_out = torch.zeros(tuple(data.shape[:2]), dtype=torch.bool, device="cuda")
            C.volume_render_cuvol_fused(spec, rays, opt, gt.cuda(), 0.0, 0.0, rgb, grads)
            torch.cuda.synchronize()
            out[budget] = (rgb, grads)
        finally:
            if old is None:
                os.environ.pop(ENV, None)
            else:
                os.environ[ENV] = old
    (r2, g2), (r1, g1) = out[None], out[0]
    np.testing.assert_array_equal(r2.cpu().numpy(), r1.cpu().numpy())
    for key in ("mask_out", "mask_background_out"):
        np.testing.assert_array_equal(getattr(g2, key).cpu().numpy(), getattr(g1, key).cpu().numpy())
    for key in ("grad_density_out", "grad_sh_out", "grad_background_out"):
        a, b = getattr(g2, key).cpu().numpy().astype(np.float64), getattr(g1, key).cpu().numpy()
        err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)
        assert err <= 1e-5, f"{Q} {key}: two-kernel vs one-kernel {err:.2e}"
