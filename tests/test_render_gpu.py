"""Parity of the CUDA ray march / fused adjoint / backward / image render with
the CPU oracle, through the reference-facing operator API (svox2_gb300.csrc ->
C ABI).  Every case checks:
  * sample indexing bit for bit against the float32 oracle (per-ray hash of
    every sample's cell and evaluated flag, plus skips) and the evaluated-sample
    count;
  * colours within 1e-5 relative of the float32 oracle and of the float64 oracle;
  * gradients per entry against the float64 oracle evaluated along the same
    samples: within 1e-5 relative, or within the float32 summation floor
    (helpers.assert_grad_f64), with the measured floor printed for the kernel and
    for the float32 oracle (the reference's algorithm in float);
  * the touched-voxel mask exactly."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S

from helpers import assert_grad_f64, assert_rgb, check_fused, grid_pair, opt_struct, rays_pair, stats_dict as _stats

pytestmark = pytest.mark.gpu


def _run_fused(spec, og, rays, o, d, gt, opt, oopt, beta=0.0, sparsity=0.0, long_rays=False, label=""):
    from svox2_gb300 import csrc as C
    Q = o.shape[0]
    N = og.density.shape[0]
    rgb = torch.zeros((Q, 3), device="cuda")
    grads = C.GridOutputGrads()
    grads.grad_density_out = torch.zeros((N, 1), device="cuda")
    grads.grad_sh_out = torch.zeros((N, og.sh.shape[1]), device="cuda")
    grads.mask_out = torch.zeros((N,), dtype=torch.bool, device="cuda")
    st = _stats(Q)
    C.volume_render_cuvol_fused(spec, rays, opt, gt.cuda(), beta, sparsity, rgb, grads, stats=st)
    torch.cuda.synchronize()
    ref, _ = check_fused(rgb, grads, st["ray_trace"].cpu().numpy(), st["eval_samples"].item(), og, oopt, o, d, gt,
                         beta=beta, sparsity=sparsity, long_rays=long_rays, label=label)
    return rgb, grads, ref


CASES = {
    # name: (reso, occupancy, basis_dim, sh dtype, n rays, options)
    "dense32_sh9": (32, None, 9, torch.float32, 1024, {}),
    "sparse48_sh9": (48, 0.2, 9, torch.float32, 1024, {}),
    "noncubic_sh4": ((20, 28, 36), 0.3, 4, torch.float32, 768, {"bg": 0.3}),
    "dense24_sh1": (24, None, 1, torch.float32, 512, {"bg": 0.0}),
    "sparse40_bf16": (40, 0.25, 9, torch.bfloat16, 768, {}),
    "sparse40_f16": (40, 0.25, 9, torch.float16, 768, {}),
    "step03_no_stop": (24, None, 9, torch.float32, 512, {"step": 0.3, "stop_thresh": 0.0}),
    "thresh_hi": (32, 0.4, 9, torch.float32, 768, {"sigma_thresh": 5.0, "stop_thresh": 1e-3}),
    "near_clip": (32, None, 9, torch.float32, 512, {"near_clip": 0.4}),
    "spheric_clip": (32, None, 9, torch.float32, 512, {"spheric": True, "near_clip": 0.1}),
}


@pytest.mark.parametrize("name", list(CASES))
def test_fused_parity(name):
    reso, occ, bd, dt, Q, kw = CASES[name]
    g = S.make_grid(reso, occupancy=occ, basis_dim=9, seed=3)
    spec, og = grid_pair(g, basis_dim=bd, sh_dtype=dt)
    o, d, gt = S.make_rays(Q, seed=4)
    opt, oopt = opt_struct(**kw)
    _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt, label=name)


def test_fused_last_sample_opaque():
    """last_sample_opaque gives the final sample a 1e9 world step.  The reference's
    forward-order adjoint forms accum = dot(C, g) - sum(w tc), a rounding residual
    near zero at the last sample, and multiplies it by that step: its float32
    density gradient there is rounding noise of order 1e-2.  The reverse-order
    adjoint accumulates the suffix sum directly (exactly 0 after an opaque
    sample), so its gradients are checked against the float64 restatement."""
    g = S.make_grid(32, occupancy=0.5, seed=3)
    spec, og = grid_pair(g)
    o, d, gt = S.make_rays(512, seed=4)
    opt, oopt = opt_struct(last_opaque=True)
    _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt, label="last_opaque")


def test_fused_sorted_batch():
    """Batches of 32768 rays and more run in coherence-key order (a permutation
    applied inside the library); results land at the rays' own positions."""
    g = S.make_grid(48, occupancy=0.3, seed=61)
    spec, og = grid_pair(g)
    o, d, gt = S.make_rays(40000, seed=62)
    opt, oopt = opt_struct()
    _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt, label="sorted48")


def test_fused_beta_sparsity():
    g = S.make_grid(32, occupancy=0.3, seed=5)
    spec, og = grid_pair(g)
    o, d, gt = S.make_rays(768, seed=6)
    opt, oopt = opt_struct()
    _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt, beta=0.5, sparsity=0.01)


def test_long_rays_colour_cache_and_checkpoint_thinning():
    """Rays with > 192 evaluated samples (colours re-gathered in the reverse pass)
    and > 64 evaluated segments (checkpoints thinned to every 2nd and 4th segment)."""
    reso = (3, 3, 1800)
    g = S.make_grid(reso, seed=7, density_mode="normal53")
    g.density.mul_(0.004)   # transparent enough that rays run the whole length
    spec, og = grid_pair(g)
    Q = 96
    gen = torch.Generator().manual_seed(8)
    o = torch.zeros((Q, 3))
    o[:, 0] = (torch.rand(Q, generator=gen) - 0.5) * 1.0
    o[:, 1] = (torch.rand(Q, generator=gen) - 0.5) * 1.0
    o[:, 2] = -1.3
    d = torch.zeros((Q, 3))
    d[:, 0] = (torch.rand(Q, generator=gen) - 0.5) * 1e-3
    d[:, 1] = (torch.rand(Q, generator=gen) - 0.5) * 1e-3
    d[:, 2] = 1.0
    d = d / d.norm(dim=-1, keepdim=True)
    gt = torch.rand((Q, 3), generator=gen)
    opt, oopt = opt_struct(stop_thresh=0.0)
    _, _, ref = _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt, long_rays=True)
    assert ref["n_eval"] > Q * 2500


def test_edge_cases():
    from svox2_gb300 import csrc as C
    # all-empty grid: every ray renders the background, no gradient, no mask
    g = S.make_grid(16, seed=9)
    g.links.fill_(-1)
    spec, og = grid_pair(g)
    o, d, gt = S.make_rays(256, seed=10)
    opt, oopt = opt_struct(bg=0.7)
    rgb, grads, _ = _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt)
    assert torch.allclose(rgb, torch.full_like(rgb, 0.7))
    assert not grads.mask_out.any()
    # smallest grid (2^3), axis-aligned rays (zero direction components), rays that miss
    g = S.make_grid(2, seed=11)
    spec, og = grid_pair(g)
    o = torch.tensor([[0.0, 0.0, -3.0], [0.1, -2.5, 0.2], [5.0, 5.0, 5.0], [0.3, 0.2, -2.0], [-2.0, 0.5, 0.5]])
    d = torch.tensor([[0.0, 0.0, 1.0], [0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.6, 0.8], [1.0, 0.0, 0.0]])
    gt = torch.rand((5, 3), generator=torch.Generator().manual_seed(0))
    opt, oopt = opt_struct()
    _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt)
    # zero rays: no launch, no error
    r = C.RaysSpec()
    r.origins = torch.zeros((0, 3), device="cuda")
    r.dirs = torch.zeros((0, 3), device="cuda")
    out = C.volume_render_cuvol(spec, r, opt)
    assert out.shape == (0, 3)


def test_forward_and_backward_only():
    from svox2_gb300 import csrc as C
    g = S.make_grid(40, occupancy=0.3, seed=12)
    spec, og = grid_pair(g)
    o, d, gt = S.make_rays(1024, seed=13)
    rays = rays_pair(o, d)
    opt, oopt = opt_struct()
    st = _stats(1024)
    rgb = C.volume_render_cuvol(spec, rays, opt, stats=st)
    torch.cuda.synchronize()
    ref = O.render(og, oopt, o.numpy(), d.numpy(), mode=0, trace=True)
    assert (st["ray_trace"].cpu().numpy().view(np.uint64) == ref["trace"]).all()
    assert_rgb(rgb.cpu().numpy(), ref["rgb"], "forward")
    # backward with an arbitrary upstream gradient
    go = torch.randn((1024, 3), generator=torch.Generator().manual_seed(14))
    N = og.density.shape[0]
    grads = C.GridOutputGrads()
    grads.grad_density_out = torch.zeros((N, 1), device="cuda")
    grads.grad_sh_out = torch.zeros((N, 27), device="cuda")
    C.volume_render_cuvol_backward(spec, rays, opt, go.cuda(), rgb, grads)
    rb = O.render(og, oopt, o.numpy(), d.numpy(), mode=2, grad_out=go.numpy(), color=ref["rgb"], prec="f64",
                  stops=ref["stops"], want_magnitude=True)
    assert_grad_f64(grads.grad_density_out.cpu().numpy(), rb["grad_density"], rb["mag_density"], "bwd grad_density")
    assert_grad_f64(grads.grad_sh_out.cpu().numpy(), rb["grad_sh"], rb["mag_sh"], "bwd grad_sh")
    # gradients accumulate into existing buffers
    C.volume_render_cuvol_backward(spec, rays, opt, go.cuda(), rgb, grads)
    assert_grad_f64(grads.grad_sh_out.cpu().numpy(), 2 * rb["grad_sh"], 2 * rb["mag_sh"], "accumulated grad_sh")


@pytest.mark.parametrize("ndc", [False, True])
def test_image_parity(ndc):
    from svox2_gb300 import csrc as C
    g = S.make_grid(48, occupancy=0.3, seed=15)
    spec, og = grid_pair(g)
    if ndc:
        c2w = torch.eye(4)
        c2w[:3, 3] = torch.tensor([0.05, -0.02, 0.0])
        ndc_c = (1.4, 1.2)
    else:
        c2w = S.look_at_c2w((0.4, -0.7, -3.2))
        ndc_c = (-1.0, -1.0)
    cam = C.CameraSpec()
    cam.c2w = c2w.cuda()
    cam.fx, cam.fy, cam.cx, cam.cy = 70.0, 72.0, 31.5, 24.0
    cam.width, cam.height = 64, 48
    cam.ndc_coeffx, cam.ndc_coeffy = ndc_c
    opt, oopt = opt_struct()
    st = _stats(64 * 48)
    img = C.volume_render_cuvol_image(spec, cam, opt, stats=st)
    torch.cuda.synchronize()
    ref = O.render_image(og, oopt, c2w.numpy(), 70.0, 72.0, 31.5, 24.0, 64, 48, ndc=ndc_c, trace=True)
    assert (st["ray_trace"].cpu().numpy().view(np.uint64) == ref["trace"]).all()
    assert_rgb(img.cpu().numpy(), ref["rgb"], "image")


def test_accelerated_links_skip():
    """Negative links below -1 (empty-space skip levels) are honoured exactly."""
    g = S.make_grid(32, occupancy=0.25, seed=16)
    links = g.links.clone()
    # mark empty 4^3 blocks with skip level -3 (2^(3-1) = 4 cells), the way accel_dist_prop encodes them
    L = links.view(8, 4, 8, 4, 8, 4).permute(0, 2, 4, 1, 3, 5).reshape(8, 8, 8, 64)
    empty = (L < 0).all(dim=-1)
    L[empty] = -3
    g.links = L.view(8, 8, 8, 4, 4, 4).permute(0, 3, 1, 4, 2, 5).reshape(32, 32, 32).contiguous()
    spec, og = grid_pair(g)
    o, d, gt = S.make_rays(1024, seed=17)
    opt, oopt = opt_struct()
    _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt)


def test_adjoint_sample_limit_is_enforced():
    """A ray may need up to diagonal / step_size samples; beyond what the adjoint's checkpoints
    cover (64 checkpoints, each at most 64 segments of 32 samples apart: 131,072 samples) the
    fused and backward renders refuse on the host; the forward runs."""
    from svox2_gb300 import csrc as C
    g = S.make_grid(32, seed=30)
    spec, og = grid_pair(g)
    o, d, gt = S.make_rays(64, seed=31)
    opt, _ = opt_struct(step=0.0004)           # 32 * sqrt(3) / 0.0004 ~ 138,566 samples > 131,072
    rays = rays_pair(o, d)
    N = og.density.shape[0]
    grads = C.GridOutputGrads()
    grads.grad_density_out = torch.zeros((N, 1), device="cuda")
    grads.grad_sh_out = torch.zeros((N, og.sh.shape[1]), device="cuda")
    grads.mask_out = torch.zeros((N,), dtype=torch.bool, device="cuda")
    rgb = torch.zeros((64, 3), device="cuda")
    with pytest.raises(RuntimeError, match="samples per ray"):
        C.volume_render_cuvol_fused(spec, rays, opt, gt.cuda(), 0.0, 0.0, rgb, grads)
    assert C.volume_render_cuvol(spec, rays, opt).shape == (64, 3)


def test_rays_near_the_adjoint_sample_limit():
    """Rays of ~126,000 evaluated samples, just inside the checkpoints' 131,072: checkpoints
    thinned to a stride of 64 segments, and colours past the colour cache's 4096 samples
    gathered again in the reverse pass.  (Every march ends at t = 2000 grid units, as the
    reference's ray_find_bounds sets it, so rays this long need a small step.)"""
    reso = (2, 2, 1900)
    g = S.make_grid(reso, seed=41, density_mode="normal53")
    g.density.mul_(1e-5)   # transparent enough that the rays run the whole length
    spec, og = grid_pair(g)
    Q = 8
    gen = torch.Generator().manual_seed(42)
    o = torch.zeros((Q, 3))
    o[:, 0] = (torch.rand(Q, generator=gen) - 0.5) * 0.5
    o[:, 1] = (torch.rand(Q, generator=gen) - 0.5) * 0.5
    o[:, 2] = -1.05
    d = torch.zeros((Q, 3))
    d[:, 0] = (torch.rand(Q, generator=gen) - 0.5) * 1e-6
    d[:, 1] = (torch.rand(Q, generator=gen) - 0.5) * 1e-6
    d[:, 2] = 1.0
    d = d / d.norm(dim=-1, keepdim=True)
    gt = torch.rand((Q, 3), generator=gen)
    opt, oopt = opt_struct(stop_thresh=0.0, step=0.015)
    _, _, ref = _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt, long_rays=True, label="near limit")
    assert ref["n_eval"] > Q * 120000, ref["n_eval"]


def test_invalid_arguments_raise():
    from svox2_gb300 import csrc as C
    g = S.make_grid(8, seed=18)
    spec, _ = grid_pair(g)
    o, d, gt = S.make_rays(4, seed=19)
    opt, _ = opt_struct()
    with pytest.raises(RuntimeError):
        C.volume_render_cuvol(spec, rays_pair(o.double(), d.double()), opt)
    bad = rays_pair(o, d)
    bad.origins = o  # CPU tensor
    with pytest.raises(RuntimeError):
        C.volume_render_cuvol(spec, bad, opt)
    spec.basis_dim = 16
    with pytest.raises(RuntimeError):
        C.volume_render_cuvol(spec, rays_pair(o, d), opt)
    # a 16-bit SH table starting at an odd element is not 4-byte aligned: refused on the host
    spec.basis_dim = 9
    N = g.density.shape[0]
    buf = torch.zeros(N * 27 + 1, dtype=torch.bfloat16, device="cuda")
    spec.sh_data = buf[1:].view(N, 27)
    with pytest.raises(RuntimeError, match="4-byte aligned"):
        C.volume_render_cuvol(spec, rays_pair(o, d), opt)
