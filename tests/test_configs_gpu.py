"""Parity at the benchmarked configurations' own sizes, and the kernel on the reference's
own outputs.

  * 64^3 dense grid, 4096 rays, seed 0 (the CPU-runnable configuration), in full;
  * the 256^3, 20%-occupancy training-step grid (3.36 M voxels) with a 40,960-ray sample of a
    training batch: at >= 32,768 rays the library runs rays in coherence order and scatters
    gradients through its padded [N][28] accumulation rows and the add pass, which is the
    path the benchmark times;
  * the 512^3, 8%-occupancy grid (32 balls, 10.7 M voxels) with SH stored as bfloat16 and as
    float16, on a 40,960-ray sample;
  * every render fixture that the reference's own CPU path wrote (tests/golden/render_*.npz,
    sigma and stop thresholds 0, the setting in which the reference's CPU path and kernels
    compute the same thing): colours and gradients of the kernel against the reference's.

Each case prints the kernel's per-entry floor and errors against the float64 oracle beside
the float32 oracle's (helpers.check_fused)."""
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S

from helpers import assert_grad_f64, check_fused, grid_pair, opt_struct, rays_pair, rel_err, run_fused_kernel

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
RENDER = sorted(GOLD.glob("render_*.npz"))


def _case(g, o, d, gt, sh_dtype=torch.float32, label="", **opt_kw):
    spec, og = grid_pair(g, sh_dtype=sh_dtype)
    opt, oopt = opt_struct(**opt_kw)
    rgb, grads, st = run_fused_kernel(spec, rays_pair(o, d), opt, gt, og.density.shape[0], og.sh.shape[1])
    check_fused(rgb, grads, st["ray_trace"].cpu().numpy(), st["eval_samples"].item(), og, oopt, o, d, gt,
                label=label)


def test_dense64_4096_rays_full():
    g = S.make_grid(64, occupancy=None, seed=0)
    o, d, gt = S.make_rays(4096, seed=0)
    _case(g, o, d, gt, label="dense64 4096 rays")


def test_train_grid_256_sorted_sample():
    g = S.make_grid(256, occupancy=0.20, n_balls=8, seed=0, device="cuda")
    assert g.density.shape[0] > 3_300_000
    o, d, gt = S.make_rays(1_000_000, seed=1)
    q = 40960
    _case(g, o[:q].contiguous(), d[:q].contiguous(), gt[:q].contiguous(), label="256^3 20% 40960 rays")


@pytest.mark.parametrize("sh_dtype", [torch.bfloat16, torch.float16], ids=["bf16", "f16"])
def test_mixed_grid_512_sample(sh_dtype):
    g = S.make_grid(512, occupancy=0.08, n_balls=32, seed=0, device="cuda")
    assert g.density.shape[0] > 10_000_000
    o, d, gt = S.make_rays(40960, seed=2000)
    _case(g, o, d, gt, sh_dtype=sh_dtype, label=f"512^3 8% {sh_dtype} 40960 rays")


@pytest.mark.parametrize("path", RENDER, ids=[p.stem for p in RENDER])
def test_kernel_on_reference_fixture(path):
    """The kernel against the colours and gradients the reference's own CPU path computed
    (volume_render(use_kernel=False) + autograd of the MSE loss), and per entry against the
    float64 oracle."""
    from svox2_gb300 import csrc as C
    z = np.load(path)
    spec = C.SparseGridSpec()
    spec.links = torch.from_numpy(z["links"]).cuda()
    spec.density_data = torch.from_numpy(z["density"]).cuda()
    spec.sh_data = torch.from_numpy(z["sh"]).cuda()
    spec._offset = torch.from_numpy(z["offset"])
    spec._scaling = torch.from_numpy(z["scaling"])
    spec.basis_dim = int(z["basis_dim"])
    spec.basis_type = 1
    o, d, gt = (torch.from_numpy(z[k]) for k in ("origins", "dirs", "rgb_gt"))
    opt, oopt = opt_struct(sigma_thresh=0.0, stop_thresh=0.0, bg=float(z["bg"]), step=float(z["step"]))
    N, Cc = z["sh"].shape
    rgb, grads, st = run_fused_kernel(spec, rays_pair(o, d), opt, gt, N, Cc)
    k_rgb = rgb.cpu().numpy()
    k_gd = grads.grad_density_out.cpu().numpy()
    k_gs = grads.grad_sh_out.cpu().numpy()
    # the reference's float32 CPU arithmetic vs this kernel (different rounding order)
    np.testing.assert_allclose(k_rgb, z["rgb"], rtol=2e-6, atol=1e-6)
    assert rel_err(k_gd, z["grad_density"]) < 1e-5
    assert rel_err(k_gs, z["grad_sh"]) < 1e-5
    touched = (z["grad_sh"] != 0).any(axis=1) | (z["grad_density"][:, 0] != 0)
    m = grads.mask_out.cpu().numpy()
    assert not np.any(touched & ~m), "a voxel the reference path gave a gradient is not marked"
    og = O.Grid(z["links"], z["density"], z["sh"], int(z["basis_dim"]), tuple(z["offset"]), tuple(z["scaling"]))
    ref = O.render(og, oopt, z["origins"], z["dirs"], mode=1, rgb_gt=z["rgb_gt"], prec="f32", trace=True)
    assert (st["ray_trace"].cpu().numpy().view(np.uint64) == ref["trace"]).all()
    r64 = O.render(og, oopt, z["origins"], z["dirs"], mode=1, rgb_gt=z["rgb_gt"], prec="f64", stops=ref["stops"],
                   want_magnitude=True)
    assert_grad_f64(k_gd, r64["grad_density"], r64["mag_density"], f"{path.stem} grad_density")
    assert_grad_f64(k_gs, r64["grad_sh"], r64["mag_sh"], f"{path.stem} grad_sh")
    print(f"{path.stem}: kernel vs reference rgb {np.abs(k_rgb - z['rgb']).max():.2e}, "
          f"grad_density {rel_err(k_gd, z['grad_density']):.2e}, grad_sh {rel_err(k_gs, z['grad_sh']):.2e}; "
          f"reference vs f64 oracle rgb {np.abs(z['rgb'] - r64['rgb']).max():.2e}")
