"""The reference-facing SparseGrid API end to end on the GPU: autograd render,
fused render, image render, sampling and a full training step, each compared
with the CPU oracle or with the other path that computes the same thing."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

from oracle import oracle as O
from svox2_gb300 import Camera, Rays, SparseGrid
from svox2_gb300 import synthetic as S

from helpers import assert_grad, assert_grad_f64, assert_rgb

pytestmark = pytest.mark.gpu


def _grid(reso=32, occ=0.35, seed=31, sh_dtype=torch.float32, z_order=False):
    g = S.make_grid(reso, occupancy=occ, seed=seed)
    grid = SparseGrid(reso=reso, basis_dim=9, device="cuda", sh_dtype=sh_dtype, use_z_order=z_order)
    if z_order:
        # keep the Morton links: rows are the allocated voxels in Morton order
        links = grid.links.cpu()
        dens = torch.zeros((links.numel(), 1))
        sh = torch.zeros((links.numel(), 27))
        m = g.links.flatten() >= 0
        dens[links.flatten()[m].long()] = g.density[g.links.flatten()[m].long()]
        sh[links.flatten()[m].long()] = g.sh[g.links.flatten()[m].long()]
        grid.density_data.data[:] = dens.cuda()
        grid.sh_data.data[:] = sh.cuda().to(sh_dtype)
    else:
        grid.links = g.links.cuda()
        grid.density_data = torch.nn.Parameter(g.density.cuda())
        grid.sh_data = torch.nn.Parameter(g.sh.cuda().to(sh_dtype))
    grid.opt.sigma_thresh = 1e-8
    grid.opt.stop_thresh = 1e-7
    return grid


def _oracle_grid(grid):
    gsz = grid._grid_size()
    return O.Grid(grid.links.cpu().numpy(), grid.density_data.detach().cpu().numpy(),
                  grid.sh_data.detach().float().cpu().numpy(), 9, tuple((grid._offset * gsz - 0.5).tolist()),
                  tuple((grid._scaling * gsz).tolist()))


@pytest.mark.parametrize("z_order", [False, True])
def test_autograd_render_matches_fused(z_order):
    grid = _grid(z_order=z_order)
    o, d, gt = S.make_rays(1500, seed=32)
    rays = Rays(o.cuda(), d.cuda())
    rgb = grid.volume_render(rays)
    F.mse_loss(rgb, gt.cuda()).backward()
    g_d = grid.density_data.grad.clone()
    g_s = grid.sh_data.grad.clone()
    grid.density_data.grad.zero_()
    grid.sh_data.grad.zero_()
    rgb2 = grid.volume_render_fused(rays, gt.cuda())
    assert torch.allclose(rgb, rgb2, rtol=0, atol=0)
    assert_grad(g_d.cpu().numpy(), grid.density_data.grad.cpu().numpy(), "density grad autograd vs fused")
    assert_grad(g_s.cpu().numpy(), grid.sh_data.grad.cpu().numpy(), "sh grad autograd vs fused")
    og = _oracle_grid(grid)
    ref = O.render(og, O.Opt(1.0, 0.5, 1e-8, 1e-7), o.numpy(), d.numpy(), mode=1, rgb_gt=gt.numpy())
    r64 = O.render(og, O.Opt(1.0, 0.5, 1e-8, 1e-7), o.numpy(), d.numpy(), mode=1, rgb_gt=gt.numpy(), prec="f64",
                   stops=ref["stops"], want_magnitude=True)
    assert_rgb(rgb.detach().cpu().numpy(), ref["rgb"])
    assert_grad_f64(grid.sh_data.grad.cpu().numpy(), r64["grad_sh"], r64["mag_sh"], "api grad_sh")
    assert_grad_f64(grid.density_data.grad.cpu().numpy(), r64["grad_density"], r64["mag_density"],
                    "api grad_density")
    np.testing.assert_array_equal(grid.sparse_grad_indexer.cpu().numpy(), ref["mask"])


def test_image_api():
    grid = _grid()
    c2w = S.look_at_c2w((0.5, 0.3, -3.0)).cuda()
    cam = Camera(c2w, fx=60.0, width=48, height=40)
    with torch.no_grad():
        img = grid.volume_render_image(cam)
    ref = O.render_image(_oracle_grid(grid), O.Opt(1.0, 0.5, 1e-8, 1e-7), c2w.cpu().numpy(), 60.0, 60.0, 24.0,
                         20.0, 48, 40)
    assert_rgb(img.cpu().numpy(), ref["rgb"], "image")
    # with grad enabled the reference renders generated rays in batches; same picture
    img2 = grid.volume_render_image(cam, batch_size=700)
    np.testing.assert_allclose(img2.detach().cpu().numpy(), img.cpu().numpy(), atol=2e-4)


def test_sample_api_autograd():
    grid = _grid()
    pts = (torch.rand((500, 3), generator=torch.Generator().manual_seed(33)) * 2 - 1).cuda()
    dens, sh = grid.sample(pts)
    (dens.sum() + sh.sum()).backward()
    assert grid.density_data.grad is not None and grid.sh_data.grad.abs().sum() > 0


def test_train_step_matches_oracle_pipeline():
    """volume_render_fused + inplace_tv_grad + inplace_tv_color_grad + RMSprop on
    both tables, against the oracle running the same steps."""
    grid = _grid(reso=24, occ=0.5, seed=34)
    og0 = _oracle_grid(grid)
    o, d, gt = S.make_rays(1024, seed=35)
    grid.volume_render_fused(Rays(o.cuda(), d.cuda()), gt.cuda())
    np.random.seed(7)
    grid.inplace_tv_grad(grid.density_data.grad, scaling=1e-2, sparse_frac=0.05)
    grid.inplace_tv_color_grad(grid.sh_data.grad, scaling=1e-2, sparse_frac=0.05)
    mask = grid.sparse_grad_indexer.clone()
    mask_sh = grid.sparse_sh_grad_indexer.clone()
    kgd = grid.density_data.grad.clone()
    kgs = grid.sh_data.grad.clone()
    d0 = grid.density_data.detach().clone()
    s0 = grid.sh_data.detach().clone()
    grid.optim_density_step(30.0, beta=0.95)
    grid.optim_sh_step(1e-2, beta=0.95)
    torch.cuda.synchronize()
    # oracle pipeline: render adjoint, then the two TV windows drawn from the host RNG
    ref = O.render(og0, O.Opt(1.0, 0.5, 1e-8, 1e-7), o.numpy(), d.numpy(), mode=1, rgb_gt=gt.numpy(), prec="f64")
    n3 = 24 ** 3
    np.random.seed(7)
    windows = []
    for _ in range(2):   # the density window, then the SH window (host RNG, as _get_rand_cells)
        start = np.random.randint(0, n3)
        c = np.arange(start, start + max(int(0.05 * n3), 1), dtype=np.int64)
        c[c >= n3] -= n3
        windows.append(c.astype(np.int32))
    gd, gs, m = ref["grad_density"], ref["grad_sh"], ref["mask"].astype(np.uint8)
    O.tv_grad(og0.links, og0.density, 0, 1, 1e-2, False, cells=windows[0], grad=gd, mask=m, prec="f64")
    m_sh = ref["mask"].astype(np.uint8)
    O.tv_grad(og0.links, og0.sh, 0, 27, 1e-2, True, cells=windows[1], grad=gs, mask=m_sh, prec="f64")
    np.testing.assert_array_equal(mask.cpu().numpy(), m.astype(bool))
    np.testing.assert_array_equal(mask_sh.cpu().numpy(), m_sh.astype(bool))
    assert_grad(kgd.cpu().numpy(), gd, "density grad after TV")
    assert_grad(kgs.cpu().numpy(), gs, "sh grad after TV")
    # the optimiser steps on the kernel's own gradients are bit-exact with the float32 restatement
    nd, _, _ = O.optim(True, d0.cpu().numpy(), np.zeros_like(og0.density), kgd.cpu().numpy(), 2,
                       mask.cpu().numpy(), beta=0.95, lr=30.0, prec="f32")
    ns, _, _ = O.optim(True, s0.cpu().numpy(), np.zeros_like(og0.sh), kgs.cpu().numpy(), 2,
                       mask_sh.cpu().numpy(), beta=0.95, lr=1e-2, prec="f32")
    np.testing.assert_array_equal(grid.density_data.detach().cpu().numpy(), nd)
    np.testing.assert_array_equal(grid.sh_data.detach().cpu().numpy(), ns)
    assert float(grid.density_data.grad.abs().max()) == 0.0   # gradients are consumed


def test_bf16_grid_trains():
    grid = _grid(sh_dtype=torch.bfloat16)
    o, d, gt = S.make_rays(2048, seed=36)
    rays = Rays(o.cuda(), d.cuda())
    losses = []
    for _ in range(5):
        rgb = grid.volume_render_fused(rays, gt.cuda())
        losses.append(float(F.mse_loss(rgb, gt.cuda())))
        grid.inplace_tv_color_grad(None, scaling=1e-3)
        grid.optim_density_step(30.0, beta=0.95)
        grid.optim_sh_step(1e-2, beta=0.95)
    assert grid.sh_data.dtype == torch.bfloat16
    assert losses[-1] < losses[0]


def test_no_cpu_path():
    grid = SparseGrid(reso=8, device="cpu")
    with pytest.raises(RuntimeError):
        grid.volume_render(Rays(torch.zeros(2, 3), torch.ones(2, 3)))
