"""Generate golden vectors from the REFERENCE implementation (sxyu/svox2's own
pure-PyTorch CPU path) for the oracle's pinning tests.

Run in a container where the reference source tree is available:
    python tests/golden/make_golden.py /path/to/reference
It imports the reference package read-only, builds small seeded grids, and
records inputs and outputs of
  * SparseGrid.volume_render(use_kernel=False) + autograd of F.mse_loss
    (svox2/svox2.py:658-884, the reference's gradcheck path), and
  * SparseGrid.sample(use_kernel=False) + autograd (svox2/svox2.py:576-653),
  * SparseGrid.save / SparseGrid.load of a checkpoint (svox2/svox2.py:1526-1628),
  * SparseGrid.resample on the CPU path without dilation (svox2/svox2.py:1223-1424),
  * SparseGrid.inplace_l2_color_grad (svox2/svox2.py:1897-1932),
  * SparseGrid.volume_render(use_kernel=False) with the MSI background model
    (svox2/svox2.py:796-876) + autograd, save / load of a grid with the background,
    and SparseGrid.sparsify_background without dilation (svox2/svox2.py:1426-1448),
into tests/golden/*.npz.  sigma_thresh = stop_thresh = 0 so that the CPU
path's semantics coincide with the CUDA kernel's (the reference's own
test/test_render_gradcheck.py uses the same setting).
"""
from __future__ import annotations

import sys
import warnings
from pathlib import Path

import numpy as np
import torch
import torch.nn.functional as F

OUT = Path(__file__).resolve().parent


def _rays(n, gen):
    o = torch.randn((n, 3), generator=gen)
    o = 1.5 * o / o.norm(dim=-1, keepdim=True)
    tgt = torch.rand((n, 3), generator=gen) - 0.5
    d = tgt - o
    d = d / d.norm(dim=-1, keepdim=True)
    gt = torch.rand((n, 3), generator=gen)
    return o, d, gt


def render_case(svox2, name, reso, basis_dim, occupancy, z_order, n_rays, bg, step, seed):
    gen = torch.Generator().manual_seed(seed)
    grid = svox2.SparseGrid(reso=reso, basis_dim=basis_dim, use_z_order=z_order, device="cpu")
    links = grid.links.clone()
    if occupancy is not None:
        # drop voxels outside a random ball union, re-index rows in raster order
        n3 = links.numel()
        keep = torch.rand(links.shape, generator=gen) < occupancy
        new = torch.full(links.shape, -1, dtype=torch.int32)
        new[keep] = torch.arange(int(keep.sum()), dtype=torch.int32)
        links = new
        grid.links = links
        N = int(keep.sum())
        grid.density_data = torch.nn.Parameter(torch.zeros(N, 1))
        grid.sh_data = torch.nn.Parameter(torch.zeros(N, 3 * basis_dim))
    N = grid.density_data.shape[0]
    dens = torch.clamp(torch.randn((N, 1), generator=gen) * 3.0 + 2.0, min=0.0)
    sh = torch.randn((N, 3 * basis_dim), generator=gen) * 0.3
    grid.density_data.data[:] = dens
    grid.sh_data.data[:] = sh
    grid.opt.sigma_thresh = 0.0
    grid.opt.stop_thresh = 0.0
    grid.opt.background_brightness = bg
    grid.opt.step_size = step
    o, d, gt = _rays(n_rays, gen)
    rgb = grid.volume_render(svox2.Rays(o, d), use_kernel=False)
    loss = F.mse_loss(rgb, gt)
    loss.backward()
    gsz = grid._grid_size()
    np.savez_compressed(
        OUT / f"render_{name}.npz",
        links=links.numpy().astype(np.int32), density=dens.numpy(), sh=sh.numpy(),
        basis_dim=basis_dim, offset=(grid._offset * gsz - 0.5).numpy(), scaling=(grid._scaling * gsz).numpy(),
        origins=o.numpy(), dirs=d.numpy(), rgb_gt=gt.numpy(), bg=bg, step=step,
        rgb=rgb.detach().numpy(), grad_density=grid.density_data.grad.numpy(),
        grad_sh=grid.sh_data.grad.numpy())
    print(name, "rays", n_rays, "voxels", N, "rgb mean", float(rgb.mean()))


def background_case(svox2, name, reso, basis_dim, nlayers, bg_reso, n_rays, bg, step, seed):
    """volume_render(use_kernel=False) of a grid with the MSI background model (svox2/svox2.py:796-876)
    and the autograd gradients of the MSE loss, background included."""
    gen = torch.Generator().manual_seed(seed)
    grid = svox2.SparseGrid(reso=reso, basis_dim=basis_dim, background_nlayers=nlayers, background_reso=bg_reso,
                            device="cpu")
    N = grid.density_data.shape[0]
    dens = torch.clamp(torch.randn((N, 1), generator=gen) * 0.6 + 0.2, min=0.0)
    sh = torch.randn((N, 3 * basis_dim), generator=gen) * 0.3
    grid.density_data.data[:] = dens
    grid.sh_data.data[:] = sh
    # drop a fifth of the background cells and re-index the rest
    keep = torch.rand(grid.background_links.shape, generator=gen) >= 0.2
    bl = torch.full(grid.background_links.shape, -1, dtype=torch.int32)
    bl[keep] = torch.arange(int(keep.sum()), dtype=torch.int32)
    grid.background_links = bl
    bd = torch.randn((int(keep.sum()), nlayers, 4), generator=gen) * 0.5
    bd[..., 3] = torch.rand((int(keep.sum()), nlayers), generator=gen) * 4.0 - 0.5
    grid.background_data = torch.nn.Parameter(bd.clone())
    grid.opt.sigma_thresh = 0.0
    grid.opt.stop_thresh = 0.0
    grid.opt.background_brightness = bg
    grid.opt.step_size = step
    o, d, gt = _rays(n_rays, gen)
    # half of the rays leave in random directions: some miss the grid and see only the background
    h = n_rays // 2
    dr = torch.randn((n_rays - h, 3), generator=gen)
    d[h:] = dr / dr.norm(dim=-1, keepdim=True)
    rgb = grid.volume_render(svox2.Rays(o, d), use_kernel=False)
    loss = F.mse_loss(rgb, gt)
    loss.backward()
    gsz = grid._grid_size()
    np.savez_compressed(
        OUT / f"background_{name}.npz",
        links=grid.links.numpy().astype(np.int32), density=dens.numpy(), sh=sh.numpy(),
        basis_dim=basis_dim, offset=(grid._offset * gsz - 0.5).numpy(), scaling=(grid._scaling * gsz).numpy(),
        bg_links=bl.numpy(), bg_data=bd.numpy(),
        origins=o.numpy(), dirs=d.numpy(), rgb_gt=gt.numpy(), bg=bg, step=step,
        rgb=rgb.detach().numpy(), grad_density=grid.density_data.grad.numpy(),
        grad_sh=grid.sh_data.grad.numpy(), grad_background=grid.background_data.grad.numpy())
    print(name, "rays", n_rays, "bg cells", int(keep.sum()), "rgb mean", float(rgb.mean()))


def sample_case(svox2, name, reso, basis_dim, n_points, seed):
    gen = torch.Generator().manual_seed(seed)
    grid = svox2.SparseGrid(reso=reso, basis_dim=basis_dim, device="cpu")
    N = grid.density_data.shape[0]
    grid.density_data.data[:] = torch.randn((N, 1), generator=gen)
    grid.sh_data.data[:] = torch.randn((N, 3 * basis_dim), generator=gen)
    pts = torch.rand((n_points, 3), generator=gen) * 2.4 - 1.2   # includes points outside the grid
    gd_out = torch.randn((n_points, 1), generator=gen)
    gs_out = torch.randn((n_points, 3 * basis_dim), generator=gen)
    d, s = grid.sample(pts.clone(), use_kernel=False)
    (d * gd_out).sum().add_((s * gs_out).sum()).backward()
    gsz = grid._grid_size()
    np.savez_compressed(
        OUT / f"sample_{name}.npz",
        links=grid.links.numpy().astype(np.int32), density=grid.density_data.data.numpy(),
        sh=grid.sh_data.data.numpy(), basis_dim=basis_dim, offset=(grid._offset * gsz - 0.5).numpy(),
        scaling=(grid._scaling * gsz).numpy(), points=pts.numpy(), grad_out_density=gd_out.numpy(),
        grad_out_sh=gs_out.numpy(), out_density=d.detach().numpy(), out_sh=s.detach().numpy(),
        grad_density=grid.density_data.grad.numpy(), grad_sh=grid.sh_data.grad.numpy())
    print(name, "points", n_points)


def checkpoint_case(svox2, name, reso, basis_dim, occupancy, radius, center, seed, bg=None):
    """SparseGrid.save (svox2/svox2.py:1526-1553) of a seeded grid, written by the reference
    itself, plus what the reference's SparseGrid.load (1555-1628) reads back from it.
    bg = (nlayers, reso): the grid also carries an MSI background with a fifth of its cells dropped."""
    gen = torch.Generator().manual_seed(seed)
    kw = {} if bg is None else {"background_nlayers": bg[0], "background_reso": bg[1]}
    grid = svox2.SparseGrid(reso=reso, basis_dim=basis_dim, radius=radius, center=center, device="cpu", **kw)
    keep = torch.rand(grid.links.shape, generator=gen) < occupancy
    links = torch.full(grid.links.shape, -1, dtype=torch.int32)
    links[keep] = torch.arange(int(keep.sum()), dtype=torch.int32)
    N = int(keep.sum())
    grid.links = links
    grid.density_data = torch.nn.Parameter(torch.randn((N, 1), generator=gen) * 3.0)
    grid.sh_data = torch.nn.Parameter(torch.randn((N, 3 * basis_dim), generator=gen) * 0.3)
    extra = {}
    if bg is not None:
        bkeep = torch.rand(grid.background_links.shape, generator=gen) >= 0.2
        bl = torch.full(grid.background_links.shape, -1, dtype=torch.int32)
        bl[bkeep] = torch.arange(int(bkeep.sum()), dtype=torch.int32)
        grid.background_links = bl
        grid.background_data = torch.nn.Parameter(torch.randn((int(bkeep.sum()), bg[0], 4), generator=gen))
    path = OUT / f"ckpt_{name}.npz"
    grid.save(str(path), compress=True)
    back = svox2.SparseGrid.load(str(path), device="cpu")
    if bg is not None:
        extra = dict(background_links=back.background_links.numpy(),
                     background_data=back.background_data.data.numpy(),
                     background_nlayers=back.background_nlayers, background_reso=back.background_reso,
                     src_background_data=grid.background_data.data.numpy())
    np.savez_compressed(
        OUT / f"ckpt_{name}_loaded.npz", links=back.links.numpy(), density_data=back.density_data.data.numpy(),
        sh_data=back.sh_data.data.numpy(), radius=back.radius.numpy(), center=back.center.numpy(),
        basis_dim=back.basis_dim, src_density=grid.density_data.data.numpy(), src_sh=grid.sh_data.data.numpy(),
        **extra)
    print(name, "checkpoint voxels", N)


def sparsify_background_case(svox2, name, nlayers, bg_reso, sigma_thresh, seed):
    """SparseGrid.sparsify_background (svox2/svox2.py:1426-1448) without dilation (the dilation
    calls the CUDA extension): the background links and data before and after."""
    gen = torch.Generator().manual_seed(seed)
    grid = svox2.SparseGrid(reso=4, basis_dim=1, background_nlayers=nlayers, background_reso=bg_reso, device="cpu")
    bkeep = torch.rand(grid.background_links.shape, generator=gen) >= 0.3
    bl = torch.full(grid.background_links.shape, -1, dtype=torch.int32)
    bl[bkeep] = torch.arange(int(bkeep.sum()), dtype=torch.int32)
    grid.background_links = bl.clone()   # sparsify_background edits the links in place
    bd = torch.randn((int(bkeep.sum()), nlayers, 4), generator=gen)
    bd[..., 3] = torch.rand((int(bkeep.sum()), nlayers), generator=gen) * 2.0
    grid.background_data = torch.nn.Parameter(bd.clone())
    grid.sparsify_background(sigma_thresh=sigma_thresh, dilate=0)
    np.savez_compressed(OUT / f"sparsify_bg_{name}.npz", links_in=bl.numpy(), data_in=bd.numpy(),
                        sigma_thresh=sigma_thresh, links_out=grid.background_links.numpy(),
                        data_out=grid.background_data.data.numpy())
    print(name, "background cells", int(bkeep.sum()), "->", int(grid.background_data.shape[0]))


def resample_case(svox2, name, reso, new_reso, occupancy, sigma_thresh, seed):
    """SparseGrid.resample (svox2/svox2.py:1223-1424) on the CPU path: no dilation (the
    reference's dilate needs its CUDA extension), density threshold, raster links."""
    gen = torch.Generator().manual_seed(seed)
    grid = svox2.SparseGrid(reso=reso, basis_dim=9, device="cpu")
    keep = torch.rand(grid.links.shape, generator=gen) < occupancy
    links = torch.full(grid.links.shape, -1, dtype=torch.int32)
    links[keep] = torch.arange(int(keep.sum()), dtype=torch.int32)
    N = int(keep.sum())
    grid.links = links
    dens = torch.rand((N, 1), generator=gen) * 20.0
    sh = torch.randn((N, 27), generator=gen) * 0.3
    grid.density_data = torch.nn.Parameter(dens.clone())
    grid.sh_data = torch.nn.Parameter(sh.clone())
    grid.resample(new_reso, sigma_thresh=sigma_thresh, dilate=0, cameras=None, use_z_order=False,
                  accelerate=False)
    np.savez_compressed(
        OUT / f"resample_{name}.npz", src_links=links.numpy(), src_density=dens.numpy(), src_sh=sh.numpy(),
        new_reso=np.array(new_reso), sigma_thresh=sigma_thresh, links=grid.links.numpy(),
        density=grid.density_data.data.numpy(), sh=grid.sh_data.data.numpy())
    print(name, "resampled voxels", grid.density_data.shape[0])


def l2_case(svox2, name, seed):
    """SparseGrid.inplace_l2_color_grad (svox2/svox2.py:1897-1932), dense and with a sparse
    SH indexer, on the CPU (plain tensor arithmetic in the reference)."""
    gen = torch.Generator().manual_seed(seed)
    grid = svox2.SparseGrid(reso=6, basis_dim=9, device="cpu")
    N = grid.sh_data.shape[0]
    grid.sh_data.data[:] = torch.randn((N, 27), generator=gen)
    g0 = torch.randn((N, 27), generator=gen)
    dense = g0.clone()
    grid.sparse_sh_grad_indexer = None
    grid.inplace_l2_color_grad(dense, start_dim=3, end_dim=-2, scaling=0.7)
    mask = torch.rand(N, generator=gen) < 0.05
    sparse = g0.clone()
    grid.sparse_sh_grad_indexer = mask
    grid.inplace_l2_color_grad(sparse, scaling=1.3)
    np.savez_compressed(OUT / f"l2_{name}.npz", sh=grid.sh_data.data.numpy(), grad0=g0.numpy(),
                        mask=mask.numpy(), dense=dense.numpy(), sparse=sparse.numpy())
    print(name, "l2 rows", N, "masked", int(mask.sum()))


def main(ref_root: str):
    sys.path.insert(0, ref_root)
    warnings.filterwarnings("ignore")
    import svox2  # the reference package (CPU path; its CUDA extension is not needed)
    torch.set_num_threads(4)
    render_case(svox2, "dense12_sh9", 12, 9, None, False, 48, 1.0, 0.5, 11)
    render_case(svox2, "sparse16_sh9", 16, 9, 0.35, False, 48, 1.0, 0.5, 12)
    render_case(svox2, "morton16_sh4", 16, 4, None, True, 40, 0.25, 0.7, 13)
    render_case(svox2, "dense10x12x14_sh1", (10, 12, 14), 1, None, False, 40, 0.0, 0.5, 14)
    sample_case(svox2, "dense10_sh9", 10, 9, 300, 15)
    checkpoint_case(svox2, "sparse10x12x14_sh9", (10, 12, 14), 9, 0.4, [1.2, 0.8, 1.0], [0.1, -0.2, 0.3], 16)
    resample_case(svox2, "sparse12_to_9x14x11", 12, [9, 14, 11], 0.5, 4.0, 17)
    l2_case(svox2, "dense6_sh9", 18)
    background_case(svox2, "dense8_sh4_l4_r6", 8, 4, 4, 6, 40, 1.0, 0.5, 19)
    background_case(svox2, "dense6_sh1_l3_r5", 6, 1, 3, 5, 40, 0.5, 0.7, 20)
    checkpoint_case(svox2, "bg_sparse6x5x4_sh4_l3_r4", (6, 5, 4), 4, 0.5, [1.0, 1.1, 0.9], [0.0, 0.1, 0.0], 21,
                    bg=(3, 4))
    sparsify_background_case(svox2, "l4_r6", 4, 6, 1.5, 22)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of a sxyu/svox2 checkout>")
    main(sys.argv[1])
