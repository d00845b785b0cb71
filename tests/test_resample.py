"""Grid resampling: SparseGrid.resample (svox2/svox2.py:1223-1424) with its kernels dilate
(svox2/csrc/misc_kernel.cu:20-48) and grid_weight_render (183-334).

Pinning: a resample that the reference itself ran on its CPU path (no dilation, density
threshold; tests/golden/make_golden.py resample_case).  The reference's dilate and
grid_weight_render have no CPU path; the oracle restates them: dilate as numpy boolean work
(exact), grid_weight_render in C (float32 and float64), pinned by known answers below."""
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S

GOLD = Path(__file__).resolve().parent / "golden" / "resample_sparse12_to_9x14x11.npz"


def test_oracle_dilate_known_answer():
    m = np.zeros((5, 6, 7), bool)
    m[0, 0, 0] = True          # a corner: its 2x2x2 block
    m[4, 3, 6] = True          # on two faces: a 2x3x2 block
    d = O.dilate(m)
    assert d.sum() == 8 + 12
    assert d[1, 1, 1] and not d[2, 2, 2] and d[3, 2, 5] and not d[2, 3, 6]


def test_oracle_grid_weight_known_answer():
    # an opaque block filling the grid: each ray stops at its first sample, weight 1 there
    data = np.full((8, 8, 8), 1e4, np.float32)
    c2w = S.look_at_c2w((0.0, 0.0, -4.0)).numpy()
    cam = dict(c2w=c2w, fx=20.0, fy=20.0, cx=4.0, cy=4.0, width=8, height=8)
    w = O.grid_weight_render(data, cam, 0.5, 0.0, False, (3.5, 3.5, 3.5), (4.0, 4.0, 4.0))
    assert w.max() == 1.0
    # only the near face (z = 0 and z = 1 corners of the first cells) is reached
    assert (w[:, :, 2:] == 0).all() and (w[:, :, :2] > 0).any()


@pytest.mark.gpu
@pytest.mark.parametrize("shape,p", [((16, 16, 16), 0.05), ((9, 14, 11), 0.2), ((2, 5, 1), 0.3), ((12, 12, 12), 0.0)])
def test_dilate_matches_oracle(shape, p):
    from svox2_gb300 import csrc as C
    rng = np.random.default_rng(7)
    m = rng.random(shape) < p
    out = C.dilate(torch.from_numpy(m).cuda())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), O.dilate(m))


@pytest.mark.gpu
@pytest.mark.parametrize("stop,opaque", [(0.2, False), (0.0, False), (0.0, True)])
def test_grid_weight_render_matches_oracle(stop, opaque):
    from svox2_gb300 import Camera
    from svox2_gb300 import csrc as C
    g = S.make_grid(24, occupancy=0.3, seed=50)
    # a dense density grid like the one resampling builds: density at every voxel, 0 where empty
    dense = torch.zeros(g.links.numel())
    occ = g.links.view(-1) >= 0
    dense[occ] = g.density.view(-1)[g.links.view(-1)[occ].long()]
    dense = dense.view(24, 24, 24)
    off, scl = S.grid_transform((24, 24, 24))
    c2w = S.look_at_c2w((1.0, 2.0, -3.5))
    cam = Camera(c2w.cuda(), fx=30.0, width=40, height=32)
    w = torch.zeros_like(dense).cuda()
    C.grid_weight_render(dense.cuda(), cam._to_cpp(), 0.5, stop, opaque, torch.tensor(off), torch.tensor(scl), w)
    torch.cuda.synchronize()
    ref = O.grid_weight_render(dense.numpy(), dict(c2w=c2w.numpy(), fx=30.0, fy=30.0, cx=20.0, cy=16.0, width=40,
                                                   height=32), 0.5, stop, opaque, off, scl)
    np.testing.assert_allclose(w.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)
    assert ref.max() > 0


@pytest.mark.gpu
def test_resample_matches_reference():
    from svox2_gb300 import SparseGrid
    z = np.load(GOLD)
    grid = SparseGrid.from_tables(torch.from_numpy(z["src_links"]).cuda(), torch.from_numpy(z["src_density"]).cuda(),
                                  torch.from_numpy(z["src_sh"]).cuda())
    grid.resample(z["new_reso"].tolist(), sigma_thresh=float(z["sigma_thresh"]), dilate=0, accelerate=False)
    np.testing.assert_array_equal(grid.links.cpu().numpy(), z["links"])
    np.testing.assert_allclose(grid.density_data.detach().cpu().numpy().reshape(-1), z["density"].reshape(-1),
                               rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(grid.sh_data.detach().cpu().numpy(), z["sh"], rtol=1e-5, atol=1e-5)


@pytest.mark.gpu
def test_resample_with_cameras_and_dilation():
    """The weight-threshold path composed from its parts: the kept voxels are the dilated mask
    of the largest camera weights; the grid is accelerated and still renders."""
    from svox2_gb300 import Camera, Rays, SparseGrid
    from svox2_gb300 import csrc as C
    g = S.make_grid(20, occupancy=0.3, seed=51)
    grid = SparseGrid.from_tables(g.links.cuda(), g.density.cuda(), g.sh.cuda())
    cams = [Camera(S.look_at_c2w(tuple(e)).cuda(), fx=24.0, width=32, height=24)
            for e in [(0.0, 0.0, -4.0), (4.0, 0.5, 0.0), (0.0, -4.0, 0.3)]]
    pts = _centres(20, 16).cuda()
    dens = grid.sample(pts, grid_coords=True, want_colors=False)[0].view(16, 16, 16)
    off, scl = S.grid_transform((16, 16, 16))
    w = torch.zeros_like(dens)
    for cam in cams:
        C.grid_weight_render(dens, cam._to_cpp(), 0.5, 0.2, False, torch.tensor(off), torch.tensor(scl), w)
    mask = C.dilate(w >= 0.01).view(-1)
    grid.resample(16, weight_thresh=0.01, dilate=1, cameras=cams, accelerate=True)
    links = grid.links.view(-1)
    assert torch.equal(links >= 0, mask)
    assert grid.density_data.shape[0] == int(mask.sum()) and int((links < -1).sum()) > 0
    o, d, _ = S.make_rays(256, seed=52)
    rgb = grid.volume_render(Rays(o.cuda(), d.cuda()))
    assert torch.isfinite(rgb).all()


@pytest.mark.gpu
def test_resample_morton_order():
    """use_z_order: the same voxels as raster order, numbered by their Morton codes."""
    from svox2_gb300 import SparseGrid
    from svox2_gb300 import utils
    g = S.make_grid(20, occupancy=0.4, seed=53)
    grid = SparseGrid.from_tables(g.links.cuda(), g.density.cuda(), g.sh.cuda())
    dens = grid.sample(_centres(20, 16).cuda(), grid_coords=True, want_colors=False)[0].view(-1)
    grid.resample(16, sigma_thresh=2.0, dilate=0, use_z_order=True, accelerate=False)
    links = grid.links.view(-1)
    kept = links >= 0
    assert torch.equal(kept, dens >= 2.0)
    codes = utils.gen_morton(16).view(-1).cuda()[kept]
    assert torch.equal(links[kept].long(), torch.argsort(torch.argsort(codes)))


def _centres(cur, new):
    f = 0.5 * cur / new
    ax = torch.linspace(f - 0.5, cur - f - 0.5, new, dtype=torch.float32)
    return torch.stack(torch.meshgrid(ax, ax, ax, indexing="ij"), -1).view(-1, 3)
