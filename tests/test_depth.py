"""Depth renders: volume_render_expected_term and volume_render_sigma_thresh
(render_lerp_kernel_cuvol.cu:122-225, 1154-1195; SparseGrid.volume_render_depth,
svox2/svox2.py:1181-1221).

The reference has no CPU path for these, so the oracle's restatement is pinned by a known
answer: in a grid filled with a very dense medium, a ray entering through a face stops at
its first sample, and both depths equal the distance from the origin to that face.
GPU: the kernel against the oracle (first-hit depth bit for bit: the same t chain and the
same trilinear density; expected depth within 1e-5 relative + 1e-6, sums reordered)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S

from helpers import grid_pair, opt_struct, rays_pair, rel_err


def _dense_wall(reso=16, density=1e4):
    g = S.make_grid(reso, seed=1)
    g.density.fill_(density)
    return g


def _axis_rays():
    # from 3 world units in front of each face, straight at it: 2 units to the grid ([-1, 1]^3)
    o = torch.tensor([[0.1, 0.2, -3.0], [0.0, -3.0, 0.3], [3.0, -0.2, 0.1], [0.25, 0.25, 3.0]])
    d = torch.tensor([[0.0, 0.0, 1.0], [0.0, 1.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.0, -1.0]])
    return o, d


def test_oracle_known_answer():
    g = _dense_wall()
    _, og = grid_pair(g, device="cpu")
    _, oopt = opt_struct()
    o, d = _axis_rays()
    first = O.render_depth(og, oopt, o.numpy(), d.numpy(), sigma_thresh=0.5)
    expected = O.render_depth(og, oopt, o.numpy(), d.numpy())
    np.testing.assert_allclose(first, 2.0, rtol=0, atol=1e-6)
    np.testing.assert_allclose(expected, 2.0, rtol=0, atol=1e-6)
    # a ray that misses the grid: 0
    away = np.array([[0.70710678, 0.70710678, 0.0]], np.float32)
    miss = O.render_depth(og, oopt, np.array([[0.0, 3.0, 0.0]], np.float32), away)
    assert miss[0] == 0.0


CASES = {
    "sparse40": (40, 0.25, {}),
    "dense24_step03": (24, None, {"step": 0.3}),
    "thresh_hi": (32, 0.4, {"sigma_thresh": 5.0, "stop_thresh": 1e-3}),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES) + ["accelerated"])
def test_depth_matches_oracle(name):
    from svox2_gb300 import csrc as C
    if name == "accelerated":
        g = S.make_grid(48, occupancy=0.15, seed=41)
        g.links = torch.from_numpy(O.accel_dist_prop(g.links.numpy()))
        opts = {}
    else:
        reso, occ, opts = CASES[name]
        g = S.make_grid(reso, occupancy=occ, seed=40)
    spec, og = grid_pair(g)
    o, d, _ = S.make_rays(2048, seed=42)
    opt, oopt = opt_struct(**opts)
    rays = rays_pair(o, d)
    exp_k = C.volume_render_expected_term(spec, rays, opt).cpu().numpy()
    exp_o = O.render_depth(og, oopt, o.numpy(), d.numpy())
    exp_64 = O.render_depth(og, oopt, o.numpy(), d.numpy(), prec="f64")
    np.testing.assert_allclose(exp_k, exp_o, rtol=1e-5, atol=1e-6)
    print(f"expected depth vs f64: kernel {rel_err(exp_k, exp_64):.2e}, oracle32 {rel_err(exp_o, exp_64):.2e}")
    for thr in (0.0, 1.5, 20.0):
        first_k = C.volume_render_sigma_thresh(spec, rays, opt, thr).cpu().numpy()
        first_o = O.render_depth(og, oopt, o.numpy(), d.numpy(), sigma_thresh=thr)
        np.testing.assert_array_equal(first_k, first_o.astype(np.float32))


@pytest.mark.gpu
def test_depth_grid_api_and_known_answer():
    from svox2_gb300 import Camera, Rays, SparseGrid
    g = _dense_wall()
    grid = SparseGrid.from_tables(g.links.cuda(), g.density.cuda(), g.sh.cuda())
    o, d = _axis_rays()
    rays = Rays(o.cuda(), d.cuda())
    torch.testing.assert_close(grid.volume_render_depth(rays), torch.full((4,), 2.0, device="cuda"),
                               rtol=0, atol=1e-6)
    torch.testing.assert_close(grid.volume_render_depth(rays, sigma_thresh=0.5),
                               torch.full((4,), 2.0, device="cuda"), rtol=0, atol=1e-6)
    cam = Camera(S.look_at_c2w((0.0, 0.0, -4.0)).cuda(), fx=40.0, width=24, height=20)
    img = grid.volume_render_depth_image(cam, batch_size=100)
    assert img.shape == (20, 24)
    flat = grid.volume_render_depth(cam.gen_rays())
    torch.testing.assert_close(img.reshape(-1), flat, rtol=0, atol=0)
