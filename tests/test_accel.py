"""accel_dist_prop (empty-space skip levels, svox2/csrc/misc_kernel.cu:108-181, 356-416).

CPU: the oracle against known answers worked out by hand from the reference kernel's
definition.  GPU: the kernel against the oracle, bit for bit, on cubic, non-cubic, thin,
empty and full grids and on the 256^3 workload grid; then a fused render through the
accelerated links against the oracle (sample indexing bit for bit, skip decisions
included)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S

from helpers import grid_pair, opt_struct, rays_pair


def test_oracle_known_answers():
    # 8^3 grid, only voxel (0, 0, 0) allocated: pyramid levels 4^3, 2^3, 1^3
    L = np.full((8, 8, 8), -1, np.int32)
    L[0, 0, 0] = 0
    out = O.accel_dist_prop(L)
    assert out[0, 0, 0] == 0                      # allocated voxels keep their link
    assert out[1, 1, 1] == -1                     # parent (0,0,0) at level 1 is occupied
    assert out[2, 2, 2] == -2 and out[3, 3, 3] == -2   # level-1 parent (1,1,1) empty, level 2 occupied
    assert out[7, 7, 7] == -3 and out[4, 4, 4] == -3   # empty up to the 1^3 root, which is occupied
    # no allocated voxel: every level is empty
    E = O.accel_dist_prop(np.full((8, 8, 8), -1, np.int32))
    assert (E == -4).all()
    # a side of 1: no pyramid level, negative links become -1
    T = np.full((1, 4, 4), -5, np.int32)
    T[0, 0, 0] = 3
    assert (O.accel_dist_prop(T)[T < 0] == -1).all()
    # non-cubic 5 x 3 x 2 -> 3x2x1 (stop: a side reached 1)
    N = np.full((5, 3, 2), -1, np.int32)
    N[4, 2, 1] = 7
    out = O.accel_dist_prop(N)
    assert out[4, 2, 1] == 7 and out[4, 2, 0] == -1 and out[0, 0, 0] == -2


def _cases():
    rng = np.random.default_rng(3)
    cases = {}
    g = S.make_grid(32, occupancy=0.2, seed=1)
    cases["sparse32"] = g.links.numpy()
    g = S.make_grid((20, 28, 36), occupancy=0.1, seed=2)
    cases["noncubic"] = g.links.numpy()
    thin = np.full((2, 5, 7), -1, np.int32)
    thin[1, 4, 6] = 0
    cases["thin"] = thin
    cases["empty"] = np.full((16, 16, 16), -1, np.int32)
    cases["full"] = np.arange(12 ** 3, dtype=np.int32).reshape(12, 12, 12)
    pre = S.make_grid(24, occupancy=0.3, seed=4).links.numpy().copy()
    pre[pre < 0] = rng.integers(-6, -1, size=int((pre < 0).sum()))      # already accelerated once
    cases["reaccelerate"] = pre
    return cases


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(_cases()))
def test_accel_matches_oracle(name):
    from svox2_gb300 import csrc as C
    L = _cases()[name]
    dev = torch.from_numpy(L.copy()).cuda()
    C.accel_dist_prop(dev)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), O.accel_dist_prop(L))


@pytest.mark.gpu
def test_accel_workload_grid_and_idempotence():
    from svox2_gb300 import csrc as C
    g = S.make_grid(256, occupancy=0.2, n_balls=8, seed=0)
    ref = O.accel_dist_prop(g.links.numpy())
    dev = g.links.cuda()
    C.accel_dist_prop(dev)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), ref)
    C.accel_dist_prop(dev)          # a second pass gives the same table
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), ref)


@pytest.mark.gpu
def test_render_through_accelerated_links():
    from svox2_gb300 import SparseGrid
    from svox2_gb300 import csrc as C
    from test_render_gpu import _run_fused
    g = S.make_grid(48, occupancy=0.15, seed=21)
    grid = SparseGrid.from_tables(g.links.cuda(), g.density.cuda(), g.sh.cuda())
    grid.accelerate()
    g.links = grid.links.cpu()
    assert int((g.links < -1).sum()) > 0
    spec, og = grid_pair(g)
    o, d, gt = S.make_rays(1024, seed=22)
    opt, oopt = opt_struct()
    _run_fused(spec, og, rays_pair(o, d), o, d, gt, opt, oopt)


@pytest.mark.gpu
def test_sphere_bound_grid_is_accelerated():
    from svox2_gb300 import SparseGrid
    grid = SparseGrid(reso=32, basis_dim=9, use_sphere_bound=True, device="cuda")
    L = grid.links.cpu().numpy()
    base = np.where(L >= 0, L, -1).astype(np.int32)
    np.testing.assert_array_equal(L, O.accel_dist_prop(base))
