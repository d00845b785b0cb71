"""The TV value, tv (svox2/csrc/loss_kernel.cu:42-109, host 483-515), and SparseGrid.tv /
tv_color through the autograd function (svox2/svox2.py:292-329, 1678-1722).

The reference has no CPU path for the value; the oracle restates the kernel and is pinned by
a known answer worked out by hand.  GPU: the kernel against the float64 oracle (a float32 sum
of up to ~5e5 terms, in per-thread, per-block and atomic stages: 1e-5 relative), and the
backward against the tv_grad kernel called directly."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S


def test_oracle_known_answer():
    # 3^3 dense grid, 8 cells, one voxel (the centre) at 256/3 so that each difference is 1
    links = np.arange(27, dtype=np.int32).reshape(3, 3, 3)
    data = np.zeros((27, 1), np.float32)
    assert O.tv_value(links, data, 0, 1, False) == pytest.approx(np.sqrt(1e-5), rel=1e-6)
    data[13] = 256.0 / 3.0
    want = (np.sqrt(3 + 1e-5) + 3 * np.sqrt(1 + 1e-5) + 4 * np.sqrt(1e-5)) / 8
    assert O.tv_value(links, data, 0, 1, False) == pytest.approx(want, rel=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["density", "sh_range", "sh_ignore_edge", "bf16"])
def test_tv_value_matches_oracle(case):
    from svox2_gb300 import csrc as C
    g = S.make_grid(32 if case != "bf16" else 24, occupancy=0.3, seed=61)
    links = g.links.cuda()
    if case == "density":
        data, lo, hi, edge = g.density.cuda(), 0, 1, False
    elif case == "sh_range":
        data, lo, hi, edge = g.sh.cuda(), 3, 20, False
    elif case == "sh_ignore_edge":
        data, lo, hi, edge = g.sh.cuda(), 0, 27, True
    else:
        data, lo, hi, edge = g.sh.cuda().to(torch.bfloat16), 0, 27, True
    v = float(C.tv(links, data, lo, hi, False, 2.0, edge, -1.0, -1.0))
    ref = O.tv_value(g.links.numpy(), data.float().cpu().numpy(), lo, hi, edge)
    assert v == pytest.approx(ref, rel=1e-5)


@pytest.mark.gpu
def test_grid_tv_autograd():
    from svox2_gb300 import SparseGrid
    from svox2_gb300 import csrc as C
    g = S.make_grid(20, occupancy=0.4, seed=62)
    grid = SparseGrid.from_tables(g.links.cuda(), g.density.cuda(), g.sh.cuda())
    tv = grid.tv()
    assert tv.dim() == 0 and tv.requires_grad
    (2.5 * tv).backward()
    ref = torch.zeros_like(grid.density_data)
    C.tv_grad(grid.links, grid.density_data.detach(), 0, 1, 1.0, False, 2.0, False, -1.0, -1.0, ref)
    torch.testing.assert_close(grid.density_data.grad, 2.5 * ref, rtol=1e-5, atol=1e-9)
    tvc = grid.tv_color(start_dim=2, end_dim=-1)
    ref_v = O.tv_value(g.links.numpy(), g.sh.numpy(), 2, 26, True)
    assert float(tvc.detach()) == pytest.approx(ref_v, rel=1e-5)
    tvc.backward()
    refc = torch.zeros_like(grid.sh_data)
    C.tv_grad(grid.links, grid.sh_data.detach(), 2, 26, 1.0, False, 2.0, True, -1.0, -1.0, refc)
    torch.testing.assert_close(grid.sh_data.grad, refc, rtol=1e-5, atol=1e-9)
