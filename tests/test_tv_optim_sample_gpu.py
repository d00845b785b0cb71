"""Parity of the TV-gradient, optimiser and point-sampling kernels with the CPU
oracle, through the reference-facing operator API."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import synthetic as S

from helpers import assert_grad, grid_pair

pytestmark = pytest.mark.gpu


def _window(n_cells, frac, start):
    num = max(int(frac * n_cells), 1)
    arr = np.arange(start, start + num, dtype=np.int64)
    arr[arr >= n_cells] -= n_cells   # wrap as _get_rand_cells does
    return arr.astype(np.int32)


@pytest.mark.parametrize("which,ignore_edge,ignore_last_z,start", [
    ("density", False, False, 100), ("density", False, True, 20000), ("sh", True, False, 31000),
    ("sh", False, False, 32700),   # window wrapping past the last cell
])
def test_tv_grad_sparse(which, ignore_edge, ignore_last_z, start):
    from svox2_gb300 import csrc as C
    g = S.make_grid(32, occupancy=0.4, seed=21)
    data = g.density if which == "density" else g.sh
    cells = _window(32 ** 3, 0.05, start)
    grad = torch.randn(data.shape, generator=torch.Generator().manual_seed(1)) * 1e-3
    mask = torch.zeros((data.shape[0],), dtype=torch.bool)
    gk, mk = grad.cuda(), mask.cuda()
    C.tv_grad_sparse(g.links.cuda(), data.cuda(), torch.from_numpy(cells).cuda(), mk, 0, data.shape[1], 0.7,
                     False, 2.0, ignore_edge, ignore_last_z, -1.0, -1.0, gk)
    go = grad.numpy().astype(np.float64).copy()
    mo = np.zeros((data.shape[0],), dtype=np.uint8)
    O.tv_grad(g.links.numpy(), data.numpy(), 0, data.shape[1], 0.7, ignore_edge, cells=cells,
              ignore_last_z=ignore_last_z, grad=go, mask=mo, prec="f64")
    assert_grad(gk.cpu().numpy(), go, "tv sparse")
    np.testing.assert_array_equal(mk.cpu().numpy(), mo.astype(bool))


@pytest.mark.parametrize("start,end,ignore_edge", [(0, 1, False), (0, 27, True), (9, 18, False)])
def test_tv_grad_dense(start, end, ignore_edge):
    from svox2_gb300 import csrc as C
    g = S.make_grid((18, 22, 26), occupancy=0.5, seed=22)
    data = g.density if end == 1 else g.sh
    gk = torch.zeros(data.shape, device="cuda")
    C.tv_grad(g.links.cuda(), data.cuda(), start, end, 1.3, False, 2.0, ignore_edge, -1.0, -1.0, gk)
    go = O.tv_grad(g.links.numpy(), data.numpy(), start, end, 1.3, ignore_edge, prec="f64")
    assert_grad(gk.cpu().numpy(), go, "tv dense")


@pytest.mark.parametrize("rms", [True, False])
@pytest.mark.parametrize("kind", ["all", "none", "mask", "list"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_optimizer_bit_exact(rms, kind, dtype):
    from svox2_gb300 import csrc as C
    gen = torch.Generator().manual_seed(23)
    N, Cc = 5000, 28
    data = (torch.randn((N, Cc), generator=gen)).to(dtype)
    grad = torch.randn((N, Cc), generator=gen)
    grad[::7] = 0.0
    rmsv = torch.rand((N, Cc), generator=gen) * 0.1
    rmsv[::5] = 0.0   # exercises the rms == 0 branch
    mask = torch.rand((N,), generator=gen) < 0.3
    idx = torch.nonzero(mask).flatten()
    indexer = {"all": torch.empty(()), "none": torch.empty((0,), dtype=torch.bool), "mask": mask,
               "list": idx}[kind]
    okind = {"all": 0, "none": 1, "mask": 2, "list": 3}[kind]
    dk, gk, rk = data.cuda(), grad.cuda(), rmsv.cuda()
    if rms:
        C.rmsprop_step(dk, rk, gk, indexer.cuda(), 0.95, 0.3, 1e-8, -1e9, 0.05)
    else:
        C.sgd_step(dk, gk, indexer.cuda(), 0.3, 0.05)
    od, orr, og = O.optim(rms, data.float().numpy(), rmsv.numpy() if rms else None, grad.numpy(), okind,
                          indexer.numpy() if okind >= 2 else None, beta=0.95, lr=0.3, eps=1e-8, minval=-1e9,
                          lr_last=0.05, prec="f32")
    od = torch.from_numpy(od).to(dtype)   # round like the kernel's store
    assert torch.equal(dk.cpu(), od), "data differs"
    np.testing.assert_array_equal(gk.cpu().numpy(), og)
    if rms:
        np.testing.assert_array_equal(rk.cpu().numpy(), orr)


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_sample_grid_fwd_bwd(dtype):
    from svox2_gb300 import csrc as C
    g = S.make_grid(20, occupancy=0.5, seed=24)
    spec, og = grid_pair(g, sh_dtype=dtype)
    gen = torch.Generator().manual_seed(25)
    pts = torch.rand((3000, 3), generator=gen) * 2.4 - 1.2
    d, s = C.sample_grid(spec, pts.cuda(), True)
    od, osh = O.sample(og, pts.numpy(), True, prec="f32")
    np.testing.assert_allclose(d.cpu().numpy(), od, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(s.cpu().numpy(), osh, rtol=1e-6, atol=1e-6)
    gd_in = torch.randn((3000, 1), generator=gen)
    gs_in = torch.randn((3000, 27), generator=gen)
    N = og.density.shape[0]
    out_d = torch.zeros((N, 1), device="cuda")
    out_s = torch.zeros((N, 27), device="cuda")
    C.sample_grid_backward(spec, pts.cuda(), gd_in.cuda(), gs_in.cuda(), out_d, out_s, True)
    rd, rs = O.sample_backward(og, pts.numpy(), gd_in.numpy(), gs_in.numpy(), True, prec="f64")
    assert_grad(out_d.cpu().numpy(), rd, "sample bwd density")
    assert_grad(out_s.cpu().numpy(), rs, "sample bwd sh")
    # density only
    d2, s2 = C.sample_grid(spec, pts.cuda(), False)
    assert s2.shape[0] == 0
    assert torch.equal(d2, d)
