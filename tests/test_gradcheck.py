"""Differentiation check (32^3 dense grid, SH degree 2, 256 rays, density
max(0, N(5, 3)), SH N(0, 0.3), sigma_thresh = stop_thresh = 0).

The adjoint is compared with central finite differences of the float64
oracle forward (eps 1e-4) on 512 seeded grid entries: the float64 oracle's
own adjoint on the CPU, and the GPU kernel's float32 adjoint (the
autograd.Function backward).  Entries whose +-eps step crosses a kink (a
colour clamp at 0 or the sigma > 0 test) are excluded and counted: they are
detected by one-sided differences that disagree."""
import numpy as np
import pytest

from oracle import oracle as O
from svox2_gb300 import synthetic as S

EPS = 1e-4
N_ENTRIES = 512


def _setup():
    g = S.make_grid(32, seed=41, density_mode="normal53")
    off, scl = S.grid_transform(g.reso)
    og = O.Grid(g.links.numpy(), g.density.numpy().astype(np.float32), g.sh.numpy(), 9, off, scl)
    o, d, gt = S.make_rays(256, seed=42)
    return g, og, o.numpy(), d.numpy(), gt.numpy()


OPT = O.Opt(1.0, 0.5, 0.0, 0.0)


def _loss64(og, o, d, gt):
    rgb = O.render(og, OPT, o, d, mode=0, prec="f64", nthreads=4)["rgb"]
    return float(np.mean((rgb - gt.astype(np.float64)) ** 2))


def test_fd_vs_float64_adjoint():
    g, og, o, d, gt = _setup()
    res = O.render(og, OPT, o, d, mode=1, rgb_gt=gt, prec="f64", nthreads=4)
    checked = excluded = 0
    worst = 0.0
    scale = max(np.abs(res["grad_sh"]).max(), np.abs(res["grad_density"]).max())
    for table, row, col, fd, kink in _fd_rounded(og, o, d, gt):
        if kink:
            excluded += 1
            continue
        an = res["grad_density"][row, 0] if table == "density" else res["grad_sh"][row, col]
        err = abs(an - fd)
        worst = max(worst, err / scale)
        assert err <= 2e-3 * abs(fd) + 1e-4 * scale, f"{table}[{row},{col}]: adjoint {an} vs fd {fd}"
        checked += 1
    print(f"FD check: {checked} entries checked, {excluded} excluded (kinks); worst err / max|grad| = {worst:.2e}")
    assert checked >= 400


def _fd_rounded(og, o, d, gt):
    """Central differences with the step actually representable in the float32 tables."""
    rng = np.random.default_rng(43)
    N = og.density.shape[0]
    out = []
    for k in range(N_ENTRIES):
        table = "density" if k % 4 == 0 else "sh"
        row = int(rng.integers(0, N))
        col = 0 if table == "density" else int(rng.integers(0, 27))
        arr = og.density if table == "density" else og.sh
        base = arr[row, col]
        up = np.float32(base + np.float32(EPS))
        dn = np.float32(base - np.float32(EPS))
        vals = []
        for v in (dn, base, up):
            arr[row, col] = v
            vals.append(_loss64(og, o, d, gt))
        arr[row, col] = base
        fm, f0, fp = vals
        h_up, h_dn = float(up) - float(base), float(base) - float(dn)
        fd = (fp - fm) / (h_up + h_dn)
        left, right = (f0 - fm) / h_dn, (fp - f0) / h_up
        kink = abs(left - right) > 2e-2 * max(abs(left), abs(right)) + 1e-9
        out.append((table, row, col, fd, kink))
    return out


@pytest.mark.gpu
def test_fd_vs_gpu_adjoint():
    import torch
    from svox2_gb300 import Rays, SparseGrid
    import torch.nn.functional as F
    g, og, o, d, gt = _setup()
    grid = SparseGrid(reso=32, basis_dim=9, device="cuda")
    grid.density_data.data[:] = g.density.cuda()
    grid.sh_data.data[:] = g.sh.cuda()
    grid.opt.sigma_thresh = 0.0
    grid.opt.stop_thresh = 0.0
    rgb = grid.volume_render(Rays(torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()))
    F.mse_loss(rgb, torch.from_numpy(gt).cuda()).backward()
    gd = grid.density_data.grad.cpu().numpy()
    gs = grid.sh_data.grad.cpu().numpy()
    res64 = O.render(og, OPT, o, d, mode=1, rgb_gt=gt, prec="f64", nthreads=4)
    scale = max(np.abs(res64["grad_sh"]).max(), np.abs(res64["grad_density"]).max())
    checked = excluded = 0
    worst = 0.0
    for table, row, col, fd, kink in _fd_rounded(og, o, d, gt):
        if kink:
            excluded += 1
            continue
        an = gd[row, 0] if table == "density" else gs[row, col]
        err = abs(an - fd)
        worst = max(worst, err / scale)
        assert err <= 2e-3 * abs(fd) + 1e-4 * scale, f"{table}[{row},{col}]: kernel {an} vs fd {fd}"
        checked += 1
    # the whole float32 adjoint against the float64 adjoint
    e_d = float(np.abs(gd - res64["grad_density"]).max() / scale)
    e_s = float(np.abs(gs - res64["grad_sh"]).max() / scale)
    print(f"GPU FD check: {checked} checked, {excluded} excluded; worst err/max|grad| {worst:.2e}; "
          f"full adjoint vs f64: density {e_d:.2e} sh {e_s:.2e}")
    assert e_d < 1e-4 and e_s < 1e-4
    assert checked >= 400
