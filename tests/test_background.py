"""MSI background model: the oracle pinned to the reference, and the host side.

* The oracle's background in the reference's pure-PyTorch semantics
  (svox2/svox2.py:796-876) against golden vectors the reference itself produced:
  colours and the gradients of the MSE loss for density, SH and the background.
  The sphere setup, intersector, equirectangular map, wrapped trilinear fetch and
  compositing that this checks are the ones the CUDA semantics use too.
* The oracle's CUDA semantics (render_lerp_kernel_cuvol.cu:386-607): its backward
  against central differences of its forward, in float64, and the plain backward
  (mode 2) against the fused one.
* Checkpoints with a background written by the reference, and sparsify_background
  without dilation, against the reference's own results.
"""
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import SparseGrid

GOLD = Path(__file__).resolve().parent / "golden"
BG = sorted(GOLD.glob("background_*.npz"))


def _grid(z):
    return O.Grid(z["links"], z["density"], z["sh"], int(z["basis_dim"]), tuple(z["offset"]), tuple(z["scaling"]),
                  bg_links=z["bg_links"], bg_data=z["bg_data"])


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


@pytest.mark.parametrize("path", BG, ids=[p.stem for p in BG])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_background_matches_reference_cpu_path(path, prec):
    z = np.load(path)
    opt = O.Opt(background_brightness=float(z["bg"]), step_size=float(z["step"]), sigma_thresh=0.0,
                stop_thresh=0.0, bg_cpu_semantics=True)
    r = O.render(_grid(z), opt, z["origins"], z["dirs"], mode=1, rgb_gt=z["rgb_gt"], prec=prec, nthreads=1)
    np.testing.assert_allclose(r["rgb"], z["rgb"], rtol=1e-5, atol=5e-6)
    assert _rel(r["grad_density"], z["grad_density"]) < 2e-5
    assert _rel(r["grad_sh"], z["grad_sh"]) < 2e-5
    assert _rel(r["grad_background"], z["grad_background"]) < 2e-5
    # every background row the reference gave a gradient is in the mask
    touched = (z["grad_background"] != 0).any(axis=-1)
    assert not np.any(touched & ~r["mask_background"])


def test_cuda_semantics_differ_from_the_cpu_path():
    """The two semantics sample different points: the restatement must not coincide with the
    CPU path (it would mean the switch does nothing)."""
    z = np.load(BG[0])
    opt = O.Opt(background_brightness=float(z["bg"]), step_size=float(z["step"]), sigma_thresh=0.0, stop_thresh=0.0)
    r = O.render(_grid(z), opt, z["origins"], z["dirs"], mode=0, prec="f64", nthreads=1)
    assert np.abs(r["rgb"] - z["rgb"]).max() > 1e-2


def _case(seed=5, reso=6, nl=3, bg_reso=5, n=24, bd=4):
    rng = np.random.default_rng(seed)
    N = reso ** 3
    links = np.arange(N, dtype=np.int32).reshape(reso, reso, reso)
    dens = np.clip(rng.normal(0.2, 0.6, (N, 1)), 0, None).astype(np.float32)
    sh = (rng.normal(0, 0.3, (N, 3 * bd))).astype(np.float32)
    keep = rng.random((2 * bg_reso, bg_reso)) >= 0.2
    bl = np.full(keep.shape, -1, np.int32)
    bl[keep] = np.arange(keep.sum(), dtype=np.int32)
    bgd = rng.normal(0, 0.5, (int(keep.sum()), nl, 4)).astype(np.float32)
    bgd[..., 3] = (rng.random((int(keep.sum()), nl)) * 4 - 0.5).astype(np.float32)
    off = (0.5 * reso - 0.5,) * 3
    scl = (0.5 * reso,) * 3
    g = O.Grid(links, dens, sh, bd, off, scl, bg_links=bl, bg_data=bgd)
    o = rng.normal(size=(n, 3))
    o = (1.5 * o / np.linalg.norm(o, axis=1, keepdims=True)).astype(np.float32)
    d = rng.random((n, 3)) - 0.5 - o
    d[n // 2:] = rng.normal(size=(n - n // 2, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    gt = rng.random((n, 3)).astype(np.float32)
    return g, o, d, gt


def _loss(g, opt, o, d, gt):
    r = O.render(g, opt, o, d, mode=0, prec="f64", nthreads=1)
    return float(np.mean((r["rgb"] - gt.astype(np.float64)) ** 2))


def _fd_check(g, opt, o, d, gt, table, grad, picks, h=2.0 ** -10):
    """Central differences of the float64 loss over float32 entries of table (exact +-h steps)."""
    scale = np.abs(grad).max()
    flat = table.reshape(-1)
    gflat = grad.reshape(-1)
    for i in picks:
        x = flat[i]
        flat[i] = x + np.float32(h)
        lp = _loss(g, opt, o, d, gt)
        flat[i] = x - np.float32(h)
        lm = _loss(g, opt, o, d, gt)
        flat[i] = x
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gflat[i]) <= 2e-3 * scale + 1e-3 * abs(fd), (i, fd, gflat[i], scale)


def test_oracle_cuda_semantics_gradient_matches_finite_differences():
    g, o, d, gt = _case()
    opt = O.Opt(background_brightness=0.8, step_size=0.5, sigma_thresh=0.0, stop_thresh=0.0)
    r = O.render(g, opt, o, d, mode=1, rgb_gt=gt, prec="f64", nthreads=1)
    gb = r["grad_background"]
    assert np.abs(gb).max() > 0 and r["mask_background"].any()
    # the largest background entries of each channel, and a few density voxels
    picks = []
    for ch in range(4):
        v = np.abs(gb[..., ch]).reshape(-1)
        picks += [int(k) * 4 + ch for k in np.argsort(v)[-3:]]
    _fd_check(g, opt, o, d, gt, g.bg_data, gb, picks)
    gd = r["grad_density"]
    _fd_check(g, opt, o, d, gt, g.density, gd, list(np.argsort(np.abs(gd).reshape(-1))[-4:]))


def test_oracle_plain_backward_matches_fused():
    """volume_render_cuvol_backward given dL/drgb of the MSE loss and the forward colour
    gives the fused gradients (no early stop, so both start the background from the same
    transmittance)."""
    g, o, d, gt = _case(seed=9)
    opt = O.Opt(background_brightness=1.0, step_size=0.5, sigma_thresh=0.0, stop_thresh=0.0)
    f = O.render(g, opt, o, d, mode=1, rgb_gt=gt, prec="f64", nthreads=1)
    go = ((f["rgb"] - gt) * (2.0 / (3 * o.shape[0]))).astype(np.float32)
    b = O.render(g, opt, o, d, mode=2, grad_out=go, color=f["rgb"], prec="f64", nthreads=1)
    for k in ("grad_density", "grad_sh", "grad_background"):
        assert _rel(b[k], f[k]) < 1e-6, k


def test_background_rays_that_miss_the_grid_see_only_the_background():
    g, o, d, gt = _case(seed=3)
    opt = O.Opt(background_brightness=0.5, step_size=0.5, sigma_thresh=0.0, stop_thresh=0.0)
    with_bg = O.render(g, opt, o, d, mode=0, prec="f64", nthreads=1)["rgb"]
    empty = O.Grid(g.links, np.zeros_like(g.density), g.sh, g.basis_dim, g.offset, g.scaling,
                   bg_links=g.bg_links, bg_data=g.bg_data)
    only_bg = O.render(empty, opt, o, d, mode=0, prec="f64", nthreads=1)["rgb"]
    nobg = O.Grid(g.links, g.density, g.sh, g.basis_dim, g.offset, g.scaling)
    fg = O.render(nobg, opt, o, d, mode=0, prec="f64", nthreads=1)["rgb"]
    # rays through an empty grid: background (+ brightness behind it) only, never the plain brightness
    assert not np.allclose(only_bg, 0.5)
    # a ray whose foreground is transparent gets exactly what the empty grid gives it
    transparent = np.all(np.abs(fg - 0.5) < 1e-12, axis=1)
    assert transparent.any()
    np.testing.assert_allclose(with_bg[transparent], only_bg[transparent], rtol=1e-12, atol=1e-12)


# ---------------------------------------------------------------- host side

CKPT = GOLD / "ckpt_bg_sparse6x5x4_sh4_l3_r4.npz"
CKPT_LOADED = GOLD / "ckpt_bg_sparse6x5x4_sh4_l3_r4_loaded.npz"


def test_load_reference_checkpoint_with_background():
    ref = np.load(CKPT_LOADED)
    grid = SparseGrid.load(str(CKPT))
    assert grid.use_background
    assert grid.background_nlayers == int(ref["background_nlayers"])
    assert grid.background_reso == int(ref["background_reso"])
    np.testing.assert_array_equal(grid.background_links.numpy(), ref["background_links"])
    np.testing.assert_array_equal(grid.background_data.data.numpy(), ref["background_data"])
    np.testing.assert_array_equal(grid.links.numpy(), ref["links"])
    np.testing.assert_array_equal(grid.sh_data.data.numpy(), ref["sh_data"])


@pytest.mark.parametrize("compress", [False, True])
def test_save_with_background_writes_the_reference_format(tmp_path, compress):
    ref_file = np.load(CKPT)
    src = np.load(CKPT_LOADED)
    grid = SparseGrid.from_tables(torch.from_numpy(ref_file["links"]), torch.from_numpy(src["src_density"]),
                                  torch.from_numpy(src["src_sh"]), radius=src["radius"].tolist(),
                                  center=src["center"].tolist())
    grid.background_nlayers = int(src["background_nlayers"])
    grid.background_reso = int(src["background_reso"])
    grid.background_links = torch.from_numpy(src["background_links"])
    grid.background_data = torch.nn.Parameter(torch.from_numpy(src["src_background_data"]))
    out = tmp_path / "grid.npz"
    grid.save(str(out), compress=compress)
    mine = np.load(out)
    assert sorted(mine.files) == sorted(ref_file.files)
    for k in ref_file.files:
        assert mine[k].dtype == ref_file[k].dtype, k
        np.testing.assert_array_equal(mine[k], ref_file[k], err_msg=k)


def test_new_grid_with_background_matches_the_reference_layout():
    g = SparseGrid(reso=4, basis_dim=1, background_nlayers=3, background_reso=5)
    assert g.use_background
    assert g.background_links.shape == (10, 5) and g.background_links.dtype == torch.int32
    np.testing.assert_array_equal(g.background_links.view(-1).numpy(), np.arange(50))
    assert g.background_data.shape == (50, 3, 4) and float(g.background_data.detach().abs().sum()) == 0.0
    spec = g._to_cpp()
    assert spec.background_links is g.background_links and spec.background_data is g.background_data
    with pytest.raises(AssertionError):
        SparseGrid(reso=4, basis_dim=1, background_nlayers=1)


def test_sparsify_background_matches_reference_without_dilation():
    z = np.load(GOLD / "sparsify_bg_l4_r6.npz")
    g = SparseGrid(reso=4, basis_dim=1, background_nlayers=z["data_in"].shape[1],
                   background_reso=z["links_in"].shape[1])
    g.background_links = torch.from_numpy(z["links_in"].copy())
    g.background_data = torch.nn.Parameter(torch.from_numpy(z["data_in"].copy()))
    g.sparsify_background(sigma_thresh=float(z["sigma_thresh"]), dilate=0)
    np.testing.assert_array_equal(g.background_links.numpy(), z["links_out"])
    np.testing.assert_array_equal(g.background_data.data.numpy(), z["data_out"])
    with pytest.raises(RuntimeError):
        g.sparsify_background(dilate=1)   # the dilation is a CUDA kernel


def test_oracle_msi_tv_known_answer():
    """msi_tv_grad_sparse (loss_kernel.cu:248-333) on a 2 x 1 x 2 MSI, worked out by hand:
    x wraps (the neighbour of column 1 is column 0), y has one row (its neighbour is itself,
    dy = 0), z stops at the last layer, where a colour channel compares with itself and sigma
    with 0.  Scales are divided by the cell count."""
    links = np.array([[0], [1]], np.int32)                    # [2 reso, reso], reso = 1
    msi = np.array([[[1.0, 2.0], [3.0, 5.0]],                 # cell (0,0): layers 0, 1; (colour, sigma)
                    [[4.0, 1.0], [0.0, 2.0]]], np.float32)    # cell (1,0)
    cells = np.array([0, 1, 2, 3], np.int32)                   # (x, y, z) = (0,0,0) (0,0,1) (1,0,0) (1,0,1)
    s, s_last = 0.8, 0.4
    g = O.msi_tv_grad(links, msi, cells, s, s_last, prec="f64")
    exp = np.zeros_like(msi, dtype=np.float64)
    sx, sy, sz = 2 / 256, 1 / 256, 2 / 256

    m64 = msi.astype(np.float64)
    s, s_last = float(np.float32(s)), float(np.float32(s_last))   # the float32 scales the call passes

    def term(x, z, ch):
        nl = 2
        v00 = m64[x, z, ch]
        vz = m64[x, z + 1, ch] if z + 1 < nl else (0.0 if ch == 1 else v00)
        v10 = m64[1 - x, z, ch]
        dx, dy, dz = v10 - v00, 0.0, vz - v00
        scale = float(np.float32(s_last) / np.float32(4)) if ch == 1 else float(np.float32(s) / np.float32(4))
        idelta = scale / np.sqrt(float(np.float32(1e-9)) + dx * dx + dy * dy + dz * dz)
        dx, dz = dx * sx, dz * sz
        exp[x, z, ch] += -(dx + dz) * idelta
        if z + 1 < nl:
            exp[x, z + 1, ch] += dz * idelta
        exp[1 - x, z, ch] += dx * idelta

    for x in range(2):
        for z in range(2):
            for ch in range(2):
                term(x, z, ch)
    np.testing.assert_allclose(g, exp, rtol=1e-12, atol=1e-15)


def test_rand_cells_background_window_wraps():
    """_get_rand_cells_background: max(int(frac * n), 1) contiguous cells over the
    [2 reso, reso, nlayers] cells from a host RNG start, wrapping at the end."""
    g = SparseGrid(reso=4, basis_dim=1, background_nlayers=3, background_reso=4)
    n = 2 * 4 * 4 * 3
    for seed in range(20):
        np.random.seed(seed)
        cells = g._get_rand_cells_background(0.25, contiguous=True).numpy()
        assert cells.shape == (int(0.25 * n),)
        assert cells.min() >= 0 and cells.max() < n
        assert np.all((np.diff(cells) == 1) | (np.diff(cells) == 1 - n))
    np.random.seed(0)
    assert g._get_rand_cells_background(0.0).shape == (1,)


def test_save_load_roundtrip_of_a_background_grid(tmp_path):
    """A grid built with a background (its links a registered buffer) goes through save / load
    with every table intact and the background layer count and resolution restored."""
    g = SparseGrid(reso=6, basis_dim=4, background_nlayers=3, background_reso=5, radius=[1.0, 1.2, 0.9],
                   center=[0.1, 0.0, -0.2])
    gen = torch.Generator().manual_seed(3)
    with torch.no_grad():
        g.density_data.copy_(torch.randn(g.density_data.shape, generator=gen))
        g.sh_data.copy_(torch.randn(g.sh_data.shape, generator=gen))
        g.background_data.copy_(torch.randn(g.background_data.shape, generator=gen))
    g.background_links[0, :2] = -1
    path = tmp_path / "bg.npz"
    g.save(str(path))
    back = SparseGrid.load(str(path))
    assert back.use_background and back.background_nlayers == 3 and back.background_reso == 5
    np.testing.assert_array_equal(back.background_links.numpy(), g.background_links.numpy())
    np.testing.assert_array_equal(back.background_data.data.numpy(), g.background_data.data.numpy())
    np.testing.assert_array_equal(back.density_data.data.numpy(), g.density_data.data.numpy())
    # SH goes through float16 on disk, as in the reference
    np.testing.assert_array_equal(back.sh_data.data.numpy(), g.sh_data.data.numpy().astype(np.float16).astype(np.float32))


def test_oracle_background_image_equals_its_rays():
    """The oracle's image path with a background gives the colours of its ray path on the
    camera's rays (the image kernel is checked against this path on the GPU)."""
    g, *_ = _case(seed=11)
    opt = O.Opt(background_brightness=0.6, step_size=0.5, sigma_thresh=1e-8, stop_thresh=1e-7)
    c2w = np.array([[1, 0, 0, 0.2], [0, 0, -1, -2.5], [0, 1, 0, 0.1]], np.float32)
    img = O.render_image(g, opt, c2w, 9.0, 9.0, 6.0, 5.0, 12, 10, prec="f64")["rgb"]
    # the same rays, formed as the pinhole camera forms them
    ys, xs = np.mgrid[0:10, 0:12]
    x = (xs + 0.5 - 6.0) / 9.0
    y = (ys + 0.5 - 5.0) / 9.0
    z = np.sqrt(x * x + y * y + 1.0)
    cam = np.stack([x / z, y / z, 1.0 / z], -1).reshape(-1, 3)
    d = (cam @ c2w[:, :3].T.astype(np.float64)).astype(np.float32)
    o = np.broadcast_to(c2w[:, 3], d.shape).astype(np.float32).copy()
    rays = O.render(g, opt, o, d, mode=0, prec="f64")["rgb"]
    np.testing.assert_allclose(img.reshape(-1, 3), rays, atol=2e-5)
