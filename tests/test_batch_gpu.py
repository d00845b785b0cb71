"""The multi-grid batch launch (svx_render_batch), the coherence order
(svx_ray_order) and the accumulation flush (svx_add_accum) through the C ABI.

Rays of three grids go into one launch, through a per-ray grid index and a
device table of grid descriptors; each grid's colours, gradients and masks are
checked against the oracle run on that grid alone, with the tolerances of the
single-grid parity tests (tests/helpers.py)."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as O
from svox2_gb300 import _lib
from svox2_gb300 import csrc
from svox2_gb300 import synthetic as S

from helpers import assert_grad, assert_grad_f64, assert_rgb, grid_pair, opt_struct

pytestmark = pytest.mark.gpu

SPECS = [(32, 0.3, 700), ((24, 40, 32), 0.25, 900), (40, 0.2, 500)]   # (reso, occupancy, rays)


def _setup(sh_dtype, seed=11):
    grids, rays = [], []
    for i, (reso, occ, q) in enumerate(SPECS):
        g = S.make_grid(reso, occupancy=occ, seed=seed + i)
        spec, og = grid_pair(g, 9, sh_dtype)
        o, d, gt = S.make_rays(q, seed=seed + 10 * i)
        grids.append((spec, og))
        rays.append((o, d, gt))
    return grids, rays


def _order(spec, o, d, opt, base, out):
    r = _lib.SvxRays(o.data_ptr(), d.data_ptr(), o.shape[0])
    _lib.call("svx_ray_order", C.byref(csrc._grid_struct(spec)), C.byref(r), C.byref(csrc._opt_struct(opt)),
              base, out.data_ptr(), torch.cuda.current_stream().cuda_stream)


def _batch(mode, grids, rays, opt, sh_dtype, use_order, accum_for=(), with_bg=0, cache_samples=0,
           record_samples=0):
    """One svx_render_batch launch over every grid's rays; returns rgb per grid and the
    per-grid gradient buffers (accumulation rows already flushed)."""
    dev = "cuda"
    n = sum(o.shape[0] for o, _, _ in rays)
    O_ = torch.cat([o for o, _, _ in rays]).to(dev)
    D_ = torch.cat([d for _, d, _ in rays]).to(dev)
    GT = torch.cat([gt for _, _, gt in rays]).to(dev)
    ray_grid = torch.cat([torch.full((o.shape[0],), i, dtype=torch.int32) for i, (o, _, _) in
                          enumerate(rays)]).to(dev)
    order = torch.full((n,), -1, dtype=torch.int32, device=dev)
    descs, bufs = [], []
    off = 0
    for i, ((spec, og), (o, d, gt)) in enumerate(zip(grids, rays)):
        N, Cc = spec.sh_data.shape
        b = {"gd": torch.zeros((N, 1), device=dev), "gs": torch.zeros((N, Cc), device=dev),
             "mask": torch.zeros((N,), dtype=torch.bool, device=dev)}
        desc = _lib.SvxBatchGrid()
        desc.grid = csrc._grid_struct(spec)
        if mode == 1:
            desc.grads = _lib.SvxGridGrads(b["gd"].data_ptr(), b["gs"].data_ptr(), b["mask"].data_ptr())
            if spec.background_data is not None:
                b["gbg"] = torch.zeros(spec.background_data.shape, device=dev)
                b["mbg"] = torch.zeros(spec.background_data.shape[:2], dtype=torch.bool, device=dev)
                desc.grads.grad_background_out = b["gbg"].data_ptr()
                desc.grads.mask_background_out = b["mbg"].data_ptr()
            desc.norm = 2.0 / (3 * o.shape[0])
            if i in accum_for:
                b["accum"] = torch.zeros((N, (Cc + 1 + 3) // 4 * 4), device=dev)
                desc.accum = b["accum"].data_ptr()
                desc.accum_stride = b["accum"].size(1)
        descs.append(bytes(desc))
        bufs.append(b)
        if use_order:
            _order(spec, O_[off:off + o.shape[0]], D_[off:off + o.shape[0]], opt, off, order[off:off + o.shape[0]])
        off += o.shape[0]
    table = torch.tensor(np.frombuffer(b"".join(descs), dtype=np.uint8), device=dev)
    n_dev = torch.tensor([n], dtype=torch.int64, device=dev)
    work = torch.zeros((4,), dtype=torch.int64, device=dev)
    rgb = torch.zeros((n, 3), device=dev)
    dt = {torch.float32: _lib.SVX_F32, torch.bfloat16: _lib.SVX_BF16, torch.float16: _lib.SVX_F16}[sh_dtype]
    st = torch.cuda.current_stream().cuda_stream
    cache = None
    if cache_samples:
        nbytes = int(_lib.load().svx_batch_colour_cache_bytes(cache_samples))
        cache = torch.empty((nbytes // 4,), dtype=torch.float32, device=dev)
    if record_samples:
        nbytes = int(_lib.load().svx_batch_record_bytes(n, record_samples))
        cache = torch.empty((nbytes // 4,), dtype=torch.float32, device=dev)
    _lib.call("svx_render_batch", mode, table.data_ptr(), 9, dt, with_bg, O_.data_ptr(), D_.data_ptr(),
              ray_grid.data_ptr(),
              order.data_ptr() if use_order else None, n_dev.data_ptr(), n, C.byref(csrc._opt_struct(opt)),
              GT.data_ptr() if mode == 1 else None, rgb.data_ptr(), work.data_ptr(),
              None if cache is None else cache.data_ptr(), 0 if cache is None else cache.numel() * 4, st)
    for (spec, _), b in zip(grids, bufs):
        if "accum" in b:
            _lib.call("svx_add_accum", b["accum"].data_ptr(), b["accum"].size(1), spec.sh_data.size(1),
                      b["accum"].size(0), b["gs"].data_ptr(), b["gd"].data_ptr(), st)
    torch.cuda.synchronize()
    if use_order:
        assert torch.equal(torch.sort(order.long()).values.cpu(), torch.arange(n))
    out, off = [], 0
    for o, _, _ in rays:
        out.append(rgb[off:off + o.shape[0]].cpu().numpy())
        off += o.shape[0]
    return out, bufs


@pytest.mark.parametrize("cache", [(0, 0), (64, 0), (0, 64), (0, 512)],
                         ids=["smem_cache", "global_cache", "records_overflow", "records"])
@pytest.mark.parametrize("sh_dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("use_order", [False, True])
def test_batch_fused_matches_oracle_per_grid(sh_dtype, use_order, cache):
    """Without a colour cache buffer the fused batch keeps 48 samples a ray in shared memory;
    with one of 64 samples a ray, rays longer than that gather colours again past it.  With a
    record buffer it runs as two kernels: with records of 64 samples the rays that evaluate more
    are listed and redone by the one-kernel step; with 512 every ray fits."""
    cache_samples, record_samples = cache
    opt, oopt = opt_struct()
    grids, rays = _setup(sh_dtype)
    rgbs, bufs = _batch(1, grids, rays, opt, sh_dtype, use_order, accum_for=(1,), cache_samples=cache_samples,
                        record_samples=record_samples)
    for (spec, og), (o, d, gt), rgb, b in zip(grids, rays, rgbs, bufs):
        ref = O.render(og, oopt, o.numpy(), d.numpy(), mode=1, rgb_gt=gt.numpy(), prec="f32")
        r64 = O.render(og, oopt, o.numpy(), d.numpy(), mode=1, rgb_gt=gt.numpy(), prec="f64", stops=ref["stops"],
                       want_magnitude=True)
        assert_rgb(rgb, ref["rgb"], "rgb")
        assert_rgb(rgb, r64["rgb"], "rgb vs float64")
        assert_grad_f64(b["gd"].cpu().numpy(), r64["grad_density"], r64["mag_density"], "batch grad_density")
        assert_grad_f64(b["gs"].cpu().numpy(), r64["grad_sh"], r64["mag_sh"], "batch grad_sh")
        np.testing.assert_array_equal(b["mask"].cpu().numpy(), ref["mask"])


def test_batch_render_order_is_bit_exact():
    """Forward colours do not depend on the processing order or on the other grids of the batch."""
    opt, oopt = opt_struct()
    grids, rays = _setup(torch.float32, seed=23)
    plain, _ = _batch(0, grids, rays, opt, torch.float32, False)
    ordered, _ = _batch(0, grids, rays, opt, torch.float32, True)
    for (spec, og), (o, d, _), a, b in zip(grids, rays, plain, ordered):
        np.testing.assert_array_equal(a, b)
        alone = csrc.volume_render_cuvol(spec, _rays(o, d), opt).cpu().numpy()
        np.testing.assert_array_equal(a, alone)
        assert_rgb(a, O.render(og, oopt, o.numpy(), d.numpy(), mode=0, prec="f32")["rgb"], "rgb")


def _rays(o, d):
    r = csrc.RaysSpec()
    r.origins, r.dirs = o.cuda().contiguous(), d.cuda().contiguous()
    return r


def test_ray_order_permutation_and_misses_last():
    opt, _ = opt_struct()
    g = S.make_grid(32, occupancy=0.3, seed=5)
    spec, _ = grid_pair(g)
    o, d, _ = S.make_rays(5000, seed=3)
    miss = torch.arange(0, 5000, 7)
    # outside the sphere around the [-1, 1]^3 grid (radius 2 > sqrt 3), pointing outwards
    u = o[miss] / o[miss].norm(dim=-1, keepdim=True)
    o[miss] = 2.0 * u
    d[miss] = u
    base = 1234
    out = torch.full((5000,), -1, dtype=torch.int32, device="cuda")
    _order(spec, o.cuda(), d.cuda(), opt, base, out)
    torch.cuda.synchronize()
    idx = out.long().cpu() - base
    assert torch.equal(torch.sort(idx).values, torch.arange(5000))
    tail = set(idx[-miss.numel():].tolist())
    assert tail == set(miss.tolist()), "rays that miss the grid must come last"
    # the same call twice gives the same order
    out2 = torch.empty_like(out)
    _order(spec, o.cuda(), d.cuda(), opt, base, out2)
    torch.cuda.synchronize()
    assert torch.equal(out, out2)


def test_add_accum_adds_nonzero_rows_only():
    gen = torch.Generator().manual_seed(4)
    N, Cc, stride = 3000, 27, 28
    acc = torch.randn((N, stride), generator=gen)
    acc[::3] = 0.0
    gs = torch.randn((N, Cc), generator=gen)
    gd = torch.randn((N, 1), generator=gen)
    gs[::3, 0] = -0.0                                   # zero rows leave even a -0.0 untouched
    ref_s = gs.clone()
    ref_d = gd.clone()
    nz = acc.abs().sum(1) != 0
    ref_s[nz] += acc[nz, :Cc]
    ref_d[nz] += acc[nz, Cc:Cc + 1]
    A, S_, D = acc.cuda(), gs.cuda(), gd.cuda()
    _lib.call("svx_add_accum", A.data_ptr(), stride, Cc, N, S_.data_ptr(), D.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(S_.cpu(), ref_s) and torch.equal(D.cpu(), ref_d)
    assert torch.equal(torch.signbit(S_.cpu()[::3, 0]), torch.ones(N // 3, dtype=torch.bool))
    with pytest.raises(RuntimeError, match="stride"):
        _lib.call("svx_add_accum", A.data_ptr(), 26, Cc, N, S_.data_ptr(), D.data_ptr(), None)


def _with_background(grids, rays, which, seed=40):
    """Give the grids listed in `which` an MSI background of their own, and send half of their
    rays off in random directions."""
    for i in which:
        spec, og = grids[i]
        gen = torch.Generator().manual_seed(seed + i)
        reso, nl = 8 + 2 * i, 4 + i
        keep = torch.rand((2 * reso, reso), generator=gen) >= 0.2
        bl = torch.full(keep.shape, -1, dtype=torch.int32)
        bl[keep] = torch.arange(int(keep.sum()), dtype=torch.int32)
        bd = torch.randn((int(keep.sum()), nl, 4), generator=gen) * 0.5
        bd[..., 3] = torch.rand((int(keep.sum()), nl), generator=gen) * 4.0 - 0.5
        spec.background_links, spec.background_data = bl.cuda(), bd.cuda()
        og.bg_links, og.bg_data = bl.numpy(), bd.numpy()
        o, d, gt = rays[i]
        q = o.shape[0]
        dr = torch.randn((q // 2, 3), generator=gen)
        d = d.clone()
        d[q // 2:] = dr / dr.norm(dim=-1, keepdim=True)
        rays[i] = (o, d.contiguous(), gt)


@pytest.mark.parametrize("use_order", [False, True])
def test_batch_with_background_matches_oracle_per_grid(use_order):
    """Grids 0 and 2 carry MSI backgrounds, grid 1 none: one launch renders and differentiates
    each ray against its own grid's background (or brightness)."""
    opt, oopt = opt_struct(stop_thresh=0.0)
    grids, rays = _setup(torch.float32, seed=31)
    _with_background(grids, rays, (0, 2))
    rgbs, bufs = _batch(1, grids, rays, opt, torch.float32, use_order, accum_for=(1,), with_bg=1)
    for i, ((spec, og), (o, d, gt), rgb, b) in enumerate(zip(grids, rays, rgbs, bufs)):
        ref = O.render(og, oopt, o.numpy(), d.numpy(), mode=1, rgb_gt=gt.numpy(), prec="f64")
        err = np.abs(rgb - ref["rgb"]).max()
        assert err <= 5e-5, (i, err)
        for k, key in (("gd", "grad_density"), ("gs", "grad_sh"), ("gbg", "grad_background")):
            if k not in b:
                continue
            r = ref[key]
            bad = np.abs(b[k].cpu().numpy() - r) > 1e-3 * np.abs(r) + 1e-4 * max(np.abs(r).max(), 1e-30)
            assert not bad.any(), (i, key, int(bad.sum()))
        if "mbg" in b:
            assert np.abs(ref["grad_background"]).max() > 0
            # a sample on a cell boundary may fall in either cell (the kernel's norms round
            # differently from the float64 oracle's): a few rows of zero weight may differ
            diff = int((b["mbg"].cpu().numpy() != ref["mask_background"]).sum())
            assert diff <= max(4, ref["mask_background"].size // 200), (i, diff)


def test_batch_render_with_background_equals_single_grid():
    """Forward colours of the batch launch equal the single-grid render of each grid, with
    and without its background."""
    opt, _ = opt_struct()
    grids, rays = _setup(torch.float32, seed=37)
    _with_background(grids, rays, (1,))
    batch, _ = _batch(0, grids, rays, opt, torch.float32, True, with_bg=1)
    for (spec, og), (o, d, _), a in zip(grids, rays, batch):
        alone = csrc.volume_render_cuvol(spec, _rays(o, d), opt).cpu().numpy()
        np.testing.assert_array_equal(a, alone)
