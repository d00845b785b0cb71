"""The allocation-free fused render (svx_volume_render_cuvol_fused_noalloc).

Callers that cannot allocate device memory while they run — work inside
another framework's callbacks, hosts that plan all device memory before they
start, processes whose device heap belongs to a foreign allocator — use this
entry instead of svx_volume_render_cuvol_fused.  It keeps its scratch (the ray
counter) in a static device array.  This test calls both entries through the
C ABI on the same inputs, two calls of the allocation-free one in a row (the
second finds the array holding the first call's contents), and requires:
  * its colours, gradients and mask to match the other entry's and the oracle's
    (indexing bit for bit, colours within 1e-5, gradients per entry against the
    float64 oracle within the float32 floor);
  * at 40,960 rays, where the other entry sorts the rays and scatters through its
    accumulation rows while this one runs them in input order with scalar atomics;
  * with the MSI background and with bfloat16 SH;
  * that the call changes neither the device's default memory pool nor PyTorch's
    caching allocator.

The file is named to be collected last, so that a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from svox2_gb300 import _lib
from svox2_gb300 import csrc as ops
from svox2_gb300 import synthetic as S

from helpers import assert_rgb, check_fused, grid_pair, opt_struct, rays_pair, stats_dict

pytestmark = pytest.mark.gpu


def _bg_tables(bg_reso, nl, seed):
    gen = torch.Generator().manual_seed(seed)
    keep = torch.rand((2 * bg_reso, bg_reso), generator=gen) >= 0.2
    links = torch.full(keep.shape, -1, dtype=torch.int32)
    links[keep] = torch.arange(int(keep.sum()), dtype=torch.int32)
    data = torch.randn((int(keep.sum()), nl, 4), generator=gen) * 0.5
    data[..., 3] = torch.rand((int(keep.sum()), nl), generator=gen) * 4.0 - 0.5
    return links, data


_cu = None


def _pool_usage():
    """(reserved, used) bytes of the current device's default memory pool, read through the
    driver API (the pool is the driver's, whichever runtime allocates from it)."""
    global _cu
    if _cu is None:
        _cu = C.CDLL("libcuda.so.1")
    dev = C.c_int()
    assert _cu.cuDeviceGet(C.byref(dev), C.c_int(torch.cuda.current_device())) == 0
    pool = C.c_void_p()
    assert _cu.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    out = []
    for attr in (5, 7):   # CU_MEMPOOL_ATTR_RESERVED_MEM_CURRENT, CU_MEMPOOL_ATTR_USED_MEM_CURRENT
        v = C.c_uint64()
        assert _cu.cuMemPoolGetAttribute(pool, C.c_int(attr), C.byref(v)) == 0
        out.append(v.value)
    return tuple(out)


def _call(name, spec, rays, opt, gt, N, n_sh, bg_shape=None, stats=None):
    rgb = torch.zeros((gt.size(0), 3), device="cuda")
    grads = ops.GridOutputGrads()
    grads.grad_density_out = torch.zeros((N, 1), device="cuda")
    grads.grad_sh_out = torch.zeros((N, n_sh), device="cuda")
    grads.mask_out = torch.zeros((N,), dtype=torch.bool, device="cuda")
    if bg_shape is not None:
        grads.grad_background_out = torch.zeros(bg_shape, device="cuda")
        grads.mask_background_out = torch.zeros(bg_shape[:2], dtype=torch.bool, device="cuda")
    g = ops._grid_struct(spec)
    r = ops._rays_struct(rays, gt.device)
    gg = ops._grads_struct(grads, N, n_sh, gt.device, True, bg_shape)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    before = (_pool_usage(), torch.cuda.memory_allocated(), torch.cuda.memory_reserved())
    _lib.call(name, C.byref(g), C.byref(r), C.byref(ops._opt_struct(opt)), gt.data_ptr(), 0.0, 0.0,
              rgb.data_ptr(), C.byref(gg), ops._stats_struct(stats), stream)
    torch.cuda.synchronize()
    after = (_pool_usage(), torch.cuda.memory_allocated(), torch.cuda.memory_reserved())
    return rgb, grads, before, after


CASES = {
    # name: (reso, occupancy, rays, sh dtype, background)
    "sparse40_3000": (40, 0.3, 3000, torch.float32, False),
    "sparse48_40960": (48, 0.3, 40960, torch.float32, False),
    "bf16_3000": (40, 0.3, 3000, torch.bfloat16, False),
    "background_2000": (24, 0.3, 2000, torch.float32, True),
}


@pytest.mark.parametrize("name", list(CASES))
def test_noalloc_fused_matches_fused_and_oracle_twice(name):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    reso, occ, Q, dt, with_bg = CASES[name]
    grid = S.make_grid(reso, occupancy=occ, seed=51)
    spec, og = grid_pair(grid, sh_dtype=dt)
    bg_shape = None
    o, d, gt = S.make_rays(Q, seed=52)
    if with_bg:
        bl, bd = _bg_tables(16, 8, 53)
        spec.background_links, spec.background_data = bl.cuda(), bd.cuda()
        og.bg_links, og.bg_data = bl.numpy(), bd.numpy()
        bg_shape = tuple(bd.shape)
        dr = torch.randn((Q // 2, 3), generator=torch.Generator().manual_seed(54))
        d[Q // 2:] = dr / dr.norm(dim=-1, keepdim=True)
        d = d.contiguous()
    rays = rays_pair(o, d)
    opt, oopt = opt_struct()
    gt_dev = gt.cuda()
    N, n_sh = og.density.shape[0], og.sh.shape[1]
    ref_rgb, ref_grads, _, _ = _call("svx_volume_render_cuvol_fused", spec, rays, opt, gt_dev, N, n_sh, bg_shape)
    for i in range(2):
        st = stats_dict(Q)
        rgb, grads, before, after = _call("svx_volume_render_cuvol_fused_noalloc", spec, rays, opt, gt_dev, N,
                                          n_sh, bg_shape, stats=st)
        assert before == after, f"call {i}: memory pools changed: {before} -> {after}"
        assert_rgb(rgb.cpu().numpy(), ref_rgb.cpu().numpy(), f"{name} call {i}: rgb vs the allocating entry")
        np.testing.assert_array_equal(grads.mask_out.cpu().numpy(), ref_grads.mask_out.cpu().numpy())
        if with_bg:
            # the background's equirectangular map differs from the host's asinf/atan2 in the
            # last bits: its gradients are held to the allocating entry, which the background
            # tests hold to the oracle and to the reference's kernels
            for key in ("grad_density_out", "grad_sh_out", "grad_background_out"):
                k, r = getattr(grads, key).cpu().numpy(), getattr(ref_grads, key).cpu().numpy()
                err = np.abs(k.astype(np.float64) - r).max() / max(np.abs(r).max(), 1e-30)
                assert err <= 1e-5, f"{name} call {i}: {key} differs from the allocating entry by {err:.2e}"
            np.testing.assert_array_equal(grads.mask_background_out.cpu().numpy(),
                                          ref_grads.mask_background_out.cpu().numpy())
        else:
            check_fused(rgb, grads, st["ray_trace"].cpu().numpy(), st["eval_samples"].item(), og, oopt, o, d, gt,
                        label=f"{name} noalloc call {i}")
