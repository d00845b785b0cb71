"""The allocation-free fused render (svx_volume_render_cuvol_fused_noalloc).

Callers that cannot allocate device memory while they run — work inside
another framework's callbacks, hosts that plan all device memory before they
start, processes whose device heap belongs to a foreign allocator — use this
entry instead of svx_volume_render_cuvol_fused.  It keeps its scratch (the ray
counter) in a static device array.  This test calls both entries through the
C ABI on the same inputs and requires the allocation-free one to give the same
colours, gradients and mask, within the parity tolerances, on two calls in a
row (the second call finds the array holding the first call's contents).

The file is named to be collected last, so that a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from svox2_gb300 import _lib
from svox2_gb300 import synthetic as S

from helpers import assert_grad, assert_rgb

pytestmark = pytest.mark.gpu


def _structs(spec_t, rays_t):
    (links, dens, sh, off, scl) = spec_t
    g = _lib.SvxGrid()
    g.density_data, g.sh_data, g.links = dens.data_ptr(), sh.data_ptr(), links.data_ptr()
    g.n_voxels = dens.size(0)
    g.size = (C.c_int32 * 3)(*links.shape)
    g.basis_dim, g.sh_data_dim, g.basis_type, g.sh_dtype, g.background_nlayers = 9, 27, 1, _lib.SVX_F32, 0
    g.offset = (C.c_float * 3)(*off)
    g.scaling = (C.c_float * 3)(*scl)
    o, d = rays_t
    r = _lib.SvxRays(o.data_ptr(), d.data_ptr(), o.size(0))
    opt = _lib.SvxRenderOpts(1.0, 0.5, 1e-8, 1e-7, 0.0, 0, 0)
    return g, r, opt


def _call(name, g, r, opt, gt, N):
    rgb = torch.zeros((gt.size(0), 3), device="cuda")
    gd = torch.zeros((N, 1), device="cuda")
    gs = torch.zeros((N, 27), device="cuda")
    mask = torch.zeros((N,), dtype=torch.bool, device="cuda")
    grads = _lib.SvxGridGrads(gd.data_ptr(), gs.data_ptr(), mask.data_ptr())
    stream = torch.cuda.current_stream().cuda_stream
    _lib.call(name, C.byref(g), C.byref(r), C.byref(opt), gt.data_ptr(), 0.0, 0.0, rgb.data_ptr(),
              C.byref(grads), None, stream)
    torch.cuda.synchronize()
    return rgb.cpu().numpy(), gd.cpu().numpy(), gs.cpu().numpy(), mask.cpu().numpy()


def test_noalloc_fused_matches_fused_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    grid = S.make_grid(40, occupancy=0.3, seed=51)
    off, scl = S.grid_transform(grid.reso)
    links, dens, sh = grid.links.cuda(), grid.density.cuda(), grid.sh.cuda()
    o, d, gt = S.make_rays(3000, seed=52)
    o, d, gt = o.cuda(), d.cuda(), gt.cuda()
    g, r, opt = _structs((links, dens, sh, off, scl), (o, d))
    N = dens.size(0)
    ref = _call("svx_volume_render_cuvol_fused", g, r, opt, gt, N)
    for _ in range(2):
        out = _call("svx_volume_render_cuvol_fused_noalloc", g, r, opt, gt, N)
        assert_rgb(out[0], ref[0], "noalloc rgb")
        assert_grad(out[1], ref[1], "noalloc grad_density")
        assert_grad(out[2], ref[2], "noalloc grad_sh")
        np.testing.assert_array_equal(out[3], ref[3])
