"""The fused step as two kernels (forward with per-ray records, then the reverse pass from them).

svx_volume_render_cuvol_fused runs an SH9 grid without the MSI background as two kernels when
the per-ray records fit the budget (SVX_FUSED_SPLIT_BYTES, read at each call), in chunks of
rays when they do not all fit at once, and as the one-kernel fused step when the budget is 0.
Every GPU fused test runs the two-kernel form at its default budget; this file holds the three
forms to one another and to the oracle on the same inputs:
  * colours and the per-ray sample trace bit for bit between the forms (the forward arithmetic is
    the same; only the gradient atomics' order differs);
  * gradients and masks of each form against the oracle (helpers.check_fused);
  * an unsorted small batch, a coherence-sorted batch with the accumulation rows, several chunks,
    BF16 storage, last_sample_opaque and the beta / sparsity terms.
"""
import os

import numpy as np
import pytest
import torch

from svox2_gb300 import synthetic as S

from helpers import check_fused, grid_pair, opt_struct, rays_pair, run_fused_kernel

pytestmark = pytest.mark.gpu

ENV = "SVX_FUSED_SPLIT_BYTES"


def _run(budget, spec, rays, opt, gt, N, n_sh, **kw):
    old = os.environ.get(ENV)
    try:
        if budget is None:
            os.environ.pop(ENV, None)
        else:
            os.environ[ENV] = str(budget)
        return run_fused_kernel(spec, rays, opt, gt, N, n_sh, **kw)
    finally:
        if old is None:
            os.environ.pop(ENV, None)
        else:
            os.environ[ENV] = old


def _record_bytes(reso, step=0.5):
    # 2 + 64 + ceil(max samples / 32) * 32 float4 entries per ray, as the host sizes them
    cap = int(np.ceil((np.sqrt(3.0) * reso / step + 2.0) / 32.0) * 32)
    return 16 * (2 + 64 + cap)


CASES = {
    # name: (reso, occupancy, rays, sh dtype, chunks, opt kwargs, beta, sparsity)
    "small_unsorted": (40, 0.3, 3000, torch.float32, 1, {}, 0.0, 0.0),
    "sorted_40960": (48, 0.3, 40960, torch.float32, 1, {}, 0.0, 0.0),
    "sorted_40960_5chunks": (48, 0.3, 40960, torch.float32, 5, {}, 0.0, 0.0),
    "bf16_sorted": (48, 0.3, 40960, torch.bfloat16, 1, {}, 0.0, 0.0),
    "opaque_beta_sparsity": (40, 0.3, 3000, torch.float32, 1, {"last_opaque": True}, 0.3, 0.01),
}


@pytest.mark.parametrize("name", list(CASES))
def test_two_kernel_fused_matches_one_kernel_and_oracle(name):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    reso, occ, Q, dt, chunks, okw, beta, sparsity = CASES[name]
    grid = S.make_grid(reso, occupancy=occ, seed=61)
    spec, og = grid_pair(grid, sh_dtype=dt)
    o, d, gt = S.make_rays(Q, seed=62)
    rays = rays_pair(o, d)
    opt, oopt = opt_struct(**okw)
    N, n_sh = og.density.shape[0], og.sh.shape[1]
    kw = dict(beta=beta, sparsity=sparsity)
    budget = None if chunks == 1 else _record_bytes(reso) * ((Q + chunks - 1) // chunks)
    two = _run(budget, spec, rays, opt, gt, N, n_sh, **kw)
    one = _run(0, spec, rays, opt, gt, N, n_sh, **kw)
    for key in ("ray_trace", "eval_samples"):
        np.testing.assert_array_equal(two[2][key].cpu().numpy(), one[2][key].cpu().numpy())
    np.testing.assert_array_equal(two[0].cpu().numpy(), one[0].cpu().numpy())
    np.testing.assert_array_equal(two[1].mask_out.cpu().numpy(), one[1].mask_out.cpu().numpy())
    for label, (rgb, grads, st) in (("two kernels", two), ("one kernel", one)):
        check_fused(rgb, grads, st["ray_trace"].cpu().numpy(), st["eval_samples"].item(), og, oopt, o, d, gt,
                    beta=beta, sparsity=sparsity, label=f"{name} {label}")
