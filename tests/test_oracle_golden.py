"""Pin the CPU oracle to the reference implementation: golden vectors made by
tests/golden/make_golden.py from sxyu/svox2's own CPU path (volume_render with
use_kernel=False + autograd, sample + autograd)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
RENDER = sorted(GOLD.glob("render_*.npz"))


def _grid(z):
    return O.Grid(z["links"], z["density"], z["sh"], int(z["basis_dim"]), tuple(z["offset"]), tuple(z["scaling"]))


def _opt(z):
    # sigma_thresh = stop_thresh = 0: the setting in which the reference CPU path and kernel agree
    return O.Opt(background_brightness=float(z["bg"]), step_size=float(z["step"]), sigma_thresh=0.0,
                 stop_thresh=0.0)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


@pytest.mark.parametrize("path", RENDER, ids=[p.stem for p in RENDER])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_render_matches_reference_cpu_path(path, prec):
    z = np.load(path)
    res = O.render(_grid(z), _opt(z), z["origins"], z["dirs"], mode=1, rgb_gt=z["rgb_gt"], prec=prec, nthreads=1)
    # colours: float32 reference arithmetic vs this restatement (different rounding order)
    np.testing.assert_allclose(res["rgb"], z["rgb"], rtol=2e-6, atol=1e-6)
    # gradients of mean((rgb - gt)^2), relative to the largest entry
    assert _rel(res["grad_density"], z["grad_density"]) < 1e-5
    assert _rel(res["grad_sh"], z["grad_sh"]) < 1e-5
    # the mask covers exactly the voxels that the reference path gave a gradient
    touched = (z["grad_sh"] != 0).any(axis=1) | (z["grad_density"][:, 0] != 0)
    assert not np.any(touched & ~res["mask"])


def test_sample_matches_reference_cpu_path():
    z = np.load(GOLD / "sample_dense10_sh9.npz")
    g = _grid(z)
    d, s = O.sample(g, z["points"], True, prec="f64")
    np.testing.assert_allclose(d, z["out_density"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(s, z["out_sh"], rtol=1e-5, atol=1e-6)
    gd, gs = O.sample_backward(g, z["points"], z["grad_out_density"], z["grad_out_sh"], True, prec="f64")
    np.testing.assert_allclose(gd, z["grad_density"], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(gs, z["grad_sh"], rtol=1e-4, atol=1e-5)
