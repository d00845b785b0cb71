"""SparseGrid.save / SparseGrid.load (svox2/svox2.py:1526-1628), against a checkpoint
that the reference itself wrote and what the reference read back from it
(tests/golden/make_golden.py, checkpoint_case)."""
from pathlib import Path

import numpy as np
import pytest
import torch

from svox2_gb300 import SparseGrid

GOLD = Path(__file__).resolve().parent / "golden"
CKPT = GOLD / "ckpt_sparse10x12x14_sh9.npz"
LOADED = GOLD / "ckpt_sparse10x12x14_sh9_loaded.npz"


def test_load_reference_checkpoint():
    ref = np.load(LOADED)
    grid = SparseGrid.load(str(CKPT))
    np.testing.assert_array_equal(grid.links.numpy(), ref["links"])
    np.testing.assert_array_equal(grid.density_data.data.numpy(), ref["density_data"])
    np.testing.assert_array_equal(grid.sh_data.data.numpy(), ref["sh_data"])
    np.testing.assert_array_equal(grid.radius.numpy(), ref["radius"])
    np.testing.assert_array_equal(grid.center.numpy(), ref["center"])
    assert grid.basis_dim == int(ref["basis_dim"]) and grid.sh_data.dtype == torch.float32


@pytest.mark.parametrize("compress", [False, True])
def test_save_writes_the_reference_format(tmp_path, compress):
    ref_file = np.load(CKPT)
    src = np.load(LOADED)
    grid = SparseGrid.from_tables(torch.from_numpy(ref_file["links"]), torch.from_numpy(src["src_density"]),
                                  torch.from_numpy(src["src_sh"]), radius=src["radius"].tolist(),
                                  center=src["center"].tolist())
    out = tmp_path / "grid.npz"
    grid.save(str(out), compress=compress)
    mine = np.load(out)
    assert sorted(mine.files) == sorted(ref_file.files)
    for k in ref_file.files:
        assert mine[k].dtype == ref_file[k].dtype, k
        np.testing.assert_array_equal(mine[k], ref_file[k], err_msg=k)


def test_low_precision_residency_and_legacy_layout(tmp_path):
    src = np.load(LOADED)
    bf = SparseGrid.load(str(CKPT), sh_dtype=torch.bfloat16)
    assert bf.sh_data.dtype == torch.bfloat16
    np.testing.assert_array_equal(bf.sh_data.data.float().numpy(),
                                  torch.from_numpy(src["sh_data"]).to(torch.bfloat16).float().numpy())
    hf = SparseGrid.load(str(CKPT), sh_dtype=torch.float16)
    np.testing.assert_array_equal(hf.sh_data.data.float().numpy(), src["sh_data"])   # float16 on disk: exact
    # the older single-table layout ("data" = [density | sh])
    legacy = tmp_path / "legacy.npz"
    np.savez(legacy, links=src["links"], data=np.concatenate([src["density_data"], src["sh_data"]], axis=1))
    g = SparseGrid.load(str(legacy))
    np.testing.assert_array_equal(g.sh_data.data.numpy(), src["sh_data"])
    np.testing.assert_array_equal(g.density_data.data.numpy(), src["density_data"])
    assert g.radius.tolist() == [1.0, 1.0, 1.0]


@pytest.mark.gpu
def test_load_to_cuda_accelerates():
    from oracle import oracle as O
    ref = np.load(LOADED)
    grid = SparseGrid.load(str(CKPT), device="cuda")
    np.testing.assert_array_equal(grid.links.cpu().numpy(), O.accel_dist_prop(ref["links"]))
    np.testing.assert_array_equal(grid.sh_data.data.cpu().numpy(), ref["sh_data"])
