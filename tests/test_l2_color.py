"""SparseGrid.inplace_l2_color_grad (svox2/svox2.py:1897-1932) against what the reference
computed on the same inputs (tests/golden/make_golden.py l2_case): dense, on a channel range,
and over the rows of a sparse SH indexer."""
from pathlib import Path

import numpy as np
import pytest
import torch

from svox2_gb300 import SparseGrid

GOLD = Path(__file__).resolve().parent / "golden" / "l2_dense6_sh9.npz"


def _grid(z, device):
    n = z["sh"].shape[0]
    links = torch.arange(n, dtype=torch.int32).view(6, 6, 6)
    return SparseGrid.from_tables(links.to(device), torch.zeros((n, 1), device=device),
                                  torch.from_numpy(z["sh"]).to(device))


@pytest.mark.parametrize("device", ["cpu", pytest.param("cuda", marks=pytest.mark.gpu)])
def test_l2_color_grad_matches_reference(device):
    z = np.load(GOLD)
    grid = _grid(z, device)
    dense = torch.from_numpy(z["grad0"]).to(device)
    grid.inplace_l2_color_grad(dense, start_dim=3, end_dim=-2, scaling=0.7)
    np.testing.assert_allclose(dense.cpu().numpy(), z["dense"], rtol=1e-6, atol=1e-7)
    sparse = torch.from_numpy(z["grad0"]).to(device)
    grid.sparse_sh_grad_indexer = torch.from_numpy(z["mask"]).to(device)
    grid.inplace_l2_color_grad(sparse, scaling=1.3)
    np.testing.assert_allclose(sparse.cpu().numpy(), z["sparse"], rtol=1e-6, atol=1e-7)
