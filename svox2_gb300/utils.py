"""Host-side helpers used by the grid API: SH constants and evaluation, Morton
order of the links table, integer helpers.

Constants are the published real spherical-harmonic normalisations
(svox2/utils.py:84-112); ``eval_sh_bases`` evaluates the same polynomials as
svox2/utils.py:115-162 for degree <= 2, which is what the renderer supports.
"""
from __future__ import annotations

from typing import Optional

import torch

SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = [1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792,
         0.5462742152960396]

# largest SH basis the reference accepts (svox2/utils.py:114); this renderer builds 1, 4 and 9.
MAX_SH_BASIS = 10


def isqrt(x: int) -> Optional[int]:
    """Exact integer square root, or None if x is not a positive square."""
    if x <= 0:
        return None
    r = int(x ** 0.5)
    while r * r > x:
        r -= 1
    while (r + 1) * (r + 1) <= x:
        r += 1
    return r if r * r == x else None


def is_pow2(x: int) -> bool:
    return x > 0 and (x & (x - 1)) == 0


def eval_sh_bases(basis_dim: int, dirs: torch.Tensor) -> torch.Tensor:
    """SH basis values (..., basis_dim) at unit directions (..., 3), degree <= 2."""
    if basis_dim not in (1, 4, 9):
        raise ValueError(f"basis_dim {basis_dim}: degree <= 2 (1, 4, 9) supported")
    out = torch.empty((*dirs.shape[:-1], basis_dim), dtype=dirs.dtype, device=dirs.device)
    out[..., 0] = SH_C0
    if basis_dim > 1:
        x, y, z = dirs.unbind(-1)
        out[..., 1] = -SH_C1 * y
        out[..., 2] = SH_C1 * z
        out[..., 3] = -SH_C1 * x
        if basis_dim > 4:
            out[..., 4] = SH_C2[0] * x * y
            out[..., 5] = SH_C2[1] * y * z
            out[..., 6] = SH_C2[2] * (2.0 * z * z - x * x - y * y)
            out[..., 7] = SH_C2[3] * x * z
            out[..., 8] = SH_C2[4] * (x * x - y * y)
    return out


def _spread_bits(v: torch.Tensor, nbits: int) -> torch.Tensor:
    """Insert two zero bits above every bit of v (bit b moves to 3b)."""
    out = torch.zeros_like(v)
    for b in range(nbits):
        out |= ((v >> b) & 1) << (3 * b)
    return out


def gen_morton(D: int, device="cpu", dtype=torch.long) -> torch.Tensor:
    """Z-order index of every cell of a D^3 grid, x the most significant axis.

    Same ordering as the reference's use_z_order links (svox2/utils.py:45-79).
    """
    if not is_pow2(D):
        raise ValueError("Morton order needs a power-of-2 resolution")
    nbits = max(D.bit_length() - 1, 1)
    a = torch.arange(D, device=device, dtype=torch.long)
    X, Y, Z = torch.meshgrid(a, a, a, indexing="ij")
    code = (_spread_bits(X, nbits) << 2) | (_spread_bits(Y, nbits) << 1) | _spread_bits(Z, nbits)
    return code.to(dtype)
