"""Basis-type constants, same values as the reference (svox2/defs.py:1-4)."""

BASIS_TYPE_SH = 1
BASIS_TYPE_3D_TEXTURE = 4
BASIS_TYPE_MLP = 255
