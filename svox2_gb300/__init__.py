"""svox2_gb300 — GB300-native (sm_103a) Plenoxels sparse-voxel renderer.

Drop-in for the reference ``svox2`` package's CUDA path: ``SparseGrid``,
``Rays``, ``Camera`` and ``RenderOptions`` keep their names and signatures;
``svox2_gb300.csrc`` is the operator module (the reference's ``svox2.csrc``),
backed by the C ABI of ``libsvox2_gb300.so`` (include/svox2_gb300.h).
"""
from .defs import BASIS_TYPE_3D_TEXTURE, BASIS_TYPE_MLP, BASIS_TYPE_SH
from .svox2 import Camera, Rays, RenderOptions, SparseGrid

__version__ = "0.1.0"

__all__ = ["SparseGrid", "Rays", "Camera", "RenderOptions", "BASIS_TYPE_SH", "BASIS_TYPE_3D_TEXTURE",
           "BASIS_TYPE_MLP", "__version__"]
