"""idwarp_gb300 — IDWarp's inverse-distance-weighted mesh warping on a GB300.

``USMesh`` is a drop-in for ``idwarp.USMesh`` on the warping path; the
evaluation runs in hand-written sm_103a CUDA kernels behind the C ABI of
``libidwarp_gb300.so`` (include/idwarp_gb300.h).
"""
from .options import Error
from .UnstructuredMesh import USMesh, pointReduce
from .MultiUnstructuredMesh import MultiUSMesh
from .complex_step import MultiUSMesh_C, USMesh_C

__version__ = "0.1.0"
__all__ = ["USMesh", "MultiUSMesh", "USMesh_C", "MultiUSMesh_C", "Error", "pointReduce"]
