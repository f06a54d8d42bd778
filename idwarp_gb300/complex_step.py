"""Names of the reference's complex-step classes (idwarp/UnstructuredMesh_C.py,
idwarp/MultiUnstructuredMesh_C.py), so that code importing them finds them.

The complex build of the warp is not part of the GPU path: derivatives come
from ``warpDeriv`` (reverse), ``warpDerivFwd`` (forward) and
``idwarp_gb300.autograd.warp``, all exact products of the same kernels; the
complex-step check of those lives in the CPU restatement used by the tests.
Constructing either class raises ``Error`` saying so.
"""
from .options import Error

_MESSAGE = (
    "%s (the complex-step build of IDWarp) is not available on the GPU path: use warpDeriv / "
    "warpDerivFwd or idwarp_gb300.autograd.warp for derivatives of the warp."
)


class USMesh_C:
    def __init__(self, *args, **kwargs):
        raise Error(_MESSAGE % "USMesh_C")


class MultiUSMesh_C:
    def __init__(self, *args, **kwargs):
        raise Error(_MESSAGE % "MultiUSMesh_C")
