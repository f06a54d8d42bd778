"""Complex-step versions of the mesh classes (idwarp/UnstructuredMesh_C.py,
idwarp/MultiUnstructuredMesh_C.py).

``USMesh_C`` takes complex surface coordinates and returns complex grids,
like the reference's USMesh over its complexified library: with a
perturbation i*h (h = 1e-40) of the surface, Im(Xv)/h is the derivative of
the warped grid along that perturbation, an independent check of
``warpDerivFwd`` and ``warpDeriv``.  It runs on the GPU's FP64 path
(``precision`` is fixed to "fp64"): the nodal properties are evaluated in
complex arithmetic from the complex coordinates, and the imaginary parts of
M_i and b_i go through the same tree walk as the real ones (the weighted
sums are linear in M and b, and the weights and decisions depend only on
the initial surface and the volume nodes).
"""
import ctypes as C

import numpy as np

from . import _lib
from .options import Error
from .UnstructuredMesh import USMesh


class USMesh_C(USMesh):
    """Complex unstructured mesh (idwarp/UnstructuredMesh_C.py:19-34)."""

    def __init__(self, options=None, comm=None, debug=False):
        if options is not None:
            if options.get("precision", "fp64") != "fp64":
                raise Error("USMesh_C evaluates the complex step in FP64; precision must be 'fp64'.")
            options = dict(options)
            options["precision"] = "fp64"
        super().__init__(options=options, comm=comm, debug=debug)
        self.dtype = "D"
        self._csCoords = None
        self._csWarped = False

    def getSurfaceCoordinates(self):
        """All surface coordinates on this processor, complex, shape (N,3)."""
        if self._csCoords is not None:
            return self._csCoords.copy()
        self._setInternalSurface()
        coords = np.zeros((self.nSurf, 3))
        self._chk(self.lib.idw_get_surface_coordinates(self.ctx, C.c_void_p(coords.ctypes.data), coords.size,
                                                         _lib.IDW_HOST), "getSurfaceCoordinates")
        return coords.astype(complex)

    def setSurfaceCoordinates(self, coordinates):
        """Set the surface coordinates (complex, or real: imaginary part zero)."""
        if len(coordinates) != self.nSurf:
            raise Error(
                "Incorrect length of coordinates supplied to setSurfaceCoordinates on proc %d. Expected aray of "
                "length %d, received an array of length %d." % (self.comm.rank, self.nSurf, len(coordinates))
            )
        coords = np.ascontiguousarray(np.asarray(coordinates, dtype=np.complex128).reshape(self.nSurf, 3))
        rc = self.lib.idw_set_surface_coordinates_cs(self.ctx, C.c_void_p(coords.ctypes.data), 3 * self.nSurf,
                                                      _lib.IDW_HOST)
        if rc == _lib.IDW_ERR_NONFINITE:
            raise Error("Non-finite surface coordinates supplied to setSurfaceCoordinates.")
        self._chk(rc, "setSurfaceCoordinates")
        self._csCoords = coords.copy()
        self._csWarped = False
        self._surfVersion += 1

    def warpMesh(self):
        """Warp the volume mesh to the complex surface coordinates."""
        self._setInternalSurface()
        self._setMeshOptions()
        if self._csCoords is None:
            self.setSurfaceCoordinates(self.getSurfaceCoordinates())
        self._chk(self.lib.idw_warp_mesh_cs(self.ctx), "warpMesh")
        self._csWarped = True

    def getWarpGrid(self):
        """Current grid in warp order, complex, flat (3*nVol,)."""
        if not self._csWarped:
            return super().getWarpGrid().astype(complex)
        out = np.zeros(3 * self.nVol, np.complex128)
        self._chk(self.lib.idw_get_volume_coordinates_cs(self.ctx, C.c_void_p(out.ctypes.data), out.size,
                                                           _lib.IDW_HOST), "getWarpGrid")
        return out

    def getCommonGrid(self):
        """Grid in the common ordering (one process: the warp ordering), complex."""
        return self.getWarpGrid()

    def getSolverGrid(self):
        """Current grid in the order set by setExternalMeshIndices(), complex."""
        if self.solverMeshDOF is None:
            raise Error("setExternalMeshIndices() must be called before getSolverGrid().")
        grid = self.getWarpGrid()
        out = np.zeros(self.solverMeshDOF, np.complex128)
        for part in ("real", "imag"):
            w = np.ascontiguousarray(getattr(grid, part))
            s = np.zeros(self.solverMeshDOF)
            self._chk(self.lib.idw_warp_to_solver_grid(self.ctx, C.c_void_p(w.ctypes.data), w.size,
                                                         C.c_void_p(s.ctypes.data), s.size, _lib.IDW_HOST),
                      "warp_to_solver_grid")
            if part == "real":
                out.real = s
            else:
                out.imag = s
        return out


class MultiUSMesh_C:
    """Complex multi-group mesh (idwarp/MultiUnstructuredMesh_C.py): not
    provided; the complex step is checked per USMesh_C instance."""

    def __init__(self, *args, **kwargs):
        raise Error("MultiUSMesh_C is not provided: use one USMesh_C per group for the complex step.")
