"""USMesh: the IDWarp unstructured-mesh warping API on a GB300.

Drop-in for ``idwarp.USMesh`` (idwarp/UnstructuredMesh.py) on the warping
path: the same method names, arguments, return shapes, option names and
error behaviour, backed by the CUDA library ``libidwarp_gb300.so`` through
its C ABI (include/idwarp_gb300.h) instead of the Fortran/PETSc f2py module.

One process drives one GPU.  The reference's MPI decomposition of the volume
nodes is not needed: the whole volume mesh lives in device memory.  ``comm``
is accepted for API compatibility and must have a single rank; several GPUs
run independent replicas, each with its own mesh object.
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from .options import BaseSolver, Error


class _SelfComm:
    rank = 0
    size = 1

    def allgather(self, x):
        return [x]

    def bcast(self, x, root=0):
        return x

    def py2f(self):
        return 0


class USMesh(BaseSolver):
    """Main unstructured-mesh warping object (idwarp/UnstructuredMesh.py:43)."""

    def __init__(self, options=None, comm=None, debug=False):
        name = "IDWarp"
        category = "Volume mesh warping"
        if comm is None:
            comm = _SelfComm()
        defOpts = self._getDefaultOptions()
        if options is None:
            raise Error(
                "The 'options' keyword argument is *NOT* optional. An options dictionary must be passed upon "
                "creation of this object"
            )
        super().__init__(name, category, defaultOptions=defOpts, options=options, comm=comm)
        if getattr(comm, "size", 1) > 1:
            raise Error(
                "USMesh on a GB300 runs one process per GPU and holds the whole volume mesh; run one replica per "
                "GPU with its own communicator of size 1."
            )
        self.printOptions()
        self.lib = _lib.load()
        self.dtype = "d"
        o = _lib.idw_options()
        self.lib.idw_default_options(C.byref(o))
        self._fill_options(o)
        ctx = C.c_void_p()
        rc = self.lib.idw_create(C.byref(o), C.byref(ctx))
        if rc != 0:
            raise _lib.LibraryError("idw_create failed with status %d (is a CUDA device visible?)" % rc)
        self.ctx = ctx
        self.warpInitialized = False
        self.faceSizes = None
        self.nSurf = 0
        self.nVol = 0
        self.solverMeshDOF = None
        self._surfVersion = 0
        self._setMeshOptions()
        self.fileType = self.getOption("fileType")
        fileName = self.getOption("gridFile")
        if fileName is not None:
            self._readGrid(fileName)

    @staticmethod
    def _getDefaultOptions():
        # idwarp/UnstructuredMesh.py:124-145, plus the GB300 precision switch and
        # the in-memory NPY grid type.
        return {
            "gridFile": [(str, type(None)), None],
            "fileType": [str, ["CGNS", "OpenFOAM", "PLOT3D", "NPY"]],
            "specifiedSurfaces": [(list, type(None)), None],
            "symmetrySurfaces": [(list, type(None)), None],
            "symmetryPlanes": [(list, type(None)), None],
            "aExp": [float, 3.0],
            "bExp": [float, 5.0],
            "LdefFact": [float, 1.0],
            "alpha": [float, 0.25],
            "errTol": [float, 0.0005],
            "evalMode": [str, ["fast", "exact"]],
            "symmTol": [float, 1e-6],
            "useRotations": [bool, True],
            "zeroCornerRotations": [bool, True],
            "cornerAngle": [float, 30.0],
            "restartFile": [(str, type(None)), None],
            "bucketSize": [int, 8],
            "precision": [str, ["mixed", "fp64"]],
            "mixedGate": [float, 2e-3],
            "diagnostics": [int, 0],
            "exactSchedule": [str, ["auto", "tiled", "walk"]],
            "adjointPrecision": [str, ["precise", "fast"]],
            "walkLists": [str, ["auto", "off"]],
            "treeBuild": [str, ["kd", "morton"]],
            "deterministic": [bool, False],
        }

    # ------------------------------------------------------------------
    # grid input
    # ------------------------------------------------------------------
    def _readGrid(self, fileName):
        if self.fileType == "NPY":
            x0 = np.load(fileName)
            self.createCommonGrid(np.asarray(x0, dtype=np.float64).reshape(-1, 3))
        elif self.fileType == "PLOT3D":
            from .plot3d import readPlot3D

            nodes, sizes = readPlot3D(fileName, return_blocks=True)
            self._plot3dShape = sizes  # writeGrid writes the same blocks back
            self.createCommonGrid(nodes)
        elif self.fileType == "CGNS":
            raise Error(
                "CGNS grid files need libcgns/HDF5, which this build does not link. Pass the volume nodes with "
                "createCommonGrid(), or use fileType 'NPY' or 'PLOT3D'."
            )
        else:
            raise Error("OpenFOAM grids need pyofm, which is not available. Pass the volume nodes with createCommonGrid().")

    def createCommonGrid(self, volNodes):
        """Set the volume grid (N,3) in common order (src/IO/createGrid.F90, libidwarp.pyf:14-17)."""
        x = volNodes
        if isinstance(x, np.ndarray):
            x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        ptr, where = _lib.vptr(x)
        n = x.shape[0]
        self._chk(self.lib.idw_create_common_grid(self.ctx, ptr, n, where), "createCommonGrid")
        self.nVol = n
        self._gridSet = True
        self.warpInitialized = False

    # ------------------------------------------------------------------
    # surface definition and coordinates
    # ------------------------------------------------------------------
    def getSurfaceCoordinates(self):
        """Return all surface coordinates on this processor, shape (N,3)."""
        self._setInternalSurface()
        coords = np.zeros((self.nSurf, 3), np.float64)
        self._chk(self.lib.idw_get_surface_coordinates(self.ctx, C.c_void_p(coords.ctypes.data), coords.size,
                                                         _lib.IDW_HOST), "getSurfaceCoordinates")
        return coords

    def setSurfaceCoordinates(self, coordinates):
        """Set all surface coordinates on this processor; same shape as getSurfaceCoordinates()."""
        if len(coordinates) != self.nSurf:
            raise Error(
                "Incorrect length of coordinates supplied to setSurfaceCoordinates on proc %d. Expected aray of "
                "length %d, received an array of length %d." % (self.comm.rank, self.nSurf, len(coordinates))
            )
        if isinstance(coordinates, np.ndarray) or not hasattr(coordinates, "data_ptr"):
            coordinates = np.ascontiguousarray(coordinates, dtype=np.float64)
        ptr, where = _lib.vptr(coordinates)
        # host arrays are checked for non-finite values by the library, which
        # then leaves the surface unchanged
        rc = self.lib.idw_set_surface_coordinates(self.ctx, ptr, 3 * self.nSurf, where)
        if rc == _lib.IDW_ERR_NONFINITE:
            raise Error("Non-finite surface coordinates supplied to setSurfaceCoordinates.")
        self._chk(rc, "setSurfaceCoordinates")
        self._surfVersion += 1

    def setExternalMeshIndices(self, ind):
        """Set the 0-based DOF indices of the solver grid into the common grid."""
        ind = np.ascontiguousarray(np.asarray(ind).ravel(), dtype=np.int32)
        self._chk(self.lib.idw_set_external_mesh_indices(self.ctx, _lib.iptr(ind), len(ind)),
                    "setExternalMeshIndices")
        self.solverMeshDOF = len(ind)

    def setSurfaceDefinition(self, pts, conn, faceSizes, cgnsBlockID=None):
        """Define the warping surface (idwarp/UnstructuredMesh.py:196-262).

        pts (M,3) nodes on this processor, conn flat 0-based connectivity,
        faceSizes the number of nodes of each face."""
        conn = np.array(conn).flatten()
        self._setSymmetryConditions()
        pts = np.ascontiguousarray(np.asarray(pts, dtype=np.float64).reshape(-1, 3))
        faceSizes = np.asarray(faceSizes).ravel()
        allPts = np.vstack(self.comm.allgather(pts))
        allFaceSizes = np.hstack(self.comm.allgather(faceSizes)).astype(np.int32)
        ptSizes = self.comm.allgather(len(pts))
        offsets = np.zeros(len(ptSizes), "intc")
        offsets[1:] = np.cumsum(ptSizes)[:-1]
        allConn = np.hstack(self.comm.allgather(conn + offsets[self.comm.rank])).astype(np.int32)

        uniquePts, link, nUnique = pointReduce(allPts, 1e-12, lib=self.lib)
        # Sort the unique points by z, y, x so the tree does not depend on the
        # input ordering (idwarp/UnstructuredMesh.py:242-256).
        ind = np.lexsort(uniquePts.T)
        uniquePts = np.ascontiguousarray(uniquePts[ind])
        inv = np.zeros_like(ind, "intc")
        rng = np.arange(len(ind)).astype("intc")
        inv[ind[rng]] = rng
        link = np.ascontiguousarray(inv[link - 1] + 1, dtype=np.int32)
        if not getattr(self, "_gridSet", False):
            raise Error("The volume grid must be set (gridFile or createCommonGrid) before setSurfaceDefinition.")
        self._setMeshOptions()
        self._chk(
            self.lib.idw_initialize_warping(self.ctx, _lib.dptr(allPts), len(allPts), _lib.dptr(uniquePts), nUnique,
                                            _lib.iptr(link), _lib.iptr(allFaceSizes), len(allFaceSizes),
                                            _lib.iptr(allConn), len(allConn)),
            "setSurfaceDefinition")
        self.nSurf = len(pts)
        self.faceSizes = allFaceSizes
        self.restartStatus = self._setDenominator0(self.getOption("restartFile"))
        self.warpInitialized = True

    def _setDenominator0(self, restartFile):
        """The denominator estimate: computed now, or through the restart file
        (initializeWarping.F90:98-312; format in idwarp_gb300.restart)."""
        if not restartFile:
            self._chk(self.lib.idw_compute_denominator0(self.ctx), "denominator0")
            return "computed"
        from .restart import CHECK_STRIDE, load_or_compute

        def load(den0):
            rc = self.lib.idw_set_denominator0(self.ctx, C.c_void_p(den0.ctypes.data), den0.size, CHECK_STRIDE, _lib.IDW_HOST)
            if rc in (_lib.IDW_ERR_RESTART, _lib.IDW_ERR_NONFINITE):
                return False
            self._chk(rc, "restartFile")
            return True

        def save():
            den0 = np.zeros(self.nVol)
            costs = np.zeros(self.nVol)
            self._chk(self.lib.idw_get_denominator0(self.ctx, C.c_void_p(den0.ctypes.data), self.nVol, _lib.IDW_HOST),
                      "denominator0")
            self._chk(self.lib.idw_dry_run_costs(self.ctx, C.c_void_p(costs.ctypes.data), self.nVol, _lib.IDW_HOST), "dryRun")
            return den0, costs

        def compute():
            self._chk(self.lib.idw_compute_denominator0(self.ctx), "denominator0")

        log = print if self.comm.rank == 0 else (lambda *a: None)
        return load_or_compute(restartFile, self.nVol, load, compute, save, log=log)

    def getLoadBalancingCosts(self):
        """dryRun cost of every volume node in common order, summed over the
        mirrors and divided by the number of unique surface points
        (kd_tree.F90:789-830, initializeWarping.F90:258-266)."""
        costs = np.zeros(self.nVol)
        self._chk(self.lib.idw_dry_run_costs(self.ctx, C.c_void_p(costs.ctypes.data), self.nVol, _lib.IDW_HOST), "dryRun")
        return costs

    def setSurfaceDefinitionFromFile(self, surfFile):
        """Surface definition from a multiblock PLOT3D surface file (quads)."""
        from .plot3d import readPlot3DSurface

        pts, conn = readPlot3DSurface(surfFile)
        self.setSurfaceDefinition(pts, conn, 4 * np.ones(len(conn), "intc"))

    def setSurfaceFromFile(self, surfFile):
        """Update the surface coordinates from a PLOT3D surface file with the same blocks."""
        from .plot3d import readPlot3DSurface

        pts, _ = readPlot3DSurface(surfFile)
        self.setSurfaceCoordinates(pts)

    # ------------------------------------------------------------------
    # grids
    # ------------------------------------------------------------------
    def getSolverGrid(self):
        """Current grid in the order set by setExternalMeshIndices(), flat (3*n,)."""
        if self.solverMeshDOF is None:
            raise Error("setExternalMeshIndices() must be called before getSolverGrid().")
        solverGrid = np.zeros(self.solverMeshDOF, np.float64)
        warpGrid = self.getWarpGrid()
        self._chk(self.lib.idw_warp_to_solver_grid(self.ctx, C.c_void_p(warpGrid.ctypes.data), warpGrid.size,
                                                     C.c_void_p(solverGrid.ctypes.data), solverGrid.size,
                                                     _lib.IDW_HOST), "warp_to_solver_grid")
        return solverGrid

    def getWarpGrid(self, out=None, wait=True):
        """Current grid in warp order, flat (3*nVol,).  ``out`` (optional) is a
        contiguous float64 host array of that size to fill, e.g. in pinned
        memory for fast repeated reads.  ``wait=False`` (with ``out``) queues
        the copy and returns at once: ``out`` is complete after
        ``synchronize()``, and the copy overlaps the work queued after it (the
        next warpMesh writes another device buffer meanwhile)."""
        if out is None:
            if not wait:
                raise Error("getWarpGrid(wait=False) needs an output array (out=...).")
            out = np.zeros(3 * self.nVol, np.float64)
        elif out.dtype != np.float64 or out.size != 3 * self.nVol or not out.flags.c_contiguous:
            raise Error("getWarpGrid(out=...) needs a contiguous float64 array of %d entries." % (3 * self.nVol))
        if wait:
            self._chk(self.lib.idw_get_volume_coordinates(self.ctx, C.c_void_p(out.ctypes.data), out.size,
                                                            _lib.IDW_HOST), "getWarpGrid")
        else:
            self._chk(self.lib.idw_get_volume_coordinates_async(self.ctx, C.c_void_p(out.ctypes.data), out.size),
                      "getWarpGrid")
        return out

    def synchronize(self):
        """Wait for the mesh's queued GPU work and asynchronous grid reads."""
        self._chk(self.lib.idw_synchronize(self.ctx), "synchronize")

    def getCommonGrid(self):
        """Grid in the original (common) ordering, flat (3*nVol,)."""
        out = np.zeros(3 * self.nVol, np.float64)
        self._chk(self.lib.idw_get_common_volume_coordinates(self.ctx, C.c_void_p(out.ctypes.data), out.size,
                                                               _lib.IDW_HOST), "getCommonGrid")
        return out

    def getdXs(self):
        """Result of the last warpDeriv(), shape (nSurf,3)."""
        dXs = np.zeros((self.nSurf, 3), np.float64)
        self._chk(self.lib.idw_get_dxs(self.ctx, C.c_void_p(dXs.ctypes.data), dXs.size, _lib.IDW_HOST), "getdXs")
        return dXs

    # ------------------------------------------------------------------
    # warping and derivatives
    # ------------------------------------------------------------------
    def warpMesh(self):
        """Warp the volume mesh to the surface set by setSurfaceCoordinates()."""
        self._setInternalSurface()
        self._setMeshOptions()
        self._chk(self.lib.idw_warp_mesh(self.ctx), "warpMesh")

    def warpDeriv(self, dXv, solverVec=True):
        """dXs = (dXv/dXs)^T dXv; the result is returned by getdXs()."""
        if solverVec:
            dXvWarp = self._solverToWarp(dXv)
        else:
            dXvWarp = dXv
        if isinstance(dXvWarp, np.ndarray) or not hasattr(dXvWarp, "data_ptr"):
            dXvWarp = np.ascontiguousarray(dXvWarp, dtype=np.float64).ravel()
        ptr, where = _lib.vptr(dXvWarp)
        n = dXvWarp.size if isinstance(dXvWarp, np.ndarray) else dXvWarp.numel()
        self._chk(self.lib.idw_warp_deriv(self.ctx, ptr, n, where), "warpDeriv")

    def warpDerivFwd(self, dXs, solverVec=True):
        """Forward-mode product dXv = (dXv/dXs) dXs (idwarp/UnstructuredMesh.py:428-459).

        dXs has the shape of getSurfaceCoordinates(); returns dXv in solver
        ordering (solverVec=True) or warp ordering, flat.  Like the reference,
        the mesh is warped first."""
        dXs = np.ascontiguousarray(np.asarray(dXs, dtype=np.float64).ravel())
        if dXs.size != 3 * self.nSurf:
            raise Error("dXs has %d entries, expected %d" % (dXs.size, 3 * self.nSurf))
        dXvWarp = np.zeros(3 * self.nVol, np.float64)
        self.warpMesh()
        self._chk(self.lib.idw_warp_deriv_fwd(self.ctx, C.c_void_p(dXs.ctypes.data), dXs.size,
                                              C.c_void_p(dXvWarp.ctypes.data), dXvWarp.size, _lib.IDW_HOST),
                  "warpDerivFwd")
        if solverVec:
            if self.solverMeshDOF is None:
                raise Error("setExternalMeshIndices() must be called before warpDerivFwd(solverVec=True).")
            dXv = np.zeros(self.solverMeshDOF, np.float64)
            self._chk(self.lib.idw_warp_to_solver_grid(self.ctx, C.c_void_p(dXvWarp.ctypes.data), dXvWarp.size,
                                                       C.c_void_p(dXv.ctypes.data), dXv.size, _lib.IDW_HOST),
                      "warp_to_solver_grid")
            return dXv
        return dXvWarp

    def verifyWarpDeriv(self, dXv=None, solverVec=True, dofStart=0, dofEnd=10, h=1e-6, randomSeed=314):
        """Compare warpDeriv with central differences on a few surface DOFs (src/warp/verifyWarpDeriv.F90)."""
        if dXv is None:
            np.random.seed(randomSeed)
            dXvWarp = np.random.random(3 * self.nVol)
        else:
            dXvWarp = self._solverToWarp(dXv) if solverVec else np.asarray(dXv, dtype=np.float64).ravel()
        nDof = 3 * self.nSurf
        dofStart = max(0, min(dofStart, nDof - 1))
        dofEnd = min(nDof - 1, max(dofEnd, 0))
        print(" Welcome to verifyWarpDeriv")
        print(" Checking ", dofEnd - dofStart, " degrees of freedom")
        print(" Doing centered differnce with h:", h)
        self.warpMesh()
        self.warpDeriv(dXvWarp, solverVec=False)
        ad = self.getdXs().ravel()
        xs0 = self.getSurfaceCoordinates().ravel().copy()
        results = []
        for dof in range(dofStart, dofEnd + 1):
            x = xs0.copy()
            x[dof] += h
            self.setSurfaceCoordinates(x.reshape(-1, 3))
            self.warpMesh()
            xp = self.getWarpGrid()
            x[dof] = xs0[dof] - h
            self.setSurfaceCoordinates(x.reshape(-1, 3))
            self.warpMesh()
            xm = self.getWarpGrid()
            fd = float(np.dot(dXvWarp, (xp - xm) / (2.0 * h)))
            a = float(ad[dof])
            err = 1e-16 if abs(0.5 * (fd + a)) < 1e-16 else (fd - a) / (0.5 * (fd + a)) * 100.0
            print("DOF:%5d OrigVal: %19.12g AD: %19.12g FD: %19.12g Err(%%): %17.10g" % (dof, xs0[dof], a, fd, err))
            results.append((dof, a, fd, err))
        self.setSurfaceCoordinates(xs0.reshape(-1, 3))
        self.warpMesh()
        return results

    # GB300 extensions ---------------------------------------------------
    def warpMeshBatch(self, coords):
        """Warp B surfaces (B, nSurf, 3) in one call; returns (B, nVol, 3)."""
        coords = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, self.nSurf, 3)
        out = np.zeros((coords.shape[0], self.nVol, 3))
        self._setMeshOptions()
        self._chk(self.lib.idw_warp_mesh_batch(self.ctx, C.c_void_p(coords.ctypes.data), coords.shape[0],
                                                 C.c_void_p(out.ctypes.data), _lib.IDW_HOST), "warpMeshBatch")
        return out

    def warpDerivFwdBatch(self, dXs):
        """Tangent products for several directions at the current surface (a
        prior warpMesh is needed): dXs (D, nSurf, 3) -> dXv (D, nVol, 3) in
        warp order."""
        dXs = np.ascontiguousarray(dXs, dtype=np.float64).reshape(-1, self.nSurf, 3)
        out = np.zeros((dXs.shape[0], self.nVol, 3))
        self._chk(self.lib.idw_warp_deriv_fwd_batch(self.ctx, C.c_void_p(dXs.ctypes.data), dXs.shape[0],
                                                    C.c_void_p(out.ctypes.data), _lib.IDW_HOST), "warpDerivFwdBatch")
        return out

    def warpDerivBatch(self, dXv):
        """S reverse products at once: dXv (S, nVol, 3) in warp order -> dXs (S, nSurf, 3)."""
        dXv = np.ascontiguousarray(dXv, dtype=np.float64).reshape(-1, self.nVol, 3)
        out = np.zeros((dXv.shape[0], self.nSurf, 3))
        self._chk(self.lib.idw_warp_deriv_batch(self.ctx, C.c_void_p(dXv.ctypes.data), dXv.shape[0],
                                                  C.c_void_p(out.ctypes.data), _lib.IDW_HOST), "warpDerivBatch")
        return out

    def autotune(self, nSurfaces=8, nSeeds=16):
        """Time the mixed form's run-time launch shapes (surfaces per batched
        walk, seeds per adjoint walk) on this mesh and keep the fastest.
        Warps the current surface first."""
        self.warpMesh()
        t = _lib.idw_tuning()
        self._chk(self.lib.idw_autotune(self.ctx, int(nSurfaces), int(nSeeds), C.byref(t)), "autotune")
        return t.as_dict()

    def getStats(self):
        """Work counters of the last warp/derivative call."""
        s = _lib.idw_stats()
        self._chk(self.lib.idw_get_stats(self.ctx, C.byref(s)), "getStats")
        return s.as_dict()

    def getDenominator0(self):
        out = np.zeros(self.nVol)
        self._chk(self.lib.idw_get_denominator0(self.ctx, C.c_void_p(out.ctypes.data), self.nVol, _lib.IDW_HOST),
                    "getDenominator0")
        return out

    def getDenominator(self):
        """sum(w) per volume node from the last warpMesh (used by warpDeriv)."""
        out = np.zeros(self.nVol)
        self._chk(self.lib.idw_get_denominator(self.ctx, C.c_void_p(out.ctypes.data), self.nVol, _lib.IDW_HOST),
                  "getDenominator")
        return out

    def getTree(self):
        """Tree arrays (preorder nodes): l, u, escape, isLeaf, X, oradius, err (12), Ai."""
        nn = self.getStats()["nTreeNodes"]
        info = np.zeros((nn, 4), np.int32)
        geom = np.zeros((nn, 4))
        err = np.zeros((nn, 12))
        ai = np.zeros(nn)
        self._chk(self.lib.idw_get_tree(self.ctx, _lib.iptr(info), _lib.dptr(geom), _lib.dptr(err), _lib.dptr(ai)),
                    "getTree")
        return {"l": info[:, 0], "u": info[:, 1], "escape": info[:, 2], "isLeaf": info[:, 3], "X": geom[:, :3],
                "oradius": geom[:, 3], "err": err, "Ai": ai}

    def getSurfaceState(self):
        n = self.getStats()["nUnique"]
        xu0 = np.zeros((n, 3))
        ai = np.zeros(n)
        n0 = np.zeros((n, 3))
        ic = np.zeros(n, np.int32)
        xi = np.zeros(n, np.int32)
        self._chk(self.lib.idw_get_surface_state(self.ctx, _lib.dptr(xu0), _lib.dptr(ai), _lib.dptr(n0),
                                                   _lib.iptr(ic), _lib.iptr(xi)), "getSurfaceState")
        return {"Xu0": xu0, "Ai": ai, "normals0": n0, "isCorner": ic, "XuInd": xi}

    def getNodalProperties(self):
        n = self.getStats()["nUnique"]
        mi = np.zeros((n, 3, 3))
        bi = np.zeros((n, 3))
        self._chk(self.lib.idw_get_nodal_properties(self.ctx, _lib.dptr(mi), _lib.dptr(bi)), "getNodalProperties")
        return mi, bi

    # ------------------------------------------------------------------
    # output
    # ------------------------------------------------------------------
    def writeGrid(self, fileName=None):
        """Write the current grid: NPY (.npy of (N,3)) or PLOT3D (single block, unformatted)."""
        if fileName is None:
            raise Error("fileName is not optional for writeGrid")
        grid = self.getCommonGrid().reshape(-1, 3)
        if self.fileType == "PLOT3D":
            from .plot3d import writePlot3D

            writePlot3D(fileName, grid, getattr(self, "_plot3dShape", None))
        elif self.fileType == "NPY":
            np.save(fileName, grid)
        else:
            raise Error("writeGrid supports the NPY and PLOT3D file types in this build.")

    def writeOFGridTecplot(self, fileName):
        """OpenFOAM grids (idwarp/UnstructuredMesh.py writeOFGridTecplot) need pyofm, which this build does
        not use; write the grid with writeGrid (NPY or PLOT3D) instead."""
        raise Error("writeOFGridTecplot needs an OpenFOAM grid (pyofm), which this build does not read.")

    # ------------------------------------------------------------------
    # internals
    # ------------------------------------------------------------------
    def _solverToWarp(self, dXv):
        dXv = np.ascontiguousarray(dXv, dtype=np.float64).ravel()
        dXvWarp = np.zeros(3 * self.nVol, np.float64)
        self._chk(self.lib.idw_solver_to_warp_grid(self.ctx, C.c_void_p(dXv.ctypes.data), dXv.size,
                                                     C.c_void_p(dXvWarp.ctypes.data), dXvWarp.size, _lib.IDW_HOST),
                    "solver_to_warp_grid")
        return dXvWarp

    def _setInternalSurface(self):
        if self.warpInitialized:
            return
        raise Error(
            "No surface definition: call setSurfaceDefinition() (the CGNS boundary-condition surfaces that "
            "the reference extracts internally need libcgns)."
        )

    def _setSymmetryConditions(self):
        symmList = self.getOption("symmetryPlanes")
        pts, normals = [], []
        if symmList is not None:
            for plane in symmList:
                pts.append(plane[0])
                normals.append(plane[1])
        normals = np.array(self.comm.bcast(np.array(normals, dtype=np.float64).reshape(-1, 3)))
        pts = np.array(self.comm.bcast(np.array(pts, dtype=np.float64).reshape(-1, 3)))
        if self.comm.rank == 0 and len(pts):
            print("+-------------------- Symmetry Planes -------------------+")
            print("|           Point                        Normal          |")
            for i in range(len(pts)):
                print("| (%7.3f %7.3f %7.3f)    (%7.3f %7.3f %7.3f) |" % (
                    pts[i][0], pts[i][1], pts[i][2], normals[i][0], normals[i][1], normals[i][2]))
            print("+--------------------------------------------------------+")
        pts = np.ascontiguousarray(pts)
        normals = np.ascontiguousarray(normals)
        self._chk(self.lib.idw_set_symmetry_planes(self.ctx, _lib.dptr(pts), _lib.dptr(normals), len(pts)),
                    "setSymmetryPlanes")

    def _fill_options(self, o):
        o.aExp = self.getOption("aExp")
        o.bExp = self.getOption("bExp")
        o.LdefFact = self.getOption("LdefFact")
        o.alpha = self.getOption("alpha")
        o.errTol = self.getOption("errTol")
        o.symmTol = self.getOption("symmTol")
        o.cornerAngle = self.getOption("cornerAngle")
        o.useRotations = int(self.getOption("useRotations"))
        o.zeroCornerRotations = int(self.getOption("zeroCornerRotations"))
        o.bucketSize = self.getOption("bucketSize")
        o.evalMode = _lib.IDW_EVAL_FAST if self.getOption("evalMode") == "fast" else _lib.IDW_EVAL_EXACT
        o.precision = _lib.IDW_PREC_MIXED if self.getOption("precision") == "mixed" else _lib.IDW_PREC_FP64
        o.mixedGate = self.getOption("mixedGate")
        o.diagnostics = self.getOption("diagnostics")
        o.exactSchedule = {"auto": 0, "tiled": 1, "walk": 2}[self.getOption("exactSchedule")]
        o.adjointPrecision = {"precise": _lib.IDW_ADJ_PRECISE, "fast": _lib.IDW_ADJ_FAST}[self.getOption("adjointPrecision")]
        o.walkLists = {"auto": _lib.IDW_WALK_LISTS_AUTO, "off": _lib.IDW_WALK_LISTS_OFF}[self.getOption("walkLists")]
        o.treeBuild = {"kd": _lib.IDW_TREE_KD, "morton": _lib.IDW_TREE_MORTON}[self.getOption("treeBuild")]
        o.deterministic = int(self.getOption("deterministic"))

    def _setMeshOptions(self):
        """Push the current options to the library (idwarp/UnstructuredMesh.py:1051-1069)."""
        o = _lib.idw_options()
        self.lib.idw_default_options(C.byref(o))
        self._fill_options(o)
        self._chk(self.lib.idw_set_options(self.ctx, C.byref(o)), "setOptions")

    def _chk(self, rc, what):
        _lib.check(self.lib, self.ctx, rc, what)

    def __del__(self):
        try:
            if getattr(self, "ctx", None):
                self.lib.idw_destroy(self.ctx)
                self.ctx = None
        except Exception:
            pass


def pointReduce(pts, tol=1e-12, lib=None):
    """Merge duplicate points: returns (uniquePts, link (1-based), nUnique) (src/utils/pointReduce.F90)."""
    L = lib or _lib.load()
    pts = np.ascontiguousarray(np.asarray(pts, dtype=np.float64).reshape(-1, 3))
    n = len(pts)
    uniq = np.zeros((max(n, 1), 3))
    link = np.zeros(max(n, 1), np.int32)
    nu = C.c_int32(0)
    rc = L.idw_point_reduce(_lib.dptr(pts), n, tol, _lib.dptr(uniq), _lib.iptr(link), C.byref(nu))
    if rc != 0:
        raise Error("pointReduce failed with status %d" % rc)
    return uniq[: nu.value].copy(), link[:n].copy(), nu.value
