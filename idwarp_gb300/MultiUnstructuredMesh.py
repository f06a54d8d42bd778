"""MultiUSMesh: independent warping of several component meshes (overset).

Drop-in for ``idwarp.MultiUSMesh`` (idwarp/MultiUnstructuredMesh.py:47-892)
without the CGNS layer.  The reference reads one combined CGNS file, groups
its domains by name (one IDWarp instance per group) and leaves the groups
without options as a fixed background.  Here the combined grid is either

* a multi-block PLOT3D file (the reference's constructor shape,
  ``MultiUSMesh(gridFile, optionsDict, comm)``) whose blocks carry names in
  the cgns_utils combine convention ``<zone>.<index>`` (``blockNames``, or one
  name per line in ``<gridFile>.names``); consecutive blocks of one zone form
  a group, as the reference's explodeByZoneName does; or
* an ordered list of ``(name, volNodes, nBlocks)`` groups: ``volNodes``
  (N, 3) are the group's nodes in combined order and ``nBlocks`` the number
  of blocks it spans.

Surface elements are routed to the groups by block ID exactly as the
reference does (:462-597).  Each warped group is a
:class:`~idwarp_gb300.USMesh` on the GPU.
"""
import os

import numpy as np

from .options import Error
from .UnstructuredMesh import USMesh


class MultiUSMesh:
    """Several IDWarp instances behind one solver-facing interface."""

    def __init__(self, grids, optionsDict, comm=None, dtype="d", debug=False, blockNames=None):
        if optionsDict is None:
            raise Error("optionsDict is not optional: one options dictionary per warped group.")
        if isinstance(grids, (str, os.PathLike)):
            grids = zone_groups_from_plot3d(grids, blockNames)
        self.comm = comm
        self.dtype = dtype
        self.meshes = []
        self.names = []
        self.cgnsBlockIntervals = []
        self.cgnsVolNodeIntervals = []  # in coordinates (3 per node) of the combined grid
        self.backgroundNodes = []
        self.backgroundIntervals = []
        blocks = 0
        coords = 0
        for name, volNodes, nBlocks in grids:
            x = np.ascontiguousarray(np.asarray(volNodes, dtype=np.float64).reshape(-1, 3))
            interval = [coords, coords + x.size]
            if name in optionsDict:
                opts = dict(optionsDict[name])
                opts.setdefault("fileType", "NPY")
                mesh = USMesh(options=opts, comm=comm, debug=debug)
                mesh.createCommonGrid(x)
                self.meshes.append(mesh)
                self.names.append(name)
                self.cgnsBlockIntervals.append([blocks, blocks + int(nBlocks)])
                self.cgnsVolNodeIntervals.append(interval)
            else:
                self.backgroundNodes.append(x.ravel())
                self.backgroundIntervals.append(interval)
            blocks += int(nBlocks)
            coords += x.size
        self.numCoorTotal = coords
        self.numSurfNodes = None
        self.numVolNodes = None
        self.cgnsVolNodeMasks = []
        self.filtered2fullMaps = []
        self.defaultSolverGrid = None

    # ------------------------------------------------------------------
    def setExternalMeshIndices(self, ind):
        """Solver ordering: 0-based coordinate indices into the combined grid
        (MultiUnstructuredMesh.py:345-432).  Must come before
        setSurfaceDefinition, as in the reference."""
        ind = np.asarray(ind).ravel()
        self.numVolNodes = len(ind)
        self.defaultSolverGrid = np.zeros(self.numVolNodes, dtype=self.dtype)
        for (start, end), nodes in zip(self.backgroundIntervals, self.backgroundNodes):
            mask = (ind >= start) & (ind < end)
            self.defaultSolverGrid[mask] = nodes[ind[mask] - start]
        self.cgnsVolNodeMasks = []
        for mesh, (start, end) in zip(self.meshes, self.cgnsVolNodeIntervals):
            mask = (ind >= start) & (ind < end)
            self.cgnsVolNodeMasks.append(mask)
            mesh.setExternalMeshIndices(ind[mask] - start)

    def getSolverGrid(self):
        if self.defaultSolverGrid is None:
            raise Error("setExternalMeshIndices must be called before getSolverGrid.")
        solverGrid = self.defaultSolverGrid.copy()
        for mesh, mask in zip(self.meshes, self.cgnsVolNodeMasks):
            solverGrid[mask] = mesh.getSolverGrid()
        return solverGrid

    def setSurfaceDefinition(self, pts, conn=None, faceSizes=None, cgnsBlockIDs=None, distTol=1e-6):
        """Route every surface element to the instance owning its block
        (MultiUnstructuredMesh.py:462-597) and define each instance's surface
        from its elements only."""
        if self.defaultSolverGrid is None:
            raise Error("The user should run self.setExternalMeshIndices before self.setSurfaceDefinition.")
        pts = np.asarray(pts, dtype=np.float64).reshape(-1, 3)
        conn = np.asarray(conn).ravel()
        faceSizes = np.asarray(faceSizes).ravel()
        cgnsBlockIDs = np.asarray(cgnsBlockIDs).ravel()
        if len(cgnsBlockIDs) != len(faceSizes):
            raise ValueError("The user should provide block IDs for every element.")
        self.numSurfNodes = pts.shape[0]
        instanceIDs = np.full(len(faceSizes), -1)
        for ii, (start, end) in enumerate(self.cgnsBlockIntervals):
            instanceIDs[(cgnsBlockIDs >= start) & (cgnsBlockIDs < end)] = ii
        offsets = np.concatenate([[0], np.cumsum(faceSizes)])
        self.filtered2fullMaps = []
        for ii, mesh in enumerate(self.meshes):
            elems = np.nonzero(instanceIDs == ii)[0]
            currFaceSizes = faceSizes[elems].astype(np.intc)
            currConn = (np.concatenate([conn[offsets[e]:offsets[e + 1]] for e in elems])
                        if len(elems) else np.zeros(0, dtype=np.intc))
            filtered2full = np.unique(currConn)
            local = np.searchsorted(filtered2full, currConn).astype(np.intc)
            mesh.setSurfaceDefinition(pts[filtered2full], local, currFaceSizes)
            self.filtered2fullMaps.append(filtered2full)

    def _need_surface(self):
        if self.numSurfNodes is None:
            raise Error("IDWarpMulti surface is not initialized. Run self.setSurfaceDefinition first.")

    def getSurfaceCoordinates(self):
        self._need_surface()
        pts = np.zeros((self.numSurfNodes, 3), dtype=self.dtype)
        for mesh, f2f in zip(self.meshes, self.filtered2fullMaps):
            pts[f2f, :] = mesh.getSurfaceCoordinates()
        return pts

    def setSurfaceCoordinates(self, pts):
        self._need_surface()
        pts = np.asarray(pts)
        for mesh, f2f in zip(self.meshes, self.filtered2fullMaps):
            mesh.setSurfaceCoordinates(pts[f2f, :])

    def getWarpGrid(self):
        """(list of the instances' flat grids, total coordinates of all instances)."""
        grids = [mesh.getCommonGrid() for mesh in self.meshes]
        return grids, int(sum(len(g) for g in grids))

    def getdXs(self):
        self._need_surface()
        dXs = np.zeros((self.numSurfNodes, 3), dtype=self.dtype)
        for mesh, f2f in zip(self.meshes, self.filtered2fullMaps):
            dXs[f2f] = dXs[f2f] + mesh.getdXs()
        return dXs

    def warpMesh(self):
        for mesh in self.meshes:
            mesh.warpMesh()

    def warpDeriv(self, dXv, solverVec=True):
        """dXv in solver ordering (solverVec) -> dXs of the whole surface."""
        dXv = np.asarray(dXv).ravel()
        for mesh, mask in zip(self.meshes, self.cgnsVolNodeMasks):
            mesh.warpDeriv(dXv[mask], solverVec=solverVec)
        return self.getdXs()

    def warpDerivFwd(self, dXs):
        """dXs of the whole surface -> dXv in solver ordering."""
        dXs = np.asarray(dXs).reshape(-1, 3)
        dXv = np.zeros(self.numVolNodes, dtype=self.dtype)
        for mesh, mask, f2f in zip(self.meshes, self.cgnsVolNodeMasks, self.filtered2fullMaps):
            dXv[mask] = mesh.warpDerivFwd(dXs[f2f])
        return dXv

    def writeGrid(self, baseName=None):
        """One NPY grid per instance: <baseName>_<name>.npy."""
        if baseName is None:
            raise Error("baseName is not optional for writeGrid")
        for name, mesh in zip(self.names, self.meshes):
            np.save("%s_%s.npy" % (baseName, name), mesh.getCommonGrid().reshape(-1, 3))

    def __del__(self):
        """Release the instances' device memory (MultiUnstructuredMesh.py:887-892):
        each USMesh destroys its context."""
        for mesh in getattr(self, "meshes", []):
            release = getattr(mesh, "__del__", None)
            if release is not None:
                try:
                    release()
                except Exception:
                    pass
        self.meshes = []


def zone_groups_from_plot3d(gridFile, blockNames=None):
    """(name, volNodes, nBlocks) groups of a multi-block PLOT3D grid: blocks
    named ``<zone>.<index>`` (cgns_utils combine), or plain zone names,
    grouped by zone in file order; ``blockNames`` defaults to the lines of
    ``<gridFile>.names``."""
    from .plot3d import readPlot3D

    nodes, sizes = readPlot3D(os.fspath(gridFile), return_blocks=True)
    if blockNames is None:
        sidecar = os.fspath(gridFile) + ".names"
        if not os.path.exists(sidecar):
            raise Error("MultiUSMesh needs the block names of %s: pass blockNames or write one name per block in %s"
                        % (gridFile, sidecar))
        with open(sidecar) as f:
            blockNames = [ln.strip() for ln in f if ln.strip()]
    if len(blockNames) != len(sizes):
        raise Error("%d block names for %d blocks in %s" % (len(blockNames), len(sizes), gridFile))
    counts = [int(a) * int(b) * int(c) for a, b, c in sizes]
    groups = []
    off = 0
    for name, n in zip(blockNames, counts):
        zone = name.rsplit(".", 1)[0] if "." in name else name
        if groups and groups[-1][0] == zone:
            groups[-1][1].append(nodes[off:off + n])
            groups[-1][2] += 1
        else:
            if any(g[0] == zone for g in groups):
                raise Error("the blocks of zone %r are not consecutive in %s" % (zone, gridFile))
            groups.append([zone, [nodes[off:off + n]], 1])
        off += n
    return [(zone, np.concatenate(parts), nb) for zone, parts, nb in groups]
