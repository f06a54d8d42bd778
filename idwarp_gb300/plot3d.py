"""Multiblock PLOT3D grids: unformatted Fortran sequential records, no iblank.

Record layout as src/IO/readPlot3d.F90 / writePlot3d.F90 use it: one record
with the number of blocks (int32), one with the block sizes (int32, 3 per
block for volume grids, 2 for surface grids), then one record per block with
the X, Y and Z arrays in Fortran order (i fastest), float64.
"""
import struct

import numpy as np


def _read_record(f):
    head = f.read(4)
    if len(head) < 4:
        raise EOFError("truncated PLOT3D file")
    (n,) = struct.unpack("<i", head)
    data = f.read(n)
    (tail,) = struct.unpack("<i", f.read(4))
    if tail != n or len(data) != n:
        raise ValueError("corrupt PLOT3D record (marker %d vs %d)" % (n, tail))
    return data


def _write_record(f, payload):
    f.write(struct.pack("<i", len(payload)))
    f.write(payload)
    f.write(struct.pack("<i", len(payload)))


def readPlot3D(fileName, return_blocks=False):
    """Volume grid -> (N,3) nodes, blocks concatenated with i fastest (readPlot3d.F90:62-80)."""
    with open(fileName, "rb") as f:
        (nZones,) = struct.unpack("<i", _read_record(f))
        sizes = np.frombuffer(_read_record(f), dtype="<i4").reshape(nZones, 3)
        blocks = []
        for z in range(nZones):
            il, jl, kl = (int(v) for v in sizes[z])
            a = np.frombuffer(_read_record(f), dtype="<f8").reshape(3, kl, jl, il)
            blocks.append(np.stack([a[0].ravel(), a[1].ravel(), a[2].ravel()], axis=1))
    nodes = np.concatenate(blocks) if blocks else np.zeros((0, 3))
    if return_blocks:
        return nodes, sizes
    return nodes


def writePlot3D(fileName, nodes, sizes=None):
    """Write (N,3) nodes as a multiblock grid; sizes (nZones,3), default one (N,1,1) block."""
    nodes = np.asarray(nodes, dtype=np.float64).reshape(-1, 3)
    if sizes is None:
        sizes = np.array([[len(nodes), 1, 1]], dtype=np.int32)
    sizes = np.asarray(sizes, dtype=np.int32).reshape(-1, 3)
    with open(fileName, "wb") as f:
        _write_record(f, struct.pack("<i", len(sizes)))
        _write_record(f, sizes.astype("<i4").tobytes())
        off = 0
        for il, jl, kl in sizes:
            n = int(il) * int(jl) * int(kl)
            blk = nodes[off:off + n]
            off += n
            _write_record(f, np.ascontiguousarray(blk.T).astype("<f8").tobytes())


def readPlot3DSurface(fileName):
    """Surface grid -> (pts (N,3), conn (nQuads,4) 0-based) (readPlot3d.F90:164-262)."""
    with open(fileName, "rb") as f:
        (nZones,) = struct.unpack("<i", _read_record(f))
        sizes = np.frombuffer(_read_record(f), dtype="<i4").reshape(nZones, 2)
        pts, conn = [], []
        off = 0
        for z in range(nZones):
            il, jl = (int(v) for v in sizes[z])
            a = np.frombuffer(_read_record(f), dtype="<f8").reshape(3, jl, il)
            j, i = np.meshgrid(np.arange(jl - 1), np.arange(il - 1), indexing="ij")
            n1 = off + j * il + i
            conn.append(np.stack([n1, n1 + 1, n1 + il + 1, n1 + il], axis=-1).reshape(-1, 4))
            pts.append(np.stack([a[0].ravel(), a[1].ravel(), a[2].ravel()], axis=1))
            off += il * jl
    return np.concatenate(pts), np.concatenate(conn).astype(np.intc)


def writePlot3DSurface(fileName, blocks):
    """blocks: list of (jl, il, 3) structured surface patches."""
    with open(fileName, "wb") as f:
        _write_record(f, struct.pack("<i", len(blocks)))
        _write_record(f, np.array([[b.shape[1], b.shape[0]] for b in blocks], dtype="<i4").tobytes())
        for b in blocks:
            b = np.asarray(b, dtype=np.float64)
            _write_record(f, np.ascontiguousarray(np.moveaxis(b, -1, 0)).astype("<f8").tobytes())
