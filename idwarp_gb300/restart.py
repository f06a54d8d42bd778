"""Restart file of the denominator estimate (src/warp/initializeWarping.F90:98-312).

The reference writes it with MPI-IO in native representation, no record
markers: one int32 ``nVol``, then ``nVol`` float64 ``denominator0``, then
``nVol`` float64 load-balancing costs (the dryRun cost of each node summed over
the mirrors, divided by the number of unique surface points), both in the
common (grid-file) order of the volume nodes.  The same bytes are read and
written here, so a file made by either side loads in the other.

``load_or_compute`` follows the reference's decisions:

* no file: compute, then save;
* a file whose node count differs: delete it, compute, save;
* otherwise load it and re-estimate every 100th node; if one has
  ``1 - estimate / loaded > 1e-15`` the file is "not accurate": delete it,
  compute, save.  Otherwise the loaded estimate is used as it is.
"""
import os

import numpy as np

CHECK_STRIDE = 100  # initializeWarping.F90:197 (j = 1, nVol, 100)


def read_restart(path):
    """``(nVol, den0, costs)`` of a restart file, or None when there is no file.
    ``den0`` and ``costs`` are None when the file is shorter than its count
    says (a file to recompute)."""
    if not os.path.exists(path):
        return None
    with open(path, "rb") as f:
        raw = f.read()
    if len(raw) < 4:
        return -1, None, None
    n = int(np.frombuffer(raw, dtype=np.int32, count=1)[0])
    if n < 0 or len(raw) < 4 + 16 * n:
        return n, None, None
    den0 = np.frombuffer(raw, dtype=np.float64, count=n, offset=4).copy()
    costs = np.frombuffer(raw, dtype=np.float64, count=n, offset=4 + 8 * n).copy()
    return n, den0, costs


def write_restart(path, den0, costs):
    den0 = np.ascontiguousarray(den0, dtype=np.float64).ravel()
    costs = np.ascontiguousarray(costs, dtype=np.float64).ravel()
    if den0.size != costs.size:
        raise ValueError("denominator0 and costs differ in length")
    with open(path, "wb") as f:
        f.write(np.int32(den0.size).tobytes())
        f.write(den0.tobytes())
        f.write(costs.tobytes())


def _delete(path):
    try:
        os.remove(path)
    except OSError:
        pass


def load_or_compute(path, nVol, load, compute, save, log=print):
    """Restart-file flow of initializeWarping.F90:98-312.

    ``load(den0)`` installs a loaded estimate and returns False when its check
    fails; ``compute()`` computes the estimate; ``save()`` returns
    ``(den0, costs)`` to write.  Returns "loaded" or "computed"."""
    rec = read_restart(path)
    if rec is not None:
        log("Loading restart file...")
        n, den0, _ = rec
        if n != nVol or den0 is None:
            log("Number of points in restart file are different...")
            _delete(path)
        else:
            log("Checking restart file...")
            if load(den0):
                return "loaded"
            log("Restart file not accurate...")
            _delete(path)
    log("Computing Denominator Estimate...")
    compute()
    log("Saving restart file...")
    write_restart(path, *save())
    return "computed"
