"""Build the native library ``libidwarp_gb300.so`` in-tree with nvcc (sm_103a).

Every translation unit is compiled in parallel, then linked into one shared
object under ``idwarp_gb300/_build``.  No cmake, no -march=native: the same
recipe runs on the x86_64 build host and on the aarch64 GPU host.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libidwarp_gb300.so")

SOURCES = ["idw_api.cu", "idw_walk.cu", "idw_mixed.cu", "idw_replay.cu", "idw_batch.cu", "idw_exact.cu", "idw_adjoint.cu", "idw_adjoint_precise.cu", "idw_nodal.cu", "idw_setup.cu",
           "idw_tree.cu", "idw_probe.cu", "idw_complex.cu", "idw_host.cpp"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else shutil.which("nvcc")


def _flags():
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
        "--expt-relaxed-constexpr", "-Xcompiler", "-pthread", "-I", CSRC, "-I", INCLUDE,
    ]


def _digest():
    h = hashlib.sha1()
    for name in sorted(os.listdir(CSRC)):
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode())
            h.update(f.read())
    with open(os.path.join(INCLUDE, "idwarp_gb300.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(_flags()).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force=False, verbose=False, jobs=None):
    """Compile (if stale) and return the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp.txt")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB
    nvcc = _nvcc()
    if nvcc is None:
        raise RuntimeError("nvcc not found: the idwarp_gb300 CUDA library cannot be built")
    objs = []
    cmds = []
    for src in SOURCES:
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [nvcc] + _flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc] + _flags() + ["-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
        cmds.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
        for msg in ex.map(run, cmds):
            if verbose and msg:
                print(msg)
    tmp = LIB + ".tmp"
    link = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"]
    run(link)
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
