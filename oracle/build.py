"""Build recipe for the oracle (test infrastructure only).

Compiles ``oracle/idw_oracle.cpp`` — the CPU FP64/complex restatement of the
IDWarp warping path — into ``oracle/_build/liboracle.so``.  No ``-march=native``
and no FMA contraction, so the restatement gives the same results on x86_64
and aarch64 hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "idw_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build_oracle(force=False, verbose=False):
    """Compile the oracle shared library if it is missing or stale."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = [
        "g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-fast-math",
        SRC, "-o", LIB + ".tmp",
    ]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_oracle_contracted():
    """The same source with FMA contraction (x86-64 with FMA only).  Not a
    second oracle: comparing the two measures how sensitive a case is to the
    rounding order of the reference formulas."""
    os.makedirs(OUT_DIR, exist_ok=True)
    out = os.path.join(OUT_DIR, "liboracle_fma.so")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
        return out
    flags = ["-ffp-contract=fast"] + (["-mfma"] if os.uname().machine == "x86_64" else [])
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp"] + flags + [SRC, "-o", out + ".tmp"],
                   check=True)
    os.replace(out + ".tmp", out)
    return out


def build_oracle_timing(force=False):
    """The timing build of the same source for the CPU baseline: -O3, tuned
    for the CPU it is built on (-mcpu=native on aarch64; built on the machine
    that runs it), FMA contraction allowed, OpenMP.  Its results differ from
    the checker build's by rounding only; it is never used as the checker."""
    os.makedirs(OUT_DIR, exist_ok=True)
    out = os.path.join(OUT_DIR, "liboracle_timing.so")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
        return out
    tune = ["-mcpu=native"] if os.uname().machine == "aarch64" else []
    subprocess.run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=fast"] + tune +
                   [SRC, "-o", out + ".tmp"], check=True)
    os.replace(out + ".tmp", out)
    return out


def timing_flags():
    """The compiler flags of the timing build (recorded beside its numbers)."""
    tune = ["-mcpu=native"] if os.uname().machine == "aarch64" else []
    return " ".join(["-O3", "-fopenmp", "-ffp-contract=fast"] + tune)


if __name__ == "__main__":
    print(build_oracle(force=True, verbose=True))
