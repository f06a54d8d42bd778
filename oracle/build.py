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


if __name__ == "__main__":
    print(build_oracle(force=True, verbose=True))
