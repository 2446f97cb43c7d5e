"""Build recipe for the CPU oracle (test infrastructure only).

Two shared libraries are built from mflbm_oracle.cpp into oracle/_build/:

  liborc_strict.so  -O2 -ffp-contract=off  : the parity oracle.  Every expression is
                    evaluated in the written order with no FMA contraction.
  liborc_fast.so    -O3 -ffp-contract=fast : the timed CPU baseline (same algorithm,
                    compiler free to contract multiply-adds).

Both use OpenMP over z slices; the result does not depend on the thread count because
every lattice node is updated independently (AA pattern) and the reductions are
sequential.  No machine-specific flags are used, so the same recipe builds on x86_64
and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "mflbm_oracle.cpp")
HEADER = os.path.join(HERE, "..", "include", "mflbm.h")

VARIANTS = {
    "liborc_strict.so": ["-O2", "-ffp-contract=off", "-fno-fast-math"],
    "liborc_fast.so": ["-O3", "-ffp-contract=fast", "-fno-fast-math"],
}


def lib_path(name="liborc_strict.so"):
    return os.path.join(OUT, name)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    procs = []
    for name, flags in VARIANTS.items():
        out = os.path.join(OUT, name)
        newest = max(os.path.getmtime(SRC), os.path.getmtime(HEADER))
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        cmd = ["g++", "-std=c++17", "-shared", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function",
               *flags, SRC, "-o", out + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), out))
    for p, out in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {out}")
        os.replace(out + ".tmp", out)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
