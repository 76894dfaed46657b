"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/yv_oracle.c and oracle/yv_oracle_build.c into
oracle/liboracle.so with gcc.  The oracle
is the checker for the CUDA path and the timed CPU baseline; the product
library never links or loads it.  -ffp-contract=off keeps one IEEE rounding
per written float operation (no fused multiply-add), which is what makes
the float instantiation bit-comparable with the CUDA kernels.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "yv_oracle.c"), os.path.join(HERE, "yv_oracle_build.c")]
OUT = os.path.join(HERE, "liboracle.so")
DEPS = SRCS + [os.path.join(HERE, "yv_oracle_impl.h"), os.path.join(HERE, "yv_oracle.h")]


def build(force=False, verbose=False):
    """Compile liboracle.so if missing or older than its sources."""
    if not force and os.path.exists(OUT):
        t = os.path.getmtime(OUT)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return OUT
    cmd = ["gcc", "-std=c11", "-O3", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-pthread", "-Wall", "-Wno-unused-function",
           *SRCS, "-o", OUT + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(OUT)
