"""Build recipe for oracle/_build/liboracle.so -- TEST INFRASTRUCTURE ONLY.

Plain C11, OpenMP, -O2 -ffp-contract=off (no implicit contraction: the only
fused multiply-adds are the explicit fmaf/fma calls), portable flags only so
that the same source gives the same results on x86-64 and aarch64.

build(fast=True) makes oracle/_build/liboracle_fast.so from the same sources
with -O3 -ffast-math -funroll-loops (contraction and reassociation allowed,
like the reference's own -Ofast): the CPU baseline is timed with it, never
compared bit for bit.  No -march=native: the flags stay the same on every
host, and the aarch64 default target already vectorises with NEON.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "liboracle.so")
OUT_FAST = os.path.join(OUT_DIR, "liboracle_fast.so")
SRCS = [os.path.join(HERE, "ubg_oracle.c"), os.path.join(HERE, "ubg_oracle_impl.h"),
        os.path.join(HERE, "ubg_tracers_oracle.c")]


def build(force: bool = False, fast: bool = False) -> str:
    out = OUT_FAST if fast else OUT
    srcs = [s for s in SRCS if os.path.exists(s)]
    if (not force and os.path.exists(out)
            and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs)):
        return out
    os.makedirs(OUT_DIR, exist_ok=True)
    csrcs = [s for s in srcs if s.endswith(".c")]
    tmp = out + ".tmp%d" % os.getpid()
    opt = (["-O3", "-ffast-math", "-funroll-loops"] if fast
           else ["-O2", "-ffp-contract=off", "-fno-fast-math"])
    cmd = ["gcc", "-std=c11", *opt, "-fopenmp", "-fPIC", "-shared", "-Wall", *csrcs, "-o", tmp,
           "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build(force="--force" in sys.argv, fast=True))
