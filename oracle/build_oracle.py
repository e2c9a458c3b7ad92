"""Build recipe for oracle/_build/liboracle.so -- TEST INFRASTRUCTURE ONLY.

Plain C11, OpenMP, -O2 -ffp-contract=off (no implicit contraction: the only
fused multiply-adds are the explicit fmaf/fma calls), portable flags only so
that the same source gives the same results on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "liboracle.so")
SRCS = [os.path.join(HERE, "ubg_oracle.c"), os.path.join(HERE, "ubg_oracle_impl.h"),
        os.path.join(HERE, "ubg_tracers_oracle.c")]


def build(force: bool = False) -> str:
    srcs = [s for s in SRCS if os.path.exists(s)]
    if (not force and os.path.exists(OUT)
            and all(os.path.getmtime(OUT) >= os.path.getmtime(s) for s in srcs)):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    csrcs = [s for s in srcs if s.endswith(".c")]
    tmp = OUT + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-Wall", *csrcs, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
