"""Build recipe for oracle/_ref/libubgref.so -- TEST INFRASTRUCTURE ONLY.

Compiles the reference's own simulation.cpp and pressure_solver.cpp
(te42kyfo/ubootgl) straight from the read-only reference checkout, with the
reference's own flags (Makefile:12: -std=c++17 -fopenmp -Ofast -march=native
-DNDEBUG), plus ref_capi.cpp.  The shim/ directory supplies a minimal GLM
subset and a declaration-only GL header, because neither library is
installed; no reference source is copied or edited.

The reference uses x86 AVX2 intrinsics (interpolators.hpp, simulation.cpp),
so this builds on x86-64 only.  Outputs go to oracle/_ref/ (git-ignored).
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
OUT = os.path.join(OUT_DIR, "libubgref.so")
# the reference checkout: UBG_REFERENCE_ROOT, else a directory "reference"
# beside the repository
REF_ROOT = os.environ.get("UBG_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(ORACLE)), "reference"))


def available() -> bool:
    return (platform.machine() in ("x86_64", "AMD64")
            and os.path.isfile(os.path.join(REF_ROOT, "simulation.cpp")))


def build(force: bool = False) -> str:
    if not available():
        raise RuntimeError("reference sources absent or not an x86-64 host")
    srcs = [os.path.join(REF_ROOT, "simulation.cpp"),
            os.path.join(REF_ROOT, "pressure_solver.cpp"),
            os.path.join(HERE, "ref_capi.cpp")]
    if (not force and os.path.exists(OUT)
            and all(os.path.getmtime(OUT) >= os.path.getmtime(s) for s in srcs)):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-fopenmp", "-Ofast", "-march=native", "-DNDEBUG",
           "-DGLM_ENABLE_EXPERIMENTAL", "-w", "-fPIC", "-shared",
           "-I", os.path.join(HERE, "shim"), "-I", REF_ROOT,
           "-I", os.path.join(REF_ROOT, "external"),
           *srcs, "-o", OUT]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
