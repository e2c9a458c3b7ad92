"""The C++ drop-in header (ubootgl_gb300/simulation.hpp): a caller written
against the reference's Simulation / MG / Single2DGrid compiles against it
(CPU test), and on a GPU its steps and MG::solve are bit-identical to the
CPU restatement of the reference (tolerance 0)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "drop_in.cpp")


def build_exe(tmp):
    from ubootgl_gb300 import build as B
    lib = B.build()
    libdir = os.path.dirname(lib)
    exe = os.path.join(tmp, "drop_in")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "ubootgl_gb300"), SRC,
           "-L", libdir, "-lubootgl_gb300", "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ absent")
def test_drop_in_compiles(tmp_path):
    assert os.path.exists(build_exe(str(tmp_path)))


@pytest.mark.gpu
def test_drop_in_steps_bit_exact(tmp_path):
    d = str(tmp_path)
    exe = build_exe(d)
    W, H, n = 130, 66, 4
    flag = WL.disc_flag(W, H, n_discs=5, seed=21)
    vx, vy = WL.initial_velocity(flag, seed=22)
    ref = O.PortSim(flag, 1.0, 1e-4)
    for k, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        ref.set(k, a)
    dts = []
    for _ in range(n):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        ref.step(dt)
        dts.append(dt)
    rng = np.random.default_rng(3)
    mp = rng.standard_normal((H, W)).astype(np.float32)
    mf = rng.standard_normal((H, W)).astype(np.float32)
    with open(os.path.join(d, "meta.txt"), "w") as f:
        f.write("%d %d %d\n" % (W, H, n))
    for k, a in (("flag", flag), ("vx", vx), ("vy", vy), ("dts", np.array(dts, np.float32)),
                 ("mg_p", mp), ("mg_f", mf)):
        np.ascontiguousarray(a, np.float32).tofile(os.path.join(d, k + ".bin"))
    subprocess.run([exe, d], check=True)
    for k, shape in (("vx", (H, W - 1)), ("vy", (H - 1, W)), ("p", (H, W))):
        out = np.fromfile(os.path.join(d, "out_%s.bin" % k), np.float32).reshape(shape)
        assert np.array_equal(out, ref.get(k)), k
    want = O.port_mg_solve(mp, mf, flag, np.float32(ref.h), zgbc=True, coarse_flag=flag)
    got = np.fromfile(os.path.join(d, "out_mg_p.bin"), np.float32).reshape(H, W)
    assert np.array_equal(got, want)
