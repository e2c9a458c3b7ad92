"""Live comparison of the CPU restatement with the reference's own code.

Runs only where the reference builds (x86-64 with the reference checkout;
oracle/ref/build_ref.py).  Tolerances as in test_oracle_golden.py.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference not buildable here")

STEP_TOL = 5e-5


def pair(W, H, seed, ndisc=12):
    flag = WL.disc_flag(W, H, n_discs=ndisc, seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1)
    port, ref = O.PortSim(flag), O.RefSim(flag)
    for s in (port, ref):
        for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
            s.set(n, a)
    return port, ref


def rel(a, b):
    return float(np.abs(a.astype(np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize("W,H,nsteps", [(1024, 512, 6), (257, 129, 8), (33, 17, 4)])
def test_steps(W, H, nsteps):
    """1024x512 is the reference's CPU-runnable configuration (12 discs)."""
    port, ref = pair(W, H, seed=W)
    for k in range(nsteps):
        dt = WL.cfl_dt(port.get("vx"), port.get("vy"), port.h)
        port.step(dt)
        ref.step(dt)
    for n in ("vx", "vy", "p"):
        assert rel(port.get(n), ref.get(n)) < STEP_TOL, n


def test_sinks_and_accumulated_velocity():
    W, H = 130, 66
    port, ref = pair(W, H, seed=7, ndisc=3)
    rng = np.random.default_rng(3)
    ax = (0.01 * rng.standard_normal((H, W - 1))).astype(np.float32)
    for s in (port, ref):
        s.set("vx_accum", ax)
        s.add_sink(0.3, 0.2, 5.0)
        s.add_sink(0.01, 0.01, 1.0)
    for k in range(3):
        dt = WL.cfl_dt(port.get("vx"), port.get("vy"), port.h)
        port.step(dt)
        ref.step(dt)
    for n in ("vx", "vy", "p", "f", "vx_accum"):
        assert rel(port.get(n), ref.get(n)) < STEP_TOL or np.abs(ref.get(n)).max() == 0, n
