"""GPU parity of the game-side field access against the oracle.

bilinearScatter / bilinearVel (interpolators.hpp:11-40,
advect_floating_items.cpp:11-14, 116-120), Simulation::setGrids
(simulation.hpp:82-98), UbootGlApp::shiftMap (ubootgl_app.cpp:245-298) and
the session snapshot.  Integer and float work in the reference's order:
bit-exact, except overlapping scatters, whose atomic sums may be ordered
differently (tolerance 1e-6 relative, stated below).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def make_sim(W=130, H=66, seed=3, steps=2):
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(W, H, n_discs=5, seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1)
    sim = Simulation(flag, 1.0, 1e-4)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    for _ in range(steps):
        sim.step(WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h))
    return sim, flag


def test_sample_velocity_exact(lib):
    from ubootgl_gb300 import _lib as L
    sim, _ = make_sim()
    rng = np.random.default_rng(7)
    n = 500
    xy = np.empty((n, 2), np.float32)
    xy[:, 0] = rng.uniform(-3, sim.width + 3, n)
    xy[:, 1] = rng.uniform(-3, sim.height + 3, n)
    out = np.empty((n, 2), np.float32)
    L.check(lib.ubg_sample_velocity(sim._h, n, fp(xy), fp(out)))
    vx, vy = sim.get("vx"), sim.get("vy")
    ref = np.array([O.bilinear_vel(vx, vy, x, y) for x, y in xy], np.float32)
    assert np.array_equal(out, ref)
    sim.close()


def test_scatter_accum_disjoint_exact(lib):
    """Items whose 2x2 stencils do not overlap: bit-identical to the
    sequential reference loop."""
    from ubootgl_gb300 import _lib as L
    sim, _ = make_sim()
    W, H = sim.width, sim.height
    rng = np.random.default_rng(11)
    pts = []
    for gy in range(4, H - 4, 5):
        for gx in range(4, W - 4, 5):
            pts.append((gx + rng.uniform(0.6, 1.4), gy + rng.uniform(0.6, 1.4)))
    xy = np.array(pts, np.float32)
    v = rng.standard_normal(xy.shape).astype(np.float32)
    ax0 = rng.standard_normal((H, W - 1)).astype(np.float32)
    ay0 = rng.standard_normal((H - 1, W)).astype(np.float32)
    sim.set("vx_accum", ax0)
    sim.set("vy_accum", ay0)
    L.check(lib.ubg_scatter_accum(sim._h, len(xy), fp(xy), fp(v)))
    ax, ay = ax0.copy(), ay0.copy()
    O.scatter_items(ax, ay, xy, v)
    assert np.array_equal(sim.get("vx_accum"), ax)
    assert np.array_equal(sim.get("vy_accum"), ay)
    sim.close()


def test_scatter_accum_overlapping_and_applied(lib):
    """Overlapping items (atomic sums, |diff| <= 1e-6 * sum of |terms|), and
    the next step applies and clears the accumulation
    (applyAccumulatedVelocity, simulation.cpp:376-396)."""
    from ubootgl_gb300 import _lib as L
    sim, _ = make_sim()
    W, H = sim.width, sim.height
    rng = np.random.default_rng(12)
    n = 2000
    xy = np.stack([rng.uniform(0, W, n), rng.uniform(0, H, n)], 1).astype(np.float32)
    v = rng.standard_normal((n, 2)).astype(np.float32)
    L.check(lib.ubg_scatter_accum(sim._h, n, fp(xy), fp(v)))
    ax, ay = np.zeros((H, W - 1), np.float32), np.zeros((H - 1, W), np.float32)
    O.scatter_items(ax, ay, xy, v)
    bx, by = np.zeros_like(ax), np.zeros_like(ay)
    O.scatter_items(bx, by, xy, np.abs(v))
    assert np.all(np.abs(sim.get("vx_accum") - ax) <= 1e-6 * bx + 1e-30)
    assert np.all(np.abs(sim.get("vy_accum") - ay) <= 1e-6 * by + 1e-30)
    sim.step(1e-4)
    assert not sim.get("vx_accum")[1:-1, 1:-1].any()
    assert not sim.get("vy_accum")[1:-1, 1:-1].any()
    sim.close()


def test_set_grids_exact(lib):
    from ubootgl_gb300 import _lib as L
    sim, flag = make_sim()
    W, H = sim.width, sim.height
    rng = np.random.default_rng(5)
    n = 400
    cells = np.stack([rng.integers(-2, W + 2, n), rng.integers(-2, H + 2, n)], 1).astype(np.int32)
    vals = rng.integers(0, 2, n).astype(np.float32)
    cells[n // 2:] = cells[: n - n // 2]  # repeated cells, later values win
    vals[n // 2:] = 1.0 - vals[: n - n // 2]
    fields = {"flag": flag.copy(), "vx": sim.get("vx"), "vy": sim.get("vy"), "p": sim.get("p")}
    for (x, y), val in zip(cells, vals):
        O.set_grids(fields, int(x), int(y), val)
    L.check(lib.ubg_set_grids(sim._h, n, cells.ctypes.data_as(C.POINTER(C.c_int)), fp(vals)))
    assert np.array_equal(sim.get("flag"), fields["flag"])
    for k in ("vx", "vy", "p"):
        assert np.array_equal(sim.get(k), fields[k]), k
    # coarse flags follow (MG::updateFields)
    port = O.PortSim(fields["flag"], 1.0, 1e-4)
    for lvl in range(port.levels()):
        assert np.array_equal(sim.mg_level_flag(lvl), port.level_flag(lvl)), lvl
    sim.close()


def test_shift_map_exact(lib):
    from ubootgl_gb300 import _lib as L
    sim, flag = make_sim(W=96, H=48)
    W, H = sim.width, sim.height
    new_flag = np.concatenate([flag[:, 1:], WL.disc_flag(W, H, n_discs=3, seed=9)[:, -1:]], 1)
    new_flag[:, 0] = flag[:, 1]
    new_flag[H // 3: H // 2, 0] = 0.0  # a solid stretch in the inflow column
    fields = {k: sim.get(k) for k in ("vx", "vx_back", "vy", "vy_back", "p")}
    fields["flag"] = flag.copy()
    O.shift_map(fields, new_flag)
    L.check(lib.ubg_shift_map(sim._h, fp(np.ascontiguousarray(new_flag, np.float32))))
    for k in ("vx", "vx_back", "vy", "vy_back", "p", "flag"):
        assert np.array_equal(sim.get(k), fields[k]), k
    # the step after the shift runs on the new hierarchy like the oracle's
    port = O.PortSim(new_flag, 1.0, 1e-4)
    for k in ("vx", "vx_back", "vy", "vy_back", "p"):
        port.set(k, fields[k])
    dt = WL.cfl_dt(fields["vx"], fields["vy"], sim.h)
    sim.step(dt)
    port.step(dt)
    for k in ("vx", "vy", "p"):
        assert np.array_equal(sim.get(k), port.get(k)), k
    sim.close()


def test_snapshot_restore_roundtrip(lib):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    sim, flag = make_sim(steps=3)
    sim.add_sink(0.3, 0.2, 1.0)
    n = C.c_size_t()
    L.check(lib.ubg_snapshot_bytes(sim._h, C.byref(n)))
    buf = (C.c_char * n.value)()
    L.check(lib.ubg_snapshot(sim._h, buf))
    other = Simulation(np.ones_like(flag), 1.0, 1e-4)
    L.check(lib.ubg_restore(other._h, buf))
    assert np.array_equal(other.get("flag"), flag)
    for _ in range(3):
        dt = WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h)
        sim.step(dt)
        other.step(dt)
    for k in ("vx", "vy", "vx_back", "vy_back", "p", "f"):
        assert np.array_equal(sim.get(k), other.get(k)), k
    bad = Simulation(np.ones((40, 64), np.float32), 1.0, 1e-4)
    assert lib.ubg_restore(bad._h, buf) == -1
    sim.close()
    other.close()
    bad.close()
