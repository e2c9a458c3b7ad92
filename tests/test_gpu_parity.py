"""GPU parity: the CUDA path against the CPU restatement of the reference.

The FP32 kernels evaluate the reference's expressions in the same order as
the restatement (oracle/ubg_oracle_impl.h), so the expected difference is
zero: tolerance 0 (bit-identical, with -0.0 == +0.0) for every field and
every stage.  Flags and coarse flags are compared exactly.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu

SIZES = [(64, 32), (130, 66), (257, 129), (129, 65), (200, 40)]


def make_pair(W, H, seed=0, ndisc=6):
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(W, H, n_discs=ndisc, seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1)
    sim = Simulation(flag, 1.0, 1e-4)
    ref = O.PortSim(flag, 1.0, 1e-4)
    for s in (sim, ref):
        s.set("vx", vx)
        s.set("vy", vy)
        s.set("vx_back", vx)
        s.set("vy_back", vy)
    return sim, ref, flag


def assert_same(sim, ref, names=("vx", "vy", "vx_back", "vy_back", "p", "f"), ctx=""):
    for n in names:
        a, b = sim.get(n), ref.get(n)
        d = np.abs(a.astype(np.float64) - b.astype(np.float64))
        assert np.array_equal(a, b), "%s %s: max |diff| %g at %s" % (
            ctx, n, d.max(), np.unravel_index(d.argmax(), d.shape))


@pytest.mark.parametrize("W,H", SIZES + [(1024, 512), (1025, 513), (33, 17)])
def test_flag_hierarchy_exact(lib, W, H):
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(W, H, n_discs=8, seed=W + H)
    sim = Simulation(flag)
    ref = O.PortSim(flag)
    assert sim.mg_levels() == ref.levels() == len(WL.mg_levels(W, H))
    for l in range(ref.levels()):
        assert np.array_equal(sim.mg_level_flag(l), ref.level_flag(l)), "level %d" % l


@pytest.mark.parametrize("W,H", SIZES)
def test_stages_bit_exact(lib, W, H):
    sim, ref, flag = make_pair(W, H, seed=W)
    dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
    sim.dt = float(dt)
    ref.set_dt(dt)
    sim.diffuse(); ref.stage("diffuse")
    assert_same(sim, ref, ctx="diffuse")
    sim.advect(); ref.stage("advect")
    assert_same(sim, ref, ctx="advect")
    sim.setVBCs(); ref.stage("set_vbcs")
    assert_same(sim, ref, ctx="setVBCs")
    sim.project(); ref.stage("project")
    assert_same(sim, ref, ctx="project")
    sim.setVBCs(); ref.stage("set_vbcs")
    assert_same(sim, ref, ctx="setVBCs 2")


@pytest.mark.parametrize("W,H", SIZES)
def test_steps_bit_exact(lib, W, H):
    sim, ref, flag = make_pair(W, H, seed=W + 7)
    for k in range(5):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        sim.step(float(dt))
        ref.step(dt)
        assert_same(sim, ref, names=("vx", "vy", "p"), ctx="step %d" % k)


# Widths at every remainder modulo 8 (the smoother loads 8-cell groups and
# the restriction writes 4 coarse cells at a time; advect stages 4-entry
# vectors), a tall narrow grid and tiny grids near the multigrid's limits.
EDGE_SIZES = [(131, 67), (134, 70), (135, 35), (45, 200), (12, 10), (9, 9), (36, 18),
              (1001, 11)]


@pytest.mark.parametrize("W,H", EDGE_SIZES)
def test_steps_bit_exact_edge_sizes(lib, W, H):
    sim, ref, flag = make_pair(W, H, seed=W + 11, ndisc=3)
    for k in range(3):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        sim.step(float(dt))
        ref.step(dt)
        assert_same(sim, ref, names=("vx", "vy", "p"), ctx="%dx%d step %d" % (W, H, k))


def test_graph_matches_direct(lib):
    W, H = 130, 66
    a, ref, flag = make_pair(W, H, seed=3)
    b, _, _ = make_pair(W, H, seed=3)
    b.set_options(use_graph=False)
    for k in range(4):
        dt = float(WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h))
        a.step(dt); b.step(dt); ref.step(dt)
    for n in ("vx", "vy", "p", "vx_back", "vy_back"):
        assert np.array_equal(a.get(n), b.get(n)), n
        assert np.array_equal(a.get(n), ref.get(n)), n


def test_accum_and_sinks(lib):
    W, H = 130, 66
    sim, ref, flag = make_pair(W, H, seed=5)
    rng = np.random.default_rng(9)
    ax = (0.01 * rng.standard_normal((H, W - 1))).astype(np.float32)
    ay = (0.01 * rng.standard_normal((H - 1, W))).astype(np.float32)
    for s in (sim, ref):
        s.set("vx_accum", ax)
        s.set("vy_accum", ay)
        s.add_sink(0.3, 0.2, 5.0)
        s.add_sink(0.5, 0.25, -3.0)
        s.add_sink(0.01, 0.01, 1.0)   # out of range: never applied, never decays
    for k in range(3):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        sim.step(float(dt)); ref.step(dt)
        assert_same(sim, ref, names=("vx", "vy", "p", "f", "vx_accum", "vy_accum"), ctx="step %d" % k)


def test_cfl_step_matches_host_dt(lib):
    """Device-side dt = 0.5 h / max|u| (max folded into the gradient and
    boundary kernels of the previous step) equals the host formula, also
    after the fields change between steps."""
    W, H = 130, 66
    a, ref, flag = make_pair(W, H, seed=8)
    rng = np.random.default_rng(1)
    for k in range(6):
        if k == 3:
            ax = (0.05 * rng.standard_normal((H, W - 1))).astype(np.float32)
            for s in (a, ref):
                s.set("vx_accum", ax)
        if k == 4:
            vy = ref.get("vy") * np.float32(1.5)
            for s in (a, ref):
                s.set("vy", vy)
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        a.step_cfl(0.5)
        if k != 3:  # with accumulated velocity, dt is taken after it is applied
            assert a.last_dt() == float(dt), k
            ref.step(dt)
        else:
            ref.step(np.float32(a.last_dt()))
        assert_same(a, ref, names=("vx", "vy", "p"), ctx="cfl step %d" % k)


def test_config0_1024x512_100_steps(lib):
    """The reference's CPU-runnable configuration: 1024x512, 12 discs, 100 steps."""
    W, H = 1024, 512
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(W, H, n_discs=12, seed=2024)
    vx, vy = WL.initial_velocity(flag, seed=2025)
    sim = Simulation(flag)
    ref = O.PortSim(flag)
    for s in (sim, ref):
        s.set("vx", vx); s.set("vy", vy); s.set("vx_back", vx); s.set("vy_back", vy)
    for k in range(100):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        sim.step(float(dt)); ref.step(dt)
        if k % 25 == 24:
            assert_same(sim, ref, names=("vx", "vy", "p"), ctx="step %d" % k)


# The advection option (extension): bilinearSample (interpolators.hpp:11-27)
# for the three samples of the back-trace instead of bicubicSample, against
# the restatement with the same option; the graph and the direct path, and
# sizes where the back-trace leaves the staged windows near the edges.
@pytest.mark.parametrize("W,H", [(130, 66), (257, 129), (135, 35), (1001, 11)])
def test_advect_bilinear_bit_exact(lib, W, H):
    sim, ref, flag = make_pair(W, H, seed=W + 3)
    sim.set_options(advect="bilinear")
    ref.set_advect_bilinear(True)
    dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
    sim.dt = float(dt)
    ref.set_dt(dt)
    sim.advect(); ref.stage("advect")
    assert_same(sim, ref, ctx="advect")
    for k in range(4):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        sim.step(float(dt))
        ref.step(dt)
        assert_same(sim, ref, names=("vx", "vy", "p"), ctx="step %d" % k)
    # the option really changes the advection
    sim2, ref2, _ = make_pair(W, H, seed=W + 3)
    dt = WL.cfl_dt(ref2.get("vx"), ref2.get("vy"), ref2.h)
    sim2.dt = float(dt)
    sim2.advect()
    sim3, _, _ = make_pair(W, H, seed=W + 3)
    sim3.set_options(advect="bilinear")
    sim3.dt = float(dt)
    sim3.advect()
    assert not np.array_equal(sim2.get("vx"), sim3.get("vx"))
