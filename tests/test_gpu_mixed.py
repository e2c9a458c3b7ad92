"""Mixed-precision projection against FP64 oracle projections.

The pre-projection state (velocity after diffuse / advect / setVBCs, the
warm-start pressure of the previous step, dt) comes from the FP32 GPU path.
Each GPU result is compared with the CPU restatement of project()
(simulation.cpp:164-208) run in double with the same algorithm:

  fp32 (the drop-in, 2 V-cycles)   vs  FP64, 2 V-cycles
  fp16 / bf16 (2 defect corrections, each one 16-bit V-cycle)
                                   vs  FP64, 2 V-cycles from p with
                                       zero-gradient edges (the same
                                       iteration in exact arithmetic)

and the test states, over the interior fluid cells,

  e_p   = max |p' - p64'| / max |p64'|      (' = minus the mean: the solver's
                                             system fixes p up to a constant)
  e_div = ||D(u) - D(u64)||_2 / ||D(u_pre)||_2

with D the cell divergence of the staggered field in FP64.  The tolerances
are written in the tests.  The tolerance-mode tests compare the residual
reduction of the three precisions over the same number of cycles.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu

# (e_p, e_div) bounds per mode.  Measured on GB300 at 512x256 after two
# cycles: fp32 3.3e-6 / 1.06e-5 (the rounding of the FP32 velocity faces),
# fp16 6.6e-4 / 2.8e-2, bf16 5.9e-3 / 2.0e-1: the last 16-bit correction's
# rounding is high-frequency noise in p, which the divergence sees through a
# discrete Laplacian.
TOL = {"fp32": (1e-5, 2e-5), "fp16": (2e-3, 0.1), "bf16": (2e-2, 0.5)}


def divergence64(vx, vy, flag):
    vx = vx.astype(np.float64)
    vy = vy.astype(np.float64)
    H, W = flag.shape
    d = np.zeros((H, W))
    d[1:H - 1, 1:W - 1] = (vx[1:H - 1, 1:W - 1] - vx[1:H - 1, 0:W - 2] +
                           vy[1:H - 1, 1:W - 1] - vy[0:H - 2, 1:W - 1])
    return d * (flag > 0)


def pre_projection_state(W, H, seed, warm_steps=2):
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(W, H, n_discs=8, seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1)
    sim = Simulation(flag, 1.0, 1e-4)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    for _ in range(warm_steps):
        sim.step(WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h))
    dt = WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h)
    sim.dt = dt
    sim.diffuse()
    sim.advect()
    sim.setVBCs()
    state = {n: sim.get(n) for n in ("vx", "vy", "vx_back", "vy_back", "p")}
    sim.close()
    return flag, state, dt


def project_gpu(flag, state, dt, precision, mode="fixed", vcycles=2, tol=1e-6, max_vcycles=60,
                graph=True):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    sim = Simulation(flag, 1.0, 1e-4)
    if mode == "tol":
        sim.set_options(solver_mode=L.SOLVE_TOLERANCE, tol=tol, max_vcycles=max_vcycles,
                        precision=precision)
    else:
        sim.set_options(solver_mode=L.SOLVE_FIXED, vcycles=vcycles, precision=precision,
                        use_graph=graph)
    for n, a in state.items():
        sim.set(n, a)
    sim.dt = dt
    sim.project()
    out = {n: sim.get(n) for n in ("vx", "vy", "p")}
    out["stats"] = sim.solver_stats()
    sim.close()
    return out


def project_fp64(flag, state, dt, ncycles=2, zgbc_first=False):
    ref = O.PortSim(flag, 1.0, 1e-4, dtype=np.float64)
    for n, a in state.items():
        ref.set(n, a.astype(np.float64))
    ref.set_dt(dt)
    ref.project(ncycles=ncycles, zgbc_first=zgbc_first)
    return {n: ref.get(n) for n in ("vx", "vy", "p")}


def errors(flag, state, out, ref):
    inner = np.zeros_like(flag, dtype=bool)
    inner[1:-1, 1:-1] = flag[1:-1, 1:-1] > 0
    p, p64 = out["p"].astype(np.float64)[inner], ref["p"][inner]
    p, p64 = p - p.mean(), p64 - p64.mean()
    e_p = np.abs(p - p64).max() / np.abs(p64).max()
    d0 = divergence64(state["vx"], state["vy"], flag)
    d = divergence64(out["vx"], out["vy"], flag)
    d64 = divergence64(ref["vx"], ref["vy"], flag)
    e_div = np.linalg.norm((d - d64)[inner]) / np.linalg.norm(d0[inner])
    return e_p, e_div


@pytest.fixture(scope="module")
def case_512(lib):
    flag, state, dt = pre_projection_state(512, 256, seed=31)
    refs = {"plain": project_fp64(flag, state, dt),
            "zgbc_first": project_fp64(flag, state, dt, zgbc_first=True)}
    return flag, state, dt, refs


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_projection_vs_fp64(case_512, precision):
    flag, state, dt, refs = case_512
    out = project_gpu(flag, state, dt, precision)
    ref = refs["plain" if precision == "fp32" else "zgbc_first"]
    e_p, e_div = errors(flag, state, out, ref)
    d0 = divergence64(state["vx"], state["vy"], flag)
    rel_div = np.linalg.norm(divergence64(out["vx"], out["vy"], flag)) / np.linalg.norm(d0)
    print("\n[mixed] 512x256 %s 2 cycles: e_p %.3e e_div %.3e (||D(u)||/||D(u_pre)|| %.3e)" %
          (precision, e_p, e_div, rel_div))
    assert out["stats"][0] == 2
    assert e_p <= TOL[precision][0]
    assert e_div <= TOL[precision][1]


@pytest.mark.parametrize("W,H", [(512, 256), (4096, 2048)])
def test_tolerance_mode_residual_reduction(lib, W, H):
    """The same number of cycles reduces the residual of the compatible
    system alike in every precision (the 16-bit correction does not slow the
    reference's V-cycle down)."""
    flag, state, dt = pre_projection_state(W, H, seed=47, warm_steps=1)
    rel = {}
    for precision in ("fp32", "fp16", "bf16"):
        out = project_gpu(flag, state, dt, precision, mode="tol", tol=1e-12, max_vcycles=20)
        cycles, rel[precision] = out["stats"]
        print("\n[mixed] %dx%d %s tolerance mode: %d cycles, ||r||/||f|| %.3e" %
              (W, H, precision, cycles, rel[precision]))
        assert cycles == 20
        assert np.isfinite(out["p"]).all()
    for precision in ("fp16", "bf16"):
        assert rel[precision] <= 2.0 * rel["fp32"]


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_mixed_fixed_graph_matches_direct(case_512, precision):
    flag, state, dt, _ = case_512
    a = project_gpu(flag, state, dt, precision, vcycles=3, graph=True)
    b = project_gpu(flag, state, dt, precision, vcycles=3, graph=False)
    for n in ("vx", "vy", "p"):
        assert np.array_equal(a[n], b[n]), n


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_mixed_steps_graph_and_direct(lib, precision):
    """Whole steps with the mixed solver in fixed mode: the captured graph
    and direct launches give identical fields, and the flow stays finite."""
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    W, H = 256, 128
    flag = WL.disc_flag(W, H, n_discs=6, seed=5)
    vx, vy = WL.initial_velocity(flag, seed=6)
    res = []
    for graph in (True, False):
        sim = Simulation(flag, 1.0, 1e-4)
        sim.set_options(solver_mode=L.SOLVE_FIXED, vcycles=2, precision=precision,
                        use_graph=graph)
        for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
            sim.set(n, a)
        for _ in range(5):
            sim.step(0.5 * sim.h / 1.2)
        res.append({n: sim.get(n) for n in ("vx", "vy", "p")})
        sim.close()
    for n in ("vx", "vy", "p"):
        assert np.isfinite(res[0][n]).all()
        assert np.array_equal(res[0][n], res[1][n]), n


def test_precision_option_errors(lib):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(64, 32, n_discs=2, seed=1)
    sim = Simulation(flag, 1.0, 1e-4)
    with pytest.raises(L.UbgError) as e:
        sim.set_options(precision=7)
    assert e.value.code == -1
    sim.set_options(precision="bf16")
    sim.set_options(precision="fp32")
    sim.close()
