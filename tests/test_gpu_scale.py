"""The plain FP32 step at scale: one 8192 x 4096 grid (33.5 M cells) with 400
seeded discs of radius 20-60 cells and 2^20 tracers (rings of 30 points),
the benchmark's second configuration.

* Fluid parity: the GPU step against the CPU restatement of the reference
  step, bit-identical (tolerance 0), for the first steps at full size.
* Tolerance mode at this size: three steps whose projections each reach a
  relative residual of 1e-6 from the previous pressure with FP32 and FP16
  coarse levels, in a bounded number of V-cycles.  BF16 coarse levels do
  not converge at this size; the solver keeps its starting pressure and the
  fields stay finite.
* Tracers: 50 fluid + tracer steps on the GPU; then one more tracer step is
  checked bit for bit against the restatement of advect_tracer_points.cs on
  the first 65536 tracers (the shader's random reseeding depends on the
  tracer's index, so a prefix of the array is checked), using the display
  texture the restatement builds from the GPU's own fields.  Size-free
  properties over all 2^20 tracers: ring pointers in range, heads finite and
  inside the domain or held where they stopped.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu

W, H = 8192, 4096
NTR, NPTS = 1 << 20, 30


def scale_flag():
    return WL.disc_flag(W, H, n_discs=400, r_range=(20.0 * 1024 / W, 60.0 * 1024 / W), seed=2026)


@pytest.fixture(scope="module")
def scale_case(lib):
    flag = scale_flag()
    vx, vy = WL.initial_velocity(flag, seed=2027)
    return flag, vx, vy


def test_scale_fluid_steps_bit_exact(scale_case):
    from ubootgl_gb300.simulation import Simulation
    flag, vx, vy = scale_case
    solid = 1.0 - flag.mean()
    assert 0.03 < solid < 0.2
    sim = Simulation(flag, 1.0, 1e-4)
    ref = O.PortSim(flag)
    for s in (sim, ref):
        for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
            s.set(n, a)
    for k in range(2):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        sim.step(float(dt))
        ref.step(dt)
        for n in ("vx", "vy", "p"):
            a, b = sim.get(n), ref.get(n)
            assert np.array_equal(a, b), "step %d %s: max |d| %g" % (k, n, np.abs(a - b).max())
    sim.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_scale_tolerance_steps(scale_case, precision):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    flag, vx, vy = scale_case
    sim = Simulation(flag, 1.0, 1e-4)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    for _ in range(2):
        sim.step_cfl(0.5)
    sim.set_options(solver_mode=L.SOLVE_TOLERANCE, tol=1e-6, max_vcycles=60, precision=precision)
    for k in range(3):
        sim.step_cfl(0.5)
        cycles, rel = sim.solver_stats()
        print("\n[tol 8192x4096 %s] step %d: %d V-cycles, ||r||/||f_c|| %.2e" % (precision, k, cycles, rel))
        if precision == "bf16":
            assert np.isfinite(rel) and rel < 1.5
        else:
            assert cycles <= 45 and rel <= 1e-6, (k, cycles, rel)
    for n in ("vx", "vy", "p"):
        assert np.isfinite(sim.get(n)).all()
    sim.close()


def test_scale_tracers(scale_case):
    from ubootgl_gb300.simulation import Simulation, Tracers
    flag, vx, vy = scale_case
    sim = Simulation(flag, 1.0, 1e-4)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    pdim = (np.float32(1.0), np.float32(np.float32(1.0) * np.float32(H) / np.float32(W)))
    tr = Tracers(sim, NTR, NPTS)
    tr.upload(*WL.seed_tracers(flag, NTR, NPTS, pdim, seed=2028))
    for k in range(50):
        sim.step_cfl(0.5)
        tr.step(sim.last_dt(), 7 + k)
    pts, st, en, ag = tr.download()
    assert (st < NPTS).all() and (en < NPTS).all()
    heads = pts[np.arange(NTR), en]
    assert np.isfinite(heads).all() and np.isfinite(ag).all()
    inside = ((heads[:, 0] >= 0) & (heads[:, 0] <= pdim[0]) & (heads[:, 1] >= 0) &
              (heads[:, 1] <= pdim[1]))
    assert inside.mean() > 0.999
    assert (st > 0).any()  # rings wrapped: 50 steps > 30 points
    # one more tracer step, bit for bit against the restatement on a prefix
    n = 65536
    dt = np.float32(sim.last_dt())
    vxy, _ = O.velocity_texture(sim.get("vx"), sim.get("vy"))
    p0, s0, e0, a0 = (np.ascontiguousarray(x[:n]).copy() for x in (pts, st, en, ag))
    O.tracers_step(p0, s0, e0, a0, vxy, flag, dt, pdim, 999)
    tr.step(float(dt), 999)
    p1, s1, e1, a1 = tr.download()
    assert np.array_equal(e1[:n], e0) and np.array_equal(s1[:n], s0)
    assert np.array_equal(a1[:n], a0)
    assert np.array_equal(p1[:n], p0)
    del tr
    sim.close()
