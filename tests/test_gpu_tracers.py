"""Display tracers and the display velocity texture on the GPU against the
CPU restatement of the GL shaders (interp_shader.cs, advect_tracer_points.cs).

The shaders themselves cannot run here (no graphics stack), so this parity is
with the restatement only.  Both sides evaluate the same FP32 operations in
the same order: tolerance 0 for positions, ages and ring pointers.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def make_sim(W=130, H=66, seed=21):
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(W, H, n_discs=4, seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1)
    sim = Simulation(flag, 1.0, 1e-4)
    sim.set("vx", vx)
    sim.set("vy", vy)
    return sim, flag


def test_velocity_texture_matches_restatement(lib):
    from ubootgl_gb300.simulation import velocity_texture
    sim, flag = make_sim()
    sim.step(float(WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h)))
    vxy, mag = velocity_texture(sim)
    rvxy, rmag = O.velocity_texture(sim.get("vx"), sim.get("vy"))
    assert vxy.shape == (2 * 66 - 1, 2 * 130 - 1, 2)
    assert np.array_equal(vxy, rvxy)
    assert np.array_equal(mag, rmag)


def test_tracers_match_restatement(lib):
    from ubootgl_gb300.simulation import Tracers
    sim, flag = make_sim()
    W, H = 130, 66
    ntr, npts = 3000, 30
    rng = np.random.default_rng(5)
    pdim = (np.float32(1.0), np.float32(np.float32(1.0) * np.float32(H) / np.float32(W)))
    pts = np.zeros((ntr, npts, 2), np.float32)
    pts[:, 0, 0] = rng.uniform(-0.02, 1.02, ntr)          # a few start outside the domain
    pts[:, 0, 1] = rng.uniform(0.0, float(pdim[1]), ntr)
    start = np.zeros(ntr, np.uint32)
    end = np.zeros(ntr, np.uint32)
    ages = rng.uniform(0.0, 6.4, ntr).astype(np.float32)  # some reseed at once
    tr = Tracers(sim, ntr, npts)
    tr.upload(pts, start, end, ages)
    for k in range(40):
        dt = np.float32(WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h))
        sim.step(float(dt))
        tr.step(float(dt), 1234 + 77 * k)
        vxy, _ = O.velocity_texture(sim.get("vx"), sim.get("vy"))
        O.tracers_step(pts, start, end, ages, vxy, flag, dt, pdim, 1234 + 77 * k)
    gp, gs, ge, ga = tr.download()
    assert np.array_equal(ge, end) and np.array_equal(gs, start)
    assert np.array_equal(ga, ages)
    assert np.array_equal(gp, pts)
    # the rings wrapped and some tracers were reseeded
    assert (start > 0).any() and (ages < 0.5).any()
