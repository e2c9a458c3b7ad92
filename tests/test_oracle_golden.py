"""The CPU restatement (oracle) against fixtures produced by the reference.

tests/golden/*.npz come from te42kyfo/ubootgl's own simulation.cpp /
pressure_solver.cpp (see tests/golden/make_golden.py).  The reference is
built with -Ofast (reassociation, reciprocal division, FMA contraction),
the restatement with plain IEEE arithmetic in source order, so they agree
to rounding: stated tolerances, relative to max|field|,
  STAGE_TOL = 5e-6   the stages of one step
  STEP_TOL  = 5e-5   after up to 10 full steps (errors grow ~1e-6 / step)
  MG_TOL    = 1e-5   multigrid solves.
A mismatch in any of the reference's quirks (advection tail columns, chunk
skipping, diffusion coefficient, face masks, coarse flags) shows up as an
O(1e-2) or larger difference, far above these tolerances.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAGE_TOL, STEP_TOL, MG_TOL = 5e-6, 5e-5, 1e-5


def rel(a, b):
    return float(np.abs(a.astype(np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


def seed_sim(z, dtype=np.float32):
    sim = O.PortSim(z["flag"], dtype=dtype)
    for n, a in (("vx", z["vx0"]), ("vy", z["vy0"]), ("vx_back", z["vx0"]), ("vy_back", z["vy0"])):
        sim.set(n, a)
    return sim


@pytest.mark.parametrize("fn", sorted(glob.glob(os.path.join(GOLD, "step_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_steps_match_reference(fn):
    z = np.load(fn)
    sim = seed_sim(z)
    assert np.float32(sim.h) == z["h"]
    kept = list(z["kept"])
    for k, dt in enumerate(z["dt"]):
        sim.step(np.float32(dt))
        if k in kept:
            i = kept.index(k)
            for n in ("vx", "vy", "p"):
                assert rel(sim.get(n), z[n][i]) < STEP_TOL, (n, k)


def test_stages_match_reference():
    z = np.load(os.path.join(GOLD, "stages_130x66.npz"))
    sim = seed_sim(z)
    sim.set_dt(np.float32(z["dt"]))
    for stage in ("diffuse", "advect", "set_vbcs", "project", "set_vbcs2"):
        sim.stage(stage.rstrip("2"))
        for n in ("vx", "vy", "vx_back", "vy_back", "p", "f"):
            assert rel(sim.get(n), z["%s_%s" % (stage, n)]) < STAGE_TOL, (stage, n)


def test_mg_flag_hierarchy_solve_matches_reference():
    z = np.load(os.path.join(GOLD, "levels_257x129.npz"))
    p = O.port_mg_solve(np.zeros_like(z["f"]), z["f"], z["flag"], z["h"], zgbc=True,
                        coarse_flag=z["flag"])
    assert rel(p, z["p"]) < MG_TOL


def test_mgtest_laplace_matches_reference():
    """mgtest.cpp's Laplace problem: Dirichlet data sinh(pi y) sin(pi x),
    MG(N, N) (every coarse flag 1), 5 V-cycles."""
    z = np.load(os.path.join(GOLD, "mg_laplace_65.npz"))
    N = 65
    u = np.zeros((N, N), np.float32)
    x = np.arange(N)
    u[N - 1, 1:N - 1] = (np.sinh(np.pi) * np.sin(x[1:N - 1] / (N - 1.0) * np.pi)).astype(np.float32)
    for c in range(5):
        u = O.port_mg_solve(u, np.zeros((N, N), np.float32), np.ones((N, N), np.float32), z["h"])
        assert rel(u, z["u"][c]) < MG_TOL, c
    # and it converges towards the analytic solution
    yy, xx = np.mgrid[0:N, 0:N] / (N - 1.0)
    exact = np.sinh(np.pi * yy) * np.sin(np.pi * xx)
    err0 = np.abs(exact[1:-1, 1:-1]).max()
    assert np.abs(u[1:-1, 1:-1] - exact[1:-1, 1:-1]).max() < 0.5 * err0


# The benchmark's first configuration over its full length: 1024x512, 12
# discs, 100 steps of the reference (long_1024x512.npz, classic red-black
# schedule), against the restatement with the same dt sequence.  Measured
# max |difference| / max |field| over the sampled rows and columns, per kept
# step (the restatement's plain IEEE order against the reference's -Ofast):
#   step            0       24      49      74      99
#   vx, vy        6.2e-6  1.9e-6  5.8e-6  8.7e-6  9.2e-6
#   p             4.3e-6  1.8e-5  2.1e-4  1.3e-4  6.9e-5
# p moves most: two V-cycles leave it unconverged, so rounding differences
# persist through the warm start.  The bounds below are ~2.5x those, and the
# GPU path equals the restatement bit for bit over the same 100 steps
# (test_gpu_parity.py), which chains the GPU to the reference at full length.
LONG_VEL_TOL = {0: 1.5e-5, 24: 1.5e-5, 49: 2e-5, 74: 2.5e-5, 99: 2.5e-5}
LONG_P_TOL = {0: 1.5e-5, 24: 5e-5, 49: 5e-4, 74: 4e-4, 99: 2e-4}


def test_100_steps_1024x512_match_reference():
    import sys
    sys.path.insert(0, GOLD)
    import make_golden as MG
    z = np.load(os.path.join(GOLD, "long_1024x512.npz"))
    flag, vx0, vy0 = MG.long_inputs()
    if MG.inputs_digest(flag, vx0, vy0) != str(z["digest"]):
        pytest.skip("the seeded inputs differ on this platform from the ones the fixture was made with")
    sim = O.PortSim(flag)
    for n, a in (("vx", vx0), ("vy", vy0), ("vx_back", vx0), ("vy_back", vy0)):
        sim.set(n, a)
    kept = [int(k) for k in z["kept"]]
    N = flag.size
    for k, dt in enumerate(z["dt"]):
        sim.step(np.float32(dt))
        if k not in kept:
            continue
        for n in ("vx", "vy", "p"):
            rows, cols, stats = MG.samples(sim.get(n))
            zr, zc, zs = z["%s_rows_%d" % (n, k)], z["%s_cols_%d" % (n, k)], z["%s_stats_%d" % (n, k)]
            tol = LONG_P_TOL[k] if n == "p" else LONG_VEL_TOL[k]
            err = max(np.abs(rows.astype(np.float64) - zr).max(),
                      np.abs(cols.astype(np.float64) - zc).max()) / zs[2]
            assert err < tol, (n, k, err)
            # L2 norm and max|.| relative; the sum relative to sqrt(N) * L2
            assert abs(stats[1] - zs[1]) < tol * zs[1], (n, k)
            assert abs(stats[2] - zs[2]) < tol * zs[2], (n, k)
            assert abs(stats[0] - zs[0]) < tol * np.sqrt(N) * zs[1], (n, k)
