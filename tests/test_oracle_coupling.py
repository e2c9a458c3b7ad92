"""CPU: the oracle's restatements of the game-side field access against the
reference itself (bilinearSample / bilinearScatter, interpolators.hpp:11-40,
and Simulation::setGrids, simulation.hpp:82-98, compiled from the reference
checkout).  The reference is built with -Ofast -march=native, which may fuse
the interpolation's multiply-adds: values agree within 2 ulp of the result
scale; setGrids is exact."""
import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference checkout (x86-64) absent")


@needs_ref
def test_bilinear_sample_and_scatter_vs_reference():
    import ctypes as C
    lib = O.ref_lib()
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    rng = np.random.default_rng(1)
    H, W = 37, 53
    g = rng.standard_normal((H, W)).astype(np.float32)
    n = 3000
    xy = np.stack([rng.uniform(-4, W + 4, n), rng.uniform(-4, H + 4, n)], 1).astype(np.float32)
    out = np.empty(n, np.float32)
    lib.ref_bilinear_sample_n(P(g), W, H, n, P(xy), P(out))
    mine = np.array([O.bilinear_sample(g, x, y) for x, y in xy], np.float32)
    assert np.all(np.abs(mine - out) <= 2 * np.spacing(np.float32(4.0)))
    v = rng.standard_normal(n).astype(np.float32)
    a = g.copy()
    lib.ref_bilinear_scatter_n(P(a), W, H, n, P(xy), P(v))
    b = g.copy()
    for (x, y), vi in zip(xy, v):
        O.bilinear_scatter(b, x, y, vi)
    assert np.allclose(a, b, rtol=0, atol=64 * np.spacing(np.float32(8.0)))


@needs_ref
def test_set_grids_vs_reference():
    W, H = 70, 40
    flag = WL.disc_flag(W, H, n_discs=3, seed=2)
    vx, vy = WL.initial_velocity(flag, seed=3)
    ref = O.RefSim(flag)
    for n, arr in (("vx", vx), ("vy", vy)):
        ref.set(n, arr)
    p = np.random.default_rng(4).standard_normal((H, W)).astype(np.float32)
    ref.set("p", p)
    fields = {"flag": flag.copy(), "vx": vx.copy(), "vy": vy.copy(), "p": p.copy()}
    rng = np.random.default_rng(5)
    for _ in range(300):
        x, y = int(rng.integers(-2, W + 2)), int(rng.integers(-2, H + 2))
        val = float(rng.integers(0, 2))
        ref.set_grids(x, y, val)
        O.set_grids(fields, x, y, np.float32(val))
    for k in ("flag", "vx", "vy", "p"):
        assert np.array_equal(ref.get(k), fields[k]), k


def test_shift_map_restatement_invariants():
    """Host-only checks of the shiftMap restatement: columns move west, the
    last column is kept, solid cells zero their faces, inflow column."""
    W, H = 40, 20
    flag = WL.disc_flag(W, H, n_discs=2, seed=1)
    vx, vy = WL.initial_velocity(flag, seed=2)
    f = {"vx": vx.copy(), "vx_back": np.zeros_like(vx), "vy": vy.copy(),
         "vy_back": np.zeros_like(vy), "p": np.arange(W * H, dtype=np.float32).reshape(H, W),
         "flag": flag.copy()}
    new = np.ones_like(flag)
    new[0, :] = new[-1, :] = 0.0
    O.shift_map(f, new)
    assert np.array_equal(f["vx"][1:-1, 1:-1], vx[1:-1, 2:])
    assert np.array_equal(f["vx_back"][1:-1, 1:-1], vx[1:-1, 2:])
    assert np.array_equal(f["p"][1:-1, :-1], np.arange(W * H, dtype=np.float32).reshape(H, W)[1:-1, 1:])
    assert not f["p"][0].any() and not f["vx"][0].any()
    u = np.float32(np.float32(0.07) * np.float32(H)) / np.float32(1.0 + (H - 2))
    assert np.array_equal(f["vx"][1:-1, 0], np.full(H - 2, u, np.float32))


def test_bilinear_advection_sampler_matches_pinned_restatement():
    """The C restatement's bilinearSample (the advection option's sampler)
    equals the numpy restatement that is pinned against the reference build
    above, bit for bit, on points inside and outside the clamp range."""
    rng = np.random.default_rng(7)
    g = rng.standard_normal((37, 53)).astype(np.float32)
    for _ in range(5000):
        cx, cy = rng.uniform(-3.0, 60.0), rng.uniform(-3.0, 45.0)
        a = O.port_bilinear_sample(g, cx, cy)
        b = O.bilinear_sample(g, cx, cy)
        assert a == b, (cx, cy, a, b)
