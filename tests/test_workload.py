"""Synthetic workload generator."""
import numpy as np

from ubootgl_gb300 import workload as WL


def test_flag_shape_and_walls():
    f = WL.disc_flag(1024, 512, n_discs=12, seed=1)
    assert f.shape == (512, 1024) and f.dtype == np.float32
    assert set(np.unique(f)) <= {0.0, 1.0}
    assert (f[0] == 0).all() and (f[-1] == 0).all()
    solid = 1.0 - f[1:-1].mean()
    assert 0.03 < solid < 0.3


def test_solid_fraction_target():
    f = WL.disc_flag(512, 256, solid_frac=0.12, seed=2)
    assert 0.12 <= 1.0 - f.mean() < 0.25


def test_velocity_respects_solids():
    f = WL.disc_flag(256, 128, n_discs=5, seed=3)
    vx, vy = WL.initial_velocity(f, seed=4)
    assert vx.shape == (128, 255) and vy.shape == (127, 256)
    assert (vx[f[:, :-1] * f[:, 1:] == 0] == 0).all()
    assert (vy[f[:-1, :] * f[1:, :] == 0] == 0).all()
    assert abs(vx[64, 0] - 1.0) < 1e-6


def test_cfl_dt_is_float32_formula():
    vx = np.full((8, 7), 2.0, np.float32)
    vy = np.full((7, 8), -3.0, np.float32)
    h = WL.grid_h(8)
    dt = WL.cfl_dt(vx, vy, h)
    assert dt.dtype == np.float32
    assert dt == np.float32(np.float32(np.float32(0.5) * np.float32(h)) / np.float32(3.0))


def test_mg_levels_match_reference_rule():
    # integer halving while both sides > 3 (pressure_solver.hpp:20-30)
    assert WL.mg_levels(1024, 512)[-1] == (8, 4) and len(WL.mg_levels(1024, 512)) == 8
    assert len(WL.mg_levels(4096, 2048)) == 10
    assert len(WL.mg_levels(8192, 4096)) == 11
