"""The allocation-free multigrid solve (ubg_mg_solve_noalloc).

Callers that may not allocate GPU memory while they run (a device-memory
budget owned by a host framework, real-time loops that must not stall in the
allocator, plug-ins whose host owns every device allocation) use this entry
point: they pass device arrays and the solver's scratch comes from a static
device array inside the library.

The test calls it through the C ABI on device arrays and checks each result
against the existing entry point (class MG: MG(flag) + solve on host arrays)
with the tolerance the parity tests use: zero (bit-identical).  The calls
come in a row: two different grids, then a 1024 x 512 grid whose p and f are
all NaN (it fills most of the shared scratch array with NaN), then a small
grid with padded row pitches (p_pitch > width, padding filled with NaN), and
that small grid once more.  The small grid must not see anything the
poisoned call left behind.  It also checks that a grid whose scratch would
exceed the static array, and an invalid h, are rejected.

This file is collected last, so a run that stops at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def _case(W, H, seed):
    rng = np.random.default_rng(seed)
    flag = WL.disc_flag(W, H, n_discs=5, seed=seed)
    p = (0.01 * rng.standard_normal((H, W))).astype(np.float32)
    f = rng.standard_normal((H, W)).astype(np.float32)
    f[0, :] = f[-1, :] = 0.0
    f[:, 0] = f[:, -1] = 0.0
    return flag, p, f


def _padded(torch, dev, a, pitch, fill):
    """a (H x W) in a device array of row pitch `pitch` elements, the padding
    set to `fill`."""
    H, W = a.shape
    buf = np.full((H, pitch), fill, dtype=a.dtype)
    buf[:, :W] = a
    return torch.from_numpy(buf).to(dev)


def _solve(lib, torch, dev, stream, flag, p0, f, h, pitch=None):
    H, W = flag.shape
    pp = pitch or W
    dp = _padded(torch, dev, p0, pp, np.float32(np.nan))
    df = _padded(torch, dev, f, pp, np.float32(np.nan))
    dflag = _padded(torch, dev, flag.astype(np.uint8), pp + 3 if pitch else W, np.uint8(7))
    rc = lib.ubg_mg_solve_noalloc(C.c_void_p(dp.data_ptr()), pp, C.c_void_p(df.data_ptr()), pp,
                                  C.c_void_p(dflag.data_ptr()), dflag.shape[1], W, H, h, 1,
                                  C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    out = dp.cpu().numpy()
    if pitch:
        # the padding of p is the caller's and stays untouched
        assert np.isnan(out[:, W:]).all()
    return rc, out[:, :W]


def test_noalloc_solve_matches_mg_class(lib):
    torch = pytest.importorskip("torch")
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import MG

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    plan = [("a", 130, 66, 11, None), ("b", 257, 129, 12, None), ("poison", 1024, 512, 13, None),
            ("c", 130, 66, 14, 157), ("c again", 130, 66, 14, 157)]
    for name, W, H, seed, pitch in plan:
        flag, p0, f = _case(W, H, seed)
        h = WL.grid_h(W)
        if name == "poison":
            p0[:] = np.nan
            f[:] = np.nan
            rc, _ = _solve(lib, torch, dev, stream, flag, p0, f, h)
            assert rc == 0, L.load().ubg_last_error()
            assert lib.ubg_last_error() == b""
            continue
        # existing entry point: MG(flag).solve on host arrays
        p_ref = p0.copy()
        MG(flag).solve(p_ref, f, flag, h, True)
        rc, got = _solve(lib, torch, dev, stream, flag, p0, f, h, pitch)
        assert rc == 0, L.load().ubg_last_error()
        assert lib.ubg_last_error() == b""
        d = np.abs(got.astype(np.float64) - p_ref.astype(np.float64)).max()
        assert np.array_equal(got, p_ref), "call %s: max |diff| %g" % (name, d)


def test_noalloc_rejects_bad_h(lib):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    W, H = 64, 32
    dp = torch.zeros((H, W), dtype=torch.float32, device=dev)
    dflag = torch.ones((H, W), dtype=torch.uint8, device=dev)
    for h in (0.0, -1.0, float("inf"), float("nan")):
        rc = lib.ubg_mg_solve_noalloc(C.c_void_p(dp.data_ptr()), W, C.c_void_p(dp.data_ptr()), W,
                                      C.c_void_p(dflag.data_ptr()), W, W, H, h, 1, None)
        assert rc == -1
        assert b"h must be" in lib.ubg_last_error()


def test_noalloc_rejects_oversize_grid(lib):
    """A 4096 x 2048 grid needs more scratch than the static array holds."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    W, H = 4096, 2048
    dp = torch.zeros((H, W), dtype=torch.float32, device=dev)
    df = torch.zeros((H, W), dtype=torch.float32, device=dev)
    dflag = torch.ones((H, W), dtype=torch.uint8, device=dev)
    rc = lib.ubg_mg_solve_noalloc(C.c_void_p(dp.data_ptr()), W, C.c_void_p(df.data_ptr()), W,
                                  C.c_void_p(dflag.data_ptr()), W, W, H, 1.0 / 4095, 1, None)
    assert rc == -1
    assert b"bytes of solver scratch" in lib.ubg_last_error()
