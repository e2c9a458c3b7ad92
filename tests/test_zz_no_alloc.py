"""The allocation-free multigrid solve (ubg_mg_solve_noalloc).

Callers that may not allocate GPU memory while they run (work recorded into
a larger CUDA graph, a device-memory budget owned by a host framework,
real-time loops) use this entry point: they pass device arrays and the
solver's scratch comes from a static device array inside the library.

The test calls it through the C ABI on device arrays, twice in a row with
different grids and data, and checks each result against the existing
entry point (class MG: MG(flag) + solve on host arrays) with the tolerance
the parity tests use: zero (bit-identical).  It also checks that a grid
whose scratch would exceed the static array is rejected.

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


def test_noalloc_solve_matches_mg_class(lib):
    torch = pytest.importorskip("torch")
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import MG

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for call, (W, H, seed) in enumerate([(130, 66, 11), (257, 129, 12)]):
        flag, p0, f = _case(W, H, seed)
        h = WL.grid_h(W)
        # existing entry point: MG(flag).solve on host arrays
        p_ref = p0.copy()
        MG(flag).solve(p_ref, f, flag, h, True)
        # allocation-free entry point on device arrays (pitch = width)
        dp = torch.from_numpy(p0.copy()).to(dev)
        df = torch.from_numpy(f).to(dev)
        dflag = torch.from_numpy(flag.astype(np.uint8)).to(dev)
        rc = lib.ubg_mg_solve_noalloc(C.c_void_p(dp.data_ptr()), W, C.c_void_p(df.data_ptr()), W,
                                      C.c_void_p(dflag.data_ptr()), W, W, H, h, 1,
                                      C.c_void_p(stream.cuda_stream))
        assert rc == 0, L.load().ubg_last_error()
        torch.cuda.synchronize(dev)
        got = dp.cpu().numpy()
        d = np.abs(got.astype(np.float64) - p_ref.astype(np.float64)).max()
        assert np.array_equal(got, p_ref), "call %d: max |diff| %g" % (call, d)


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
