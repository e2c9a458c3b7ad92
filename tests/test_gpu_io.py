"""Asynchronous host I/O (ubg_io_*): a pipeline of steps whose inputs are
uploaded and whose results are downloaded asynchronously gives exactly the
fields of the synchronous upload / step / download sequence."""
import numpy as np
import pytest

from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def test_async_io_pipeline_matches_sync(lib):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    W, H, n = 200, 100, 6
    flag = WL.disc_flag(W, H, n_discs=4, seed=8)
    ins = [WL.initial_velocity(flag, seed=20 + i) for i in range(n)]
    ref = Simulation(flag, 1.0, 1e-4)
    want = []
    for vx, vy in ins:
        ref.set("vx", vx)
        ref.set("vy", vy)
        ref.step_cfl(0.5)
        want.append((ref.get("vx_current"), ref.get("vy_current")))
    sim = Simulation(flag, 1.0, 1e-4)
    hin = [(L.PinnedArray((H, W - 1)), L.PinnedArray((H - 1, W))) for _ in range(n)]
    hout = [(L.PinnedArray((H, W - 1)), L.PinnedArray((H - 1, W))) for _ in range(n)]
    for (a, b), (vx, vy) in zip(hin, ins):
        a.array[:] = vx
        b.array[:] = vy
    for i in range(n):
        L.check(lib.ubg_io_upload_async(sim._h, L.fptr(hin[i][0].array), L.fptr(hin[i][1].array)))
        sim.step_cfl(0.5)
        L.check(lib.ubg_io_download_async(sim._h, L.fptr(hout[i][0].array),
                                          L.fptr(hout[i][1].array)))
    L.check(lib.ubg_io_wait(sim._h))
    for i in range(n):
        assert np.array_equal(hout[i][0].array, want[i][0]), i
        assert np.array_equal(hout[i][1].array, want[i][1]), i
    ref.close()
    sim.close()


@pytest.mark.parametrize("d", [1.0001, 2.0001, 3.0, 3.0001, 4.0001, 1.00020003, 1.37, 4.999])
def test_division_by_reciprocal_exact(lib, d):
    """The kernels' x / d (Markstein's correction of x * RN(1/d)) equals
    CUDA's IEEE division bit for bit: random bit patterns over every
    exponent (zeros, subnormals, infinities, NaNs included)."""
    import ctypes as C
    from ubootgl_gb300 import _lib as L
    rng = np.random.default_rng(int(d * 1000))
    x = rng.integers(0, 2 ** 32, 1 << 22, dtype=np.uint64).astype(np.uint32).view(np.float32)
    x = np.concatenate([x, np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-38,
                                     3.4e38, 1.0, -1.0], np.float32)])
    bad = C.c_uint()
    L.check(lib.ubg_selftest_div(L.fptr(np.ascontiguousarray(x)), len(x), np.float32(d),
                                 C.byref(bad)))
    assert bad.value == 0
