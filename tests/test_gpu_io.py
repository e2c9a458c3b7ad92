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
