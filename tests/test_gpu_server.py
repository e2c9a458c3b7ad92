"""The step server: results independent of the mix, admission by budget,
latency statistics.

Each session's kernels touch only that session's memory.  In the stream
mode they run the single-simulation path; in the fused mode one launch per
kernel covers every in-flight request, and the fused kernels run the same
per-member arithmetic.  Either way a session stepped among many others must
be bit-identical (tolerance 0) to the same session stepped alone.
"""
import numpy as np
import pytest

from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def session_inputs(W, H, seed, u_in=1.0):
    flag = WL.disc_flag(W, H, n_discs=4, seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1, u_in=u_in)
    return flag, vx, vy


@pytest.mark.parametrize("mode", ["fused", "streams"])
def test_alone_vs_mixed_bit_identical(lib, mode):
    from ubootgl_gb300.simulation import Server
    sizes = [(256, 128), (512, 256), (128, 64), (384, 192), (1024, 512), (192, 96)]
    rng = np.random.default_rng(0)
    # alone: one session, its requests one after another
    target = (300, 150, 41)
    solo = Server(8 << 30, max_active=4, mode=mode)
    sid = solo.open(*session_inputs(*target))
    reqs = [3, 1, 5, 2]
    for k in reqs:
        solo.wait(solo.submit(sid, k))
    alone = {n: solo.get(sid, n) for n in ("vx", "vy", "p")}
    solo.close()
    # in a mix: the same session among others, requests interleaved
    mix = Server(8 << 30, max_active=4, mode=mode)
    others = [mix.open(*session_inputs(W, H, 50 + i, 0.6 + 0.15 * i))
              for i, (W, H) in enumerate(sizes)]
    sid = mix.open(*session_inputs(*target))
    pending = []
    for k in reqs:
        for o in rng.permutation(others)[:4]:
            pending.append(mix.submit(int(o), int(rng.integers(1, 6))))
        pending.append(mix.submit(sid, k))
    for r in pending:
        mix.wait(r)
    for n in ("vx", "vy", "p"):
        assert np.array_equal(mix.get(sid, n), alone[n]), n
    st = mix.stats()
    assert st["completed"] == len(pending)
    assert st["queued"] == 0 and st["active"] == 0
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    mix.close()


def test_admission_by_budget(lib):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Server
    import ctypes as C
    b = C.c_size_t()
    L.check(lib.ubg_device_bytes(512, 256, C.byref(b)))
    srv = Server(int(2.5 * b.value), max_active=2)
    ids = [srv.open(*session_inputs(512, 256, s)) for s in range(4)]
    assert ids[0] is not None and ids[1] is not None
    assert ids[2] is None and ids[3] is None
    st = srv.stats()
    assert st["rejected_sessions"] == 2 and st["sessions"] == 2
    assert st["device_bytes_used"] <= int(2.5 * b.value)
    srv.close_session(ids[0])  # memory frees up: a new session is admitted
    assert srv.open(*session_inputs(512, 256, 9)) is not None
    srv.close()


def test_mixed_precision_sessions(lib):
    from ubootgl_gb300.simulation import Server
    srv = Server(8 << 30, max_active=8)
    a = srv.open(*session_inputs(256, 128, 3), precision="fp16")
    b = srv.open(*session_inputs(256, 128, 3), precision="fp32")
    ra, rb = srv.submit(a, 4), srv.submit(b, 4)
    srv.wait(ra)
    srv.wait(rb)
    # same flow, two solvers: the velocities agree to the mixed solver's
    # accuracy (p itself is fixed only up to a constant by the solver's
    # singular system, and the two solvers drift differently in it)
    va, vb = srv.get(a, "vx"), srv.get(b, "vx")
    assert np.isfinite(srv.get(a, "p")).all()
    assert np.abs(va - vb).max() <= 0.05 * np.abs(vb).max()
    srv.close()


@pytest.mark.parametrize("fuse_cells", [None, 50000])
def test_fused_many_sessions_match_plain_steps(lib, fuse_cells):
    """24 sessions of uneven sizes, requests of 1..8 steps submitted in a
    burst (requests join and leave the fused step at different step
    boundaries): every session ends bit-identical to a plain simulation
    stepped the same number of times.  With a 50000-cell fuse limit the
    larger sessions run as stream requests beside the fused ones."""
    from ubootgl_gb300.simulation import Server, Simulation
    rng = np.random.default_rng(4)
    sizes = [(int(w), int(w) // 2) for w in rng.choice([96, 128, 192, 256, 320, 512, 768], 24)]
    srv = Server(16 << 30, max_active=24, mode="fused", fuse_cells=fuse_cells)
    sids, total = [], []
    for i, (W, H) in enumerate(sizes):
        sids.append(srv.open(*session_inputs(W, H, 300 + i, 0.5 + 0.05 * i)))
        total.append(0)
    pending = []
    for rnd in range(3):
        for j in rng.permutation(len(sids)):
            k = int(rng.integers(1, 9))
            pending.append(srv.submit(sids[j], k))
            total[j] += k
    for r in pending:
        srv.wait(r)
    assert srv.stats()["completed"] == len(pending)
    for i, (W, H) in enumerate(sizes):
        flag, vx, vy = session_inputs(W, H, 300 + i, 0.5 + 0.05 * i)
        sim = Simulation(flag, 1.0, 1e-4)
        for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
            sim.set(n, a)
        for _ in range(total[i]):
            sim.step_cfl(0.5)
        for n in ("vx", "vy", "p"):
            assert np.array_equal(srv.get(sids[i], n), sim.get(n)), (W, n)
        sim.close()
    srv.close()


def test_queue_admission_admits_after_close(lib):
    """UBG_ADMIT_QUEUE: sessions over the budget wait instead of failing;
    their requests start once a close frees memory, and the late session
    steps exactly as if it had been admitted at once."""
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Server, Simulation
    import ctypes as C
    b = C.c_size_t()
    L.check(lib.ubg_device_bytes(512, 256, C.byref(b)))
    srv = Server(int(2.5 * b.value), max_active=2, admission="queue")
    inputs = [session_inputs(512, 256, 70 + s) for s in range(4)]
    ids = [srv.open(*x) for x in inputs]
    assert all(i is not None for i in ids)
    st = srv.stats()
    assert st["sessions"] == 4 and st["pending_sessions"] == 2 and st["rejected_sessions"] == 0
    reqs = [srv.submit(i, 3) for i in ids]
    srv.wait(reqs[0])
    srv.wait(reqs[1])
    srv.drain()  # returns with the waiting sessions' requests still queued
    st = srv.stats()
    assert st["completed"] == 2 and st["queued"] == 2
    srv.close_session(ids[0])  # frees memory: the first waiting session is built
    srv.wait(reqs[2])
    st = srv.stats()
    assert st["admitted_from_queue"] == 1 and st["pending_sessions"] == 1
    srv.close_session(ids[1])
    srv.wait(reqs[3])
    assert srv.stats()["admitted_from_queue"] == 2
    for k in (2, 3):
        sim = Simulation(inputs[k][0], 1.0, 1e-4)
        for n, a in (("vx", inputs[k][1]), ("vy", inputs[k][2]), ("vx_back", inputs[k][1]),
                     ("vy_back", inputs[k][2])):
            sim.set(n, a)
        for _ in range(3):
            sim.step_cfl(0.5)
        for n in ("vx", "vy", "p"):
            assert np.array_equal(srv.get(ids[k], n), sim.get(n)), (k, n)
        sim.close()
    # a session larger than the whole budget is still refused
    assert srv.open(*session_inputs(2048, 1024, 5)) is None
    srv.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_tolerance_sessions_alone_vs_mixed(lib, precision):
    """Tolerance-mode sessions run on the pool threads beside fused and
    stream requests.  The solver's reductions combine their partial sums in
    a fixed order, so a session's result is the same bits alone and in the
    mix (each projection solved to a relative residual of 1e-6)."""
    from ubootgl_gb300.simulation import Server
    target = session_inputs(384, 192, 91)
    solo = Server(8 << 30, max_active=4)
    sid = solo.open(*target, precision=precision, tol=1e-6)
    for k in (2, 3):
        solo.wait(solo.submit(sid, k))
    alone = {n: solo.get(sid, n) for n in ("vx", "vy")}
    solo.close()
    mix = Server(8 << 30, max_active=4)
    others = [mix.open(*session_inputs(W, H, 60 + i)) for i, (W, H) in
              enumerate([(256, 128), (512, 256), (1024, 512)])]
    others.append(mix.open(*session_inputs(256, 128, 65), tol=1e-6))
    sid = mix.open(*target, precision=precision, tol=1e-6)
    pending = []
    for k in (2, 3):
        for o in others:
            pending.append(mix.submit(o, 3))
        pending.append(mix.submit(sid, k))
    for r in pending:
        mix.wait(r)
    for n in ("vx", "vy"):
        assert np.array_equal(mix.get(sid, n), alone[n]), n
    mix.close()
