"""Batches and the autotuner: results identical to stepping alone.

A batch step is one CUDA graph: small FP32 members are stepped by fused
launches (one launch per kernel over all of them), the other members'
fixed-cycle step bodies are parallel branches.  The members only touch
their own memory and every kernel runs the single-simulation arithmetic, so
each member must be bit-identical to the same simulation stepped alone
(tolerance 0).  The autotuner only changes tile shapes and the coarse-tail
size, which must not change a bit either.
"""
import numpy as np
import pytest

from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu

SIZES = [(128, 64), (192, 96), (256, 128), (96, 48), (320, 160), (512, 256)]


def build(W, H, seed, precision="fp32", u_in=1.0):
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(W, H, n_discs=4, seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1, u_in=u_in)
    sim = Simulation(flag, 1.0, 1e-4)
    if precision != "fp32":
        sim.set_options(precision=precision)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    return sim


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_batch_device_dt_matches_alone(lib, precision):
    from ubootgl_gb300.simulation import Batch
    alone = [build(W, H, 10 + i, precision, 0.5 + 0.2 * i) for i, (W, H) in enumerate(SIZES)]
    members = [build(W, H, 10 + i, precision, 0.5 + 0.2 * i) for i, (W, H) in enumerate(SIZES)]
    batch = Batch(members)
    for _ in range(4):
        for s in alone:
            s.step_cfl(0.5)
        batch.step(cfl=0.5)
    batch.sync()
    for a, b in zip(alone, members):
        for n in ("vx", "vy", "vx_back", "vy_back", "p"):
            assert np.array_equal(a.get(n), b.get(n)), (a.width, n)
        assert a.last_dt() == b.last_dt()
    batch.close()
    for s in alone + members:
        s.close()


def test_batch_host_dt_accum_and_member_steps(lib):
    """Host time steps, an accumulation applied before a batch step, and
    members stepped alone between batch steps."""
    from ubootgl_gb300.simulation import Batch
    alone = [build(W, H, 30 + i) for i, (W, H) in enumerate(SIZES[:4])]
    members = [build(W, H, 30 + i) for i, (W, H) in enumerate(SIZES[:4])]
    batch = Batch(members)
    rng = np.random.default_rng(3)
    for it in range(5):
        dts = np.array([WL.cfl_dt(s.get("vx"), s.get("vy"), s.h) for s in alone], np.float32)
        if it == 2:
            for a, b in zip(alone, members):
                acc = (1e-3 * rng.standard_normal((a.height, a.width - 1))).astype(np.float32)
                a.set("vx_accum", acc)
                b.set("vx_accum", acc)
        if it == 3:
            for a, b, dt in zip(alone, members, dts):
                a.step(float(dt))
                b.step(float(dt))
            continue
        for a, dt in zip(alone, dts):
            a.step(float(dt))
        batch.step(dts)
    for a, b in zip(alone, members):
        for n in ("vx", "vy", "p"):
            assert np.array_equal(a.get(n), b.get(n)), (a.width, n)
    batch.close()
    for s in alone + members:
        s.close()


def test_autotune_bit_identical(lib):
    """The autotuner's choices (tiles, tail size, the cluster coarse solve's
    first level or the launches per level) give the same bits as the
    defaults (which start the cluster coarse solve two levels above the
    tail where the device can hold the cluster)."""
    import ctypes as C
    import json
    buf = C.create_string_buffer(1024)
    assert lib.ubg_device_info(buf, len(buf)) == 0
    cluster = json.loads(buf.value.decode())["cluster_coarse_solve"].startswith("available")
    a = build(1024, 512, 77)
    b = build(1024, 512, 77)
    rep = b.autotune()
    assert rep["levels"] and "tail_cells" in rep and rep["vcycle_us"] > 0
    assert all(t["vcycle_us"] > 0 for t in rep["trials"])
    assert "cluster_top" in rep
    if cluster:  # every feasible first level was timed
        assert sum(t["what"] == "cluster" for t in rep["trials"]) >= 2
    for _ in range(3):
        a.step_cfl(0.5)
        b.step_cfl(0.5)
    for n in ("vx", "vy", "p"):
        assert np.array_equal(a.get(n), b.get(n)), n
    a.close()
    b.close()


def test_batch_rejects_tolerance_members(lib):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Batch
    s = build(96, 48, 1)
    s.set_options(solver_mode=L.SOLVE_TOLERANCE, tol=1e-3)
    b = Batch([s])
    with pytest.raises(L.UbgError):
        b.step(cfl=0.5)
    b.close()
    s.close()


def test_fused_batch_uneven_many(lib):
    """A fused batch (one launch per kernel over all members) of 24 members
    with uneven sizes, hence different multigrid depths and coarse tails:
    every member bit-identical to stepping alone, also after a member is
    stepped alone between batch steps (the plan follows its indices)."""
    from ubootgl_gb300.simulation import Batch
    rng = np.random.default_rng(9)
    sizes = [(int(w), int(w) // 2) for w in rng.choice([96, 128, 160, 192, 256, 320, 384, 512], 24)]
    alone = [build(W, H, 200 + i, u_in=0.5 + 0.04 * i) for i, (W, H) in enumerate(sizes)]
    members = [build(W, H, 200 + i, u_in=0.5 + 0.04 * i) for i, (W, H) in enumerate(sizes)]
    batch = Batch(members)
    for it in range(5):
        if it == 2:
            alone[3].step_cfl(0.5)
            members[3].step_cfl(0.5)
        for s in alone:
            s.step_cfl(0.5)
        batch.step(cfl=0.5)
    batch.sync()
    for a, b in zip(alone, members):
        for n in ("vx", "vy", "vx_back", "vy_back", "p"):
            assert np.array_equal(a.get(n), b.get(n)), (a.width, n)
    batch.close()
    for s in alone + members:
        s.close()


def test_hybrid_batch_fused_and_branches(lib):
    """Small FP32 members fused, a member above 2^20 cells and a mixed-
    precision member as graph branches of the same batch step: all
    bit-identical to stepping alone."""
    from ubootgl_gb300.simulation import Batch
    cfg = [(1536, 768, "fp32"), (128, 64, "fp32"), (256, 128, "fp16"), (320, 160, "fp32"),
           (96, 48, "fp32")]
    alone = [build(W, H, 400 + i, p, 0.6 + 0.1 * i) for i, (W, H, p) in enumerate(cfg)]
    members = [build(W, H, 400 + i, p, 0.6 + 0.1 * i) for i, (W, H, p) in enumerate(cfg)]
    batch = Batch(members)
    for _ in range(4):
        for s in alone:
            s.step_cfl(0.5)
        batch.step(cfl=0.5)
    batch.sync()
    for a, b in zip(alone, members):
        for n in ("vx", "vy", "vx_back", "vy_back", "p"):
            assert np.array_equal(a.get(n), b.get(n)), (a.width, n)
    batch.close()
    for s in alone + members:
        s.close()


def test_fused_batch_odd_sizes(lib):
    """Fused members whose widths leave every remainder modulo 8 and odd
    heights: bit-identical to stepping alone."""
    from ubootgl_gb300.simulation import Batch
    sizes = [(97, 49), (131, 67), (202, 101), (259, 130), (333, 111), (64, 33), (75, 41),
             (150, 75)]
    alone = [build(W, H, 500 + i, u_in=0.7 + 0.05 * i) for i, (W, H) in enumerate(sizes)]
    members = [build(W, H, 500 + i, u_in=0.7 + 0.05 * i) for i, (W, H) in enumerate(sizes)]
    batch = Batch(members)
    for _ in range(4):
        for s in alone:
            s.step_cfl(0.5)
        batch.step(cfl=0.5)
    batch.sync()
    for a, b in zip(alone, members):
        for n in ("vx", "vy", "vx_back", "vy_back", "p"):
            assert np.array_equal(a.get(n), b.get(n)), (a.width, n)
    batch.close()
    for s in alone + members:
        s.close()
