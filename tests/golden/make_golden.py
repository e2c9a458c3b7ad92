"""Generates the golden fixtures in this directory from the reference itself.

Runs te42kyfo/ubootgl's own Simulation::step / MG::solve (simulation.cpp and
pressure_solver.cpp compiled from the reference checkout by
oracle/ref/build_ref.py, classic red-black schedule) on seeded synthetic
inputs and stores inputs and outputs as compressed .npz files:

  step_<W>x<H>.npz   flag, initial vx / vy, the dt of every step, and vx,
                     vy, p after the steps listed in `kept` of a short run
  stages_130x66.npz  one step taken stage by stage (diffuse, advect,
                     setVBCs, project, setVBCs): all fields after each stage
  levels_257x129.npz the multigrid flag hierarchy (MG::updateFields)
  mg_laplace_65.npz  mgtest.cpp's Laplace problem (sinh(pi y) sin(pi x)
                     Dirichlet data, all flags 1, MG(N, N)) after 5 V-cycles
  long_1024x512.npz  the 1024x512, 12-disc flow of the benchmark's first
                     configuration over 100 steps: the dt of every step and,
                     after steps 0, 24, 49, 74 and 99, sampled rows and
                     columns of vx, vy and p plus their sum, L2 norm and
                     max|.| (the full fields would be 6 MB per kept step).
                     The inputs are regenerated from their seeds by the
                     test; a SHA-256 of them is stored to prove it.

Run from the repository root on an x86-64 machine with the reference
checkout:  python tests/golden/make_golden.py [steps|stages|levels|mgtest|long ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from ubootgl_gb300 import workload as WL  # noqa: E402

STEP_CASES = [(64, 32, 5, 101), (130, 66, 6, 102), (256, 128, 10, 103), (200, 40, 5, 104)]


def run_steps(W, H, nsteps, seed):
    flag = WL.disc_flag(W, H, n_discs=6, seed=seed)
    vx0, vy0 = WL.initial_velocity(flag, seed=seed + 1)
    ref = O.RefSim(flag, 1.0, 1e-4)
    for n, a in (("vx", vx0), ("vy", vy0), ("vx_back", vx0), ("vy_back", vy0)):
        ref.set(n, a)
    dts, vxs, vys, ps = [], [], [], []
    for _ in range(nsteps):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        ref.step(dt)
        dts.append(dt)
        vxs.append(ref.get("vx"))
        vys.append(ref.get("vy"))
        ps.append(ref.get("p"))
    kept = [0, nsteps // 2, nsteps - 1] if W * H > 64 * 64 else list(range(nsteps))
    np.savez_compressed(os.path.join(HERE, "step_%dx%d.npz" % (W, H)), flag=flag, vx0=vx0, vy0=vy0,
                        dt=np.array(dts, np.float32), kept=np.array(kept),
                        vx=np.stack([vxs[k] for k in kept]), vy=np.stack([vys[k] for k in kept]),
                        p=np.stack([ps[k] for k in kept]), h=np.float32(ref.h))


LONG = dict(W=1024, H=512, steps=100, seed=2024, kept=(0, 24, 49, 74, 99),
            rows=(100, 256, 400), cols=(300, 700))


def long_inputs():
    W, H, seed = LONG["W"], LONG["H"], LONG["seed"]
    flag = WL.disc_flag(W, H, n_discs=12, r_range=(20, 60), seed=seed)
    vx0, vy0 = WL.initial_velocity(flag, seed=seed + 1)
    return flag, vx0, vy0


def inputs_digest(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, np.float32).tobytes())
    return h.hexdigest()


def samples(a):
    a64 = a.astype(np.float64)
    rows = np.stack([a[r] for r in LONG["rows"]])
    cols = np.stack([a[:, c] for c in LONG["cols"]])
    stats = np.array([a64.sum(), np.sqrt((a64 * a64).sum()), np.abs(a64).max()])
    return rows, cols, stats


def run_long():
    flag, vx0, vy0 = long_inputs()
    ref = O.RefSim(flag, 1.0, 1e-4)
    for n, a in (("vx", vx0), ("vy", vy0), ("vx_back", vx0), ("vy_back", vy0)):
        ref.set(n, a)
    out = {"digest": np.array(inputs_digest(flag, vx0, vy0)), "kept": np.array(LONG["kept"])}
    dts = []
    for k in range(LONG["steps"]):
        dt = WL.cfl_dt(ref.get("vx"), ref.get("vy"), ref.h)
        ref.step(dt)
        dts.append(dt)
        if k in LONG["kept"]:
            for n in ("vx", "vy", "p"):
                rows, cols, stats = samples(ref.get(n))
                out["%s_rows_%d" % (n, k)] = rows
                out["%s_cols_%d" % (n, k)] = cols
                out["%s_stats_%d" % (n, k)] = stats
    out["dt"] = np.array(dts, np.float32)
    np.savez_compressed(os.path.join(HERE, "long_1024x512.npz"), **out)


def run_stages():
    W, H, seed = 130, 66, 105
    flag = WL.disc_flag(W, H, n_discs=6, seed=seed)
    vx0, vy0 = WL.initial_velocity(flag, seed=seed + 1)
    ref = O.RefSim(flag, 1.0, 1e-4)
    for n, a in (("vx", vx0), ("vy", vy0), ("vx_back", vx0), ("vy_back", vy0)):
        ref.set(n, a)
    dt = WL.cfl_dt(vx0, vy0, ref.h)
    ref.set_dt(dt)
    out = {"flag": flag, "vx0": vx0, "vy0": vy0, "dt": np.float32(dt)}
    for key in ("diffuse", "advect", "set_vbcs", "project", "set_vbcs2"):
        ref.stage(key.rstrip("2"))
        for n in ("vx", "vy", "vx_back", "vy_back", "p", "f"):
            out["%s_%s" % (key, n)] = ref.get(n)
    np.savez_compressed(os.path.join(HERE, "stages_130x66.npz"), **out)


def run_levels():
    # MG(flag)'s coarse flags are private to the reference's class; they are
    # pinned through a solve that depends on every one of them.
    W, H = 257, 129
    flag = WL.disc_flag(W, H, n_discs=8, seed=106)
    rng = np.random.default_rng(107)
    f = rng.standard_normal((H, W)).astype(np.float32)
    p0 = np.zeros((H, W), np.float32)
    h = np.float32(1.0 / (W - 1))
    p = O.ref_mg_solve(p0, f, flag, h, zgbc=True, coarse_flag=flag)
    np.savez_compressed(os.path.join(HERE, "levels_257x129.npz"), flag=flag, f=f, p=p, h=h)


def run_mgtest():
    N = 65
    h = np.float32(1.0 / (N - 1))
    u = np.zeros((N, N), np.float32)
    x = np.arange(N)
    u[N - 1, 1:N - 1] = (np.sinh(np.pi) * np.sin(x[1:N - 1] / (N - 1.0) * np.pi)).astype(np.float32)
    rhs = np.zeros((N, N), np.float32)
    flag = np.ones((N, N), np.float32)
    lib = O.ref_lib()
    lib.ref_set_threads(1)
    mg = lib.ref_mg_create(N, N, None)
    cycles = []
    ptr = lambda a: a.ctypes.data_as(O.C.POINTER(O.C.c_float))
    for _ in range(5):
        lib.ref_mg_solve(mg, ptr(u), ptr(rhs), ptr(flag), N, N, h, 0)
        cycles.append(u.copy())
    lib.ref_mg_destroy(mg)
    np.savez_compressed(os.path.join(HERE, "mg_laplace_65.npz"), u=np.stack(cycles), h=h)


if __name__ == "__main__":
    if not O.ref_available():
        sys.exit("the reference checkout (x86-64) is needed to generate fixtures")
    only = sys.argv[1:]
    if not only or "steps" in only:
        for case in STEP_CASES:
            run_steps(*case)
    if not only or "stages" in only:
        run_stages()
    if not only or "levels" in only:
        run_levels()
    if not only or "mgtest" in only:
        run_mgtest()
    if not only or "long" in only:
        run_long()
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(HERE, fn)))
