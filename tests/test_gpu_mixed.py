"""Mixed-precision projection against FP64 oracle projections.

The pre-projection state (velocity after diffuse / advect / setVBCs, the
warm-start pressure of the previous step, dt) comes from the FP32 GPU path.
Each GPU result is compared with the CPU restatement of project()
(simulation.cpp:164-208) run in double with the same algorithm:

  fp32 (the drop-in, 2 V-cycles)   vs  FP64, 2 V-cycles
  fp16 / bf16 (2 defect corrections, each one 16-bit V-cycle)
                                   vs  FP64, 2 V-cycles from p with
                                       zero-gradient edges (the same
                                       iteration in exact arithmetic)

and the test states, over the interior fluid cells,

  e_p   = max |p' - p64'| / max |p64'|      (' = minus the mean: the solver's
                                             system fixes p up to a constant)
  e_div = ||D(u) - D(u64)||_2 / ||D(u_pre)||_2

with D the cell divergence of the staggered field in FP64.  The tolerances
are written in the tests.  The fixed mode runs the reference's two cycles,
so its 16-bit corrections leave their rounding in p (the bounds below say
how much); equal accuracy is the tolerance mode's contract, tested at the
end of this file.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ubootgl_gb300 import workload as WL

pytestmark = pytest.mark.gpu

# (e_p, e_div) bounds per mode.  Measured on GB300 at 512x256 after two
# cycles: fp32 3.3e-6 / 1.06e-5 (the rounding of the FP32 velocity faces),
# fp16 6.6e-4 / 2.8e-2, bf16 5.9e-3 / 2.0e-1: the last 16-bit correction's
# rounding is high-frequency noise in p, which the divergence sees through a
# discrete Laplacian.
TOL = {"fp32": (1e-5, 2e-5), "fp16": (2e-3, 0.1), "bf16": (2e-2, 0.5)}


def divergence64(vx, vy, flag):
    vx = vx.astype(np.float64)
    vy = vy.astype(np.float64)
    H, W = flag.shape
    d = np.zeros((H, W))
    d[1:H - 1, 1:W - 1] = (vx[1:H - 1, 1:W - 1] - vx[1:H - 1, 0:W - 2] +
                           vy[1:H - 1, 1:W - 1] - vy[0:H - 2, 1:W - 1])
    return d * (flag > 0)


def pre_projection_state(W, H, seed, warm_steps=2):
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(W, H, n_discs=8, seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1)
    sim = Simulation(flag, 1.0, 1e-4)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    for _ in range(warm_steps):
        sim.step(WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h))
    dt = WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h)
    sim.dt = dt
    sim.diffuse()
    sim.advect()
    sim.setVBCs()
    state = {n: sim.get(n) for n in ("vx", "vy", "vx_back", "vy_back", "p")}
    sim.close()
    return flag, state, dt


def project_gpu(flag, state, dt, precision, mode="fixed", vcycles=2, tol=1e-6, max_vcycles=60,
                graph=True):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    sim = Simulation(flag, 1.0, 1e-4)
    if mode == "tol":
        sim.set_options(solver_mode=L.SOLVE_TOLERANCE, tol=tol, max_vcycles=max_vcycles,
                        precision=precision)
    else:
        sim.set_options(solver_mode=L.SOLVE_FIXED, vcycles=vcycles, precision=precision,
                        use_graph=graph)
    for n, a in state.items():
        sim.set(n, a)
    sim.dt = dt
    sim.project()
    out = {n: sim.get(n) for n in ("vx", "vy", "p")}
    out["stats"] = sim.solver_stats()
    sim.close()
    return out


def project_fp64(flag, state, dt, ncycles=2, zgbc_first=False):
    ref = O.PortSim(flag, 1.0, 1e-4, dtype=np.float64)
    for n, a in state.items():
        ref.set(n, a.astype(np.float64))
    ref.set_dt(dt)
    ref.project(ncycles=ncycles, zgbc_first=zgbc_first)
    return {n: ref.get(n) for n in ("vx", "vy", "p")}


def errors(flag, state, out, ref):
    inner = np.zeros_like(flag, dtype=bool)
    inner[1:-1, 1:-1] = flag[1:-1, 1:-1] > 0
    p, p64 = out["p"].astype(np.float64)[inner], ref["p"][inner]
    p, p64 = p - p.mean(), p64 - p64.mean()
    e_p = np.abs(p - p64).max() / np.abs(p64).max()
    d0 = divergence64(state["vx"], state["vy"], flag)
    d = divergence64(out["vx"], out["vy"], flag)
    d64 = divergence64(ref["vx"], ref["vy"], flag)
    e_div = np.linalg.norm((d - d64)[inner]) / np.linalg.norm(d0[inner])
    return e_p, e_div


@pytest.fixture(scope="module")
def case_512(lib):
    flag, state, dt = pre_projection_state(512, 256, seed=31)
    refs = {"plain": project_fp64(flag, state, dt),
            "zgbc_first": project_fp64(flag, state, dt, zgbc_first=True)}
    return flag, state, dt, refs


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_projection_vs_fp64(case_512, precision):
    flag, state, dt, refs = case_512
    out = project_gpu(flag, state, dt, precision)
    ref = refs["plain" if precision == "fp32" else "zgbc_first"]
    e_p, e_div = errors(flag, state, out, ref)
    d0 = divergence64(state["vx"], state["vy"], flag)
    rel_div = np.linalg.norm(divergence64(out["vx"], out["vy"], flag)) / np.linalg.norm(d0)
    print("\n[mixed] 512x256 %s 2 cycles: e_p %.3e e_div %.3e (||D(u)||/||D(u_pre)|| %.3e)" %
          (precision, e_p, e_div, rel_div))
    assert out["stats"][0] == 2
    assert e_p <= TOL[precision][0]
    assert e_div <= TOL[precision][1]


# ------------------------------------------------------------ tolerance mode
# The tolerance solver (flexible CG preconditioned by the tolerance
# hierarchy's V-cycle, FP64 pressure iterate) on the zero-gradient system
# with the net edge flux moved to the outflow column x = W-2.  Its FP64
# oracle is exact: for the exact solution p64 of L p = -f_c, the gradient
# update (simulation.cpp:196-207) leaves D(u64) = D(u_pre) + h L p64 =
# -h (f - f_c), i.e. the divergence is zero except for the compatibility
# correction on the outflow column.  So
#   e_div = ||D(u) - D(u64)|| / ||D(u_pre)||
# is measured against that closed form at every size, and at 512x256 the
# pressure is also compared with an FP64 solve of the same system (scipy
# conjugate gradients on the cell graph Laplacian, independent of the
# multigrid code).  Bounds: the solver's own true residual <= tol, the 16-bit
# modes within 2x of FP32's e_div, and e_div <= 1e-5 beyond the floor that
# storing the velocity faces in FP32 sets by itself: each updated face is
# rounded once, an error of about ulp(u)^2 / 12 in variance, so
#   floor = sqrt(sum over cells of the variances of their four faces) / ||D(u_pre)||
# (the faces are near 1 in a channel flow, where ulp is 1.2e-7, while
# D(u_pre) shrinks with h: at 4096x2048 the floor alone is about 1e-5).
TOL_SOLVE = 1e-6
E_DIV_MAX = 1e-5


def fp32_floor(flag, state, out):
    """Expected e_div of an exact projection whose result is rounded to FP32
    once per updated face."""
    H, W = flag.shape
    fl = flag > 0
    var = np.zeros((H, W))
    ux = np.spacing(np.abs(out["vx"]).astype(np.float32)).astype(np.float64) ** 2 / 12.0
    uy = np.spacing(np.abs(out["vy"]).astype(np.float32)).astype(np.float64) ** 2 / 12.0
    mx = np.zeros_like(ux, dtype=bool)
    mx[1:H - 1, 1:W - 2] = fl[1:H - 1, 1:W - 2] & fl[1:H - 1, 2:W - 1]
    my = np.zeros_like(uy, dtype=bool)
    my[1:H - 2, 1:W - 1] = fl[1:H - 2, 1:W - 1] & fl[2:H - 1, 1:W - 1]
    ux, uy = ux * mx, uy * my
    var[1:H - 1, 1:W - 1] += ux[1:H - 1, 1:W - 1] + ux[1:H - 1, 0:W - 2]
    var[1:H - 1, 1:W - 1] += uy[1:H - 1, 1:W - 1] + uy[0:H - 2, 1:W - 1]
    inner = np.zeros_like(fl)
    inner[1:-1, 1:-1] = fl[1:-1, 1:-1]
    d0 = divergence64(state["vx"], state["vy"], flag)
    return np.sqrt(var[inner].sum()) / np.linalg.norm(d0[inner])


def compat_rhs(flag, state, h):
    """f = -D(u_pre)/h on the interior fluid cells and f_c (the solver's
    compatible right-hand side) in FP64."""
    H, W = flag.shape
    inner = np.zeros_like(flag, dtype=bool)
    inner[1:-1, 1:-1] = flag[1:-1, 1:-1] > 0
    f = -divergence64(state["vx"], state["vy"], flag) / h
    f[~inner] = 0.0
    col = inner[:, W - 2]
    fc = f.copy()
    if col.any():
        fc[col, W - 2] -= f[inner].sum() / col.sum()
    else:
        fc[inner] -= f[inner].mean()
    return inner, f, fc


def fp64_pressure(flag, fc, h):
    """FP64 solution of the zero-gradient system, scipy CG to 1e-12."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    H, W = flag.shape
    inner = np.zeros_like(flag, dtype=bool)
    inner[1:-1, 1:-1] = flag[1:-1, 1:-1] > 0
    idx = -np.ones((H, W), dtype=np.int64)
    n = int(inner.sum())
    idx[inner] = np.arange(n)
    rows, cols, vals = [], [], []
    diag = np.zeros(n)
    ys, xs = np.nonzero(inner)
    me = idx[ys, xs]
    for dy, dx in ((0, 1), (0, -1), (1, 0), (-1, 0)):
        ny, nx = ys + dy, xs + dx
        ok = inner[ny, nx]
        rows.append(me[ok])
        cols.append(idx[ny[ok], nx[ok]])
        vals.append(-np.ones(int(ok.sum())))
        diag[me[ok]] += 1.0
    A = sp.csr_matrix((np.concatenate(vals + [diag]),
                       (np.concatenate(rows + [np.arange(n)]), np.concatenate(cols + [np.arange(n)]))),
                      shape=(n, n)) / (h * h)
    b = fc[inner]
    Minv = sp.diags(np.where(A.diagonal() > 0, 1.0 / np.maximum(A.diagonal(), 1e-300), 0.0))
    try:
        x, info = sla.cg(A, b, rtol=1e-12, atol=0.0, maxiter=50000, M=Minv)
    except TypeError:  # scipy < 1.12 names the relative tolerance `tol`
        x, info = sla.cg(A, b, tol=1e-12, atol=0.0, maxiter=50000, M=Minv)
    p = np.zeros((H, W))
    p[inner] = x
    return p, np.linalg.norm(A @ x - b) / np.linalg.norm(b)


def tolerance_errors(flag, state, out, h):
    inner, f, fc = compat_rhs(flag, state, h)
    d0 = divergence64(state["vx"], state["vy"], flag)
    d = divergence64(out["vx"], out["vy"], flag)
    d64 = -h * (f - fc)
    e_div = np.linalg.norm((d - d64)[inner]) / np.linalg.norm(d0[inner])
    return inner, fc, e_div


@pytest.fixture(scope="module")
def tol_512(lib):
    flag, state, dt = pre_projection_state(512, 256, seed=31)
    h = WL.grid_h(512)
    res = {}
    for precision in ("fp32", "fp16", "bf16"):
        out = project_gpu(flag, state, dt, precision, mode="tol", tol=TOL_SOLVE, max_vcycles=100)
        inner, fc, e_div = tolerance_errors(flag, state, out, h)
        res[precision] = (out, e_div)
    p64, r64 = fp64_pressure(flag, fc, h)
    return flag, state, h, res, p64, r64


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_tolerance_solver_vs_fp64_512(tol_512, precision):
    from scipy import ndimage
    flag, state, h, res, p64, r64 = tol_512
    out, e_div = res[precision]
    cycles, rel = out["stats"]
    inner = np.zeros_like(flag, dtype=bool)
    inner[1:-1, 1:-1] = flag[1:-1, 1:-1] > 0
    # the pressure is fixed up to a constant on each connected fluid region
    lab, nreg = ndimage.label(inner)
    p = out["p"].astype(np.float64)
    dp = np.zeros_like(p)
    for k in range(1, nreg + 1):
        m = lab == k
        dp[m] = (p[m] - p[m].mean()) - (p64[m] - p64[m].mean())
    big = lab == np.bincount(lab[inner]).argmax()
    e_p = np.abs(dp[big]).max() / np.abs(p64[big] - p64[big].mean()).max()
    floor = fp32_floor(flag, state, out)
    print("\n[tol] 512x256 %s: %d V-cycles, ||r||/||f_c|| %.2e, e_div %.2e (FP32 floor %.2e), "
          "e_p %.2e (fp64 oracle residual %.1e)" % (precision, cycles, rel, e_div, floor, e_p, r64))
    assert r64 < 1e-9
    assert rel <= TOL_SOLVE
    assert e_div <= E_DIV_MAX
    assert e_p <= 1e-4
    assert e_div <= 2.0 * res["fp32"][1]
    assert cycles <= 2 * res["fp32"][0]["stats"][0] + 2


def test_tolerance_solver_4096(lib):
    """Config 3's grid: every precision reaches the tolerance, e_div beyond
    the FP32 velocity floor <= 1e-5 against the exact FP64 projection, 16-bit
    modes within 2x of FP32."""
    W, H = 4096, 2048
    flag, state, dt = pre_projection_state(W, H, seed=47, warm_steps=1)
    h = WL.grid_h(W)
    e = {}
    for precision in ("fp32", "fp16", "bf16"):
        out = project_gpu(flag, state, dt, precision, mode="tol", tol=TOL_SOLVE, max_vcycles=100)
        cycles, rel = out["stats"]
        _, _, e[precision] = tolerance_errors(flag, state, out, h)
        floor = fp32_floor(flag, state, out)
        print("\n[tol] %dx%d %s: %d V-cycles, ||r||/||f_c|| %.2e, e_div %.2e (FP32 floor %.2e)" %
              (W, H, precision, cycles, rel, e[precision], floor))
        assert np.isfinite(out["p"]).all()
        assert rel <= TOL_SOLVE
        assert e[precision] <= np.hypot(E_DIV_MAX, floor)
    for precision in ("fp16", "bf16"):
        assert e[precision] <= 2.0 * e["fp32"]


def test_tolerance_steps_stay_converged(lib):
    """Whole steps in tolerance mode: each projection reaches the tolerance
    from the previous step's pressure, in every precision."""
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    W, H = 256, 128
    flag = WL.disc_flag(W, H, n_discs=6, seed=5)
    vx, vy = WL.initial_velocity(flag, seed=6)
    for precision in ("fp32", "fp16", "bf16"):
        sim = Simulation(flag, 1.0, 1e-4)
        sim.set_options(solver_mode=L.SOLVE_TOLERANCE, tol=TOL_SOLVE, max_vcycles=100,
                        precision=precision)
        for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
            sim.set(n, a)
        for _ in range(4):
            sim.step(WL.cfl_dt(sim.get("vx"), sim.get("vy"), sim.h))
            cycles, rel = sim.solver_stats()
            assert 0 <= cycles <= 100 and rel <= TOL_SOLVE, (precision, cycles, rel)
        for n in ("vx", "vy", "p"):
            assert np.isfinite(sim.get(n)).all()
        sim.close()


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_mixed_fixed_graph_matches_direct(case_512, precision):
    flag, state, dt, _ = case_512
    a = project_gpu(flag, state, dt, precision, vcycles=3, graph=True)
    b = project_gpu(flag, state, dt, precision, vcycles=3, graph=False)
    for n in ("vx", "vy", "p"):
        assert np.array_equal(a[n], b[n]), n


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_mixed_steps_graph_and_direct(lib, precision):
    """Whole steps with the mixed solver in fixed mode: the captured graph
    and direct launches give identical fields, and the flow stays finite."""
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    W, H = 256, 128
    flag = WL.disc_flag(W, H, n_discs=6, seed=5)
    vx, vy = WL.initial_velocity(flag, seed=6)
    res = []
    for graph in (True, False):
        sim = Simulation(flag, 1.0, 1e-4)
        sim.set_options(solver_mode=L.SOLVE_FIXED, vcycles=2, precision=precision,
                        use_graph=graph)
        for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
            sim.set(n, a)
        for _ in range(5):
            sim.step(0.5 * sim.h / 1.2)
        res.append({n: sim.get(n) for n in ("vx", "vy", "p")})
        sim.close()
    for n in ("vx", "vy", "p"):
        assert np.isfinite(res[0][n]).all()
        assert np.array_equal(res[0][n], res[1][n]), n


def test_precision_option_errors(lib):
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation
    flag = WL.disc_flag(64, 32, n_discs=2, seed=1)
    sim = Simulation(flag, 1.0, 1e-4)
    with pytest.raises(L.UbgError) as e:
        sim.set_options(precision=7)
    assert e.value.code == -1
    sim.set_options(precision="bf16")
    sim.set_options(precision="fp32")
    sim.close()
