"""Seeded synthetic workloads for the ubootgl fluid step.

The reference's game builds its flag mask from a level PNG
(terrain.cpp:20-49) and its velocity from the simulation's constructor
(simulation.hpp:32-67).  Benchmarks and tests here use seeded synthetic
stand-ins with the shapes the step is quoted on:

* flag: 1 = fluid, 0 = solid; solid rows y = 0 and y = H-1 (no-slip walls),
  fluid inflow column x = 0 and outflow column x = W-1, plus seeded solid
  discs.  Values are exactly 0.0 or 1.0, like Terrain::subSample's output
  (terrain.cpp:3-11).
* velocity: vx = 1 + 0.1*n1, vy = 0.1*n2 with n1, n2 Gaussian-smoothed
  (sigma = 8 cells) white noise normalised to unit standard deviation; faces
  touching a solid cell are zeroed (the rule of Simulation::setGrids,
  simulation.hpp:82-98); inflow vx(0, y) = u_in on fluid rows.
* time step: dt = cfl * h / max|u| with cfl = 0.5, computed by the caller
  from the current fields.
"""
import math

import numpy as np


def disc_flag(W, H, n_discs=12, r_range=(20, 60), seed=0, solid_frac=None):
    """Channel with solid top/bottom rows and seeded solid discs.

    r_range is in cells for W = 1024 and scales with W / 1024, so the same
    flow set-up holds at every size.  With solid_frac, discs are added
    (rejection-free, one at a time) until the solid fraction reaches it.
    """
    rng = np.random.default_rng(seed)
    flag = np.ones((H, W), dtype=np.float32)
    flag[0, :] = 0.0
    flag[H - 1, :] = 0.0
    scale = W / 1024.0
    rmin, rmax = r_range[0] * scale, r_range[1] * scale
    yy, xx = np.mgrid[0:H, 0:W]

    def add_disc():
        r = rng.uniform(rmin, rmax)
        cx = rng.uniform(0.1 * W + r, 0.95 * W - r) if 0.85 * W > 2 * r else 0.5 * W
        cy = rng.uniform(r, H - r) if H > 2 * r else 0.5 * H
        y0, y1 = max(1, int(cy - r) - 1), min(H - 1, int(cy + r) + 2)
        x0, x1 = max(1, int(cx - r) - 1), min(W - 1, int(cx + r) + 2)
        sub = (xx[y0:y1, x0:x1] - cx) ** 2 + (yy[y0:y1, x0:x1] - cy) ** 2 <= r * r
        flag[y0:y1, x0:x1][sub] = 0.0

    if solid_frac is None:
        for _ in range(n_discs):
            add_disc()
    else:
        guard = 0
        while 1.0 - flag.mean() < solid_frac and guard < 100000:
            add_disc()
            guard += 1
    return flag


def _smooth_noise(rng, shape, sigma):
    from scipy.ndimage import gaussian_filter

    n = rng.standard_normal(shape).astype(np.float64)
    n = gaussian_filter(n, sigma=sigma, mode="wrap")
    s = n.std()
    return (n / (s if s > 0 else 1.0)).astype(np.float32)


def initial_velocity(flag, seed=1, amp=0.1, sigma=8.0, u_in=1.0):
    """Return (vx, vy) with shapes (H, W-1) and (H-1, W)."""
    H, W = flag.shape
    rng = np.random.default_rng(seed)
    vx = (1.0 + amp * _smooth_noise(rng, (H, W - 1), sigma)).astype(np.float32)
    vy = (amp * _smooth_noise(rng, (H - 1, W), sigma)).astype(np.float32)
    vx[:, 0] = u_in
    vx[:, :] *= flag[:, :-1] * flag[:, 1:]
    vy[:, :] *= flag[:-1, :] * flag[1:, :]
    vy[0, :] = 0.0
    return np.ascontiguousarray(vx), np.ascontiguousarray(vy)


def cfl_dt(vx, vy, h, cfl=0.5):
    """dt = cfl * h / max|u| over both staggered components, in float32
    arithmetic ((cfl * h) / umax with umax >= 1e-7), which is what the
    device-side CFL step computes."""
    f = np.float32
    umax = max(f(np.abs(vx).max()), f(np.abs(vy).max()))
    umax = umax if umax > f(1e-7) else f(1e-7)
    return f(f(f(cfl) * f(h)) / umax)


def grid_h(W, pwidth=1.0):
    """Simulation::h = pwidth / (width - 1.0f) (simulation.hpp:63), in float32."""
    return float(np.float32(pwidth) / (np.float32(W) - np.float32(1.0)))


def mg_levels(W, H):
    """Level sizes of MG(width, height), pressure_solver.hpp:16-31."""
    out = []
    while W > 3 and H > 3:
        out.append((W, H))
        W //= 2
        H //= 2
    return out


def batch_sizes(n, wmin=128, wmax=2048, seed=0, multiple=32):
    """Widths log-uniform in [wmin, wmax] rounded to `multiple`, height = w/2."""
    rng = np.random.default_rng(seed)
    ws = np.exp(rng.uniform(math.log(wmin), math.log(wmax), size=n))
    ws = np.clip((np.round(ws / multiple) * multiple).astype(int), wmin, wmax)
    return [(int(w), int(w) // 2) for w in ws]


# ---------------------------------------------------------------------------
# Many-instance workloads (batched and served simulations).

def log_uniform_widths(n, wmin, wmax, seed, multiple=32):
    """n widths drawn log-uniform in [wmin, wmax], rounded to `multiple`."""
    rng = np.random.default_rng(seed)
    w = np.exp(rng.uniform(math.log(wmin), math.log(wmax), n))
    return [int(max(wmin, min(wmax, multiple * round(x / multiple)))) for x in w]


def fast_velocity(flag, seed=1, amp=0.1, cell=8, u_in=1.0):
    """Like initial_velocity, with the smoothed noise made by bilinear
    up-sampling of white noise on a grid `cell` times coarser (a cheap
    stand-in for the Gaussian filter, for workloads of many instances)."""
    H, W = flag.shape
    rng = np.random.default_rng(seed)

    def noise(h, w):
        ch, cw = h // cell + 2, w // cell + 2
        c = rng.standard_normal((ch, cw))
        ys = np.linspace(0, ch - 1.001, h)
        xs = np.linspace(0, cw - 1.001, w)
        y0, x0 = ys.astype(int), xs.astype(int)
        fy, fx = (ys - y0)[:, None], (xs - x0)[None, :]
        a = c[y0][:, x0] * (1 - fx) + c[y0][:, x0 + 1] * fx
        b = c[y0 + 1][:, x0] * (1 - fx) + c[y0 + 1][:, x0 + 1] * fx
        n = a * (1 - fy) + b * fy
        return (n / max(n.std(), 1e-12)).astype(np.float32)

    vx = (1.0 + amp * noise(H, W - 1)).astype(np.float32)
    vy = (amp * noise(H - 1, W)).astype(np.float32)
    vx[:, 0] = u_in
    vx *= flag[:, :-1] * flag[:, 1:]
    vy *= flag[:-1, :] * flag[1:, :]
    vy[0, :] = 0.0
    return np.ascontiguousarray(vx), np.ascontiguousarray(vy)


def instance(W, H, seed, solid_range=(0.08, 0.15), u_in=None):
    """One instance of a many-instance workload: its own seeded disc mask
    with a solid fraction drawn from solid_range, its own inflow speed
    (uniform in [0.5, 1.5] unless given)."""
    rng = np.random.default_rng(seed)
    frac = rng.uniform(*solid_range)
    u = rng.uniform(0.5, 1.5) if u_in is None else u_in
    flag = disc_flag(W, H, seed=seed + 1, solid_frac=frac)
    vx, vy = fast_velocity(flag, seed=seed + 2, u_in=u)
    return flag, vx, vy


def seed_tracers(flag, ntr, npts, pdim, seed):
    """ntr tracer heads uniform over the fluid cells (positions in [0, pdim]);
    empty rings, ages uniform in [0, 2*pi) so that reseeding is spread out."""
    H, W = flag.shape
    rng = np.random.default_rng(seed)
    pts = np.zeros((ntr, npts, 2), np.float32)
    got = 0
    while got < ntr:
        n = 2 * (ntr - got)
        x = rng.uniform(0.0, 1.0, n)
        y = rng.uniform(0.0, 1.0, n)
        ok = flag[np.minimum((y * H).astype(int), H - 1), np.minimum((x * W).astype(int), W - 1)] > 0
        x, y = x[ok][:ntr - got], y[ok][:ntr - got]
        pts[got:got + len(x), 0, 0] = x * pdim[0]
        pts[got:got + len(x), 0, 1] = y * pdim[1]
        got += len(x)
    ages = rng.uniform(0.0, 6.28, ntr).astype(np.float32)
    return pts, np.zeros(ntr, np.uint32), np.zeros(ntr, np.uint32), ages
