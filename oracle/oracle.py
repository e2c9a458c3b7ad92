"""ctypes front end of the test oracle -- TEST INFRASTRUCTURE ONLY.

PortSim     -- the CPU restatement (ubg_oracle.c), REAL=float or REAL=double.
RefSim      -- the reference's own Simulation (simulation.cpp,
               pressure_solver.cpp of te42kyfo/ubootgl) built by
               ref/build_ref.py; present only where that build can run
               (x86-64 with the reference checkout).
Both expose the same methods, so tests can swap one for the other.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

FIELD = {"vx": 0, "vy": 1, "vx_back": 2, "vy_back": 3, "p": 4, "f": 5, "flag": 6,
         "vx_accum": 7, "vy_accum": 8}

_port = None
_port_fast = None
_ref = None


def _fp(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def port_lib(fast=False):
    """The restatement built for parity (default) or, with fast, the same
    sources built for speed (the CPU baseline timing only)."""
    global _port, _port_fast
    if fast:
        if _port_fast is None:
            _port_fast = _bind_port(C.CDLL(build_oracle.build(fast=True)))
        return _port_fast
    if _port is None:
        _port = _bind_port(C.CDLL(build_oracle.build()))
    return _port


def _bind_port(lib):
    for sfx, ct in (("f", C.c_float), ("d", C.c_double)):
        P = C.POINTER(ct)
        g = lambda n: getattr(lib, "ubo_%s_%s" % (sfx, n))
        g("create").restype = C.c_void_p
        g("create").argtypes = [P, C.c_int, C.c_int, ct, ct]
        g("destroy").argtypes = [C.c_void_p]
        for n in ("step",):
            g(n).argtypes = [C.c_void_p, ct]
        g("step_ncycles").argtypes = [C.c_void_p, ct, C.c_int]
        g("set_dt").argtypes = [C.c_void_p, ct]
        for n in ("apply_accum", "diffuse", "advect", "set_vbcs", "set_pbc", "project"):
            g(n).argtypes = [C.c_void_p]
        g("project_ncycles").argtypes = [C.c_void_p, C.c_int]
        g("project_opts").argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        g("sim_mg_solve").argtypes = [C.c_void_p, C.c_int]
        g("get_field").argtypes = [C.c_void_p, C.c_int, P]
        g("set_field").argtypes = [C.c_void_p, C.c_int, P]
        g("update_flag").argtypes = [C.c_void_p, P]
        g("get_h").restype = ct
        g("get_h").argtypes = [C.c_void_p]
        g("mg_levels").argtypes = [C.c_void_p]
        g("mg_level_flag").argtypes = [C.c_void_p, C.c_int, P]
        g("mg_level_size").argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int),
                                       C.POINTER(C.c_int)]
        g("add_sink").argtypes = [C.c_void_p, ct, ct, ct]
        g("mg_create").restype = C.c_void_p
        g("mg_create").argtypes = [C.c_int, C.c_int, P]
        g("mg_destroy").argtypes = [C.c_void_p]
        g("mg_nlevels").argtypes = [C.c_void_p]
        g("mg_solve").argtypes = [C.c_void_p, P, P, P, ct, C.c_int]
        g("rbgs").argtypes = [P, P, P, C.c_int, C.c_int, ct, ct]
        g("residual").restype = C.c_double
        g("residual").argtypes = [P, P, P, P, C.c_int, C.c_int, ct]
        g("set_advect_bilinear").argtypes = [C.c_void_p, C.c_int]
        g("bilinear_sample").restype = ct
        g("bilinear_sample").argtypes = [P, C.c_int, C.c_int, ct, ct]
        g("advect_mask_vx").argtypes = [P, C.c_int, C.c_int, C.c_int]
        g("advect_mask_vy").argtypes = [P, C.c_int, C.c_int, C.c_int]
    lib.ubo_omp_set_threads.argtypes = [C.c_int]
    if hasattr(lib, "ubo_tracers_f_step"):
        _bind_tracers(lib)
    return lib


def _bind_tracers(lib):
    P = C.POINTER(C.c_float)
    U = C.POINTER(C.c_uint32)
    lib.ubo_tracers_f_step.argtypes = [P, P, C.c_int, C.c_int, P, C.c_int, C.c_int, C.c_int,
                                       C.c_int, U, U, P, C.c_float, C.c_float, C.c_float,
                                       C.c_uint32]
    lib.ubo_velocity_texture_f.argtypes = [P, P, C.c_int, C.c_int, P, P]


def velocity_texture(vx, vy):
    """interp_shader.cs restated: (vxy (2H-1, 2W-1, 2), mag (2H-1, 2W-1))."""
    lib = port_lib()
    H, W = vy.shape[0] + 1, vy.shape[1]
    vx = np.ascontiguousarray(vx, np.float32)
    vy = np.ascontiguousarray(vy, np.float32)
    vxy = np.zeros((2 * H - 1, 2 * W - 1, 2), np.float32)
    mag = np.zeros((2 * H - 1, 2 * W - 1), np.float32)
    lib.ubo_velocity_texture_f(_fp(vx, C.c_float), _fp(vy, C.c_float), W, H,
                               _fp(vxy, C.c_float), _fp(mag, C.c_float))
    return vxy, mag


def tracers_step(points, start, end, ages, vxy, flag, dt, pdim, rand_seed):
    """advect_tracer_points.cs restated; arrays are updated in place."""
    lib = port_lib()
    ntr, npts = points.shape[0], points.shape[1]
    th, tw = vxy.shape[0], vxy.shape[1]
    nfy, nfx = flag.shape
    lib.ubo_tracers_f_step(_fp(points, C.c_float), _fp(vxy, C.c_float), tw, th,
                           _fp(np.ascontiguousarray(flag, np.float32), C.c_float), nfx, nfy, ntr,
                           npts, start.ctypes.data_as(C.POINTER(C.c_uint32)),
                           end.ctypes.data_as(C.POINTER(C.c_uint32)), _fp(ages, C.c_float),
                           dt, pdim[0], pdim[1], rand_seed)


def ref_available():
    from .ref import build_ref
    return build_ref.available()


def ref_lib():
    global _ref
    if _ref is None:
        from .ref import build_ref
        lib = C.CDLL(build_ref.build())
        P = C.POINTER(C.c_float)
        lib.ref_create.restype = C.c_void_p
        lib.ref_create.argtypes = [P, C.c_int, C.c_int, C.c_float, C.c_float]
        lib.ref_destroy.argtypes = [C.c_void_p]
        lib.ref_set_field.argtypes = [C.c_void_p, C.c_int, P]
        lib.ref_get_field.argtypes = [C.c_void_p, C.c_int, P]
        lib.ref_update_flag.argtypes = [C.c_void_p, P]
        lib.ref_get_h.restype = C.c_float
        lib.ref_get_h.argtypes = [C.c_void_p]
        lib.ref_set_dt.argtypes = [C.c_void_p, C.c_float]
        lib.ref_step.argtypes = [C.c_void_p, C.c_float]
        for n in ("apply_accum", "diffuse", "advect", "set_vbcs", "set_pbc", "project"):
            getattr(lib, "ref_" + n).argtypes = [C.c_void_p]
        lib.ref_mg_solve_sim.argtypes = [C.c_void_p, C.c_int]
        lib.ref_add_sink.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float]
        lib.ref_mg_create.restype = C.c_void_p
        lib.ref_mg_create.argtypes = [C.c_int, C.c_int, P]
        lib.ref_mg_destroy.argtypes = [C.c_void_p]
        lib.ref_mg_solve.argtypes = [C.c_void_p, P, P, P, C.c_int, C.c_int, C.c_float, C.c_int]
        lib.ref_rbgs.argtypes = [P, P, P, C.c_int, C.c_int, C.c_float]
        lib.ref_residual.restype = C.c_float
        lib.ref_residual.argtypes = [P, P, P, P, C.c_int, C.c_int, C.c_float]
        lib.ref_set_threads.argtypes = [C.c_int]
        lib.ref_bilinear_sample_n.argtypes = [P, C.c_int, C.c_int, C.c_int, P, P]
        lib.ref_bilinear_scatter_n.argtypes = [P, C.c_int, C.c_int, C.c_int, P, P]
        lib.ref_set_grids.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float]
        _ref = lib
    return _ref


def field_shape(name, W, H):
    if name in ("vx", "vx_back", "vx_accum"):
        return (H, W - 1)
    if name in ("vy", "vy_back", "vy_accum"):
        return (H - 1, W)
    return (H, W)


class PortSim:
    """The CPU restatement's Simulation (dtype float32 or float64)."""

    def __init__(self, flag, pwidth=1.0, mu=1e-4, dtype=np.float32, fast=False):
        self.lib = port_lib(fast)
        self.dtype = np.dtype(dtype)
        self.sfx = "f" if self.dtype == np.float32 else "d"
        self.ct = C.c_float if self.sfx == "f" else C.c_double
        flag = np.ascontiguousarray(flag, dtype=self.dtype)
        self.H, self.W = flag.shape
        self.h_ = self._fn("create")(_fp(flag, self.ct), self.W, self.H, pwidth, mu)
        if not self.h_:
            raise ValueError("oracle create failed")

    def _fn(self, n):
        return getattr(self.lib, "ubo_%s_%s" % (self.sfx, n))

    def __del__(self):
        if getattr(self, "h_", None):
            self._fn("destroy")(self.h_)
            self.h_ = None

    @property
    def h(self):
        return self._fn("get_h")(self.h_)

    def get(self, name):
        out = np.empty(field_shape(name, self.W, self.H), dtype=self.dtype)
        self._fn("get_field")(self.h_, FIELD[name], _fp(out, self.ct))
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        assert a.shape == field_shape(name, self.W, self.H), (name, a.shape)
        self._fn("set_field")(self.h_, FIELD[name], _fp(a, self.ct))

    def update_flag(self, flag):
        a = np.ascontiguousarray(flag, dtype=self.dtype)
        self._fn("update_flag")(self.h_, _fp(a, self.ct))

    def step(self, dt, ncycles=2):
        self._fn("step_ncycles")(self.h_, dt, ncycles)

    def set_dt(self, dt):
        self._fn("set_dt")(self.h_, dt)

    def stage(self, name):
        self._fn(name)(self.h_)

    def mg_solve(self, zgbc=True):
        self._fn("sim_mg_solve")(self.h_, 1 if zgbc else 0)

    def project(self, ncycles=2, meanfree=False, zgbc_first=False):
        """project() with `ncycles` V-cycles (simulation.cpp:164-208).
        meanfree: subtract the mean of f over the interior fluid cells first
        (the tolerance modes' compatible system); zgbc_first: zero-gradient
        edges on p before the first V-cycle (the mixed solver's start)."""
        self._fn("project_opts")(self.h_, ncycles, 1 if meanfree else 0, 1 if zgbc_first else 0)

    def add_sink(self, x, y, z):
        self._fn("add_sink")(self.h_, x, y, z)

    def set_advect_bilinear(self, on=True):
        """Advection samples with bilinearSample instead of bicubicSample
        (the extension's option; the reference advects bicubically)."""
        self._fn("set_advect_bilinear")(self.h_, 1 if on else 0)

    def levels(self):
        return self._fn("mg_levels")(self.h_)

    def level_flag(self, level):
        w, h = C.c_int(), C.c_int()
        self._fn("mg_level_size")(self.h_, level, C.byref(w), C.byref(h))
        out = np.empty((h.value, w.value), dtype=self.dtype)
        self._fn("mg_level_flag")(self.h_, level, _fp(out, self.ct))
        return out


class RefSim:
    """The reference's own Simulation, compiled from its sources (float32)."""

    def __init__(self, flag, pwidth=1.0, mu=1e-4, threads=None):
        self.lib = ref_lib()
        flag = np.ascontiguousarray(flag, dtype=np.float32)
        self.H, self.W = flag.shape
        self.dtype = np.dtype(np.float32)
        self.set_threads(threads)
        self.h_ = self.lib.ref_create(_fp(flag, C.c_float), self.W, self.H, pwidth, mu)

    def set_threads(self, threads=None):
        # Classic (deterministic) red-black schedule needs H/threads < 100 at
        # every level with H >= 20 (pressure_solver.cpp:52, 65).
        if threads is None:
            threads = max(1, self.H // 100 + 1)
        self.lib.ref_set_threads(threads)

    def __del__(self):
        if getattr(self, "h_", None):
            self.lib.ref_destroy(self.h_)
            self.h_ = None

    @property
    def h(self):
        return self.lib.ref_get_h(self.h_)

    def get(self, name):
        out = np.empty(field_shape(name, self.W, self.H), dtype=np.float32)
        self.lib.ref_get_field(self.h_, FIELD[name], _fp(out, C.c_float))
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        assert a.shape == field_shape(name, self.W, self.H), (name, a.shape)
        self.lib.ref_set_field(self.h_, FIELD[name], _fp(a, C.c_float))

    def update_flag(self, flag):
        a = np.ascontiguousarray(flag, dtype=np.float32)
        self.lib.ref_update_flag(self.h_, _fp(a, C.c_float))

    def step(self, dt, ncycles=2):
        assert ncycles == 2, "the reference always runs two V-cycles"
        self.lib.ref_step(self.h_, dt)

    def set_dt(self, dt):
        self.lib.ref_set_dt(self.h_, dt)

    def stage(self, name):
        getattr(self.lib, "ref_" + name)(self.h_)

    def mg_solve(self, zgbc=True):
        self.lib.ref_mg_solve_sim(self.h_, 1 if zgbc else 0)

    def add_sink(self, x, y, z):
        self.lib.ref_add_sink(self.h_, x, y, z)

    def set_grids(self, x, y, val):
        self.lib.ref_set_grids(self.h_, x, y, val)


def port_mg_solve(p, f, flag, h, zgbc=False, coarse_flag=None, dtype=np.float32):
    """Standalone MG::solve on copies (class MG, pressure_solver.hpp:13-76).
    coarse_flag=None builds MG(width, height) (all coarse flags 1.0, as
    mgtest does); otherwise MG(coarse_flag)."""
    lib = port_lib()
    sfx = "f" if np.dtype(dtype) == np.float32 else "d"
    ct = C.c_float if sfx == "f" else C.c_double
    g = lambda n: getattr(lib, "ubo_%s_%s" % (sfx, n))
    Hh, Ww = p.shape
    pp = np.ascontiguousarray(p, dtype=dtype).copy()
    ff = np.ascontiguousarray(f, dtype=dtype)
    fl = np.ascontiguousarray(flag, dtype=dtype)
    cf = None if coarse_flag is None else np.ascontiguousarray(coarse_flag, dtype=dtype)
    mg = g("mg_create")(Ww, Hh, None if cf is None else _fp(cf, ct))
    try:
        g("mg_solve")(mg, _fp(pp, ct), _fp(ff, ct), _fp(fl, ct), h, 1 if zgbc else 0)
    finally:
        g("mg_destroy")(mg)
    return pp


def ref_mg_solve(p, f, flag, h, zgbc=False, coarse_flag=None, threads=None):
    lib = ref_lib()
    Hh, Ww = p.shape
    lib.ref_set_threads(threads or max(1, Hh // 100 + 1))
    pp = np.ascontiguousarray(p, dtype=np.float32).copy()
    ff = np.ascontiguousarray(f, dtype=np.float32)
    fl = np.ascontiguousarray(flag, dtype=np.float32)
    cf = None if coarse_flag is None else np.ascontiguousarray(coarse_flag, dtype=np.float32)
    mg = lib.ref_mg_create(Ww, Hh, None if cf is None else _fp(cf, C.c_float))
    try:
        lib.ref_mg_solve(mg, _fp(pp, C.c_float), _fp(ff, C.c_float), _fp(fl, C.c_float), Ww, Hh,
                         h, 1 if zgbc else 0)
    finally:
        lib.ref_mg_destroy(mg)
    return pp


def port_residual(p, f, flag, h, dtype=np.float32):
    lib = port_lib()
    sfx = "f" if np.dtype(dtype) == np.float32 else "d"
    ct = C.c_float if sfx == "f" else C.c_double
    Hh, Ww = p.shape
    a = [np.ascontiguousarray(x, dtype=dtype) for x in (p, f, flag)]
    r = np.zeros((Hh, Ww), dtype=dtype)
    n = getattr(lib, "ubo_%s_residual" % sfx)(*[_fp(x, ct) for x in a], _fp(r, ct), Ww, Hh, h)
    return r, n


def set_threads(n, fast=False):
    port_lib(fast).ubo_omp_set_threads(n)


# ---------------------------------------------------------------------------
# Game-side field access, restated in numpy float32 scalar arithmetic in the
# reference's evaluation order (test infrastructure only).

def _f32(v):
    return np.float32(v)


def bilinear_sample(grid, cx, cy):
    """bilinearSample, interpolators.hpp:11-27 (grid indexed [y, x])."""
    gh, gw = grid.shape
    cx = min(max(_f32(cx), _f32(0.0)), _f32(gw) - _f32(1.1))
    cy = min(max(_f32(cy), _f32(0.0)), _f32(gh) - _f32(1.1))
    ix, iy = int(cx), int(cy)
    sx, sy = cx - np.floor(cx), cy - np.floor(cy)
    v1, v2 = grid[iy, ix], grid[iy, ix + 1]
    v3, v4 = grid[iy + 1, ix], grid[iy + 1, ix + 1]
    vm1 = v1 + (v2 - v1) * sx
    vm2 = v3 + (v4 - v3) * sx
    return vm1 + (vm2 - vm1) * sy


def port_bilinear_sample(grid, cx, cy):
    """The C restatement's bilinearSample (the advection option's sampler)."""
    g = np.ascontiguousarray(grid, dtype=np.float32)
    gh, gw = g.shape
    return np.float32(port_lib().ubo_f_bilinear_sample(_fp(g, C.c_float), gw, gh,
                                                       np.float32(cx), np.float32(cy)))


def bilinear_scatter(grid, cx, cy, v):
    """bilinearScatter, interpolators.hpp:29-40 (in place)."""
    gh, gw = grid.shape
    cx = min(max(_f32(cx), _f32(0.0)), _f32(gw) - _f32(1.1))
    cy = min(max(_f32(cy), _f32(0.0)), _f32(gh) - _f32(1.1))
    ix, iy = int(cx), int(cy)
    sx, sy = cx - np.floor(cx), cy - np.floor(cy)
    ax, ay = _f32(1.0) - sx, _f32(1.0) - sy
    v = _f32(v)
    grid[iy + 1, ix + 1] += sx * sy * v
    grid[iy + 1, ix] += ax * sy * v
    grid[iy, ix + 1] += sx * ay * v
    grid[iy, ix] += ax * ay * v


def bilinear_vel(vx, vy, cx, cy):
    """Simulation::bilinearVel, advect_floating_items.cpp:11-14."""
    return (bilinear_sample(vx, _f32(cx) - _f32(0.5), _f32(cy) - _f32(0.0)),
            bilinear_sample(vy, _f32(cx) - _f32(0.0), _f32(cy) - _f32(0.5)))


def scatter_items(vx_accum, vy_accum, xy, v):
    """The floating items' force transfer, advect_floating_items.cpp:116-120."""
    for (cx, cy), (a, b) in zip(xy, v):
        bilinear_scatter(vx_accum, _f32(cx) - _f32(0.5), _f32(cy) - _f32(0.0), a)
        bilinear_scatter(vy_accum, _f32(cx) - _f32(0.0), _f32(cy) - _f32(0.5), b)


def set_grids(fields, x, y, val):
    """Simulation::setGrids, simulation.hpp:82-98; fields: dict of flag, vx,
    vy, p (front buffers), modified in place."""
    flag = fields["flag"]
    H, W = flag.shape
    if not (x >= 0 and y >= 0 and x < W and y < H):
        return
    flag[y, x] = val
    if val == 0:
        if x < W - 1:
            fields["vx"][y, x] = 0.0
        if x > 0:
            fields["vx"][y, x - 1] = 0.0
        if y < H - 1:
            fields["vy"][y, x] = 0.0
        if y > 0:
            fields["vy"][y - 1, x] = 0.0
        fields["p"][y, x] = 0.0


def shift_map(fields, new_flag):
    """UbootGlApp::shiftMap, ubootgl_app.cpp:245-298; fields: dict of vx,
    vx_back, vy, vy_back, p, flag (float32), modified in place."""
    for c in ("vx", "vy"):
        f, b = fields[c], fields[c + "_back"]
        w = f.shape[1]
        for x in range(2, w):
            f[:, x - 1] = f[:, x]
            b[:, x - 1] = f[:, x]
    p = fields["p"]
    for x in range(1, p.shape[1]):
        p[:, x - 1] = p[:, x]
    H, W = new_flag.shape
    for y in range(H):
        for x in range(W):
            set_grids(fields, x, y, new_flag[y, x])
    area = np.float32(1.0)
    for y in range(fields["vy"].shape[0]):
        area = np.float32(area + fields["flag"][y, 0])
    for y in range(fields["vx"].shape[0]):
        u = np.float32(np.float32(0.07) * np.float32(H)) / area
        fields["vx"][y, 0] = fields["vx_back"][y, 0] = np.float32(u * fields["flag"][y, 0])
