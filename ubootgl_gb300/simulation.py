"""Python mirror of the reference's Simulation and MG classes over the C ABI.

class Simulation   -- simulation.hpp:18-141 (constructor from a flag grid,
                      step, the stage methods, the public fields).
class MG           -- pressure_solver.hpp:13-76 (MG(width, height), MG(flag),
                      updateFields, solve).
rbgs, calculateResidualField -- the free functions of pressure_solver.hpp.

Fields are numpy float32 arrays indexed [y, x] (row-major, idx = y*width+x as
in db2dgrid.hpp:19).  Reads download from the device; assignments upload.
All compute runs in the CUDA library; there is no CPU path.
"""
import ctypes as C

import numpy as np

from . import _lib as L


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        raise ValueError("expected shape %s, got %s" % (shape, a.shape))
    return a


class Simulation:
    """Simulation(flag, pwidth, mu), simulation.hpp:32-67."""

    BC = L.BC

    def __init__(self, flag, pwidth=1.0, mu=1e-4):
        self._lib = L.load()
        flag = _f32(flag)
        self.height, self.width = flag.shape
        self.pwidth = float(np.float32(pwidth))
        self.mu = float(np.float32(mu))
        h = C.c_void_p()
        L.check(self._lib.ubg_create(L.fptr(flag), self.width, self.height, pwidth, mu,
                                     C.byref(h)))
        self._h = h
        self.dt = 0.0
        # h = pwidth / (width - 1.0f), simulation.hpp:63
        self.h = float(np.float32(pwidth) / (np.float32(self.width) - np.float32(1.0)))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ubg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------ options
    def set_options(self, solver_mode=None, vcycles=None, tol=None, max_vcycles=None,
                    use_graph=None, precision=None, advect=None):
        """Solver options (extension).  precision: "fp32", "fp16" or "bf16"
        (the mixed-precision defect-correction solver).  advect: "bicubic"
        (the reference) or "bilinear" (bilinearSample for the back-trace)."""
        o = L.Options()
        L.check(self._lib.ubg_default_options(C.byref(o)))
        cur = getattr(self, "_opts", None)
        if cur is not None:
            C.memmove(C.byref(o), C.byref(cur), C.sizeof(o))
        if precision is not None:
            o.precision = {"fp32": L.FP32, "fp16": L.MIXED_FP16,
                           "bf16": L.MIXED_BF16}.get(precision, precision)
        if solver_mode is not None:
            o.solver_mode = solver_mode
        if vcycles is not None:
            o.vcycles = vcycles
        if tol is not None:
            o.tol = tol
        if max_vcycles is not None:
            o.max_vcycles = max_vcycles
        if use_graph is not None:
            o.use_graph = int(use_graph)
        if advect is not None:
            o.advect_bilinear = {"bicubic": 0, "bilinear": 1}[advect]
        L.check(self._lib.ubg_set_options(self._h, C.byref(o)))
        self._opts = o

    def set_bcs(self, west="INFLOW", east="OUTFLOW_ZERO_PRESSURE", north="NOSLIP",
                south="NOSLIP"):
        L.check(self._lib.ubg_set_bcs(self._h, L.BC[west], L.BC[east], L.BC[north],
                                      L.BC[south]))

    # ------------------------------------------------------------ the step
    def step(self, timestep):
        """Simulation::step, simulation.cpp:356-374."""
        self.dt = timestep
        L.check(self._lib.ubg_step(self._h, timestep))

    def step_cfl(self, cfl=0.5):
        L.check(self._lib.ubg_step_cfl(self._h, cfl))

    def last_dt(self):
        v = C.c_float()
        L.check(self._lib.ubg_last_dt(self._h, C.byref(v)))
        return v.value

    def autotune(self):
        """Tunes the multigrid tiles and tail size (extension); returns the
        report as a dict."""
        import json
        buf = C.create_string_buffer(1 << 16)
        L.check(self._lib.ubg_autotune(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def snapshot(self):
        """Session state as bytes (ubg_snapshot)."""
        n = C.c_size_t()
        L.check(self._lib.ubg_snapshot_bytes(self._h, C.byref(n)))
        buf = (C.c_char * n.value)()
        L.check(self._lib.ubg_snapshot(self._h, buf))
        return bytes(buf)

    def restore(self, blob):
        buf = C.create_string_buffer(blob, len(blob))
        L.check(self._lib.ubg_restore(self._h, buf))

    def solver_stats(self):
        """(V-cycles or corrections of the last solve, final ||r||/||f|| in
        tolerance mode else -1)."""
        n, r = C.c_int(), C.c_double()
        L.check(self._lib.ubg_solver_stats(self._h, C.byref(n), C.byref(r)))
        return n.value, r.value

    def applyAccumulatedVelocity(self):
        L.check(self._lib.ubg_apply_accumulated_velocity(self._h))

    def diffuse(self):
        L.check(self._lib.ubg_diffuse(self._h, self.dt))

    def advect(self):
        L.check(self._lib.ubg_advect(self._h, self.dt))

    def setVBCs(self):
        L.check(self._lib.ubg_set_vbcs(self._h))

    def setPBC(self):
        L.check(self._lib.ubg_set_pbc(self._h))

    def project(self):
        L.check(self._lib.ubg_project(self._h, self.dt))

    def add_sink(self, x, y, strength):
        """sinks.push_back(glm::vec3(x, y, strength))."""
        L.check(self._lib.ubg_add_sink(self._h, x, y, strength))

    def mg_solve(self, zero_gradient_bc=True):
        L.check(self._lib.ubg_mg_solve_sim(self._h, int(zero_gradient_bc)))

    def sync(self):
        L.check(self._lib.ubg_sync(self._h))

    # ------------------------------------------------------------- fields
    def _shape(self, name):
        W, H = self.width, self.height
        if name.startswith("vx"):
            return (H, W - 1)
        if name.startswith("vy"):
            return (H - 1, W)
        return (H, W)

    def get(self, name):
        out = np.empty(self._shape(name), dtype=np.float32)
        L.check(self._lib.ubg_download(self._h, L.FIELDS[name], L.fptr(out)))
        return out

    def set(self, name, arr):
        a = _f32(arr, self._shape(name))
        L.check(self._lib.ubg_upload(self._h, L.FIELDS[name], L.fptr(a)))

    def update_flag(self, flag):
        """memcpy(sim.flag.data(), ...) + sim.mg.updateFields(sim.flag)."""
        self.set("flag", flag)

    def mg_levels(self):
        n = C.c_int()
        L.check(self._lib.ubg_mg_levels(self._h, C.byref(n)))
        return n.value

    def mg_level_flag(self, level):
        w, h = C.c_int(), C.c_int()
        L.check(self._lib.ubg_mg_level_flag(self._h, level, C.byref(w), C.byref(h), None))
        out = np.empty((h.value, w.value), dtype=np.float32)
        L.check(self._lib.ubg_mg_level_flag(self._h, level, None, None, L.fptr(out)))
        return out

    def device_field(self, name):
        """(device pointer, pitch in elements, width, height) of a field."""
        ptr, pitch, w, h = C.c_void_p(), C.c_int(), C.c_int(), C.c_int()
        L.check(self._lib.ubg_field_device(self._h, L.FIELDS[name], C.byref(ptr), C.byref(pitch),
                                           C.byref(w), C.byref(h)))
        return ptr.value, pitch.value, w.value, h.value

    def profile(self, on=True):
        L.check(self._lib.ubg_profile_enable(self._h, int(on)))

    def profile_reset(self):
        L.check(self._lib.ubg_profile_reset(self._h))

    def profile_classes(self):
        """{kernel class: (total ms, launches)} accumulated while profiling."""
        out = {}
        for kc in range(20):
            name, ms, n = C.c_char_p(), C.c_double(), C.c_int()
            L.check(self._lib.ubg_profile_class(self._h, kc, C.byref(name), C.byref(ms),
                                                C.byref(n)))
            if n.value:
                out[name.value.decode()] = (ms.value, n.value)
        return out

    def profile_read(self):
        sm, sl, st, kl = C.c_double(), C.c_int(), C.c_double(), C.c_int()
        L.check(self._lib.ubg_profile_read(self._h, C.byref(sm), C.byref(sl), C.byref(st),
                                           C.byref(kl)))
        return {"smoother_ms": sm.value, "smoother_launches": sl.value, "step_ms": st.value,
                "kernel_launches": kl.value}

    vx = property(lambda s: s.get("vx"), lambda s, a: s.set("vx", a))
    vy = property(lambda s: s.get("vy"), lambda s, a: s.set("vy", a))
    p = property(lambda s: s.get("p"), lambda s, a: s.set("p", a))
    f = property(lambda s: s.get("f"), lambda s, a: s.set("f", a))
    flag = property(lambda s: s.get("flag"), lambda s, a: s.set("flag", a))
    vx_current = property(lambda s: s.get("vx_current"))
    vy_current = property(lambda s: s.get("vy_current"))


class Batch:
    """Several simulations advanced by one CUDA graph launch per step
    (extension).  The members stay usable on their own."""

    def __init__(self, sims):
        self._lib = L.load()
        self.sims = list(sims)
        arr = (C.c_void_p * len(self.sims))(*[s._h.value for s in self.sims])
        h = C.c_void_p()
        L.check(self._lib.ubg_batch_create(len(self.sims), arr, C.byref(h)))
        self._h = h

    def step(self, dts=None, cfl=0.5):
        if dts is None:
            L.check(self._lib.ubg_batch_step(self._h, None, cfl))
        else:
            d = np.ascontiguousarray(dts, np.float32)
            assert d.shape == (len(self.sims),)
            L.check(self._lib.ubg_batch_step(self._h, L.fptr(d), cfl))

    def sync(self):
        L.check(self._lib.ubg_batch_sync(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ubg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Step server over resident sessions (extension; ubg_server_*)."""

    def __init__(self, budget_bytes, max_active=16, mode="fused", fuse_cells=None,
                 admission="reject"):
        """mode "fused": one step of every in-flight FP32 request of at most
        `fuse_cells` cells (library default 2^20) per launch sequence
        (continuous batching); "streams": each request's steps on its
        session's own stream.  admission "reject": an open over the memory
        budget returns None; "queue": it waits for closes to free memory."""
        self._lib = L.load()
        h = C.c_void_p()
        L.check(self._lib.ubg_server_create(int(budget_bytes), int(max_active), C.byref(h)))
        self._h = h
        L.check(self._lib.ubg_server_set_mode(h, {"streams": 0, "fused": 1}[mode]))
        L.check(self._lib.ubg_server_set_admission(h, {"reject": 0, "queue": 1}[admission]))
        if fuse_cells is not None:
            L.check(self._lib.ubg_server_set_fuse_cells(h, int(fuse_cells)))

    def open(self, flag, vx=None, vy=None, pwidth=1.0, mu=1e-4, precision="fp32", vcycles=2,
             tol=None, max_vcycles=100):
        """Returns the session id, or None when the memory budget rejects it.
        tol: the tolerance solver (relative residual) instead of `vcycles`
        fixed V-cycles."""
        flag = _f32(flag)
        H, W = flag.shape
        o = L.Options()
        L.check(self._lib.ubg_default_options(C.byref(o)))
        o.precision = {"fp32": L.FP32, "fp16": L.MIXED_FP16, "bf16": L.MIXED_BF16}[precision]
        o.vcycles = vcycles
        if tol is not None:
            o.solver_mode = L.SOLVE_TOLERANCE
            o.tol = tol
            o.max_vcycles = max_vcycles
        sid = C.c_int()
        rc = self._lib.ubg_server_open(
            self._h, L.fptr(flag), W, H, pwidth, mu,
            None if vx is None else L.fptr(_f32(vx, (H, W - 1))),
            None if vy is None else L.fptr(_f32(vy, (H - 1, W))), C.byref(o), C.byref(sid))
        if rc == -6:
            return None
        L.check(rc)
        return sid.value

    def close_session(self, sid):
        L.check(self._lib.ubg_server_close(self._h, sid))

    def submit(self, sid, steps, cfl=0.5):
        r = C.c_uint64()
        L.check(self._lib.ubg_server_submit(self._h, sid, steps, cfl, C.byref(r)))
        return r.value

    def wait(self, req):
        ms = C.c_double()
        L.check(self._lib.ubg_server_wait(self._h, req, C.byref(ms)))
        return ms.value

    def drain(self):
        L.check(self._lib.ubg_server_drain(self._h))

    def get(self, sid, name):
        """A field of an idle session."""
        h = C.c_void_p()
        L.check(self._lib.ubg_server_session_sim(self._h, sid, C.byref(h)))
        view = Simulation.__new__(Simulation)
        view._lib, view._h = self._lib, h
        W, H = C.c_int(), C.c_int()
        # level 0 of the multigrid gives the grid size
        L.check(self._lib.ubg_mg_level_flag(h, 0, C.byref(W), C.byref(H), None))
        view.width, view.height = W.value, H.value
        out = view.get(name)
        view._h = None
        return out

    def stats(self):
        st = L.ServeStats()
        L.check(self._lib.ubg_server_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in L.ServeStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ubg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tracers:
    """Fluid tracers of a Simulation (draw_tracers_cs.cpp GLTracers +
    advect_tracer_points.cs), device-resident."""

    def __init__(self, sim, ntracers, npoints=30):
        self._lib = L.load()
        self.sim = sim
        self.ntracers, self.npoints = int(ntracers), int(npoints)
        h = C.c_void_p()
        L.check(self._lib.ubg_tracers_create(sim._h, self.ntracers, self.npoints, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ubg_tracers_destroy(self._h)
            self._h = None

    def upload(self, points=None, start=None, end=None, ages=None):
        U = C.POINTER(C.c_uint32)
        pts = None if points is None else _f32(points, (self.ntracers, self.npoints, 2))
        st = None if start is None else np.ascontiguousarray(start, np.uint32)
        en = None if end is None else np.ascontiguousarray(end, np.uint32)
        ag = None if ages is None else _f32(ages, (self.ntracers,))
        L.check(self._lib.ubg_tracers_upload(
            self._h, None if pts is None else L.fptr(pts),
            None if st is None else st.ctypes.data_as(U),
            None if en is None else en.ctypes.data_as(U), None if ag is None else L.fptr(ag)))

    def download(self):
        U = C.POINTER(C.c_uint32)
        pts = np.empty((self.ntracers, self.npoints, 2), np.float32)
        st = np.empty(self.ntracers, np.uint32)
        en = np.empty(self.ntracers, np.uint32)
        ag = np.empty(self.ntracers, np.float32)
        L.check(self._lib.ubg_tracers_download(self._h, L.fptr(pts), st.ctypes.data_as(U),
                                               en.ctypes.data_as(U), L.fptr(ag)))
        return pts, st, en, ag

    def step(self, dt, rand_seed):
        """updateTracers (draw_tracers_cs.cpp:131-156)."""
        L.check(self._lib.ubg_tracers_step(self._h, dt, rand_seed))


def velocity_texture(sim):
    """interp_shader.cs on the simulation's current fields: (vxy, mag)."""
    lib = L.load()
    th, tw = 2 * sim.height - 1, 2 * sim.width - 1
    vxy = np.empty((th, tw, 2), np.float32)
    mag = np.empty((th, tw), np.float32)
    L.check(lib.ubg_velocity_texture(sim._h, L.fptr(vxy), L.fptr(mag)))
    return vxy, mag


class MG:
    """class MG, pressure_solver.hpp:13-76.  MG(width, height) or MG(flag)."""

    def __init__(self, width_or_flag, height=None):
        self._lib = L.load()
        h = C.c_void_p()
        if height is None:
            flag = _f32(width_or_flag)
            self.height, self.width = flag.shape
            L.check(self._lib.ubg_mg_create(self.width, self.height, L.fptr(flag), C.byref(h)))
        else:
            self.width, self.height = int(width_or_flag), int(height)
            L.check(self._lib.ubg_mg_create(self.width, self.height, None, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ubg_mg_destroy(self._h)
            self._h = None

    def updateFields(self, flag):
        L.check(self._lib.ubg_mg_update_fields(self._h, L.fptr(_f32(flag))))

    def solve(self, p, f, flag, h, zeroGradientBC=False):
        """MG::solve: updates p (a float32 array) in place and returns it."""
        shape = (self.height, self.width)
        if not (isinstance(p, np.ndarray) and p.dtype == np.float32 and p.flags.c_contiguous
                and p.shape == shape):
            raise ValueError("p must be a C-contiguous float32 array of shape %s" % (shape,))
        L.check(self._lib.ubg_mg_solve(self._h, L.fptr(p), L.fptr(_f32(f, shape)),
                                       L.fptr(_f32(flag, shape)), h, int(zeroGradientBC)))
        return p


def rbgs(p, f, flag, h, alpha=1.0):
    """rbgs(p, f, flag, h, alpha), pressure_solver.cpp:35-89; returns the new p."""
    lib = L.load()
    p = _f32(p).copy()
    H, W = p.shape
    L.check(lib.ubg_rbgs(L.fptr(p), L.fptr(_f32(f, (H, W))), L.fptr(_f32(flag, (H, W))), W, H,
                         h, alpha))
    return p


def calculateResidualField(p, f, flag, h):
    """calculateResidualField, pressure_solver.cpp:91-116 -> (r, ||r||_2)."""
    lib = L.load()
    p = _f32(p)
    H, W = p.shape
    r = np.zeros((H, W), dtype=np.float32)
    n = C.c_double()
    L.check(lib.ubg_residual(L.fptr(p), L.fptr(_f32(f, (H, W))), L.fptr(_f32(flag, (H, W))),
                             L.fptr(r), W, H, h, C.byref(n)))
    return r, n.value
