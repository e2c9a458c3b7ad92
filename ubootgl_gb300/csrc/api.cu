// C ABI of ubootgl_gb300 (include/ubootgl_gb300.h): simulation handles,
// host <-> device transfers, the step sequence of Simulation::step
// (simulation.cpp:356-374), the standalone MG class and the free solver
// functions.  All device work of a handle goes to its own stream.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>
#include <algorithm>
#include <atomic>

#include "ubg_internal.cuh"

using namespace ubg;

namespace {
thread_local std::string g_err;
}  // namespace

void ubg::set_last_error(const std::string &msg) { g_err = msg; }

namespace {

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

template <class F>
int guarded(F &&f) {
  try {
    g_err.clear();
    return f();
  } catch (const ArgError &e) {
    return fail(UBG_EINVAL, e.what());
  } catch (const CudaError &e) {
    return fail(UBG_ECUDA, e.what());
  } catch (const std::bad_alloc &) {
    return fail(UBG_ENOMEM, "allocation failed");
  } catch (const std::exception &e) {
    return fail(UBG_ESTATE, e.what());
  }
}

constexpr int kRing = 64;
constexpr int kMaxSinks = 256;

// Flags cross the ABI as float 0.0 / 1.0 and live on the device as bytes.
void flag_to_u8(const float *flag, int W, int H, std::vector<uint8_t> &out, int pitch) {
  out.assign((size_t)pitch * H, 0);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      float v = flag[(size_t)y * W + x];
      if (v == 0.0f)
        out[(size_t)y * pitch + x] = 0;
      else if (v == 1.0f)
        out[(size_t)y * pitch + x] = 1;
      else
        throw ArgError("flag values must be exactly 0.0 or 1.0 (cell " + std::to_string(x) + "," +
                       std::to_string(y) + ")");
    }
}

StepScalars make_scalars(float dt, float mu, float pwidth, int W, float h) {
  // simulation.cpp:105, 165, 242, 276, 286
  StepScalars s;
  s.dt = dt;
  s.a = dt * mu * ((float)W - 1.0f) / pwidth;
  s.den = 1.0f + 4.0f * s.a;
  s.rden = 1.0f / s.den;
  s.ih = 1.0f / h;
  s.chalf = 0.5f * dt * s.ih;
  s.cfull = dt * s.ih;
  return s;
}

struct HostSink {
  float x, y, z;
};

}  // namespace

struct ubg_sim {
  int W = 0, H = 0, P = 0;
  float pwidth = 1.0f, mu = 0.0f, h = 0.0f;
  Bcs bc{UBG_BC_INFLOW, UBG_BC_OUTFLOW_ZERO_PRESSURE, UBG_BC_NOSLIP, UBG_BC_NOSLIP};
  ubg_options opt{};
  cudaStream_t st = nullptr;
  void *arena = nullptr;
  size_t arena_bytes = 0;
  VelBufs v{};
  int fx = 0, fy = 0;
  float *ax = nullptr, *ay = nullptr;
  uint8_t *codes_x = nullptr, *codes_y = nullptr;
  MgHier mg;
  MgLow lo;       // 16-bit correction hierarchy of the fixed-mode mixed solver
  FcgSolver fcg;  // tolerance-mode solver (allocated when that mode is set)
  StepScalars *d_sc = nullptr;
  unsigned int *d_umax = nullptr;
  SinkCell *d_sinks = nullptr;
  // pinned host staging
  StepScalars *h_ring = nullptr;
  SinkCell *h_sinks = nullptr;
  double *h_norm = nullptr;
  cudaEvent_t ring_ev[kRing] = {};
  bool ring_used[kRing] = {};
  int ring_i = 0;
  std::vector<HostSink> sinks;
  std::vector<float> flag_host;
  bool accum_dirty = false;
  bool umax_ready = false;  // d_umax holds max|u| of the current fields
  float last_dt = 0.0f;
  int last_vcycles = 0;
  double last_rel = -1.0;  // ||r|| / ||f|| after the last tolerance-mode solve
  // CUDA graph of the fixed-cycle step body
  // captured step bodies: a step flips the velocity buffers, so steps
  // alternate between two index states and two graphs
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    int key = -1;
    long gen = -1;
    long launches = 0;
    int fx = 0, fy = 0, cur0 = 0;  // indices after the body
  };
  StepGraph graphs[2];
  int graph_next = 0;
  long gen = 0;  // bumped whenever something baked into a captured step changes
  // profiling
  bool prof = false;
  Profiler profiler;
  cudaEvent_t ev_step[2] = {nullptr, nullptr};
  long launches_last = 0;
  double step_ms_total = 0.0;
  long steps_profiled = 0;
  // grow-only device scratch for the item / cell lists of the game-side calls
  void *scratch = nullptr;
  size_t scratch_bytes = 0;
  // asynchronous host I/O (ubg_io_*): staging buffers and a copy stream
  float *io_in[2] = {nullptr, nullptr}, *io_out[2] = {nullptr, nullptr};
  void *io_arena = nullptr;
  cudaStream_t io_st = nullptr, io_out_st = nullptr;  // host->device, device->host
  cudaEvent_t io_in_ready = nullptr, io_in_free = nullptr, io_out_copied = nullptr,
              io_out_done = nullptr;
  bool io_staged = false;

  void io_init() {
    if (io_arena) return;
    size_t fb = ((size_t)P * H * 4 + 255) / 256 * 256;
    if (cudaMalloc(&io_arena, 4 * fb) != cudaSuccess) {
      cudaGetLastError();
      io_arena = nullptr;
      throw std::bad_alloc();
    }
    char *p = (char *)io_arena;
    for (int k = 0; k < 2; k++, p += fb) io_in[k] = (float *)p;
    for (int k = 0; k < 2; k++, p += fb) io_out[k] = (float *)p;
    UBG_CUDA(cudaStreamCreateWithFlags(&io_st, cudaStreamNonBlocking));
    UBG_CUDA(cudaStreamCreateWithFlags(&io_out_st, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&io_in_ready, &io_in_free, &io_out_copied, &io_out_done})
      UBG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    UBG_CUDA(cudaEventRecord(io_in_free, st));
    UBG_CUDA(cudaEventRecord(io_out_done, io_out_st));
  }

  // staged inputs become the front velocity before the next step's kernels
  void io_consume() {
    if (!io_staged) return;
    UBG_CUDA(cudaStreamWaitEvent(st, io_in_ready, 0));
    launch_stage_in(v, fx, fy, io_in[0], io_in[1], d_umax, st);
    UBG_CUDA(cudaEventRecord(io_in_free, st));
    io_staged = false;
    umax_ready = true;  // the copy kernel folded max|u| of the new fields
  }

  void *scratch_get(size_t bytes) {
    if (bytes > scratch_bytes) {
      sync();
      if (scratch) cudaFree(scratch);
      scratch = nullptr;
      scratch_bytes = 0;
      size_t b = std::max(bytes, (size_t)1 << 16);
      if (cudaMalloc(&scratch, b) != cudaSuccess) {
        cudaGetLastError();
        throw std::bad_alloc();
      }
      scratch_bytes = b;
    }
    return scratch;
  }

  // The flag changed on the device: coarse flags and every stencil code
  // (MG::updateFields on the device flag, plus the face codes).
  void flag_changed() {
    fcg.dirty = true;
    mg_update_fields(mg, st);
    launch_face_codes(v, flag(), codes_x, codes_y, st);
    umax_ready = false;
  }

  ~ubg_sim() {
    if (st) cudaStreamSynchronize(st);
    for (auto &g : graphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    for (auto &e : ring_ev)
      if (e) cudaEventDestroy(e);
    for (auto &e : ev_step)
      if (e) cudaEventDestroy(e);
    if (h_ring) cudaFreeHost(h_ring);
    if (h_sinks) cudaFreeHost(h_sinks);
    if (h_norm) cudaFreeHost(h_norm);
    mg_low_free(lo);
    fcg_free(fcg);
    if (scratch) cudaFree(scratch);
    if (io_st) cudaStreamSynchronize(io_st);
    if (io_out_st) cudaStreamSynchronize(io_out_st);
    for (cudaEvent_t e : {io_in_ready, io_in_free, io_out_copied, io_out_done})
      if (e) cudaEventDestroy(e);
    if (io_st) cudaStreamDestroy(io_st);
    if (io_out_st) cudaStreamDestroy(io_out_st);
    if (io_arena) cudaFree(io_arena);
    mg_free(mg);
    if (arena) cudaFree(arena);
    if (st) cudaStreamDestroy(st);
  }

  float *p() { return mg.lv[0].e[mg.cur0]; }
  float *f() { return mg.lv[0].rhs; }
  uint8_t *flag() { return mg.lv[0].flag; }

  // Stages the dt-dependent scalars for the next kernels of this stream.
  void push_scalars(float dt) {
    int slot = ring_i;
    ring_i = (ring_i + 1) % kRing;
    if (ring_used[slot]) UBG_CUDA(cudaEventSynchronize(ring_ev[slot]));
    h_ring[slot] = make_scalars(dt, mu, pwidth, W, h);
    UBG_CUDA(cudaMemcpyAsync(d_sc, &h_ring[slot], sizeof(StepScalars), cudaMemcpyHostToDevice, st));
    UBG_CUDA(cudaEventRecord(ring_ev[slot], st));
    ring_used[slot] = true;
    last_dt = dt;
  }

  void set_vbcs() { launch_vbc(v, fx, fy, bc, true, true, st); }

  void apply_accum() {
    launch_accum(v, fx, fy, ax, ay, st);
    accum_dirty = false;
  }

  // diffuse(), simulation.cpp:104-162.  The vx and vy sweeps are independent
  // (setVBCs treats the components separately), so each sweep launch does
  // both; the vy boundary is refreshed first because the reference's vy
  // sweeps run after a setVBCs.
  void diffuse() {
    launch_vbc(v, fx, fy, bc, false, true, st);
    for (int i = 0; i < 2; i++) {
      launch_diffuse_sweep(v, fx, fy, d_sc, 3, st);
      fx ^= 1;
      fy ^= 1;
      set_vbcs();
    }
  }

  void advect() {
    launch_advect(v, fx, fy, d_sc, st);
    fx ^= 1;
    fy ^= 1;
  }

  // The sinks of project() (simulation.cpp:173-187), resolved on the host.
  int stage_sinks(float dt) {
    int n = 0;
    std::vector<HostSink> keep;
    for (auto &s : sinks) {
      float gx = s.x / h + 0.5f, gy = s.y / h + 0.5f;
      if (!(gx <= 3 || gx > (float)(W - 3) || gy <= 3 || gy > (float)(H - 3))) {
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            if (n >= kMaxSinks * 9) break;
            h_sinks[n++] = SinkCell{(int)(gx + (float)dx), (int)(gy + (float)dy), s.z};
          }
        s.z = (float)((double)s.z * std::pow(0.000001, (double)(dt * 50.0f)));
      }
    }
    for (auto &s : sinks)
      if (!(s.z < 0.05f)) keep.push_back(s);
    sinks.swap(keep);
    if (n) UBG_CUDA(cudaMemcpyAsync(d_sinks, h_sinks, sizeof(SinkCell) * n, cudaMemcpyHostToDevice, st));
    return n;
  }

  void solve_pressure() {
    if (opt.precision != UBG_FP32) {
      solve_mixed();
      return;
    }
    for (int c = 0; c < opt.vcycles; c++) mg_solve(mg, true, st);
    last_vcycles = opt.vcycles;
    last_rel = -1.0;
  }

  // Extension, fixed mode: FP32 defect correction around a 16-bit V-cycle,
  // `vcycles` corrections (no host synchronisation, capturable), equal in
  // exact arithmetic to `vcycles` V-cycles started from p with
  // zero-gradient edges.
  void solve_mixed() {
    if (lo.levels != mg.levels || lo.prec != opt.precision)
      throw std::runtime_error("mixed-precision hierarchy not allocated (ubg_set_options)");
    last_vcycles = mg_solve_mixed(mg, lo, 0.0, opt.vcycles, 0.0, nullptr, st);
    last_rel = -1.0;
  }

  // project(), simulation.cpp:164-208 (without the trailing setVBCs of step).
  // The gradient kernel also starts the max|u| reduction for the next CFL dt.
  // Tolerance mode (extension): flexible CG preconditioned by the tolerance
  // hierarchy's V-cycle (k_krylov.cu) until ||r|| <= tol ||f_c||; the
  // gradient update reads its double-float pressure.
  void project(int nsink_cells) {
    launch_divergence(v, fx, fy, f(), d_sc, st);
    launch_sinks(f(), P, d_sinks, nsink_cells, st);
    if (opt.solver_mode == UBG_SOLVE_TOLERANCE) {
      if (!fcg.arena) throw std::runtime_error("tolerance solver not allocated (ubg_set_options)");
      fcg_set_precision(fcg, opt.precision);
      last_vcycles = fcg_solve(fcg, flag(), f(), p(), (double)opt.tol, opt.max_vcycles, &last_rel, st);
      launch_pbc(p(), P, W, H, bc, st);
      UBG_CUDA(cudaMemsetAsync(d_umax, 0, sizeof(unsigned int), st));
      launch_gradient_df(v, fx, fy, fcg.xh, fcg.xl, d_sc, d_umax, st);
      return;
    }
    solve_pressure();
    launch_pbc(p(), P, W, H, bc, st);
    UBG_CUDA(cudaMemsetAsync(d_umax, 0, sizeof(unsigned int), st));
    launch_gradient(v, fx, fy, p(), d_sc, d_umax, st);
  }

  // Everything of step() after the scalars are staged and the accumulated
  // velocity is applied; captured into a graph in fixed-cycle mode.  The
  // final setVBCs completes max|u| over all faces.
  void step_body(int nsink_cells) {
    diffuse();
    advect();
    set_vbcs();
    project(nsink_cells);
    launch_vbc(v, fx, fy, bc, true, true, st, d_umax);
  }

  void step(float dt, bool device_dt, float cfl) {
    long l0 = g_stats.launches;
    bool accum_dirty_at_start = accum_dirty;
    struct ProfInstall {
      bool on;
      ProfInstall(bool on_, Profiler *p) : on(on_) {
        if (on) g_prof = p;
      }
      ~ProfInstall() {
        if (on) g_prof = nullptr;
      }
    } pi(prof, &profiler);
    if (prof) UBG_CUDA(cudaEventRecord(ev_step[0], st));
    io_consume();
    if (accum_dirty) apply_accum();
    int nsc = 0;
    if (device_dt) {
      launch_cfl(v, fx, fy, cfl, h, mu, pwidth, d_umax, d_sc, st, umax_ready && !accum_dirty_at_start);
    } else {
      push_scalars(dt);
      nsc = sinks.empty() ? 0 : stage_sinks(dt);
    }
    bool graphable = opt.use_graph && opt.solver_mode == UBG_SOLVE_FIXED && nsc == 0 && !prof;
    if (graphable) {
      // The body only depends on (fx, fy, cur0) parity and the cycle count.
      int key = (fx << 2) | (fy << 1) | mg.cur0 | (opt.vcycles << 3) | (opt.precision << 24);
      StepGraph *g = nullptr;
      for (auto &c : graphs)
        if (c.exec && c.key == key && c.gen == gen) g = &c;
      if (!g) g = &capture(key);
      UBG_CUDA(cudaGraphLaunch(g->exec, st));
      // replay the index bookkeeping of the captured body
      fx = g->fx;
      fy = g->fy;
      mg.cur0 = g->cur0;
      g_stats.launches += g->launches;
    } else {
      step_body(nsc);
    }
    umax_ready = true;
    if (prof) {
      UBG_CUDA(cudaEventRecord(ev_step[1], st));
      // per-step collection keeps the event pool small
      UBG_CUDA(cudaStreamSynchronize(st));
      float ms = 0.0f;
      UBG_CUDA(cudaEventElapsedTime(&ms, ev_step[0], ev_step[1]));
      step_ms_total += ms;
      steps_profiled++;
      profiler.collect();
    }
    launches_last = g_stats.launches - l0;
  }

  // Captures the step body for the current indices into the older of the
  // two graph slots (an executable graph still in flight is freed by the
  // driver when it completes).
  StepGraph &capture(int key) {
    StepGraph &sg = graphs[graph_next];
    graph_next ^= 1;
    if (sg.exec) {
      cudaGraphExecDestroy(sg.exec);
      sg.exec = nullptr;
    }
    int fx0 = fx, fy0 = fy, c0 = mg.cur0;
    long l0 = g_stats.launches;
    cudaGraph_t g = nullptr;
    UBG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      step_body(0);
    } catch (...) {
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    UBG_CUDA(cudaStreamEndCapture(st, &g));
    UBG_CUDA(cudaGraphInstantiate(&sg.exec, g, 0));
    cudaGraphDestroy(g);
    sg.launches = g_stats.launches - l0;
    g_stats.launches = l0;
    sg.fx = fx;
    sg.fy = fy;
    sg.cur0 = mg.cur0;
    fx = fx0;
    fy = fy0;
    mg.cur0 = c0;
    sg.key = key;
    sg.gen = gen;
    return sg;
  }

  void sync() { UBG_CUDA(cudaStreamSynchronize(st)); }
};

struct ubg_mg {
  MgHier mg;
  cudaStream_t st = nullptr;
  int W = 0, H = 0;
  ~ubg_mg() {
    if (st) cudaStreamSynchronize(st);
    mg_free(mg);
    if (st) cudaStreamDestroy(st);
  }
};

namespace {

struct FieldView {
  float *dev;
  int w, h;
};

FieldView field_view(ubg_sim *s, int field) {
  int W = s->W, H = s->H;
  switch (field) {
    case UBG_VX: case UBG_VX_CURRENT: return {s->v.vx[s->fx], W - 1, H};
    case UBG_VY: case UBG_VY_CURRENT: return {s->v.vy[s->fy], W, H - 1};
    case UBG_VX_BACK: return {s->v.vx[1 - s->fx], W - 1, H};
    case UBG_VY_BACK: return {s->v.vy[1 - s->fy], W, H - 1};
    case UBG_P: return {s->p(), W, H};
    case UBG_F: return {s->f(), W, H};
    case UBG_VX_ACCUM: return {s->ax, W - 1, H};
    case UBG_VY_ACCUM: return {s->ay, W, H - 1};
  }
  throw ArgError("unknown field id " + std::to_string(field));
}

void upload_flag_u8(MgLevel &L0, const float *flag, int W, int H, cudaStream_t st) {
  std::vector<uint8_t> u8;
  flag_to_u8(flag, W, H, u8, L0.pitch);
  UBG_CUDA(cudaMemcpyAsync(L0.flag, u8.data(), u8.size(), cudaMemcpyHostToDevice, st));
  UBG_CUDA(cudaStreamSynchronize(st));
}

void check_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    throw CudaError("no CUDA device available (this library has no CPU path)");
  }
}

}  // namespace

extern "C" {

const char *ubg_last_error(void) { return g_err.c_str(); }

int ubg_device_info(char *buf, size_t len) {
  return guarded([&] {
    check_device();
    int dev = 0;
    UBG_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp p;
    UBG_CUDA(cudaGetDeviceProperties(&p, dev));
    snprintf(buf, len,
             "{\"name\": \"%s\", \"sm\": \"%d.%d\", \"sms\": %d, \"mem_gb\": %.1f, "
             "\"cluster_coarse_solve\": \"%s\"}",
             p.name, p.major, p.minor, p.multiProcessorCount, p.totalGlobalMem / 1e9,
             cluster_coarse_solve_status());
    return UBG_OK;
  });
}

int ubg_host_alloc(size_t bytes, void **ptr) {
  return guarded([&] {
    if (!ptr) throw ArgError("null argument");
    check_device();
    UBG_CUDA(cudaMallocHost(ptr, bytes));
    return UBG_OK;
  });
}

int ubg_host_free(void *ptr) {
  return guarded([&] {
    if (ptr) UBG_CUDA(cudaFreeHost(ptr));
    return UBG_OK;
  });
}

int ubg_default_options(ubg_options *o) {
  if (!o) return fail(UBG_EINVAL, "null options");
  o->solver_mode = UBG_SOLVE_FIXED;
  o->vcycles = 2;
  o->tol = 1e-6f;
  o->max_vcycles = 100;
  o->precision = UBG_FP32;
  o->use_graph = 1;
  o->advect_bilinear = 0;
  return UBG_OK;
}

int ubg_create(const float *flag, int width, int height, float pwidth, float mu, ubg_sim **out) {
  return guarded([&] {
    if (!flag || !out) throw ArgError("null argument");
    if (width < 8 || height < 8) throw ArgError("width and height must be >= 8");
    if ((long long)width * height > (1LL << 31)) throw ArgError("grid too large");
    check_device();
    std::unique_ptr<ubg_sim> s(new ubg_sim());
    s->W = width;
    s->H = height;
    s->P = round_up(width, 32);
    s->pwidth = pwidth;
    s->mu = mu;
    s->h = pwidth / ((float)width - 1.0f);  // simulation.hpp:63
    ubg_default_options(&s->opt);
    UBG_CUDA(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
    size_t n = (size_t)s->P * height;
    size_t fb = (n * 4 + 255) / 256 * 256;
    size_t bb = (n + 255) / 256 * 256;
    size_t extra = 256 * 3 + (size_t)kMaxSinks * 9 * sizeof(SinkCell);
    size_t total = 6 * fb + 2 * bb + extra;
    s->arena_bytes = total;
    if (cudaMalloc(&s->arena, total) != cudaSuccess) {
      cudaGetLastError();
      throw std::bad_alloc();
    }
    UBG_CUDA(cudaMemsetAsync(s->arena, 0, total, s->st));
    char *p = (char *)s->arena;
    s->v.vx[0] = (float *)p; p += fb;
    s->v.vx[1] = (float *)p; p += fb;
    s->v.vy[0] = (float *)p; p += fb;
    s->v.vy[1] = (float *)p; p += fb;
    s->ax = (float *)p; p += fb;
    s->ay = (float *)p; p += fb;
    s->codes_x = (uint8_t *)p; p += bb;
    s->codes_y = (uint8_t *)p; p += bb;
    s->v.cx = s->codes_x;
    s->v.cy = s->codes_y;
    s->d_sc = (StepScalars *)p; p += 256;
    s->d_umax = (unsigned int *)p; p += 256;
    p += 256;
    s->d_sinks = (SinkCell *)p;
    s->v.pitch = s->P;
    s->v.W = width;
    s->v.H = height;
    mg_alloc(s->mg, width, height, s->h);
    UBG_CUDA(cudaMallocHost(&s->h_ring, sizeof(StepScalars) * kRing));
    UBG_CUDA(cudaMallocHost(&s->h_sinks, sizeof(SinkCell) * kMaxSinks * 9));
    UBG_CUDA(cudaMallocHost(&s->h_norm, sizeof(double)));
    for (auto &e : s->ring_ev) UBG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto &e : s->ev_step) UBG_CUDA(cudaEventCreate(&e));
    // flag + multigrid hierarchy (MG(flag), simulation.hpp:62)
    s->flag_host.assign(flag, flag + (size_t)width * height);
    upload_flag_u8(s->mg.lv[0], flag, width, height, s->st);
    mg_update_fields(s->mg, s->st);
    launch_face_codes(s->v, s->flag(), s->codes_x, s->codes_y, s->st);
    // vy(x, 0) = 0 and vx(0, y) = 1 in both buffers (simulation.hpp:55-60)
    std::vector<float> col((size_t)height, 1.0f);
    for (int b = 0; b < 2; b++)
      UBG_CUDA(cudaMemcpy2DAsync(s->v.vx[b], (size_t)s->P * 4, col.data(), 4, 4, height,
                                 cudaMemcpyHostToDevice, s->st));
    UBG_CUDA(cudaStreamSynchronize(s->st));
    *out = s.release();
    return UBG_OK;
  });
}

int ubg_destroy(ubg_sim *sim) {
  return guarded([&] {
    delete sim;
    return UBG_OK;
  });
}

int ubg_set_options(ubg_sim *s, const ubg_options *o) {
  return guarded([&] {
    if (!s || !o) throw ArgError("null argument");
    if (o->solver_mode != UBG_SOLVE_FIXED && o->solver_mode != UBG_SOLVE_TOLERANCE)
      throw ArgError("solver_mode");
    if (o->vcycles < 0 || o->vcycles > 1000) throw ArgError("vcycles out of range");
    if (o->max_vcycles < 1 || o->max_vcycles > 100000) throw ArgError("max_vcycles out of range");
    if (o->precision != UBG_FP32 && o->precision != UBG_MIXED_FP16 &&
        o->precision != UBG_MIXED_BF16)
      throw ArgError("precision");
    if (o->solver_mode == UBG_SOLVE_TOLERANCE && !(o->tol > 0.0f)) throw ArgError("tol must be > 0");
    if (o->advect_bilinear != 0 && o->advect_bilinear != 1) throw ArgError("advect_bilinear");
    UBG_CUDA(cudaStreamSynchronize(s->st));
    if (o->solver_mode == UBG_SOLVE_TOLERANCE) {
      // flexible CG over the tolerance hierarchy; the fixed-mode 16-bit
      // hierarchy is not needed
      mg_low_free(s->lo);
      if (!s->fcg.arena) fcg_alloc(s->fcg, s->W, s->H, s->P, s->h);
      fcg_set_precision(s->fcg, o->precision);
    } else {
      fcg_free(s->fcg);
      if (o->precision == UBG_FP32)
        mg_low_free(s->lo);
      else if (s->lo.prec != o->precision || s->lo.levels != s->mg.levels)
        mg_low_alloc(s->lo, s->mg, o->precision);
    }
    s->opt = *o;
    s->v.advect_bilinear = o->advect_bilinear;
    s->gen++;
    return UBG_OK;
  });
}

int ubg_set_bcs(ubg_sim *s, int west, int east, int north, int south) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    for (int b : {west, east, north, south})
      if (b < 0 || b > 3) throw ArgError("boundary type");
    s->bc = Bcs{west, east, north, south};
    s->gen++;  // boundary types are baked into the captured step
    return UBG_OK;
  });
}

int ubg_step(ubg_sim *s, float dt) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->step(dt, false, 0.0f);
    return UBG_OK;
  });
}

int ubg_step_cfl(ubg_sim *s, float cfl) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    if (!s->sinks.empty()) throw ArgError("sinks need a host dt (use ubg_step)");
    s->step(0.0f, true, cfl);
    return UBG_OK;
  });
}

int ubg_solver_stats(ubg_sim *s, int *vcycles, double *rel_residual) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    if (vcycles) *vcycles = s->last_vcycles;
    if (rel_residual) *rel_residual = s->last_rel;
    return UBG_OK;
  });
}

int ubg_last_dt(ubg_sim *s, float *dt) {
  return guarded([&] {
    if (!s || !dt) throw ArgError("null argument");
    StepScalars sc;
    UBG_CUDA(cudaMemcpyAsync(&sc, s->d_sc, sizeof(sc), cudaMemcpyDeviceToHost, s->st));
    UBG_CUDA(cudaStreamSynchronize(s->st));
    *dt = sc.dt;
    return UBG_OK;
  });
}

int ubg_apply_accumulated_velocity(ubg_sim *s) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->umax_ready = false;
    s->apply_accum();
    return UBG_OK;
  });
}

int ubg_diffuse(ubg_sim *s, float dt) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->umax_ready = false;
    s->push_scalars(dt);
    s->diffuse();
    return UBG_OK;
  });
}

int ubg_advect(ubg_sim *s, float dt) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->umax_ready = false;
    s->push_scalars(dt);
    s->advect();
    return UBG_OK;
  });
}

int ubg_set_vbcs(ubg_sim *s) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->umax_ready = false;
    s->set_vbcs();
    return UBG_OK;
  });
}

int ubg_set_pbc(ubg_sim *s) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    launch_pbc(s->p(), s->P, s->W, s->H, s->bc, s->st);
    return UBG_OK;
  });
}

int ubg_project(ubg_sim *s, float dt) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->umax_ready = false;
    s->push_scalars(dt);
    int n = s->sinks.empty() ? 0 : s->stage_sinks(dt);
    s->project(n);
    return UBG_OK;
  });
}

int ubg_add_sink(ubg_sim *s, float x, float y, float strength) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    if ((int)s->sinks.size() >= kMaxSinks) throw ArgError("too many sinks");
    s->sinks.push_back(HostSink{x, y, strength});
    return UBG_OK;
  });
}

int ubg_upload(ubg_sim *s, int field, const float *src) {
  return guarded([&] {
    if (!s || !src) throw ArgError("null argument");
    s->umax_ready = false;
    if (field == UBG_FLAG) {
      upload_flag_u8(s->mg.lv[0], src, s->W, s->H, s->st);
      s->flag_host.assign(src, src + (size_t)s->W * s->H);
      s->flag_changed();
      s->sync();
      return UBG_OK;
    }
    if (field == UBG_VX_CURRENT || field == UBG_VY_CURRENT) throw ArgError("current fields are read-only");
    FieldView fv = field_view(s, field);
    UBG_CUDA(cudaMemcpy2DAsync(fv.dev, (size_t)s->P * 4, src, (size_t)fv.w * 4, (size_t)fv.w * 4, fv.h,
                               cudaMemcpyHostToDevice, s->st));
    if (field == UBG_VX_ACCUM || field == UBG_VY_ACCUM) s->accum_dirty = true;
    s->sync();
    return UBG_OK;
  });
}

int ubg_download(ubg_sim *s, int field, float *dst) {
  return guarded([&] {
    if (!s || !dst) throw ArgError("null argument");
    if (field == UBG_FLAG) {
      s->sync();
      std::memcpy(dst, s->flag_host.data(), sizeof(float) * s->flag_host.size());
      return UBG_OK;
    }
    FieldView fv = field_view(s, field);
    UBG_CUDA(cudaMemcpy2DAsync(dst, (size_t)fv.w * 4, fv.dev, (size_t)s->P * 4, (size_t)fv.w * 4, fv.h,
                               cudaMemcpyDeviceToHost, s->st));
    s->sync();
    return UBG_OK;
  });
}

int ubg_mg_levels(ubg_sim *s, int *levels) {
  return guarded([&] {
    if (!s || !levels) throw ArgError("null argument");
    *levels = s->mg.levels;
    return UBG_OK;
  });
}

int ubg_mg_level_flag(ubg_sim *s, int level, int *w, int *h, float *dst) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    if (level < 0 || level >= s->mg.levels) throw ArgError("level out of range");
    MgLevel &L = s->mg.lv[level];
    if (w) *w = L.w;
    if (h) *h = L.h;
    if (!dst) return UBG_OK;
    std::vector<uint8_t> u8((size_t)L.pitch * L.h);
    UBG_CUDA(cudaMemcpyAsync(u8.data(), L.flag, u8.size(), cudaMemcpyDeviceToHost, s->st));
    s->sync();
    for (int y = 0; y < L.h; y++)
      for (int x = 0; x < L.w; x++) dst[(size_t)y * L.w + x] = (float)u8[(size_t)y * L.pitch + x];
    return UBG_OK;
  });
}

int ubg_mg_solve_sim(ubg_sim *s, int zgbc) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    mg_solve(s->mg, zgbc != 0, s->st);
    return UBG_OK;
  });
}

int ubg_field_device(ubg_sim *s, int field, void **ptr, int *pitch, int *w, int *h) {
  return guarded([&] {
    if (!s || !ptr) throw ArgError("null argument");
    s->umax_ready = false;
    if (field == UBG_FLAG) {
      *ptr = s->flag();
      if (pitch) *pitch = s->P;
      if (w) *w = s->W;
      if (h) *h = s->H;
      return UBG_OK;
    }
    FieldView fv = field_view(s, field);
    *ptr = fv.dev;
    if (pitch) *pitch = s->P;
    if (w) *w = fv.w;
    if (h) *h = fv.h;
    return UBG_OK;
  });
}

int ubg_stream(ubg_sim *s, void **stream) {
  if (!s || !stream) return fail(UBG_EINVAL, "null argument");
  *stream = (void *)s->st;
  return UBG_OK;
}

int ubg_sync(ubg_sim *s) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->sync();
    return UBG_OK;
  });
}

int ubg_profile_enable(ubg_sim *s, int on) {
  if (!s) return fail(UBG_EINVAL, "null handle");
  s->prof = on != 0;
  return UBG_OK;
}

int ubg_profile_read(ubg_sim *s, double *smoother_ms, int *smoother_launches, double *step_ms,
                     int *kernel_launches) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->sync();
    long n = s->profiler.count[KC_SMOOTH_L0];
    if (smoother_ms) *smoother_ms = n ? s->profiler.total_ms[KC_SMOOTH_L0] / n : 0.0;
    if (smoother_launches) *smoother_launches = (int)n;
    if (step_ms) *step_ms = s->steps_profiled ? s->step_ms_total / s->steps_profiled : 0.0;
    if (kernel_launches) *kernel_launches = (int)s->launches_last;
    return UBG_OK;
  });
}

int ubg_profile_class(ubg_sim *s, int kc, const char **name, double *total_ms, int *count) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    if (kc < 0 || kc >= KC_COUNT) throw ArgError("kernel class out of range");
    s->sync();
    if (name) *name = kernel_class_name(kc);
    if (total_ms) *total_ms = s->profiler.total_ms[kc];
    if (count) *count = (int)s->profiler.count[kc];
    return UBG_OK;
  });
}

int ubg_profile_reset(ubg_sim *s) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->sync();
    for (int k = 0; k < KC_COUNT; k++) {
      s->profiler.total_ms[k] = 0.0;
      s->profiler.count[k] = 0;
    }
    s->step_ms_total = 0.0;
    s->steps_profiled = 0;
    return UBG_OK;
  });
}

// ------------------------------------------------------- display tracers

struct ubg_tracers {
  ubg_sim *sim = nullptr;
  int ntr = 0, npts = 0;
  void *mem = nullptr;
  float2 *points = nullptr;
  uint32_t *start = nullptr, *end = nullptr;
  float *ages = nullptr;
  ~ubg_tracers() {
    if (sim && sim->st) cudaStreamSynchronize(sim->st);
    if (mem) cudaFree(mem);
  }
};

int ubg_velocity_texture(ubg_sim *s, float *vxy, float *mag) {
  return guarded([&] {
    if (!s || !vxy) throw ArgError("null argument");
    size_t n = (size_t)(2 * s->W - 1) * (2 * s->H - 1);
    void *mem = nullptr;
    UBG_CUDA(cudaMallocAsync(&mem, n * 12, s->st));
    float2 *dv = (float2 *)mem;
    float *dm = (float *)((char *)mem + n * 8);
    launch_velocity_texture(s->v.vx[s->fx], s->v.vy[s->fy], s->P, s->W, s->H, dv, dm, s->st);
    UBG_CUDA(cudaMemcpyAsync(vxy, dv, n * 8, cudaMemcpyDeviceToHost, s->st));
    if (mag) UBG_CUDA(cudaMemcpyAsync(mag, dm, n * 4, cudaMemcpyDeviceToHost, s->st));
    UBG_CUDA(cudaFreeAsync(mem, s->st));
    s->sync();
    return UBG_OK;
  });
}

int ubg_tracers_create(ubg_sim *s, int ntracers, int npoints, ubg_tracers **out) {
  return guarded([&] {
    if (!s || !out) throw ArgError("null argument");
    if (ntracers < 1 || npoints < 1 || (long long)ntracers * npoints > (1LL << 31))
      throw ArgError("tracer counts out of range");
    std::unique_ptr<ubg_tracers> t(new ubg_tracers());
    t->sim = s;
    t->ntr = ntracers;
    t->npts = npoints;
    size_t np = (size_t)ntracers * npoints * 8, nt = (size_t)ntracers * 4;
    auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    size_t total = al(np) + 3 * al(nt);
    if (cudaMalloc(&t->mem, total) != cudaSuccess) {
      cudaGetLastError();
      throw std::bad_alloc();
    }
    UBG_CUDA(cudaMemsetAsync(t->mem, 0, total, s->st));
    char *p = (char *)t->mem;
    t->points = (float2 *)p; p += al(np);
    t->start = (uint32_t *)p; p += al(nt);
    t->end = (uint32_t *)p; p += al(nt);
    t->ages = (float *)p;
    s->sync();
    *out = t.release();
    return UBG_OK;
  });
}

int ubg_tracers_destroy(ubg_tracers *t) {
  return guarded([&] {
    delete t;
    return UBG_OK;
  });
}

int ubg_tracers_upload(ubg_tracers *t, const float *points, const uint32_t *start,
                       const uint32_t *end, const float *ages) {
  return guarded([&] {
    if (!t) throw ArgError("null handle");
    cudaStream_t st = t->sim->st;
    size_t np = (size_t)t->ntr * t->npts * 8, nt = (size_t)t->ntr * 4;
    if (points) UBG_CUDA(cudaMemcpyAsync(t->points, points, np, cudaMemcpyHostToDevice, st));
    if (start) UBG_CUDA(cudaMemcpyAsync(t->start, start, nt, cudaMemcpyHostToDevice, st));
    if (end) UBG_CUDA(cudaMemcpyAsync(t->end, end, nt, cudaMemcpyHostToDevice, st));
    if (ages) UBG_CUDA(cudaMemcpyAsync(t->ages, ages, nt, cudaMemcpyHostToDevice, st));
    UBG_CUDA(cudaStreamSynchronize(st));
    return UBG_OK;
  });
}

int ubg_tracers_download(ubg_tracers *t, float *points, uint32_t *start, uint32_t *end,
                         float *ages) {
  return guarded([&] {
    if (!t) throw ArgError("null handle");
    cudaStream_t st = t->sim->st;
    size_t np = (size_t)t->ntr * t->npts * 8, nt = (size_t)t->ntr * 4;
    if (points) UBG_CUDA(cudaMemcpyAsync(points, t->points, np, cudaMemcpyDeviceToHost, st));
    if (start) UBG_CUDA(cudaMemcpyAsync(start, t->start, nt, cudaMemcpyDeviceToHost, st));
    if (end) UBG_CUDA(cudaMemcpyAsync(end, t->end, nt, cudaMemcpyDeviceToHost, st));
    if (ages) UBG_CUDA(cudaMemcpyAsync(ages, t->ages, nt, cudaMemcpyDeviceToHost, st));
    UBG_CUDA(cudaStreamSynchronize(st));
    return UBG_OK;
  });
}

int ubg_tracers_step(ubg_tracers *t, float dt, uint32_t rand_seed) {
  return guarded([&] {
    if (!t) throw ArgError("null handle");
    ubg_sim *s = t->sim;
    TracerArgs a{};
    a.points = t->points;
    a.start = t->start;
    a.end = t->end;
    a.ages = t->ages;
    a.vx = s->v.vx[s->fx];
    a.vy = s->v.vy[s->fy];
    a.P = s->P;
    a.W = s->W;
    a.H = s->H;
    a.flag = s->flag();
    a.nfx = s->W;
    a.nfy = s->H;
    a.fpitch = s->P;
    a.ntracers = t->ntr;
    a.npoints = t->npts;
    a.dt = dt;
    // pdim = (pwidth, pwidth * ny / nx), draw_tracers_cs.cpp:147
    a.pdx = s->pwidth;
    a.pdy = s->pwidth * (float)s->H / (float)s->W;
    a.seed = rand_seed;
    launch_tracers(a, s->st);
    return UBG_OK;
  });
}

// --------------------------------------------------------------- class MG

int ubg_mg_create(int width, int height, const float *flag, ubg_mg **out) {
  return guarded([&] {
    if (!out) throw ArgError("null argument");
    if (width < 8 || height < 8) throw ArgError("width and height must be >= 8");
    check_device();
    std::unique_ptr<ubg_mg> m(new ubg_mg());
    m->W = width;
    m->H = height;
    UBG_CUDA(cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking));
    mg_alloc(m->mg, width, height, 1.0f);
    if (flag) {
      upload_flag_u8(m->mg.lv[0], flag, width, height, m->st);
      mg_update_fields(m->mg, m->st);
    } else {
      mg_fill_coarse_flags_one(m->mg, m->st);
    }
    UBG_CUDA(cudaStreamSynchronize(m->st));
    *out = m.release();
    return UBG_OK;
  });
}

int ubg_mg_destroy(ubg_mg *m) {
  return guarded([&] {
    delete m;
    return UBG_OK;
  });
}

int ubg_mg_update_fields(ubg_mg *m, const float *flag) {
  return guarded([&] {
    if (!m || !flag) throw ArgError("null argument");
    upload_flag_u8(m->mg.lv[0], flag, m->W, m->H, m->st);
    mg_update_fields(m->mg, m->st);
    UBG_CUDA(cudaStreamSynchronize(m->st));
    return UBG_OK;
  });
}

int ubg_mg_solve(ubg_mg *m, float *p, const float *f, const float *flag, float h, int zgbc) {
  return guarded([&] {
    if (!m || !p || !f || !flag) throw ArgError("null argument");
    MgLevel &L = m->mg.lv[0];
    size_t hp = (size_t)m->W * 4, dp = (size_t)L.pitch * 4;
    upload_flag_u8(L, flag, m->W, m->H, m->st);
    level_make_code(L, m->st);
    UBG_CUDA(cudaMemcpy2DAsync(L.e[m->mg.cur0], dp, p, hp, hp, m->H, cudaMemcpyHostToDevice, m->st));
    UBG_CUDA(cudaMemcpy2DAsync(L.rhs, dp, f, hp, hp, m->H, cudaMemcpyHostToDevice, m->st));
    mg_set_h(m->mg, h);
    mg_solve(m->mg, zgbc != 0, m->st);
    UBG_CUDA(cudaMemcpy2DAsync(p, hp, L.e[m->mg.cur0], dp, hp, m->H, cudaMemcpyDeviceToHost, m->st));
    UBG_CUDA(cudaStreamSynchronize(m->st));
    return UBG_OK;
  });
}

int ubg_mg_solve_device(ubg_mg *m, float *p, int p_pitch, const float *f, int f_pitch,
                        const uint8_t *flag, int flag_pitch, float h, int zgbc, void *stream) {
  return guarded([&] {
    if (!m || !p || !f || !flag) throw ArgError("null argument");
    cudaStream_t st = stream ? (cudaStream_t)stream : m->st;
    MgLevel &L = m->mg.lv[0];
    size_t w4 = (size_t)m->W * 4, dp = (size_t)L.pitch * 4;
    UBG_CUDA(cudaMemcpy2DAsync(L.flag, L.pitch, flag, flag_pitch, m->W, m->H, cudaMemcpyDeviceToDevice, st));
    level_make_code(L, st);
    UBG_CUDA(cudaMemcpy2DAsync(L.e[m->mg.cur0], dp, p, (size_t)p_pitch * 4, w4, m->H,
                               cudaMemcpyDeviceToDevice, st));
    UBG_CUDA(cudaMemcpy2DAsync(L.rhs, dp, f, (size_t)f_pitch * 4, w4, m->H, cudaMemcpyDeviceToDevice, st));
    mg_set_h(m->mg, h);
    mg_solve(m->mg, zgbc != 0, st);
    UBG_CUDA(cudaMemcpy2DAsync(p, (size_t)p_pitch * 4, L.e[m->mg.cur0], dp, w4, m->H,
                               cudaMemcpyDeviceToDevice, st));
    return UBG_OK;
  });
}

// ------------------------------------------------ free solver functions

namespace {
struct TmpLevel {
  MgLevel L{};
  void *mem = nullptr;
  cudaStream_t st = nullptr;
  TmpLevel(int w, int h) {
    L.w = w;
    L.h = h;
    L.pitch = round_up(w, 32);
    size_t n = (size_t)L.pitch * h;
    size_t fb = (n * 4 + 255) / 256 * 256;
    size_t bb = (n + 255) / 256 * 256;
    if (cudaMalloc(&mem, 3 * fb + 2 * bb + 256) != cudaSuccess) {
      cudaGetLastError();
      throw std::bad_alloc();
    }
    char *p = (char *)mem;
    L.e[0] = (float *)p; p += fb;
    L.e[1] = (float *)p; p += fb;
    L.rhs = (float *)p; p += fb;
    L.flag = (uint8_t *)p; p += bb;
    L.code = (uint8_t *)p;
    UBG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    UBG_CUDA(cudaMemsetAsync(mem, 0, 3 * fb + 2 * bb + 256, st));
  }
  ~TmpLevel() {
    if (st) cudaStreamSynchronize(st);
    if (mem) cudaFree(mem);
    if (st) cudaStreamDestroy(st);
  }
  void load(const float *p, const float *f, const float *flag) {
    size_t hp = (size_t)L.w * 4, dp = (size_t)L.pitch * 4;
    if (p) UBG_CUDA(cudaMemcpy2DAsync(L.e[0], dp, p, hp, hp, L.h, cudaMemcpyHostToDevice, st));
    UBG_CUDA(cudaMemcpy2DAsync(L.rhs, dp, f, hp, hp, L.h, cudaMemcpyHostToDevice, st));
    upload_flag_u8(L, flag, L.w, L.h, st);
    level_make_code(L, st);
  }
};
}  // namespace

int ubg_rbgs(float *p, const float *f, const float *flag, int width, int height, float h,
             float alpha) {
  return guarded([&] {
    if (!p || !f || !flag) throw ArgError("null argument");
    if (width < 3 || height < 3) throw ArgError("grid too small");
    check_device();
    TmpLevel t(width, height);
    t.L.hh = h;
    t.load(p, f, flag);
    int cur = 0;
    level_rbgs(t.L, cur, alpha, t.st);
    size_t hp = (size_t)width * 4, dp = (size_t)t.L.pitch * 4;
    UBG_CUDA(cudaMemcpy2DAsync(p, hp, t.L.e[cur], dp, hp, height, cudaMemcpyDeviceToHost, t.st));
    UBG_CUDA(cudaStreamSynchronize(t.st));
    return UBG_OK;
  });
}

int ubg_residual(const float *p, const float *f, const float *flag, float *r, int width, int height,
                 float h, double *l2norm) {
  return guarded([&] {
    if (!p || !f || !flag) throw ArgError("null argument");
    if (width < 3 || height < 3) throw ArgError("grid too small");
    check_device();
    TmpLevel t(width, height);
    t.L.hh = h;
    t.load(p, f, flag);
    double *dn = nullptr;
    UBG_CUDA(cudaMallocAsync((void **)&dn, sizeof(double), t.st));
    UBG_CUDA(cudaMemsetAsync(dn, 0, sizeof(double), t.st));
    level_residual(t.L, 0, t.L.e[1], dn, t.st);
    double nh = 0.0;
    UBG_CUDA(cudaMemcpyAsync(&nh, dn, sizeof(double), cudaMemcpyDeviceToHost, t.st));
    size_t hp = (size_t)width * 4, dp = (size_t)t.L.pitch * 4;
    if (r) UBG_CUDA(cudaMemcpy2DAsync(r, hp, t.L.e[1], dp, hp, height, cudaMemcpyDeviceToHost, t.st));
    UBG_CUDA(cudaFreeAsync(dn, t.st));
    UBG_CUDA(cudaStreamSynchronize(t.st));
    if (l2norm) *l2norm = std::sqrt(nh);
    return UBG_OK;
  });
}

}  // extern "C"

// ------------------------------------------------ game-side field access

int ubg_scatter_accum(ubg_sim *s, int n, const float *xy, const float *v) {
  return guarded([&] {
    if (!s || n < 0 || (n > 0 && (!xy || !v))) throw ArgError("null argument");
    if (n == 0) return UBG_OK;
    size_t b = (size_t)n * sizeof(float2);
    char *d = (char *)s->scratch_get(2 * b);
    UBG_CUDA(cudaMemcpyAsync(d, xy, b, cudaMemcpyHostToDevice, s->st));
    UBG_CUDA(cudaMemcpyAsync(d + b, v, b, cudaMemcpyHostToDevice, s->st));
    launch_scatter_accum(s->ax, s->ay, s->P, s->W, s->H, (const float2 *)d,
                         (const float2 *)(d + b), n, s->st);
    s->accum_dirty = true;
    s->sync();
    return UBG_OK;
  });
}

int ubg_sample_velocity(ubg_sim *s, int n, const float *xy, float *out) {
  return guarded([&] {
    if (!s || n < 0 || (n > 0 && (!xy || !out))) throw ArgError("null argument");
    if (n == 0) return UBG_OK;
    size_t b = (size_t)n * sizeof(float2);
    char *d = (char *)s->scratch_get(2 * b);
    UBG_CUDA(cudaMemcpyAsync(d, xy, b, cudaMemcpyHostToDevice, s->st));
    launch_sample_velocity(s->v.vx[s->fx], s->v.vy[s->fy], s->P, s->W, s->H, (const float2 *)d,
                           (float2 *)(d + b), n, s->st);
    UBG_CUDA(cudaMemcpyAsync(out, d + b, b, cudaMemcpyDeviceToHost, s->st));
    s->sync();
    return UBG_OK;
  });
}

int ubg_set_grids(ubg_sim *s, int n, const int *xy, const float *vals) {
  return guarded([&] {
    if (!s || n < 0 || (n > 0 && (!xy || !vals))) throw ArgError("null argument");
    if (n == 0) return UBG_OK;
    // In call order: the last value of a cell wins; a cell set to 0 at any
    // point has its faces and p zeroed.  Cells outside the grid are ignored
    // (the reference's bounds test).
    std::vector<int> slot((size_t)0);
    std::vector<int2> cells;
    std::vector<uint8_t> val, zero;
    std::unordered_map<long long, int> at;
    for (int i = 0; i < n; i++) {
      int x = xy[2 * i], y = xy[2 * i + 1];
      float f = vals[i];
      if (!(x >= 0 && y >= 0 && x < s->W && y < s->H)) continue;
      if (f != 0.0f && f != 1.0f) throw ArgError("flag values must be exactly 0.0 or 1.0");
      long long key = (long long)y * s->W + x;
      auto it = at.find(key);
      int k;
      if (it == at.end()) {
        k = (int)cells.size();
        at.emplace(key, k);
        cells.push_back(make_int2(x, y));
        val.push_back(0);
        zero.push_back(0);
      } else {
        k = it->second;
      }
      val[k] = f != 0.0f;
      if (f == 0.0f) zero[k] = 1;
      s->flag_host[(size_t)key] = f;
    }
    int m = (int)cells.size();
    if (m == 0) return UBG_OK;
    size_t b = (size_t)m * sizeof(int2);
    char *d = (char *)s->scratch_get(b + 2 * (size_t)m + 16);
    UBG_CUDA(cudaMemcpyAsync(d, cells.data(), b, cudaMemcpyHostToDevice, s->st));
    UBG_CUDA(cudaMemcpyAsync(d + b, val.data(), m, cudaMemcpyHostToDevice, s->st));
    UBG_CUDA(cudaMemcpyAsync(d + b + m, zero.data(), m, cudaMemcpyHostToDevice, s->st));
    launch_set_grids((const int2 *)d, (const uint8_t *)(d + b), (const uint8_t *)(d + b + m), m,
                     s->flag(), s->v.vx[s->fx], s->v.vy[s->fy], s->p(), s->P, s->W, s->H, s->st);
    s->flag_changed();
    s->sync();
    return UBG_OK;
  });
}

int ubg_shift_map(ubg_sim *s, const float *new_flag) {
  return guarded([&] {
    if (!s || !new_flag) throw ArgError("null argument");
    const int W = s->W, H = s->H;
    std::vector<uint8_t> u8;
    flag_to_u8(new_flag, W, H, u8, s->P);
    // inletArea and inletVelocity in float, in the reference's order
    float area = 1.0f;
    for (int y = 0; y < H - 1; y++) area += new_flag[(size_t)y * W];
    float u = 0.07f * (float)H / area;
    MgLevel &L0 = s->mg.lv[0];
    float *p_in = L0.e[s->mg.cur0], *p_out = L0.e[1 - s->mg.cur0];
    UBG_CUDA(cudaMemcpyAsync(L0.flag, u8.data(), u8.size(), cudaMemcpyHostToDevice, s->st));
    launch_shift_map(s->v, s->fx, s->fy, p_in, p_out, L0.flag, s->P, W, H, u, s->st);
    s->mg.cur0 ^= 1;
    s->flag_host.assign(new_flag, new_flag + (size_t)W * H);
    s->flag_changed();
    s->sync();
    return UBG_OK;
  });
}

// ----------------------------------------------------- snapshot / restore
namespace {
struct SnapHeader {
  char magic[8];  // "UBGSNAP1"
  int32_t version, width, height, nsinks;
  float pwidth, mu, h, last_dt;
  int32_t bc[4];
  int32_t reserved[4];
};
constexpr int kSnapFields[] = {UBG_VX, UBG_VX_BACK, UBG_VY, UBG_VY_BACK, UBG_P,
                               UBG_F,  UBG_VX_ACCUM, UBG_VY_ACCUM};

size_t snap_bytes(const ubg_sim *s) {
  size_t W = s->W, H = s->H;
  size_t fl = 2 * ((W - 1) * H + W * (H - 1)) + 2 * W * H + ((W - 1) * H + W * (H - 1));
  return sizeof(SnapHeader) + (size_t)kMaxSinks * 3 * sizeof(float) + fl * sizeof(float) + W * H;
}
}  // namespace

int ubg_snapshot_bytes(ubg_sim *s, size_t *bytes) {
  return guarded([&] {
    if (!s || !bytes) throw ArgError("null argument");
    *bytes = snap_bytes(s);
    return UBG_OK;
  });
}

int ubg_snapshot(ubg_sim *s, void *dst) {
  return guarded([&] {
    if (!s || !dst) throw ArgError("null argument");
    char *o = (char *)dst;
    SnapHeader hd{};
    std::memcpy(hd.magic, "UBGSNAP1", 8);
    hd.version = 1;
    hd.width = s->W;
    hd.height = s->H;
    hd.nsinks = (int32_t)s->sinks.size();
    hd.pwidth = s->pwidth;
    hd.mu = s->mu;
    hd.h = s->h;
    hd.last_dt = s->last_dt;
    hd.bc[0] = s->bc.w;
    hd.bc[1] = s->bc.e;
    hd.bc[2] = s->bc.n;
    hd.bc[3] = s->bc.s;
    std::memcpy(o, &hd, sizeof(hd));
    o += sizeof(hd);
    float *sk = (float *)o;
    for (size_t i = 0; i < (size_t)kMaxSinks; i++) {
      bool have = i < s->sinks.size();
      sk[3 * i] = have ? s->sinks[i].x : 0.0f;
      sk[3 * i + 1] = have ? s->sinks[i].y : 0.0f;
      sk[3 * i + 2] = have ? s->sinks[i].z : 0.0f;
    }
    o += (size_t)kMaxSinks * 3 * sizeof(float);
    for (int f : kSnapFields) {
      FieldView fv = field_view(s, f);
      UBG_CUDA(cudaMemcpy2DAsync(o, (size_t)fv.w * 4, fv.dev, (size_t)s->P * 4, (size_t)fv.w * 4,
                                 fv.h, cudaMemcpyDeviceToHost, s->st));
      o += (size_t)fv.w * fv.h * 4;
    }
    s->sync();
    for (size_t i = 0; i < s->flag_host.size(); i++) o[i] = s->flag_host[i] != 0.0f ? 1 : 0;
    return UBG_OK;
  });
}

int ubg_restore(ubg_sim *s, const void *src) {
  return guarded([&] {
    if (!s || !src) throw ArgError("null argument");
    const char *o = (const char *)src;
    SnapHeader hd;
    std::memcpy(&hd, o, sizeof(hd));
    if (std::memcmp(hd.magic, "UBGSNAP1", 8) != 0 || hd.version != 1)
      throw ArgError("not a snapshot of this format");
    if (hd.width != s->W || hd.height != s->H) throw ArgError("snapshot grid size differs");
    if (hd.nsinks < 0 || hd.nsinks > kMaxSinks) throw ArgError("snapshot sink count");
    o += sizeof(hd);
    const float *sk = (const float *)o;
    s->sinks.clear();
    for (int i = 0; i < hd.nsinks; i++) s->sinks.push_back(HostSink{sk[3 * i], sk[3 * i + 1], sk[3 * i + 2]});
    o += (size_t)kMaxSinks * 3 * sizeof(float);
    s->sync();
    for (int f : kSnapFields) {
      FieldView fv = field_view(s, f);
      UBG_CUDA(cudaMemcpy2DAsync(fv.dev, (size_t)s->P * 4, o, (size_t)fv.w * 4, (size_t)fv.w * 4,
                                 fv.h, cudaMemcpyHostToDevice, s->st));
      o += (size_t)fv.w * fv.h * 4;
    }
    std::vector<float> fl((size_t)s->W * s->H);
    for (size_t i = 0; i < fl.size(); i++) fl[i] = o[i] ? 1.0f : 0.0f;
    upload_flag_u8(s->mg.lv[0], fl.data(), s->W, s->H, s->st);
    s->flag_host.swap(fl);
    s->bc = Bcs{hd.bc[0], hd.bc[1], hd.bc[2], hd.bc[3]};
    s->last_dt = hd.last_dt;
    s->accum_dirty = true;
    s->gen++;
    s->flag_changed();
    s->sync();
    return UBG_OK;
  });
}

// -------------------------------------------------------------- autotuner
int ubg_autotune(ubg_sim *s, char *report, size_t len) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    s->sync();
    std::string rep;
    mg_autotune(s->mg, s->st, &rep);
    s->gen++;  // the captured step uses the old tiles
    if (report && len) {
      size_t n = std::min(len - 1, rep.size());
      std::memcpy(report, rep.data(), n);
      report[n] = 0;
    }
    return UBG_OK;
  });
}

// ------------------------------------------------------- fused stepping
// Records the launches of one step of every member as fused slots, in the
// order of ubg_sim::step_body, for the members' current indices; cfl[i] is
// member i's dt factor.  afx / afy receive the indices after the step.
void fused_plan(const std::vector<ubg_sim *> &sims, const float *cfl,
                std::vector<MultiSlot> &slots, std::vector<int> &afx, std::vector<int> &afy) {
  const int n = (int)sims.size();
  std::vector<int> fx(n), fy(n);
  for (int i = 0; i < n; i++) {
    fx[i] = sims[i]->fx;
    fy[i] = sims[i]->fy;
  }
  auto add = [&](MultiSlot &sl, const void *a, size_t bytes, int blocks) {
    const char *p = (const char *)a;
    sl.args.insert(sl.args.end(), p, p + bytes);
    if (sl.bs.empty()) sl.bs.push_back(0);
    sl.bs.push_back(sl.bs.back() + blocks);
    sl.blocks += blocks;
    sl.n++;
  };
  auto vbc = [&](bool dvx, bool dvy, bool umax) {
    MultiSlot sl;
    sl.kind = MK_VBC;
    for (int i = 0; i < n; i++) {
      ubg_sim *s = sims[i];
      VbcM a{s->v, fx[i], fy[i], dvx, dvy, s->bc, umax ? s->d_umax : nullptr};
      add(sl, &a, sizeof(a), multi_blocks_vbc(a));
    }
    slots.push_back(std::move(sl));
  };
  {  // dt = cfl h / max|u| from the previous step's max|u|
    MultiSlot sl;
    sl.kind = MK_CFL;
    for (int i = 0; i < n; i++) {
      ubg_sim *s = sims[i];
      CflM a{s->d_umax, cfl[i], s->h, s->mu, s->pwidth, s->W, s->d_sc};
      add(sl, &a, sizeof(a), 0);
    }
    slots.push_back(std::move(sl));
  }
  // diffuse (simulation.cpp:104-162)
  vbc(false, true, false);
  for (int k = 0; k < 2; k++) {
    MultiSlot sl;
    sl.kind = MK_DIFFUSE;
    for (int i = 0; i < n; i++) {
      ubg_sim *s = sims[i];
      DiffuseM a{s->v, fx[i], fy[i], 3, 0, 0, s->d_sc};
      int b = multi_blocks_diffuse(a);
      add(sl, &a, sizeof(a), b);
      fx[i] ^= 1;
      fy[i] ^= 1;
    }
    slots.push_back(std::move(sl));
    vbc(true, true, false);
  }
  {  // advect
    MultiSlot sl;
    sl.kind = MK_ADVECT;
    for (int i = 0; i < n; i++) {
      ubg_sim *s = sims[i];
      AdvectM a{s->v, fx[i], fy[i], 0, s->d_sc};
      int b = multi_blocks_advect(a);
      add(sl, &a, sizeof(a), b);
      fx[i] ^= 1;
      fy[i] ^= 1;
    }
    slots.push_back(std::move(sl));
  }
  vbc(true, true, false);
  {  // project: divergence
    MultiSlot sl;
    sl.kind = MK_DIVERGENCE;
    for (int i = 0; i < n; i++) {
      ubg_sim *s = sims[i];
      DivergenceM a{s->v.vx[fx[i]], s->v.vy[fy[i]], s->f(), s->P, s->W, s->H, 0, s->d_sc};
      int b = multi_blocks_divergence(a);
      add(sl, &a, sizeof(a), b);
    }
    slots.push_back(std::move(sl));
  }
  std::vector<MgHier *> mgs;
  for (auto *s : sims) mgs.push_back(&s->mg);
  const int vc = sims[0]->opt.vcycles;
  for (auto *s : sims)
    if (s->opt.vcycles != vc) throw ArgError("fused batch: members need the same V-cycle count");
  for (int c = 0; c < vc; c++) mg_multi_vcycle(mgs, slots);
  {  // setPBC, then the gradient update with max|u| (umax zeroed first)
    MultiSlot sl;
    sl.kind = MK_PBC;
    for (int i = 0; i < n; i++) {
      ubg_sim *s = sims[i];
      PbcM a{s->p(), s->P, s->W, s->H, s->bc, s->d_umax};
      add(sl, &a, sizeof(a), multi_blocks_pbc(a));
    }
    slots.push_back(std::move(sl));
  }
  {
    MultiSlot sl;
    sl.kind = MK_GRADIENT;
    for (int i = 0; i < n; i++) {
      ubg_sim *s = sims[i];
      GradientM a{s->v, fx[i], fy[i], 0, s->p(), s->d_sc, s->d_umax};
      int b = multi_blocks_gradient(a);
      add(sl, &a, sizeof(a), b);
    }
    slots.push_back(std::move(sl));
  }
  vbc(true, true, true);
  afx = fx;
  afy = fy;
}


// Packs the slots into one table: arguments and block prefix sums of each
// slot, 256-byte aligned, each prefix-sum array followed by `tag` (the word
// the kernels check); returns the bytes.
size_t fused_pack(const std::vector<MultiSlot> &slots, unsigned tag, std::vector<char> &host,
                  std::vector<size_t> &aoff, std::vector<size_t> &boff) {
  aoff.assign(slots.size(), 0);
  boff.assign(slots.size(), 0);
  size_t bytes = 0;
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  for (size_t i = 0; i < slots.size(); i++) {
    aoff[i] = bytes;
    bytes += al(slots[i].args.size());
    boff[i] = bytes;
    bytes += al((slots[i].bs.size() + 1) * sizeof(int));
  }
  host.assign(bytes, 0);
  for (size_t i = 0; i < slots.size(); i++) {
    const MultiSlot &sl = slots[i];
    if (sl.bs.size() != (size_t)sl.n + 1) throw std::logic_error("fused slot prefix sums");
    std::memcpy(host.data() + aoff[i], sl.args.data(), sl.args.size());
    std::memcpy(host.data() + boff[i], sl.bs.data(), sl.bs.size() * sizeof(int));
    std::memcpy(host.data() + boff[i] + sl.bs.size() * sizeof(int), &tag, sizeof(tag));
  }
  return bytes;
}

// A fresh tag for each packed table.
unsigned fused_tag() {
  static std::atomic<unsigned> next{0x5eed0001u};
  return next.fetch_add(2u);
}

// A word in mapped pinned host memory that the fused kernels flag errors in.
unsigned *alloc_err_word() {
  void *p = nullptr;
  if (cudaHostAlloc(&p, 64, cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    throw std::bad_alloc();
  }
  *(volatile unsigned *)p = 0u;
  return (unsigned *)p;
}

void fused_launch(const std::vector<MultiSlot> &slots, const char *dtable,
                  const std::vector<size_t> &aoff, const std::vector<size_t> &boff, unsigned tag,
                  unsigned *err, cudaStream_t st) {
  for (size_t i = 0; i < slots.size(); i++) {
    const MultiSlot &sl = slots[i];
    const int *bs = (const int *)(dtable + boff[i]);
    if (sl.kind == MK_MG || sl.kind == MK_TAIL)
      launch_multi_mg(sl, dtable + aoff[i], bs, tag, err, st);
    else
      launch_multi_step(sl.kind, dtable + aoff[i], bs, sl.n, sl.blocks, tag, err, st);
  }
}

namespace ubg {
struct FusedStepper::Impl {
  static constexpr int kSlots = 2;  // steps in flight
  cudaStream_t st = nullptr;
  cudaEvent_t ev[kSlots] = {}, join_ev = nullptr;
  unsigned *err = nullptr;  // mapped host word
  bool used[kSlots] = {};
  char *host[kSlots] = {};
  void *dev[kSlots] = {};
  size_t cap[kSlots] = {};
  int next = 0;
  std::vector<MultiSlot> slots;
  std::vector<char> pack;
  std::vector<size_t> aoff, boff;
  std::vector<int> afx, afy;
};

FusedStepper::FusedStepper() : p_(new Impl()) {
  try {
    // high priority: a fused step is many short dependent launches, which
    // would otherwise queue behind the long kernels of other streams
    int lo = 0, hi = 0;
    UBG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    UBG_CUDA(cudaStreamCreateWithPriority(&p_->st, cudaStreamNonBlocking, hi));
    UBG_CUDA(cudaEventCreateWithFlags(&p_->join_ev, cudaEventDisableTiming));
    for (auto &e : p_->ev) UBG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    p_->err = alloc_err_word();
  } catch (...) {
    this->~FusedStepper();
    throw;
  }
}

FusedStepper::~FusedStepper() {
  if (!p_) return;
  if (p_->st) cudaStreamSynchronize(p_->st);
  for (int k = 0; k < Impl::kSlots; k++) {
    if (p_->host[k]) cudaFreeHost(p_->host[k]);
    if (p_->dev[k]) cudaFree(p_->dev[k]);
    if (p_->ev[k]) cudaEventDestroy(p_->ev[k]);
  }
  if (p_->join_ev) cudaEventDestroy(p_->join_ev);
  if (p_->err) cudaFreeHost(p_->err);
  if (p_->st) cudaStreamDestroy(p_->st);
  delete p_;
  p_ = nullptr;
}

bool FusedStepper::eligible(const ubg_sim *s) {
  return s->opt.precision == UBG_FP32 && s->opt.solver_mode == UBG_SOLVE_FIXED &&
         !s->opt.advect_bilinear && s->opt.vcycles >= 1 && s->mg.tail_top >= 1 &&
         s->sinks.empty() && !s->prof;
}

int FusedStepper::group(const ubg_sim *s) { return s->opt.vcycles; }

void FusedStepper::join(ubg_sim *s) {
  s->io_consume();
  bool accum = s->accum_dirty;
  if (accum) s->apply_accum();
  // max|u| of the current fields for the first fused step's dt (the
  // scalars this also writes are recomputed by that step's own CFL launch
  // with the request's factor)
  if (!s->umax_ready || accum)
    launch_cfl(s->v, s->fx, s->fy, 0.5f, s->h, s->mu, s->pwidth, s->d_umax, s->d_sc, s->st, false);
  s->umax_ready = true;
  UBG_CUDA(cudaEventRecord(p_->join_ev, s->st));
  UBG_CUDA(cudaStreamWaitEvent(p_->st, p_->join_ev, 0));
}

bool FusedStepper::ready() const {
  return !p_->used[p_->next] || cudaEventQuery(p_->ev[p_->next]) != cudaErrorNotReady;
}

void FusedStepper::step(const std::vector<ubg_sim *> &sims, const std::vector<float> &cfl) {
  if (sims.empty()) return;
  if (cfl.size() != sims.size()) throw ArgError("one cfl per member");
  Impl &m = *p_;
  const int k = m.next;
  m.next = (m.next + 1) % Impl::kSlots;
  if (m.used[k]) UBG_CUDA(cudaEventSynchronize(m.ev[k]));
  m.slots.clear();
  fused_plan(sims, cfl.data(), m.slots, m.afx, m.afy);
  const unsigned tag = fused_tag();
  size_t bytes = fused_pack(m.slots, tag, m.pack, m.aoff, m.boff);
  if (bytes > m.cap[k]) {
    if (m.host[k]) cudaFreeHost(m.host[k]);
    if (m.dev[k]) cudaFree(m.dev[k]);
    m.host[k] = nullptr;
    m.dev[k] = nullptr;
    m.cap[k] = 0;
    size_t b = std::max(bytes * 2, (size_t)1 << 16);
    if (cudaMallocHost((void **)&m.host[k], b) != cudaSuccess ||
        cudaMalloc(&m.dev[k], b) != cudaSuccess) {
      cudaGetLastError();
      throw std::bad_alloc();
    }
    m.cap[k] = b;
  }
  std::memcpy(m.host[k], m.pack.data(), bytes);
  UBG_CUDA(cudaMemcpyAsync(m.dev[k], m.host[k], bytes, cudaMemcpyHostToDevice, m.st));
  fused_launch(m.slots, (const char *)m.dev[k], m.aoff, m.boff, tag, m.err, m.st);
  UBG_CUDA(cudaEventRecord(m.ev[k], m.st));
  m.used[k] = true;
  for (size_t i = 0; i < sims.size(); i++) {
    ubg_sim *s = sims[i];
    s->fx = m.afx[i];
    s->fy = m.afy[i];
    s->umax_ready = true;
    s->last_vcycles = s->opt.vcycles;
  }
}

bool FusedStepper::failed() const { return *(volatile unsigned *)p_->err != 0u; }

void FusedStepper::leave(ubg_sim *s, cudaEvent_t ev) {
  UBG_CUDA(cudaEventRecord(ev, p_->st));
  UBG_CUDA(cudaStreamWaitEvent(s->st, ev, 0));
}
}  // namespace ubg

// ----------------------------------------------------------------- batch
// Many independent simulations advanced by one graph launch: each member's
// fixed-cycle step body is captured on its own stream as a parallel branch
// of one CUDA graph, so the members' kernels run concurrently and the host
// issues one launch per batch step.
struct ubg_batch {
  static constexpr size_t kMaxBranches = 32;
  std::vector<ubg_sim *> sims;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> pre, join;
  // branch form: one graph per index state (steps alternate between two)
  struct Branch {
    cudaGraphExec_t exec = nullptr;
    std::vector<long long> key;
    float cfl = -1.0f;
    std::vector<int> after_fx, after_fy, after_cur0;
    long launches = 0;
  };
  Branch br[2];
  int br_next = 0;
  // fused form: every launch covers all members (one graph per index parity)
  struct Fused {
    std::vector<long long> key;
    cudaGraphExec_t exec = nullptr;
    void *table = nullptr;
    std::vector<int> after_fx, after_fy, after_cur0;
    long launches = 0;
  };
  Fused fused[2];
  int fused_next = 0;
  bool use_fused = true;
  unsigned *err = nullptr;  // mapped host word the fused kernels flag errors in

  void check_fused() const {
    if (err && *(volatile unsigned *)err)
      throw CudaError("fused batch step: a launch found a table it was not made for");
  }

  ~ubg_batch() {
    if (st) cudaStreamSynchronize(st);
    for (auto &f : fused) {
      if (f.exec) cudaGraphExecDestroy(f.exec);
      if (f.table) cudaFree(f.table);
    }
    for (auto &b : br)
      if (b.exec) cudaGraphExecDestroy(b.exec);
    for (auto e : pre) cudaEventDestroy(e);
    for (auto e : join) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (done) cudaEventDestroy(done);
    if (err) cudaFreeHost(err);
    if (st) cudaStreamDestroy(st);
  }

  std::vector<long long> make_key(bool device_dt) const {
    std::vector<long long> k;
    k.push_back(device_dt);
    for (auto *s : sims)
      k.push_back(((long long)s->fx << 2) | (s->fy << 1) | s->mg.cur0 |
                  ((long long)s->opt.vcycles << 3) | ((long long)s->opt.precision << 24) |
                  ((long long)s->mg.tail_top << 32));
    for (auto *s : sims) k.push_back(s->gen);
    return k;
  }

  Branch &capture(bool device_dt, float cfl) {
    Branch &b = br[br_next];
    br_next ^= 1;
    if (b.exec) {
      cudaGraphExecDestroy(b.exec);
      b.exec = nullptr;
    }
    long l0 = g_stats.launches;
    size_t n = sims.size();
    b.after_fx.assign(n, 0);
    b.after_fy.assign(n, 0);
    b.after_cur0.assign(n, 0);
    std::vector<int> fx0(n), fy0(n), c00(n);
    for (size_t i = 0; i < n; i++) {
      fx0[i] = sims[i]->fx;
      fy0[i] = sims[i]->fy;
      c00[i] = sims[i]->mg.cur0;
    }
    cudaGraph_t g = nullptr;
    UBG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      UBG_CUDA(cudaEventRecord(fork, st));
      for (size_t i = 0; i < n; i++) {
        ubg_sim *s = sims[i];
        UBG_CUDA(cudaStreamWaitEvent(s->st, fork, 0));
        if (device_dt)
          launch_cfl(s->v, s->fx, s->fy, cfl, s->h, s->mu, s->pwidth, s->d_umax, s->d_sc, s->st,
                     true);
        s->step_body(0);
        UBG_CUDA(cudaEventRecord(join[i], s->st));
        UBG_CUDA(cudaStreamWaitEvent(st, join[i], 0));
        b.after_fx[i] = s->fx;
        b.after_fy[i] = s->fy;
        b.after_cur0[i] = s->mg.cur0;
        s->fx = fx0[i];
        s->fy = fy0[i];
        s->mg.cur0 = c00[i];
      }
    } catch (...) {
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      for (size_t i = 0; i < n; i++) {
        sims[i]->fx = fx0[i];
        sims[i]->fy = fy0[i];
        sims[i]->mg.cur0 = c00[i];
      }
      throw;
    }
    UBG_CUDA(cudaStreamEndCapture(st, &g));
    UBG_CUDA(cudaGraphInstantiate(&b.exec, g, 0));
    cudaGraphDestroy(g);
    b.launches = g_stats.launches - l0;
    g_stats.launches = l0;
    b.key = make_key(device_dt);
    b.cfl = cfl;
    return b;
  }

  // Members the fused launches take: FP32, fixed V-cycle count, a coarse
  // tail, at most kFuseMaxCells cells; the others become graph branches of
  // the same step.  Measured on GB300: fused launches win by far for small
  // members (64 x 128x64: 0.24 vs 3.9 ms per batch step; 64 x 512x256: 1.8
  // vs 5.6 ms); members of 2 M cells run ~7 % faster as concurrent
  // branches.  The fused form needs a device-side dt and two small members.
  bool partition(bool device_dt, std::vector<int> &small, std::vector<int> &big) const {
    small.clear();
    big.clear();
    if (!use_fused || !device_dt) return false;
    const int vc = sims[0]->opt.vcycles;
    for (size_t i = 0; i < sims.size(); i++) {
      ubg_sim *s = sims[i];
      if (FusedStepper::eligible(s) && s->opt.vcycles == vc &&
          (long long)s->W * s->H <= kFuseMaxCells)
        small.push_back((int)i);
      else
        big.push_back((int)i);
    }
    return small.size() >= 2;
  }

  // One graph per index state: fused launches over the small members on
  // the batch stream, the big members' step bodies as branches beside them.
  Fused &fused_graph(float cfl, const std::vector<int> &small, const std::vector<int> &big) {
    std::vector<long long> k = make_key(true);
    k.push_back((long long)__builtin_bit_cast(unsigned, cfl));
    for (auto &f : fused)
      if (f.exec && f.key == k) return f;
    Fused &f = fused[fused_next];
    fused_next ^= 1;
    if (f.exec) {
      UBG_CUDA(cudaStreamSynchronize(st));
      cudaGraphExecDestroy(f.exec);
      f.exec = nullptr;
    }
    if (f.table) {
      cudaFree(f.table);
      f.table = nullptr;
    }
    const size_t n = sims.size();
    f.after_fx.assign(n, 0);
    f.after_fy.assign(n, 0);
    f.after_cur0.assign(n, 0);
    std::vector<ubg_sim *> ss;
    for (int i : small) ss.push_back(sims[i]);
    std::vector<MultiSlot> slots;
    std::vector<float> cfls(ss.size(), cfl);
    std::vector<int> afx, afy;
    fused_plan(ss, cfls.data(), slots, afx, afy);
    for (size_t j = 0; j < small.size(); j++) {
      f.after_fx[small[j]] = afx[j];
      f.after_fy[small[j]] = afy[j];
      f.after_cur0[small[j]] = ss[j]->mg.cur0;
    }
    std::vector<char> host;
    std::vector<size_t> aoff, boff;
    const unsigned tag = fused_tag();
    size_t bytes = fused_pack(slots, tag, host, aoff, boff);
    if (cudaMalloc(&f.table, bytes) != cudaSuccess) {
      cudaGetLastError();
      f.table = nullptr;
      throw std::bad_alloc();
    }
    if (!err) err = alloc_err_word();
    // on the batch stream, complete before the graph can run
    UBG_CUDA(cudaMemcpyAsync(f.table, host.data(), bytes, cudaMemcpyHostToDevice, st));
    UBG_CUDA(cudaStreamSynchronize(st));
    long l0 = g_stats.launches;
    std::vector<int> fx0(n), fy0(n), c00(n);
    for (size_t i = 0; i < n; i++) {
      fx0[i] = sims[i]->fx;
      fy0[i] = sims[i]->fy;
      c00[i] = sims[i]->mg.cur0;
    }
    auto restore = [&] {
      for (size_t i = 0; i < n; i++) {
        sims[i]->fx = fx0[i];
        sims[i]->fy = fy0[i];
        sims[i]->mg.cur0 = c00[i];
      }
    };
    cudaGraph_t g = nullptr;
    UBG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      if (!big.empty()) UBG_CUDA(cudaEventRecord(fork, st));
      for (int i : big) {
        ubg_sim *s = sims[i];
        UBG_CUDA(cudaStreamWaitEvent(s->st, fork, 0));
        launch_cfl(s->v, s->fx, s->fy, cfl, s->h, s->mu, s->pwidth, s->d_umax, s->d_sc, s->st,
                   true);
        s->step_body(0);
        UBG_CUDA(cudaEventRecord(join[i], s->st));
        f.after_fx[i] = s->fx;
        f.after_fy[i] = s->fy;
        f.after_cur0[i] = s->mg.cur0;
      }
      fused_launch(slots, (const char *)f.table, aoff, boff, tag, err, st);
      for (int i : big) UBG_CUDA(cudaStreamWaitEvent(st, join[i], 0));
    } catch (...) {
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      restore();
      throw;
    }
    restore();
    UBG_CUDA(cudaStreamEndCapture(st, &g));
    UBG_CUDA(cudaGraphInstantiate(&f.exec, g, 0));
    cudaGraphDestroy(g);
    f.launches = g_stats.launches - l0;
    g_stats.launches = l0;
    f.key = k;
    return f;
  }

  void step(const float *dts, float cfl) {
    check_fused();
    bool device_dt = dts == nullptr;
    for (size_t i = 0; i < sims.size(); i++) {
      ubg_sim *s = sims[i];
      if (!s->sinks.empty()) throw ArgError("a member has pending sinks (step it with ubg_step)");
      if (s->opt.solver_mode != UBG_SOLVE_FIXED) throw ArgError("batch steps need the fixed solver mode");
      if (s->prof) throw ArgError("a member is profiling");
    }
    {
      // Many members and no fused launches (every member mixed-precision or
      // large): one graph with a branch per member ran 256 members at 0.69x
      // the members' own step graphs launched on their own streams
      // (GB300), so past kMaxBranches each member launches its own graph.
      std::vector<int> small, big;
      if (!partition(device_dt, small, big) && sims.size() > kMaxBranches) {
        for (size_t i = 0; i < sims.size(); i++)
          sims[i]->step(device_dt ? 0.0f : dts[i], device_dt, cfl);
        return;
      }
    }
    for (size_t i = 0; i < sims.size(); i++) {
      ubg_sim *s = sims[i];
      // work outside the graph, on the member's stream
      s->io_consume();
      bool accum = s->accum_dirty;
      if (accum) s->apply_accum();
      if (!device_dt)
        s->push_scalars(dts[i]);
      else if (!s->umax_ready || accum)
        launch_cfl(s->v, s->fx, s->fy, cfl, s->h, s->mu, s->pwidth, s->d_umax, s->d_sc, s->st,
                   false);
      UBG_CUDA(cudaEventRecord(pre[i], s->st));
    }
    std::vector<int> small, big;
    if (partition(device_dt, small, big)) {
      Fused &f = fused_graph(cfl, small, big);
      for (size_t i = 0; i < sims.size(); i++) UBG_CUDA(cudaStreamWaitEvent(st, pre[i], 0));
      UBG_CUDA(cudaGraphLaunch(f.exec, st));
      UBG_CUDA(cudaEventRecord(done, st));
      for (size_t i = 0; i < sims.size(); i++) {
        ubg_sim *s = sims[i];
        UBG_CUDA(cudaStreamWaitEvent(s->st, done, 0));
        s->fx = f.after_fx[i];
        s->fy = f.after_fy[i];
        s->mg.cur0 = f.after_cur0[i];
        s->umax_ready = true;
        s->last_vcycles = s->opt.vcycles;
      }
      g_stats.launches += f.launches;
      return;
    }
    auto k = make_key(device_dt);
    Branch *b = nullptr;
    for (auto &c : br)
      if (c.exec && c.key == k && c.cfl == cfl) b = &c;
    if (!b) b = &capture(device_dt, cfl);
    for (size_t i = 0; i < sims.size(); i++) UBG_CUDA(cudaStreamWaitEvent(st, pre[i], 0));
    UBG_CUDA(cudaGraphLaunch(b->exec, st));
    UBG_CUDA(cudaEventRecord(done, st));
    for (size_t i = 0; i < sims.size(); i++) {
      ubg_sim *s = sims[i];
      UBG_CUDA(cudaStreamWaitEvent(s->st, done, 0));
      s->fx = b->after_fx[i];
      s->fy = b->after_fy[i];
      s->mg.cur0 = b->after_cur0[i];
      s->umax_ready = true;
      s->last_vcycles = s->opt.vcycles;
    }
    g_stats.launches += b->launches;
  }
};

int ubg_batch_create(int n, ubg_sim *const *sims, ubg_batch **out) {
  return guarded([&] {
    if (n < 1 || !sims || !out) throw ArgError("null argument");
    std::unique_ptr<ubg_batch> b(new ubg_batch());
    for (int i = 0; i < n; i++) {
      if (!sims[i]) throw ArgError("null member");
      for (int j = 0; j < i; j++)
        if (sims[j] == sims[i]) throw ArgError("a simulation appears twice in the batch");
      b->sims.push_back(sims[i]);
    }
    UBG_CUDA(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
    UBG_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    UBG_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    b->pre.assign(n, nullptr);
    b->join.assign(n, nullptr);
    for (int i = 0; i < n; i++) {
      UBG_CUDA(cudaEventCreateWithFlags(&b->pre[i], cudaEventDisableTiming));
      UBG_CUDA(cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming));
    }
    *out = b.release();
    return UBG_OK;
  });
}

int ubg_batch_destroy(ubg_batch *b) {
  return guarded([&] {
    delete b;
    return UBG_OK;
  });
}

int ubg_batch_step(ubg_batch *b, const float *dts, float cfl) {
  return guarded([&] {
    if (!b) throw ArgError("null handle");
    if (!dts && !(cfl > 0.0f)) throw ArgError("cfl must be > 0 when dts is NULL");
    b->step(dts, cfl);
    return UBG_OK;
  });
}

int ubg_batch_stream(ubg_batch *b, void **stream) {
  if (!b || !stream) return fail(UBG_EINVAL, "null argument");
  *stream = (void *)b->st;
  return UBG_OK;
}

int ubg_batch_sync(ubg_batch *b) {
  return guarded([&] {
    if (!b) throw ArgError("null handle");
    UBG_CUDA(cudaStreamSynchronize(b->st));
    b->check_fused();
    return UBG_OK;
  });
}

// Device bytes a simulation of this size holds (fields + multigrid), and the
// bytes a live handle holds now (plus the mixed-precision hierarchy and
// scratch buffers it allocated).
static size_t sim_bytes_for(int W, int H) {
  size_t P = (size_t)round_up(W, 32), n = P * (size_t)H;
  size_t fb = (n * 4 + 255) / 256 * 256, bb = (n + 255) / 256 * 256;
  return 6 * fb + 2 * bb + 256 * 3 + (size_t)kMaxSinks * 9 * sizeof(SinkCell) + mg_arena_bytes(W, H);
}

int ubg_device_bytes(int width, int height, size_t *bytes) {
  return guarded([&] {
    if (!bytes || width < 8 || height < 8) throw ArgError("bad argument");
    *bytes = sim_bytes_for(width, height);
    return UBG_OK;
  });
}

int ubg_sim_device_bytes(ubg_sim *s, size_t *bytes) {
  return guarded([&] {
    if (!s || !bytes) throw ArgError("null argument");
    size_t lo = 0;
    if (s->lo.levels) {
      for (auto &L : s->mg.lv) lo += 3 * (((size_t)L.pitch * L.h * 2 + 255) / 256 * 256);
      lo += ((size_t)s->P * s->H * 4 + 255) / 256 * 256 + 256;
    }
    size_t fb = 0;
    if (s->fcg.arena) fb = fcg_bytes(s->W, s->H, s->P, s->fcg.prec);
    *bytes = s->arena_bytes + s->mg.arena_bytes + lo + fb + s->scratch_bytes;
    return UBG_OK;
  });
}

// ------------------------------------------------------ asynchronous host I/O
int ubg_io_upload_async(ubg_sim *s, const float *vx, const float *vy) {
  return guarded([&] {
    if (!s || !vx || !vy) throw ArgError("null argument");
    s->io_init();
    // the staging buffers are free once the previous staged inputs were consumed
    UBG_CUDA(cudaStreamWaitEvent(s->io_st, s->io_in_free, 0));
    UBG_CUDA(cudaMemcpy2DAsync(s->io_in[0], (size_t)s->P * 4, vx, (size_t)(s->W - 1) * 4,
                               (size_t)(s->W - 1) * 4, s->H, cudaMemcpyHostToDevice, s->io_st));
    UBG_CUDA(cudaMemcpy2DAsync(s->io_in[1], (size_t)s->P * 4, vy, (size_t)s->W * 4, (size_t)s->W * 4,
                               s->H - 1, cudaMemcpyHostToDevice, s->io_st));
    UBG_CUDA(cudaEventRecord(s->io_in_ready, s->io_st));
    s->io_staged = true;
    return UBG_OK;
  });
}

int ubg_io_download_async(ubg_sim *s, float *vx, float *vy) {
  return guarded([&] {
    if (!s || !vx || !vy) throw ArgError("null argument");
    s->io_init();
    // snapshot the current fields on the simulation's stream (the next step
    // overwrites them), then copy to the host on the I/O stream
    UBG_CUDA(cudaStreamWaitEvent(s->st, s->io_out_done, 0));
    launch_stage_out(s->v, s->fx, s->fy, s->io_out[0], s->io_out[1], s->st);
    UBG_CUDA(cudaEventRecord(s->io_out_copied, s->st));
    UBG_CUDA(cudaStreamWaitEvent(s->io_out_st, s->io_out_copied, 0));
    UBG_CUDA(cudaMemcpy2DAsync(vx, (size_t)(s->W - 1) * 4, s->io_out[0], (size_t)s->P * 4,
                               (size_t)(s->W - 1) * 4, s->H, cudaMemcpyDeviceToHost, s->io_out_st));
    UBG_CUDA(cudaMemcpy2DAsync(vy, (size_t)s->W * 4, s->io_out[1], (size_t)s->P * 4, (size_t)s->W * 4,
                               s->H - 1, cudaMemcpyDeviceToHost, s->io_out_st));
    UBG_CUDA(cudaEventRecord(s->io_out_done, s->io_out_st));
    return UBG_OK;
  });
}

int ubg_io_wait(ubg_sim *s) {
  return guarded([&] {
    if (!s) throw ArgError("null handle");
    if (s->io_st) UBG_CUDA(cudaStreamSynchronize(s->io_st));
    if (s->io_out_st) UBG_CUDA(cudaStreamSynchronize(s->io_out_st));
    return UBG_OK;
  });
}

int ubg_selftest_div(const float *x, int n, float d, unsigned *mismatches) {
  return guarded([&] {
    if (!x || n < 1 || !mismatches || !(d > 0.0f)) throw ArgError("bad argument");
    selftest_div_rn(x, n, d, mismatches);
    return UBG_OK;
  });
}
