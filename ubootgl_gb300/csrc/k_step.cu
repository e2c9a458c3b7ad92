// Step kernels of the fluid time step: boundary conditions, diffusion,
// semi-Lagrangian bicubic advection, divergence, pressure gradient, and the
// accumulated-velocity update.  Each kernel restates one reference function
// (te42kyfo/ubootgl, file:line in the comments) in the reference's operation
// order; the library is compiled with -fmad=false, so results match the FP32
// CPU restatement bit for bit.
#include "ubg_internal.cuh"

namespace ubg {

thread_local LaunchStats g_stats;
thread_local Profiler *g_prof = nullptr;

const char *kernel_class_name(int kc) {
  static const char *n[KC_COUNT] = {"vbc", "accum", "diffuse", "advect", "divergence", "sinks",
                                    "pbc", "gradient", "cfl", "smooth_l0", "smooth_coarse",
                                    "resid_restrict_l0", "resid_restrict_coarse", "coarsen",
                                    "residual", "tracers", "other"};
  return (kc >= 0 && kc < KC_COUNT) ? n[kc] : "?";
}

cudaEvent_t Profiler::next() {
  if (used == pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    pool.push_back(e);
  }
  return pool[used++];
}

void Profiler::collect() {
  for (auto &m : marks) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, pool[m.a], pool[m.b]) == cudaSuccess) {
      total_ms[m.kc] += ms;
      count[m.kc] += 1;
    }
  }
  cudaGetLastError();
  marks.clear();
  used = 0;
}

Profiler::~Profiler() {
  for (auto e : pool) cudaEventDestroy(e);
}

namespace {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ float ld(const float *p, int pitch, int x, int y) {
  return __ldg(p + (size_t)y * pitch + x);
}
__device__ __forceinline__ float fl(const uint8_t *f, int pitch, int x, int y) {
  return (float)__ldg(f + (size_t)y * pitch + x);
}

// VBCPar / VBCPer / singlePBC, simulation.cpp:22-78.
__device__ __forceinline__ float vbc_par(int bc, float a, float b) {
  if (bc == UBG_BC_INFLOW) return b;
  if (bc == UBG_BC_OUTFLOW || bc == UBG_BC_OUTFLOW_ZERO_PRESSURE) return a > 0.0f ? a : 0.0f;
  return 0.0f;
}
__device__ __forceinline__ float vbc_per(int bc, float a, float b) {
  if (bc == UBG_BC_INFLOW) return b;
  if (bc == UBG_BC_OUTFLOW || bc == UBG_BC_OUTFLOW_ZERO_PRESSURE) return a > 0.0f ? a : 0.0f;
  return -a;
}
__device__ __forceinline__ float single_pbc(int bc, float a) {
  return bc == UBG_BC_OUTFLOW_ZERO_PRESSURE ? -a : a;
}

// ------------------------------------------------------------------ setVBCs
// The reference first sets the x-edges for every row, then the y-edges for
// every column (which fixes the corners), reading the front buffer and
// writing both buffers.  Phase-1 threads own rows 1..h-2 of the two edge
// columns; phase-2 threads own whole columns of the two edge rows and
// recompute the phase-1 value they need.  The two columns next to each
// corner are handled by the corner's thread, because the corner's phase-1
// value reads the old row-0 value of its neighbour.
template <bool XPAR>
__device__ void vbc_component(const float *s, float *b0, float *b1, int pitch, int w, int h,
                              Bcs bc, int t) {
  // XPAR: x-edges use VBCPar and y-edges VBCPer (vx); otherwise swapped (vy).
  auto edge_x = [&](int side_bc, float a, float b) {
    return XPAR ? vbc_par(side_bc, a, b) : vbc_per(side_bc, a, b);
  };
  auto edge_y = [&](int side_bc, float a, float b) {
    return XPAR ? vbc_per(side_bc, a, b) : vbc_par(side_bc, a, b);
  };
  auto S = [&](int x, int y) { return s[(size_t)y * pitch + x]; };
  auto put = [&](int x, int y, float v) {
    b0[(size_t)y * pitch + x] = v;
    b1[(size_t)y * pitch + x] = v;
  };
  auto p1 = [&](int x, int y) {
    if (x == 0) return edge_x(bc.w, S(1, y), S(0, y));
    if (x == w - 1) return edge_x(bc.e, S(w - 2, y), S(w - 1, y));
    return S(x, y);
  };
  int n1 = h - 2;
  if (t < n1) {
    int y = t + 1;
    float l = edge_x(bc.w, S(1, y), S(0, y));
    float r = edge_x(bc.e, S(w - 2, y), S(w - 1, y));
    put(0, y, l);
    put(w - 1, y, r);
    return;
  }
  t -= n1;
  if (t >= w) return;
  int x = t;
  if (x == 1 || x == w - 2) return;  // handled by the corner threads
  float bot = edge_y(bc.s, p1(x, 1), p1(x, 0));
  float top = edge_y(bc.n, p1(x, h - 2), p1(x, h - 1));
  float bot2 = 0.f, top2 = 0.f;
  int x2 = -1;
  if (x == 0) x2 = 1;
  if (x == w - 1) x2 = w - 2;
  if (x2 >= 0) {
    bot2 = edge_y(bc.s, S(x2, 1), S(x2, 0));
    top2 = edge_y(bc.n, S(x2, h - 2), S(x2, h - 1));
  }
  put(x, 0, bot);
  put(x, h - 1, top);
  if (x2 >= 0) {
    put(x2, 0, bot2);
    put(x2, h - 1, top2);
  }
}

__global__ void k_vbc(VelBufs v, int fx, int fy, Bcs bc, int do_vx, int do_vy) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int W = v.W, H = v.H;
  int nx = (H - 2) + (W - 1);
  if (t < nx) {
    if (do_vx)
      vbc_component<true>(v.vx[fx], v.vx[0], v.vx[1], v.pitch, W - 1, H, bc, t);
    return;
  }
  t -= nx;
  if (do_vy) vbc_component<false>(v.vy[fy], v.vy[0], v.vy[1], v.pitch, W, H - 1, bc, t);
}

// ---------------------------------------------- applyAccumulatedVelocity
__global__ void k_accum(float *vx, float *vy, float *ax, float *ay, int pitch, int W, int H) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  size_t i = (size_t)y * pitch + x;
  if (x >= 1 && x < W - 2 && y >= 1 && y < H - 1) {
    vx[i] = vx[i] + ax[i];
    ax[i] = 0.0f;
  }
  if (x >= 1 && x < W - 1 && y >= 1 && y < H - 2) {
    vy[i] = vy[i] + ay[i];
    ay[i] = 0.0f;
  }
}

// ---------------------------------------------------------------- diffuse
// One Jacobi sweep, simulation.cpp:114-128 (vx) and 140-154 (vy).
__global__ void k_diffuse(VelBufs v, int srcx, int srcy, const uint8_t *__restrict__ flag,
                          const StepScalars *__restrict__ sc, int comps) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  int W = v.W, H = v.H, P = v.pitch;
  float a = sc->a, den = sc->den;
  if (blockIdx.z == 0) {
    if (!(comps & 1) || x < 1 || x >= W - 2 || y < 1 || y >= H - 1) return;
    const float *s = v.vx[srcx];
    float c = ld(s, P, x, y);
    float val = 0.0f;
    val = val + ld(s, P, x + 1, y) * fl(flag, P, x + 1, y) * fl(flag, P, x + 2, y);
    val = val + ld(s, P, x - 1, y) * fl(flag, P, x, y) * fl(flag, P, x - 1, y);
    float fvn = fl(flag, P, x, y + 1) * fl(flag, P, x - 1, y + 1);
    val = val + (ld(s, P, x, y + 1) * fvn + (1.0f - fvn) * -c);
    float fvs = fl(flag, P, x, y - 1) * fl(flag, P, x - 1, y - 1);
    val = val + (ld(s, P, x, y - 1) * fvs + (1.0f - fvs) * -c);
    v.vx[1 - srcx][(size_t)y * P + x] =
        fl(flag, P, x, y) * fl(flag, P, x + 1, y) * (c + a * val) / den;
  } else {
    if (!(comps & 2) || x < 1 || x >= W - 1 || y < 1 || y >= H - 2) return;
    const float *s = v.vy[srcy];
    float c = ld(s, P, x, y);
    float val = 0.0f;
    val = val + ld(s, P, x, y - 1) * fl(flag, P, x, y) * fl(flag, P, x, y - 1);
    val = val + ld(s, P, x, y + 1) * fl(flag, P, x, y + 1) * fl(flag, P, x, y + 2);
    float fve = fl(flag, P, x + 1, y) * fl(flag, P, x + 1, y + 1);
    val = val + (ld(s, P, x + 1, y) * fve + (1.0f - fve) * -c);
    float fvw = fl(flag, P, x - 1, y) * fl(flag, P, x - 1, y + 1);
    val = val + (ld(s, P, x - 1, y) * fvw + (1.0f - fvw) * -c);
    v.vy[1 - srcy][(size_t)y * P + x] =
        fl(flag, P, x, y) * fl(flag, P, x, y + 1) * (c + a * val) / den;
  }
}

// ----------------------------------------------------------------- advect
// CubicHermite (interpolators.hpp:78-85): Catmull-Rom coefficients of the
// reference, evaluated as a Horner polynomial with fused multiply-adds.
__device__ __forceinline__ float cubic_hermite(float t, float A, float B, float C, float D) {
  float a = ((-0.5f * A + 1.5f * B) - 1.5f * C) + 0.5f * D;
  float b = ((A - 2.5f * B) + 2.0f * C) - 0.5f * D;
  float c = 0.5f * (C - A);
  return __fmaf_rn(__fmaf_rn(__fmaf_rn(a, t, b), t, c), t, B);
}

// bicubicSample (interpolators.hpp:92-206): clamp to [3, size-3], truncate,
// vertical pass over 4 rows for 4 columns, then the horizontal pass.
__device__ __forceinline__ float bicubic(const float *__restrict__ g, int pitch, int gw, int gh,
                                         float cx, float cy) {
  float hx = (float)gw - 3.0f, hy = (float)gh - 3.0f;
  cx = cx < hx ? cx : hx;
  cx = cx > 3.0f ? cx : 3.0f;
  cy = cy < hy ? cy : hy;
  cy = cy > 3.0f ? cy : 3.0f;
  int ix = (int)cx, iy = (int)cy;
  float sx = cx - (float)ix, sy = cy - (float)iy;
  const float *r0 = g + (size_t)(iy - 1) * pitch + (ix - 1);
  float col[4];
#pragma unroll
  for (int j = 0; j < 4; j++)
    col[j] = cubic_hermite(sy, __ldg(r0 + j), __ldg(r0 + pitch + j), __ldg(r0 + 2 * pitch + j),
                           __ldg(r0 + 3 * pitch + j));
  return cubic_hermite(sx, col[0], col[1], col[2], col[3]);
}

// The reference advects in chunks of 8 faces from x = 1 while x < width-8
// and skips a chunk when no lane passes the fluid test (simulation.cpp:248,
// 254-256, 300, 302-304).  Returns whether face x of row y is advected.
__device__ __forceinline__ bool advect_mask(const uint8_t *__restrict__ flag, int P, int W,
                                            int x, int y, bool is_vx) {
  int xs = 1 + ((x - 1) >> 3) * 8;
  if (is_vx) {
    if (!(xs < (W - 1) - 8)) return false;
    const uint8_t *r = flag + (size_t)y * P;
#pragma unroll
    for (int i = 0; i < 8; i++)
      if (__ldg(r + xs - 1 + i) && __ldg(r + xs + i)) return true;
    return false;
  } else {
    if (!(xs < W - 8)) return false;
    const uint8_t *r = flag + (size_t)y * P;
    const uint8_t *rm = r - P;
#pragma unroll
    for (int i = 0; i < 8; i++)
      if (__ldg(r + xs + i) && __ldg(rm + xs + i)) return true;
    return false;
  }
}

__global__ void k_advect(VelBufs v, int srcx, int srcy, const uint8_t *__restrict__ flag,
                         const StepScalars *__restrict__ sc) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  int W = v.W, H = v.H, P = v.pitch;
  const float *vx = v.vx[srcx];
  const float *vy = v.vy[srcy];
  float chalf = sc->chalf, cfull = sc->cfull;
  if (blockIdx.z == 0) {
    // vx faces, simulation.cpp:247-298
    if (x < 1 || x >= W - 2 || y < 1 || y >= H - 1) return;
    if (!advect_mask(flag, P, W, x, y, true)) return;
    float posx = (float)x + 0.5f, posy = (float)y;
    float vx1 = ld(vx, P, x, y);
    float vy1 = ((ld(vy, P, x, y) + ld(vy, P, x, y - 1)) + (ld(vy, P, x + 1, y) + ld(vy, P, x + 1, y - 1))) *
                0.25f;
    float midx = posx - vx1 * chalf;
    float midy = posy - vy1 * chalf;
    float vx2 = bicubic(vx, P, W - 1, H, midx - 0.5f, midy);
    float vy2 = bicubic(vy, P, W, H - 1, midx, midy - 0.5f);
    float endx = posx - vx2 * cfull;
    float endy = posy - vy2 * cfull;
    float r = bicubic(vx, P, W - 1, H, endx - 0.5f, endy);
    v.vx[1 - srcx][(size_t)y * P + x] = r * fl(flag, P, x, y) * fl(flag, P, x + 1, y);
  } else {
    // vy faces, simulation.cpp:300-347 (rows 1..H-2 of the vx loop)
    if (x < 1 || x >= W - 1 || y < 1 || y >= H - 1) return;
    if (!advect_mask(flag, P, W, x, y, false)) return;
    float posx = (float)x, posy = (float)y + 0.5f;
    float vy1 = ld(vy, P, x, y);
    // The reference reads vx at flat index x+1+y*(W-1): for x = W-2 that is
    // element 0 of the next row.
    float a0 = ld(vx, P, x, y), a1 = ld(vx, P, x, y - 1);
    float a2 = (x + 1 < W - 1) ? ld(vx, P, x + 1, y) : ld(vx, P, 0, y + 1);
    float a3 = (x + 1 < W - 1) ? ld(vx, P, x + 1, y - 1) : ld(vx, P, 0, y);
    float vx1 = ((a0 + a1) + (a2 + a3)) * 0.25f;
    float midx = posx - vx1 * chalf;
    float midy = posy - vy1 * chalf;
    float vx2 = bicubic(vx, P, W - 1, H, midx - 0.5f, midy);
    float vy2 = bicubic(vy, P, W, H - 1, midx, midy - 0.5f);
    float endx = posx - vx2 * cfull;
    float endy = posy - vy2 * cfull;
    float r = bicubic(vy, P, W, H - 1, endx, endy - 0.5f);
    v.vy[1 - srcy][(size_t)y * P + x] = r * fl(flag, P, x, y) * fl(flag, P, x, y + 1);
  }
}

// ------------------------------------------------------------- divergence
__global__ void k_divergence(const float *__restrict__ vx, const float *__restrict__ vy,
                             float *__restrict__ f, int P, int W, int H,
                             const StepScalars *__restrict__ sc) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x < 1 || x >= W - 1 || y < 1 || y >= H - 1) return;
  float ih = sc->ih;
  f[(size_t)y * P + x] =
      -ih * (ld(vx, P, x, y) - ld(vx, P, x - 1, y) + ld(vy, P, x, y) - ld(vy, P, x, y - 1));
}

__global__ void k_sinks(float *f, int P, const SinkCell *cells, int n) {
  // The reference writes the cells in list order; later sinks win.
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int i = 0; i < n; i++) f[(size_t)cells[i].y * P + cells[i].x] = cells[i].v;
}

// ------------------------------------------------------------------ setPBC
__global__ void k_pbc(float *p, int P, int W, int H, Bcs bc) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  auto at = [&](int x, int y) -> float & { return p[(size_t)y * P + x]; };
  if (t < H - 2) {
    int y = t + 1;
    at(0, y) = single_pbc(bc.w, at(1, y));
    at(W - 1, y) = single_pbc(bc.e, at(W - 2, y));
    return;
  }
  t -= H - 2;
  if (t >= W) return;
  int x = t;
  // value of column x in rows 1 and H-2 after the x-edge loop
  float a1, a2;
  if (x == 0) {
    a1 = single_pbc(bc.w, at(1, 1));
    a2 = single_pbc(bc.w, at(1, H - 2));
  } else if (x == W - 1) {
    a1 = single_pbc(bc.e, at(W - 2, 1));
    a2 = single_pbc(bc.e, at(W - 2, H - 2));
  } else {
    a1 = at(x, 1);
    a2 = at(x, H - 2);
  }
  at(x, 0) = single_pbc(bc.s, a1);
  at(x, H - 1) = single_pbc(bc.n, a2);
}

// ---------------------------------------------------------------- gradient
__global__ void k_gradient(float *vx, float *vy, const float *__restrict__ p,
                           const uint8_t *__restrict__ flag, int P, int W, int H,
                           const StepScalars *__restrict__ sc) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  float ih = sc->ih;
  size_t i = (size_t)y * P + x;
  if (x >= 1 && x < W - 2 && y >= 1 && y < H - 1)
    vx[i] = vx[i] - fl(flag, P, x, y) * fl(flag, P, x + 1, y) * ih * (ld(p, P, x + 1, y) - ld(p, P, x, y));
  if (x >= 1 && x < W - 1 && y >= 1 && y < H - 2)
    vy[i] = vy[i] - fl(flag, P, x, y) * fl(flag, P, x, y + 1) * ih * (ld(p, P, x, y + 1) - ld(p, P, x, y));
}

// --------------------------------------------------------------------- CFL
__global__ void k_umax(const float *__restrict__ vx, const float *__restrict__ vy, int P, int W,
                       int H, unsigned int *umax_bits) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  float m = 0.0f;
  if (x < W - 1 && y < H) m = fabsf(ld(vx, P, x, y));
  if (x < W && y < H - 1) m = fmaxf(m, fabsf(ld(vy, P, x, y)));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(umax_bits, __float_as_uint(m));
}

__global__ void k_cfl_scalars(const unsigned int *umax_bits, float cfl, float h, float mu,
                              float pwidth, int W, StepScalars *sc) {
  float umax = __uint_as_float(*umax_bits);
  umax = umax > 1e-7f ? umax : 1e-7f;
  float dt = cfl * h / umax;
  StepScalars s;
  s.dt = dt;
  s.a = dt * mu * ((float)W - 1.0f) / pwidth;
  s.den = 1.0f + 4.0f * s.a;
  s.ih = 1.0f / h;
  s.chalf = 0.5f * dt * s.ih;
  s.cfull = dt * s.ih;
  *sc = s;
}

inline dim3 grid2(int w, int h, int z = 1) { return dim3((w + BX - 1) / BX, (h + BY - 1) / BY, z); }

}  // namespace

void launch_vbc(const VelBufs &v, int fx, int fy, Bcs bc, bool do_vx, bool do_vy, cudaStream_t st) {
  ProfScope ps_(KC_VBC, st);
  int n = (v.H - 2) + (v.W - 1) + (v.H - 3) + v.W;
  k_vbc<<<(n + 255) / 256, 256, 0, st>>>(v, fx, fy, bc, do_vx, do_vy);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_accum(const VelBufs &v, int fx, int fy, float *ax, float *ay, cudaStream_t st) {
  ProfScope ps_(KC_ACCUM, st);
  k_accum<<<grid2(v.W, v.H), dim3(BX, BY), 0, st>>>(v.vx[fx], v.vy[fy], ax, ay, v.pitch, v.W, v.H);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_diffuse_sweep(const VelBufs &v, int srcx, int srcy, const uint8_t *flag,
                          const StepScalars *sc, int comps, cudaStream_t st) {
  ProfScope ps_(KC_DIFFUSE, st);
  k_diffuse<<<grid2(v.W, v.H, 2), dim3(BX, BY), 0, st>>>(v, srcx, srcy, flag, sc, comps);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_advect(const VelBufs &v, int srcx, int srcy, const uint8_t *flag,
                   const StepScalars *sc, cudaStream_t st) {
  ProfScope ps_(KC_ADVECT, st);
  k_advect<<<grid2(v.W, v.H, 2), dim3(BX, BY), 0, st>>>(v, srcx, srcy, flag, sc);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_divergence(const VelBufs &v, int fx, int fy, float *f, const StepScalars *sc,
                       cudaStream_t st) {
  ProfScope ps_(KC_DIVERGENCE, st);
  k_divergence<<<grid2(v.W, v.H), dim3(BX, BY), 0, st>>>(v.vx[fx], v.vy[fy], f, v.pitch, v.W, v.H, sc);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_sinks(float *f, int pitch, const SinkCell *cells, int n, cudaStream_t st) {
  if (n <= 0) return;
  ProfScope ps_(KC_SINKS, st);
  k_sinks<<<1, 32, 0, st>>>(f, pitch, cells, n);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_pbc(float *p, int pitch, int W, int H, Bcs bc, cudaStream_t st) {
  ProfScope ps_(KC_PBC, st);
  int n = (H - 2) + W;
  k_pbc<<<(n + 255) / 256, 256, 0, st>>>(p, pitch, W, H, bc);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_gradient(const VelBufs &v, int fx, int fy, const float *p, const uint8_t *flag,
                     const StepScalars *sc, cudaStream_t st) {
  ProfScope ps_(KC_GRADIENT, st);
  k_gradient<<<grid2(v.W, v.H), dim3(BX, BY), 0, st>>>(v.vx[fx], v.vy[fy], p, flag, v.pitch, v.W,
                                                        v.H, sc);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_cfl(const VelBufs &v, int fx, int fy, float cfl, float h, float mu, float pwidth,
                unsigned int *umax_bits, StepScalars *sc, cudaStream_t st) {
  ProfScope ps_(KC_CFL, st);
  UBG_CUDA(cudaMemsetAsync(umax_bits, 0, sizeof(unsigned int), st));
  k_umax<<<grid2(v.W, v.H), dim3(BX, BY), 0, st>>>(v.vx[fx], v.vy[fy], v.pitch, v.W, v.H, umax_bits);
  UBG_LAUNCH_CHECK();
  k_cfl_scalars<<<1, 1, 0, st>>>(umax_bits, cfl, h, mu, pwidth, v.W, sc);
  UBG_LAUNCH_CHECK();
  g_stats.launches += 2;
}

}  // namespace ubg
