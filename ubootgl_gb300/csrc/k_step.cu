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
                                    "residual", "tracers", "other", "smooth_l1", "tail", "krylov"};
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
                              Bcs bc, int t, float &m) {
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
    m = fmaxf(m, fabsf(v));
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

__device__ __forceinline__ void k_vbc_body(VelBufs v, int fx, int fy, Bcs bc, int do_vx, int do_vy,
                      unsigned int *umax_bits, const int bx, const int by, const int bz) {
  int t = bx * blockDim.x + threadIdx.x;
  int W = v.W, H = v.H;
  int nx = (H - 2) + (W - 1);
  float m = 0.0f;
  if (t < nx) {
    if (do_vx) vbc_component<true>(pick(v.vx, fx), v.vx[0], v.vx[1], v.pitch, W - 1, H, bc, t, m);
  } else if (do_vy) {
    vbc_component<false>(pick(v.vy, fy), v.vy[0], v.vy[1], v.pitch, W, H - 1, bc, t - nx, m);
  }
  // max |boundary value| for the next step's CFL dt (interior faces come
  // from the gradient kernel)
  if (umax_bits) {
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(umax_bits, __float_as_uint(m));
  }
}
__global__ void k_vbc(VelBufs v, int fx, int fy, Bcs bc, int do_vx, int do_vy,
                      unsigned int *umax_bits) {
  griddep_wait();
  k_vbc_body(v, fx, fy, bc, do_vx, do_vy, umax_bits, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---------------------------------------------- applyAccumulatedVelocity
__global__ void k_accum(float *vx, float *vy, float *ax, float *ay, int pitch, int W, int H) {
  griddep_wait();
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

// ------------------------------------------------------------- face codes
// vx face (x, y) sits between cells x and x+1; vy face (x, y) between cells
// y and y+1.  Diffusion terms (simulation.cpp:118-126 and 144-152):
//   vx: T1 = vx(x+1,y)*f(x+1,y)*f(x+2,y), T2 = vx(x-1,y)*f(x,y)*f(x-1,y),
//       T3 uses fvn = f(x,y+1)*f(x-1,y+1), T4 uses fvs = f(x,y-1)*f(x-1,y-1)
//   vy: T1 = vy(x,y-1)*f(x,y)*f(x,y-1), T2 = vy(x,y+1)*f(x,y+1)*f(x,y+2),
//       T3 uses fve = f(x+1,y)*f(x+1,y+1), T4 uses fvw = f(x-1,y)*f(x-1,y+1)
// FC_A reproduces the chunked advection loop (simulation.cpp:248-256,
// 300-304): faces from x = 1 in chunks of 8 while the chunk start is below
// width-8, a chunk skipped when none of its lanes passes the fluid test.
__global__ void k_face_codes(const uint8_t *__restrict__ flag, uint8_t *cx, uint8_t *cy, int P,
                             int W, int H) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  auto F = [&](int xx, int yy) -> unsigned { return flag[(size_t)yy * P + xx]; };
  if (x < W - 1 && y < H) {
    unsigned c = 0;
    if (x >= 1 && x < W - 2 && y >= 1 && y < H - 1) {
      if (F(x, y) & F(x + 1, y)) c |= FC_M;
      if (F(x + 1, y) & F(x + 2, y)) c |= FC_T1;
      if (F(x, y) & F(x - 1, y)) c |= FC_T2;
      if (F(x, y + 1) & F(x - 1, y + 1)) c |= FC_T3;
      if (F(x, y - 1) & F(x - 1, y - 1)) c |= FC_T4;
      int xs = 1 + ((x - 1) >> 3) * 8;
      if (xs < (W - 1) - 8)
        for (int i = 0; i < 8; i++)
          if (F(xs - 1 + i, y) & F(xs + i, y)) {
            c |= FC_A;
            break;
          }
    }
    cx[(size_t)y * P + x] = (uint8_t)c;
  }
  if (x < W && y < H - 1) {
    unsigned c = 0;
    if (x >= 1 && x < W - 1 && y >= 1) {
      // rows 1..H-2: the advection loop also covers vy's last row H-2
      if (F(x, y) & F(x, y + 1)) c |= FC_M;
      if (y < H - 2) {
        if (F(x, y) & F(x, y - 1)) c |= FC_T1;
        if (F(x, y + 1) & F(x, y + 2)) c |= FC_T2;
        if (F(x + 1, y) & F(x + 1, y + 1)) c |= FC_T3;
        if (F(x - 1, y) & F(x - 1, y + 1)) c |= FC_T4;
      }
      int xs = 1 + ((x - 1) >> 3) * 8;
      if (xs < W - 8)
        for (int i = 0; i < 8; i++)
          if (F(xs + i, y) & F(xs + i, y - 1)) {
            c |= FC_A;
            break;
          }
    }
    cy[(size_t)y * P + x] = (uint8_t)c;
  }
}

// ---------------------------------------------------------------- diffuse
// One Jacobi sweep, simulation.cpp:114-128 (vx) and 140-154 (vy).  With
// flags in {0, 1}: v*f*f is f*f ? v : 0, v*fv + (1-fv)*(-c) is fv ? v : -c,
// and the running sum starts at +0, so the face codes give the reference's
// values (a zero's sign aside).
// Row-vector access: a thread handles 4 consecutive faces of one row with
// float4 loads (x is a multiple of 4 and rows are 128-byte aligned); a block
// of 64 x 4 threads covers 256 x 4 faces.
constexpr int VX = 64, VY = 4;
__device__ __forceinline__ float4 ld4(const float *p, int P, int x, int y) {
  return __ldg(reinterpret_cast<const float4 *>(p + (size_t)y * P + x));
}
__device__ __forceinline__ float comp(const float4 &v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}
__device__ __forceinline__ unsigned compu(const uchar4 &v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}
// Stores the faces of [x, x+4) that lie in [lo, hi] (a whole float4 when all do).
__device__ __forceinline__ void st4_masked(float *row, int x, int lo, int hi, const float o[4]) {
  if (x >= lo && x + 3 <= hi) {
    *reinterpret_cast<float4 *>(row + x) = make_float4(o[0], o[1], o[2], o[3]);
  } else {
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (x + j >= lo && x + j <= hi) row[x + j] = o[j];
  }
}

__device__ __forceinline__ void k_diffuse_body(VelBufs v, int srcx, int srcy,
                                                 const StepScalars *__restrict__ sc, int comps, const int bx, const int by, const int bz) {
  const int x = 4 * (bx * VX + threadIdx.x), y = by * VY + threadIdx.y;
  const int W = v.W, H = v.H, P = v.pitch;
  const float a = sc->a, den = sc->den, rden = sc->rden;
  // both components per thread (independent arrays; twice the loads in
  // flight per thread)
  (void)bz;
  if ((comps & 1) && y >= 1 && y < H - 1 && x <= W - 3 && x + 3 >= 1) {
    // vx: interior faces x in [1, W-3], y in [1, H-2]
    const float *s = pick(v.vx, srcx);
    float4 C = ld4(s, P, x, y), N = ld4(s, P, x, y + 1), S = ld4(s, P, x, y - 1);
    uchar4 K = __ldg(reinterpret_cast<const uchar4 *>(v.cx + (size_t)y * P + x));
    float L = x >= 1 ? ld(s, P, x - 1, y) : 0.0f;
    float R = x + 4 < W - 1 ? ld(s, P, x + 4, y) : 0.0f;
    float o[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      unsigned k = compu(K, j);
      float c = comp(C, j);
      float t1 = j < 3 ? comp(C, j + 1) : R, t2 = j > 0 ? comp(C, j - 1) : L;
      float val = 0.0f;
      val = val + ((k & FC_T1) ? t1 : 0.0f);
      val = val + ((k & FC_T2) ? t2 : 0.0f);
      val = val + ((k & FC_T3) ? comp(N, j) : -c);
      val = val + ((k & FC_T4) ? comp(S, j) : -c);
      o[j] = (k & FC_M) ? div_rn(c + a * val, den, rden) : 0.0f;
    }
    st4_masked(pick(v.vx, 1 - srcx) + (size_t)y * P, x, 1, W - 3, o);
  }
  if ((comps & 2) && y >= 1 && y < H - 2 && x <= W - 2 && x + 3 >= 1) {
    // vy: interior faces x in [1, W-2], y in [1, H-3]
    const float *s = pick(v.vy, srcy);
    float4 C = ld4(s, P, x, y), N = ld4(s, P, x, y + 1), S = ld4(s, P, x, y - 1);
    uchar4 K = __ldg(reinterpret_cast<const uchar4 *>(v.cy + (size_t)y * P + x));
    float L = x >= 1 ? ld(s, P, x - 1, y) : 0.0f;
    float R = x + 4 < W ? ld(s, P, x + 4, y) : 0.0f;
    float o[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      unsigned k = compu(K, j);
      float c = comp(C, j);
      float t3 = j < 3 ? comp(C, j + 1) : R, t4 = j > 0 ? comp(C, j - 1) : L;
      float val = 0.0f;
      val = val + ((k & FC_T1) ? comp(S, j) : 0.0f);
      val = val + ((k & FC_T2) ? comp(N, j) : 0.0f);
      val = val + ((k & FC_T3) ? t3 : -c);
      val = val + ((k & FC_T4) ? t4 : -c);
      o[j] = (k & FC_M) ? div_rn(c + a * val, den, rden) : 0.0f;
    }
    st4_masked(pick(v.vy, 1 - srcy) + (size_t)y * P, x, 1, W - 2, o);
  }
}
__global__ void __launch_bounds__(256) k_diffuse(VelBufs v, int srcx, int srcy,
                                                 const StepScalars *__restrict__ sc, int comps) {
  griddep_wait();
  k_diffuse_body(v, srcx, srcy, sc, comps, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ----------------------------------------------------------------- advect
// CubicHermite (interpolators.hpp:78-85) is the Catmull-Rom cubic; it is
// evaluated through its four weights of t (the same polynomial, regrouped),
// wA = t(-1/2 + t(1 - t/2)), wB = 1 + t^2(-5/2 + 3t/2),
// wC = t(1/2 + t(2 - 3t/2)), wD = t^2(-1/2 + t/2), with explicit fused
// multiply-adds, exactly as the CPU restatement does.
struct CrW {
  float a, b, c, d;
};
__device__ __forceinline__ CrW cr_weights(float t) {
  float t2 = t * t;
  CrW w;
  w.a = t * __fmaf_rn(t, __fmaf_rn(-0.5f, t, 1.0f), -0.5f);
  w.b = __fmaf_rn(t2, __fmaf_rn(1.5f, t, -2.5f), 1.0f);
  w.c = t * __fmaf_rn(t, __fmaf_rn(-1.5f, t, 2.0f), 0.5f);
  w.d = t2 * __fmaf_rn(0.5f, t, -0.5f);
  return w;
}
__device__ __forceinline__ float cr_dot(const CrW &w, float A, float B, float C, float D) {
  return __fmaf_rn(w.d, D, __fmaf_rn(w.c, C, __fmaf_rn(w.b, B, w.a * A)));
}



// The two weight sets of one sample at once: lane x for t.x, lane y for t.y
// (the operations of cr_weights, lane by lane).
struct CrW2 {
  float2 a, b, c, d;
};
__device__ __forceinline__ CrW2 cr_weights2(float2 t) {
  const float2 t2 = f2_mul(t, t);
  CrW2 w;
  w.a = f2_mul(t, f2_fma(t, f2_fma(f2(-0.5f), t, f2(1.0f)), f2(-0.5f)));
  w.b = f2_fma(t2, f2_fma(f2(1.5f), t, f2(-2.5f)), f2(1.0f));
  w.c = f2_mul(t, f2_fma(t, f2_fma(f2(-1.5f), t, f2(2.0f)), f2(0.5f)));
  w.d = f2_mul(t2, f2_fma(f2(0.5f), t, f2(-0.5f)));
  return w;
}

// Catmull-Rom sample from 16 values (rows r0..r3 of a 4x4 stencil): the
// four vertical dots cr_dot(wy, column j) two columns per instruction, then
// the horizontal dot.
__device__ __forceinline__ float bicubic16(const float *b, int stride, float sx, float sy) {
  const CrW2 w = cr_weights2(make_float2(sy, sx));
  const float2 wa = f2(w.a.x), wb = f2(w.b.x), wc = f2(w.c.x), wd = f2(w.d.x);
  float2 col[2];
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const float2 A = make_float2(b[2 * j], b[2 * j + 1]);
    const float2 B = make_float2(b[stride + 2 * j], b[stride + 2 * j + 1]);
    const float2 C = make_float2(b[2 * stride + 2 * j], b[2 * stride + 2 * j + 1]);
    const float2 D = make_float2(b[3 * stride + 2 * j], b[3 * stride + 2 * j + 1]);
    col[j] = f2_fma(wd, D, f2_fma(wc, C, f2_fma(wb, B, f2_mul(wa, A))));
  }
  const CrW wx{w.a.y, w.b.y, w.c.y, w.d.y};
  return cr_dot(wx, col[0].x, col[0].y, col[1].x, col[1].y);
}

// A staged window of one staggered component: region [sx0, sx0+SW) x
// [sy0, sy0+SH) of the grid in shared memory.
struct Win {
  const float *s;
  int sx0, sy0;
};

// bicubicSample (interpolators.hpp:92-206) reading the 4x4 stencil from the
// shared-memory window when it lies inside, else from global memory.
template <int SW, int SH>
__device__ __forceinline__ float bicubic_win(const Win &wn, const float *__restrict__ g, int P,
                                             int gw, int gh, float cx, float cy) {
  float hx = (float)gw - 3.0f, hy = (float)gh - 3.0f;
  cx = cx < hx ? cx : hx;
  cx = cx > 3.0f ? cx : 3.0f;
  cy = cy < hy ? cy : hy;
  cy = cy > 3.0f ? cy : 3.0f;
  int ix = (int)cx, iy = (int)cy;
  float sx = cx - (float)ix, sy = cy - (float)iy;
  int lx = ix - 1 - wn.sx0, ly = iy - 1 - wn.sy0;
  if (lx >= 0 && lx + 3 < SW && ly >= 0 && ly + 3 < SH)
    return bicubic16(wn.s + ly * SW + lx, SW, sx, sy);
  return bicubic16(g + (size_t)(iy - 1) * P + (ix - 1), P, sx, sy);
}

// bilinearSample (interpolators.hpp:11-27) for the advection option: clamp
// to [0, size - 1.1] (glm::clamp = min(max(c, lo), hi)), truncate,
// interpolate along x, then along y; the four values from the shared-memory
// window when they lie inside, else from global memory.
template <int SW, int SH>
__device__ __forceinline__ float bilinear_win(const Win &wn, const float *__restrict__ g, int P,
                                              int gw, int gh, float cx, float cy) {
  const float hx = (float)gw - 1.1f, hy = (float)gh - 1.1f;
  cx = cx < 0.0f ? 0.0f : cx;
  cx = hx < cx ? hx : cx;
  cy = cy < 0.0f ? 0.0f : cy;
  cy = hy < cy ? hy : cy;
  const int ix = (int)cx, iy = (int)cy;
  const float sx = cx - (float)ix, sy = cy - (float)iy;
  const int lx = ix - wn.sx0, ly = iy - wn.sy0;
  float v1, v2, v3, v4;
  if (lx >= 0 && lx + 1 < SW && ly >= 0 && ly + 1 < SH) {
    const float *b = wn.s + ly * SW + lx;
    v1 = b[0];
    v2 = b[1];
    v3 = b[SW];
    v4 = b[SW + 1];
  } else {
    const float *b = g + (size_t)iy * P + ix;
    v1 = b[0];
    v2 = b[1];
    v3 = b[P];
    v4 = b[P + 1];
  }
  const float vm1 = v1 + (v2 - v1) * sx;
  const float vm2 = v3 + (v4 - v3) * sx;
  return vm1 + (vm2 - vm1) * sy;
}

// advect, simulation.cpp:241-354.  A block handles the vx and vy faces of a
// 64 x 16 tile of cells; both velocity components are staged in shared
// memory with a 4-cell halo, which holds every stencil of a back-trace that
// moves up to about one cell (the CFL-0.5 step moves at most half a cell);
// longer traces read from global memory.
constexpr int AD_TX = 64, AD_TY = 16, AD_H = 4;
constexpr int AD_SW = AD_TX + 2 * AD_H, AD_SH = AD_TY + 2 * AD_H;

// BIL: the advection option's bilinearSample instead of bicubicSample.
template <bool BIL>
__device__ __forceinline__ void k_advect_body(VelBufs v, int srcx, int srcy,
                                                const StepScalars *__restrict__ sc, const int bx, const int by, const int bz) {
  __shared__ __align__(16) float sxv[AD_SH * AD_SW];
  __shared__ __align__(16) float syv[AD_SH * AD_SW];
  __shared__ __align__(16) uint8_t scx[AD_TY * AD_TX], scy[AD_TY * AD_TX];
  const int W = v.W, H = v.H, P = v.pitch;
  const float *vx = pick(v.vx, srcx);
  const float *vy = pick(v.vy, srcy);
  const int X0 = bx * AD_TX, Y0 = by * AD_TY;
  const int sx0 = X0 - AD_H, sy0 = Y0 - AD_H;
  const int tid = threadIdx.y * BX + threadIdx.x;
  // staging: 4 entries per load (sx0 and X0 are multiples of 4, so every
  // float4 / uchar4 lies inside its row's pitch); entries outside a
  // component's extent are 0
  static_assert(AD_SW % 4 == 0 && AD_H % 4 == 0 && AD_TX % 4 == 0, "vector staging");
  for (int i = tid; i < AD_SH * (AD_SW / 4); i += 256) {
    const int ry = i / (AD_SW / 4), rx = 4 * (i - ry * (AD_SW / 4));
    const int gx = sx0 + rx, gy = sy0 + ry;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (gx >= 0 && gy >= 0) {
      if (gx < W - 1 && gy < H) a = *reinterpret_cast<const float4 *>(vx + (size_t)gy * P + gx);
      if (gx < W && gy < H - 1) b = *reinterpret_cast<const float4 *>(vy + (size_t)gy * P + gx);
      if (gx + 3 >= W - 1) {
        if (gx + 1 >= W - 1) a.y = 0.f;
        if (gx + 2 >= W - 1) a.z = 0.f;
        a.w = 0.f;
      }
      if (gx + 3 >= W) {
        if (gx + 1 >= W) b.y = 0.f;
        if (gx + 2 >= W) b.z = 0.f;
        b.w = 0.f;
      }
    }
    *reinterpret_cast<float4 *>(sxv + ry * AD_SW + rx) = a;
    *reinterpret_cast<float4 *>(syv + ry * AD_SW + rx) = b;
  }
  for (int i = tid; i < AD_TY * (AD_TX / 4); i += 256) {
    const int ty = i / (AD_TX / 4), tx = 4 * (i - ty * (AD_TX / 4));
    const int x = X0 + tx, y = Y0 + ty;
    unsigned a = 0u, b = 0u;
    if (x < W && y < H) {
      a = __ldg(reinterpret_cast<const unsigned *>(v.cx + (size_t)y * P + x));
      b = __ldg(reinterpret_cast<const unsigned *>(v.cy + (size_t)y * P + x));
    }
    *reinterpret_cast<unsigned *>(scx + ty * AD_TX + tx) = a;
    *reinterpret_cast<unsigned *>(scy + ty * AD_TX + tx) = b;
  }
  __syncthreads();
  const Win wx{sxv, sx0, sy0}, wy{syv, sx0, sy0};
  const float chalf = sc->chalf, cfull = sc->cfull;
  auto SX = [&](int x, int y) { return sxv[(y - sy0) * AD_SW + (x - sx0)]; };
  auto SY = [&](int x, int y) { return syv[(y - sy0) * AD_SW + (x - sx0)]; };
  float *outx = pick(v.vx, 1 - srcx), *outy = pick(v.vy, 1 - srcy);
  auto SAMPLE = [&](const Win &wn, const float *__restrict__ g, int P_, int gw, int gh, float cx,
                    float cy) {
    if constexpr (BIL)
      return bilinear_win<AD_SW, AD_SH>(wn, g, P_, gw, gh, cx, cy);
    else
      return bicubic_win<AD_SW, AD_SH>(wn, g, P_, gw, gh, cx, cy);
  };
  for (int i = tid; i < AD_TX * AD_TY; i += 256) {
    int ty = i / AD_TX, tx = i - ty * AD_TX;
    int x = X0 + tx, y = Y0 + ty;
    if (y < 1 || y >= H - 1 || x < 1) continue;
    // vx face (x, y), simulation.cpp:247-298
    if (x < W - 2) {
      unsigned k = scx[i];
      if (k & FC_A) {
        float posx = (float)x + 0.5f, posy = (float)y;
        float vx1 = SX(x, y);
        float vy1 = ((SY(x, y) + SY(x, y - 1)) + (SY(x + 1, y) + SY(x + 1, y - 1))) * 0.25f;
        float midx = posx - vx1 * chalf;
        float midy = posy - vy1 * chalf;
        float vx2 = SAMPLE(wx, vx, P, W - 1, H, midx - 0.5f, midy);
        float vy2 = SAMPLE(wy, vy, P, W, H - 1, midx, midy - 0.5f);
        float endx = posx - vx2 * cfull;
        float endy = posy - vy2 * cfull;
        float r = SAMPLE(wx, vx, P, W - 1, H, endx - 0.5f, endy);
        outx[(size_t)y * P + x] = (k & FC_M) ? r : 0.0f;
      }
    }
    // vy face (x, y), simulation.cpp:300-347 (rows 1..H-2 of the vx loop)
    if (x < W - 1) {
      unsigned k = scy[i];
      if (k & FC_A) {
        float posx = (float)x, posy = (float)y + 0.5f;
        float vy1 = SY(x, y);
        // The reference reads vx at flat index x+1+y*(W-1): for x = W-2 that
        // is element 0 of the next row.
        float a2 = (x + 1 < W - 1) ? SX(x + 1, y) : ld(vx, P, 0, y + 1);
        float a3 = (x + 1 < W - 1) ? SX(x + 1, y - 1) : ld(vx, P, 0, y);
        float vx1 = ((SX(x, y) + SX(x, y - 1)) + (a2 + a3)) * 0.25f;
        float midx = posx - vx1 * chalf;
        float midy = posy - vy1 * chalf;
        float vx2 = SAMPLE(wx, vx, P, W - 1, H, midx - 0.5f, midy);
        float vy2 = SAMPLE(wy, vy, P, W, H - 1, midx, midy - 0.5f);
        float endx = posx - vx2 * cfull;
        float endy = posy - vy2 * cfull;
        float r = SAMPLE(wy, vy, P, W, H - 1, endx, endy - 0.5f);
        outy[(size_t)y * P + x] = (k & FC_M) ? r : 0.0f;
      }
    }
  }
}
template <bool BIL>
__global__ void __launch_bounds__(256) k_advect(VelBufs v, int srcx, int srcy,
                                                const StepScalars *__restrict__ sc) {
  griddep_wait();
  k_advect_body<BIL>(v, srcx, srcy, sc, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ------------------------------------------------------------- divergence
__device__ __forceinline__ void k_divergence_body(const float *__restrict__ vx,
                                                    const float *__restrict__ vy,
                                                    float *__restrict__ f, int P, int W, int H,
                                                    const StepScalars *__restrict__ sc, const int bx, const int by, const int bz) {
  const int x = 4 * (bx * VX + threadIdx.x), y = by * VY + threadIdx.y;
  if (y < 1 || y >= H - 1 || x > W - 2 || x + 3 < 1) return;
  const float ih = sc->ih;
  float4 U = ld4(vx, P, x, y), V = ld4(vy, P, x, y), Vs = ld4(vy, P, x, y - 1);
  float L = x >= 1 ? ld(vx, P, x - 1, y) : 0.0f;
  float o[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    float um = j > 0 ? comp(U, j - 1) : L;
    o[j] = -ih * (comp(U, j) - um + comp(V, j) - comp(Vs, j));
  }
  st4_masked(f + (size_t)y * P, x, 1, W - 2, o);
}
__global__ void __launch_bounds__(256) k_divergence(const float *__restrict__ vx,
                                                    const float *__restrict__ vy,
                                                    float *__restrict__ f, int P, int W, int H,
                                                    const StepScalars *__restrict__ sc) {
  griddep_wait();
  k_divergence_body(vx, vy, f, P, W, H, sc, blockIdx.x, blockIdx.y, blockIdx.z);
}

__global__ void k_sinks(float *f, int P, const SinkCell *cells, int n) {
  griddep_wait();
  // The reference writes the cells in list order; later sinks win.
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int i = 0; i < n; i++) f[(size_t)cells[i].y * P + cells[i].x] = cells[i].v;
}

// ------------------------------------------------------------------ setPBC
__device__ __forceinline__ void k_pbc_body(float *p, int P, int W, int H, Bcs bc, const int bx, const int by, const int bz) {
  int t = bx * blockDim.x + threadIdx.x;
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
__global__ void k_pbc(float *p, int P, int W, int H, Bcs bc) {
  griddep_wait();
  k_pbc_body(p, P, W, H, bc, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---------------------------------------------------------------- gradient
// Pressure-gradient update; also folds max(|vx|, |vy|) of every interior
// face (after the update) into *umax_bits for the next step's CFL dt.
__device__ __forceinline__ void k_gradient_body(VelBufs v, int fx, int fy,
                                                  const float *__restrict__ p,
                                                  const StepScalars *__restrict__ sc,
                                                  unsigned int *umax_bits, const int bx, const int by, const int bz) {
  const int x = 4 * (bx * VX + threadIdx.x), y = by * VY + threadIdx.y;
  const int W = v.W, H = v.H, P = v.pitch;
  float m = 0.0f;
  if (y >= 1 && y < H - 1 && x <= W - 2 && x + 3 >= 1) {
    const float ih = sc->ih;
    float *vx = pick(v.vx, fx), *vy = pick(v.vy, fy);
    float4 P0 = ld4(p, P, x, y), PN = ld4(p, P, x, y + 1);
    float PR = x + 4 < W ? ld(p, P, x + 4, y) : 0.0f;
    float4 U = *reinterpret_cast<const float4 *>(vx + (size_t)y * P + x);
    float4 V = *reinterpret_cast<const float4 *>(vy + (size_t)y * P + x);
    uchar4 KX = __ldg(reinterpret_cast<const uchar4 *>(v.cx + (size_t)y * P + x));
    uchar4 KY = __ldg(reinterpret_cast<const uchar4 *>(v.cy + (size_t)y * P + x));
    float ox[4], oy[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      float p0 = comp(P0, j), pe = j < 3 ? comp(P0, j + 1) : PR;
      float u = comp(U, j), w = comp(V, j);
      bool inx = x + j >= 1 && x + j <= W - 3;
      bool iny = x + j >= 1 && x + j <= W - 2 && y <= H - 3;
      ox[j] = (inx && (compu(KX, j) & FC_M)) ? u - ih * (pe - p0) : u;
      oy[j] = (iny && (compu(KY, j) & FC_M)) ? w - ih * (comp(PN, j) - p0) : w;
      if (inx) m = fmaxf(m, fabsf(ox[j]));
      if (iny) m = fmaxf(m, fabsf(oy[j]));
    }
    st4_masked(vx + (size_t)y * P, x, 1, W - 3, ox);
    if (y <= H - 3) st4_masked(vy + (size_t)y * P, x, 1, W - 2, oy);
  }
  if (umax_bits) {
    // one atomic per block: per-warp atomics on one address serialise
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float red[VX * VY / 32];
    const int tid = threadIdx.y * VX + threadIdx.x;
    if ((tid & 31) == 0) red[tid >> 5] = m;
    __syncthreads();
    if (tid == 0) {
      for (int i = 1; i < VX * VY / 32; i++) m = fmaxf(m, red[i]);
      atomicMax(umax_bits, __float_as_uint(m));
    }
  }
}
__global__ void __launch_bounds__(256) k_gradient(VelBufs v, int fx, int fy,
                                                  const float *__restrict__ p,
                                                  const StepScalars *__restrict__ sc,
                                                  unsigned int *umax_bits) {
  griddep_wait();
  k_gradient_body(v, fx, fy, p, sc, umax_bits, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ------------------------------------------------------ staged host I/O
// Staged inputs become the front velocity (whole arrays, ghosts included),
// with max|u| over every element folded in as k_umax computes it; and the
// current velocity is snapshotted for an asynchronous download.  Kernels
// rather than 2-D device copies: a pitched cudaMemcpy2D between device
// buffers measured ~0.9 TB/s on GB300.
__global__ void __launch_bounds__(256) k_stage_in(const float *__restrict__ inx,
                                                  const float *__restrict__ iny, float *vx,
                                                  float *vy, int P, int W, int H,
                                                  unsigned int *umax_bits) {
  griddep_wait();
  const int x = 4 * (blockIdx.x * VX + threadIdx.x), y = blockIdx.y * VY + threadIdx.y;
  float m = 0.0f;
  if (x < W && y < H) {
    const size_t i = (size_t)y * P + x;
    const float4 a = *reinterpret_cast<const float4 *>(inx + i);
    const float ax[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (x + j < W - 1) m = fmaxf(m, fabsf(ax[j]));
    st4_masked(vx + (size_t)y * P, x, 0, W - 2, ax);
    if (y < H - 1) {
      const float4 b = *reinterpret_cast<const float4 *>(iny + i);
      const float bx[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (x + j < W) m = fmaxf(m, fabsf(bx[j]));
      st4_masked(vy + (size_t)y * P, x, 0, W - 1, bx);
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float red[VX * VY / 32];
  const int tid = threadIdx.y * VX + threadIdx.x;
  if ((tid & 31) == 0) red[tid >> 5] = m;
  __syncthreads();
  if (tid == 0) {
    for (int i = 1; i < VX * VY / 32; i++) m = fmaxf(m, red[i]);
    atomicMax(umax_bits, __float_as_uint(m));
  }
}

__global__ void __launch_bounds__(256) k_stage_out(const float *__restrict__ vx,
                                                   const float *__restrict__ vy, float *outx,
                                                   float *outy, int P, int W, int H) {
  griddep_wait();
  const int x = 4 * (blockIdx.x * VX + threadIdx.x), y = blockIdx.y * VY + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t i = (size_t)y * P + x;
  *reinterpret_cast<float4 *>(outx + i) = *reinterpret_cast<const float4 *>(vx + i);
  if (y < H - 1) *reinterpret_cast<float4 *>(outy + i) = *reinterpret_cast<const float4 *>(vy + i);
}

// --------------------------------------------------------------------- CFL
__global__ void __launch_bounds__(256) k_umax(const float *__restrict__ vx,
                                              const float *__restrict__ vy, int P, int W, int H,
                                              unsigned int *umax_bits) {
  griddep_wait();
  // grid-stride over rows; one atomic per block
  float m = 0.0f;
  for (int y = blockIdx.y * 8 + threadIdx.y; y < H; y += gridDim.y * 8)
    for (int x = blockIdx.x * 32 + threadIdx.x; x < W; x += gridDim.x * 32) {
      if (x < W - 1) m = fmaxf(m, fabsf(ld(vx, P, x, y)));
      if (y < H - 1) m = fmaxf(m, fabsf(ld(vy, P, x, y)));
    }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float red[8];
  if (threadIdx.x == 0) red[threadIdx.y] = m;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    for (int i = 1; i < 8; i++) m = fmaxf(m, red[i]);
    atomicMax(umax_bits, __float_as_uint(m));
  }
}

__device__ __forceinline__ void k_cfl_scalars_body(const unsigned int *umax_bits, float cfl, float h, float mu,
                              float pwidth, int W, StepScalars *sc, const int bx, const int by, const int bz) {
  float umax = __uint_as_float(*umax_bits);
  umax = umax > 1e-7f ? umax : 1e-7f;
  float dt = cfl * h / umax;
  StepScalars s;
  s.dt = dt;
  s.a = dt * mu * ((float)W - 1.0f) / pwidth;
  s.den = 1.0f + 4.0f * s.a;
  s.rden = __frcp_rn(s.den);
  s.ih = 1.0f / h;
  s.chalf = 0.5f * dt * s.ih;
  s.cfull = dt * s.ih;
  *sc = s;
}
__global__ void k_cfl_scalars(const unsigned int *umax_bits, float cfl, float h, float mu,
                              float pwidth, int W, StepScalars *sc) {
  griddep_wait();
  k_cfl_scalars_body(umax_bits, cfl, h, mu, pwidth, W, sc, blockIdx.x, blockIdx.y, blockIdx.z);
}

inline dim3 grid2(int w, int h, int z = 1) { return dim3((w + BX - 1) / BX, (h + BY - 1) / BY, z); }
inline dim3 grid_vec(int w, int h, int z = 1) {
  return dim3((w + 4 * VX - 1) / (4 * VX), (h + VY - 1) / VY, z);
}


// ---------------------------------------------------- multi-member kernels
__global__ void k_vbc_m(const VbcM *__restrict__ A, const int *__restrict__ bs, int n,
        unsigned tag, unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  const int m = member_of(bs, n);
  const VbcM a = A[m];
  k_vbc_body(a.v, a.fx, a.fy, a.bc, a.do_vx, a.do_vy, a.umax, (int)blockIdx.x - __ldg(bs + m), 0, 0);
}
__global__ void __launch_bounds__(256) k_diffuse_m(const DiffuseM *__restrict__ A, const int *__restrict__ bs, int n,
            unsigned tag, unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  const int m = member_of(bs, n);
  const DiffuseM a = A[m];
  const int l = (int)blockIdx.x - __ldg(bs + m);
  k_diffuse_body(a.v, a.srcx, a.srcy, a.sc, a.comps, l % a.gx, (l / a.gx) % a.gy, l / (a.gx * a.gy));
}
__global__ void __launch_bounds__(256) k_advect_m(const AdvectM *__restrict__ A, const int *__restrict__ bs, int n,
           unsigned tag, unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  const int m = member_of(bs, n);
  const AdvectM a = A[m];
  const int l = (int)blockIdx.x - __ldg(bs + m);
  // fused members advect bicubically (the bilinear option is not fused)
  k_advect_body<false>(a.v, a.srcx, a.srcy, a.sc, l % a.gx, l / a.gx, 0);
}
__global__ void __launch_bounds__(256) k_divergence_m(const DivergenceM *__restrict__ A, const int *__restrict__ bs, int n,
               unsigned tag, unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  const int m = member_of(bs, n);
  const DivergenceM a = A[m];
  const int l = (int)blockIdx.x - __ldg(bs + m);
  k_divergence_body(a.vx, a.vy, a.f, a.P, a.W, a.H, a.sc, l % a.gx, l / a.gx, 0);
}
__global__ void k_pbc_m(const PbcM *__restrict__ A, const int *__restrict__ bs, int n,
        unsigned tag, unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  const int m = member_of(bs, n);
  const PbcM a = A[m];
  const int l = (int)blockIdx.x - __ldg(bs + m);
  if (l == 0 && threadIdx.x == 0 && a.umax_zero) *a.umax_zero = 0u;
  k_pbc_body(a.p, a.P, a.W, a.H, a.bc, l, 0, 0);
}
__global__ void __launch_bounds__(256) k_gradient_m(const GradientM *__restrict__ A, const int *__restrict__ bs, int n,
             unsigned tag, unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  const int m = member_of(bs, n);
  const GradientM a = A[m];
  const int l = (int)blockIdx.x - __ldg(bs + m);
  k_gradient_body(a.v, a.fx, a.fy, a.p, a.sc, a.umax, l % a.gx, l / a.gx, 0);
}
__global__ void k_cfl_m(const CflM *__restrict__ A, const int *__restrict__ bs, int n, unsigned tag,
                        unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const CflM a = A[m];
  k_cfl_scalars_body(a.umax, a.cfl, a.h, a.mu, a.pwidth, a.W, a.sc, 0, 0, 0);
}
}  // namespace

void launch_face_codes(const VelBufs &v, const uint8_t *flag, uint8_t *cx, uint8_t *cy,
                       cudaStream_t st) {
  k_face_codes<<<grid2(v.W, v.H), dim3(BX, BY), 0, st>>>(flag, cx, cy, v.pitch, v.W, v.H);
  UBG_LAUNCH_CHECK();
}

void launch_vbc(const VelBufs &v, int fx, int fy, Bcs bc, bool do_vx, bool do_vy, cudaStream_t st,
                unsigned int *umax_bits) {
  ProfScope ps_(KC_VBC, st);
  int n = (v.H - 2) + (v.W - 1) + (v.H - 3) + v.W;
  launch_pdl(k_vbc, dim3((n + 255) / 256), dim3(256), 0, st, v, fx, fy, bc, do_vx, do_vy, umax_bits);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_accum(const VelBufs &v, int fx, int fy, float *ax, float *ay, cudaStream_t st) {
  ProfScope ps_(KC_ACCUM, st);
  launch_pdl(k_accum, grid2(v.W, v.H), dim3(BX, BY), 0, st, v.vx[fx], v.vy[fy], ax, ay, v.pitch, v.W, v.H);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_diffuse_sweep(const VelBufs &v, int srcx, int srcy, const StepScalars *sc, int comps,
                          cudaStream_t st) {
  ProfScope ps_(KC_DIFFUSE, st);
  launch_pdl(k_diffuse, grid_vec(v.W, v.H), dim3(VX, VY), 0, st, v, srcx, srcy, sc, comps);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_advect(const VelBufs &v, int srcx, int srcy, const StepScalars *sc, cudaStream_t st) {
  ProfScope ps_(KC_ADVECT, st);
  dim3 grid((v.W + AD_TX - 1) / AD_TX, (v.H + AD_TY - 1) / AD_TY);
  if (v.advect_bilinear)
    launch_pdl(k_advect<true>, grid, dim3(BX, BY), 0, st, v, srcx, srcy, sc);
  else
    launch_pdl(k_advect<false>, grid, dim3(BX, BY), 0, st, v, srcx, srcy, sc);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_divergence(const VelBufs &v, int fx, int fy, float *f, const StepScalars *sc,
                       cudaStream_t st) {
  ProfScope ps_(KC_DIVERGENCE, st);
  launch_pdl(k_divergence, grid_vec(v.W, v.H), dim3(VX, VY), 0, st, v.vx[fx], v.vy[fy], f,
             v.pitch, v.W, v.H, sc);
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
  launch_pdl(k_pbc, dim3((n + 255) / 256), dim3(256), 0, st, p, pitch, W, H, bc);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_gradient(const VelBufs &v, int fx, int fy, const float *p, const StepScalars *sc,
                     unsigned int *umax_bits, cudaStream_t st) {
  ProfScope ps_(KC_GRADIENT, st);
  launch_pdl(k_gradient, grid_vec(v.W, v.H), dim3(VX, VY), 0, st, v, fx, fy, p, sc, umax_bits);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_stage_in(VelBufs &v, int fx, int fy, const float *inx, const float *iny,
                     unsigned int *umax_bits, cudaStream_t st) {
  ProfScope ps_(KC_OTHER, st);
  UBG_CUDA(cudaMemsetAsync(umax_bits, 0, sizeof(unsigned int), st));
  launch_pdl(k_stage_in, grid_vec(v.W, v.H), dim3(VX, VY), 0, st, inx, iny, v.vx[fx], v.vy[fy],
             v.pitch, v.W, v.H, umax_bits);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_stage_out(const VelBufs &v, int fx, int fy, float *outx, float *outy, cudaStream_t st) {
  ProfScope ps_(KC_OTHER, st);
  launch_pdl(k_stage_out, grid_vec(v.W, v.H), dim3(VX, VY), 0, st, v.vx[fx], v.vy[fy], outx, outy,
             v.pitch, v.W, v.H);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_cfl(const VelBufs &v, int fx, int fy, float cfl, float h, float mu, float pwidth,
                unsigned int *umax_bits, StepScalars *sc, cudaStream_t st, bool umax_ready) {
  ProfScope ps_(KC_CFL, st);
  if (umax_ready) {
    launch_pdl(k_cfl_scalars, dim3(1), dim3(1), 0, st, umax_bits, cfl, h, mu, pwidth, v.W, sc);
    UBG_LAUNCH_CHECK();
    g_stats.launches++;
    return;
  }
  UBG_CUDA(cudaMemsetAsync(umax_bits, 0, sizeof(unsigned int), st));
  dim3 g((v.W + BX - 1) / BX, 64);
  if (g.x > 16) g.x = 16;
  launch_pdl(k_umax, g, dim3(BX, BY), 0, st, v.vx[fx], v.vy[fy], v.pitch, v.W, v.H, umax_bits);
  UBG_LAUNCH_CHECK();
  launch_pdl(k_cfl_scalars, dim3(1), dim3(1), 0, st, umax_bits, cfl, h, mu, pwidth, v.W, sc);
  UBG_LAUNCH_CHECK();
  g_stats.launches += 2;
}

}  // namespace ubg

namespace ubg {
int multi_blocks_vbc(const VbcM &a) {
  int n = (a.v.H - 2) + (a.v.W - 1) + (a.v.H - 3) + a.v.W;
  return (n + 255) / 256;
}
int multi_blocks_diffuse(DiffuseM &a) {
  dim3 g = grid_vec(a.v.W, a.v.H);
  a.gx = (int)g.x;
  a.gy = (int)g.y;
  return (int)(g.x * g.y * g.z);
}
int multi_blocks_advect(AdvectM &a) {
  a.gx = (a.v.W + AD_TX - 1) / AD_TX;
  return a.gx * ((a.v.H + AD_TY - 1) / AD_TY);
}
int multi_blocks_divergence(DivergenceM &a) {
  dim3 g = grid_vec(a.W, a.H);
  a.gx = (int)g.x;
  return (int)(g.x * g.y);
}
int multi_blocks_pbc(const PbcM &a) { return ((a.H - 2) + a.W + 255) / 256; }
int multi_blocks_gradient(GradientM &a) {
  dim3 g = grid_vec(a.v.W, a.v.H);
  a.gx = (int)g.x;
  return (int)(g.x * g.y);
}

void launch_multi_step(int kind, const void *args, const int *bs, int n, int blocks,
                       unsigned tag, unsigned *err, cudaStream_t st) {
  switch (kind) {
    case MK_VBC:
      launch_pdl(k_vbc_m, dim3(blocks), dim3(256), 0, st, (const VbcM *)args, bs, n, tag, err);
      break;
    case MK_DIFFUSE:
      launch_pdl(k_diffuse_m, dim3(blocks), dim3(VX, VY), 0, st, (const DiffuseM *)args, bs, n, tag, err);
      break;
    case MK_ADVECT:
      launch_pdl(k_advect_m, dim3(blocks), dim3(BX, BY), 0, st, (const AdvectM *)args, bs, n, tag, err);
      break;
    case MK_DIVERGENCE:
      launch_pdl(k_divergence_m, dim3(blocks), dim3(VX, VY), 0, st, (const DivergenceM *)args, bs,
                 n, tag, err);
      break;
    case MK_PBC:
      launch_pdl(k_pbc_m, dim3(blocks), dim3(256), 0, st, (const PbcM *)args, bs, n, tag, err);
      break;
    case MK_GRADIENT:
      launch_pdl(k_gradient_m, dim3(blocks), dim3(VX, VY), 0, st, (const GradientM *)args, bs, n, tag, err);
      break;
    case MK_CFL:
      launch_pdl(k_cfl_m, dim3((n + 127) / 128), dim3(128), 0, st, (const CflM *)args, bs, n, tag,
                 err);
      break;
    default:
      throw ArgError("multi-member launch kind");
  }
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}
}  // namespace ubg
