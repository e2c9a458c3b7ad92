// Device-side versions of what the reference's game code does to the
// simulation's fields from the host:
//
//  k_scatter_accum   bilinearScatter into vx_accum / vy_accum
//                    (interpolators.hpp:29-40) at pos/h - (0.5, 0) and
//                    pos/h - (0, 0.5), as advect_floating_items.cpp:116-120
//                    and 239-244 call it; one thread per item, atomic adds.
//  k_sample_velocity bilinearVel (advect_floating_items.cpp:11-14): the
//                    bilinearSample (interpolators.hpp:11-27) of vx at
//                    c - (0.5, 0) and of vy at c - (0, 0.5).
//  k_set_grids       Simulation::setGrids (simulation.hpp:82-98) for a list
//                    of distinct cells.
//  k_shift_*         UbootGlApp::shiftMap (ubootgl_app.cpp:245-298): fields
//                    moved one column west, the new terrain applied with
//                    setGrids, inflow column reset.
// Arithmetic in the reference's order (no contraction).
#include "ubg_internal.cuh"

namespace ubg {
namespace {

// glm::clamp(c, (0, 0), (w - 1.1f, h - 1.1f)), ivec2(c), fract(c)
struct Bil {
  int ix, iy;
  float sx, sy;
};
__device__ __forceinline__ Bil bil_coords(float cx, float cy, int gw, int gh) {
  cx = fminf(fmaxf(cx, 0.0f), (float)gw - 1.1f);
  cy = fminf(fmaxf(cy, 0.0f), (float)gh - 1.1f);
  Bil b;
  b.ix = (int)cx;
  b.iy = (int)cy;
  b.sx = cx - floorf(cx);
  b.sy = cy - floorf(cy);
  return b;
}

__device__ __forceinline__ float bil_sample(const float *g, int P, int gw, int gh, float cx,
                                            float cy) {
  Bil b = bil_coords(cx, cy, gw, gh);
  const float *r0 = g + (size_t)b.iy * P + b.ix;
  float v1 = r0[0], v2 = r0[1], v3 = r0[P], v4 = r0[P + 1];
  float vm1 = v1 + (v2 - v1) * b.sx;
  float vm2 = v3 + (v4 - v3) * b.sx;
  return vm1 + (vm2 - vm1) * b.sy;
}

__device__ __forceinline__ void bil_scatter(float *g, int P, int gw, int gh, float cx, float cy,
                                            float v) {
  Bil b = bil_coords(cx, cy, gw, gh);
  float ax = 1.0f - b.sx, ay = 1.0f - b.sy;
  float *r0 = g + (size_t)b.iy * P + b.ix;
  atomicAdd(r0 + P + 1, b.sx * b.sy * v);
  atomicAdd(r0 + P, ax * b.sy * v);
  atomicAdd(r0 + 1, b.sx * ay * v);
  atomicAdd(r0, ax * ay * v);
}

__global__ void k_scatter_accum(float *ax, float *ay, int P, int W, int H, const float2 *xy,
                                const float2 *v, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 c = xy[i], d = v[i];
  bil_scatter(ax, P, W - 1, H, c.x - 0.5f, c.y - 0.0f, d.x);
  bil_scatter(ay, P, W, H - 1, c.x - 0.0f, c.y - 0.5f, d.y);
}

__global__ void k_sample_velocity(const float *vx, const float *vy, int P, int W, int H,
                                  const float2 *xy, float2 *out, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 c = xy[i];
  out[i] = make_float2(bil_sample(vx, P, W - 1, H, c.x - 0.5f, c.y - 0.0f),
                       bil_sample(vy, P, W, H - 1, c.x - 0.0f, c.y - 0.5f));
}

// setGrids on distinct cells: flag = val; a cell set to 0 (at any point of
// the caller's sequence: `zero`) zeroes its four faces (front buffers) and p.
__global__ void k_set_grids(const int2 *cells, const uint8_t *val, const uint8_t *zero, int n,
                            uint8_t *flag, float *vx, float *vy, float *p, int P, int W, int H) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int x = cells[i].x, y = cells[i].y;
  flag[(size_t)y * P + x] = val[i];
  if (!zero[i]) return;
  if (x < W - 1) vx[(size_t)y * P + x] = 0.0f;
  if (x > 0) vx[(size_t)y * P + x - 1] = 0.0f;
  if (y < H - 1) vy[(size_t)y * P + x] = 0.0f;
  if (y > 0) vy[(size_t)(y - 1) * P + x] = 0.0f;
  p[(size_t)y * P + x] = 0.0f;
}

// shiftMap, first part: back(x-1) = front(x) for x in [2, w-1] of a
// staggered component (both buffers take the old front value).
__global__ void k_shift_to_back(const float *front, float *back, int P, int w, int h) {
  int x = blockIdx.x * 32 + threadIdx.x + 2, y = blockIdx.y * 8 + threadIdx.y;
  if (x >= w || y >= h) return;
  back[(size_t)y * P + x - 1] = front[(size_t)y * P + x];
}
__global__ void k_copy_cols(const float *src, float *dst, int P, int x0, int x1, int h) {
  int x = blockIdx.x * 32 + threadIdx.x + x0, y = blockIdx.y * 8 + threadIdx.y;
  if (x >= x1 || y >= h) return;
  dst[(size_t)y * P + x] = src[(size_t)y * P + x];
}
// p(x-1) = p(x) for x in [1, W-1] into the other buffer, column W-1 kept.
__global__ void k_shift_p(const float *p, float *out, int P, int W, int H) {
  int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  if (x >= W || y >= H) return;
  out[(size_t)y * P + x] = p[(size_t)y * P + (x < W - 1 ? x + 1 : x)];
}
// setGrids for every cell of the new terrain (flag already stored): zero
// the faces and p of solid cells.
__global__ void k_apply_solid(const uint8_t *flag, float *vx, float *vy, float *p, int P, int W,
                              int H) {
  int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  if (x >= W || y >= H) return;
  if (flag[(size_t)y * P + x]) return;
  if (x < W - 1) vx[(size_t)y * P + x] = 0.0f;
  if (x > 0) vx[(size_t)y * P + x - 1] = 0.0f;
  if (y < H - 1) vy[(size_t)y * P + x] = 0.0f;
  if (y > 0) vy[(size_t)(y - 1) * P + x] = 0.0f;
  p[(size_t)y * P + x] = 0.0f;
}
// vx.f(0, y) = vx.b(0, y) = inletVelocity * flag(0, y)
__global__ void k_inflow(float *vf, float *vb, const uint8_t *flag, int P, int H, float u) {
  int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= H) return;
  float v = u * (float)flag[(size_t)y * P];
  vf[(size_t)y * P] = v;
  vb[(size_t)y * P] = v;
}

dim3 grid2(int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); }

}  // namespace

void launch_scatter_accum(float *ax, float *ay, int P, int W, int H, const float2 *xy,
                          const float2 *v, int n, cudaStream_t st) {
  if (n <= 0) return;
  k_scatter_accum<<<(n + 255) / 256, 256, 0, st>>>(ax, ay, P, W, H, xy, v, n);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_sample_velocity(const float *vx, const float *vy, int P, int W, int H,
                            const float2 *xy, float2 *out, int n, cudaStream_t st) {
  if (n <= 0) return;
  k_sample_velocity<<<(n + 255) / 256, 256, 0, st>>>(vx, vy, P, W, H, xy, out, n);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_set_grids(const int2 *cells, const uint8_t *val, const uint8_t *zero, int n,
                      uint8_t *flag, float *vx, float *vy, float *p, int P, int W, int H,
                      cudaStream_t st) {
  if (n <= 0) return;
  k_set_grids<<<(n + 255) / 256, 256, 0, st>>>(cells, val, zero, n, flag, vx, vy, p, P, W, H);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_shift_map(VelBufs &v, int fx, int fy, const float *p_in, float *p_out,
                      const uint8_t *flag, int P, int W, int H, float inlet_u, cudaStream_t st) {
  const int wx = W - 1, wy = W;
  k_shift_to_back<<<grid2(wx - 2, H), dim3(32, 8), 0, st>>>(v.vx[fx], v.vx[1 - fx], P, wx, H);
  UBG_LAUNCH_CHECK();
  k_copy_cols<<<grid2(wx - 2, H), dim3(32, 8), 0, st>>>(v.vx[1 - fx], v.vx[fx], P, 1, wx - 1, H);
  UBG_LAUNCH_CHECK();
  k_shift_to_back<<<grid2(wy - 2, H - 1), dim3(32, 8), 0, st>>>(v.vy[fy], v.vy[1 - fy], P, wy,
                                                                H - 1);
  UBG_LAUNCH_CHECK();
  k_copy_cols<<<grid2(wy - 2, H - 1), dim3(32, 8), 0, st>>>(v.vy[1 - fy], v.vy[fy], P, 1, wy - 1,
                                                            H - 1);
  UBG_LAUNCH_CHECK();
  k_shift_p<<<grid2(W, H), dim3(32, 8), 0, st>>>(p_in, p_out, P, W, H);
  UBG_LAUNCH_CHECK();
  k_apply_solid<<<grid2(W, H), dim3(32, 8), 0, st>>>(flag, v.vx[fx], v.vy[fy], p_out, P, W, H);
  UBG_LAUNCH_CHECK();
  k_inflow<<<(H + 127) / 128, 128, 0, st>>>(v.vx[fx], v.vx[1 - fx], flag, P, H, inlet_u);
  UBG_LAUNCH_CHECK();
  g_stats.launches += 7;
}

}  // namespace ubg

// ------------------------------------------------------------ self-test
namespace ubg {
namespace {
__global__ void k_div_check(const float *x, int n, float d, float r, unsigned *bad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float a = div_rn(x[i], d, r), b = x[i] / d;
  if (__float_as_uint(a) != __float_as_uint(b) && !(a != a && b != b)) atomicAdd(bad, 1u);
}
}  // namespace

int selftest_div_rn(const float *x, int n, float d, unsigned *mismatches) {
  // both buffers are freed on every path, including a failing CUDA call
  struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
      if (p) cudaFree(p);
    }
  } bx, bb;
  UBG_CUDA(cudaMalloc(&bx.p, (size_t)n * sizeof(float)));
  UBG_CUDA(cudaMalloc(&bb.p, sizeof(unsigned)));
  float *dx = (float *)bx.p;
  unsigned *dbad = (unsigned *)bb.p;
  UBG_CUDA(cudaMemcpy(dx, x, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
  UBG_CUDA(cudaMemset(dbad, 0, sizeof(unsigned)));
  k_div_check<<<(n + 255) / 256, 256>>>(dx, n, d, 1.0f / d, dbad);
  UBG_LAUNCH_CHECK();
  UBG_CUDA(cudaMemcpy(mismatches, dbad, sizeof(unsigned), cudaMemcpyDeviceToHost));
  return 0;
}
}  // namespace ubg
