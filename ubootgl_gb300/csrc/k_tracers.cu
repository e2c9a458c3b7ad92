// Display tracers and the display velocity texture, the two GL compute
// shaders of te42kyfo/ubootgl restated as CUDA kernels over the device-
// resident staggered fields (no graphics interop: the texture is a plain
// device buffer).
//
//  k_velocity_texture  interp_shader.cs:14-34 (velocity_textures.cpp:63-93):
//                      texel (i, j) of (2W-1) x (2H-1) samples vx at
//                      (i/(2W-2), (j+1)/(2H)) and vy at ((i+1)/(2W), j/(2H-2))
//                      with GL bilinear filtering (texel centres (k+0.5)/n,
//                      wrap REPEAT), magnitude = length(vec2(vx, vy)).
//  k_tracers           advect_tracer_points.cs:42-82: RK2 midpoint step of
//                      every tracer's newest point, stop and age 0.1 outside
//                      the domain or where the flag (bilinear, CLAMP_TO_EDGE
//                      in s, REPEAT in t) is < 0.6, reseed from
//                      wang_hash(gid + seed) and the Numerical Recipes LCG
//                      once the age exceeds 2*3.141, else advance the ring.
//                      The reference samples the display texture, which the
//                      GL path rebuilds every frame; here each lookup forms
//                      the four texels it blends straight from the
//                      staggered vx / vy with the texture kernel's own
//                      arithmetic (texel()), so no (2W-1) x (2H-1) texture
//                      is written per step (1.07 GB at 8192 x 4096) and the
//                      results are the same bits.
// One thread per texel / tracer; arithmetic in the shaders' order (FP32
// weights instead of GL's fixed-point filter weights).
#include "ubg_internal.cuh"

namespace ubg {
namespace {

__device__ __forceinline__ float frac_floor(float u, int &i0) {
  float fl = floorf(u);
  i0 = (int)fl;
  return u - fl;
}
__device__ __forceinline__ int wrap_repeat(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}
__device__ __forceinline__ int wrap_clamp(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }

// Bilinear fetch of a pitched float texture (REPEAT in both directions).
__device__ __forceinline__ float tex_f(const float *__restrict__ t, int P, int nx, int ny, float s,
                                       float tt) {
  int i0, j0;
  float a = frac_floor(s * (float)nx - 0.5f, i0);
  float b = frac_floor(tt * (float)ny - 0.5f, j0);
  int i1 = wrap_repeat(i0 + 1, nx), j1 = wrap_repeat(j0 + 1, ny);
  i0 = wrap_repeat(i0, nx);
  j0 = wrap_repeat(j0, ny);
  float t00 = __ldg(t + (size_t)j0 * P + i0), t10 = __ldg(t + (size_t)j0 * P + i1);
  float t01 = __ldg(t + (size_t)j1 * P + i0), t11 = __ldg(t + (size_t)j1 * P + i1);
  float r0 = t00 * (1.0f - a) + t10 * a;
  float r1 = t01 * (1.0f - a) + t11 * a;
  return r0 * (1.0f - b) + r1 * b;
}

// Texel (i, j) of the display texture (interp_shader.cs:20-31).
__device__ __forceinline__ float2 texel(const float *__restrict__ vx, const float *__restrict__ vy,
                                        int P, int W, int H, int i, int j) {
  float sx = (float)i / (2.0f * (float)W - 2.0f), tx = (float)(j + 1) / (2.0f * (float)H);
  float sy = (float)(i + 1) / (2.0f * (float)W), ty = (float)j / (2.0f * (float)H - 2.0f);
  return make_float2(tex_f(vx, P, W - 1, H, sx, tx), tex_f(vy, P, W, H - 1, sy, ty));
}

__global__ void k_velocity_texture(const float *__restrict__ vx, const float *__restrict__ vy,
                                   int P, int W, int H, float2 *vxy, float *mag) {
  int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  int tw = 2 * W - 1, th = 2 * H - 1;
  if (i >= tw || j >= th) return;
  const float2 t = texel(vx, vy, P, W, H, i, j);
  const float a = t.x, b = t.y;
  size_t k = (size_t)j * tw + i;
  vxy[k] = make_float2(a, b);
  if (mag) mag[k] = sqrtf(a * a + b * b);
}

// Bilinear lookup of the display texture (REPEAT in both directions), its
// four texels formed from the staggered fields.
__device__ __forceinline__ float2 tex_vxy(const float *__restrict__ vx,
                                          const float *__restrict__ vy, int P, int W, int H,
                                          float s, float tt) {
  const int nx = 2 * W - 1, ny = 2 * H - 1;
  int i0, j0;
  float a = frac_floor(s * (float)nx - 0.5f, i0);
  float b = frac_floor(tt * (float)ny - 0.5f, j0);
  int i1 = wrap_repeat(i0 + 1, nx), j1 = wrap_repeat(j0 + 1, ny);
  i0 = wrap_repeat(i0, nx);
  j0 = wrap_repeat(j0, ny);
  float2 t00 = texel(vx, vy, P, W, H, i0, j0), t10 = texel(vx, vy, P, W, H, i1, j0);
  float2 t01 = texel(vx, vy, P, W, H, i0, j1), t11 = texel(vx, vy, P, W, H, i1, j1);
  float2 r;
  float r0 = t00.x * (1.0f - a) + t10.x * a;
  float r1 = t01.x * (1.0f - a) + t11.x * a;
  r.x = r0 * (1.0f - b) + r1 * b;
  r0 = t00.y * (1.0f - a) + t10.y * a;
  r1 = t01.y * (1.0f - a) + t11.y * a;
  r.y = r0 * (1.0f - b) + r1 * b;
  return r;
}

// Flag texture: the cell flags as 0.0 / 1.0, CLAMP_TO_EDGE in s, REPEAT in t.
__device__ __forceinline__ float tex_flag(const uint8_t *__restrict__ f, int P, int nx, int ny,
                                          float s, float tt) {
  int i0, j0;
  float a = frac_floor(s * (float)nx - 0.5f, i0);
  float b = frac_floor(tt * (float)ny - 0.5f, j0);
  int i1 = wrap_clamp(i0 + 1, nx), j1 = wrap_repeat(j0 + 1, ny);
  i0 = wrap_clamp(i0, nx);
  j0 = wrap_repeat(j0, ny);
  float t00 = (float)__ldg(f + (size_t)j0 * P + i0), t10 = (float)__ldg(f + (size_t)j0 * P + i1);
  float t01 = (float)__ldg(f + (size_t)j1 * P + i0), t11 = (float)__ldg(f + (size_t)j1 * P + i1);
  float r0 = t00 * (1.0f - a) + t10 * a;
  float r1 = t01 * (1.0f - a) + t11 * a;
  return r0 * (1.0f - b) + r1 * b;
}

__device__ __forceinline__ uint32_t wang_hash(uint32_t seed) {
  seed = (seed ^ 61u) ^ (seed >> 16);
  seed *= 9u;
  seed = seed ^ (seed >> 4);
  seed *= 0x27d4eb2du;
  seed = seed ^ (seed >> 15);
  return seed;
}

__global__ void __launch_bounds__(256) k_tracers(TracerArgs a) {
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.ntracers) return;
  uint32_t rng = wang_hash((uint32_t)gid + a.seed);
  size_t base = (size_t)gid * a.npoints;
  uint32_t e = a.end[gid];
  uint32_t curr = e % (uint32_t)a.npoints, next = (e + 1u) % (uint32_t)a.npoints;
  float2 cp = a.points[base + curr];
  const float pdx = a.pdx, pdy = a.pdy, dt = a.dt;
  float2 v1 = tex_vxy(a.vx, a.vy, a.P, a.W, a.H, cp.x / pdx, cp.y / pdy);
  float mx = cp.x + v1.x * dt * 0.5f, my = cp.y + v1.y * dt * 0.5f;
  float2 v2 = tex_vxy(a.vx, a.vy, a.P, a.W, a.H, mx / pdx, my / pdy);
  float nx = cp.x + v2.x * dt, ny = cp.y + v2.y * dt;
  bool out = cp.x < 0.0f || cp.y < 0.0f || cp.x > pdx || cp.y > pdy;
  float fl = tex_flag(a.flag, a.fpitch, a.nfx, a.nfy, cp.x / pdx, cp.y / pdy);
  float age = a.ages[gid];
  if (out || fl < 0.6f) {
    nx = cp.x;
    ny = cp.y;
    age += 0.1f;
  }
  if (age > 2.0f * 3.141f) {
    a.start[gid] = 0;
    a.end[gid] = 0;
    rng = 1664525u * rng + 1013904223u;
    float rx = (float)(rng % 100000u) / 100000.0f;
    rng = 1664525u * rng + 1013904223u;
    float ry = (float)(rng % 100000u) / 100000.0f;
    a.points[base] = make_float2(rx * pdx, ry * pdy);
    a.ages[gid] = 0.0f;
  } else {
    a.end[gid] = next;
    uint32_t s = a.start[gid];
    if (s == next) a.start[gid] = (s + 1u) % (uint32_t)a.npoints;
    a.points[base + next] = make_float2(nx, ny);
    a.ages[gid] = age + 0.02f;
  }
}

}  // namespace

void launch_velocity_texture(const float *vx, const float *vy, int P, int W, int H, float2 *vxy,
                             float *mag, cudaStream_t st) {
  ProfScope ps_(KC_TRACERS, st);
  dim3 grid((2 * W - 1 + 31) / 32, (2 * H - 1 + 7) / 8);
  k_velocity_texture<<<grid, dim3(32, 8), 0, st>>>(vx, vy, P, W, H, vxy, mag);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void launch_tracers(const TracerArgs &a, cudaStream_t st) {
  ProfScope ps_(KC_TRACERS, st);
  if (a.ntracers <= 0) return;
  k_tracers<<<(a.ntracers + 255) / 256, 256, 0, st>>>(a);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

}  // namespace ubg
