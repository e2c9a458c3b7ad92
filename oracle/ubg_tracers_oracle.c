/*
 * CPU restatement of ubootgl's display tracers -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference computes these only in OpenGL compute shaders, which cannot
 * run on this machine (no graphics stack), so parity with the shaders
 * themselves is unpinned; this file restates their arithmetic in plain C and
 * the CUDA kernels are checked against it.
 *
 *  - ubo_velocity_texture_f: interp_shader.cs:14-34 / velocity_textures.cpp
 *    :63-93.  Texel (i, j) of the (2W-1) x (2H-1) texture samples the
 *    staggered vx ((W-1) x H) at (i/(2W-2), (j+1)/(2H)) and vy (W x (H-1)) at
 *    ((i+1)/(2W), j/(2H-2)) with GL bilinear filtering (texel centres at
 *    (k+0.5)/n, wrap mode REPEAT: the textures set no wrap parameter), and
 *    its magnitude is length(vec2(vx, vy)).
 *  - ubo_tracers_f_step: advect_tracer_points.cs:42-82.  RK2 midpoint step of
 *    each tracer's newest point through the velocity texture (REPEAT), stop
 *    and age by 0.1 outside [0, pdim] or where the flag texture (bilinear,
 *    CLAMP_TO_EDGE in s as draw_2dbuf.cpp sets it, REPEAT in t) is < 0.6,
 *    reseed with wang_hash(gid + seed) -> LCG -> (x % 100000) / 100000.0 once
 *    the age exceeds 2*3.141, else advance the ring pointers and add 0.02.
 * Filtering weights are full FP32 here (GL hardware uses fixed-point
 * weights); operations are written out in evaluation order.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

typedef struct {
  float x, y;
} f2;

static inline float frac_floor(float u, int *i0) {
  float fl = floorf(u);
  *i0 = (int)fl;
  return u - fl;
}

static inline int wrap_repeat(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}
static inline int wrap_clamp(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }

/* Bilinear sample of a scalar texture of n_x x n_y texels at normalised
 * (s, t); mode_s / mode_t: 0 = REPEAT, 1 = CLAMP_TO_EDGE. */
static float tex_bilinear(const float *tex, int nx, int ny, float s, float t, int mode_s,
                          int mode_t) {
  int i0, j0;
  float a = frac_floor(s * (float)nx - 0.5f, &i0);
  float b = frac_floor(t * (float)ny - 0.5f, &j0);
  int i1 = i0 + 1, j1 = j0 + 1;
  i0 = mode_s ? wrap_clamp(i0, nx) : wrap_repeat(i0, nx);
  i1 = mode_s ? wrap_clamp(i1, nx) : wrap_repeat(i1, nx);
  j0 = mode_t ? wrap_clamp(j0, ny) : wrap_repeat(j0, ny);
  j1 = mode_t ? wrap_clamp(j1, ny) : wrap_repeat(j1, ny);
  float t00 = tex[(size_t)j0 * nx + i0], t10 = tex[(size_t)j0 * nx + i1];
  float t01 = tex[(size_t)j1 * nx + i0], t11 = tex[(size_t)j1 * nx + i1];
  float r0 = t00 * (1.0f - a) + t10 * a;
  float r1 = t01 * (1.0f - a) + t11 * a;
  return r0 * (1.0f - b) + r1 * b;
}

static f2 tex_bilinear2(const float *vxy, int nx, int ny, float s, float t) {
  int i0, j0;
  float a = frac_floor(s * (float)nx - 0.5f, &i0);
  float b = frac_floor(t * (float)ny - 0.5f, &j0);
  int i1 = wrap_repeat(i0 + 1, nx), j1 = wrap_repeat(j0 + 1, ny);
  i0 = wrap_repeat(i0, nx);
  j0 = wrap_repeat(j0, ny);
  f2 r;
  for (int c = 0; c < 2; c++) {
    float t00 = vxy[2 * ((size_t)j0 * nx + i0) + c], t10 = vxy[2 * ((size_t)j0 * nx + i1) + c];
    float t01 = vxy[2 * ((size_t)j1 * nx + i0) + c], t11 = vxy[2 * ((size_t)j1 * nx + i1) + c];
    float r0 = t00 * (1.0f - a) + t10 * a;
    float r1 = t01 * (1.0f - a) + t11 * a;
    float v = r0 * (1.0f - b) + r1 * b;
    if (c == 0)
      r.x = v;
    else
      r.y = v;
  }
  return r;
}

/* vx: (W-1) x H, vy: W x (H-1), row-major; out vxy: (2W-1) x (2H-1) x 2,
 * mag: (2W-1) x (2H-1). */
void ubo_velocity_texture_f(const float *vx, const float *vy, int W, int H, float *vxy,
                            float *mag) {
  int tw = 2 * W - 1, th = 2 * H - 1;
  int j;
#pragma omp parallel for schedule(static)
  for (j = 0; j < th; j++)
    for (int i = 0; i < tw; i++) {
      float sx = (float)i / (2.0f * (float)W - 2.0f), tx = (float)(j + 1) / (2.0f * (float)H);
      float sy = (float)(i + 1) / (2.0f * (float)W), ty = (float)j / (2.0f * (float)H - 2.0f);
      float a = tex_bilinear(vx, W - 1, H, sx, tx, 0, 0);
      float b = tex_bilinear(vy, W, H - 1, sy, ty, 0, 0);
      size_t k = (size_t)j * tw + i;
      vxy[2 * k] = a;
      vxy[2 * k + 1] = b;
      mag[k] = sqrtf(a * a + b * b);
    }
}

static inline uint32_t wang_hash(uint32_t seed) {
  seed = (seed ^ 61u) ^ (seed >> 16);
  seed *= 9u;
  seed = seed ^ (seed >> 4);
  seed *= 0x27d4eb2du;
  seed = seed ^ (seed >> 15);
  return seed;
}

/* One tracer step.  points: ntracers * npoints * 2 floats; start/end: ring
 * pointers; ages.  vxy: velocity texture (tw x th x 2); flag: nfx x nfy. */
void ubo_tracers_f_step(float *points, const float *vxy, int tw, int th, const float *flag, int nfx,
                        int nfy, int ntracers, int npoints, uint32_t *start, uint32_t *end,
                        float *ages, float dt, float pdx, float pdimy, uint32_t rand_seed) {
  int gid;
#pragma omp parallel for schedule(static)
  for (gid = 0; gid < ntracers; gid++) {
    uint32_t rng = wang_hash((uint32_t)gid + rand_seed);
    size_t base = (size_t)gid * npoints;
    uint32_t curr = end[gid] % (uint32_t)npoints;
    uint32_t next = (end[gid] + 1u) % (uint32_t)npoints;
    float px = points[2 * (base + curr)], py = points[2 * (base + curr) + 1];
    f2 v1 = tex_bilinear2(vxy, tw, th, px / pdx, py / pdimy);
    float mx = px + v1.x * dt * 0.5f, my = py + v1.y * dt * 0.5f;
    f2 v2 = tex_bilinear2(vxy, tw, th, mx / pdx, my / pdimy);
    float nx_ = px + v2.x * dt, ny_ = py + v2.y * dt;
    int out = px < 0.0f || py < 0.0f || px > pdx || py > pdimy;
    float fl = tex_bilinear(flag, nfx, nfy, px / pdx, py / pdimy, 1, 0);
    if (out || fl < 0.6f) {
      nx_ = px;
      ny_ = py;
      ages[gid] += 0.1f;
    }
    if (ages[gid] > 2.0f * 3.141f) {
      start[gid] = 0;
      end[gid] = 0;
      rng = 1664525u * rng + 1013904223u;
      float rx = (float)(rng % 100000u) / 100000.0f;
      rng = 1664525u * rng + 1013904223u;
      float ry = (float)(rng % 100000u) / 100000.0f;
      points[2 * base] = rx * pdx;
      points[2 * base + 1] = ry * pdimy;
      ages[gid] = 0.0f;
    } else {
      end[gid] = next;
      if (start[gid] == end[gid]) start[gid] = (start[gid] + 1u) % (uint32_t)npoints;
      points[2 * (base + next)] = nx_;
      points[2 * (base + next) + 1] = ny_;
      ages[gid] = ages[gid] + 0.02f;
    }
  }
}
