// Tolerance-mode pressure solver: flexible conjugate gradients (FCG(1),
// Y. Notay, "Flexible conjugate gradients", SIAM J. Sci. Comput. 22(4),
// 2000) on the zero-gradient pressure system of MG::solve
// (pressure_solver.cpp:91-116: r = f + (1/h^2) sum_n flag_n (p_n - p) on
// the interior fluid cells), preconditioned by one V-cycle of the
// tolerance hierarchy (ext_vcycle, k_mg.cu), run until
// ||r|| <= tol ||f_c|| in FP64 norms.
//
// The reference always runs two V-cycles and never reaches a tolerance
// (simulation.cpp:189-190); this solver is the extension that does.
//
// Precision: the pressure iterate x is a double-float (two FP32 arrays,
// about 48 significant bits).  Rounding p to FP32 alone leaves a relative
// residual of 2e-4 at 512x256 and 6e-4 at 1024x512 for a flow state's
// pressure (its smooth part is large against the neighbour differences the
// residual is made of), so no FP32 p reaches 1e-6.  The Krylov vectors r,
// d, q and the preconditioner output z are FP32; stencil sums add their
// rounding errors back (TwoSum); dot products and norms are FP32 per thread
// and FP64 across threads, combined in a fixed order (the same bits on
// every run).  The mean of z over the interior fluid cells is taken out
// of every search direction (the constant the V-cycle leaves in z would
// otherwise turn the dot products into rounding noise).  The V-cycle runs
// its level 0 in FP32 and its coarse levels in FP32, FP16 or BF16
// (ubg_options precision).
//
// Compatibility: the system is singular (constants on each connected fluid
// region), and f sums to the net flux through the domain edges, which is
// not zero when inflow and outflow differ.  The solver moves that sum to
// the outflow column x = W-2 (f_c = f - sum(f) / n on its n fluid cells;
// all fluid cells when that column has none), where the reference's
// outflow boundary (setVBCs, simulation.cpp:80-102) takes up the
// imbalance.  Enclosed pockets have zero net flux and keep their f.
#include "ubg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace ubg {
namespace {

constexpr int BX = 32, BY = 8;  // 32 x 8 threads, 4 cells of a row per thread

__device__ __forceinline__ bool interior(int x, int y, int W, int H) {
  return x >= 1 && x < W - 1 && y >= 1 && y < H - 1;
}

// a + b = s + e exactly (Knuth's TwoSum; the library is built without FMA
// contraction, so every operation rounds as written).
__device__ __forceinline__ float two_sum(float a, float b, float *e) {
  const float s = a + b, bb = s - a;
  *e = (a - (s - bb)) + (b - bb);
  return s;
}
// a + b + c + d with the rounding errors of the three additions added back:
// the stencil's neighbour differences are exact in FP32 but cancel in the
// sum by orders of magnitude for a smooth field, so a plain FP32 sum loses
// the digits the residual is made of.
__device__ __forceinline__ float sum4(float a, float b, float c, float d) {
  float e1, e2, e3;
  const float s1 = two_sum(a, b, &e1), s2 = two_sum(c, d, &e2);
  const float s = two_sum(s1, s2, &e3);
  return s + ((e1 + e2) + e3);
}

// The pressure iterate is a double-float: x = xh + xl, |xl| <= ulp(xh) / 2
// (about 48 significant bits, all arithmetic in FP32: on GB300's FP64 pipe
// an FP64 iterate made the residual pass the slowest kernel of the loop).
// (xh_n + xl_n) - (xh + xl) as a head (the exact difference of the heads
// with its rounding error moved to the tail) and a small tail.
__device__ __forceinline__ float df_diff(float hn, float ln, float h, float l, float *tail) {
  float e;
  const float d = two_sum(hn, -h, &e);
  *tail = e + (ln - l);
  return d;
}
// The neighbour sum of a cell from up to four double-float differences:
// heads summed with their rounding errors added back, tails added plainly.
__device__ __forceinline__ float df_sum4(const float (&dh)[4], const float (&dl)[4]) {
  return sum4(dh[0], dh[1], dh[2], dh[3]) + ((dl[0] + dl[1]) + (dl[2] + dl[3]));
}
// (h, l) + a * d, with the product exact (FMA error term) and the result
// renormalised.
__device__ __forceinline__ void df_axpy(float &h, float &l, float a, float d) {
  const float p = a * d, pe = __fmaf_rn(a, d, -p);
  float e;
  const float s = two_sum(h, p, &e);
  const float t = (e + pe) + l;
  h = s + t;
  l = t - (h - s);
}

// Reduction of up to three sums and a max over the grid, in a fixed order:
// each block reduces its threads (warp shuffles, then its warps in order)
// and writes its partials; the last block to finish (a ticket counter)
// adds the partials of all blocks in block order and stores the results
// (dst[k] = sum; *mdst = max), then resets the ticket.  The results are the
// same bits on every run, and no same-address atomics pile up (FP64 atomics
// to one address from 8192 blocks cost ~90 us per kernel).
template <int N>
__device__ __forceinline__ void block_reduce(double (&v)[N], unsigned mx, double *const (&dst)[N],
                                             unsigned *mdst, FcgPartials *pr) {
  const int tid = threadIdx.y * BX + threadIdx.x;
#pragma unroll
  for (int k = 0; k < N; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  mx = __reduce_max_sync(0xffffffffu, mx);
  __shared__ double red[N][BY];
  __shared__ unsigned redm[BY];
  __shared__ bool last;
  if ((tid & 31) == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) red[k][tid >> 5] = v[k];
    redm[tid >> 5] = mx;
  }
  __syncthreads();
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) {
      double t = 0.0;
      for (int i = 0; i < BY; i++) t += red[k][i];
      pr->v[blockIdx.x][k] = t;
    }
    unsigned m = 0;
    for (int i = 0; i < BY; i++) m = max(m, redm[i]);
    pr->m[blockIdx.x] = m;
    __threadfence();
    last = atomicAdd(&pr->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last block: every thread adds the partials of blocks tid, tid + 256,
  // ... (independent loads, all in flight), then the block reduces in a
  // fixed order as above
  const int nb = (int)gridDim.x;
  double t[N];
  unsigned m = 0;
#pragma unroll
  for (int k = 0; k < N; k++) t[k] = 0.0;
  for (int b = tid; b < nb; b += BX * BY) {
#pragma unroll
    for (int k = 0; k < N; k++) t[k] += __ldcg(&pr->v[b][k]);
    m = max(m, __ldcg(&pr->m[b]));
  }
#pragma unroll
  for (int k = 0; k < N; k++)
    for (int o = 16; o > 0; o >>= 1) t[k] += __shfl_xor_sync(0xffffffffu, t[k], o);
  m = __reduce_max_sync(0xffffffffu, m);
  __syncthreads();  // red / redm are reused
  if ((tid & 31) == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) red[k][tid >> 5] = t[k];
    redm[tid >> 5] = m;
  }
  __syncthreads();
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) {
      double sum = 0.0;
      for (int i = 0; i < BY; i++) sum += red[k][i];
      if (dst[k]) *dst[k] = sum;
    }
    unsigned mm = 0;
    for (int i = 0; i < BY; i++) mm = max(mm, redm[i]);
    if (mdst) *mdst = mm;
  }
  if (tid == 0) pr->ticket = 0u;
}

// Sum of f over the interior fluid cells, the fluid cells of the outflow
// column x = W-2 and all interior fluid cells (counts).
__global__ void __launch_bounds__(BX *BY) k_fcg_fsum(const float *__restrict__ f,
                                                     const uint8_t *__restrict__ code, int W,
                                                     int H, int P, FcgScalars *sc,
                                                     FcgPartials *pr) {
  griddep_wait();
  float s = 0.0f;
  int ne = 0, nf = 0;
  // grid-stride over tiles of 128 x 8 cells: a few blocks per SM, so few
  // same-address atomics in the final reduction
  const int tiles_x = (W + 4 * BX - 1) / (4 * BX), ntiles = tiles_x * ((H + BY - 1) / BY);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int x4 = ((t % tiles_x) * BX + threadIdx.x) * 4, y = (t / tiles_x) * BY + threadIdx.y;
    if (y >= 1 && y < H - 1) {
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int x = x4 + j;
        if (x >= 1 && x < W - 1) {
          const size_t i = (size_t)y * P + x;
          if (__ldg(code + i) & 1u) {
            s += __ldg(f + i);
            nf++;
            if (x == W - 2) ne++;
          }
        }
      }
    }
  }
  double v[3] = {(double)s, (double)ne, (double)nf};
  double *const dst[3] = {&sc->fsum, &sc->neast, &sc->nfluid};
  block_reduce<3>(v, 0u, dst, nullptr, pr);
}

// The compatibility correction: (on the outflow column, everywhere else)
// in FP32, formed once per launch.
__device__ __forceinline__ float2 compat_corr(const FcgScalars *sc) {
  const double ne = sc->neast, nf = sc->nfluid;
  if (ne > 0.0) return make_float2((float)(sc->fsum / ne), 0.0f);
  const float a = nf > 0.0 ? (float)(sc->fsum / nf) : 0.0f;
  return make_float2(a, a);
}

// r = f_c + ihsq * sum_n flag_n (x_n - x) on the interior fluid cells (0
// elsewhere), the neighbour differences in double-float; neighbours on the
// domain edge are zero-gradient copies (difference 0).  Writes r and
// accumulates ||r||^2 and max|r|, and with want_ff also ||f_c||^2.
__global__ void __launch_bounds__(BX *BY) k_fcg_resid(const float *__restrict__ xh,
                                                      const float *__restrict__ xl,
                                                      const float *__restrict__ f,
                                                      const uint8_t *__restrict__ code, int W,
                                                      int H, int P, float ihsq, float *r,
                                                      FcgScalars *sc, int want_ff, FcgPartials *pr) {
  griddep_wait();
  float ff = 0.0f, rr = 0.0f;
  unsigned mx = 0;
  const float2 corr = compat_corr(sc);
  // grid-stride over tiles of 128 x 8 cells: a few blocks per SM, so few
  // partial sums to combine
  const int tiles_x = (W + 4 * BX - 1) / (4 * BX), ntiles = tiles_x * ((H + BY - 1) / BY);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int x4 = ((t % tiles_x) * BX + threadIdx.x) * 4, y = (t / tiles_x) * BY + threadIdx.y;
    if (x4 >= W || y >= H) continue;
    float rv[4] = {0.f, 0.f, 0.f, 0.f};
    const size_t i0 = (size_t)y * P + x4;
    auto cell = [&](int j, unsigned c, float hc, float lc, float hw, float lw, float he, float le,
                    float hs, float ls, float hn, float ln, float fv) {
      float dh[4], dl[4];
      dh[0] = (c & 2u) ? df_diff(hw, lw, hc, lc, &dl[0]) : (dl[0] = 0.0f);
      dh[1] = (c & 4u) ? df_diff(he, le, hc, lc, &dl[1]) : (dl[1] = 0.0f);
      dh[2] = (c & 8u) ? df_diff(hs, ls, hc, lc, &dl[2]) : (dl[2] = 0.0f);
      dh[3] = (c & 16u) ? df_diff(hn, ln, hc, lc, &dl[3]) : (dl[3] = 0.0f);
      const float fc = fv - (x4 + j == W - 2 ? corr.x : corr.y);
      rv[j] = fc + ihsq * df_sum4(dh, dl);
      ff = __fmaf_rn(fc, fc, ff);
      rr = __fmaf_rn(rv[j], rv[j], rr);
      mx = max(mx, __float_as_uint(fabsf(rv[j])));
    };
    if (x4 >= 2 && x4 + 4 <= W - 2 && y >= 2 && y <= H - 3) {
      // interior: every neighbour is an interior cell; rows as float4
      auto R4 = [&](const float *a, size_t i, float *o) {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(a + i));
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
        o[3] = v.w;
      };
      float hc[4], lc[4], hs[4], ls[4], hn[4], ln[4];
      R4(xh, i0, hc);
      R4(xl, i0, lc);
      R4(xh, i0 - P, hs);
      R4(xl, i0 - P, ls);
      R4(xh, i0 + P, hn);
      R4(xl, i0 + P, ln);
      const float hw = __ldg(xh + i0 - 1), lw = __ldg(xl + i0 - 1);
      const float he = __ldg(xh + i0 + 4), le = __ldg(xl + i0 + 4);
      const uchar4 cv = __ldg(reinterpret_cast<const uchar4 *>(code + i0));
      const float4 fv = __ldg(reinterpret_cast<const float4 *>(f + i0));
      const unsigned C4[4] = {cv.x, cv.y, cv.z, cv.w};
      const float F4[4] = {fv.x, fv.y, fv.z, fv.w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        if (!(C4[j] & 1u)) continue;
        cell(j, C4[j], hc[j], lc[j], j > 0 ? hc[j - 1] : hw, j > 0 ? lc[j - 1] : lw,
             j < 3 ? hc[j + 1] : he, j < 3 ? lc[j + 1] : le, hs[j], ls[j], hn[j], ln[j], F4[j]);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int x = x4 + j;
        if (x >= W || !interior(x, y, W, H)) continue;
        const size_t i = i0 + j;
        unsigned c = __ldg(code + i);
        if (!(c & 1u)) continue;
        // neighbours on the domain edge: zero-gradient copies
        if (x - 1 < 1) c &= ~2u;
        if (x + 1 >= W - 1) c &= ~4u;
        if (y - 1 < 1) c &= ~8u;
        if (y + 1 >= H - 1) c &= ~16u;
        auto H1 = [&](size_t k, bool on) { return on ? __ldg(xh + k) : 0.0f; };
        auto L1 = [&](size_t k, bool on) { return on ? __ldg(xl + k) : 0.0f; };
        cell(j, c, __ldg(xh + i), __ldg(xl + i), H1(i - 1, c & 2u), L1(i - 1, c & 2u),
             H1(i + 1, c & 4u), L1(i + 1, c & 4u), H1(i - P, c & 8u), L1(i - P, c & 8u),
             H1(i + P, c & 16u), L1(i + P, c & 16u), __ldg(f + i));
      }
    }
    float *o = r + i0;
    if (x4 + 3 < W) {
      *reinterpret_cast<float4 *>(o) = make_float4(rv[0], rv[1], rv[2], rv[3]);
    } else {
      for (int j = 0; j < 4 && x4 + j < W; j++) o[j] = rv[j];
    }
  }
  double v[2] = {(double)ff, (double)rr};
  double *const dst[2] = {want_ff ? &sc->ff : nullptr, &sc->rr};
  block_reduce<2>(v, mx, dst, &sc->maxbits, pr);
}

// Sum of z over the interior fluid cells.  A maps a constant on a fluid
// region to 0, so nothing in the iteration removes the constant that the
// V-cycle leaves in z (its coarsest level is singular, and its right-hand
// side sums to zero only up to rounding).  Carried into the direction d,
// that constant enters (z, q), (d, q) and (d, r) through the rounding of
// sum(q) and sum(r) over the region; once the constant dominates d, those
// dot products are rounding noise and the iteration diverges from the
// accuracy it had reached (at 8192 x 4096 with 400 discs the residual
// climbed from 1e-6 to 1e-3).  k_fcg_zq and k_fcg_dir subtract the mean.
__global__ void __launch_bounds__(BX *BY) k_fcg_zsum(const float *__restrict__ z,
                                                     const uint8_t *__restrict__ code, int W,
                                                     int H, int P, FcgScalars *sc,
                                                     FcgPartials *pr) {
  griddep_wait();
  float s = 0.0f;
  // grid-stride over tiles of 128 x 8 cells, four tiles per pass with
  // their loads issued together (rows are padded to the pitch, a multiple
  // of 32 cells, so a float4 / uchar4 at x4 < W stays in the row)
  const int tiles_x = (W + 4 * BX - 1) / (4 * BX), ntiles = tiles_x * ((H + BY - 1) / BY);
  const int G = (int)gridDim.x;
  for (int t0 = blockIdx.x; t0 < ntiles; t0 += 4 * G) {
    float4 a[4];
    uchar4 c[4];
    int xs[4];
    bool ok[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int t = t0 + u * G;
      const int x4 = ((t % tiles_x) * BX + threadIdx.x) * 4, y = (t / tiles_x) * BY + threadIdx.y;
      ok[u] = t < ntiles && x4 < W && y >= 1 && y < H - 1;
      xs[u] = x4;
      if (ok[u]) {
        const size_t i = (size_t)y * P + x4;
        a[u] = *reinterpret_cast<const float4 *>(z + i);
        c[u] = __ldg(reinterpret_cast<const uchar4 *>(code + i));
      }
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if (!ok[u]) continue;
      const int x4 = xs[u];
      const float A[4] = {a[u].x, a[u].y, a[u].z, a[u].w};
      const unsigned C[4] = {c[u].x, c[u].y, c[u].z, c[u].w};
      float t4[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
        t4[j] = (x4 + j >= 1 && x4 + j < W - 1 && (C[j] & 1u)) ? A[j] : 0.0f;
      s = s + ((t4[0] + t4[1]) + (t4[2] + t4[3]));
    }
  }
  double v[1] = {(double)s};
  double *const dst[1] = {&sc->zsum};
  block_reduce<1>(v, 0u, dst, nullptr, pr);
}

__device__ __forceinline__ float z_mean(const FcgScalars *sc) {
  return sc->nfluid > 0.0 ? (float)(sc->zsum / sc->nfluid) : 0.0f;
}

// zq = (z - zm, q_prev), zm the mean of z over the interior fluid cells;
// zeroes the accumulators of k_fcg_dir.
__global__ void __launch_bounds__(BX *BY) k_fcg_zq(const float *__restrict__ z,
                                                   const float *__restrict__ q, int W, int H,
                                                   int P, FcgScalars *sc, int slot,
                                                   FcgPartials *pr) {
  griddep_wait();
  const float zm = z_mean(sc);
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    sc->dq[slot] = 0.0;
    sc->dr = 0.0;
  }
  float s = 0.0f;
  // grid-stride over tiles of 128 x 8 cells, four tiles per pass with
  // their loads issued together
  const int tiles_x = (W + 4 * BX - 1) / (4 * BX), ntiles = tiles_x * ((H + BY - 1) / BY);
  const int G = (int)gridDim.x;
  for (int t0 = blockIdx.x; t0 < ntiles; t0 += 4 * G) {
    float4 a[4], b[4];
    bool ok[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int t = t0 + u * G;
      const int x4 = ((t % tiles_x) * BX + threadIdx.x) * 4, y = (t / tiles_x) * BY + threadIdx.y;
      ok[u] = t < ntiles && x4 < W && y < H;
      if (ok[u]) {
        const size_t i = (size_t)y * P + x4;
        a[u] = *reinterpret_cast<const float4 *>(z + i);
        b[u] = *reinterpret_cast<const float4 *>(q + i);
      }
    }
    // q is 0 outside the interior fluid cells and beyond the width
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (ok[u])
        s = s + ((((a[u].x - zm) * b[u].x + (a[u].y - zm) * b[u].y) + (a[u].z - zm) * b[u].z) +
                 (a[u].w - zm) * b[u].w);
  }
  double v[1] = {(double)s};
  double *const dst[1] = {&sc->zq};
  block_reduce<1>(v, 0u, dst, nullptr, pr);
}

// d = (z - zm) + beta d_old (beta = -zq / dq_prev; 0 on the first
// iteration) on the interior fluid cells and the edges, d = 0 on the
// interior solid cells (where z and d_old are 0), q = A d = -ihsq * sum_n
// flag_n (d_n - d) on the interior fluid cells (0 elsewhere), (d, q) and
// (d, r); zeroes the accumulators of k_fcg_update.  The shift by zm is
// applied to every value read, so q sees the stored d of each fluid cell;
// the values of solid neighbours never enter q.
__global__ void __launch_bounds__(BX *BY) k_fcg_dir(const float *__restrict__ z,
                                                    const float *__restrict__ dold, float *dnew,
                                                    float *q, const float *__restrict__ r,
                                                    const uint8_t *__restrict__ code, int W,
                                                    int H, int P, float ihsq, FcgScalars *sc,
                                                    int first, int slot, FcgPartials *pr) {
  griddep_wait();
  const float beta = first ? 0.0f : (float)(-sc->zq / sc->dq[slot ^ 1]);
  const float zm = z_mean(sc);
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    sc->rr = 0.0;
    sc->maxbits = 0u;
  }
  float dq = 0.0f, dr = 0.0f;
  // grid-stride over tiles of 128 x 8 cells: a few blocks per SM, so few
  // same-address atomics in the final reduction
  const int tiles_x = (W + 4 * BX - 1) / (4 * BX), ntiles = tiles_x * ((H + BY - 1) / BY);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int x4 = ((t % tiles_x) * BX + threadIdx.x) * 4, y = (t / tiles_x) * BY + threadIdx.y;
    if (x4 < W && y < H) {
      auto D = [&](size_t i) {
        return first ? __ldg(z + i) - zm : (__ldg(z + i) - zm) + beta * __ldg(dold + i);
      };
      const size_t i0 = (size_t)y * P + x4;
      float dc[4], qv[4] = {0.f, 0.f, 0.f, 0.f};
      if (x4 >= 2 && x4 + 4 <= W - 2 && y >= 2 && y <= H - 3) {
        // interior: every neighbour is an interior cell; rows as float4
        auto D4 = [&](size_t i, float *o) {
          const float4 a = __ldg(reinterpret_cast<const float4 *>(z + i));
          o[0] = a.x - zm;
          o[1] = a.y - zm;
          o[2] = a.z - zm;
          o[3] = a.w - zm;
          if (!first) {
            const float4 b = __ldg(reinterpret_cast<const float4 *>(dold + i));
            o[0] = o[0] + beta * b.x;
            o[1] = o[1] + beta * b.y;
            o[2] = o[2] + beta * b.z;
            o[3] = o[3] + beta * b.w;
          }
        };
        float S4[4], N4[4];
        D4(i0, dc);
        D4(i0 - P, S4);
        D4(i0 + P, N4);
        const float dw = D(i0 - 1), de = D(i0 + 4);
        const uchar4 cv = __ldg(reinterpret_cast<const uchar4 *>(code + i0));
        const float4 rv = __ldg(reinterpret_cast<const float4 *>(r + i0));
        const unsigned C4[4] = {cv.x, cv.y, cv.z, cv.w};
        const float R4[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const unsigned c = C4[j];
          if (!(c & 1u)) continue;
          const float a0 = (c & 2u) ? (j > 0 ? dc[j - 1] : dw) - dc[j] : 0.0f;
          const float a1 = (c & 4u) ? (j < 3 ? dc[j + 1] : de) - dc[j] : 0.0f;
          const float a2 = (c & 8u) ? S4[j] - dc[j] : 0.0f;
          const float a3 = (c & 16u) ? N4[j] - dc[j] : 0.0f;
          qv[j] = -ihsq * sum4(a0, a1, a2, a3);
          dq = __fmaf_rn(dc[j], qv[j], dq);
          dr = __fmaf_rn(dc[j], R4[j], dr);
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (!(C4[j] & 1u)) dc[j] = 0.0f;
      } else {
#pragma unroll
        for (int j = 0; j < 4; j++) dc[j] = (x4 + j < W) ? D(i0 + j) : 0.0f;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int x = x4 + j;
          if (x >= W || !interior(x, y, W, H)) continue;
          const size_t i = i0 + j;
          const unsigned c = __ldg(code + i);
          if (!(c & 1u)) continue;
          const float a0 = ((c & 2u) && x - 1 >= 1) ? (j > 0 ? dc[j - 1] : D(i - 1)) - dc[j] : 0.0f;
          const float a1 = ((c & 4u) && x + 1 < W - 1) ? (j < 3 ? dc[j + 1] : D(i + 1)) - dc[j] : 0.0f;
          const float a2 = ((c & 8u) && y - 1 >= 1) ? D(i - P) - dc[j] : 0.0f;
          const float a3 = ((c & 16u) && y + 1 < H - 1) ? D(i + P) - dc[j] : 0.0f;
          qv[j] = -ihsq * sum4(a0, a1, a2, a3);
          dq = __fmaf_rn(dc[j], qv[j], dq);
          dr = __fmaf_rn(dc[j], __ldg(r + i), dr);
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (x4 + j < W && interior(x4 + j, y, W, H) && !(__ldg(code + i0 + j) & 1u)) dc[j] = 0.0f;
      }
      if (x4 + 3 < W) {
        *reinterpret_cast<float4 *>(dnew + i0) = make_float4(dc[0], dc[1], dc[2], dc[3]);
        *reinterpret_cast<float4 *>(q + i0) = make_float4(qv[0], qv[1], qv[2], qv[3]);
      } else {
        for (int j = 0; j < 4 && x4 + j < W; j++) {
          dnew[i0 + j] = dc[j];
          q[i0 + j] = qv[j];
        }
      }
    }
  }
  double v[2] = {(double)dq, (double)dr};
  double *const dst[2] = {&sc->dq[slot], &sc->dr};
  block_reduce<2>(v, 0u, dst, nullptr, pr);
}

// alpha = dr / dq; x += alpha d (double-float, the product exact); r -=
// alpha q; ||r||^2 and max|r|; zeroes the accumulator of the next k_fcg_zq.
__global__ void __launch_bounds__(BX *BY) k_fcg_update(float *xh, float *xl,
                                                       const float *__restrict__ d, float *r,
                                                       const float *__restrict__ q, int W, int H,
                                                       int P, FcgScalars *sc, int slot,
                                                       FcgPartials *pr) {
  griddep_wait();
  const double dqv = sc->dq[slot];
  const float af = (float)(dqv != 0.0 ? sc->dr / dqv : 0.0);
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) sc->zq = 0.0;
  float rr = 0.0f;
  unsigned mx = 0;
  const int tiles_x = (W + 4 * BX - 1) / (4 * BX), ntiles = tiles_x * ((H + BY - 1) / BY);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int x4 = ((t % tiles_x) * BX + threadIdx.x) * 4, y = (t / tiles_x) * BY + threadIdx.y;
    if (x4 >= W || y >= H) continue;
    const size_t i0 = (size_t)y * P + x4;
    if (x4 + 3 < W) {
      const float4 dv = *reinterpret_cast<const float4 *>(d + i0);
      const float4 qv = *reinterpret_cast<const float4 *>(q + i0);
      float4 rv = *reinterpret_cast<const float4 *>(r + i0);
      float4 h4 = *reinterpret_cast<const float4 *>(xh + i0);
      float4 l4 = *reinterpret_cast<const float4 *>(xl + i0);
      df_axpy(h4.x, l4.x, af, dv.x);
      df_axpy(h4.y, l4.y, af, dv.y);
      df_axpy(h4.z, l4.z, af, dv.z);
      df_axpy(h4.w, l4.w, af, dv.w);
      *reinterpret_cast<float4 *>(xh + i0) = h4;
      *reinterpret_cast<float4 *>(xl + i0) = l4;
      rv.x -= af * qv.x;
      rv.y -= af * qv.y;
      rv.z -= af * qv.z;
      rv.w -= af * qv.w;
      *reinterpret_cast<float4 *>(r + i0) = rv;
      const float R[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        rr = __fmaf_rn(R[j], R[j], rr);
        mx = max(mx, __float_as_uint(fabsf(R[j])));
      }
    } else {
      for (int j = 0; j < 4 && x4 + j < W; j++) {
        const size_t i = i0 + j;
        float hh = xh[i], ll = xl[i];
        df_axpy(hh, ll, af, d[i]);
        xh[i] = hh;
        xl[i] = ll;
        const float rj = r[i] - af * q[i];
        r[i] = rj;
        rr = __fmaf_rn(rj, rj, rr);
        mx = max(mx, __float_as_uint(fabsf(rj)));
      }
    }
  }
  double v[1] = {(double)rr};
  double *const dst[1] = {&sc->rr};
  block_reduce<1>(v, mx, dst, &sc->maxbits, pr);
}

// x = p on every cell (warm start from the current pressure; tail 0).
__global__ void __launch_bounds__(BX *BY) k_fcg_load(const float *__restrict__ p, float *xh,
                                                     float *xl, int W, int H, int P) {
  griddep_wait();
  const int x4 = (blockIdx.x * BX + threadIdx.x) * 4, y = blockIdx.y * BY + threadIdx.y;
  if (x4 >= W || y >= H) return;
  const size_t i = (size_t)y * P + x4;
  if (x4 + 3 < W) {
    *reinterpret_cast<float4 *>(xh + i) = __ldg(reinterpret_cast<const float4 *>(p + i));
    *reinterpret_cast<float4 *>(xl + i) = make_float4(0.f, 0.f, 0.f, 0.f);
  } else {
    for (int j = 0; j < 4 && x4 + j < W; j++) {
      xh[i + j] = p[i + j];
      xl[i + j] = 0.0f;
    }
  }
}

// p = xh + xl (rounded) on the interior cells (the edges are set by setPBC
// next).
__global__ void __launch_bounds__(BX *BY) k_fcg_store(const float *__restrict__ xh,
                                                      const float *__restrict__ xl, float *p,
                                                      int W, int H, int P) {
  griddep_wait();
  const int x4 = (blockIdx.x * BX + threadIdx.x) * 4, y = blockIdx.y * BY + threadIdx.y;
  if (y < 1 || y >= H - 1) return;
  const size_t i = (size_t)y * P + x4;
  for (int j = 0; j < 4; j++) {
    const int x = x4 + j;
    if (x >= 1 && x < W - 1) p[i + j] = xh[i + j] + xl[i + j];
  }
}

// The pressure-gradient update (simulation.cpp:196-207) from the
// double-float pressure: vx -= ih * dp on the faces whose two cells are
// fluid, x in [1, W-3], with dp = x(x+1) - x(x) in double-float rounded
// once; vy likewise, y in [1, H-3].  max|u| of the interior faces in range
// is folded into *umax_bits.
__global__ void __launch_bounds__(BX *BY) k_gradient_df(float *vx, float *vy,
                                                        const uint8_t *__restrict__ cx,
                                                        const uint8_t *__restrict__ cy,
                                                        const float *__restrict__ xh,
                                                        const float *__restrict__ xl, int W, int H,
                                                        int P, const StepScalars *__restrict__ sc,
                                                        unsigned *umax_bits) {
  griddep_wait();
  const int x4 = (blockIdx.x * BX + threadIdx.x) * 4, y = blockIdx.y * BY + threadIdx.y;
  float m = 0.0f;
  auto dp = [&](size_t a, size_t b) {
    float tail;
    const float head = df_diff(__ldg(xh + a), __ldg(xl + a), __ldg(xh + b), __ldg(xl + b), &tail);
    return head + tail;
  };
  if (y >= 1 && y < H - 1) {
    const float ih = sc->ih;
    for (int j = 0; j < 4; j++) {
      const int x = x4 + j;
      const size_t i = (size_t)y * P + x;
      if (x >= 1 && x <= W - 3) {
        float u = vx[i];
        if (__ldg(cx + i) & FC_M) u = u - ih * dp(i + 1, i);
        vx[i] = u;
        m = fmaxf(m, fabsf(u));
      }
      if (x >= 1 && x <= W - 2 && y <= H - 3) {
        float w = vy[i];
        if (__ldg(cy + i) & FC_M) w = w - ih * dp(i + P, i);
        vy[i] = w;
        m = fmaxf(m, fabsf(w));
      }
    }
  }
  if (umax_bits) {
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float red[BY];
    const int tid = threadIdx.y * BX + threadIdx.x;
    if ((tid & 31) == 0) red[tid >> 5] = m;
    __syncthreads();
    if (tid == 0) {
      for (int k = 1; k < BY; k++) m = fmaxf(m, red[k]);
      atomicMax(umax_bits, __float_as_uint(m));
    }
  }
}

size_t a256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

void fcg_alloc(FcgSolver &fs, int W, int H, int P, float h) {
  fcg_free(fs);
  ext_hier_alloc(fs.mg, W, H, h);
  size_t n = (size_t)P * H;
  size_t total = a256(sizeof(FcgScalars)) + a256(sizeof(FcgPartials)) + 5 * a256(n * 4);
  void *arena = nullptr;
  if (cudaMalloc(&arena, total) != cudaSuccess) {
    cudaGetLastError();
    fcg_free(fs);
    throw std::bad_alloc();
  }
  UBG_CUDA(cudaMemsetAsync(arena, 0, total, cudaStreamLegacy));
  UBG_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
  void *host = nullptr;
  if (cudaHostAlloc(&host, sizeof(FcgScalars), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(arena);
    fcg_free(fs);
    throw std::bad_alloc();
  }
  char *p = (char *)arena;
  fs.dev = (FcgScalars *)p;
  p += a256(sizeof(FcgScalars));
  fs.part = (FcgPartials *)p;
  p += a256(sizeof(FcgPartials));
  fs.xh = (float *)p;
  p += a256(n * 4);
  fs.xl = (float *)p;
  p += a256(n * 4);
  fs.d[0] = (float *)p;
  p += a256(n * 4);
  fs.d[1] = (float *)p;
  p += a256(n * 4);
  fs.q = (float *)p;
  fs.arena = arena;
  fs.host = (FcgScalars *)host;
  fs.W = W;
  fs.H = H;
  fs.P = P;
  fs.h = h;
  fs.dirty = true;
  fs.prec = UBG_FP32;
}

void fcg_free(FcgSolver &fs) {
  mg_low_free(fs.lo);
  mg_free(fs.mg);
  fs.mg = MgHier{};
  if (fs.arena) cudaFree(fs.arena);
  if (fs.host) cudaFreeHost(fs.host);
  fs.arena = nullptr;
  fs.host = nullptr;
  fs.dev = nullptr;
  fs.part = nullptr;
  fs.xh = fs.xl = nullptr;
  fs.d[0] = fs.d[1] = fs.q = nullptr;
}

size_t fcg_bytes(int W, int H, int P, int prec) {
  size_t n = (size_t)P * H;
  size_t b = ext_hier_bytes(W, H) + a256(sizeof(FcgScalars)) + a256(sizeof(FcgPartials)) +
             5 * a256(n * 4);
  if (prec != UBG_FP32) b += b / 2;  // 16-bit copies of the hierarchy's arrays (upper bound)
  return b;
}

void fcg_set_precision(FcgSolver &fs, int prec) {
  if (prec == fs.prec && (prec == UBG_FP32 || fs.lo.levels == fs.mg.levels)) return;
  if (prec == UBG_FP32)
    mg_low_free(fs.lo);
  else
    mg_low_alloc(fs.lo, fs.mg, prec);
  fs.prec = prec;
}

int fcg_solve(FcgSolver &fs, const uint8_t *flag, const float *f, float *p, double tol,
              int max_iter, double *rel, cudaStream_t st) {
  const int W = fs.W, H = fs.H, P = fs.P;
  MgHier &mg = fs.mg;
  MgLevel &L0 = mg.lv[0];
  if (fs.dirty) {
    ext_hier_update_fields(mg, flag, P, st);
    fs.dirty = false;
  }
  const float ihsq = 1.0f / fs.h / fs.h;
  const dim3 grid((W + 4 * BX - 1) / (4 * BX), (H + BY - 1) / BY), blk(BX, BY);
  // the reducing kernels: grid-stride, one wave of resident blocks each
  int dev = 0, nsm = 0;
  UBG_CUDA(cudaGetDevice(&dev));
  UBG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  auto wave = [&](auto kern) {
    int per_sm = 0;
    UBG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BX * BY, 0));
    long long n = std::min<long long>((long long)grid.x * grid.y, (long long)std::max(1, per_sm) * nsm);
    return dim3((unsigned)std::min<long long>(n, kFcgMaxBlocks));
  };
  const dim3 g_fsum = wave(k_fcg_fsum), g_resid = wave(k_fcg_resid), g_zq = wave(k_fcg_zq),
             g_zsum = wave(k_fcg_zsum),
             g_dir = wave(k_fcg_dir), g_update = wave(k_fcg_update);
  float *r = L0.rhs;  // the V-cycle's level-0 right-hand side is the residual
  UBG_CUDA(cudaMemsetAsync(fs.dev, 0, sizeof(FcgScalars), st));
  {
    ProfScope ps_(KC_KRYLOV, st);
    k_fcg_load<<<grid, blk, 0, st>>>(p, fs.xh, fs.xl, W, H, P);
  }
  UBG_LAUNCH_CHECK();
  {
    ProfScope ps_(KC_KRYLOV, st);
    k_fcg_fsum<<<g_fsum, blk, 0, st>>>(f, L0.code, W, H, P, fs.dev, fs.part);
  }
  UBG_LAUNCH_CHECK();
  {
    ProfScope ps_(KC_KRYLOV, st);
    k_fcg_resid<<<g_resid, blk, 0, st>>>(fs.xh, fs.xl, f, L0.code, W, H, P, ihsq, r, fs.dev, 1,
                                       fs.part);
  }
  UBG_LAUNCH_CHECK();
  g_stats.launches += 3;
  auto read = [&]() {
    UBG_CUDA(cudaMemcpyAsync(fs.host, fs.dev, sizeof(FcgScalars), cudaMemcpyDeviceToHost, st));
    UBG_CUDA(cudaStreamSynchronize(st));
  };
  read();
  const double ff = fs.host->ff, target2 = tol * tol * ff;
  // The recurrence r -= alpha q drifts from f_c + L x by FP32 rounding; when
  // it meets the tolerance, r is recomputed from x (residual replacement)
  // and, if that misses the tolerance, the iteration restarts from it.  A
  // replacement that finds the residual not at least halved since the last
  // one ends the solve: the tolerance is below what the FP32 vectors
  // resolve.
  // A solve that ends above the residual it started from (the iteration
  // diverged: 16-bit coarse levels too coarse in precision for the grid,
  // BF16 at 8192 x 4096) keeps its starting pressure instead; a recurrence
  // residual 100 times the starting one ends it early.
  double rr = fs.host->rr, last_true = rr;
  const double start_rr = rr;
  bool diverged = false;
  bool fresh = true, first = true;
  int it = 0, cur_d = 0;
  auto replace_residual = [&]() {
    UBG_CUDA(cudaMemsetAsync(&fs.dev->rr, 0, sizeof(double), st));
    UBG_CUDA(cudaMemsetAsync(&fs.dev->maxbits, 0, sizeof(unsigned), st));
    {
      ProfScope ps_(KC_KRYLOV, st);
      k_fcg_resid<<<g_resid, blk, 0, st>>>(fs.xh, fs.xl, f, L0.code, W, H, P, ihsq, r, fs.dev, 0,
                                         fs.part);
    }
    UBG_LAUNCH_CHECK();
    g_stats.launches++;
    read();
    rr = fs.host->rr;
    fresh = true;
    first = true;
  };
  for (;;) {
    if (!std::isfinite(rr)) throw CudaError("tolerance solver: non-finite residual");
    if (rr <= target2) {
      if (fresh) break;
      replace_residual();
      if (rr > 0.25 * last_true) break;
      last_true = rr;
      continue;
    }
    if (it >= max_iter) {
      if (!fresh) replace_residual();
      break;
    }
    ext_vcycle(mg, fs.prec == UBG_FP32 ? nullptr : &fs.lo, fs.prec, &fs.dev->maxbits, st);
    const float *z = L0.e[mg.cur0];
    const int slot = it & 1;
    {
      ProfScope ps_(KC_KRYLOV, st);
      k_fcg_zsum<<<g_zsum, blk, 0, st>>>(z, L0.code, W, H, P, fs.dev, fs.part);
    }
    UBG_LAUNCH_CHECK();
    g_stats.launches++;
    if (it > 0) {  // (also zeroes the accumulators of k_fcg_dir)
      {
        ProfScope ps_(KC_KRYLOV, st);
        k_fcg_zq<<<g_zq, blk, 0, st>>>(z, fs.q, W, H, P, fs.dev, slot, fs.part);
      }
      UBG_LAUNCH_CHECK();
      g_stats.launches++;
    }
    {
      ProfScope ps_(KC_KRYLOV, st);
      k_fcg_dir<<<g_dir, blk, 0, st>>>(z, fs.d[cur_d], fs.d[cur_d ^ 1], fs.q, r, L0.code, W, H, P,
                                      ihsq, fs.dev, first ? 1 : 0, slot, fs.part);
    }
    UBG_LAUNCH_CHECK();
    cur_d ^= 1;
    {
      ProfScope ps_(KC_KRYLOV, st);
      k_fcg_update<<<g_update, blk, 0, st>>>(fs.xh, fs.xl, fs.d[cur_d], r, fs.q, W, H, P, fs.dev, slot,
                                            fs.part);
    }
    UBG_LAUNCH_CHECK();
    g_stats.launches += 2;
    it++;
    first = false;
    fresh = false;
    read();
    rr = fs.host->rr;
    if (rr > 1.0e4 * start_rr) {
      diverged = true;
      break;
    }
  }
  if (diverged || rr > start_rr) {
    {
      ProfScope ps_(KC_KRYLOV, st);
      k_fcg_load<<<grid, blk, 0, st>>>(p, fs.xh, fs.xl, W, H, P);
    }
    UBG_LAUNCH_CHECK();
    g_stats.launches++;
    rr = start_rr;
  } else {
    {
      ProfScope ps_(KC_KRYLOV, st);
      k_fcg_store<<<grid, blk, 0, st>>>(fs.xh, fs.xl, p, W, H, P);
    }
    UBG_LAUNCH_CHECK();
    g_stats.launches++;
  }
  if (rel) *rel = std::sqrt(rr / (ff > 0.0 ? ff : 1.0));
  return it;
}

void launch_gradient_df(const VelBufs &v, int fx, int fy, const float *xh, const float *xl,
                        const StepScalars *sc, unsigned *umax_bits, cudaStream_t st) {
  ProfScope ps_(KC_GRADIENT, st);
  const dim3 grid((v.W + 4 * BX - 1) / (4 * BX), (v.H + BY - 1) / BY);
  k_gradient_df<<<grid, dim3(BX, BY), 0, st>>>(fx ? v.vx[1] : v.vx[0], fy ? v.vy[1] : v.vy[0], v.cx,
                                                v.cy, xh, xl, v.W, v.H, v.pitch, sc, umax_bits);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

}  // namespace ubg
