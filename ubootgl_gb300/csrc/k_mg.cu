// Multigrid pressure solver (class MG, pressure_solver.{hpp,cpp} of
// te42kyfo/ubootgl) on the GPU.
//
//  k_mg        red-black Gauss-Seidel (rbgs + smoothingKernel,
//              pressure_solver.cpp:10-24, 35-89), up to 5 sweeps temporally
//              blocked in shared memory, with an optional prologue
//              (prolongate + correct, pressure_solver.cpp:134-181), the
//              zero-gradient boundary after every sweep on level 0
//              (setZeroGradientBC, pressure_solver.cpp:183-192), and an
//              optional epilogue that computes the residual and restricts it
//              to the next level (calculateResidualField + restrict,
//              pressure_solver.cpp:91-132) without writing the fine residual.
//  k_mg_tail   the coarse end of the V-cycle in one CTA, in shared memory.
//  k_mg_ctail  the coarse end from a larger level down in one launch of a
//              16-CTA cluster: row bands with ghost rows exchanged through
//              distributed shared memory, the tail's levels in CTA 0.
//  k_residual  the residual field and its squared L2 norm.
//  k_coarsen   MG::updateFields (pressure_solver.hpp:34-57), integer exact.
//
// Red points are those with x+y odd (pressure_solver.cpp:36); a sweep updates
// all red points, then all black points, which is the reference's
// deterministic schedule.  Every kernel reads one buffer and writes another,
// so tiles never race on their halos.
#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "ubg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>

#define ALPHA_IS_ONE(a) ((a) == 1.0f)

namespace ubg {
namespace {

// Per-cell stencil code of a level: bit 0 = the cell's flag, bits 1..4 = the
// flags of its west, east, south (y-1) and north (y+1) neighbours (0 on the
// domain boundary, whose cells are never smoothed).
constexpr unsigned C_CENTER = 1, C_W = 2, C_E = 4, C_S = 8, C_N = 16;

__global__ void k_make_code(const uint8_t *__restrict__ flag, uint8_t *code, int w, int h,
                            int P) {
  int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  if (x >= w || y >= h) return;
  size_t i = (size_t)y * P + x;
  unsigned c = flag[i] ? C_CENTER : 0u;
  if (x >= 1 && x < w - 1 && y >= 1 && y < h - 1) {
    if (flag[i - 1]) c |= C_W;
    if (flag[i + 1]) c |= C_E;
    if (flag[i - P]) c |= C_S;
    if (flag[i + P]) c |= C_N;
  }
  code[i] = (uint8_t)c;
}

// smoothingKernel (pressure_solver.cpp:10-24) for alpha = 1.  With flags in
// {0, 1}, p*flag inside the sum equals flag ? p : 0 (the running sum starts
// at +0 and never becomes -0), val/sum is exact as a multiplication for
// sum = 1, 2, 4 and a true division for sum = 3, and flag*val equals
// flag ? val : 0 up to the sign of a zero.
// x / 3 (correctly rounded either way)
__device__ __forceinline__ float div3(float x) { return div_rn(x, 3.0f, 1.0f / 3.0f); }
__device__ __forceinline__ double div3(double x) { return x / 3.0; }

// T = float is the reference's arithmetic; T = double serves the FP64
// coarse solve of the mixed-precision solver.
template <class T>
__device__ __forceinline__ T rb_update1(unsigned c, T pw, T pe, T ps, T pn, T f, T hh) {
  T val = T(0);
  val = val + ((c & C_W) ? pw : T(0));
  val = val + ((c & C_E) ? pe : T(0));
  val = val + ((c & C_S) ? ps : T(0));
  val = val + ((c & C_N) ? pn : T(0));
  val = val + f * hh * hh;
  int s = __popc((c >> 1) & 15u);
  if (s == 3)
    val = div3(val);
  else
    val = val * (s == 4 ? T(0.25) : (s == 2 ? T(0.5) : (s == 1 ? T(1) : T(0))));
  if (s == 0) val = T(0);
  return (c & C_CENTER) ? val : T(0);
}

// General alpha (the free function rbgs(p, f, flag, h, alpha)).
__device__ __forceinline__ float rb_update_alpha(unsigned c, float pc, float pw, float pe,
                                                 float ps, float pn, float f, float hh,
                                                 float alpha) {
  float fw = (c & C_W) ? 1.0f : 0.0f, fe = (c & C_E) ? 1.0f : 0.0f;
  float fs = (c & C_S) ? 1.0f : 0.0f, fn = (c & C_N) ? 1.0f : 0.0f;
  float sum = 0.0f;
  sum = sum + (fw + fe + fn + fs);
  float val = 0.0f;
  val = val + pw * fw;
  val = val + pe * fe;
  val = val + ps * fs;
  val = val + pn * fn;
  val = val + f * hh * hh;
  val = val / sum;
  if (sum == 0.0f) val = 0.0f;
  return ((c & C_CENTER) ? 1.0f : 0.0f) * (alpha * val + (1.0f - alpha) * pc);
}

// calculateResidualField at one cell (pressure_solver.cpp:100-110): a
// neighbour term p_n*flag_n + p*(1-flag_n) is flag_n ? p_n : p.
template <class T>
__device__ __forceinline__ T resid1(unsigned c, T pc, T pw, T pe, T ps, T pn, T f, T ihsq) {
  T val = T(0);
  val = val + ((c & C_W) ? pw : pc);
  val = val + ((c & C_E) ? pe : pc);
  val = val + ((c & C_S) ? ps : pc);
  val = val + ((c & C_N) ? pn : pc);
  val = val + T(-4) * pc;
  val = val * ihsq;
  return (c & C_CENTER) ? (f + val) : T(0);
}

// Storage of the smoothed arrays: float (the reference's arithmetic, and the
// only type whose results are compared bit for bit) or __half /
// __nv_bfloat16 for the low-precision correction V-cycle of the mixed
// solver.  Arithmetic is always FP32 in registers.
template <class S>
struct Sto;
template <>
struct Sto<float> {
  static __device__ __forceinline__ float4 ldg4(const float *p) {
    return __ldg(reinterpret_cast<const float4 *>(p));
  }
  static __device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
  static __device__ __forceinline__ float4 lds4(const float *p) {
    return *reinterpret_cast<const float4 *>(p);
  }
  static __device__ __forceinline__ void sts4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
  static __device__ __forceinline__ float2 lds2(const float *p) {
    return *reinterpret_cast<const float2 *>(p);
  }
  static __device__ __forceinline__ void sts2(float *p, float a, float b) {
    *reinterpret_cast<float2 *>(p) = make_float2(a, b);
  }
  static __device__ __forceinline__ float tof(float v) { return v; }
  static __device__ __forceinline__ float fromf(float v) { return v; }
  static __device__ __forceinline__ float ldg1(const float *p) { return __ldg(p); }
};
template <>
struct Sto<__half> {
  static __device__ __forceinline__ float4 unpack(uint2 u) {
    float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&u.x));
    float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
  }
  static __device__ __forceinline__ uint2 pack(float4 v) {
    __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
    return make_uint2(*reinterpret_cast<unsigned *>(&a), *reinterpret_cast<unsigned *>(&b));
  }
  static __device__ __forceinline__ float4 ldg4(const __half *p) {
    return unpack(__ldg(reinterpret_cast<const uint2 *>(p)));
  }
  static __device__ __forceinline__ void st4(__half *p, float4 v) { *reinterpret_cast<uint2 *>(p) = pack(v); }
  static __device__ __forceinline__ float4 lds4(const __half *p) {
    return unpack(*reinterpret_cast<const uint2 *>(p));
  }
  static __device__ __forceinline__ void sts4(__half *p, float4 v) { *reinterpret_cast<uint2 *>(p) = pack(v); }
  static __device__ __forceinline__ float2 lds2(const __half *p) {
    return __half22float2(*reinterpret_cast<const __half2 *>(p));
  }
  static __device__ __forceinline__ void sts2(__half *p, float a, float b) {
    *reinterpret_cast<__half2 *>(p) = __floats2half2_rn(a, b);
  }
  static __device__ __forceinline__ float tof(__half v) { return __half2float(v); }
  static __device__ __forceinline__ __half fromf(float v) { return __float2half_rn(v); }
  static __device__ __forceinline__ float ldg1(const __half *p) { return __half2float(__ldg(p)); }
};
template <>
struct Sto<__nv_bfloat16> {
  static __device__ __forceinline__ float4 unpack(uint2 u) {
    float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u.x));
    float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
  }
  static __device__ __forceinline__ uint2 pack(float4 v) {
    __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y), b = __floats2bfloat162_rn(v.z, v.w);
    return make_uint2(*reinterpret_cast<unsigned *>(&a), *reinterpret_cast<unsigned *>(&b));
  }
  static __device__ __forceinline__ float4 ldg4(const __nv_bfloat16 *p) {
    return unpack(__ldg(reinterpret_cast<const uint2 *>(p)));
  }
  static __device__ __forceinline__ void st4(__nv_bfloat16 *p, float4 v) {
    *reinterpret_cast<uint2 *>(p) = pack(v);
  }
  static __device__ __forceinline__ float4 lds4(const __nv_bfloat16 *p) {
    return unpack(*reinterpret_cast<const uint2 *>(p));
  }
  static __device__ __forceinline__ void sts4(__nv_bfloat16 *p, float4 v) {
    *reinterpret_cast<uint2 *>(p) = pack(v);
  }
  static __device__ __forceinline__ float2 lds2(const __nv_bfloat16 *p) {
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(p));
  }
  static __device__ __forceinline__ void sts2(__nv_bfloat16 *p, float a, float b) {
    *reinterpret_cast<__nv_bfloat162 *>(p) = __floats2bfloat162_rn(a, b);
  }
  static __device__ __forceinline__ float tof(__nv_bfloat16 v) { return __bfloat162float(v); }
  static __device__ __forceinline__ __nv_bfloat16 fromf(float v) { return __float2bfloat16_rn(v); }
  static __device__ __forceinline__ float ldg1(const __nv_bfloat16 *p) {
    return __bfloat162float(__ldg(p));
  }
};

// S: storage of the level's own arrays (in, out, rhs); SC: storage of the
// next coarser level's arrays that the launch reads (ec) or writes (rc).
template <class S, class SC = S>
struct MgArgsT {
  const S *in;
  S *out;
  const S *rhs;
  const uint8_t *code;
  int w, h, pitch;
  float hh, alpha, ihsq;
  int nsweeps, zgbc, zero_init;
  // prologue: p += prolongate(ec) (post-smoothing)
  const SC *ec;
  const uint8_t *codec;
  int cpitch;
  float wsum[5];   // (float)((double)k + 0.0001)
  float rwsum[5];  // RN(1 / wsum[k]), for div_rn
  // epilogue: rc = restrict(residual) (pre-smoothing)
  SC *rc;
  int cw, ch;
  float rfac;  // restriction weight: 1/16 (reference), 1/16 * (hc/h)^2 (scaled form)
  int tile;    // smoother tile id (-1: by level width), host side only
  // epilogue: sum of r^2 over the tile's interior cells
  double *norm2;
  // Tolerance-solver hierarchy (ext != 0): zero-gradient edges on every
  // level include the four corner cells, and the prolongation has no
  // zero columns / rows at the east and north ends (the coarse edges there
  // are zero-gradient copies, not zeros).
  int ext;
  // Scaled 16-bit coarse levels below an FP32 level (scale_bits != null):
  // s = 2^-(e + scale_kexp) with max|rhs| * scale_h1sq = m 2^e, m in
  // [0.5, 1) (max|rhs| as float bits on the device); the restriction
  // writes rfac * s * scale_h1sq * (...) and the prolongation adds e_c / s.
  const unsigned *scale_bits;
  float scale_h1sq;
  int scale_kexp;
};
using MgArgs = MgArgsT<float>;

// Scale of the 16-bit coarse levels from max|r| (float bits): returns s and
// sets *inv = 1 / s (both powers of two; 0 when r is zero).
__device__ __forceinline__ float coarse_scale(const unsigned *bits, float h1sq, int kexp,
                                              float *inv) {
  const float m = __uint_as_float(*bits) * h1sq;
  if (!(m > 0.0f)) {
    *inv = 0.0f;
    return 0.0f;
  }
  int ex;
  frexpf(m, &ex);
  *inv = ldexpf(1.0f, ex + kexp);
  return ldexpf(1.0f, -ex - kexp);
}

template <int TX, int TY, int HALO>
struct Tile {
  static constexpr int RX = TX + 2 * HALO, RY = TY + 2 * HALO, HX = RX / 2;
  // coarse window for the prolongation prologue (rows padded to a multiple
  // of 4 entries for vector access)
  static constexpr int CW = HX + 4, CH = RY / 2 + 2;
  static_assert(RX % 4 == 0 && HALO % 4 == 0 && TX % 4 == 0 && TY % 2 == 0, "tile alignment");
  // shared memory for element size ES: p and f in the split layout, codes,
  // the coarse window (values of element size ESC, and flags)
  static constexpr size_t smem(size_t ES = 4, size_t ESC = 0) {
    return (size_t)2 * RY * HX * (2 * ES + 1) +
           (((size_t)CW * CH * (ESC ? ESC : ES) + 15) / 16 * 16) + ((size_t)CW * CH + 15) / 16 * 16;
  }
};

// One multigrid smoothing launch on a tile of TX x TY cells with a halo of
// HALO cells, all in shared memory in a red/black-split layout: cell (rx, ry)
// of the region lives in colour array (rx+ry)&1 at [ry][rx/2], so the four
// neighbours of a cell are consecutive entries of the other colour's rows
// (no bank conflicts).  Red = (x+y) odd; region parity equals global parity
// because x0 + y0 is even.  After half sweep i only cells within HALO - i of
// the tile are still exact, so each half sweep updates just that cone.
// EXT: the tolerance hierarchy's rules (a.ext, a.scale_bits) compiled in;
// the reference's path is built without them.
template <int TX, int TY, int HALO, bool ALPHA1, int NT, class S, class SC, bool EXT = false>
__device__ __forceinline__ void k_mg_body(const MgArgsT<S, SC> &a, const int bx, const int by) {
  constexpr int NTY = NT / 32;
  using T = Tile<TX, TY, HALO>;
  using St = Sto<S>;
  using Sc = Sto<SC>;
  constexpr int RX = T::RX, RY = T::RY, HX = T::HX;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S *sp = reinterpret_cast<S *>(smem_raw);  // [2][RY][HX]
  S *sf = sp + 2 * RY * HX;
  uint8_t *sc = reinterpret_cast<uint8_t *>(sf + 2 * RY * HX);
  auto IDX = [](int rx, int ry) { return (((rx + ry) & 1) * RY + ry) * HX + (rx >> 1); };

  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  const int x0 = bx * TX - HALO, y0 = by * TY - HALO;
  const int w = a.w, h = a.h, P = a.pitch;

  // ---- load p, f, code: 8 consecutive cells per thread and item (two
  // float4 / two uchar4 loads; x0 is a multiple of 4), stored as 4 cells of
  // each colour (one 128-bit store per colour, codes one 32-bit store).
  // One array at a time, all of a thread's loads of that array in flight
  // together, into the red/black-split layout.
  static_assert(RX % 8 == 0, "8-cell load groups");
  constexpr int NQ = RY * (RX / 8), NIT = (NQ + NT - 1) / NT;
  using Items = float4[NIT][2];
  auto load_issue = [&](const S *src, bool zero, Items &v) {
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int q = tid + it * NT;
      const int ry = q / (RX / 8), g = q - ry * (RX / 8);
      const int gx = x0 + 8 * g, gy = y0 + ry;
      const bool row = !zero && q < NQ && gy >= 0 && gy < h;
#pragma unroll
      for (int hf = 0; hf < 2; hf++) {
        const int x = gx + 4 * hf;
        v[it][hf] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (row && x >= 0 && x < w) v[it][hf] = St::ldg4(src + (size_t)gy * P + x);
      }
    }
  };
  auto load_store = [&](S *dst, const Items &v) {
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int q = tid + it * NT;
      if (q >= NQ) break;
      const int ry = q / (RX / 8), g = q - ry * (RX / 8);
      const int gx = x0 + 8 * g;
      float c[8] = {v[it][0].x, v[it][0].y, v[it][0].z, v[it][0].w,
                    v[it][1].x, v[it][1].y, v[it][1].z, v[it][1].w};
      if (gx + 7 >= w) {  // cells at and beyond the grid's width are 0
#pragma unroll
        for (int i = 1; i < 8; i++)
          if (gx + i >= w) c[i] = 0.f;
      }
      const int c0 = ry & 1;
      St::sts4(dst + (c0 * RY + ry) * HX + 4 * g, make_float4(c[0], c[2], c[4], c[6]));
      St::sts4(dst + ((c0 ^ 1) * RY + ry) * HX + 4 * g, make_float4(c[1], c[3], c[5], c[7]));
    }
  };
  {
    Items vp;
    load_issue(a.in, a.zero_init != 0, vp);
    load_store(sp, vp);
  }
  {
    // f, the codes and the coarse window: all loads in flight together
    Items vf;
    load_issue(a.rhs, false, vf);
    unsigned cv[NIT][2];
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int q = tid + it * NT;
      const int ry = q / (RX / 8), g = q - ry * (RX / 8);
      const int gx = x0 + 8 * g, gy = y0 + ry;
      const bool row = q < NQ && gy >= 0 && gy < h;
#pragma unroll
      for (int hf = 0; hf < 2; hf++) {
        const int x = gx + 4 * hf;
        cv[it][hf] = 0u;
        if (row && x >= 0 && x < w)
          cv[it][hf] = __ldg(reinterpret_cast<const unsigned *>(a.code + (size_t)gy * P + x));
      }
    }
    // coarse window of the prolongation prologue (post-smoothing): loaded
    // while the code loads are in flight, stored before the same barrier
    if (a.ec) {
      constexpr int CW = T::CW, CH = T::CH;
      SC *sec = reinterpret_cast<SC *>(sc + 2 * RY * HX);
      uint8_t *scf = reinterpret_cast<uint8_t *>(sc + 2 * RY * HX) +
                     ((size_t)CW * CH * sizeof(SC) + 15) / 16 * 16;
      const int cxa = x0 >> 1, cya = y0 >> 1;
      // all of a thread's loads in flight together, then the stores
      if constexpr (HALO % 8 == 0) {
        // cxa is a multiple of 4: 4 coarse entries per load (value and flag)
        constexpr int CQ4 = (CW / 4) * CH, CIT = (CQ4 + NT - 1) / NT;
        static_assert(CW % 4 == 0, "window rows of whole vectors");
        float4 ev[CIT];
        unsigned fv[CIT];
  #pragma unroll
        for (int it = 0; it < CIT; it++) {
          const int q = tid + it * NT;
          const int ly = q / (CW / 4), lx = 4 * (q - ly * (CW / 4));
          const int cx = cxa + lx, cy = cya + ly;
          ev[it] = make_float4(0.f, 0.f, 0.f, 0.f);
          fv[it] = 0u;
          if (q < CQ4 && cx >= 0 && cx < a.cw && cy >= 0 && cy < a.ch) {
            ev[it] = Sc::ldg4(a.ec + (size_t)cy * a.cpitch + cx);
            fv[it] = __ldg(reinterpret_cast<const unsigned *>(a.codec + (size_t)cy * a.cpitch + cx)) &
                     0x01010101u;
            if (cx + 3 >= a.cw) {  // entries at and beyond the level's width are 0
              if (cx + 1 >= a.cw) ev[it].y = 0.f, fv[it] &= 0x000000ffu;
              if (cx + 2 >= a.cw) ev[it].z = 0.f, fv[it] &= 0x0000ffffu;
              ev[it].w = 0.f;
              fv[it] &= 0x00ffffffu;
            }
          }
        }
  #pragma unroll
        for (int it = 0; it < CIT; it++) {
          const int q = tid + it * NT;
          if (q < CQ4) {
            Sc::sts4(sec + 4 * q, ev[it]);
            *reinterpret_cast<unsigned *>(scf + 4 * q) = fv[it];
          }
        }
      } else {
        constexpr int CQ = CW * CH, CIT = (CQ + NT - 1) / NT;
        float ev[CIT];
        uint8_t fv[CIT];
  #pragma unroll
        for (int it = 0; it < CIT; it++) {
          int q = tid + it * NT;
          int ly = q / CW, lx = q - ly * CW;
          int cx = cxa + lx, cy = cya + ly;
          ev[it] = 0.0f;
          fv[it] = 0;
          if (q < CQ && cx >= 0 && cx < a.cw && cy >= 0 && cy < a.ch) {
            ev[it] = Sc::ldg1(a.ec + (size_t)cy * a.cpitch + cx);
            fv[it] = __ldg(a.codec + (size_t)cy * a.cpitch + cx) & 1u;
          }
        }
  #pragma unroll
        for (int it = 0; it < CIT; it++) {
          int q = tid + it * NT;
          if (q < CQ) {
            sec[q] = Sc::fromf(ev[it]);
            scf[q] = fv[it];
          }
        }
      }
    }
    load_store(sf, vf);
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int q = tid + it * NT;
      if (q >= NQ) break;
      const int ry = q / (RX / 8), g = q - ry * (RX / 8);
      const int gx = x0 + 8 * g;
      unsigned lo = cv[it][0], hi = cv[it][1];
      if (gx + 7 >= w) {  // byte i of (lo, hi) is cell gx + i
#pragma unroll
        for (int i = 1; i < 8; i++)
          if (gx + i >= w) {
            if (i < 4)
              lo &= ~(0xffu << (8 * i));
            else
              hi &= ~(0xffu << (8 * (i - 4)));
          }
      }
      // even bytes to the row's colour, odd bytes to the other one
      const unsigned ev = __byte_perm(lo, hi, 0x6420), od = __byte_perm(lo, hi, 0x7531);
      const int c0 = ry & 1;
      *reinterpret_cast<unsigned *>(sc + (c0 * RY + ry) * HX + 4 * g) = ev;
      *reinterpret_cast<unsigned *>(sc + ((c0 ^ 1) * RY + ry) * HX + 4 * g) = od;
    }
  }
  __syncthreads();

  // Row mapping of the vectorised phases: a thread handles 4 consecutive
  // cells of one colour in one row (128-bit shared-memory accesses).  A
  // warp covers 32 entries (k) of 4 rows two apart, 8 lanes per row (each
  // quarter-warp one row: no bank conflicts); its partner warp takes the
  // rows in between.  So a row's parity is the same across a warp and,
  // because a pass covers an even number of rows, fixed for a thread
  // through a pass: parity-dependent choices are warp-uniform.  The compact
  // 4-row footprint also keeps fewer warps straddling obstacle edges (at
  // 4096x2048 with 12 discs: 9 % of warp passes instead of 16 % for 2 rows
  // of 64 entries).
  constexpr int KH = HX / 32, RPP = NT / (HX / 4);
  static_assert(HX % 32 == 0 && (NT / 32) % (2 * KH) == 0, "vector layout");
  const int lane = tid & 31, wid = tid >> 5;
  const int kh = wid % KH, wpar = (wid / KH) & 1;
  const int k0 = 4 * ((lane & 7) + 8 * kh);
  const int rsub = (wid / (2 * KH)) * 8 + wpar + 2 * (lane >> 3);
  // The prolongation prologue measures faster with wide rows: G threads per
  // row, a warp on 32 / G rows two apart, its partner warp between them.
  constexpr int G = HX / 4, RW = 32 / G;
  static_assert(NT % G == 0 && 32 % G == 0, "vector layout");
  const int k0w = 4 * (lane % G);
  const int rsubw = (wid >> 1) * (2 * RW) + (wid & 1) + 2 * (lane / G);

  // ---- prologue: correct(p, prolongate(ec)) on the interior cells, from
  // the coarse window staged with the field loads above
  if (a.ec) {
    constexpr int CW = T::CW, CH = T::CH;
    SC *sec = reinterpret_cast<SC *>(sc + 2 * RY * HX);
    uint8_t *scf = reinterpret_cast<uint8_t *>(sc + 2 * RY * HX) +
                   ((size_t)CW * CH * sizeof(SC) + 15) / 16 * 16;
    // correction scale of scaled 16-bit coarse levels (1 otherwise)
    float ecmul = 1.0f;
    if (EXT && a.scale_bits) coarse_scale(a.scale_bits, a.scale_h1sq, a.scale_kexp, &ecmul);
    const bool ext = EXT && a.ext != 0;
    // prolongate (pressure_solver.cpp:134-172); e * fine flag = e here.
    // Fine cell (rx, ry) = (2k + par, ry) lies over coarse column k of the
    // window and coarse row ry / 2; x parity is par and y parity ry & 1, both
    // fixed across the thread's 4 cells.
#pragma unroll
    for (int color = 0; color < 2; color++) {
      for (int ry = rsubw; ry < RY; ry += RPP) {
        const int par = (ry + color) & 1, yo = ry & 1;
        const int gy = y0 + ry;
        if (gy < 1 || gy >= h - 1) continue;
        const int row = (color * RY + ry) * HX + k0w;
        const unsigned cw4 = *reinterpret_cast<const unsigned *>(sc + row);
        if ((cw4 & 0x01010101u) == 0u) continue;  // no fluid cell among the 4
        const int eo = (ry >> 1) * CW + k0w;
        const float4 ea = Sc::lds4(sec + eo);
        const float E0[5] = {ea.x, ea.y, ea.z, ea.w, Sc::tof(sec[eo + 4])};
        const unsigned fa = *reinterpret_cast<const unsigned *>(scf + eo);
        const unsigned F0[5] = {fa & 0xffu, (fa >> 8) & 0xffu, (fa >> 16) & 0xffu, fa >> 24,
                                scf[eo + 4]};
        float E1[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        unsigned F1[5] = {0u, 0u, 0u, 0u, 0u};
        if (yo) {
          const float4 eb = Sc::lds4(sec + eo + CW);
          E1[0] = eb.x;
          E1[1] = eb.y;
          E1[2] = eb.z;
          E1[3] = eb.w;
          E1[4] = Sc::tof(sec[eo + CW + 4]);
          const unsigned fb = *reinterpret_cast<const unsigned *>(scf + eo + CW);
          F1[0] = fb & 0xffu;
          F1[1] = (fb >> 8) & 0xffu;
          F1[2] = (fb >> 16) & 0xffu;
          F1[3] = fb >> 24;
          F1[4] = scf[eo + CW + 4];
        }
        const float4 pv = St::lds4(sp + row);
        float out[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int gx = x0 + 2 * (k0w + j) + par;
          if (gx < 1 || gx >= w - 1 || !((cw4 >> (8 * j)) & C_CENTER)) continue;
          float pe;
          if (!par && !yo) {
            pe = E0[j];
          } else if (par && !yo) {
            const int k = F0[j] + F0[j + 1];
            pe = (!ext && gx >= w - 2) ? 0.0f : div_rn(E0[j] + E0[j + 1], a.wsum[k], a.rwsum[k]);
          } else if (!par && yo) {
            const int k = F0[j] + F1[j];
            pe = (!ext && gy >= h - 2) ? 0.0f : div_rn(E0[j] + E1[j], a.wsum[k], a.rwsum[k]);
          } else {
            const int k = F0[j] + F1[j + 1] + F0[j + 1] + F1[j];
            pe = (!ext && (gx >= w - 2 || gy >= h - 2))
                     ? 0.0f
                     : div_rn(((E0[j] + E1[j + 1]) + E0[j + 1]) + E1[j], a.wsum[k], a.rwsum[k]);
          }
          if (EXT && a.scale_bits) pe = pe * ecmul;
          out[j] = out[j] + pe;
        }
        St::sts4(sp + row, make_float4(out[0], out[1], out[2], out[3]));
      }
    }
    __syncthreads();
  }

  // setZeroGradientBC on this region (only tiles that touch the domain edge)
  const bool edge = x0 <= 0 || y0 <= 0 || x0 + RX >= w || y0 + RY >= h;
  auto zero_gradient = [&]() {
    for (int q = tid; q < 2 * RY; q += NT) {
      int ry = q >> 1, side = q & 1;
      int gy = y0 + ry;
      if (gy < 1 || gy >= h - 1) continue;
      int rx = side ? (w - 1 - x0) : (0 - x0);
      int rn = side ? rx - 1 : rx + 1;
      if (rx < 0 || rx >= RX || rn < 0 || rn >= RX) continue;
      sp[IDX(rx, ry)] = sp[IDX(rn, ry)];
    }
    for (int q = tid; q < 2 * RX; q += NT) {
      int rx = q >> 1, side = q & 1;
      int gx = x0 + rx;
      if (gx < 1 || gx >= w - 1) continue;
      int ry = side ? (h - 1 - y0) : (0 - y0);
      int rn = side ? ry - 1 : ry + 1;
      if (ry < 0 || ry >= RY || rn < 0 || rn >= RY) continue;
      sp[IDX(rx, ry)] = sp[IDX(rx, rn)];
    }
    if (EXT && a.ext && tid < 4) {  // corner cell <- its diagonal interior neighbour
      const int cxg = (tid & 1) ? w - 1 : 0, cyg = (tid & 2) ? h - 1 : 0;
      const int rx = cxg - x0, ry = cyg - y0;
      const int rnx = rx + ((tid & 1) ? -1 : 1), rny = ry + ((tid & 2) ? -1 : 1);
      if (rx >= 0 && rx < RX && ry >= 0 && ry < RY && rnx >= 0 && rnx < RX && rny >= 0 &&
          rny < RY)
        sp[IDX(rx, ry)] = sp[IDX(rnx, rny)];
    }
  };
  if (a.zgbc && edge && a.ec) {
    zero_gradient();
    __syncthreads();
  }

  // ---- red-black sweeps: a thread updates the 4 cells of its row group
  // (see the row mapping above)
  const float hh = a.hh;
  const bool inner = x0 >= 1 && y0 >= 1 && x0 + RX <= w - 1 && y0 + RY <= h - 1;
  // which of the thread's 4 cells may be smoothed, per row parity: k >= 1 -
  // par and k <= HX - 1 - par keep all neighbours in the region; the column
  // must be inside the domain's interior
  unsigned cmask[2];
#pragma unroll
  for (int par = 0; par < 2; par++) {
    unsigned m = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int k = k0 + j, gx = x0 + 2 * k + par;
      const bool ok = k >= 1 - par && k <= HX - 1 - par && gx >= 1 && gx < w - 1;
      m |= ok ? (1u << j) : 0u;
    }
    cmask[par] = m;
  }
  auto sweep = [&](auto parc, const int color, const int half) {
    constexpr int PAR = decltype(parc)::value;
    S *self = sp + color * RY * HX;
    const S *oth = sp + (color ^ 1) * RY * HX;
    const S *fs = sf + color * RY * HX;
    const uint8_t *cs = sc + color * RY * HX;
    const unsigned cm = cmask[PAR];
    for (int ry = half + rsub; ry <= RY - 1 - half; ry += RPP) {
      if (!inner) {
        const int gy = y0 + ry;
        if (gy < 1 || gy >= h - 1) continue;  // boundary row: kept as it is
      }
      const int row = ry * HX + k0;
      const float4 o = St::lds4(oth + row);
      const float ex = St::tof(PAR ? oth[row + 4] : oth[row - 1]);
      const float4 os = St::lds4(oth + row - HX);
      const float4 on = St::lds4(oth + row + HX);
      const float4 fv = St::lds4(fs + row);
      const unsigned cw = *reinterpret_cast<const unsigned *>(cs + row);
      const float W4[4] = {PAR ? o.x : ex, PAR ? o.y : o.x, PAR ? o.z : o.y, PAR ? o.w : o.z};
      const float E4[4] = {PAR ? o.y : o.x, PAR ? o.z : o.y, PAR ? o.w : o.z, PAR ? ex : o.w};
      const float S4[4] = {os.x, os.y, os.z, os.w}, N4[4] = {on.x, on.y, on.z, on.w};
      const float F4[4] = {fv.x, fv.y, fv.z, fv.w};
      float out[4];
      if (ALPHA1) {
        // all-fluid neighbourhoods take val / 4, and cells that are all
        // solid (inside obstacles, outside the domain) are 0 (a per-thread
        // choice: a warp vote here cost more than the divergence it saves)
        if (cw == 0x1f1f1f1fu) {
#pragma unroll
          for (int j = 0; j < 4; j++)
            out[j] = ((((W4[j] + E4[j]) + S4[j]) + N4[j]) + F4[j] * hh * hh) * 0.25f;
        } else if ((cw & 0x01010101u) == 0u) {
#pragma unroll
          for (int j = 0; j < 4; j++) out[j] = 0.0f;
        } else {
#pragma unroll
          for (int j = 0; j < 4; j++)
            out[j] = rb_update1((cw >> (8 * j)) & 0xffu, W4[j], E4[j], S4[j], N4[j], F4[j], hh);
        }
        if (cm != 0xfu) {  // edge columns keep their values
          const float4 sv = St::lds4(self + row);
          const float P4[4] = {sv.x, sv.y, sv.z, sv.w};
#pragma unroll
          for (int j = 0; j < 4; j++)
            if (!((cm >> j) & 1u)) out[j] = P4[j];
        }
      } else {
        const float4 sv = St::lds4(self + row);
        const float P4[4] = {sv.x, sv.y, sv.z, sv.w};
#pragma unroll
        for (int j = 0; j < 4; j++)
          out[j] = ((cm >> j) & 1u) ? rb_update_alpha((cw >> (8 * j)) & 0xffu, P4[j], W4[j], E4[j],
                                                      S4[j], N4[j], F4[j], hh, a.alpha)
                                    : P4[j];
      }
      St::sts4(self + row, make_float4(out[0], out[1], out[2], out[3]));
    }
  };
  int half = 0;
  for (int s = 0; s < a.nsweeps; s++) {
#pragma unroll
    for (int color = 1; color >= 0; color--) {
      half++;
      // parity of this thread's rows: (half + rsub) & 1, rsub's parity is wpar
      if (((half + wpar + color) & 1) != 0)
        sweep(std::integral_constant<int, 1>{}, color, half);
      else
        sweep(std::integral_constant<int, 0>{}, color, half);
      __syncthreads();
    }
    if (a.zgbc && edge) {
      zero_gradient();
      __syncthreads();
    }
  }

  // ---- write the tile (float4; gx is a multiple of 4)
  for (int q = tid; q < TY * (TX / 4); q += NT) {
    int ty2 = q / (TX / 4), g = q - ty2 * (TX / 4);
    int ry = HALO + ty2, rx = HALO + 4 * g;
    int gx = x0 + rx, gy = y0 + ry;
    if (gy >= h || gx >= w) continue;
    int c0 = (rx + ry) & 1;
    int b0 = (c0 * RY + ry) * HX + (rx >> 1), b1 = ((c0 ^ 1) * RY + ry) * HX + (rx >> 1);
    float2 u = St::lds2(sp + b0);
    float2 v = St::lds2(sp + b1);
    float4 o = make_float4(u.x, v.x, u.y, v.y);
    S *dst = a.out + (size_t)gy * P + gx;
    if (gx + 3 < w) {
      St::st4(dst, o);
    } else {
      dst[0] = St::fromf(o.x);
      if (gx + 1 < w) dst[1] = St::fromf(o.y);
      if (gx + 2 < w) dst[2] = St::fromf(o.z);
    }
  }

  if (!a.rc && !a.norm2) return;
  // ---- residual on the tile grown by one cell (in place into f) ----------
  // (per-thread partial sums of r^2 in FP32, a handful of terms each; the
  // block and global sums are FP64.  No FP64 arithmetic in the cell loop:
  // GB300's FP64 rate is a small fraction of FP32.)
  float acc = 0.0f;
  const int rlo = a.rc ? HALO - 1 : HALO;
  const int rhix = a.rc ? HALO + TX : HALO + TX - 1, rhiy = a.rc ? HALO + TY : HALO + TY - 1;
#pragma unroll
  for (int color = 0; color < 2; color++) {
    const S *self = sp + color * RY * HX;
    const S *oth = sp + (color ^ 1) * RY * HX;
    S *fs = sf + color * RY * HX;
    const uint8_t *cs = sc + color * RY * HX;
    for (int ry = rlo + rsub; ry <= rhiy; ry += RPP) {
      const int par = (ry + color) & 1;
      const int gy = y0 + ry;
      const int row = ry * HX + k0;
      const float4 o = St::lds4(oth + row);
      const float ex = St::tof(par ? oth[row + 4] : oth[row - 1]);
      const float4 os = St::lds4(oth + row - HX);
      const float4 on = St::lds4(oth + row + HX);
      const float4 fv = St::lds4(fs + row);
      const float4 sv = St::lds4(self + row);
      const uchar4 cv = *reinterpret_cast<const uchar4 *>(cs + row);
      const float W4[4] = {par ? o.x : ex, par ? o.y : o.x, par ? o.z : o.y, par ? o.w : o.z};
      const float E4[4] = {par ? o.y : o.x, par ? o.z : o.y, par ? o.w : o.z, par ? ex : o.w};
      const float S4[4] = {os.x, os.y, os.z, os.w}, N4[4] = {on.x, on.y, on.z, on.w};
      const float F4[4] = {fv.x, fv.y, fv.z, fv.w}, P4[4] = {sv.x, sv.y, sv.z, sv.w};
      const unsigned C4[4] = {cv.x, cv.y, cv.z, cv.w};
      float out[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int rx = 2 * (k0 + j) + par, gx = x0 + rx;
        float r = 0.0f;
        if (rx >= rlo && rx <= rhix && gx >= 1 && gx < w - 1 && gy >= 1 && gy < h - 1) {
          r = resid1(C4[j], P4[j], W4[j], E4[j], S4[j], N4[j], F4[j], a.ihsq);
          if (a.norm2 && rx >= HALO && rx < HALO + TX && ry >= HALO && ry < HALO + TY)
            acc = __fmaf_rn(r, r, acc);
        }
        out[j] = r;
      }
      if (a.rc) St::sts4(fs + row, make_float4(out[0], out[1], out[2], out[3]));
    }
  }
  __syncthreads();
  if (a.norm2) {
    __shared__ double red[NTY];
    double dacc = (double)acc;
    for (int o = 16; o > 0; o >>= 1) dacc += __shfl_xor_sync(0xffffffffu, dacc, o);
    if (tx == 0) red[ty] = dacc;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int i = 0; i < NTY; i++) t += red[i];
      atomicAdd(a.norm2, t);
    }
  }
  // ---- restrict (pressure_solver.cpp:118-132) onto the coarse tile -------
  if (a.rc) {
    const int cx0 = bx * (TX / 2), cy0 = by * (TY / 2);
    float rfac = a.rfac;
    if (EXT && a.scale_bits) {
      float inv;
      rfac = rfac * (coarse_scale(a.scale_bits, a.scale_h1sq, a.scale_kexp, &inv) * a.scale_h1sq);
    }
    // one coarse cell: full weighting of the 3x3 fine residuals around it
    auto restrict1 = [&](float m1, float c0, float p1, float m2, float c2, float p2, float m3,
                         float c3, float p3) {
      float v = (m1 * 1.0f + c0 * 2.0f) + p1 * 1.0f;
      v = v + ((m2 * 2.0f + c2 * 4.0f) + p2 * 2.0f);
      v = v + ((m3 * 1.0f + c3 * 2.0f) + p3 * 1.0f);
      return v * rfac;
    };
    if constexpr (HALO % 8 == 0 && (TX / 2) % 4 == 0) {
      // 4 consecutive coarse cells per thread.  Coarse column X sits over
      // fine column rx = 2X - x0 (even): its centre values are entries kc =
      // rx / 2 of the colour-(ry & 1) rows, its west / east neighbours
      // entries kc - 1 / kc of the other colour; kc is a multiple of 4.
      constexpr int CXG = TX / 8, NQR = CXG * (TY / 2);
      for (int q = tid; q < NQR; q += NT) {
        const int cyy = q / CXG, g = q - cyy * CXG;
        const int X0 = cx0 + 4 * g, Y = cy0 + cyy;
        if (X0 >= a.cw || Y >= a.ch) continue;
        const int ry = 2 * Y - y0, kc = (2 * X0 - x0) >> 1;
        float cen[3][4], oth[3][5];
#pragma unroll
        for (int e = 0; e < 3; e++) {
          const int r = ry + e - 1, c = r & 1;
          const float4 u = St::lds4(sf + (c * RY + r) * HX + kc);
          const float4 o = St::lds4(sf + ((c ^ 1) * RY + r) * HX + kc);
          cen[e][0] = u.x;
          cen[e][1] = u.y;
          cen[e][2] = u.z;
          cen[e][3] = u.w;
          oth[e][0] = St::tof(sf[((c ^ 1) * RY + r) * HX + kc - 1]);
          oth[e][1] = o.x;
          oth[e][2] = o.y;
          oth[e][3] = o.z;
          oth[e][4] = o.w;
        }
        float v[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int X = X0 + j;
          v[j] = 0.0f;
          if (X >= 1 && X < a.cw - 1 && Y >= 1 && Y < a.ch - 1)
            v[j] = restrict1(oth[0][j], cen[0][j], oth[0][j + 1], oth[1][j], cen[1][j],
                             oth[1][j + 1], oth[2][j], cen[2][j], oth[2][j + 1]);
        }
        SC *dst = a.rc + (size_t)Y * a.cpitch + X0;
        if (X0 + 3 < a.cw) {
          Sc::st4(dst, make_float4(v[0], v[1], v[2], v[3]));
        } else {
#pragma unroll
          for (int j = 0; j < 4; j++)
            if (X0 + j < a.cw) dst[j] = Sc::fromf(v[j]);
        }
      }
    } else {
      for (int q = tid; q < (TX / 2) * (TY / 2); q += NT) {
        int cyy = q / (TX / 2), cxx = q - cyy * (TX / 2);
        int X = cx0 + cxx, Y = cy0 + cyy;
        if (X >= a.cw || Y >= a.ch) continue;
        float v = 0.0f;
        if (X >= 1 && X < a.cw - 1 && Y >= 1 && Y < a.ch - 1) {
          int rx = 2 * X - x0, ry = 2 * Y - y0;
          auto R = [&](int dx, int dy) { return St::tof(sf[IDX(rx + dx, ry + dy)]); };
          v = restrict1(R(-1, -1), R(0, -1), R(1, -1), R(-1, 0), R(0, 0), R(1, 0), R(-1, 1),
                        R(0, 1), R(1, 1));
        }
        a.rc[(size_t)Y * a.cpitch + X] = Sc::fromf(v);
      }
    }
  }
}

template <int TX, int TY, int HALO, bool ALPHA1, int NT, class S = float, class SC = S,
          bool EXT = false>
__global__ void __launch_bounds__(NT, NT >= 1024 ? 1 : (NT == 512 ? 2 : 4))
    k_mg(MgArgsT<S, SC> a) {
  griddep_wait();
  k_mg_body<TX, TY, HALO, ALPHA1, NT, S, SC, EXT>(a, blockIdx.x, blockIdx.y);
}
// One launch over the members of a batch (FP32): block -> member -> tile.
template <int TX, int TY, int HALO, bool ALPHA1, int NT>
__global__ void __launch_bounds__(NT, NT >= 1024 ? 1 : (NT == 512 ? 2 : 4))
    k_mg_m(const MgArgs *__restrict__ A, const int *__restrict__ bs, int n, unsigned tag,
           unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  const int m = member_of(bs, n);
  const MgArgs &a = A[m];
  const int l = (int)blockIdx.x - __ldg(bs + m), gx = (a.w + TX - 1) / TX;
  k_mg_body<TX, TY, HALO, ALPHA1, NT, float, float>(a, l % gx, l / gx);
}

// ------------------------------------------------------ residual field only
__global__ void k_residual(const float *__restrict__ p, const float *__restrict__ rhs,
                           const uint8_t *__restrict__ flag, int w, int h, int P, float ihsq,
                           float *r, double *norm2) {
  griddep_wait();
  int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  double acc = 0.0;
  if (x < w && y < h) {
    float rv = 0.0f;
    if (x >= 1 && x < w - 1 && y >= 1 && y < h - 1) {
      size_t i = (size_t)y * P + x;
      float pc = p[i];
      float fw = (float)flag[i - 1], fe = (float)flag[i + 1];
      float fs = (float)flag[i - P], fn = (float)flag[i + P];
      float val = 0.0f;
      val = val + (p[i - 1] * fw + pc * (1.0f - fw));
      val = val + (p[i + 1] * fe + pc * (1.0f - fe));
      val = val + (p[i - P] * fs + pc * (1.0f - fs));
      val = val + (p[i + P] * fn + pc * (1.0f - fn));
      val = val + -4.0f * pc;
      val = val * ihsq;
      rv = (rhs[i] + val) * (float)flag[i];
      acc = (double)rv * (double)rv;
    }
    if (r) r[(size_t)y * P + x] = rv;
  }
  // 2-D block of 32 x 8: reduce over the whole block
  __shared__ double red[8];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (threadIdx.x == 0) red[threadIdx.y] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && threadIdx.x == 0 && norm2) {
    double s = 0.0;
    for (int i = 0; i < 8; i++) s += red[i];
    atomicAdd(norm2, s);
  }
}

// --------------------------------------------------------- flag coarsening
__global__ void k_coarsen(const uint8_t *__restrict__ f, int fp, uint8_t *fc, int cw, int ch,
                          int cp) {
  int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  if (x >= cw || y >= ch) return;
  uint8_t v = 1;
  if (x >= 1 && x < cw - 1 && y >= 1 && y < ch - 1) {
    auto F = [&](int xx, int yy) { return (int)f[(size_t)yy * fp + xx]; };
    int s = F(2 * x - 1, 2 * y - 1) + 2 * F(2 * x, 2 * y - 1) + F(2 * x + 1, 2 * y - 1) +
            2 * F(2 * x - 1, 2 * y) + 4 * F(2 * x, 2 * y) + 2 * F(2 * x + 1, 2 * y) +
            F(2 * x - 1, 2 * y + 1) + 2 * F(2 * x, 2 * y + 1) + F(2 * x + 1, 2 * y + 1);
    // (s / 16.0f) > 0.2 in the reference, exact for integer s.
    v = s >= 4 ? 1 : 0;
  }
  fc[(size_t)y * cp + x] = v;
}

__global__ void k_fill_u8(uint8_t *p, int w, int h, int pitch, uint8_t v) {
  int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  if (x < w && y < h) p[(size_t)y * pitch + x] = v;
}

// ------------------------------------------------------------ tail solver
// The coarse end of the V-cycle (levels lt .. levels-2) in one launch of one
// 1024-thread CTA, every level resident in shared memory: down (zero initial
// guess, 3 sweeps, residual, restrict), 5 sweeps on the coarsest level, up
// (prolongate + correct, 3 sweeps).  Same arithmetic as the tiled kernels.
constexpr int TAIL_MAXL = 12;
constexpr int TAIL_THREADS = 1024;
constexpr size_t TAIL_SMEM_MAX = 160 * 1024;

struct TailLevel {
  int w, h;
  float hh, ihsq, rfac;
  int oe, orr, orhs, oc;  // offsets: elements for e / r / rhs, bytes for code
};
template <class S>
struct TailArgs {
  int nlev;
  TailLevel L[TAIL_MAXL];
  const uint8_t *code[TAIL_MAXL];
  int code_pitch[TAIL_MAXL];
  const S *rhs_top;
  int rhs_pitch;
  S *e_top;
  int e_pitch;
  int float_words;  // elements of the arithmetic part of shared memory
  float wsum[5];
  float rwsum[5];  // RN(1 / wsum[k])
  // Tolerance-solver hierarchy: zero-gradient edges (corners included) on
  // every level after every sweep and after the correction, no zero
  // columns / rows in the prolongation, `ncoarse` sweeps on the coarsest
  // level (the last one of the tail) instead of 5.
  int ext, ncoarse;
};

// A level may be worked by a team of threads (a prefix of the block, with
// named barrier 1 or a warp barrier); measured on GB300, the whole block on
// every level is fastest, so every level's team is the full block.
__device__ __forceinline__ void team_sync(int team) {
  if (team >= TAIL_THREADS)
    __syncthreads();
  else if (team > 32)
    asm volatile("bar.sync 1, %0;" ::"r"(team) : "memory");
  else
    __syncwarp();
}

// S: storage of the top level's rhs and result (float, or the 16-bit type of
// the mixed solver); T: arithmetic and shared-memory type (float, or double
// for the FP64 coarse solve of the mixed solver).
// Loads the tail's codes and zeroes its e arrays; level 0's rhs comes from
// rhs_top (from_global) or is zeroed for its producer to fill.
template <class S, class T>
__device__ __forceinline__ void tail_load(const TailArgs<S> &a, T *fm, uint8_t *bm,
                                          bool from_global) {
  using St = Sto<S>;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nl = a.nlev;
  for (int t = 0; t < nl; t++) {
    const TailLevel &L = a.L[t];
    for (int y = ty; y < L.h; y += 32)
      for (int x = tx; x < L.w; x += 32) {
        int q = y * L.w + x;
        bm[L.oc + q] = a.code[t][(size_t)y * a.code_pitch[t] + x];
        fm[L.oe + q] = T(0);
        if (t == 0)
          fm[L.orhs + q] = from_global ? (T)St::tof(a.rhs_top[(size_t)y * a.rhs_pitch + x]) : T(0);
      }
  }
}

// The tail's levels on shared memory (fm: arithmetic arrays, bm: codes),
// with level 0's rhs and zeroed e arrays in place: down, the coarsest level,
// up.  Block-local barriers only.
template <class S, class T>
__device__ __forceinline__ void tail_levels(const TailArgs<S> &a, T *fm, uint8_t *bm) {
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  const int nl = a.nlev;
  const float ws0 = a.wsum[0], ws1 = a.wsum[1], ws2 = a.wsum[2], ws3 = a.wsum[3], ws4 = a.wsum[4];
  const float rw0 = a.rwsum[0], rw1 = a.rwsum[1], rw2 = a.rwsum[2], rw3 = a.rwsum[3],
              rw4 = a.rwsum[4];
  // x / wsum[k], correctly rounded (div_rn for float, the division for double)
  auto DIVW = [&](T x, int k) -> T {
    const float d = k == 0 ? ws0 : (k == 1 ? ws1 : (k == 2 ? ws2 : (k == 3 ? ws3 : ws4)));
    if constexpr (std::is_same<T, float>::value) {
      const float r = k == 0 ? rw0 : (k == 1 ? rw1 : (k == 2 ? rw2 : (k == 3 ? rw3 : rw4)));
      return div_rn(x, d, r);
    } else {
      return x / (T)d;
    }
  };
  auto team_of = [&](int t) {
    (void)t;
    return TAIL_THREADS;
  };


  // setZeroGradientBC on level t, plus the corners in ext mode
  auto zero_gradient = [&](int t, int team) {
    const TailLevel &L = a.L[t];
    T *e = fm + L.oe;
    const int w = L.w, hh2 = L.h, ny = hh2 - 2, nx = w - 2;
    for (int q = tid; q < 2 * ny + 2 * nx + 4; q += team) {
      if (q < 2 * ny) {
        const int y = 1 + (q >> 1);
        if (q & 1)
          e[y * w + w - 1] = e[y * w + w - 2];
        else
          e[y * w] = e[y * w + 1];
      } else if (q < 2 * ny + 2 * nx) {
        const int k = q - 2 * ny, x = 1 + (k >> 1);
        if (k & 1)
          e[(hh2 - 1) * w + x] = e[(hh2 - 2) * w + x];
        else
          e[x] = e[w + x];
      } else {
        const int c = q - 2 * ny - 2 * nx;
        const int cx = (c & 1) ? w - 1 : 0, cy = (c & 2) ? hh2 - 1 : 0;
        const int nxx = (c & 1) ? w - 2 : 1, nyy = (c & 2) ? hh2 - 2 : 1;
        e[cy * w + cx] = e[nyy * w + nxx];
      }
    }
    team_sync(team);
  };

  auto sweeps = [&](int t, int ns, int team) {
    const TailLevel &L = a.L[t];
    T *e = fm + L.oe;
    const T *f = fm + L.orhs;
    const uint8_t *c = bm + L.oc;
    const int w = L.w, hw2 = (w + 1) / 2, ystep = team / 32;
    const T hh = (T)L.hh;
    for (int s = 0; s < ns; s++) {
      for (int color = 1; color >= 0; color--) {
        for (int y = 1 + ty; y < L.h - 1; y += ystep) {
          int par = (y + color) & 1;
          for (int j = tx; j < hw2; j += 32) {
            int x = 2 * j + par;
            if (x < 1 || x >= w - 1) continue;
            int i = y * w + x;
            unsigned ci = c[i];
            T pw = e[i - 1], pe = e[i + 1], ps = e[i - w], pn = e[i + w], fi = f[i];
            if (ci == (C_CENTER | C_W | C_E | C_S | C_N))
              e[i] = ((((pw + pe) + ps) + pn) + fi * hh * hh) * T(0.25);
            else
              e[i] = rb_update1<T>(ci, pw, pe, ps, pn, fi, hh);
          }
        }
        team_sync(team);
      }
      if (a.ext) zero_gradient(t, team);
    }
  };

  // down
  for (int t = 0; t < nl; t++) {
    const int team = team_of(t);
    if (tid >= team) continue;
    const int ystep = team / 32;
    if (t == nl - 1) {
      sweeps(t, a.ext ? a.ncoarse : 5, team);
      break;
    }
    sweeps(t, 3, team);
    const TailLevel &L = a.L[t], &C = a.L[t + 1];
    T *e = fm + L.oe, *r = fm + L.orr;
    const T *f = fm + L.orhs;
    const uint8_t *c = bm + L.oc;
    for (int y = ty; y < L.h; y += ystep)
      for (int x = tx; x < L.w; x += 32) {
        int q = y * L.w + x;
        T rv = T(0);
        if (x >= 1 && x < L.w - 1 && y >= 1 && y < L.h - 1)
          rv = resid1<T>(c[q], e[q], e[q - 1], e[q + 1], e[q - L.w], e[q + L.w], f[q], (T)L.ihsq);
        r[q] = rv;
      }
    team_sync(team);
    T *rc = fm + C.orhs;
    const T rfac = (T)L.rfac;
    for (int Y = ty; Y < C.h; Y += ystep)
      for (int X = tx; X < C.w; X += 32) {
        T v = T(0);
        if (X >= 1 && X < C.w - 1 && Y >= 1 && Y < C.h - 1) {
          const T *R0 = r + (2 * Y) * L.w + 2 * X;
          v = (R0[-L.w - 1] * T(1) + R0[-L.w] * T(2)) + R0[-L.w + 1] * T(1);
          v = v + ((R0[-1] * T(2) + R0[0] * T(4)) + R0[1] * T(2));
          v = v + ((R0[L.w - 1] * T(1) + R0[L.w] * T(2)) + R0[L.w + 1] * T(1));
          v = v * rfac;
        }
        rc[Y * C.w + X] = v;
      }
    team_sync(team);
  }
  // up
  for (int t = nl - 2; t >= 0; t--) {
    const int team = team_of(t);
    if (tid >= team) continue;
    const int ystep = team / 32;
    team_sync(team);  // the coarser level's team has finished
    const TailLevel &L = a.L[t], &C = a.L[t + 1];
    T *e = fm + L.oe;
    const T *ec = fm + C.oe;
    const uint8_t *c = bm + L.oc, *cc = bm + C.oc;
    for (int y = 1 + ty; y < L.h - 1; y += ystep)
      for (int x = 1 + tx; x < L.w - 1; x += 32) {
        int q = y * L.w + x;
        if (!(c[q] & C_CENTER)) continue;
        int cx = x >> 1, cy = y >> 1;
        auto E = [&](int xx, int yy) { return ec[yy * C.w + xx]; };
        auto F = [&](int xx, int yy) { return (int)(cc[yy * C.w + xx] & 1u); };
        bool xo = x & 1, yo = y & 1;
        const bool ext = a.ext != 0;
        T ev;
        if (!xo && !yo)
          ev = E(cx, cy);
        else if (xo && !yo)
          ev = (!ext && x >= L.w - 2) ? T(0)
                                      : DIVW(E(cx, cy) + E(cx + 1, cy), F(cx, cy) + F(cx + 1, cy));
        else if (!xo && yo)
          ev = (!ext && y >= L.h - 2) ? T(0)
                                      : DIVW(E(cx, cy) + E(cx, cy + 1), F(cx, cy) + F(cx, cy + 1));
        else
          ev = (!ext && (x >= L.w - 2 || y >= L.h - 2))
                   ? T(0)
                   : DIVW(((E(cx, cy) + E(cx + 1, cy + 1)) + E(cx + 1, cy)) + E(cx, cy + 1),
                          F(cx, cy) + F(cx + 1, cy + 1) + F(cx + 1, cy) + F(cx, cy + 1));
        e[q] = e[q] + ev;
      }
    team_sync(team);
    if (a.ext) zero_gradient(t, team);
    sweeps(t, 3, team);
  }
}

template <class S, class T>
__device__ __forceinline__ void k_mg_tail_body(const TailArgs<S> &a) {
  using St = Sto<S>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *fm = reinterpret_cast<T *>(smem_raw);
  uint8_t *bm = smem_raw + (size_t)a.float_words * sizeof(T);
  const int tx = threadIdx.x, ty = threadIdx.y;
  tail_load<S, T>(a, fm, bm, true);
  __syncthreads();
  tail_levels<S, T>(a, fm, bm);
  __syncthreads();
  const TailLevel &L0 = a.L[0];
  for (int y = ty; y < L0.h; y += 32)
    for (int x = tx; x < L0.w; x += 32)
      a.e_top[(size_t)y * a.e_pitch + x] = St::fromf((float)fm[L0.oe + y * L0.w + x]);
}

template <class S, class T>
__global__ void __launch_bounds__(TAIL_THREADS, 1) k_mg_tail(TailArgs<S> a) {
  griddep_wait();
  k_mg_tail_body<S, T>(a);
}
// One block per member of a batch (FP32).
__global__ void __launch_bounds__(TAIL_THREADS, 1)
    k_mg_tail_m(const TailArgs<float> *__restrict__ A, const int *__restrict__ bs, int n,
                unsigned tag, unsigned *err) {
  griddep_wait();
  if (!table_ok(bs, n, tag, err)) return;
  k_mg_tail_body<float, float>(A[blockIdx.x]);
}

// ------------------------------------------------ cluster coarse solve
// The coarse end of the V-cycle from a level of up to ~512x256 cells down,
// in one launch of a cluster of CT_CTAS thread blocks (the reference's
// hierarchy, FP32).  Levels cluster_top .. tail_top-1 are split into row
// bands, one per block, each in its block's shared memory with one ghost
// row on either side.  After a phase changes the first or last row of a
// band, the block writes those cells into its neighbours' ghost rows
// through distributed shared memory, and the cluster barrier makes them
// visible.  The bands nest: block k owns rows [2b, 2b') of a level when it
// owns rows [b, b') of the next coarser one (the last block also takes the
// extra rows of odd heights), so a restriction reads only its band and the
// ghost row below it, and a prolongation its coarse band and the ghost row
// above.  The tail's levels (tail_top down) run in block 0 alone, as in the
// one-block tail kernel.  Every cell goes through the arithmetic of the
// tiled kernels and the tail, so the results are the same bits.  Each
// sweep's half only sends the cells of the colour it updated: the
// neighbour reads only the other colour of its ghost rows in that phase.
namespace cg = cooperative_groups;
constexpr int CT_MAXD = 6;
constexpr int CT_CTAS = 16;
constexpr size_t CT_SMEM_MAX = 227 * 1024;

struct CtLevel {
  int w, h, rows;     // level size; local rows per block (largest band + 2)
  float hh, ihsq, rfac;
  int oe, orr, orhs;  // float offsets of the local e / r / rhs arrays (rows x w)
  int oc;             // byte offset of the local codes
  int band[CT_CTAS + 1];
  const uint8_t *code;
  int code_pitch;
};
struct CTailArgs {
  int nd;                    // banded levels
  CtLevel D[CT_MAXD];
  int tband[CT_CTAS + 1];    // row bands of the tail's top level (restriction targets)
  TailArgs<float> tail;      // the tail's levels, run by block 0
  int tail_fo, tail_bo;      // float / byte offsets of the tail's region
  int float_words;           // floats before the byte region
  const float *rhs_top;      // level cluster_top's rhs and result (global)
  int rhs_pitch;
  float *e_top;
  int e_pitch;
  float wsum[5], rwsum[5];
};

__global__ void __launch_bounds__(TAIL_THREADS, 1) k_mg_ctail(const __grid_constant__ CTailArgs a) {
  griddep_wait();
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  constexpr int C = CT_CTAS;
  constexpr int NT = TAIL_THREADS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *fm = reinterpret_cast<float *>(smem_raw);
  uint8_t *bm = smem_raw + (size_t)a.float_words * sizeof(float);
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const float ws0 = a.wsum[0], ws1 = a.wsum[1], ws2 = a.wsum[2], ws3 = a.wsum[3], ws4 = a.wsum[4];
  const float rw0 = a.rwsum[0], rw1 = a.rwsum[1], rw2 = a.rwsum[2], rw3 = a.rwsum[3],
              rw4 = a.rwsum[4];
  auto DIVW = [&](float x, int k) -> float {
    const float d = k == 0 ? ws0 : (k == 1 ? ws1 : (k == 2 ? ws2 : (k == 3 ? ws3 : ws4)));
    const float r = k == 0 ? rw0 : (k == 1 ? rw1 : (k == 2 ? rw2 : (k == 3 ? rw3 : rw4)));
    return div_rn(x, d, r);
  };
  // (row, 32-column segment) items to warps, columns to lanes: one
  // division per warp item instead of one per cell
  const int wid = tid >> 5, lane = tid & 31;
  auto for_cells = [&](int nrows, int ncols, auto &&fn) {
    const int nseg = (ncols + 31) >> 5;
    for (int it = wid; it < nrows * nseg; it += NT / 32) {
      const int r = it / nseg, c = (it - r * nseg) * 32 + lane;
      if (c < ncols) fn(r, c);
    }
  };

  // load: codes of the band and ghost rows, zeroed e / r, level 0's rhs
  for (int d = 0; d < a.nd; d++) {
    const CtLevel &L = a.D[d];
    const int y0 = L.band[rank], y1 = L.band[rank + 1], w = L.w;
    for_cells(y1 - y0 + 2, w, [&](int lr, int x) {
      const int y = y0 - 1 + lr, k = lr * w + x;
      const bool in = y >= 0 && y < L.h;
      bm[L.oc + k] = in ? L.code[(size_t)y * L.code_pitch + x] : (uint8_t)0;
      fm[L.oe + k] = 0.0f;
      fm[L.orr + k] = 0.0f;
      fm[L.orhs + k] = (d == 0 && y >= y0 && y < y1) ? a.rhs_top[(size_t)y * a.rhs_pitch + x] : 0.0f;
    });
  }
  if (rank == 0) tail_load<float, float>(a.tail, fm + a.tail_fo, bm + a.tail_bo, false);
  cl.sync();

  // The first / last band row of array `off` of level d into the
  // neighbours' ghost rows: the cells of colour `color` ((x + y + color)
  // even), or whole rows for color < 0.
  auto send_rows = [&](int d, int off, int color, bool first, bool last) {
    const CtLevel &L = a.D[d];
    const int y0 = L.band[rank], y1 = L.band[rank + 1], w = L.w;
    float *arr = fm + off;
    if (first && rank > 0) {
      float *dst = cl.map_shared_rank(arr, rank - 1) + (y0 - L.band[rank - 1] + 1) * w;
      const float *src = arr + w;
      for (int x = tid; x < w; x += NT)
        if (color < 0 || ((x + y0 + color) & 1) == 0) dst[x] = src[x];
    }
    if (last && rank < C - 1) {
      float *dst = cl.map_shared_rank(arr, rank + 1);
      const float *src = arr + (y1 - y0) * w;
      for (int x = tid; x < w; x += NT)
        if (color < 0 || ((x + y1 - 1 + color) & 1) == 0) dst[x] = src[x];
    }
  };

  // one half-sweep (colour `color`) of level d's band, then the exchange
  auto dsweep = [&](int d, int color) {
    const CtLevel &L = a.D[d];
    const int w = L.w, y0 = L.band[rank], y1 = L.band[rank + 1], hw2 = (w + 1) / 2;
    float *e = fm + L.oe;
    const float *f = fm + L.orhs;
    const uint8_t *c = bm + L.oc;
    const float hh = L.hh;
    const int ya = max(y0, 1), yb = min(y1, L.h - 1);
    for_cells(max(yb - ya, 0), hw2, [&](int ry, int j) {
      const int y = ya + ry;
      const int x = 2 * j + ((y + color) & 1);
      if (x < 1 || x >= w - 1) return;
      const int i = (y - y0 + 1) * w + x;
      const unsigned ci = c[i];
      const float pw = e[i - 1], pe = e[i + 1], ps = e[i - w], pn = e[i + w], fi = f[i];
      if (ci == (C_CENTER | C_W | C_E | C_S | C_N))
        e[i] = ((((pw + pe) + ps) + pn) + fi * hh * hh) * 0.25f;
      else
        e[i] = rb_update1<float>(ci, pw, pe, ps, pn, fi, hh);
    });
    __syncthreads();
    send_rows(d, L.oe, color, true, true);
    cl.sync();
  };

  // residual of level d's band; the last band row goes to the next block
  auto dresid = [&](int d) {
    const CtLevel &L = a.D[d];
    const int w = L.w, y0 = L.band[rank], y1 = L.band[rank + 1];
    const float *e = fm + L.oe, *f = fm + L.orhs;
    float *r = fm + L.orr;
    const uint8_t *c = bm + L.oc;
    const float ihsq = L.ihsq;
    for_cells(y1 - y0, w, [&](int ry, int x) {
      const int y = y0 + ry, q = (ry + 1) * w + x;
      float rv = 0.0f;
      if (x >= 1 && x < w - 1 && y >= 1 && y < L.h - 1)
        rv = resid1<float>(c[q], e[q], e[q - 1], e[q + 1], e[q - w], e[q + w], f[q], ihsq);
      r[q] = rv;
    });
    __syncthreads();
    send_rows(d, L.orr, -1, false, true);
    cl.sync();
  };

  // full-weighting restriction of level d's residual into the next level's
  // rhs: its band (local) or, below the banded levels, the tail's top level
  // in block 0
  auto drestrict = [&](int d) {
    const CtLevel &L = a.D[d];
    const bool to_tail = d + 1 == a.nd;
    const int w = L.w, y0 = L.band[rank];
    const int wc = to_tail ? a.tail.L[0].w : a.D[d + 1].w;
    const int hc = to_tail ? a.tail.L[0].h : a.D[d + 1].h;
    const int Y0 = to_tail ? a.tband[rank] : a.D[d + 1].band[rank];
    const int Y1 = to_tail ? a.tband[rank + 1] : a.D[d + 1].band[rank + 1];
    float *rc = to_tail ? cl.map_shared_rank(fm + a.tail_fo + a.tail.L[0].orhs, 0)
                        : fm + a.D[d + 1].orhs;
    const float *r = fm + L.orr;
    const float rfac = L.rfac;
    for_cells(Y1 - Y0, wc, [&](int rY, int X) {
      const int Y = Y0 + rY;
      if (X < 1 || X >= wc - 1 || Y < 1 || Y >= hc - 1) return;
      const float *R0 = r + (2 * Y - y0 + 1) * w + 2 * X;
      float v = (R0[-w - 1] * 1.0f + R0[-w] * 2.0f) + R0[-w + 1] * 1.0f;
      v = v + ((R0[-1] * 2.0f + R0[0] * 4.0f) + R0[1] * 2.0f);
      v = v + ((R0[w - 1] * 1.0f + R0[w] * 2.0f) + R0[w + 1] * 1.0f);
      v = v * rfac;
      if (to_tail)
        rc[Y * wc + X] = v;
      else
        rc[(Y - Y0 + 1) * wc + X] = v;
    });
    cl.sync();
  };

  // prolongation of the next level's e onto level d's band, correction,
  // then whole first / last rows to the neighbours
  auto dprolong = [&](int d) {
    const CtLevel &L = a.D[d];
    const bool from_tail = d + 1 == a.nd;
    const int w = L.w, y0 = L.band[rank], y1 = L.band[rank + 1];
    float *e = fm + L.oe;
    const uint8_t *c = bm + L.oc;
    const int wc = from_tail ? a.tail.L[0].w : a.D[d + 1].w;
    const int Y0 = from_tail ? 0 : a.D[d + 1].band[rank] - 1;
    const float *ec = from_tail ? cl.map_shared_rank(fm + a.tail_fo + a.tail.L[0].oe, 0)
                                : fm + a.D[d + 1].oe;
    const uint8_t *cg_ = from_tail ? a.tail.code[0] : bm + a.D[d + 1].oc;
    const int cpitch = from_tail ? a.tail.code_pitch[0] : wc;
    auto E = [&](int xx, int yy) { return ec[(yy - Y0) * wc + xx]; };
    auto F = [&](int xx, int yy) {
      return (int)((from_tail ? __ldg(cg_ + (size_t)yy * cpitch + xx)
                              : cg_[(size_t)(yy - Y0) * cpitch + xx]) &
                   1u);
    };
    for_cells(y1 - y0, w, [&](int ry, int x) {
      const int y = y0 + ry;
      if (x < 1 || x >= w - 1 || y < 1 || y >= L.h - 1) return;
      const int q = (ry + 1) * w + x;
      if (!(c[q] & C_CENTER)) return;
      const int cx = x >> 1, cy = y >> 1;
      const bool xo = x & 1, yo = y & 1;
      float ev;
      if (!xo && !yo)
        ev = E(cx, cy);
      else if (xo && !yo)
        ev = (x >= w - 2) ? 0.0f : DIVW(E(cx, cy) + E(cx + 1, cy), F(cx, cy) + F(cx + 1, cy));
      else if (!xo && yo)
        ev = (y >= L.h - 2) ? 0.0f : DIVW(E(cx, cy) + E(cx, cy + 1), F(cx, cy) + F(cx, cy + 1));
      else
        ev = (x >= w - 2 || y >= L.h - 2)
                 ? 0.0f
                 : DIVW(((E(cx, cy) + E(cx + 1, cy + 1)) + E(cx + 1, cy)) + E(cx, cy + 1),
                        F(cx, cy) + F(cx + 1, cy + 1) + F(cx + 1, cy) + F(cx, cy + 1));
      e[q] = e[q] + ev;
    });
    __syncthreads();
    send_rows(d, L.oe, -1, true, true);
    cl.sync();
  };

  for (int d = 0; d < a.nd; d++) {
    for (int s = 0; s < 3; s++) {
      dsweep(d, 1);
      dsweep(d, 0);
    }
    dresid(d);
    drestrict(d);
  }
  if (rank == 0) tail_levels<float, float>(a.tail, fm + a.tail_fo, bm + a.tail_bo);
  cl.sync();
  for (int d = a.nd - 1; d >= 0; d--) {
    dprolong(d);
    for (int s = 0; s < 3; s++) {
      dsweep(d, 1);
      dsweep(d, 0);
    }
  }
  {
    const CtLevel &L = a.D[0];
    const int w = L.w, y0 = L.band[rank], y1 = L.band[rank + 1];
    for_cells(y1 - y0, w, [&](int ry, int x) {
      a.e_top[(size_t)(y0 + ry) * a.e_pitch + x] = fm[L.oe + (ry + 1) * w + x];
    });
  }
  cl.sync();  // no block leaves while another may still read its memory
}

// ------------------------------------------------------------ launches
// The tiles the tolerance hierarchy uses (chosen by level width): the only
// ones built with its rules.
template <int TX, int TY, int HALO, bool A1>
constexpr bool ext_tile() {
  return A1 && HALO == 8 && ((TX == 112 && TY == 50) || (TX == 48 && TY == 16));
}

template <int TX, int TY, int HALO, bool A1, int NT = 256, class S = float, class SC = S>
void launch_mg_t(const MgArgsT<S, SC> &a, cudaStream_t st) {
  using T = Tile<TX, TY, HALO>;
  dim3 grid((a.w + TX - 1) / TX, (a.h + TY - 1) / TY);
  if (a.ext) {
    if constexpr (ext_tile<TX, TY, HALO, A1>()) {
      launch_pdl(k_mg<TX, TY, HALO, A1, NT, S, SC, true>, grid, dim3(32, NT / 32),
                 T::smem(sizeof(S), sizeof(SC)), st, a);
    } else {
      throw ArgError("tolerance hierarchy: tile not built with its rules");
    }
  } else if constexpr (std::is_same<S, SC>::value) {
    launch_pdl(k_mg<TX, TY, HALO, A1, NT, S, SC, false>, grid, dim3(32, NT / 32),
               T::smem(sizeof(S), sizeof(SC)), st, a);
  } else {
    throw ArgError("mixed storage types only in the tolerance hierarchy");
  }
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

template <int TX, int TY, int HALO, bool A1, int NT = 256, class S = float, class SC = S,
          bool EXT = false>
void set_smem_attr() {
  UBG_CUDA(cudaFuncSetAttribute(k_mg<TX, TY, HALO, A1, NT, S, SC, EXT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)Tile<TX, TY, HALO>::smem(sizeof(S), sizeof(SC))));
  // one carveout for every kernel of a V-cycle: no L1 / shared-memory
  // reconfiguration between consecutive launches
  UBG_CUDA(cudaFuncSetAttribute(k_mg<TX, TY, HALO, A1, NT, S, SC, EXT>,
                                cudaFuncAttributePreferredSharedMemoryCarveout, 100));
}

template <class S, class T>
void set_tail_attr() {
  UBG_CUDA(cudaFuncSetAttribute(k_mg_tail<S, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TAIL_SMEM_MAX));
  UBG_CUDA(cudaFuncSetAttribute(k_mg_tail<S, T>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
}

template <class S>
void set_vcycle_attrs() {
  set_smem_attr<112, 50, 8, true, 512, S>();
  set_smem_attr<48, 16, 8, true, 256, S>();
  set_smem_attr<40, 8, 12, true, 256, S>();
  set_smem_attr<112, 24, 8, true, 256, S>();
  set_smem_attr<48, 40, 8, true, 256, S>();
  set_smem_attr<112, 114, 8, true, 1024, S>();
}

template <int TX, int TY, int HALO>
void set_multi_attr() {
  constexpr int NT = TX == 112 && TY == 50 ? 512 : (TX == 112 && TY == 114 ? 1024 : 256);
  UBG_CUDA(cudaFuncSetAttribute(k_mg_m<TX, TY, HALO, true, NT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)Tile<TX, TY, HALO>::smem(4)));
  UBG_CUDA(cudaFuncSetAttribute(k_mg_m<TX, TY, HALO, true, NT>,
                                cudaFuncAttributePreferredSharedMemoryCarveout, 100));
}

// Sets the shared-memory attributes of every smoother and tail kernel, once
// per process (function-local static initialisation is thread-safe; the
// server's worker thread and the caller's threads may race here).
bool g_ctail_ok = false;  // a cluster of the coarse solve fits this device
char g_ctail_why[160] = "not probed";

static void set_all_kernel_attributes() {
  set_multi_attr<112, 50, 8>();
  set_multi_attr<48, 16, 8>();
  set_multi_attr<40, 8, 12>();
  set_multi_attr<112, 24, 8>();
  set_multi_attr<48, 40, 8>();
  set_multi_attr<112, 114, 8>();
  UBG_CUDA(cudaFuncSetAttribute(k_mg_tail_m, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TAIL_SMEM_MAX));
  UBG_CUDA(cudaFuncSetAttribute(k_mg_tail_m, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  set_vcycle_attrs<float>();
  set_smem_attr<56, 24, 4, false>();
  set_tail_attr<float, float>();
  set_vcycle_attrs<__half>();
  set_vcycle_attrs<__nv_bfloat16>();
  set_tail_attr<__half, double>();
  set_tail_attr<__nv_bfloat16, double>();
  // the tolerance solver: its rules on the width-chosen tiles, FP32 level 0
  // over 16-bit coarse levels, FP32 arithmetic in the tail over 16-bit
  // storage
  set_smem_attr<112, 50, 8, true, 512, float, float, true>();
  set_smem_attr<48, 16, 8, true, 256, float, float, true>();
  set_smem_attr<112, 50, 8, true, 512, __half, __half, true>();
  set_smem_attr<48, 16, 8, true, 256, __half, __half, true>();
  set_smem_attr<112, 50, 8, true, 512, __nv_bfloat16, __nv_bfloat16, true>();
  set_smem_attr<48, 16, 8, true, 256, __nv_bfloat16, __nv_bfloat16, true>();
  set_smem_attr<112, 50, 8, true, 512, float, __half, true>();
  set_smem_attr<48, 16, 8, true, 256, float, __half, true>();
  set_smem_attr<112, 50, 8, true, 512, float, __nv_bfloat16, true>();
  set_smem_attr<48, 16, 8, true, 256, float, __nv_bfloat16, true>();
  set_tail_attr<__half, float>();
  set_tail_attr<__nv_bfloat16, float>();
  // the cluster coarse solve: 16 blocks of up to 227 KB each, if the device
  // can hold such a cluster (else the launches per level are used)
  g_ctail_ok = false;
  cudaError_t e1 = cudaFuncSetAttribute(k_mg_ctail, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)CT_SMEM_MAX);
  cudaError_t e2 = e1 == cudaSuccess
                       ? cudaFuncSetAttribute(k_mg_ctail,
                                              cudaFuncAttributeNonPortableClusterSizeAllowed, 1)
                       : e1;
  if (e2 != cudaSuccess) {
    snprintf(g_ctail_why, sizeof(g_ctail_why), "attributes: %s", cudaGetErrorString(e2));
  } else {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(CT_CTAS);
    cfg.blockDim = dim3(32, TAIL_THREADS / 32);
    cfg.dynamicSmemBytes = CT_SMEM_MAX;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CT_CTAS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    cudaError_t e3 = cudaOccupancyMaxActiveClusters(&nclusters, k_mg_ctail, &cfg);
    g_ctail_ok = e3 == cudaSuccess && nclusters >= 1;
    if (g_ctail_ok)
      snprintf(g_ctail_why, sizeof(g_ctail_why), "available (%d clusters of %d blocks)",
               nclusters, CT_CTAS);
    else
      snprintf(g_ctail_why, sizeof(g_ctail_why), "occupancy: %s, %d clusters",
               cudaGetErrorString(e3), nclusters);
  }
  cudaGetLastError();
}

void init_kernel_attributes() {
  static const bool done = (set_all_kernel_attributes(), true);
  (void)done;
}

// 3 sweeps with an optional restriction epilogue need HALO >= 8; the tile
// is chosen by level width so small levels still fill the GPU.
// Smoother tiles the autotuner chooses from (3-sweep launches need a halo of
// 8, 5-sweep launches 12): id -> TX x TY, halo, threads.
constexpr int kTiles = 6;
const char *const kTileNames[kTiles] = {"112x50/h8/512", "48x16/h8/256", "40x8/h12/256",
                                        "112x24/h8/256", "48x40/h8/256", "112x114/h8/1024"};
bool tile_ok(int id, int nsweeps) { return id >= 0 && id < kTiles && (nsweeps <= 3 || id == 2); }

template <class S>
void launch_mg_tile(const MgArgsT<S> &a, int id, cudaStream_t st) {
  switch (id) {
    case 0: launch_mg_t<112, 50, 8, true, 512, S>(a, st); break;
    case 1: launch_mg_t<48, 16, 8, true, 256, S>(a, st); break;
    case 2: launch_mg_t<40, 8, 12, true, 256, S>(a, st); break;
    case 3: launch_mg_t<112, 24, 8, true, 256, S>(a, st); break;
    case 4: launch_mg_t<48, 40, 8, true, 256, S>(a, st); break;
    case 5: launch_mg_t<112, 114, 8, true, 1024, S>(a, st); break;
    default: throw ArgError("smoother tile id");
  }
}

// An FP32 level over 16-bit coarse arrays (the tolerance solver's level 0):
// 3 sweeps, tile by level width.
template <class SC>
void launch_mg_mixed_top(const MgArgsT<float, SC> &a, cudaStream_t st) {
  if (!ALPHA_IS_ONE(a.alpha) || a.nsweeps < 1 || a.nsweeps > 3)
    throw ArgError("mixed top level: alpha = 1, at most 3 sweeps");
  if (a.w >= 1200)
    launch_mg_t<112, 50, 8, true, 512, float, SC>(a, st);
  else
    launch_mg_t<48, 16, 8, true, 256, float, SC>(a, st);
}

template <class S>
void launch_mg(const MgArgsT<S> &a, cudaStream_t st) {
  if (ALPHA_IS_ONE(a.alpha) && a.nsweeps > 1 && a.nsweeps <= 5 && tile_ok(a.tile, a.nsweeps)) {
    launch_mg_tile(a, a.tile, st);
    return;
  }
  if (!ALPHA_IS_ONE(a.alpha) || a.nsweeps == 1) {
    if constexpr (std::is_same<S, float>::value) {
      if (a.nsweeps != 1) throw ArgError("general alpha: one sweep per launch");
      launch_mg_t<56, 24, 4, false>(a, st);
    } else {
      throw ArgError("16-bit smoother: alpha = 1 only");
    }
  } else if (a.nsweeps <= 3) {
    if (a.w >= 1200)
      launch_mg_t<112, 50, 8, true, 512, S>(a, st);
    else
      launch_mg_t<48, 16, 8, true, 256, S>(a, st);
  } else if (a.nsweeps <= 5) {
    launch_mg_t<40, 8, 12, true, 256, S>(a, st);
  } else {
    throw ArgError("smoother: at most 5 sweeps per launch");
  }
}

MgArgs level_args(MgLevel &L, const float *in, float *out, int ns, float alpha) {
  MgArgs a{};
  a.in = in;
  a.out = out;
  a.rhs = L.rhs;
  a.code = L.code;
  a.w = L.w;
  a.h = L.h;
  a.pitch = L.pitch;
  a.hh = L.hh;
  a.alpha = alpha;
  a.ihsq = 1.0f / L.hh / L.hh;
  a.nsweeps = ns;
  for (int k = 0; k < 5; k++) {
    a.wsum[k] = (float)((double)(float)k + 0.0001);
    a.rwsum[k] = 1.0f / a.wsum[k];
  }
  a.rfac = 1.0f / 16.0f;
  a.tile = -1;
  return a;
}

// Shared-memory bytes of the tail for levels lt .. last (default
// levels-2, the reference's coarsest level) with arithmetic type of
// elem_bytes.
size_t tail_smem_bytes(const std::vector<MgLevel> &lv, int lt, size_t elem_bytes, int last = -1) {
  size_t fw = 0, bw = 0;
  if (last < 0) last = (int)lv.size() - 2;
  for (int t = lt; t <= last; t++) {
    size_t n = (size_t)lv[t].w * lv[t].h;
    fw += 3 * ((n + 3) / 4 * 4);
    bw += (n + 15) / 16 * 16;
  }
  return fw * elem_bytes + bw;
}

// scaled: the h^2-scaled form of the mixed solver (hh = 1, ihsq = 1,
// restriction weights rfac[level]); else the reference's form.
template <class S, class T>
TailArgs<S> tail_args(MgHier &mg, int lt, const S *rhs_top, S *e_top, const float *rfac,
                      size_t *smem_out) {
  TailArgs<S> a{};
  int nl = mg_coarsest(mg) + 1 - lt;
  a.nlev = nl;
  a.ext = mg.ext ? 1 : 0;
  a.ncoarse = mg.ncoarse;
  size_t fw = 0, bw = 0;
  for (int t = 0; t < nl; t++) {
    MgLevel &L = mg.lv[lt + t];
    TailLevel &TL = a.L[t];
    int n = L.w * L.h;
    TL.w = L.w;
    TL.h = L.h;
    TL.hh = rfac ? 1.0f : L.hh;
    TL.ihsq = rfac ? 1.0f : 1.0f / L.hh / L.hh;
    TL.rfac = rfac ? rfac[lt + t] : 1.0f / 16.0f;
    TL.oe = (int)fw;
    fw += (n + 3) / 4 * 4;
    TL.orr = (int)fw;
    fw += (n + 3) / 4 * 4;
    TL.orhs = (int)fw;
    fw += (n + 3) / 4 * 4;
    TL.oc = (int)bw;
    bw += (n + 15) / 16 * 16;
    a.code[t] = L.code;
    a.code_pitch[t] = L.pitch;
  }
  a.float_words = (int)fw;
  MgLevel &top = mg.lv[lt];
  a.rhs_top = rhs_top;
  a.rhs_pitch = top.pitch;
  a.e_top = e_top;
  a.e_pitch = top.pitch;
  for (int k = 0; k < 5; k++) {
    a.wsum[k] = (float)((double)(float)k + 0.0001);
    a.rwsum[k] = 1.0f / a.wsum[k];
  }
  size_t smem = fw * sizeof(T) + bw;
  if (smem > TAIL_SMEM_MAX) throw ArgError("coarse levels exceed the tail kernel's shared memory");
  *smem_out = smem;
  return a;
}

template <class S, class T>
void run_tail_t(MgHier &mg, int lt, const S *rhs_top, S *e_top, const float *rfac,
                cudaStream_t st) {
  ProfScope ps_(KC_TAIL, st);
  size_t smem = 0;
  TailArgs<S> a = tail_args<S, T>(mg, lt, rhs_top, e_top, rfac, &smem);
  launch_pdl(k_mg_tail<S, T>, dim3(1), dim3(32, 32), smem, st, a);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void run_tail(MgHier &mg, int lt, cudaStream_t st) {
  run_tail_t<float, float>(mg, lt, mg.lv[lt].rhs, mg.lv[lt].e[0], nullptr, st);
}

// Arguments of the cluster coarse solve from level ct (banded levels ct ..
// tail_top-1, the tail below); false if the hierarchy or the shared memory
// does not allow it.
bool ctail_args(MgHier &mg, int ct, CTailArgs &a, size_t &smem) {
  const int T = mg.tail_top;
  if (mg.ext || ct < 1 || T < 2 || ct >= T || T - ct > CT_MAXD || T > mg_coarsest(mg))
    return false;
  constexpr int C = CT_CTAS;
  if (mg.lv[T].h < C) return false;
  for (int l = ct; l < T; l++)
    if (mg.lv[l + 1].h != mg.lv[l].h / 2 || mg.lv[l + 1].w != mg.lv[l].w / 2) return false;
  a = CTailArgs{};
  size_t tsm = 0;
  try {
    a.tail = tail_args<float, float>(mg, T, nullptr, nullptr, nullptr, &tsm);
  } catch (const ArgError &) {
    return false;
  }
  a.nd = T - ct;
  // bands: the tail's top level split evenly, each finer level's bands the
  // doubled ones (the last block takes the extra rows of odd heights)
  const int hT = mg.lv[T].h;
  for (int k = 0; k < C; k++) a.tband[k] = (int)(((long long)k * hT) / C);
  a.tband[C] = hT;
  const int *next = a.tband;
  for (int d = a.nd - 1; d >= 0; d--) {
    CtLevel &D = a.D[d];
    const MgLevel &L = mg.lv[ct + d];
    for (int k = 0; k < C; k++) D.band[k] = 2 * next[k];
    D.band[C] = L.h;
    int rows = 0;
    for (int k = 0; k < C; k++) {
      if (D.band[k + 1] <= D.band[k]) return false;
      rows = std::max(rows, D.band[k + 1] - D.band[k]);
    }
    D.rows = rows + 2;
    D.w = L.w;
    D.h = L.h;
    D.hh = L.hh;
    D.ihsq = 1.0f / L.hh / L.hh;
    D.rfac = 1.0f / 16.0f;
    D.code = L.code;
    D.code_pitch = L.pitch;
    next = D.band;
  }
  size_t fo = 0, bo = 0;
  for (int d = 0; d < a.nd; d++) {
    CtLevel &D = a.D[d];
    const size_t n = (size_t)D.rows * D.w;
    D.oe = (int)fo;
    fo += (n + 3) / 4 * 4;
    D.orr = (int)fo;
    fo += (n + 3) / 4 * 4;
    D.orhs = (int)fo;
    fo += (n + 3) / 4 * 4;
    D.oc = (int)bo;
    bo += (n + 15) / 16 * 16;
  }
  a.tail_fo = (int)fo;
  fo += (size_t)a.tail.float_words;
  a.tail_bo = (int)bo;
  bo += tsm - (size_t)a.tail.float_words * sizeof(float);
  a.float_words = (int)fo;
  smem = fo * sizeof(float) + bo;
  if (smem > CT_SMEM_MAX) return false;
  const MgLevel &top = mg.lv[ct];
  a.rhs_top = top.rhs;
  a.rhs_pitch = top.pitch;
  a.e_top = top.e[0];
  a.e_pitch = top.pitch;
  for (int k = 0; k < 5; k++) {
    a.wsum[k] = (float)((double)(float)k + 0.0001);
    a.rwsum[k] = 1.0f / a.wsum[k];
  }
  return true;
}

// The lowest level from which the cluster coarse solve covers the rest of
// the V-cycle, or -1.
int choose_cluster(MgHier &mg) {
  init_kernel_attributes();
  if (!g_ctail_ok) return -1;
  int best = -1;
  for (int ct = mg.tail_top - 1; ct >= 1; ct--) {
    CTailArgs a;
    size_t smem = 0;
    if (!ctail_args(mg, ct, a, smem)) break;
    best = ct;
  }
  return best;
}

void run_ctail(MgHier &mg, int ct, cudaStream_t st) {
  ProfScope ps_(KC_TAIL, st);
  CTailArgs a;
  size_t smem = 0;
  if (!ctail_args(mg, ct, a, smem)) throw ArgError("cluster coarse solve: hierarchy does not fit");
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(CT_CTAS);
  cfg.blockDim = dim3(32, TAIL_THREADS / 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CT_CTAS;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  UBG_CUDA(cudaLaunchKernelEx(&cfg, k_mg_ctail, a));
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

// MG::solveLevel, pressure_solver.cpp:201-248.
void solve_level(MgHier &mg, std::vector<int> &cur, int l, bool zgbc, cudaStream_t st) {
  bool bc = zgbc && l == 0;
  MgLevel &L = mg.lv[l];
  if (l >= 1 && l == mg.cluster_top) {
    run_ctail(mg, l, st);
    cur[l] = 0;
    return;
  }
  if (l >= 1 && l == mg.tail_top) {
    run_tail(mg, l, st);
    cur[l] = 0;
    return;
  }
  if (l == mg.levels - 2) {
    ProfScope ps_(l == 0 ? KC_SMOOTH_L0 : (l == 1 ? KC_SMOOTH_L1 : KC_SMOOTH_COARSE), st);
    MgArgs a = level_args(L, L.e[cur[l]], L.e[1 - cur[l]], 5, 1.0f);
    a.zero_init = l > 0;
    launch_mg(a, st);
    cur[l] ^= 1;
    return;
  }
  MgLevel &C = mg.lv[l + 1];
  {
    ProfScope ps_(l == 0 ? KC_SMOOTH_L0 : (l == 1 ? KC_SMOOTH_L1 : KC_SMOOTH_COARSE), st);
    MgArgs a = level_args(L, L.e[cur[l]], L.e[1 - cur[l]], 3, 1.0f);
    a.zgbc = bc;
    a.zero_init = l > 0;
    a.tile = L.tile_pre;
    a.rc = C.rhs;
    a.cw = C.w;
    a.ch = C.h;
    a.cpitch = C.pitch;
    launch_mg(a, st);
    cur[l] ^= 1;
  }
  solve_level(mg, cur, l + 1, false, st);
  {
    ProfScope ps_(l == 0 ? KC_SMOOTH_L0 : (l == 1 ? KC_SMOOTH_L1 : KC_SMOOTH_COARSE), st);
    MgArgs a = level_args(L, L.e[cur[l]], L.e[1 - cur[l]], 3, 1.0f);
    a.zgbc = bc;
    a.tile = L.tile_post;
    a.ec = C.e[cur[l + 1]];
    a.codec = C.code;
    a.cpitch = C.pitch;
    a.cw = C.w;
    a.ch = C.h;
    if (l == 0) a.norm2 = mg.post_norm2;
    launch_mg(a, st);
    cur[l] ^= 1;
  }
}

// ------------------------------------------------ mixed-precision solver
// Defect correction (iterative refinement) around a 16-bit V-cycle.  The
// outer loop keeps p, f and the residual in FP32 with FP64 norms; the inner
// V-cycle solves the correction equation in the h^2-scaled form
//   n e - sum(e_nbr) = g,  g = s h^2 r
// (the smoother's own form with hh = 1: no 1/h^2 factors, so e and g share
// one magnitude range), with s a power of two chosen from max|r| so that the
// 16-bit values stay in range; the correction applied is e / s.
template <class S>
struct DcArgs {
  const float *p;         // current pressure (FP32, level 0)
  const S *e;             // correction of the last V-cycle (null: none yet)
  const DcScalars *sc_in;  // its 1/s
  float *pout;            // p + e / s with the zero-gradient edges
  const float *f;
  const uint8_t *code;
  int w, h, pitch;
  float ihsq;
  float *r;          // residual of pout (0 on the edges)
  DcScalars *sc;     // norm2 / maxbits accumulate here
};

// p' = p + e/s everywhere (edge cells take their interior neighbour's value,
// corners untouched: setZeroGradientBC, pressure_solver.cpp:183-192), then
// r = f + A p' (calculateResidualField, pressure_solver.cpp:100-110) with
// ||r||^2 (FP32 per warp, FP64 across warps) and max|r|.
template <class S>
__global__ void __launch_bounds__(256) k_dc_resid(DcArgs<S> a) {
  griddep_wait();
  using St = Sto<S>;
  // 4 cells per thread (x4 .. x4 + 3 of row y)
  const int x4 = (blockIdx.x * 32 + threadIdx.x) * 4, y = blockIdx.y * 8 + threadIdx.y;
  const int w = a.w, h = a.h, P = a.pitch;
  const float is = a.e ? a.sc_in->inv_s : 0.0f;
  auto PV = [&](int xx, int yy) {
    if (yy >= 1 && yy <= h - 2) xx = xx == 0 ? 1 : (xx == w - 1 ? w - 2 : xx);
    if (xx >= 1 && xx <= w - 2) yy = yy == 0 ? 1 : (yy == h - 1 ? h - 2 : yy);
    size_t i = (size_t)yy * P + xx;
    float v = __ldg(a.p + i);
    if (a.e) v = v + St::ldg1(a.e + i) * is;
    return v;
  };
  float sq = 0.0f;
  unsigned mb = 0u;
  if (x4 < w && y < h) {
    float pc[4], rv[4] = {0.f, 0.f, 0.f, 0.f};
    const size_t i0 = (size_t)y * P + x4;
    if (x4 >= 4 && x4 + 4 <= w - 2 && y >= 2 && y <= h - 3) {
      // interior: no edge mapping; rows y-1, y, y+1 as float4 plus the
      // west / east neighbours
      auto row4 = [&](int yy, float *o) {
        const size_t i = (size_t)yy * P + x4;
        float4 v = __ldg(reinterpret_cast<const float4 *>(a.p + i));
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
        o[3] = v.w;
        if (a.e) {
          const float4 e = St::ldg4(a.e + i);
          o[0] = o[0] + e.x * is;
          o[1] = o[1] + e.y * is;
          o[2] = o[2] + e.z * is;
          o[3] = o[3] + e.w * is;
        }
      };
      float s4[4], n4[4];
      row4(y, pc);
      row4(y - 1, s4);
      row4(y + 1, n4);
      const float pw = PV(x4 - 1, y), pe = PV(x4 + 4, y);
      const float4 fv = __ldg(reinterpret_cast<const float4 *>(a.f + i0));
      const uchar4 cv = __ldg(reinterpret_cast<const uchar4 *>(a.code + i0));
      const float F4[4] = {fv.x, fv.y, fv.z, fv.w};
      const unsigned C4[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
      for (int j = 0; j < 4; j++)
        rv[j] = resid1<float>(C4[j], pc[j], j > 0 ? pc[j - 1] : pw, j < 3 ? pc[j + 1] : pe, s4[j],
                              n4[j], F4[j], a.ihsq);
      *reinterpret_cast<float4 *>(a.pout + i0) = make_float4(pc[0], pc[1], pc[2], pc[3]);
      *reinterpret_cast<float4 *>(a.r + i0) = make_float4(rv[0], rv[1], rv[2], rv[3]);
    } else {
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int x = x4 + j;
        if (x >= w) break;
        const size_t i = i0 + j;
        pc[j] = PV(x, y);
        a.pout[i] = pc[j];
        if (x >= 1 && x < w - 1 && y >= 1 && y < h - 1)
          rv[j] = resid1<float>(__ldg(a.code + i), pc[j], PV(x - 1, y), PV(x + 1, y),
                                PV(x, y - 1), PV(x, y + 1), __ldg(a.f + i), a.ihsq);
        a.r[i] = rv[j];
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      sq = __fmaf_rn(rv[j], rv[j], sq);
      mb = max(mb, __float_as_uint(fabsf(rv[j])));
    }
  }
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  mb = __reduce_max_sync(0xffffffffu, mb);
  __shared__ double red[8];
  __shared__ unsigned redm[8];
  if (threadIdx.x == 0) {
    red[threadIdx.y] = (double)sq;
    redm[threadIdx.y] = mb;
  }
  __syncthreads();
  if (threadIdx.y == 0 && threadIdx.x == 0) {
    double t = 0.0;
    unsigned m = 0;
    for (int k = 0; k < 8; k++) {
      t += red[k];
      m = max(m, redm[k]);
    }
    atomicAdd(&a.sc->norm2, t);
    atomicMax(&a.sc->maxbits, m);
  }
}

// g = r * h0^2 * s into the 16-bit rhs of level 0, s = 2^-(ex + kexp) where
// max|r| h0^2 = m 2^ex, m in [0.5, 1); records 1/s for the correction.
template <class S>
__global__ void __launch_bounds__(256) k_dc_scale(const float *__restrict__ r, S *g, int w, int h,
                                                  int pitch, DcScalars *sc, float h0sq, int kexp) {
  griddep_wait();
  using St = Sto<S>;
  const float m = __uint_as_float(sc->maxbits) * h0sq;
  float mul = 0.0f, inv = 0.0f;
  if (m > 0.0f) {
    int ex;
    frexpf(m, &ex);
    mul = h0sq * ldexpf(1.0f, -ex - kexp);
    inv = ldexpf(1.0f, ex + kexp);
  }
  const int x4 = (blockIdx.x * 32 + threadIdx.x) * 4, y = blockIdx.y * 8 + threadIdx.y;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) sc->inv_s = inv;
  if (x4 >= w || y >= h) return;
  const size_t i = (size_t)y * pitch + x4;
  float4 v = __ldg(reinterpret_cast<const float4 *>(r + i));
  v.x *= mul;
  v.y *= mul;
  v.z *= mul;
  v.w *= mul;
  St::st4(g + i, v);
}

// Mean of f over the interior fluid cells: sum, sum of squares and count
// (FP32 within a warp, FP64 across warps), then f -= mean on those cells.
// The zero-gradient system of the solver is singular (constants span its
// null space); the tolerance and mixed solvers solve its compatible part.
__global__ void __launch_bounds__(256) k_fmean_reduce(const float *__restrict__ f,
                                                      const uint8_t *__restrict__ code, int w,
                                                      int h, int pitch, double *acc) {
  griddep_wait();
  const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  float v = 0.0f;
  bool in = false;
  if (x >= 1 && x < w - 1 && y >= 1 && y < h - 1) {
    size_t i = (size_t)y * pitch + x;
    in = (__ldg(code + i) & C_CENTER) != 0;
    if (in) v = __ldg(f + i);
  }
  float s1 = v, s2 = v * v;
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  int n = __popc(__ballot_sync(0xffffffffu, in));
  __shared__ double r1[8], r2[8], rn[8];
  if (threadIdx.x == 0) {
    r1[threadIdx.y] = (double)s1;
    r2[threadIdx.y] = (double)s2;
    rn[threadIdx.y] = (double)n;
  }
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    double a1 = 0.0, a2 = 0.0, an = 0.0;
    for (int k = 0; k < 8; k++) {
      a1 += r1[k];
      a2 += r2[k];
      an += rn[k];
    }
    if (an > 0.0) {
      atomicAdd(acc + 0, a1);
      atomicAdd(acc + 1, a2);
      atomicAdd(acc + 2, an);
    }
  }
}

__global__ void __launch_bounds__(256) k_fmean_apply(float *f, const uint8_t *__restrict__ code,
                                                     int w, int h, int pitch,
                                                     const double *acc) {
  griddep_wait();
  const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  if (x < 1 || x >= w - 1 || y < 1 || y >= h - 1) return;
  const double n = acc[2];
  const float mean = n > 0.0 ? (float)(acc[0] / n) : 0.0f;
  size_t i = (size_t)y * pitch + x;
  if (__ldg(code + i) & C_CENTER) f[i] = f[i] - mean;
}

template <class S>
MgArgsT<S> level_args_lo(MgHier &mg, MgLow &lo, int l, int cin, int ns) {
  MgLevel &L = mg.lv[l];
  MgArgsT<S> a{};
  a.in = (const S *)lo.e[cin][l];
  a.out = (S *)lo.e[1 - cin][l];
  a.rhs = (const S *)lo.rhs[l];
  a.code = L.code;
  a.w = L.w;
  a.h = L.h;
  a.pitch = L.pitch;
  a.hh = 1.0f;
  a.alpha = 1.0f;
  a.ihsq = 1.0f;
  a.nsweeps = ns;
  a.zero_init = 0;
  for (int k = 0; k < 5; k++) {
    a.wsum[k] = (float)((double)(float)k + 0.0001);
    a.rwsum[k] = 1.0f / a.wsum[k];
  }
  a.rfac = lo.rfac[l];
  a.tile = -1;
  return a;
}

// One V-cycle of the correction equation from e = 0 (solveLevel's schedule:
// V(3,3), 5 sweeps on the coarsest level, zero-gradient edges on level 0).
template <class S>
void solve_level_lo(MgHier &mg, MgLow &lo, std::vector<int> &cur, int l, cudaStream_t st) {
  const KernelClass kc = l == 0 ? KC_SMOOTH_L0 : (l == 1 ? KC_SMOOTH_L1 : KC_SMOOTH_COARSE);
  if (l >= 1 && l == mg.tail_top_fp64) {
    run_tail_t<S, double>(mg, l, (const S *)lo.rhs[l], (S *)lo.e[0][l], lo.rfac.data(), st);
    cur[l] = 0;
    return;
  }
  if (l == mg.levels - 2) {
    ProfScope ps_(kc, st);
    MgArgsT<S> a = level_args_lo<S>(mg, lo, l, cur[l], 5);
    a.zero_init = 1;
    a.zgbc = l == 0;
    launch_mg(a, st);
    cur[l] ^= 1;
    return;
  }
  MgLevel &C = mg.lv[l + 1];
  {
    ProfScope ps_(kc, st);
    MgArgsT<S> a = level_args_lo<S>(mg, lo, l, cur[l], 3);
    a.zero_init = 1;
    a.zgbc = l == 0;
    a.tile = mg.lv[l].tile_pre;
    a.rc = (S *)lo.rhs[l + 1];
    a.cw = C.w;
    a.ch = C.h;
    a.cpitch = C.pitch;
    launch_mg(a, st);
    cur[l] ^= 1;
  }
  solve_level_lo<S>(mg, lo, cur, l + 1, st);
  {
    ProfScope ps_(kc, st);
    MgArgsT<S> a = level_args_lo<S>(mg, lo, l, cur[l], 3);
    a.zgbc = l == 0;
    a.tile = mg.lv[l].tile_post;
    a.ec = (const S *)lo.e[cur[l + 1]][l + 1];
    a.codec = C.code;
    a.cpitch = C.pitch;
    a.cw = C.w;
    a.ch = C.h;
    launch_mg(a, st);
    cur[l] ^= 1;
  }
}

// One residual pass: p <- p + e/s (e = null: none), r, norm, max.
template <class S>
void dc_resid(MgHier &mg, MgLow &lo, const S *e, cudaStream_t st) {
  ProfScope ps_(KC_RESIDUAL, st);
  MgLevel &L = mg.lv[0];
  UBG_CUDA(cudaMemsetAsync(lo.dev, 0, offsetof(DcScalars, inv_s), st));
  DcArgs<S> a{};
  a.p = L.e[mg.cur0];
  a.e = e;
  a.sc_in = lo.dev;
  a.pout = L.e[1 - mg.cur0];
  a.f = L.rhs;
  a.code = L.code;
  a.w = L.w;
  a.h = L.h;
  a.pitch = L.pitch;
  a.ihsq = 1.0f / L.hh / L.hh;
  a.r = lo.r32;
  a.sc = lo.dev;
  dim3 grid((L.w + 127) / 128, (L.h + 7) / 8);
  k_dc_resid<S><<<grid, dim3(32, 8), 0, st>>>(a);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
  mg.cur0 ^= 1;
}

template <class S>
int solve_mixed_t(MgHier &mg, MgLow &lo, double tol, int max_cycles, double fnorm2, double *rel,
                  cudaStream_t st) {
  MgLevel &L0 = mg.lv[0];
  const float h0sq = L0.hh * L0.hh;
  const S *e_last = nullptr;
  int c = 0;
  auto converged = [&]() {
    UBG_CUDA(cudaMemcpyAsync(lo.host, lo.dev, sizeof(DcScalars), cudaMemcpyDeviceToHost, st));
    UBG_CUDA(cudaStreamSynchronize(st));
    return lo.host->norm2 <= tol * tol * fnorm2;
  };
  for (;;) {
    dc_resid<S>(mg, lo, e_last, st);
    if (tol > 0.0 && converged()) break;
    if (c >= max_cycles) break;
    {
      ProfScope ps_(KC_RESIDUAL, st);
      dim3 grid((L0.w + 127) / 128, (L0.h + 7) / 8);
      k_dc_scale<S><<<grid, dim3(32, 8), 0, st>>>(lo.r32, (S *)lo.rhs[0], L0.w, L0.h, L0.pitch,
                                                  lo.dev, h0sq, lo.kexp);
      UBG_LAUNCH_CHECK();
      g_stats.launches++;
    }
    std::vector<int> cur(mg.levels, 0);
    solve_level_lo<S>(mg, lo, cur, 0, st);
    e_last = (const S *)lo.e[cur[0]][0];
    c++;
  }
  if (rel) *rel = tol > 0.0 ? std::sqrt(lo.host->norm2 / (fnorm2 > 0.0 ? fnorm2 : 1.0)) : -1.0;
  return c;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// The first level whose whole coarse end fits the tail kernel (arithmetic
// elements of elem_bytes: 4 for FP32, 8 for the mixed solver's FP64) with a
// top level of at most max_cells.
int choose_tail(const std::vector<MgLevel> &lv, int max_cells, size_t elem_bytes = 4,
                int last = -1) {
  int L = (int)lv.size();
  if (last < 0) last = L - 2;
  for (int lt = 1; lt <= last; lt++) {
    if (tail_smem_bytes(lv, lt, elem_bytes, last) <= TAIL_SMEM_MAX &&
        (size_t)lv[lt].w * lv[lt].h <= (size_t)max_cells)
      return lt;
  }
  return -1;
}

}  // namespace

const char *cluster_coarse_solve_status() {
  init_kernel_attributes();
  return g_ctail_why;
}

namespace {
std::vector<MgLevel> level_shapes(int W, int H, float h0) {
  int cw = W, ch = H;
  float hh = h0;
  std::vector<MgLevel> lv;
  while (cw > 3 && ch > 3) {
    MgLevel L{};
    L.w = cw;
    L.h = ch;
    L.pitch = round_up(cw, 32);
    L.hh = hh;
    lv.push_back(L);
    int nw = cw / 2, nh = ch / 2;
    // h * (r.width - 1.0f) / (rc.width - 1.0f), pressure_solver.cpp:225
    hh = hh * ((float)cw - 1.0f) / ((float)nw - 1.0f);
    cw = nw;
    ch = nh;
  }
  if (lv.size() < 2) throw ArgError("grid too small for the multigrid hierarchy (need W, H >= 8)");
  return lv;
}
}  // namespace

size_t mg_arena_bytes(int W, int H) {
  size_t total = 0;
  for (auto &L : level_shapes(W, H, 1.0f)) {
    size_t n = (size_t)L.pitch * L.h;
    total += 3 * align256(n * 4) + 2 * align256(n);
  }
  return total + 512;  // norm scalars
}

void mg_bind(MgHier &mg, int W, int H, float h0, void *arena, size_t bytes) {
  std::vector<MgLevel> lv = level_shapes(W, H, h0);
  if (bytes < mg_arena_bytes(W, H)) throw ArgError("multigrid arena too small");
  init_kernel_attributes();
  char *p = (char *)arena;
  for (auto &L : lv) {
    size_t n = (size_t)L.pitch * L.h;
    L.e[0] = (float *)p;
    p += align256(n * 4);
    L.e[1] = (float *)p;
    p += align256(n * 4);
    L.rhs = (float *)p;
    p += align256(n * 4);
    L.flag = (uint8_t *)p;
    p += align256(n);
    L.code = (uint8_t *)p;
    p += align256(n);
  }
  mg.norm = (double *)p;
  mg.post_norm2 = nullptr;
  mg.tail_top = choose_tail(lv, mg.tail_cells);
  mg.tail_top_fp64 = choose_tail(lv, 128, 8);
  mg.lv = lv;
  mg.levels = (int)lv.size();
  // the cluster coarse solve from two levels above the tail (the autotuner
  // measured that choice fastest at 1024x512, 4096x2048 and 8192x4096;
  // from larger levels its 16 blocks have too much work per phase)
  {
    const int lowest = choose_cluster(mg);
    mg.cluster_top = lowest >= 1 ? std::max(lowest, mg.tail_top - 2) : -1;
  }
  mg.arena = nullptr;  // not owned
  mg.arena_bytes = bytes;
  mg.cur0 = 0;
}

void mg_alloc(MgHier &mg, int W, int H, float h0) {
  mg_free(mg);
  size_t total = mg_arena_bytes(W, H);
  void *arena = nullptr;
  if (cudaMalloc(&arena, total) != cudaSuccess) {
    cudaGetLastError();
    throw std::bad_alloc();
  }
  // zeroed before any stream of the caller uses it
  UBG_CUDA(cudaMemsetAsync(arena, 0, total, cudaStreamLegacy));
  UBG_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
  mg_bind(mg, W, H, h0, arena, total);
  mg.arena = arena;
}

void mg_free(MgHier &mg) {
  if (mg.arena) cudaFree(mg.arena);
  mg.arena = nullptr;
  mg.lv.clear();
  mg.levels = 0;
}

void level_make_code(MgLevel &L, cudaStream_t st) {
  dim3 grid((L.w + 31) / 32, (L.h + 7) / 8);
  k_make_code<<<grid, dim3(32, 8), 0, st>>>(L.flag, L.code, L.w, L.h, L.pitch);
  UBG_LAUNCH_CHECK();
}

void mg_update_fields(MgHier &mg, cudaStream_t st) {
  ProfScope ps_(KC_COARSEN, st);
  for (int l = 1; l < mg.levels; l++) {
    MgLevel &F = mg.lv[l - 1], &C = mg.lv[l];
    dim3 grid((C.w + 31) / 32, (C.h + 7) / 8);
    k_coarsen<<<grid, dim3(32, 8), 0, st>>>(F.flag, F.pitch, C.flag, C.w, C.h, C.pitch);
    UBG_LAUNCH_CHECK();
  }
  for (int l = 0; l < mg.levels; l++) level_make_code(mg.lv[l], st);
}

void mg_fill_coarse_flags_one(MgHier &mg, cudaStream_t st) {
  for (int l = 1; l < mg.levels; l++) {
    MgLevel &C = mg.lv[l];
    dim3 grid((C.w + 31) / 32, (C.h + 7) / 8);
    k_fill_u8<<<grid, dim3(32, 8), 0, st>>>(C.flag, C.w, C.h, C.pitch, 1);
    UBG_LAUNCH_CHECK();
  }
  for (int l = 0; l < mg.levels; l++) level_make_code(mg.lv[l], st);
}

void mg_solve(MgHier &mg, bool zgbc, cudaStream_t st) {
  std::vector<int> cur(mg.levels, 0);
  cur[0] = mg.cur0;
  solve_level(mg, cur, 0, zgbc, st);
  mg.cur0 = cur[0];
}

double mg_meanfree_rhs(MgHier &mg, cudaStream_t st, bool want_norm) {
  ProfScope ps_(KC_RESIDUAL, st);
  MgLevel &L = mg.lv[0];
  double *acc = mg.norm + 8;
  UBG_CUDA(cudaMemsetAsync(acc, 0, 3 * sizeof(double), st));
  dim3 grid((L.w + 31) / 32, (L.h + 7) / 8);
  k_fmean_reduce<<<grid, dim3(32, 8), 0, st>>>(L.rhs, L.code, L.w, L.h, L.pitch, acc);
  UBG_LAUNCH_CHECK();
  k_fmean_apply<<<grid, dim3(32, 8), 0, st>>>(L.rhs, L.code, L.w, L.h, L.pitch, acc);
  UBG_LAUNCH_CHECK();
  g_stats.launches += 2;
  if (!want_norm) return -1.0;
  double h[3];
  UBG_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st));
  UBG_CUDA(cudaStreamSynchronize(st));
  return h[2] > 0.0 ? std::max(0.0, h[1] - h[0] * h[0] / h[2]) : h[1];
}

// ------------------------------------------------------------- autotuner
namespace {
struct EvPair {
  cudaEvent_t a = nullptr, b = nullptr;
  EvPair() {
    UBG_CUDA(cudaEventCreate(&a));
    UBG_CUDA(cudaEventCreate(&b));
  }
  ~EvPair() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

// Mean milliseconds of `reps` calls of f after `warm` untimed calls.
template <class F>
double time_ms(EvPair &ev, cudaStream_t st, int warm, int reps, F &&f) {
  for (int i = 0; i < warm; i++) f();
  UBG_CUDA(cudaEventRecord(ev.a, st));
  for (int i = 0; i < reps; i++) f();
  UBG_CUDA(cudaEventRecord(ev.b, st));
  UBG_CUDA(cudaEventSynchronize(ev.b));
  float ms = 0.0f;
  UBG_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
  return (double)ms / reps;
}
}  // namespace

// The autotuner times whole V-cycles, captured into a CUDA graph as the step
// runs them, so launch gaps and the cache state between launches count:
// coordinate descent over the tail size, then each tiled level's pre- and
// post-smoothing tile.  The pressure is saved first and restored after the
// trials (a V-cycle leaves p in the buffer it started in).
// Tuning results by grid size: the choices depend on the level shapes, so
// simulations of one size (the members of a batch, the sessions of a
// server) share the first one's trials.
struct TuneChoice {
  int tail_cells = 0, tail_top = 0, cluster_top = -1;
  std::vector<int> pre, post;
};
std::mutex g_tune_mu;
std::map<std::pair<int, int>, TuneChoice> g_tune_cache;

void mg_autotune(MgHier &mg, cudaStream_t st, std::string *report) {
  init_kernel_attributes();
  const int nl = mg.levels;
  const std::pair<int, int> key(mg.lv[0].w, mg.lv[0].h);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end() && (int)it->second.pre.size() == nl) {
      mg.tail_cells = it->second.tail_cells;
      mg.tail_top = it->second.tail_top;
      mg.cluster_top = it->second.cluster_top;
      for (int l = 0; l < nl; l++) {
        mg.lv[l].tile_pre = it->second.pre[l];
        mg.lv[l].tile_post = it->second.post[l];
      }
      if (report) {
        char buf[160];
        snprintf(buf, sizeof(buf),
                 "{\"cached\": true, \"tail_cells\": %d, \"tail_top\": %d, \"cluster_top\": %d, \"levels\": [",
                 mg.tail_cells, mg.tail_top, mg.cluster_top);
        std::string rep = buf;
        const int last = (mg.tail_top >= 1 ? mg.tail_top : nl - 1) - 1;
        for (int l = 0; l <= std::min(last, nl - 3); l++) {
          const MgLevel &L = mg.lv[l];
          snprintf(buf, sizeof(buf), "%s{\"level\": %d, \"w\": %d, \"h\": %d, \"pre\": \"%s\", \"post\": \"%s\"}",
                   l ? ", " : "", l, L.w, L.h, L.tile_pre >= 0 ? kTileNames[L.tile_pre] : "default",
                   L.tile_post >= 0 ? kTileNames[L.tile_post] : "default");
          rep += buf;
        }
        rep += "]}";
        *report += rep;
      }
      return;
    }
  }
  EvPair ev;
  MgLevel &L0 = mg.lv[0];
  const size_t pbytes = (size_t)L0.pitch * L0.h * sizeof(float);
  float *saved = nullptr;
  if (cudaMalloc(&saved, pbytes) != cudaSuccess) {
    cudaGetLastError();
    throw std::bad_alloc();
  }
  const int c0 = mg.cur0;
  UBG_CUDA(cudaMemcpyAsync(saved, L0.e[c0], pbytes, cudaMemcpyDeviceToDevice, st));
  auto vcycle_us = [&]() {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    UBG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      mg_solve(mg, true, st);
    } catch (...) {
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      mg.cur0 = c0;
      throw;
    }
    UBG_CUDA(cudaStreamEndCapture(st, &g));
    mg.cur0 = c0;
    UBG_CUDA(cudaGraphInstantiate(&ge, g, 0));
    cudaGraphDestroy(g);
    double ms = time_ms(ev, st, 2, 6, [&] { UBG_CUDA(cudaGraphLaunch(ge, st)); });
    cudaGraphExecDestroy(ge);
    return 1e3 * ms;
  };
  // the tail and the tiles are tuned with launches per level; the cluster
  // coarse solve is tried last
  mg.cluster_top = -1;
  std::string rep = "{\"trials\": [";
  bool first = true;
  auto note = [&](const char *what, int level, const char *choice, double us) {
    char buf[200];
    snprintf(buf, sizeof(buf), "%s{\"what\": \"%s\", \"level\": %d, \"choice\": \"%s\", \"vcycle_us\": %.2f}",
             first ? "" : ", ", what, level, choice, us);
    rep += buf;
    first = false;
  };
  double best = vcycle_us();
  note("start", -1, "default", best);
  // tail size
  const int tail_cand[] = {512, 1024, 2048, 4096, 8192};
  int best_tc = mg.tail_cells, best_lt = mg.tail_top;
  for (int tc : tail_cand) {
    int lt = choose_tail(mg.lv, tc);
    if (lt < 1 || lt == best_lt) continue;
    int keep = mg.tail_top;
    mg.tail_top = lt;
    double t = vcycle_us();
    char c[32];
    snprintf(c, sizeof(c), "%d cells", tc);
    note("tail", lt, c, t);
    if (t < best) {
      best = t;
      best_tc = tc;
      best_lt = lt;
    } else {
      mg.tail_top = keep;
    }
  }
  mg.tail_top = best_lt;
  mg.tail_cells = best_tc;
  // tiles of the tiled levels (coordinate descent, pre then post)
  const int last = (mg.tail_top >= 1 ? mg.tail_top : nl - 1) - 1;
  for (int l = 0; l <= std::min(last, nl - 3); l++) {
    for (int which = 0; which < 2; which++) {
      int &slot = which ? mg.lv[l].tile_post : mg.lv[l].tile_pre;
      int keep = slot;
      for (int id = 0; id < kTiles; id++) {
        if (id == keep) continue;
        slot = id;
        double t = vcycle_us();
        note(which ? "post" : "pre", l, kTileNames[id], t);
        if (t < best) {
          best = t;
          keep = id;
        }
      }
      slot = keep;
    }
  }
  {
    // every feasible first level of the cluster coarse solve
    const int lowest = choose_cluster(mg);
    int keep = -1;
    for (int ct = mg.tail_top - 1; lowest >= 1 && ct >= lowest; ct--) {
      mg.cluster_top = ct;
      double t = vcycle_us();
      note("cluster", ct, "on", t);
      if (t < best) {
        best = t;
        keep = ct;
      }
    }
    mg.cluster_top = keep;
  }
  UBG_CUDA(cudaMemcpyAsync(L0.e[c0], saved, pbytes, cudaMemcpyDeviceToDevice, st));
  UBG_CUDA(cudaStreamSynchronize(st));
  cudaFree(saved);
  char buf[256];
  snprintf(buf, sizeof(buf), "], \"vcycle_us\": %.2f, \"tail_cells\": %d, \"tail_top\": %d, \"cluster_top\": %d, \"levels\": [",
           best, mg.tail_cells, mg.tail_top, mg.cluster_top);
  rep += buf;
  for (int l = 0; l <= std::min(last, nl - 3); l++) {
    const MgLevel &L = mg.lv[l];
    snprintf(buf, sizeof(buf), "%s{\"level\": %d, \"w\": %d, \"h\": %d, \"pre\": \"%s\", \"post\": \"%s\"}",
             l ? ", " : "", l, L.w, L.h, L.tile_pre >= 0 ? kTileNames[L.tile_pre] : "default",
             L.tile_post >= 0 ? kTileNames[L.tile_post] : "default");
    rep += buf;
  }
  rep += "]}";
  if (report) *report += rep;
  TuneChoice tc;
  tc.tail_cells = mg.tail_cells;
  tc.tail_top = mg.tail_top;
  tc.cluster_top = mg.cluster_top;
  for (int l = 0; l < nl; l++) {
    tc.pre.push_back(mg.lv[l].tile_pre);
    tc.post.push_back(mg.lv[l].tile_post);
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[key] = tc;
}

void mg_low_alloc(MgLow &lo, const MgHier &mg, int prec) {
  mg_low_free(lo);
  if (prec != UBG_MIXED_FP16 && prec != UBG_MIXED_BF16) throw ArgError("unknown precision mode");
  init_kernel_attributes();
  size_t total = align256(sizeof(DcScalars));
  for (auto &L : mg.lv) total += 3 * align256((size_t)L.pitch * L.h * 2);
  const MgLevel &L0 = mg.lv[0];
  total += align256((size_t)L0.pitch * L0.h * 4);
  void *arena = nullptr;
  if (cudaMalloc(&arena, total) != cudaSuccess) {
    cudaGetLastError();
    throw std::bad_alloc();
  }
  UBG_CUDA(cudaMemsetAsync(arena, 0, total, cudaStreamLegacy));
  UBG_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
  void *host = nullptr;
  if (cudaHostAlloc(&host, sizeof(DcScalars), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(arena);
    throw std::bad_alloc();
  }
  char *p = (char *)arena;
  lo.dev = (DcScalars *)p;
  p += align256(sizeof(DcScalars));
  lo.r32 = (float *)p;
  p += align256((size_t)L0.pitch * L0.h * 4);
  for (int k = 0; k < 2; k++) lo.e[k].assign(mg.levels, nullptr);
  lo.rhs.assign(mg.levels, nullptr);
  lo.rfac.assign(mg.levels, 0.0f);
  for (int l = 0; l < mg.levels; l++) {
    size_t b = align256((size_t)mg.lv[l].pitch * mg.lv[l].h * 2);
    lo.e[0][l] = p;
    p += b;
    lo.e[1][l] = p;
    p += b;
    lo.rhs[l] = p;
    p += b;
    if (l + 1 < mg.levels) {
      double q = (double)mg.lv[l + 1].hh / (double)mg.lv[l].hh;
      lo.rfac[l] = (float)(q * q / 16.0);
    }
  }
  // e = A^-1 g is bounded by about max|g| * max(W, H)^2 / 2 (a channel with
  // one Dirichlet end); keep it below 2^14 in FP16.  BF16 has FP32's range.
  int kexp = 0;
  if (prec == UBG_MIXED_FP16) {
    double n = (double)std::max(L0.w, L0.h);
    kexp = std::max(0, (int)std::ceil(std::log2(0.5 * n * n)) - 14);
  }
  lo.kexp = kexp;
  lo.prec = prec;
  lo.levels = mg.levels;
  lo.arena = arena;
  lo.host = (DcScalars *)host;
}

void mg_low_free(MgLow &lo) {
  if (lo.arena) cudaFree(lo.arena);
  if (lo.host) cudaFreeHost(lo.host);
  lo = MgLow{};
}

int mg_solve_mixed(MgHier &mg, MgLow &lo, double tol, int max_cycles, double fnorm2, double *rel,
                   cudaStream_t st) {
  if (lo.levels != mg.levels) throw std::runtime_error("mixed-precision hierarchy not allocated");
  if (lo.prec == UBG_MIXED_FP16) return solve_mixed_t<__half>(mg, lo, tol, max_cycles, fnorm2, rel, st);
  return solve_mixed_t<__nv_bfloat16>(mg, lo, tol, max_cycles, fnorm2, rel, st);
}

// ------------------------------------------------- fused batch V-cycle
namespace {
int tile_for(const MgLevel &L, int choice) {
  if (tile_ok(choice, 3)) return choice;
  return L.w >= 1200 ? 0 : 1;  // the width rule of launch_mg for 3 sweeps
}
int tile_tx(int id) { return id == 0 || id == 3 || id == 5 ? 112 : (id == 2 ? 40 : 48); }
int tile_ty(int id) {
  const int ty[kTiles] = {50, 16, 8, 24, 40, 114};
  return ty[id];
}
template <class A>
void slot_add(MultiSlot &s, const A &a, int blocks) {
  const char *p = reinterpret_cast<const char *>(&a);
  s.args.insert(s.args.end(), p, p + sizeof(A));
  if (s.bs.empty()) s.bs.push_back(0);
  s.bs.push_back(s.bs.back() + blocks);
  s.blocks += blocks;
  s.n++;
}
}  // namespace

void mg_multi_vcycle(const std::vector<MgHier *> &mgs, std::vector<MultiSlot> &out) {
  init_kernel_attributes();
  const int n = (int)mgs.size();
  int maxt = 0;
  for (auto *m : mgs) {
    if (m->tail_top < 1) throw ArgError("fused batch: a member has no coarse tail");
    maxt = std::max(maxt, m->tail_top);
  }
  // per member and level: which e[] holds the level's current values
  std::vector<std::vector<int>> cur(n);
  for (int i = 0; i < n; i++) {
    cur[i].assign(mgs[i]->levels, 0);
    cur[i][0] = mgs[i]->cur0;
  }
  auto level_slots = [&](int l, bool pre) {
    std::map<int, MultiSlot> by_tile;
    for (int i = 0; i < n; i++) {
      MgHier &mg = *mgs[i];
      if (l >= mg.tail_top) continue;
      MgLevel &L = mg.lv[l], &C = mg.lv[l + 1];
      MgArgs a = level_args(L, L.e[cur[i][l]], L.e[1 - cur[i][l]], 3, 1.0f);
      a.zgbc = l == 0;
      if (pre) {
        a.zero_init = l > 0;
        a.rc = C.rhs;
        a.cw = C.w;
        a.ch = C.h;
        a.cpitch = C.pitch;
      } else {
        a.ec = C.e[cur[i][l + 1]];
        a.codec = C.code;
        a.cpitch = C.pitch;
        a.cw = C.w;
        a.ch = C.h;
      }
      const int id = tile_for(L, pre ? L.tile_pre : L.tile_post);
      a.tile = id;
      MultiSlot &sl = by_tile[id];
      sl.kind = MK_MG;
      sl.tile = id;
      const int tx = tile_tx(id), ty = tile_ty(id);
      slot_add(sl, a, ((L.w + tx - 1) / tx) * ((L.h + ty - 1) / ty));
      cur[i][l] ^= 1;
    }
    for (auto &kv : by_tile) out.push_back(std::move(kv.second));
  };
  for (int l = 0; l < maxt; l++) level_slots(l, true);
  {
    MultiSlot sl;
    sl.kind = MK_TAIL;
    for (int i = 0; i < n; i++) {
      MgHier &mg = *mgs[i];
      const int lt = mg.tail_top;
      size_t smem = 0;
      TailArgs<float> a = tail_args<float, float>(mg, lt, mg.lv[lt].rhs, mg.lv[lt].e[0], nullptr,
                                                  &smem);
      sl.smem = std::max(sl.smem, smem);
      slot_add(sl, a, 1);
      cur[i][lt] = 0;
    }
    out.push_back(std::move(sl));
  }
  for (int l = maxt - 1; l >= 0; l--) level_slots(l, false);
  for (int i = 0; i < n; i++)
    if (cur[i][0] != mgs[i]->cur0) throw std::runtime_error("fused V-cycle parity");
}

void launch_multi_mg(const MultiSlot &slot, const void *dargs, const int *dbs, unsigned tag,
                     unsigned *err, cudaStream_t st) {
  if (slot.kind == MK_TAIL) {
    launch_pdl(k_mg_tail_m, dim3(slot.n), dim3(32, 32), slot.smem, st,
               (const TailArgs<float> *)dargs, dbs, slot.n, tag, err);
  } else {
    const MgArgs *A = (const MgArgs *)dargs;
    switch (slot.tile) {
#define UBG_MULTI_TILE(ID, TX, TY, HALO, NT)                                                   \
  case ID:                                                                                     \
    launch_pdl(k_mg_m<TX, TY, HALO, true, NT>, dim3(slot.blocks), dim3(32, NT / 32),          \
               Tile<TX, TY, HALO>::smem(4), st, A, dbs, slot.n, tag, err);                     \
    break;
      UBG_MULTI_TILE(0, 112, 50, 8, 512)
      UBG_MULTI_TILE(1, 48, 16, 8, 256)
      UBG_MULTI_TILE(2, 40, 8, 12, 256)
      UBG_MULTI_TILE(3, 112, 24, 8, 256)
      UBG_MULTI_TILE(4, 48, 40, 8, 256)
      UBG_MULTI_TILE(5, 112, 114, 8, 1024)
#undef UBG_MULTI_TILE
      default:
        throw ArgError("fused batch: smoother tile id");
    }
  }
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

void mg_set_h(MgHier &mg, float h0) {
  float hh = h0;
  for (int l = 0; l < mg.levels; l++) {
    mg.lv[l].hh = hh;
    if (l + 1 < mg.levels)
      hh = hh * ((float)mg.lv[l].w - 1.0f) / ((float)mg.lv[l + 1].w - 1.0f);
  }
}

void level_rbgs(MgLevel &L, int &cur, float alpha, cudaStream_t st) {
  ProfScope ps_(KC_SMOOTH_L0, st);
  init_kernel_attributes();
  MgArgs a = level_args(L, L.e[cur], L.e[1 - cur], 1, alpha);
  launch_mg_t<56, 24, 4, false>(a, st);
  cur = 1 - cur;
}

void level_residual(const MgLevel &L, int cur, float *r, double *norm2, cudaStream_t st) {
  ProfScope ps_(KC_RESIDUAL, st);
  dim3 grid((L.w + 31) / 32, (L.h + 7) / 8);
  float ihsq = 1.0f / L.hh / L.hh;
  k_residual<<<grid, dim3(32, 8), 0, st>>>(L.e[cur], L.rhs, L.flag, L.w, L.h, L.pitch, ihsq, r,
                                           norm2);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}


// ------------------------------------------- tolerance-solver hierarchy
// The tolerance solver (k_krylov.cu) preconditions its Krylov loop with a
// V-cycle of its own hierarchy, built for convergence rather than for
// parity with MG::solveLevel:
//  * level sizes floor(w/2)+1, so coarse cell X sits over fine cell 2X for
//    every interior fine cell up to the last one and coarse edges sit over
//    fine edges (the reference's floor(w/2) leaves the last fine columns
//    and rows without a coarse cell);
//  * spacing doubles exactly per level;
//  * a coarse cell is fluid if any of the nine fine cells of its
//    full-weighting stencil is (the reference keeps it only above a
//    weighted fraction of 0.2, which closes narrow gaps on coarse levels);
//    coarse edge cells are fluid, as in the reference;
//  * zero-gradient edges (corners included) on every level, so every level
//    solves the zero-gradient system; no zero columns / rows in the
//    prolongation;
//  * the last level is the coarsest, with 40 sweeps.
namespace {
std::vector<MgLevel> ext_shapes(int W, int H, float h0) {
  std::vector<MgLevel> lv;
  int w = W, h = H;
  float hh = h0;
  for (;;) {
    MgLevel L{};
    L.w = w;
    L.h = h;
    L.pitch = round_up(w, 32);
    L.hh = hh;
    lv.push_back(L);
    const int nw = w / 2 + 1, nh = h / 2 + 1;
    if (nw < 5 || nh < 5 || nw >= w || nh >= h) break;
    w = nw;
    h = nh;
    hh = 2.0f * hh;
  }
  if (lv.size() < 2) throw ArgError("grid too small for the tolerance solver (need W, H >= 8)");
  return lv;
}

// Coarse flags of the tolerance hierarchy: interior cell (X, Y) is fluid if
// any fine cell (2X + dx, 2Y + dy), |dx|, |dy| <= 1, is; edge cells are 1.
__global__ void k_coarsen_ext(const uint8_t *__restrict__ f, int fp, uint8_t *fc, int cw, int ch,
                              int cp) {
  const int X = blockIdx.x * 32 + threadIdx.x, Y = blockIdx.y * 8 + threadIdx.y;
  if (X >= cw || Y >= ch) return;
  uint8_t v = 1;
  if (X >= 1 && X < cw - 1 && Y >= 1 && Y < ch - 1) {
    unsigned any = 0;
#pragma unroll
    for (int dy = -1; dy <= 1; dy++)
#pragma unroll
      for (int dx = -1; dx <= 1; dx++) any |= __ldg(f + (size_t)(2 * Y + dy) * fp + 2 * X + dx);
    v = any ? 1 : 0;
  }
  fc[(size_t)Y * cp + X] = v;
}

template <class S>
void ext_fill_common(MgArgsT<S> &a) {
  for (int k = 0; k < 5; k++) {
    a.wsum[k] = (float)((double)(float)k + 0.0001);
    a.rwsum[k] = 1.0f / a.wsum[k];
  }
  a.alpha = 1.0f;
  a.tile = -1;
  a.ext = 1;
  a.zgbc = 1;
}

// Level l >= 1 of the tolerance hierarchy: FP32 arrays of mg (unscaled
// form) or the 16-bit arrays of lo (h^2-scaled form: hh = 1, restriction
// weight (1/16) (h_c / h)^2 = 1/4 because the spacing doubles).
template <class SC>
MgArgsT<SC> ext_level_args(MgHier &mg, MgLow *lo, int l, int cin, int ns) {
  constexpr bool scaled = !std::is_same<SC, float>::value;
  MgLevel &L = mg.lv[l];
  MgArgsT<SC> a{};
  if (scaled) {
    a.in = (const SC *)lo->e[cin][l];
    a.out = (SC *)lo->e[1 - cin][l];
    a.rhs = (const SC *)lo->rhs[l];
  } else {
    a.in = (const SC *)L.e[cin];
    a.out = (SC *)L.e[1 - cin];
    a.rhs = (const SC *)L.rhs;
  }
  a.code = L.code;
  a.w = L.w;
  a.h = L.h;
  a.pitch = L.pitch;
  a.hh = scaled ? 1.0f : L.hh;
  a.ihsq = scaled ? 1.0f : 1.0f / L.hh / L.hh;
  a.nsweeps = ns;
  a.rfac = scaled ? 0.25f : 1.0f / 16.0f;
  ext_fill_common(a);
  return a;
}

template <class SC>
void ext_vcycle_t(MgHier &mg, MgLow *lo, const unsigned *scale_bits, cudaStream_t st) {
  constexpr bool scaled = !std::is_same<SC, float>::value;
  const int T = mg.tail_top;
  if (T < 1) throw ArgError("tolerance hierarchy without a coarse tail");
  auto arr = [&](int l, int c) -> SC * {
    return scaled ? (SC *)lo->e[c][l] : (SC *)mg.lv[l].e[c];
  };
  auto rhs = [&](int l) -> SC * { return scaled ? (SC *)lo->rhs[l] : (SC *)mg.lv[l].rhs; };
  std::vector<int> cur(mg.levels, 0);
  MgLevel &L0 = mg.lv[0], &L1 = mg.lv[1];
  int kexp = 0;
  if (std::is_same<SC, __half>::value) {
    // e = A^-1 g stays below about max|g| * n^2 / 2 on level 1 (n = its
    // larger side); keep it below 2^14 in FP16
    double n = (double)std::max(L1.w, L1.h);
    kexp = std::max(0, (int)std::ceil(std::log2(0.5 * n * n)) - 14);
  }
  auto top_args = [&](int cin) {
    MgArgsT<float, SC> a{};
    a.in = L0.e[cin];
    a.out = L0.e[1 - cin];
    a.rhs = L0.rhs;
    a.code = L0.code;
    a.w = L0.w;
    a.h = L0.h;
    a.pitch = L0.pitch;
    a.hh = L0.hh;
    a.ihsq = 1.0f / L0.hh / L0.hh;
    a.nsweeps = 3;
    a.rfac = 1.0f / 16.0f;
    for (int k = 0; k < 5; k++) {
      a.wsum[k] = (float)((double)(float)k + 0.0001);
      a.rwsum[k] = 1.0f / a.wsum[k];
    }
    a.alpha = 1.0f;
    a.tile = -1;
    a.ext = 1;
    a.zgbc = 1;
    a.cw = L1.w;
    a.ch = L1.h;
    a.cpitch = L1.pitch;
    if (scaled) {
      a.scale_bits = scale_bits;
      a.scale_h1sq = L1.hh * L1.hh;
      a.scale_kexp = kexp;
    }
    return a;
  };
  auto launch_top = [&](const MgArgsT<float, SC> &a) {
    ProfScope ps_(KC_SMOOTH_L0, st);
    if constexpr (scaled)
      launch_mg_mixed_top<SC>(a, st);
    else
      launch_mg(a, st);
  };
  // down
  {
    MgArgsT<float, SC> a = top_args(0);
    a.zero_init = 1;
    a.rc = rhs(1);
    launch_top(a);
    cur[0] = 1;
  }
  for (int l = 1; l < T; l++) {
    ProfScope ps_(l == 1 ? KC_SMOOTH_L1 : KC_SMOOTH_COARSE, st);
    MgArgsT<SC> a = ext_level_args<SC>(mg, lo, l, cur[l], 3);
    a.zero_init = 1;
    a.rc = rhs(l + 1);
    a.cw = mg.lv[l + 1].w;
    a.ch = mg.lv[l + 1].h;
    a.cpitch = mg.lv[l + 1].pitch;
    launch_mg(a, st);
    cur[l] ^= 1;
  }
  {
    std::vector<float> rf(mg.levels, 0.25f);
    run_tail_t<SC, float>(mg, T, rhs(T), arr(T, 0), scaled ? rf.data() : nullptr, st);
    cur[T] = 0;
  }
  // up
  for (int l = T - 1; l >= 1; l--) {
    ProfScope ps_(l == 1 ? KC_SMOOTH_L1 : KC_SMOOTH_COARSE, st);
    MgArgsT<SC> a = ext_level_args<SC>(mg, lo, l, cur[l], 3);
    a.ec = arr(l + 1, cur[l + 1]);
    a.codec = mg.lv[l + 1].code;
    a.cpitch = mg.lv[l + 1].pitch;
    a.cw = mg.lv[l + 1].w;
    a.ch = mg.lv[l + 1].h;
    launch_mg(a, st);
    cur[l] ^= 1;
  }
  {
    MgArgsT<float, SC> a = top_args(cur[0]);
    a.ec = arr(1, cur[1]);
    a.codec = L1.code;
    launch_top(a);
    cur[0] ^= 1;
  }
  mg.cur0 = cur[0];
}
}  // namespace

size_t ext_hier_bytes(int W, int H) {
  size_t total = 512;
  for (auto &L : ext_shapes(W, H, 1.0f)) {
    size_t n = (size_t)L.pitch * L.h;
    total += 3 * align256(n * 4) + 2 * align256(n);
  }
  return total;
}

void ext_hier_alloc(MgHier &mg, int W, int H, float h0) {
  mg_free(mg);
  std::vector<MgLevel> lv = ext_shapes(W, H, h0);
  init_kernel_attributes();
  size_t total = ext_hier_bytes(W, H);
  void *arena = nullptr;
  if (cudaMalloc(&arena, total) != cudaSuccess) {
    cudaGetLastError();
    throw std::bad_alloc();
  }
  UBG_CUDA(cudaMemsetAsync(arena, 0, total, cudaStreamLegacy));
  UBG_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
  char *p = (char *)arena;
  for (auto &L : lv) {
    size_t n = (size_t)L.pitch * L.h;
    L.e[0] = (float *)p;
    p += align256(n * 4);
    L.e[1] = (float *)p;
    p += align256(n * 4);
    L.rhs = (float *)p;
    p += align256(n * 4);
    L.flag = (uint8_t *)p;
    p += align256(n);
    L.code = (uint8_t *)p;
    p += align256(n);
  }
  mg.norm = (double *)p;
  mg.post_norm2 = nullptr;
  mg.ext = true;
  mg.ncoarse = 16;
  mg.lv = lv;
  mg.levels = (int)lv.size();
  mg.tail_top = choose_tail(lv, 4096, 4, mg.levels - 1);
  if (mg.tail_top < 1) mg.tail_top = mg.levels - 1;
  mg.tail_top_fp64 = -1;
  mg.arena = arena;
  mg.arena_bytes = total;
  mg.cur0 = 0;
}

void ext_hier_update_fields(MgHier &mg, const uint8_t *flag0, int pitch0, cudaStream_t st) {
  ProfScope ps_(KC_COARSEN, st);
  MgLevel &L0 = mg.lv[0];
  UBG_CUDA(cudaMemcpy2DAsync(L0.flag, L0.pitch, flag0, pitch0, L0.w, L0.h,
                             cudaMemcpyDeviceToDevice, st));
  for (int l = 1; l < mg.levels; l++) {
    MgLevel &F = mg.lv[l - 1], &C = mg.lv[l];
    dim3 grid((C.w + 31) / 32, (C.h + 7) / 8);
    k_coarsen_ext<<<grid, dim3(32, 8), 0, st>>>(F.flag, F.pitch, C.flag, C.w, C.h, C.pitch);
    UBG_LAUNCH_CHECK();
  }
  for (int l = 0; l < mg.levels; l++) level_make_code(mg.lv[l], st);
}

void ext_vcycle(MgHier &mg, MgLow *lo, int prec, const unsigned *scale_bits, cudaStream_t st) {
  if (prec == UBG_FP32)
    ext_vcycle_t<float>(mg, nullptr, nullptr, st);
  else if (prec == UBG_MIXED_FP16)
    ext_vcycle_t<__half>(mg, lo, scale_bits, st);
  else if (prec == UBG_MIXED_BF16)
    ext_vcycle_t<__nv_bfloat16>(mg, lo, scale_bits, st);
  else
    throw ArgError("precision");
}

}  // namespace ubg
