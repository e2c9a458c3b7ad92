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
//  k_residual  the residual field and its squared L2 norm.
//  k_coarsen   MG::updateFields (pressure_solver.hpp:34-57), integer exact.
//
// Red points are those with x+y odd (pressure_solver.cpp:36); a sweep updates
// all red points, then all black points, which is the reference's
// deterministic schedule.  Every kernel reads one buffer and writes another,
// so tiles never race on their halos.
#include "ubg_internal.cuh"

#include <cstdlib>
#include <cstring>

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
__device__ __forceinline__ float rb_update1(unsigned c, float pw, float pe, float ps, float pn,
                                            float f, float hh) {
  float val = 0.0f;
  val = val + ((c & C_W) ? pw : 0.0f);
  val = val + ((c & C_E) ? pe : 0.0f);
  val = val + ((c & C_S) ? ps : 0.0f);
  val = val + ((c & C_N) ? pn : 0.0f);
  val = val + f * hh * hh;
  int s = __popc((c >> 1) & 15u);
  if (s == 3)
    val = val / 3.0f;
  else
    val = val * (s == 4 ? 0.25f : (s == 2 ? 0.5f : (s == 1 ? 1.0f : 0.0f)));
  if (s == 0) val = 0.0f;
  return (c & C_CENTER) ? val : 0.0f;
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
__device__ __forceinline__ float resid1(unsigned c, float pc, float pw, float pe, float ps,
                                        float pn, float f, float ihsq) {
  float val = 0.0f;
  val = val + ((c & C_W) ? pw : pc);
  val = val + ((c & C_E) ? pe : pc);
  val = val + ((c & C_S) ? ps : pc);
  val = val + ((c & C_N) ? pn : pc);
  val = val + -4.0f * pc;
  val = val * ihsq;
  return (c & C_CENTER) ? (f + val) : 0.0f;
}

struct MgArgs {
  const float *in;
  float *out;
  const float *rhs;
  const uint8_t *code;
  int w, h, pitch;
  float hh, alpha, ihsq;
  int nsweeps, zgbc, zero_init;
  // prologue: p += prolongate(ec) (post-smoothing)
  const float *ec;
  const uint8_t *codec;
  int cpitch;
  float wsum[5];  // (float)((double)k + 0.0001)
  // epilogue: rc = restrict(residual) (pre-smoothing)
  float *rc;
  int cw, ch;
  // epilogue: sum of r^2 over the tile's interior cells
  double *norm2;
};

// prolongate (pressure_solver.cpp:134-172) at one fine interior cell whose
// own flag is set.
__device__ __forceinline__ float prolong_at(const MgArgs &a, int gx, int gy) {
  int cx = gx >> 1, cy = gy >> 1;
  const float *ec = a.ec;
  const uint8_t *fc = a.codec;
  int cp = a.cpitch;
  auto E = [&](int x, int y) { return __ldg(ec + (size_t)y * cp + x); };
  auto F = [&](int x, int y) { return (int)(__ldg(fc + (size_t)y * cp + x) & 1u); };
  bool xo = gx & 1, yo = gy & 1;
  if (!xo && !yo) return E(cx, cy);
  if (xo && !yo) {
    if (gx >= a.w - 2) return 0.0f;
    float sum = a.wsum[F(cx, cy) + F(cx + 1, cy)];
    return (E(cx, cy) + E(cx + 1, cy)) / sum;
  }
  if (!xo && yo) {
    if (gy >= a.h - 2) return 0.0f;
    float sum = a.wsum[F(cx, cy) + F(cx, cy + 1)];
    return (E(cx, cy) + E(cx, cy + 1)) / sum;
  }
  if (gx >= a.w - 2 || gy >= a.h - 2) return 0.0f;
  float sum = a.wsum[F(cx, cy) + F(cx + 1, cy + 1) + F(cx + 1, cy) + F(cx, cy + 1)];
  return (((E(cx, cy) + E(cx + 1, cy + 1)) + E(cx + 1, cy)) + E(cx, cy + 1)) / sum;
}

template <int TX, int TY, int HALO>
struct Tile {
  static constexpr int RX = TX + 2 * HALO, RY = TY + 2 * HALO, HX = RX / 2;
  // coarse window for the prolongation prologue
  static constexpr int CW = HX + 2, CH = RY / 2 + 2;
  static_assert(RX % 4 == 0 && HALO % 4 == 0 && TX % 4 == 0 && TY % 2 == 0, "tile alignment");
  static constexpr size_t smem() {
    return (size_t)2 * RY * HX * (4 + 4 + 1) + (size_t)CW * CH * 4 + ((size_t)CW * CH + 15) / 16 * 16;
  }
};

// One multigrid smoothing launch on a tile of TX x TY cells with a halo of
// HALO cells, all in shared memory in a red/black-split layout: cell (rx, ry)
// of the region lives in colour array (rx+ry)&1 at [ry][rx/2], so the four
// neighbours of a cell are consecutive entries of the other colour's rows
// (no bank conflicts).  Red = (x+y) odd; region parity equals global parity
// because x0 + y0 is even.  After half sweep i only cells within HALO - i of
// the tile are still exact, so each half sweep updates just that cone.
template <int TX, int TY, int HALO, bool ALPHA1, int NT>
__global__ void __launch_bounds__(NT, NT == 512 ? 2 : 4) k_mg(MgArgs a) {
  constexpr int NTY = NT / 32;
  using T = Tile<TX, TY, HALO>;
  constexpr int RX = T::RX, RY = T::RY, HX = T::HX;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *sp = reinterpret_cast<float *>(smem_raw);  // [2][RY][HX]
  float *sf = sp + 2 * RY * HX;
  uint8_t *sc = reinterpret_cast<uint8_t *>(sf + 2 * RY * HX);
  auto IDX = [](int rx, int ry) { return (((rx + ry) & 1) * RY + ry) * HX + (rx >> 1); };

  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  const int x0 = blockIdx.x * TX - HALO, y0 = blockIdx.y * TY - HALO;
  const int w = a.w, h = a.h, P = a.pitch;

  // ---- load p, f, code (float4 / uchar4 per thread; x0 is a multiple of 4).
  // One array at a time, all of a thread's loads of that array in flight
  // together, into the red/black-split layout.
  constexpr int NQ = RY * (RX / 4), NIT = (NQ + NT - 1) / NT;
  auto load_split = [&](const float *src, float *dst, bool zero) {
    float4 v[NIT];
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      int q = tid + it * NT;
      int ry = q / (RX / 4), g = q - ry * (RX / 4);
      int gx = x0 + 4 * g, gy = y0 + ry;
      v[it] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (!zero && q < NQ && gy >= 0 && gy < h && gx >= 0 && gx < w)
        v[it] = __ldg(reinterpret_cast<const float4 *>(src + (size_t)gy * P + gx));
    }
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      int q = tid + it * NT;
      if (q >= NQ) break;
      int ry = q / (RX / 4), g = q - ry * (RX / 4);
      int gx = x0 + 4 * g;
      float4 p4 = v[it];
      if (gx + 3 >= w) {
        if (gx + 1 >= w) p4.y = 0.f;
        if (gx + 2 >= w) p4.z = 0.f;
        p4.w = 0.f;
      }
      int c0 = ry & 1;
      *reinterpret_cast<float2 *>(dst + (c0 * RY + ry) * HX + 2 * g) = make_float2(p4.x, p4.z);
      *reinterpret_cast<float2 *>(dst + ((c0 ^ 1) * RY + ry) * HX + 2 * g) = make_float2(p4.y, p4.w);
    }
  };
  load_split(a.in, sp, a.zero_init != 0);
  load_split(a.rhs, sf, false);
  {
    uchar4 cv[NIT];
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      int q = tid + it * NT;
      int ry = q / (RX / 4), g = q - ry * (RX / 4);
      int gx = x0 + 4 * g, gy = y0 + ry;
      cv[it] = make_uchar4(0, 0, 0, 0);
      if (q < NQ && gy >= 0 && gy < h && gx >= 0 && gx < w)
        cv[it] = __ldg(reinterpret_cast<const uchar4 *>(a.code + (size_t)gy * P + gx));
    }
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      int q = tid + it * NT;
      if (q >= NQ) break;
      int ry = q / (RX / 4), g = q - ry * (RX / 4);
      int gx = x0 + 4 * g;
      uchar4 c4 = cv[it];
      if (gx + 3 >= w) {
        if (gx + 1 >= w) c4.y = 0;
        if (gx + 2 >= w) c4.z = 0;
        c4.w = 0;
      }
      int c0 = ry & 1;
      int base0 = (c0 * RY + ry) * HX + 2 * g, base1 = ((c0 ^ 1) * RY + ry) * HX + 2 * g;
      sc[base0] = c4.x;
      sc[base0 + 1] = c4.z;
      sc[base1] = c4.y;
      sc[base1 + 1] = c4.w;
    }
  }
  __syncthreads();

  // ---- prologue: correct(p, prolongate(ec)) on the interior cells, with
  // the coarse window staged in shared memory
  if (a.ec) {
    constexpr int CW = T::CW, CH = T::CH;
    float *sec = reinterpret_cast<float *>(sc + 2 * RY * HX);
    uint8_t *scf = reinterpret_cast<uint8_t *>(sec + CW * CH);
    const int cxa = x0 >> 1, cya = y0 >> 1;
    for (int q = tid; q < CW * CH; q += NT) {
      int ly = q / CW, lx = q - ly * CW;
      int cx = cxa + lx, cy = cya + ly;
      float e = 0.0f;
      uint8_t fc = 0;
      if (cx >= 0 && cx < a.cw && cy >= 0 && cy < a.ch) {
        e = __ldg(a.ec + (size_t)cy * a.cpitch + cx);
        fc = __ldg(a.codec + (size_t)cy * a.cpitch + cx) & 1u;
      }
      sec[q] = e;
      scf[q] = fc;
    }
    __syncthreads();
#pragma unroll
    for (int color = 0; color < 2; color++) {
      for (int ry = ty; ry < RY; ry += NTY) {
        const int par = (ry + color) & 1;
        const int gy = y0 + ry;
        if (gy < 1 || gy >= h - 1) continue;
        for (int k = tx; k < HX; k += 32) {
          int rx = 2 * k + par, gx = x0 + rx;
          int i = (color * RY + ry) * HX + k;
          if (gx < 1 || gx >= w - 1 || !(sc[i] & C_CENTER)) continue;
          // prolongate (pressure_solver.cpp:134-172); e * fine flag = e here
          const float *E = sec + (ry >> 1) * CW + (rx >> 1);
          const uint8_t *F = scf + (ry >> 1) * CW + (rx >> 1);
          bool xo = gx & 1, yo = gy & 1;
          float ev;
          if (!xo && !yo) {
            ev = E[0];
          } else if (xo && !yo) {
            ev = (gx >= w - 2) ? 0.0f : (E[0] + E[1]) / a.wsum[F[0] + F[1]];
          } else if (!xo && yo) {
            ev = (gy >= h - 2) ? 0.0f : (E[0] + E[CW]) / a.wsum[F[0] + F[CW]];
          } else {
            ev = (gx >= w - 2 || gy >= h - 2)
                     ? 0.0f
                     : (((E[0] + E[CW + 1]) + E[1]) + E[CW]) / a.wsum[F[0] + F[CW + 1] + F[1] + F[CW]];
          }
          sp[i] = sp[i] + ev;
        }
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
  };
  if (a.zgbc && edge && a.ec) {
    zero_gradient();
    __syncthreads();
  }

  // ---- red-black sweeps: a thread updates 4 consecutive cells of one colour
  // in one row (128-bit shared-memory accesses); G threads cover a row.
  constexpr int G = HX / 4, RPP = NT / G;
  static_assert(HX % 4 == 0 && NT % G == 0, "vector layout");
  const int k0 = 4 * (tid % G), rsub = tid / G;
  const float hh = a.hh;
  const bool inner = x0 >= 1 && y0 >= 1 && x0 + RX <= w - 1 && y0 + RY <= h - 1;
  // which of the thread's 4 cells may be smoothed (both parities):
  // k >= 1 - par and k <= HX - 1 - par keep all neighbours in the region
  auto cell_ok = [&](int k, int par, int gy) {
    bool ok = k >= 1 - par && k <= HX - 1 - par;
    if (!inner) {
      int gx = x0 + 2 * k + par;
      ok = ok && gx >= 1 && gx < w - 1 && gy >= 1 && gy < h - 1;
    }
    return ok;
  };
  int half = 0;
  for (int s = 0; s < a.nsweeps; s++) {
#pragma unroll
    for (int color = 1; color >= 0; color--) {
      half++;
      float *self = sp + color * RY * HX;
      const float *oth = sp + (color ^ 1) * RY * HX;
      const float *fs = sf + color * RY * HX;
      const uint8_t *cs = sc + color * RY * HX;
      for (int ry = half + rsub; ry <= RY - 1 - half; ry += RPP) {
        const int par = (ry + color) & 1;
        const int gy = y0 + ry;
        const int row = ry * HX + k0;
        const float4 o = *reinterpret_cast<const float4 *>(oth + row);
        const float ex = par ? oth[row + 4] : oth[row - 1];
        const float4 os = *reinterpret_cast<const float4 *>(oth + row - HX);
        const float4 on = *reinterpret_cast<const float4 *>(oth + row + HX);
        const float4 fv = *reinterpret_cast<const float4 *>(fs + row);
        const float4 sv = *reinterpret_cast<const float4 *>(self + row);
        const uchar4 cv = *reinterpret_cast<const uchar4 *>(cs + row);
        const float W4[4] = {par ? o.x : ex, par ? o.y : o.x, par ? o.z : o.y, par ? o.w : o.z};
        const float E4[4] = {par ? o.y : o.x, par ? o.z : o.y, par ? o.w : o.z, par ? ex : o.w};
        const float S4[4] = {os.x, os.y, os.z, os.w}, N4[4] = {on.x, on.y, on.z, on.w};
        const float F4[4] = {fv.x, fv.y, fv.z, fv.w}, P4[4] = {sv.x, sv.y, sv.z, sv.w};
        const unsigned C4[4] = {cv.x, cv.y, cv.z, cv.w};
        float out[4];
        if (ALPHA1) {
          const unsigned all = (unsigned)cv.x | ((unsigned)cv.y << 8) | ((unsigned)cv.z << 16) |
                               ((unsigned)cv.w << 24);
          // warp-uniform choice: all-fluid neighbourhoods take val / 4
          if (__all_sync(__activemask(), all == 0x1f1f1f1fu)) {
#pragma unroll
            for (int j = 0; j < 4; j++)
              out[j] = ((((W4[j] + E4[j]) + S4[j]) + N4[j]) + F4[j] * hh * hh) * 0.25f;
          } else {
#pragma unroll
            for (int j = 0; j < 4; j++) out[j] = rb_update1(C4[j], W4[j], E4[j], S4[j], N4[j], F4[j], hh);
          }
        } else {
#pragma unroll
          for (int j = 0; j < 4; j++)
            out[j] = rb_update_alpha(C4[j], P4[j], W4[j], E4[j], S4[j], N4[j], F4[j], hh, a.alpha);
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (!cell_ok(k0 + j, par, gy)) out[j] = P4[j];
        *reinterpret_cast<float4 *>(self + row) = make_float4(out[0], out[1], out[2], out[3]);
      }
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
    float2 u = *reinterpret_cast<const float2 *>(sp + b0);
    float2 v = *reinterpret_cast<const float2 *>(sp + b1);
    float4 o = make_float4(u.x, v.x, u.y, v.y);
    float *dst = a.out + (size_t)gy * P + gx;
    if (gx + 3 < w) {
      *reinterpret_cast<float4 *>(dst) = o;
    } else {
      dst[0] = o.x;
      if (gx + 1 < w) dst[1] = o.y;
      if (gx + 2 < w) dst[2] = o.z;
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
    const float *self = sp + color * RY * HX;
    const float *oth = sp + (color ^ 1) * RY * HX;
    float *fs = sf + color * RY * HX;
    const uint8_t *cs = sc + color * RY * HX;
    for (int ry = rlo + rsub; ry <= rhiy; ry += RPP) {
      const int par = (ry + color) & 1;
      const int gy = y0 + ry;
      const int row = ry * HX + k0;
      const float4 o = *reinterpret_cast<const float4 *>(oth + row);
      const float ex = par ? oth[row + 4] : oth[row - 1];
      const float4 os = *reinterpret_cast<const float4 *>(oth + row - HX);
      const float4 on = *reinterpret_cast<const float4 *>(oth + row + HX);
      const float4 fv = *reinterpret_cast<const float4 *>(fs + row);
      const float4 sv = *reinterpret_cast<const float4 *>(self + row);
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
      if (a.rc) *reinterpret_cast<float4 *>(fs + row) = make_float4(out[0], out[1], out[2], out[3]);
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
    const int cx0 = blockIdx.x * (TX / 2), cy0 = blockIdx.y * (TY / 2);
    for (int q = tid; q < (TX / 2) * (TY / 2); q += NT) {
      int cyy = q / (TX / 2), cxx = q - cyy * (TX / 2);
      int X = cx0 + cxx, Y = cy0 + cyy;
      if (X >= a.cw || Y >= a.ch) continue;
      float v = 0.0f;
      if (X >= 1 && X < a.cw - 1 && Y >= 1 && Y < a.ch - 1) {
        int rx = 2 * X - x0, ry = 2 * Y - y0;
        auto R = [&](int dx, int dy) { return sf[IDX(rx + dx, ry + dy)]; };
        v = (R(-1, -1) * 1.0f + R(0, -1) * 2.0f) + R(1, -1) * 1.0f;
        v = v + ((R(-1, 0) * 2.0f + R(0, 0) * 4.0f) + R(1, 0) * 2.0f);
        v = v + ((R(-1, 1) * 1.0f + R(0, 1) * 2.0f) + R(1, 1) * 1.0f);
        v = v * (1.0f / 16.0f);
      }
      a.rc[(size_t)Y * a.cpitch + X] = v;
    }
  }
}

// ------------------------------------------------------ residual field only
__global__ void k_residual(const float *__restrict__ p, const float *__restrict__ rhs,
                           const uint8_t *__restrict__ flag, int w, int h, int P, float ihsq,
                           float *r, double *norm2) {
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
  float hh, ihsq;
  int oe, orr, orhs, oc;  // offsets: floats for e / r / rhs, bytes for code
};
struct TailArgs {
  int nlev;
  TailLevel L[TAIL_MAXL];
  const uint8_t *code[TAIL_MAXL];
  int code_pitch[TAIL_MAXL];
  const float *rhs_top;
  int rhs_pitch;
  float *e_top;
  int e_pitch;
  int float_words;  // size of the float part of shared memory
  float wsum[5];
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

__global__ void __launch_bounds__(TAIL_THREADS, 1) k_mg_tail(TailArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *fm = reinterpret_cast<float *>(smem_raw);
  uint8_t *bm = smem_raw + (size_t)a.float_words * 4;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  const int nl = a.nlev;
  const float ws0 = a.wsum[0], ws1 = a.wsum[1], ws2 = a.wsum[2], ws3 = a.wsum[3], ws4 = a.wsum[4];
  auto WS = [&](int k) {
    return k == 0 ? ws0 : (k == 1 ? ws1 : (k == 2 ? ws2 : (k == 3 ? ws3 : ws4)));
  };
  auto team_of = [&](int t) {
    (void)t;
    return TAIL_THREADS;
  };

  for (int t = 0; t < nl; t++) {
    const TailLevel &L = a.L[t];
    for (int y = ty; y < L.h; y += 32)
      for (int x = tx; x < L.w; x += 32) {
        int q = y * L.w + x;
        bm[L.oc + q] = a.code[t][(size_t)y * a.code_pitch[t] + x];
        fm[L.oe + q] = 0.0f;
        if (t == 0) fm[L.orhs + q] = a.rhs_top[(size_t)y * a.rhs_pitch + x];
      }
  }
  __syncthreads();

  auto sweeps = [&](int t, int ns, int team) {
    const TailLevel &L = a.L[t];
    float *e = fm + L.oe;
    const float *f = fm + L.orhs;
    const uint8_t *c = bm + L.oc;
    const int w = L.w, hw2 = (w + 1) / 2, ystep = team / 32;
    const float hh = L.hh;
    for (int s = 0; s < ns; s++) {
      for (int color = 1; color >= 0; color--) {
        for (int y = 1 + ty; y < L.h - 1; y += ystep) {
          int par = (y + color) & 1;
          for (int j = tx; j < hw2; j += 32) {
            int x = 2 * j + par;
            if (x < 1 || x >= w - 1) continue;
            int i = y * w + x;
            unsigned ci = c[i];
            float pw = e[i - 1], pe = e[i + 1], ps = e[i - w], pn = e[i + w], fi = f[i];
            if (__all_sync(__activemask(), ci == (C_CENTER | C_W | C_E | C_S | C_N)))
              e[i] = ((((pw + pe) + ps) + pn) + fi * hh * hh) * 0.25f;
            else
              e[i] = rb_update1(ci, pw, pe, ps, pn, fi, hh);
          }
        }
        team_sync(team);
      }
    }
  };

  // down
  for (int t = 0; t < nl; t++) {
    const int team = team_of(t);
    if (tid >= team) continue;
    const int ystep = team / 32;
    if (t == nl - 1) {
      sweeps(t, 5, team);
      break;
    }
    sweeps(t, 3, team);
    const TailLevel &L = a.L[t], &C = a.L[t + 1];
    float *e = fm + L.oe, *r = fm + L.orr;
    const float *f = fm + L.orhs;
    const uint8_t *c = bm + L.oc;
    for (int y = ty; y < L.h; y += ystep)
      for (int x = tx; x < L.w; x += 32) {
        int q = y * L.w + x;
        float rv = 0.0f;
        if (x >= 1 && x < L.w - 1 && y >= 1 && y < L.h - 1)
          rv = resid1(c[q], e[q], e[q - 1], e[q + 1], e[q - L.w], e[q + L.w], f[q], L.ihsq);
        r[q] = rv;
      }
    team_sync(team);
    float *rc = fm + C.orhs;
    for (int Y = ty; Y < C.h; Y += ystep)
      for (int X = tx; X < C.w; X += 32) {
        float v = 0.0f;
        if (X >= 1 && X < C.w - 1 && Y >= 1 && Y < C.h - 1) {
          const float *R0 = r + (2 * Y) * L.w + 2 * X;
          v = (R0[-L.w - 1] * 1.0f + R0[-L.w] * 2.0f) + R0[-L.w + 1] * 1.0f;
          v = v + ((R0[-1] * 2.0f + R0[0] * 4.0f) + R0[1] * 2.0f);
          v = v + ((R0[L.w - 1] * 1.0f + R0[L.w] * 2.0f) + R0[L.w + 1] * 1.0f);
          v = v * (1.0f / 16.0f);
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
    float *e = fm + L.oe;
    const float *ec = fm + C.oe;
    const uint8_t *c = bm + L.oc, *cc = bm + C.oc;
    for (int y = 1 + ty; y < L.h - 1; y += ystep)
      for (int x = 1 + tx; x < L.w - 1; x += 32) {
        int q = y * L.w + x;
        if (!(c[q] & C_CENTER)) continue;
        int cx = x >> 1, cy = y >> 1;
        auto E = [&](int xx, int yy) { return ec[yy * C.w + xx]; };
        auto F = [&](int xx, int yy) { return (int)(cc[yy * C.w + xx] & 1u); };
        bool xo = x & 1, yo = y & 1;
        float ev;
        if (!xo && !yo)
          ev = E(cx, cy);
        else if (xo && !yo)
          ev = (x >= L.w - 2) ? 0.0f : (E(cx, cy) + E(cx + 1, cy)) / WS(F(cx, cy) + F(cx + 1, cy));
        else if (!xo && yo)
          ev = (y >= L.h - 2) ? 0.0f : (E(cx, cy) + E(cx, cy + 1)) / WS(F(cx, cy) + F(cx, cy + 1));
        else
          ev = (x >= L.w - 2 || y >= L.h - 2)
                   ? 0.0f
                   : (((E(cx, cy) + E(cx + 1, cy + 1)) + E(cx + 1, cy)) + E(cx, cy + 1)) /
                         WS(F(cx, cy) + F(cx + 1, cy + 1) + F(cx + 1, cy) + F(cx, cy + 1));
        e[q] = e[q] + ev;
      }
    team_sync(team);
    sweeps(t, 3, team);
  }
  __syncthreads();
  const TailLevel &L0 = a.L[0];
  for (int y = ty; y < L0.h; y += 32)
    for (int x = tx; x < L0.w; x += 32) a.e_top[(size_t)y * a.e_pitch + x] = fm[L0.oe + y * L0.w + x];
}

// ------------------------------------------------------------ launches
template <int TX, int TY, int HALO, bool A1, int NT = 256>
void launch_mg_t(const MgArgs &a, cudaStream_t st) {
  using T = Tile<TX, TY, HALO>;
  dim3 grid((a.w + TX - 1) / TX, (a.h + TY - 1) / TY);
  k_mg<TX, TY, HALO, A1, NT><<<grid, dim3(32, NT / 32), T::smem(), st>>>(a);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

template <int TX, int TY, int HALO, bool A1, int NT = 256>
void set_smem_attr() {
  UBG_CUDA(cudaFuncSetAttribute(k_mg<TX, TY, HALO, A1, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)Tile<TX, TY, HALO>::smem()));
  // one carveout for every kernel of a V-cycle: no L1 / shared-memory
  // reconfiguration between consecutive launches
  UBG_CUDA(cudaFuncSetAttribute(k_mg<TX, TY, HALO, A1, NT>,
                                cudaFuncAttributePreferredSharedMemoryCarveout, 100));
}

void init_kernel_attributes() {
  static bool done = false;
  if (done) return;
  set_smem_attr<112, 50, 8, true, 512>();
  set_smem_attr<48, 16, 8, true>();
  set_smem_attr<40, 8, 12, true>();
  set_smem_attr<56, 24, 4, false>();
  UBG_CUDA(cudaFuncSetAttribute(k_mg_tail, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TAIL_SMEM_MAX));
  UBG_CUDA(cudaFuncSetAttribute(k_mg_tail, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  done = true;
}

// 3 sweeps with an optional restriction epilogue need HALO >= 8; the tile
// is chosen by level width so small levels still fill the GPU.
void launch_mg(const MgArgs &a, cudaStream_t st) {
  if (!ALPHA_IS_ONE(a.alpha) || a.nsweeps == 1) {
    if (a.nsweeps != 1) throw ArgError("general alpha: one sweep per launch");
    launch_mg_t<56, 24, 4, false>(a, st);
  } else if (a.nsweeps <= 3) {
    if (a.w >= 1200)
      launch_mg_t<112, 50, 8, true, 512>(a, st);
    else
      launch_mg_t<48, 16, 8, true>(a, st);
  } else if (a.nsweeps <= 5) {
    launch_mg_t<40, 8, 12, true>(a, st);
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
  for (int k = 0; k < 5; k++) a.wsum[k] = (float)((double)(float)k + 0.0001);
  return a;
}

void run_tail(MgHier &mg, int lt, cudaStream_t st) {
  ProfScope ps_(KC_TAIL, st);
  TailArgs a{};
  int nl = mg.levels - 1 - lt;
  a.nlev = nl;
  size_t fw = 0, bw = 0;
  for (int t = 0; t < nl; t++) {
    MgLevel &L = mg.lv[lt + t];
    TailLevel &T = a.L[t];
    int n = L.w * L.h;
    T.w = L.w;
    T.h = L.h;
    T.hh = L.hh;
    T.ihsq = 1.0f / L.hh / L.hh;
    T.oe = (int)fw;
    fw += (n + 3) / 4 * 4;
    T.orr = (int)fw;
    fw += (n + 3) / 4 * 4;
    T.orhs = (int)fw;
    fw += (n + 3) / 4 * 4;
    T.oc = (int)bw;
    bw += (n + 15) / 16 * 16;
    a.code[t] = L.code;
    a.code_pitch[t] = L.pitch;
  }
  a.float_words = (int)fw;
  MgLevel &top = mg.lv[lt];
  a.rhs_top = top.rhs;
  a.rhs_pitch = top.pitch;
  a.e_top = top.e[0];
  a.e_pitch = top.pitch;
  for (int k = 0; k < 5; k++) a.wsum[k] = (float)((double)(float)k + 0.0001);
  size_t smem = fw * 4 + bw;
  k_mg_tail<<<1, dim3(32, 32), smem, st>>>(a);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

// MG::solveLevel, pressure_solver.cpp:201-248.
void solve_level(MgHier &mg, std::vector<int> &cur, int l, bool zgbc, cudaStream_t st) {
  bool bc = zgbc && l == 0;
  MgLevel &L = mg.lv[l];
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

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

int choose_tail(const std::vector<MgLevel> &lv) {
  int L = (int)lv.size();
  for (int lt = 1; lt <= L - 2; lt++) {
    size_t bytes = 0;
    for (int t = lt; t <= L - 2; t++) {
      size_t n = (size_t)lv[t].w * lv[t].h;
      bytes += 3 * ((n + 3) / 4 * 4) * 4 + (n + 15) / 16 * 16;
    }
    if (bytes <= TAIL_SMEM_MAX && (size_t)lv[lt].w * lv[lt].h <= 2048) return lt;
  }
  return -1;
}

}  // namespace

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
  mg.tail_top = choose_tail(lv);
  mg.lv = lv;
  mg.levels = (int)lv.size();
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
  UBG_CUDA(cudaMemset(arena, 0, total));
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

}  // namespace ubg
