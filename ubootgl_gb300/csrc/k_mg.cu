// Multigrid pressure solver (class MG, pressure_solver.{hpp,cpp} of
// te42kyfo/ubootgl) on the GPU.
//
//  k_smooth          red-black Gauss-Seidel (rbgs + smoothingKernel,
//                    pressure_solver.cpp:10-24, 35-89), NS sweeps temporally
//                    blocked in shared memory; optional prologue that applies
//                    prolongate + correct (pressure_solver.cpp:134-181) and
//                    optional zero-gradient boundary after every sweep
//                    (setZeroGradientBC, pressure_solver.cpp:183-192).
//  k_resid_restrict  calculateResidualField + restrict fused
//                    (pressure_solver.cpp:91-132); the fine residual never
//                    goes to memory.
//  k_residual        the residual field and its squared L2 norm.
//  k_coarsen         MG::updateFields (pressure_solver.hpp:34-57), integer
//                    exact.
//
// Red points are those with x+y odd (pressure_solver.cpp:36); a sweep updates
// all red points, then all black points, which is the reference's
// deterministic schedule.  Every kernel reads one buffer and writes another,
// so tiles never race on their halos.
#include "ubg_internal.cuh"

#include <cstring>

namespace ubg {
namespace {

struct ProlongArgs {
  const float *ec;       // coarse error (level l+1), null = no prolongation
  const uint8_t *flagc;  // coarse flag
  int cpitch;
  float wsum[5];         // (float)((double)k + 0.0001), k = 0..4
};

struct SmoothArgs {
  const float *in;
  float *out;
  const float *rhs;
  const uint8_t *flag;
  int w, h, pitch;
  float hh;
  float alpha;
  int nsweeps;
  int zgbc;
  int zero_init;
  ProlongArgs pr;
};

template <int TX, int TY, int HALO>
struct SmoothTile {
  static constexpr int RX = TX + 2 * HALO;
  static constexpr int RY = TY + 2 * HALO;
  static constexpr size_t smem() { return (size_t)RX * RY * (4 + 4 + 1); }
};

// prolongate (pressure_solver.cpp:134-172) evaluated at one fine cell.
__device__ __forceinline__ float prolong_at(const ProlongArgs &pr, int gx, int gy, int w, int h,
                                            float fine) {
  int cx = gx >> 1, cy = gy >> 1;
  const float *ec = pr.ec;
  const uint8_t *fc = pr.flagc;
  int cp = pr.cpitch;
  auto E = [&](int x, int y) { return __ldg(ec + (size_t)y * cp + x); };
  auto F = [&](int x, int y) { return (int)__ldg(fc + (size_t)y * cp + x); };
  bool xo = gx & 1, yo = gy & 1;
  if (!xo && !yo) return E(cx, cy) * fine;
  if (xo && !yo) {
    if (gx >= w - 2) return 0.0f;
    float sum = pr.wsum[F(cx, cy) + F(cx + 1, cy)];
    return fine * (E(cx, cy) + E(cx + 1, cy)) / sum;
  }
  if (!xo && yo) {
    if (gy >= h - 2) return 0.0f;
    float sum = pr.wsum[F(cx, cy) + F(cx, cy + 1)];
    return fine * (E(cx, cy) + E(cx, cy + 1)) / sum;
  }
  if (gx >= w - 2 || gy >= h - 2) return 0.0f;
  float sum = pr.wsum[F(cx, cy) + F(cx + 1, cy + 1) + F(cx + 1, cy) + F(cx, cy + 1)];
  return fine * (((E(cx, cy) + E(cx + 1, cy + 1)) + E(cx + 1, cy)) + E(cx, cy + 1)) / sum;
}

template <int TX, int TY, int HALO>
__global__ void __launch_bounds__(256) k_smooth(SmoothArgs a) {
  using T = SmoothTile<TX, TY, HALO>;
  constexpr int RX = T::RX, RY = T::RY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *sp = reinterpret_cast<float *>(smem_raw);
  float *sf = sp + RX * RY;
  uint8_t *sfl = reinterpret_cast<uint8_t *>(sf + RX * RY);

  const int tid = threadIdx.x, nt = blockDim.x;
  const int x0 = blockIdx.x * TX - HALO, y0 = blockIdx.y * TY - HALO;
  const int w = a.w, h = a.h, P = a.pitch;

  for (int i = tid; i < RX * RY; i += nt) {
    int ry = i / RX, rx = i - ry * RX;
    int gx = x0 + rx, gy = y0 + ry;
    bool in = gx >= 0 && gx < w && gy >= 0 && gy < h;
    size_t gi = (size_t)gy * P + gx;
    float pv = 0.0f, fv = 0.0f;
    uint8_t flv = 0;
    if (in) {
      if (!a.zero_init) pv = __ldg(a.in + gi);
      fv = __ldg(a.rhs + gi);
      flv = __ldg(a.flag + gi);
    }
    if (a.pr.ec && in && gx >= 1 && gx < w - 1 && gy >= 1 && gy < h - 1)
      pv = pv + prolong_at(a.pr, gx, gy, w, h, (float)flv);
    sp[i] = pv;
    sf[i] = fv;
    sfl[i] = flv;
  }
  __syncthreads();

  auto zero_gradient = [&]() {
    // setZeroGradientBC on the cells of this region (corners untouched).
    for (int i = tid; i < RX * RY; i += nt) {
      int ry = i / RX, rx = i - ry * RX;
      int gx = x0 + rx, gy = y0 + ry;
      if (gy >= 1 && gy < h - 1) {
        if (gx == 0 && rx + 1 < RX) sp[i] = sp[i + 1];
        if (gx == w - 1 && rx >= 1) sp[i] = sp[i - 1];
      }
      if (gx >= 1 && gx < w - 1) {
        if (gy == 0 && ry + 1 < RY) sp[i] = sp[i + RX];
        if (gy == h - 1 && ry >= 1) sp[i] = sp[i - RX];
      }
    }
  };
  if (a.zgbc && a.pr.ec) {
    zero_gradient();
    __syncthreads();
  }

  const float hh = a.hh, alpha = a.alpha;
  constexpr int HALFW = (RX - 2) / 2;
  constexpr int NCELL = (RY - 2) * HALFW;
  for (int s = 0; s < a.nsweeps; s++) {
#pragma unroll
    for (int color = 1; color >= 0; color--) {  // red (x+y odd) first, then black
      for (int k = tid; k < NCELL; k += nt) {
        int ry = 1 + k / HALFW;
        int j = k - (ry - 1) * HALFW;
        int off = color ? (ry & 1) : ((ry + 1) & 1);
        int rx = 1 + 2 * j + off;
        int gx = x0 + rx, gy = y0 + ry;
        if (gx < 1 || gx >= w - 1 || gy < 1 || gy >= h - 1) continue;
        int i = ry * RX + rx;
        float fw = (float)sfl[i - 1], fe = (float)sfl[i + 1];
        float fs = (float)sfl[i - RX], fn = (float)sfl[i + RX];
        float sum = 0.0f;
        sum = sum + (fw + fe + fn + fs);
        float val = 0.0f;
        val = val + sp[i - 1] * fw;
        val = val + sp[i + 1] * fe;
        val = val + sp[i - RX] * fs;
        val = val + sp[i + RX] * fn;
        val = val + sf[i] * hh * hh;
        val = val / sum;
        if (sum == 0.0f) val = 0.0f;
        sp[i] = (float)sfl[i] * (alpha * val + (1.0f - alpha) * sp[i]);
      }
      __syncthreads();
    }
    if (a.zgbc) {
      zero_gradient();
      __syncthreads();
    }
  }

  for (int i = tid; i < TX * TY; i += nt) {
    int ty = i / TX, tx = i - ty * TX;
    int gx = x0 + HALO + tx, gy = y0 + HALO + ty;
    if (gx < w && gy < h) a.out[(size_t)gy * P + gx] = sp[(ty + HALO) * RX + tx + HALO];
  }
}

// ---------------------------------------------------- residual + restrict
struct RRArgs {
  const float *p, *rhs;
  const uint8_t *flag;
  int w, h, pitch;
  float ihsq;
  float *rc;      // coarse output
  int cw, ch, cpitch;
  double *norm2;  // optional: sum of r^2 over the fine interior
};

constexpr int CTX = 32, CTY = 8;

__device__ __forceinline__ float residual_at(const float *sp, const uint8_t *sfl, int i, int RX,
                                             float f, float ihsq) {
  float pc = sp[i];
  float fw = (float)sfl[i - 1], fe = (float)sfl[i + 1];
  float fs = (float)sfl[i - RX], fn = (float)sfl[i + RX];
  float val = 0.0f;
  val = val + (sp[i - 1] * fw + pc * (1.0f - fw));
  val = val + (sp[i + 1] * fe + pc * (1.0f - fe));
  val = val + (sp[i - RX] * fs + pc * (1.0f - fs));
  val = val + (sp[i + RX] * fn + pc * (1.0f - fn));
  val = val + -4.0f * pc;
  val = val * ihsq;
  return (f + val) * (float)sfl[i];
}

__device__ __forceinline__ void block_add_double(double v, double *out) {
  if (!out) return;
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
    v = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) atomicAdd(out, v);
  }
}

__global__ void __launch_bounds__(256) k_resid_restrict(RRArgs a) {
  constexpr int PRX = 2 * CTX + 3, PRY = 2 * CTY + 3;  // p / flag region
  constexpr int RRX = 2 * CTX + 1, RRY = 2 * CTY + 1;  // residual region
  __shared__ float sp[PRY * PRX];
  __shared__ uint8_t sfl[PRY * PRX];
  __shared__ float sr[RRY * RRX];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int X0 = blockIdx.x * CTX, Y0 = blockIdx.y * CTY;
  const int px0 = 2 * X0 - 2, py0 = 2 * Y0 - 2;
  const int w = a.w, h = a.h, P = a.pitch;
  for (int i = tid; i < PRX * PRY; i += nt) {
    int ry = i / PRX, rx = i - ry * PRX;
    int gx = px0 + rx, gy = py0 + ry;
    bool in = gx >= 0 && gx < w && gy >= 0 && gy < h;
    sp[i] = in ? __ldg(a.p + (size_t)gy * P + gx) : 0.0f;
    sfl[i] = in ? __ldg(a.flag + (size_t)gy * P + gx) : (uint8_t)0;
  }
  __syncthreads();
  double acc = 0.0;
  for (int i = tid; i < RRX * RRY; i += nt) {
    int j = i / RRX, k = i - j * RRX;
    int gx = px0 + 1 + k, gy = py0 + 1 + j;
    float r = 0.0f;
    if (gx >= 1 && gx < w - 1 && gy >= 1 && gy < h - 1) {
      float f = __ldg(a.rhs + (size_t)gy * P + gx);
      r = residual_at(sp, sfl, (j + 1) * PRX + (k + 1), PRX, f, a.ihsq);
      if (a.norm2 && gx >= 2 * X0 && gx < 2 * (X0 + CTX) && gy >= 2 * Y0 && gy < 2 * (Y0 + CTY))
        acc += (double)r * (double)r;
    }
    sr[i] = r;
  }
  __syncthreads();
  for (int i = tid; i < CTX * CTY; i += nt) {
    int ty = i / CTX, tx = i - ty * CTX;
    int X = X0 + tx, Y = Y0 + ty;
    if (X >= a.cw || Y >= a.ch) continue;
    float v = 0.0f;
    if (X >= 1 && X < a.cw - 1 && Y >= 1 && Y < a.ch - 1) {
      const float *c = sr + (2 * ty + 1) * RRX + (2 * tx + 1);
      v = (c[-RRX - 1] * 1.0f + c[-RRX] * 2.0f) + c[-RRX + 1] * 1.0f;
      v = v + ((c[-1] * 2.0f + c[0] * 4.0f) + c[1] * 2.0f);
      v = v + ((c[RRX - 1] * 1.0f + c[RRX] * 2.0f) + c[RRX + 1] * 1.0f);
      v = v * (1.0f / 16.0f);
    }
    a.rc[(size_t)Y * a.cpitch + X] = v;
  }
  block_add_double(acc, a.norm2);
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

// ---------------------------------------------------------------- helpers
template <int TX, int TY, int HALO>
void launch_smooth_t(const SmoothArgs &a, cudaStream_t st) {
  using T = SmoothTile<TX, TY, HALO>;
  static_assert(T::smem() <= 48 * 1024, "smoother tile exceeds the default shared-memory limit");
  size_t sm = T::smem();
  dim3 grid((a.w + TX - 1) / TX, (a.h + TY - 1) / TY);
  k_smooth<TX, TY, HALO><<<grid, 256, sm, st>>>(a);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

// Halo of a temporally blocked tile: each red-black sweep needs two cells,
// plus one so that the zero-gradient copy of a tile whose first column is
// the domain's last column (p(w-1, y) = p(w-2, y)) reads a valid neighbour.
// x0 + y0 stays even, so region parity equals global parity.
void launch_smooth(const SmoothArgs &a, cudaStream_t st) {
  switch (a.nsweeps) {
    case 1: launch_smooth_t<64, 32, 3>(a, st); break;
    case 2: launch_smooth_t<64, 32, 5>(a, st); break;
    case 3: launch_smooth_t<64, 32, 7>(a, st); break;
    case 4: launch_smooth_t<64, 32, 9>(a, st); break;
    case 5: launch_smooth_t<64, 32, 11>(a, st); break;
    default: throw ArgError("smoother: 1..5 sweeps per launch");
  }
}

ProlongArgs make_prolong(const MgLevel *coarse, int cur) {
  ProlongArgs pr{};
  if (!coarse) return pr;
  pr.ec = coarse->e[cur];
  pr.flagc = coarse->flag;
  pr.cpitch = coarse->pitch;
  for (int k = 0; k < 5; k++) pr.wsum[k] = (float)((double)(float)k + 0.0001);
  return pr;
}

void smooth(MgHier &mg, std::vector<int> &cur, int l, int ns, bool zgbc, bool zero_init,
            const MgLevel *prolong_from, int prolong_cur, float alpha, cudaStream_t st) {
  MgLevel &L = mg.lv[l];
  ProfScope ps_(l == 0 ? KC_SMOOTH_L0 : KC_SMOOTH_COARSE, st);
  SmoothArgs a{};
  a.in = L.e[cur[l]];
  a.out = L.e[1 - cur[l]];
  a.rhs = L.rhs;
  a.flag = L.flag;
  a.w = L.w;
  a.h = L.h;
  a.pitch = L.pitch;
  a.hh = L.hh;
  a.alpha = alpha;
  a.nsweeps = ns;
  a.zgbc = zgbc ? 1 : 0;
  a.zero_init = zero_init ? 1 : 0;
  a.pr = make_prolong(prolong_from, prolong_cur);
  launch_smooth(a, st);
  cur[l] = 1 - cur[l];
}

void resid_restrict(MgHier &mg, std::vector<int> &cur, int l, double *norm2, cudaStream_t st) {
  ProfScope ps_(l == 0 ? KC_RESTRICT_L0 : KC_RESTRICT_COARSE, st);
  MgLevel &F = mg.lv[l];
  MgLevel &C = mg.lv[l + 1];
  RRArgs a{};
  a.p = F.e[cur[l]];
  a.rhs = F.rhs;
  a.flag = F.flag;
  a.w = F.w;
  a.h = F.h;
  a.pitch = F.pitch;
  a.ihsq = 1.0f / F.hh / F.hh;
  a.rc = C.rhs;
  a.cw = C.w;
  a.ch = C.h;
  a.cpitch = C.pitch;
  a.norm2 = norm2;
  dim3 grid((C.w + CTX - 1) / CTX, (C.h + CTY - 1) / CTY);
  k_resid_restrict<<<grid, 256, 0, st>>>(a);
  UBG_LAUNCH_CHECK();
  g_stats.launches++;
}

// MG::solveLevel, pressure_solver.cpp:201-248.
void solve_level(MgHier &mg, std::vector<int> &cur, int l, bool zgbc, cudaStream_t st) {
  bool bc = zgbc && l == 0;
  if (l == mg.levels - 2) {
    smooth(mg, cur, l, 5, false, l > 0, nullptr, 0, 1.0f, st);
    return;
  }
  smooth(mg, cur, l, 3, bc, l > 0, nullptr, 0, 1.0f, st);
  resid_restrict(mg, cur, l, nullptr, st);
  solve_level(mg, cur, l + 1, false, st);
  smooth(mg, cur, l, 3, bc, false, &mg.lv[l + 1], cur[l + 1], 1.0f, st);
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

void mg_alloc(MgHier &mg, int W, int H, float h0) {
  mg_free(mg);
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
  size_t total = 0;
  for (auto &L : lv) {
    size_t n = (size_t)L.pitch * L.h;
    total += 3 * align256(n * 4) + align256(n);
  }
  total += 256;  // norm scalar
  void *arena = nullptr;
  if (cudaMalloc(&arena, total) != cudaSuccess) {
    cudaGetLastError();
    throw std::bad_alloc();
  }
  UBG_CUDA(cudaMemset(arena, 0, total));
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
  }
  mg.norm = (double *)p;
  mg.lv = lv;
  mg.levels = (int)lv.size();
  mg.arena = arena;
  mg.arena_bytes = total;
  mg.cur0 = 0;
}

void mg_free(MgHier &mg) {
  if (mg.arena) cudaFree(mg.arena);
  mg.arena = nullptr;
  mg.lv.clear();
  mg.levels = 0;
}

void mg_update_fields(MgHier &mg, cudaStream_t st) {
  for (int l = 1; l < mg.levels; l++) {
    MgLevel &F = mg.lv[l - 1], &C = mg.lv[l];
    ProfScope ps_(KC_COARSEN, st);
    dim3 grid((C.w + 31) / 32, (C.h + 7) / 8);
    k_coarsen<<<grid, dim3(32, 8), 0, st>>>(F.flag, F.pitch, C.flag, C.w, C.h, C.pitch);
    UBG_LAUNCH_CHECK();
    g_stats.launches++;
  }
}

void mg_fill_coarse_flags_one(MgHier &mg, cudaStream_t st) {
  for (int l = 1; l < mg.levels; l++) {
    MgLevel &C = mg.lv[l];
    dim3 grid((C.w + 31) / 32, (C.h + 7) / 8);
    k_fill_u8<<<grid, dim3(32, 8), 0, st>>>(C.flag, C.w, C.h, C.pitch, 1);
    UBG_LAUNCH_CHECK();
  }
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
  SmoothArgs a{};
  a.in = L.e[cur];
  a.out = L.e[1 - cur];
  a.rhs = L.rhs;
  a.flag = L.flag;
  a.w = L.w;
  a.h = L.h;
  a.pitch = L.pitch;
  a.hh = L.hh;
  a.alpha = alpha;
  a.nsweeps = 1;
  launch_smooth(a, st);
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
