// Internal declarations of the ubootgl_gb300 CUDA library.
//
// Device layout (one simulation of W x H pressure cells):
//   every level-0 field is a pitched, row-major float array with row pitch
//   P = round_up(W, 32) elements (128-byte rows); vx uses columns 0..W-2 of
//   H rows, vy columns 0..W-1 of H-1 rows.  The flag is one byte per cell
//   with the same element pitch.  Coarse multigrid levels have their own
//   pitch round_up(w_l, 32).
//
// Arithmetic: the library is compiled with -fmad=false; every kernel
// evaluates the reference's expressions in the reference's source order in
// IEEE float, with explicit __fmaf_rn only in the Catmull-Rom sampler.  That
// is what makes the FP32 path bit-identical to the CPU restatement of the
// reference used as the test oracle.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ubootgl_gb300.h"

namespace ubg {

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct ArgError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define UBG_CUDA(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      throw ::ubg::CudaError(std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + \
                             __FILE__ + ":" + std::to_string(__LINE__) + ")");           \
  } while (0)

#define UBG_LAUNCH_CHECK() UBG_CUDA(cudaGetLastError())

// Programmatic dependent launch: the kernel may be scheduled while its
// predecessor on the stream drains (the launch latency overlaps the
// predecessor's last wave); every kernel launched this way starts with
// griddep_wait(), so no thread reads memory before the predecessor grid has
// completed and its writes are visible.
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  UBG_CUDA(cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...));
}
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// Sets the message returned by ubg_last_error() on the calling thread.
void set_last_error(const std::string &msg);

// ------------------------------------------------------------ step scalars
// Quantities that depend on dt, formed exactly as the reference forms them
// (simulation.cpp:105, 165, 242, 276, 286) in float.  They live in device
// memory so that a captured step graph does not depend on dt.
struct StepScalars {
  float dt;
  float a;      // dt * mu * (width - 1.0f) / pwidth
  float den;    // 1.0f + 4.0f * a
  float rden;   // RN(1 / den), for div_rn
  float ih;     // 1.0f / h
  float chalf;  // 0.5f * dt * ih
  float cfull;  // dt * ih
};

struct SinkCell {
  int x, y;
  float v;
};

// Boundary types per edge, order West, East, North, South.
struct Bcs {
  int w, e, n, s;
};

// ------------------------------------------------------------- kernels
// Velocity fields of one simulation, for the step kernels.
struct VelBufs {
  float *vx[2];
  float *vy[2];
  int pitch, W, H;
  // Per-face stencil codes (static per flag mask, pitched like the fields):
  // FC_M = face mask flag*flag of the two cells, FC_T1..FC_T4 = weights of
  // the four diffusion neighbour terms in the reference's order, FC_A = the
  // reference's advection loop covers this face.
  const uint8_t *cx, *cy;
  int advect_bilinear;  // advection option: bilinearSample instead of bicubicSample
};
constexpr unsigned FC_M = 1, FC_T1 = 2, FC_T2 = 4, FC_T3 = 8, FC_T4 = 16, FC_A = 32;
// Buffer f of a pair, chosen without indexing the array: a run-time index
// into a kernel parameter's array makes the compiler copy the parameter to
// local memory.
__device__ __forceinline__ float *pick(float *const (&b)[2], int f) { return f ? b[1] : b[0]; }
// Builds the face codes from the cell flags.
void launch_face_codes(const VelBufs &v, const uint8_t *flag, uint8_t *cx, uint8_t *cy,
                       cudaStream_t st);

// setVBCs (simulation.cpp:80-102): boundary values computed from the front
// buffers (fx, fy), written to both buffers of each component.
void launch_vbc(const VelBufs &v, int fx, int fy, Bcs bc, bool do_vx, bool do_vy,
                cudaStream_t st, unsigned int *umax_bits = nullptr);
// applyAccumulatedVelocity (simulation.cpp:376-396).
void launch_accum(const VelBufs &v, int fx, int fy, float *ax, float *ay, cudaStream_t st);
// One Jacobi diffusion sweep, buffer src -> buffer 1-src of each component
// (simulation.cpp:112-129, 138-155); comps bit 0 = vx, bit 1 = vy.
void launch_diffuse_sweep(const VelBufs &v, int srcx, int srcy, const StepScalars *sc, int comps,
                          cudaStream_t st);
// advect (simulation.cpp:241-354): reads buffer `src` of vx / vy, writes the
// advected faces into buffer 1-src (faces the reference does not advect keep
// their value).
void launch_advect(const VelBufs &v, int srcx, int srcy, const StepScalars *sc, cudaStream_t st);
// Divergence into f (simulation.cpp:166-171).
void launch_divergence(const VelBufs &v, int fx, int fy, float *f, const StepScalars *sc,
                       cudaStream_t st);
// Sinks (simulation.cpp:173-183), already resolved to cells on the host.
void launch_sinks(float *f, int pitch, const SinkCell *cells, int n, cudaStream_t st);
// setPBC (simulation.cpp:36-45).
void launch_pbc(float *p, int pitch, int W, int H, Bcs bc, cudaStream_t st);
// Pressure-gradient update (simulation.cpp:196-207); if umax_bits is set,
// max(|u|) of the updated interior faces is folded into it (atomicMax on
// the float bits).
void launch_gradient(const VelBufs &v, int fx, int fy, const float *p, const StepScalars *sc,
                     unsigned int *umax_bits, cudaStream_t st);
// max(|vx|, |vy|) over the front buffers -> dt = cfl*h/max (extension) and
// the derived scalars.  With umax_ready the maximum left in *umax_bits by
// the previous step's gradient and boundary kernels is used as is.
// Staged host I/O: staging -> front velocity (+ max|u| into *umax_bits,
// zeroed first), and front velocity -> staging.
void launch_stage_in(VelBufs &v, int fx, int fy, const float *inx, const float *iny,
                     unsigned int *umax_bits, cudaStream_t st);
void launch_stage_out(const VelBufs &v, int fx, int fy, float *outx, float *outy, cudaStream_t st);
void launch_cfl(const VelBufs &v, int fx, int fy, float cfl, float h, float mu, float pwidth,
                unsigned int *umax_bits, StepScalars *sc, cudaStream_t st, bool umax_ready);

// Packed FP32 (two lanes per instruction, sm_100 and later): each lane is
// the IEEE single-precision operation with round-to-nearest, so every lane
// equals the scalar operation it replaces.  ptxas may fuse a packed product
// that feeds a packed addition into one fused multiply-add (observed on
// sm_103a despite .rn), so these are used only where no product is added.
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }

// x / d, correctly rounded, for a divisor d > 0 with r = RN(1 / d):
// Markstein's correction (P. Markstein, "Computation of elementary functions
// on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990):
// q0 = RN(x r), the remainder x - q0 d is exact in one FMA, and RN(q0 + rem r)
// is RN(x / d) when nothing underflows or overflows.  Zeros, tiny, huge and
// non-finite x take the division itself.
__device__ __forceinline__ float div_rn(float x, float d, float r) {
  const float ax = fabsf(x);
  if (ax >= 0x1p-100f && ax <= 0x1p+100f) {
    const float q0 = x * r;
    const float rem = __fmaf_rn(-q0, d, x);
    return __fmaf_rn(rem, r, q0);
  }
  return x / d;
}

// Compares div_rn(x[i], d, RN(1/d)) with x[i] / d bit for bit on the device
// (NaNs compare equal); host arrays.
int selftest_div_rn(const float *x, int n, float d, unsigned *mismatches);

// ------------------------------------------------- game-side field access
void launch_scatter_accum(float *ax, float *ay, int P, int W, int H, const float2 *xy,
                          const float2 *v, int n, cudaStream_t st);
void launch_sample_velocity(const float *vx, const float *vy, int P, int W, int H,
                            const float2 *xy, float2 *out, int n, cudaStream_t st);
void launch_set_grids(const int2 *cells, const uint8_t *val, const uint8_t *zero, int n,
                      uint8_t *flag, float *vx, float *vy, float *p, int P, int W, int H,
                      cudaStream_t st);
void launch_shift_map(VelBufs &v, int fx, int fy, const float *p_in, float *p_out,
                      const uint8_t *flag, int P, int W, int H, float inlet_u, cudaStream_t st);

// ------------------------------------- multi-member (fused batch) launches
// One launch covers every member of a batch: the grid is the concatenation
// of the members' grids, bs[m] the first block of member m (bs[n] = total),
// and each block runs the single-simulation kernel body on its member's
// arguments.  Arguments live in a device table built by the host.
enum MultiKind {
  MK_VBC = 0, MK_DIFFUSE, MK_ADVECT, MK_DIVERGENCE, MK_PBC, MK_GRADIENT, MK_CFL, MK_MG, MK_TAIL
};
struct VbcM {
  VelBufs v;
  int fx, fy, do_vx, do_vy;
  Bcs bc;
  unsigned int *umax;
};
struct DiffuseM {
  VelBufs v;
  int srcx, srcy, comps, gx, gy;
  const StepScalars *sc;
};
struct AdvectM {
  VelBufs v;
  int srcx, srcy, gx;
  const StepScalars *sc;
};
struct DivergenceM {
  const float *vx, *vy;
  float *f;
  int P, W, H, gx;
  const StepScalars *sc;
};
struct PbcM {
  float *p;
  int P, W, H;
  Bcs bc;
  unsigned int *umax_zero;  // zeroed by the member's first thread (next: gradient)
};
struct GradientM {
  VelBufs v;
  int fx, fy, gx;
  const float *p;
  const StepScalars *sc;
  unsigned int *umax;
};
struct CflM {
  const unsigned int *umax;
  float cfl, h, mu, pwidth;
  int W;
  StepScalars *sc;
};
// The member of the block in a multi-member launch: the largest m with
// bs[m] <= blockIdx.x.
__device__ __forceinline__ int member_of(const int *__restrict__ bs, int n) {
  const int b = (int)blockIdx.x;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(bs + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Every fused launch first checks its table: the word after the member
// prefix sums, bs[n + 1], must equal the launch's tag (written with the
// table).  A launch that finds another value (a table not yet written, or
// not the one the launch was made for) sets *err and returns without
// touching any field.
__device__ __forceinline__ bool table_ok(const int *__restrict__ bs, int n, unsigned tag,
                                         unsigned *err) {
  if ((unsigned)__ldg(bs + n + 1) == tag) return true;
  if (threadIdx.x == 0 && threadIdx.y == 0) atomicOr(err, 1u);
  return false;
}

// One launch of a fused batch step: `n` members, their argument structs
// back to back, the block prefix sums and the dynamic shared memory.
struct MultiSlot {
  int kind = 0;
  int tile = -1;  // MK_MG: smoother tile id
  int n = 0;
  int blocks = 0;
  size_t smem = 0;
  std::vector<char> args;
  std::vector<int> bs;
};
// Blocks a member needs for each kind (and fills the grid width fields).
int multi_blocks_vbc(const VbcM &a);
int multi_blocks_diffuse(DiffuseM &a);
int multi_blocks_advect(AdvectM &a);
int multi_blocks_divergence(DivergenceM &a);
int multi_blocks_pbc(const PbcM &a);
int multi_blocks_gradient(GradientM &a);
// Launches over n members (device tables args, bs; total blocks).
void launch_multi_step(int kind, const void *args, const int *bs, int n, int blocks,
                       unsigned tag, unsigned *err, cudaStream_t st);

// ------------------------------------------------------------ multigrid
struct MgLevel {
  int w, h, pitch;
  float hh;            // grid spacing of this level
  uint8_t *flag;       // w x h, pitched, 0 / 1
  uint8_t *code;       // per-cell stencil code (own flag + the 4 neighbours' flags)
  float *e[2];         // level 0: pressure ping-pong; coarse: error ping-pong
  float *rhs;          // level 0: f; coarse: restricted residual
  int tile_pre = -1;   // smoother tile of the pre- / post-smoothing launch
  int tile_post = -1;  //   (-1: chosen by level width; else set by the autotuner)
};

struct MgHier {
  int levels = 0;
  std::vector<MgLevel> lv;
  int cur0 = 0;                  // which e[] of level 0 holds p
  int tail_top = -1;             // first level solved by the one-CTA tail kernel
  int tail_cells = 2048;         // largest top level the tail takes (autotuned)
  int tail_top_fp64 = -1;        // the same for the mixed solver's FP64 tail
  // First level of the cluster coarse solve (levels cluster_top ..
  // tail_top-1 in row bands over a thread-block cluster, the tail's levels
  // in its first CTA; one launch), or -1: launches per level.
  int cluster_top = -1;
  void *arena = nullptr;
  size_t arena_bytes = 0;
  double *norm = nullptr;        // device scalar for residual norms
  double *post_norm2 = nullptr;  // if set: ||r||^2 after each level-0 post-smoothing
  // The tolerance solver's own hierarchy (ext_hier_*): level sizes
  // floor(w/2)+1, zero-gradient edges on every level, coarsest level = the
  // last one, solved with `ncoarse` sweeps.  The reference's hierarchy
  // (ext = false) ends one level earlier (levels-2) with 5 sweeps.
  bool ext = false;
  int ncoarse = 5;
};
inline int mg_coarsest(const MgHier &mg) { return mg.ext ? mg.levels - 1 : mg.levels - 2; }
// Whether the cluster coarse solve can run on this device, and why not.
const char *cluster_coarse_solve_status();

// Times the candidate smoother tiles of every level and the tail sizes on
// this hierarchy's own arrays (state preserved: trials write only scratch
// buffers) and keeps the fastest; results are bit-identical for every
// choice.  Appends a JSON report to *report if given.
void mg_autotune(MgHier &mg, cudaStream_t st, std::string *report);

// The launches of one V-cycle (MG::solve with zero-gradient edges, FP32) of
// every member, fused level by level: pre-smoothing launches from level 0
// down, one tail launch (each member's one-CTA coarse solve), then the
// post-smoothing launches back up.  Members of a level are grouped by their
// smoother tile.  Every member needs a coarse tail (tail_top >= 1).
void mg_multi_vcycle(const std::vector<MgHier *> &mgs, std::vector<MultiSlot> &out);
// Launches one MK_MG / MK_TAIL slot whose tables are at dargs / dbs.
void launch_multi_mg(const MultiSlot &slot, const void *dargs, const int *dbs, unsigned tag,
                     unsigned *err, cudaStream_t st);

// Allocates the hierarchy for a W x H level-0 grid with spacing h0.
void mg_alloc(MgHier &mg, int W, int H, float h0);
// Device bytes of the hierarchy of a W x H grid, and laying it out in a
// caller-provided arena (not owned; nothing is allocated or cleared).
size_t mg_arena_bytes(int W, int H);
void mg_bind(MgHier &mg, int W, int H, float h0, void *arena, size_t bytes);
void mg_free(MgHier &mg);
// MG::updateFields on the device: level 0 flag must already be set; also
// rebuilds the stencil codes of every level.
void mg_update_fields(MgHier &mg, cudaStream_t st);
// Stencil codes of one level from its flags.
void level_make_code(MgLevel &L, cudaStream_t st);
// Sets all coarse flags to 1.0 (MG(width, height) without a flag).
void mg_fill_coarse_flags_one(MgHier &mg, cudaStream_t st);
// One call of MG::solve(p, f, flag, h, zgbc) on level 0's e[cur0] / rhs.
void mg_solve(MgHier &mg, bool zgbc, cudaStream_t st);
// Recomputes every level's spacing from the level-0 spacing h0
// (h * (w-1) / (wc-1) per level, pressure_solver.cpp:225).
void mg_set_h(MgHier &mg, float h0);
// One red-black sweep of a single level (free function rbgs), e[cur] -> e[1-cur].
void level_rbgs(MgLevel &L, int &cur, float alpha, cudaStream_t st);
// Residual field of one level into `r` (pitched like the level, may be null)
// with its squared L2 norm accumulated into *norm2 (device double, may be null).
void level_residual(const MgLevel &L, int cur, float *r, double *norm2, cudaStream_t st);

// ------------------------------------------- mixed-precision multigrid
// Device scalars of the defect-correction loop.
struct DcScalars {
  double norm2;      // ||r||^2 of the last residual pass (FP64)
  unsigned maxbits;  // max |r| of the last residual pass, as float bits
  float inv_s;       // 1 / s of the correction in flight (s = scale of the 16-bit rhs)
};

// Low-precision correction hierarchy: the level shapes and stencil codes of
// an MgHier, error and right-hand side stored in 16 bits (FP16 or BF16).
struct MgLow {
  int prec = 0;  // UBG_MIXED_FP16 or UBG_MIXED_BF16
  int levels = 0;
  std::vector<void *> e[2], rhs;  // per level, pitch of the MgHier level
  std::vector<float> rfac;        // restriction weight of each fine level, scaled form
  float *r32 = nullptr;           // level-0 residual in FP32
  DcScalars *dev = nullptr;       // device scalars
  DcScalars *host = nullptr;      // pinned copy for the convergence test
  void *arena = nullptr;
  int kexp = 0;  // the scaled rhs g satisfies max|g| in [2^-(kexp+1), 2^-kexp)
};

// Subtracts the mean of level 0's rhs over the interior fluid cells from
// those cells (device-side; capturable).  With want_norm, synchronises and
// returns ||f - mean||^2 over them (FP64), else -1.
double mg_meanfree_rhs(MgHier &mg, cudaStream_t st, bool want_norm);
void mg_low_alloc(MgLow &lo, const MgHier &mg, int prec);
void mg_low_free(MgLow &lo);

// Mixed-precision MG::solve of level 0 of `mg` (p = e[cur0], rhs f): an FP32
// defect-correction loop whose correction is one V-cycle of the scaled
// system in 16-bit storage (FP32 arithmetic, FP64 coarse solve).  Runs
// max_cycles corrections; when tol > 0 it stops as soon as
// ||r|| <= tol * sqrt(fnorm2) (FP64 norms, one host read per cycle).
// Returns the corrections run; *rel (may be null) = ||r|| / sqrt(fnorm2) of
// the final p when tol > 0, else -1.
int mg_solve_mixed(MgHier &mg, MgLow &lo, double tol, int max_cycles, double fnorm2, double *rel,
                   cudaStream_t st);

// ------------------------------------------------ tolerance-mode solver
// The tolerance solver's hierarchy (sizes floor(w/2)+1, zero-gradient
// edges on every level; k_mg.cu) and one preconditioning V-cycle of it:
// z = M r with r = level 0's rhs and z = level 0's e[cur0] after the call
// (zero start).  prec selects the storage of the coarse levels: FP32 (mg's
// arrays) or 16 bits (lo's arrays, h^2-scaled, scale from *scale_bits =
// max|r| as float bits); level 0 is FP32 in every mode.
size_t ext_hier_bytes(int W, int H);
void ext_hier_alloc(MgHier &mg, int W, int H, float h0);
// Level-0 flag from flag0 (pitch0 bytes per row), coarse flags, codes.
void ext_hier_update_fields(MgHier &mg, const uint8_t *flag0, int pitch0, cudaStream_t st);
void ext_vcycle(MgHier &mg, MgLow *lo, int prec, const unsigned *scale_bits, cudaStream_t st);

// Device scalars of the flexible CG loop (k_krylov.cu).
struct FcgScalars {
  double ff;       // ||f_c||^2
  double rr;       // ||r||^2 of the recurrence
  double zq;       // (z, q_prev)
  double dr;       // (d, r)
  double dq[2];    // (d, q) of this and of the previous iteration
  double fsum;     // sum of f over the interior fluid cells
  double neast;    // fluid cells of the outflow column x = W-2
  double nfluid;   // interior fluid cells
  double zsum;     // sum of the preconditioned residual z over the interior fluid cells
  unsigned maxbits;  // max|r| as float bits
  unsigned pad;
};

// Per-block partial sums of the Krylov reductions (summed in block order by
// the last block of each launch) and the ticket that finds that block.
constexpr int kFcgMaxBlocks = 2048;
struct FcgPartials {
  double v[kFcgMaxBlocks][4];
  unsigned m[kFcgMaxBlocks];
  unsigned ticket;
};

struct FcgSolver {
  MgHier mg;  // the tolerance hierarchy (level 0: rhs = r, e = z)
  MgLow lo;   // its 16-bit arrays (mixed precision)
  int prec = UBG_FP32;
  float *xh = nullptr, *xl = nullptr;  // double-float pressure iterate, pitched like the fields
  float *d[2] = {nullptr, nullptr}, *q = nullptr;
  FcgScalars *dev = nullptr, *host = nullptr;
  FcgPartials *part = nullptr;  // zeroed at allocation (ticket 0)
  void *arena = nullptr;
  bool dirty = true;  // the flag changed since the coarse flags were built
  int W = 0, H = 0, P = 0;
  float h = 0.0f;
};
void fcg_alloc(FcgSolver &fs, int W, int H, int P, float h);
void fcg_free(FcgSolver &fs);
size_t fcg_bytes(int W, int H, int P, int prec);
void fcg_set_precision(FcgSolver &fs, int prec);
// Solves the zero-gradient system for p (warm start: p as given; result:
// p's interior cells, and fs.xh + fs.xl as a double-float) until ||r|| <= tol ||f_c||, at most
// max_iter iterations (one V-cycle each).  Synchronises once per
// iteration.  Returns the iterations run; *rel = ||f_c + L x|| / ||f_c||
// of the final x.
int fcg_solve(FcgSolver &fs, const uint8_t *flag, const float *f, float *p, double tol,
              int max_iter, double *rel, cudaStream_t st);
// The pressure-gradient update from the double-float pressure xh + xl.
void launch_gradient_df(const VelBufs &v, int fx, int fy, const float *xh, const float *xl,
                        const StepScalars *sc, unsigned *umax_bits, cudaStream_t st);

// ------------------------------------------------------------- tracers
struct TracerArgs {
  float2 *points;       // ntracers x npoints ring of positions
  uint32_t *start, *end;
  float *ages;
  const float *vx, *vy;  // front velocity buffers (the texels are formed from them)
  int P, W, H;
  const uint8_t *flag;  // cell flags, nfx x nfy, row pitch fpitch
  int nfx, nfy, fpitch;
  int ntracers, npoints;
  float dt, pdx, pdy;
  uint32_t seed;
};
// interp_shader.cs: the (2W-1) x (2H-1) display texture (and magnitude if
// mag is non-null) from the front velocity buffers.
void launch_velocity_texture(const float *vx, const float *vy, int P, int W, int H, float2 *vxy,
                             float *mag, cudaStream_t st);
// advect_tracer_points.cs: one step of every tracer.
void launch_tracers(const TracerArgs &a, cudaStream_t st);

// Counters for the benchmark.
struct LaunchStats {
  long launches = 0;
};
extern thread_local LaunchStats g_stats;

// Optional per-kernel timing: when a Profiler is installed for the calling
// thread (profiling mode, never during graph capture), every launch site
// records a CUDA event pair on its stream, tagged with its kernel class.
enum KernelClass {
  KC_VBC = 0, KC_ACCUM, KC_DIFFUSE, KC_ADVECT, KC_DIVERGENCE, KC_SINKS, KC_PBC, KC_GRADIENT,
  KC_CFL, KC_SMOOTH_L0, KC_SMOOTH_COARSE, KC_RESTRICT_L0, KC_RESTRICT_COARSE, KC_COARSEN,
  KC_RESIDUAL, KC_TRACERS, KC_OTHER, KC_SMOOTH_L1, KC_TAIL, KC_KRYLOV, KC_COUNT
};
const char *kernel_class_name(int kc);

struct Profiler {
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  struct Mark {
    int kc;
    size_t a, b;
  };
  std::vector<Mark> marks;
  double total_ms[KC_COUNT] = {};
  long count[KC_COUNT] = {};
  cudaEvent_t next();
  void collect();  // after the stream is synchronised
  ~Profiler();
};
extern thread_local Profiler *g_prof;

struct ProfScope {
  Profiler *p;
  size_t a = 0;
  int kc;
  cudaStream_t st;
  ProfScope(int kc_, cudaStream_t st_) : p(g_prof), kc(kc_), st(st_) {
    if (p) {
      a = p->used;
      cudaEventRecord(p->next(), st);
    }
  }
  ~ProfScope() {
    if (p) {
      size_t b = p->used;
      cudaEventRecord(p->next(), st);
      p->marks.push_back({kc, a, b});
    }
  }
};

// Largest member (in cells) that fused launches take by default; larger
// grids fill the GPU on their own and overlap better as separate streams.
constexpr long long kFuseMaxCells = 1LL << 20;

// Steps a changing set of simulations together, one launch per kernel over
// the whole set per step (continuous batching).  The work runs on the
// stepper's own stream, in order; members join and leave between steps.
// The members must be eligible(): FP32, fixed V-cycle count, a coarse
// tail, no sinks, not profiling.  Each member's results are bit-identical
// to stepping it alone.
class FusedStepper {
 public:
  FusedStepper();
  ~FusedStepper();
  FusedStepper(const FusedStepper &) = delete;
  FusedStepper &operator=(const FusedStepper &) = delete;
  static bool eligible(const ubg_sim *s);
  // Members stepped together need the same group (their V-cycle count).
  static int group(const ubg_sim *s);
  // Orders the stepper's stream after the work on s's stream so far and
  // readies s's dt input (pending staged input, accumulation, max|u|).
  void join(ubg_sim *s);
  // True when the next step can be enqueued without waiting on the device
  // (at most two steps in flight).
  bool ready() const;
  // One device-CFL step of every member; cfl[i] is member i's factor.  The
  // members need the same V-cycle count.
  void step(const std::vector<ubg_sim *> &sims, const std::vector<float> &cfl);
  // Records ev on the stepper's stream after s's last fused step and makes
  // s's own stream wait for it.
  void leave(ubg_sim *s, cudaEvent_t ev);
  // True once a fused launch found a table it was not made for (that
  // launch skipped its work); read after the steps in question completed.
  bool failed() const;

 private:
  struct Impl;
  Impl *p_;
};

}  // namespace ubg
