/*
 * CPU restatement of ubootgl's fluid step -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the oracle the CUDA path is checked against.  Only tests,
 * the smoke check and the CPU-baseline leg of the benchmark may load it; the
 * product library never links it.
 *
 * It is included twice by ubg_oracle.c, once with REAL=float (the parity
 * oracle) and once with REAL=double (the FP64 oracle used for accuracy
 * statements).  Every function follows the reference's code path line by line
 * (citations are to te42kyfo/ubootgl, path:line) in plain IEEE arithmetic:
 * the file is compiled with -ffp-contract=off, so the only fused multiply-adds
 * are the explicit FMA() calls in the Catmull-Rom sampler.  The CUDA kernels
 * evaluate the same operations in the same order, which makes the FP32 GPU
 * path bit-identical to REAL=float here.  The reference itself is compiled
 * with -Ofast (reassociation, reciprocal division, contraction), so it agrees
 * with this restatement only to a few ulp per operation; that difference is
 * measured by tests/test_oracle_vs_reference.py.
 *
 * Red-black Gauss-Seidel follows the reference's deterministic ("classic")
 * schedule, pressure_solver.cpp:65-71: all red points of a sweep, then all
 * black points.  Each half sweep reads only the other colour, so the OpenMP
 * loops below give the same result for any thread count.
 *
 * Required macros: REAL, SFX (name suffix), FMA (fused multiply-add for REAL).
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(CAT(ubo_, SFX), CAT(_, name))
#define SIM_T CAT(ubo_sim_, SFX)
#define MG_T CAT(ubo_mg_, SFX)

/* ------------------------------------------------------------------ grids */
/* Row-major storage, idx = y*width + x (db2dgrid.hpp:19). */
#define AT(arr, w, x, y) ((arr)[(size_t)(y) * (size_t)(w) + (size_t)(x)])

typedef struct {
  int levels;
  int lw[UBO_MAXL], lh[UBO_MAXL];
  REAL *rs[UBO_MAXL], *rcs[UBO_MAXL], *ecs[UBO_MAXL], *es[UBO_MAXL];
  REAL *flagcs[UBO_MAXL];
} MG_T;

typedef struct {
  int W, H;
  REAL pwidth, mu, h, dt;
  int bcWest, bcEast, bcNorth, bcSouth;
  REAL *vxb[2], *vyb[2];
  int fx, fy; /* front index of vx and of vy (each DoubleBuffered2DGrid swaps on its own) */
  REAL *vx_accum, *vy_accum;
  REAL *p, *f, *flag, *r;
  MG_T mg;
  int nsinks;
  REAL sinks[UBO_MAXSINKS][3];
  int bilinear; /* advection samples: 0 bicubicSample (the reference), 1 bilinearSample */
} SIM_T;

static REAL *FN(alloc)(size_t n) {
  REAL *v = (REAL *)calloc(n ? n : 1, sizeof(REAL));
  return v;
}

static void FN(fill)(REAL *v, size_t n, REAL val) {
  for (size_t i = 0; i < n; i++) v[i] = val;
}

/* -------------------------------------------------------------- MG setup */
/* Level sizes by integer halving while both sides are > 3
 * (pressure_solver.hpp:16-31); coarse flag arrays start filled with 1.0
 * (pressure_solver.hpp:26). */
static int FN(mg_init)(MG_T *mg, int width, int height) {
  memset(mg, 0, sizeof(*mg));
  int cw = width, ch = height;
  int l = 0;
  while (cw > 3 && ch > 3) {
    if (l >= UBO_MAXL) return -1;
    size_t n = (size_t)cw * ch;
    mg->lw[l] = cw;
    mg->lh[l] = ch;
    mg->rs[l] = FN(alloc)(n);
    mg->rcs[l] = FN(alloc)(n);
    mg->ecs[l] = FN(alloc)(n);
    mg->es[l] = FN(alloc)(n);
    mg->flagcs[l] = FN(alloc)(n);
    FN(fill)(mg->flagcs[l], n, (REAL)1.0);
    cw /= 2;
    ch /= 2;
    l++;
  }
  mg->levels = l;
  return 0;
}

static void FN(mg_free)(MG_T *mg) {
  for (int l = 0; l < mg->levels; l++) {
    free(mg->rs[l]);
    free(mg->rcs[l]);
    free(mg->ecs[l]);
    free(mg->es[l]);
    free(mg->flagcs[l]);
  }
  mg->levels = 0;
}

/* MG::updateFields, pressure_solver.hpp:34-57: level 0 is a copy of the flag;
 * coarse levels are refilled with 1.0 and their interior set to
 * (1-2-1 x 1-2-1 weighted average of the finer flag > 0.2) ? 1 : 0. */
void FN(mg_update_fields)(MG_T *mg, const REAL *flag) {
  memcpy(mg->flagcs[0], flag, sizeof(REAL) * (size_t)mg->lw[0] * mg->lh[0]);
  for (int level = 1; level < mg->levels; level++) {
    REAL *fc = mg->flagcs[level];
    const REAL *f = mg->flagcs[level - 1];
    int fw = mg->lw[level - 1];
    int cw = mg->lw[level], ch = mg->lh[level];
    FN(fill)(fc, (size_t)cw * ch, (REAL)1.0);
    for (int y = 1; y < ch - 1; y++) {
      for (int x = 1; x < cw - 1; x++) {
        REAL v = 0;
        v = AT(f, fw, 2 * x - 1, 2 * y - 1) * 1 + AT(f, fw, 2 * x + 0, 2 * y - 1) * 2 +
            AT(f, fw, 2 * x + 1, 2 * y - 1) * 1;
        v += AT(f, fw, 2 * x - 1, 2 * y + 0) * 2 + AT(f, fw, 2 * x + 0, 2 * y + 0) * 4 +
             AT(f, fw, 2 * x + 1, 2 * y + 0) * 2;
        v += AT(f, fw, 2 * x - 1, 2 * y + 1) * 1 + AT(f, fw, 2 * x + 0, 2 * y + 1) * 2 +
             AT(f, fw, 2 * x + 1, 2 * y + 1) * 1;
        v *= (REAL)1.0 / (REAL)16.0;
        AT(fc, cw, x, y) = ((double)v > 0.2) ? (REAL)1.0 : (REAL)0.0;
      }
    }
  }
}

/* ------------------------------------------------------- MG components */
/* smoothingKernel, pressure_solver.cpp:10-24 (alpha = 1 everywhere on the
 * step's path; the general form is kept). */
static inline REAL FN(smooth_pt)(const REAL *p, const REAL *f, const REAL *flag, int w,
                                 REAL h, REAL alpha, int x, int y) {
  REAL val = 0;
  REAL sum = 0;
  sum += AT(flag, w, x - 1, y) + AT(flag, w, x + 1, y) + AT(flag, w, x, y + 1) +
         AT(flag, w, x, y - 1);
  val += AT(p, w, x - 1, y) * AT(flag, w, x - 1, y);
  val += AT(p, w, x + 1, y) * AT(flag, w, x + 1, y);
  val += AT(p, w, x, y - 1) * AT(flag, w, x, y - 1);
  val += AT(p, w, x, y + 1) * AT(flag, w, x, y + 1);
  val += AT(f, w, x, y) * h * h;
  val /= sum;
  if (sum == 0) val = 0;
  return AT(flag, w, x, y) * (alpha * val + ((REAL)1.0 - alpha) * AT(p, w, x, y));
}

/* rbgs, pressure_solver.cpp:35-89, classic schedule: red points (x+y odd,
 * x = 1 + y%2, pressure_solver.cpp:36) of every row, then black points. */
void FN(rbgs)(REAL *p, const REAL *f, const REAL *flag, int w, int hgt, REAL h,
              REAL alpha) {
  int y;
#pragma omp parallel for schedule(static)
  for (y = 1; y < hgt - 1; y++)
    for (int x = 1 + (y % 2); x < w - 1; x += 2)
      AT(p, w, x, y) = FN(smooth_pt)(p, f, flag, w, h, alpha, x, y);
#pragma omp parallel for schedule(static)
  for (y = 1; y < hgt - 1; y++)
    for (int x = 1 + ((y + 1) % 2); x < w - 1; x += 2)
      AT(p, w, x, y) = FN(smooth_pt)(p, f, flag, w, h, alpha, x, y);
}

/* calculateResidualField, pressure_solver.cpp:91-116.  Returns the L2 norm,
 * accumulated in double (the reference's float reduction order depends on
 * the thread count; the norm is discarded on the step's path). */
double FN(residual)(const REAL *p, const REAL *f, const REAL *flag, REAL *r, int w,
                    int hgt, REAL h) {
  double l2r = 0;
  REAL ihsq = (REAL)1.0 / h / h;
  int y;
#pragma omp parallel for schedule(static) reduction(+ : l2r)
  for (y = 1; y < hgt - 1; y++) {
    for (int x = 1; x < w - 1; x++) {
      REAL pc = AT(p, w, x, y);
      REAL val = 0;
      val += AT(p, w, x - 1, y) * AT(flag, w, x - 1, y) + pc * ((REAL)1.0 - AT(flag, w, x - 1, y));
      val += AT(p, w, x + 1, y) * AT(flag, w, x + 1, y) + pc * ((REAL)1.0 - AT(flag, w, x + 1, y));
      val += AT(p, w, x, y - 1) * AT(flag, w, x, y - 1) + pc * ((REAL)1.0 - AT(flag, w, x, y - 1));
      val += AT(p, w, x, y + 1) * AT(flag, w, x, y + 1) + pc * ((REAL)1.0 - AT(flag, w, x, y + 1));
      val += (REAL)-4.0 * pc;
      val *= ihsq;
      REAL rv = (AT(f, w, x, y) + val) * AT(flag, w, x, y);
      AT(r, w, x, y) = rv;
      l2r += (double)rv * (double)rv;
    }
  }
  return sqrt(l2r);
}

/* restrict, pressure_solver.cpp:118-132: full weighting onto the coarse
 * interior. */
void FN(restrict_fw)(const REAL *r, int fw, REAL *rc, int cw, int ch) {
  int y;
#pragma omp parallel for schedule(static)
  for (y = 1; y < ch - 1; y++) {
    for (int x = 1; x < cw - 1; x++) {
      REAL v = 0;
      v = AT(r, fw, 2 * x - 1, 2 * y - 1) * 1 + AT(r, fw, 2 * x + 0, 2 * y - 1) * 2 +
          AT(r, fw, 2 * x + 1, 2 * y - 1) * 1;
      v += AT(r, fw, 2 * x - 1, 2 * y + 0) * 2 + AT(r, fw, 2 * x + 0, 2 * y + 0) * 4 +
           AT(r, fw, 2 * x + 1, 2 * y + 0) * 2;
      v += AT(r, fw, 2 * x - 1, 2 * y + 1) * 1 + AT(r, fw, 2 * x + 0, 2 * y + 1) * 2 +
           AT(r, fw, 2 * x + 1, 2 * y + 1) * 1;
      AT(rc, cw, x, y) = v * ((REAL)1.0 / (REAL)16.0);
    }
  }
}

/* prolongate, pressure_solver.cpp:134-172.  The "+ 0.0001" is a double
 * literal in the reference, so the weight sum is formed in double and
 * rounded to REAL. */
void FN(prolongate)(REAL *e, int w, int hgt, const REAL *ec, const REAL *flagc, int cw,
                    const REAL *flag) {
  FN(fill)(e, (size_t)w * hgt, 0);
  int y;
#pragma omp parallel for schedule(static)
  for (y = 2; y < hgt - 1; y += 2)
    for (int x = 2; x < w - 1; x += 2)
      AT(e, w, x, y) = AT(ec, cw, x / 2, y / 2) * AT(flag, w, x, y);
#pragma omp parallel for schedule(static)
  for (y = 2; y < hgt - 1; y += 2)
    for (int x = 1; x < w - 2; x += 2) {
      REAL sum = (REAL)((double)(AT(flagc, cw, x / 2, y / 2) + AT(flagc, cw, x / 2 + 1, y / 2)) +
                        0.0001);
      AT(e, w, x, y) =
          AT(flag, w, x, y) * (AT(ec, cw, x / 2, y / 2) + AT(ec, cw, x / 2 + 1, y / 2)) / sum;
    }
#pragma omp parallel for schedule(static)
  for (y = 1; y < hgt - 2; y += 2)
    for (int x = 2; x < w - 1; x += 2) {
      REAL sum = (REAL)((double)(AT(flagc, cw, x / 2, y / 2) + AT(flagc, cw, x / 2, y / 2 + 1)) +
                        0.0001);
      AT(e, w, x, y) =
          AT(flag, w, x, y) * (AT(ec, cw, x / 2, y / 2) + AT(ec, cw, x / 2, y / 2 + 1)) / sum;
    }
#pragma omp parallel for schedule(static)
  for (y = 1; y < hgt - 2; y += 2)
    for (int x = 1; x < w - 2; x += 2) {
      REAL sum = (REAL)((double)(AT(flagc, cw, x / 2, y / 2) + AT(flagc, cw, x / 2 + 1, y / 2 + 1) +
                                 AT(flagc, cw, x / 2 + 1, y / 2) + AT(flagc, cw, x / 2, y / 2 + 1)) +
                        0.0001);
      AT(e, w, x, y) = AT(flag, w, x, y) *
                       (AT(ec, cw, x / 2, y / 2) + AT(ec, cw, x / 2 + 1, y / 2 + 1) +
                        AT(ec, cw, x / 2 + 1, y / 2) + AT(ec, cw, x / 2, y / 2 + 1)) /
                       sum;
    }
}

/* correct, pressure_solver.cpp:174-181 (p += e*1.0; the double round trip
 * of the reference equals a float add, since double has > 2*24+2 bits). */
void FN(correct)(REAL *p, const REAL *e, int w, int hgt) {
  int y;
#pragma omp parallel for schedule(static)
  for (y = 1; y < hgt - 1; y++)
    for (int x = 1; x < w - 1; x++) AT(p, w, x, y) += AT(e, w, x, y);
}

/* setZeroGradientBC, pressure_solver.cpp:183-192 (corners untouched). */
void FN(zero_gradient_bc)(REAL *p, int w, int hgt) {
  for (int y = 1; y < hgt - 1; y++) {
    AT(p, w, 0, y) = AT(p, w, 1, y);
    AT(p, w, w - 1, y) = AT(p, w, w - 2, y);
  }
  for (int x = 1; x < w - 1; x++) {
    AT(p, w, x, 0) = AT(p, w, x, 1);
    AT(p, w, x, hgt - 1) = AT(p, w, x, hgt - 2);
  }
}

/* MG::solveLevel, pressure_solver.cpp:201-248: V(3,3) cycle; the level
 * levels-2 is "solved" by 5 RB-GS sweeps; the zero-gradient BC is applied on
 * level 0 only; coarse h = h*(w-1)/(wc-1). */
static void FN(solve_level)(MG_T *mg, REAL *p, const REAL *f, const REAL *flag, REAL h,
                            int level, int zgbc) {
  int w = mg->lw[level], hgt = mg->lh[level];
  if (level == mg->levels - 2) {
    for (int i = 0; i < 5; i++) FN(rbgs)(p, f, flag, w, hgt, h, (REAL)1.0);
    return;
  }
  for (int i = 0; i < 3; i++) {
    FN(rbgs)(p, f, flag, w, hgt, h, (REAL)1.0);
    if (level == 0 && zgbc) FN(zero_gradient_bc)(p, w, hgt);
  }
  REAL *r = mg->rs[level];
  FN(fill)(r, (size_t)w * hgt, 0);
  FN(residual)(p, f, flag, r, w, hgt, h);
  int cw = mg->lw[level + 1], ch = mg->lh[level + 1];
  REAL *rc = mg->rcs[level + 1];
  FN(fill)(rc, (size_t)cw * ch, 0);
  FN(restrict_fw)(r, w, rc, cw, ch);
  REAL *ec = mg->ecs[level + 1];
  FN(fill)(ec, (size_t)cw * ch, 0);
  REAL *flagc = mg->flagcs[level + 1];
  REAL hc = h * ((REAL)w - (REAL)1.0) / ((REAL)cw - (REAL)1.0);
  FN(solve_level)(mg, ec, rc, flagc, hc, level + 1, 0);
  REAL *e = mg->es[level];
  FN(prolongate)(e, w, hgt, ec, flagc, cw, flag);
  FN(correct)(p, e, w, hgt);
  if (level == 0 && zgbc) FN(zero_gradient_bc)(p, w, hgt);
  for (int i = 0; i < 3; i++) {
    FN(rbgs)(p, f, flag, w, hgt, h, (REAL)1.0);
    if (level == 0 && zgbc) FN(zero_gradient_bc)(p, w, hgt);
  }
}

/* MG::solve, pressure_solver.hpp:59-62. */
void FN(mg_solve)(MG_T *mg, REAL *p, const REAL *f, const REAL *flag, REAL h, int zgbc) {
  FN(solve_level)(mg, p, f, flag, h, 0, zgbc);
}

/* --------------------------------------------------------- boundary rules */
/* singlePBC / VBCPar / VBCPer, simulation.cpp:22-78. */
static inline REAL FN(single_pbc)(int bc, REAL a) {
  if (bc == UBO_BC_OUTFLOW_ZERO_PRESSURE) return -a;
  return a;
}
static inline REAL FN(vbc_par)(int bc, REAL a, REAL b) {
  if (bc == UBO_BC_INFLOW) return b;
  if (bc == UBO_BC_OUTFLOW || bc == UBO_BC_OUTFLOW_ZERO_PRESSURE) return a > 0 ? a : (REAL)0.0;
  return 0;
}
static inline REAL FN(vbc_per)(int bc, REAL a, REAL b) {
  if (bc == UBO_BC_INFLOW) return b;
  if (bc == UBO_BC_OUTFLOW || bc == UBO_BC_OUTFLOW_ZERO_PRESSURE) return a > 0 ? a : (REAL)0.0;
  return -a;
}

/* setPBC, simulation.cpp:36-45. */
void FN(set_pbc)(SIM_T *s) {
  int W = s->W, H = s->H;
  REAL *p = s->p;
  for (int y = 0; y < H; y++) {
    AT(p, W, 0, y) = FN(single_pbc)(s->bcWest, AT(p, W, 1, y));
    AT(p, W, W - 1, y) = FN(single_pbc)(s->bcEast, AT(p, W, W - 2, y));
  }
  for (int x = 0; x < W; x++) {
    AT(p, W, x, 0) = FN(single_pbc)(s->bcSouth, AT(p, W, x, 1));
    AT(p, W, x, H - 1) = FN(single_pbc)(s->bcNorth, AT(p, W, x, H - 2));
  }
}

/* setVBCs, simulation.cpp:80-102: values computed from the front buffer and
 * written to both buffers, x-edges first, then y-edges (which fixes the
 * corners). */
void FN(set_vbcs)(SIM_T *s) {
  int W = s->W, H = s->H;
  int vxw = W - 1, vxh = H, vyw = W, vyh = H - 1;
  REAL *xf = s->vxb[s->fx], *xb = s->vxb[1 - s->fx];
  REAL *yf = s->vyb[s->fy], *yb = s->vyb[1 - s->fy];
  for (int y = 0; y < vxh; y++) {
    REAL v = FN(vbc_par)(s->bcWest, AT(xf, vxw, 1, y), AT(xf, vxw, 0, y));
    AT(xf, vxw, 0, y) = AT(xb, vxw, 0, y) = v;
    v = FN(vbc_par)(s->bcEast, AT(xf, vxw, vxw - 2, y), AT(xf, vxw, vxw - 1, y));
    AT(xf, vxw, vxw - 1, y) = AT(xb, vxw, vxw - 1, y) = v;
  }
  for (int x = 0; x < vxw; x++) {
    REAL v = FN(vbc_per)(s->bcSouth, AT(xf, vxw, x, 1), AT(xf, vxw, x, 0));
    AT(xf, vxw, x, 0) = AT(xb, vxw, x, 0) = v;
    v = FN(vbc_per)(s->bcNorth, AT(xf, vxw, x, vxh - 2), AT(xf, vxw, x, vxh - 1));
    AT(xf, vxw, x, vxh - 1) = AT(xb, vxw, x, vxh - 1) = v;
  }
  for (int y = 0; y < vyh; y++) {
    REAL v = FN(vbc_per)(s->bcWest, AT(yf, vyw, 1, y), AT(yf, vyw, 0, y));
    AT(yf, vyw, 0, y) = AT(yb, vyw, 0, y) = v;
    v = FN(vbc_per)(s->bcEast, AT(yf, vyw, vyw - 2, y), AT(yf, vyw, vyw - 1, y));
    AT(yf, vyw, vyw - 1, y) = AT(yb, vyw, vyw - 1, y) = v;
  }
  for (int x = 0; x < vyw; x++) {
    REAL v = FN(vbc_par)(s->bcSouth, AT(yf, vyw, x, 1), AT(yf, vyw, x, 0));
    AT(yf, vyw, x, 0) = AT(yb, vyw, x, 0) = v;
    v = FN(vbc_par)(s->bcNorth, AT(yf, vyw, x, vyh - 2), AT(yf, vyw, x, vyh - 1));
    AT(yf, vyw, x, vyh - 1) = AT(yb, vyw, x, vyh - 1) = v;
  }
}

/* ------------------------------------------------------------- diffusion */
/* diffuse, simulation.cpp:104-162: two Jacobi sweeps of vx (front -> back,
 * swap, setVBCs), then two of vy.  a = dt*mu*(width-1)/pwidth. */
void FN(diffuse)(SIM_T *s) {
  int W = s->W, H = s->H;
  const REAL *flag = s->flag;
  REAL a = s->dt * s->mu * ((REAL)W - (REAL)1.0) / s->pwidth;
  REAL den = (REAL)1.0 + (REAL)4.0 * a;
  int vxw = W - 1, vxh = H, vyw = W, vyh = H - 1;
  for (int i = 1; i < 3; i++) {
    const REAL *vf = s->vxb[s->fx];
    REAL *vb = s->vxb[1 - s->fx];
    int y;
#pragma omp parallel for schedule(static)
    for (y = 1; y < vxh - 1; y++) {
      for (int x = 1; x < vxw - 1; x++) {
        REAL c = AT(vf, vxw, x, y);
        REAL val = 0;
        val += AT(vf, vxw, x + 1, y) * AT(flag, W, x + 1, y) * AT(flag, W, x + 2, y);
        val += AT(vf, vxw, x - 1, y) * AT(flag, W, x, y) * AT(flag, W, x - 1, y);
        REAL fvn = AT(flag, W, x, y + 1) * AT(flag, W, x - 1, y + 1);
        val += AT(vf, vxw, x, y + 1) * fvn + ((REAL)1.0 - fvn) * -c;
        REAL fvs = AT(flag, W, x, y - 1) * AT(flag, W, x - 1, y - 1);
        val += AT(vf, vxw, x, y - 1) * fvs + ((REAL)1.0 - fvs) * -c;
        AT(vb, vxw, x, y) = AT(flag, W, x, y) * AT(flag, W, x + 1, y) * (c + a * val) / den;
      }
    }
    s->fx = 1 - s->fx;
    FN(set_vbcs)(s);
  }
  for (int i = 1; i < 3; i++) {
    const REAL *vf = s->vyb[s->fy];
    REAL *vb = s->vyb[1 - s->fy];
    int y;
#pragma omp parallel for schedule(static)
    for (y = 1; y < vyh - 1; y++) {
      for (int x = 1; x < vyw - 1; x++) {
        REAL c = AT(vf, vyw, x, y);
        REAL val = 0;
        val += AT(vf, vyw, x, y - 1) * AT(flag, W, x, y) * AT(flag, W, x, y - 1);
        val += AT(vf, vyw, x, y + 1) * AT(flag, W, x, y + 1) * AT(flag, W, x, y + 2);
        REAL fve = AT(flag, W, x + 1, y) * AT(flag, W, x + 1, y + 1);
        val += AT(vf, vyw, x + 1, y) * fve + ((REAL)1.0 - fve) * -c;
        REAL fvw = AT(flag, W, x - 1, y) * AT(flag, W, x - 1, y + 1);
        val += AT(vf, vyw, x - 1, y) * fvw + ((REAL)1.0 - fvw) * -c;
        AT(vb, vyw, x, y) = AT(flag, W, x, y) * AT(flag, W, x, y + 1) * (c + a * val) / den;
      }
    }
    s->fy = 1 - s->fy;
    FN(set_vbcs)(s);
  }
}

/* ------------------------------------------------------------- advection */
/* CubicHermite, interpolators.hpp:78-85, is the Catmull-Rom cubic through
 * A, B, C, D at parameter t.  It is evaluated here through its four weights
 * (the same polynomial, regrouped):
 *   wA = t(-1/2 + t(1 - t/2)),  wB = 1 + t^2(-5/2 + 3t/2),
 *   wC = t(1/2 + t(2 - 3t/2)),  wD = t^2(-1/2 + t/2),
 * with explicit fused multiply-adds; the weights of one t serve all four
 * columns of a bicubic sample. */
static inline void FN(cr_weights)(REAL t, REAL w[4]) {
  REAL t2 = t * t;
  w[0] = t * FMA(t, FMA((REAL)-0.5, t, (REAL)1.0), (REAL)-0.5);
  w[1] = FMA(t2, FMA((REAL)1.5, t, (REAL)-2.5), (REAL)1.0);
  w[2] = t * FMA(t, FMA((REAL)-1.5, t, (REAL)2.0), (REAL)0.5);
  w[3] = t2 * FMA((REAL)0.5, t, (REAL)-0.5);
}
static inline REAL FN(cr_dot)(const REAL w[4], REAL A, REAL B, REAL C, REAL D) {
  return FMA(w[3], D, FMA(w[2], C, FMA(w[1], B, w[0] * A)));
}

/* bicubicSample, interpolators.hpp:92-206: clamp to [3, size-3], truncate,
 * vertical Catmull-Rom over rows iy-1..iy+2 for the four columns ix-1..ix+2,
 * then horizontal. */
static inline REAL FN(bicubic)(const REAL *g, int gw, int gh, REAL cx, REAL cy) {
  REAL hx = (REAL)gw - (REAL)3.0, hy = (REAL)gh - (REAL)3.0;
  cx = cx < hx ? cx : hx;
  cx = cx > (REAL)3.0 ? cx : (REAL)3.0;
  cy = cy < hy ? cy : hy;
  cy = cy > (REAL)3.0 ? cy : (REAL)3.0;
  int ix = (int)cx, iy = (int)cy;
  REAL sx = cx - (REAL)ix, sy = cy - (REAL)iy;
  REAL wy[4], wx[4], col[4];
  FN(cr_weights)(sy, wy);
  FN(cr_weights)(sx, wx);
  for (int j = 0; j < 4; j++) {
    int x = ix - 1 + j;
    col[j] = FN(cr_dot)(wy, AT(g, gw, x, iy - 1), AT(g, gw, x, iy), AT(g, gw, x, iy + 1),
                        AT(g, gw, x, iy + 2));
  }
  return FN(cr_dot)(wx, col[0], col[1], col[2], col[3]);
}

/* bilinearSample, interpolators.hpp:11-27: clamp to [0, size - 1.1]
 * (glm::clamp = min(max(c, lo), hi)), truncate, interpolate along x, then
 * along y.  The advection option samples with it instead of bicubicSample
 * (extension; the reference advects bicubically). */
static inline REAL FN(bilinear)(const REAL *g, int gw, int gh, REAL cx, REAL cy) {
  REAL hx = (REAL)gw - (REAL)1.1f, hy = (REAL)gh - (REAL)1.1f;
  cx = cx < (REAL)0.0 ? (REAL)0.0 : cx;
  cx = hx < cx ? hx : cx;
  cy = cy < (REAL)0.0 ? (REAL)0.0 : cy;
  cy = hy < cy ? hy : cy;
  int ix = (int)cx, iy = (int)cy;
  REAL sx = cx - (REAL)ix, sy = cy - (REAL)iy;
  REAL v1 = AT(g, gw, ix, iy), v2 = AT(g, gw, ix + 1, iy);
  REAL v3 = AT(g, gw, ix, iy + 1), v4 = AT(g, gw, ix + 1, iy + 1);
  REAL vm1 = v1 + (v2 - v1) * sx;
  REAL vm2 = v3 + (v4 - v3) * sx;
  return vm1 + (vm2 - vm1) * sy;
}
REAL FN(bilinear_sample)(const REAL *g, int gw, int gh, REAL cx, REAL cy) {
  return FN(bilinear)(g, gw, gh, cx, cy);
}
void FN(set_advect_bilinear)(SIM_T *s, int on) { s->bilinear = on ? 1 : 0; }

/* Whether the reference advects face x of row y.  The x loops run in chunks
 * of 8 from x = 1 while x < width-8 (simulation.cpp:248, 300), so the last
 * columns are never advected, and a chunk is skipped when none of its 8
 * lanes has both cells of the skip test fluid (simulation.cpp:254-256 for
 * vx, 302-304 for vy). */
int FN(advect_mask_vx)(const REAL *flag, int W, int x, int y) {
  int xs = 1 + ((x - 1) / 8) * 8;
  if (!(xs < (W - 1) - 8)) return 0;
  for (int i = 0; i < 8; i++)
    if (AT(flag, W, xs - 1 + i, y) + AT(flag, W, xs + i, y) == (REAL)2.0) return 1;
  return 0;
}
int FN(advect_mask_vy)(const REAL *flag, int W, int x, int y) {
  int xs = 1 + ((x - 1) / 8) * 8;
  if (!(xs < W - 8)) return 0;
  for (int i = 0; i < 8; i++)
    if (AT(flag, W, xs + i, y) + AT(flag, W, xs + i, y - 1) == (REAL)2.0) return 1;
  return 0;
}

/* advect, simulation.cpp:241-354: RK2 back-trace per face, three bicubic
 * samples (bilinear with the advection option), result * face mask into the
 * back buffer, then swap both grids.
 * The vy loop runs over the vx rows 1..H-2 (simulation.cpp:247), so it also
 * writes vy row H-2; setVBCs overwrites that row afterwards.  The vx average
 * of the vy loop reads flat index x+1+y*(W-1), which for x = W-2 is element 0
 * of the next row; REF_VX reproduces that. */
#define REF_VX(vx, W, x, y) ((vx)[(size_t)(y) * (size_t)((W)-1) + (size_t)(x)])
#define SAMPLE(g, gw, gh, cx, cy) \
  (bil ? FN(bilinear)(g, gw, gh, cx, cy) : FN(bicubic)(g, gw, gh, cx, cy))
void FN(advect)(SIM_T *s) {
  int W = s->W, H = s->H;
  const int bil = s->bilinear;
  const REAL *flag = s->flag;
  REAL ih = (REAL)1.0 / s->h;
  REAL chalf = (REAL)0.5 * s->dt * ih;
  REAL cfull = s->dt * ih;
  const REAL *vx = s->vxb[s->fx], *vy = s->vyb[s->fy];
  REAL *vxo = s->vxb[1 - s->fx], *vyo = s->vyb[1 - s->fy];
  int vxw = W - 1, vxh = H, vyw = W, vyh = H - 1;
  int y;
#pragma omp parallel for schedule(dynamic, 16)
  for (y = 1; y < vxh - 1; y++) {
    for (int x = 1; x < vxw - 1; x++) {
      if (!FN(advect_mask_vx)(flag, W, x, y)) continue;
      REAL posx = (REAL)x + (REAL)0.5, posy = (REAL)y;
      REAL vx1 = AT(vx, vxw, x, y);
      REAL vy1 = ((AT(vy, vyw, x, y) + AT(vy, vyw, x, y - 1)) +
                  (AT(vy, vyw, x + 1, y) + AT(vy, vyw, x + 1, y - 1))) *
                 (REAL)0.25;
      REAL midx = posx - vx1 * chalf;
      REAL midy = posy - vy1 * chalf;
      REAL vx2 = SAMPLE(vx, vxw, vxh, midx - (REAL)0.5, midy);
      REAL vy2 = SAMPLE(vy, vyw, vyh, midx, midy - (REAL)0.5);
      REAL endx = posx - vx2 * cfull;
      REAL endy = posy - vy2 * cfull;
      REAL v = SAMPLE(vx, vxw, vxh, endx - (REAL)0.5, endy);
      AT(vxo, vxw, x, y) = v * AT(flag, W, x, y) * AT(flag, W, x + 1, y);
    }
    for (int x = 1; x < vyw - 1; x++) {
      if (!FN(advect_mask_vy)(flag, W, x, y)) continue;
      REAL posx = (REAL)x, posy = (REAL)y + (REAL)0.5;
      REAL vy1 = AT(vy, vyw, x, y);
      REAL vx1 = ((REF_VX(vx, W, x, y) + REF_VX(vx, W, x, y - 1)) +
                  (REF_VX(vx, W, x + 1, y) + REF_VX(vx, W, x + 1, y - 1))) *
                 (REAL)0.25;
      REAL midx = posx - vx1 * chalf;
      REAL midy = posy - vy1 * chalf;
      REAL vx2 = SAMPLE(vx, vxw, vxh, midx - (REAL)0.5, midy);
      REAL vy2 = SAMPLE(vy, vyw, vyh, midx, midy - (REAL)0.5);
      REAL endx = posx - vx2 * cfull;
      REAL endy = posy - vy2 * cfull;
      REAL v = SAMPLE(vy, vyw, vyh, endx, endy - (REAL)0.5);
      AT(vyo, vyw, x, y) = v * AT(flag, W, x, y) * AT(flag, W, x, y + 1);
    }
  }
  (void)vyh;
  s->fx = 1 - s->fx;
  s->fy = 1 - s->fy;
}
#undef SAMPLE

/* -------------------------------------------------------------- projection */
/* project, simulation.cpp:164-208: divergence into f, explosion sinks, two
 * MG V-cycles, setPBC, pressure-gradient update of the interior faces.
 * Options of the extension solvers:
 *  meanfree: the solver's system has zero-gradient edges everywhere, so it
 *    is singular and only the part of f orthogonal to the constants is
 *    solvable; the mean of f over the interior fluid cells (sum in double)
 *    is subtracted from those cells before the V-cycles (tolerance modes);
 *  zgbc_first: the zero-gradient edges are applied to p before the first
 *    V-cycle, which makes k V-cycles equal (in exact arithmetic) to the
 *    mixed-precision solver's k defect corrections. */
void FN(project_opts)(SIM_T *s, int ncycles, int meanfree, int zgbc_first) {
  int W = s->W, H = s->H;
  REAL ih = (REAL)1.0 / s->h;
  REAL *vx = s->vxb[s->fx], *vy = s->vyb[s->fy];
  const REAL *flag = s->flag;
  int vxw = W - 1, vyw = W;
  int y;
#pragma omp parallel for schedule(static)
  for (y = 1; y < H - 1; y++)
    for (int x = 1; x < W - 1; x++)
      AT(s->f, W, x, y) = -ih * (AT(vx, vxw, x, y) - AT(vx, vxw, x - 1, y) + AT(vy, vyw, x, y) -
                                 AT(vy, vyw, x, y - 1));
  /* sinks, simulation.cpp:173-187 */
  int keep = 0;
  for (int i = 0; i < s->nsinks; i++) {
    REAL gx = s->sinks[i][0] / s->h + (REAL)0.5;
    REAL gy = s->sinks[i][1] / s->h + (REAL)0.5;
    if (!(gx <= 3 || gx > (REAL)(W - 3) || gy <= 3 || gy > (REAL)(H - 3))) {
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++)
          AT(s->f, W, (int)(gx + (REAL)dx), (int)(gy + (REAL)dy)) = s->sinks[i][2];
      s->sinks[i][2] = (REAL)((double)s->sinks[i][2] * pow(0.000001, (double)(s->dt * (REAL)50)));
    }
  }
  for (int i = 0; i < s->nsinks; i++) {
    if (!(s->sinks[i][2] < (REAL)0.05)) {
      s->sinks[keep][0] = s->sinks[i][0];
      s->sinks[keep][1] = s->sinks[i][1];
      s->sinks[keep][2] = s->sinks[i][2];
      keep++;
    }
  }
  s->nsinks = keep;
  if (meanfree) {
    double sum = 0.0, n = 0.0;
    for (y = 1; y < H - 1; y++)
      for (int x = 1; x < W - 1; x++)
        if (AT(flag, W, x, y) != (REAL)0) {
          sum += (double)AT(s->f, W, x, y);
          n += 1.0;
        }
    REAL mean = n > 0.0 ? (REAL)(sum / n) : (REAL)0;
    for (y = 1; y < H - 1; y++)
      for (int x = 1; x < W - 1; x++)
        if (AT(flag, W, x, y) != (REAL)0) AT(s->f, W, x, y) -= mean;
  }
  if (zgbc_first) FN(zero_gradient_bc)(s->p, W, H);
  for (int c = 0; c < ncycles; c++) FN(mg_solve)(&s->mg, s->p, s->f, flag, s->h, 1);
  FN(set_pbc)(s);
#pragma omp parallel for schedule(static)
  for (y = 1; y < H - 1; y++)
    for (int x = 1; x < W - 2; x++)
      AT(vx, vxw, x, y) -= AT(flag, W, x, y) * AT(flag, W, x + 1, y) * ih *
                           (AT(s->p, W, x + 1, y) - AT(s->p, W, x, y));
#pragma omp parallel for schedule(static)
  for (y = 1; y < H - 2; y++)
    for (int x = 1; x < W - 1; x++)
      AT(vy, vyw, x, y) -= AT(flag, W, x, y) * AT(flag, W, x, y + 1) * ih *
                           (AT(s->p, W, x, y + 1) - AT(s->p, W, x, y));
}

void FN(project_ncycles)(SIM_T *s, int ncycles) { FN(project_opts)(s, ncycles, 0, 0); }
void FN(project)(SIM_T *s) { FN(project_ncycles)(s, 2); }

/* applyAccumulatedVelocity, simulation.cpp:376-396. */
void FN(apply_accum)(SIM_T *s) {
  int W = s->W, H = s->H;
  int vxw = W - 1, vxh = H, vyw = W, vyh = H - 1;
  REAL *vx = s->vxb[s->fx], *vy = s->vyb[s->fy];
  int y;
#pragma omp parallel for schedule(static)
  for (y = 1; y < vxh - 1; y++)
    for (int x = 1; x < vxw - 1; x++) {
      AT(vx, vxw, x, y) += AT(s->vx_accum, vxw, x, y);
      AT(s->vx_accum, vxw, x, y) = 0;
    }
#pragma omp parallel for schedule(static)
  for (y = 1; y < vyh - 1; y++)
    for (int x = 1; x < vyw - 1; x++) {
      AT(vy, vyw, x, y) += AT(s->vy_accum, vyw, x, y);
      AT(s->vy_accum, vyw, x, y) = 0;
    }
}

/* step, simulation.cpp:356-374. */
void FN(step_ncycles)(SIM_T *s, REAL dt, int ncycles) {
  s->dt = dt;
  FN(apply_accum)(s);
  FN(diffuse)(s);
  FN(advect)(s);
  FN(set_vbcs)(s);
  FN(project_ncycles)(s, ncycles);
  FN(set_vbcs)(s);
}
void FN(step)(SIM_T *s, REAL dt) { FN(step_ncycles)(s, dt, 2); }

/* --------------------------------------------------------- construction */
/* Simulation(flag, pwidth, mu), simulation.hpp:32-67. */
SIM_T *FN(create)(const REAL *flag, int W, int H, REAL pwidth, REAL mu) {
  if (W < 8 || H < 8) return NULL;
  SIM_T *s = (SIM_T *)calloc(1, sizeof(SIM_T));
  s->W = W;
  s->H = H;
  s->pwidth = pwidth;
  s->mu = mu;
  size_t nx = (size_t)(W - 1) * H, ny = (size_t)W * (H - 1), n = (size_t)W * H;
  for (int b = 0; b < 2; b++) {
    s->vxb[b] = FN(alloc)(nx);
    s->vyb[b] = FN(alloc)(ny);
  }
  s->vx_accum = FN(alloc)(nx);
  s->vy_accum = FN(alloc)(ny);
  s->p = FN(alloc)(n);
  s->f = FN(alloc)(n);
  s->flag = FN(alloc)(n);
  s->r = FN(alloc)(n);
  memcpy(s->flag, flag, n * sizeof(REAL));
  s->bcSouth = UBO_BC_NOSLIP;
  s->bcNorth = UBO_BC_NOSLIP;
  s->bcWest = UBO_BC_INFLOW;
  s->bcEast = UBO_BC_OUTFLOW_ZERO_PRESSURE;
  for (int x = 0; x < W; x++) s->vyb[0][x] = s->vyb[1][x] = 0;
  for (int y = 0; y < H; y++) AT(s->vxb[0], W - 1, 0, y) = AT(s->vxb[1], W - 1, 0, y) = 1;
  if (FN(mg_init)(&s->mg, W, H) != 0) {
    free(s);
    return NULL;
  }
  FN(mg_update_fields)(&s->mg, s->flag);
  s->h = pwidth / ((REAL)W - (REAL)1.0);
  return s;
}

void FN(destroy)(SIM_T *s) {
  if (!s) return;
  for (int b = 0; b < 2; b++) {
    free(s->vxb[b]);
    free(s->vyb[b]);
  }
  free(s->vx_accum);
  free(s->vy_accum);
  free(s->p);
  free(s->f);
  free(s->flag);
  free(s->r);
  FN(mg_free)(&s->mg);
  free(s);
}

/* Field access for the harness: which = UBO_FIELD_*. */
REAL *FN(field)(SIM_T *s, int which, int *w, int *h) {
  int W = s->W, H = s->H;
  switch (which) {
    case UBO_FIELD_VX: *w = W - 1; *h = H; return s->vxb[s->fx];
    case UBO_FIELD_VY: *w = W; *h = H - 1; return s->vyb[s->fy];
    case UBO_FIELD_VX_BACK: *w = W - 1; *h = H; return s->vxb[1 - s->fx];
    case UBO_FIELD_VY_BACK: *w = W; *h = H - 1; return s->vyb[1 - s->fy];
    case UBO_FIELD_P: *w = W; *h = H; return s->p;
    case UBO_FIELD_F: *w = W; *h = H; return s->f;
    case UBO_FIELD_FLAG: *w = W; *h = H; return s->flag;
    case UBO_FIELD_VX_ACCUM: *w = W - 1; *h = H; return s->vx_accum;
    case UBO_FIELD_VY_ACCUM: *w = W; *h = H - 1; return s->vy_accum;
    default: return NULL;
  }
}

void FN(get_field)(SIM_T *s, int which, REAL *dst) {
  int w, h;
  REAL *src = FN(field)(s, which, &w, &h);
  if (src) memcpy(dst, src, sizeof(REAL) * (size_t)w * h);
}
void FN(set_field)(SIM_T *s, int which, const REAL *src) {
  int w, h;
  REAL *dst = FN(field)(s, which, &w, &h);
  if (dst) memcpy(dst, src, sizeof(REAL) * (size_t)w * h);
}
/* memcpy(sim.flag...) + mg.updateFields (ubootgl_app.cpp:111-112). */
void FN(update_flag)(SIM_T *s, const REAL *flag) {
  memcpy(s->flag, flag, sizeof(REAL) * (size_t)s->W * s->H);
  FN(mg_update_fields)(&s->mg, s->flag);
}
void FN(set_dt)(SIM_T *s, REAL dt) { s->dt = dt; }
REAL FN(get_h)(SIM_T *s) { return s->h; }
int FN(mg_levels)(SIM_T *s) { return s->mg.levels; }
void FN(mg_level_flag)(SIM_T *s, int level, REAL *dst) {
  memcpy(dst, s->mg.flagcs[level], sizeof(REAL) * (size_t)s->mg.lw[level] * s->mg.lh[level]);
}
void FN(mg_level_size)(SIM_T *s, int level, int *w, int *h) {
  *w = s->mg.lw[level];
  *h = s->mg.lh[level];
}
void FN(sim_mg_solve)(SIM_T *s, int zgbc) { FN(mg_solve)(&s->mg, s->p, s->f, s->flag, s->h, zgbc); }
int FN(add_sink)(SIM_T *s, REAL x, REAL y, REAL z) {
  if (s->nsinks >= UBO_MAXSINKS) return -1;
  s->sinks[s->nsinks][0] = x;
  s->sinks[s->nsinks][1] = y;
  s->sinks[s->nsinks][2] = z;
  s->nsinks++;
  return 0;
}

/* Standalone MG (class MG): MG(width, height) keeps all coarse flags at 1.0
 * unless update is given a flag (MG(flag) calls updateFields). */
MG_T *FN(mg_create)(int w, int h, const REAL *flag) {
  MG_T *mg = (MG_T *)calloc(1, sizeof(MG_T));
  if (FN(mg_init)(mg, w, h) != 0 || mg->levels < 2) {
    FN(mg_free)(mg);
    free(mg);
    return NULL;
  }
  if (flag) FN(mg_update_fields)(mg, flag);
  return mg;
}
void FN(mg_destroy)(MG_T *mg) {
  if (!mg) return;
  FN(mg_free)(mg);
  free(mg);
}
int FN(mg_nlevels)(MG_T *mg) { return mg->levels; }

#undef SIM_T
#undef MG_T
#undef FN
