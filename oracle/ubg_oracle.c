/*
 * CPU restatement of ubootgl's fluid step -- TEST INFRASTRUCTURE ONLY.
 *
 * Builds liboracle.so (see build_oracle.py) with an FP32 instance (ubo_f_*,
 * the parity oracle) and an FP64 instance (ubo_d_*, the accuracy oracle) of
 * ubg_oracle_impl.h.  Loaded by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py only.
 *
 * Parity pin: tests/test_oracle_vs_reference.py checks the FP32 instance
 * against the reference's own simulation.cpp + pressure_solver.cpp, compiled
 * from source into oracle/_ref by oracle/ref/build_ref.py, and against the
 * golden fixtures in tests/golden/ that the same reference build produced.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define UBO_MAXL 24
#define UBO_MAXSINKS 256

enum { UBO_BC_INFLOW = 0, UBO_BC_OUTFLOW = 1, UBO_BC_OUTFLOW_ZERO_PRESSURE = 2, UBO_BC_NOSLIP = 3 };
enum {
  UBO_FIELD_VX = 0,
  UBO_FIELD_VY = 1,
  UBO_FIELD_VX_BACK = 2,
  UBO_FIELD_VY_BACK = 3,
  UBO_FIELD_P = 4,
  UBO_FIELD_F = 5,
  UBO_FIELD_FLAG = 6,
  UBO_FIELD_VX_ACCUM = 7,
  UBO_FIELD_VY_ACCUM = 8
};

#define REAL float
#define SFX f
#define FMA(a, b, c) fmaf((a), (b), (c))
#include "ubg_oracle_impl.h"
#undef REAL
#undef SFX
#undef FMA

#define REAL double
#define SFX d
#define FMA(a, b, c) fma((a), (b), (c))
#include "ubg_oracle_impl.h"
#undef REAL
#undef SFX
#undef FMA

int ubo_omp_max_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void ubo_omp_set_threads(int n) {
#ifdef _OPENMP
  extern void omp_set_num_threads(int);
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
