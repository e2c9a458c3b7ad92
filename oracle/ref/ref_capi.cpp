// C entry points over the reference's own Simulation / MG classes, so that
// the tests can drive the unmodified reference (simulation.cpp,
// pressure_solver.cpp of te42kyfo/ubootgl) through ctypes.  Compiled into
// oracle/_ref/libubgref.so by build_ref.py; TEST INFRASTRUCTURE ONLY.
#include <omp.h>
#include <cstring>
#include "simulation.hpp"
#include "interpolators.hpp"

namespace {
enum { F_VX = 0, F_VY = 1, F_VX_BACK = 2, F_VY_BACK = 3, F_P = 4, F_F = 5, F_FLAG = 6,
       F_VX_ACCUM = 7, F_VY_ACCUM = 8 };

float *field_ptr(Simulation *s, int which, size_t *n) {
  switch (which) {
    case F_VX: *n = (size_t)s->vx.width * s->vx.height; return s->vx.data();
    case F_VY: *n = (size_t)s->vy.width * s->vy.height; return s->vy.data();
    case F_VX_BACK: *n = (size_t)s->vx.width * s->vx.height; return s->vx.back_data();
    case F_VY_BACK: *n = (size_t)s->vy.width * s->vy.height; return s->vy.back_data();
    case F_P: *n = (size_t)s->p.width * s->p.height; return s->p.data();
    case F_F: *n = (size_t)s->f.width * s->f.height; return s->f.data();
    case F_FLAG: *n = (size_t)s->flag.width * s->flag.height; return s->flag.data();
    case F_VX_ACCUM: *n = (size_t)s->vx_accum.width * s->vx_accum.height; return s->vx_accum.data();
    case F_VY_ACCUM: *n = (size_t)s->vy_accum.width * s->vy_accum.height; return s->vy_accum.data();
  }
  *n = 0;
  return nullptr;
}
}  // namespace

extern "C" {

void ref_set_threads(int n) { omp_set_num_threads(n); }

void *ref_create(const float *flag, int w, int h, float pwidth, float mu) {
  Single2DGrid fl(w, h);
  std::memcpy(fl.data(), flag, sizeof(float) * (size_t)w * h);
  return new Simulation(fl, pwidth, mu);
}
void ref_destroy(void *s) { delete static_cast<Simulation *>(s); }

void ref_set_field(void *sp, int which, const float *src) {
  size_t n;
  float *dst = field_ptr(static_cast<Simulation *>(sp), which, &n);
  if (dst) std::memcpy(dst, src, n * sizeof(float));
}
void ref_get_field(void *sp, int which, float *dst) {
  size_t n;
  float *src = field_ptr(static_cast<Simulation *>(sp), which, &n);
  if (src) std::memcpy(dst, src, n * sizeof(float));
}
void ref_update_flag(void *sp, const float *flag) {
  auto *s = static_cast<Simulation *>(sp);
  std::memcpy(s->flag.data(), flag, sizeof(float) * (size_t)s->width * s->height);
  s->mg.updateFields(s->flag);
}
float ref_get_h(void *sp) { return static_cast<Simulation *>(sp)->h; }
void ref_set_dt(void *sp, float dt) { static_cast<Simulation *>(sp)->dt = dt; }
void ref_step(void *sp, float dt) { static_cast<Simulation *>(sp)->step(dt); }
void ref_apply_accum(void *sp) { static_cast<Simulation *>(sp)->applyAccumulatedVelocity(); }
void ref_diffuse(void *sp) { static_cast<Simulation *>(sp)->diffuse(); }
void ref_advect(void *sp) { static_cast<Simulation *>(sp)->advect(); }
void ref_set_vbcs(void *sp) { static_cast<Simulation *>(sp)->setVBCs(); }
void ref_set_pbc(void *sp) { static_cast<Simulation *>(sp)->setPBC(); }
void ref_project(void *sp) { static_cast<Simulation *>(sp)->project(); }
void ref_mg_solve_sim(void *sp, int zgbc) {
  auto *s = static_cast<Simulation *>(sp);
  s->mg.solve(s->p, s->f, s->flag, s->h, zgbc != 0);
}
void ref_add_sink(void *sp, float x, float y, float z) {
  static_cast<Simulation *>(sp)->sinks.push_back(glm::vec3(x, y, z));
}

// Standalone MG (class MG) and the free functions of pressure_solver.hpp.
void *ref_mg_create(int w, int h, const float *flag) {
  if (!flag) return new MG(w, h);
  Single2DGrid fl(w, h);
  std::memcpy(fl.data(), flag, sizeof(float) * (size_t)w * h);
  return new MG(fl);
}
void ref_mg_destroy(void *m) { delete static_cast<MG *>(m); }
void ref_mg_solve(void *m, float *p, const float *f, const float *flag, int w, int h, float hh,
                  int zgbc) {
  Single2DGrid P(w, h), F(w, h), FL(w, h);
  size_t n = (size_t)w * h;
  std::memcpy(P.data(), p, n * 4);
  std::memcpy(F.data(), f, n * 4);
  std::memcpy(FL.data(), flag, n * 4);
  static_cast<MG *>(m)->solve(P, F, FL, hh, zgbc != 0);
  std::memcpy(p, P.data(), n * 4);
}
void ref_rbgs(float *p, const float *f, const float *flag, int w, int h, float hh) {
  Single2DGrid P(w, h), F(w, h), FL(w, h);
  size_t n = (size_t)w * h;
  std::memcpy(P.data(), p, n * 4);
  std::memcpy(F.data(), f, n * 4);
  std::memcpy(FL.data(), flag, n * 4);
  rbgs(P, F, FL, hh, 1.0f);
  std::memcpy(p, P.data(), n * 4);
}
float ref_residual(const float *p, const float *f, const float *flag, float *r, int w, int h,
                   float hh) {
  Single2DGrid P(w, h), F(w, h), FL(w, h), R(w, h);
  size_t n = (size_t)w * h;
  std::memcpy(P.data(), p, n * 4);
  std::memcpy(F.data(), f, n * 4);
  std::memcpy(FL.data(), flag, n * 4);
  float l2 = calculateResidualField(P, F, FL, R, hh);
  std::memcpy(r, R.data(), n * 4);
  return l2;
}

// bilinearSample / bilinearScatter (interpolators.hpp:11-40) over n points,
// the scatter sequential in item order, on a copy of a w x h grid.
void ref_bilinear_sample_n(const float *grid, int w, int h, int n, const float *xy, float *out) {
  Single2DGrid G(w, h);
  std::memcpy(G.data(), grid, (size_t)w * h * 4);
  for (int i = 0; i < n; i++) out[i] = bilinearSample(G, glm::vec2(xy[2 * i], xy[2 * i + 1]));
}
void ref_bilinear_scatter_n(float *grid, int w, int h, int n, const float *xy, const float *v) {
  Single2DGrid G(w, h);
  std::memcpy(G.data(), grid, (size_t)w * h * 4);
  for (int i = 0; i < n; i++) bilinearScatter(G, glm::vec2(xy[2 * i], xy[2 * i + 1]), v[i]);
  std::memcpy(grid, G.data(), (size_t)w * h * 4);
}
// Simulation::setGrids (simulation.hpp:82-98).
void ref_set_grids(void *sp, int x, int y, float val) {
  static_cast<Simulation *>(sp)->setGrids(glm::ivec2(x, y), val);
}

}  // extern "C"
