// C++ drop-in for the reference's Simulation and MG classes
// (simulation.hpp:18-141, pressure_solver.hpp:13-76, db2dgrid.hpp:12-108 of
// te42kyfo/ubootgl) over the C ABI in include/ubootgl_gb300.h.
//
// Same class names, constructors, methods and public members, so callers
// written against the reference compile unchanged.  The fields live on the
// GPU; the public grid members are host mirrors:
//   * step() uploads vx_accum / vy_accum (under accum_mutex) and new sinks,
//     steps on the device, and refreshes vx_current / vy_current;
//   * pull() refreshes every mirror from the device, push() sends the
//     mirrors of vx, vy (both buffers), p and flag back (for code that edits
//     the fields directly);
//   * mg.updateFields(flag) uploads the flag and rebuilds the hierarchy on
//     the device;
//   * setGrids edits the mirrors and the device in one call; bilinearVel
//     samples the device's current velocity.
// Errors from the library throw std::runtime_error with its message.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../include/ubootgl_gb300.h"

namespace ubootgl_gb300 {

inline void ubg_check(int rc) {
  if (rc != UBG_OK) throw std::runtime_error(std::string("ubootgl_gb300: ") + ubg_last_error());
}

// db2dgrid.hpp:12-50: row-major w x h floats, v[y * width + x].
class Single2DGrid {
 public:
  Single2DGrid(int width, int height)
      : width(width), height(height), v((size_t)width * height, 0.0f) {}
  Single2DGrid() : width(0), height(0) {}
  int idx(int x, int y) const { return y * width + x; }
  float *data() { return v.data(); }
  const float *data() const { return v.data(); }
  float &operator()(int x, int y) { return v[(size_t)idx(x, y)]; }
  float operator()(int x, int y) const { return v[(size_t)idx(x, y)]; }
  // glm::ivec2 (or any type with x, y; floating coordinates truncate)
  template <class V>
  float &operator()(const V &c) {
    return (*this)((int)c.x, (int)c.y);
  }
  template <class V>
  float operator()(const V &c) const {
    return (*this)((int)c.x, (int)c.y);
  }
  void fill(float val) { std::fill(v.begin(), v.end(), val); }
  int width, height;
  std::vector<float> v;
};

// db2dgrid.hpp:52-108: front / back buffers, f() / b(), swap().
class DoubleBuffered2DGrid {
 public:
  DoubleBuffered2DGrid(int width, int height)
      : width(width), height(height), front(0), back(1),
        v{std::vector<float>((size_t)width * height), std::vector<float>((size_t)width * height)} {}
  DoubleBuffered2DGrid() : width(0), height(0), front(0), back(1) {}
  int idx(int x, int y) const { return y * width + x; }
  void swap() { std::swap(front, back); }
  float &f(int x, int y) { return v[front][(size_t)idx(x, y)]; }
  float &b(int x, int y) { return v[back][(size_t)idx(x, y)]; }
  float f(int x, int y) const { return v[front][(size_t)idx(x, y)]; }
  float b(int x, int y) const { return v[back][(size_t)idx(x, y)]; }
  template <class V>
  float &f(const V &c) {
    return f((int)c.x, (int)c.y);
  }
  template <class V>
  float &b(const V &c) {
    return b((int)c.x, (int)c.y);
  }
  float &operator()(int x, int y) { return f(x, y); }
  float operator()(int x, int y) const { return f(x, y); }
  template <class V>
  float &operator()(const V &c) {
    return f((int)c.x, (int)c.y);
  }
  float *data() { return v[front].data(); }
  const float *data() const { return v[front].data(); }
  float *back_data() { return v[back].data(); }
  int width, height;
  int front, back;
  std::vector<float> v[2];
};

// class MG (pressure_solver.hpp:13-76).  A standalone MG owns a device
// hierarchy; the Simulation's member mg is bound to the simulation.
class MG {
 public:
  MG() {}
  MG(int width, int height) { ubg_check(ubg_mg_create(width, height, nullptr, &h_)); }
  explicit MG(Single2DGrid &flag) {
    ubg_check(ubg_mg_create(flag.width, flag.height, flag.data(), &h_));
  }
  MG(const MG &) = delete;
  MG &operator=(const MG &) = delete;
  MG(MG &&o) noexcept : h_(o.h_), sim_(o.sim_) {
    o.h_ = nullptr;
    o.sim_ = nullptr;
  }
  MG &operator=(MG &&o) noexcept {
    if (this != &o) {
      reset();
      h_ = o.h_;
      sim_ = o.sim_;
      o.h_ = nullptr;
      o.sim_ = nullptr;
    }
    return *this;
  }
  ~MG() { reset(); }

  // MG::updateFields(flag), pressure_solver.hpp:34-57
  void updateFields(Single2DGrid &flag) {
    if (sim_)
      ubg_check(ubg_upload(sim_, UBG_FLAG, flag.data()));
    else if (h_)
      ubg_check(ubg_mg_update_fields(h_, flag.data()));
    else
      throw std::runtime_error("ubootgl_gb300: MG not constructed");
  }

  // MG::solve(p, f, flag, h, zeroGradientBC), pressure_solver.hpp:59-62, on
  // host grids (p in place).  A Simulation's bound mg solves its own
  // device-resident p / f instead: use Simulation::project.
  void solve(Single2DGrid &p, Single2DGrid &f, Single2DGrid &flag, float h,
             bool zeroGradientBC = false) {
    if (!h_) throw std::runtime_error("ubootgl_gb300: standalone MG needed for host-grid solve");
    ubg_check(ubg_mg_solve(h_, p.data(), f.data(), flag.data(), h, zeroGradientBC ? 1 : 0));
  }

 private:
  friend class Simulation;
  void reset() {
    if (h_) ubg_mg_destroy(h_);
    h_ = nullptr;
    sim_ = nullptr;
  }
  ubg_mg *h_ = nullptr;
  ubg_sim *sim_ = nullptr;
};

// glm::vec3 stand-in for the sinks vector (any type with x, y, z converts).
struct Sink {
  float x = 0, y = 0, z = 0;
  Sink() {}
  Sink(float x, float y, float z) : x(x), y(y), z(z) {}
  template <class V>
  Sink(const V &v) : x(v.x), y(v.y), z(v.z) {}
};

class Simulation {
 public:
  enum class BC { INFLOW, OUTFLOW, OUTFLOW_ZERO_PRESSURE, NOSLIP };

  // Simulation(const Single2DGrid &flag, float pwidth, float mu),
  // simulation.hpp:32-67
  Simulation(const Single2DGrid &flagInput, float pwidth, float mu)
      : pwidth(pwidth), mu(mu), width(flagInput.width), height(flagInput.height) {
    vx = DoubleBuffered2DGrid(width - 1, height);
    vy = DoubleBuffered2DGrid(width, height - 1);
    vx_accum = Single2DGrid(width - 1, height);
    vy_accum = Single2DGrid(width, height - 1);
    vx_current = Single2DGrid(width - 1, height);
    vy_current = Single2DGrid(width, height - 1);
    p = Single2DGrid(width, height);
    f = Single2DGrid(width, height);
    flag = flagInput;
    r = Single2DGrid(width, height);
    bcSouth = BC::NOSLIP;
    bcNorth = BC::NOSLIP;
    bcWest = BC::INFLOW;
    bcEast = BC::OUTFLOW_ZERO_PRESSURE;
    ubg_check(ubg_create(flag.data(), width, height, pwidth, mu, &h_));
    mg.sim_ = h_;
    h = pwidth / (width - 1.0f);
    applied_bc_[0] = bcWest;
    applied_bc_[1] = bcEast;
    applied_bc_[2] = bcNorth;
    applied_bc_[3] = bcSouth;
    pull();
  }
  Simulation(const Simulation &) = delete;
  Simulation &operator=(const Simulation &) = delete;
  ~Simulation() {
    mg.sim_ = nullptr;
    if (h_) ubg_destroy(h_);
  }

  // Simulation::step(float timestep), simulation.cpp:356-374
  void step(float timestep) {
    dt = timestep;
    sync_in();
    ubg_check(ubg_step(h_, timestep));
    download(UBG_VX_CURRENT, vx_current);
    download(UBG_VY_CURRENT, vy_current);
  }

  // The stages, on the device with the member dt (simulation.cpp:104-396).
  void applyAccumulatedVelocity() {
    sync_in();
    ubg_check(ubg_apply_accumulated_velocity(h_));
  }
  void diffuse() { ubg_check(ubg_diffuse(h_, dt)); }
  void advect() { ubg_check(ubg_advect(h_, dt)); }
  void setVBCs() { ubg_check(ubg_set_vbcs(h_)); }
  void setPBC() { ubg_check(ubg_set_pbc(h_)); }
  void project() {
    sync_in();
    ubg_check(ubg_project(h_, dt));
  }
  void saveCurrentVelocityFields() {
    download(UBG_VX_CURRENT, vx_current);
    download(UBG_VY_CURRENT, vy_current);
  }

  // getDT, simulation.cpp:226-238, on the device's current fields
  float getDT() {
    pull();
    float max_vel = 1.0e-7f;
    for (int y = 1; y < height - 1; y++)
      for (int x = 1; x < width - 1; x++) max_vel = std::max(max_vel, std::max(vx(x, y), vy(x, y)));
    return pwidth / (width - 1.0f) / max_vel * 2.5f;
  }

  // centerP, simulation.cpp:209-223
  void centerP() {
    download(UBG_P, p);
    float avgP = 0;
    for (int y = 1; y < height - 1; y++)
      for (int x = 1; x < width - 1; x++) avgP += p(x, y);
    for (int y = 1; y < height - 1; y++)
      for (int x = 1; x < width - 1; x++) p(x, y) -= avgP / width / height;
    ubg_check(ubg_upload(h_, UBG_P, p.data()));
  }

  // setGrids(glm::ivec2 c, float val), simulation.hpp:82-98: the mirrors
  // and the device (which also rebuilds the multigrid flags)
  template <class IV>
  void setGrids(IV c, float val) {
    int x = (int)c.x, y = (int)c.y;
    if (!(x >= 0 && y >= 0 && x < width && y < height)) return;
    flag(x, y) = val;
    if (val == 0) {
      if (x < vx.width) vx.f(x, y) = 0.0f;
      if (x > 0) vx.f(x - 1, y) = 0.0f;
      if (y < vy.height) vy.f(x, y) = 0.0f;
      if (y > 0) vy.f(x, y - 1) = 0.0f;
      p(x, y) = 0.0f;
    }
    int xy[2] = {x, y};
    ubg_check(ubg_set_grids(h_, 1, xy, &val));
  }

  // bilinearVel(c), advect_floating_items.cpp:11-14, on the device
  template <class V>
  V bilinearVel(V c) {
    float in[2] = {(float)c.x, (float)c.y}, out[2];
    ubg_check(ubg_sample_velocity(h_, 1, in, out));
    V r = c;
    r.x = out[0];
    r.y = out[1];
    return r;
  }

  // psampleFlag*, simulation.cpp:398-425, on the flag mirror
  template <class V>
  float psampleFlagNearest(V pc) {
    float gx = pc.x / (pwidth / (flag.width)), gy = pc.y / (pwidth / (flag.width));
    return flag((int)gx, (int)gy);
  }
  template <class V>
  float psampleFlagLinear(V pc) {
    float cx = pc.x / (pwidth / (flag.width)) - 0.5f, cy = pc.y / (pwidth / (flag.width)) - 0.5f;
    int ix = (int)cx, iy = (int)cy;
    ix = std::max(0, std::min(flag.width - 2, ix));
    iy = std::max(0, std::min(flag.height - 2, iy));
    float sx = cx - std::floor(cx), sy = cy - std::floor(cy);
    float p01 = flag(ix, iy + 1), p11 = flag(ix + 1, iy + 1);
    float p00 = flag(ix, iy), p10 = flag(ix + 1, iy);
    float a = p00 * (1.0f - sx) + p10 * sx, b = p01 * (1.0f - sx) + p11 * sx;
    return a * (1.0f - sy) + b * sy;
  }
  template <class V>
  V psampleFlagNormal(V pc) {
    V q = pc;
    auto at = [&](float dx, float dy) {
      q.x = pc.x + dx;
      q.y = pc.y + dy;
      return psampleFlagLinear(q);
    };
    float p01 = at(-h, h), p11 = at(h, h), p00 = at(-h, -h), p10 = at(h, -h);
    V r = pc;
    r.x = p11 + p10 - p01 - p00;
    r.y = p01 + p11 - p00 - p10;
    return r;
  }

  // ---- mirror synchronisation (extension)
  void pull() {
    ubg_check(ubg_sync(h_));
    download(UBG_VX, vx.v[vx.front]);
    download(UBG_VX_BACK, vx.v[vx.back]);
    download(UBG_VY, vy.v[vy.front]);
    download(UBG_VY_BACK, vy.v[vy.back]);
    download(UBG_P, p);
    download(UBG_F, f);
    download(UBG_FLAG, flag);
    download(UBG_VX_CURRENT, vx_current);
    download(UBG_VY_CURRENT, vy_current);
  }
  void push() {
    ubg_check(ubg_upload(h_, UBG_VX, vx.v[vx.front].data()));
    ubg_check(ubg_upload(h_, UBG_VX_BACK, vx.v[vx.back].data()));
    ubg_check(ubg_upload(h_, UBG_VY, vy.v[vy.front].data()));
    ubg_check(ubg_upload(h_, UBG_VY_BACK, vy.v[vy.back].data()));
    ubg_check(ubg_upload(h_, UBG_P, p.data()));
    ubg_check(ubg_upload(h_, UBG_FLAG, flag.data()));
  }
  ubg_sim *handle() const { return h_; }

  float pwidth;
  float mu;
  int width, height;
  float dt = 0.0f;
  BC bcWest, bcEast, bcNorth, bcSouth;
  DoubleBuffered2DGrid vx, vy;
  Single2DGrid vx_accum, vy_accum;
  Single2DGrid vx_current, vy_current;
  std::mutex accum_mutex;
  Single2DGrid p, f, flag, r;
  MG mg;
  float h;
  std::vector<Sink> sinks;

 private:
  void download(int field, Single2DGrid &g) { ubg_check(ubg_download(h_, field, g.data())); }
  void download(int field, std::vector<float> &v) { ubg_check(ubg_download(h_, field, v.data())); }

  // boundary types, accumulated velocity and sinks before a step / stage
  void sync_in() {
    BC now[4] = {bcWest, bcEast, bcNorth, bcSouth};
    if (!std::equal(now, now + 4, applied_bc_)) {
      ubg_check(ubg_set_bcs(h_, (int)bcWest, (int)bcEast, (int)bcNorth, (int)bcSouth));
      std::copy(now, now + 4, applied_bc_);
    }
    {
      std::lock_guard<std::mutex> lock(accum_mutex);
      ubg_check(ubg_upload(h_, UBG_VX_ACCUM, vx_accum.data()));
      ubg_check(ubg_upload(h_, UBG_VY_ACCUM, vy_accum.data()));
      // applyAccumulatedVelocity zeroes the interior (simulation.cpp:376-396)
      for (int y = 1; y < vx_accum.height - 1; y++)
        for (int x = 1; x < vx_accum.width - 1; x++) vx_accum(x, y) = 0.0f;
      for (int y = 1; y < vy_accum.height - 1; y++)
        for (int x = 1; x < vy_accum.width - 1; x++) vy_accum(x, y) = 0.0f;
    }
    for (const Sink &s : sinks) ubg_check(ubg_add_sink(h_, s.x, s.y, s.z));
    sinks.clear();
  }

  ubg_sim *h_ = nullptr;
  BC applied_bc_[4];
};

}  // namespace ubootgl_gb300

#ifndef UBOOTGL_GB300_NO_GLOBAL_NAMES
using ubootgl_gb300::DoubleBuffered2DGrid;
using ubootgl_gb300::MG;
using ubootgl_gb300::Simulation;
using ubootgl_gb300::Single2DGrid;
#endif
