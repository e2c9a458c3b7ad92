// Caller written against the reference's classes (Simulation, MG,
// Single2DGrid), compiled against the drop-in header.  Reads a case from
// <dir>: meta.txt (W H nsteps), flag.bin, vx.bin, vy.bin, dts.bin,
// mg_p.bin, mg_f.bin (float32, row-major); writes out_vx.bin, out_vy.bin,
// out_p.bin (after the steps) and out_mg_p.bin (one MG::solve with
// zero-gradient edges on a standalone MG(flag)).
#include <cstdio>
#include <string>
#include <vector>

#include "simulation.hpp"

static std::vector<float> load(const std::string &fn, size_t n) {
  std::vector<float> v(n);
  FILE *f = std::fopen(fn.c_str(), "rb");
  if (!f || std::fread(v.data(), 4, n, f) != n) throw std::runtime_error("read " + fn);
  std::fclose(f);
  return v;
}
static void save(const std::string &fn, const float *p, size_t n) {
  FILE *f = std::fopen(fn.c_str(), "wb");
  if (!f || std::fwrite(p, 4, n, f) != n) throw std::runtime_error("write " + fn);
  std::fclose(f);
}

struct ivec2 {
  int x, y;
};

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  std::string d = argv[1];
  int W = 0, H = 0, n = 0;
  FILE *m = std::fopen((d + "/meta.txt").c_str(), "r");
  if (!m || std::fscanf(m, "%d %d %d", &W, &H, &n) != 3) return 2;
  std::fclose(m);
  try {
    Single2DGrid flag(W, H);
    flag.v = load(d + "/flag.bin", (size_t)W * H);
    Simulation sim(flag, 1.0f, 1e-4f);
    auto vx = load(d + "/vx.bin", (size_t)(W - 1) * H);
    auto vy = load(d + "/vy.bin", (size_t)W * (H - 1));
    sim.vx.v[0] = vx;
    sim.vx.v[1] = vx;
    sim.vy.v[0] = vy;
    sim.vy.v[1] = vy;
    sim.push();
    auto dts = load(d + "/dts.bin", (size_t)n);
    for (int i = 0; i < n; i++) sim.step(dts[i]);
    sim.pull();
    save(d + "/out_vx.bin", sim.vx.data(), (size_t)(W - 1) * H);
    save(d + "/out_vy.bin", sim.vy.data(), (size_t)W * (H - 1));
    save(d + "/out_p.bin", sim.p.data(), (size_t)W * H);
    // the display mirrors equal the front buffers after a step
    for (size_t i = 0; i < sim.vx_current.v.size(); i++)
      if (sim.vx_current.v[i] != sim.vx.v[sim.vx.front][i]) return 3;
    // setGrids through the drop-in, then one more step
    sim.setGrids(ivec2{W / 2, H / 2}, 0.0f);
    if (sim.flag(W / 2, H / 2) != 0.0f) return 4;

    MG mg(flag);
    Single2DGrid p(W, H), f(W, H);
    p.v = load(d + "/mg_p.bin", (size_t)W * H);
    f.v = load(d + "/mg_f.bin", (size_t)W * H);
    mg.solve(p, f, flag, sim.h, true);
    save(d + "/out_mg_p.bin", p.data(), (size_t)W * H);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
