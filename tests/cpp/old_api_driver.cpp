// A driver written against the earlier generator's class members
// (static_<i>_<name>, size0(), memorySize0(), lowerMargin0(), as in
// examples/Life/main.cu and examples/Hydro/main-kh.cu), cross-checked with
// the current accessors of the same object.
#include <cmath>
#include <cstdio>
#include <vector>

#include "Hydro.hpp"
#include "Life.hpp"

int main() {
  int bad = 0;
  {
    Life sim(64, 40);
    sim.init();
    const int W = sim.memorySize0(), H = sim.memorySize1();
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) sim.static_2_cell[y * W + x] = ((x * 7 + y * 3) % 5) == 0;
    for (int t = 0; t < 10; ++t) sim.proceed();
    std::vector<int> cells = sim.static_2_cell;
    long pop = 0;
    for (int c : cells) pop += c;
    const int p_old = sim.static_0_population, g_old = sim.static_1_generation;
    if (pop != p_old || p_old != sim.population() || g_old != 10 || (int)cells.size() != W * H)
      ++bad;
    std::printf("life %d %d %ld\n", p_old, g_old, pop);
  }
  {
    Hydro sim(96, 64);
    const int W = sim.size0(), H = sim.size1();
    sim.static_1_time = 0;
    sim.static_2_cfl = 0.5;
    sim.static_5_extent0 = 1.0;
    sim.static_6_extent1 = 1.0;
    sim.static_3_dR0 = sim.static_5_extent0 / W;
    sim.static_4_dR1 = sim.static_6_extent1 / H;
    sim.init();
    for (int t = 0; t < 5; ++t) sim.proceed();
    std::vector<float> dens = sim.static_7_density;
    const double t_old = sim.static_1_time;
    const int i = sim.memorySize0() * (H / 2 + sim.lowerMargin1()) + W / 2 + sim.lowerMargin0();
    if (t_old != sim.time() || !(t_old > 0) || dens[i] != (float)sim.density(W / 2, H / 2) ||
        sim.dR0() != 1.0 / W)
      ++bad;
    std::printf("hydro %.17g %.9g\n", t_old, dens[i]);
  }
  std::printf("%s\n", bad ? "MISMATCH" : "ok");
  return bad;
}
