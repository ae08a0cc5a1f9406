// shim_driver.cpp -- a driver written against the generated-class interface
// (include/Life.hpp, include/Hydro.hpp), as examples/Life/main.cpp and
// examples/Hydro/main-kh.cpp are.  Built and run by tests/test_shims.py.
//   shim_driver life N0 N1 STEPS    -> prints "generation population" lines
//   shim_driver hydro N STEPS       -> prints "time" and the total mass
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "Hydro.hpp"
#include "Life.hpp"

int main(int argc, char **argv) {
  if (argc >= 5 && !std::strcmp(argv[1], "life")) {
    Life sim(std::atoi(argv[2]), std::atoi(argv[3]));
    const int W = sim.om_size_0(), H = sim.om_size_1();
    sim.init();
    // a glider and a blinker, written through the element accessor
    const int g[5][2] = {{1, 0}, {2, 1}, {0, 2}, {1, 2}, {2, 2}};
    for (auto &c : g) sim.cell(c[0] + 3, c[1] + 3) = 1;
    for (int x = 0; x < 3; ++x) sim.cell(W / 2 + x, H / 2) = 1;
    for (int t = 0; t < std::atoi(argv[4]); ++t) {
      sim.proceed();
      std::printf("%d %d\n", sim.generation(), sim.population());
    }
    long alive = 0;
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) alive += sim.cell(x, y);
    std::printf("alive %ld\n", alive);
    return 0;
  }
  if (argc >= 4 && !std::strcmp(argv[1], "hydro")) {
    const int n = std::atoi(argv[2]);
    Hydro sim(n, n, 1.4, OM_BOUNDARY_CYCLIC);
    sim.time() = 0;
    sim.cfl() = 0.4;
    sim.extent0() = 1.0;
    sim.extent1() = 1.0;
    sim.dR0() = sim.extent0() / n;
    sim.dR1() = sim.extent1() / n;
    sim.init();
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        const bool band = y > n / 4 && y < 3 * n / 4;
        sim.density(x, y) = band ? 2.0 : 1.0;
        sim.velocity0(x, y) = band ? 0.5 : -0.5;
        sim.velocity1(x, y) = 0.01 * ((x * 7 + y * 3) % 11 - 5) / 5.0;
        sim.pressure(x, y) = 2.5;
      }
    double mass0 = 0;
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) mass0 += sim.density(x, y);
    for (int t = 0; t < std::atoi(argv[3]); ++t) sim.proceed();
    double mass = 0;
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) mass += sim.density(x, y);
    std::printf("time %.17g\nmass0 %.17g\nmass %.17g\n", sim.time(), mass0, mass);
    return 0;
  }
  if (argc >= 4 && !std::strcmp(argv[1], "hydro_open")) {
    // the generated class's defaults: open boundary, gamma 5/3, jet init
    const int n = std::atoi(argv[2]);
    Hydro sim(n, n);
    sim.time() = 0;
    sim.cfl() = 0.5;
    sim.extent0() = 1.0;
    sim.extent1() = 1.0;
    sim.dR0() = sim.extent0() / n;
    sim.dR1() = sim.extent1() / n;
    sim.init();
    for (int t = 0; t < std::atoi(argv[3]); ++t) sim.proceed();
    double mass = 0, px = 0;
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        mass += sim.density(x, y);
        px += sim.density(x, y) * sim.velocity0(x, y);
      }
    std::printf("time %.17g\nmass %.17g\npx %.17g\nmargin %d\n", sim.time(), mass, px,
                sim.om_lower_margin_0());
    return 0;
  }
  std::fprintf(stderr,
               "usage: shim_driver life N0 N1 STEPS | hydro N STEPS | hydro_open N STEPS\n");
  return 2;
}
