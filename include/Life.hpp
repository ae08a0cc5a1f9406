// Life.hpp -- drop-in for the class Paraiso generates from
// examples/Life/Generator.hs (statics cell :: Array Int, population and
// generation :: Scalar Int; kernels init and proceed), backed by the GB300
// runtime.  examples/Life/main.cpp builds against it unchanged:
//   g++ main.cpp -I<repo>/include -L<repo>/paraiso_gb300 -lom_gb300
// The earlier generator's members (static_0_population,
// static_1_generation, static_2_cell, memorySize0(), ...) are here too, so
// examples/Life/main.cu builds unchanged as well.
#pragma once

#include "om_shim.hpp"

class Life : public om_shim::machine {
 public:
  // the example's Native.Setup: 80 x 48, cyclic (Generator.hs:39-44)
  Life() : Life(80, 48) {}
  Life(int n0, int n1, int boundary = OM_BOUNDARY_CYCLIC)
      : om_shim::machine(OM_KIND_LIFE, n0, n1, config(boundary)), cell_(h_, "cell"),
        static_0_population(h_, "population"), static_1_generation(h_, "generation"),
        static_2_cell(h_, "cell") {}

  int &population() { return scalar<int>("population"); }
  int &generation() { return scalar<int>("generation"); }
  om_shim::host_array<int> &cell() { return cell_; }
  int &cell(int i0, int i1) { return element<int>("cell", i0, i1); }

  void init() { run("init"); }
  void proceed() { run("proceed"); }

 private:
  om_shim::host_array<int> cell_;

 public:
  // the earlier generator's statics (examples-old/Life-exampled/dist/Life.hpp)
  om_shim::scalar_member<int> static_0_population, static_1_generation;
  om_shim::array_member<int> static_2_cell;

 private:
  static om_config config(int boundary) {
    om_config c;
    om_config_default(&c);
    c.boundary = boundary;
    return c;
  }
};
