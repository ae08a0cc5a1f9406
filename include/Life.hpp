// Life.hpp -- drop-in for the class Paraiso generates from
// examples/Life/Generator.hs (statics cell :: Array Int, population and
// generation :: Scalar Int; kernels init and proceed), backed by the GB300
// runtime.  examples/Life/main.cpp builds against it unchanged:
//   g++ main.cpp -I<repo>/include -L<repo>/paraiso_gb300 -lom_gb300
#pragma once

#include "om_shim.hpp"

class Life : public om_shim::machine {
 public:
  // the example's Native.Setup: 80 x 48, cyclic (Generator.hs:39-44)
  Life() : Life(80, 48) {}
  Life(int n0, int n1, int boundary = OM_BOUNDARY_CYCLIC)
      : om_shim::machine(OM_KIND_LIFE, n0, n1, config(boundary)), cell_(h_, "cell") {}

  int &population() { return scalar<int>("population"); }
  int &generation() { return scalar<int>("generation"); }
  om_shim::host_array<int> &cell() { return cell_; }
  int &cell(int i0, int i1) { return element<int>("cell", i0, i1); }

  void init() { run("init"); }
  void proceed() { run("proceed"); }

 private:
  static om_config config(int boundary) {
    om_config c;
    om_config_default(&c);
    c.boundary = boundary;
    return c;
  }
  om_shim::host_array<int> cell_;
};
