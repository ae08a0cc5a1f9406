// Hydro.hpp -- drop-in for the class Paraiso generates from
// examples/Hydro/HydroMain.hs (statics generation :: Int; time, cfl, dR0,
// dR1, extent0, extent1 :: Real; density, velocity0, velocity1, pressure ::
// Array Real; kernels init and proceed), backed by the GB300 runtime.
// examples/Hydro/main-kh.cpp builds against it unchanged.
//
// Real is double as in examples/Hydro/Hydro.hs:37; define OM_HYDRO_FP32 to
// store the arrays in float and run the FP32 fused kernel (scalars stay
// double: time is accumulated in FP64).  The default mesh is the generated
// one: 1024 x 1024 with the open boundary of the generator's default setup
// (Language/Paraiso/Generator/Native.hs:36): 3-cell margins that take the
// jet state every step (HydroMain.hs:105-131).
//
// The earlier generator's members (static_0_generation .. static_10_pressure,
// size0(), memorySize0(), lowerMargin0(), ...) are here too, so
// examples/Hydro/main-kh.cu builds unchanged as well.
#pragma once

#include "om_shim.hpp"

class Hydro : public om_shim::machine {
 public:
#ifdef OM_HYDRO_FP32
  typedef float Real;
#else
  typedef double Real;
#endif
  // the example's mesh (HydroMain.hs:290-302), open, gamma 5/3
  Hydro() : Hydro(1024, 1024) {}
  Hydro(int n0, int n1, double gamma = 5.0 / 3.0, int boundary = OM_BOUNDARY_OPEN)
      : om_shim::machine(OM_KIND_HYDRO, n0, n1, config(gamma, boundary)),
        density_(h_, "density"), velocity0_(h_, "velocity0"),
        velocity1_(h_, "velocity1"), pressure_(h_, "pressure"),
        static_0_generation(h_, "generation"), static_1_time(h_, "time"),
        static_2_cfl(h_, "cfl"), static_3_dR0(h_, "dR0"), static_4_dR1(h_, "dR1"),
        static_5_extent0(h_, "extent0"), static_6_extent1(h_, "extent1"),
        static_7_density(h_, "density"), static_8_velocity0(h_, "velocity0"),
        static_9_velocity1(h_, "velocity1"), static_10_pressure(h_, "pressure") {}

  int &generation() { return scalar<int>("generation"); }
  double &time() { return scalar<double>("time"); }
  double &cfl() { return scalar<double>("cfl"); }
  double &dR0() { return scalar<double>("dR0"); }
  double &dR1() { return scalar<double>("dR1"); }
  double &extent0() { return scalar<double>("extent0"); }
  double &extent1() { return scalar<double>("extent1"); }

  om_shim::host_array<Real> &density() { return density_; }
  om_shim::host_array<Real> &velocity0() { return velocity0_; }
  om_shim::host_array<Real> &velocity1() { return velocity1_; }
  om_shim::host_array<Real> &pressure() { return pressure_; }
  Real &density(int i0, int i1) { return element<Real>("density", i0, i1); }
  Real &velocity0(int i0, int i1) { return element<Real>("velocity0", i0, i1); }
  Real &velocity1(int i0, int i1) { return element<Real>("velocity1", i0, i1); }
  Real &pressure(int i0, int i1) { return element<Real>("pressure", i0, i1); }

  void init() { run("init"); }
  void proceed() { run("proceed"); }

 private:
  om_shim::host_array<Real> density_, velocity0_, velocity1_, pressure_;

 public:
  // the earlier generator's statics (examples-old/Hydro-exampled/dist/Hydro.hpp)
  om_shim::scalar_member<int> static_0_generation;
  om_shim::scalar_member<double> static_1_time, static_2_cfl, static_3_dR0, static_4_dR1,
      static_5_extent0, static_6_extent1;
  om_shim::array_member<Real> static_7_density, static_8_velocity0, static_9_velocity1,
      static_10_pressure;

 private:
  static om_config config(double gamma, int boundary) {
    om_config c;
    om_config_default(&c);
    c.gamma = gamma;
    c.boundary = boundary;
#ifdef OM_HYDRO_FP32
    c.precision = 32;
#else
    c.precision = 64;
#endif
    return c;
  }
};
