// hydro_ref.cpp -- C entry points around the reference's pre-generated Hydro
// class (examples-old/Hydro-exampled/dist/Hydro.{hpp,cpp}: 1024x1024, float,
// open boundary, gamma 5/3; or a copy resized by oracle/resize_ref.py).  Compiled together with that Hydro.cpp by
// oracle/Makefile into oracle/_ref/libref_hydro.so.  Test infrastructure only.
#include <cstdint>
#include "Hydro.hpp"

extern "C" int ref_hydro_size0(void) { Hydro s; return s.size0(); }
extern "C" int ref_hydro_memory_size(void) { Hydro s; return s.memorySize(); }

// Scalars as in examples-old/Hydro-exampled/main-kh.cpp: time 0, extent 1,
// dR = extent / size.  init(); optionally replace the four memory arrays
// (rho, vx, vy, p, each memory-sized); then `steps` x proceed().
extern "C" void ref_hydro_run(const float *initial, int steps, float cfl,
                              float *out, float *out_time) {
  Hydro *s = new Hydro();
  s->static_1_time = 0;
  s->static_2_cfl = cfl;
  s->static_5_extent0 = 1.0;
  s->static_6_extent1 = 1.0;
  s->static_3_dR0 = s->static_5_extent0 / s->size0();
  s->static_4_dR1 = s->static_6_extent1 / s->size1();
  s->init();
  const int n = s->memorySize();
  if (initial)
    for (int i = 0; i < n; ++i) {
      s->static_7_density[i] = initial[i];
      s->static_8_velocity0[i] = initial[n + i];
      s->static_9_velocity1[i] = initial[2 * n + i];
      s->static_10_pressure[i] = initial[3 * n + i];
    }
  for (int t = 0; t < steps; ++t) {
    s->proceed();
    if (out_time) out_time[t] = s->static_1_time;
  }
  for (int i = 0; i < n; ++i) {
    out[i] = s->static_7_density[i];
    out[n + i] = s->static_8_velocity0[i];
    out[2 * n + i] = s->static_9_velocity1[i];
    out[3 * n + i] = s->static_10_pressure[i];
  }
  delete s;
}
