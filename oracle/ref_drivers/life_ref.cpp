// life_ref.cpp -- C entry points around the reference's pre-generated Life
// class (examples-old/Life-exampled/dist/Life.{hpp,cpp}: 128x128, open
// boundary, old accessor API; or a copy resized by oracle/resize_ref.py).
// Compiled together with that Life.cpp by oracle/Makefile into
// oracle/_ref/libref_life.so.  Test infrastructure only.
#include <cstdint>
#include <cstring>
#include "Life.hpp"

extern "C" int ref_life_size0(void) { Life s; return s.size0(); }
extern "C" int ref_life_size1(void) { Life s; return s.size1(); }
extern "C" int ref_life_memory_size(void) { Life s; return s.memorySize(); }

// init(); optionally replace the whole memory array of `cell`; then
// `steps` x proceed().  Writes the final memory array and the population
// after every generation.
extern "C" void ref_life_run(const int32_t *initial, int steps,
                             int32_t *out_cells, int32_t *out_pops) {
  Life *s = new Life();
  s->init();
  const int n = s->memorySize();
  if (initial)
    for (int i = 0; i < n; ++i) s->static_2_cell[i] = initial[i];
  for (int t = 0; t < steps; ++t) {
    s->proceed();
    if (out_pops) out_pops[t] = s->static_0_population;
  }
  for (int i = 0; i < n; ++i) out_cells[i] = s->static_2_cell[i];
  delete s;
}
