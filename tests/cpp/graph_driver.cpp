// A driver in the style of examples/ShiftExample/main.cpp, built against a
// header emitted by paraiso_gb300.omgraph.emit_header (TableMaker.hpp on the
// include path).  Prints the table, margins included, after each kernel and
// the total.  Built and run by tests/test_shims.py.
#include <cstdio>

#include "TableMaker.hpp"

static void dump(TableMaker &m) {
  std::printf("value:");
  for (int x = -m.om_lower_margin_0(); x < m.om_size_0() + m.om_upper_margin_0(); ++x)
    std::printf(" %d", m.table(x));
  std::printf("\n");
}

int main() {
  TableMaker maker;
  maker.init();
  dump(maker);
  maker.increment();
  dump(maker);
  maker.calculate();
  dump(maker);
  std::printf("total: %d\n", maker.total());
  return 0;
}
