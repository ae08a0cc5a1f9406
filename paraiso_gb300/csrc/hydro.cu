// hydro.cu -- placeholder until the Hydro kernels land.
#include "om_internal.cuh"

namespace om {
om_status hydro_setup(Handle *h) {
  (void)h;
  set_error("Hydro: not built yet");
  return OM_ERR_UNSUPPORTED;
}
}  // namespace om

using namespace om;
extern "C" om_status om_hydro_init_kh(om_handle, uint64_t) { set_error("Hydro: not built yet"); return OM_ERR_UNSUPPORTED; }
extern "C" om_status om_hydro_totals(om_handle, double *) { set_error("Hydro: not built yet"); return OM_ERR_UNSUPPORTED; }
extern "C" om_status om_hydro_dt_history(om_handle, double *, int, int *) { set_error("Hydro: not built yet"); return OM_ERR_UNSUPPORTED; }
