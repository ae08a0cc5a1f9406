// hydro.cu -- the examples/Hydro Orthotope Machine on GB300: handle setup,
// the `init` and `proceed` kernels, Kelvin-Helmholtz input, FP64 totals.
//
// Reference: examples/Hydro/HydroMain.hs:44-164 (statics, buildInit,
// buildProceed) and the generated class of
// examples-old/Hydro-exampled/dist-cuda/Hydro.{hpp,cu}.
//
// Paths (om_config.precision / .variant):
//   precision 32, variant 0  fused tiled step, FP32, multiply-add contraction
//   precision 32, variant 2  fused tiled step, FP32, exact operation order
//   precision 64, variant 0  fused tiled step, FP64, exact operation order
//   precision 32/64, variant 1  plain path: the generated structure (timescale
//                            pass, min-reduce with a host round trip,
//                            all-Delayed recompute step, manifest copies)
// Every path is cyclic (periodic); the CFL minimum of the state a fused step
// writes is reduced in its epilogue, so consecutive steps need no extra pass
// and no host round trip.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "hydro_launch.cuh"
#include "om_internal.cuh"

namespace om {

struct HydroState {
  int fp64 = 0;
  int variant = 0;
  int tile = kTile32x16;
  bool ts_valid = false;       // sc->tsmin[slot] holds the min of the current state
  int slot = 0;
  double ts_dR0 = 0, ts_dR1 = 0;  // dR the cached minimum was computed with
  double ts_ext1 = 0;             // extent1 it was computed with (open grids)
  int lm = 0;                     // margin width: 3 on an open grid, else 0
  unsigned long long *d_margin = nullptr;  // open grid: margin cells' CFL minimum
  double *d_dt = nullptr;      // dt history of the last run
  int dt_cap = 0;
  int last_n = 0;
  void *d_ts = nullptr;        // plain path: timescale manifest
  unsigned long long *d_min = nullptr, *h_min = nullptr;  // plain path reduce result
  double *d_partials = nullptr, *d_totals = nullptr, *h_totals = nullptr;
  int totals_blocks = 1024;
};

static HydroState *hst(Handle *h) { return (HydroState *)h->impl; }
static HydroScalars *hsc_host(Handle *h) { return (HydroScalars *)h->h_scalars; }
static HydroScalars *hsc_dev(Handle *h) { return (HydroScalars *)h->d_scalars; }

static int reduce_grid(Handle *h) { return 2 * sm_count(h->device); }

static om_status hydro_reserve(Handle *h, int kernel_id, int n) {
  (void)kernel_id;
  HydroState *st = hst(h);
  if (n <= st->dt_cap) return OM_OK;
  const int cap = std::max(n, 1024);
  double *p = nullptr;
  if (cudaMalloc(&p, sizeof(double) * cap) != cudaSuccess) {
    cudaGetLastError();
    set_error("Hydro: cannot allocate the dt history");
    return OM_ERR_NOMEM;
  }
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  if (st->d_dt) cudaFree(st->d_dt);
  st->d_dt = p;
  st->dt_cap = cap;
  return OM_OK;
}

static om_status hydro_init(Handle *h, int n) {
  (void)n;
  HydroState *st = hst(h);
  OM_CUDA_CHECK(hydro_init_jet(st->fp64, h->arrays[0].d(), h->arrays[1].d(), h->arrays[2].d(),
                               h->arrays[3].d(), h->size[0], h->size[1], st->lm, h->cfg.gamma,
                               hsc_dev(h), h->stream));
  h->launches++;
  st->ts_valid = false;
  st->last_n = 0;
  return OM_OK;
}

// the cached minimum (and on an open grid the margin minimum, a function of
// dR and extent1) still belongs to the current scalars
static bool ts_current(Handle *h) {
  const HydroState *st = hst(h);
  const HydroScalars *hs_ = hsc_host(h);
  return st->ts_valid && st->ts_dR0 == hs_->dR0 && st->ts_dR1 == hs_->dR1 &&
         (st->lm == 0 || st->ts_ext1 == hs_->extent1);
}

static void ts_mark_current(Handle *h) {
  HydroState *st = hst(h);
  const HydroScalars *hs_ = hsc_host(h);
  st->ts_valid = true;
  st->ts_dR0 = hs_->dR0;
  st->ts_dR1 = hs_->dR1;
  st->ts_ext1 = hs_->extent1;
}

// ensure sc->tsmin[slot] holds the CFL minimum of the current state
static om_status ensure_tsmin(Handle *h) {
  HydroState *st = hst(h);
  if (ts_current(h)) return OM_OK;
  OM_CUDA_CHECK(cudaMemsetAsync(&hsc_dev(h)->tsmin[st->slot], 0xFF, sizeof(unsigned long long),
                                h->stream));
  cudaEvent_t ev = prof_begin(h);
  if (st->lm > 0) {
    OM_CUDA_CHECK(hydro_tsmin_open(st->fp64, h->arrays[0].d(), h->arrays[1].d(),
                                   h->arrays[2].d(), h->arrays[3].d(), h->size[0], h->size[1],
                                   st->lm, h->cfg.gamma, hsc_dev(h), st->slot, st->d_margin,
                                   reduce_grid(h), h->stream));
    h->launches += 2;
  } else {
    OM_CUDA_CHECK(hydro_tsmin(st->fp64, h->arrays[0].d(), h->arrays[1].d(), h->arrays[2].d(),
                              h->arrays[3].d(), h->memory_size_total(), h->cfg.gamma,
                              hsc_dev(h), st->slot, reduce_grid(h), h->stream));
    h->launches++;
  }
  prof_end(h, ev, "hydro_tsmin_kernel", (double)h->memory_size_total());
  ts_mark_current(h);
  return OM_OK;
}

static om_status proceed_fused(Handle *h, int n) {
  HydroState *st = hst(h);
  OM_TRY(ensure_tsmin(h));
  const double cells = (double)h->size[0] * h->size[1];
  const bool persist = !st->fp64 && st->variant != 2 && st->lm == 0 &&
                       hydro_tile_is_persistent(st->tile) &&
                       hydro_persist_fits(h->size[0], h->size[1]);
  // the persistent kernel's form that runs (the profile name follows it)
  const int form = persist ? hydro_persist_form_for(hydro_persist_form(st->tile),
                                                    (long long)(h->size[0] / 32) * (h->size[1] / 32),
                                                    h->device, h->cfg.grid_limit)
                           : -1;
  const char *kname = st->fp64 ? "hydro_fused_kernel_f64"
                      : st->variant == 2 ? "hydro_fused_kernel_f32_exact"
                      : persist          ? (form == 2   ? "hydro_pair2_kernel"
                                            : form == 1 ? "hydro_pair_kernel"
                                                        : "hydro_persist_kernel")
                                         : "hydro_fused_kernel_f32";
  for (int k = 0; k < n; ++k) {
    OM_CUDA_CHECK(cudaMemsetAsync(&hsc_dev(h)->tsmin[1 - st->slot], 0xFF,
                                  sizeof(unsigned long long), h->stream));
    HydroStepArgs a;
    a.rho = h->arrays[0].d(); a.v0 = h->arrays[1].d();
    a.v1 = h->arrays[2].d(); a.p = h->arrays[3].d();
    a.nrho = h->arrays[0].d_next(); a.nv0 = h->arrays[1].d_next();
    a.nv1 = h->arrays[2].d_next(); a.np = h->arrays[3].d_next();
    a.n0 = h->size[0]; a.n1 = h->size[1];
    a.nt0 = 0;
    a.gamma = h->cfg.gamma;
    a.gamma_f = (float)h->cfg.gamma;
    a.sc = hsc_dev(h);
    a.read_slot = st->slot;
    a.dt_hist = st->d_dt + k;
    a.lm = st->lm;
    a.ms0 = (int)h->memory_size(0);
    a.margin_min = st->d_margin;
    a.grid_limit = h->cfg.grid_limit;
    cudaEvent_t ev = prof_begin(h);
    cudaError_t e = st->fp64 ? hydro_fused_f64(a, st->tile, h->stream, nullptr)
                             : hydro_fused_f32(a, st->tile, st->variant == 2, h->stream, nullptr);
    if (e != cudaSuccess) {
      set_error(std::string("Hydro fused step: ") + cudaGetErrorString(e));
      return OM_ERR_CUDA;
    }
    prof_end(h, ev, kname, cells);
    h->launches++;
    for (int i = 0; i < 4; ++i) h->arrays[i].swap();
    st->slot = 1 - st->slot;
  }
  st->last_n = n;
  return OM_OK;
}

// The generated structure: timescale manifest, reduce-min returned to the
// host (thrust::min_element), dt formed on the host in the OM's Real type,
// the all-Delayed step kernel into manifests, manifests copied to statics.
static om_status proceed_plain(Handle *h, int n) {
  HydroState *st = hst(h);
  const size_t cells = h->memory_size_total();
  const int grid = reduce_grid(h) * 4;
  const size_t bytes = cells * (st->fp64 ? 8 : 4);
  for (int k = 0; k < n; ++k) {
    const HydroScalars *hs_ = hsc_host(h);
    OM_CUDA_CHECK(hydro_plain_timescale(st->fp64, h->arrays[0].d(), h->arrays[1].d(),
                                        h->arrays[2].d(), h->arrays[3].d(), st->d_ts, cells,
                                        h->cfg.gamma, hsc_dev(h), grid, h->stream));
    h->launches++;
    OM_CUDA_CHECK(cudaMemsetAsync(st->d_min, 0xFF, sizeof(unsigned long long), h->stream));
    OM_CUDA_CHECK(hydro_plain_reduce_min(st->fp64, st->d_ts, cells, st->d_min, grid, h->stream));
    h->launches++;
    OM_CUDA_CHECK(cudaMemcpyAsync(st->h_min, st->d_min, sizeof(unsigned long long),
                                  cudaMemcpyDeviceToHost, h->stream));
    OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
    double dtG;
    if (st->fp64) {
      double tsmin;
      std::memcpy(&tsmin, st->h_min, sizeof(double));
      dtG = hs_->cfl * tsmin;
    } else {
      const uint32_t bits = (uint32_t)*st->h_min;
      float tsmin;
      std::memcpy(&tsmin, &bits, sizeof(float));
      dtG = (double)((float)hs_->cfl * tsmin);
    }
    cudaEvent_t ev = prof_begin(h);
    OM_CUDA_CHECK(hydro_plain_step(st->fp64, h->arrays[0].d(), h->arrays[1].d(),
                                   h->arrays[2].d(), h->arrays[3].d(), h->arrays[0].d_next(),
                                   h->arrays[1].d_next(), h->arrays[2].d_next(),
                                   h->arrays[3].d_next(), h->size[0], h->size[1], h->cfg.gamma,
                                   dtG, hs_->dR0, hs_->dR1, grid, h->stream));
    prof_end(h, ev, "hydro_plain_step_kernel", (double)cells);
    h->launches++;
    OM_CUDA_CHECK(hydro_scalar_advance(hsc_dev(h), dtG, st->d_dt + k, h->stream));
    h->launches++;
    for (int i = 0; i < 4; ++i)
      OM_CUDA_CHECK(cudaMemcpyAsync(h->arrays[i].d(), h->arrays[i].d_next(), bytes,
                                    cudaMemcpyDeviceToDevice, h->stream));
  }
  st->ts_valid = false;
  st->last_n = n;
  return OM_OK;
}

static om_status hydro_proceed(Handle *h, int n) {
  HydroState *st = hst(h);
  if (n > st->dt_cap) {
    set_error("Hydro: dt history not reserved");
    return OM_ERR_STATE;
  }
  return st->variant == 1 ? proceed_plain(h, n) : proceed_fused(h, n);
}

static uint64_t hydro_state_key(Handle *h) {
  HydroState *st = hst(h);
  return (ts_current(h) ? 1 : 0) | (uint64_t)st->slot << 1;
}

static void hydro_restore_key(Handle *h, uint64_t key) {
  HydroState *st = hst(h);
  st->ts_valid = (key & 1) != 0;
  st->slot = (int)((key >> 1) & 1);
  if (st->ts_valid) ts_mark_current(h);
}

struct HydroCkState;
static size_t hydro_save_state(Handle *h, void *out, size_t cap);
static void hydro_load_state(Handle *h, const void *in, size_t n);

static bool hydro_graph_ok(Handle *h, int kernel_id) {
  (void)kernel_id;
  return hst(h)->variant != 1;  // the plain path round-trips to the host
}

static void hydro_after_replay(Handle *h, int kernel_id, int n) {
  HydroState *st = hst(h);
  if (h->kernels[kernel_id].name == "proceed") {
    ts_mark_current(h);
    st->slot ^= (n & 1);
    st->last_n = n;
  } else {
    st->ts_valid = false;
    st->last_n = 0;
  }
}

static void hydro_array_written(Handle *h, Array *a) {
  (void)a;
  hst(h)->ts_valid = false;
}

void adjoint_release(Handle *h);

static void hydro_free(Handle *h) {
  HydroState *st = hst(h);
  if (!st) return;
  adjoint_release(h);
  cudaFree(st->d_dt);
  cudaFree(st->d_ts);
  cudaFree(st->d_min);
  cudaFree(st->d_margin);
  if (st->h_min) cudaFreeHost(st->h_min);
  cudaFree(st->d_partials);
  cudaFree(st->d_totals);
  if (st->h_totals) cudaFreeHost(st->h_totals);
  delete st;
  h->impl = nullptr;
}

// the device address of the CFL minimum of the current state (computed
// first if the cached one does not belong to it)
om_status hydro_tsmin_device(Handle *h, unsigned long long **ptr) {
  OM_TRY(upload_scalars(h));
  OM_TRY(ensure_tsmin(h));
  *ptr = &hsc_dev(h)->tsmin[hst(h)->slot];
  return OM_OK;
}

struct HydroCkState {
  bool ts_valid;
  int slot;
  double ts_dR0, ts_dR1, ts_ext1;
};
static_assert(sizeof(HydroCkState) <= 64, "checkpoint bookkeeping size");

// the cached-minimum bookkeeping travels with om_save / om_load, so a
// restart continues bit-identically (no re-reduction in another build)
static size_t hydro_save_state(Handle *h, void *out, size_t cap) {
  const HydroState *st = hst(h);
  const HydroCkState k{st->ts_valid, st->slot, st->ts_dR0, st->ts_dR1, st->ts_ext1};
  if (cap < sizeof k) return 0;
  std::memcpy(out, &k, sizeof k);
  return sizeof k;
}

static void hydro_load_state(Handle *h, const void *in, size_t n) {
  if (n != sizeof(HydroCkState)) return;  // keep the invalidated cache
  HydroCkState k;
  std::memcpy(&k, in, sizeof k);
  HydroState *st = hst(h);
  st->ts_valid = k.ts_valid;
  st->slot = k.slot;
  st->ts_dR0 = k.ts_dR0;
  st->ts_dR1 = k.ts_dR1;
  st->ts_ext1 = k.ts_ext1;
}

// the four arrays of a checkpoint share one allocation (f[0] is its base)
om_status hydro_checkpoint_alloc(Handle *h, HydroCheckpoint *c) {
  const size_t bytes = h->memory_size_total() * h->arrays[0].elem_size;
  const size_t pitch = (bytes + 255) / 256 * 256;
  char *base = nullptr;
  if (cudaMalloc(&base, pitch * 4) != cudaSuccess) {
    cudaGetLastError();
    set_error("Hydro checkpoint allocation failed");
    return OM_ERR_NOMEM;
  }
  for (int i = 0; i < 4; ++i) c->f[i] = base + pitch * i;
  return OM_OK;
}

void hydro_checkpoint_free(HydroCheckpoint *c) {
  if (c->f[0]) cudaFree(c->f[0]);
  for (int i = 0; i < 4; ++i) c->f[i] = nullptr;
}

om_status hydro_save(Handle *h, HydroCheckpoint *c) {
  const size_t bytes = h->memory_size_total() * h->arrays[0].elem_size;
  for (int i = 0; i < 4; ++i) {
    OM_TRY(bring_device(h, h->arrays[i]));
    OM_CUDA_CHECK(cudaMemcpyAsync(c->f[i], h->arrays[i].d(), bytes, cudaMemcpyDeviceToDevice,
                                  h->stream));
  }
  std::memcpy(c->sc, h->h_scalars, sizeof(HydroScalars));
  HydroState *st = hst(h);
  HydroCkState k{st->ts_valid, st->slot, st->ts_dR0, st->ts_dR1, st->ts_ext1};
  std::memcpy(c->state, &k, sizeof(k));
  return OM_OK;
}

om_status hydro_restore(Handle *h, const HydroCheckpoint *c) {
  const size_t bytes = h->memory_size_total() * h->arrays[0].elem_size;
  // the host scalar block is pinned: a copy from it that is still queued
  // reads it when it runs, so it is rewritten only once the stream is idle
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  for (int i = 0; i < 4; ++i) {
    OM_CUDA_CHECK(cudaMemcpyAsync(h->arrays[i].d(), c->f[i], bytes, cudaMemcpyDeviceToDevice,
                                  h->stream));
    h->arrays[i].newer = h->arrays[i].host ? Newer::kDevice : Newer::kBoth;
  }
  std::memcpy(h->h_scalars, c->sc, sizeof(HydroScalars));
  OM_TRY(upload_scalars(h));
  HydroState *st = hst(h);
  HydroCkState k;
  std::memcpy(&k, c->state, sizeof(k));
  st->ts_valid = k.ts_valid;
  st->slot = k.slot;
  st->ts_dR0 = k.ts_dR0;
  st->ts_dR1 = k.ts_dR1;
  st->ts_ext1 = k.ts_ext1;
  return OM_OK;
}

om_status hydro_setup(Handle *h) {
  if (!h->cyclic && h->cfg.variant == 1) {
    set_error("Hydro: the open boundary runs on the fused path (variant 0 or 2), not plain");
    return OM_ERR_UNSUPPORTED;
  }
  if (h->cfg.precision != 32 && h->cfg.precision != 64) {
    set_error("Hydro: precision must be 32 or 64");
    return OM_ERR_ARG;
  }
  if (h->cfg.variant < 0 || h->cfg.variant > 2 || (h->cfg.precision == 64 && h->cfg.variant == 2)) {
    set_error("Hydro: variant must be 0 (fused), 1 (plain) or 2 (fused exact FP32)");
    return OM_ERR_ARG;
  }
  if (!(h->cfg.gamma > 1.0)) {
    set_error("Hydro: gamma must be > 1");
    return OM_ERR_ARG;
  }
  // open grids keep 3-cell margins (the stencil radius of both stages,
  // Hydro.hpp:12-13 of the generated class); periodic grids none
  const int lm = h->cyclic ? 0 : 3;
  for (int ax = 0; ax < 2; ++ax) {
    h->lower_margin[ax] = lm;
    h->upper_margin[ax] = lm;
  }
  HydroState *st = new HydroState();
  st->fp64 = h->cfg.precision == 64;
  st->variant = h->cfg.variant;
  st->lm = lm;
  st->tile = hydro_tile_of(h->cfg.tile_x, h->cfg.tile_y, !st->fp64 && st->variant == 0);
  h->impl = st;
  h->impl_free = hydro_free;
  h->ops.state_key = hydro_state_key;
  h->ops.after_replay = hydro_after_replay;
  h->ops.restore_key = hydro_restore_key;
  h->ops.array_written = hydro_array_written;
  h->ops.reserve = hydro_reserve;
  h->ops.graph_ok = hydro_graph_ok;
  h->ops.save_state = hydro_save_state;
  h->ops.load_state = hydro_load_state;
  h->ops.before_upload = [](Handle *hh) { hydro_scalars_refresh(hsc_host(hh)); };
  h->ops.after_run = [](Handle *hh) -> om_status {
    HydroScalars *sc = hsc_host(hh);
    if (!sc->wait_error) return OM_OK;
    sc->wait_error = 0;  // cleared on the device by the next upload
    set_error("Hydro: a kernel's bounded wait for its tensor copies ran out; the state of this "
              "run is unspecified");
    return OM_ERR_CUDA;
  };
  const int es = st->fp64 ? 8 : 4;
  OM_TRY(alloc_array(h, "density", es));
  OM_TRY(alloc_array(h, "velocity0", es));
  OM_TRY(alloc_array(h, "velocity1", es));
  OM_TRY(alloc_array(h, "pressure", es));
  h->scalars.push_back({"generation", kInt, offsetof(HydroScalars, generation)});
  h->scalars.push_back({"time", kDouble, offsetof(HydroScalars, time)});
  h->scalars.push_back({"cfl", kDouble, offsetof(HydroScalars, cfl)});
  h->scalars.push_back({"dR0", kDouble, offsetof(HydroScalars, dR0)});
  h->scalars.push_back({"dR1", kDouble, offsetof(HydroScalars, dR1)});
  h->scalars.push_back({"extent0", kDouble, offsetof(HydroScalars, extent0)});
  h->scalars.push_back({"extent1", kDouble, offsetof(HydroScalars, extent1)});
  h->scalar_bytes = sizeof(HydroScalars);
  h->kernels.push_back({"init", hydro_init});
  h->kernels.push_back({"proceed", hydro_proceed});
  const size_t cells = h->memory_size_total();
  if (cudaMalloc(&st->d_ts, cells * es) != cudaSuccess ||
      cudaMalloc(&st->d_min, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&st->d_margin, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&st->h_min, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&st->d_partials, sizeof(double) * 8 * st->totals_blocks) != cudaSuccess ||
      cudaMalloc(&st->d_totals, sizeof(double) * 4) != cudaSuccess ||
      cudaMallocHost(&st->h_totals, sizeof(double) * 4) != cudaSuccess) {
    cudaGetLastError();
    set_error("Hydro: scratch allocation failed");
    return OM_ERR_NOMEM;
  }
  return OM_OK;
}

}  // namespace om

using namespace om;

static om_status hydro_handle(om_handle H, Handle **out) {
  Handle *h = handle_of(H);
  if (!h) { set_error("null handle"); return OM_ERR_ARG; }
  if (h->kind != OM_KIND_HYDRO) { set_error("not a Hydro handle"); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  *out = h;
  return OM_OK;
}

extern "C" om_status om_hydro_init_kh(om_handle H, uint64_t seed) {
  Handle *h;
  OM_TRY(hydro_handle(H, &h));
  HydroState *st = hst(h);
  if (st->lm > 0) {
    set_error("om_hydro_init_kh: the Kelvin-Helmholtz start is periodic (open grids use init)");
    return OM_ERR_UNSUPPORTED;
  }
  OM_CUDA_CHECK(hydro_init_kh(st->fp64, h->arrays[0].d(), h->arrays[1].d(), h->arrays[2].d(),
                              h->arrays[3].d(), h->size[0], h->size[1], mix64(seed), h->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  for (int i = 0; i < 4; ++i) {
    Array &a = h->arrays[i];
    a.newer = a.host ? Newer::kDevice : Newer::kBoth;
  }
  HydroScalars *s = hsc_host(h);
  s->time = 0;
  s->extent0 = 1.0;
  s->extent1 = 1.0;
  s->dR0 = 1.0 / h->size[0];
  s->dR1 = 1.0 / h->size[1];
  if (s->cfl == 0) s->cfl = 0.4;
  st->ts_valid = false;
  return OM_OK;
}

extern "C" om_status om_hydro_totals(om_handle H, double *out) {
  if (!out) { set_error("om_hydro_totals: out is NULL"); return OM_ERR_ARG; }
  Handle *h;
  OM_TRY(hydro_handle(H, &h));
  HydroState *st = hst(h);
  for (int i = 0; i < 4; ++i) OM_TRY(bring_device(h, h->arrays[i]));
  OM_CUDA_CHECK(hydro_totals(st->fp64, h->arrays[0].d(), h->arrays[1].d(), h->arrays[2].d(),
                             h->arrays[3].d(), h->size[0], h->size[1], st->lm, h->cfg.gamma,
                             st->d_partials, st->totals_blocks, st->d_totals, h->stream));
  OM_CUDA_CHECK(cudaMemcpyAsync(st->h_totals, st->d_totals, sizeof(double) * 4,
                                cudaMemcpyDeviceToHost, h->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  bool finite = true;
  for (int k = 0; k < 4; ++k) {
    out[k] = st->h_totals[k];
    finite = finite && std::isfinite(out[k]);
  }
  if (!finite) {
    set_error("Hydro: non-finite conserved total (NaN or Inf in the state)");
    return OM_ERR_NONFINITE;
  }
  return OM_OK;
}

extern "C" om_status om_hydro_dt_history(om_handle H, double *out, int n, int *written) {
  Handle *h;
  OM_TRY(hydro_handle(H, &h));
  if (!out && n > 0) { set_error("om_hydro_dt_history: out is NULL"); return OM_ERR_ARG; }
  HydroState *st = hst(h);
  const int m = std::min(n, st->last_n);
  if (m > 0) {
    OM_CUDA_CHECK(cudaMemcpyAsync(out, st->d_dt, sizeof(double) * m, cudaMemcpyDeviceToHost,
                                  h->stream));
    OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  }
  if (written) *written = std::max(m, 0);
  return OM_OK;
}
