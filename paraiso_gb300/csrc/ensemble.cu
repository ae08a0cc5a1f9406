// ensemble.cu -- batched Hydro: many independent periodic Kelvin-Helmholtz
// (or user-supplied) grids of uneven sizes advanced together, one
// persistent launch per step over every (instance, tile) work item, each
// instance with its own CFL dt and time; multi-step runs replay a captured
// CUDA graph.  No counterpart in the reference (it advances one compile-time
// sized grid per generated object, examples/Hydro/main-kh.cpp:49-59).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "hydro_launch.cuh"
#include "om_internal.cuh"

namespace om {

__global__ void ensemble_reset_slots_kernel(HydroScalars *sc, int count, int slot) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) sc[k].tsmin[slot] = ~0ull;
}

}  // namespace om

using namespace om;

struct om_ensemble_s {
  int count = 0;
  int fp64 = 0;
  bool exact = false;
  int tile = kTile32x32;
  int tx = 32, ty = 16;
  double gamma = 1.4;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<int> n0, n1;
  std::vector<size_t> offset;
  size_t total_cells = 0;
  size_t es = 4;
  void *field[4][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
  int cur = 0;  // current buffer parity == CFL slot holding its minimum
  HydroScalars *d_sc = nullptr, *h_sc = nullptr;
  HydroStepArgs *d_args[2] = {nullptr, nullptr};
  std::vector<int> prefix;
  int *d_prefix = nullptr;
  // persistent kernel: 4 tensor maps per instance and buffer parity,
  // [parity][instance][field]
  CUtensorMap *d_maps = nullptr;
  bool ts_valid = false;
  int grid = 0;
  double *d_partials = nullptr, *d_totals = nullptr, *h_totals = nullptr;
  int totals_blocks = 1024;
  std::map<std::tuple<int, int>, cudaGraphExec_t> graphs;  // (n, cur) -> graph
  int last_launches = 0;
  bool profiling = false;
  float last_kernel_ms = 0;
};

static const char *kFields[4] = {"density", "velocity0", "velocity1", "pressure"};

static int field_index(const char *name) {
  for (int i = 0; i < 4; ++i)
    if (!std::strcmp(name, kFields[i])) return i;
  return -1;
}

static om_status ens_upload_args(om_ensemble E) {
  for (int p = 0; p < 2; ++p) {
    std::vector<HydroStepArgs> a(E->count);
    for (int k = 0; k < E->count; ++k) {
      HydroStepArgs &x = a[k];
      const size_t off = E->offset[k] * E->es;
      x.rho = (char *)E->field[0][p] + off;
      x.v0 = (char *)E->field[1][p] + off;
      x.v1 = (char *)E->field[2][p] + off;
      x.p = (char *)E->field[3][p] + off;
      x.nrho = (char *)E->field[0][1 - p] + off;
      x.nv0 = (char *)E->field[1][1 - p] + off;
      x.nv1 = (char *)E->field[2][1 - p] + off;
      x.np = (char *)E->field[3][1 - p] + off;
      x.n0 = E->n0[k];
      x.n1 = E->n1[k];
      x.nt0 = (E->n0[k] + E->tx - 1) / E->tx;
      x.gamma = E->gamma;
      x.gamma_f = (float)E->gamma;
      x.sc = E->d_sc + k;
      x.read_slot = p;
      x.dt_hist = &E->d_sc[k].dt_last;
      x.lm = 0;
      x.ms0 = E->n0[k];
      x.margin_min = nullptr;
    }
    OM_CUDA_CHECK(cudaMemcpyAsync(E->d_args[p], a.data(), sizeof(HydroStepArgs) * E->count,
                                  cudaMemcpyHostToDevice, E->stream));
  }
  OM_CUDA_CHECK(cudaStreamSynchronize(E->stream));
  return OM_OK;
}

// Issue n ensemble steps on the stream (graph-capturable: no host sync).
static om_status ens_issue(om_ensemble E, int n) {
  for (int s = 0; s < n; ++s) {
    ensemble_reset_slots_kernel<<<(E->count + 127) / 128, 128, 0, E->stream>>>(E->d_sc, E->count,
                                                                            1 - E->cur);
    OM_CUDA_CHECK(cudaGetLastError());
    cudaError_t e = E->fp64 ? hydro_ensemble_f64(E->d_args[E->cur], E->d_prefix, E->count,
                                                 E->tile, E->grid, E->stream)
                            : hydro_ensemble_f32(E->d_args[E->cur], E->d_prefix, E->count,
                                                 E->tile, E->exact, E->grid, E->stream,
                                                 E->d_maps ? E->d_maps + (size_t)E->cur * E->count * 4
                                                           : nullptr);
    if (e != cudaSuccess) {
      set_error(std::string("ensemble step: ") + cudaGetErrorString(e));
      return OM_ERR_CUDA;
    }
    E->cur = 1 - E->cur;
  }
  E->last_launches = 2 * n;
  return OM_OK;
}

extern "C" {

om_status om_ensemble_create(int count, const int *sizes, const om_config *cfg,
                             om_ensemble *out) {
  if (!out || !sizes || count < 1 || count > (1 << 20)) {
    set_error("om_ensemble_create: need count >= 1, sizes[count][2] and out");
    return OM_ERR_ARG;
  }
  *out = nullptr;
  om_config c;
  if (cfg) c = *cfg; else om_config_default(&c);
  if (c.boundary != OM_BOUNDARY_CYCLIC) {
    set_error("om_ensemble_create: ensembles are periodic (cyclic boundary)");
    return OM_ERR_UNSUPPORTED;
  }
  if ((c.precision != 32 && c.precision != 64) || !(c.gamma > 1.0) ||
      (c.variant != 0 && c.variant != 2) || (c.precision == 64 && c.variant == 2)) {
    set_error("om_ensemble_create: precision 32/64, gamma > 1, variant 0 (fused) or 2 (exact FP32)");
    return OM_ERR_ARG;
  }
  for (int k = 0; k < count; ++k)
    if (sizes[2 * k] < 1 || sizes[2 * k + 1] < 1 || sizes[2 * k] > (1 << 16) ||
        sizes[2 * k + 1] > (1 << 16)) {
      set_error("om_ensemble_create: instance sizes must be in [1, 65536]");
      return OM_ERR_ARG;
    }
  OM_CUDA_CHECK(cudaSetDevice(c.device));
  om_ensemble E = new om_ensemble_s();
  E->count = count;
  E->fp64 = c.precision == 64;
  E->exact = c.variant == 2 || E->fp64;
  E->tile = hydro_tile_of(c.tile_x, c.tile_y, !E->exact && !E->fp64);
  if (hydro_tile_is_sweep(E->tile)) E->tile = kTile32x32;  // items are tiles
  if (hydro_tile_is_persistent(E->tile))
    for (int k = 0; k < count; ++k)
      if (!hydro_persist_fits(sizes[2 * k], sizes[2 * k + 1])) E->tile = kTile32x32;
  if (E->tile == kPairGroups32x32) {
    long long items = 0;
    for (int k = 0; k < count; ++k) items += (long long)(sizes[2 * k] / 32) * (sizes[2 * k + 1] / 32);
    if (hydro_persist_form_for(2, items, c.device, c.grid_limit) != 2) E->tile = kPair32x32;
  }
  hydro_tile_dims(E->tile, &E->tx, &E->ty);
  E->gamma = c.gamma;
  E->device = c.device;
  E->es = E->fp64 ? 8 : 4;
  om_status st = OM_OK;
  if (cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete E;
    set_error("om_ensemble_create: stream creation failed");
    return OM_ERR_CUDA;
  }
  E->prefix.assign(count + 1, 0);
  for (int k = 0; k < count; ++k) {
    E->n0.push_back(sizes[2 * k]);
    E->n1.push_back(sizes[2 * k + 1]);
    E->offset.push_back(E->total_cells);
    // align every instance to 64 cells (256 B) for coalesced tile loads
    E->total_cells += ((size_t)sizes[2 * k] * sizes[2 * k + 1] + 63) / 64 * 64;
    const long long tiles = (long long)((sizes[2 * k] + E->tx - 1) / E->tx) *
                            ((sizes[2 * k + 1] + E->ty - 1) / E->ty);
    if (E->prefix[k] + tiles > 0x7fffffffLL) {
      set_error("om_ensemble_create: too many tiles");
      om_ensemble_destroy(E);
      return OM_ERR_ARG;
    }
    E->prefix[k + 1] = E->prefix[k] + (int)tiles;
  }
  auto alloc = [&](void **p, size_t bytes) {
    if (st == OM_OK && cudaMalloc(p, bytes) != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
      set_error("om_ensemble_create: device allocation failed");
      st = OM_ERR_NOMEM;
    }
  };
  for (int f = 0; f < 4; ++f)
    for (int b = 0; b < 2; ++b) alloc(&E->field[f][b], E->total_cells * E->es);
  alloc((void **)&E->d_sc, sizeof(HydroScalars) * count);
  alloc((void **)&E->d_args[0], sizeof(HydroStepArgs) * count);
  alloc((void **)&E->d_args[1], sizeof(HydroStepArgs) * count);
  alloc((void **)&E->d_prefix, sizeof(int) * (count + 1));
  alloc((void **)&E->d_partials, sizeof(double) * 8 * E->totals_blocks);
  alloc((void **)&E->d_totals, sizeof(double) * 4);
  if (st == OM_OK && (cudaMallocHost(&E->h_sc, sizeof(HydroScalars) * count) != cudaSuccess ||
                      cudaMallocHost(&E->h_totals, sizeof(double) * 4) != cudaSuccess)) {
    cudaGetLastError();
    set_error("om_ensemble_create: pinned allocation failed");
    st = OM_ERR_NOMEM;
  }
  if (st != OM_OK) {
    std::string keep = om_last_error();
    om_ensemble_destroy(E);
    set_error(keep);
    return st;
  }
  std::memset(E->h_sc, 0, sizeof(HydroScalars) * count);
  for (int k = 0; k < count; ++k) {
    E->h_sc[k].cfl = 0.4;
    E->h_sc[k].extent0 = E->h_sc[k].extent1 = 1.0;
    E->h_sc[k].dR0 = 1.0 / E->n0[k];
    E->h_sc[k].dR1 = 1.0 / E->n1[k];
  }
  for (int f = 0; f < 4; ++f)
    for (int b = 0; b < 2; ++b)
      if (cudaMemsetAsync(E->field[f][b], 0, E->total_cells * E->es, E->stream) != cudaSuccess) {
        cudaGetLastError();
      }
  if (cudaMemcpyAsync(E->d_prefix, E->prefix.data(), sizeof(int) * (count + 1),
                      cudaMemcpyHostToDevice, E->stream) != cudaSuccess) {
    om_ensemble_destroy(E);
    set_error("om_ensemble_create: upload failed");
    return OM_ERR_CUDA;
  }
  if (hydro_tile_is_persistent(E->tile)) {
    std::vector<CUtensorMap> maps((size_t)2 * count * 4);
    for (int p = 0; p < 2 && st == OM_OK; ++p)
      for (int k = 0; k < count && st == OM_OK; ++k) {
        HydroStepArgs x{};
        const size_t off = E->offset[k] * E->es;
        x.rho = (char *)E->field[0][p] + off;
        x.v0 = (char *)E->field[1][p] + off;
        x.v1 = (char *)E->field[2][p] + off;
        x.p = (char *)E->field[3][p] + off;
        x.n0 = E->n0[k];
        x.n1 = E->n1[k];
        if (!hydro_persist_encode(&maps[((size_t)p * count + k) * 4], x)) {
          set_error("om_ensemble_create: tensor map encoding failed");
          st = OM_ERR_CUDA;
        }
      }
    alloc((void **)&E->d_maps, sizeof(CUtensorMap) * maps.size());
    if (st == OM_OK && cudaMemcpy(E->d_maps, maps.data(), sizeof(CUtensorMap) * maps.size(),
                                  cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      set_error("om_ensemble_create: tensor map upload failed");
      st = OM_ERR_CUDA;
    }
    if (st != OM_OK) {
      std::string keep = om_last_error();
      om_ensemble_destroy(E);
      set_error(keep);
      return st;
    }
  }
  const int occ = hydro_ensemble_occupancy(E->fp64, E->tile, E->exact);
  E->grid = std::max(1, std::min(occ * sm_count(E->device), E->prefix[count]));
  if (c.grid_limit > 0) E->grid = std::min(E->grid, c.grid_limit);
  st = ens_upload_args(E);
  if (st != OM_OK) {
    om_ensemble_destroy(E);
    return st;
  }
  *out = E;
  return OM_OK;
}

om_status om_ensemble_destroy(om_ensemble E) {
  if (!E) return OM_OK;
  cudaSetDevice(E->device);
  if (E->stream) cudaStreamSynchronize(E->stream);
  for (auto &kv : E->graphs) cudaGraphExecDestroy(kv.second);
  for (int f = 0; f < 4; ++f)
    for (int b = 0; b < 2; ++b) cudaFree(E->field[f][b]);
  cudaFree(E->d_sc);
  cudaFree(E->d_args[0]);
  cudaFree(E->d_args[1]);
  cudaFree(E->d_prefix);
  cudaFree(E->d_maps);
  cudaFree(E->d_partials);
  cudaFree(E->d_totals);
  if (E->h_sc) cudaFreeHost(E->h_sc);
  if (E->h_totals) cudaFreeHost(E->h_totals);
  if (E->stream) cudaStreamDestroy(E->stream);
  cudaGetLastError();
  delete E;
  return OM_OK;
}

om_status om_ensemble_info(om_ensemble E, int *count, long long *total_cells, int *grid,
                           int *work_items) {
  if (!E) { set_error("null ensemble"); return OM_ERR_ARG; }
  if (count) *count = E->count;
  if (total_cells) {
    long long t = 0;
    for (int k = 0; k < E->count; ++k) t += (long long)E->n0[k] * E->n1[k];
    *total_cells = t;
  }
  if (grid) *grid = E->grid;
  if (work_items) *work_items = E->prefix[E->count];
  return OM_OK;
}

om_status om_ensemble_init_kh(om_ensemble E, uint64_t base_seed) {
  if (!E) { set_error("null ensemble"); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(E->device));
  for (int k = 0; k < E->count; ++k) {
    const size_t off = E->offset[k] * E->es;
    OM_CUDA_CHECK(hydro_init_kh(E->fp64, (char *)E->field[0][E->cur] + off,
                                (char *)E->field[1][E->cur] + off,
                                (char *)E->field[2][E->cur] + off,
                                (char *)E->field[3][E->cur] + off, E->n0[k], E->n1[k],
                                mix64(base_seed + (uint64_t)k), E->stream));
    E->h_sc[k].time = 0;
    E->h_sc[k].cfl = 0.4;
    E->h_sc[k].extent0 = E->h_sc[k].extent1 = 1.0;
    E->h_sc[k].dR0 = 1.0 / E->n0[k];
    E->h_sc[k].dR1 = 1.0 / E->n1[k];
  }
  OM_CUDA_CHECK(cudaStreamSynchronize(E->stream));
  E->ts_valid = false;
  return OM_OK;
}

static om_status ens_tsmin_all(om_ensemble E) {
  if (E->ts_valid) return OM_OK;
  ensemble_reset_slots_kernel<<<(E->count + 127) / 128, 128, 0, E->stream>>>(E->d_sc, E->count,
                                                                          E->cur);
  OM_CUDA_CHECK(cudaGetLastError());
  const int grid = 2 * sm_count(E->device);
  for (int k = 0; k < E->count; ++k) {
    const size_t off = E->offset[k] * E->es;
    OM_CUDA_CHECK(hydro_tsmin(E->fp64, (char *)E->field[0][E->cur] + off,
                              (char *)E->field[1][E->cur] + off,
                              (char *)E->field[2][E->cur] + off,
                              (char *)E->field[3][E->cur] + off, (size_t)E->n0[k] * E->n1[k],
                              E->gamma, E->d_sc + k, E->cur, grid, E->stream));
  }
  E->ts_valid = true;
  return OM_OK;
}

// after a run's scalar blocks came back: a kernel whose bounded wait for
// its tensor copies ran out has raised wait_error (cleared here; the next
// upload clears it on the device)
static om_status ens_check_waits(om_ensemble E) {
  bool raised = false;
  for (int k = 0; k < E->count; ++k)
    if (E->h_sc[k].wait_error) {
      raised = true;
      E->h_sc[k].wait_error = 0;
    }
  if (!raised) return OM_OK;
  set_error("ensemble step: a kernel's bounded wait for its tensor copies ran out; the states "
            "of this run are unspecified");
  return OM_ERR_CUDA;
}

// the CUDA graph of n steps from buffer parity E->cur (captured on first use)
static om_status ens_graph(om_ensemble E, int n, cudaGraphExec_t *out) {
  auto key = std::make_tuple(n, E->cur);
  auto it = E->graphs.find(key);
  if (it == E->graphs.end()) {
    const int cur0 = E->cur;
    cudaGraph_t g = nullptr;
    OM_CUDA_CHECK(cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeThreadLocal));
    om_status s = ens_issue(E, n);
    cudaError_t ce = cudaStreamEndCapture(E->stream, &g);
    E->cur = cur0;
    if (s != OM_OK) { if (g) cudaGraphDestroy(g); return s; }
    if (ce != cudaSuccess) {
      set_error(std::string("ensemble graph capture: ") + cudaGetErrorString(ce));
      return OM_ERR_CUDA;
    }
    cudaGraphExec_t ex = nullptr;
    ce = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      set_error(std::string("ensemble graph instantiate: ") + cudaGetErrorString(ce));
      return OM_ERR_CUDA;
    }
    it = E->graphs.emplace(key, ex).first;
  }
  *out = it->second;
  return OM_OK;
}

// replay the graph of n steps (n > 1)
static om_status ens_replay(om_ensemble E, int n) {
  cudaGraphExec_t ex = nullptr;
  OM_TRY(ens_graph(E, n, &ex));
  OM_CUDA_CHECK(cudaGraphLaunch(ex, E->stream));
  if (n & 1) E->cur = 1 - E->cur;
  E->last_launches = 2 * n;
  return OM_OK;
}

static om_status ens_run(om_ensemble E, int n, bool use_graph) {
  OM_CUDA_CHECK(cudaSetDevice(E->device));
  for (int k = 0; k < E->count; ++k) hydro_scalars_refresh(&E->h_sc[k]);
  OM_CUDA_CHECK(cudaMemcpyAsync(E->d_sc, E->h_sc, sizeof(HydroScalars) * E->count,
                                cudaMemcpyHostToDevice, E->stream));
  OM_TRY(ens_tsmin_all(E));
  if (use_graph && n > 1) {
    OM_TRY(ens_replay(E, n));
  } else {
    OM_TRY(ens_issue(E, n));
  }
  OM_CUDA_CHECK(cudaMemcpyAsync(E->h_sc, E->d_sc, sizeof(HydroScalars) * E->count,
                                cudaMemcpyDeviceToHost, E->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(E->stream));
  return ens_check_waits(E);
}

om_status om_ensemble_step(om_ensemble E, int n) {
  if (!E || n < 0) { set_error("om_ensemble_step: bad arguments"); return OM_ERR_ARG; }
  if (n == 0) return OM_OK;
  return ens_run(E, n, true);
}

om_status om_ensemble_time_step(om_ensemble E, int n, float *ms) {
  if (!E || n < 1 || !ms) { set_error("om_ensemble_time_step: bad arguments"); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(E->device));
  // capture (or find) the graph first so the timed region is the replay
  for (int k = 0; k < E->count; ++k) hydro_scalars_refresh(&E->h_sc[k]);
  OM_CUDA_CHECK(cudaMemcpyAsync(E->d_sc, E->h_sc, sizeof(HydroScalars) * E->count,
                                cudaMemcpyHostToDevice, E->stream));
  OM_TRY(ens_tsmin_all(E));
  cudaGraphExec_t ex = nullptr;
  if (n > 1) OM_TRY(ens_graph(E, n, &ex));
  cudaEvent_t e0, e1;
  OM_CUDA_CHECK(cudaEventCreate(&e0));
  OM_CUDA_CHECK(cudaEventCreate(&e1));
  OM_CUDA_CHECK(cudaStreamSynchronize(E->stream));
  OM_CUDA_CHECK(cudaEventRecord(e0, E->stream));
  if (ex) {
    OM_CUDA_CHECK(cudaGraphLaunch(ex, E->stream));
    if (n & 1) E->cur = 1 - E->cur;
    E->last_launches = 2 * n;
  } else {
    OM_TRY(ens_issue(E, n));
  }
  OM_CUDA_CHECK(cudaEventRecord(e1, E->stream));
  OM_CUDA_CHECK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  OM_CUDA_CHECK(cudaMemcpyAsync(E->h_sc, E->d_sc, sizeof(HydroScalars) * E->count,
                                cudaMemcpyDeviceToHost, E->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(E->stream));
  return ens_check_waits(E);
}

om_status om_ensemble_read(om_ensemble E, int k, const char *name, void *dst, size_t bytes) {
  if (!E || !name || !dst || k < 0 || k >= E->count) {
    set_error("om_ensemble_read: bad arguments");
    return OM_ERR_ARG;
  }
  const int f = field_index(name);
  if (f < 0) { set_error(std::string("no field named ") + name); return OM_ERR_ARG; }
  if (bytes != (size_t)E->n0[k] * E->n1[k] * E->es) {
    set_error("om_ensemble_read: byte count must be n0*n1*element size");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(E->device));
  OM_CUDA_CHECK(cudaMemcpyAsync(dst, (char *)E->field[f][E->cur] + E->offset[k] * E->es, bytes,
                                cudaMemcpyDefault, E->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(E->stream));
  return OM_OK;
}

om_status om_ensemble_write(om_ensemble E, int k, const char *name, const void *src,
                            size_t bytes) {
  if (!E || !name || !src || k < 0 || k >= E->count) {
    set_error("om_ensemble_write: bad arguments");
    return OM_ERR_ARG;
  }
  const int f = field_index(name);
  if (f < 0) { set_error(std::string("no field named ") + name); return OM_ERR_ARG; }
  if (bytes != (size_t)E->n0[k] * E->n1[k] * E->es) {
    set_error("om_ensemble_write: byte count must be n0*n1*element size");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(E->device));
  OM_CUDA_CHECK(cudaMemcpyAsync((char *)E->field[f][E->cur] + E->offset[k] * E->es, src, bytes,
                                cudaMemcpyDefault, E->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(E->stream));
  E->ts_valid = false;
  return OM_OK;
}

om_status om_ensemble_scalar(om_ensemble E, int k, const char *name, double *value) {
  if (!E || !name || !value || k < 0 || k >= E->count) {
    set_error("om_ensemble_scalar: bad arguments");
    return OM_ERR_ARG;
  }
  const HydroScalars &s = E->h_sc[k];
  if (!std::strcmp(name, "time")) *value = s.time;
  else if (!std::strcmp(name, "cfl")) *value = s.cfl;
  else if (!std::strcmp(name, "dR0")) *value = s.dR0;
  else if (!std::strcmp(name, "dR1")) *value = s.dR1;
  else if (!std::strcmp(name, "dt")) *value = s.dt_last;
  else { set_error(std::string("no ensemble scalar named ") + name); return OM_ERR_ARG; }
  return OM_OK;
}

om_status om_ensemble_set_scalar(om_ensemble E, int k, const char *name, double value) {
  if (!E || !name || k < 0 || k >= E->count) {
    set_error("om_ensemble_set_scalar: bad arguments");
    return OM_ERR_ARG;
  }
  HydroScalars &s = E->h_sc[k];
  if (!std::strcmp(name, "time")) s.time = value;
  else if (!std::strcmp(name, "cfl")) s.cfl = value;
  else if (!std::strcmp(name, "dR0")) { s.dR0 = value; E->ts_valid = false; }
  else if (!std::strcmp(name, "dR1")) { s.dR1 = value; E->ts_valid = false; }
  else { set_error(std::string("no settable ensemble scalar named ") + name); return OM_ERR_ARG; }
  return OM_OK;
}

om_status om_ensemble_totals(om_ensemble E, int k, double *out) {
  if (!E || !out || k < 0 || k >= E->count) {
    set_error("om_ensemble_totals: bad arguments");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(E->device));
  const size_t off = E->offset[k] * E->es;
  OM_CUDA_CHECK(hydro_totals(E->fp64, (char *)E->field[0][E->cur] + off,
                             (char *)E->field[1][E->cur] + off, (char *)E->field[2][E->cur] + off,
                             (char *)E->field[3][E->cur] + off, E->n0[k], E->n1[k], 0,
                             E->gamma, E->d_partials, E->totals_blocks, E->d_totals, E->stream));
  OM_CUDA_CHECK(cudaMemcpyAsync(E->h_totals, E->d_totals, sizeof(double) * 4,
                                cudaMemcpyDeviceToHost, E->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(E->stream));
  bool finite = true;
  for (int i = 0; i < 4; ++i) {
    out[i] = E->h_totals[i];
    finite = finite && std::isfinite(out[i]);
  }
  if (!finite) {
    set_error("ensemble instance has a non-finite conserved total");
    return OM_ERR_NONFINITE;
  }
  return OM_OK;
}

om_status om_ensemble_last_launch_count(om_ensemble E, int *launches) {
  if (!E || !launches) { set_error("null argument"); return OM_ERR_ARG; }
  *launches = E->last_launches;
  return OM_OK;
}

}  // extern "C"
