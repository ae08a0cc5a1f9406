// autotune.cu -- measured search over the GB300 kernels' launch knobs.
//
// The reference tunes its generated CUDA with a genetic algorithm over a
// genome of cudaGridSize (16+16 bits), a Manifest/Delayed choice per OM node
// and __syncthreads hints (Language/Paraiso/Tuning/Genetic.hs:138-172,
// examples-old/GA/*), scoring each genome by regenerating, recompiling and
// timing the program.  Here the knobs that matter on GB300 are few and known
// at run time, so the tuner times every candidate of a small grid directly,
// on the caller's mesh size, through the public C ABI, and keeps the best per
// (kind, size, precision, device) for the life of the process:
//   Life  : kernel family (register-resident blocks, warp-specialised,
//           shared-memory tiles), temporal depth, block rows
//   Hydro : fused-step tile shape (32x8, 32x16, 64x16, 32x32, 64x8) and
//           column sweeps (32 x 8, 32 x 16 and 64 x 8 rows per chunk)
//   Ensemble: tile shape and persistent grid size (all resident CTAs, or
//           one CTA per SM)
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "om_internal.cuh"

namespace {

struct Key {
  int kind, n0, n1, precision, device;
  bool operator<(const Key &o) const {
    return std::tie(kind, n0, n1, precision, device) <
           std::tie(o.kind, o.n0, o.n1, o.precision, o.device);
  }
};

struct Entry {
  om_config cfg;
  double rate;
};

std::mutex g_mu;
std::map<Key, Entry> g_cache;

// cell-updates per second of one candidate (0 when the candidate fails)
double time_candidate(int kind, const int *sizes, const om_config &cfg, int steps) {
  om_handle h = nullptr;
  if (om_create(kind, 2, sizes, &cfg, &h) != OM_OK) return 0.0;
  double rate = 0.0;
  bool ok = true;
  if (kind == OM_KIND_LIFE) {
    ok = om_life_fill_random(h, 1, 0.3) == OM_OK;
  } else {
    ok = om_hydro_init_kh(h, 1) == OM_OK;
  }
  int kid = -1;
  ok = ok && om_kernel_id(h, "proceed", &kid) == OM_OK;
  float ms = 0;
  // one run to settle (allocations, first-touch), then the best of two
  ok = ok && om_time_run(h, kid, steps, &ms) == OM_OK;
  float best = 1e30f;
  for (int r = 0; ok && r < 2; ++r) {
    ok = om_time_run(h, kid, steps, &ms) == OM_OK;
    if (ok && ms < best) best = ms;
  }
  if (ok && best > 0) rate = (double)sizes[0] * sizes[1] * steps / (best * 1e-3);
  om_destroy(h);
  return ok ? rate : 0.0;
}

}  // namespace

extern "C" om_status om_autotune(int kind, int ndim, const int *sizes, const om_config *base,
                                 om_config *best, double *best_rate) {
  if (!sizes || !best || ndim != 2 || (kind != OM_KIND_LIFE && kind != OM_KIND_HYDRO)) {
    om::set_error("om_autotune: bad arguments");
    return OM_ERR_ARG;
  }
  om_config b;
  if (base) b = *base; else om_config_default(&b);
  const Key key{kind, sizes[0], sizes[1], kind == OM_KIND_HYDRO ? b.precision : 0, b.device};
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      *best = it->second.cfg;
      if (best_rate) *best_rate = it->second.rate;
      return OM_OK;
    }
  }
  std::vector<om_config> cands;
  int steps = 0;
  if (kind == OM_KIND_LIFE) {
    steps = 96;
    const bool packed = b.boundary == OM_BOUNDARY_CYCLIC && sizes[0] % 32 == 0 && b.variant == 0;
    if (!packed) {
      cands.push_back(b);  // only the integer kernel applies
    } else {
      for (int depth : {24, 32})
        for (int th : {0, 128, 192, 256, 320}) {
          om_config c = b;
          c.depth = depth;
          c.tile_x = 0;
          c.tile_y = th;
          c.life_kernel = 0;
          cands.push_back(c);
        }
      for (int k = 1; k <= (sizes[0] >= 1024 ? 16 : 4); ++k) {
        om_config c = b;
        c.depth = 32;
        c.tile_x = 0;
        c.tile_y = 0;
        c.life_kernel = k;
        cands.push_back(c);
      }
      for (int th : {128, 192}) {
        om_config c = b;
        c.depth = 32;
        c.tile_x = 30;
        c.tile_y = th;
        c.life_kernel = 0;
        cands.push_back(c);
      }
    }
  } else {
    steps = 8;
    // the persistent 32 x 32 kernel, paired with two groups per CTA (0, 0),
    // paired with two CTAs per SM (16, 0) and one wall per thread (32, 0),
    // tile kernels, then column sweeps (a negative tile_y: rows per chunk)
    const int shapes[11][2] = {{0, 0}, {16, 0}, {32, 0}, {0, 32}, {0, 8}, {64, 0}, {0, 16},
                               {64, 8}, {0, -8}, {0, -16}, {64, -8}};
    const int nshapes = (b.precision == 64 || b.variant != 0) ? 1 : 11;
    for (int s = 0; s < nshapes; ++s) {
      om_config c = b;
      c.tile_x = shapes[s][0];
      c.tile_y = shapes[s][1];
      cands.push_back(c);
    }
  }
  double best_r = 0;
  om_config best_c = cands[0];
  for (const om_config &c : cands) {
    const double r = time_candidate(kind, sizes, c, steps);
    if (r > best_r) {
      best_r = r;
      best_c = c;
    }
  }
  if (best_r <= 0) {
    om::set_error("om_autotune: no candidate ran (see om_last_error of om_create)");
    return OM_ERR_CUDA;
  }
  {
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache[key] = Entry{best_c, best_r};
  }
  *best = best_c;
  if (best_rate) *best_rate = best_r;
  return OM_OK;
}

extern "C" om_status om_autotune_ensemble(int count, const int *sizes, const om_config *base,
                                          om_config *best, double *best_rate) {
  if (!sizes || !best || count < 1) {
    om::set_error("om_autotune_ensemble: bad arguments");
    return OM_ERR_ARG;
  }
  om_config b;
  if (base) b = *base; else om_config_default(&b);
  const int shapes[8][2] = {{0, 0}, {16, 0}, {32, 0}, {0, 32}, {0, 8}, {64, 0}, {0, 16}, {64, 8}};
  const int nshapes = (b.precision == 64 || b.variant != 0) ? 1 : 8;
  long long cells = 0;
  for (int k = 0; k < count; ++k) cells += (long long)sizes[2 * k] * sizes[2 * k + 1];
  int dev = b.device;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
    cudaGetLastError();
    sms = 0;
  }
  double best_r = 0;
  om_config best_c = b;
  for (int s = 0; s < 2 * nshapes; ++s) {
    om_config c = b;
    c.tile_x = shapes[s / 2][0];
    c.tile_y = shapes[s / 2][1];
    // persistent grid: every resident CTA (0), or one CTA per SM
    c.grid_limit = (s & 1) ? sms : 0;
    if ((s & 1) && sms == 0) continue;
    om_ensemble e = nullptr;
    if (om_ensemble_create(count, sizes, &c, &e) != OM_OK) continue;
    // 8 steps per timing, best of three after a settling run: candidates
    // within a few per cent of each other are told apart
    float ms = 0, bestms = 1e30f;
    bool ok = om_ensemble_init_kh(e, 1) == OM_OK && om_ensemble_time_step(e, 8, &ms) == OM_OK;
    for (int r = 0; ok && r < 3; ++r) {
      ok = om_ensemble_time_step(e, 8, &ms) == OM_OK;
      if (ok && ms < bestms) bestms = ms;
    }
    om_ensemble_destroy(e);
    if (!ok) continue;
    const double rate = (double)cells * 8 / (bestms * 1e-3);
    if (rate > best_r) {
      best_r = rate;
      best_c = c;
    }
  }
  if (best_r <= 0) {
    om::set_error("om_autotune_ensemble: no candidate ran");
    return OM_ERR_CUDA;
  }
  *best = best_c;
  if (best_rate) *best_rate = best_r;
  return OM_OK;
}
