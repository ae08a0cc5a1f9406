// hydro_launch.cuh -- host-side launchers of the Hydro kernels, declared for
// hydro.cu and defined in the translation units that compile the kernels
// (hydro_exact.cu without multiply-add contraction, hydro_fast.cu with it).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/om_gb300.h"
#include "hydro_kernels.cuh"

namespace om {

// Tile shapes of the fused kernel available to the tuner (FP32 production
// build; FP64 and the exact FP32 variant run 32x16).
// The sweep shapes (kSweep*) walk strips of TX columns down the grid in
// chunks of TY rows (hydro_sweep.cuh).  kPersist32x32, kPair32x32 and
// kPairGroups32x32 are the persistent 32 x 32 kernel with prefetched boxes
// (hydro_persist.cuh): one wall or cell per thread, two with packed f32x2
// instructions, and the latter as one CTA of two groups half a tile apart;
// on grids whose sides are multiples of 32 and at least 64, else the
// 32 x 32 tile kernel.
enum HydroTile {
  kTile32x8 = 0, kTile32x16 = 1, kTile64x16 = 2, kTile32x32 = 3, kTile64x8 = 4,
  kSweep32x8 = 5, kSweep32x16 = 6, kSweep64x8 = 7, kPersist32x32 = 8, kPair32x32 = 9,
  kPairGroups32x32 = 10, kTileCount = 11
};
inline bool hydro_tile_is_persistent(int tile) {
  return tile == kPersist32x32 || tile == kPair32x32 || tile == kPairGroups32x32;
}
// the persistent kernel's form: 0 one wall per thread, 1 paired, 2 paired
// with two groups per CTA
inline int hydro_persist_form(int tile) {
  return tile == kPairGroups32x32 ? 2 : tile == kPair32x32 ? 1 : 0;
}
inline bool hydro_tile_is_sweep(int tile) { return tile >= kSweep32x8 && tile <= kSweep64x8; }
void hydro_tile_dims(int tile, int *tx, int *ty);
// the tile a configuration's tile_x / tile_y select (0 = default): x 64
// with y 8 is 64x8, else 64x16; x 0 or 32 with y 8, 16 or 32 is 32x8,
// 32x16 or the 32x32 tile kernel; with y 0 the persistent 32 x 32 kernel:
// x 0 (the production default) paired, as one CTA per SM of two groups half
// a tile apart; x 16 paired, two CTAs per SM; x 32 one wall or cell per
// thread.
// A negative tile_y selects a sweep of -tile_y rows per chunk (x 32 or 64).
inline int hydro_tile_of(int tile_x, int tile_y, bool production) {
  if (!production) return kTile32x16;
  if (tile_y < 0) {
    if (tile_x == 64) return kSweep64x8;
    return tile_y == -16 ? kSweep32x16 : kSweep32x8;
  }
  if (tile_x == 64) return tile_y == 8 ? kTile64x8 : kTile64x16;
  if (tile_y == 8) return kTile32x8;
  if (tile_y == 16) return kTile32x16;
  if (tile_y == 32) return kTile32x32;
  if (tile_x == 16) return kPair32x32;
  return tile_x == 32 ? kPersist32x32 : kPairGroups32x32;
}

// fused two-stage step; `exact` selects the no-contraction build
cudaError_t hydro_fused_f32(const HydroStepArgs &a, int tile, bool exact, cudaStream_t s,
                            int *grid_out);
cudaError_t hydro_fused_f64(const HydroStepArgs &a, int tile, cudaStream_t s, int *grid_out);
// one fused step of a periodic grid that also writes the tape of the
// reverse sweep (32x16 tiles; the build of the handle's variant)
cudaError_t hydro_fused_tape(int fp64, bool exact, const HydroStepArgs &a, const HydroTapeOut &t,
                             cudaStream_t s, int tile);

// ensemble step over every instance (persistent grid of `grid` blocks, 0 =
// resident blocks x SMs); args/prefix in device memory.  The persistent
// tiles take `table` (4 tensor maps per instance, hydro_persist_encode of
// the instance's args) and fall back to the 32 x 32 tile kernel without one.
cudaError_t hydro_ensemble_f32(const HydroStepArgs *args, const int *prefix, int count, int tile,
                               bool exact, int grid, cudaStream_t s,
                               const CUtensorMap *table = nullptr);

// the persistent 32 x 32 production step (hydro_persist.cu): grids whose
// sides are multiples of 32 and at least 64 (periodic)
bool hydro_persist_fits(int n0, int n1);
// the four field tensor maps of a's current state
bool hydro_persist_encode(CUtensorMap *maps4, const HydroStepArgs &a);
// the form that runs for `tiles` tiles: two groups per CTA only when every
// group has at least 16 tiles (grid_limit > 0: that many CTAs at most),
// else the paired form
int hydro_persist_form_for(int form, long long tiles, int device, int grid_limit);
// resident CTAs per SM of the persistent ensemble kernel of a form
// (hydro_persist_form; a CTA of form 2 holds two groups)
int hydro_persist_occupancy(int form);
cudaError_t hydro_persist_step(const HydroStepArgs &a, int form, cudaStream_t s, int *grid_out);
cudaError_t hydro_persist_tape(const HydroStepArgs &a, int form, const HydroTapeOut &t,
                               cudaStream_t s);
cudaError_t hydro_persist_ensemble(const HydroStepArgs *args, const int *prefix, int count,
                                   const CUtensorMap *table, int form, int grid,
                                   cudaStream_t s);
cudaError_t hydro_ensemble_f64(const HydroStepArgs *args, const int *prefix, int count, int tile,
                               int grid, cudaStream_t s);
// resident blocks per SM of the ensemble kernel for (fp64, tile, exact)
int hydro_ensemble_occupancy(int fp64, int tile, bool exact);

// CFL minimum of a state into sc->tsmin[slot] (slot pre-set to all ones)
cudaError_t hydro_tsmin(int fp64, const void *rho, const void *v0, const void *v1,
                        const void *p, size_t n, double gamma, HydroScalars *sc, int slot,
                        int grid, cudaStream_t s);
// the same for an open grid with margins lm: the margin cells' (jet)
// minimum into *margin_min, then interior and margin into sc->tsmin[slot]
cudaError_t hydro_tsmin_open(int fp64, const void *rho, const void *v0, const void *v1,
                             const void *p, int n0, int n1, int lm, double gamma,
                             HydroScalars *sc, int slot, unsigned long long *margin_min, int grid,
                             cudaStream_t s);

// plain path pieces
cudaError_t hydro_plain_timescale(int fp64, const void *rho, const void *v0, const void *v1,
                                  const void *p, void *ts, size_t n, double gamma,
                                  const HydroScalars *sc, int grid, cudaStream_t s);
cudaError_t hydro_plain_reduce_min(int fp64, const void *ts, size_t n, unsigned long long *out,
                                   int grid, cudaStream_t s);
cudaError_t hydro_plain_step(int fp64, const void *rho, const void *v0, const void *v1,
                             const void *p, void *orho, void *ov0, void *ov1, void *op, int n0,
                             int n1, double gamma, double dtG, double dR0, double dR1, int grid,
                             cudaStream_t s);
cudaError_t hydro_scalar_advance(HydroScalars *sc, double dt, double *dt_hist, cudaStream_t s);

// initial states
cudaError_t hydro_init_jet(int fp64, void *rho, void *v0, void *v1, void *p, int n0, int n1,
                           int lm, double gamma, const HydroScalars *sc, cudaStream_t s);
cudaError_t hydro_init_kh(int fp64, void *rho, void *v0, void *v1, void *p, int n0, int n1,
                          unsigned long long seed_mix, cudaStream_t s);

// compensated FP64 totals over the n0 x n1 interior of memory arrays with
// margins lm: partials[blocks][8], then out[4] (device)
cudaError_t hydro_totals(int fp64, const void *rho, const void *v0, const void *v1,
                         const void *p, int n0, int n1, int lm, double gamma, double *partials,
                         int blocks, double *out, cudaStream_t s);

// A saved Hydro state (hydro.cu): the four arrays (device copies), the
// scalar block and the cached-minimum bookkeeping, so that a restore
// continues bit-identically.  Used by the adjoint's checkpointing.
struct Handle;
struct HydroCheckpoint {
  void *f[4] = {nullptr, nullptr, nullptr, nullptr};
  unsigned char sc[sizeof(HydroScalars)];
  unsigned char state[64];
};
om_status hydro_checkpoint_alloc(Handle *h, HydroCheckpoint *c);
void hydro_checkpoint_free(HydroCheckpoint *c);
om_status hydro_save(Handle *h, HydroCheckpoint *c);
om_status hydro_restore(Handle *h, const HydroCheckpoint *c);
// the device address of the CFL minimum of h's current state (computed first
// when the cached one does not belong to it)
om_status hydro_tsmin_device(Handle *h, unsigned long long **ptr);

}  // namespace om
