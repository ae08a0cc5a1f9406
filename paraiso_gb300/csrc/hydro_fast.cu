// hydro_fast.cu -- the production FP32 build of the fused Hydro step:
// the tile code of the exact build (hydro_kernels.cuh) with the production
// algebra (hf:: in hydro_scheme.cuh), compiled with multiply-add
// contraction and fast single-precision division and square root, in the
// tile shapes the tuner chooses from.
#include <cuda_runtime.h>

#include "hydro_launch.cuh"
#include "hydro_sweep.cuh"
#include "om_internal.cuh"

namespace om {

cudaError_t hydro_fused_f32_exact(const HydroStepArgs &a, cudaStream_t s, int *grid_out);

template <int TX, int TY, int NT, bool OPEN = false>
static cudaError_t launch_fast(const HydroStepArgs &a0, cudaStream_t s, int *grid_out) {
  HydroStepArgs a = a0;
  a.nt0 = (a.n0 + TX - 1) / TX;
  const int nt1 = (a.n1 + TY - 1) / TY;
  const size_t smem = sizeof(FusedSmem<float, TX, TY>);
  cudaError_t e = cudaFuncSetAttribute(hydro_fused_kernel<float, TX, TY, NT, OPEN, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  hydro_fused_kernel<float, TX, TY, NT, OPEN, true><<<a.nt0 * nt1, NT, smem, s>>>(a);
  if (grid_out) *grid_out = a.nt0 * nt1;
  return cudaGetLastError();
}

// The production sweep over a periodic grid: strips of TX columns, segments
// sized to fill the resident blocks about once.  With `tape`, the taped step.
template <int TX, int TY, int NT, bool TAPE>
static cudaError_t launch_sweep(const HydroStepArgs &a0, const HydroTapeOut *tape,
                                cudaStream_t s, int *grid_out) {
  using K = void (*)(HydroStepArgs, SweepGeom, const HydroTapeOut);
  K k = hydro_sweep_kernel<float, TX, TY, NT, TAPE, true>;
  const size_t smem = sizeof(SweepSmem<float, TX, TY>);
  static int resident_per_sm = 0;  // the same on every device of one kind
  if (!resident_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NT, smem);
    if (e != cudaSuccess) return e;
    resident_per_sm = n > 0 ? n : 1;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  HydroStepArgs a = a0;
  a.nt0 = 0;
  const SweepGeom geo = sweep_geometry(a.n0, a.n1, TX, TY, resident_per_sm * sm_count(dev));
  HydroTapeOut t{};
  if (tape) t = *tape;
  const int grid = geo.strips * geo.segs;
  k<<<grid, NT, smem, s>>>(a, geo, t);
  if (grid_out) *grid_out = grid;
  return cudaGetLastError();
}

cudaError_t hydro_ensemble_f32_exact(const HydroStepArgs *args, const int *prefix, int count,
                                     int grid, cudaStream_t s);
int hydro_ensemble_occupancy_exact(int fp64);

template <int TX, int TY, int NT>
static cudaError_t launch_ens(const HydroStepArgs *args, const int *prefix, int count, int grid,
                              cudaStream_t s) {
  const size_t smem = sizeof(FusedSmem<float, TX, TY>);
  cudaError_t e = cudaFuncSetAttribute(hydro_ensemble_kernel<float, TX, TY, NT, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  hydro_ensemble_kernel<float, TX, TY, NT, true><<<grid, NT, smem, s>>>(args, prefix, count);
  return cudaGetLastError();
}

template <int TX, int TY, int NT> static int occ_fast() {
  const size_t smem = sizeof(FusedSmem<float, TX, TY>);
  cudaFuncSetAttribute(hydro_ensemble_kernel<float, TX, TY, NT, true>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, hydro_ensemble_kernel<float, TX, TY, NT, true>,
                                                    NT, smem) != cudaSuccess || n < 1) {
    cudaGetLastError();
    n = 1;
  }
  return n;
}

cudaError_t hydro_ensemble_f32(const HydroStepArgs *args, const int *prefix, int count, int tile,
                               bool exact, int grid, cudaStream_t s, const CUtensorMap *table) {
  if (exact) return hydro_ensemble_f32_exact(args, prefix, count, grid, s);
  if (hydro_tile_is_persistent(tile) && table)
    return hydro_persist_ensemble(args, prefix, count, table, hydro_persist_form(tile), grid, s);
  switch (tile) {
    case kTile32x8: return launch_ens<32, 8, 256>(args, prefix, count, grid, s);
    case kTile64x16: return launch_ens<64, 16, 512>(args, prefix, count, grid, s);
    case kTile32x32: return launch_ens<32, 32, 512>(args, prefix, count, grid, s);
    case kTile64x8: return launch_ens<64, 8, 256>(args, prefix, count, grid, s);
    case kTile32x16: return launch_ens<32, 16, 256>(args, prefix, count, grid, s);
    default: return launch_ens<32, 32, 512>(args, prefix, count, grid, s);
  }
}

int hydro_ensemble_occupancy(int fp64, int tile, bool exact) {
  if (fp64 || exact) return hydro_ensemble_occupancy_exact(fp64);
  switch (tile) {
    case kPersist32x32:
    case kPair32x32:
    case kPairGroups32x32: return hydro_persist_occupancy(hydro_persist_form(tile));
    case kTile32x8: return occ_fast<32, 8, 256>();
    case kTile64x16: return occ_fast<64, 16, 512>();
    case kTile32x32: return occ_fast<32, 32, 512>();
    case kTile64x8: return occ_fast<64, 8, 256>();
    case kTile32x16: return occ_fast<32, 16, 256>();
    default: return occ_fast<32, 32, 512>();
  }
}

cudaError_t hydro_fused_tape_exact(int fp64, const HydroStepArgs &a, const HydroTapeOut &t,
                                   cudaStream_t s);

// the taped production step on TX x TY tiles
template <int TX, int TY, int NT>
static cudaError_t launch_tape_fast(const HydroStepArgs &a0, const HydroTapeOut &t,
                                   cudaStream_t s) {
  HydroStepArgs a = a0;
  a.nt0 = (a.n0 + TX - 1) / TX;
  const int nt1 = (a.n1 + TY - 1) / TY;
  const size_t smem = sizeof(FusedSmem<float, TX, TY>);
  cudaError_t e = cudaFuncSetAttribute(hydro_fused_tape_kernel<float, TX, TY, NT, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  hydro_fused_tape_kernel<float, TX, TY, NT, true><<<a.nt0 * nt1, NT, smem, s>>>(a, t);
  return cudaGetLastError();
}

cudaError_t hydro_fused_tape(int fp64, bool exact, const HydroStepArgs &a0, const HydroTapeOut &t,
                             cudaStream_t s, int tile) {
  if (fp64 || exact) return hydro_fused_tape_exact(fp64, a0, t, s);
  // the taped step runs the code of the handle's production step, so a
  // recomputed state equals the forward pass's bit for bit
  switch (tile) {
    case kPersist32x32:
    case kPair32x32:
    case kPairGroups32x32:
      if (hydro_persist_fits(a0.n0, a0.n1))
        return hydro_persist_tape(a0, hydro_persist_form(tile), t, s);
      return launch_tape_fast<32, 32, 512>(a0, t, s);
    case kTile32x8: return launch_tape_fast<32, 8, 256>(a0, t, s);
    case kTile64x16: return launch_tape_fast<64, 16, 512>(a0, t, s);
    case kTile32x16: return launch_tape_fast<32, 16, 256>(a0, t, s);
    case kTile64x8: return launch_tape_fast<64, 8, 256>(a0, t, s);
    case kSweep32x8: return launch_sweep<32, 8, 256, true>(a0, &t, s, nullptr);
    case kSweep32x16: return launch_sweep<32, 16, 512, true>(a0, &t, s, nullptr);
    case kSweep64x8: return launch_sweep<64, 8, 512, true>(a0, &t, s, nullptr);
    default: return launch_tape_fast<32, 32, 512>(a0, t, s);
  }
}

cudaError_t hydro_fused_f32(const HydroStepArgs &a, int tile, bool exact, cudaStream_t s,
                            int *grid_out) {
  if (exact) return hydro_fused_f32_exact(a, s, grid_out);
  // an open grid (margins, jet boundary condition) runs the 32x16 tile
  if (a.lm > 0) return launch_fast<32, 16, 256, true>(a, s, grid_out);
  switch (tile) {
    case kPersist32x32:
    case kPair32x32:
    case kPairGroups32x32:
      if (hydro_persist_fits(a.n0, a.n1))
        return hydro_persist_step(a, hydro_persist_form(tile), s, grid_out);
      return launch_fast<32, 32, 512>(a, s, grid_out);
    case kTile32x8: return launch_fast<32, 8, 256>(a, s, grid_out);
    case kTile64x16: return launch_fast<64, 16, 512>(a, s, grid_out);
    case kTile32x32: return launch_fast<32, 32, 512>(a, s, grid_out);
    case kTile64x8: return launch_fast<64, 8, 256>(a, s, grid_out);
    case kSweep32x8: return launch_sweep<32, 8, 256, false>(a, nullptr, s, grid_out);
    case kSweep32x16: return launch_sweep<32, 16, 512, false>(a, nullptr, s, grid_out);
    case kSweep64x8: return launch_sweep<64, 8, 512, false>(a, nullptr, s, grid_out);
    case kTile32x16: return launch_fast<32, 16, 256>(a, s, grid_out);
    default: return launch_fast<32, 32, 512>(a, s, grid_out);
  }
}

}  // namespace om
