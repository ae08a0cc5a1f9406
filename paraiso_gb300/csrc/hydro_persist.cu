// hydro_persist.cu -- launchers of the persistent production FP32 step
// (hydro_persist.cuh): single grids (plain and taped) and ensembles.
// Compiled with the production build's fast single-precision math, like
// hydro_fast.cu, so the two tile codes give the same bits.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "hydro_launch.cuh"
#include "hydro_persist.cuh"
#include "om_internal.cuh"

namespace om {

// The two-group form pays half a tile per group for its start; it runs when
// each of its groups (two per CTA, one CTA per SM or grid_limit CTAs) has at
// least 16 tiles, else the paired form with two CTAs per SM does.
int hydro_persist_form_for(int form, long long tiles, int device, int grid_limit) {
  if (form != 2) return form;
  int ctas = sm_count(device);
  if (grid_limit > 0 && grid_limit < ctas) ctas = grid_limit;
  return tiles >= 16LL * 2 * ctas ? 2 : 1;
}

bool hydro_persist_fits(int n0, int n1) {
  return n0 % hp::TX == 0 && n1 % hp::TY == 0 && n0 >= 2 * hp::TX && n1 >= 2 * hp::TY;
}

// one field of an n0 x n1 FP32 grid as a 2-D tensor of 40 x 38 boxes
static bool encode_field(CUtensorMap *m, const void *base, int n0, int n1) {
  const uint64_t dims[2] = {(uint64_t)n0, (uint64_t)n1};
  const uint64_t strides[1] = {(uint64_t)n0 * sizeof(float)};
  const uint32_t box[2] = {(uint32_t)hp::BW, (uint32_t)hp::BH};
  return tma::encode_tiled(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims,
                           strides, box, CU_TENSOR_MAP_SWIZZLE_NONE);
}

bool hydro_persist_encode(CUtensorMap *maps4, const HydroStepArgs &a) {
  const void *f[4] = {a.rho, a.v0, a.v1, a.p};
  for (int k = 0; k < 4; ++k)
    if (!encode_field(&maps4[k], f[k], a.n0, a.n1)) return false;
  return true;
}

template <class K> static int resident_per_sm(K kernel, int threads, int groups = 1) {
  const int smem = (int)sizeof(hp::Smem) * groups;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int hydro_persist_occupancy(int form) {
  static int n[3] = {-1, -1, -1};
  int &v = n[form];
  if (v < 0)
    v = form == 2 ? resident_per_sm(hp::hydro_pair2_ensemble_kernel, 2 * hp::NT2, 2)
        : form == 1 ? resident_per_sm(hp::hydro_persist_ensemble_kernel<true>, hp::NT2)
                    : resident_per_sm(hp::hydro_persist_ensemble_kernel<false>, hp::NT);
  return v > 0 ? v : 1;
}

// FORM 0: one wall or cell per thread; 1: paired; 2: paired, two groups per CTA
template <bool TAPE, int FORM>
static cudaError_t persist_launch(const HydroStepArgs &a0, const HydroTapeOut *tape,
                                  cudaStream_t s, int *grid_out) {
  auto kernel = FORM == 2 ? hp::hydro_pair2_kernel<TAPE>
                : FORM == 1 ? hp::hydro_pair_kernel<TAPE> : hp::hydro_persist_kernel<TAPE>;
  const int groups = FORM == 2 ? 2 : 1;
  const int threads = (FORM == 0 ? hp::NT : hp::NT2) * groups;
  const size_t smem = sizeof(hp::Smem) * groups;
  static int occ = -1;
  if (occ < 0) occ = resident_per_sm(kernel, threads, groups);
  if (occ <= 0) return cudaErrorInvalidConfiguration;
  HydroStepArgs a = a0;
  a.nt0 = a.n0 / hp::TX;
  CUtensorMap m[4];
  if (!hydro_persist_encode(m, a)) return cudaErrorInvalidValue;
  int dev = 0;
  cudaGetDevice(&dev);
  const int tiles = a.nt0 * (a.n1 / hp::TY);
  // every group of a CTA takes at least one tile
  int grid = std::min((tiles + groups - 1) / groups, occ * sm_count(dev));
  if (a.grid_limit > 0) grid = std::min(grid, a.grid_limit);
  HydroTapeOut t{};
  if (tape) t = *tape;
  kernel<<<grid, threads, smem, s>>>(a, m[0], m[1], m[2], m[3], t);
  if (grid_out) *grid_out = grid;
  return cudaGetLastError();
}

cudaError_t hydro_persist_step(const HydroStepArgs &a, int form, cudaStream_t s, int *grid_out) {
  int dev = 0;
  cudaGetDevice(&dev);
  form = hydro_persist_form_for(form, (long long)(a.n0 / hp::TX) * (a.n1 / hp::TY), dev,
                                a.grid_limit);
  return form == 2 ? persist_launch<false, 2>(a, nullptr, s, grid_out)
         : form == 1 ? persist_launch<false, 1>(a, nullptr, s, grid_out)
                     : persist_launch<false, 0>(a, nullptr, s, grid_out);
}

cudaError_t hydro_persist_tape(const HydroStepArgs &a, int form, const HydroTapeOut &t,
                               cudaStream_t s) {
  int dev = 0;
  cudaGetDevice(&dev);
  form = hydro_persist_form_for(form, (long long)(a.n0 / hp::TX) * (a.n1 / hp::TY), dev,
                                a.grid_limit);
  return form == 2 ? persist_launch<true, 2>(a, &t, s, nullptr)
         : form == 1 ? persist_launch<true, 1>(a, &t, s, nullptr)
                     : persist_launch<true, 0>(a, &t, s, nullptr);
}

cudaError_t hydro_persist_ensemble(const HydroStepArgs *args, const int *prefix, int count,
                                   const CUtensorMap *table, int form, int grid,
                                   cudaStream_t s) {
  if (hydro_persist_occupancy(form) < 1) return cudaErrorInvalidConfiguration;
  if (form == 2)
    hp::hydro_pair2_ensemble_kernel<<<grid, 2 * hp::NT2, 2 * sizeof(hp::Smem), s>>>(
        args, prefix, count, table);
  else if (form == 1)
    hp::hydro_persist_ensemble_kernel<true><<<grid, hp::NT2, sizeof(hp::Smem), s>>>(
        args, prefix, count, table);
  else
    hp::hydro_persist_ensemble_kernel<false><<<grid, hp::NT, sizeof(hp::Smem), s>>>(
        args, prefix, count, table);
  return cudaGetLastError();
}

}  // namespace om
