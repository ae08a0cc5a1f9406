// hydro_fast.cu -- the production FP32 build of the fused Hydro step:
// same source as the exact build (hydro_kernels.cuh), compiled with
// multiply-add contraction, in the tile shapes the tuner chooses from.
#include <cuda_runtime.h>

#include "hydro_launch.cuh"

namespace om {

cudaError_t hydro_fused_f32_exact(const HydroStepArgs &a, cudaStream_t s, int *grid_out);

template <int TX, int TY, int NT>
static cudaError_t launch_fast(const HydroStepArgs &a0, cudaStream_t s, int *grid_out) {
  HydroStepArgs a = a0;
  a.nt0 = (a.n0 + TX - 1) / TX;
  const int nt1 = (a.n1 + TY - 1) / TY;
  const size_t smem = sizeof(FusedSmem<float, TX, TY>);
  cudaError_t e = cudaFuncSetAttribute(hydro_fused_kernel<float, TX, TY, NT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  hydro_fused_kernel<float, TX, TY, NT><<<a.nt0 * nt1, NT, smem, s>>>(a);
  if (grid_out) *grid_out = a.nt0 * nt1;
  return cudaGetLastError();
}

cudaError_t hydro_fused_f32(const HydroStepArgs &a, int tile, bool exact, cudaStream_t s,
                            int *grid_out) {
  if (exact) return hydro_fused_f32_exact(a, s, grid_out);
  switch (tile) {
    case kTile32x8: return launch_fast<32, 8, 256>(a, s, grid_out);
    case kTile64x16: return launch_fast<64, 16, 512>(a, s, grid_out);
    default: return launch_fast<32, 16, 256>(a, s, grid_out);
  }
}

}  // namespace om
