// life_noalloc.cu -- a Life entry point that allocates no memory at all.
//
// Some callers cannot call cudaMalloc: host frameworks whose device
// allocator owns all device memory and forbids allocations by anyone else,
// and real-time loops that must not block on the allocator (cudaMalloc can
// wait for the whole device).  They own the cell grids; this entry point
// only needs a few per-generation counters, which live in a file-scope
// device array instead of memory allocated per call.
//
// The call returns with the caller's stream synchronised: it reads back the
// cell-value flag and copies the populations before it returns.
//
// The array is OM_LIFE_NOALLOC_MAX_GENERATIONS + 1 words: one population
// counter per generation and a flag raised when a cell is neither 0 nor 1.
// Every GPU that loads this library holds it until the process exits.
// Every call shares it and it keeps the last call's contents, so each call
// clears it before use; calls that overlap on the GPU (different streams,
// or several host threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "om_internal.cuh"

namespace om {

cudaError_t life_tb_launch_into(const int32_t *cur, int32_t *next, int n0, int n1, int gens,
                                uint32_t *pop, cudaStream_t s);
cudaError_t life_check_cells_into(const int32_t *cells, size_t n, uint32_t *flag,
                                  cudaStream_t s);

static __device__ __align__(256) uint32_t
    g_life_noalloc_scratch[OM_LIFE_NOALLOC_MAX_GENERATIONS + 1];

// Device address of the scratch array, looked up once per device with that
// device current.  A host-side reference to g_life_noalloc_scratch is only
// a stand-in for the symbol and must never be handed to a kernel.
static const int kMaxDevices = 64;
static uint32_t *g_scratch_ptr[kMaxDevices];
static std::mutex g_scratch_mu;

static om_status scratch_for_current_device(uint32_t **out) {
  int dev = -1;
  OM_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("om_life_proceed_noalloc: device ordinal out of range");
    return OM_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_life_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("om_life_proceed_noalloc: cudaGetSymbolAddress failed: ") +
                cudaGetErrorString(e));
      return OM_ERR_CUDA;
    }
    g_scratch_ptr[dev] = (uint32_t *)p;
  }
  *out = g_scratch_ptr[dev];
  return OM_OK;
}

}  // namespace om

using namespace om;

extern "C" om_status om_life_proceed_noalloc(const int32_t *cells_in, int32_t *cells_out,
                                             int n0, int n1, int generations,
                                             int32_t *populations, void *stream) {
  if (!cells_in || !cells_out || !populations) {
    set_error("om_life_proceed_noalloc: null pointer argument");
    return OM_ERR_ARG;
  }
  if (cells_in == cells_out) {
    set_error("om_life_proceed_noalloc: cells_in and cells_out must be different buffers");
    return OM_ERR_ARG;
  }
  if (generations < 1 || generations > OM_LIFE_NOALLOC_MAX_GENERATIONS) {
    set_error("om_life_proceed_noalloc: generations must be in [1, " +
              std::to_string(OM_LIFE_NOALLOC_MAX_GENERATIONS) +
              "]: the shared scratch holds one population counter per generation");
    return OM_ERR_ARG;
  }
  if (n0 < 32 || n1 < 1 || n0 % 32 != 0 || n0 > (1 << 20) || n1 > (1 << 20)) {
    set_error("om_life_proceed_noalloc: n0 must be a multiple of 32 in [32, 2^20] and "
              "n1 in [1, 2^20]");
    return OM_ERR_ARG;
  }
  // populations are int32: a grid of more than INT32_MAX cells could report a
  // wrapped count
  if ((size_t)n0 * (size_t)n1 > (size_t)INT32_MAX) {
    set_error("om_life_proceed_noalloc: n0 * n1 must be at most 2^31 - 1 cells (the "
              "populations are int32)");
    return OM_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t *scratch = nullptr;
  OM_TRY(scratch_for_current_device(&scratch));
  const size_t bytes = sizeof(uint32_t) * (OM_LIFE_NOALLOC_MAX_GENERATIONS + 1);
  OM_CUDA_CHECK(cudaMemsetAsync(scratch, 0, bytes, s));
  const size_t n = (size_t)n0 * n1;
  uint32_t *flag = scratch + OM_LIFE_NOALLOC_MAX_GENERATIONS;
  OM_CUDA_CHECK(life_check_cells_into(cells_in, n, flag, s));
  OM_CUDA_CHECK(life_tb_launch_into(cells_in, cells_out, n0, n1, generations, scratch, s));
  uint32_t bad = 0;
  OM_CUDA_CHECK(cudaMemcpyAsync(&bad, flag, sizeof(bad), cudaMemcpyDeviceToHost, s));
  OM_CUDA_CHECK(cudaMemcpyAsync(populations, scratch, sizeof(int32_t) * generations,
                                cudaMemcpyDefault, s));
  OM_CUDA_CHECK(cudaStreamSynchronize(s));
  if (bad) {
    set_error("om_life_proceed_noalloc: every cell must be 0 or 1 (cells_out is unspecified)");
    return OM_ERR_ARG;
  }
  return OM_OK;
}
