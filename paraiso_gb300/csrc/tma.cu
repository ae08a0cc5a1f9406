// tma.cu -- host side of tma.cuh: tensor-map encoding through the driver
// entry point (the runtime hands out the driver's cuTensorMapEncodeTiled, so
// the library needs no link against the driver library).
#include <mutex>
#include <string>

#include "om_internal.cuh"
#include "tma.cuh"

namespace om {
namespace tma {

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    else
      cudaGetLastError();
  });
  return fn;
}

bool encode_tiled(CUtensorMap *map, CUtensorMapDataType type, int rank, void *base,
                  const uint64_t *dims, const uint64_t *strides_bytes, const uint32_t *box,
                  CUtensorMapSwizzle swizzle) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || rank < 1 || rank > 5) return false;
  cuuint64_t d[5], st[4];
  cuuint32_t b[5], es[5];
  for (int i = 0; i < rank; ++i) {
    d[i] = dims[i];
    b[i] = box[i];
    es[i] = 1;
    if (i + 1 < rank) st[i] = strides_bytes[i];
  }
  CUtensorMap m;
  const CUresult r = fn(&m, type, (cuuint32_t)rank, base, d, st, b, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  *map = m;
  return true;
}

// An mbarrier armed for 128 bytes that no copy delivers (none is issued, so
// nothing is in flight): the bounded wait must give up and raise *err.
__global__ void wait_bound_selftest_kernel(uint32_t *err, uint32_t polls) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar, 128);
    mbar_wait(&bar, 0, err, polls);
  }
}

}  // namespace tma
}  // namespace om

using namespace om;

// See include/om_gb300.h.
extern "C" om_status om_selftest_wait_bound(int device) {
  OM_CUDA_CHECK(cudaSetDevice(device));
  uint32_t *err = nullptr;
  if (cudaMalloc(&err, sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    set_error("om_selftest_wait_bound: cannot allocate the error word");
    return OM_ERR_NOMEM;
  }
  uint32_t h = 0;
  cudaError_t e = cudaMemset(err, 0, sizeof(uint32_t));
  // 200 polls of at most 20 us each: the wait gives up within about 4 ms
  if (e == cudaSuccess) {
    tma::wait_bound_selftest_kernel<<<1, 32>>>(err, 200);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (e != cudaSuccess) {
    set_error(std::string("om_selftest_wait_bound: ") + cudaGetErrorString(e));
    return OM_ERR_CUDA;
  }
  if (h != 1) {
    set_error("om_selftest_wait_bound: the bounded wait did not report its time-out");
    return OM_ERR_STATE;
  }
  return OM_OK;
}
