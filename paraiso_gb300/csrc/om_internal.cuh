// om_internal.cuh -- shared declarations of the GB300 Orthotope Machine
// runtime: the handle, storage with its host mirror, error plumbing.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/om_gb300.h"

namespace om {

// Thread-local error text returned by om_last_error().
void set_error(const std::string &msg);

#define OM_CUDA_CHECK(expr)                                                   \
  do {                                                                        \
    cudaError_t _e = (expr);                                                  \
    if (_e != cudaSuccess) {                                                  \
      ::om::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));    \
      return OM_ERR_CUDA;                                                     \
    }                                                                         \
  } while (0)

#define OM_TRY(expr)                                                          \
  do {                                                                        \
    om_status _s = (expr);                                                    \
    if (_s != OM_OK) return _s;                                               \
  } while (0)

// Which copy of an array holds the newest data.  Same three states as the
// generated CUDA container's host/device mirror
// (Language/Paraiso/Generator/PlanTrans.hs:724-728): reading on the host
// brings the host copy up to date; a non-const host access marks the host
// newer; a kernel launch brings the device copy up to date first.
enum class Newer { kBoth, kHost, kDevice };

struct Array {
  std::string name;
  int elem_size = 4;      // bytes per element
  size_t count = 0;       // memory-sized element count (margins included)
  void *dev[2] = {nullptr, nullptr};  // double buffer: [cur], [1-cur]
  int cur = 0;
  void *host = nullptr;   // pinned host mirror, allocated on first access
  Newer newer = Newer::kBoth;
  void *d() const { return dev[cur]; }
  void *d_next() const { return dev[1 - cur]; }
  void swap() { cur = 1 - cur; }
};

enum ScalarType { kInt = 0, kDouble = 1, kFloat = 2 };

struct Scalar {
  std::string name;
  ScalarType type;
  size_t offset;  // byte offset inside the host/device scalar blocks
};

struct Handle;
typedef om_status (*KernelFn)(Handle *, int n);

// Hooks a kind (Life, Hydro) gives the generic runtime.
struct KindOps {
  // host-side state that decides which launches a run issues; a captured
  // CUDA graph is replayed only while it matches
  uint64_t (*state_key)(Handle *) = nullptr;
  // apply the host-side effects of a run whose graph was replayed
  void (*after_replay)(Handle *, int kernel_id, int n) = nullptr;
  // put back the host-side state described by a state_key (capturing a run
  // executes its host bookkeeping once; the replay applies it again)
  void (*restore_key)(Handle *, uint64_t key) = nullptr;
  // an array's contents were replaced from outside (host mirror or copy)
  void (*array_written)(Handle *, Array *) = nullptr;
  // allocate whatever a run of n steps needs, before any stream capture
  om_status (*reserve)(Handle *, int kernel_id, int n) = nullptr;
  // false when a kernel synchronises with the host mid-run (no graph capture)
  bool (*graph_ok)(Handle *, int kernel_id) = nullptr;
  // after a run has completed and its scalars are back on the host: report
  // a failure that kernels recorded in the scalar block
  om_status (*after_run)(Handle *) = nullptr;
  // derive host-side scalar fields from the user-visible ones right before
  // the scalar block is uploaded
  void (*before_upload)(Handle *) = nullptr;
  // host-side state a checkpoint carries besides the statics (bytes written
  // into out, at most cap; returns the size), and its restoration
  size_t (*save_state)(Handle *, void *out, size_t cap) = nullptr;
  void (*load_state)(Handle *, const void *in, size_t n) = nullptr;
};

struct Kernel {
  std::string name;
  KernelFn fn;
};

// Device time of individual launches, bracketed by CUDA events on the
// handle's stream while profiling is enabled (never inside graph capture).
struct ProfPending {
  std::string name;
  cudaEvent_t e0, e1;
  double units;
};
struct ProfAgg {
  long launches = 0;
  double ms = 0, units = 0;
};

// Scalar block shared by host (pinned mirror) and device.  Layout is fixed
// per OM kind; see life.cu / hydro.cu.
struct Handle {
  int kind = 0;
  int ndim = 2;
  int size[2] = {0, 0};
  int lower_margin[2] = {0, 0};
  int upper_margin[2] = {0, 0};
  int cyclic = 1;
  om_config cfg{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<Array> arrays;
  std::vector<Scalar> scalars;
  std::vector<Kernel> kernels;
  size_t scalar_bytes = 0;
  void *h_scalars = nullptr;  // pinned
  void *d_scalars = nullptr;
  bool scalars_dirty = true;  // host scalar block changed since last upload
  void *impl = nullptr;       // kind-specific state
  void (*impl_free)(Handle *) = nullptr;
  KindOps ops;
  int launches = 0;           // kernel launches issued by the current run
  int current_kernel = -1;    // index of the kernel whose function is running
  bool profiling = false;
  bool capturing = false;
  std::vector<ProfPending> prof_pending;
  std::map<std::string, ProfAgg> prof;

  size_t memory_size(int ax) const {
    return (size_t)size[ax] + lower_margin[ax] + upper_margin[ax];
  }
  size_t memory_size_total() const { return memory_size(0) * memory_size(1); }
  Array *find_array(const char *n);
  Scalar *find_scalar(const char *n);
};

// Create a handle: stream, then `setup` (which adds arrays, scalars and
// kernels), then the scalar block.  Used by om_create and om_create_graph.
om_status create_handle(int kind, const int sizes[2], const om_config &cfg,
                        om_status (*setup)(Handle *, void *), void *ctx, om_handle *out);

// Allocate an OM array (double-buffered device storage, zero-filled).
om_status alloc_array(Handle *h, const char *name, int elem_size);
// Device copy up to date (uploads the host mirror if the host is newer).
om_status bring_device(Handle *h, Array &a);
// OM_FAIL_ALLOC_AFTER=N (environment): every allocation request after the
// first N reports failure (tests of the out-of-memory paths)
bool injected_alloc_failure();
// Host copy up to date (downloads if the device is newer).
om_status bring_host(Handle *h, Array &a);
// Upload the host scalar block before a kernel; download it after.
om_status upload_scalars(Handle *h);
om_status download_scalars(Handle *h);

// Kind-specific constructors (life.cu, hydro.cu).
om_status life_setup(Handle *h);
om_status hydro_setup(Handle *h);

// Bracket one launch with events when profiling: call prof_begin before
// the launch and prof_end after it.
cudaEvent_t prof_begin(Handle *h);
void prof_end(Handle *h, cudaEvent_t e0, const char *name, double units);
// Fold finished event pairs into h->prof (called after a stream sync).
void prof_collect(Handle *h);

// SM count of the handle's device (cached).
int sm_count(int device);

// The runtime handle behind an opaque om_handle (om_abi.cu).
Handle *handle_of(om_handle H);

// splitmix64 finaliser; the synthetic-input hash is
// mix64(mix64(seed) + index * 0x9E3779B97F4A7C15).
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

}  // namespace om
