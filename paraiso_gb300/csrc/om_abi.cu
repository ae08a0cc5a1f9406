// om_abi.cu -- the C ABI of include/om_gb300.h: handles, the host/device
// mirror of OM arrays, scalar blocks, kernel dispatch and CUDA-graph replay
// of multi-step runs.
//
// Reference interface being replaced: the class Paraiso's generator prints
// per OM (Language/Paraiso/Generator/PlanTrans.hs:51-277) together with its
// host/device container (PlanTrans.hs:724-728).
#include <cuda_runtime.h>
#include <cstdlib>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "om_internal.cuh"

namespace om {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int sm_count(int device) {
  static std::mutex mu;
  static std::map<int, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(device);
  if (it != cache.end()) return it->second;
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0) n = 148;
  cache[device] = n;
  return n;
}

Array *Handle::find_array(const char *n) {
  for (auto &a : arrays)
    if (a.name == n) return &a;
  return nullptr;
}

Scalar *Handle::find_scalar(const char *n) {
  for (auto &s : scalars)
    if (s.name == n) return &s;
  return nullptr;
}

// Fault injection for tests, on the host: with OM_FAIL_ALLOC_AFTER=n in the
// environment, array allocations after the first n (counted from when the
// variable took its current value) report failure without calling the
// allocator, so every caller's OM_ERR_NOMEM path can be exercised.
bool injected_alloc_failure() {
  static std::mutex mu;
  static std::string seen;
  static long count = 0;
  const char *e = std::getenv("OM_FAIL_ALLOC_AFTER");
  std::lock_guard<std::mutex> lock(mu);
  const std::string now = e ? e : "";
  if (now != seen) {
    seen = now;
    count = 0;
  }
  if (now.empty()) return false;
  return count++ >= std::atol(now.c_str());
}

om_status alloc_array(Handle *h, const char *name, int elem_size) {
  Array a;
  a.name = name;
  a.elem_size = elem_size;
  a.count = h->memory_size_total();
  const size_t bytes = a.count * (size_t)elem_size;
  if (injected_alloc_failure()) {
    set_error(std::string("cudaMalloc failed for array ") + name + " (injected by "
              "OM_FAIL_ALLOC_AFTER)");
    return OM_ERR_NOMEM;
  }
  for (int b = 0; b < 2; ++b) {
    if (cudaMalloc(&a.dev[b], bytes) != cudaSuccess) {
      cudaGetLastError();
      if (b == 1) cudaFree(a.dev[0]);
      set_error(std::string("cudaMalloc failed for array ") + name + " (" +
                std::to_string(bytes) + " bytes)");
      return OM_ERR_NOMEM;
    }
    OM_CUDA_CHECK(cudaMemsetAsync(a.dev[b], 0, bytes, h->stream));
  }
  h->arrays.push_back(a);
  return OM_OK;
}

static om_status ensure_host(Handle *h, Array &a) {
  if (a.host) return OM_OK;
  const size_t bytes = a.count * (size_t)a.elem_size;
  if (cudaMallocHost(&a.host, bytes) != cudaSuccess) {
    cudaGetLastError();
    a.host = nullptr;
    set_error("cudaMallocHost failed for the host mirror of " + a.name);
    return OM_ERR_NOMEM;
  }
  // the device copy is authoritative until the host mirror is first read
  if (a.newer == Newer::kBoth) a.newer = Newer::kDevice;
  (void)h;
  return OM_OK;
}

om_status bring_device(Handle *h, Array &a) {
  if (a.newer == Newer::kHost) {
    OM_CUDA_CHECK(cudaMemcpyAsync(a.d(), a.host, a.count * (size_t)a.elem_size,
                                  cudaMemcpyHostToDevice, h->stream));
    a.newer = Newer::kBoth;
  }
  return OM_OK;
}

om_status bring_host(Handle *h, Array &a) {
  OM_TRY(ensure_host(h, a));
  if (a.newer == Newer::kDevice) {
    OM_CUDA_CHECK(cudaMemcpyAsync(a.host, a.d(), a.count * (size_t)a.elem_size,
                                  cudaMemcpyDeviceToHost, h->stream));
    OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
    a.newer = Newer::kBoth;
  }
  return OM_OK;
}

om_status upload_scalars(Handle *h) {
  if (!h->scalar_bytes) return OM_OK;
  if (h->ops.before_upload) h->ops.before_upload(h);
  OM_CUDA_CHECK(cudaMemcpyAsync(h->d_scalars, h->h_scalars, h->scalar_bytes,
                                cudaMemcpyHostToDevice, h->stream));
  return OM_OK;
}

om_status download_scalars(Handle *h) {
  if (!h->scalar_bytes) return OM_OK;
  OM_CUDA_CHECK(cudaMemcpyAsync(h->h_scalars, h->d_scalars, h->scalar_bytes,
                                cudaMemcpyDeviceToHost, h->stream));
  return OM_OK;
}

cudaEvent_t prof_begin(Handle *h) {
  if (!h->profiling || h->capturing) return nullptr;
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  cudaEventRecord(e, h->stream);
  return e;
}

void prof_end(Handle *h, cudaEvent_t e0, const char *name, double units) {
  if (!e0) return;
  cudaEvent_t e1 = nullptr;
  if (cudaEventCreate(&e1) != cudaSuccess) { cudaGetLastError(); cudaEventDestroy(e0); return; }
  cudaEventRecord(e1, h->stream);
  h->prof_pending.push_back({name, e0, e1, units});
}

void prof_collect(Handle *h) {
  for (auto &p : h->prof_pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.e0, p.e1) == cudaSuccess) {
      ProfAgg &a = h->prof[p.name];
      a.launches += 1;
      a.ms += ms;
      a.units += p.units;
    } else {
      cudaGetLastError();
    }
    cudaEventDestroy(p.e0);
    cudaEventDestroy(p.e1);
  }
  h->prof_pending.clear();
}

}  // namespace om

using namespace om;

struct om_handle_s {
  Handle h;
  // CUDA graphs of multi-step runs, keyed by (kernel, n, buffer parity)
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    std::vector<int> end_cur;
    int launches = 0;
  };
  std::map<std::tuple<int, int, uint64_t>, GraphEntry> graphs;
  int last_launches = 0;
};

namespace om {
Handle *handle_of(om_handle H) { return H ? &H->h : nullptr; }
}  // namespace om

namespace om {

om_status create_handle(int kind, const int sizes[2], const om_config &cfg,
                        om_status (*setup)(Handle *, void *), void *ctx, om_handle *out) {
  om_config c = cfg;
  *out = nullptr;
  if (c.boundary != OM_BOUNDARY_CYCLIC && c.boundary != OM_BOUNDARY_OPEN) {
    set_error("om_create: boundary must be cyclic (0) or open (1)");
    return OM_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("om_create: no CUDA device available");
    return OM_ERR_CUDA;
  }
  if (c.device < 0 || c.device >= ndev) {
    set_error("om_create: device ordinal out of range");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(c.device));
  om_handle H = new om_handle_s();
  Handle *h = &H->h;
  h->kind = kind;
  h->ndim = 2;
  h->size[0] = sizes[0];
  h->size[1] = sizes[1];
  h->cyclic = c.boundary == OM_BOUNDARY_CYCLIC;
  h->cfg = c;
  h->device = c.device;
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete H;
    set_error("om_create: cudaStreamCreate failed");
    return OM_ERR_CUDA;
  }
  h->own_stream = true;
  om_status s = setup(h, ctx);
  if (s == OM_OK && h->scalar_bytes) {
    if (cudaMallocHost(&h->h_scalars, h->scalar_bytes) != cudaSuccess ||
        cudaMalloc(&h->d_scalars, h->scalar_bytes) != cudaSuccess) {
      cudaGetLastError();
      set_error("om_create: scalar block allocation failed");
      s = OM_ERR_NOMEM;
    } else {
      std::memset(h->h_scalars, 0, h->scalar_bytes);
    }
  }
  if (s == OM_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) {
    set_error(std::string("om_create: ") + cudaGetErrorString(cudaGetLastError()));
    s = OM_ERR_CUDA;
  }
  if (s != OM_OK) {
    std::string keep = g_last_error;
    om_destroy(H);
    set_error(keep);
    return s;
  }
  *out = H;
  return OM_OK;
}

}  // namespace om

extern "C" {

void om_config_default(om_config *cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->boundary = OM_BOUNDARY_CYCLIC;
  cfg->precision = 32;
  cfg->gamma = 5.0 / 3.0;
  cfg->device = 0;
  cfg->use_graph = 1;
}

const char *om_last_error(void) { return g_last_error.c_str(); }

const char *om_version(void) { return "paraiso_gb300 0.1 (sm_103a)"; }

om_status om_create(int kind, int ndim, const int *sizes, const om_config *cfg,
                    om_handle *out) {
  if (!out) { set_error("om_create: out is NULL"); return OM_ERR_ARG; }
  *out = nullptr;
  if (kind != OM_KIND_LIFE && kind != OM_KIND_HYDRO) {
    set_error("om_create: unknown kind " + std::to_string(kind));
    return OM_ERR_ARG;
  }
  if (ndim != 2 || !sizes) {
    set_error("om_create: only 2-dimensional orthotopes are supported");
    return OM_ERR_ARG;
  }
  if (sizes[0] <= 0 || sizes[1] <= 0 || sizes[0] > (1 << 20) || sizes[1] > (1 << 20)) {
    set_error("om_create: sizes must be in [1, 2^20]");
    return OM_ERR_ARG;
  }
  om_config c;
  if (cfg) c = *cfg; else om_config_default(&c);
  struct Kind {
    static om_status setup(Handle *h, void *) {
      return h->kind == OM_KIND_LIFE ? life_setup(h) : hydro_setup(h);
    }
  };
  return create_handle(kind, sizes, c, Kind::setup, nullptr, out);
}

om_status om_destroy(om_handle H) {
  if (!H) return OM_OK;
  Handle *h = &H->h;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto &kv : H->graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  if (h->impl_free) h->impl_free(h);
  for (auto &a : h->arrays) {
    cudaFree(a.dev[0]);
    cudaFree(a.dev[1]);
    if (a.host) cudaFreeHost(a.host);
  }
  if (h->h_scalars) cudaFreeHost(h->h_scalars);
  if (h->d_scalars) cudaFree(h->d_scalars);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  cudaGetLastError();
  delete H;
  return OM_OK;
}

static om_status axis_query(om_handle H, int axis, int *out, int which) {
  if (!H || !out) { set_error("null handle or output"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  if (axis < -1 || axis >= h->ndim) { set_error("axis out of range"); return OM_ERR_ARG; }
  auto one = [&](int ax) -> long long {
    switch (which) {
      case 0: return h->size[ax];
      case 1: return (long long)h->memory_size(ax);
      case 2: return h->lower_margin[ax];
      default: return h->upper_margin[ax];
    }
  };
  long long v;
  if (axis >= 0) v = one(axis);
  else v = one(0) * one(1);
  if (v > 0x7fffffffLL) { set_error("size exceeds int range"); return OM_ERR_ARG; }
  *out = (int)v;
  return OM_OK;
}

om_status om_size(om_handle h, int axis, int *out) { return axis_query(h, axis, out, 0); }
om_status om_memory_size(om_handle h, int axis, int *out) { return axis_query(h, axis, out, 1); }
om_status om_lower_margin(om_handle h, int axis, int *out) { return axis_query(h, axis, out, 2); }
om_status om_upper_margin(om_handle h, int axis, int *out) { return axis_query(h, axis, out, 3); }

om_status om_kernel_id(om_handle H, const char *name, int *id) {
  if (!H || !name || !id) { set_error("om_kernel_id: null argument"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  for (size_t i = 0; i < h->kernels.size(); ++i)
    if (h->kernels[i].name == name) { *id = (int)i; return OM_OK; }
  set_error(std::string("om_kernel_id: no kernel named ") + name);
  return OM_ERR_ARG;
}

static om_status prepare(Handle *h) {
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  for (auto &a : h->arrays) {
    if (a.newer == Newer::kHost) {
      OM_TRY(bring_device(h, a));
      if (h->ops.array_written) h->ops.array_written(h, &a);
    }
    // from here on the kernel owns the newest copy
    if (a.host) a.newer = Newer::kBoth;
  }
  OM_TRY(upload_scalars(h));
  return OM_OK;
}

static om_status finish(Handle *h) {
  OM_TRY(download_scalars(h));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  prof_collect(h);
  for (auto &a : h->arrays)
    if (a.newer == Newer::kBoth && a.host) a.newer = Newer::kDevice;
  if (h->ops.after_run) OM_TRY(h->ops.after_run(h));
  return OM_OK;
}

static om_status run_plain(om_handle H, int kernel_id, int n) {
  Handle *h = &H->h;
  h->launches = 0;
  h->current_kernel = kernel_id;
  om_status s = h->kernels[kernel_id].fn(h, n);
  H->last_launches = h->launches;
  return s;
}

om_status om_run_n(om_handle H, int kernel_id, int n) {
  if (!H) { set_error("om_run: null handle"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  if (kernel_id < 0 || kernel_id >= (int)h->kernels.size()) {
    set_error("om_run: kernel id out of range");
    return OM_ERR_ARG;
  }
  if (n < 0) { set_error("om_run_n: n < 0"); return OM_ERR_ARG; }
  if (n == 0) return OM_OK;
  if (h->ops.reserve) OM_TRY(h->ops.reserve(h, kernel_id, n));
  OM_TRY(prepare(h));
  const bool graph_ok = h->cfg.use_graph && n > 1 && !h->profiling &&
                        (!h->ops.graph_ok || h->ops.graph_ok(h, kernel_id));
  if (!graph_ok) {
    OM_TRY(run_plain(H, kernel_id, n));
    return finish(h);
  }
  uint64_t mask = 0;
  for (size_t i = 0; i < h->arrays.size(); ++i)
    mask |= (uint64_t)h->arrays[i].cur << i;
  const uint64_t skey = h->ops.state_key ? h->ops.state_key(h) : 0;
  const uint64_t key2 = mask ^ (skey << 32);
  auto key = std::make_tuple(kernel_id, n, key2);
  auto it = H->graphs.find(key);
  if (it == H->graphs.end()) {
    om_handle_s::GraphEntry e;
    cudaGraph_t g = nullptr;
    OM_CUDA_CHECK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    h->capturing = true;
    om_status s = run_plain(H, kernel_id, n);
    h->capturing = false;
    cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (s != OM_OK) { if (g) cudaGraphDestroy(g); return s; }
    if (ce != cudaSuccess) {
      set_error(std::string("graph capture: ") + cudaGetErrorString(ce));
      return OM_ERR_CUDA;
    }
    ce = cudaGraphInstantiate(&e.exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      set_error(std::string("graph instantiate: ") + cudaGetErrorString(ce));
      return OM_ERR_CUDA;
    }
    for (auto &a : h->arrays) e.end_cur.push_back(a.cur);
    e.launches = H->last_launches;
    // the capture changed the host-side state; roll it back so the
    // replay below applies it once
    for (size_t i = 0; i < h->arrays.size(); ++i)
      h->arrays[i].cur = (int)((mask >> i) & 1);
    if (h->ops.restore_key) h->ops.restore_key(h, skey);
    it = H->graphs.emplace(key, e).first;
  }
  OM_CUDA_CHECK(cudaGraphLaunch(it->second.exec, h->stream));
  for (size_t i = 0; i < h->arrays.size(); ++i) h->arrays[i].cur = it->second.end_cur[i];
  H->last_launches = it->second.launches;
  if (h->ops.after_replay) h->ops.after_replay(h, kernel_id, n);
  return finish(h);
}

om_status om_run(om_handle H, int kernel_id) {
  if (!H) { set_error("om_run: null handle"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  if (kernel_id < 0 || kernel_id >= (int)h->kernels.size()) {
    set_error("om_run: kernel id out of range");
    return OM_ERR_ARG;
  }
  if (h->ops.reserve) OM_TRY(h->ops.reserve(h, kernel_id, 1));
  OM_TRY(prepare(h));
  OM_TRY(run_plain(H, kernel_id, 1));
  return finish(h);
}

om_status om_scalar_ptr(om_handle H, const char *name, void **ptr, int *type) {
  if (!H || !name || !ptr) { set_error("om_scalar_ptr: null argument"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  Scalar *s = h->find_scalar(name);
  if (!s) { set_error(std::string("no scalar named ") + name); return OM_ERR_ARG; }
  *ptr = (char *)h->h_scalars + s->offset;
  if (type) *type = s->type;
  return OM_OK;
}

om_status om_array_host(om_handle H, const char *name, void **ptr, size_t *count,
                        int *elem_size) {
  if (!H || !name || !ptr) { set_error("om_array_host: null argument"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  Array *a = h->find_array(name);
  if (!a) { set_error(std::string("no array named ") + name); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  OM_TRY(bring_host(h, *a));
  a->newer = Newer::kHost;
  *ptr = a->host;
  if (count) *count = a->count;
  if (elem_size) *elem_size = a->elem_size;
  return OM_OK;
}

om_status om_array_host_const(om_handle H, const char *name, const void **ptr,
                              size_t *count, int *elem_size) {
  if (!H || !name || !ptr) { set_error("om_array_host_const: null argument"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  Array *a = h->find_array(name);
  if (!a) { set_error(std::string("no array named ") + name); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  OM_TRY(bring_host(h, *a));
  *ptr = a->host;
  if (count) *count = a->count;
  if (elem_size) *elem_size = a->elem_size;
  return OM_OK;
}

om_status om_array_device(om_handle H, const char *name, void **dptr) {
  if (!H || !name || !dptr) { set_error("om_array_device: null argument"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  Array *a = h->find_array(name);
  if (!a) { set_error(std::string("no array named ") + name); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  OM_TRY(bring_device(h, *a));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  if (a->host) a->newer = Newer::kDevice;
  *dptr = a->d();
  return OM_OK;
}

om_status om_array_read(om_handle H, const char *name, void *dst, size_t bytes) {
  if (!H || !name || !dst) { set_error("om_array_read: null argument"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  Array *a = h->find_array(name);
  if (!a) { set_error(std::string("no array named ") + name); return OM_ERR_ARG; }
  if (bytes != a->count * (size_t)a->elem_size) {
    set_error("om_array_read: byte count must equal the memory-sized array");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  if (a->newer == Newer::kHost) {
    std::memcpy(dst, a->host, bytes);  // host copy is authoritative
    return OM_OK;
  }
  OM_CUDA_CHECK(cudaMemcpyAsync(dst, a->d(), bytes, cudaMemcpyDefault, h->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  return OM_OK;
}

om_status om_array_write(om_handle H, const char *name, const void *src, size_t bytes) {
  if (!H || !name || !src) { set_error("om_array_write: null argument"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  Array *a = h->find_array(name);
  if (!a) { set_error(std::string("no array named ") + name); return OM_ERR_ARG; }
  if (bytes != a->count * (size_t)a->elem_size) {
    set_error("om_array_write: byte count must equal the memory-sized array");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  OM_CUDA_CHECK(cudaMemcpyAsync(a->d(), src, bytes, cudaMemcpyDefault, h->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  if (a->host) a->newer = Newer::kDevice;
  else a->newer = Newer::kBoth;
  // the written contents are arbitrary: let the kind re-validate its state
  if (h->ops.array_written) h->ops.array_written(h, a);
  return OM_OK;
}

om_status om_time_run(om_handle H, int kernel_id, int n, float *ms) {
  if (!H || !ms) { set_error("om_time_run: null argument"); return OM_ERR_ARG; }
  Handle *h = &H->h;
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  cudaEvent_t e0, e1;
  OM_CUDA_CHECK(cudaEventCreate(&e0));
  OM_CUDA_CHECK(cudaEventCreate(&e1));
  if (kernel_id < 0 || kernel_id >= (int)h->kernels.size() || n < 1) {
    set_error("om_time_run: bad kernel id or n");
    return OM_ERR_ARG;
  }
  if (h->ops.reserve) OM_TRY(h->ops.reserve(h, kernel_id, n));
  OM_TRY(prepare(h));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  OM_CUDA_CHECK(cudaEventRecord(e0, h->stream));
  om_status s = run_plain(H, kernel_id, n);
  OM_CUDA_CHECK(cudaEventRecord(e1, h->stream));
  OM_CUDA_CHECK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != OM_OK) return s;
  return finish(h);
}

om_status om_profile_enable(om_handle H, int enable) {
  if (!H) { set_error("null handle"); return OM_ERR_ARG; }
  H->h.profiling = enable != 0;
  if (!enable) H->h.prof.clear();
  return OM_OK;
}

om_status om_profile_query(om_handle H, const char *kernel, long *launches,
                           double *total_ms, double *total_units) {
  if (!H || !kernel) { set_error("null argument"); return OM_ERR_ARG; }
  auto it = H->h.prof.find(kernel);
  if (it == H->h.prof.end()) {
    if (launches) *launches = 0;
    if (total_ms) *total_ms = 0;
    if (total_units) *total_units = 0;
    return OM_OK;
  }
  if (launches) *launches = it->second.launches;
  if (total_ms) *total_ms = it->second.ms;
  if (total_units) *total_units = it->second.units;
  return OM_OK;
}

om_status om_last_launch_count(om_handle H, int *launches) {
  if (!H || !launches) { set_error("null argument"); return OM_ERR_ARG; }
  *launches = H->last_launches;
  return OM_OK;
}

}  // extern "C"
