// snapshot.cu -- checkpoint/restart of a handle's statics and the text
// snapshots of the Hydro driver.  The generated class keeps its statics as
// public containers and scalars (Language/Paraiso/Generator/PlanTrans.hs:
// 117-157) and has no I/O of its own; its drivers write text snapshots
// through the accessors (examples/Hydro/main-kh.cpp:17-31).  Host code only.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "om_internal.cuh"

namespace om {
namespace {

const char kMagic[8] = {'O', 'M', 'G', 'B', '3', '0', '0', '\0'};
const uint32_t kVersion = 1;

struct Writer {
  std::ofstream f;
  void raw(const void *p, size_t n) { f.write(static_cast<const char *>(p), (std::streamsize)n); }
  template <class T> void put(T v) { raw(&v, sizeof v); }
  void str(const std::string &s) {
    put<uint32_t>((uint32_t)s.size());
    raw(s.data(), s.size());
  }
};

struct Reader {
  std::ifstream f;
  bool ok = true;
  void raw(void *p, size_t n) {
    if (!f.read(static_cast<char *>(p), (std::streamsize)n)) ok = false;
  }
  template <class T> T get() {
    T v{};
    raw(&v, sizeof v);
    return v;
  }
  std::string str() {
    const uint32_t n = get<uint32_t>();
    if (!ok || n > 4096) { ok = false; return std::string(); }
    std::string s(n, '\0');
    raw(&s[0], n);
    return s;
  }
};

// layout of a handle as written in the header
void write_layout(Writer &w, const Handle *h) {
  w.put<int32_t>(h->kind);
  for (int d = 0; d < 2; ++d) {
    w.put<int32_t>(h->size[d]);
    w.put<int32_t>(h->lower_margin[d]);
    w.put<int32_t>(h->upper_margin[d]);
  }
  w.put<uint64_t>(h->scalar_bytes);
  w.put<uint32_t>((uint32_t)h->scalars.size());
  for (const Scalar &s : h->scalars) {
    w.str(s.name);
    w.put<int32_t>((int32_t)s.type);
    w.put<uint64_t>(s.offset);
  }
  w.put<uint32_t>((uint32_t)h->arrays.size());
  for (const Array &a : h->arrays) {
    w.str(a.name);
    w.put<int32_t>(a.elem_size);
    w.put<uint64_t>(a.count);
  }
}

bool layout_matches(Reader &r, const Handle *h, std::string *why) {
  if (r.get<int32_t>() != h->kind) { *why = "kind differs"; return false; }
  for (int d = 0; d < 2; ++d) {
    const int32_t n = r.get<int32_t>(), lo = r.get<int32_t>(), hi = r.get<int32_t>();
    if (n != h->size[d] || lo != h->lower_margin[d] || hi != h->upper_margin[d]) {
      *why = "mesh size or margins differ on axis " + std::to_string(d);
      return false;
    }
  }
  if (r.get<uint64_t>() != h->scalar_bytes) { *why = "scalar block differs"; return false; }
  const uint32_t ns = r.get<uint32_t>();
  if (ns != h->scalars.size()) { *why = "number of scalars differs"; return false; }
  for (const Scalar &s : h->scalars) {
    const std::string name = r.str();
    const int32_t type = r.get<int32_t>();
    const uint64_t off = r.get<uint64_t>();
    if (name != s.name || type != (int32_t)s.type || off != s.offset) {
      *why = "scalar " + s.name + " differs";
      return false;
    }
  }
  const uint32_t na = r.get<uint32_t>();
  if (na != h->arrays.size()) { *why = "number of arrays differs"; return false; }
  for (const Array &a : h->arrays) {
    const std::string name = r.str();
    const int32_t es = r.get<int32_t>();
    const uint64_t n = r.get<uint64_t>();
    if (name != a.name || es != a.elem_size || n != a.count) {
      *why = "array " + a.name + " differs";
      return false;
    }
  }
  if (!r.ok) { *why = "truncated header"; return false; }
  return true;
}

}  // namespace
}  // namespace om

using namespace om;

extern "C" om_status om_save(om_handle H, const char *path) {
  Handle *h = handle_of(H);
  if (!h || !path) { set_error("om_save: null argument"); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  Writer w;
  w.f.open(path, std::ios::binary | std::ios::trunc);
  if (!w.f) { set_error(std::string("om_save: cannot open ") + path); return OM_ERR_ARG; }
  w.raw(kMagic, sizeof kMagic);
  w.put<uint32_t>(kVersion);
  write_layout(w, h);
  w.raw(h->h_scalars, h->scalar_bytes);
  unsigned char kind_state[256];
  const size_t ks = h->ops.save_state ? h->ops.save_state(h, kind_state, sizeof kind_state) : 0;
  w.put<uint32_t>((uint32_t)ks);
  w.raw(kind_state, ks);
  std::vector<char> buf;
  for (Array &a : h->arrays) {
    const size_t bytes = a.count * (size_t)a.elem_size;
    buf.resize(bytes);
    OM_TRY(om_array_read(H, a.name.c_str(), buf.data(), bytes));
    w.raw(buf.data(), bytes);
  }
  w.f.flush();
  if (!w.f) { set_error(std::string("om_save: write failed: ") + path); return OM_ERR_ARG; }
  return OM_OK;
}

extern "C" om_status om_load(om_handle H, const char *path) {
  Handle *h = handle_of(H);
  if (!h || !path) { set_error("om_load: null argument"); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  Reader r;
  r.f.open(path, std::ios::binary);
  if (!r.f) { set_error(std::string("om_load: cannot open ") + path); return OM_ERR_ARG; }
  char magic[8];
  r.raw(magic, sizeof magic);
  if (!r.ok || std::memcmp(magic, kMagic, sizeof magic) != 0 || r.get<uint32_t>() != kVersion) {
    set_error(std::string("om_load: not a checkpoint of this runtime: ") + path);
    return OM_ERR_ARG;
  }
  std::string why;
  if (!layout_matches(r, h, &why)) {
    set_error("om_load: checkpoint does not fit this handle: " + why);
    return OM_ERR_ARG;
  }
  std::vector<char> scal(h->scalar_bytes);
  r.raw(scal.data(), scal.size());
  const uint32_t ks = r.get<uint32_t>();
  if (!r.ok || ks > 256) { set_error("om_load: corrupt checkpoint"); return OM_ERR_ARG; }
  std::vector<char> kind_state(ks);
  r.raw(kind_state.data(), ks);
  std::vector<std::vector<char>> data(h->arrays.size());
  for (size_t i = 0; i < h->arrays.size(); ++i) {
    data[i].resize(h->arrays[i].count * (size_t)h->arrays[i].elem_size);
    r.raw(data[i].data(), data[i].size());
  }
  if (!r.ok) { set_error("om_load: truncated checkpoint"); return OM_ERR_ARG; }
  // arrays through om_array_write: every kind drops what it cached about them
  for (size_t i = 0; i < h->arrays.size(); ++i)
    OM_TRY(om_array_write(H, h->arrays[i].name.c_str(), data[i].data(), data[i].size()));
  std::memcpy(h->h_scalars, scal.data(), scal.size());
  h->scalars_dirty = true;
  if (h->ops.load_state) h->ops.load_state(h, kind_state.data(), kind_state.size());
  return OM_OK;
}

// The text snapshot of examples/Hydro/main-kh.cpp:17-31 (antiAlias 1): per
// interior cell "x y density velocity0 velocity1 pressure" with x = dR0
// (ix + 0.5), y = dR1 (iy + 0.5), a blank line after each row, written with
// the default std::ostream formatting that main-kh.cpp uses.
extern "C" om_status om_hydro_write_snapshot(om_handle H, const char *path) {
  Handle *h = handle_of(H);
  if (!h || !path || h->kind != OM_KIND_HYDRO) {
    set_error("om_hydro_write_snapshot: needs a Hydro handle and a path");
    return OM_ERR_ARG;
  }
  const char *names[4] = {"density", "velocity0", "velocity1", "pressure"};
  std::vector<std::vector<char>> f(4);
  int es = 0;
  for (int k = 0; k < 4; ++k) {
    const Array *a = h->find_array(names[k]);
    es = a->elem_size;
    f[k].resize(a->count * (size_t)a->elem_size);
    OM_TRY(om_array_read(H, names[k], f[k].data(), f[k].size()));
  }
  double dR0 = 0, dR1 = 0;
  {
    void *p;
    int t;
    OM_TRY(om_scalar_ptr(H, "dR0", &p, &t));
    dR0 = *static_cast<double *>(p);
    OM_TRY(om_scalar_ptr(H, "dR1", &p, &t));
    dR1 = *static_cast<double *>(p);
  }
  std::ofstream ofs(path);
  if (!ofs) { set_error(std::string("om_hydro_write_snapshot: cannot open ") + path); return OM_ERR_ARG; }
  const int W = h->size[0], Hn = h->size[1];
  const size_t ms0 = h->memory_size(0);
  auto at = [&](int k, size_t i) -> double {
    if (es == 8) {
      double v;
      std::memcpy(&v, f[k].data() + 8 * i, 8);
      return v;
    }
    float v;
    std::memcpy(&v, f[k].data() + 4 * i, 4);
    return v;
  };
  for (int iy = 0; iy < Hn; ++iy) {
    for (int ix = 0; ix < W; ++ix) {
      const size_t i = ms0 * (iy + h->lower_margin[1]) + ix + h->lower_margin[0];
      const double x = dR0 * (ix + 0.5), y = dR1 * (iy + 0.5);
      ofs << x << " " << y << " ";
      if (es == 8)
        ofs << at(0, i) << " " << at(1, i) << " " << at(2, i) << " " << at(3, i) << std::endl;
      else
        ofs << (float)at(0, i) << " " << (float)at(1, i) << " " << (float)at(2, i) << " "
            << (float)at(3, i) << std::endl;
    }
    ofs << std::endl;
  }
  if (!ofs) { set_error(std::string("om_hydro_write_snapshot: write failed: ") + path); return OM_ERR_ARG; }
  return OM_OK;
}
