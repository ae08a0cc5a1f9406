// om_shim.hpp -- helpers shared by the header-only shims Life.hpp and
// Hydro.hpp, which rebuild the class Paraiso's generator prints
// (Language/Paraiso/Generator/PlanTrans.hs:51-277) on top of the C ABI in
// om_gb300.h.  Errors, which the generated class never reports, surface as
// std::runtime_error carrying om_last_error().
#pragma once

#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "om_gb300.h"

namespace om_shim {

inline void check(om_status s, const char *what) {
  if (s != OM_OK) throw std::runtime_error(std::string(what) + ": " + om_last_error());
}

// The generated Array container seen from the host: element access marks the
// host copy newer, like thrust_vector::operator[] (PlanTrans.hs:724-728).
template <class T> class host_array {
 public:
  host_array(om_handle h, const char *name) : h_(h), name_(name) {}
  T &operator[](std::size_t i) { return data()[i]; }
  const T &operator[](std::size_t i) const { return cdata()[i]; }
  std::size_t size() const {
    const void *p;
    std::size_t n;
    int es;
    check(om_array_host_const(h_, name_, &p, &n, &es), name_);
    return n;
  }
  T *data() {
    void *p;
    check(om_array_host(h_, name_, &p, nullptr, nullptr), name_);
    return static_cast<T *>(p);
  }
  const T *cdata() const {
    const void *p;
    check(om_array_host_const(h_, name_, &p, nullptr, nullptr), name_);
    return static_cast<const T *>(p);
  }
  T *begin() { return data(); }
  T *end() { return data() + size(); }

 private:
  om_handle h_;
  const char *name_;
};

// The earlier generator's public static members (static_<i>_<name>, the
// i-th static of the OM; examples-old/*/dist/*.hpp): a Scalar reads and
// writes through the handle's host scalar block, an Array indexes the host
// copy and converts to any container built from an iterator pair (the
// drivers copy it into std::vector or thrust::host_vector).
template <class T> class scalar_member {
 public:
  scalar_member(om_handle h, const char *name) : h_(h), name_(name) {}
  operator T() const { return *ptr(); }
  scalar_member &operator=(T v) {
    *ptr() = v;
    return *this;
  }
  scalar_member &operator=(const scalar_member &o) { return *this = (T)o; }

 private:
  T *ptr() const {
    void *p;
    check(om_scalar_ptr(h_, name_, &p, nullptr), name_);
    return static_cast<T *>(p);
  }
  om_handle h_;
  const char *name_;
};

template <class T> class array_member : public host_array<T> {
 public:
  array_member(om_handle h, const char *name) : host_array<T>(h, name) {}
  template <class V, class = typename std::enable_if<
                         std::is_constructible<V, const T *, const T *>::value>::type>
  operator V() const {
    const T *b = this->cdata();
    return V(b, b + this->size());
  }
};

// Common part of a generated OM class: the handle, sizes, margins, kernels.
class machine {
 public:
  machine(int kind, int n0, int n1, const om_config &cfg) {
    const int sizes[2] = {n0, n1};
    check(om_create(kind, 2, sizes, &cfg, &h_), "om_create");
  }
  // a general OM graph (om_create_graph), compiled for this GPU
  explicit machine(const char *graph_text) {
    check(om_create_graph(graph_text, nullptr, &h_), "om_create_graph");
  }
  ~machine() { om_destroy(h_); }
  machine(const machine &) = delete;
  machine &operator=(const machine &) = delete;

  int om_size() { return q(::om_size, -1); }
  int om_size_0() { return q(::om_size, 0); }
  int om_size_1() { return q(::om_size, 1); }
  int om_memory_size() { return q(::om_memory_size, -1); }
  int om_memory_size_0() { return q(::om_memory_size, 0); }
  int om_memory_size_1() { return q(::om_memory_size, 1); }
  int om_lower_margin_0() { return q(::om_lower_margin, 0); }
  int om_lower_margin_1() { return q(::om_lower_margin, 1); }
  int om_upper_margin_0() { return q(::om_upper_margin, 0); }
  int om_upper_margin_1() { return q(::om_upper_margin, 1); }
  // the earlier generator's names for the same
  int size() { return om_size(); }
  int size0() { return om_size_0(); }
  int size1() { return om_size_1(); }
  int memorySize() { return om_memory_size(); }
  int memorySize0() { return om_memory_size_0(); }
  int memorySize1() { return om_memory_size_1(); }
  int lowerMargin0() { return om_lower_margin_0(); }
  int lowerMargin1() { return om_lower_margin_1(); }
  int upperMargin0() { return om_upper_margin_0(); }
  int upperMargin1() { return om_upper_margin_1(); }

  om_handle handle() const { return h_; }

 protected:
  void run(const char *kernel) {
    int id;
    check(om_kernel_id(h_, kernel, &id), kernel);
    check(om_run(h_, id), kernel);
  }
  template <class T> T &scalar(const char *name) {
    void *p;
    check(om_scalar_ptr(h_, name, &p, nullptr), name);
    return *static_cast<T *>(p);
  }
  template <class T> T &element(const char *name, int i0, int i1) {
    void *p;
    check(om_array_host(h_, name, &p, nullptr, nullptr), name);
    const std::size_t addr = (std::size_t)(om_lower_margin_0() + i0) +
                             (std::size_t)om_memory_size_0() * (om_lower_margin_1() + i1);
    return static_cast<T *>(p)[addr];
  }
  om_handle h_ = nullptr;

 private:
  int q(om_status (*f)(om_handle, int, int *), int axis) {
    int v;
    check(f(h_, axis, &v), "size query");
    return v;
  }
};

}  // namespace om_shim
