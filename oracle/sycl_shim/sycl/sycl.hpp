// Host-only stand-in for the slice of SYCL 2020 that sycl-bench's PolyBench
// contraction benchmarks and their harness headers use.  TEST INFRASTRUCTURE:
// it exists so that the reference's own, unmodified source files compile with
// a plain C++ compiler (oracle/build_ref.sh), and their kernels and host
// verification loops can be run to pin the oracle.  It is never part of the
// GPU product.
//
// Semantics kept: buffers are shared handles over their own storage
// (initialised from the host pointer; no write-back), accessors index that
// storage row-major, parallel_for runs the kernel body once per work-item on
// the host (rows in parallel under OpenMP; each work-item's body runs as
// written, so results do not depend on the thread count).  Every buffer
// constructed is recorded in detail::buffer_log() so a driver can read the
// final device contents.
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace sycl {

class exception : public std::exception {
public:
  explicit exception(std::string w = "sycl shim exception") : what_(std::move(w)) {}
  const char* what() const noexcept override { return what_.c_str(); }

private:
  std::string what_;
};

template <int D>
class range {
public:
  range() { v_.fill(0); }
  template <int DD = D, typename = std::enable_if_t<DD == 1>>
  range(std::size_t a) : v_{a} {}
  template <int DD = D, typename = std::enable_if_t<DD == 2>>
  range(std::size_t a, std::size_t b) : v_{a, b} {}
  template <int DD = D, typename = std::enable_if_t<DD == 3>>
  range(std::size_t a, std::size_t b, std::size_t c) : v_{a, b, c} {}
  std::size_t operator[](int i) const { return v_[i]; }
  std::size_t& operator[](int i) { return v_[i]; }
  std::size_t get(int i) const { return v_[i]; }
  std::size_t size() const {
    std::size_t s = 1;
    for(auto x : v_) s *= x;
    return s;
  }

private:
  std::array<std::size_t, D> v_;
};

template <int D>
class id : public range<D> {
public:
  using range<D>::range;
  id() : range<D>() {}
  friend id operator+(const id& a, const id& b) {
    id r;
    for(int d = 0; d < D; ++d) r[d] = a[d] + b[d];
    return r;
  }
};

template <int D>
class item {
public:
  std::size_t operator[](int i) const { return idx_[i]; }
  std::size_t get_id(int i) const { return idx_[i]; }
  range<D> get_range() const { return r_; }
  operator id<D>() const { return idx_; }
  std::size_t get_linear_id() const {
    std::size_t l = 0;
    for(int i = 0; i < D; ++i) l = l * r_[i] + idx_[i];
    return l;
  }

private:
  friend class handler;
  item(id<D> i, range<D> r) : idx_(i), r_(r) {}
  id<D> idx_;
  range<D> r_;
};

namespace access {
enum class mode { read, write, read_write, discard_write, discard_read_write, atomic };
enum class target { device, host_buffer };
}  // namespace access
using target = access::target;

namespace detail {
struct storage_base {
  virtual ~storage_base() = default;
  void* data = nullptr;
  std::size_t count = 0;
};
template <class T>
struct storage : storage_base {
  std::vector<T> v;
  explicit storage(std::size_t n) : v(n) {
    data = v.data();
    count = n;
  }
};
// Every buffer storage created, in construction order.
inline std::vector<std::shared_ptr<storage_base>>& buffer_log() {
  static std::vector<std::shared_ptr<storage_base>> log;
  return log;
}
}  // namespace detail

template <class T, int D>
class accessor {
public:
  accessor(T* p, range<D> r) : p_(p), r_(r) {}
  T& operator[](id<D> i) const { return p_[linear(i)]; }
  T& operator[](const item<D>& it) const {
    id<D> i;
    for(int d = 0; d < D; ++d) i[d] = it[d];
    return p_[linear(i)];
  }
  template <int DD = D, typename = std::enable_if_t<DD == 1>>
  T& operator[](std::size_t i) const {
    return p_[i];
  }
  T* get_pointer() const { return p_; }
  range<D> get_range() const { return r_; }

private:
  std::size_t linear(const id<D>& i) const {
    std::size_t l = 0;
    for(int d = 0; d < D; ++d) l = l * r_[d] + i[d];
    return l;
  }
  T* p_;
  range<D> r_;
};

class handler;

template <class T, int D = 1>
class buffer {
public:
  explicit buffer(range<D> r) : r_(r), s_(std::make_shared<detail::storage<T>>(r.size())) {
    detail::buffer_log().push_back(s_);
  }
  buffer(const T* data, range<D> r) : buffer(r) {
    for(std::size_t i = 0; i < r.size(); ++i) s_->v[i] = data[i];
  }
  buffer(T* data, range<D> r) : buffer(static_cast<const T*>(data), r) {}
  void set_write_back(bool) {}
  template <access::mode M, access::target Tg = access::target::device>
  accessor<T, D> get_access(handler&) {
    return accessor<T, D>(s_->v.data(), r_);
  }
  template <access::mode M>
  accessor<T, D> get_access() {
    return accessor<T, D>(s_->v.data(), r_);
  }
  accessor<T, D> get_host_access() { return accessor<T, D>(s_->v.data(), r_); }
  range<D> get_range() const { return r_; }

private:
  range<D> r_;
  std::shared_ptr<detail::storage<T>> s_;
};

class event {
public:
  void wait() {}
  void wait_and_throw() {}
};

class handler {
public:
  template <class Name = void, class F>
  void parallel_for(range<2> r, F f) {
#pragma omp parallel for schedule(static)
    for(long i = 0; i < long(r[0]); ++i)
      for(std::size_t j = 0; j < r[1]; ++j) f(item<2>(id<2>(std::size_t(i), j), r));
  }
  template <class Name = void, class F>
  void parallel_for(range<1> r, F f) {
#pragma omp parallel for schedule(static)
    for(long i = 0; i < long(r[0]); ++i) f(item<1>(id<1>(std::size_t(i)), r));
  }
  template <class Name = void, class F>
  void single_task(F f) {
    f();
  }
};

namespace info {
namespace device {
struct name {};
}  // namespace device
namespace event_profiling {
struct command_submit {};
struct command_start {};
struct command_end {};
}  // namespace event_profiling
}  // namespace info

enum class aspect { cpu, gpu, fp16, fp64 };

class device {
public:
  template <class Info>
  std::string get_info() const {
    return "host CPU (sycl-bench reference via host-only shim)";
  }
  bool has(aspect a) const { return a != aspect::gpu; }
};

namespace property {
namespace queue {
struct in_order {};
struct enable_profiling {};
}  // namespace queue
}  // namespace property

class property_list {
public:
  template <class... P>
  property_list(P...) {}
};

struct cpu_selector_t {};
struct gpu_selector_t {};
inline constexpr cpu_selector_t cpu_selector_v{};
inline constexpr gpu_selector_t gpu_selector_v{};

class queue {
public:
  queue() = default;
  explicit queue(const property_list&) {}
  template <class Selector>
  queue(const Selector&, const property_list&) {}
  template <class F>
  event submit(F f) {
    handler h;
    f(h);
    return event{};
  }
  void wait() {}
  void wait_and_throw() {}
  device get_device() const { return device{}; }
  template <class T>
  event copy(const T* src, T* dst, std::size_t count) {
    for(std::size_t i = 0; i < count; ++i) dst[i] = src[i];
    return event{};
  }
};

// Built-in math used by the kernels (covariance/correlation): the host's
// correctly rounded square roots.
inline float sqrt(float x) { return std::sqrt(x); }
inline double sqrt(double x) { return std::sqrt(x); }

namespace usm {
enum class alloc { host, device, shared, unknown };
}
inline void* malloc(std::size_t bytes, queue&, usm::alloc) { return std::malloc(bytes); }
inline void* malloc_host(std::size_t bytes, queue&) { return std::malloc(bytes); }
template <class T>
void free(T* p, queue&) {
  std::free(p);
}

}  // namespace sycl
