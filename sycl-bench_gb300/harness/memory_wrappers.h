// Device buffers of the benchmarks.
//
// PrefetchedBuffer keeps the semantics of sycl-bench's
// include/memory_wrappers.h:39-92: initialize() allocates on the device and
// copies the host data there before the timed region (no write-back to the
// host array); get_host_access() copies the device contents back (the
// reference's host accessor, e.g. polybench/gemm.cpp:99).  On the host
// device (--device=cpu) the "device" copy is host memory.
#pragma once

#include <cstring>
#include <memory>
#include <vector>

#include "device.h"

template <class T, int Dimensions = 1>
class PrefetchedBuffer {
  static_assert(Dimensions >= 1 && Dimensions <= 3, "1 to 3 dimensions");

public:
  PrefetchedBuffer() = default;
  PrefetchedBuffer(const PrefetchedBuffer&) = delete;
  PrefetchedBuffer& operator=(const PrefetchedBuffer&) = delete;
  ~PrefetchedBuffer() { release(); }

  // Allocate without initial data (forceDataAllocation).
  void initialize(const gb::Queue& q, std::size_t count) {
    release();
    q_ = q;
    count_ = count;
    if(q.is_host()) {
      host_.assign(count, T{});
    } else {
      gb::check(gbpoly_malloc(q.ctx(), reinterpret_cast<void**>(&dev_), count * sizeof(T)), "device allocation");
      gb::check(gbpoly_memset(q.ctx(), dev_, 0, count * sizeof(T)), "device memset");
      q.wait_and_throw();
    }
  }

  // Allocate and copy `count` elements from `data` (forceDataTransfer).
  void initialize(const gb::Queue& q, const T* data, std::size_t count) {
    release();
    q_ = q;
    count_ = count;
    if(q.is_host()) {
      host_.assign(data, data + count);
    } else {
      gb::check(gbpoly_malloc(q.ctx(), reinterpret_cast<void**>(&dev_), count * sizeof(T)), "device allocation");
      gb::check(gbpoly_memcpy_h2d(q.ctx(), dev_, data, count * sizeof(T)), "host to device copy");
      q.wait_and_throw();
    }
  }

  // Device address (host address on the host device).
  T* get() { return q_.is_host() ? host_.data() : dev_; }
  const T* get() const { return q_.is_host() ? host_.data() : dev_; }
  std::size_t size() const { return count_; }

  // Copy of the current contents on the host.
  const T* get_host_access() {
    if(q_.is_host()) return host_.data();
    readback_.resize(count_);
    q_.wait_and_throw();
    gb::check(gbpoly_memcpy_d2h(q_.ctx(), readback_.data(), dev_, count_ * sizeof(T)), "device to host copy");
    q_.wait_and_throw();
    return readback_.data();
  }

private:
  void release() {
    if(dev_ && q_.valid() && !q_.is_host()) gbpoly_free(q_.ctx(), dev_);
    dev_ = nullptr;
    host_.clear();
  }

  gb::Queue q_;
  T* dev_ = nullptr;
  std::size_t count_ = 0;
  std::vector<T> host_;
  std::vector<T> readback_;
};
