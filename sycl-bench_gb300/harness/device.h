// Device queue of the SYCL-free harness.
//
// Replaces the sycl::queue held in BenchmarkArgs (include/command_line.h:133-134
// of sycl-bench) with a handle over either
//   * a libgbpoly context on a CUDA device (--device=gpu / default), or
//   * the host cores (--device=cpu), where kernels run as OpenMP loops.
// Copies of a Queue share one underlying device, as copies of a sycl::queue do.
//
// submit() mirrors queue::submit(command group): it hands the command group a
// Handler that says where to run, and returns an Event carrying the timing
// data the reference reads through event::get_profiling_info
// (include/common.h:88-96): device start/end (CUDA events around the
// command's launches, queued behind a bounded stream hold so that they time
// device execution) and the host time the command was submitted.
#pragma once

#include <chrono>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbpoly.h"

namespace gb {

class Error : public std::runtime_error {
public:
  Error(gbpoly_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  gbpoly_status status;
};

inline void check(gbpoly_status s, const char* what = "gbpoly call") {
  if(s != GBPOLY_OK) throw Error(s, std::string(what) + ": " + gbpoly_last_error());
}

using clock = std::chrono::steady_clock;

struct DeviceImpl {
  bool host = false;
  gbpoly_ctx* ctx = nullptr;
  std::string name;
  // timeline origin: an event recorded when the timed region begins, and the host time of that record
  gbpoly_event* origin = nullptr;
  clock::time_point origin_host;

  ~DeviceImpl() {
    if(ctx) {
      if(origin) gbpoly_event_destroy(ctx, origin);
      gbpoly_destroy(ctx);
    }
  }
};

// Timing record of one submitted command group.
class Event {
public:
  Event() = default;
  Event(std::shared_ptr<DeviceImpl> d, gbpoly_event* s, gbpoly_event* e, clock::time_point submit)
      : dev(std::move(d)), start(s), end(e), submit_host(submit) {}
  Event(clock::time_point submit, clock::time_point host_start, clock::time_point host_end)
      : submit_host(submit), hstart(host_start), hend(host_end) {}
  Event(Event&& o) noexcept { *this = std::move(o); }
  Event& operator=(Event&& o) noexcept {
    release();
    dev = std::move(o.dev);
    start = o.start;
    end = o.end;
    submit_host = o.submit_host;
    hstart = o.hstart;
    hend = o.hend;
    o.start = o.end = nullptr;
    return *this;
  }
  Event(const Event&) = delete;
  Event& operator=(const Event&) = delete;
  ~Event() { release(); }

  // command_end - command_start
  std::chrono::nanoseconds kernel_time() const {
    if(!dev) return std::chrono::duration_cast<std::chrono::nanoseconds>(hend - hstart);
    float ms = 0.f;
    check(gbpoly_event_elapsed_ms(dev->ctx, start, end, &ms), "event elapsed time");
    return std::chrono::nanoseconds(static_cast<long long>(double(ms) * 1e6));
  }

  // command_start - command_submit.  On the GPU the device start is placed on
  // the host timeline through the origin event recorded when the timed
  // region began (the stream is idle then, so the origin's device time is
  // its host record time).
  std::chrono::nanoseconds submit_time() const {
    if(!dev) return std::chrono::duration_cast<std::chrono::nanoseconds>(hstart - submit_host);
    if(!dev->origin) return std::chrono::nanoseconds(0);
    float ms = 0.f;
    check(gbpoly_event_elapsed_ms(dev->ctx, dev->origin, start, &ms), "event elapsed time");
    const double start_ns = double(ms) * 1e6;
    const double submit_ns =
        double(std::chrono::duration_cast<std::chrono::nanoseconds>(submit_host - dev->origin_host).count());
    return std::chrono::nanoseconds(static_cast<long long>(start_ns > submit_ns ? start_ns - submit_ns : 0.0));
  }

private:
  void release() {
    if(dev && dev->ctx) {
      if(start) gbpoly_event_destroy(dev->ctx, start);
      if(end) gbpoly_event_destroy(dev->ctx, end);
    }
    start = end = nullptr;
  }

  std::shared_ptr<DeviceImpl> dev;
  gbpoly_event* start = nullptr;
  gbpoly_event* end = nullptr;
  clock::time_point submit_host, hstart, hend;
};

// What a command group sees: where it runs.
class Queue;

class Handler {
public:
  explicit Handler(DeviceImpl* d) : dev(d) {}
  explicit Handler(const Queue& q);
  bool on_host() const { return dev->host; }
  gbpoly_ctx* ctx() const { return dev->ctx; }

private:
  DeviceImpl* dev;
};

class Queue {
public:
  Queue() = default;
  // Longest a submitted command group's launches may take to queue before
  // the stream starts without waiting for them.
  static constexpr uint32_t kHoldTimeoutUs = 20000;

  // "cpu", "gpu" or "default" (include/command_line.h:193-201).  The GPU
  // index is taken from GBPOLY_DEVICE (default 0).
  static Queue create(const std::string& type) {
    Queue q;
    q.impl = std::make_shared<DeviceImpl>();
    if(type == "cpu") {
      q.impl->host = true;
      q.impl->name = host_cpu_name();
    } else if(type == "gpu" || type == "default") {
      const char* env = std::getenv("GBPOLY_DEVICE");
      const int dev = env ? std::atoi(env) : 0;
      check(gbpoly_init(dev, &q.impl->ctx), "gbpoly_init");
      char buf[256];
      check(gbpoly_device_name(q.impl->ctx, buf, sizeof buf), "gbpoly_device_name");
      q.impl->name = buf;
    } else {
      throw std::invalid_argument{"unknown device type: " + type};
    }
    return q;
  }

  bool valid() const { return static_cast<bool>(impl); }
  bool is_host() const { return impl->host; }
  gbpoly_ctx* ctx() const { return impl->ctx; }
  const std::string& device_name() const { return impl->name; }
  std::string implementation() const { return impl->host ? "gbpoly host (OpenMP)" : "gbpoly CUDA (sm_103a)"; }

  // queue::wait_and_throw()
  void wait_and_throw() const {
    if(impl && impl->ctx) check(gbpoly_synchronize(impl->ctx), "wait_and_throw");
  }

  // Marks the start of a timed region (see Event::submit_time).
  void mark_timeline_origin() const {
    if(!impl || !impl->ctx) return;
    if(!impl->origin) check(gbpoly_event_create(impl->ctx, &impl->origin), "event create");
    impl->origin_host = clock::now();
    check(gbpoly_event_record(impl->ctx, impl->origin), "event record");
  }

  template <class CommandGroup>
  Event submit(CommandGroup&& cg) const {
    const auto submit = clock::now();
    Handler h(impl.get());
    if(impl->host) {
      const auto t0 = clock::now();
      cg(h);
      const auto t1 = clock::now();
      return Event(submit, t0, t1);
    }
    gbpoly_event *s = nullptr, *e = nullptr;
    check(gbpoly_event_create(impl->ctx, &s), "event create");
    check(gbpoly_event_create(impl->ctx, &e), "event create");
    Event ev(impl, s, e, submit);
    // The stream waits (bounded) until the command group is queued, so the
    // start event is timestamped when its kernels can start: the pair times
    // device execution, not the host's launch latency.
    check(gbpoly_stream_hold(impl->ctx, kHoldTimeoutUs), "stream hold");
    struct Release {
      gbpoly_ctx* ctx;
      ~Release() { gbpoly_stream_release(ctx); }
    } release{impl->ctx};
    check(gbpoly_event_record(impl->ctx, s), "event record");
    cg(h);
    check(gbpoly_event_record(impl->ctx, e), "event record");
    return ev;
  }

  DeviceImpl* impl_ptr() const { return impl.get(); }

private:
  static std::string host_cpu_name();
  std::shared_ptr<DeviceImpl> impl;
};

}  // namespace gb

#include <cstdlib>
#include <fstream>

inline gb::Handler::Handler(const Queue& q) : dev(q.impl_ptr()) {}

inline std::string gb::Queue::host_cpu_name() {
  std::ifstream f("/proc/cpuinfo");
  std::string line;
  while(std::getline(f, line)) {
    for(const char* key : {"model name", "Model name"}) {
      if(line.rfind(key, 0) == 0) {
        auto p = line.find(':');
        if(p != std::string::npos) return line.substr(p + 2);
      }
    }
  }
  return "host CPU";
}
