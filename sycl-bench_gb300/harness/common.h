// Benchmark driver of the SYCL-free harness (sycl-bench include/common.h).
//
// A benchmark class B provides
//   B(const BenchmarkArgs&), void setup(), void run(std::vector<gb::Event>&)
//   (or void run()), static std::string getBenchmarkName(BenchmarkArgs&),
// and optionally bool verify(VerificationSetting&) and
// static ThroughputMetric getThroughputMetric(const BenchmarkArgs&).
//
// BenchmarkManager<B>::run() keeps the reference's sequence
// (include/common.h:37-147): emit problem-size / local-size / device-name /
// sycl-implementation; then for each of --num-runs runs, while every run so
// far verified: construct B, setup(), wait, time run()+wait ("run-time"),
// record kernel/submit/system time from the returned events, verify().
// Then the timing statistics, hook results and Verification PASS/FAIL/N/A,
// and flush.  Any exception discards the benchmark's results and is
// reported on stderr by BenchmarkApp::run (:208-212).
#pragma once

#include <chrono>
#include <iostream>
#include <string>
#include <unordered_set>
#include <vector>

#include "benchmark_hook.h"
#include "benchmark_traits.h"
#include "command_line.h"
#include "memory_wrappers.h"
#include "result_consumer.h"
#include "time_metrics.h"
#include "type_traits.h"

#ifndef SYCL_BENCH_HAS_FP64_SUPPORT
#define SYCL_BENCH_HAS_FP64_SUPPORT 0
#endif

template <class Benchmark>
class BenchmarkManager {
public:
  explicit BenchmarkManager(const BenchmarkArgs& args) : args_(args) {}

  void addHook(BenchmarkHook& h) { hooks_.push_back(&h); }

  template <typename... Extra>
  void run(Extra&&... extra) {
    auto& out = *args_.result_consumer;
    out.proceedToBenchmark(Benchmark{args_, extra...}.getBenchmarkName(args_));
    out.consumeResult("problem-size", std::to_string(args_.problem_size));
    out.consumeResult("local-size", std::to_string(args_.local_size));
    out.consumeResult("device-name", args_.device_queue.device_name());
    out.consumeResult("sycl-implementation", args_.device_queue.implementation());

    TimeMetricsProcessor<Benchmark> metrics(args_);
    for(auto* h : hooks_) h->atInit();

    bool all_pass = true;
    try {
      const std::size_t total = args_.num_runs + (args_.warmup_run ? 1 : 0);
      for(std::size_t r = 0; r < total && all_pass; ++r) {
        const bool record = !(args_.warmup_run && r == 0);
        Benchmark b(args_, extra...);
        for(auto* h : hooks_) h->preSetup();
        b.setup();
        args_.device_queue.wait_and_throw();
        for(auto* h : hooks_) h->postSetup();

        std::vector<gb::Event> events;
        events.reserve(64);
        for(auto* h : hooks_) h->preKernel();
        args_.device_queue.mark_timeline_origin();
        const auto t0 = std::chrono::high_resolution_clock::now();
        if constexpr(detail::BenchmarkTraits<Benchmark>::supportsQueueProfiling)
          b.run(events);
        else
          b.run();
        args_.device_queue.wait_and_throw();
        const auto t1 = std::chrono::high_resolution_clock::now();
        for(auto* h : hooks_) h->postKernel();

        const auto run_time = std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0);
        if(record) {
          metrics.addTimingResult("run-time", run_time);
          if constexpr(detail::BenchmarkTraits<Benchmark>::supportsQueueProfiling) {
#if defined(SYCL_BENCH_ENABLE_QUEUE_PROFILING)
            std::chrono::nanoseconds kernel{0}, submit{0};
            for(const auto& e : events) {
              kernel += e.kernel_time();
              submit += e.submit_time();
            }
            metrics.addTimingResult("kernel-time", kernel);
            metrics.addTimingResult("submit-time", submit);
            metrics.addTimingResult("system-time", run_time - kernel);
#else
            mark_unavailable(metrics, r);
#endif
          } else {
            mark_unavailable(metrics, r);
          }
        }

        if constexpr(detail::BenchmarkTraits<Benchmark>::hasVerify) {
          if(args_.verification.range.size() > 0 && args_.verification.enabled && !b.verify(args_.verification))
            all_pass = false;
        }
      }
    } catch(...) {
      out.discard();
      throw;
    }

    metrics.emitResults(out);
    for(auto* h : hooks_) h->emitResults(out);

    if(args_.verification.range.size() == 0 || !args_.verification.enabled ||
        !detail::BenchmarkTraits<Benchmark>::hasVerify)
      out.consumeResult("Verification", "N/A");
    else
      out.consumeResult("Verification", all_pass ? "PASS" : "FAIL");
    out.flush();
  }

private:
  template <class M>
  void mark_unavailable(M& metrics, std::size_t run_index) {
    const bool first_recorded = run_index == (args_.warmup_run ? 1u : 0u);
    if(!first_recorded) return;
    metrics.markAsUnavailable("kernel-time");
    metrics.markAsUnavailable("submit-time");
    metrics.markAsUnavailable("system-time");
  }

  BenchmarkArgs args_;
  std::vector<BenchmarkHook*> hooks_;
};

class BenchmarkApp {
public:
  BenchmarkApp(int argc, char** argv) {
    try {
      args_ = BenchmarkCommandLine{argc, argv}.getBenchmarkArgs();
    } catch(std::exception& e) {
      std::cerr << "Error while parsing command lines: " << e.what() << std::endl;
    }
  }

  const BenchmarkArgs& getArgs() const { return args_; }
  bool shouldRunNDRangeKernels() const { return !args_.cli.isFlagSet("--no-ndrange-kernels"); }
  bool deviceSupportsFP64() const { return true; }  // CUDA devices and host cores do FP64

  template <class Benchmark, typename... Extra>
  void run(Extra&&... extra) {
    if(!args_.device_queue.valid()) {
      std::cerr << "Error: no device queue (command line could not be parsed)" << std::endl;
      return;
    }
    try {
      const auto name = Benchmark{args_, extra...}.getBenchmarkName(args_);
      if(!names_.insert(name).second) {
        std::cerr << "Benchmark with name '" << name << "' has already been run\n";
        throw std::runtime_error("Duplicate benchmark name");
      }
      BenchmarkManager<Benchmark> mgr(args_);
      mgr.run(extra...);
    } catch(gb::Error& e) {
      std::cerr << "Device error: " << e.what() << std::endl;
    } catch(std::exception& e) {
      std::cerr << "Error: " << e.what() << std::endl;
    }
  }

private:
  BenchmarkArgs args_;
  std::unordered_set<std::string> names_;
};
