// Timing statistics (sycl-bench include/time_metrics.h:26-153).
//
// For each timing name, in sorted name order, emits
//   <name>-mean, -stddev (sample, n-1), -median (upper median), -min,
//   -samples (sorted, space separated, quoted), -throughput (metric / min)
// in seconds, or "N/A" for all six when the timing is unavailable.  Before
// them, "throughput-metric" (the benchmark's getThroughputMetric or "N/A").
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <numeric>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "benchmark_traits.h"
#include "command_line.h"
#include "result_consumer.h"

// The metric a throughput is computed from (e.g. FLOP), not the throughput itself.
struct ThroughputMetric {
  double metric = 0.0;
  std::string unit;
};

template <typename Benchmark>
class TimeMetricsProcessor {
public:
  explicit TimeMetricsProcessor(const BenchmarkArgs& args) : args_(args) {}

  void addTimingResult(const std::string& name, std::chrono::nanoseconds t) {
    if(unavailable_.count(name)) throw std::invalid_argument{"Cannot add result for unavailable timing " + name};
    results_[name].push_back(t);
  }

  void markAsUnavailable(const std::string& name) {
    if(results_.count(name)) throw std::invalid_argument{"Cannot mark timing " + name + " with existing results as unavailable"};
    unavailable_.insert(name);
  }

  void emitResults(ResultConsumer& out) const {
    ThroughputMetric tpm;
    bool has_tpm = false;
    if constexpr(detail::BenchmarkTraits<Benchmark>::hasGetThroughputMetric) {
      tpm = Benchmark::getThroughputMetric(args_);
      has_tpm = true;
      out.consumeResult("throughput-metric", std::to_string(tpm.metric), tpm.unit);
    } else {
      out.consumeResult("throughput-metric", "N/A", "");
    }

    std::set<std::string> names(unavailable_.begin(), unavailable_.end());
    for(const auto& r : results_) names.insert(r.first);

    for(const auto& name : names) {
      if(unavailable_.count(name)) {
        for(const char* s : {"-mean", "-stddev", "-median", "-min", "-samples", "-throughput"})
          out.consumeResult(name + s, "N/A");
        continue;
      }
      std::vector<double> sec;
      for(auto t : results_.at(name)) sec.push_back(double(t.count()) / 1.0e9);
      std::sort(sec.begin(), sec.end());
      const double n = double(sec.size());
      const double mean = std::accumulate(sec.begin(), sec.end(), 0.0) / n;
      double var = 0.0;
      for(double x : sec) var += (mean - x) * (mean - x);
      const double stddev = sec.size() > 1 ? std::sqrt(var / (n - 1.0)) : 0.0;
      out.consumeResult(name + "-mean", std::to_string(mean), "s");
      out.consumeResult(name + "-stddev", std::to_string(stddev), "s");
      out.consumeResult(name + "-median", std::to_string(sec[sec.size() / 2]), "s");
      out.consumeResult(name + "-min", std::to_string(sec.front()), "s");
      std::ostringstream samples;
      samples << '"';
      for(std::size_t i = 0; i < sec.size(); ++i) samples << (i ? " " : "") << std::to_string(sec[i]);
      samples << '"';
      out.consumeResult(name + "-samples", samples.str());
      if(has_tpm && tpm.metric > 0.0)
        out.consumeResult(name + "-throughput", std::to_string(tpm.metric / sec.front()), tpm.unit + "/s");
      else
        out.consumeResult(name + "-throughput", "N/A", "");
    }
  }

private:
  const BenchmarkArgs args_;
  std::map<std::string, std::vector<std::chrono::nanoseconds>> results_;
  std::set<std::string> unavailable_;
};
