// Command line of the PolyBench executables (sycl-bench include/command_line.h).
//
//   --size=<n> (3072)  --local=<n> (256)  --num-runs=<n> (5)
//   --device=cpu|gpu|default (default)  --output=stdio|<csv file> (stdio)
//   --verification-begin=x,y,z  --verification-range=x,y,z
//   --no-verification  --no-ndrange-kernels  --warmup-run
// plus benchmark-specific `--key=value` options read through
// args.cli.getOrDefault (e.g. --precision, --init, --seed, --error-report).
//
// Arguments are `--key=value` pairs (a repeated key is an error) or flags.
// Differences from the reference, on purpose:
//   * --warmup-run is parsed (the reference never reads it, command_line.h:166-167)
//     and runs one extra, untimed run first;
//   * x,y,z lists parse by element count (the reference tests the string
//     length, so only one-character values parse, command_line.h:44-53).
#pragma once

#include <array>
#include <cstddef>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "device.h"
#include "result_consumer.h"

#include <iostream>

struct Range3 {
  std::array<std::size_t, 3> v{1, 1, 1};
  std::size_t size() const { return v[0] * v[1] * v[2]; }
  std::size_t operator[](int i) const { return v[i]; }
};
using Id3 = Range3;

namespace detail {
template <class T>
inline T simple_cast(const std::string& s) {
  std::stringstream in{s};
  T out{};
  in >> out;
  if(in.fail()) throw std::invalid_argument{"cannot parse command line value: " + s};
  return out;
}
template <>
inline std::string simple_cast<std::string>(const std::string& s) {
  return s;
}

inline Range3 parse3(const std::string& s, std::size_t fill) {
  std::vector<std::size_t> parts;
  std::stringstream in{s};
  std::string item;
  while(std::getline(in, item, ',')) parts.push_back(simple_cast<std::size_t>(item));
  if(parts.empty() || parts.size() > 3) throw std::invalid_argument{"Invalid range/id: " + s};
  Range3 r;
  for(int i = 0; i < 3; ++i) r.v[i] = i < int(parts.size()) ? parts[i] : fill;
  return r;
}
}  // namespace detail

template <class T>
inline T cast(const std::string& s) {
  return detail::simple_cast<T>(s);
}

class CommandLine {
public:
  CommandLine() = default;
  CommandLine(int argc, char** argv) {
    for(int i = 0; i < argc; ++i) {
      const std::string arg = argv[i];
      const auto pos = arg.find('=');
      if(pos == std::string::npos) {
        flags_.insert(arg);
        continue;
      }
      const std::string key = arg.substr(0, pos);
      if(args_.count(key)) throw std::invalid_argument{"Encountered command line argument several times: " + key};
      args_[key] = arg.substr(pos + 1);
    }
  }

  bool isArgSet(const std::string& key) const { return args_.count(key) != 0; }
  bool isFlagSet(const std::string& flag) const { return flags_.count(flag) != 0; }

  template <class T>
  T getOrDefault(const std::string& key, const T& fallback) const {
    return isArgSet(key) ? cast<T>(args_.at(key)) : fallback;
  }

  template <class T>
  T get(const std::string& key) const {
    if(!isArgSet(key)) throw std::invalid_argument{"Command line argument was requested but missing: " + key};
    return cast<T>(args_.at(key));
  }

private:
  std::unordered_map<std::string, std::string> args_;
  std::unordered_set<std::string> flags_;
};

template <>
inline Range3 CommandLine::getOrDefault<Range3>(const std::string& key, const Range3& fallback) const {
  return isArgSet(key) ? detail::parse3(args_.at(key), key == "--verification-begin" ? 0 : 1) : fallback;
}

struct VerificationSetting {
  bool enabled = true;
  Id3 begin{{0, 0, 0}};
  Range3 range{{1, 1, 1}};
};

struct BenchmarkArgs {
  std::size_t problem_size = 0;
  std::size_t local_size = 0;
  std::size_t num_runs = 0;
  gb::Queue device_queue;
  gb::Queue device_queue_in_order;  // one CUDA stream is already in order: same queue
  VerificationSetting verification;
  CommandLine cli;
  std::shared_ptr<ResultConsumer> result_consumer;
  bool warmup_run = false;
};

class BenchmarkCommandLine {
public:
  BenchmarkCommandLine(int argc, char** argv) : cli_{argc, argv} {}

  BenchmarkArgs getBenchmarkArgs() const {
    BenchmarkArgs a;
    a.problem_size = cli_.getOrDefault<std::size_t>("--size", 3072);
    a.local_size = cli_.getOrDefault<std::size_t>("--local", 256);
    a.num_runs = cli_.getOrDefault<std::size_t>("--num-runs", 5);
    const std::string device = cli_.getOrDefault<std::string>("--device", "default");
    a.device_queue = gb::Queue::create(device);
    a.device_queue_in_order = a.device_queue;
    a.verification.enabled = !cli_.isFlagSet("--no-verification");
    a.verification.begin = cli_.getOrDefault<Id3>("--verification-begin", Id3{{0, 0, 0}});
    a.verification.range = cli_.getOrDefault<Range3>("--verification-range", Range3{{1, 1, 1}});
    a.result_consumer = makeResultConsumer(cli_.getOrDefault<std::string>("--output", "stdio"));
    a.warmup_run = cli_.isFlagSet("--warmup-run");
    a.cli = cli_;
    return a;
  }

private:
  static std::shared_ptr<ResultConsumer> makeResultConsumer(const std::string& name) {
    if(name == "stdio") return std::make_shared<OstreamResultConsumer>(std::cout);
    return std::make_shared<AppendingCsvResultConsumer>(name);
  }

  CommandLine cli_;
};
