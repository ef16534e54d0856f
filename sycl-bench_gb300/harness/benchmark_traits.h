// Compile-time detection of the optional parts of a benchmark class
// (sycl-bench include/benchmark_traits.h:9-33):
//   run(std::vector<gb::Event>&)  -> the benchmark reports per-command timings
//   verify(VerificationSetting&)  -> results are checked
//   getThroughputMetric(args)     -> *-throughput columns are filled
#pragma once

#include <type_traits>
#include <utility>
#include <vector>

#include "device.h"

struct VerificationSetting;
struct BenchmarkArgs;

namespace detail {

template <typename T, typename = void>
struct SupportsQueueProfiling : std::false_type {};
template <typename T>
struct SupportsQueueProfiling<T, std::void_t<decltype(std::declval<T&>().run(std::declval<std::vector<gb::Event>&>()))>>
    : std::true_type {};

template <typename T, typename = void>
struct HasVerify : std::false_type {};
template <typename T>
struct HasVerify<T, std::void_t<decltype(&T::verify)>> : std::true_type {};

template <typename T, typename = void>
struct HasThroughputMetric : std::false_type {};
template <typename T>
struct HasThroughputMetric<T, std::void_t<decltype(&T::getThroughputMetric)>> : std::true_type {};

template <typename T>
struct BenchmarkTraits {
  static constexpr bool supportsQueueProfiling = SupportsQueueProfiling<T>::value;
  static constexpr bool hasVerify = HasVerify<T>::value;
  static constexpr bool hasGetThroughputMetric = HasThroughputMetric<T>::value;
};

}  // namespace detail
