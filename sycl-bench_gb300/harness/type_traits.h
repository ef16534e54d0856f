// Readable element-type names used as benchmark-name suffixes, as in
// sycl-bench's include/type_traits.h:14-23 ("fp32", "fp64", ...).
#pragma once

template <class T>
struct ReadableTypename;

template <>
struct ReadableTypename<float> {
  static constexpr const char* name = "fp32";
};
template <>
struct ReadableTypename<double> {
  static constexpr const char* name = "fp64";
};
template <>
struct ReadableTypename<int> {
  static constexpr const char* name = "int32";
};
template <>
struct ReadableTypename<long long> {
  static constexpr const char* name = "int64";
};
