// Observer interface around each benchmark run (sycl-bench include/benchmark_hook.h:6-16).
#pragma once

#include "result_consumer.h"

class BenchmarkHook {
public:
  virtual void atInit() = 0;
  virtual void preSetup() = 0;
  virtual void postSetup() = 0;
  virtual void preKernel() = 0;
  virtual void postKernel() = 0;
  virtual void emitResults(ResultConsumer&) {}
  virtual ~BenchmarkHook() = default;
};
