// Phase profiler: when enabled, CUDA events bracket every instrumented region on the library
// stream; the report sums device time, launches, algorithmic flops and bytes per region name.
#pragma once

#include <string>

#include "common.hpp"

namespace pgpu {

bool profile_enabled();
void profile_enable(bool on);
void profile_reset();
// JSON object {name: {"calls", "ms", "flops", "bytes"}} (synchronizes the stream).
std::string profile_report();

class ProfScope {
 public:
  ProfScope(const char* name, double flops = 0, double bytes = 0);
  ~ProfScope();
  ProfScope(const ProfScope&) = delete;
  ProfScope& operator=(const ProfScope&) = delete;

 private:
  int slot_ = -1;
};

}  // namespace pgpu
