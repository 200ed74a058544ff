// profile.h -- optional per-kernel CUDA-event timing of the fused timestep.
//
// When enabled (gb300_profile_enable), the fused solve records an event on
// the launch stream before each kernel and one after the last; after the
// step's closing synchronisation the gaps are added to a per-name table that
// gb300_profile_entry reports.  Disabled, it costs one branch per launch.
#pragma once

#include <cuda_runtime.h>

namespace flow {

class StepProfiler {
 public:
  // Starts a step on stream s (no-op when profiling is off).
  void begin(cudaStream_t s);
  // Marks the start of the named kernel (its end is the next mark).
  void mark(const char* name);
  // Closes the step; call after the stream has been synchronised.
  void end();

 private:
  bool active_ = false;
  cudaStream_t stream_ = nullptr;
  int n_ = 0;
  const char* names_[48];
};

bool profiling_enabled();

}  // namespace flow
