// Phase timers and kernel-launch counter, the GPU counterpart of the
// reference's IMSRGProfiler (src/IMSRGProfiler.cc:14-137): named timers
// accumulate CUDA-event durations on the stream the phase ran on.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

namespace imsrg {

extern std::atomic<long long> g_kernel_launches;
inline void count_launch(int n = 1) { g_kernel_launches.fetch_add(n, std::memory_order_relaxed); }

bool prof_enabled();
// returns an opaque slot, or -1 when profiling is off
int prof_begin(const char* name, cudaStream_t st);
void prof_end(int slot, cudaStream_t st);

struct ProfScope {
  int slot;
  cudaStream_t st;
  ProfScope(const char* name, cudaStream_t s) : slot(prof_begin(name, s)), st(s) {}
  ~ProfScope() { prof_end(slot, st); }
};

}  // namespace imsrg
