// Phase timers (CUDA events) and the kernel-launch counter; see prof.hpp.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "prof.hpp"

namespace imsrg {

std::atomic<long long> g_kernel_launches{0};

namespace {
struct Pending {
  std::string name;
  cudaEvent_t e0, e1;
};
std::mutex g_pmu;
bool g_on = false;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free;
std::map<std::string, std::pair<double, long long>> g_timer;

cudaEvent_t get_event()
{
  if (!g_free.empty()) {
    cudaEvent_t e = g_free.back();
    g_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void resolve_locked()
{
  for (Pending& p : g_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(p.e1) == cudaSuccess && cudaEventElapsedTime(&ms, p.e0, p.e1) == cudaSuccess) {
      auto& t = g_timer[p.name];
      t.first += ms;
      t.second += 1;
    }
    g_free.push_back(p.e0);
    g_free.push_back(p.e1);
  }
  g_pending.clear();
}
}  // namespace

bool prof_enabled() { return g_on; }

int prof_begin(const char* name, cudaStream_t st)
{
  if (!g_on) return -1;
  std::lock_guard<std::mutex> g(g_pmu);
  Pending p;
  p.name = name;
  p.e0 = get_event();
  p.e1 = get_event();
  cudaEventRecord(p.e0, st);
  g_pending.push_back(p);
  return (int)g_pending.size() - 1;
}

void prof_end(int slot, cudaStream_t st)
{
  if (slot < 0) return;
  std::lock_guard<std::mutex> g(g_pmu);
  if (slot < (int)g_pending.size()) cudaEventRecord(g_pending[slot].e1, st);
}

}  // namespace imsrg

using namespace imsrg;

extern "C" {

int imsrg_profiler_enable(int on)
{
  std::lock_guard<std::mutex> g(g_pmu);
  g_on = on != 0;
  // events are created here, not inside the timed phases (a phase takes two
  // and they return to the pool only when the timers are read)
  while (g_on && g_free.size() < 1024) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) break;
    g_free.push_back(e);
  }
  return IMSRG_OK;
}

int imsrg_profiler_reset(void)
{
  std::lock_guard<std::mutex> g(g_pmu);
  resolve_locked();
  g_timer.clear();
  g_kernel_launches.store(0);
  return IMSRG_OK;
}

int imsrg_profiler_get(const char* name, double* total_ms, long long* count)
{
  if (!name) return IMSRG_ERR_ARG;
  std::lock_guard<std::mutex> g(g_pmu);
  resolve_locked();
  auto it = g_timer.find(name);
  if (total_ms) *total_ms = it == g_timer.end() ? 0.0 : it->second.first;
  if (count) *count = it == g_timer.end() ? 0 : it->second.second;
  return IMSRG_OK;
}

int imsrg_profiler_names(char* buf, int buflen)
{
  std::lock_guard<std::mutex> g(g_pmu);
  resolve_locked();
  std::string all;
  for (auto& kv : g_timer) {
    all += kv.first;
    all += '\n';
  }
  if (!buf || buflen <= 0) return (int)all.size() + 1;
  int n = std::min<int>((int)all.size(), buflen - 1);
  all.copy(buf, n);
  buf[n] = 0;
  return IMSRG_OK;
}

long long imsrg_kernel_launches(void) { return g_kernel_launches.load(); }

}  // extern "C"
