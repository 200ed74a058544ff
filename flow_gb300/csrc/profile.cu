// profile.cu -- per-kernel event timing table (see profile.h) and its C ABI.
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/flow_gb300.h"
#include "profile.h"

namespace flow {
namespace {

struct Entry {
  std::string name;
  long long launches = 0;
  double total_ms = 0.0;
};

std::mutex g_mu;
bool g_enabled = false;
std::vector<Entry> g_table;
cudaEvent_t g_events[49];
bool g_events_ready = false;

void add(const char* name, float ms) {
  for (auto& e : g_table) {
    if (e.name == name) {
      e.launches += 1;
      e.total_ms += ms;
      return;
    }
  }
  g_table.push_back(Entry{name, 1, ms});
}

}  // namespace

bool profiling_enabled() { return g_enabled; }

void StepProfiler::begin(cudaStream_t s) {
  active_ = g_enabled;
  stream_ = s;
  n_ = 0;
  if (active_ && !g_events_ready) {
    for (auto& ev : g_events) cudaEventCreate(&ev);
    g_events_ready = true;
  }
}

void StepProfiler::mark(const char* name) {
  if (!active_ || n_ >= 48) return;
  cudaEventRecord(g_events[n_], stream_);
  names_[n_++] = name;
}

void StepProfiler::end() {
  if (!active_ || n_ == 0) return;
  cudaEventRecord(g_events[n_], stream_);
  cudaEventSynchronize(g_events[n_]);
  std::lock_guard<std::mutex> lock(g_mu);
  for (int k = 0; k < n_; ++k) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, g_events[k], g_events[k + 1]);
    add(names_[k], ms);
  }
  active_ = false;
}

}  // namespace flow

extern "C" {

int gb300_profile_enable(int on) {
  flow::g_enabled = (on != 0);
  return GB300_OK;
}

int gb300_profile_reset(void) {
  std::lock_guard<std::mutex> lock(flow::g_mu);
  flow::g_table.clear();
  return GB300_OK;
}

int gb300_profile_count(void) {
  std::lock_guard<std::mutex> lock(flow::g_mu);
  return (int)flow::g_table.size();
}

int gb300_profile_entry(int i, char* name, int name_len, long long* launches,
                        double* total_ms) {
  std::lock_guard<std::mutex> lock(flow::g_mu);
  if (i < 0 || i >= (int)flow::g_table.size() || !name || name_len <= 0) {
    return GB300_ERR_ARG;
  }
  const auto& e = flow::g_table[(size_t)i];
  std::strncpy(name, e.name.c_str(), (size_t)name_len - 1);
  name[name_len - 1] = '\0';
  if (launches) *launches = e.launches;
  if (total_ms) *total_ms = e.total_ms;
  return GB300_OK;
}

}  // extern "C"
