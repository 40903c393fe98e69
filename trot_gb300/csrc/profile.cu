// Optional per-kernel timers: when enabled, every launch the C ABI issues is
// bracketed by a pair of CUDA events recorded on the launching stream, and
// trot_profile_collect() sums the elapsed times per kernel name.  Disabled by
// default (zero cost); must stay disabled while a stream is being captured
// into a CUDA graph.  Events come from a pool created at enable time.
#include <atomic>
#include <cstring>
#include <mutex>
#include <vector>

#include "kernels.h"
#include "profile.h"

namespace trot {

namespace {
struct Rec {
  const char* name;
  int a, b;
};
std::mutex g_mu;
std::atomic<bool> g_on{false};
std::atomic<long long> g_launches{0};
std::vector<cudaEvent_t> g_pool;
size_t g_next = 0;
std::vector<Rec> g_recs;
}  // namespace

void prof_count_launch() {
  if (g_on.load(std::memory_order_relaxed)) g_launches.fetch_add(1, std::memory_order_relaxed);
}

int prof_begin(cudaStream_t st) {
  if (!g_on) return -1;
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_next + 2 > g_pool.size()) return -1;
  int i = (int)g_next;
  g_next += 2;
  cudaEventRecord(g_pool[i], st);
  return i;
}

void prof_end(int slot, const char* name, cudaStream_t st) {
  if (slot < 0) return;
  cudaEventRecord(g_pool[slot + 1], st);
  std::lock_guard<std::mutex> lk(g_mu);
  g_recs.push_back(Rec{name, slot, slot + 1});
}

}  // namespace trot

using namespace trot;

extern "C" {

int trot_profile_enable(int max_launches) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto e : g_pool) cudaEventDestroy(e);
  g_pool.clear();
  g_recs.clear();
  g_next = 0;
  g_launches = 0;
  g_on = max_launches > 0;
  for (int i = 0; i < 2 * max_launches; ++i) {
    cudaEvent_t e;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) { g_on = false; return cuda_status(r, "cudaEventCreate"); }
    g_pool.push_back(e);
  }
  return TROT_OK;
}

// Synchronises on the recorded events and writes up to max_names distinct
// kernel names (each in a 48-byte slot of `names`), total milliseconds and
// launch counts; returns the number of names or a negative status.  Clears the
// records (the pool is reused).
int trot_profile_collect(int max_names, char* names, double* total_ms, int* launches) {
  std::lock_guard<std::mutex> lk(g_mu);
  int n = 0;
  for (const Rec& r : g_recs) {
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(g_pool[r.b]);
    if (e != cudaSuccess) return -cuda_status(e, "cudaEventSynchronize");
    cudaEventElapsedTime(&ms, g_pool[r.a], g_pool[r.b]);
    int k = 0;
    for (; k < n; ++k)
      if (strncmp(names + 48 * k, r.name, 47) == 0) break;
    if (k == n) {
      if (n == max_names) continue;
      strncpy(names + 48 * k, r.name, 47);
      names[48 * k + 47] = 0;
      total_ms[k] = 0.0;
      launches[k] = 0;
      ++n;
    }
    total_ms[k] += ms;
    launches[k] += 1;
  }
  g_recs.clear();
  g_next = 0;
  return n;
}

// Kernel launches the library issued since trot_profile_enable (every launch,
// timed or not).
long long trot_profile_launch_count(void) { return g_launches.load(); }

}  // extern "C"
