// Diagnostics: kernel-launch counter and CUDA-event timing of the dominant
// kernel (enabled on request; off it costs one relaxed atomic per launch).
#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "diag.cuh"

namespace {
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_timing{0};
std::mutex g_mu;
struct Pending {
  cudaEvent_t a, b;
  double flops, bytes;
};
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free;
double g_ms = 0, g_flops = 0, g_bytes = 0;
uint64_t g_dom_launches = 0;
thread_local cudaEvent_t g_open = nullptr;   // one open bracket per host thread

cudaEvent_t get_event() {
  if (!g_free.empty()) {
    cudaEvent_t e = g_free.back();
    g_free.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

void fold_locked() {
  for (auto& p : g_pending) {
    float ms = 0;
    cudaEventSynchronize(p.b);
    cudaEventElapsedTime(&ms, p.a, p.b);
    g_ms += ms;
    g_flops += p.flops;
    g_bytes += p.bytes;
    ++g_dom_launches;
    g_free.push_back(p.a);
    g_free.push_back(p.b);
  }
  g_pending.clear();
}
}  // namespace

namespace mgt {
void count_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

void dom_begin(cudaStream_t s) {
  if (!g_timing.load(std::memory_order_relaxed)) return;
  std::lock_guard<std::mutex> lk(g_mu);
  g_open = get_event();
  cudaEventRecord(g_open, s);
}

void dom_end(cudaStream_t s, double flops, double bytes) {
  if (!g_timing.load(std::memory_order_relaxed)) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_open) return;
  cudaEvent_t b = get_event();
  cudaEventRecord(b, s);
  g_pending.push_back({g_open, b, flops, bytes});
  g_open = nullptr;
  if (g_pending.size() > 4096) fold_locked();
}
}  // namespace mgt

extern "C" int mgt_diag_reset(int enable_timing) {
  std::lock_guard<std::mutex> lk(g_mu);
  fold_locked();
  g_launches.store(0);
  g_ms = g_flops = g_bytes = 0;
  g_dom_launches = 0;
  g_timing.store(enable_timing ? 1 : 0);
  return MGT_OK;
}

extern "C" int mgt_diag_read(uint64_t* launches, uint64_t* dom_launches, double* dom_ms, double* dom_flops,
                             double* dom_bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  fold_locked();
  if (launches) *launches = g_launches.load();
  if (dom_launches) *dom_launches = g_dom_launches;
  if (dom_ms) *dom_ms = g_ms;
  if (dom_flops) *dom_flops = g_flops;
  if (dom_bytes) *dom_bytes = g_bytes;
  return MGT_OK;
}
