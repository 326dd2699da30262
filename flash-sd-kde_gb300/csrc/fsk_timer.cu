// fsk_timer.cu - optional per-kernel device timing for measurement.
//
// When enabled (fsk_timer_enable(1)), each hot-path kernel launch is
// bracketed by cudaEventRecord on the stream it is launched on, tagged with a
// kernel id and its algorithmic work (pair evaluations).  fsk_timer_collect
// waits for the recorded events and returns, per kernel id, the launch count,
// total device milliseconds and total work.  Disabled by default; costs two
// event records per launch when enabled.
#include <mutex>
#include <vector>

#include "fsk_kernels.cuh"

namespace fsk {

namespace {
struct Rec {
  int id;
  double work;
  cudaEvent_t a, b;
};
std::mutex g_mu;
bool g_enabled = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

TimerScope::TimerScope(int id, double work, cudaStream_t s) : active_(false), idx_(0), s_(s) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_enabled) return;
  Rec r{id, work, take_event(), take_event()};
  cudaEventRecord(r.a, s);
  g_recs.push_back(r);
  idx_ = g_recs.size() - 1;
  active_ = true;
}

TimerScope::~TimerScope() {
  if (!active_) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (idx_ < g_recs.size()) cudaEventRecord(g_recs[idx_].b, s_);
}

}  // namespace fsk

extern "C" {

void fsk_timer_enable(int on) {
  std::lock_guard<std::mutex> lk(fsk::g_mu);
  fsk::g_enabled = on != 0;
}

// Fills up to `cap` entries of ids/launches/ms/work (host arrays) with one row
// per kernel id seen since the last collect; returns the number of rows or a
// negative fsk status.  Waits for the recorded events.
int fsk_timer_collect(int* ids, int64_t* launches, double* ms, double* work, int cap) {
  std::lock_guard<std::mutex> lk(fsk::g_mu);
  int rows = 0;
  for (auto& r : fsk::g_recs) {
    if (cudaEventSynchronize(r.b) != cudaSuccess) return -FSK_ERR_CUDA;
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    int k = 0;
    while (k < rows && ids[k] != r.id) ++k;
    if (k == rows) {
      if (rows == cap) continue;
      ids[k] = r.id;
      launches[k] = 0;
      ms[k] = 0.0;
      work[k] = 0.0;
      ++rows;
    }
    launches[k] += 1;
    ms[k] += t;
    work[k] += r.work;
    fsk::g_pool.push_back(r.a);
    fsk::g_pool.push_back(r.b);
  }
  fsk::g_recs.clear();
  return rows;
}

}  // extern "C"
