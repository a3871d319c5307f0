// Launch counting and optional CUDA-event timing of one kernel family.
//
// The bench reports how many of the library's kernels ran in its timed
// region (gpu_launches) and the average device time of the dominant kernel,
// measured with events recorded on the stream that launches it.
#include <atomic>
#include <mutex>
#include <set>
#include <utility>
#include <vector>
#include "tg_common.cuh"
#include "tg_ops.cuh"
#include "../../include/topopt_gb300.h"

namespace tg {

static std::atomic<int64_t> g_launches{0};
void count_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_smem_limit(const void* func, int bytes) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  TG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({func, dev})) return;
  TG_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done.insert({func, dev});
}
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

namespace {
std::mutex g_mu;
int g_kind = PK_NONE;
std::vector<cudaEvent_t> g_pool;     // recorded pairs (start, stop)
size_t g_used = 0;
int g_open = 0;
double g_ms = 0.0;
int64_t g_count = 0;

cudaEvent_t next_event() {
  if (g_used == g_pool.size()) {
    cudaEvent_t e;
    TG_CUDA(cudaEventCreate(&e));
    g_pool.push_back(e);
  }
  return g_pool[g_used++];
}

// fold finished pairs into the totals once the pool grows large
void drain_locked() {
  for (size_t i = 0; i + 1 < g_used; i += 2) {
    TG_CUDA(cudaEventSynchronize(g_pool[i + 1]));
    float ms = 0.f;
    TG_CUDA(cudaEventElapsedTime(&ms, g_pool[i], g_pool[i + 1]));
    g_ms += ms;
    g_count += 1;
  }
  g_used = 0;
}
}  // namespace

int prof_kind() { return g_kind; }

namespace {
std::atomic<int64_t> g_small_pairs{150000};
std::atomic<int> g_oc_timeout{0};
std::atomic<int> g_tail{0};
std::atomic<int> g_pdl{1};
std::atomic<int> g_tail_timeout{0};
std::atomic<int> g_conv_umma{1};
std::atomic<int> g_conv_timeout{0};
}  // namespace
bool tune_conv_umma() { return g_conv_umma.load(std::memory_order_relaxed) != 0; }
bool tune_take_conv_timeout() { return g_conv_timeout.exchange(0) != 0; }
int64_t tune_stencil_small_pairs() { return g_small_pairs.load(std::memory_order_relaxed); }
bool tune_take_oc_barrier_timeout() { return g_oc_timeout.exchange(0) != 0; }
int tune_coarse_tail() { return g_tail.load(std::memory_order_relaxed); }
namespace {
thread_local int tl_pdl = 1;
}
bool pdl_on() { return tl_pdl != 0 && g_pdl.load(std::memory_order_relaxed) != 0; }
int pdl_scope(int on) {
  const int prev = tl_pdl;
  tl_pdl = on;
  return prev;
}
bool tune_take_tail_barrier_timeout() { return g_tail_timeout.exchange(0) != 0; }

namespace {
thread_local ProfCapture* g_cap = nullptr;
}

void ProfCapture::release() {
  for (auto& pr : pairs) {
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  pairs.clear();
  if (open) cudaEventDestroy(open);
  open = nullptr;
}

void prof_capture_begin(ProfCapture* pc) {
  pc->release();
  pc->kind = g_kind;
  g_cap = pc;
}
void prof_capture_end() { g_cap = nullptr; }

void prof_collect(const ProfCapture& pc) {
  if (pc.kind != g_kind || pc.kind == PK_NONE) return;
  std::lock_guard<std::mutex> lk(g_mu);
  for (const auto& pr : pc.pairs) {
    float ms = 0.f;
    TG_CUDA(cudaEventElapsedTime(&ms, pr.first, pr.second));
    g_ms += ms;
    g_count += 1;
  }
}

void prof_begin(int kind, cudaStream_t st) {
  if (kind != g_kind || kind == PK_NONE) return;
  if (g_cap) {
    // external record: becomes an event node of the graph (a plain record
    // during capture only expresses a dependency)
    TG_CUDA(cudaEventCreate(&g_cap->open));
    TG_CUDA(cudaEventRecordWithFlags(g_cap->open, st, cudaEventRecordExternal));
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_used >= 4096 && g_open == 0) drain_locked();
  TG_CUDA(cudaEventRecord(next_event(), st));
  g_open = 1;
}

void prof_end(int kind, cudaStream_t st) {
  if (kind != g_kind || kind == PK_NONE) return;
  if (g_cap) {
    cudaEvent_t e;
    TG_CUDA(cudaEventCreate(&e));
    TG_CUDA(cudaEventRecordWithFlags(e, st, cudaEventRecordExternal));
    g_cap->pairs.emplace_back(g_cap->open, e);
    g_cap->open = nullptr;
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  TG_CUDA(cudaEventRecord(next_event(), st));
  g_open = 0;
}

}  // namespace tg

extern "C" {

int32_t tg_profile_kernel(int32_t kind) {
  try {
    std::lock_guard<std::mutex> lk(tg::g_mu);
    tg::drain_locked();
    tg::g_kind = kind;
    tg::g_ms = 0.0;
    tg::g_count = 0;
    return TG_OK;
  } catch (const tg::Error& e) {
    return e.code;
  }
}

int32_t tg_stats(int32_t reset, int64_t* launches, double* prof_ms, int64_t* prof_launches) {
  try {
    std::lock_guard<std::mutex> lk(tg::g_mu);
    tg::drain_locked();
    if (launches) *launches = tg::g_launches.load();
    if (prof_ms) *prof_ms = tg::g_ms;
    if (prof_launches) *prof_launches = tg::g_count;
    if (reset) {
      tg::g_launches.store(0);
      tg::g_ms = 0.0;
      tg::g_count = 0;
    }
    return TG_OK;
  } catch (const tg::Error& e) {
    return e.code;
  }
}

}  // extern "C"

extern "C" int32_t tg_tune(int32_t key, int64_t value) {
  switch (key) {
    case TG_TUNE_STENCIL_SMALL_PAIRS:
      if (value < 0) return TG_EINVAL;
      tg::g_small_pairs.store(value);
      return TG_OK;
    case TG_TUNE_OC_BARRIER_TIMEOUT:
      tg::g_oc_timeout.store(value != 0 ? 1 : 0);
      return TG_OK;
    case TG_TUNE_COARSE_TAIL:
      if (value < 0 || value > 4096) return TG_EINVAL;
      tg::g_tail.store((int)value);
      return TG_OK;
    case TG_TUNE_TAIL_BARRIER_TIMEOUT:
      tg::g_tail_timeout.store(value != 0 ? 1 : 0);
      return TG_OK;
    case TG_TUNE_PDL:
      tg::g_pdl.store(value != 0 ? 1 : 0);
      return TG_OK;
    case TG_TUNE_STENCIL_TMA:
      if (value < 0 || value > 64) return TG_EINVAL;
      tg::tune_set_stencil_tma((int)value);
      return TG_OK;
    case TG_TUNE_CONV_UMMA:
      tg::g_conv_umma.store(value != 0 ? 1 : 0);
      return TG_OK;
    case TG_TUNE_CONV_TIMEOUT:
      tg::g_conv_timeout.store(value != 0 ? 1 : 0);
      return TG_OK;
    default:
      return TG_EINVAL;
  }
}
