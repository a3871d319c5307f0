// OC update that allocates nothing on the device.
//
// Some callers cannot call cudaMalloc: a host application whose device memory
// is owned by its own pool allocator, or code that must not change the
// device's allocation state while other work runs (for example between the
// set-up and the replay of a captured CUDA graph of that application).  They
// still own their inputs and outputs, so this entry point takes device
// pointers for those; the only memory it needs beyond them -- the per-element
// bisection factors, the per-block partial sums and the bisection state --
// lives in one file-scope __device__ array that every GPU loading this library
// holds until the process exits.
//
// Limits and sharing:
//  * at most TG_NOALLOC_MAX_N design variables (2,097,152); larger n is
//    rejected with TG_EINVAL before any device work;
//  * all calls share the one array and it keeps the last call's contents;
//    everything that must start at zero (the reduction ticket) is cleared by
//    each call, but calls that overlap on the GPU (two streams, two host
//    threads) race on the array and must be serialised by the caller;
//  * every call looks up the array's device address with cudaGetSymbolAddress
//    on the current device (cheap once the module is loaded, and never stale
//    after a device reset);
//  * every call copies the bisection state back and synchronises the stream,
//    so it must not be called while that stream is being captured into a CUDA
//    graph: such a call is refused with TG_EINVAL before any work.
#include <string>
#include "tg_design.cuh"
#include "../../include/topopt_gb300.h"

namespace {

constexpr int64_t kMaxN = TG_NOALLOC_MAX_N;

struct NoAllocScratch {
  double S[kMaxN];                 // x*sqrt(-dc/dv) per design variable
  double part[tg::RED_BLOCKS];     // per-block partial sums
  tg::OCState state;               // bisection interval, carry, step count
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

thread_local std::string g_err;

int32_t fail(int32_t code, const std::string& msg) {
  g_err = msg;
  return code;
}

}  // namespace

extern "C" {

const char* tg_noalloc_last_error(void) { return g_err.c_str(); }

int32_t tg_oc_noalloc(int64_t n, const double* x, const double* dc, const double* dv, double g,
                      const int8_t* el_flags, double move, double l1, double l2, double* xnew,
                      double* gt, int32_t* nsteps, void* stream) {
  if (!x || !dc || !dv || !xnew || n <= 0)
    return fail(TG_EINVAL, "tg_oc_noalloc: NULL pointer or n <= 0");
  if (n > kMaxN)
    return fail(TG_EINVAL, "tg_oc_noalloc: n = " + std::to_string(n) +
                               " exceeds the static scratch limit of " + std::to_string(kMaxN) +
                               " design variables");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess)
    return fail(TG_ECUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(TG_EINVAL, "tg_oc_noalloc: the stream is being captured; this call synchronises "
                           "the stream and cannot be part of a CUDA graph");
  // the host-side name of the array is not its device address: look the
  // address up on the current device
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(TG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  NoAllocScratch* s = static_cast<NoAllocScratch*>(p);
  try {
    tg::OCState h{};
    // one scratch array: the move-limit bounds are recomputed from x each step
    const tg::OCScratch ocs{s->S, nullptr, nullptr};
    tg::oc_begin(n, x, dc, dv, el_flags, move, ocs, &s->state, g, st, l1, l2);
    tg::oc_steps(n, x, ocs, dv, el_flags, move, s->part, &s->state, 256, st);
    TG_CUDA(cudaMemcpyAsync(&h, &s->state, sizeof(tg::OCState), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    if (h.bar.err) return fail(TG_ETIMEOUT, "tg_oc_noalloc: a grid barrier wait timed out");
    if (!h.done) return fail(TG_ENOTCONV, "tg_oc_noalloc: OC bisection did not terminate");
    tg::oc_finish(n, x, ocs, el_flags, move, xnew, &s->state, st);
    TG_CUDA(cudaStreamSynchronize(st));
    if (gt) *gt = h.gt;
    if (nsteps) *nsteps = h.nsteps;
    return TG_OK;
  } catch (const tg::Error& err) {
    return fail(err.code, err.msg);
  }
}

}  // extern "C"
