// Context of one optimisation problem: device buffers, multigrid hierarchy,
// solver drivers.  Internal to the library (the ABI sees an opaque tg_ctx).
#pragma once
#include <vector>
#include <string>
#include "tg_common.cuh"
#include "tg_ops.cuh"
#include "tg_design.cuh"
#include "../../include/topopt_gb300.h"

namespace tg {

template <typename T> struct DevBuf {
  T* p = nullptr;
  int64_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  void alloc(int64_t count) {
    release();
    if (count <= 0) return;
    TG_CUDA(cudaMalloc(&p, sizeof(T) * count));
    n = count;
  }
  void zero(cudaStream_t st) {
    if (p) TG_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * n, st));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DevBuf() { release(); }
  operator T*() const { return p; }
};

struct Level {
  Grid g;
  DevBuf<uint8_t> fix;
  DevBuf<double> A64;       // stencil (levels >= 1)
  DevBuf<float> A32;
  DevBuf<double> dinv64, b64, x64, t64, r64;
  DevBuf<float> dinv32, b32, x32, t32, r32;
};

struct Ctx {
  int dev = 0;
  cudaStream_t st = nullptr;
  std::string err;
  // problem
  Grid g;                       // fine grid on the device (element counts in nex/ney/nez)
  Grid rg;                      // the caller's grid; g == rg unless padded
  bool padded = false;          // g has padding layers at the high end of each axis
  DevBuf<double> emb;           // caller-numbered staging buffer (padded grids)
  int ne = 0;                   // element matrix dim
  double volfrac = 0.5, rmin = 1.5, eps = 1e-9, penal = 3.0, move = 0.2;
  int ft = 1;
  int precond = 0, precision = 0, nsmooth = 2, maxiter = 2000, learned = 0;
  int unsmoothed = 0;           // bit l: level l not smoothed (tg_problem.unsmoothed)
  int nsmooth_coarse = 2;       // sweeps before / after on levels >= 1
  double omega = 0.6, rtol = 1e-8, inner_rtol = 1e-4;
  double bnorm = 0.0;           // ||M f|| of load case 0
  int nload = 1;                // load cases: f and u hold nload vectors each
  FineOp op;
  std::vector<double> KEh;      // corner-bit order, host
  // device: problem data
  DevBuf<uint8_t> touch;
  DevBuf<int8_t> flags;
  DevBuf<double> KE64, Q;
  DevBuf<float> Q32;            // Q in FP32 (mixed: coarse operators built in FP32)
  DevBuf<float> KE32;
  DevBuf<double> f, u, x, xPhys, xold, xnew, dc, dcf, dv, Hs, S, s64;
  DevBuf<double> xsolved;       // the design the scale factors and hierarchy were built for
  DevBuf<float> S32;            // FP32 copies screening the OC bisection (5 nel)
  bool built = false;           // a hierarchy exists (tg_adjoint reuses it)
  DevBuf<float> s32;
  DevBuf<__nv_bfloat16> s16;
  DevBuf<double> fw;            // filter weights
  FilterStencil fs;
  DevBuf<double> part, part2;   // reduction partials
  DevBuf<double> scal;          // scalar results (obj, vol, change)
  DevBuf<OCState> oc;
  DevBuf<PCGState> pcg, pcg_out;
  // PCG vectors
  DevBuf<double> r, z, p, q, z2;   // z2: FP64 PCG iterate (fixed address for the graph)
  DevBuf<float> r32, z32, p32, q32, d32;
  // hierarchy
  std::vector<Level*> lv;
  int L = 1;
  int64_t nc = 0, ldc = 0;
  DevBuf<double> Dc, gjwork;
  DevBuf<float> Dc32;           // mixed contexts: the coarsest inverse in FP32 for the FP32 V-cycle
  DevBuf<GridBar> tailbar;      // barrier of the cooperative V-cycle bottom
  double g_oc = 0.0;            // OC carry
  int iter = 0;
  // pinned host mirrors
  OCState* h_oc = nullptr;
  PCGState* h_pcg = nullptr;
  double* h_scal = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, tev0 = nullptr, tev1 = nullptr;
  // one PCG iteration captured as a CUDA graph (FP64 / FP32 loop); every
  // pointer and kernel argument it uses is fixed for the context's lifetime
  struct IterGraph {
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;        // kernels per replay
    int kind = 0;                // profiled family the graph was captured for
    ProfCapture prof;            // its event pairs
  } g64, g32;
  // the whole PCG loop as one graph: a WHILE conditional node whose body is
  // one iteration plus a one-thread kernel that sets the condition from the
  // PCG state on the device (no host round trip per iteration)
  struct LoopGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle h = 0;
    int64_t body_launches = 0;   // kernels per iteration
  } l64, l32;
  bool use_graphs = true;
  struct Cnn* cnn = nullptr;     // learned warm start (not owned)
  // the learned start of this step awaits its test after the first cycle;
  // the FP32 PCG graphs were captured for this deflation vector (null: none)
  bool ws_pending = false;
  // side stream of a design step (learned warm start, then the first FP64
  // residual of the mixed solve, beside the hierarchy build); r_ready: c.r
  // and c.pcg_out hold f - K u and its norm for the solve that follows
  cudaStream_t side = nullptr;
  cudaEvent_t sev_fork = nullptr, sev_join = nullptr;
  bool r_ready = false;
  int last_fallback = 0;
  double last_warm_ratio = 0.0;
  const float* g32_corr = nullptr;
  // Helmholtz PDE filter: the screened Poisson problem on the same device
  // grid, one scalar DOF per node, as its own context (owned); events order
  // its stream after this context's and back
  Ctx* hf = nullptr;
  cudaEvent_t hev0 = nullptr, hev1 = nullptr;
  int64_t filter_iters = 0;      // PCG iterations of all filter solves so far
  // statistics of the last solve
  int last_iters = 0, last_vcycles = 0, last_refine = 0, last_converged = 0;
  double last_relres = 0.0;

  ~Ctx();
};

void ctx_init(Ctx& c, const ::tg_problem& p);
void ctx_step(Ctx& c, ::tg_iter_out& out);
void build_hierarchy(Ctx& c);     // uses c.s64 / c.s32 / c.s16 of the current xPhys
void set_density(Ctx& c, const double* xPhys_dev);   // scale factors for xPhys
// solve K u = b (b, u device FP64, u holds the warm start)
void solve(Ctx& c, const double* b, double* u);
// TG_ETIMEOUT (and a reset flag or barrier) if a bounded wait of a V-cycle
// kernel (TMA copy, grid barrier of the cooperative bottom) ran out since the
// last check; synchronises c.st
void check_waits(Ctx& c);
// prescaled: the level's scratch buffer already holds omega D^-1 b (fused
// into the restriction that produced b); dot_op >= 0: also the PCG dot b . x
// of the result into c.pcg (DOT_RHO), fused into the last fine sweep
template <typename T>
void vcycle(Ctx& c, int l, const T* b, T* x, bool prescaled = false, int dot_op = -1);
// Helmholtz PDE filter: set-up (KF: screened Poisson element matrix, host)
// and y = TF^T KF^-1 TF (v * mul) [/ max(1e-3, xdiv)]; mul and xdiv may be
// null; with part_sum / part_max also the sums of the density filter
// (sum y per block, max |x - xold| per block)
void helmholtz_init(Ctx& c, const double* KF);
void helmholtz_apply(Ctx& c, const double* v, const double* mul, const double* xdiv, double* y,
                     const double* x = nullptr, const double* xold = nullptr,
                     double* part_sum = nullptr, double* part_max = nullptr);

}  // namespace tg
