// Design-variable kernels: distance filter stencil, SIMP scale factors,
// OC bisection with device-side control, deterministic reductions, PCG
// vector updates.
//
// Replaces: assemble_matrix_filter + the three sparse H products per
// iteration (filter/matrix_filter.py:101-232, topology_optimization.py:545-572,
// :637-649), simp (material_interpolation.py:6-32), oc_top88
// (optimizer/optimality_criterion.py:9-79), the change/volume reductions
// (topology_optimization.py:516, :654, :670) and the PCG vector algebra
// (linear_solvers.py:114-134).
#include <algorithm>
#include "tg_ops.cuh"
#include "tg_design.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// filter: weights max(0, rmin - |d|) over |d_i| <= R; H is never formed
// ---------------------------------------------------------------------------
template <int NDIM, int MODE>
__global__ void __launch_bounds__(RED_THREADS) k_filter(Grid g, int R, int rex, int rey, int rez,
                                                       const double* __restrict__ w,
                                                       const double* __restrict__ x,
                                                       const double* __restrict__ d,
                                                       const double* __restrict__ Hs,
                                                       double* __restrict__ y,
                                                       const double* __restrict__ xold,
                                                       double* part_sum, double* part_max) {
  pdl_wait();
  pdl_trigger();
  __shared__ double sh[32];
  const int64_t nel = g.nel();
  const int W = 2 * R + 1;
  double psum = 0.0, pmax = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nel;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int ey = (int)(e % g.ney);
    const int ex = (int)((e / g.ney) % g.nex);
    const int ez = (int)(e / ((int64_t)g.ney * g.nex));
    if (ex >= rex || ey >= rey || ez >= rez) {   // padding element
      y[e] = 0.0;
      continue;
    }
    double acc = 0.0;
    const int zlo = (NDIM == 3) ? -R : 0, zhi = (NDIM == 3) ? R : 0;
    for (int oz = zlo; oz <= zhi && MODE != 4; ++oz) {
      const int nz = ez + oz;
      if (nz < 0 || nz >= rez) continue;
      for (int ox = -R; ox <= R; ++ox) {
        const int nx = ex + ox;
        if (nx < 0 || nx >= rex) continue;
        for (int oy = -R; oy <= R; ++oy) {
          const int ny = ey + oy;
          if (ny < 0 || ny >= rey) continue;
          const double wt = w[((NDIM == 3 ? (oz + R) * W : 0) + (ox + R)) * W + (oy + R)];
          if (wt == 0.0) continue;          // uniform over the block: taps beyond rmin
          const int64_t nb = g.elem(nx, ny, nz);
          if (MODE == 0 || MODE == 5) acc += wt * x[nb];
          else if (MODE == 1) acc += wt * (x[nb] / Hs[nb]);
          else if (MODE == 2) acc += wt * (x[nb] * d[nb]);
          else acc += wt;
        }
      }
    }
    double out;
    if (MODE == 0) out = acc / Hs[e];
    else if (MODE == 1) out = acc;
    else if (MODE == 2) out = acc / Hs[e] / fmax(0.001, x[e]);
    else if (MODE == 3 || MODE == 5) out = acc;
    else out = x[e];
    y[e] = out;
    if (part_sum) psum += out;
    if (xold) pmax = fmax(pmax, fabs(x[e] - xold[e]));
  }
  if (part_sum) {
    const double s = block_sum(psum, sh);
    if (threadIdx.x == 0) part_sum[blockIdx.x] = s;
  }
  if (xold) {
    const double m = block_max(pmax, sh);
    if (threadIdx.x == 0) part_max[blockIdx.x] = m;
  }
}

__global__ void k_div(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                      double* __restrict__ q) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) q[i] = a[i] / b[i];
}

void filter_apply_ex(const Grid& g, const FilterStencil& fs, const double* x, const double* d,
                     const double* Hs, double* y, int mode, const double* xold, double* part_sum,
                     double* part_max, cudaStream_t st) {
  const unsigned blocks = red_blocks(g.nel());
  prof_begin(PK_FILTER, st);
  if (mode == 1 && fs.tmp) {
    // H (x / Hs): the quotient once per element (GB300's FP64 divide is a
    // multi-instruction sequence on the narrow FP64 pipe), then a plain sum
    launch_pdl(k_div, dim3((unsigned)cdiv(g.nel(), 256)), dim3(256), 0, st, g.nel(), x, Hs, fs.tmp);
    TG_CHECK_LAUNCH();
    x = fs.tmp;
    mode = 5;
  }
#define TG_F(ND, M) launch_pdl(k_filter<ND, M>, dim3(blocks), dim3(RED_THREADS), 0, st, g, fs.R, fs.rex, fs.rey, fs.rez, fs.w, x, d, Hs, y, xold, part_sum, part_max)
  if (g.ndim == 3) {
    if (mode == 0) TG_F(3, 0); else if (mode == 1) TG_F(3, 1); else if (mode == 2) TG_F(3, 2);
    else if (mode == 3) TG_F(3, 3); else if (mode == 5) TG_F(3, 5); else TG_F(3, 4);
  } else {
    if (mode == 0) TG_F(2, 0); else if (mode == 1) TG_F(2, 1); else if (mode == 2) TG_F(2, 2);
    else if (mode == 3) TG_F(2, 3); else if (mode == 5) TG_F(2, 5); else TG_F(2, 4);
  }
#undef TG_F
  prof_end(PK_FILTER, st);
  TG_CHECK_LAUNCH();
}

void filter_apply(const Grid& g, const FilterStencil& fs, const double* x, const double* d,
                  const double* Hs, double* y, int mode, cudaStream_t st) {
  filter_apply_ex(g, fs, x, d, Hs, y, mode, nullptr, nullptr, nullptr, st);
}

// ---------------------------------------------------------------------------
// SIMP scale factors eps + (1-eps) x^p in FP64 / FP32 / BF16
// ---------------------------------------------------------------------------
__global__ void k_simp(int64_t n, const double* __restrict__ x, double eps, double penal,
                       double* s64, float* s32, __nv_bfloat16* s16, const int8_t* flags) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xv = x[i];
  const double xp = (penal == 3.0) ? xv * xv * xv : pow(xv, penal);
  double s = eps + (1.0 - eps) * xp;
  if (flags && flags[i] == EL_OUTSIDE) s = 0.0;
  if (s64) s64[i] = s;
  if (s32) s32[i] = (float)s;
  if (s16) s16[i] = __double2bfloat16(s);
}

void simp_scale(int64_t n, const double* x, double eps, double penal, double* s64, float* s32,
                __nv_bfloat16* s16, cudaStream_t st, const int8_t* flags) {
  launch_pdl(k_simp, dim3((unsigned)cdiv(n, 256)), dim3(256), 0, st, n, x, eps, penal, s64, s32, s16, flags);
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// deterministic finalisation of block partials (single block, fixed order)
// ---------------------------------------------------------------------------
__device__ double max_partials(const double* part, int nb, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v = fmax(v, __ldcg(part + i));
  return block_max(v, sh);
}

__global__ void k_reduce_to(const double* part, int nb, double* out, int is_max) {
  pdl_wait();
  pdl_trigger();
  __shared__ double sh[32];
  const double v = is_max ? max_partials(part, nb, sh) : sum_partials(part, nb, sh);
  if (threadIdx.x == 0) *out = v;
}

void reduce_partials(const double* part, int nb, double* out, bool is_max, cudaStream_t st) {
  launch_pdl(k_reduce_to, dim3(1), dim3(RED_THREADS), 0, st, part, nb, out, is_max ? 1 : 0);
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// OC bisection (optimizer/optimality_criterion.py:59-79)
// ---------------------------------------------------------------------------
// bar_count0 = 0; a value no arrival sequence of the grid reaches (a test of
// the bounded barrier wait) keeps every block waiting until its limit
__global__ void k_oc_init(OCState* s, double g, double l1, double l2, unsigned int bar_count0) {
  pdl_wait();
  pdl_trigger();
  s->l1 = l1;
  s->l2 = l2;
  s->g = g;
  s->gt = g;
  s->nsteps = 0;
  s->nsteps64 = 0;
  s->done = ((l2 - l1) / (l1 + l2) > 1e-3) ? 0 : 1;
  s->lmid = 0.5 * (l2 + l1);
  s->sc = 1.0 / sqrt(s->lmid);
  s->sc_last = s->sc;
  s->ticket = 0;
  s->bar.count = bar_count0;
  s->bar.err = 0;
}

// Per design iteration: P = x * sqrt(-dc/dv) and, when stored, the bounds
// lo = max(0, x - move), hi = min(1, x + move) (flags: lo = hi = 0 or 1).
// The step value max(lo, min(hi, P / sqrt(lmid))) equals the reference's
// max(0, max(x - move, min(1, min(x + move, x sqrt(-dc/dv/lmid))))) with the
// square root of the quotient split as sqrt(-dc/dv) / sqrt(lmid).
__global__ void __launch_bounds__(RED_THREADS) k_oc_prep(int64_t n, const double* __restrict__ x,
                                                        const double* __restrict__ dc,
                                                        const double* __restrict__ dv,
                                                        const int8_t* __restrict__ flags,
                                                        double move, OCScratch sc) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xi = x[i];
  const bool outside = flags && flags[i] == EL_OUTSIDE;
  const double P = outside ? 0.0 : xi * sqrt(-dc[i] / dv[i]);
  sc.P[i] = P;
  if (sc.lo) {
    double lo = fmax(0.0, xi - move), hi = fmin(1.0, xi + move);
    if (flags) {
      if (flags[i] == 1 || outside) lo = hi = 0.0;
      else if (flags[i] == 2) lo = hi = 1.0;
    }
    sc.lo[i] = lo;
    sc.hi[i] = hi;
    if (sc.f32) {
      sc.f32[i] = (float)P;
      sc.f32[n + i] = (float)lo;
      sc.f32[2 * n + i] = (float)hi;
      sc.f32[3 * n + i] = (float)xi;
      sc.f32[4 * n + i] = (float)dv[i];
    }
  }
}

template <bool BOUNDS>
__device__ __forceinline__ double oc_value(int64_t i, double xi, const OCScratch& sc,
                                           const int8_t* __restrict__ flags, double move,
                                           double s) {
  const double b = sc.P[i] * s;
  if (BOUNDS) return fmax(sc.lo[i], fmin(sc.hi[i], b));
  double xn = fmax(0.0, fmax(xi - move, fmin(1.0, fmin(xi + move, b))));
  if (flags) {
    if (flags[i] == 1 || flags[i] == EL_OUTSIDE) xn = 0.0;
    else if (flags[i] == 2) xn = 1.0;
  }
  return xn;
}

// The whole bisection in one cooperative launch (all blocks co-resident):
// per step every block sums its elements' dv * (xnew - x) in a fixed
// grid-stride order, writes the block sum to the partials of the step's
// parity, meets the others at a grid barrier and then sums all partials in
// the same fixed order, so every block takes the same decision on (l1, l2)
// without another launch or a host round trip.  Double-buffered partials need
// one barrier per reduction: a block writes reduction k+1's partials only
// after every block has passed reduction k's barrier, i.e. finished reading
// reduction k-1's.  Block 0 writes the final state.  Runs at most max_steps
// steps.
//
// SCREEN (GB300 issues ~64 FP32 operations per FP64 one): each step first
// evaluates the sum in FP32 from FP32 copies of P, lo, hi, x, dv, together
// with a bound on its distance from the FP64 sum.  Per element the FP32 term
// differs from the FP64 one by at most 4u (|dv| (P s + 1 + |x| + 2 |d|) + |t|)
// (u = 2^-24: the roundings of P, s, their product, lo / hi (both in [0, 1]),
// x, the difference d, dv and the product t = dv d; the clamp is 1-Lipschitz),
// and a thread's sum of m terms adds at most m u sum |t|; the FP64 sum's own
// rounding is far below.  With A = sum (|dv| (P s + 1 + |x| + 2 |d|) + |t|),
// |g + T32| > (16 + 2m) u A means the FP64 evaluation has the same sign: the
// decision is the FP64 decision.  Otherwise (near the root) the step is
// evaluated in FP64 as without SCREEN.  The carry gt of the last step is
// always an FP64 sum.
template <bool BOUNDS, bool SCREEN>
__global__ void __launch_bounds__(RED_THREADS) k_oc_bisect(int64_t n, const double* __restrict__ x,
                                                          OCScratch sc,
                                                          const double* __restrict__ dv,
                                                          const int8_t* __restrict__ flags,
                                                          double move, double* part, OCState* st,
                                                          int max_steps) {
  __shared__ double sh[32];
  __shared__ double tot_s, tot_a;
  double l1 = st->l1, l2 = st->l2, lmid = st->lmid, s = st->sc, s_last = st->sc_last;
  double gt = st->gt;
  const double g = st->g;
  int done = st->done, steps = 0, steps64 = 0;
  bool gt_exact = true;
  const unsigned int nb = gridDim.x;
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t ts = (int64_t)gridDim.x * blockDim.x;
  int red = 0;                                   // reductions so far (partials parity)
  // one FP64 reduction of g + sum dv (xnew(s) - x); false: a barrier timed out
  auto fp64_sum = [&](double sv, double& out) -> bool {
    double acc = 0.0;
    for (int64_t i = t0; i < n; i += ts) {
      const double xi = x[i];
      acc += dv[i] * (oc_value<BOUNDS>(i, xi, sc, flags, move, sv) - xi);
    }
    double* pp = part + (red & 1) * (SCREEN ? 2 : 1) * nb;
    const double bs = block_sum(acc, sh);
    if (threadIdx.x == 0) pp[blockIdx.x] = bs;
    if (!grid_sync(&st->bar)) return false;
    ++red;
    const double t = sum_partials(pp, (int)nb, sh);
    if (threadIdx.x == 0) tot_s = t;
    __syncthreads();
    out = g + tot_s;
    return true;
  };
  while (!done && steps < max_steps) {
    bool decided = false, up = false;
    if constexpr (SCREEN) {
      const float s32 = (float)s;
      const float* P32 = sc.f32;
      const float* lo32 = sc.f32 + n;
      const float* hi32 = sc.f32 + 2 * n;
      const float* x32 = sc.f32 + 3 * n;
      const float* dv32 = sc.f32 + 4 * n;
      float tsum = 0.f, asum = 0.f;
      for (int64_t i = t0; i < n; i += ts) {
        const float ps = P32[i] * s32;
        const float xi = x32[i], di = dv32[i];
        const float d = fmaxf(lo32[i], fminf(hi32[i], ps)) - xi;
        const float t = di * d;
        tsum += t;
        asum += fabsf(di) * (ps + 1.f + fabsf(xi) + 2.f * fabsf(d)) + fabsf(t);
      }
      double* pp = part + (red & 1) * 2 * nb;
      const double bt = block_sum((double)tsum, sh);
      const double ba = block_sum((double)asum, sh);
      if (threadIdx.x == 0) {
        pp[blockIdx.x] = bt;
        pp[nb + blockIdx.x] = ba;
      }
      if (!grid_sync(&st->bar)) return;
      ++red;
      const double tt = sum_partials(pp, (int)nb, sh);
      if (threadIdx.x == 0) tot_s = tt;
      const double ta = sum_partials(pp + nb, (int)nb, sh);
      if (threadIdx.x == 0) tot_a = ta;
      __syncthreads();
      const double m = (double)((n + ts - 1) / ts);
      const double g32 = g + tot_s;
      const double margin = ldexp(tot_a, -24) * (16.0 + 2.0 * m);
      if (fabs(g32) > margin) {        // false for NaN or infinite values: FP64 below
        decided = true;
        up = g32 > 0;
        gt = g32;
        gt_exact = false;
      }
    }
    if (!decided) {
      if (!fp64_sum(s, gt)) return;
      up = gt > 0;
      gt_exact = true;
      ++steps64;
    }
    s_last = s;
    if (up) l1 = lmid;
    else l2 = lmid;
    ++steps;
    if ((l2 - l1) / (l1 + l2) > 1e-3) {
      lmid = 0.5 * (l2 + l1);
      s = 1.0 / sqrt(lmid);
    } else {
      done = 1;
    }
  }
  if (SCREEN && !gt_exact) {
    if (!fp64_sum(s_last, gt)) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->l1 = l1;
    st->l2 = l2;
    st->lmid = lmid;
    st->sc = s;
    st->sc_last = s_last;
    st->gt = gt;
    st->done = done;
    st->nsteps += steps;
    st->nsteps64 += steps64;
  }
}

template <bool BOUNDS>
__global__ void __launch_bounds__(RED_THREADS) k_oc_finish(int64_t n, const double* __restrict__ x,
                                                          OCScratch sc,
                                                          const int8_t* __restrict__ flags,
                                                          double move, double* __restrict__ xnew,
                                                          const OCState* st) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) xnew[i] = oc_value<BOUNDS>(i, x[i], sc, flags, move, st->sc_last);
}

void oc_begin(int64_t n, const double* x, const double* dc, const double* dv, const int8_t* flags,
              double move, OCScratch sc, OCState* st, double g, cudaStream_t s, double l1,
              double l2) {
  prof_begin(PK_OC, s);
  launch_pdl(k_oc_prep, dim3((unsigned)cdiv(n, RED_THREADS)), dim3(RED_THREADS), 0, s, n, x, dc, dv, flags, move, sc);
  launch_pdl(k_oc_init, dim3(1), dim3(1), 0, s, st, g, l1, l2, tune_take_oc_barrier_timeout() ? 0x40000000u : 0u);
  prof_end(PK_OC, s);
  count_launches(1);
  TG_CHECK_LAUNCH();
}
void oc_steps(int64_t n, const double* x, OCScratch sc, const double* dv, const int8_t* flags,
              double move, double* part, OCState* st, int nsteps, cudaStream_t s) {
  // co-resident grid: at most half the partial slots (double-buffered) and
  // what the device holds at once (the per-element FP64 work of a step needs
  // all the warps it can get on GB300's narrow FP64 pipe)
  int dev = 0, nsm = 0, per_sm = 0;
  TG_CUDA(cudaGetDevice(&dev));
  TG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const bool screen = sc.lo && sc.f32;
  const void* fn = screen ? (const void*)k_oc_bisect<true, true>
                   : sc.lo ? (const void*)k_oc_bisect<true, false>
                           : (const void*)k_oc_bisect<false, false>;
  TG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, RED_THREADS, 0));
  // double-buffered partials: 2 (4 with the screen's second sum) per block
  const int64_t cap = std::min<int64_t>(RED_BLOCKS / (screen ? 4 : 2), (int64_t)nsm * std::max(per_sm, 1));
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, RED_THREADS), cap));
  void* args[] = {(void*)&n, (void*)&x, (void*)&sc, (void*)&dv, (void*)&flags, (void*)&move,
                  (void*)&part, (void*)&st, (void*)&nsteps};
  prof_begin(PK_OC, s);
  TG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(RED_THREADS), args, 0, s));
  prof_end(PK_OC, s);
  TG_CHECK_LAUNCH();
}
void oc_finish(int64_t n, const double* x, OCScratch sc, const int8_t* flags, double move,
               double* xnew, const OCState* st, cudaStream_t s) {
  const unsigned blocks = (unsigned)cdiv(n, RED_THREADS);
  prof_begin(PK_OC, s);
  if (sc.lo) launch_pdl(k_oc_finish<true>, dim3(blocks), dim3(RED_THREADS), 0, s, n, x, sc, flags, move, xnew, st);
  else launch_pdl(k_oc_finish<false>, dim3(blocks), dim3(RED_THREADS), 0, s, n, x, sc, flags, move, xnew, st);
  prof_end(PK_OC, s);
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// PCG vector algebra (scalars live in device memory)
// ---------------------------------------------------------------------------
// Arithmetic runs in the vector's own type (GB300's FP64 pipe is ~1/64 of
// FP32, so FP64 work per element would dominate an FP32 vector kernel); each
// thread's partial sum is widened to FP64 for the block and grid reduction.
template <typename TA, typename TB>
__global__ void __launch_bounds__(RED_THREADS) k_dot(int64_t n, const TA* __restrict__ a,
                                                    const TB* __restrict__ b, double* part,
                                                    PCGState* st, int op) {
  pdl_wait();
  pdl_trigger();
  __shared__ double sh[32];
  __shared__ int last;
  TA acc = TA(0);
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t ts = (int64_t)gridDim.x * blockDim.x;
  if constexpr (sizeof(TA) == 4 && sizeof(TB) == 4) {
    // FP32: 16-byte loads (the vectors start at allocation boundaries), scalar tail
    const int64_t n4 = n / 4;
    const float4* a4 = reinterpret_cast<const float4*>(a);
    const float4* b4 = reinterpret_cast<const float4*>(b);
#pragma unroll 2
    for (int64_t i = t0; i < n4; i += ts) {
      const float4 x = a4[i], y = b4[i];
      acc = fmaf(x.x, y.x, acc);
      acc = fmaf(x.y, y.y, acc);
      acc = fmaf(x.z, y.z, acc);
      acc = fmaf(x.w, y.w, acc);
    }
    for (int64_t i = 4 * n4 + t0; i < n; i += ts) acc = fmaf(a[i], b[i], acc);
  } else {
#pragma unroll 4
    for (int64_t i = t0; i < n; i += ts) acc = fma(a[i], (TA)b[i], acc);
  }
  const double s = block_sum((double)acc, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s;
    __threadfence();
    const unsigned t = atomicAdd(&st->ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const double tot = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    pcg_dot_finish(st, op, tot);
    st->ticket = 0;
  }
}

template <typename TA, typename TB>
void dot(int64_t n, const TA* a, const TB* b, double* part, PCGState* st, int op, cudaStream_t s) {
  launch_pdl(k_dot<TA, TB>, dim3(red_blocks(n)), dim3(RED_THREADS), 0, s, n, a, b, part, st, op);
  TG_CHECK_LAUNCH();
}
template void dot<double, double>(int64_t, const double*, const double*, double*, PCGState*, int, cudaStream_t);
template void dot<float, float>(int64_t, const float*, const float*, double*, PCGState*, int, cudaStream_t);

template <typename T>
__global__ void k_update_p(int64_t n, const T* __restrict__ z, T* __restrict__ p, const PCGState* st) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const T beta = (T)st->beta;
  const bool first = st->iter == 0;
  if constexpr (sizeof(T) == 4) {         // thread per 4 values, 16-byte accesses
    const int64_t n4 = n / 4;
    if (i < n4) {
      const float4 zv = reinterpret_cast<const float4*>(z)[i];
      float4 pv = first ? zv : reinterpret_cast<const float4*>(p)[i];
      if (!first) {
        pv.x = fmaf(beta, pv.x, zv.x); pv.y = fmaf(beta, pv.y, zv.y);
        pv.z = fmaf(beta, pv.z, zv.z); pv.w = fmaf(beta, pv.w, zv.w);
      }
      reinterpret_cast<float4*>(p)[i] = pv;
    } else if (i < n4 + (n - 4 * n4)) {
      const int64_t j = 4 * n4 + (i - n4);
      p[j] = first ? z[j] : fma(beta, p[j], z[j]);
    }
  } else {
    if (i >= n) return;
    p[i] = first ? z[i] : fma(beta, p[i], z[i]);
  }
}
template <typename T>
void update_p(int64_t n, const T* z, T* p, const PCGState* st, cudaStream_t s) {
  const int64_t nt = sizeof(T) == 4 ? n / 4 + (n % 4) : n;
  launch_pdl(k_update_p<T>, dim3((unsigned)cdiv(nt, 256)), dim3(256), 0, s, n, z, p, st);
  TG_CHECK_LAUNCH();
}
template void update_p<double>(int64_t, const double*, double*, const PCGState*, cudaStream_t);
template void update_p<float>(int64_t, const float*, float*, const PCGState*, cudaStream_t);

__global__ void k_update_p_corr(int64_t n, const float* __restrict__ z, const float* __restrict__ w,
                                float* __restrict__ p, const PCGState* st) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const float beta = (float)st->beta;
  const float gam = -(float)(st->wz * st->wawinv);
  const bool first = st->iter == 0;
  const int64_t n4 = n / 4;
  if (i < n4) {
    const float4 zv = reinterpret_cast<const float4*>(z)[i];
    const float4 wv = reinterpret_cast<const float4*>(w)[i];
    float4 v;
    v.x = fmaf(gam, wv.x, zv.x); v.y = fmaf(gam, wv.y, zv.y);
    v.z = fmaf(gam, wv.z, zv.z); v.w = fmaf(gam, wv.w, zv.w);
    if (!first) {
      const float4 pv = reinterpret_cast<const float4*>(p)[i];
      v.x = fmaf(beta, pv.x, v.x); v.y = fmaf(beta, pv.y, v.y);
      v.z = fmaf(beta, pv.z, v.z); v.w = fmaf(beta, pv.w, v.w);
    }
    reinterpret_cast<float4*>(p)[i] = v;
  } else if (i < n4 + (n - 4 * n4)) {
    const int64_t j = 4 * n4 + (i - n4);
    const float v = fmaf(gam, w[j], z[j]);
    p[j] = first ? v : fmaf(beta, p[j], v);
  }
}
void update_p_corr(int64_t n, const float* z, const float* w, float* p, const PCGState* st,
                   cudaStream_t s) {
  const int64_t nt = n / 4 + (n % 4);
  launch_pdl(k_update_p_corr, dim3((unsigned)cdiv(nt, 256)), dim3(256), 0, s, n, z, w, p, st);
  TG_CHECK_LAUNCH();
}
__global__ void k_deflate_start(int64_t n, const float* __restrict__ w, const float* __restrict__ aw,
                                float* __restrict__ d, float* __restrict__ r, const PCGState* st) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gam = (float)(st->wr * st->wawinv);
  d[i] = gam * w[i];
  r[i] = fmaf(-gam, aw[i], r[i]);
}
void deflate_start(int64_t n, const float* w, const float* aw, float* d, float* r,
                   const PCGState* st, cudaStream_t s) {
  k_deflate_start<<<(unsigned)cdiv(n, 256), 256, 0, s>>>(n, w, aw, d, r, st);
  TG_CHECK_LAUNCH();
}
__global__ void k_set_correction(PCGState* st, double v) {
  st->wawinv = v;
  st->wr = st->wz = 0.0;
}
void set_correction(PCGState* st, double v, cudaStream_t s) {
  k_set_correction<<<1, 1, 0, s>>>(st, v);
  TG_CHECK_LAUNCH();
}

// x += alpha p ; r -= alpha q ; rr = r.r (finalised by the last block)
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) k_update_xr(int64_t n, const T* __restrict__ p,
                                                          const T* __restrict__ q, T* __restrict__ x,
                                                          T* __restrict__ r, double* part, PCGState* st) {
  pdl_wait();
  pdl_trigger();
  __shared__ double sh[32];
  __shared__ int last;
  const T alpha = (T)st->alpha;
  T acc = T(0);
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t ts = (int64_t)gridDim.x * blockDim.x;
  int64_t i0 = 0;
  if constexpr (sizeof(T) == 4) {
    const int64_t n4 = n / 4;
    const float4* p4 = reinterpret_cast<const float4*>(p);
    const float4* q4 = reinterpret_cast<const float4*>(q);
    float4* x4 = reinterpret_cast<float4*>(x);
    float4* r4 = reinterpret_cast<float4*>(r);
    for (int64_t i = t0; i < n4; i += ts) {
      const float4 pv = p4[i], qv = q4[i];
      float4 xv = x4[i], rv = r4[i];
      xv.x = fmaf(alpha, pv.x, xv.x); xv.y = fmaf(alpha, pv.y, xv.y);
      xv.z = fmaf(alpha, pv.z, xv.z); xv.w = fmaf(alpha, pv.w, xv.w);
      rv.x = fmaf(-alpha, qv.x, rv.x); rv.y = fmaf(-alpha, qv.y, rv.y);
      rv.z = fmaf(-alpha, qv.z, rv.z); rv.w = fmaf(-alpha, qv.w, rv.w);
      x4[i] = xv;
      r4[i] = rv;
      acc = fmaf(rv.x, rv.x, acc); acc = fmaf(rv.y, rv.y, acc);
      acc = fmaf(rv.z, rv.z, acc); acc = fmaf(rv.w, rv.w, acc);
    }
    i0 = 4 * n4;
  }
#pragma unroll 4
  for (int64_t i = i0 + t0; i < n; i += ts) {
    x[i] = fma(alpha, p[i], x[i]);
    const T ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    acc = fma(ri, ri, acc);
  }
  const double s = block_sum((double)acc, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s;
    __threadfence();
    const unsigned t = atomicAdd(&st->ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const double tot = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    st->rr = tot;
    st->iter += 1;
    st->ticket = 0;
  }
}
template <typename T>
void update_xr(int64_t n, const T* p, const T* q, T* x, T* r, double* part, PCGState* st,
               cudaStream_t s) {
  launch_pdl(k_update_xr<T>, dim3(red_blocks(n)), dim3(RED_THREADS), 0, s, n, p, q, x, r, part, st);
  TG_CHECK_LAUNCH();
}
template void update_xr<double>(int64_t, const double*, const double*, double*, double*, double*, PCGState*, cudaStream_t);
template void update_xr<float>(int64_t, const float*, const float*, float*, float*, double*, PCGState*, cudaStream_t);

__global__ void k_pcg_reset(PCGState* st) {
  pdl_wait();
  pdl_trigger();
  st->iter = 0;
  st->rho = st->beta = st->alpha = st->pq = 0.0;
  st->ticket = 0;
}
void pcg_reset(PCGState* st, cudaStream_t s) {
  launch_pdl(k_pcg_reset, dim3(1), dim3(1), 0, s, st);
  TG_CHECK_LAUNCH();
}

// r32 = r64 / ||r64|| ;   x64 += ||r64|| * d32   (the norm comes from DOT_RR)
__global__ void k_to_unit_f32(int64_t n, const double* __restrict__ r, const PCGState* st,
                              float* __restrict__ r32) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  r32[i] = (float)r[i] * (float)st->rinv;
}
__global__ void k_add_scaled_f32(int64_t n, const float* __restrict__ d, const PCGState* st,
                                 double* __restrict__ x) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = fma(st->rnorm, (double)d[i], x[i]);
}
void to_unit_f32(int64_t n, const double* r, const PCGState* st, float* r32, cudaStream_t s) {
  launch_pdl(k_to_unit_f32, dim3((unsigned)cdiv(n, 256)), dim3(256), 0, s, n, r, st, r32);
  TG_CHECK_LAUNCH();
}
void add_scaled_f32(int64_t n, const float* d, const PCGState* st, double* x, cudaStream_t s) {
  launch_pdl(k_add_scaled_f32, dim3((unsigned)cdiv(n, 256)), dim3(256), 0, s, n, d, st, x);
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_scale_mul(int64_t n, T a, const T* __restrict__ d, const T* __restrict__ b,
                            T* __restrict__ x) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if constexpr (sizeof(T) == 4) {         // thread per 4 values, 16-byte accesses
    const int64_t n4 = n / 4;
    if (i < n4) {
      const float4 dv = reinterpret_cast<const float4*>(d)[i];
      const float4 bv = reinterpret_cast<const float4*>(b)[i];
      reinterpret_cast<float4*>(x)[i] = make_float4(a * dv.x * bv.x, a * dv.y * bv.y,
                                                    a * dv.z * bv.z, a * dv.w * bv.w);
    } else if (i < n4 + (n - 4 * n4)) {
      const int64_t j = 4 * n4 + (i - n4);
      x[j] = a * d[j] * b[j];
    }
  } else {
    if (i < n) x[i] = a * d[i] * b[i];
  }
}
template <typename T>
void scale_mul(int64_t n, double a, const T* d, const T* b, T* x, cudaStream_t s) {
  const int64_t nt = sizeof(T) == 4 ? n / 4 + (n % 4) : n;
  launch_pdl(k_scale_mul<T>, dim3((unsigned)cdiv(nt, 256)), dim3(256), 0, s, n, (T)a, d, b, x);
  TG_CHECK_LAUNCH();
}
template void scale_mul<double>(int64_t, double, const double*, const double*, double*, cudaStream_t);
template void scale_mul<float>(int64_t, double, const float*, const float*, float*, cudaStream_t);

__global__ void k_d2f(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
void d2f(int64_t n, const double* a, float* b, cudaStream_t s) {
  launch_pdl(k_d2f, dim3((unsigned)cdiv(n, 256)), dim3(256), 0, s, n, a, b);
  TG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_axpby(int64_t n, double a, const T* __restrict__ x, double b, T* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = (T)(a * (double)x[i] + b * (double)y[i]);
}
template <typename T>
void axpby(int64_t n, double a, const T* x, double b, T* y, cudaStream_t st) {
  k_axpby<T><<<(unsigned)cdiv(n, 256), 256, 0, st>>>(n, a, x, b, y);
  TG_CHECK_LAUNCH();
}
template void axpby<double>(int64_t, double, const double*, double, double*, cudaStream_t);
template void axpby<float>(int64_t, double, const float*, double, float*, cudaStream_t);

__global__ void k_mask(int64_t nnodes, int ndof, const uint8_t* fix, double* v) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nnodes * ndof) return;
  if ((fix[i / ndof] >> (i % ndof)) & 1) v[i] = 0.0;
}
// user's grid numbering <-> device grid numbering (same coordinates; the
// device grid has extra element / node layers at the high end of each axis)
__global__ void k_embed(Grid rg, Grid g, int nodes, const double* __restrict__ src,
                        double* __restrict__ dst, int to_dev) {
  const int per = nodes ? g.ndof : 1;
  const int64_t nr = nodes ? rg.nnodes() : rg.nel();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nr * per) return;
  const int64_t i = t / per;
  const int c = (int)(t - i * per);
  const int ny = nodes ? rg.nny : rg.ney, nx = nodes ? rg.nnx : rg.nex;
  const int y = (int)(i % ny), x = (int)((i / ny) % nx), z = (int)(i / ((int64_t)ny * nx));
  const int64_t j = (nodes ? g.node(x, y, z) : g.elem(x, y, z)) * per + c;
  if (to_dev) dst[j] = src[t];
  else dst[t] = src[j];
}

void embed_copy(const Grid& rg, const Grid& g, bool nodes, const double* src, double* dst,
                bool to_device_grid, cudaStream_t st) {
  const int64_t n = (nodes ? rg.nnodes() * g.ndof : rg.nel());
  k_embed<<<(unsigned)cdiv(n, 256), 256, 0, st>>>(rg, g, nodes ? 1 : 0, src, dst,
                                                  to_device_grid ? 1 : 0);
  TG_CHECK_LAUNCH();
}

void mask_vec_f64(int64_t nnodes, int ndof, const uint8_t* fix, double* v, cudaStream_t st) {
  launch_pdl(k_mask, dim3((unsigned)cdiv(nnodes * ndof, 256)), dim3(256), 0, st, nnodes, ndof, fix, v);
  TG_CHECK_LAUNCH();
}

// edofMat straight from the element coordinates (reference local node order)
__global__ void k_edofmat(Grid g, int32_t* out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  const int ey = (int)(e % g.ney);
  const int ex = (int)((e / g.ney) % g.nex);
  const int ez = (int)(e / ((int64_t)g.ney * g.nex));
  // reference local order as (dx, dy, dz): 2-D (0,1),(1,1),(1,0),(0,0);
  // 3-D adds the same four at dz = 1
  const int lx[4] = {0, 1, 1, 0}, ly[4] = {1, 1, 0, 0};
  const int nc = (g.ndim == 3) ? 8 : 4;
  const int nd = g.ndof;
  for (int k = 0; k < nc; ++k) {
    const int64_t n = g.node(ex + lx[k & 3], ey + ly[k & 3], ez + (k >> 2));
    for (int c = 0; c < nd; ++c) out[e * nc * nd + k * nd + c] = (int32_t)(n * nd + c);
  }
}
void edofmat(const Grid& g, int32_t* out, cudaStream_t st) {
  k_edofmat<<<(unsigned)cdiv(g.nel(), 256), 256, 0, st>>>(g, out);
  TG_CHECK_LAUNCH();
}

}  // namespace tg
