// Device-resident solver / optimiser state and the launchers of tg_design.cu.
#pragma once
#include "tg_common.cuh"
#include "tg_ops.cuh"

namespace tg {

// OC bisection state (optimizer/optimality_criterion.py:59-77)
struct OCState {
  double l1, l2, lmid, g, gt;
  double sc;         // 1/sqrt(lmid) of the next step (computed once per step)
  double sc_last;    // 1/sqrt(lmid) of the last evaluated step
  int done, nsteps;
  int nsteps64;      // steps decided by an FP64 pass (the rest by the FP32 screen)
  unsigned int ticket;
  GridBar bar;       // barrier of the one-launch bisection (bar.err: a wait timed out)
};
// per-call scratch: P = x*sqrt(-dc/dv); lo/hi = the move-limit bounds with the
// passive/active flags folded in (both null: recomputed from x every step)
struct OCScratch {
  double* P;
  double* lo;
  double* hi;
  // optional (with lo/hi): 5 n floats, the FP32 copies of P, lo, hi, x and dv
  // that screen each bisection decision (null: every step in FP64)
  float* f32 = nullptr;
};

// PCG scalars (linear_solvers.py:114-134)
enum DotOp : int { DOT_RHO = 0, DOT_ALPHA = 1, DOT_RR = 2, DOT_BB = 3, DOT_WR = 4, DOT_WZ = 5 };
struct PCGState {
  double rho, beta, alpha, pq, rr, bb, rnorm, rinv;
  int iter;
  unsigned int ticket;
  double tol;        // device-side PCG loop: continue while sqrt(rr) >= tol
  int maxit;         //   and iter < maxit (and rr finite)
  // deflation by one vector w (deflated CG, Saad et al. 2000): each pass
  // starts with the residual made orthogonal to w (wr = w.r, DOT_WR) and
  // every search direction is made A-orthogonal to w, p = z - mu w + beta p
  // with mu = (Aw . z) / (w^T A w) (wz = Aw . z, DOT_WZ); wawinv =
  // 1 / (w^T A w), 0 = no deflation
  double wr, wz, wawinv;
};

// PCG scalars from a finished dot product (the last block of a reduction)
__device__ inline void pcg_dot_finish(PCGState* st, int op, double tot) {
  if (op == DOT_RHO) {
    st->beta = (st->iter > 0) ? tot / st->rho : 0.0;
    st->rho = tot;
  } else if (op == DOT_ALPHA) {
    st->pq = tot;
    st->alpha = st->rho / tot;
  } else if (op == DOT_RR) {
    st->rr = tot;
    st->rnorm = sqrt(tot);
    st->rinv = tot > 0.0 ? 1.0 / st->rnorm : 0.0;
  } else if (op == DOT_BB) {
    st->bb = tot;
  } else if (op == DOT_WR) {
    st->wr = tot;
  } else if (op == DOT_WZ) {
    st->wz = tot;
  }
}

// fine_apply that also forms a PCG dot of its output, finalised into the PCG
// state like dot(): DOT_ALPHA = u . y (mode AM_Y), DOT_RHO = b . y (AM_JACOBI)
template <typename T, typename S>
void fine_apply_dot(const FineOp& op, const S* scale, const T* u, T* y, const T* b, const T* dinv,
                    double omega, int mode, double* part, PCGState* pst, int dot_op,
                    cudaStream_t st);

void filter_apply_ex(const Grid& g, const FilterStencil& fs, const double* x, const double* d,
                     const double* Hs, double* y, int mode, const double* xold, double* part_sum,
                     double* part_max, cudaStream_t st);
void reduce_partials(const double* part, int nb, double* out, bool is_max, cudaStream_t st);

void oc_begin(int64_t n, const double* x, const double* dc, const double* dv, const int8_t* flags,
              double move, OCScratch sc, OCState* st, double g, cudaStream_t s, double l1 = 0.0,
              double l2 = 1e9);
// up to nsteps bisection steps in one cooperative launch (none once `done`);
// st->bar.err set: a grid barrier timed out
void oc_steps(int64_t n, const double* x, OCScratch sc, const double* dv, const int8_t* flags,
              double move, double* part, OCState* st, int nsteps, cudaStream_t s);
// xnew at the last evaluated lmid (call once `done` is set)
void oc_finish(int64_t n, const double* x, OCScratch sc, const int8_t* flags, double move,
               double* xnew, const OCState* st, cudaStream_t s);

template <typename TA, typename TB>
void dot(int64_t n, const TA* a, const TB* b, double* part, PCGState* st, int op, cudaStream_t s);
template <typename T>
void update_p(int64_t n, const T* z, T* p, const PCGState* st, cudaStream_t s);
// deflated search direction p = (z - mu w) + beta p, mu = st->wz * st->wawinv (FP32)
void update_p_corr(int64_t n, const float* z, const float* w, float* p, const PCGState* st,
                   cudaStream_t s);
// start of a deflated pass: gamma = st->wr * st->wawinv, d = gamma w,
// r -= gamma Aw (the residual orthogonal to w; FP32)
void deflate_start(int64_t n, const float* w, const float* aw, float* d, float* r,
                   const PCGState* st, cudaStream_t s);
// st->wawinv = v (one thread)
void set_correction(PCGState* st, double v, cudaStream_t s);
template <typename T>
void update_xr(int64_t n, const T* p, const T* q, T* x, T* r, double* part, PCGState* st,
               cudaStream_t s);
void pcg_reset(PCGState* st, cudaStream_t s);
void to_unit_f32(int64_t n, const double* r, const PCGState* st, float* r32, cudaStream_t s);
void add_scaled_f32(int64_t n, const float* d, const PCGState* st, double* x, cudaStream_t s);
template <typename T>
void scale_mul(int64_t n, double a, const T* d, const T* b, T* x, cudaStream_t s);
void d2f(int64_t n, const double* a, float* b, cudaStream_t s);
void edofmat(const Grid& g, int32_t* out, cudaStream_t st);

}  // namespace tg
