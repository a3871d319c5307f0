/*
 * topopt_gb300 -- C ABI of the GB300 (sm_103a) SIMP compliance-minimisation
 * library.  Plain pointers and sizes only; every host array is C-contiguous,
 * FP64 (double), int64 (indices) or int32/int8 as stated.
 *
 * The library is a drop-in for the per-iteration hot path of the reference
 * topoptlab driver (topoptlab/topology_optimization.py:411-673): SIMP
 * scaling, assembly + Dirichlet slicing + linear solve, compliance and
 * sensitivities, sensitivity / density filter, OC update, change / volume.
 * A context (tg_ctx) owns every device buffer of one problem and one CUDA
 * stream; it is not re-entrant, separate contexts may run concurrently.
 *
 * Return codes: TG_OK, or one of the TG_E* codes with a message available
 * from tg_last_error().  The Python wrapper maps TG_EINVAL to ValueError and
 * TG_ENOTCONV / TG_ETIMEOUT / TG_ENAN / TG_ECUDA to RuntimeError, like the
 * reference's ValueError("Unknown ...") (topology_optimization.py:262, :367)
 * and RuntimeError("... did not converge") (solve_linsystem.py:349-351).
 */
#ifndef TOPOPT_GB300_H
#define TOPOPT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TG_ABI_VERSION 6

enum {
  TG_OK = 0,
  TG_EINVAL = 1,     /* bad argument / unsupported combination */
  TG_ENOTCONV = 2,   /* PCG or OC bisection did not converge within its cap */
  TG_ETIMEOUT = 3,   /* a device loop hit its wall-clock limit */
  TG_ENAN = 4,       /* NaN / Inf in a residual or objective */
  TG_ECUDA = 5,      /* CUDA runtime error */
  TG_ENOMEM = 6
};

enum { TG_PREC_FP64 = 0, TG_PREC_MIXED = 1 };
enum { TG_LEARNED_WARM_START = 1, TG_LEARNED_COARSE_CORRECTION = 2 };
enum { TG_PRECOND_GMG = 0, TG_PRECOND_JACOBI = 1 };
enum {
  TG_FIELD_X = 0,      /* design variables x            (nel)  */
  TG_FIELD_XPHYS = 1,  /* physical densities xPhys      (nel)  */
  TG_FIELD_U = 2,      /* state (displacement / temp.)  (ndof) */
  TG_FIELD_DC = 3,     /* filtered objective sensitivity (nel) */
  TG_FIELD_DV = 4,     /* filtered volume sensitivity   (nel)  */
  TG_FIELD_F = 5       /* load vector                   (ndof) */
};

/* Problem description; mirrors the arguments of the reference main()
 * (topology_optimization.py:47-79) that the hot path consumes. */
typedef struct tg_problem {
  int32_t ndim;          /* 2 or 3 */
  int32_t nnode_dof;     /* 1 (Poisson) or ndim (elasticity) */
  int32_t nelx, nely, nelz;   /* nelz ignored for ndim == 2 */
  const double* KE;      /* element matrix, (2^ndim*nnode_dof)^2, row major,
                            reference local node order (lk(l=l) output) */
  const int64_t* fixed;  /* fixed DOF indices (bcs() output) */
  int64_t nfixed;
  const double* f;       /* load vector, ndof (bcs() output, one load case) */
  double volfrac, rmin, eps, penal, move;
  int32_t ft;            /* -1 none, 0 sensitivity filter, 1 density filter */
  const int8_t* el_flags;/* NULL or nel flags: 1 passive (0), 2 active (1) */
  int32_t precond;       /* TG_PRECOND_* */
  int32_t precision;     /* TG_PREC_* */
  int32_t nlevels;       /* multigrid levels, 0 = automatic */
  int32_t nsmooth;       /* damped-Jacobi sweeps before / after (default 2) */
  double omega;          /* Jacobi damping (default 0.6) */
  double rtol;           /* FP64 relative residual target (default 1e-8) */
  int32_t maxiter;       /* PCG iteration cap (default 2000) */
  double inner_rtol;     /* mixed precision: FP32 inner solve target (1e-4) */
  int32_t learned;       /* bit mask, used once a trained network is attached
                            (tg_cnn_attach): TG_LEARNED_WARM_START = the
                            network's warm start, TG_LEARNED_COARSE_CORRECTION
                            = its vector as the deflation vector of the mixed
                            solver's FP32 PCG; 0 = the warm start alone once a
                            network is attached */
  int32_t device;        /* CUDA device ordinal */
  int32_t nload;         /* load cases (columns of bcs()'s f, topology_optimization.py:
                            463-500): f holds nload vectors of ndof one after another;
                            0 or 1 = one load case */
  int32_t filter_pde;    /* 1: Helmholtz PDE filter for ft 0/1 instead of the distance
                            filter (topology_optimization.py:360-365, 554-555, 568-570,
                            646-647; filter/helmholtz_filter.py:133-200) */
  const double* KF;      /* filter_pde: screened Poisson element matrix, (2^ndim)^2 row
                            major, reference local node order (lk_screened_poisson_2d/_3d
                            with k = (rmin / (2 sqrt 3))^2, elements/screenedpoisson_2d.py:8) */
  int32_t unsmoothed;    /* multigrid: bit l set (0 < l < nlevels - 1) = level l is not
                            smoothed: its right-hand side is restricted on as it is and
                            the coarser correction prolongated back (the Galerkin coarse
                            correction through the composite interpolation of levels
                            l-1 -> l+1); 0 = every level smoothed (TG_EINVAL for other
                            bits) */
  int32_t nsmooth_coarse;/* multigrid: damped-Jacobi sweeps before / after on the coarse
                            levels (1 .. nlevels-2); 0 = nsmooth */
} tg_problem;

typedef struct tg_iter_out {
  double obj;            /* compliance of the design that was solved */
  double vol;            /* mean(xPhys) after the update */
  double change;         /* max |x_new - x_old| */
  double g;              /* OC carry (optimality_criterion.py:73) */
  double rel_res;        /* true FP64 ||f - K u|| / ||f|| after the solve */
  int32_t pcg_iters;     /* (inner) PCG iterations */
  int32_t vcycles;       /* V-cycles applied */
  int32_t refinements;   /* FP64 refinement steps (mixed precision) */
  int32_t oc_steps;      /* OC bisection steps */
  int32_t fallback;      /* 1 if the learned warm start was rejected */
  int32_t nlevels;       /* multigrid levels used */
  double t_solve_ms;     /* device time of the linear solve */
  double t_step_ms;      /* host wall time of the whole step */
  double warm_ratio;     /* learned warm start: FP64 residual norm of the learned
                            start over the plain start's (u_prev); 0 without one */
} tg_iter_out;

typedef struct tg_solve_info {
  int32_t iters, vcycles, refinements, converged;
  double rel_res;
} tg_solve_info;

typedef struct tg_ctx tg_ctx;

int32_t tg_abi_version(void);

/* Message of the last failing call on ctx, or of the last failing
 * tg_create / context-free call when ctx is NULL. */
const char* tg_last_error(const tg_ctx* ctx);

/* Replaces the set-up half of main() (topology_optimization.py:203-409):
 * element matrix, edofMat (implicit), filter, BCs, initial design x = volfrac.*/
int32_t tg_create(const tg_problem* prob, tg_ctx** out);
void tg_destroy(tg_ctx* ctx);

/* One design iteration (topology_optimization.py:411-673, OC branch). */
int32_t tg_step(tg_ctx* ctx, tg_iter_out* out);

/* One design iteration of each of n independent contexts (a batch of
 * designs, e.g. heat plates of different sizes), run concurrently by
 * nthreads host threads (<= 0: min(n, 16)), each context on its own CUDA
 * stream.  Each context's result equals its own tg_step.  rcs[i] receives
 * the status of ctxs[i]; the return value is the first non-OK status (or OK).
 * No reference counterpart: the reference runs one design per process. */
int32_t tg_step_many(tg_ctx* const* ctxs, int32_t n, tg_iter_out* outs, int32_t* rcs,
                     int32_t nthreads);

/* Host <-> device copies of a field (TG_FIELD_*), n = number of doubles. */
int32_t tg_get(tg_ctx* ctx, int32_t field, double* host, int64_t n);
int32_t tg_set(tg_ctx* ctx, int32_t field, const double* host, int64_t n);

/* Unit entry points (host buffers), used by the solve_lin / filter / OC /
 * objective mirrors and by the tests. */
/* y = M K(xPhys) M u  (fem.py:141-237 + SpMV); precision TG_PREC_FP64 or
 * TG_PREC_MIXED (FP32 arithmetic, result widened to FP64). */
int32_t tg_kmul(tg_ctx* ctx, const double* xPhys, const double* u, double* y, int32_t precision);
/* K u = rhs on the free DOFs (solve_linsystem.py:20-365 slot).  u0 may be NULL. */
int32_t tg_solve(tg_ctx* ctx, const double* xPhys, const double* rhs, const double* u0, double* u,
                 tg_solve_info* info);
/* Adjoint solve and sensitivity of an objective that is not self-adjoint
 * (topology_optimization.py:473-500): adj = K^-1 rhs_adj on the free DOFs,
 * with the scale factors, multigrid hierarchy and coarsest inverse of the
 * last state solve (tg_step or tg_solve) -- nothing is rebuilt, as the
 * reference reuses its factorisation / preconditioner -- and, when dobj is
 * not NULL, dobj_e = simp_dx(xPhys_e) adj_e^T KE u_e for the design of that
 * solve (the reference's dobj accumulation).  u: the state of that solve
 * (ndof); rhs_adj: the objective's adjoint right-hand side (the reference
 * objectives' rhs_adj, e.g. objectives.py:121-157).  Not for padded grids. */
int32_t tg_adjoint(tg_ctx* ctx, const double* u, const double* rhs_adj, double* adj, double* dobj,
                   tg_solve_info* info);
/* PCG on an assembled CSR matrix (indptr int64 [n+1], indices int32, data
 * FP64), Jacobi-preconditioned when jacobi != 0, stopping at
 * ||b - A x|| < max(atol, rtol ||b||): the pcg / solve_lin path for callers
 * that pass an assembled matrix (linear_solvers.py:50-136,
 * solve_linsystem.py:341-352).  x0 may be NULL.  Errors: tg_csr_last_error(). */
int32_t tg_csr_pcg(int64_t n, const int64_t* indptr, const int32_t* indices, const double* data,
                   const double* rhs, const double* x0, double* x, double rtol, double atol,
                   int32_t maxiter, int32_t jacobi, tg_solve_info* info, int32_t device);
const char* tg_csr_last_error(void);
/* mode 0: (H x)/Hs   1: H(x/Hs)   2: H(x*d)/Hs/max(1e-3,x)   3: Hs
 * (filter/matrix_filter.py:101-232 + topology_optimization.py:545-558, :639)
 * contexts with filter_pde:  6: TF^T KF^-1 TF x   7: TF^T KF^-1 TF (x*d) / max(1e-3,x)
 * (topology_optimization.py:555, :569, :647) */
int32_t tg_filter(tg_ctx* ctx, const double* x, const double* d, double* y, int32_t mode);
/* obj = sum simp(xPhys) u_e^T KE u_e, dc = -simp_dx(xPhys) u_e^T KE u_e
 * (objectives.py:51-55, topology_optimization.py:491-500) */
int32_t tg_compliance(tg_ctx* ctx, const double* xPhys, const double* u, double* obj, double* dc);
/* oc_top88 (optimizer/optimality_criterion.py:9-79) */
int32_t tg_oc(tg_ctx* ctx, const double* x, const double* dc, const double* dv, double g,
              double* xnew, double* gt, int32_t* nsteps);
/* oc_top88 without a context: n design variables, optional el_flags (int8,
 * 1 passive, 2 active), bisection bounds l1 < l2 */
int32_t tg_oc_raw(int64_t n, const double* x, const double* dc, const double* dv, double g,
                  const int8_t* el_flags, double move, double l1, double l2, double* xnew,
                  double* gt, int32_t* nsteps, int32_t device);
/* Allocation-free OC update.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory themselves -- applications
 * whose device memory belongs to their own pool allocator, or code that must
 * not change the device's allocation state while its other work runs.  x, dc,
 * dv, el_flags (may be NULL) and xnew are DEVICE pointers owned by the caller;
 * gt and nsteps are host pointers.  The only extra device memory is a static
 * array inside the library sized for TG_NOALLOC_MAX_N design variables; larger
 * n returns TG_EINVAL.  The array is shared by all calls and keeps the last
 * call's contents, so calls that overlap on the GPU race and must be
 * serialised by the caller.  Every call looks up the array's device address
 * on the current device and synchronises stream before it returns, so it
 * must never be called while stream is being captured into a CUDA graph
 * (refused with TG_EINVAL).  stream is a cudaStream_t (NULL = legacy default
 * stream).  Errors: message from tg_noalloc_last_error(). */
#define TG_NOALLOC_MAX_N 2097152
int32_t tg_oc_noalloc(int64_t n, const double* x, const double* dc, const double* dv, double g,
                      const int8_t* el_flags, double move, double l1, double l2, double* xnew,
                      double* gt, int32_t* nsteps, void* stream);
const char* tg_noalloc_last_error(void);
/* one multigrid V-cycle x = V(b) for the densities xPhys */
int32_t tg_vcycle(tg_ctx* ctx, const double* xPhys, const double* b, double* x, int32_t precision);
/* number of multigrid levels and the DOF count of one level */
int32_t tg_levels(tg_ctx* ctx, int32_t* nlevels, int64_t* ndofs_per_level /* >= 8 entries */);
/* assembled stencil of level >= 1 for the densities xPhys, layout
 * [(dir*ndof+ci)*ndof+cj][node], n = 3^ndim*ndof^2*nnodes(level) */
int32_t tg_coarse_stencil(tg_ctx* ctx, const double* xPhys, int32_t level, double* out, int64_t n);
/* Learned warm start (no counterpart in the reference: new capability of the
 * GB300 solver).  A 3-level 3-D convolutional encoder-decoder (16/32/64
 * channels, FP32) on the context's multigrid level-1 node grid predicts a
 * level-1 displacement correction y from the filtered density, the previous
 * displacement and the residual of the previous displacement restricted to
 * the level-1 grid.  w = P y (prolongated to the fine grid) gives the warm
 * start, the energy-optimal combination c1 u_prev + c2 w, and optionally
 * (TG_LEARNED_COARSE_CORRECTION) the deflation vector of the mixed solver's
 * FP32 PCG, a coarse-grid correction by one extra basis vector.  After the
 * first cycle of the solve, tg_step compares the residual with the plain
 * warm start's (u_prev); when it is not below, the step falls back to plain
 * PCG from u_prev (tg_iter_out.fallback = 1).  The network runs on its own
 * CUDA stream, overlapping the build of the multigrid hierarchy.  Training
 * runs on the GPU with the library's own forward / backward / Adam kernels. */
typedef struct tg_cnn tg_cnn;
/* network for ctx (3-D elasticity, >= 2 multigrid levels); capacity = number
 * of training samples to hold; seed = weight initialisation */
int32_t tg_cnn_create(tg_ctx* ctx, int32_t capacity, uint64_t seed, tg_cnn** out);
void tg_cnn_destroy(tg_cnn* cnn);
/* use cnn for the warm starts (and coarse-grid corrections) of ctx's tg_step
 * (NULL detaches); the parts used are tg_problem.learned's bits, the warm
 * start alone when it was 0 */
int32_t tg_cnn_attach(tg_ctx* ctx, tg_cnn* cnn);
/* record one training pair around a tg_step of ctx: begin (features of the
 * current design and displacement) before the step, end (target = new -
 * previous displacement) after it; ctx is the network's own context or any
 * mixed-precision context on the same device with the same grids (runs of
 * other volume fractions or start designs) */
int32_t tg_cnn_record_begin(tg_cnn* cnn, tg_ctx* ctx);
int32_t tg_cnn_record_end(tg_cnn* cnn, tg_ctx* ctx);
/* Adam (lr, beta 0.9 / 0.999) over the recorded pairs; final mean loss */
int32_t tg_cnn_train(tg_cnn* cnn, int32_t epochs, double lr, uint64_t seed, double* final_loss);
/* Adam (lr, beta 0.9 / 0.999, continuing the network's optimiser state) over
 * n caller-provided pairs: host features x0s [n][nodes][7] and targets
 * [n][nodes][3], one step per pair, pairs in a seeded shuffled order per
 * epoch; final mean loss */
int32_t tg_cnn_fit(tg_cnn* cnn, int32_t n, const float* x0s, const float* targets, int32_t epochs,
                   double lr, uint64_t seed, double* final_loss);
/* parameter count, level-1 grid (nx, ny, nz), recorded samples */
int32_t tg_cnn_info(tg_cnn* cnn, int64_t* nparams, int32_t* grid_dims, int32_t* nsamples);
/* copy the flat parameter vector out (set = 0) or in (set = 1) */
int32_t tg_cnn_params(tg_cnn* cnn, int32_t set, float* host, int64_t n);
/* forward pass on host features x0 [nodes][7] -> y [nodes][3]; with a target
 * also the MSE loss and the parameter gradient (host buffers, y / loss /
 * grads may be NULL) */
int32_t tg_cnn_eval(tg_cnn* cnn, const float* x0, const float* target, float* y, double* loss,
                    float* grads);
/* the forward pass as the warm start runs it (single TF32 products instead of
 * the split FP32-level ones of tg_cnn_eval): host x0 [nodes][7] -> y [nodes][3] */
int32_t tg_cnn_infer(tg_cnn* cnn, const float* x0, float* y);
/* Device time between two calls on the context's stream: op 0 records the
 * start event, op 1 records the stop event, synchronises and writes the
 * elapsed milliseconds to *ms. */
int32_t tg_timer(tg_ctx* ctx, int32_t op, double* ms);
/* Event timing of one kernel family (0 off, 1 fine FP64 K.u, 2 fine FP32
 * K.u, 3 fine FP32 K.u with BF16 densities, 4 FP32 coarse stencil (levels
 * >= 2), 5 FP64 coarse stencil, 6 filter, 7 OC step, 8 FP32 level-1
 * stencil, 9 coarse operator build, 10 coarsest inverse, 11 vector kernels,
 * 12 transfers, 13 compliance, 14 learned warm start, 15 the V-cycle's
 * cooperative bottom); resets the accumulated time. */
int32_t tg_profile_kernel(int32_t kind);
/* Kernel launches made by the library (all contexts) and the accumulated
 * device time / launch count of the profiled family; reset != 0 zeroes them. */
int32_t tg_stats(int32_t reset, int64_t* launches, double* prof_ms, int64_t* prof_launches);
/* Library-wide switches for tests and tuning (no counterpart in the
 * reference).  TG_TUNE_STENCIL_SMALL_PAIRS: coarse levels with fewer
 * (node, DOF) rows than value run the small-grid stencil kernel, the others
 * the row-plane kernel (default 150000; 0 runs the row-plane kernel on every
 * level, so tests can compare it with the oracle on small grids).
 * TG_TUNE_OC_BARRIER_TIMEOUT: value != 0 makes the next OC bisection's grid
 * barrier wait for one block more than its grid holds, so every block's
 * bounded wait runs out (seconds) and the call returns TG_ETIMEOUT;
 * the switch clears itself.  TG_TUNE_COARSE_TAIL: value 1 runs the bottom
 * of every V-cycle -- restriction into the last smoothed level, its sweeps,
 * the coarsest dense solve and both prolongations -- as one launch of one
 * thread-block cluster (up to 16 CTAs, hardware cluster barriers between
 * the phases); 2 as one cooperative launch with bounded grid barriers, one
 * block per SM (value > 2: that many blocks); 0 runs the separate kernels.
 * Same arithmetic, same results.
 * TG_TUNE_STENCIL_TMA: value 1 runs the FP32 3-D coarse sweeps of levels
 * too large for the small-grid kernel with TMA-staged coefficients (value
 * > 1: at most value - 1 node rows per CTA); 0 (default) runs the
 * register-path kernel.  Same results.
 * TG_TUNE_PDL: value != 0 (default) launches the kernels of the PCG iteration
 * with programmatic dependent launch (a kernel is scheduled while its
 * predecessor finishes and waits for it before touching memory); 0 launches
 * them one after another.  Same results.
 * TG_TUNE_TAIL_BARRIER_TIMEOUT:
 * like TG_TUNE_OC_BARRIER_TIMEOUT for the next such launch (the solve or
 * tg_vcycle call returns TG_ETIMEOUT).  TG_TUNE_CONV_UMMA: value != 0
 * (default) runs the learned warm start's TF32 inference convolutions on the
 * 5th-generation tensor cores (tcgen05, accumulators in tensor memory); 0 on
 * warp-level mma.sync.  Both round the operands to TF32 the same way and
 * accumulate in FP32 in the same order (bit-identical outputs).  TG_TUNE_CONV_TIMEOUT:
 * value != 0 makes one CTA of the next tensor-core convolution launch wait on
 * a barrier phase that never completes, so its bounded wait runs out (about
 * a second), it frees its tensor memory and leaves, and the call that ran the
 * launch returns TG_ETIMEOUT; the switch clears itself.
 * Unknown keys return TG_EINVAL. */
enum {
  TG_TUNE_STENCIL_SMALL_PAIRS = 1,
  TG_TUNE_OC_BARRIER_TIMEOUT = 2,
  TG_TUNE_COARSE_TAIL = 3,
  TG_TUNE_TAIL_BARRIER_TIMEOUT = 4,
  TG_TUNE_STENCIL_TMA = 5,
  TG_TUNE_PDL = 6,
  TG_TUNE_CONV_UMMA = 7,
  TG_TUNE_CONV_TIMEOUT = 8
};
int32_t tg_tune(int32_t key, int64_t value);
/* edofMat (elements/bilinear_quadrilateral.py:7-48, trilinear_hexahedron.py:7-58)
 * generated on the device; out has nel*(2^ndim*nnode_dof) int32 entries */
/* Inverse of a dense SPD matrix A (row-major n x n, n <= 8192) by the
 * library's coarsest-level method, the symmetric block sweep operator:
 * mode 0 in FP64, mode 1 in double-word FP32 arithmetic (about 48
 * significant bits; what mixed-precision contexts use: each step's update
 * launch also forms the next step's panel), mode 2 the same double-word
 * sweep with panel and update as separate launches (same result as mode 1).
 * Diagnostic (no reference counterpart); synchronous. */
int32_t tg_dense_inverse(const double* A, int64_t n, double* Ainv, int32_t mode, int32_t device);
int32_t tg_edofmat(int32_t ndim, int32_t nelx, int32_t nely, int32_t nelz, int32_t nnode_dof,
                   int32_t* out, int32_t device);

#ifdef __cplusplus
}
#endif
#endif /* TOPOPT_GB300_H */
