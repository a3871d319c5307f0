// Jacobi-preconditioned CG on an assembled CSR matrix, for callers of the
// solve_lin / pcg interface that hand over an assembled operator
// (solve_linsystem.py:20-365, linear_solvers.py:50-136) instead of a
// structured-grid problem.  FP64 throughout, PCG exactly as the reference
// (r = b - A x; z = D^-1 r; rho = r.z; ... ; stop when ||r|| < rtol ||b||).
#include <algorithm>
#include <cmath>
#include <vector>
#include "tg_ctx.cuh"
#include "../../include/topopt_gb300.h"

namespace tg {

// y = A x, one warp per row
__global__ void k_csr_spmv(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                           const double* __restrict__ val, const double* __restrict__ x,
                           double* __restrict__ y) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  double s = 0.0;
  for (int64_t k = ptr[row] + lane; k < ptr[row + 1]; k += 32) s += val[k] * x[idx[k]];
  s = warp_sum(s);
  if (lane == 0) y[row] = s;
}

__global__ void k_csr_diag_inv(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                               const double* __restrict__ val, double* __restrict__ dinv) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= n) return;
  double d = 0.0;
  for (int64_t k = ptr[row]; k < ptr[row + 1]; ++k)
    if (idx[k] == row) d += val[k];
  dinv[row] = d != 0.0 ? 1.0 / d : 0.0;
}

__global__ void k_sub(int64_t n, const double* a, const double* b, double* c) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) c[i] = a[i] - b[i];
}

}  // namespace tg

namespace {
thread_local std::string g_csr_err;
}

extern "C" {

const char* tg_csr_last_error(void) { return g_csr_err.c_str(); }

int32_t tg_csr_pcg(int64_t n, const int64_t* indptr, const int32_t* indices, const double* data,
                   const double* rhs, const double* x0, double* x, double rtol, double atol,
                   int32_t maxiter, int32_t jacobi, tg_solve_info* info, int32_t device) {
  using namespace tg;
  if (n <= 0 || !indptr || !indices || !data || !rhs || !x) {
    g_csr_err = "tg_csr_pcg: bad arguments";
    return TG_EINVAL;
  }
  try {
    TG_CUDA(cudaSetDevice(device));
    cudaStream_t st = 0;
    const int64_t nnz = indptr[n];
    DevBuf<int64_t> ptr;
    DevBuf<int32_t> idx;
    DevBuf<double> val, b, xd, r, z, p, q, dinv, part;
    DevBuf<PCGState> ps;
    ptr.alloc(n + 1); idx.alloc(nnz); val.alloc(nnz);
    b.alloc(n); xd.alloc(n); r.alloc(n); z.alloc(n); p.alloc(n); q.alloc(n); dinv.alloc(n);
    part.alloc(RED_BLOCKS); ps.alloc(1);
    TG_CUDA(cudaMemcpy(ptr.p, indptr, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    TG_CUDA(cudaMemcpy(idx.p, indices, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
    TG_CUDA(cudaMemcpy(val.p, data, sizeof(double) * nnz, cudaMemcpyHostToDevice));
    TG_CUDA(cudaMemcpy(b.p, rhs, sizeof(double) * n, cudaMemcpyHostToDevice));
    if (x0) TG_CUDA(cudaMemcpy(xd.p, x0, sizeof(double) * n, cudaMemcpyHostToDevice));
    else TG_CUDA(cudaMemset(xd.p, 0, sizeof(double) * n));
    const unsigned wb = (unsigned)cdiv(n * 32, 256), eb = (unsigned)cdiv(n, 256);
    k_csr_diag_inv<<<eb, 256, 0, st>>>(n, ptr, idx, val, dinv);
    TG_CHECK_LAUNCH();
    PCGState h{};
    auto read = [&] {
      TG_CUDA(cudaMemcpy(&h, ps.p, sizeof(PCGState), cudaMemcpyDeviceToHost));
    };
    pcg_reset(ps, st);
    dot<double, double>(n, b.p, b.p, part, ps, DOT_BB, st);
    read();
    const double tol = std::max(atol, rtol * std::sqrt(h.bb));
    k_csr_spmv<<<wb, 256, 0, st>>>(n, ptr, idx, val, xd, q);
    TG_CHECK_LAUNCH();
    k_sub<<<eb, 256, 0, st>>>(n, b, q, r);
    TG_CHECK_LAUNCH();
    pcg_reset(ps, st);
    dot<double, double>(n, r.p, r.p, part, ps, DOT_RR, st);
    read();
    int it = 0;
    bool conv = std::sqrt(h.rr) < tol;
    while (!conv && it < maxiter) {
      if (jacobi) scale_mul<double>(n, 1.0, dinv.p, r.p, z.p, st);
      else TG_CUDA(cudaMemcpyAsync(z.p, r.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      dot<double, double>(n, r.p, z.p, part, ps, DOT_RHO, st);
      update_p<double>(n, z.p, p.p, ps, st);
      k_csr_spmv<<<wb, 256, 0, st>>>(n, ptr, idx, val, p, q);
      TG_CHECK_LAUNCH();
      dot<double, double>(n, p.p, q.p, part, ps, DOT_ALPHA, st);
      update_xr<double>(n, p.p, q.p, xd.p, r.p, part, ps, st);
      ++it;
      read();
      if (!std::isfinite(h.rr)) throw Error{ENAN, "tg_csr_pcg: non-finite residual"};
      conv = std::sqrt(h.rr) < tol;
    }
    TG_CUDA(cudaMemcpy(x, xd.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (info) {
      info->iters = it;
      info->vcycles = 0;
      info->refinements = 0;
      info->converged = conv;
      info->rel_res = h.bb > 0 ? std::sqrt(h.rr / h.bb) : 0.0;
    }
    if (!conv) {
      g_csr_err = "pcg iteration did not converge";
      return TG_ENOTCONV;
    }
    return TG_OK;
  } catch (const Error& e) {
    g_csr_err = e.msg;
    return e.code;
  }
}

}  // extern "C"
