// Helmholtz PDE filter (filter/helmholtz_filter.py:133-200, applied as in
// topology_optimization.py:554-555, 568-570, 646-647):
//
//   y = TF^T KF^-1 TF v
//
// TF spreads each element value over the element's 2^d nodes with weight
// 2^-d; KF is the screened Poisson operator (Laplacian scaled by
// k = (rmin / (2 sqrt 3))^2 plus the consistent mass matrix) with no boundary
// conditions.  KF is the stiffness operator of a scalar problem on the same
// device grid with unit densities, so it is solved by a second context of
// this library: FP64 matrix-free multigrid PCG on one DOF per node.  KF never
// changes, so that context's hierarchy (Galerkin coarse operators, coarsest
// inverse) is built once, where the reference factorises KF once
// (topology_optimization.py:365).  The solve runs to a relative residual of
// 1e-12 so that filtered fields agree with the factorised solve to ~1e-12.
#include "tg_ctx.cuh"

namespace tg {

// rhs = TF (v * mul) on the nodes; padding elements contribute nothing and
// fixed (padding) nodes get 0
template <int NDIM>
__global__ void k_tf(Grid g, const double* __restrict__ v, const double* __restrict__ mul,
                     const int8_t* __restrict__ flags, const uint8_t* __restrict__ fix,
                     double* __restrict__ rhs) {
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= g.nnodes()) return;
  const int y = (int)(n % g.nny), x = (int)((n / g.nny) % g.nnx);
  const int z = (int)(n / ((int64_t)g.nny * g.nnx));
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < (1 << NDIM); ++c) {
    const int ex = x - (c & 1), ey = y - ((c >> 1) & 1), ez = (NDIM == 3) ? z - (c >> 2) : 0;
    if (ex < 0 || ey < 0 || ez < 0 || ex >= g.nex || ey >= g.ney || ez >= g.nez) continue;
    const int64_t e = g.elem(ex, ey, ez);
    if (flags && flags[e] == EL_OUTSIDE) continue;
    s += mul ? v[e] * mul[e] : v[e];
  }
  rhs[n] = fix[n] ? 0.0 : s * (NDIM == 3 ? 0.125 : 0.25);
}

// y = TF^T u per element (divided by max(1e-3, xdiv) for the ft=0 form);
// optionally the fused sums of the density filter: sum y and max |x - xold|
template <int NDIM>
__global__ void __launch_bounds__(RED_THREADS)
k_tft(Grid g, const double* __restrict__ u, const double* __restrict__ xdiv,
      const int8_t* __restrict__ flags, double* __restrict__ y, const double* __restrict__ x,
      const double* __restrict__ xold, double* part_sum, double* part_max) {
  __shared__ double sh[32];
  const int64_t nel = g.nel();
  double psum = 0.0, pmax = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nel;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (flags && flags[e] == EL_OUTSIDE) {
      y[e] = 0.0;
      continue;
    }
    const int ey = (int)(e % g.ney), ex = (int)((e / g.ney) % g.nex);
    const int ez = (int)(e / ((int64_t)g.ney * g.nex));
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < (1 << NDIM); ++c)
      s += u[g.node(ex + (c & 1), ey + ((c >> 1) & 1), NDIM == 3 ? ez + (c >> 2) : 0)];
    double out = s * (NDIM == 3 ? 0.125 : 0.25);
    if (xdiv) out /= fmax(0.001, xdiv[e]);
    y[e] = out;
    psum += out;
    if (xold) pmax = fmax(pmax, fabs(x[e] - xold[e]));
  }
  if (part_sum) {
    const double s = block_sum(psum, sh);
    if (threadIdx.x == 0) part_sum[blockIdx.x] = s;
  }
  if (part_max) {
    const double m = block_max(pmax, sh);
    if (threadIdx.x == 0) part_max[blockIdx.x] = m;
  }
}

void helmholtz_init(Ctx& c, const double* KF) {
  TG_REQUIRE(KF != nullptr, "filter_pde needs the screened Poisson element matrix KF");
  TG_REQUIRE(c.ft == 0 || c.ft == 1, "the Helmholtz filter applies to ft 0 and 1");
  const Grid& g = c.g;
  const Grid& rg = c.rg;
  // the filter problem lives on the device grid itself: on a padded grid the
  // padding elements are outside and the padding nodes fixed, as for the
  // physics problem, so its context needs no padding of its own
  std::vector<int64_t> fixed;
  std::vector<int8_t> fl;
  if (c.padded) {
    for (int z = 0; z < g.nnz; ++z)
      for (int x = 0; x < g.nnx; ++x)
        for (int y = 0; y < g.nny; ++y)
          if (x >= rg.nnx || y >= rg.nny || z >= rg.nnz) fixed.push_back(g.node(x, y, z));
    fl.assign(g.nel(), 0);
    for (int ez = 0; ez < g.nez; ++ez)
      for (int ex = 0; ex < g.nex; ++ex)
        for (int ey = 0; ey < g.ney; ++ey)
          if (ex >= rg.nex || ey >= rg.ney || ez >= rg.nez) fl[g.elem(ex, ey, ez)] = EL_OUTSIDE;
  }
  std::vector<double> zero(g.nnodes(), 0.0);
  ::tg_problem q{};
  q.ndim = g.ndim;
  q.nnode_dof = 1;
  q.nelx = g.nex; q.nely = g.ney; q.nelz = g.ndim == 3 ? g.nez : 0;
  q.KE = KF;
  q.fixed = fixed.data(); q.nfixed = (int64_t)fixed.size();
  q.f = zero.data();
  // unit densities with eps = 0 and penalty 1: every element scale is exactly 1
  q.volfrac = 1.0; q.rmin = 1.0; q.eps = 0.0; q.penal = 1.0; q.move = 0.2;
  q.ft = -1;
  q.el_flags = c.padded ? fl.data() : nullptr;
  q.precond = c.precond;
  q.precision = TG_PREC_FP64;
  q.nlevels = c.precond == TG_PRECOND_GMG ? c.L : 0;   // the physics grid's hierarchy depth
  q.nsmooth = c.nsmooth; q.omega = c.omega;
  q.rtol = 1e-12; q.maxiter = 2000;
  q.device = c.dev;
  q.nload = 1;
  c.hf = new Ctx();
  ctx_init(*c.hf, q);
  Ctx& h = *c.hf;
  TG_REQUIRE(!h.padded && h.g.nex == g.nex && h.g.ney == g.ney && h.g.nez == g.nez,
             "Helmholtz filter grid differs from the design grid");
  set_density(h, h.xPhys);
  build_hierarchy(h);
  TG_CUDA(cudaEventCreateWithFlags(&c.hev0, cudaEventDisableTiming));
  TG_CUDA(cudaEventCreateWithFlags(&c.hev1, cudaEventDisableTiming));
  TG_CUDA(cudaStreamSynchronize(h.st));
}

void helmholtz_apply(Ctx& c, const double* v, const double* mul, const double* xdiv, double* y,
                     const double* x, const double* xold, double* part_sum, double* part_max) {
  Ctx& h = *c.hf;
  const Grid& g = c.g;
  ProfScope ps(PK_FILTER, c.st);
  // the filter context has its own stream: order it after the caller's work
  TG_CUDA(cudaEventRecord(c.hev0, c.st));
  TG_CUDA(cudaStreamWaitEvent(h.st, c.hev0, 0));
  const unsigned nb = (unsigned)cdiv(g.nnodes(), 256);
  if (g.ndim == 3) k_tf<3><<<nb, 256, 0, h.st>>>(g, v, mul, c.flags.p, h.op.fix, h.f.p);
  else k_tf<2><<<nb, 256, 0, h.st>>>(g, v, mul, c.flags.p, h.op.fix, h.f.p);
  TG_CHECK_LAUNCH();
  h.u.zero(h.st);
  solve(h, h.f.p, h.u.p);
  c.filter_iters += h.last_iters;
  const unsigned rb = red_blocks(g.nel());
  if (g.ndim == 3)
    k_tft<3><<<rb, RED_THREADS, 0, h.st>>>(g, h.u, xdiv, c.flags.p, y, x, xold, part_sum, part_max);
  else
    k_tft<2><<<rb, RED_THREADS, 0, h.st>>>(g, h.u, xdiv, c.flags.p, y, x, xold, part_sum, part_max);
  TG_CHECK_LAUNCH();
  TG_CUDA(cudaEventRecord(c.hev1, h.st));
  TG_CUDA(cudaStreamWaitEvent(c.st, c.hev1, 0));
}

}  // namespace tg
