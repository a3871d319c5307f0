// Problem set-up, multigrid hierarchy, PCG drivers and the design step.
//
// The design step follows topology_optimization.py:411-673 (OC branch):
// scale -> solve -> compliance/sensitivity -> sensitivity filter -> OC ->
// density filter -> change/volume.  Every array stays on the device; the
// host reads back four scalars per step.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include "tg_ctx.cuh"
#include "tg_cnn.cuh"
#include "../../include/topopt_gb300.h"

namespace tg {

Ctx::~Ctx() {
  if (g64.exec) cudaGraphExecDestroy(g64.exec);
  if (g32.exec) cudaGraphExecDestroy(g32.exec);
  for (LoopGraph* l : {&l64, &l32}) {
    if (l->exec) cudaGraphExecDestroy(l->exec);
    if (l->graph) cudaGraphDestroy(l->graph);
  }
  for (Level* l : lv) delete l;
  delete hf;
  if (hev0) cudaEventDestroy(hev0);
  if (hev1) cudaEventDestroy(hev1);
  if (h_oc) cudaFreeHost(h_oc);
  if (h_pcg) cudaFreeHost(h_pcg);
  if (h_scal) cudaFreeHost(h_scal);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (tev0) cudaEventDestroy(tev0);
  if (tev1) cudaEventDestroy(tev1);
  if (side) {
    cudaStreamSynchronize(side);
    cudaStreamDestroy(side);
  }
  if (sev_fork) cudaEventDestroy(sev_fork);
  if (sev_join) cudaEventDestroy(sev_join);
  if (st) cudaStreamDestroy(st);
}

// reference local node order -> corner bits (dx | dy<<1 | dz<<2)
static int corner_bits(int k, int ndim) {
  static const int lx[4] = {0, 1, 1, 0}, ly[4] = {1, 1, 0, 0};
  const int dz = (ndim == 3) ? (k >> 2) : 0;
  return lx[k & 3] | (ly[k & 3] << 1) | (dz << 2);
}

static void setup_element(Ctx& c, const double* KEref) {
  const int nd = c.g.ndim, nf = c.g.ndof, NC = 1 << nd, NE = NC * nf;
  c.ne = NE;
  // permute to corner-bit order
  std::vector<int> perm(NE);   // bit index -> reference index
  for (int k = 0; k < NC; ++k)
    for (int q = 0; q < nf; ++q) perm[corner_bits(k, nd) * nf + q] = k * nf + q;
  c.KEh.assign(NE * NE, 0.0);
  for (int i = 0; i < NE; ++i)
    for (int j = 0; j < NE; ++j) c.KEh[i * NE + j] = KEref[perm[i] * NE + perm[j]];
  // sector blocks  B = H KE H / 4^nd
  std::vector<double> B(NE * NE, 0.0);
  auto hsign = [](int s, int d) { return (__builtin_popcount(s & d) & 1) ? -1.0 : 1.0; };
  double bmax = 0.0;
  for (int s = 0; s < NC; ++s)
    for (int a = 0; a < nf; ++a)
      for (int t = 0; t < NC; ++t)
        for (int b = 0; b < nf; ++b) {
          double acc = 0.0;
          for (int d = 0; d < NC; ++d)
            for (int e = 0; e < NC; ++e)
              acc += hsign(s, d) * c.KEh[(d * nf + a) * NE + e * nf + b] * hsign(t, e);
          acc /= (double)(NC * NC);
          B[(s * nf + a) * NE + t * nf + b] = acc;
          bmax = std::max(bmax, std::fabs(acc));
        }
  auto sigf = [&](int chi, int q) { return (nf == nd) ? (chi ^ (1 << q)) : chi; };
  const bool vec_ok = (nf == nd) || (nf == 1);
  double off = 0.0;
  for (int s = 0; s < NC; ++s)
    for (int a = 0; a < nf; ++a)
      for (int t = 0; t < NC; ++t)
        for (int b = 0; b < nf; ++b) {
          const int chi1 = (nf == nd) ? (s ^ (1 << a)) : s;
          const int chi2 = (nf == nd) ? (t ^ (1 << b)) : t;
          if (chi1 != chi2) off = std::max(off, std::fabs(B[(s * nf + a) * NE + t * nf + b]));
        }
  c.op.sector = vec_ok && off <= 1e-12 * bmax;
  std::memset(&c.op.B64, 0, sizeof(c.op.B64));
  std::memset(&c.op.B32, 0, sizeof(c.op.B32));
  // hex8 elasticity: does the block zero pattern match the reference element's?
  bool hex8 = c.op.sector && nd == 3 && nf == 3;
  if (hex8)
    for (int chi = 0; chi < NC; ++chi)
      for (int a = 0; a < nf; ++a)
        for (int b = 0; b < nf; ++b) {
          const double v = B[(sigf(chi, a) * nf + a) * NE + sigf(chi, b) * nf + b];
          const bool nz = std::fabs(v) > 1e-12 * bmax;
          if (nz != (((hex8_mask(chi) >> (a * 3 + b)) & 1u) != 0)) hex8 = false;
        }
  c.op.kind = !c.op.sector ? EK_DENSE : (hex8 ? EK_SECTOR_HEX8 : EK_SECTOR);
  if (c.op.sector)
    for (int chi = 0; chi < NC; ++chi)
      for (int a = 0; a < nf; ++a)
        for (int b = 0; b < nf; ++b) {
          double v = B[(sigf(chi, a) * nf + a) * NE + sigf(chi, b) * nf + b];
          if (hex8 && !((hex8_mask(chi) >> (a * 3 + b)) & 1u)) v = 0.0;   // exact zeros
          c.op.B64.b[chi][a][b] = v;
          c.op.B32.b[chi][a][b] = (float)v;
        }
  for (int i = 0; i < NE; ++i) c.op.KEdiag[i] = c.KEh[i * NE + i];
  // Q_o = P_o^T KE P_o for the 2^nd child octants (level-1 Galerkin blocks)
  std::vector<double> Qh((size_t)NC * NE * NE, 0.0);
  auto pw = [&](int o, int p, int a) {
    double w = 1.0;
    for (int k = 0; k < nd; ++k) {
      const int pos = ((o >> k) & 1) + ((p >> k) & 1);
      const int dist = std::abs(pos - 2 * ((a >> k) & 1));
      w *= dist == 0 ? 1.0 : (dist == 1 ? 0.5 : 0.0);
    }
    return w;
  };
  for (int o = 0; o < NC; ++o)
    for (int a = 0; a < NC; ++a)
      for (int b = 0; b < NC; ++b)
        for (int ci = 0; ci < nf; ++ci)
          for (int cj = 0; cj < nf; ++cj) {
            double acc = 0.0;
            for (int p = 0; p < NC; ++p) {
              const double wp = pw(o, p, a);
              if (wp == 0.0) continue;
              for (int q = 0; q < NC; ++q) {
                const double wq = pw(o, q, b);
                if (wq == 0.0) continue;
                acc += wp * wq * c.KEh[(p * nf + ci) * NE + q * nf + cj];
              }
            }
            Qh[(size_t)o * NE * NE + (a * nf + ci) * NE + b * nf + cj] = acc;
          }
  c.KE64.alloc(NE * NE);
  c.KE32.alloc(NE * NE);
  c.Q.alloc((int64_t)NC * NE * NE);
  std::vector<float> k32(NE * NE);
  for (int i = 0; i < NE * NE; ++i) k32[i] = (float)c.KEh[i];
  TG_CUDA(cudaMemcpy(c.KE64.p, c.KEh.data(), sizeof(double) * NE * NE, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c.KE32.p, k32.data(), sizeof(float) * NE * NE, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c.Q.p, Qh.data(), sizeof(double) * Qh.size(), cudaMemcpyHostToDevice));
  std::vector<float> q32(Qh.begin(), Qh.end());
  c.Q32.alloc((int64_t)q32.size());
  TG_CUDA(cudaMemcpy(c.Q32.p, q32.data(), sizeof(float) * q32.size(), cudaMemcpyHostToDevice));
  c.op.KE64 = c.KE64.p;
  c.op.KE32 = c.KE32.p;
}

static int choose_levels(const Grid& g, int requested);
static int choose_levels_nat(const Grid& g) { return choose_levels(g, 0); }

static Grid coarsest_of(const Grid& g, int L) {
  Grid c = g;
  for (int l = 1; l < L; ++l) c = coarsen(c);
  return c;
}

// Grids whose element counts do not halve down to a small coarsest level
// (odd counts, e.g. a 65x65 heat plate) are embedded in the smallest grid
// with counts that are multiples of 2^k whose k-times coarsened grid has at
// most 1200 DOFs.  The padding layers sit at the high end of each axis:
// padding elements have zero stiffness (flag EL_OUTSIDE) and padding nodes
// are fixed, so the caller's nodes see exactly the caller's operator; the
// filter, volume, compliance and OC skip padding elements.
static Grid embedding_grid(const Grid& rg, int requested_levels) {
  if (requested_levels > 0) return rg;
  if (coarsest_of(rg, choose_levels_nat(rg)).ndofs() <= 1200) return rg;
  for (int k = 1; k <= 12; ++k) {
    const int m = 1 << k;
    auto up = [m](int v) { return ((v + m - 1) / m) * m; };
    const Grid gp = make_grid(rg.ndim, rg.ndof, up(rg.nex), up(rg.ney), rg.ndim == 3 ? up(rg.nez) : 1);
    Grid c = gp;
    for (int l = 0; l < k; ++l) c = coarsen(c);
    if (c.ndofs() <= 1200) return gp;
  }
  return rg;
}

static int choose_levels(const Grid& g, int requested) {
  int L = 1;
  Grid cur = g;
  const int cap = requested > 0 ? requested : 12;
  while (L < cap) {
    const bool even = (cur.nex % 2 == 0) && (cur.ney % 2 == 0) && (cur.ndim == 2 || cur.nez % 2 == 0);
    if (!even || cur.nex < 2 || cur.ney < 2 || (cur.ndim == 3 && cur.nez < 2)) break;
    if (requested <= 0 && cur.ndofs() <= 1200) break;
    cur = coarsen(cur);
    ++L;
  }
  return L;
}

void ctx_init(Ctx& c, const tg_problem& p) {
  TG_REQUIRE(p.ndim == 2 || p.ndim == 3, "ndim must be 2 or 3");
  TG_REQUIRE(p.nnode_dof == 1 || p.nnode_dof == p.ndim,
             "nnode_dof must be 1 (scalar) or ndim (elasticity)");
  TG_REQUIRE(p.nelx > 0 && p.nely > 0 && (p.ndim == 2 || p.nelz > 0), "element counts must be > 0");
  TG_REQUIRE(p.KE != nullptr && p.f != nullptr, "KE and f are required");
  TG_REQUIRE(p.ft >= -1 && p.ft <= 1, "ft must be -1, 0 or 1");
  TG_REQUIRE(p.precision == TG_PREC_FP64 || p.precision == TG_PREC_MIXED, "unknown precision");
  TG_REQUIRE(p.precond == TG_PRECOND_GMG || p.precond == TG_PRECOND_JACOBI, "unknown preconditioner");
  {   // argument checks that need no device: fixed DOF indices
    const Grid rg0 = make_grid(p.ndim, p.nnode_dof, p.nelx, p.nely, p.nelz);
    TG_REQUIRE(p.nfixed >= 0 && (p.nfixed == 0 || p.fixed != nullptr), "fixed DOF list missing");
    for (int64_t i = 0; i < p.nfixed; ++i)
      TG_REQUIRE(p.fixed[i] >= 0 && p.fixed[i] < rg0.ndofs(), "fixed DOF index out of range");
  }
  c.dev = p.device;
  TG_CUDA(cudaSetDevice(c.dev));
  TG_CUDA(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
  TG_CUDA(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking));
  TG_CUDA(cudaEventCreateWithFlags(&c.sev_fork, cudaEventDisableTiming));
  TG_CUDA(cudaEventCreateWithFlags(&c.sev_join, cudaEventDisableTiming));
  TG_CUDA(cudaEventCreate(&c.ev0));
  TG_CUDA(cudaEventCreate(&c.ev1));
  TG_CUDA(cudaEventCreate(&c.tev0));
  TG_CUDA(cudaEventCreate(&c.tev1));
  c.rg = make_grid(p.ndim, p.nnode_dof, p.nelx, p.nely, p.nelz);
  c.g = (p.precond == TG_PRECOND_GMG) ? embedding_grid(c.rg, p.nlevels) : c.rg;
  c.padded = c.g.nex != c.rg.nex || c.g.ney != c.rg.ney || c.g.nez != c.rg.nez;
  c.volfrac = p.volfrac; c.rmin = p.rmin; c.eps = p.eps; c.penal = p.penal;
  c.move = p.move > 0 ? p.move : 0.2;
  c.ft = p.ft; c.precond = p.precond; c.precision = p.precision;
  c.nsmooth = p.nsmooth > 0 ? p.nsmooth : 2;
  c.nsmooth_coarse = p.nsmooth_coarse > 0 ? p.nsmooth_coarse : c.nsmooth;
  c.omega = p.omega > 0 ? p.omega : 0.6;
  c.rtol = p.rtol > 0 ? p.rtol : 1e-8;
  c.maxiter = p.maxiter > 0 ? p.maxiter : 2000;
  c.inner_rtol = p.inner_rtol > 0 ? p.inner_rtol : 1e-4;
  c.learned = p.learned;
  c.nload = p.nload > 1 ? p.nload : 1;
  const Grid& g = c.g;
  const int64_t nn = g.nnodes(), nd = g.ndofs(), nel = g.nel();
  c.op.g = g;
  c.op.flat64 = c.precision == TG_PREC_FP64;
  setup_element(c, p.KE);

  // fixed-DOF bits per node (caller's DOF numbers mapped to the device grid;
  // padding nodes fully fixed), and per element "touches a fixed DOF"
  const Grid& rg = c.rg;
  const int64_t rnd = rg.ndofs(), rnel = rg.nel();
  auto dev_node = [&](int64_t rn) {
    const int y = (int)(rn % rg.nny), x = (int)((rn / rg.nny) % rg.nnx);
    const int z = (int)(rn / ((int64_t)rg.nny * rg.nnx));
    return g.node(x, y, z);
  };
  std::vector<uint8_t> fix(nn, 0);
  if (c.padded) {
    const uint8_t all = (uint8_t)((1u << g.ndof) - 1u);
    for (int z = 0; z < g.nnz; ++z)
      for (int x = 0; x < g.nnx; ++x)
        for (int y = 0; y < g.nny; ++y)
          if (x >= rg.nnx || y >= rg.nny || z >= rg.nnz) fix[g.node(x, y, z)] = all;
  }
  for (int64_t i = 0; i < p.nfixed; ++i) {
    const int64_t d = p.fixed[i];
    TG_REQUIRE(d >= 0 && d < rnd, "fixed DOF index out of range");
    fix[dev_node(d / g.ndof)] |= (uint8_t)(1u << (d % g.ndof));
  }
  std::vector<uint8_t> touch(nel, 0);
  for (int ez = 0; ez < g.nez; ++ez)
    for (int ex = 0; ex < g.nex; ++ex)
      for (int ey = 0; ey < g.ney; ++ey) {
        uint8_t t = 0;
        for (int d = 0; d < (1 << g.ndim); ++d)
          t |= fix[g.node(ex + (d & 1), ey + ((d >> 1) & 1), g.ndim == 3 ? ez + ((d >> 2) & 1) : 0)];
        touch[g.elem(ex, ey, ez)] = t ? 1 : 0;
      }
  // hierarchy grids and coarse fixed bits (coincident fine DOF)
  // L == 1 with multigrid: the fine grid is the coarsest level and the
  // "V-cycle" is the dense direct solve of the fine operator
  c.L = (c.precond == TG_PRECOND_GMG) ? choose_levels(g, p.nlevels) : 1;
  c.unsmoothed = p.unsmoothed;
  TG_REQUIRE(c.unsmoothed == 0 ||
                 (c.precond == TG_PRECOND_GMG && (c.unsmoothed & 1) == 0 &&
                  (c.unsmoothed >> std::max(c.L - 1, 0)) == 0),
             "unsmoothed: only levels 1 .. nlevels-2 can be left unsmoothed");
  std::vector<std::vector<uint8_t>> fixl{fix};
  c.lv.push_back(new Level());
  c.lv[0]->g = g;
  for (int l = 1; l < c.L; ++l) {
    const Grid gf = c.lv[l - 1]->g, gc = coarsen(gf);
    std::vector<uint8_t> fc(gc.nnodes(), 0);
    for (int z = 0; z < gc.nnz; ++z)
      for (int x = 0; x < gc.nnx; ++x)
        for (int y = 0; y < gc.nny; ++y)
          fc[gc.node(x, y, z)] = fixl[l - 1][gf.node(2 * x, 2 * y, gf.ndim == 3 ? 2 * z : 0)];
    fixl.push_back(fc);
    c.lv.push_back(new Level());
    c.lv[l]->g = gc;
  }
  if (c.precond == TG_PRECOND_GMG) {
    const Grid gc = c.lv[c.L - 1]->g;
    c.nc = gc.ndofs();
    TG_REQUIRE(c.nc <= 8192, "coarsest multigrid level too large for the dense solve "
                             "(use element counts divisible by a higher power of 2, or "
                             "preconditioner gb300-jacobi)");
    c.ldc = cdiv(c.nc, 32) * 32;
    c.Dc.alloc(c.ldc * c.ldc);
    if (c.precision == TG_PREC_MIXED && c.L > 1) c.Dc32.alloc(c.ldc * c.ldc);
    c.gjwork.alloc(32 * 32 + 2 * 32 * c.ldc);   // pivot tile, row panel R, saved panel X
    c.tailbar.alloc(1);
    TG_CUDA(cudaMemsetAsync(c.tailbar.p, 0, sizeof(GridBar), c.st));
  }
  const bool mixed = c.precision == TG_PREC_MIXED;
  for (int l = 0; l < c.L; ++l) {
    Level& v = *c.lv[l];
    const int64_t n = v.g.ndofs();
    v.fix.alloc(v.g.nnodes());
    TG_CUDA(cudaMemcpy(v.fix.p, fixl[l].data(), fixl[l].size(), cudaMemcpyHostToDevice));
    const int64_t ns = v.g.slds() * stencil_half_dirs(g.ndim) * g.ndof * g.ndof;
    // mixed precision: the coarse operators (levels >= 1) exist in FP32 only,
    // built in FP32 for the FP32 V-cycle; the fine level keeps its FP64 data
    const bool last = (l == c.L - 1) && c.precond == TG_PRECOND_GMG;
    if (l >= 1 || last) {
      if (mixed && l >= 1) v.A32.alloc(ns);
      else v.A64.alloc(ns);
    }
    if (!last || l == 0) {
      if (!mixed || l == 0) { v.dinv64.alloc(n); v.t64.alloc(n); v.r64.alloc(n); }
      if (mixed) { v.dinv32.alloc(n); v.t32.alloc(n); v.r32.alloc(n); }
    }
    if (l >= 1) {
      if (mixed) { v.b32.alloc(n); v.x32.alloc(n); }
      else { v.b64.alloc(n); v.x64.alloc(n); }
    }
  }
  c.op.fix = c.lv[0]->fix.p;
  c.touch.alloc(nel);
  TG_CUDA(cudaMemcpy(c.touch.p, touch.data(), nel, cudaMemcpyHostToDevice));
  if (p.el_flags || c.padded) {
    std::vector<int8_t> fl(nel, EL_OUTSIDE);
    for (int ez = 0; ez < rg.nez; ++ez)
      for (int ex = 0; ex < rg.nex; ++ex)
        for (int ey = 0; ey < rg.ney; ++ey)
          fl[g.elem(ex, ey, ez)] = p.el_flags ? p.el_flags[rg.elem(ex, ey, ez)] : 0;
    c.flags.alloc(nel);
    TG_CUDA(cudaMemcpy(c.flags.p, fl.data(), nel, cudaMemcpyHostToDevice));
  }
  if (c.padded) c.emb.alloc(std::max(rnd, rnel));
  // vectors
  c.f.alloc(nd * c.nload); c.u.alloc(nd * c.nload);
  c.x.alloc(nel); c.xPhys.alloc(nel); c.xold.alloc(nel); c.xnew.alloc(nel); c.xsolved.alloc(nel);
  c.dc.alloc(nel); c.dcf.alloc(nel); c.dv.alloc(nel); c.Hs.alloc(nel); c.S.alloc(3 * nel);
  c.S32.alloc(5 * nel);
  c.s64.alloc(nel);
  if (mixed) { c.s32.alloc(nel); c.s16.alloc(nel); }
  c.part.alloc(RED_BLOCKS); c.part2.alloc(RED_BLOCKS); c.scal.alloc(8);
  c.oc.alloc(1); c.pcg.alloc(1); c.pcg_out.alloc(1);
  c.oc.zero(c.st); c.pcg.zero(c.st); c.pcg_out.zero(c.st);
  c.r.alloc(nd); c.z.alloc(nd); c.p.alloc(nd); c.q.alloc(nd); c.z2.alloc(nd);
  if (mixed) { c.r32.alloc(nd); c.z32.alloc(nd); c.p32.alloc(nd); c.q32.alloc(nd); c.d32.alloc(nd); }
  TG_CUDA(cudaMallocHost(&c.h_oc, sizeof(OCState)));
  TG_CUDA(cudaMallocHost(&c.h_pcg, sizeof(PCGState)));
  TG_CUDA(cudaMallocHost(&c.h_scal, 8 * sizeof(double)));

  // loads (masked to the free DOFs), one device vector per load case
  for (int lc = 0; lc < c.nload; ++lc) {
    std::vector<double> fh(nd, 0.0);
    const double* fsrc = p.f + (int64_t)lc * rnd;
    for (int64_t i = 0; i < rnd; ++i) fh[dev_node(i / g.ndof) * g.ndof + i % g.ndof] = fsrc[i];
    double bb = 0.0;
    for (int64_t i = 0; i < nd; ++i) {
      if ((fix[i / g.ndof] >> (i % g.ndof)) & 1) fh[i] = 0.0;
      bb += fh[i] * fh[i];
    }
    if (lc == 0) c.bnorm = std::sqrt(bb);
    TG_CUDA(cudaMemcpy(c.f.p + (int64_t)lc * nd, fh.data(), sizeof(double) * nd,
                       cudaMemcpyHostToDevice));
  }
  c.u.zero(c.st);

  // filter stencil weights and the normaliser Hs (filter/matrix_filter.py:185-231)
  const int R = std::max(0, (int)std::ceil(c.rmin) - 1);
  const int W = 2 * R + 1;
  const int nw = (g.ndim == 3) ? W * W * W : W * W;
  std::vector<double> w(nw);
  for (int i = 0; i < nw; ++i) {
    const int oy = i % W - R, ox = (i / W) % W - R, oz = (g.ndim == 3) ? i / (W * W) - R : 0;
    w[i] = std::max(0.0, c.rmin - std::sqrt((double)(ox * ox + oy * oy + oz * oz)));
  }
  c.fw.alloc(nw);
  TG_CUDA(cudaMemcpy(c.fw.p, w.data(), sizeof(double) * nw, cudaMemcpyHostToDevice));
  c.fs.R = R; c.fs.nw = nw; c.fs.w = c.fw.p;
  c.fs.rex = rg.nex; c.fs.rey = rg.ney; c.fs.rez = rg.nez;
  c.fs.tmp = c.S.p + nel;   // OC scratch, idle while a filter runs
  filter_apply(g, c.fs, nullptr, nullptr, nullptr, c.Hs, 3, c.st);
  // dv: ones, filtered once for the density filter (topology_optimization.py:520, :558)
  std::vector<double> ones(nel, 0.0);
  for (int ez = 0; ez < rg.nez; ++ez)
    for (int ex = 0; ex < rg.nex; ++ex)
      for (int ey = 0; ey < rg.ney; ++ey) ones[g.elem(ex, ey, ez)] = 1.0;
  TG_CUDA(cudaMemcpy(c.xnew.p, ones.data(), sizeof(double) * nel, cudaMemcpyHostToDevice));
  if (p.filter_pde) {
    // dv = TF^T KF^-1 TF 1 for the density form (topology_optimization.py:570)
    helmholtz_init(c, p.KF);
    if (c.ft == 1) helmholtz_apply(c, c.xnew, nullptr, nullptr, c.dv);
    else TG_CUDA(cudaMemcpyAsync(c.dv.p, c.xnew.p, sizeof(double) * nel, cudaMemcpyDeviceToDevice, c.st));
  } else if (c.ft == 1) {
    filter_apply(g, c.fs, c.xnew, nullptr, c.Hs, c.dv, 1, c.st);
  } else {
    TG_CUDA(cudaMemcpyAsync(c.dv.p, c.xnew.p, sizeof(double) * nel, cudaMemcpyDeviceToDevice, c.st));
  }
  // initial design x = xPhys = volfrac (topology_optimization.py:216-219)
  std::vector<double> x0(nel, 0.0);
  for (int ez = 0; ez < rg.nez; ++ez)
    for (int ex = 0; ex < rg.nex; ++ex)
      for (int ey = 0; ey < rg.ney; ++ey) x0[g.elem(ex, ey, ez)] = c.volfrac;
  TG_CUDA(cudaMemcpy(c.x.p, x0.data(), sizeof(double) * nel, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c.xPhys.p, x0.data(), sizeof(double) * nel, cudaMemcpyHostToDevice));
  c.g_oc = 0.0;
  TG_CUDA(cudaStreamSynchronize(c.st));
}

// ---------------------------------------------------------------------------
// hierarchy
// ---------------------------------------------------------------------------
void set_density(Ctx& c, const double* xPhys) {
  ProfScope ps(PK_COARSE_BUILD, c.st);
  simp_scale(c.g.nel(), xPhys, c.eps, c.penal, c.s64, c.s32.p, c.s16.p, c.st, c.flags.p);
  TG_CUDA(cudaMemcpyAsync(c.xsolved.p, xPhys, sizeof(double) * c.g.nel(), cudaMemcpyDeviceToDevice,
                          c.st));
}

void build_hierarchy(Ctx& c) {
  const bool mixed = c.precision == TG_PREC_MIXED;
  Level& f = *c.lv[0];
  {
  ProfScope ps(PK_COARSE_BUILD, c.st);
  fine_dinv<double, double>(c.op, c.s64, f.dinv64, c.st);
  if (mixed) fine_dinv<float, __nv_bfloat16>(c.op, c.s16, f.dinv32, c.st);
  if (c.precond != TG_PRECOND_GMG) {
    c.built = true;
    return;
  }
  // mixed: level operators in FP32 (they only serve the FP32 V-cycle, which
  // would round FP64 ones to FP32 anyway); the coarsest matrix is inverted in FP64
  for (int l = 1; l < c.L; ++l) {
    Level& v = *c.lv[l];
    if (mixed) {
      if (l == 1) build_level1<float>(c.op, c.s32, c.touch, c.Q32, c.KE32, v.g, v.fix, v.A32, c.st);
      else build_galerkin<float>(c.lv[l - 1]->g, c.lv[l - 1]->A32, v.g, v.fix, v.A32, c.st);
      if (l < c.L - 1) stencil_dinv<float>(v.g, v.fix, v.A32, v.dinv32, c.st);
    } else {
      if (l == 1) build_level1<double>(c.op, c.s64, c.touch, c.Q, c.KE64, v.g, v.fix, v.A64, c.st);
      else build_galerkin<double>(c.lv[l - 1]->g, c.lv[l - 1]->A64, v.g, v.fix, v.A64, c.st);
      if (l < c.L - 1) stencil_dinv<double>(v.g, v.fix, v.A64, v.dinv64, c.st);
    }
  }
  Level& cl = *c.lv[c.L - 1];
  if (c.L == 1) {
    build_fine_stencil(c.op, c.s64, cl.A64, c.st);
    stencil_to_dense<double>(cl.g, cl.fix, cl.A64, c.Dc, c.nc, c.ldc, c.st);
  } else if (mixed) {
    stencil_to_dense<float>(cl.g, cl.fix, cl.A32, c.Dc, c.nc, c.ldc, c.st);
  } else {
    stencil_to_dense<double>(cl.g, cl.fix, cl.A64, c.Dc, c.nc, c.ldc, c.st);
  }
  }
  ProfScope ps(PK_COARSE_INV, c.st);
  if (mixed && c.L > 1) gj_inverse_dw(c.Dc, c.nc, c.ldc, c.gjwork, c.st);
  else gj_inverse(c.Dc, c.nc, c.ldc, c.gjwork, c.st);
  if (c.Dc32.p) d2f(c.ldc * c.ldc, c.Dc, c.Dc32, c.st);
  c.built = true;
}

// ---------------------------------------------------------------------------
// V-cycle (zero initial guess, nsmooth damped-Jacobi sweeps before and after)
// ---------------------------------------------------------------------------
template <typename T> struct LvBufs;
template <> struct LvBufs<double> {
  static double* dinv(Level& v) { return v.dinv64; }
  static double* b(Level& v) { return v.b64; }
  static double* x(Level& v) { return v.x64; }
  static double* t(Level& v) { return v.t64; }
  static double* r(Level& v) { return v.r64; }
  static const double* A(Level& v) { return v.A64; }
};
template <> struct LvBufs<float> {
  static float* dinv(Level& v) { return v.dinv32; }
  static float* b(Level& v) { return v.b32; }
  static float* x(Level& v) { return v.x32; }
  static float* t(Level& v) { return v.t32; }
  static float* r(Level& v) { return v.r32; }
  static const float* A(Level& v) { return v.A32; }
};

template <typename T>
static void level_apply(Ctx& c, int l, const T* in, T* out, const T* b, int mode) {
  Level& v = *c.lv[l];
  if (l == 0) {
    if (std::is_same<T, double>::value)
      fine_apply<double, double>(c.op, c.s64, (const double*)in, (double*)out, (const double*)b,
                                 (const double*)LvBufs<T>::dinv(v), c.omega, mode, c.st);
    else
      fine_apply<float, __nv_bfloat16>(c.op, c.s16, (const float*)in, (float*)out,
                                       (const float*)b, (const float*)LvBufs<T>::dinv(v), c.omega,
                                       mode, c.st);
  } else {
    ProfScope ps(sizeof(T) == 8 ? PK_STENCIL_F64 : (l == 1 ? PK_STENCIL1_F32 : PK_STENCIL_F32), c.st);
    stencil_apply<T>(v.g, LvBufs<T>::A(v), in, out, b, LvBufs<T>::dinv(v), c.omega, mode, c.st);
  }
}

template <typename T> void vcycle(Ctx& c, int l, const T* b, T* x, bool prescaled, int dot_op) {
  Level& v = *c.lv[l];
  const int64_t n = v.g.ndofs();
  if (l == c.L - 1) {
    {
      ProfScope ps(PK_TRANSFER, c.st);
      // GJ scratch is idle here
      if constexpr (std::is_same<T, float>::value) {
        if (c.Dc32.p) dense_apply(c.Dc32.p, c.nc, c.ldc, b, x, c.gjwork, c.st);
        else dense_apply<T>(c.Dc, c.nc, c.ldc, b, x, c.gjwork, c.st);
      } else {
        dense_apply<T>(c.Dc, c.nc, c.ldc, b, x, c.gjwork, c.st);
      }
    }
    if (dot_op >= 0) {
      ProfScope ps(PK_VECTOR, c.st);
      dot<T, T>(n, b, x, c.part, c.pcg, dot_op, c.st);
    }
    return;
  }
  auto smoothed = [&](int k) { return k < c.L - 1 && !((c.unsmoothed >> k) & 1); };
  if (l > 0 && !smoothed(l)) {
    // no smoothing on this level (x = 0, residual = b): restrict b on, take
    // the coarser correction and prolongate it back
    Level& w = *c.lv[l + 1];
    const bool fuse = smoothed(l + 1);
    {
      ProfScope ps(PK_TRANSFER, c.st);
      if (fuse)
        restrict_<T>(v.g, w.g, w.fix, b, LvBufs<T>::b(w), c.st, LvBufs<T>::dinv(w),
                     LvBufs<T>::t(w), c.omega);
      else
        restrict_<T>(v.g, w.g, w.fix, b, LvBufs<T>::b(w), c.st);
    }
    vcycle<T>(c, l + 1, LvBufs<T>::b(w), LvBufs<T>::x(w), fuse);
    ProfScope ps(PK_TRANSFER, c.st);
    prolong_set<T>(v.g, w.g, v.fix, LvBufs<T>::x(w), x, c.st);
    return;
  }
  const int nsm = l == 0 ? c.nsmooth : c.nsmooth_coarse;
  // 2*nsm - 1 sweeps swap the buffers an odd number of times: starting in
  // the scratch buffer ends in x (no copy at the end of the level)
  T* bufs[2] = {x, LvBufs<T>::t(v)};
  int cur = 1;
  if (!prescaled) {
    ProfScope ps(PK_VECTOR, c.st);
    scale_mul<T>(n, c.omega, LvBufs<T>::dinv(v), b, bufs[cur], c.st);
  }
  for (int s = 1; s < nsm; ++s) {
    level_apply<T>(c, l, bufs[cur], bufs[1 - cur], b, AM_JACOBI);
    cur = 1 - cur;
  }
  T* r = LvBufs<T>::r(v);
  level_apply<T>(c, l, bufs[cur], r, b, AM_RES);
  Level& w = *c.lv[l + 1];
  const bool fuse = smoothed(l + 1);       // the coarsest level has no smoother
  // the two levels below this one (the last smoothed level, on the small-grid
  // stencil, and the coarsest solve) in one cooperative launch
  const int64_t tail_pairs = w.g.nnodes() * w.g.ndof;
  if (l + 3 == c.L && tune_coarse_tail() && tail_pairs < tune_stencil_small_pairs() &&
      tail_pairs <= TAIL_MAX_PAIRS && smoothed(l + 1)) {
    Level& k = *c.lv[c.L - 1];
    TailArgs<T> a;
    a.gp = v.g; a.gt = w.g; a.gc = k.g;
    a.fixt = w.fix; a.fixc = k.fix; a.fixp = v.fix;
    a.rp = r; a.xp = bufs[cur];
    a.At = LvBufs<T>::A(w); a.dinvt = LvBufs<T>::dinv(w);
    a.bt = LvBufs<T>::b(w); a.xt = LvBufs<T>::x(w); a.tt = LvBufs<T>::t(w);
    a.rt = LvBufs<T>::r(w);
    a.bc = LvBufs<T>::b(k); a.xc = LvBufs<T>::x(k);
    a.Dc = c.Dc; a.nc = c.nc; a.ldc = c.ldc; a.part = c.gjwork;
    a.Dc32 = std::is_same<T, float>::value ? c.Dc32.p : nullptr;
    a.omega = (T)c.omega; a.nsmooth = c.nsmooth_coarse; a.bar = c.tailbar;
    const int mode = tune_coarse_tail();
    a.cluster = mode == 1 ? 16 : 0;
    a.blocks = mode > 2 ? mode : 0;
    ProfScope ps(PK_TAIL, c.st);
    coarse_tail<T>(a, c.st);
  } else {
    {
      ProfScope ps(PK_TRANSFER, c.st);
      if (fuse)
        restrict_<T>(v.g, w.g, w.fix, r, LvBufs<T>::b(w), c.st, LvBufs<T>::dinv(w),
                     LvBufs<T>::t(w), c.omega);
      else
        restrict_<T>(v.g, w.g, w.fix, r, LvBufs<T>::b(w), c.st);
    }
    vcycle<T>(c, l + 1, LvBufs<T>::b(w), LvBufs<T>::x(w), fuse);
    {
      ProfScope ps(PK_TRANSFER, c.st);
      prolong_add<T>(v.g, w.g, v.fix, LvBufs<T>::x(w), bufs[cur], c.st);
    }
  }
  // the fine level's last sweep of the FP32 cycle also forms the PCG dot b . x
  const bool fused_dot = dot_op >= 0 && l == 0 && std::is_same<T, float>::value;
  for (int s = 0; s < nsm; ++s) {
    if (fused_dot && s == nsm - 1)
      fine_apply_dot<float, __nv_bfloat16>(c.op, c.s16, (const float*)bufs[cur],
                                           (float*)bufs[1 - cur], (const float*)b,
                                           (const float*)LvBufs<T>::dinv(v), c.omega, AM_JACOBI,
                                           c.part, c.pcg, dot_op, c.st);
    else
      level_apply<T>(c, l, bufs[cur], bufs[1 - cur], b, AM_JACOBI);
    cur = 1 - cur;
  }
  if (dot_op >= 0 && !fused_dot) {
    ProfScope ps(PK_VECTOR, c.st);
    dot<T, T>(n, b, bufs[cur], c.part, c.pcg, dot_op, c.st);
  }
  if (bufs[cur] != x) {
    ProfScope ps(PK_VECTOR, c.st);
    TG_CUDA(cudaMemcpyAsync(x, bufs[cur], sizeof(T) * n, cudaMemcpyDeviceToDevice, c.st));
  }
}
template void vcycle<double>(Ctx&, int, const double*, double*, bool, int);
template void vcycle<float>(Ctx&, int, const float*, float*, bool, int);

template <typename T>
static void precondition(Ctx& c, const T* r, T* z) {
  if (c.precond == TG_PRECOND_GMG) {
    vcycle<T>(c, 0, r, z);
  } else {
    ProfScope ps(PK_VECTOR, c.st);
    scale_mul<T>(c.g.ndofs(), 1.0, LvBufs<T>::dinv(*c.lv[0]), r, z, c.st);
  }
}

// ---------------------------------------------------------------------------
// solvers
// ---------------------------------------------------------------------------
static void read_pcg(Ctx& c, PCGState* d) {
  TG_CUDA(cudaMemcpyAsync(c.h_pcg, d, sizeof(PCGState), cudaMemcpyDeviceToHost, c.st));
  TG_CUDA(cudaStreamSynchronize(c.st));
}

static void check_finite(double v, const char* what) {
  if (!std::isfinite(v)) throw Error{ENAN, std::string("non-finite value in ") + what};
}

// Run one PCG iteration body: replayed from a CUDA graph captured on first
// use (one launch per iteration instead of ~35).  While a kernel family is
// event-timed the graph is captured again with the family's event pairs as
// graph nodes, read after each replay.  Ends with the PCG scalars in h_pcg.
template <typename F>
static void run_iteration(Ctx& c, Ctx::IterGraph& gr, F&& body) {
  if (!c.use_graphs) {
    body();
    TG_CUDA(cudaStreamSynchronize(c.st));
    return;
  }
  const int kind = prof_kind();
  if (gr.exec && gr.kind != kind) {
    cudaGraphExecDestroy(gr.exec);
    gr.exec = nullptr;
    gr.prof.release();
  }
  if (!gr.exec) {
    const int64_t before = launch_count();
    cudaGraph_t graph = nullptr;
    TG_CUDA(cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal));
    if (kind != PK_NONE) prof_capture_begin(&gr.prof);
    try {
      body();
    } catch (...) {
      prof_capture_end();
      cudaStreamEndCapture(c.st, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    prof_capture_end();
    gr.kind = kind;
    TG_CUDA(cudaStreamEndCapture(c.st, &graph));
    const cudaError_t e = cudaGraphInstantiate(&gr.exec, graph, 0);
    cudaGraphDestroy(graph);
    TG_CUDA(e);
    gr.launches = launch_count() - before;
    count_launches(-gr.launches);      // capture recorded, did not launch
  }
  TG_CUDA(cudaGraphLaunch(gr.exec, c.st));
  count_launches(gr.launches);
  TG_CUDA(cudaStreamSynchronize(c.st));
  if (kind != PK_NONE) prof_collect(gr.prof);
}

__global__ void k_loop_ctl(PCGState* s, double tol, int maxit) {
  pdl_wait();
  pdl_trigger();
  s->tol = tol;
  s->maxit = maxit;
}
// continue while not converged (finite rr) and under the iteration cap
__device__ __host__ inline bool pcg_continue(const PCGState& s) {
  return isfinite(s.rr) && sqrt(s.rr) >= s.tol && s.iter < s.maxit;
}
__global__ void k_loop_continue(cudaGraphConditionalHandle h, const PCGState* s) {
  pdl_wait();
  cudaGraphSetConditional(h, pcg_continue(*s) ? 1u : 0u);
}

// Run PCG iterations (body = one iteration, no host read inside) until
// sqrt(rr) < tol, the PCG state's iter (counted since its reset; `start` at
// entry, so a loop can resume one that stopped) reaches maxit, or rr is not
// finite: as one WHILE-node graph replay, captured on first use; while a
// kernel family is event-timed or graphs are off, one iteration at a time
// from the host.  Leaves the PCG state in h_pcg and returns the number of
// iterations run by this call.
template <typename F>
static int run_loop(Ctx& c, Ctx::IterGraph& gr, Ctx::LoopGraph& lg, double tol, int maxit,
                    F&& body, int start = 0) {
  if (maxit - start <= 0) {
    read_pcg(c, c.pcg);
    return 0;
  }
  if (!c.use_graphs || prof_kind() != PK_NONE) {
    int it = 0;
    while (start + it < maxit) {
      run_iteration(c, gr, [&] {
        body();
        TG_CUDA(cudaMemcpyAsync(c.h_pcg, c.pcg.p, sizeof(PCGState), cudaMemcpyDeviceToHost, c.st));
      });
      ++it;
      PCGState s = *c.h_pcg;
      s.tol = tol;
      s.maxit = maxit;
      if (!pcg_continue(s)) break;
    }
    return it;
  }
  if (!lg.exec) {
    TG_CUDA(cudaGraphCreate(&lg.graph, 0));
    TG_CUDA(cudaGraphConditionalHandleCreate(&lg.h, lg.graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = lg.h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    TG_CUDA(cudaGraphAddNode(&node, lg.graph, nullptr, nullptr, 0, &np));
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    const int64_t before = launch_count();
    TG_CUDA(cudaStreamBeginCaptureToGraph(c.st, bodyg, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    try {
      body();
      launch_pdl(k_loop_continue, dim3(1), dim3(1), 0, c.st, lg.h, (const PCGState*)c.pcg.p);
      TG_CHECK_LAUNCH();
    } catch (...) {
      cudaGraph_t g2 = nullptr;
      cudaStreamEndCapture(c.st, &g2);
      cudaGraphDestroy(lg.graph);
      lg.graph = nullptr;
      throw;
    }
    cudaGraph_t g2 = nullptr;
    TG_CUDA(cudaStreamEndCapture(c.st, &g2));
    TG_CUDA(cudaGraphInstantiate(&lg.exec, lg.graph, 0));
    lg.body_launches = launch_count() - before;
    count_launches(-lg.body_launches);    // captured, not launched
  }
  // the PCG state was reset (iter = 0) by the caller just before the loop
  k_loop_ctl<<<1, 1, 0, c.st>>>(c.pcg, tol, maxit);
  TG_CHECK_LAUNCH();
  TG_CUDA(cudaGraphLaunch(lg.exec, c.st));
  read_pcg(c, c.pcg);
  const int it = c.h_pcg->iter - start;
  count_launches(lg.body_launches * it);
  return it;
}

static void drop_loop_graphs(Ctx::IterGraph& gr, Ctx::LoopGraph& lg) {
  if (gr.exec) cudaGraphExecDestroy(gr.exec);
  gr.exec = nullptr;
  gr.prof.release();
  if (lg.exec) cudaGraphExecDestroy(lg.exec);
  if (lg.graph) cudaGraphDestroy(lg.graph);
  lg.exec = nullptr;
  lg.graph = nullptr;
}

// plain FP64 PCG (linear_solvers.py:114-134), x in/out
static int pcg64(Ctx& c, const double* b, double* x, double tol_abs, int maxiter, bool& conv) {
  const int64_t n = c.g.ndofs();
  fine_apply<double, double>(c.op, c.s64, x, c.r, b, nullptr, 0.0, AM_RES, c.st);
  pcg_reset(c.pcg, c.st);
  dot<double, double>(n, c.r.p, c.r.p, c.part, c.pcg, DOT_RR, c.st);
  read_pcg(c, c.pcg);
  double rr = c.h_pcg->rr;
  check_finite(rr, "PCG residual");
  conv = std::sqrt(rr) < tol_abs;
  int it = 0;
  // x lives in the caller's buffer; the captured body must not depend on it
  double* xs = c.z2.p;
  TG_CUDA(cudaMemcpyAsync(xs, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.st));
  if (!conv) {
    it = run_loop(c, c.g64, c.l64, tol_abs, maxiter, [&] {
      precondition<double>(c, c.r, c.z);
      {
        ProfScope ps(PK_VECTOR, c.st);
        dot<double, double>(n, c.r.p, c.z.p, c.part, c.pcg, DOT_RHO, c.st);
        update_p<double>(n, c.z, c.p, c.pcg, c.st);
      }
      fine_apply<double, double>(c.op, c.s64, c.p, c.q, nullptr, nullptr, 0.0, AM_Y, c.st);
      ProfScope ps(PK_VECTOR, c.st);
      dot<double, double>(n, c.p.p, c.q.p, c.part, c.pcg, DOT_ALPHA, c.st);
      update_xr<double>(n, c.p, c.q, xs, c.r, c.part, c.pcg, c.st);
    });
    rr = c.h_pcg->rr;
    check_finite(rr, "PCG residual");
    conv = std::sqrt(rr) < tol_abs;
  }
  TG_CUDA(cudaMemcpyAsync(x, xs, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.st));
  return it;
}

// the deflation vector of the FP32 PCG (the coarse-grid correction), when
// the context uses one (a learned network attached with that part enabled)
static const float* correction_vector(const Ctx& c) {
  return (c.cnn && (c.learned & TG_LEARNED_COARSE_CORRECTION)) ? c.cnn->w32.p : nullptr;
}

// FP32 PCG on the unit-norm residual r32 (d32 = 0 initial), FP64 dots:
// pcg32_begin resets, pcg32_run iterates until the inner tolerance or the
// state's iteration count reaches maxit (so a second call resumes a first).
// With a deflation vector w the pass starts from d32 = gamma w, the residual
// made orthogonal to w (a no-op while the state's wawinv is 0).
static void pcg32_begin(Ctx& c) {
  const int64_t n = c.g.ndofs();
  TG_CUDA(cudaMemsetAsync(c.d32.p, 0, sizeof(float) * n, c.st));
  pcg_reset(c.pcg, c.st);
  if (const float* w = correction_vector(c)) {
    ProfScope ps(PK_VECTOR, c.st);
    dot<float, float>(n, w, c.r32.p, c.part, c.pcg, DOT_WR, c.st);
    deflate_start(n, w, c.cnn->aw32.p, c.d32, c.r32, c.pcg, c.st);
  }
}
static int pcg32_run(Ctx& c, double tol_abs, int maxit, int start) {
  const int64_t n = c.g.ndofs();
  const float* w = correction_vector(c);
  const float* aw = w ? c.cnn->aw32.p : nullptr;
  if (w != c.g32_corr) {               // the captured iteration is for another vector
    drop_loop_graphs(c.g32, c.l32);
    c.g32_corr = w;
  }
  const int it = run_loop(c, c.g32, c.l32, tol_abs, maxit, [&] {
    // z = M r with rho = r . z fused into the cycle's last fine sweep; with a
    // deflation vector w, Aw . z for the deflated search direction; q = A p
    // with p . q (alpha) fused into the product
    if (c.precond == TG_PRECOND_GMG) {
      vcycle<float>(c, 0, c.r32, c.z32, false, DOT_RHO);
    } else {
      precondition<float>(c, c.r32, c.z32);
      ProfScope ps(PK_VECTOR, c.st);
      dot<float, float>(n, c.r32.p, c.z32.p, c.part, c.pcg, DOT_RHO, c.st);
    }
    {
      ProfScope ps(PK_VECTOR, c.st);
      if (w) {
        dot<float, float>(n, aw, c.z32.p, c.part, c.pcg, DOT_WZ, c.st);
        update_p_corr(n, c.z32, w, c.p32, c.pcg, c.st);
      } else {
        update_p<float>(n, c.z32, c.p32, c.pcg, c.st);
      }
    }
    fine_apply_dot<float, float>(c.op, c.s32, c.p32, c.q32, nullptr, nullptr, 0.0, AM_Y, c.part,
                                 c.pcg, DOT_ALPHA, c.st);
    ProfScope ps(PK_VECTOR, c.st);
    update_xr<float>(n, c.p32, c.q32, c.d32, c.r32, c.part, c.pcg, c.st);
  }, start);
  check_finite(c.h_pcg->rr, "inner PCG residual");
  return it;
}

void check_waits(Ctx& c) {
  if (take_wait_error(c.st))
    throw Error{ETIMEOUT, "multigrid V-cycle: a bounded wait for a TMA copy timed out"};
  if (c.cnn && take_conv_error(c.st))
    throw Error{ETIMEOUT, "learned warm start: a bounded wait of the tensor-core convolution timed out"};
  if (!c.tailbar.p) return;
  int err = 0;
  TG_CUDA(cudaMemcpyAsync(&err, &c.tailbar.p->err, sizeof(int), cudaMemcpyDeviceToHost, c.st));
  TG_CUDA(cudaStreamSynchronize(c.st));
  if (err) {
    TG_CUDA(cudaMemsetAsync(c.tailbar.p, 0, sizeof(GridBar), c.st));
    TG_CUDA(cudaStreamSynchronize(c.st));
    throw Error{ETIMEOUT, "multigrid V-cycle: a grid barrier wait of the coarse levels timed out"};
  }
}

void solve(Ctx& c, const double* b, double* u) {
  const int64_t n = c.g.ndofs();
  // c.r / c.pcg_out already hold b - K u and its norm (formed beside the
  // hierarchy build by ctx_step); consumed by this call only
  const bool r_ready = c.r_ready;
  c.r_ready = false;
  double bb;
  {
    pcg_reset(c.pcg_out, c.st);
    dot<double, double>(n, b, b, c.part, c.pcg_out, DOT_BB, c.st);
    read_pcg(c, c.pcg_out);
    bb = c.h_pcg->bb;
  }
  const double bnorm = std::sqrt(bb);
  const double tol = c.rtol * bnorm;
  c.last_iters = c.last_vcycles = c.last_refine = 0;
  c.last_converged = 0;
  if (bnorm == 0.0) {
    TG_CUDA(cudaMemsetAsync(u, 0, sizeof(double) * n, c.st));
    c.last_converged = 1;
    c.last_relres = 0.0;
    return;
  }
  mask_vec_f64(c.g.nnodes(), c.g.ndof, c.op.fix, u, c.st);
  if (c.precision == TG_PREC_FP64) {
    bool conv = false;
    const int it = pcg64(c, b, u, tol, c.maxiter, conv);
    c.last_iters = it;
    c.last_vcycles = (c.precond == TG_PRECOND_GMG) ? it : 0;
    c.last_converged = conv;
  } else {
    // FP64 iterative refinement around the FP32 PCG; every pass starts from
    // the true FP64 residual, so the last one is the reported residual
    int total = 0;
    bool conv = false;
    double rr = 0.0;
    for (int k = 0; k < 64 && total < c.maxiter; ++k) {
      if (!(k == 0 && r_ready)) {      // else formed on the side stream during the build
        fine_apply<double, double>(c.op, c.s64, u, c.r, b, nullptr, 0.0, AM_RES, c.st);
        ProfScope ps(PK_VECTOR, c.st);
        pcg_reset(c.pcg_out, c.st);
        dot<double, double>(n, c.r.p, c.r.p, c.part, c.pcg_out, DOT_RR, c.st);
      }
      read_pcg(c, c.pcg_out);
      rr = c.h_pcg->rr;
      check_finite(rr, "FP64 residual");
      if (std::sqrt(rr) < tol) {
        conv = true;
        break;
      }
      {
        ProfScope ps(PK_VECTOR, c.st);
        to_unit_f32(n, c.r, c.pcg_out, c.r32, c.st);
      }
      const double inner = std::max(c.inner_rtol, 0.5 * tol / std::sqrt(rr));
      // with multigrid at most 200 iterations per pass (a pass normally takes
      // 20-60): an FP32 recurrence that stalls -- seen on one design of a
      // 200-iteration run from random densities -- is restarted from the true
      // FP64 residual by the next pass
      const int cap = std::min(c.maxiter - total, c.precond == TG_PRECOND_GMG ? 200 : c.maxiter);
      pcg32_begin(c);
      int it = 0;
      if (c.ws_pending) {
        // the learned start is kept only if the residual after its first
        // cycle is below the plain warm start's (u_prev's) residual;
        // otherwise plain PCG from u_prev, without the deflation
        c.ws_pending = false;
        it = pcg32_run(c, inner, 1, 0);
        const double inner1 = std::sqrt(c.h_pcg->rr);
        const double r1 = std::sqrt(rr) * inner1;
        TG_CUDA(cudaMemcpyAsync(c.h_scal + 5, c.cnn->plain_rr(), sizeof(double),
                                cudaMemcpyDeviceToHost, c.st));
        TG_CUDA(cudaStreamSynchronize(c.st));
        const double r_plain = std::sqrt(c.h_scal[5]);
        c.last_warm_ratio = r_plain > 0.0 ? std::sqrt(rr) / r_plain : 0.0;
        if (!(r1 < r_plain)) {
          TG_CUDA(cudaMemcpyAsync(u, c.cnn->uprev.p, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                  c.st));
          set_correction(c.pcg, 0.0, c.st);
          c.last_fallback = 1;
          total += it;
          continue;    // the next pass starts from u_prev's true residual
        }
        if (inner1 >= inner && it < cap) it += pcg32_run(c, inner, cap, it);
      } else {
        it = pcg32_run(c, inner, cap, 0);
      }
      total += it;
      ProfScope ps(PK_VECTOR, c.st);
      add_scaled_f32(n, c.d32, c.pcg_out, u, c.st);
      c.last_refine = k + 1;
    }
    c.last_iters = total;
    c.last_vcycles = (c.precond == TG_PRECOND_GMG) ? total : 0;
    c.last_converged = conv;
    if (conv) c.last_relres = std::sqrt(rr) / bnorm;
  }
  if (c.precision == TG_PREC_FP64 || !c.last_converged) {
    // true FP64 residual (the FP64 PCG's recursive residual can drift from it)
    fine_apply<double, double>(c.op, c.s64, u, c.r, b, nullptr, 0.0, AM_RES, c.st);
    pcg_reset(c.pcg_out, c.st);
    dot<double, double>(n, c.r.p, c.r.p, c.part, c.pcg_out, DOT_RR, c.st);
    read_pcg(c, c.pcg_out);
    c.last_relres = std::sqrt(c.h_pcg->rr) / bnorm;
  }
  if (c.precond == TG_PRECOND_GMG) check_waits(c);
  if (!c.last_converged)
    throw Error{ENOTCONV, "gb300 pcg iteration did not converge (iterations: " +
                              std::to_string(c.last_iters) +
                              ", relative residual: " + std::to_string(c.last_relres) + ")"};
}

// ---------------------------------------------------------------------------
// one design iteration
// ---------------------------------------------------------------------------
void ctx_step(Ctx& c, tg_iter_out& out) {
  const auto t0 = std::chrono::steady_clock::now();
  const Grid& g = c.g;
  const int64_t nel = g.nel();
  set_density(c, c.xPhys);
  TG_CUDA(cudaEventRecord(c.ev0, c.st));
  // learned warm start and coarse-grid correction (kept only if the residual
  // after the solve's first cycle is below the plain warm start's; else the
  // solve falls back to plain PCG from the previous displacement); it needs
  // only the new scale factors, so it runs on the network's stream while
  // this stream builds the hierarchy
  const int lmask = c.learned & (TG_LEARNED_WARM_START | TG_LEARNED_COARSE_CORRECTION);
  const bool warm = lmask && c.cnn && c.cnn->trained && c.iter > 0 && c.nload == 1 &&
                    c.precision == TG_PREC_MIXED;
  c.last_fallback = 0;
  c.last_warm_ratio = 0.0;
  c.ws_pending = false;
  c.r_ready = false;
  if (!warm && correction_vector(c)) set_correction(c.pcg, 0.0, c.st);   // plain PCG
  // the mixed solve's first FP64 residual f - K u needs only the scale
  // factors too: on the side stream (after the warm start, which changes u)
  const bool side = c.precision == TG_PREC_MIXED && c.nload == 1;
  if (side) {
    TG_CUDA(cudaEventRecord(c.sev_fork, c.st));
    TG_CUDA(cudaStreamWaitEvent(c.side, c.sev_fork, 0));
    if (warm) {
      c.cnn->warm_start(c, (lmask & TG_LEARNED_WARM_START) != 0,
                        (lmask & TG_LEARNED_COARSE_CORRECTION) != 0, c.side);
      c.ws_pending = true;
    }
    fine_apply<double, double>(c.op, c.s64, c.u, c.r, c.f, nullptr, 0.0, AM_RES, c.side);
    {
      ProfScope ps(PK_VECTOR, c.side);
      pcg_reset(c.pcg_out, c.side);
      dot<double, double>(g.ndofs(), c.r.p, c.r.p, c.part, c.pcg_out, DOT_RR, c.side);
    }
    TG_CUDA(cudaEventRecord(c.sev_join, c.side));
  }
  build_hierarchy(c);
  if (side) {
    TG_CUDA(cudaStreamWaitEvent(c.st, c.sev_join, 0));
    c.r_ready = true;
  }
  // one solve per load case with the same hierarchy (topology_optimization.py:446-459)
  const int64_t nd = g.ndofs();
  int iters = 0, vcycles = 0, refine = 0;
  double relres = 0.0;
  for (int lc = 0; lc < c.nload; ++lc) {
    solve(c, c.f.p + lc * nd, c.u.p + lc * nd);
    iters += c.last_iters;
    vcycles += c.last_vcycles;
    refine += c.last_refine;
    relres = std::max(relres, c.last_relres);
  }
  TG_CUDA(cudaEventRecord(c.ev1, c.st));
  // compliance + raw sensitivity
  const int nbe = (int)red_blocks(nel);
  {
    ProfScope ps(PK_COMPLIANCE, c.st);
    // compliance and sensitivities summed over the load cases in fixed order
    // (topology_optimization.py:463-500; compliance is self-adjoint)
    for (int lc = 0; lc < c.nload; ++lc)
      fine_compliance(c.op, c.xPhys, c.u.p + lc * nd, c.eps, c.penal, c.dc, c.part, c.st,
                      c.flags.p, lc > 0);
    reduce_partials(c.part, nbe, c.scal.p + 0, false, c.st);
  }
  // sensitivity filter
  if (c.hf && c.ft == 1) helmholtz_apply(c, c.dc, nullptr, nullptr, c.dcf);
  else if (c.hf && c.ft == 0) helmholtz_apply(c, c.dc, c.xPhys, c.x, c.dcf);
  else if (c.ft == 1) filter_apply(g, c.fs, c.dc, nullptr, c.Hs, c.dcf, 1, c.st);
  else if (c.ft == 0) filter_apply(g, c.fs, c.x, c.dc, c.Hs, c.dcf, 2, c.st);
  else TG_CUDA(cudaMemcpyAsync(c.dcf.p, c.dc.p, sizeof(double) * nel, cudaMemcpyDeviceToDevice, c.st));
  // OC
  const OCScratch ocs{c.S.p, c.S.p + nel, c.S.p + 2 * nel, c.S32.p};
  // the whole bisection in one launch; its state is read back with the
  // iteration's scalars at the end (no host round trip in between)
  oc_begin(nel, c.x, c.dcf, c.dv, c.flags.p, c.move, ocs, c.oc, c.g_oc, c.st);
  oc_steps(nel, c.x, ocs, c.dv, c.flags.p, c.move, c.part2, c.oc, 256, c.st);
  oc_finish(nel, c.x, ocs, c.flags.p, c.move, c.xnew, c.oc, c.st);
  TG_CUDA(cudaMemcpyAsync(c.h_oc, c.oc.p, sizeof(OCState), cudaMemcpyDeviceToHost, c.st));
  // x_old <- x ; x <- x_new
  std::swap(c.xold.p, c.x.p);
  std::swap(c.x.p, c.xnew.p);
  // density filter (or copy) fused with the volume sum and max |x - x_old|
  if (c.hf && c.ft == 1)
    helmholtz_apply(c, c.x, nullptr, nullptr, c.xPhys, c.x, c.xold, c.part, c.part2);
  else
    filter_apply_ex(g, c.fs, c.x, nullptr, c.Hs, c.xPhys, c.ft == 1 ? 0 : 4, c.xold, c.part,
                    c.part2, c.st);
  reduce_partials(c.part, nbe, c.scal.p + 1, false, c.st);
  reduce_partials(c.part2, nbe, c.scal.p + 2, true, c.st);
  TG_CUDA(cudaMemcpyAsync(c.h_scal, c.scal.p, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.st));
  TG_CUDA(cudaStreamSynchronize(c.st));
  if (c.h_oc->bar.err) throw Error{ETIMEOUT, "OC bisection: a grid barrier wait timed out"};
  if (!c.h_oc->done) throw Error{ENOTCONV, "OC bisection did not terminate within 256 steps"};
  c.g_oc = c.h_oc->gt;
  const int fallback = c.last_fallback;
  const double vol_sum = c.h_scal[1];
  float ms = 0.f;
  TG_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
  out.obj = c.h_scal[0];
  out.vol = vol_sum / (double)c.rg.nel();   // padding elements hold 0
  out.change = c.h_scal[2];
  out.g = c.g_oc;
  out.rel_res = relres;
  out.pcg_iters = iters;
  out.vcycles = vcycles;
  out.refinements = refine;
  out.oc_steps = c.h_oc->nsteps;
  out.fallback = fallback;
  out.nlevels = c.L;
  out.t_solve_ms = ms;
  out.warm_ratio = c.last_warm_ratio;
  check_finite(out.obj, "objective");
  c.iter++;
  out.t_step_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace tg
