// extern "C" entry points (include/topopt_gb300.h).  Every call catches the
// library's exceptions and turns them into a status code plus a message;
// nothing aborts and no device code traps.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>
#include "tg_ctx.cuh"
#include "tg_cnn.cuh"
#include "../../include/topopt_gb300.h"

struct tg_ctx {
  tg::Ctx c;
};

namespace {
thread_local std::string g_last_error;

// programmatic dependent launch for mixed-precision contexts only (restored
// on every exit)
struct PdlScope {
  int prev;
  explicit PdlScope(tg_ctx* ctx)
      : prev(tg::pdl_scope(!ctx || ctx->c.precision == TG_PREC_MIXED ? 1 : 0)) {}
  ~PdlScope() { tg::pdl_scope(prev); }
};

template <typename F>
int32_t guarded(tg_ctx* ctx, F&& fn) {
  PdlScope pdl(ctx);
  try {
    if (ctx) TG_CUDA(cudaSetDevice(ctx->c.dev));
    fn();
    return TG_OK;
  } catch (const tg::Error& e) {
    if (ctx) ctx->c.err = e.msg;
    g_last_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->c.err = "host out of memory";
    g_last_error = "host out of memory";
    return TG_ENOMEM;
  } catch (const std::exception& e) {
    if (ctx) ctx->c.err = e.what();
    g_last_error = e.what();
    return TG_ECUDA;
  }
}

template <typename T>
void h2d(T* dst, const T* src, int64_t n, cudaStream_t st) {
  TG_CUDA(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, st));
}
template <typename T>
void d2h(T* dst, const T* src, int64_t n, cudaStream_t st) {
  TG_CUDA(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
  TG_CUDA(cudaStreamSynchronize(st));
}

// device array of a field; n = its length in the caller's numbering (u and f:
// all load cases, one vector after another)
double* field_ptr(tg::Ctx& c, int32_t field, int64_t& n, bool& nodes) {
  nodes = field == TG_FIELD_U || field == TG_FIELD_F;
  n = nodes ? c.rg.ndofs() * c.nload : c.rg.nel();
  switch (field) {
    case TG_FIELD_X: return c.x;
    case TG_FIELD_XPHYS: return c.xPhys;
    case TG_FIELD_U: return c.u;
    case TG_FIELD_DC: return c.dcf;
    case TG_FIELD_DV: return c.dv;
    case TG_FIELD_F: return c.f;
    default: throw tg::Error{TG_EINVAL, "unknown field"};
  }
}

// host (caller numbering) -> device array (device numbering), and back; on a
// padded grid through the staging buffer and the embedding kernel (the
// padding entries of dst keep their values)
void put_field(tg::Ctx& c, double* dev, const double* host, bool nodes) {
  const int64_t n = nodes ? c.rg.ndofs() : c.rg.nel();
  if (!c.padded) {
    h2d(dev, host, n, c.st);
    return;
  }
  h2d(c.emb.p, host, n, c.st);
  tg::embed_copy(c.rg, c.g, nodes, c.emb, dev, true, c.st);
}
void get_field(tg::Ctx& c, double* host, const double* dev, bool nodes) {
  const int64_t n = nodes ? c.rg.ndofs() : c.rg.nel();
  if (!c.padded) {
    d2h(host, dev, n, c.st);
    return;
  }
  tg::embed_copy(c.rg, c.g, nodes, dev, c.emb, false, c.st);
  d2h(host, c.emb.p, n, c.st);
}
void require_unpadded(const tg::Ctx& c, const char* what) {
  if (c.padded)
    throw tg::Error{TG_EINVAL, std::string(what) + ": not available for a grid embedded in a "
                               "padded device grid (its element counts do not coarsen)"};
}
}  // namespace

extern "C" {

int32_t tg_abi_version(void) { return TG_ABI_VERSION; }

const char* tg_last_error(const tg_ctx* ctx) {
  if (ctx) return ctx->c.err.c_str();
  return g_last_error.c_str();
}

int32_t tg_create(const tg_problem* prob, tg_ctx** out) {
  if (!prob || !out) {
    g_last_error = "tg_create: NULL argument";
    return TG_EINVAL;
  }
  *out = nullptr;
  tg_ctx* ctx = nullptr;
  try {
    ctx = new tg_ctx();
  } catch (...) {
    g_last_error = "host out of memory";
    return TG_ENOMEM;
  }
  const int32_t rc = guarded(nullptr, [&] { tg::ctx_init(ctx->c, *prob); });
  if (rc != TG_OK) {
    delete ctx;
    return rc;
  }
  *out = ctx;
  return TG_OK;
}

void tg_destroy(tg_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->c.dev);
  if (ctx->c.st) cudaStreamSynchronize(ctx->c.st);
  delete ctx;
}

int32_t tg_step(tg_ctx* ctx, tg_iter_out* out) {
  if (!ctx || !out) return TG_EINVAL;
  return guarded(ctx, [&] { tg::ctx_step(ctx->c, *out); });
}

int32_t tg_step_many(tg_ctx* const* ctxs, int32_t n, tg_iter_out* outs, int32_t* rcs,
                     int32_t nthreads) {
  if (!ctxs || !outs || !rcs || n < 0) return TG_EINVAL;
  for (int32_t i = 0; i < n; ++i)
    if (!ctxs[i]) return TG_EINVAL;
  const int nt = (int)std::max<int32_t>(1, std::min<int32_t>(n, nthreads > 0 ? nthreads : 16));
  std::atomic<int32_t> next{0};
  auto worker = [&] {
    for (int32_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
      tg_ctx* ctx = ctxs[i];
      rcs[i] = guarded(ctx, [&] {
        TG_CUDA(cudaSetDevice(ctx->c.dev));
        tg::ctx_step(ctx->c, outs[i]);
      });
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
  for (int32_t i = 0; i < n; ++i)
    if (rcs[i] != TG_OK) return rcs[i];
  return TG_OK;
}

int32_t tg_get(tg_ctx* ctx, int32_t field, double* host, int64_t n) {
  if (!ctx || !host) return TG_EINVAL;
  return guarded(ctx, [&] {
    int64_t m = 0;
    bool nodes = false;
    double* p = field_ptr(ctx->c, field, m, nodes);
    TG_REQUIRE(n == m, "tg_get: wrong element count");
    const int nv = nodes ? ctx->c.nload : 1;
    for (int k = 0; k < nv; ++k)
      get_field(ctx->c, host + k * (m / nv), p + k * ctx->c.g.ndofs(), nodes);
  });
}

int32_t tg_set(tg_ctx* ctx, int32_t field, const double* host, int64_t n) {
  if (!ctx || !host) return TG_EINVAL;
  return guarded(ctx, [&] {
    tg::Ctx& c = ctx->c;
    int64_t m = 0;
    bool nodes = false;
    double* p = field_ptr(c, field, m, nodes);
    TG_REQUIRE(n == m, "tg_set: wrong element count");
    const int nv = nodes ? c.nload : 1;
    for (int k = 0; k < nv; ++k) put_field(c, p + k * c.g.ndofs(), host + k * (m / nv), nodes);
    if (field == TG_FIELD_F || field == TG_FIELD_U)
      for (int k = 0; k < c.nload; ++k)
        tg::mask_vec_f64(c.g.nnodes(), c.g.ndof, c.op.fix, p + k * c.g.ndofs(), c.st);
    TG_CUDA(cudaStreamSynchronize(c.st));
  });
}

int32_t tg_kmul(tg_ctx* ctx, const double* xPhys, const double* u, double* y, int32_t precision) {
  if (!ctx || !xPhys || !u || !y) return TG_EINVAL;
  return guarded(ctx, [&] {
    tg::Ctx& c = ctx->c;
    require_unpadded(c, "tg_kmul");
    const int64_t nel = c.g.nel(), nd = c.g.ndofs();
    h2d(c.xnew.p, xPhys, nel, c.st);
    h2d(c.r.p, u, nd, c.st);
    // the operator expects inputs that are zero on fixed DOFs
    tg::mask_vec_f64(c.g.nnodes(), c.g.ndof, c.op.fix, c.r, c.st);
    if (precision == TG_PREC_FP64) {
      tg::simp_scale(nel, c.xnew, c.eps, c.penal, c.s64, nullptr, nullptr, c.st);
      tg::fine_apply<double, double>(c.op, c.s64, c.r, c.q, nullptr, nullptr, 0.0, tg::AM_Y, c.st);
      d2h(y, c.q.p, nd, c.st);
    } else {
      TG_REQUIRE(c.precision == TG_PREC_MIXED, "tg_kmul: FP32 path needs a mixed-precision context");
      tg::simp_scale(nel, c.xnew, c.eps, c.penal, nullptr, c.s32, nullptr, c.st);
      tg::d2f(nd, c.r, c.p32, c.st);
      tg::fine_apply<float, float>(c.op, c.s32, c.p32, c.q32, nullptr, nullptr, 0.0, tg::AM_Y, c.st);
      std::vector<float> tmp(nd);
      d2h(tmp.data(), c.q32.p, nd, c.st);
      for (int64_t i = 0; i < nd; ++i) y[i] = tmp[i];
    }
  });
}

int32_t tg_solve(tg_ctx* ctx, const double* xPhys, const double* rhs, const double* u0, double* u,
                 tg_solve_info* info) {
  if (!ctx || !xPhys || !rhs || !u) return TG_EINVAL;
  tg::Ctx& c = ctx->c;
  const int32_t rc = guarded(ctx, [&] {
    const int64_t nd = c.g.ndofs();
    TG_CUDA(cudaMemsetAsync(c.xnew.p, 0, sizeof(double) * c.g.nel(), c.st));
    TG_CUDA(cudaMemsetAsync(c.z.p, 0, sizeof(double) * nd, c.st));
    TG_CUDA(cudaMemsetAsync(c.p.p, 0, sizeof(double) * nd, c.st));
    put_field(c, c.xnew.p, xPhys, false);
    tg::set_density(c, c.xnew);
    tg::build_hierarchy(c);
    put_field(c, c.z.p, rhs, true);
    tg::mask_vec_f64(c.g.nnodes(), c.g.ndof, c.op.fix, c.z, c.st);
    if (u0) put_field(c, c.p.p, u0, true);
    // solve() uses r, q and the level buffers; rhs lives in z, the iterate in a
    // dedicated copy so the PCG vectors stay free
    std::vector<double> host(nd);
    tg::DevBuf<double> b, x;
    b.alloc(nd);
    x.alloc(nd);
    TG_CUDA(cudaMemcpyAsync(b.p, c.z.p, sizeof(double) * nd, cudaMemcpyDeviceToDevice, c.st));
    TG_CUDA(cudaMemcpyAsync(x.p, c.p.p, sizeof(double) * nd, cudaMemcpyDeviceToDevice, c.st));
    tg::solve(c, b, x);
    get_field(c, u, x.p, true);
  });
  if (info) {
    info->iters = c.last_iters;
    info->vcycles = c.last_vcycles;
    info->refinements = c.last_refine;
    info->converged = c.last_converged;
    info->rel_res = c.last_relres;
  }
  return rc;
}

int32_t tg_adjoint(tg_ctx* ctx, const double* u, const double* rhs_adj, double* adj, double* dobj,
                   tg_solve_info* info) {
  if (!ctx || !u || !rhs_adj || !adj) return TG_EINVAL;
  tg::Ctx& c = ctx->c;
  const int32_t rc = guarded(ctx, [&] {
    require_unpadded(c, "tg_adjoint");
    TG_REQUIRE(c.built, "tg_adjoint reuses the operator of a state solve: call tg_step or "
                        "tg_solve first");
    const int64_t nd = c.g.ndofs(), nel = c.g.nel();
    tg::DevBuf<double> uu, b, x;
    uu.alloc(nd);
    b.alloc(nd);
    x.alloc(nd);
    h2d(uu.p, u, nd, c.st);
    h2d(b.p, rhs_adj, nd, c.st);
    tg::mask_vec_f64(c.g.nnodes(), c.g.ndof, c.op.fix, b, c.st);
    tg::mask_vec_f64(c.g.nnodes(), c.g.ndof, c.op.fix, uu, c.st);
    x.zero(c.st);
    tg::solve(c, b, x);                 // the state solve's scale factors and hierarchy
    d2h(adj, x.p, nd, c.st);
    if (dobj) {
      tg::fine_adjoint_sens(c.op, c.xsolved, uu, x, c.eps, c.penal, c.dc, c.st, c.flags.p);
      d2h(dobj, c.dc.p, nel, c.st);
    }
  });
  if (info) {
    info->iters = c.last_iters;
    info->vcycles = c.last_vcycles;
    info->refinements = c.last_refine;
    info->converged = c.last_converged;
    info->rel_res = c.last_relres;
  }
  return rc;
}

int32_t tg_filter(tg_ctx* ctx, const double* x, const double* d, double* y, int32_t mode) {
  const bool pde = mode == 6 || mode == 7;
  if (!ctx || !y || mode < 0 || (mode > 3 && !pde) || (mode != 3 && !x) ||
      ((mode == 2 || mode == 7) && !d))
    return TG_EINVAL;
  if (pde && !ctx->c.hf) return TG_EINVAL;
  return guarded(ctx, [&] {
    tg::Ctx& c = ctx->c;
    require_unpadded(c, "tg_filter");
    const int64_t nel = c.g.nel();
    if (x) h2d(c.xnew.p, x, nel, c.st);
    if (d) h2d(c.S.p, d, nel, c.st);
    if (mode == 6) tg::helmholtz_apply(c, c.xnew, nullptr, nullptr, c.dc);
    else if (mode == 7) tg::helmholtz_apply(c, c.S, c.xnew, c.xnew, c.dc);
    else tg::filter_apply(c.g, c.fs, c.xnew, c.S, c.Hs, c.dc, mode, c.st);
    d2h(y, c.dc.p, nel, c.st);
  });
}

int32_t tg_compliance(tg_ctx* ctx, const double* xPhys, const double* u, double* obj, double* dc) {
  if (!ctx || !xPhys || !u || !obj) return TG_EINVAL;
  return guarded(ctx, [&] {
    tg::Ctx& c = ctx->c;
    require_unpadded(c, "tg_compliance");
    const int64_t nel = c.g.nel(), nd = c.g.ndofs();
    h2d(c.xnew.p, xPhys, nel, c.st);
    h2d(c.r.p, u, nd, c.st);
    tg::fine_compliance(c.op, c.xnew, c.r, c.eps, c.penal, c.dc, c.part, c.st);
    tg::reduce_partials(c.part, (int)tg::red_blocks(nel), c.scal.p, false, c.st);
    d2h(obj, c.scal.p, 1, c.st);
    if (dc) d2h(dc, c.dc.p, nel, c.st);
  });
}

int32_t tg_oc(tg_ctx* ctx, const double* x, const double* dc, const double* dv, double g,
              double* xnew, double* gt, int32_t* nsteps) {
  if (!ctx || !x || !dc || !dv || !xnew) return TG_EINVAL;
  return guarded(ctx, [&] {
    tg::Ctx& c = ctx->c;
    require_unpadded(c, "tg_oc");
    const int64_t nel = c.g.nel();
    tg::DevBuf<double> xd, dcd, dvd, xn;
    xd.alloc(nel); dcd.alloc(nel); dvd.alloc(nel); xn.alloc(nel);
    h2d(xd.p, x, nel, c.st);
    h2d(dcd.p, dc, nel, c.st);
    h2d(dvd.p, dv, nel, c.st);
    const tg::OCScratch ocs{c.S.p, c.S.p + nel, c.S.p + 2 * nel, c.S32.p};
    tg::oc_begin(nel, xd, dcd, dvd, c.flags.p, c.move, ocs, c.oc, g, c.st);
    tg::oc_steps(nel, xd, ocs, dvd, c.flags.p, c.move, c.part2, c.oc, 256, c.st);
    d2h(c.h_oc, c.oc.p, 1, c.st);
    if (c.h_oc->bar.err) throw tg::Error{TG_ETIMEOUT, "OC bisection: a grid barrier wait timed out"};
    if (!c.h_oc->done) throw tg::Error{TG_ENOTCONV, "OC bisection did not terminate"};
    tg::oc_finish(nel, xd, ocs, c.flags.p, c.move, xn, c.oc, c.st);
    d2h(xnew, xn.p, nel, c.st);
    if (gt) *gt = c.h_oc->gt;
    if (nsteps) *nsteps = c.h_oc->nsteps;
  });
}

int32_t tg_oc_raw(int64_t n, const double* x, const double* dc, const double* dv, double g,
                  const int8_t* el_flags, double move, double l1, double l2, double* xnew,
                  double* gt, int32_t* nsteps, int32_t device) {
  if (!x || !dc || !dv || !xnew || n <= 0) return TG_EINVAL;
  return guarded(nullptr, [&] {
    TG_CUDA(cudaSetDevice(device));
    cudaStream_t st = 0;
    tg::DevBuf<double> xd, dcd, dvd, xn, S, part;
    tg::DevBuf<float> S32;
    tg::DevBuf<int8_t> fl;
    tg::DevBuf<tg::OCState> oc;
    xd.alloc(n); dcd.alloc(n); dvd.alloc(n); xn.alloc(n); S.alloc(3 * n); part.alloc(tg::RED_BLOCKS);
    S32.alloc(5 * n);
    oc.alloc(1);
    h2d(xd.p, x, n, st);
    h2d(dcd.p, dc, n, st);
    h2d(dvd.p, dv, n, st);
    if (el_flags) {
      fl.alloc(n);
      h2d(fl.p, el_flags, n, st);
    }
    tg::OCState h;
    const tg::OCScratch ocs{S.p, S.p + n, S.p + 2 * n, S32.p};
    tg::oc_begin(n, xd, dcd, dvd, fl.p, move, ocs, oc, g, st, l1, l2);
    tg::oc_steps(n, xd, ocs, dvd, fl.p, move, part, oc, 256, st);
    d2h(&h, oc.p, 1, st);
    if (h.bar.err) throw tg::Error{TG_ETIMEOUT, "OC bisection: a grid barrier wait timed out"};
    if (!h.done) throw tg::Error{TG_ENOTCONV, "OC bisection did not terminate"};
    tg::oc_finish(n, xd, ocs, fl.p, move, xn, oc, st);
    d2h(xnew, xn.p, n, st);
    if (gt) *gt = h.gt;
    if (nsteps) *nsteps = h.nsteps;
  });
}

int32_t tg_vcycle(tg_ctx* ctx, const double* xPhys, const double* b, double* x, int32_t precision) {
  if (!ctx || !xPhys || !b || !x) return TG_EINVAL;
  return guarded(ctx, [&] {
    tg::Ctx& c = ctx->c;
    TG_REQUIRE(c.precond == TG_PRECOND_GMG, "tg_vcycle needs a multigrid context");
    require_unpadded(c, "tg_vcycle");
    const int64_t nel = c.g.nel(), nd = c.g.ndofs();
    h2d(c.xnew.p, xPhys, nel, c.st);
    tg::set_density(c, c.xnew);
    tg::build_hierarchy(c);
    h2d(c.r.p, b, nd, c.st);
    tg::mask_vec_f64(c.g.nnodes(), c.g.ndof, c.op.fix, c.r, c.st);
    if (precision == TG_PREC_FP64) {
      TG_REQUIRE(c.precision == TG_PREC_FP64 || c.L == 1,
                 "an FP64 V-cycle needs an fp64 context (mixed contexts build FP32 levels)");
      tg::vcycle<double>(c, 0, c.r, c.z);
      d2h(x, c.z.p, nd, c.st);
      tg::check_waits(c);
    } else {
      TG_REQUIRE(c.precision == TG_PREC_MIXED, "FP32 V-cycle needs a mixed-precision context");
      tg::d2f(nd, c.r, c.r32, c.st);
      tg::vcycle<float>(c, 0, c.r32, c.z32);
      std::vector<float> tmp(nd);
      d2h(tmp.data(), c.z32.p, nd, c.st);
      for (int64_t i = 0; i < nd; ++i) x[i] = tmp[i];
      tg::check_waits(c);
    }
  });
}

int32_t tg_levels(tg_ctx* ctx, int32_t* nlevels, int64_t* ndofs) {
  if (!ctx || !nlevels) return TG_EINVAL;
  return guarded(ctx, [&] {
    *nlevels = ctx->c.L;
    if (ndofs)
      for (int l = 0; l < ctx->c.L && l < 8; ++l) ndofs[l] = ctx->c.lv[l]->g.ndofs();
  });
}

int32_t tg_coarse_stencil(tg_ctx* ctx, const double* xPhys, int32_t level, double* out, int64_t n) {
  if (!ctx || !xPhys || !out) return TG_EINVAL;
  return guarded(ctx, [&] {
    tg::Ctx& c = ctx->c;
    TG_REQUIRE(c.precond == TG_PRECOND_GMG, "no multigrid hierarchy");
    require_unpadded(c, "tg_coarse_stencil");
    TG_REQUIRE(level >= 1 && level < c.L, "level out of range");
    tg::Level& v = *c.lv[level];
    TG_REQUIRE(n == v.g.nnodes() * (v.g.ndim == 3 ? 27 : 9) * v.g.ndof * v.g.ndof,
               "tg_coarse_stencil: wrong element count");
    h2d(c.xnew.p, xPhys, c.g.nel(), c.st);
    tg::set_density(c, c.xnew);
    tg::build_hierarchy(c);
    tg::DevBuf<double> full;
    full.alloc(n);
    if (c.precision == TG_PREC_MIXED) tg::stencil_expand<float>(v.g, v.A32, full, c.st);
    else tg::stencil_expand<double>(v.g, v.A64, full, c.st);
    d2h(out, full.p, n, c.st);
  });
}

int32_t tg_timer(tg_ctx* ctx, int32_t op, double* ms) {
  if (!ctx) return TG_EINVAL;
  return guarded(ctx, [&] {
    tg::Ctx& c = ctx->c;
    if (op == 0) {
      TG_CUDA(cudaEventRecord(c.tev0, c.st));
    } else {
      TG_CUDA(cudaEventRecord(c.tev1, c.st));
      TG_CUDA(cudaEventSynchronize(c.tev1));
      float t = 0.f;
      TG_CUDA(cudaEventElapsedTime(&t, c.tev0, c.tev1));
      if (ms) *ms = t;
    }
  });
}

int32_t tg_dense_inverse(const double* A, int64_t n, double* Ainv, int32_t mode, int32_t device) {
  if (!A || !Ainv || n <= 0 || n > 8192 || mode < 0 || mode > 2) return TG_EINVAL;
  return guarded(nullptr, [&] {
    TG_CUDA(cudaSetDevice(device));
    const int64_t ld = tg::cdiv(n, 32) * 32;
    // padding rows and columns hold the identity
    std::vector<double> h((size_t)(ld * ld), 0.0);
    for (int64_t i = 0; i < n; ++i)
      for (int64_t j = 0; j < n; ++j) h[(size_t)(i * ld + j)] = A[i * n + j];
    for (int64_t i = n; i < ld; ++i) h[(size_t)(i * ld + i)] = 1.0;
    tg::DevBuf<double> D, work;
    D.alloc(ld * ld);
    work.alloc(32 * 32 + 2 * 32 * ld);
    TG_CUDA(cudaMemcpy(D.p, h.data(), sizeof(double) * ld * ld, cudaMemcpyHostToDevice));
    if (mode == 0) tg::gj_inverse(D, n, ld, work, 0);
    else tg::gj_inverse_dw(D, n, ld, work, 0, mode == 1);
    TG_CUDA(cudaMemcpy(h.data(), D.p, sizeof(double) * ld * ld, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; ++i)
      for (int64_t j = 0; j < n; ++j) Ainv[i * n + j] = h[(size_t)(i * ld + j)];
  });
}

int32_t tg_edofmat(int32_t ndim, int32_t nelx, int32_t nely, int32_t nelz, int32_t nnode_dof,
                   int32_t* out, int32_t device) {
  if (!out) return TG_EINVAL;
  return guarded(nullptr, [&] {
    TG_REQUIRE((ndim == 2 || ndim == 3) && nelx > 0 && nely > 0 && (ndim == 2 || nelz > 0) &&
                   nnode_dof > 0 && nnode_dof <= 3,
               "tg_edofmat: bad arguments");
    TG_CUDA(cudaSetDevice(device));
    const tg::Grid g = tg::make_grid(ndim, nnode_dof, nelx, nely, nelz);
    const int64_t n = g.nel() * (1 << ndim) * nnode_dof;
    tg::DevBuf<int32_t> d;
    d.alloc(n);
    tg::edofmat(g, d, 0);
    TG_CUDA(cudaMemcpy(out, d.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  });
}

// ---------------------------------------------------------------------------
// learned warm start
// ---------------------------------------------------------------------------
struct tg_cnn {
  tg_ctx* owner;
  tg::Cnn* net;
};

int32_t tg_cnn_create(tg_ctx* ctx, int32_t capacity, uint64_t seed, tg_cnn** out) {
  if (!ctx || !out || capacity < 0) return TG_EINVAL;
  *out = nullptr;
  return guarded(ctx, [&] {
    tg_cnn* w = new tg_cnn{ctx, nullptr};
    try {
      w->net = new tg::Cnn(ctx->c, capacity, seed);
    } catch (...) {
      delete w;
      throw;
    }
    *out = w;
  });
}

void tg_cnn_destroy(tg_cnn* cnn) {
  if (!cnn) return;
  if (cnn->owner && cnn->owner->c.cnn == cnn->net) cnn->owner->c.cnn = nullptr;
  cudaSetDevice(cnn->owner->c.dev);
  cudaStreamSynchronize(cnn->owner->c.st);
  delete cnn->net;
  delete cnn;
}

int32_t tg_cnn_attach(tg_ctx* ctx, tg_cnn* cnn) {
  if (!ctx) return TG_EINVAL;
  return guarded(ctx, [&] {
    TG_REQUIRE(!cnn || cnn->owner == ctx, "the network belongs to another context");
    ctx->c.cnn = cnn ? cnn->net : nullptr;
    if (cnn && (ctx->c.learned & (TG_LEARNED_WARM_START | TG_LEARNED_COARSE_CORRECTION)) == 0)
      ctx->c.learned = TG_LEARNED_WARM_START;
  });
}

// training pairs may come from any context on the same device with the
// network's grids (e.g. runs of other volume fractions or start designs)
static void require_same_grids(const tg_cnn* cnn, const tg_ctx* ctx) {
  const tg::Ctx& a = cnn->owner->c;
  const tg::Ctx& b = ctx->c;
  TG_REQUIRE(a.dev == b.dev && a.g.nex == b.g.nex && a.g.ney == b.g.ney && a.g.nez == b.g.nez &&
                 a.g.ndof == b.g.ndof && b.L >= 2 && b.lv[1]->g.nnx == a.lv[1]->g.nnx &&
                 b.lv[1]->g.nny == a.lv[1]->g.nny && b.lv[1]->g.nnz == a.lv[1]->g.nnz,
             "the context's grids differ from the network's");
}

int32_t tg_cnn_record_begin(tg_cnn* cnn, tg_ctx* ctx) {
  if (!cnn || !ctx) return TG_EINVAL;
  return guarded(ctx, [&] {
    require_same_grids(cnn, ctx);
    cnn->net->record_begin(ctx->c);
  });
}

int32_t tg_cnn_record_end(tg_cnn* cnn, tg_ctx* ctx) {
  if (!cnn || !ctx) return TG_EINVAL;
  return guarded(ctx, [&] {
    require_same_grids(cnn, ctx);
    cnn->net->record_end(ctx->c);
  });
}

int32_t tg_cnn_train(tg_cnn* cnn, int32_t epochs, double lr, uint64_t seed, double* final_loss) {
  if (!cnn || epochs < 1) return TG_EINVAL;
  return guarded(cnn->owner, [&] {
    const double l = cnn->net->train(epochs, (float)lr, seed);
    if (final_loss) *final_loss = l;
  });
}

int32_t tg_cnn_fit(tg_cnn* cnn, int32_t n, const float* x0s, const float* targets, int32_t epochs,
                   double lr, uint64_t seed, double* final_loss) {
  if (!cnn || n < 1 || !x0s || !targets || epochs < 1) return TG_EINVAL;
  return guarded(cnn->owner, [&] {
    const double l = cnn->net->fit(n, x0s, targets, epochs, (float)lr, seed);
    if (final_loss) *final_loss = l;
  });
}

int32_t tg_cnn_info(tg_cnn* cnn, int64_t* nparams, int32_t* grid_dims, int32_t* nsamples) {
  if (!cnn) return TG_EINVAL;
  return guarded(cnn->owner, [&] {
    if (nparams) *nparams = cnn->net->nparams;
    if (grid_dims) {
      grid_dims[0] = cnn->net->A.nx;
      grid_dims[1] = cnn->net->A.ny;
      grid_dims[2] = cnn->net->A.nz;
    }
    if (nsamples) *nsamples = cnn->net->nsamples;
  });
}

int32_t tg_cnn_params(tg_cnn* cnn, int32_t set, float* host, int64_t n) {
  if (!cnn || !host) return TG_EINVAL;
  return guarded(cnn->owner, [&] {
    TG_REQUIRE(n == cnn->net->nparams, "tg_cnn_params: wrong element count");
    cudaStream_t st = cnn->owner->c.st;
    if (set) {
      h2d(cnn->net->params.p, host, n, st);
      TG_CUDA(cudaStreamSynchronize(st));
      cnn->net->trained = true;   // loaded weights count as a trained network
    } else {
      d2h(host, cnn->net->params.p, n, st);
    }
  });
}

int32_t tg_cnn_eval(tg_cnn* cnn, const float* x0, const float* target, float* y, double* loss,
                    float* grads) {
  if (!cnn || !x0) return TG_EINVAL;
  return guarded(cnn->owner, [&] {
    tg::Cnn& net = *cnn->net;
    cudaStream_t st = cnn->owner->c.st;
    const int64_t na = net.A.n();
    h2d(net.x0.p, x0, na * 7, st);
    net.forward(st);
    if (y) d2h(y, net.y.p, na * 3, st);
    if (target) {
      h2d(net.tgt.p, target, na * 3, st);
      const double l = net.backward(st, true);
      if (loss) *loss = l;
      if (grads) d2h(grads, net.grads.p, net.nparams, st);
    }
    TG_CUDA(cudaStreamSynchronize(st));
  });
}

int32_t tg_cnn_infer(tg_cnn* cnn, const float* x0, float* y) {
  if (!cnn || !x0 || !y) return TG_EINVAL;
  return guarded(cnn->owner, [&] {
    tg::Cnn& net = *cnn->net;
    cudaStream_t st = cnn->owner->c.st;
    const int64_t na = net.A.n();
    h2d(net.x0.p, x0, na * 7, st);
    net.forward(st, false);
    d2h(y, net.y.p, na * 3, st);
    TG_CUDA(cudaStreamSynchronize(st));
    if (tg::take_conv_error(st))
      throw tg::Error{tg::ETIMEOUT, "tensor-core convolution: a bounded wait timed out"};
  });
}

}  // extern "C"
