// The learned warm-start network (see tg_cnn.cu).
#pragma once
#include <vector>
#include "tg_ctx.cuh"

namespace tg {

// node grid of one network level
struct NG {
  int nx, ny, nz;
  __host__ __device__ int64_t n() const { return (int64_t)nx * ny * nz; }
};

struct Layer {
  int cin, cout;
  int64_t w_off, b_off;    // offsets of W[27][cin][cout] and b[cout] in the parameter buffer
};

struct Cnn {
  Ctx* ctx;
  NG A{}, B{}, Cg{};               // full / half / quarter of the level-1 node grid
  std::vector<Layer> layers;
  int64_t nparams = 0;
  DevBuf<float> params, grads, adam_m, adam_v, wt;
  // per layer the TF32 weight images the tensor-core convolution streams
  // into shared memory (rebuilt from params by every TF32 forward)
  DevBuf<float> wpack;
  int64_t wpack_off[6] = {};
  // activations (channels-last) and their gradients
  DevBuf<float> x0, e1, p1, e2, p2, e3, u2, d2, u1, d1, y, tgt;
  DevBuf<float> g_a16, g_a32, g_b64, g_b32, g_b16, g_c64, g_c32, g_e1, g_e2, g_y;
  DevBuf<float> dw_part;
  DevBuf<double> loss_part, loss_out;
  // training set recorded from solver runs
  int capacity_ = 0, nsamples = 0;
  DevBuf<float> data_x, data_t;
  // solver-state scratch; w32: the prolongated network output (the deflation
  // vector of the FP32 PCG in the solve that follows), aw32 = K w32; rc32:
  // the residual restricted to the level-1 grid, a network input
  DevBuf<double> uprev, corr;
  DevBuf<float> r32a, w32, aw32, rc32;
  DevBuf<PCGState> su, sr, src;  // norms of u_prev, of its residual, of the restricted residual
  DevBuf<PCGState> gal;          // the five products of the 2x2 Galerkin combination
  DevBuf<double> wsb;            // c1, c2, valid of the last warm start
  DevBuf<double> rpart;          // reduction partials of the network's own dots
  float lr = 1e-3f;
  int adam_t = 0;
  bool trained = false;

  Cnn(Ctx& c, int capacity, uint64_t seed);
  Cnn(const Cnn&) = delete;
  Cnn& operator=(const Cnn&) = delete;
  // split: FP32-level split-TF32 products (training, checks); otherwise TF32
  void forward(cudaStream_t st, bool split = true);
  void pack_umma(cudaStream_t st);
  double backward(cudaStream_t st, bool want_loss);
  void adam_step(cudaStream_t st);
  void features(Ctx& c, const double* u_prev);
  void record_begin(Ctx& c);
  void record_end(Ctx& c);
  double train(int epochs, float lr, uint64_t seed);
  // Adam over n caller-provided pairs (host x0s [n][nodes][7], targets
  // [n][nodes][3]), one step per pair in a seeded shuffled order per epoch
  double fit(int n, const float* x0s, const float* targets, int epochs, float lr, uint64_t seed);
  // Candidate warm start and coarse-grid correction for the current design:
  // uprev <- u; with combine, u <- c1 u + c2 w (w = P y, energy-optimal c);
  // with correction, c.pcg gets 1 / (w^T K w) and w deflates the FP32 PCG
  // (else 0).  The plain warm start's residual norm^2 stays in plain_rr()
  // (device) for the fallback test after the first cycle of the solve.
  // The work is enqueued on stream s (the context's side stream, which the
  // caller has made wait for the design's scale factors); it does not touch
  // the multigrid hierarchy, so it overlaps the hierarchy's build.
  void warm_start(Ctx& c, bool combine, bool correction, cudaStream_t s);
  const double* plain_rr() const { return &sr.p->rr; }
};

}  // namespace tg
