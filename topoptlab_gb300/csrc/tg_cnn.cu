// Learned warm start: a small 3-D convolutional encoder-decoder trained on the
// GPU by the library's own forward / backward / Adam kernels.
//
// No counterpart in the reference (a new capability of this solver).
//
// Grid: the multigrid's level-1 node grid (every second fine node), tensors
// channels-last FP32, node index ((z*nnx)+x)*nny+y like every other array.
// Network (3 levels, 16/32/64 channels, 3x3x3 stride-1 convolutions):
//   x0 (7 ch: filtered density, u_prev/s_u, r/s_r)
//   e1 = relu(conv 7->16)         level A (full)
//   e2 = relu(conv 16->32 (pool e1))      level B (half)
//   e3 = relu(conv 32->64 (pool e2))      level C (quarter)
//   d2 = relu(conv 64->32 (up e3) + e2)   level B
//   d1 = relu(conv 32->16 (up d2) + e1)   level A
//   y  = conv 16->3 (d1)                  level A, linear
// y * s_u is a level-1 displacement correction; the warm start is
// u_prev + P (y * s_u) with the multigrid prolongation P.
#include <algorithm>
#include <type_traits>
#include <cmath>
#include <random>
#include <vector>
#include "tg_ctx.cuh"
#include "tg_cnn.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// grid helpers
// ---------------------------------------------------------------------------
static NG half_grid(const NG& g) { return NG{(g.nx + 1) / 2, (g.ny + 1) / 2, (g.nz + 1) / 2}; }

__device__ __forceinline__ void ng_xyz(const NG& g, int64_t i, int& x, int& y, int& z) {
  y = (int)(i % g.ny);
  x = (int)((i / g.ny) % g.nx);
  z = (int)(i / ((int64_t)g.ny * g.nx));
}
__device__ __forceinline__ int64_t ng_idx(const NG& g, int x, int y, int z) {
  return ((int64_t)z * g.nx + x) * g.ny + y;
}

// ---------------------------------------------------------------------------
// 3x3x3 convolution, stride 1, zero padding (forward; also the input gradient
// with flipped / transposed weights).  Epilogue: + bias, + skip, relu,
// * (mask > 0).
// ---------------------------------------------------------------------------
// The convolution runs on the tensor cores as an implicit GEMM
// out[n][co] = sum_{k, ci} in[nbr(n, k)][ci] W[k][ci][co] with warp-level
// mma.sync m16n8k8 TF32 and FP32 accumulation.
// SPLIT: each FP32 operand is split as hi = tf32(v), lo = tf32(v - hi) and
// the product taken as hi*hi + hi*lo + lo*hi (three MMAs), which keeps
// FP32-level accuracy (training, and every check against the FP32 oracle);
// without SPLIT one TF32 MMA (the warm-start inference: its output is a
// correction whose use the fallback rule guards, so TF32 rounding of the
// operands is immaterial).  A CTA of 4 warps
// computes 128 consecutive nodes (a warp: two 16-row tiles) times 8*NT output
// channels (blockIdx.y selects the chunk); A fragments are gathered from the
// channels-last input (zero outside the grid), B fragments read through the
// read-only cache; input channels past CIN (CIN not a multiple of 8) read as
// zero.  Fragment layouts of m16n8k8 (PTX ISA): with g = lane / 4,
// t = lane % 4, A holds (g, t), (g + 8, t), (g, t + 4), (g + 8, t + 4); B
// holds (t, g), (t + 4, g); C holds (g, 2t), (g, 2t + 1), (g + 8, 2t),
// (g + 8, 2t + 1).
__device__ __forceinline__ uint32_t f2tf32(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// CTA tile: a block of 8 (y) x 4 (x) x 4 (z) output nodes; its input block
// with a one-node halo (10 x 6 x 6 node rows, zero outside the grid) is
// staged in shared memory once, and all 27 taps read their A fragments from
// it (no barrier inside the tap loop).  Warp w computes z-layer w: two
// 16-row tiles of 8 y x 2 x nodes.
template <int CIN, int NT>
struct ConvTile {
  static constexpr int TY = 8, TX = 4, TZ = 4;
  static constexpr int HY = TY + 2, HX = TX + 2, HZ = TZ + 2;
  static constexpr int CP = (CIN + 7) / 8 * 8;   // input channels padded to the MMA k
  static constexpr int AS = CP + 4;              // row stride (words): conflict-free fragments
  static constexpr size_t smem() { return sizeof(float) * HZ * HX * HY * AS; }
};

template <int CIN, int NT, bool SPLIT>
__global__ void __launch_bounds__(128) k_conv3_mma(NG g, const float* __restrict__ in,
                                                   const float* __restrict__ W, int cout,
                                                   const float* __restrict__ bias,
                                                   const float* __restrict__ skip, int relu,
                                                   const float* __restrict__ mask,
                                                   float* __restrict__ out) {
  using TT = ConvTile<CIN, NT>;
  constexpr int CP = TT::CP, AS = TT::AS, HY = TT::HY, HX = TT::HX, HZ = TT::HZ;
  extern __shared__ __align__(16) float hs[];       // [HZ][HX][HY][AS]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gq = lane >> 2, tq = lane & 3;
  const int y0 = blockIdx.x * TT::TY, x0 = blockIdx.y * TT::TX;
  const int zb = gridDim.z / ((cout + 8 * NT - 1) / (8 * NT));   // z blocks per channel chunk
  const int z0 = (blockIdx.z % zb) * TT::TZ;
  const int co0 = (blockIdx.z / zb) * 8 * NT;
  // stage the halo block (zero outside the grid): 16-byte pieces of a node's
  // channels when CIN is a multiple of 8 (a node's channels are contiguous, AS
  // is a multiple of 4 and there are no padding columns), single values
  // (padding columns zero) otherwise
  constexpr int VW = (CIN % 8 == 0) ? 4 : 1;     // CIN % 8 == 0: no padding columns
  constexpr int NV = (CIN % 8 == 0) ? CIN / 4 : CP;
  for (int i = tid; i < HZ * HX * HY * NV; i += 128) {
    const int v = i % NV, hy = (i / NV) % HY, hx = (i / (NV * HY)) % HX, hz = i / (NV * HY * HX);
    const int X = x0 - 1 + hx, Y = y0 - 1 + hy, Z = z0 - 1 + hz;
    const bool in_grid = X >= 0 && X < g.nx && Y >= 0 && Y < g.ny && Z >= 0 && Z < g.nz;
    float* dst = hs + ((hz * HX + hx) * HY + hy) * AS + v * VW;
    if constexpr (VW == 4) {
      float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
      if (in_grid) val = __ldg(reinterpret_cast<const float4*>(in + ng_idx(g, X, Y, Z) * CIN) + v);
      *reinterpret_cast<float4*>(dst) = val;
    } else {
      *dst = (in_grid && v < CIN) ? __ldg(in + ng_idx(g, X, Y, Z) * CIN + v) : 0.f;
    }
  }

  __syncthreads();
  float acc[2][NT][4];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[m][j][q] = 0.f;
  // this thread's B values of a tap (rows c0 + t and c0 + t + 4, column 8 j + g),
  // loaded one tap ahead so that the read-only-cache latency overlaps the
  // current tap's MMAs
  constexpr int NCH = CP / 8;
  float wn[NCH][NT][2];
  auto load_w = [&](int k, float (&w)[NCH][NT][2]) {
    const float* wk = W + (int64_t)k * CIN * cout;
#pragma unroll
    for (int ch = 0; ch < NCH; ++ch)
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int co = co0 + j * 8 + gq, c = ch * 8 + tq;
        w[ch][j][0] = co < cout && c < CIN ? __ldg(wk + (int64_t)c * cout + co) : 0.f;
        w[ch][j][1] = co < cout && c + 4 < CIN ? __ldg(wk + (int64_t)(c + 4) * cout + co) : 0.f;
      }
  };
  load_w(0, wn);
#pragma unroll 1
  for (int k = 0; k < 27; ++k) {
    const int dy = k % 3 - 1, dx = (k / 3) % 3 - 1, dz = k / 9 - 1;
    // halo row of node (ly, lx, lz) shifted by the tap: lz = warp, lx = 2m (+1 for rows 8..15)
    const float* base = hs + (((warp + 1 + dz) * HX + (1 + dx)) * HY + (1 + dy + gq)) * AS + tq;
    float wc[NCH][NT][2];
#pragma unroll
    for (int ch = 0; ch < NCH; ++ch)
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        wc[ch][j][0] = wn[ch][j][0];
        wc[ch][j][1] = wn[ch][j][1];
      }
    if (k + 1 < 27) load_w(k + 1, wn);
#pragma unroll
    for (int c0 = 0; c0 < CP; c0 += 8) {
      uint32_t ahi[2][4], alo[2][4];
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const float* r0 = base + (2 * m) * HY * AS + c0;       // x = 2m,     y = gq
        const float* r1 = base + (2 * m + 1) * HY * AS + c0;   // x = 2m + 1, y = gq
        const float v[4] = {r0[0], r1[0], r0[4], r1[4]};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          ahi[m][q] = f2tf32(v[q]);
          if (SPLIT) alo[m][q] = f2tf32(v[q] - __uint_as_float(ahi[m][q]));
        }
      }
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const float w0 = wc[c0 / 8][j][0], w1 = wc[c0 / 8][j][1];
        uint32_t bhi[2], blo[2];
        bhi[0] = f2tf32(w0);
        bhi[1] = f2tf32(w1);
        if (SPLIT) {
          blo[0] = f2tf32(w0 - __uint_as_float(bhi[0]));
          blo[1] = f2tf32(w1 - __uint_as_float(bhi[1]));
        }
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          if (SPLIT) {
            mma_tf32(acc[m][j], alo[m], bhi);
            mma_tf32(acc[m][j], ahi[m], blo);
          }
          mma_tf32(acc[m][j], ahi[m], bhi);
        }
      }
    }
  }
  // epilogue: c0 (g, 2t), c1 (g, 2t + 1), c2 (g + 8, 2t), c3 (g + 8, 2t + 1); tile row
  // r < 8 is node (y = r, x = 2m), r >= 8 node (y = r - 8, x = 2m + 1)
  const int Z = z0 + warp;
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int X = x0 + 2 * m + (q >> 1), Y = y0 + gq;
      if (X >= g.nx || Y >= g.ny || Z >= g.nz) continue;
      const int64_t node = ng_idx(g, X, Y, Z);
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int co = co0 + j * 8 + 2 * tq + (q & 1);
        if (co >= cout) continue;
        float v = acc[m][j][q] + (bias ? bias[co] : 0.f);
        if (skip) v += skip[node * cout + co];
        if (relu) v = fmaxf(v, 0.f);
        if (mask && !(mask[node * cout + co] > 0.f)) v = 0.f;
        out[node * cout + co] = v;
      }
    }
}

template <int CIN, bool SPLIT>
static void conv3_launch(const NG& g, const float* in, const float* W, int cout, const float* bias,
                         const float* skip, int relu, const float* mask, float* out,
                         cudaStream_t st) {
  auto go = [&](auto nt_tag, unsigned chunks) {
    constexpr int NT = decltype(nt_tag)::value;
    using TT = ConvTile<CIN, NT>;
    constexpr size_t smem = TT::smem();
    const dim3 grid((unsigned)cdiv(g.ny, TT::TY), (unsigned)cdiv(g.nx, TT::TX),
                    (unsigned)cdiv(g.nz, TT::TZ) * chunks);
    set_smem_limit((const void*)k_conv3_mma<CIN, NT, SPLIT>, (int)smem);
    k_conv3_mma<CIN, NT, SPLIT><<<grid, 128, smem, st>>>(g, in, W, cout, bias, skip, relu, mask,
                                                         out);
  };
  // coarse network levels have few nodes: 8 output channels per CTA there, so
  // that enough warps run (each CTA stages its small halo block again)
  if (cout <= 8 || g.n() < 65536) go(std::integral_constant<int, 1>{}, (unsigned)cdiv(cout, 8));
  else if (cout <= 16) go(std::integral_constant<int, 2>{}, 1);
  else go(std::integral_constant<int, 4>{}, (unsigned)cdiv(cout, 32));
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// The same convolution on the 5th-generation tensor cores (tcgen05), for the
// warm start's TF32 inference.
// ---------------------------------------------------------------------------
// A CTA of 4 warps computes 128 output nodes -- 8 (y) x 16 (x) of one z plane
// -- times NN output channels (blockIdx.z / nz selects the chunk) as one
// M = 128, N = NN FP32 accumulator in tensor memory (TMEM): tile row r is
// TMEM lane r, node (y0 + r % 8, x0 + r / 8); column n is output channel
// co0 + n.  Both operands sit in shared memory in the MMA's K-major layout
// without swizzle: core matrices of 8 rows x 16 bytes (4 TF32 values), the 8
// rows 16 bytes apart, neighbouring core matrices along K `lbo` bytes apart
// and along M (or N) `sbo` bytes apart.
//  * A (input): the tile's input block with a one-node halo, 3 (z) x 18 (x)
//    x 10 (y) nodes, as planes [chunk of 8 channels][half of 4] of [z][x][y]
//    16-byte entries (zero outside the grid and past CIN), staged once by all
//    threads.  For a tap (dz, dx, dy) the 128 rows are 16 runs of 8
//    consecutive y entries, one run per x, so the tap's A matrix is a view of
//    the block: start at the shifted entry, sbo = one x column (10 entries),
//    lbo = one plane.
//  * B (one tap's weights): the image [chunk][half][n] of 16-byte entries (4
//    input channels of output channel co0 + n; sbo = 8 entries, lbo = NN
//    entries), packed in global memory once per forward pass (k_pack_umma)
//    and streamed by bulk copies (cp.async.bulk) into a ring of WSTAGES
//    stages: a stage's "full" barrier completes when its copy has landed, its
//    "empty" barrier when the MMAs that read it have completed.
// One thread drives the ring and the tensor core: per tap it waits for the
// stage to be full, issues the NCH MMAs (K = 8 each), commits them to the
// stage's empty barrier, and refills the previous tap's stage once those
// MMAs are done.  A last commit completes the "done" barrier, on which the
// other threads wait before they read their 32 TMEM lanes (tcgen05.ld) and
// apply bias, skip and relu.  Operands are rounded to TF32 as the mma.sync
// kernel rounds them (cvt.rna) and accumulated in FP32 in the same order
// (tap, chunk of 8 channels), so the two kernels give the same results.
// Every wait is bounded (about a second of %globaltimer): a wait that runs
// out makes the CTA issue nothing more, wait once more (bounded) for its
// copies and MMAs in flight, free its TMEM and leave without storing; the
// convolution error flag tells the host (TG_ETIMEOUT).
__device__ int g_conv_err = 0;

namespace um {
constexpr int TY = 8, TX = 16, HY = TY + 2, HX = TX + 2, HZ = 3;
constexpr int HN = HZ * HX * HY;                 // 540 halo entries per plane
// bytes per [chunk][half] plane: one entry of padding puts the 8 planes that
// a quarter warp stores to in distinct 16-byte bank groups
constexpr int PLANE = (HN + 1) * 16;
constexpr int WSTAGES = 4;
constexpr uint64_t WAIT_NS = 1000000000ull;
// mbarriers: full[WSTAGES], empty[WSTAGES], done, stall (never completes)
constexpr int B_FULL = 0, B_EMPTY = WSTAGES, B_DONE = 2 * WSTAGES, B_STALL = 2 * WSTAGES + 1;
constexpr int NBARS = 2 * WSTAGES + 2;
}  // namespace um

// output channels per CTA for a layer of cout channels (the MMA's N)
inline int umma_nn(int cout) { return cout <= 16 ? 16 : cout <= 32 ? 32 : 64; }

template <int CIN, int NN>
struct UmmaConv {
  static constexpr int CP = (CIN + 7) / 8 * 8;
  static constexpr int NCH = CP / 8;
  static constexpr int A_BYTES = NCH * 2 * um::PLANE;
  static constexpr int W_BYTES = NCH * 2 * NN * 16;        // one tap's weight image
  static constexpr int TCOLS = NN < 32 ? 32 : NN;          // TMEM columns: a power of 2, >= 32
  // 128 bytes of alignment slack, 128 of mbarriers, TMEM address and flag
  static constexpr size_t smem() {
    return 256 + (size_t)A_BYTES + (size_t)um::WSTAGES * W_BYTES;
  }
};

// shared-memory matrix descriptor: start address, leading (K) and stride
// (M / N) byte offsets, each in 16-byte units; bits 46-48 hold the fixed
// value 0b001; base offset 0, no swizzle
__device__ __forceinline__ uint64_t umma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9 and 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
      :: "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               ::"r"(smem_u32(bar)) : "memory");
}
// bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to shared memory, completing on `bar` with its byte count
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
// 16 consecutive 32-bit TMEM columns of this thread's lane; the wait carries
// the registers, so nothing reads them before the load has completed
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr) : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]),
                 "+r"(v[6]), "+r"(v[7]), "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]),
                 "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15])
               :: "memory");
}
__device__ __forceinline__ float tf32r(float v) { return __uint_as_float(f2tf32(v)); }

// weight images of the tensor-core kernel: out[((chunk * 27 + k) * NCH2 + p)
// * NN + n][j] = tf32(W[k][4 p + j][chunk * NN + n]), zero past cin / cout
struct PackJob {
  const float* W;
  float* out;
  int cin, cout, nn, nch2, chunks;
};
struct PackJobs {
  PackJob j[6];
};
__global__ void k_pack_umma(PackJobs jobs) {
  const PackJob& jb = jobs.j[blockIdx.y];
  const int64_t per_tap = (int64_t)jb.nch2 * jb.nn * 4;
  const int64_t total = (int64_t)jb.chunks * 27 * per_tap;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(i & 3), n = (int)((i >> 2) % jb.nn);
    const int p = (int)((i / (4 * jb.nn)) % jb.nch2);
    const int k = (int)((i / per_tap) % 27), ch = (int)(i / (per_tap * 27));
    const int ci = 4 * p + j, co = ch * jb.nn + n;
    jb.out[i] = (ci < jb.cin && co < jb.cout) ? tf32r(jb.W[((int64_t)k * jb.cin + ci) * jb.cout + co])
                                               : 0.f;
  }
}

template <int CIN, int NN>
__global__ void __launch_bounds__(128) k_conv3_umma(NG g, const float* __restrict__ in,
                                                    const float* __restrict__ Wp, int cout,
                                                    const float* __restrict__ bias,
                                                    const float* __restrict__ skip, int relu,
                                                    float* __restrict__ out, int stall) {
  using U = UmmaConv<CIN, NN>;
  constexpr int NCH = U::NCH, NS = um::WSTAGES;
  extern __shared__ __align__(128) unsigned char um_smem[];
  unsigned char* base = um_smem + ((128u - (smem_u32(um_smem) & 127u)) & 127u);
  uint64_t* bar = reinterpret_cast<uint64_t*>(base);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(base + 8 * um::NBARS);
  int* s_fail = reinterpret_cast<int*>(base + 8 * um::NBARS + 4);
  unsigned char* As = base + 128;
  unsigned char* Ws = As + U::A_BYTES;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int z = (int)(blockIdx.z % (unsigned)g.nz), chunk = (int)(blockIdx.z / (unsigned)g.nz);
  const int co0 = chunk * NN;
  const int y0 = blockIdx.x * um::TY, x0 = blockIdx.y * um::TX;
  const float* wimg = Wp + (int64_t)chunk * 27 * (U::W_BYTES / 4);
  auto tap_image = [&](int k) { return wimg + (int64_t)k * (U::W_BYTES / 4); };

  if (tid == 0) {
    *s_fail = 0;
#pragma unroll
    for (int k = 0; k < um::NBARS; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[k])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // the first WSTAGES taps' weights start moving while the block is staged
#pragma unroll
    for (int k = 0; k < NS; ++k)
      bulk_g2s(Ws + k * U::W_BYTES, tap_image(k), U::W_BYTES, &bar[um::B_FULL + k]);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(tslot)), "r"((uint32_t)U::TCOLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  // input block, (chunk, half) fastest so that a warp reads whole node rows;
  // four entries in flight per thread
  constexpr int NE = NCH * 2 * um::HN;
  auto load_entry = [&](int i) {
    const int p = i % (NCH * 2), e = i / (NCH * 2);
    const int hy = e % um::HY, hx = (e / um::HY) % um::HX, hz = e / (um::HY * um::HX);
    const int X = x0 - 1 + hx, Y = y0 - 1 + hy, Z = z - 1 + hz;
    const int c0 = p * 4;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (X >= 0 && X < g.nx && Y >= 0 && Y < g.ny && Z >= 0 && Z < g.nz && c0 < CIN) {
      const float* src = in + ng_idx(g, X, Y, Z) * CIN + c0;
      if constexpr (CIN % 4 == 0) {
        v = __ldg(reinterpret_cast<const float4*>(src));
      } else {
        v.x = __ldg(src);
        v.y = c0 + 1 < CIN ? __ldg(src + 1) : 0.f;
        v.z = c0 + 2 < CIN ? __ldg(src + 2) : 0.f;
        v.w = c0 + 3 < CIN ? __ldg(src + 3) : 0.f;
      }
    }
    return v;
  };
  for (int i0 = tid; i0 < NE; i0 += 4 * 128) {
    float4 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      v[u] = (i0 + u * 128 < NE) ? load_entry(i0 + u * 128) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * 128;
      if (i < NE)
        *reinterpret_cast<float4*>(As + (i % (NCH * 2)) * um::PLANE + (i / (NCH * 2)) * 16) =
            make_float4(tf32r(v[u].x), tf32r(v[u].y), tf32r(v[u].z), tf32r(v[u].w));
    }
  }
  // generic-proxy stores -> visible to the tensor core's (async-proxy) reads;
  // the TMEM address written by the allocation
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  bool failed = false;
  if (tid == 0) {
    constexpr uint32_t IDESC = umma_idesc_tf32(128, NN);
    const uint32_t a0 = smem_u32(As), w0 = smem_u32(Ws);
    int issued = NS - 1;          // the last tap whose weight copy was issued
    int consumed = -1;            // the last tap whose copy was waited for
    int committed = -1;           // the last tap whose MMAs were committed
    if (stall) failed = !mbar_wait_bounded(&bar[um::B_STALL], 0, um::WAIT_NS);
#pragma unroll 1
    for (int k = 0; k < 27 && !failed; ++k) {
      const int s = k % NS;
      if (!mbar_wait_bounded(&bar[um::B_FULL + s], (k / NS) & 1, um::WAIT_NS)) {
        failed = true;
        break;
      }
      consumed = k;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int dy = k % 3 - 1, dx = (k / 3) % 3 - 1, dz = k / 9 - 1;
      const uint32_t aoff = (uint32_t)((((1 + dz) * um::HX + (1 + dx)) * um::HY + (1 + dy)) * 16);
#pragma unroll
      for (int c = 0; c < NCH; ++c) {
        const uint64_t ad = umma_sdesc(a0 + 2 * c * um::PLANE + aoff, um::PLANE, um::HY * 16);
        const uint64_t bd = umma_sdesc(w0 + s * U::W_BYTES + 2 * c * NN * 16, NN * 16, 128);
        umma_tf32(tmem, ad, bd, IDESC, (k | c) != 0 ? 1u : 0u);
      }
      umma_commit(&bar[um::B_EMPTY + s]);
      committed = k;
      // refill the previous tap's stage once its MMAs are done (this tap's
      // MMAs keep the tensor core busy meanwhile)
      const int kp = k - 1, kn = kp + NS;
      if (kp >= 0 && kn < 27) {
        const int sp = kp % NS;
        if (!mbar_wait_bounded(&bar[um::B_EMPTY + sp], (kp / NS) & 1, um::WAIT_NS)) {
          failed = true;
          break;
        }
        bulk_g2s(Ws + sp * U::W_BYTES, tap_image(kn), U::W_BYTES, &bar[um::B_FULL + sp]);
        issued = kn;
      }
    }
    if (!failed) {
      umma_commit(&bar[um::B_DONE]);     // completes when every MMA above has
    } else {
      // nothing more is issued; wait (bounded) for what is in flight, then
      // release the other threads
      for (int j = consumed + 1; j <= issued; ++j)
        (void)mbar_wait_bounded(&bar[um::B_FULL + j % NS], (j / NS) & 1, um::WAIT_NS);
      if (committed >= 0)
        (void)mbar_wait_bounded(&bar[um::B_EMPTY + committed % NS], (committed / NS) & 1,
                                um::WAIT_NS);
      *s_fail = 1;
      asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n"
                   ::"r"(smem_u32(&bar[um::B_DONE])) : "memory");
    }
  }
  // thread 0 arrives within a few of its own bounded waits, even on failure
  if (!mbar_wait_bounded(&bar[um::B_DONE], 0, 8 * um::WAIT_NS)) failed = true;
  failed = __syncthreads_or(failed || *s_fail != 0) != 0;
  if (!failed) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int r = warp * 32 + lane;
    const int Y = y0 + (r & 7), X = x0 + (r >> 3);
    const bool valid = X < g.nx && Y < g.ny;
    const int64_t node = valid ? ng_idx(g, X, Y, z) : 0;
#pragma unroll
    for (int cb = 0; cb < NN; cb += 16) {
      uint32_t v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
      if (!valid) continue;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int co = co0 + cb + j;
        if (co >= cout) continue;
        float val = __uint_as_float(v[j]) + (bias ? bias[co] : 0.f);
        if (skip) val += skip[node * cout + co];
        if (relu) val = fmaxf(val, 0.f);
        out[node * cout + co] = val;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"((uint32_t)U::TCOLS) : "memory");
  }
  if (failed && tid == 0) atomicExch(&g_conv_err, 1);
}

int take_conv_error(cudaStream_t st) {
  int v = 0;
  TG_CUDA(cudaMemcpyFromSymbolAsync(&v, g_conv_err, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
  TG_CUDA(cudaStreamSynchronize(st));
  if (v) {
    static const int zero = 0;
    TG_CUDA(cudaMemcpyToSymbolAsync(g_conv_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st));
    TG_CUDA(cudaStreamSynchronize(st));
  }
  return v;
}

template <int CIN, int NN>
static void conv3_umma_launch(const NG& g, const float* in, const float* Wp, int cout,
                              const float* bias, const float* skip, int relu, float* out,
                              cudaStream_t st) {
  using U = UmmaConv<CIN, NN>;
  const dim3 grid((unsigned)cdiv(g.ny, um::TY), (unsigned)cdiv(g.nx, um::TX),
                  (unsigned)(g.nz * cdiv(cout, NN)));
  set_smem_limit((const void*)k_conv3_umma<CIN, NN>, (int)U::smem());
  const int stall = tune_take_conv_timeout() ? 1 : 0;
  k_conv3_umma<CIN, NN><<<grid, 128, U::smem(), st>>>(g, in, Wp, cout, bias, skip, relu, out, stall);
  TG_CHECK_LAUNCH();
}

// Wp: the layer's weight images (k_pack_umma); false: no tensor-core variant
// for this shape (the caller uses mma.sync)
static bool conv3_umma(const NG& g, int cin, const float* in, const float* Wp, int cout,
                       const float* bias, const float* skip, int relu, float* out,
                       cudaStream_t st) {
  if (cout > 64) return false;
  auto go = [&](auto cin_tag) {
    constexpr int CI = decltype(cin_tag)::value;
    switch (umma_nn(cout)) {
      case 16: conv3_umma_launch<CI, 16>(g, in, Wp, cout, bias, skip, relu, out, st); break;
      case 32: conv3_umma_launch<CI, 32>(g, in, Wp, cout, bias, skip, relu, out, st); break;
      default: conv3_umma_launch<CI, 64>(g, in, Wp, cout, bias, skip, relu, out, st); break;
    }
  };
  switch (cin) {
    case 7: go(std::integral_constant<int, 7>{}); return true;
    case 16: go(std::integral_constant<int, 16>{}); return true;
    case 32: go(std::integral_constant<int, 32>{}); return true;
    case 64: go(std::integral_constant<int, 64>{}); return true;
    default: return false;
  }
}

// floats of one layer's weight images
static int64_t umma_pack_size(int cin, int cout) {
  const int nn = umma_nn(cout);
  return (int64_t)cdiv(cout, nn) * 27 * ((cin + 7) / 8 * 2) * nn * 4;
}

// Wp: the layer's tensor-core weight images (TF32 inference only), or null
static void conv3(const NG& g, int cin, const float* in, const float* W, int cout,
                  const float* bias, const float* skip, int relu, const float* mask, float* out,
                  cudaStream_t st, bool split = true, const float* Wp = nullptr) {
  if (Wp && !split && !mask && conv3_umma(g, cin, in, Wp, cout, bias, skip, relu, out, st))
    return;
#define TG_C3(CI)                                                                                \
  if (split) conv3_launch<CI, true>(g, in, W, cout, bias, skip, relu, mask, out, st);            \
  else conv3_launch<CI, false>(g, in, W, cout, bias, skip, relu, mask, out, st);
  switch (cin) {
    case 3: TG_C3(3) break;
    case 7: TG_C3(7) break;
    case 16: TG_C3(16) break;
    case 32: TG_C3(32) break;
    case 64: TG_C3(64) break;
    default: throw Error{EINVAL_, "conv3: unsupported input channel count"};
  }
#undef TG_C3
}

// W'[k'][co][ci] = W[26-k'][ci][co]: the input gradient is a convolution of the
// output gradient with these weights
__global__ void k_flip_transpose(const float* W, int cin, int cout, float* Wt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)27 * cin * cout) return;
  const int ci = (int)(i % cin), co = (int)((i / cin) % cout), k = (int)(i / ((int64_t)cin * cout));
  Wt[i] = W[((int64_t)(26 - k) * cin + ci) * cout + co];
}

// ---------------------------------------------------------------------------
// weight gradient: dW[k][ci][co] = sum_n in[n+off_k][ci] g[n][co]; one CTA per
// (k, chunk of nodes) writes a partial, a second kernel sums the partials in
// fixed order (deterministic, no atomics)
// ---------------------------------------------------------------------------
constexpr int DW_CHUNK = 2048;
constexpr int DW_BATCH = 32;

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv3_dw(NG g, const float* __restrict__ in,
                                                  const float* __restrict__ gout,
                                                  float* __restrict__ part) {
  constexpr int NP = CIN * COUT;
  constexpr int PER = (NP + 255) / 256;
  __shared__ float sin[DW_BATCH][CIN];
  __shared__ float sgo[DW_BATCH][COUT];
  const int k = blockIdx.y;
  const int dy = k % 3 - 1, dx = (k / 3) % 3 - 1, dz = k / 9 - 1;
  const int64_t n0 = (int64_t)blockIdx.x * DW_CHUNK;
  const int64_t n1 = (n0 + DW_CHUNK < g.n()) ? n0 + DW_CHUNK : g.n();
  float acc[PER];
#pragma unroll
  for (int p = 0; p < PER; ++p) acc[p] = 0.f;
  for (int64_t b0 = n0; b0 < n1; b0 += DW_BATCH) {
    for (int i = threadIdx.x; i < DW_BATCH * CIN; i += blockDim.x) {
      const int v = i / CIN, ci = i % CIN;
      const int64_t n = b0 + v;
      float val = 0.f;
      if (n < n1) {
        int x, y, z;
        ng_xyz(g, n, x, y, z);
        const int X = x + dx, Y = y + dy, Z = z + dz;
        if (X >= 0 && X < g.nx && Y >= 0 && Y < g.ny && Z >= 0 && Z < g.nz)
          val = in[ng_idx(g, X, Y, Z) * CIN + ci];
      }
      sin[v][ci] = val;
    }
    for (int i = threadIdx.x; i < DW_BATCH * COUT; i += blockDim.x) {
      const int v = i / COUT, co = i % COUT;
      const int64_t n = b0 + v;
      sgo[v][co] = (n < n1) ? gout[n * COUT + co] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int pi = threadIdx.x + p * 256;
      if (pi < NP) {
        const int ci = pi / COUT, co = pi % COUT;
        float a = acc[p];
#pragma unroll 8
        for (int v = 0; v < DW_BATCH; ++v) a = fmaf(sin[v][ci], sgo[v][co], a);
        acc[p] = a;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int pi = threadIdx.x + p * 256;
    if (pi < NP) part[((int64_t)blockIdx.x * 27 + k) * NP + pi] = acc[p];
  }
}

__global__ void k_sum_parts(const float* part, int nchunks, int64_t m, float* out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int c = 0; c < nchunks; ++c) s += part[(int64_t)c * m + i];
  out[i] = (float)s;
}

// bias gradient db[co] = sum_n g[n][co] (one block per channel, fixed order)
__global__ void k_bias_grad(const float* gout, int64_t n, int cout, float* db) {
  __shared__ double sh[32];
  const int co = blockIdx.x;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += gout[i * cout + co];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) db[co] = (float)s;
}

template <int CIN, int COUT>
static void dw_launch(const NG& g, const float* in, const float* gout, float* part, float* dW,
                      cudaStream_t st) {
  const int nch = (int)cdiv(g.n(), DW_CHUNK);
  k_conv3_dw<CIN, COUT><<<dim3(nch, 27), 256, 0, st>>>(g, in, gout, part);
  TG_CHECK_LAUNCH();
  const int64_t m = (int64_t)27 * CIN * COUT;
  k_sum_parts<<<(unsigned)cdiv(m, 256), 256, 0, st>>>(part, nch, m, dW);
  TG_CHECK_LAUNCH();
}

static void conv3_dw(const NG& g, int cin, int cout, const float* in, const float* gout,
                     float* part, float* dW, float* db, cudaStream_t st) {
  const int key = cin * 1000 + cout;
  switch (key) {
    case 7016: dw_launch<7, 16>(g, in, gout, part, dW, st); break;
    case 16032: dw_launch<16, 32>(g, in, gout, part, dW, st); break;
    case 32064: dw_launch<32, 64>(g, in, gout, part, dW, st); break;
    case 64032: dw_launch<64, 32>(g, in, gout, part, dW, st); break;
    case 32016: dw_launch<32, 16>(g, in, gout, part, dW, st); break;
    case 16003: dw_launch<16, 3>(g, in, gout, part, dW, st); break;
    default: throw Error{EINVAL_, "conv3_dw: unsupported channel pair"};
  }
  k_bias_grad<<<cout, 256, 0, st>>>(gout, g.n(), cout, db);
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// pooling (average of the present children), nearest upsampling, and their
// adjoints; elementwise helpers
// ---------------------------------------------------------------------------
__global__ void k_pool(NG gf, NG gc, int C, const float* in, float* out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= gc.n() * C) return;
  const int c = (int)(t % C);
  const int64_t I = t / C;
  int X, Y, Z;
  ng_xyz(gc, I, X, Y, Z);
  float s = 0.f;
  int cnt = 0;
  for (int a = 0; a < 8; ++a) {
    const int x = 2 * X + (a & 1), y = 2 * Y + ((a >> 1) & 1), z = 2 * Z + (a >> 2);
    if (x < gf.nx && y < gf.ny && z < gf.nz) {
      s += in[ng_idx(gf, x, y, z) * C + c];
      ++cnt;
    }
  }
  out[t] = s / (float)cnt;
}
__global__ void k_pool_bwd(NG gf, NG gc, int C, const float* gout, float* gin, int accumulate) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= gf.n() * C) return;
  const int c = (int)(t % C);
  const int64_t i = t / C;
  int x, y, z;
  ng_xyz(gf, i, x, y, z);
  const int X = x / 2, Y = y / 2, Z = z / 2;
  int cnt = 0;
  for (int a = 0; a < 8; ++a) {
    const int xx = 2 * X + (a & 1), yy = 2 * Y + ((a >> 1) & 1), zz = 2 * Z + (a >> 2);
    if (xx < gf.nx && yy < gf.ny && zz < gf.nz) ++cnt;
  }
  const float v = gout[ng_idx(gc, X, Y, Z) * C + c] / (float)cnt;
  gin[t] = accumulate ? gin[t] + v : v;
}
__global__ void k_up(NG gf, NG gc, int C, const float* in, float* out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= gf.n() * C) return;
  const int c = (int)(t % C);
  int x, y, z;
  ng_xyz(gf, t / C, x, y, z);
  out[t] = in[ng_idx(gc, x / 2, y / 2, z / 2) * C + c];
}
__global__ void k_up_bwd(NG gf, NG gc, int C, const float* gout, float* gin) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= gc.n() * C) return;
  const int c = (int)(t % C);
  int X, Y, Z;
  ng_xyz(gc, t / C, X, Y, Z);
  float s = 0.f;
  for (int a = 0; a < 8; ++a) {
    const int x = 2 * X + (a & 1), y = 2 * Y + ((a >> 1) & 1), z = 2 * Z + (a >> 2);
    if (x < gf.nx && y < gf.ny && z < gf.nz) s += gout[ng_idx(gf, x, y, z) * C + c];
  }
  gin[t] = s;
}
__global__ void k_add_inplace(int64_t n, const float* a, float* b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] += a[i];
}
// gradient through relu: g *= (act > 0)
__global__ void k_relu_mask(int64_t n, const float* act, float* g) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && !(act[i] > 0.f)) g[i] = 0.f;
}
// MSE: L = mean((y - t)^2), dL/dy = 2 (y - t) / N; partial loss per block
__global__ void k_mse(int64_t n, const float* y, const float* t, float* g, double* part) {
  __shared__ double sh[32];
  double s = 0.0;
  const float scale = 2.f / (float)n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    g[i] = scale * d;
    s += (double)d * (double)d;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}
// Adam (Kingma & Ba), bias-corrected
__global__ void k_adam(int64_t n, float* w, const float* g, float* m, float* v, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

static unsigned nb(int64_t n) { return (unsigned)cdiv(n, 256); }

// ---------------------------------------------------------------------------
// features and targets from the solver state
// ---------------------------------------------------------------------------
// x0[I] = (density at fine node 2I, u(2I)/s_u, (P^T r)(I)/s_r) with the
// density averaged over the fine elements touching the node and P^T r the
// residual restricted to the level-1 grid (a smooth coarse picture of the
// rough fine residual), s_r its norm
__global__ void k_features(Grid gf, NG g1, const double* __restrict__ xPhys,
                           const double* __restrict__ u, const float* __restrict__ rc,
                           const PCGState* su, const PCGState* sr, float* __restrict__ x0) {
  const int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (I >= g1.n()) return;
  int X, Y, Z;
  ng_xyz(g1, I, X, Y, Z);
  const int fx = 2 * X, fy = 2 * Y, fz = (gf.ndim == 3) ? 2 * Z : 0;
  double dsum = 0.0;
  int cnt = 0;
  for (int a = 0; a < 8; ++a) {
    const int ex = fx - (a & 1), ey = fy - ((a >> 1) & 1), ez = fz - (a >> 2);
    if (ex < 0 || ex >= gf.nex || ey < 0 || ey >= gf.ney || ez < 0 || ez >= gf.nez) continue;
    dsum += xPhys[gf.elem(ex, ey, ez)];
    ++cnt;
  }
  const int64_t fn = gf.node(fx, fy, fz);
  const float iu = (float)su->rinv, ir = (float)sr->rinv;
  float* o = x0 + I * 7;
  o[0] = (float)(dsum / cnt);
  for (int c = 0; c < 3; ++c) {
    o[1 + c] = (float)u[fn * 3 + c] * iu;
    o[4 + c] = rc[I * 3 + c] * ir;
  }
}
// target t[I] = (u_new(2I) - u_prev(2I)) / s_u
__global__ void k_target(Grid gf, NG g1, const double* __restrict__ unew,
                         const double* __restrict__ uprev, const PCGState* su, float* __restrict__ t) {
  const int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (I >= g1.n()) return;
  int X, Y, Z;
  ng_xyz(g1, I, X, Y, Z);
  const int64_t fn = gf.node(2 * X, 2 * Y, (gf.ndim == 3) ? 2 * Z : 0);
  const float iu = (float)su->rinv;
  for (int c = 0; c < 3; ++c) t[I * 3 + c] = (float)(unew[fn * 3 + c] - uprev[fn * 3 + c]) * iu;
}
// level-1 correction in FP64: d[I] = y[I] * s_u
__global__ void k_correction(int64_t n, const float* y, const PCGState* su, double* d) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) d[i] = (double)y[i] * su->rnorm;
}

// ---------------------------------------------------------------------------
// the network object
// ---------------------------------------------------------------------------
Cnn::Cnn(Ctx& c, int capacity, uint64_t seed) : ctx(&c) {
  TG_REQUIRE(c.g.ndim == 3 && c.g.ndof == 3, "the learned warm start is built for 3-D elasticity");
  TG_REQUIRE(c.L >= 2, "the learned warm start needs a multigrid context (>= 2 levels)");
  const Grid& g1 = c.lv[1]->g;
  A = NG{g1.nnx, g1.nny, g1.nnz};
  B = half_grid(A);
  Cg = half_grid(B);
  const int spec[6][2] = {{7, 16}, {16, 32}, {32, 64}, {64, 32}, {32, 16}, {16, 3}};
  int64_t off = 0;
  for (auto& s : spec) {
    Layer l{s[0], s[1], off, 0};
    off += (int64_t)27 * s[0] * s[1];
    l.b_off = off;
    off += s[1];
    layers.push_back(l);
  }
  nparams = off;
  params.alloc(nparams); grads.alloc(nparams); adam_m.alloc(nparams); adam_v.alloc(nparams);
  wt.alloc((int64_t)27 * 64 * 64);
  int64_t poff = 0;
  for (size_t i = 0; i < layers.size(); ++i) {
    wpack_off[i] = poff;
    poff += umma_pack_size(layers[i].cin, layers[i].cout);
  }
  wpack.alloc(poff);
  adam_m.zero(c.st);
  adam_v.zero(c.st);
  // He-normal initialisation from a seeded generator
  std::vector<float> h(nparams, 0.f);
  std::mt19937_64 rng(seed);
  for (auto& l : layers) {
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (27.f * l.cin)));
    for (int64_t i = 0; i < (int64_t)27 * l.cin * l.cout; ++i) h[l.w_off + i] = nd(rng);
  }
  TG_CUDA(cudaMemcpy(params.p, h.data(), sizeof(float) * nparams, cudaMemcpyHostToDevice));
  const int64_t na = A.n(), nbn = B.n(), nc = Cg.n();
  x0.alloc(na * 7); e1.alloc(na * 16); p1.alloc(nbn * 16); e2.alloc(nbn * 32); p2.alloc(nc * 32);
  e3.alloc(nc * 64); u2.alloc(nbn * 64); d2.alloc(nbn * 32); u1.alloc(na * 32); d1.alloc(na * 16);
  y.alloc(na * 3); tgt.alloc(na * 3);
  g_a16.alloc(na * 16); g_a32.alloc(na * 32); g_b64.alloc(nbn * 64); g_b32.alloc(nbn * 32);
  g_b16.alloc(nbn * 16); g_c64.alloc(nc * 64); g_c32.alloc(nc * 32); g_e1.alloc(na * 16);
  g_e2.alloc(nbn * 32); g_y.alloc(na * 3);
  dw_part.alloc(cdiv(na, DW_CHUNK) * 27 * 64 * 64);
  loss_part.alloc(RED_BLOCKS);
  loss_out.alloc(1);
  capacity_ = capacity;
  data_x.alloc((int64_t)capacity * na * 7);
  data_t.alloc((int64_t)capacity * na * 3);
  uprev.alloc(c.g.ndofs());
  corr.alloc(g1.ndofs());
  r32a.alloc(c.g.ndofs());
  w32.alloc(c.g.ndofs());
  w32.zero(c.st);
  aw32.alloc(c.g.ndofs());
  aw32.zero(c.st);
  rc32.alloc(g1.ndofs());
  su.alloc(1); sr.alloc(1); src.alloc(1); su.zero(c.st); sr.zero(c.st); src.zero(c.st);
  gal.alloc(6); gal.zero(c.st);
  wsb.alloc(4); wsb.zero(c.st);
  rpart.alloc(RED_BLOCKS);
  TG_CUDA(cudaStreamSynchronize(c.st));
}

// the tensor-core weight images of every layer, from the current parameters
void Cnn::pack_umma(cudaStream_t st) {
  PackJobs jobs{};
  int64_t most = 0;
  for (size_t i = 0; i < layers.size(); ++i) {
    const Layer& l = layers[i];
    const int nn = umma_nn(l.cout);
    jobs.j[i] = PackJob{params.p + l.w_off, wpack.p + wpack_off[i], l.cin, l.cout, nn,
                        (l.cin + 7) / 8 * 2, (int)cdiv(l.cout, nn)};
    most = std::max(most, umma_pack_size(l.cin, l.cout));
  }
  k_pack_umma<<<dim3((unsigned)std::min<int64_t>(cdiv(most, 256), 128), (unsigned)layers.size()),
                256, 0, st>>>(jobs);
  TG_CHECK_LAUNCH();
}

void Cnn::forward(cudaStream_t st, bool split) {
  const float* P = params.p;
  auto W = [&](int i) { return P + layers[i].w_off; };
  auto b = [&](int i) { return P + layers[i].b_off; };
  // TF32 inference on the tensor cores (tcgen05) unless switched off
  const bool tc = !split && tune_conv_umma();
  if (tc) pack_umma(st);
  auto Wp = [&](int i) { return tc ? wpack.p + wpack_off[i] : nullptr; };
  conv3(A, 7, x0, W(0), 16, b(0), nullptr, 1, nullptr, e1, st, split, Wp(0));
  k_pool<<<nb(B.n() * 16), 256, 0, st>>>(A, B, 16, e1, p1);
  TG_CHECK_LAUNCH();
  conv3(B, 16, p1, W(1), 32, b(1), nullptr, 1, nullptr, e2, st, split, Wp(1));
  k_pool<<<nb(Cg.n() * 32), 256, 0, st>>>(B, Cg, 32, e2, p2);
  TG_CHECK_LAUNCH();
  conv3(Cg, 32, p2, W(2), 64, b(2), nullptr, 1, nullptr, e3, st, split, Wp(2));
  k_up<<<nb(B.n() * 64), 256, 0, st>>>(B, Cg, 64, e3, u2);
  TG_CHECK_LAUNCH();
  conv3(B, 64, u2, W(3), 32, b(3), e2, 1, nullptr, d2, st, split, Wp(3));
  k_up<<<nb(A.n() * 32), 256, 0, st>>>(A, B, 32, d2, u1);
  TG_CHECK_LAUNCH();
  conv3(A, 32, u1, W(4), 16, b(4), e1, 1, nullptr, d1, st, split, Wp(4));
  conv3(A, 16, d1, W(5), 3, b(5), nullptr, 0, nullptr, y, st, split, Wp(5));
}

// loss against tgt, gradients into grads (forward must have run)
double Cnn::backward(cudaStream_t st, bool want_loss) {
  const float* P = params.p;
  float* G = grads.p;
  auto gW = [&](int i) { return G + layers[i].w_off; };
  auto gb = [&](int i) { return G + layers[i].b_off; };
  auto flip = [&](int i) {
    const Layer& l = layers[i];
    k_flip_transpose<<<nb((int64_t)27 * l.cin * l.cout), 256, 0, st>>>(P + l.w_off, l.cin, l.cout, wt);
    TG_CHECK_LAUNCH();
  };
  const int64_t na = A.n(), nbn = B.n(), nc = Cg.n();
  const unsigned lb = red_blocks(na * 3);
  k_mse<<<lb, RED_THREADS, 0, st>>>(na * 3, y, tgt, g_y, loss_part);
  TG_CHECK_LAUNCH();
  // head: y = conv(d1)
  conv3_dw(A, 16, 3, d1, g_y, dw_part, gW(5), gb(5), st);
  flip(5);
  conv3(A, 3, g_y, wt, 16, nullptr, nullptr, 0, d1, g_a16, st);        // g(pre d1) = dx * (d1 > 0)
  // d1 = relu(conv(u1) + e1)
  conv3_dw(A, 32, 16, u1, g_a16, dw_part, gW(4), gb(4), st);
  TG_CUDA(cudaMemcpyAsync(g_e1.p, g_a16.p, sizeof(float) * na * 16, cudaMemcpyDeviceToDevice, st));
  flip(4);
  conv3(A, 16, g_a16, wt, 32, nullptr, nullptr, 0, nullptr, g_a32, st);  // g(u1)
  k_up_bwd<<<nb(nbn * 32), 256, 0, st>>>(A, B, 32, g_a32, g_b32);       // g(d2)
  TG_CHECK_LAUNCH();
  k_relu_mask<<<nb(nbn * 32), 256, 0, st>>>(nbn * 32, d2, g_b32);        // g(pre d2)
  TG_CHECK_LAUNCH();
  // d2 = relu(conv(u2) + e2)
  conv3_dw(B, 64, 32, u2, g_b32, dw_part, gW(3), gb(3), st);
  TG_CUDA(cudaMemcpyAsync(g_e2.p, g_b32.p, sizeof(float) * nbn * 32, cudaMemcpyDeviceToDevice, st));
  flip(3);
  conv3(B, 32, g_b32, wt, 64, nullptr, nullptr, 0, nullptr, g_b64, st);  // g(u2)
  k_up_bwd<<<nb(nc * 64), 256, 0, st>>>(B, Cg, 64, g_b64, g_c64);        // g(e3)
  TG_CHECK_LAUNCH();
  k_relu_mask<<<nb(nc * 64), 256, 0, st>>>(nc * 64, e3, g_c64);
  TG_CHECK_LAUNCH();
  // e3 = relu(conv(p2))
  conv3_dw(Cg, 32, 64, p2, g_c64, dw_part, gW(2), gb(2), st);
  flip(2);
  conv3(Cg, 64, g_c64, wt, 32, nullptr, nullptr, 0, nullptr, g_c32, st); // g(p2)
  k_pool_bwd<<<nb(nbn * 32), 256, 0, st>>>(B, Cg, 32, g_c32, g_e2, 1);  // g(e2) += pool^T g(p2)
  TG_CHECK_LAUNCH();
  k_relu_mask<<<nb(nbn * 32), 256, 0, st>>>(nbn * 32, e2, g_e2);
  TG_CHECK_LAUNCH();
  // e2 = relu(conv(p1))
  conv3_dw(B, 16, 32, p1, g_e2, dw_part, gW(1), gb(1), st);
  flip(1);
  conv3(B, 32, g_e2, wt, 16, nullptr, nullptr, 0, nullptr, g_b16, st);  // g(p1)
  k_pool_bwd<<<nb(na * 16), 256, 0, st>>>(A, B, 16, g_b16, g_e1, 1);    // g(e1) += pool^T g(p1)
  TG_CHECK_LAUNCH();
  k_relu_mask<<<nb(na * 16), 256, 0, st>>>(na * 16, e1, g_e1);
  TG_CHECK_LAUNCH();
  // e1 = relu(conv(x0))
  conv3_dw(A, 7, 16, x0, g_e1, dw_part, gW(0), gb(0), st);
  if (!want_loss) return 0.0;
  reduce_partials(loss_part, (int)lb, loss_out, false, st);
  double l = 0.0;
  TG_CUDA(cudaMemcpyAsync(&l, loss_out.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  TG_CUDA(cudaStreamSynchronize(st));
  return l / (double)(na * 3);
}

void Cnn::adam_step(cudaStream_t st) {
  ++adam_t;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
  k_adam<<<nb(nparams), 256, 0, st>>>(nparams, params, grads, adam_m, adam_v, lr, b1, b2, 1e-8f,
                                      c1, c2);
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// solver-state interface
// ---------------------------------------------------------------------------
// r32a = f - K(xPhys) u in FP32 (scale factors s32 must hold simp(xPhys))
// out = f - K u in FP32; leaves p32 = u and z32 = f (FP32 copies)
static void residual32(Ctx& c, const double* u, float* out) {
  const int64_t n = c.g.ndofs();
  d2f(n, u, c.p32, c.st);
  d2f(n, c.f, c.z32, c.st);
  fine_apply<float, float>(c.op, c.s32, c.p32, out, c.z32, nullptr, 0.0, AM_RES, c.st);
}

void Cnn::features(Ctx& c, const double* u_prev) {
  const int64_t n = c.g.ndofs();
  const Level& l1 = *c.lv[1];
  residual32(c, u_prev, r32a);
  pcg_reset(su, c.st);
  dot<double, double>(n, u_prev, u_prev, rpart, su, DOT_RR, c.st);
  pcg_reset(sr, c.st);
  dot<float, float>(n, r32a.p, r32a.p, rpart, sr, DOT_RR, c.st);   // the plain start's residual
  restrict_<float>(c.g, l1.g, l1.fix, r32a, rc32, c.st);
  pcg_reset(src, c.st);
  dot<float, float>(l1.g.ndofs(), rc32.p, rc32.p, rpart, src, DOT_RR, c.st);
  k_features<<<nb(A.n()), 256, 0, c.st>>>(c.g, A, c.xPhys, u_prev, rc32, su, src, x0);
  TG_CHECK_LAUNCH();
}

void Cnn::record_begin(Ctx& c) {
  TG_REQUIRE(nsamples < capacity_, "training set is full");
  TG_REQUIRE(c.precision == TG_PREC_MIXED, "recording needs a mixed-precision context");
  set_density(c, c.xPhys);
  TG_CUDA(cudaMemcpyAsync(uprev.p, c.u.p, sizeof(double) * c.g.ndofs(), cudaMemcpyDeviceToDevice, c.st));
  features(c, uprev);
  TG_CUDA(cudaMemcpyAsync(data_x.p + (int64_t)nsamples * A.n() * 7, x0.p, sizeof(float) * A.n() * 7,
                          cudaMemcpyDeviceToDevice, c.st));
}

void Cnn::record_end(Ctx& c) {
  k_target<<<nb(A.n()), 256, 0, c.st>>>(c.g, A, c.u, uprev, su,
                                        data_t.p + (int64_t)nsamples * A.n() * 3);
  TG_CHECK_LAUNCH();
  ++nsamples;
  TG_CUDA(cudaStreamSynchronize(c.st));
}

double Cnn::train(int epochs, float lr_, uint64_t seed) {
  TG_REQUIRE(nsamples > 0, "no training samples recorded");
  lr = lr_;
  cudaStream_t st = ctx->st;
  std::mt19937_64 rng(seed);
  std::vector<int> order(nsamples);
  double last = 0.0;
  for (int e = 0; e < epochs; ++e) {
    for (int i = 0; i < nsamples; ++i) order[i] = i;
    std::shuffle(order.begin(), order.end(), rng);
    double sum = 0.0;
    for (int i = 0; i < nsamples; ++i) {
      const int s = order[i];
      TG_CUDA(cudaMemcpyAsync(x0.p, data_x.p + (int64_t)s * A.n() * 7, sizeof(float) * A.n() * 7,
                              cudaMemcpyDeviceToDevice, st));
      TG_CUDA(cudaMemcpyAsync(tgt.p, data_t.p + (int64_t)s * A.n() * 3, sizeof(float) * A.n() * 3,
                              cudaMemcpyDeviceToDevice, st));
      forward(st);
      sum += backward(st, e == epochs - 1);
      adam_step(st);
    }
    if (e == epochs - 1) last = sum / nsamples;
  }
  TG_CUDA(cudaStreamSynchronize(st));
  trained = true;
  return last;
}

double Cnn::fit(int n, const float* x0s, const float* targets, int epochs, float lr_,
                uint64_t seed) {
  TG_REQUIRE(n > 0 && x0s && targets, "tg_cnn_fit: no pairs");
  lr = lr_;
  cudaStream_t st = ctx->st;
  std::mt19937_64 rng(seed);
  std::vector<int> order(n);
  const int64_t na = A.n();
  double last = 0.0;
  for (int e = 0; e < epochs; ++e) {
    for (int i = 0; i < n; ++i) order[i] = i;
    std::shuffle(order.begin(), order.end(), rng);
    double sum = 0.0;
    for (int i = 0; i < n; ++i) {
      const int s = order[i];
      TG_CUDA(cudaMemcpyAsync(x0.p, x0s + (int64_t)s * na * 7, sizeof(float) * na * 7,
                              cudaMemcpyHostToDevice, st));
      TG_CUDA(cudaMemcpyAsync(tgt.p, targets + (int64_t)s * na * 3, sizeof(float) * na * 3,
                              cudaMemcpyHostToDevice, st));
      forward(st);
      sum += backward(st, e == epochs - 1);
      adam_step(st);
    }
    if (e == epochs - 1) last = sum / n;
  }
  TG_CUDA(cudaStreamSynchronize(st));
  trained = true;
  return last;
}

// The five products of the 2x2 Galerkin combination in one pass over the
// vectors: v1.Kv1, v1.Kv2, v2.Kv2, v1.f, v2.f (FP32 products, each thread's
// sums widened to FP64 for the block and grid sums, finished in fixed order
// by the last block into out[k].bb)
constexpr int DOT5_BLOCKS = RED_BLOCKS / 5;
__global__ void __launch_bounds__(RED_THREADS) k_dot5(int64_t n, const float* __restrict__ v1,
                                                     const float* __restrict__ v2,
                                                     const float* __restrict__ k1,
                                                     const float* __restrict__ k2,
                                                     const float* __restrict__ f, double* part,
                                                     PCGState* out) {
  __shared__ double sh[32];
  __shared__ int last;
  float a[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t ts = (int64_t)gridDim.x * blockDim.x;
  const int64_t n4 = n / 4;
  for (int64_t i = t0; i < n4; i += ts) {
    const float4 x1 = reinterpret_cast<const float4*>(v1)[i];
    const float4 x2 = reinterpret_cast<const float4*>(v2)[i];
    const float4 y1 = reinterpret_cast<const float4*>(k1)[i];
    const float4 y2 = reinterpret_cast<const float4*>(k2)[i];
    const float4 ff = reinterpret_cast<const float4*>(f)[i];
    const float xs1[4] = {x1.x, x1.y, x1.z, x1.w}, xs2[4] = {x2.x, x2.y, x2.z, x2.w};
    const float ys1[4] = {y1.x, y1.y, y1.z, y1.w}, ys2[4] = {y2.x, y2.y, y2.z, y2.w};
    const float fs[4] = {ff.x, ff.y, ff.z, ff.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      a[0] = fmaf(xs1[q], ys1[q], a[0]);
      a[1] = fmaf(xs1[q], ys2[q], a[1]);
      a[2] = fmaf(xs2[q], ys2[q], a[2]);
      a[3] = fmaf(xs1[q], fs[q], a[3]);
      a[4] = fmaf(xs2[q], fs[q], a[4]);
    }
  }
  for (int64_t i = 4 * n4 + t0; i < n; i += ts) {
    a[0] = fmaf(v1[i], k1[i], a[0]);
    a[1] = fmaf(v1[i], k2[i], a[1]);
    a[2] = fmaf(v2[i], k2[i], a[2]);
    a[3] = fmaf(v1[i], f[i], a[3]);
    a[4] = fmaf(v2[i], f[i], a[4]);
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const double bs = block_sum((double)a[k], sh);
    if (threadIdx.x == 0) part[k * gridDim.x + blockIdx.x] = bs;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(&out[0].ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int k = 0; k < 5; ++k) {
    const double tot = sum_partials(part + k * gridDim.x, (int)gridDim.x, sh);
    if (threadIdx.x == 0) out[k].bb = tot;
  }
  if (threadIdx.x == 0) out[0].ticket = 0;
}


// The 2x2 Galerkin solve on the device: ws = {c1, c2, valid}; with
// `correction` also the deflation scalar pcg->wawinv = 1 / (w^T K w) (0 when
// the products are not usable)
__global__ void k_ws_solve(const PCGState* gal, double* ws, PCGState* pcg, int correction) {
  const double g11 = gal[0].bb, g12 = gal[1].bb, g22 = gal[2].bb, f1 = gal[3].bb, f2 = gal[4].bb;
  const double det = g11 * g22 - g12 * g12;
  const bool ok = isfinite(det) && det > 1e-12 * fabs(g11 * g22) && g11 > 0 && g22 > 0;
  ws[0] = ok ? (f1 * g22 - f2 * g12) / det : 0.0;
  ws[1] = ok ? (f2 * g11 - f1 * g12) / det : 0.0;
  ws[2] = ok ? 1.0 : 0.0;
  pcg->wawinv = (correction && isfinite(g22) && g22 > 0.0) ? 1.0 / g22 : 0.0;
  pcg->wr = pcg->wz = 0.0;
}
// u <- c1 u + c2 v2 when the 2x2 solve was usable
__global__ void k_ws_apply(int64_t n, const double* ws, double* u, const double* v2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && ws[2] != 0.0) u[i] = ws[0] * u[i] + ws[1] * v2[i];
}

// Warm start and coarse-grid correction for the current design.  The
// network's level-1 correction is prolongated to the fine grid (w = P y) and
// combined with the previous displacement (v1 = u_prev) by the energy-optimal
// (Galerkin) 2x2 solve
//   [v_i^T K v_j] c = [v_i^T f],   u0 = c1 v1 + c2 w,
// with the products in FP32 (the energy error of u0 is at most u_prev's).
// With `correction` the same w deflates the FP32 PCG of the solve (deflated
// CG: each pass starts with its residual made orthogonal to w, every search
// direction is made K-orthogonal to w), a coarse-grid correction by one
// extra basis vector.  Whether the learned start is kept is decided after the
// first cycle of the solve, against the plain warm start's residual (solve()).
void Cnn::warm_start(Ctx& c, bool combine, bool correction, cudaStream_t side) {
  // everything below is enqueued on the side stream (the helpers take the
  // context's stream member); the context's own stream comes back at the end
  struct Swap {
    Ctx& c;
    cudaStream_t keep;
    Swap(Ctx& c_, cudaStream_t s) : c(c_), keep(c_.st) { c.st = s; }
    ~Swap() { c.st = keep; }
  } swap(c, side);
  {
    ProfScope ps(PK_LEARNED, c.st);
    const int64_t n = c.g.ndofs();
    double* v2 = c.z2.p;
    features(c, c.u);            // p32 = u_prev, z32 = f, r32a = f - K u_prev, sr.rr = |r32a|^2
    forward(c.st, false);        // TF32 inference
    k_correction<<<nb(c.lv[1]->g.ndofs()), 256, 0, c.st>>>(c.lv[1]->g.ndofs(), y, su, corr);
    TG_CHECK_LAUNCH();
    TG_CUDA(cudaMemsetAsync(v2, 0, sizeof(double) * n, c.st));
    prolong_add<double>(c.g, c.lv[1]->g, c.op.fix, corr, v2, c.st);
    TG_CUDA(cudaMemcpyAsync(uprev.p, c.u.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.st));
    // w32 = w, q32 = K v1, aw32 = K w
    d2f(n, v2, w32, c.st);
    fine_apply<float, float>(c.op, c.s32, c.p32, c.q32, nullptr, nullptr, 0.0, AM_Y, c.st);
    fine_apply<float, float>(c.op, c.s32, w32, aw32, nullptr, nullptr, 0.0, AM_Y, c.st);
    const unsigned b5 = std::min<unsigned>(red_blocks(n), (unsigned)DOT5_BLOCKS);
    k_dot5<<<b5, RED_THREADS, 0, c.st>>>(n, c.p32, w32, c.q32, aw32, c.z32, rpart, gal.p);
    TG_CHECK_LAUNCH();
    k_ws_solve<<<1, 1, 0, c.st>>>(gal.p, wsb.p, c.pcg.p, correction ? 1 : 0);
    TG_CHECK_LAUNCH();
    if (combine) {
      k_ws_apply<<<nb(n), 256, 0, c.st>>>(n, wsb.p, c.u.p, v2);
      TG_CHECK_LAUNCH();
    }
  }
}

}  // namespace tg
