// Geometric multigrid on structured grids: assembled coarse stencils,
// exact (masked) Galerkin coarse operators, transfers, damped Jacobi, and the
// dense FP64 coarsest-grid inverse.
//
// The reference's multigrid (multigrid.py:89-154 V-cycle, gmg.py:148-189
// stride-2 coarse nodes, linear_solvers.py:306-372 damped Jacobi) forms
// P^T A P with SciPy on every V-cycle call and its interpolator
// (gmg.py:34-146) does not run.  Here:
//  * P is trilinear (bilinear) interpolation from the stride-2 nodes, per DOF
//    component, masked on both sides: Pt = M_f P M_c;
//  * level 1 is built straight from the element scale factors as
//    A_1 = Pt^T (M K(rho) M) Pt: an unmasked child element contributes
//    rho_c * Q_c with Q_c = P_c^T KE P_c precomputed once per problem, a
//    child touching a fixed DOF contributes the exact masked product;
//  * deeper levels are Galerkin products of the assembled stencils;
//  * stencils are symmetric and half-stored (the centre and the 13 upper
//    directions in 3-D, 4 in 2-D), structure-of-arrays
//    A[(dir*ndof+ci)*ndof+cj][node], so consecutive threads read coalesced
//    coefficients; a lower direction reads the neighbour's upper block
//    transposed;
//  * the coarsest level (a few hundred to ~8000 DOFs) is inverted once per
//    design iteration by the block sweep operator in FP64 (16-wide pivots)
//    and applied as one dense mat-vec per V-cycle.
#include <algorithm>
#include <atomic>
#include <cuda.h>

#include "tg_ops.cuh"

namespace tg {

template <int NDIM> __host__ __device__ constexpr int ndir() { return NDIM == 3 ? 27 : 9; }

__device__ __forceinline__ void node_xyz(const Grid& g, int64_t n, int& x, int& y, int& z) {
  y = (int)(n % g.nny);
  x = (int)((n / g.nny) % g.nnx);
  z = (int)(n / ((int64_t)g.nny * g.nnx));
}
// direction index: dy fastest, then dx, then dz; components in {-1,0,1}
__device__ __forceinline__ void dir_xyz(int d, int ndim, int& dx, int& dy, int& dz) {
  dy = d % 3 - 1;
  dx = (d / 3) % 3 - 1;
  dz = (ndim == 3) ? d / 9 - 1 : 0;
}
__device__ __forceinline__ int dir_index(int dx, int dy, int dz, int ndim) {
  return (ndim == 3 ? (dz + 1) * 9 : 0) + (dx + 1) * 3 + (dy + 1);
}
__device__ __forceinline__ bool in_grid(const Grid& g, int x, int y, int z) {
  return x >= 0 && x < g.nnx && y >= 0 && y < g.nny && z >= 0 && z < g.nnz;
}

// ---------------------------------------------------------------------------
// stencil mat-vec with fused residual / Jacobi epilogues
// ---------------------------------------------------------------------------
// Coarse operators are symmetric, so only the centre block and the blocks of
// the "upper" directions (index >= centre: dz, dx, dy lexicographically >= 0)
// are stored: A_h[((d - C)*ndof + ci)*ndof + cj][node].  The block of a lower
// direction d at node n is the transpose of the block of direction -d (index
// 2C - d) stored at the neighbour m = n + d.
template <int NDIM> __host__ __device__ constexpr int ndir_half() { return ndir<NDIM>() / 2 + 1; }

template <int NDIM, int NDOF, typename T>
__device__ __forceinline__ T coef(const T* __restrict__ A, int64_t ld, int d, int ci, int cj,
                                  int64_t n, int64_t m) {
  constexpr int C = ndir<NDIM>() / 2;
  return d >= C ? __ldg(A + (((d - C) * NDOF + ci) * NDOF + cj) * ld + n)
                : __ldg(A + (((C - d) * NDOF + cj) * NDOF + ci) * ld + m);
}

// One CTA per (TY x TX) patch of a node plane, NDOF x 256 threads: thread
// (ci, node) computes row ci of its node (81 coefficient loads in 3-D
// elasticity), so there are NDOF times more warps in flight than with a
// thread per node and fewer registers each -- the level-1 sweep is bound by
// the latency of its coefficient loads, not by their bandwidth.  TY spans
// whole y-rows where the grid allows, so consecutive threads own consecutive
// nodes and every coefficient load of a warp is contiguous.  The u values of
// the patch and its one-node halo in the planes z-1, z, z+1 are staged in
// shared memory, component-major (stride-1 reads across a warp), with zeros
// outside the grid.  A lower-direction block is read at the neighbour;
// outside the grid the node's own (finite) block is read instead and meets a
// zero u, so the loads need no branches.
template <int NDIM, int NDOF, typename T, int MODE>
__global__ void __launch_bounds__(NDOF * 256) k_stencil_apply(Grid g, int TY, int TX,
                                                             const T* __restrict__ A,
                                                             const T* __restrict__ u,
                                                             T* __restrict__ y,
                                                             const T* __restrict__ b,
                                                             const T* __restrict__ dinv, T omega) {
  pdl_wait();
  pdl_trigger();
  constexpr int NP = (NDIM == 3) ? 3 : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* us = reinterpret_cast<T*>(smem_raw);
  const int RY = TY + 2, PL = (TX + 2) * RY;
  const int y0 = blockIdx.x * TY, x0 = blockIdx.y * TX, z = blockIdx.z;
  const int64_t ld = g.slds();
  const int tid = threadIdx.x;
  // stage u (global order: component fastest)
  for (int i = tid; i < NDOF * NP * PL; i += blockDim.x) {
    const int c = i % NDOF, hy = (i / NDOF) % RY, hx = (i / (NDOF * RY)) % (TX + 2);
    const int pz = i / (NDOF * PL);
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = (NDIM == 3) ? z - 1 + pz : 0;
    T v = T(0);
    if (in_grid(g, gx, gy, gz)) v = __ldg(u + g.node(gx, gy, gz) * NDOF + c);
    us[(c * NP + pz) * PL + hx * RY + hy] = v;
  }
  __syncthreads();
  const int ci = tid >> 8, tn = tid & 255;      // row (warp-uniform), node of the patch
  const int ty = tn % TY, tx = tn / TY;
  const int xx = x0 + tx, yy = y0 + ty;
  if (tx >= TX || xx >= g.nnx || yy >= g.nny) return;
  const int64_t n = g.node(xx, yy, z);
  const bool ok[3][3] = {{xx > 0, true, xx + 1 < g.nnx},
                         {yy > 0, true, yy + 1 < g.nny},
                         {z > 0, true, z + 1 < g.nnz}};
  const int64_t sx = g.nny, sz = (int64_t)g.nny * g.nnx;
  const T* uc = us + ((NDIM == 3) ? PL : 0) + (tx + 1) * RY + (ty + 1);   // centre, plane z
  T acc = T(0);
#pragma unroll
  for (int d = 0; d < ndir<NDIM>(); ++d) {
    int dx, dy, dz;
    dir_xyz(d, NDIM, dx, dy, dz);
    const bool v = ok[0][dx + 1] && ok[1][dy + 1] && ok[2][dz + 1];
    const int64_t m = v ? n + dz * sz + dx * sx + dy : n;
    const int so = dz * PL + dx * RY + dy;
#pragma unroll
    for (int cj = 0; cj < NDOF; ++cj)
      acc = fma(coef<NDIM, NDOF, T>(A, ld, d, ci, cj, n, m), uc[cj * NP * PL + so], acc);
  }
  const int64_t k = n * NDOF + ci;
  T out;
  if (MODE == AM_Y) out = acc;
  else if (MODE == AM_RES) out = b[k] - acc;
  else out = uc[ci * NP * PL] + omega * dinv[k] * (b[k] - acc);
  y[k] = out;
}

// Loads of vectors: through the read-only cache in separate launches; at L2
// (coherent) inside the cooperative tail kernel, where the vector was written
// by other blocks earlier in the same launch.
template <bool CG, typename T>
__device__ __forceinline__ T ldv(const T* p) {
  if constexpr (CG) return __ldcg(p);
  else return __ldg(p);
}

// Small levels (too few (row, node) pairs to hide the coefficient-load
// latency): several threads per pair, each summing the 3 directions of one
// neighbour row (dz, dx fixed, dy = -1, 0, +1; 9 rows in 3-D, 3 in 2-D), the
// partial sums added in fixed order through shared memory -- a short load
// chain per thread and more CTAs on grids too small to fill the GPU.
template <int NDIM> __host__ __device__ constexpr int small_split() { return NDIM == 3 ? 9 : 3; }
template <int NDIM> __host__ __device__ constexpr int small_pairs() { return NDIM == 3 ? 64 : 128; }
template <int NDIM> __host__ __device__ constexpr int small_threads() {
  return small_split<NDIM>() * small_pairs<NDIM>();
}
// one block's work: pairs [vb * SP, (vb + 1) * SP) with small_threads
// threads; ends with a barrier, so part can be reused
template <int NDIM, int NDOF, typename T, int MODE, bool CG = false>
__device__ __forceinline__ void stencil_small_vb(const Grid& g, const T* __restrict__ A,
                                                 const T* __restrict__ u, T* __restrict__ y,
                                                 const T* __restrict__ b,
                                                 const T* __restrict__ dinv, T omega, int64_t vb,
                                                 T (&part)[small_split<NDIM>()][small_pairs<NDIM>()]) {
  constexpr int SP = small_pairs<NDIM>(), NS = small_split<NDIM>();
  const int slot = threadIdx.x % SP, pz = threadIdx.x / SP;
  const int64_t ld = g.nnodes(), lda = g.slds();
  const int64_t t = vb * SP + slot;
  const bool active = t < ld * NDOF;
  T acc = T(0);
  int ci = 0;
  int64_t n = 0;
  if (active) {
    ci = (int)(t / ld);
    n = t - (int64_t)ci * ld;
    int x, yy, z;
    node_xyz(g, n, x, yy, z);
    const int64_t sx = g.nny, sz = (int64_t)g.nny * g.nnx;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      // the row pz: 3-D (dz, dx) = (pz / 3 - 1, pz % 3 - 1), 2-D dx = pz - 1
      const int d = pz * 3 + e;
      int dx, dy, dz;
      dir_xyz(d, NDIM, dx, dy, dz);
      const bool v = in_grid(g, x + dx, yy + dy, z + dz);
      const int64_t m = v ? n + dz * sz + dx * sx + dy : n;
#pragma unroll
      for (int cj = 0; cj < NDOF; ++cj) {
        const T uu = ldv<CG>(u + m * NDOF + cj);
        acc = fma(coef<NDIM, NDOF, T>(A, lda, d, ci, cj, n, m), v ? uu : T(0), acc);
      }
    }
  }
  part[pz][slot] = acc;
  __syncthreads();
  if (pz == 0 && active) {
    T s = part[0][slot];
#pragma unroll
    for (int r = 1; r < NS; ++r) s += part[r][slot];
    const int64_t k = n * NDOF + ci;
    T out;
    if (MODE == AM_Y) out = s;
    else if (MODE == AM_RES) out = ldv<CG>(b + k) - s;
    else out = ldv<CG>(u + k) + omega * dinv[k] * (ldv<CG>(b + k) - s);
    y[k] = out;
  }
  __syncthreads();
}
template <int NDIM, int NDOF, typename T, int MODE>
__global__ void __launch_bounds__(small_threads<NDIM>()) k_stencil_small(Grid g, const T* __restrict__ A,
                                                                  const T* __restrict__ u,
                                                                  T* __restrict__ y,
                                                                  const T* __restrict__ b,
                                                                  const T* __restrict__ dinv,
                                                                  T omega) {
  pdl_wait();
  pdl_trigger();
  __shared__ T part[small_split<NDIM>()][small_pairs<NDIM>()];
  stencil_small_vb<NDIM, NDOF, T, MODE>(g, A, u, y, b, dinv, omega, blockIdx.x, part);
}

// ---------------------------------------------------------------------------
// 3-D FP32 stencil sweep with TMA-staged coefficients
// ---------------------------------------------------------------------------
// k_stencil_apply waits on its 81 coefficient loads per row one after another
// (long-scoreboard stalls).  Here one thread of the CTA issues, per direction
// d, one 2-D TMA copy of the NDOF^2 coefficient arrays of that direction over
// the CTA's node range into shared memory: a CTA owns TX whole y-rows of a
// plane, nodes [n0, n0 + P) contiguous, and a lower direction's blocks are
// read at the neighbour range [n0 + off(d), n0 + off(d) + P).  The tensor map
// views the stencil as (node, array) with the 128-byte-aligned array stride
// slds; each copy starts at the range start rounded down to a multiple of 4
// nodes (the TMA rule for 4-byte elements) and reads BX >= P + 3 nodes, zeros
// beyond the grid.  Three mbarriers (dz = -1, 0, +1) let the rows start on the
// first nine directions while the rest arrive; u is staged as in
// k_stencil_apply.  Same products in the same order as k_stencil_apply, so
// the results are bit-identical.  Every wait is bounded (about a second of
// %globaltimer); a wait that runs out sets the library's wait-error flag,
// waits once more for the copies in flight and leaves.
__device__ int g_wait_err = 0;


constexpr int STMA_PT = 128;           // node slots per CTA at most (threads = NDOF * PT)
constexpr int STMA_SMEM_MAX = 112 * 1024;

template <int NDOF, int MODE, int PT>
__global__ void __launch_bounds__(NDOF * PT) k_stencil_tma(const __grid_constant__ CUtensorMap tmA,
                                                                Grid g, int TX, int BX, int tstride,
                                                                const float* __restrict__ u,
                                                                float* __restrict__ y,
                                                                const float* __restrict__ b,
                                                                const float* __restrict__ dinv,
                                                                float omega) {
  constexpr int NB = NDOF * NDOF;
  constexpr int C = 13;
  extern __shared__ __align__(128) unsigned char stma_smem[];
  // 128-byte aligned start (the launch adds 128 bytes for this)
  unsigned char* base = stma_smem + ((128u - (smem_u32(stma_smem) & 127u)) & 127u);
  uint64_t* bar = reinterpret_cast<uint64_t*>(base);
  float* tiles = reinterpret_cast<float*>(base + 128);
  float* us = tiles + 27 * tstride;
  const int x0 = blockIdx.x * TX, z = blockIdx.y;
  const int TXe = min(TX, g.nnx - x0);
  const int P = TXe * g.nny;
  const int64_t n0 = g.node(x0, 0, z);
  const int64_t sx = g.nny, sz = (int64_t)g.nny * g.nnx;
  const int tid = threadIdx.x;
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[k])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    const uint32_t bytes = (uint32_t)(BX * NB * 4);
    for (int gz = 0; gz < 3; ++gz) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                   ::"r"(smem_u32(&bar[gz])), "r"(9 * bytes) : "memory");
      for (int e = 0; e < 9; ++e) {
        const int d = gz * 9 + e;
        int dx, dy, dz;
        dir_xyz(d, 3, dx, dy, dz);
        const int64_t off = (d >= C) ? 0 : dz * sz + dx * sx + dy;
        const int xs = (int)((n0 + off) & ~(int64_t)3);
        const int krow = (d >= C ? d - C : C - d) * NB;
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3}], [%4];"
            ::"r"(smem_u32(tiles + d * tstride)), "l"(reinterpret_cast<uint64_t>(&tmA)),
              "r"(xs), "r"(krow), "r"(smem_u32(&bar[gz]))
            : "memory");
      }
    }
  }
  // u of planes z-1..z+1, rows x0-1..x0+TX, y -1..nny (zeros outside the grid)
  const int RY = g.nny + 2, PL = (TX + 2) * RY;
  for (int i = tid; i < NDOF * 3 * PL; i += blockDim.x) {
    const int c = i % NDOF, hy = (i / NDOF) % RY, hx = (i / (NDOF * RY)) % (TX + 2);
    const int pz = i / (NDOF * PL);
    const int gx = x0 - 1 + hx, gy = -1 + hy, gz = z - 1 + pz;
    float v = 0.f;
    if (in_grid(g, gx, gy, gz)) v = __ldg(u + g.node(gx, gy, gz) * NDOF + c);
    us[(c * 3 + pz) * PL + hx * RY + hy] = v;
  }
  __syncthreads();
  const int ci = tid / PT, p = tid % PT;
  const bool active = p < P;
  const int tx = p / g.nny, ty = p % g.nny;
  const float* uc = us + PL + (tx + 1) * RY + (ty + 1);     // centre, plane z
  float acc = 0.f;
  bool ok = true;
#pragma unroll
  for (int gz = 0; gz < 3; ++gz) {
    if (!mbar_wait_bounded(&bar[gz], 0, 1000000000ull)) {
      ok = false;
      break;
    }
    if (active) {
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        const int d = gz * 9 + e;
        int dx, dy, dz;
        dir_xyz(d, 3, dx, dy, dz);
        const int64_t off = (d >= C) ? 0 : dz * sz + dx * sx + dy;
        const int xi = p + (int)((n0 + off) & 3);
        const float* tl = tiles + d * tstride + xi;
        const int so = dz * PL + dx * RY + dy;
#pragma unroll
        for (int cj = 0; cj < NDOF; ++cj) {
          const int r = (d >= C) ? ci * NDOF + cj : cj * NDOF + ci;
          acc = fmaf(tl[r * BX], uc[cj * 3 * PL + so], acc);
        }
      }
    }
  }
  if (!ok) {
    if (tid == 0) atomicExch(&g_wait_err, 1);
    for (int gz = 0; gz < 3; ++gz) mbar_wait_bounded(&bar[gz], 0, 1000000000ull);
    return;
  }
  if (!active) return;
  const int64_t n = n0 + p;
  const int64_t k = n * NDOF + ci;
  float out;
  if (MODE == AM_Y) out = acc;
  else if (MODE == AM_RES) out = b[k] - acc;
  else out = uc[ci * 3 * PL] + omega * dinv[k] * (b[k] - acc);
  y[k] = out;
}

namespace {
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    TG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q));
    TG_REQUIRE(q == cudaDriverEntryPointSuccess && p, "cuTensorMapEncodeTiled unavailable");
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}
// rows TX per CTA and the copy width BX for the TMA sweep, 0 when it does not apply
struct StmaShape {
  int TX = 0, BX = 0, tstride = 0, PT = 0;
  size_t smem = 0;
};
std::atomic<int> g_stma_on{0};
StmaShape stma_shape(const Grid& g) {
  StmaShape s;
  if (g.ndim != 3 || (g.ndof != 3 && g.ndof != 1)) return s;
  const int nb = g.ndof * g.ndof;
  const int cap = g_stma_on.load(std::memory_order_relaxed) > 1 ? g_stma_on.load() - 1 : 1 << 20;
  for (int tx = std::min(std::min(STMA_PT / g.nny, g.nnx), cap); tx >= 1; --tx) {
    const int bx = (tx * g.nny + 3 + 3) / 4 * 4;
    if (bx > 256) continue;
    const int ts = (bx * nb + 31) / 32 * 32;
    const size_t sm = 256 + sizeof(float) * (27 * (size_t)ts + (size_t)g.ndof * 3 * (tx + 2) * (g.nny + 2));
    if (sm <= (size_t)STMA_SMEM_MAX) {
      s.TX = tx; s.BX = bx; s.tstride = ts; s.smem = sm;
      s.PT = tx * g.nny <= 64 ? 64 : 128;
      return s;
    }
  }
  return s;
}
}  // namespace

void tune_set_stencil_tma(int on) { g_stma_on.store(on); }

int take_wait_error(cudaStream_t st) {
  int v = 0;
  TG_CUDA(cudaMemcpyFromSymbolAsync(&v, g_wait_err, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
  TG_CUDA(cudaStreamSynchronize(st));
  if (v) {
    static const int z = 0;
    TG_CUDA(cudaMemcpyToSymbolAsync(g_wait_err, &z, sizeof(int), 0, cudaMemcpyHostToDevice, st));
    TG_CUDA(cudaStreamSynchronize(st));
  }
  return v;
}

static bool stencil_apply_tma(const Grid& g, const float* A, const float* u, float* y,
                              const float* b, const float* dinv, double omega, int mode,
                              cudaStream_t st) {
  if (!g_stma_on.load(std::memory_order_relaxed)) return false;
  const StmaShape s = stma_shape(g);
  if (!s.TX) return false;
  TG_REQUIRE((reinterpret_cast<uintptr_t>(A) & 127) == 0, "stencil arrays must be 128-byte aligned");
  CUtensorMap tm;
  const cuuint64_t dims[2] = {(cuuint64_t)g.nnodes(), (cuuint64_t)(14 * g.ndof * g.ndof)};
  const cuuint64_t strides[1] = {(cuuint64_t)g.slds() * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)s.BX, (cuuint32_t)(g.ndof * g.ndof)};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode_tiled()(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(A),
                                    dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  TG_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed for the stencil");
  const dim3 grid((unsigned)cdiv(g.nnx, s.TX), (unsigned)g.nnz);
  const unsigned nt = (unsigned)(g.ndof * s.PT);
  const float om = (float)omega;
#define TG_ST(NF, M, PTV)                                                                      \
  {                                                                                            \
    static bool attr = false;                                                                  \
    if (!attr) {                                                                               \
      TG_CUDA(cudaFuncSetAttribute(k_stencil_tma<NF, M, PTV>,                                  \
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, STMA_SMEM_MAX)); \
      attr = true;                                                                             \
    }                                                                                          \
    k_stencil_tma<NF, M, PTV><<<grid, nt, s.smem, st>>>(tm, g, s.TX, s.BX, s.tstride, u, y, b, dinv, om); \
  }
#define TG_STM(NF, PTV)                                                                        \
  if (mode == AM_Y) TG_ST(NF, AM_Y, PTV) else if (mode == AM_RES) TG_ST(NF, AM_RES, PTV) else TG_ST(NF, AM_JACOBI, PTV)
  if (g.ndof == 3) {
    if (s.PT == 64) { TG_STM(3, 64) } else { TG_STM(3, 128) }
  } else {
    if (s.PT == 64) { TG_STM(1, 64) } else { TG_STM(1, 128) }
  }
#undef TG_STM
#undef TG_ST
  TG_CHECK_LAUNCH();
  return true;
}

template <typename T>
void stencil_apply(const Grid& g, const T* A, const T* u, T* y, const T* b, const T* dinv,
                   double omega, int mode, cudaStream_t st) {
  const int64_t pairs = g.nnodes() * g.ndof;
  if (pairs < tune_stencil_small_pairs()) {
#define TG_SS(ND, NF)                                                                          \
  {                                                                                            \
    const dim3 grid((unsigned)cdiv(pairs, small_pairs<ND>())), blk(small_threads<ND>());      \
    if (mode == AM_Y) launch_pdl(k_stencil_small<ND, NF, T, AM_Y>, grid, blk, 0, st, g, A, u, y, b, dinv, (T)omega); \
    else if (mode == AM_RES) launch_pdl(k_stencil_small<ND, NF, T, AM_RES>, grid, blk, 0, st, g, A, u, y, b, dinv, (T)omega); \
    else launch_pdl(k_stencil_small<ND, NF, T, AM_JACOBI>, grid, blk, 0, st, g, A, u, y, b, dinv, (T)omega); \
  }
    switch (g.ndim * 10 + g.ndof) {
      case 33: TG_SS(3, 3) break;
      case 31: TG_SS(3, 1) break;
      case 22: TG_SS(2, 2) break;
      case 21: TG_SS(2, 1) break;
      default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
    }
#undef TG_SS
    TG_CHECK_LAUNCH();
    return;
  }
  if constexpr (std::is_same<T, float>::value) {
    if (stencil_apply_tma(g, A, u, y, b, dinv, omega, mode, st)) return;
  }
  const int TY = std::min(g.nny, 256);
  const int TX = std::max(1, std::min(g.nnx, 256 / TY));
  const dim3 grid((unsigned)cdiv(g.nny, TY), (unsigned)cdiv(g.nnx, TX), (unsigned)g.nnz);
  const size_t smem = sizeof(T) * g.ndof * (g.ndim == 3 ? 3 : 1) * (TX + 2) * (TY + 2);
  const unsigned nt = 256u * (unsigned)g.ndof;
  const int key = g.ndim * 10 + g.ndof;
#define TG_SA(ND, NF)                                                                          \
  if (mode == AM_Y) launch_pdl(k_stencil_apply<ND, NF, T, AM_Y>, dim3(grid), dim3(nt), smem, st, g, TY, TX, A, u, y, b, dinv, (T)omega); \
  else if (mode == AM_RES) launch_pdl(k_stencil_apply<ND, NF, T, AM_RES>, dim3(grid), dim3(nt), smem, st, g, TY, TX, A, u, y, b, dinv, (T)omega); \
  else launch_pdl(k_stencil_apply<ND, NF, T, AM_JACOBI>, dim3(grid), dim3(nt), smem, st, g, TY, TX, A, u, y, b, dinv, (T)omega);
  switch (key) {
    case 33: TG_SA(3, 3) break;
    case 31: TG_SA(3, 1) break;
    case 22: TG_SA(2, 2) break;
    case 21: TG_SA(2, 1) break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
#undef TG_SA
  TG_CHECK_LAUNCH();
}
template void stencil_apply<double>(const Grid&, const double*, const double*, double*,
                                    const double*, const double*, double, int, cudaStream_t);
template void stencil_apply<float>(const Grid&, const float*, const float*, float*, const float*,
                                   const float*, double, int, cudaStream_t);

template <int NDIM, int NDOF, typename T>
__global__ void k_stencil_dinv(Grid g, const uint8_t* fix, const T* A, T* dinv) {
  pdl_wait();
  pdl_trigger();
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= g.nnodes()) return;
  const int64_t ld = g.slds();
#pragma unroll
  for (int c = 0; c < NDOF; ++c) {
    const T dg = A[(c * NDOF + c) * ld + n];     // centre block (half index 0)
    dinv[n * NDOF + c] = (((fix[n] >> c) & 1) || dg == T(0)) ? T(0) : T(1) / dg;
  }
}

template <typename T>
void stencil_dinv(const Grid& g, const uint8_t* fix, const T* A, T* dinv, cudaStream_t st) {
  const unsigned blocks = (unsigned)cdiv(g.nnodes(), 256);
  const int key = g.ndim * 10 + g.ndof;
  switch (key) {
    case 33: launch_pdl(k_stencil_dinv<3, 3, T>, dim3(blocks), dim3(256), 0, st, g, fix, A, dinv); break;
    case 31: launch_pdl(k_stencil_dinv<3, 1, T>, dim3(blocks), dim3(256), 0, st, g, fix, A, dinv); break;
    case 22: launch_pdl(k_stencil_dinv<2, 2, T>, dim3(blocks), dim3(256), 0, st, g, fix, A, dinv); break;
    case 21: launch_pdl(k_stencil_dinv<2, 1, T>, dim3(blocks), dim3(256), 0, st, g, fix, A, dinv); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
  TG_CHECK_LAUNCH();
}
template void stencil_dinv<double>(const Grid&, const uint8_t*, const double*, double*, cudaStream_t);
template void stencil_dinv<float>(const Grid&, const uint8_t*, const float*, float*, cudaStream_t);

// ---------------------------------------------------------------------------
// level 1 from the element scale factors
// ---------------------------------------------------------------------------
// weight of coarse corner a for child-element corner p of child octant o
__device__ __forceinline__ double pweight(int o, int p, int a, int ndim) {
  double w = 1.0;
  for (int k = 0; k < ndim; ++k) {
    const int pos = ((o >> k) & 1) + ((p >> k) & 1);   // 0..2 inside the coarse element
    const int dist = abs(pos - 2 * ((a >> k) & 1));
    w *= (dist == 0) ? 1.0 : (dist == 1 ? 0.5 : 0.0);
  }
  return w;
}

template <int NDIM, int NDOF, typename T>
__global__ void __launch_bounds__(256, 3) k_build_level1(Grid gf, Grid gc, const T* __restrict__ scale,
                                                      const uint8_t* __restrict__ touch,
                                                      const uint8_t* __restrict__ fixf,
                                                      const T* __restrict__ Q,
                                                      const T* __restrict__ KE,
                                                      const uint8_t* __restrict__ fixc,
                                                      T* __restrict__ Ac) {
  pdl_wait();
  pdl_trigger();
  constexpr int NC = 1 << NDIM;
  constexpr int NE = NC * NDOF;
  const int64_t ldc = gc.nnodes();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= ldc * ndir_half<NDIM>()) return;
  const int64_t I = t % ldc;
  const int DH = (int)(t / ldc), D = DH + ndir<NDIM>() / 2;   // upper directions only
  int ix, iy, iz, dx, dy, dz;
  node_xyz(gc, I, ix, iy, iz);
  dir_xyz(D, NDIM, dx, dy, dz);
  const int jx = ix + dx, jy = iy + dy, jz = iz + dz;
  T acc[NDOF][NDOF];
#pragma unroll
  for (int a = 0; a < NDOF; ++a)
#pragma unroll
    for (int b = 0; b < NDOF; ++b) acc[a][b] = T(0);
  if (in_grid(gc, jx, jy, jz)) {
    const int64_t J = gc.node(jx, jy, jz);
    const int exl = max(max(ix, jx) - 1, 0), exh = min(min(ix, jx), gc.nex - 1);
    const int eyl = max(max(iy, jy) - 1, 0), eyh = min(min(iy, jy), gc.ney - 1);
    const int ezl = (NDIM == 3) ? max(max(iz, jz) - 1, 0) : 0;
    const int ezh = (NDIM == 3) ? min(min(iz, jz), gc.nez - 1) : 0;
    for (int ez = ezl; ez <= ezh; ++ez)
      for (int ex = exl; ex <= exh; ++ex)
        for (int ey = eyl; ey <= eyh; ++ey) {
          const int ca = (ix - ex) | ((iy - ey) << 1) | ((NDIM == 3 ? iz - ez : 0) << 2);
          const int cb = (jx - ex) | ((jy - ey) << 1) | ((NDIM == 3 ? jz - ez : 0) << 2);
          // children touching no fixed DOF, the common case, in one unrolled
          // pass (their density and table loads independent of each other)
          const int64_t fe0 = gf.elem(2 * ex, 2 * ey, (NDIM == 3) ? 2 * ez : 0);
          const int64_t fsx = gf.ney, fsz = (int64_t)gf.nex * gf.ney;
          bool any_touch = false;
#pragma unroll
          for (int o = 0; o < NC; ++o)
            any_touch |= touch[fe0 + (o & 1) * fsx + ((o >> 1) & 1) + ((o >> 2) & 1) * fsz] != 0;
          if (!any_touch) {
#pragma unroll
            for (int o = 0; o < NC; ++o) {
              const T rho = scale[fe0 + (o & 1) * fsx + ((o >> 1) & 1) + ((o >> 2) & 1) * fsz];
              const T* Qo = Q + (int64_t)o * NE * NE;
#pragma unroll
              for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
                for (int cj = 0; cj < NDOF; ++cj)
                  acc[ci][cj] += rho * __ldg(Qo + (ca * NDOF + ci) * NE + cb * NDOF + cj);
            }
            continue;
          }
#pragma unroll 1
          for (int o = 0; o < NC; ++o) {
            const int fx = 2 * ex + (o & 1), fy = 2 * ey + ((o >> 1) & 1);
            const int fz = (NDIM == 3) ? 2 * ez + ((o >> 2) & 1) : 0;
            const int64_t fe = gf.elem(fx, fy, fz);
            const T rho = scale[fe];
            if (!touch[fe]) {
              const T* Qo = Q + (int64_t)o * NE * NE;
#pragma unroll
              for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
                for (int cj = 0; cj < NDOF; ++cj)
                  acc[ci][cj] += rho * __ldg(Qo + (ca * NDOF + ci) * NE + cb * NDOF + cj);
            } else {
              // exact: sum_{p,q} P[p,a] P[q,b] m(p,ci) m(q,cj) KE[(p,ci),(q,cj)]
              for (int p = 0; p < NC; ++p) {
                const T wp = (T)pweight(o, p, ca, NDIM);
                if (wp == T(0)) continue;
                const uint8_t mp = fixf[gf.node(fx + (p & 1), fy + ((p >> 1) & 1),
                                                 (NDIM == 3) ? fz + ((p >> 2) & 1) : 0)];
                for (int q = 0; q < NC; ++q) {
                  const T wq = (T)pweight(o, q, cb, NDIM);
                  if (wq == T(0)) continue;
                  const uint8_t mq = fixf[gf.node(fx + (q & 1), fy + ((q >> 1) & 1),
                                                   (NDIM == 3) ? fz + ((q >> 2) & 1) : 0)];
                  for (int ci = 0; ci < NDOF; ++ci) {
                    if ((mp >> ci) & 1) continue;
                    for (int cj = 0; cj < NDOF; ++cj) {
                      if ((mq >> cj) & 1) continue;
                      acc[ci][cj] += rho * wp * wq * KE[(p * NDOF + ci) * NE + q * NDOF + cj];
                    }
                  }
                }
              }
            }
          }
        }
    const uint8_t mi = fixc[I], mj = fixc[J];
#pragma unroll
    for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
      for (int cj = 0; cj < NDOF; ++cj)
        if (((mi >> ci) & 1) || ((mj >> cj) & 1)) acc[ci][cj] = T(0);
  }
#pragma unroll
  for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
    for (int cj = 0; cj < NDOF; ++cj) Ac[((DH * NDOF + ci) * NDOF + cj) * gc.slds() + I] = acc[ci][cj];
}

template <typename T>
void build_level1(const FineOp& op, const T* scale, const uint8_t* touch, const T* Q, const T* KE,
                  const Grid& gc, const uint8_t* fixc, T* Ac, cudaStream_t st) {
  const int64_t nt = gc.nnodes() * (op.g.ndim == 3 ? 14 : 5);
  const unsigned blocks = (unsigned)cdiv(nt, 256);
  const int key = op.g.ndim * 10 + op.g.ndof;
  switch (key) {
    case 33: launch_pdl(k_build_level1<3, 3, T>, dim3(blocks), dim3(256), 0, st, op.g, gc, scale, touch, op.fix, Q, KE, fixc, Ac); break;
    case 31: launch_pdl(k_build_level1<3, 1, T>, dim3(blocks), dim3(256), 0, st, op.g, gc, scale, touch, op.fix, Q, KE, fixc, Ac); break;
    case 22: launch_pdl(k_build_level1<2, 2, T>, dim3(blocks), dim3(256), 0, st, op.g, gc, scale, touch, op.fix, Q, KE, fixc, Ac); break;
    case 21: launch_pdl(k_build_level1<2, 1, T>, dim3(blocks), dim3(256), 0, st, op.g, gc, scale, touch, op.fix, Q, KE, fixc, Ac); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
  TG_CHECK_LAUNCH();
}
template void build_level1<double>(const FineOp&, const double*, const uint8_t*, const double*,
                                   const double*, const Grid&, const uint8_t*, double*, cudaStream_t);
template void build_level1<float>(const FineOp&, const float*, const uint8_t*, const float*,
                                  const float*, const Grid&, const uint8_t*, float*, cudaStream_t);

// fine-level stencil assembled from the element scale factors (used when the
// fine grid is itself the coarsest level): A[I][D] = sum_e s_e M KE M
template <int NDIM, int NDOF>
__global__ void __launch_bounds__(256) k_build_fine(Grid g, const double* __restrict__ scale,
                                                    const uint8_t* __restrict__ fix,
                                                    const double* __restrict__ KE,
                                                    double* __restrict__ A) {
  constexpr int NE = (1 << NDIM) * NDOF;
  const int64_t ld = g.nnodes();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= ld * ndir_half<NDIM>()) return;
  const int64_t I = t % ld;
  const int DH = (int)(t / ld), D = DH + ndir<NDIM>() / 2;
  int ix, iy, iz, dx, dy, dz;
  node_xyz(g, I, ix, iy, iz);
  dir_xyz(D, NDIM, dx, dy, dz);
  const int jx = ix + dx, jy = iy + dy, jz = iz + dz;
  double acc[NDOF][NDOF];
#pragma unroll
  for (int a = 0; a < NDOF; ++a)
#pragma unroll
    for (int b = 0; b < NDOF; ++b) acc[a][b] = 0.0;
  if (in_grid(g, jx, jy, jz)) {
    const int64_t J = g.node(jx, jy, jz);
    const int exl = max(max(ix, jx) - 1, 0), exh = min(min(ix, jx), g.nex - 1);
    const int eyl = max(max(iy, jy) - 1, 0), eyh = min(min(iy, jy), g.ney - 1);
    const int ezl = (NDIM == 3) ? max(max(iz, jz) - 1, 0) : 0;
    const int ezh = (NDIM == 3) ? min(min(iz, jz), g.nez - 1) : 0;
    for (int ez = ezl; ez <= ezh; ++ez)
      for (int ex = exl; ex <= exh; ++ex)
        for (int ey = eyl; ey <= eyh; ++ey) {
          const int ca = (ix - ex) | ((iy - ey) << 1) | ((NDIM == 3 ? iz - ez : 0) << 2);
          const int cb = (jx - ex) | ((jy - ey) << 1) | ((NDIM == 3 ? jz - ez : 0) << 2);
          const double s = scale[g.elem(ex, ey, ez)];
#pragma unroll
          for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
            for (int cj = 0; cj < NDOF; ++cj)
              acc[ci][cj] += s * KE[(ca * NDOF + ci) * NE + cb * NDOF + cj];
        }
    const uint8_t mi = fix[I], mj = fix[J];
#pragma unroll
    for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
      for (int cj = 0; cj < NDOF; ++cj)
        if (((mi >> ci) & 1) || ((mj >> cj) & 1)) acc[ci][cj] = 0.0;
  }
#pragma unroll
  for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
    for (int cj = 0; cj < NDOF; ++cj) A[((DH * NDOF + ci) * NDOF + cj) * g.slds() + I] = acc[ci][cj];
}

void build_fine_stencil(const FineOp& op, const double* scale, double* A, cudaStream_t st) {
  const int64_t nt = op.g.nnodes() * (op.g.ndim == 3 ? 14 : 5);
  const unsigned blocks = (unsigned)cdiv(nt, 256);
  const int key = op.g.ndim * 10 + op.g.ndof;
  switch (key) {
    case 33: k_build_fine<3, 3><<<blocks, 256, 0, st>>>(op.g, scale, op.fix, op.KE64, A); break;
    case 31: k_build_fine<3, 1><<<blocks, 256, 0, st>>>(op.g, scale, op.fix, op.KE64, A); break;
    case 22: k_build_fine<2, 2><<<blocks, 256, 0, st>>>(op.g, scale, op.fix, op.KE64, A); break;
    case 21: k_build_fine<2, 1><<<blocks, 256, 0, st>>>(op.g, scale, op.fix, op.KE64, A); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// Galerkin product of an assembled stencil
// ---------------------------------------------------------------------------
// Valid (a, b) pairs per axis for coarse offset d = j - i: fine nodes 2i + a
// and 2j + b (a, b in {-1, 0, 1}) that lie within one fine cell of each other
// (r = 2d + b - a in {-1, 0, 1}): 3, 7 and 3 pairs for d = -1, 0, 1.
__constant__ int8_t c_gal_a[3][7] = {{-1, -1, 0, 0, 0, 0, 0}, {-1, -1, 0, 0, 0, 1, 1}, {0, 1, 1, 0, 0, 0, 0}};
__constant__ int8_t c_gal_b[3][7] = {{0, 1, 1, 0, 0, 0, 0}, {-1, 0, -1, 0, 1, 0, 1}, {-1, -1, 0, 0, 0, 0, 0}};
__host__ __device__ constexpr int gal_pairs(int d) { return d == 0 ? 7 : 3; }

// Galerkin product of a half-stored stencil, Ac(I, J) = sum P(f, I) Af(f, g)
// P(g, J): a group of 8 threads per (coarse node I, upper direction D), lane
// k taking the k-th valid pair of the slowest axis (z in 3-D, x in 2-D) and
// looping over the valid pairs of the other axes, so only contributing fine
// pairs are visited (1270 of 27 x 27 per node in 3-D) and the small coarse
// levels get 8x the threads; the group's partial blocks are added by a fixed
// shuffle tree.
constexpr int GAL_LANES = 8;
template <int NDIM, int NDOF, typename T>
__global__ void __launch_bounds__(256) k_galerkin(Grid gf, const T* __restrict__ Af, Grid gc,
                                                  const uint8_t* __restrict__ fixc,
                                                  T* __restrict__ Ac) {
  pdl_wait();
  pdl_trigger();
  const int64_t ldc = gc.nnodes();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x % GAL_LANES;
  const int64_t grp = t / GAL_LANES;
  const bool active = grp < ldc * ndir_half<NDIM>();
  const int64_t I = active ? grp % ldc : 0;
  const int DH = active ? (int)(grp / ldc) : 0, D = DH + ndir<NDIM>() / 2;
  int ix, iy, iz, dx, dy, dz;
  node_xyz(gc, I, ix, iy, iz);
  dir_xyz(D, NDIM, dx, dy, dz);
  const int jx = ix + dx, jy = iy + dy, jz = iz + dz;
  const bool jin = active && in_grid(gc, jx, jy, jz);
  T acc[NDOF][NDOF];
#pragma unroll
  for (int a = 0; a < NDOF; ++a)
#pragma unroll
    for (int b = 0; b < NDOF; ++b) acc[a][b] = T(0);
  // slowest axis of the lane: z in 3-D, x in 2-D
  const int ds = (NDIM == 3) ? dz : dx;
  if (jin && lane < gal_pairs(ds)) {
    const int as = c_gal_a[ds + 1][lane], bs = c_gal_b[ds + 1][lane];
    const int fs = 2 * ((NDIM == 3) ? iz : ix) + as, gs = 2 * ((NDIM == 3) ? jz : jx) + bs;
    const int ns = (NDIM == 3) ? gf.nnz : gf.nnx;
    if (fs >= 0 && fs < ns && gs >= 0 && gs < ns) {
      const T ws = T((as ? 0.5 : 1.0) * (bs ? 0.5 : 1.0));
      const int rs = gs - fs;
      // the middle axis (x in 3-D; none in 2-D) and y
      const int nm = (NDIM == 3) ? gal_pairs(dx) : 1;
      for (int km = 0; km < nm; ++km) {
        const int am = (NDIM == 3) ? c_gal_a[dx + 1][km] : 0;
        const int bm = (NDIM == 3) ? c_gal_b[dx + 1][km] : 0;
        const int fx = (NDIM == 3) ? 2 * ix + am : fs, gx = (NDIM == 3) ? 2 * jx + bm : gs;
        if (fx < 0 || fx >= gf.nnx || gx < 0 || gx >= gf.nnx) continue;
        const T wm = ws * T((am ? 0.5 : 1.0) * (bm ? 0.5 : 1.0));
        const int fz = (NDIM == 3) ? fs : 0, gz = (NDIM == 3) ? gs : 0;
        const int rx = gx - fx, rz = (NDIM == 3) ? rs : 0;
#pragma unroll
        for (int ky = 0; ky < 7; ++ky) {
          if (ky >= gal_pairs(dy)) break;
          const int ay = c_gal_a[dy + 1][ky], by = c_gal_b[dy + 1][ky];
          const int fy = 2 * iy + ay, gy = 2 * jy + by;
          if (fy < 0 || fy >= gf.nny || gy < 0 || gy >= gf.nny) continue;
          const T w = wm * T((ay ? 0.5 : 1.0) * (by ? 0.5 : 1.0));
          const int dd = dir_index(rx, gy - fy, rz, NDIM);
          const int64_t fi = gf.node(fx, fy, fz), gi = gf.node(gx, gy, gz);
#pragma unroll
          for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
            for (int cj = 0; cj < NDOF; ++cj)
              acc[ci][cj] += w * coef<NDIM, NDOF, T>(Af, gf.slds(), dd, ci, cj, fi, gi);
        }
      }
    }
  }
#pragma unroll
  for (int off = GAL_LANES / 2; off > 0; off >>= 1)
#pragma unroll
    for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
      for (int cj = 0; cj < NDOF; ++cj)
        acc[ci][cj] += __shfl_xor_sync(0xffffffffu, acc[ci][cj], off);
  if (!active || lane != 0) return;
  if (jin) {
    const int64_t J = gc.node(jx, jy, jz);
    const uint8_t mi = fixc[I], mj = fixc[J];
#pragma unroll
    for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
      for (int cj = 0; cj < NDOF; ++cj)
        if (((mi >> ci) & 1) || ((mj >> cj) & 1)) acc[ci][cj] = T(0);
  }
#pragma unroll
  for (int ci = 0; ci < NDOF; ++ci)
#pragma unroll
    for (int cj = 0; cj < NDOF; ++cj) Ac[((DH * NDOF + ci) * NDOF + cj) * gc.slds() + I] = acc[ci][cj];
}

template <typename T>
void build_galerkin(const Grid& gf, const T* Af, const Grid& gc, const uint8_t* fixc, T* Ac,
                    cudaStream_t st) {
  const int64_t nt = gc.nnodes() * (gf.ndim == 3 ? 14 : 5) * GAL_LANES;
  const unsigned blocks = (unsigned)cdiv(nt, 256);
  const int key = gf.ndim * 10 + gf.ndof;
  switch (key) {
    case 33: launch_pdl(k_galerkin<3, 3, T>, dim3(blocks), dim3(256), 0, st, gf, Af, gc, fixc, Ac); break;
    case 31: launch_pdl(k_galerkin<3, 1, T>, dim3(blocks), dim3(256), 0, st, gf, Af, gc, fixc, Ac); break;
    case 22: launch_pdl(k_galerkin<2, 2, T>, dim3(blocks), dim3(256), 0, st, gf, Af, gc, fixc, Ac); break;
    case 21: launch_pdl(k_galerkin<2, 1, T>, dim3(blocks), dim3(256), 0, st, gf, Af, gc, fixc, Ac); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
  TG_CHECK_LAUNCH();
}
template void build_galerkin<double>(const Grid&, const double*, const Grid&, const uint8_t*,
                                     double*, cudaStream_t);
template void build_galerkin<float>(const Grid&, const float*, const Grid&, const uint8_t*,
                                    float*, cudaStream_t);

template <int NDIM, int NDOF, typename T>
__global__ void k_stencil_expand(Grid g, const T* __restrict__ Ah, double* __restrict__ Af) {
  const int64_t ld = g.nnodes();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= ld * ndir<NDIM>() * NDOF * NDOF) return;
  const int64_t n = t % ld;
  const int k = (int)(t / ld);
  const int cj = k % NDOF, ci = (k / NDOF) % NDOF, d = k / (NDOF * NDOF);
  int x, y, z, dx, dy, dz;
  node_xyz(g, n, x, y, z);
  dir_xyz(d, NDIM, dx, dy, dz);
  Af[t] = in_grid(g, x + dx, y + dy, z + dz)
              ? (double)coef<NDIM, NDOF, T>(Ah, g.slds(), d, ci, cj, n, g.node(x + dx, y + dy, z + dz))
              : 0.0;
}

template <typename T>
void stencil_expand(const Grid& g, const T* Ah, double* Af, cudaStream_t st) {
  const unsigned blocks = (unsigned)cdiv(g.nnodes() * (g.ndim == 3 ? 27 : 9) * g.ndof * g.ndof, 256);
  switch (g.ndim * 10 + g.ndof) {
    case 33: k_stencil_expand<3, 3, T><<<blocks, 256, 0, st>>>(g, Ah, Af); break;
    case 31: k_stencil_expand<3, 1, T><<<blocks, 256, 0, st>>>(g, Ah, Af); break;
    case 22: k_stencil_expand<2, 2, T><<<blocks, 256, 0, st>>>(g, Ah, Af); break;
    case 21: k_stencil_expand<2, 1, T><<<blocks, 256, 0, st>>>(g, Ah, Af); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
  TG_CHECK_LAUNCH();
}
template void stencil_expand<double>(const Grid&, const double*, double*, cudaStream_t);
template void stencil_expand<float>(const Grid&, const float*, double*, cudaStream_t);

// ---------------------------------------------------------------------------
// transfers
// ---------------------------------------------------------------------------
// restriction: one thread per (component, coarse node), fully unrolled over
// the 3^ndim fine nodes of the coarse node's support
// (optionally fused with the coarse level's first smoothing step from a zero
// guess, xc = omega * dinvc * bc)
template <int NDIM, int NDOF, typename T, bool CG = false>
__device__ __forceinline__ void restrict_one(const Grid& gf, const Grid& gc, const uint8_t* fixc,
                                             const T* __restrict__ rf, T* __restrict__ bc,
                                             const T* __restrict__ dinvc, T* __restrict__ xc,
                                             T omega, int64_t t) {
  const int64_t ldc = gc.nnodes();
  const int c = (int)(t / ldc);
  const int64_t I = t - (int64_t)c * ldc;
  int ix, iy, iz;
  node_xyz(gc, I, ix, iy, iz);
  T acc = T(0);
#pragma unroll
  for (int al = 0; al < ndir<NDIM>(); ++al) {
    int ax, ay, az;
    dir_xyz(al, NDIM, ax, ay, az);
    const int fx = 2 * ix + ax, fy = 2 * iy + ay, fz = 2 * iz + az;
    if (!in_grid(gf, fx, fy, fz)) continue;
    const T w = T((ax ? 0.5 : 1.0) * (ay ? 0.5 : 1.0) * (az ? 0.5 : 1.0));
    acc += w * ldv<CG>(rf + gf.node(fx, fy, fz) * NDOF + c);
  }
  const T bv = ((fixc[I] >> c) & 1) ? T(0) : acc;
  bc[I * NDOF + c] = bv;
  if (xc) xc[I * NDOF + c] = omega * dinvc[I * NDOF + c] * bv;
}
template <int NDIM, int NDOF, typename T>
__global__ void __launch_bounds__(256) k_restrict(Grid gf, Grid gc, const uint8_t* fixc,
                                                  const T* __restrict__ rf, T* __restrict__ bc,
                                                  const T* __restrict__ dinvc, T* __restrict__ xc,
                                                  T omega) {
  pdl_wait();
  pdl_trigger();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < gc.nnodes() * NDOF) restrict_one<NDIM, NDOF, T>(gf, gc, fixc, rf, bc, dinvc, xc, omega, t);
}

template <typename T>
void restrict_(const Grid& gf, const Grid& gc, const uint8_t* fixc, const T* rf, T* bc,
               cudaStream_t st, const T* dinvc, T* xc, double omega) {
  const unsigned blocks = (unsigned)cdiv(gc.nnodes() * gc.ndof, 256);
  switch (gf.ndim * 10 + gf.ndof) {
    case 33: launch_pdl(k_restrict<3, 3, T>, dim3(blocks), dim3(256), 0, st, gf, gc, fixc, rf, bc, dinvc, xc, (T)omega); break;
    case 31: launch_pdl(k_restrict<3, 1, T>, dim3(blocks), dim3(256), 0, st, gf, gc, fixc, rf, bc, dinvc, xc, (T)omega); break;
    case 22: launch_pdl(k_restrict<2, 2, T>, dim3(blocks), dim3(256), 0, st, gf, gc, fixc, rf, bc, dinvc, xc, (T)omega); break;
    case 21: launch_pdl(k_restrict<2, 1, T>, dim3(blocks), dim3(256), 0, st, gf, gc, fixc, rf, bc, dinvc, xc, (T)omega); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
  TG_CHECK_LAUNCH();
}
template void restrict_<double>(const Grid&, const Grid&, const uint8_t*, const double*, double*, cudaStream_t,
                                const double*, double*, double);
template void restrict_<float>(const Grid&, const Grid&, const uint8_t*, const float*, float*, cudaStream_t,
                               const float*, float*, double);

// prolongation: one thread per fine node, all components; the 1, 2, 4 or 8
// coarse parents follow from the parity of the fine coordinates
template <int NDIM, int NDOF, typename T, bool CG = false, bool SET = false>
__device__ __forceinline__ void prolong_one(const Grid& gf, const Grid& gc, const uint8_t* fixf,
                                            const T* __restrict__ xc, T* __restrict__ xf,
                                            int64_t i) {
  int fx, fy, fz;
  node_xyz(gf, i, fx, fy, fz);
  const int ox = fx & 1, oy = fy & 1, oz = (NDIM == 3) ? (fz & 1) : 0;
  const int cx0 = fx >> 1, cy0 = fy >> 1, cz0 = (NDIM == 3) ? fz >> 1 : 0;
  const T w = T((ox ? 0.5 : 1.0) * (oy ? 0.5 : 1.0) * (oz ? 0.5 : 1.0));
  T acc[NDOF];
#pragma unroll
  for (int c = 0; c < NDOF; ++c) acc[c] = T(0);
#pragma unroll
  for (int k = 0; k < (1 << NDIM); ++k) {
    const int a = k & 1, b = (k >> 1) & 1, d = (k >> 2) & 1;
    if ((a && !ox) || (b && !oy) || (d && !oz)) continue;
    const int64_t I = gc.node(cx0 + a, cy0 + b, cz0 + d);
#pragma unroll
    for (int c = 0; c < NDOF; ++c) acc[c] += ldv<CG>(xc + I * NDOF + c);
  }
  const uint8_t m = fixf[i];
#pragma unroll
  for (int c = 0; c < NDOF; ++c) {
    if (SET) xf[i * NDOF + c] = ((m >> c) & 1) ? T(0) : w * acc[c];
    else if (!((m >> c) & 1)) xf[i * NDOF + c] += w * acc[c];
  }
}
template <int NDIM, int NDOF, typename T, bool SET>
__global__ void __launch_bounds__(256) k_prolong_add(Grid gf, Grid gc, const uint8_t* fixf,
                                                     const T* __restrict__ xc,
                                                     T* __restrict__ xf) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < gf.nnodes()) prolong_one<NDIM, NDOF, T, false, SET>(gf, gc, fixf, xc, xf, i);
}

template <typename T, bool SET>
static void prolong_launch(const Grid& gf, const Grid& gc, const uint8_t* fixf, const T* xc, T* xf,
                           cudaStream_t st) {
  const unsigned blocks = (unsigned)cdiv(gf.nnodes(), 256);
  switch (gf.ndim * 10 + gf.ndof) {
    case 33: launch_pdl(k_prolong_add<3, 3, T, SET>, dim3(blocks), dim3(256), 0, st, gf, gc, fixf, xc, xf); break;
    case 31: launch_pdl(k_prolong_add<3, 1, T, SET>, dim3(blocks), dim3(256), 0, st, gf, gc, fixf, xc, xf); break;
    case 22: launch_pdl(k_prolong_add<2, 2, T, SET>, dim3(blocks), dim3(256), 0, st, gf, gc, fixf, xc, xf); break;
    case 21: launch_pdl(k_prolong_add<2, 1, T, SET>, dim3(blocks), dim3(256), 0, st, gf, gc, fixf, xc, xf); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
  TG_CHECK_LAUNCH();
}
template <typename T>
void prolong_add(const Grid& gf, const Grid& gc, const uint8_t* fixf, const T* xc, T* xf,
                 cudaStream_t st) {
  prolong_launch<T, false>(gf, gc, fixf, xc, xf, st);
}
template <typename T>
void prolong_set(const Grid& gf, const Grid& gc, const uint8_t* fixf, const T* xc, T* xf,
                 cudaStream_t st) {
  prolong_launch<T, true>(gf, gc, fixf, xc, xf, st);
}
template void prolong_add<double>(const Grid&, const Grid&, const uint8_t*, const double*, double*, cudaStream_t);
template void prolong_add<float>(const Grid&, const Grid&, const uint8_t*, const float*, float*, cudaStream_t);
template void prolong_set<double>(const Grid&, const Grid&, const uint8_t*, const double*, double*, cudaStream_t);
template void prolong_set<float>(const Grid&, const Grid&, const uint8_t*, const float*, float*, cudaStream_t);

// ---------------------------------------------------------------------------
// coarsest level: dense matrix and blocked Gauss-Jordan inverse (FP64)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_stencil_to_dense(Grid g, const uint8_t* fix, const T* __restrict__ A,
                                   double* D, int64_t n, int64_t ld) {
  pdl_wait();
  pdl_trigger();
  const int64_t ldA = g.nnodes();
  const int C = g.ndim == 3 ? 13 : 4;
  const int nh = C + 1;
  const int ndof = g.ndof;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= ldA * nh * ndof * ndof) return;
  const int64_t I = t % ldA;
  const int k = (int)(t / ldA);          // (dh*ndof+ci)*ndof+cj
  const int cj = k % ndof, ci = (k / ndof) % ndof, dh = k / (ndof * ndof);
  int ix, iy, iz, dx, dy, dz;
  node_xyz(g, I, ix, iy, iz);
  dir_xyz(C + dh, g.ndim, dx, dy, dz);
  if (!in_grid(g, ix + dx, iy + dy, iz + dz)) return;
  const int64_t J = g.node(ix + dx, iy + dy, iz + dz);
  const double v = (double)A[(int64_t)k * g.slds() + I];
  D[(I * ndof + ci) * ld + J * ndof + cj] = v;
  if (dh > 0) D[(J * ndof + cj) * ld + I * ndof + ci] = v;   // mirrored lower block
}
__global__ void k_dense_fix_diag(Grid g, const uint8_t* fix, double* D, int64_t n, int64_t ld) {
  pdl_wait();
  pdl_trigger();
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= ld) return;
  if (r >= n) {
    D[r * ld + r] = 1.0;
    return;
  }
  const int64_t node = r / g.ndof;
  const int c = (int)(r % g.ndof);
  if ((fix[node] >> c) & 1) D[r * ld + r] = 1.0;
}

template <typename T>
void stencil_to_dense(const Grid& g, const uint8_t* fix, const T* A, double* D, int64_t n,
                      int64_t ld, cudaStream_t st) {
  TG_CUDA(cudaMemsetAsync(D, 0, sizeof(double) * ld * ld, st));
  const int64_t nt = g.nnodes() * (g.ndim == 3 ? 14 : 5) * g.ndof * g.ndof;
  launch_pdl(k_stencil_to_dense<T>, dim3((unsigned)cdiv(nt, 256)), dim3(256), 0, st, g, fix, A, D, n, ld);
  TG_CHECK_LAUNCH();
  launch_pdl(k_dense_fix_diag, dim3((unsigned)cdiv(ld, 256)), dim3(256), 0, st, g, fix, D, n, ld);
  TG_CHECK_LAUNCH();
}
template void stencil_to_dense<double>(const Grid&, const uint8_t*, const double*, double*,
                                       int64_t, int64_t, cudaStream_t);
template void stencil_to_dense<float>(const Grid&, const uint8_t*, const float*, double*, int64_t,
                                      int64_t, cudaStream_t);

constexpr int GJB = 32;   // tile of the final mirror / negate pass
constexpr int SWB = 16;   // pivot block of the sweep operator

// Invert a TB x TB SPD tile in shared memory (Gauss-Jordan without pivoting)
// with TB*TB threads, (i, j) = (y, x).  Every pivot step reads tile a and
// writes tile b (two shared buffers: no hazard inside a step) and costs one
// barrier: the thread that computes the next pivot element also computes its
// reciprocal in the same step (GB300's FP64 pipe is narrow and a divide is a
// long dependent sequence, so there is one per step, off the other threads'
// path); all other elements take one multiply or FMA.  A single warp would
// use only its own sub-partition's share of the FP64 pipe.  TB is even, so
// the inverse ends in a.
template <int TB>
__device__ __forceinline__ void gj_tile_inverse(double (&a)[TB][TB + 1], double (&b)[TB][TB + 1],
                                                double (&rpiv)[2], int i, int j) {
  if (i == 0 && j == 0) rpiv[0] = 1.0 / a[0][0];
  __syncthreads();
  for (int p = 0; p < TB; p += 2) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      double (&src)[TB][TB + 1] = h ? b : a;
      double (&dst)[TB][TB + 1] = h ? a : b;
      const int q = p + h;
      const double rp = rpiv[h];
      const double aiq = src[i][q], aqj = src[q][j];
      double v;
      if (i == q && j == q) v = rp;
      else if (i == q) v = aqj * rp;
      else if (j == q) v = -aiq * rp;
      else v = fma(-aiq, aqj * rp, src[i][j]);
      dst[i][j] = v;
      if (i == q + 1 && j == q + 1) rpiv[h ^ 1] = 1.0 / v;   // next pivot (q + 1 < TB here)
      __syncthreads();
    }
  }
}

// The coarsest matrix is SPD, so it is inverted with the block sweep operator,
// which keeps the matrix symmetric at every step (pivot block K, P = A_KK^-1):
//   A_KK <- -P,  A_KJ <- P A_KJ,  A_IK <- A_IK P,  A_IJ <- A_IJ - A_IK P A_KJ,
// ending with -A^-1.  Only blocks (ib <= jb) are kept up to date, which halves
// the rank-TB update flops of a plain Gauss-Jordan inverse and removes its
// column-panel product (A_IK P is the transpose of the row panel P A_KI).
// Two launches per pivot step:
//  (1) panel: every CTA jb inverts the pivot tile itself (no serial pivot
//      launch), saves the original panel tile X_J = A_KJ to Xb and writes
//      R_J = P X_J; CTA K writes P;
//  (2) update: D_IJ -= X_I^T R_J for ib <= jb off the pivot row/column, and
//      the panel row/column and the pivot tile are overwritten with R and -P
//      in the same launch (the update reads X from Xb, so no tile is read
//      and written by different CTAs of one launch); one CTA per tile of the
//      upper triangle.
// Pivot block 16, not 32: the step's critical path (pivot-tile inverse and
// panel product, TB^3 FP64 FMAs each on one SM) shrinks 8x while the update
// work per matrix stays n^3 / 2; on GB300's narrow FP64 pipe the 32-wide
// panel cost more than the update it precedes.
template <int TB>
__global__ void __launch_bounds__(TB * TB) k_sw_panel(const double* D, int64_t ld, int k,
                                                     double* P, double* R, double* Xb) {
  pdl_wait();
  pdl_trigger();
  __shared__ double a[TB][TB + 1], xs[TB][TB + 1], tb[TB][TB + 1];
  __shared__ double rpiv[2];
  const int jb = blockIdx.x;
  const int i = threadIdx.y, j = threadIdx.x;
  a[i][j] = D[(int64_t)(k * TB + i) * ld + k * TB + j];
  if (jb != k) {
    if (k < jb) xs[i][j] = D[(int64_t)(k * TB + i) * ld + jb * TB + j];
    else xs[j][i] = D[(int64_t)(jb * TB + i) * ld + k * TB + j];   // coalesced, transposed in smem
  }
  __syncthreads();
  gj_tile_inverse<TB>(a, tb, rpiv, i, j);
  if (jb == k) {
    P[i * TB + j] = a[i][j];
    return;
  }
  double acc = 0.0;
#pragma unroll
  for (int m = 0; m < TB; ++m) acc = fma(a[i][m], xs[m][j], acc);
  R[(int64_t)i * ld + jb * TB + j] = acc;
  Xb[(int64_t)i * ld + jb * TB + j] = xs[i][j];
}

// upper-triangle tile of linear index t, column by column: (ib, jb), ib <= jb
// (FP32 estimate, corrected exactly in integers: an FP64 sqrt per thread would
// cost more on GB300's narrow FP64 pipe than the tile's own FMAs)
__device__ __forceinline__ void tri_tile(int t, int& ib, int& jb) {
  int c = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  c = max(c, 0);
  while (c * (c + 1) / 2 > t) --c;
  while ((c + 1) * (c + 2) / 2 <= t) ++c;
  jb = c;
  ib = t - c * (c + 1) / 2;
}

template <int TB>
__global__ void __launch_bounds__(TB * TB) k_sw_update(double* D, int64_t ld, int k,
                                                      const double* P, const double* R,
                                                      const double* Xb) {
  pdl_wait();
  pdl_trigger();
  int ib, jb;
  tri_tile(blockIdx.x, ib, jb);
  const int i = threadIdx.y, j = threadIdx.x;
  if (ib == k && jb == k) {                       // pivot tile <- -P
    D[(int64_t)(k * TB + i) * ld + k * TB + j] = -P[i * TB + j];
    return;
  }
  if (ib == k) {                                  // panel row (upper orientation) <- R_J
    D[(int64_t)(k * TB + i) * ld + jb * TB + j] = R[(int64_t)i * ld + jb * TB + j];
    return;
  }
  __shared__ double xs[TB][TB + 1], rs[TB][TB + 1];
  if (jb == k) {                                  // panel column (ib < k) <- R_I^T
    rs[i][j] = R[(int64_t)i * ld + ib * TB + j];
    __syncthreads();
    D[(int64_t)(ib * TB + i) * ld + k * TB + j] = rs[j][i];
    return;
  }
  xs[i][j] = Xb[(int64_t)i * ld + ib * TB + j];   // X_I[m = i][c = j]
  rs[i][j] = R[(int64_t)i * ld + jb * TB + j];
  __syncthreads();
  double acc = 0.0;
#pragma unroll
  for (int m = 0; m < TB; ++m) acc = fma(xs[m][i], rs[m][j], acc);
  D[(int64_t)(ib * TB + i) * ld + jb * TB + j] -= acc;
}
// D <- -D on the upper blocks, mirrored into the lower ones: the full A^-1
// (GJB is a multiple of SWB)
__global__ void __launch_bounds__(GJB * GJB) k_sw_mirror(double* D, int64_t ld) {
  pdl_wait();
  pdl_trigger();
  const int ib = blockIdx.y, jb = blockIdx.x;
  if (ib > jb) return;
  __shared__ double ts[GJB][GJB + 1];
  const int i = threadIdx.y, j = threadIdx.x;
  const double v = -D[(int64_t)(ib * GJB + i) * ld + jb * GJB + j];
  ts[i][j] = v;
  __syncthreads();
  if (ib == jb) {
    // the sweep keeps only pivot-block tiles with row block <= column block up
    // to date: below them take the transpose, on them enforce exact symmetry
    const int ri = i / SWB, cj = j / SWB;
    const double w = ri > cj ? ts[j][i] : (ri < cj ? v : 0.5 * (v + ts[j][i]));
    D[(int64_t)(ib * GJB + i) * ld + jb * GJB + j] = w;
  } else {
    D[(int64_t)(ib * GJB + i) * ld + jb * GJB + j] = v;
    D[(int64_t)(jb * GJB + i) * ld + ib * GJB + j] = ts[j][i];
  }
}

void gj_inverse(double* D, int64_t n, int64_t ld, double* work, cudaStream_t st) {
  TG_REQUIRE(ld % GJB == 0, "dense leading dimension must be a multiple of 32");
  const int nb = (int)(ld / SWB);
  double* P = work;                  // SWB*SWB
  double* R = work + SWB * SWB;      // SWB*ld
  double* Xb = R + SWB * ld;         // SWB*ld
  const dim3 thr(SWB, SWB);
  const unsigned tiles = (unsigned)(nb * (nb + 1) / 2);
  for (int k = 0; k < nb; ++k) {
    launch_pdl(k_sw_panel<SWB>, dim3(nb), thr, 0, st, (const double*)D, ld, k, P, R, Xb);
    launch_pdl(k_sw_update<SWB>, dim3(tiles), thr, 0, st, D, ld, k, (const double*)P, (const double*)R, (const double*)Xb);
  }
  const int nm = (int)(ld / GJB);
  launch_pdl(k_sw_mirror, dim3(nm, nm), dim3(GJB, GJB), 0, st, D, ld);
  count_launches(2 * (int64_t)nb);   // + the mirror, counted below
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// the same block sweep in double-word arithmetic on the FP32 pipes
// ---------------------------------------------------------------------------
// GB300 issues about 2 FP64 FMAs per SM per clock against 128 FP32 ones.  A
// double-word number is the unevaluated sum h + l of two FP32 numbers (about
// 48 significant bits); its error-free building blocks are Knuth's TwoSum,
// Dekker's FastTwoSum and the FMA-based TwoProd, and the accurate DW + DW
// and DW x DW of Joldes, Muller and Popescu, "Tight and rigorous error bounds
// for basic building blocks of double-word arithmetic" (ACM TOMS 44, 2017,
// Algorithms 6 and 12).  The update's 16-term sums follow the compensated
// dot product of Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM
// J. Sci. Comput. 26, 2005), extended by the cross terms of DW operands.
// Every operation is an explicit round-to-nearest intrinsic, so none is
// contracted into an FMA.  A matrix element is a float2 (h, l) in the same
// 8 bytes as the FP64 element it replaces.
struct DW {
  float h, l;
};
__device__ __forceinline__ DW two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DW fast_two_sum(float a, float b) {   // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DW dw_add(DW x, DW y) {
  const DW s = two_sum(x.h, y.h);
  const DW t = two_sum(x.l, y.l);
  const DW v = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
  return fast_two_sum(v.h, __fadd_rn(t.l, v.l));
}
__device__ __forceinline__ DW dw_neg(DW x) { return {-x.h, -x.l}; }
__device__ __forceinline__ DW dw_mul(DW x, DW y) {
  const float ch = __fmul_rn(x.h, y.h);
  const float cl1 = __fmaf_rn(x.h, y.h, -ch);
  const float tl1 = __fmaf_rn(x.h, y.l, __fmul_rn(x.l, y.l));
  const float cl2 = __fmaf_rn(x.l, y.h, tl1);
  return fast_two_sum(ch, __fadd_rn(cl1, cl2));
}
// 1 / a: the correctly rounded FP32 reciprocal r0 of a.h, then one Newton
// step r0 + r0 (1 - a r0) with the residual 1 - a r0 formed in DW
__device__ __forceinline__ DW dw_rcp(DW a) {
  const float r0 = __frcp_rn(a.h);
  const DW p = dw_mul(a, DW{r0, 0.f});
  const DW e = dw_add(DW{1.f, 0.f}, dw_neg(p));
  return fast_two_sum(r0, __fmul_rn(r0, __fadd_rn(e.h, e.l)));
}
// compensated sum of products: (sh, sl) += x y
__device__ __forceinline__ void dw_dot_step(float& sh, float& sl, DW x, DW y) {
  const float p = __fmul_rn(x.h, y.h);
  float pe = __fmaf_rn(x.h, y.h, -p);
  pe = __fmaf_rn(x.h, y.l, pe);
  pe = __fmaf_rn(x.l, y.h, pe);
  const DW s = two_sum(sh, p);
  sh = s.h;
  sl = __fadd_rn(sl, __fadd_rn(s.l, pe));
}
__device__ __forceinline__ DW ld_dw(const float2* p) {
  const float2 v = *p;
  return {v.x, v.y};
}
__device__ __forceinline__ void st_dw(float2* p, DW v) { *p = make_float2(v.h, v.l); }

// gj_tile_inverse in DW (same step structure and barriers)
template <int TB>
__device__ __forceinline__ void dw_tile_inverse(float2 (&a)[TB][TB + 1], float2 (&b)[TB][TB + 1],
                                                DW (&rpiv)[2], int i, int j) {
  if (i == 0 && j == 0) rpiv[0] = dw_rcp(ld_dw(&a[0][0]));
  __syncthreads();
  for (int p = 0; p < TB; p += 2) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float2 (&src)[TB][TB + 1] = h ? b : a;
      float2 (&dst)[TB][TB + 1] = h ? a : b;
      const int q = p + h;
      const DW rp = rpiv[h];
      const DW aiq = ld_dw(&src[i][q]), aqj = ld_dw(&src[q][j]);
      DW v;
      if (i == q && j == q) v = rp;
      else if (i == q) v = dw_mul(aqj, rp);
      else if (j == q) v = dw_neg(dw_mul(aiq, rp));
      else v = dw_add(ld_dw(&src[i][j]), dw_neg(dw_mul(aiq, dw_mul(aqj, rp))));
      st_dw(&dst[i][j], v);
      if (i == q + 1 && j == q + 1) rpiv[h ^ 1] = dw_rcp(v);
      __syncthreads();
    }
  }
}

// k_sw_panel / k_sw_update in DW on float2 storage
template <int TB>
__global__ void __launch_bounds__(TB * TB) k_dw_panel(const float2* D, int64_t ld, int k,
                                                     float2* P, float2* R, float2* Xb) {
  pdl_wait();
  pdl_trigger();
  __shared__ float2 a[TB][TB + 1], xs[TB][TB + 1], tb[TB][TB + 1];
  __shared__ DW rpiv[2];
  const int jb = blockIdx.x;
  const int i = threadIdx.y, j = threadIdx.x;
  a[i][j] = D[(int64_t)(k * TB + i) * ld + k * TB + j];
  if (jb != k) {
    if (k < jb) xs[i][j] = D[(int64_t)(k * TB + i) * ld + jb * TB + j];
    else xs[j][i] = D[(int64_t)(jb * TB + i) * ld + k * TB + j];
  }
  __syncthreads();
  dw_tile_inverse<TB>(a, tb, rpiv, i, j);
  if (jb == k) {
    P[i * TB + j] = a[i][j];
    return;
  }
  float sh = 0.f, sl = 0.f;
#pragma unroll
  for (int m = 0; m < TB; ++m) dw_dot_step(sh, sl, ld_dw(&a[i][m]), ld_dw(&xs[m][j]));
  st_dw(&R[(int64_t)i * ld + jb * TB + j], two_sum(sh, sl));
  Xb[(int64_t)i * ld + jb * TB + j] = xs[i][j];
}

template <int TB>
__global__ void __launch_bounds__(TB * TB) k_dw_update(float2* D, int64_t ld, int k,
                                                      const float2* P, const float2* R,
                                                      const float2* Xb) {
  pdl_wait();
  pdl_trigger();
  int ib, jb;
  tri_tile(blockIdx.x, ib, jb);
  const int i = threadIdx.y, j = threadIdx.x;
  if (ib == k && jb == k) {
    const float2 v = P[i * TB + j];
    D[(int64_t)(k * TB + i) * ld + k * TB + j] = make_float2(-v.x, -v.y);
    return;
  }
  if (ib == k) {
    D[(int64_t)(k * TB + i) * ld + jb * TB + j] = R[(int64_t)i * ld + jb * TB + j];
    return;
  }
  __shared__ float2 xs[TB][TB + 1], rs[TB][TB + 1];
  if (jb == k) {
    rs[i][j] = R[(int64_t)i * ld + ib * TB + j];
    __syncthreads();
    D[(int64_t)(ib * TB + i) * ld + k * TB + j] = rs[j][i];
    return;
  }
  xs[i][j] = Xb[(int64_t)i * ld + ib * TB + j];
  rs[i][j] = R[(int64_t)i * ld + jb * TB + j];
  __syncthreads();
  float sh = 0.f, sl = 0.f;
#pragma unroll
  for (int m = 0; m < TB; ++m) dw_dot_step(sh, sl, ld_dw(&xs[m][i]), ld_dw(&rs[m][j]));
  float2* d = D + (int64_t)(ib * TB + i) * ld + jb * TB + j;
  st_dw(d, dw_add(ld_dw(d), dw_neg(two_sum(sh, sl))));
}

// Step k of the sweep together with step k+1's panel (look-ahead), one
// launch: the first nb CTAs form panel column J of pivot block K = k+1 from
// the matrix as step k leaves it -- the pivot tile and tile (K, J), each
// updated in the CTA by the same double-word expression k_dw_update applies
// (tile (K, k) is step k's R) --, invert the pivot tile and write P, R, Xb of
// step K into the other buffer; the other CTAs update the upper tiles as
// k_dw_update does, except those of row / column K, which step K overwrites
// anyway.  Same values as the two-launch sweep; the panel's serial chain
// (pivot-tile inverse) runs beside the update instead of after it.
template <int TB>
__global__ void __launch_bounds__(TB * TB) k_dw_update_la(float2* D, int64_t ld, int k, int nb,
                                                         const float2* P, const float2* R,
                                                         const float2* Xb, float2* Pn, float2* Rn,
                                                         float2* Xbn) {
  pdl_wait();
  pdl_trigger();
  const int i = threadIdx.y, j = threadIdx.x;
  const int K = k + 1;
  __shared__ float2 xs[TB][TB + 1], rs[TB][TB + 1];
  if ((int)blockIdx.x < nb) {
    __shared__ float2 a[TB][TB + 1], tb[TB][TB + 1], xk[TB][TB + 1], ys[TB][TB + 1];
    __shared__ DW rpiv[2];
    const int J = blockIdx.x;
    // X_K and R_K of step k (k_dw_update's xs / rs for block K)
    xs[i][j] = Xb[(int64_t)i * ld + K * TB + j];
    rs[i][j] = R[(int64_t)i * ld + K * TB + j];
    if (J != K && J != k) ys[i][j] = (K < J) ? R[(int64_t)i * ld + J * TB + j]     // R_J
                                             : Xb[(int64_t)i * ld + J * TB + j];   // X_J
    __syncthreads();
    {
      // pivot tile (K, K) after step k
      float sh = 0.f, sl = 0.f;
#pragma unroll
      for (int m = 0; m < TB; ++m) dw_dot_step(sh, sl, ld_dw(&xs[m][i]), ld_dw(&rs[m][j]));
      const float2* d = D + (int64_t)(K * TB + i) * ld + K * TB + j;
      st_dw(&a[i][j], dw_add(ld_dw(d), dw_neg(two_sum(sh, sl))));
    }
    if (J == k) {
      // tile (k, K) is step k's R at block K: A'(K*TB+i, k*TB+j) = R[j][K*TB+i]
      xk[i][j] = R[(int64_t)j * ld + K * TB + i];
    } else if (K < J) {
      // tile (K, J) after step k
      float sh = 0.f, sl = 0.f;
#pragma unroll
      for (int m = 0; m < TB; ++m) dw_dot_step(sh, sl, ld_dw(&xs[m][i]), ld_dw(&ys[m][j]));
      const float2* d = D + (int64_t)(K * TB + i) * ld + J * TB + j;
      st_dw(&xk[i][j], dw_add(ld_dw(d), dw_neg(two_sum(sh, sl))));
    } else if (J < K) {
      // tile (J, K) after step k, element (j, i) of the upper tile
      float sh = 0.f, sl = 0.f;
#pragma unroll
      for (int m = 0; m < TB; ++m) dw_dot_step(sh, sl, ld_dw(&ys[m][j]), ld_dw(&rs[m][i]));
      const float2* d = D + (int64_t)(J * TB + j) * ld + K * TB + i;
      st_dw(&xk[i][j], dw_add(ld_dw(d), dw_neg(two_sum(sh, sl))));
    }
    __syncthreads();
    dw_tile_inverse<TB>(a, tb, rpiv, i, j);
    if (J == K) {
      Pn[i * TB + j] = a[i][j];
      return;
    }
    float sh = 0.f, sl = 0.f;
#pragma unroll
    for (int m = 0; m < TB; ++m) dw_dot_step(sh, sl, ld_dw(&a[i][m]), ld_dw(&xk[m][j]));
    st_dw(&Rn[(int64_t)i * ld + J * TB + j], two_sum(sh, sl));
    Xbn[(int64_t)i * ld + J * TB + j] = xk[i][j];
    return;
  }
  int ib, jb;
  tri_tile((int)blockIdx.x - nb, ib, jb);
  if (ib == K || jb == K) return;
  if (ib == k && jb == k) {
    const float2 v = P[i * TB + j];
    D[(int64_t)(k * TB + i) * ld + k * TB + j] = make_float2(-v.x, -v.y);
    return;
  }
  if (ib == k) {
    D[(int64_t)(k * TB + i) * ld + jb * TB + j] = R[(int64_t)i * ld + jb * TB + j];
    return;
  }
  if (jb == k) {
    rs[i][j] = R[(int64_t)i * ld + ib * TB + j];
    __syncthreads();
    D[(int64_t)(ib * TB + i) * ld + k * TB + j] = rs[j][i];
    return;
  }
  xs[i][j] = Xb[(int64_t)i * ld + ib * TB + j];
  rs[i][j] = R[(int64_t)i * ld + jb * TB + j];
  __syncthreads();
  float sh = 0.f, sl = 0.f;
#pragma unroll
  for (int m = 0; m < TB; ++m) dw_dot_step(sh, sl, ld_dw(&xs[m][i]), ld_dw(&rs[m][j]));
  float2* d = D + (int64_t)(ib * TB + i) * ld + jb * TB + j;
  st_dw(d, dw_add(ld_dw(d), dw_neg(two_sum(sh, sl))));
}

// FP64 -> DW in place (h = the FP64 value rounded to FP32, l = the rounded rest)
__global__ void k_dw_split(double* D, int64_t n) {
  pdl_wait();
  pdl_trigger();
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const double v = D[e];
  const float h = __double2float_rn(v);
  const float l = __double2float_rn(v - (double)h);
  reinterpret_cast<float2*>(D)[e] = make_float2(h, l);
}
// k_sw_mirror reading DW and writing FP64 in place: each block reads only its
// own upper tile (before its barrier) and the lower tiles it writes are read
// by no block
__global__ void __launch_bounds__(GJB * GJB) k_dw_mirror(double* D, int64_t ld) {
  pdl_wait();
  pdl_trigger();
  const int ib = blockIdx.y, jb = blockIdx.x;
  if (ib > jb) return;
  __shared__ double ts[GJB][GJB + 1];
  const int i = threadIdx.y, j = threadIdx.x;
  const int64_t e = (int64_t)(ib * GJB + i) * ld + jb * GJB + j;
  const float2 f = reinterpret_cast<const float2*>(D)[e];
  const double v = -((double)f.x + (double)f.y);
  ts[i][j] = v;
  __syncthreads();
  if (ib == jb) {
    const int ri = i / SWB, cj = j / SWB;
    const double w = ri > cj ? ts[j][i] : (ri < cj ? v : 0.5 * (v + ts[j][i]));
    D[e] = w;
  } else {
    D[e] = v;
    D[(int64_t)(jb * GJB + i) * ld + ib * GJB + j] = ts[j][i];
  }
}

void gj_inverse_dw(double* D, int64_t n, int64_t ld, double* work, cudaStream_t st, bool lookahead) {
  TG_REQUIRE(ld % GJB == 0, "dense leading dimension must be a multiple of 32");
  const int nb = (int)(ld / SWB);
  float2* Df = reinterpret_cast<float2*>(D);
  // two (P, R, Xb) sets: the look-ahead writes step k+1's while step k reads its own
  const int64_t set = SWB * SWB + 2 * SWB * ld;
  float2* P[2];
  float2* R[2];
  float2* Xb[2];
  for (int b = 0; b < 2; ++b) {
    P[b] = reinterpret_cast<float2*>(work) + b * set;
    R[b] = P[b] + SWB * SWB;
    Xb[b] = R[b] + SWB * ld;
  }
  launch_pdl(k_dw_split, dim3((unsigned)cdiv(ld * ld, 256)), dim3(256), 0, st, D, ld * ld);
  const dim3 thr(SWB, SWB);
  const unsigned tiles = (unsigned)(nb * (nb + 1) / 2);
  if (lookahead) {
    launch_pdl(k_dw_panel<SWB>, dim3(nb), thr, 0, st, Df, ld, 0, P[0], R[0], Xb[0]);
    for (int k = 0; k + 1 < nb; ++k) {
      const int b = k & 1;
      launch_pdl(k_dw_update_la<SWB>, dim3(nb + tiles), thr, 0, st, Df, ld, k, nb,
                 (const float2*)P[b], (const float2*)R[b], (const float2*)Xb[b], P[b ^ 1], R[b ^ 1],
                 Xb[b ^ 1]);
    }
    const int b = (nb - 1) & 1;
    launch_pdl(k_dw_update<SWB>, dim3(tiles), thr, 0, st, Df, ld, nb - 1, (const float2*)P[b],
               (const float2*)R[b], (const float2*)Xb[b]);
    count_launches((int64_t)nb + 2);     // panel, nb - 1 fused steps, last update, split
  } else {
    for (int k = 0; k < nb; ++k) {
      launch_pdl(k_dw_panel<SWB>, dim3(nb), thr, 0, st, Df, ld, k, P[0], R[0], Xb[0]);
      launch_pdl(k_dw_update<SWB>, dim3(tiles), thr, 0, st, Df, ld, k, (const float2*)P[0],
                 (const float2*)R[0], (const float2*)Xb[0]);
    }
    count_launches(2 * (int64_t)nb + 1);   // and the split
  }
  const int nm = (int)(ld / GJB);
  launch_pdl(k_dw_mirror, dim3(nm, nm), dim3(GJB, GJB), 0, st, D, ld);
  TG_CHECK_LAUNCH();                     // the mirror
}

// x = Dinv b: a warp per (row, column chunk) writes a partial sum, a second
// kernel adds the DA_CHUNKS partials of a row in fixed order (deterministic;
// 8x the parallelism of a warp per row on the ~1200-row coarsest matrix).
// Fixed rows of Dinv hold the identity and b is 0 there.
constexpr int DA_CHUNKS = 8;
// one warp: the partial sum of row `row` over column chunk `chunk`
template <typename T, bool CG = false>
__device__ __forceinline__ void dense_partial_one(const double* __restrict__ Dinv, int64_t n,
                                                  int64_t ld, const T* __restrict__ b,
                                                  double* __restrict__ part, int64_t row,
                                                  int chunk, int lane) {
  const int64_t w = (n + DA_CHUNKS - 1) / DA_CHUNKS;
  const int64_t j0 = chunk * w, j1 = min(n, j0 + w);
  double acc = 0.0;
#pragma unroll 4
  for (int64_t j = j0 + lane; j < j1; j += 32) acc = fma(Dinv[row * ld + j], (double)ldv<CG>(b + j), acc);
  acc = warp_sum(acc);
  if (lane == 0) part[chunk * n + row] = acc;
}
template <typename T, bool CG = false>
__device__ __forceinline__ void dense_sum_one(const double* __restrict__ part, int64_t n,
                                              T* __restrict__ x, int64_t row) {
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < DA_CHUNKS; ++k) s += ldv<CG>(part + k * n + row);
  x[row] = (T)s;
}
// the same with the inverse stored in FP32 (the FP32 V-cycle of mixed
// contexts): half the bytes per cycle, FP32 products summed per lane in FP32,
// the warp and chunk sums in FP64
template <bool CG = false>
__device__ __forceinline__ void dense_partial32_one(const float* __restrict__ Dinv, int64_t n,
                                                    int64_t ld, const float* __restrict__ b,
                                                    double* __restrict__ part, int64_t row,
                                                    int chunk, int lane) {
  const int64_t w = (n + DA_CHUNKS - 1) / DA_CHUNKS;
  const int64_t j0 = chunk * w, j1 = min(n, j0 + w);
  float acc = 0.f;
#pragma unroll 4
  for (int64_t j = j0 + lane; j < j1; j += 32) acc = fmaf(Dinv[row * ld + j], ldv<CG>(b + j), acc);
  const double s = warp_sum((double)acc);
  if (lane == 0) part[chunk * n + row] = s;
}
template <typename T>
__global__ void __launch_bounds__(256) k_dense_partial(const double* __restrict__ Dinv, int64_t n,
                                                      int64_t ld, const T* __restrict__ b,
                                                      double* __restrict__ part) {
  pdl_wait();
  pdl_trigger();
  const int64_t row = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (row < n) dense_partial_one<T>(Dinv, n, ld, b, part, row, blockIdx.y, threadIdx.x & 31);
}
template <typename T>
__global__ void k_dense_sum(const double* __restrict__ part, int64_t n, T* __restrict__ x) {
  pdl_wait();
  pdl_trigger();
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row < n) dense_sum_one<T>(part, n, x, row);
}

template <typename T>
void dense_apply(const double* Dinv, int64_t n, int64_t ld, const T* b, T* x, double* work,
                 cudaStream_t st) {
  launch_pdl(k_dense_partial<T>, dim3(dim3((unsigned)cdiv(n, 8), DA_CHUNKS)), dim3(256), 0, st, Dinv, n, ld, b, work);
  TG_CHECK_LAUNCH();
  launch_pdl(k_dense_sum<T>, dim3((unsigned)cdiv(n, 256)), dim3(256), 0, st, work, n, x);
  TG_CHECK_LAUNCH();
}
template void dense_apply<double>(const double*, int64_t, int64_t, const double*, double*, double*, cudaStream_t);
template void dense_apply<float>(const double*, int64_t, int64_t, const float*, float*, double*, cudaStream_t);

__global__ void __launch_bounds__(256) k_dense_partial_f32(const float* __restrict__ Dinv, int64_t n,
                                                          int64_t ld, const float* __restrict__ b,
                                                          double* __restrict__ part) {
  pdl_wait();
  pdl_trigger();
  const int64_t row = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (row < n) dense_partial32_one<false>(Dinv, n, ld, b, part, row, blockIdx.y, threadIdx.x & 31);
}
void dense_apply(const float* Dinv, int64_t n, int64_t ld, const float* b, float* x, double* work,
                 cudaStream_t st) {
  launch_pdl(k_dense_partial_f32, dim3(dim3((unsigned)cdiv(n, 8), DA_CHUNKS)), dim3(256), 0, st, Dinv, n, ld, b, work);
  TG_CHECK_LAUNCH();
  launch_pdl(k_dense_sum<float>, dim3((unsigned)cdiv(n, 256)), dim3(256), 0, st, work, n, x);
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// the bottom of the V-cycle in one cooperative launch
// ---------------------------------------------------------------------------
// Every phase is a grid-stride loop over the same work units as the separate
// kernels (restrict_one, stencil_small_vb, dense_partial_one, dense_sum_one,
// prolong_one), so each value is computed in the same order as with those
// launches; grid_sync separates the phases.  One block per SM: the tail and
// coarsest levels are small (a few thousand rows), so the launch and drain of
// ~10 separate kernels per V-cycle, not their work, was the cost.
// phase barrier: the hardware cluster barrier (release / acquire at cluster
// scope) when the launch is one thread-block cluster, else the bounded grid
// barrier of a cooperative launch
template <bool CLUSTER>
__device__ __forceinline__ bool tail_sync(GridBar* bar) {
  if constexpr (CLUSTER) {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;"
                 ::: "memory");
    return true;
  } else {
    return grid_sync(bar);
  }
}

template <int NDIM, int NDOF, typename T, bool CLUSTER>
__global__ void __launch_bounds__(small_threads<NDIM>()) k_coarse_tail(TailArgs<T> a) {
  __shared__ T spart[small_split<NDIM>()][small_pairs<NDIM>()];
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t gsz = (int64_t)gridDim.x * blockDim.x;
  const int64_t rows_t = a.gt.nnodes() * NDOF;
  const int64_t nvb = cdiv(rows_t, small_pairs<NDIM>());
  auto sweep = [&](const T* in, T* out, int mode) {
    for (int64_t vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      if (mode == AM_JACOBI)
        stencil_small_vb<NDIM, NDOF, T, AM_JACOBI, true>(a.gt, a.At, in, out, a.bt, a.dinvt, a.omega, vb, spart);
      else
        stencil_small_vb<NDIM, NDOF, T, AM_RES, true>(a.gt, a.At, in, out, a.bt, a.dinvt, a.omega, vb, spart);
    }
  };
  // restriction into the tail level with its first step from zero (t = omega D^-1 b)
  for (int64_t t = gtid; t < rows_t; t += gsz)
    restrict_one<NDIM, NDOF, T, true>(a.gp, a.gt, a.fixt, a.rp, a.bt, a.dinvt, a.tt, a.omega, t);
  if (!tail_sync<CLUSTER>(a.bar)) return;
  T* bufs[2] = {a.xt, a.tt};
  int cur = 1;
  for (int s = 1; s < a.nsmooth; ++s) {
    sweep(bufs[cur], bufs[1 - cur], AM_JACOBI);
    cur = 1 - cur;
    if (!tail_sync<CLUSTER>(a.bar)) return;
  }
  sweep(bufs[cur], a.rt, AM_RES);
  if (!tail_sync<CLUSTER>(a.bar)) return;
  // restriction to the coarsest level
  const int64_t rows_c = a.gc.nnodes() * NDOF;
  for (int64_t t = gtid; t < rows_c; t += gsz)
    restrict_one<NDIM, NDOF, T, true>(a.gt, a.gc, a.fixc, a.rt, a.bc, nullptr, nullptr, T(0), t);
  if (!tail_sync<CLUSTER>(a.bar)) return;
  // coarsest solve: a warp per (row, column chunk), then the fixed-order sums
  {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = gtid >> 5, nw = gsz >> 5;
    for (int64_t w = w0; w < a.nc * DA_CHUNKS; w += nw) {
      if constexpr (std::is_same<T, float>::value) {
        if (a.Dc32) {
          dense_partial32_one<true>(a.Dc32, a.nc, a.ldc, a.bc, a.part, w % a.nc, (int)(w / a.nc), lane);
          continue;
        }
      }
      dense_partial_one<T, true>(a.Dc, a.nc, a.ldc, a.bc, a.part, w % a.nc, (int)(w / a.nc), lane);
    }
  }
  if (!tail_sync<CLUSTER>(a.bar)) return;
  for (int64_t r = gtid; r < a.nc; r += gsz) dense_sum_one<T, true>(a.part, a.nc, a.xc, r);
  if (!tail_sync<CLUSTER>(a.bar)) return;
  for (int64_t i = gtid; i < a.gt.nnodes(); i += gsz)
    prolong_one<NDIM, NDOF, T, true>(a.gt, a.gc, a.fixt, a.xc, bufs[cur], i);
  if (!tail_sync<CLUSTER>(a.bar)) return;
  for (int s = 0; s < a.nsmooth; ++s) {
    sweep(bufs[cur], bufs[1 - cur], AM_JACOBI);
    cur = 1 - cur;
    if (!tail_sync<CLUSTER>(a.bar)) return;
  }
  // the tail level's result (ends in xt for an even number of steps; the
  // parent reads bufs[cur])
  for (int64_t i = gtid; i < a.gp.nnodes(); i += gsz)
    prolong_one<NDIM, NDOF, T, true>(a.gp, a.gt, a.fixp, bufs[cur], a.xp, i);
}

template <typename T>
void coarse_tail(const TailArgs<T>& a, cudaStream_t st) {
  TG_REQUIRE(a.gt.nnodes() * a.gt.ndof <= TAIL_MAX_PAIRS, "coarse_tail: tail level too large");
  TG_REQUIRE(a.nsmooth >= 1, "coarse_tail: nsmooth >= 1");
  TG_REQUIRE(a.gc.ndofs() == a.nc && a.ldc >= a.nc, "coarse_tail: coarsest matrix size");
  int dev = 0, nsm = 0;
  TG_CUDA(cudaGetDevice(&dev));
  TG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const bool cl = a.cluster > 0;
  const void* fn = nullptr;
  int slot = 0;
  switch (a.gt.ndim * 10 + a.gt.ndof) {
    case 33: fn = cl ? (const void*)k_coarse_tail<3, 3, T, true> : (const void*)k_coarse_tail<3, 3, T, false>; slot = 0; break;
    case 31: fn = cl ? (const void*)k_coarse_tail<3, 1, T, true> : (const void*)k_coarse_tail<3, 1, T, false>; slot = 1; break;
    case 22: fn = cl ? (const void*)k_coarse_tail<2, 2, T, true> : (const void*)k_coarse_tail<2, 2, T, false>; slot = 2; break;
    case 21: fn = cl ? (const void*)k_coarse_tail<2, 1, T, true> : (const void*)k_coarse_tail<2, 1, T, false>; slot = 3; break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof)"};
  }
  cudaLaunchConfig_t cfg = {};
  const int nthr = a.gt.ndim == 3 ? small_threads<3>() : small_threads<2>();
  cfg.blockDim = dim3((unsigned)nthr);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cl) {
    // one cluster of 16 CTAs (non-portable size) where the GPU can place it, else 8
    static std::atomic<int> csize[4] = {};
    int cs = csize[slot].load(std::memory_order_relaxed);
    if (!cs) {
      TG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      for (cs = 16; cs >= 2; cs /= 2) {
        cfg.gridDim = dim3((unsigned)cs);
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) == cudaSuccess && nclusters >= 1)
          break;
        (void)cudaGetLastError();
      }
      TG_REQUIRE(cs >= 2, "coarse_tail: no thread-block cluster fits");
      csize[slot].store(cs, std::memory_order_relaxed);
    }
    cs = std::min(cs, a.cluster);
    cfg.gridDim = dim3((unsigned)cs);
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
  } else {
    static std::atomic<int> fits[4] = {};      // resident blocks per SM, found once per variant
    int per_sm = fits[slot].load(std::memory_order_relaxed);
    if (!per_sm) {
      TG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, nthr, 0));
      TG_REQUIRE(per_sm >= 1, "coarse_tail: kernel does not fit on an SM");
      fits[slot].store(per_sm, std::memory_order_relaxed);
    }
    if (tune_take_tail_barrier_timeout()) {
      // the first barrier waits for one block more than the grid holds (the
      // same count OC's bounded-wait test uses), so every wait runs out
      static const unsigned int big = 0x40000000u;
      TG_CUDA(cudaMemcpyAsync(&a.bar->count, &big, sizeof(big), cudaMemcpyHostToDevice, st));
    }
    // all blocks co-resident (the cooperative launch refuses more)
    cfg.gridDim = dim3((unsigned)std::min(a.blocks > 0 ? a.blocks : nsm, nsm * per_sm));
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
  }
  TailArgs<T> args = a;
  void* kargs[] = {(void*)&args};
  TG_CUDA(cudaLaunchKernelExC(&cfg, fn, kargs));
  TG_CHECK_LAUNCH();
}
template void coarse_tail<float>(const TailArgs<float>&, cudaStream_t);
template void coarse_tail<double>(const TailArgs<double>&, cudaStream_t);

}  // namespace tg
