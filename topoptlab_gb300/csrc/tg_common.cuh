// Shared definitions for the GB300 SIMP compliance library (sm_103a).
//
// Data layout in HBM (the reference's own numbering, so host<->device copies
// are plain memcpys and edofMat parity is structural):
//   node (x, y, z)    -> ((z * nnx) + x) * nny + y          (y fastest)
//   DOF  (node, c)    -> node * ndof + c
//   element (x, y, z) -> ((z * nex) + x) * ney + y
// (elements/bilinear_quadrilateral.py:41-47, trilinear_hexahedron.py:45-57,
//  filter/matrix_filter.py:178-183).  In 2-D z = 0 and nnz = nez = 1.
//
// Dirichlet conditions: one byte per node, bit c set when DOF c is fixed.
// Every operator works on all DOFs with fixed rows and columns zeroed
// (A = M K M, M the 0/1 mask of free DOFs); every vector is kept zero on
// fixed DOFs.
#pragma once
#include <cuda_runtime.h>
#include <utility>
#include <vector>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string>

namespace tg {

struct Grid {
  int ndim;              // 2 or 3
  int ndof;              // DOFs per node (1, 2, 3)
  int nex, ney, nez;     // elements per axis (nez = 1 in 2-D)
  int nnx, nny, nnz;     // nodes per axis (nnz = 1 in 2-D)
  __host__ __device__ int64_t nnodes() const { return (int64_t)nnx * nny * nnz; }
  // stride between the coefficient arrays of an assembled stencil: nnodes
  // rounded up to 32, so every array starts 128-byte aligned (TMA copies)
  __host__ __device__ int64_t slds() const { return (nnodes() + 31) / 32 * 32; }
  __host__ __device__ int64_t ndofs() const { return nnodes() * ndof; }
  __host__ __device__ int64_t nel() const { return (int64_t)nex * ney * nez; }
  __host__ __device__ int64_t node(int x, int y, int z) const {
    return ((int64_t)z * nnx + x) * nny + y;
  }
  __host__ __device__ int64_t elem(int x, int y, int z) const {
    return ((int64_t)z * nex + x) * ney + y;
  }
};

inline Grid make_grid(int ndim, int ndof, int nex, int ney, int nez) {
  Grid g;
  g.ndim = ndim; g.ndof = ndof;
  g.nex = nex; g.ney = ney; g.nez = (ndim == 3) ? nez : 1;
  g.nnx = nex + 1; g.nny = ney + 1; g.nnz = (ndim == 3) ? nez + 1 : 1;
  return g;
}

inline Grid coarsen(const Grid& f) {
  return make_grid(f.ndim, f.ndof, f.nex / 2, f.ney / 2, f.ndim == 3 ? f.nez / 2 : 1);
}

// Status codes shared with the C ABI.
enum : int {
  OK = 0, EINVAL_ = 1, ENOTCONV = 2, ETIMEOUT = 3, ENAN = 4, ECUDA = 5, ENOMEM_ = 6
};

struct Error {
  int code;
  std::string msg;
};

#define TG_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess)                                                   \
      throw ::tg::Error{::tg::ECUDA, std::string(#call) + ": " +             \
                                         cudaGetErrorString(_e)};            \
  } while (0)

// Every kernel launch of the library goes through TG_CHECK_LAUNCH (or
// count_launches for loops), which also counts launches for the bench's
// gpu_launches figure.
void count_launches(int64_t n);
// Raise a kernel's dynamic shared-memory limit to `bytes` on the current
// device, once per (kernel, device): the attribute belongs to the device that
// is current when it is set, and contexts may live on different devices.
void set_smem_limit(const void* func, int bytes);
#define TG_CHECK_LAUNCH()                 \
  do {                                    \
    ::tg::count_launches(1);              \
    TG_CUDA(cudaGetLastError());          \
  } while (0)

// Programmatic dependent launch for the small kernels of the PCG iteration:
// launched with launch_pdl, a kernel may be scheduled while its predecessor
// on the stream still runs (once every block of the predecessor has passed
// pdl_trigger), which hides the launch and block ramp-up between dependent
// kernels.  Every kernel launched this way calls pdl_wait() first, in every
// thread, before any global memory access: it returns once the predecessor
// grid has completed and its writes are visible, so the stream order of the
// data is unchanged.  Both are no-ops for a kernel launched normally.
bool pdl_on();            // tg_tune(TG_TUNE_PDL) (default on) and the calling thread's scope
// the calling thread's scope: the library turns programmatic dependent launch
// off while it works for an FP64 context (its long FP64 kernels gain nothing,
// and blocks parked early cost concurrently stepped designs SM slots);
// returns the previous setting
int pdl_scope(int on);
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <typename... ExpTypes, typename... ActTypes>
inline void launch_pdl(void (*kernel)(ExpTypes...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t st, ActTypes&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_on() ? 1 : 0;
  TG_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<ActTypes>(args)...));
}

// Optional event timing of one kernel family (see tg_profile_kernel):
// prof_begin/prof_end bracket the launches of family `kind` on stream st.
// Families are disjoint; a composite region (e.g. the coarsest inverse) is
// timed as a whole.
enum ProfKind : int {
  PK_NONE = 0, PK_FINE_F64 = 1, PK_FINE_F32 = 2, PK_FINE_BF16 = 3,
  PK_STENCIL_F32 = 4,     // coarse stencil sweeps, FP32, levels >= 2
  PK_STENCIL_F64 = 5, PK_FILTER = 6, PK_OC = 7,
  PK_STENCIL1_F32 = 8,    // coarse stencil sweeps, FP32, level 1
  PK_COARSE_BUILD = 9,    // level operators, diagonals, dense coarsest matrix
  PK_COARSE_INV = 10,     // coarsest dense inverse
  PK_VECTOR = 11,         // PCG / refinement vector kernels and reductions
  PK_TRANSFER = 12,       // restriction, prolongation, coarsest dense apply
  PK_COMPLIANCE = 13,     // compliance and sensitivities
  PK_LEARNED = 14,        // learned warm start inference
  PK_TAIL = 15,           // the V-cycle's bottom levels in one cooperative launch
  PK_NKINDS = 16
};
void prof_begin(int kind, cudaStream_t st);
void prof_end(int kind, cudaStream_t st);
int prof_kind();              // family being timed (PK_NONE when off)
// brackets the enclosed launches of family k (no nesting of one family)
struct ProfScope {
  int k;
  cudaStream_t s;
  ProfScope(int k_, cudaStream_t s_) : k(k_), s(s_) { prof_begin(k, s); }
  ~ProfScope() {
    try {
      prof_end(k, s);
    } catch (...) {
    }
  }
  ProfScope(const ProfScope&) = delete;
  ProfScope& operator=(const ProfScope&) = delete;
};
// Event pairs recorded while a CUDA graph is captured: they become event
// nodes of the graph and are read after every replay (device time of the
// family inside the graph, without the host launch gaps of direct launches).
struct ProfCapture {
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pairs;
  cudaEvent_t open = nullptr;
  int kind = 0;
  void release();
  ~ProfCapture() { release(); }
};
void prof_capture_begin(ProfCapture* pc);   // prof_begin/end now record into pc
void prof_capture_end();
void prof_collect(const ProfCapture& pc);   // after a replay has completed
int64_t launch_count();       // kernels launched so far
// Library-wide switches set through tg_tune (include/topopt_gb300.h):
// the (row, node) pair count below which coarse stencils use the small-grid
// kernel, and a one-shot request that the next OC bisection's grid barrier
// wait for one block more than its grid holds (its bounded wait runs out).
int64_t tune_stencil_small_pairs();
bool tune_take_oc_barrier_timeout();
// the V-cycle's bottom (the last smoothed level and the coarsest solve) as
// one cooperative launch (default off: on GB300 its nine grid barriers cost
// more than the ten separate launches they replace inside the PCG graph),
// and the one-shot barrier-timeout request for its next launch
int tune_coarse_tail();   // 0 off, 1 one cluster, 2 cooperative (one block per SM), > 2 that many blocks
bool tune_take_tail_barrier_timeout();
bool tune_conv_umma();           // warm-start inference convolutions on tcgen05 (default on)
bool tune_take_conv_timeout();   // one-shot: the next tcgen05 convolution's waits run out

#define TG_REQUIRE(cond, msg)                                                \
  do {                                                                       \
    if (!(cond)) throw ::tg::Error{::tg::EINVAL_, (msg)};                    \
  } while (0)

__host__ __device__ inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// type helpers
// ---------------------------------------------------------------------------
template <typename S> __device__ __forceinline__ float to_f(S v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}
template <typename T, typename S> __device__ __forceinline__ T load_scale(const S* p, int64_t i);
template <> __device__ __forceinline__ double load_scale<double, double>(const double* p, int64_t i) {
  return __ldg(p + i);
}
template <> __device__ __forceinline__ float load_scale<float, float>(const float* p, int64_t i) {
  return __ldg(p + i);
}
template <> __device__ __forceinline__ float load_scale<float, __nv_bfloat16>(const __nv_bfloat16* p,
                                                                            int64_t i) {
  return __bfloat162float(p[i]);
}

// ---------------------------------------------------------------------------
// deterministic block reductions (fixed shuffle tree, fixed partial order)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
// result valid in thread 0; blockDim.x must be a multiple of 32, <= 1024
__device__ inline double block_sum(double v, double* sh /* >= 32 */) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  return v;
}
__device__ inline double block_max(double v, double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_max(v);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : -1.0e308;
  if (w == 0) v = warp_max(v);
  __syncthreads();
  return v;
}

// sum of nb per-block partials in fixed order (bypassing L1: other blocks
// wrote them); result valid in thread 0
__device__ inline double sum_partials(const double* part, int nb, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v += __ldcg(part + i);
  return block_sum(v, sh);
}

// Grid-wide barrier of a cooperative launch (all blocks co-resident):
// arrival count plus a generation number.  Every wait is bounded: a block that
// polls about 2^22 times (a fraction of a second) without the generation
// moving, or that sees another block's error, records the error flag and
// returns false; callers then leave the kernel and the host reports
// TG_ETIMEOUT.  count and err start at zero.
struct GridBar {
  unsigned int count, gen;
  int err;
};
__device__ __forceinline__ bool grid_sync(GridBar* b) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
    const unsigned int g = *(volatile unsigned int*)&b->gen;
    __threadfence();
    if (atomicAdd(&b->count, 1u) == nb - 1) {
      atomicExch(&b->count, 0u);
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      unsigned int polls = 0;
      while (*(volatile unsigned int*)&b->gen == g) {
        if (*(volatile int*)&b->err != 0 || ++polls > (1u << 22)) {
          atomicExch(&b->err, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// mbarrier helpers: the shared-window address of a shared-memory pointer, the
// global nanosecond timer, and a parity wait that gives up after limit_ns
// (false: the phase did not complete in time).
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  const uint32_t a = smem_u32(bar);
  const uint64_t t0 = global_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(a), "r"(parity) : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// Number of partial-sum slots used by every grid-wide reduction.  Grids that
// reduce are launched with at most this many blocks (grid-stride loops), so
// the summation order depends only on the problem size, never on timing.
constexpr int RED_BLOCKS = 1216;   // 8 per SM on 152 SMs
constexpr int RED_THREADS = 256;
inline unsigned red_blocks(int64_t n) {
  const int64_t b = cdiv(n, RED_THREADS);
  return (unsigned)(b < RED_BLOCKS ? (b < 1 ? 1 : b) : RED_BLOCKS);
}

}  // namespace tg
