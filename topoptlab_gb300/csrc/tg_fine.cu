// Fine-level matrix-free SIMP operator y = M K(rho) M u on structured quad4 /
// hex8 grids, its inverse diagonal, and the fused compliance + sensitivity.
//
// Replaces the reference's per-iteration  Kes = KE*simp(xPhys)  +  COO->CSC
// assembly + Dirichlet slicing + CSR SpMV (topology_optimization.py:419-451,
// fem.py:141-237, linear_solvers.py:130) and the compliance / sensitivity
// gathers (objectives.py:51-55, topology_optimization.py:491-500).
//
// Design (GB300).  3-D: k_fine_zstream -- a CTA owns a 15 x 15 column of
// nodes and a chunk of z planes (as many chunks as make one wave of resident
// CTAs); its 256 threads are the 16 x 16 elements touching the column; node
// planes stream through a 3-plane shared-memory ring (cp.async, one plane
// ahead), each layer's element outputs go to shared memory and every owned
// node gathers its 8 contributions in a fixed order, so results are
// bit-reproducible without atomics.  Optional fused epilogues form a PCG dot
// product of the output (one FP64 partial per CTA, finished by the last CTA).
// 2-D: k_fine_apply -- a CTA owns a 32 x 32 brick of nodes and accumulates
// element outputs in 4 colour passes (elements of one colour share no node).
// The element product uses the reflection-sector form KE = H B H
// (Walsh-Hadamard over corner bits, B block diagonal), ~240 flops per hex8
// element instead of 1152: GB300's FP64 pipe is narrow, and the FP64
// residual is the one K.u the mixed-precision solver cannot avoid; the
// differences are taken exactly first, which keeps the FP32 product accurate
// for smooth fields.
#include <algorithm>
#include <type_traits>
#include "tg_ops.cuh"
#include "tg_design.cuh"

namespace tg {

template <int NDIM> struct Tile;
template <> struct Tile<3> { static constexpr int X = 8, Y = 16, Z = 8; };
template <> struct Tile<2> { static constexpr int X = 32, Y = 32, Z = 1; };

template <int NDIM, int NDOF>
__host__ __device__ constexpr int sig(int chi, int c) {
  return (NDOF == NDIM) ? (chi ^ (1 << c)) : chi;
}

template <int NDIM, int NDOF, typename T>
__device__ __forceinline__ void wht(T (&v)[1 << NDIM][NDOF]) {
#pragma unroll
  for (int a = 0; a < NDIM; ++a)
#pragma unroll
    for (int d = 0; d < (1 << NDIM); ++d)
      if (!((d >> a) & 1)) {
        const int e = d | (1 << a);
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          const T t0 = v[d][c], t1 = v[e][c];
          v[d][c] = t0 + t1;
          v[e][c] = t0 - t1;
        }
      }
}

// y = KE u for one element, sector form (u is destroyed); the density is
// applied by the caller's fused multiply-add into the accumulator.
template <int NDIM, int NDOF, typename T, int KIND>
__device__ __forceinline__ void elem_sector(T (&u)[1 << NDIM][NDOF], const Sector<T>& B,
                                            T (&y)[1 << NDIM][NDOF]) {
  constexpr int NC = 1 << NDIM;
  wht<NDIM, NDOF, T>(u);
#pragma unroll
  for (int chi = 0; chi < NC; ++chi)
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      T acc = T(0);
#pragma unroll
      for (int c2 = 0; c2 < NDOF; ++c2)
        if (KIND != EK_SECTOR_HEX8 || ((hex8_mask(chi) >> (c * 3 + c2)) & 1u))
          acc += B.b[chi][c][c2] * u[sig<NDIM, NDOF>(chi, c2)][c2];
      y[sig<NDIM, NDOF>(chi, c)][c] = acc;
    }
  wht<NDIM, NDOF, T>(y);
}

template <int NDIM, int NDOF, typename T>
__device__ __forceinline__ void elem_dense(const T (&u)[1 << NDIM][NDOF], const T* KEs,
                                           T (&y)[1 << NDIM][NDOF]) {
  constexpr int NE = (1 << NDIM) * NDOF;
#pragma unroll 4
  for (int i = 0; i < NE; ++i) {
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < NE; ++j) acc += KEs[i * NE + j] * u[j / NDOF][j % NDOF];
    y[i / NDOF][i % NDOF] = acc;
  }
}

template <typename T, typename S> struct ApplyArgs {
  Grid g;
  const uint8_t* fix;
  const S* scale;
  const T* u;
  T* y;
  const T* b;
  const T* dinv;
  T omega;
  const T* KE;      // dense path
  Sector<T> B;
  double* part;     // fused PCG dot: per-CTA partial sums
  PCGState* pst;    //   and the state it finalises
  bool flat64;      // FineOp::flat64
};

template <int NDIM, int NDOF, typename T, bool SECTOR>
constexpr size_t apply_smem() {
  using TL = Tile<NDIM>;
  constexpr int HZ = (NDIM == 3) ? TL::Z + 2 : 1;
  constexpr int EZ = (NDIM == 3) ? TL::Z + 1 : 1;
  constexpr int NE = (1 << NDIM) * NDOF;
  return sizeof(T) * ((size_t)HZ * (TL::X + 2) * (TL::Y + 2) * NDOF +
                      (size_t)TL::Z * TL::X * TL::Y * NDOF + (SECTOR ? 0 : NE * NE) +
                      (size_t)EZ * (TL::X + 1) * (TL::Y + 1));
}

// asynchronous global -> shared copies (all of a thread's copies in flight at once)
template <int BYTES> __device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if (BYTES == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// The input u must be zero on fixed DOFs (every producer in the library keeps
// that invariant; the unit entry point masks its input explicitly), so the
// halo is a plain copy; the output is masked in the epilogue.
// Shared-memory layout of a node tile (halo included): component-major, and
// each y-row split into even and odd y so that the 2-strided accesses of one
// colour pass hit consecutive words; the half-row pitch is padded so that
// neighbouring x-rows of a warp land on different banks.
template <int NDIM> struct SLayout {
  using TL = Tile<NDIM>;
  static constexpr int HX = TL::X + 2, HY = TL::Y + 2, HZ = (NDIM == 3) ? TL::Z + 2 : 1;
  static constexpr int HH = HY / 2 + (NDIM == 3 ? 1 : 3);          // half-row pitch
  static constexpr int ROWS = HZ * HX;
  static constexpr int NODE_WORDS = ROWS * 2 * HH;                  // per component
  __device__ static constexpr int at(int c, int hz, int hx, int hy) {
    return c * NODE_WORDS + (hz * HX + hx) * 2 * HH + (hy & 1) * HH + (hy >> 1);
  }
  // element scale factors, same parity split along y
  static constexpr int EX = TL::X + 1, EY = TL::Y + 1, EZ = (NDIM == 3) ? TL::Z + 1 : 1;
  static constexpr int EH = (EY + 1) / 2 + 1;
  static constexpr int ELEM_WORDS = EZ * EX * 2 * EH;
  __device__ static constexpr int eat(int lz, int lx, int ly) {
    return (lz * EX + lx) * 2 * EH + (ly & 1) * EH + (ly >> 1);
  }
};

template <int NDIM, int NDOF, typename T, int KIND>
constexpr size_t apply_smem_v2() {
  using L = SLayout<NDIM>;
  constexpr int NE = (1 << NDIM) * NDOF;
  return sizeof(T) * ((size_t)2 * NDOF * L::NODE_WORDS + L::ELEM_WORDS + (KIND != EK_DENSE ? 0 : NE * NE));
}

template <int NDIM, int NDOF, typename T, typename S, int KIND, int MODE>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 2 : 4) k_fine_apply(ApplyArgs<T, S> a) {
  pdl_wait();
  pdl_trigger();
  using TL = Tile<NDIM>;
  using L = SLayout<NDIM>;
  constexpr int TX = TL::X, TY = TL::Y, TZ = TL::Z;
  constexpr int HX = L::HX, HY = L::HY, HZ = L::HZ;
  constexpr int EX = L::EX, EY = L::EY, EZ = L::EZ;
  constexpr int NC = 1 << NDIM;
  constexpr int NE = NC * NDOF;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* us = reinterpret_cast<T*>(smem_raw);       // u tile with halo
  T* ys = us + NDOF * L::NODE_WORDS;             // accumulator, same shape (halo discarded)
  T* rs = ys + NDOF * L::NODE_WORDS;             // element scale factors
  T* KEs = rs + L::ELEM_WORDS;                   // dense path only
  const Grid& g = a.g;
  const int y0 = blockIdx.x * TY, x0 = blockIdx.y * TX, z0 = blockIdx.z * TZ;
  const int tid = threadIdx.x, nth = blockDim.x;

  // stage u with a one-node halo (global order for coalescing)
  for (int i = tid; i < HZ * HX * HY * NDOF; i += nth) {
    const int c = i % NDOF;
    const int hy = (i / NDOF) % HY;
    const int hx = (i / (NDOF * HY)) % HX;
    const int hz = i / (NDOF * HY * HX);
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = (NDIM == 3) ? z0 - 1 + hz : 0;
    T* dst = us + L::at(c, hz, hx, hy);
    if (gx >= 0 && gx < g.nnx && gy >= 0 && gy < g.nny && gz >= 0 && gz < g.nnz)
      cp_async<sizeof(T)>(dst, a.u + g.node(gx, gy, gz) * NDOF + c);
    else
      *dst = T(0);
  }
  // stage the scale factors of the elements touching the tile
  for (int i = tid; i < EZ * EX * EY; i += nth) {
    const int ly = i % EY, lx = (i / EY) % EX, lz = i / (EY * EX);
    const int ex = x0 - 1 + lx, ey = y0 - 1 + ly, ez = (NDIM == 3) ? z0 - 1 + lz : 0;
    T* dst = rs + L::eat(lz, lx, ly);
    if (ex >= 0 && ex < g.nex && ey >= 0 && ey < g.ney && ez >= 0 && ez < g.nez) {
      if (sizeof(S) == sizeof(T))
        cp_async<sizeof(T)>(dst, a.scale + g.elem(ex, ey, ez));
      else
        *dst = load_scale<T, S>(a.scale, g.elem(ex, ey, ez));
    } else {
      *dst = T(0);
    }
  }
  for (int i = tid; i < NDOF * L::NODE_WORDS; i += nth) ys[i] = T(0);
  if (KIND == EK_DENSE)
    for (int i = tid; i < NE * NE; i += nth) KEs[i] = a.KE[i];
  cp_async_wait_all();
  __syncthreads();

  // elements with local coords l in [0, T+1) (global = origin - 1 + l), in
  // 2^ndim colour passes; the accumulator covers the halo, so corners need no
  // bounds test.  Elements outside the grid have rho = 0 and u = 0.
#pragma unroll
  for (int col = 0; col < NC; ++col) {
    const int cx = col & 1, cy = (col >> 1) & 1, cz = (col >> 2) & 1;
    const int nyc = (EY - cy + 1) / 2, nxc = (EX - cx + 1) / 2;
    const int nzc = (NDIM == 3) ? (EZ - cz + 1) / 2 : 1;
    for (int t = tid; t < nyc * nxc * nzc; t += nth) {
      const int ly = cy + 2 * (t % nyc);
      const int lx = cx + 2 * ((t / nyc) % nxc);
      const int lz = (NDIM == 3) ? cz + 2 * (t / (nyc * nxc)) : 0;
      const T rho = rs[L::eat(lz, lx, ly)];
      T ue[NC][NDOF], ye[NC][NDOF];
#pragma unroll
      for (int d = 0; d < NC; ++d) {
        const int hx = lx + (d & 1), hy = ly + ((d >> 1) & 1), hz = (NDIM == 3) ? lz + ((d >> 2) & 1) : 0;
#pragma unroll
        for (int c = 0; c < NDOF; ++c) ue[d][c] = us[L::at(c, hz, hx, hy)];
      }
      if (KIND != EK_DENSE)
        elem_sector<NDIM, NDOF, T, KIND>(ue, a.B, ye);
      else
        elem_dense<NDIM, NDOF, T>(ue, KEs, ye);
#pragma unroll
      for (int d = 0; d < NC; ++d) {
        const int hx = lx + (d & 1), hy = ly + ((d >> 1) & 1), hz = (NDIM == 3) ? lz + ((d >> 2) & 1) : 0;
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          T& acc = ys[L::at(c, hz, hx, hy)];
          acc = fma(rho, ye[d][c], acc);
        }
      }
    }
    __syncthreads();
  }

  // epilogue: owned nodes (interior of the halo tile)
  for (int i = tid; i < TZ * TX * TY * NDOF; i += nth) {
    const int c = i % NDOF;
    const int oy = (i / NDOF) % TY;
    const int ox = (i / (NDOF * TY)) % TX;
    const int oz = i / (NDOF * TY * TX);
    const int gx = x0 + ox, gy = y0 + oy, gz = z0 + oz;
    if (gx >= g.nnx || gy >= g.nny || gz >= g.nnz) continue;
    const int64_t n = g.node(gx, gy, gz);
    const int64_t k = n * NDOF + c;
    const int s = L::at(c, (NDIM == 3) ? oz + 1 : 0, ox + 1, oy + 1);
    // loads issued without a dependency on the fixed flag; the flag selects
    const bool fixed = (a.fix[n] >> c) & 1;
    const T au = ys[s];
    T out;
    if (MODE == AM_Y) {
      out = au;
    } else if (MODE == AM_RES) {
      out = a.b[k] - au;
    } else {
      out = us[s] + a.omega * a.dinv[k] * (a.b[k] - au);
    }
    a.y[k] = fixed ? T(0) : out;
  }
}

// ---------------------------------------------------------------------------
// 3-D: z-streaming variant.  A CTA owns a 15 x 15 column of nodes (x, y) over
// a chunk of node planes and marches up in z: per element layer each of its
// 256 threads evaluates one of the 16 x 16 elements touching the column
// (every element once per layer, no colour passes), writes rho * KE u_e to a
// shared element-output buffer, and after one barrier each owned node sums
// the four element outputs below and above it in a fixed order (bit-
// reproducible, no atomics).  Node planes stream through a 3-slot shared ring
// filled by cp.async one layer ahead; densities, b and dinv are loaded into
// registers one layer ahead.  Recomputed elements: (16*16)/(15*15) in x-y and
// one extra layer per z chunk, against (9*17*9)/(8*16*8) for the brick kernel.
// ---------------------------------------------------------------------------
namespace zs {
constexpr int EXT = 16, EYT = 16;          // element tile = threads (x, y)
constexpr int OX = EXT - 1, OY = EYT - 1;  // owned nodes per tile
constexpr int PX = EXT + 1, PY = EYT + 1;  // node plane incl. halo
constexpr int PITCH = 48;                  // row pitch in words: the two x-rows of a warp
                                           // (16 lanes each) fall on disjoint banks
constexpr int PLANE = PX * PITCH;          // words per component plane
constexpr int NT = EXT * EYT;
template <int NDOF> __host__ __device__ constexpr int ncopy() { return (NDOF * PX * PY + NT - 1) / NT; }
template <int NDOF, typename T, int KIND> constexpr size_t smem() {
  constexpr int NE = 8 * NDOF;
  return sizeof(T) * ((size_t)3 * NDOF * PLANE + (size_t)NE * NT + (KIND == EK_DENSE ? NE * NE : 0));
}
}  // namespace zs

// DOTK >= 0: also the PCG dot DOTK of the output with the input (AM_Y: u . y)
// or with b (AM_JACOBI: b . y) over the owned nodes, one FP64 partial per CTA,
// summed in fixed order by the last CTA to finish.
template <int NDOF, typename T, typename S, int KIND, int MODE, int DOTK = -1>
__global__ void __launch_bounds__(zs::NT, sizeof(T) == 8 ? 2 : 4) k_fine_zstream(ApplyArgs<T, S> a,
                                                                                int zc) {
  pdl_wait();
  pdl_trigger();
  using namespace zs;
  constexpr int NC = 8;
  constexpr int NE = NC * NDOF;
  constexpr int SLOT = NDOF * PLANE;
  constexpr int NCP = ncopy<NDOF>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* us = reinterpret_cast<T*>(smem_raw);        // 3 node-plane slots [c][x][PITCH]
  T* yo = us + 3 * SLOT;                          // element outputs [corner*NDOF+c][NT]
  T* KEs = yo + NE * NT;                          // dense path only
  const Grid& g = a.g;
  const int tid = threadIdx.x;
  const int y0 = blockIdx.x * OY, x0 = blockIdx.y * OX;
  const int zbeg = blockIdx.z * zc, zend = min(zbeg + zc, g.nnz);
  const int64_t pstride = (int64_t)g.nnx * g.nny * NDOF;   // words per global node plane
  const int64_t lstride = (int64_t)g.nex * g.ney;           // elements per layer

  // per-thread plane-copy descriptors (same (x, y) pattern for every plane)
  int goff[NCP], soff[NCP];
#pragma unroll
  for (int k = 0; k < NCP; ++k) {
    const int i = tid + k * NT;
    soff[k] = -1;
    goff[k] = 0;
    if (i < NDOF * PX * PY) {
      const int hx = i / (PY * NDOF), j = i % (PY * NDOF);
      const int hy = j / NDOF, c = j % NDOF;
      const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
      if (gx >= 0 && gx < g.nnx && gy >= 0 && gy < g.nny) {
        soff[k] = c * PLANE + hx * PITCH + hy;
        goff[k] = (gx * g.nny + gy) * NDOF + c;
      }
    }
  }
  // slots never written by a copy (outside the grid in x or y) stay zero
  for (int i = tid; i < 3 * SLOT; i += NT) us[i] = T(0);
  if (KIND == EK_DENSE)
    for (int i = tid; i < NE * NE; i += NT) KEs[i] = a.KE[i];
  __syncthreads();
  auto load_plane = [&](int p, int slot) {
    if (p < 0 || p >= g.nnz) return;
    const T* src = a.u + p * pstride;
    T* dst = us + slot * SLOT;
#pragma unroll
    for (int k = 0; k < NCP; ++k)
      if (soff[k] >= 0) cp_async<sizeof(T)>(dst + soff[k], src + goff[k]);
  };

  // element handled by this thread
  const int exl = tid / EYT, eyl = tid % EYT;
  const int ex = x0 - 1 + exl, ey = y0 - 1 + eyl;
  const bool evalid = ex >= 0 && ex < g.nex && ey >= 0 && ey < g.ney;
  const int64_t eoff = (int64_t)ex * g.ney + ey;
  auto load_rho = [&](int ez) -> T {
    return (evalid && ez >= 0 && ez < g.nez) ? load_scale<T, S>(a.scale, ez * lstride + eoff) : T(0);
  };
  const int ubase = exl * PITCH + eyl;
  // node owned by this thread (tid < OX*OY)
  const int ox = tid / OY, oy = tid % OY;
  const int nx = x0 + ox, ny = y0 + oy;
  const bool nvalid = tid < OX * OY && nx < g.nnx && ny < g.nny;
  const int obase = (ox + 1) * EYT + (oy + 1);     // element (ox+1, oy+1) has this node as corner 0
  const int nubase = (ox + 1) * PITCH + (oy + 1);

  int s0 = 0, s1 = 1, s2 = 2;     // slots of planes ez, ez+1, ez+2
  load_plane(zbeg - 1, s0);
  load_plane(zbeg, s1);
  cp_async_wait_all();
  __syncthreads();
  T rho = load_rho(zbeg - 1);
  T dacc = T(0);
  T acc[NDOF];
#pragma unroll
  for (int c = 0; c < NDOF; ++c) acc[c] = T(0);

  for (int ez = zbeg - 1; ez < zend; ++ez) {
    if (ez + 1 < zend) load_plane(ez + 2, s2);
    const T rho_next = load_rho(ez + 1);
    // epilogue inputs of plane ez (issued early, used after the barrier)
    const bool owned = nvalid && ez >= zbeg;
    const int64_t nid = ((int64_t)ez * g.nnx + nx) * g.nny + ny;
    T bv[NDOF], dv[NDOF];
    uint8_t fx = 0;
    if (owned) {
      fx = a.fix[nid];
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        bv[c] = (MODE != AM_Y) ? a.b[nid * NDOF + c] : T(0);
        dv[c] = (MODE == AM_JACOBI) ? a.dinv[nid * NDOF + c] : T(0);
      }
    }
    const bool lvalid = ez >= 0 && ez < g.nez;   // uniform over the CTA
    if (lvalid) {
      const T* p0 = us + s0 * SLOT + ubase;
      const T* p1 = us + s1 * SLOT + ubase;
      T ue[NC][NDOF], ye[NC][NDOF];
#pragma unroll
      for (int d = 0; d < NC; ++d)
#pragma unroll
        for (int c = 0; c < NDOF; ++c)
          ue[d][c] = ((d >> 2) ? p1 : p0)[c * PLANE + (d & 1) * PITCH + ((d >> 1) & 1)];
      if (KIND != EK_DENSE)
        elem_sector<3, NDOF, T, KIND>(ue, a.B, ye);
      else
        elem_dense<3, NDOF, T>(ue, KEs, ye);
#pragma unroll
      for (int d = 0; d < NC; ++d)
#pragma unroll
        for (int c = 0; c < NDOF; ++c) yo[(d * NDOF + c) * NT + tid] = rho * ye[d][c];
    }
    __syncthreads();
    if (nvalid) {
      T hi[NDOF];
#pragma unroll
      for (int c = 0; c < NDOF; ++c) hi[c] = T(0);
      if (lvalid) {
        // element (ox+1-dx, oy+1-dy) of this layer has the node as corner (dx, dy, dz)
#pragma unroll
        for (int d = 0; d < NC; ++d) {
          const int e = obase - (d & 1) * EYT - ((d >> 1) & 1);
#pragma unroll
          for (int c = 0; c < NDOF; ++c) {
            const T v = yo[(d * NDOF + c) * NT + e];
            if (d >> 2) hi[c] += v;
            else acc[c] += v;
          }
        }
      }
      if (owned) {
        const T* pu = us + s0 * SLOT + nubase;
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          T out;
          if (MODE == AM_Y) out = acc[c];
          else if (MODE == AM_RES) out = bv[c] - acc[c];
          else out = pu[c * PLANE] + a.omega * dv[c] * (bv[c] - acc[c]);
          out = ((fx >> c) & 1) ? T(0) : out;
          a.y[nid * NDOF + c] = out;
          if (DOTK == DOT_ALPHA) dacc = fma(pu[c * PLANE], out, dacc);
          else if (DOTK == DOT_RHO) dacc = fma(bv[c], out, dacc);
        }
      }
#pragma unroll
      for (int c = 0; c < NDOF; ++c) acc[c] = hi[c];
    }
    rho = rho_next;
    cp_async_wait_all();
    __syncthreads();
    const int t = s0;
    s0 = s1; s1 = s2; s2 = t;
  }
  if constexpr (DOTK >= 0) {
    __shared__ double sh[32];
    __shared__ int last;
    const double bs = block_sum((double)dacc, sh);
    const unsigned nblk = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    if (tid == 0) {
      a.part[bid] = bs;
      __threadfence();
      last = (atomicAdd(&a.pst->ticket, 1u) == nblk - 1);
    }
    __syncthreads();
    if (last) {
      __threadfence();
      const double tot = sum_partials(a.part, (int)nblk, sh);
      if (tid == 0) {
        pcg_dot_finish(a.pst, DOTK, tot);
        a.pst->ticket = 0;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 3-D, FP32: z-streaming with two y-adjacent elements per thread.  The CTA's
// 256 threads cover 16 (x) x 32 (y) elements (15 x 31 owned nodes); a thread's
// two elements share their middle node face, so per element layer it reads 3
// node faces instead of 4 and does the x/z butterflies of the reflection
// transform once per face; the two elements' outputs on the shared face are
// added in transform space before the inverse x/z butterflies.  Node
// contributions are merged without the element-output buffer: the face a
// thread shares with its y-neighbour arrives by a warp shuffle (lane + 1 is
// the next element pair in y), the x-neighbour's by one small shared-memory
// exchange, and the z-neighbour's stays in registers until the next layer.
// Node rows are stored even y first, then odd y, with a pitch of 48 words, so
// every shared-memory access of a warp (two x-rows of 16 lanes, stride-2 in
// y) is bank-conflict free.  Every sum runs in a fixed order: results are
// bit-reproducible.
// ---------------------------------------------------------------------------
namespace zp {
// JY = 16: a warp is exactly two x-rows of pairs, so the y-neighbour of every
// lane but the first of a row is lane - 1 of the same warp (the shuffle)
constexpr int EXT = 16, JY = 16;            // threads: element columns in x, pairs in y
constexpr int EYT = 2 * JY;                 // 32 elements in y
constexpr int OX = EXT - 1, OY = EYT - 1;   // owned nodes per tile: 15 x 31
constexpr int PX = EXT + 1, PY = EYT + 1;   // node rows / nodes per row incl. halo: 17 x 33
constexpr int ODD = JY + 1;                 // odd-y nodes of a row start here (even y: 0..16)
// the two x-rows of a warp land 16 banks apart for every face access
constexpr int PITCH = 48;
constexpr int PLANE = PX * PITCH;           // words per component plane
constexpr int NT = EXT * JY;
template <int NDOF> __host__ __device__ constexpr int ncopy() { return (NDOF * PX * PY + NT - 1) / NT; }
template <int NDOF, typename T> constexpr size_t smem() {
  return sizeof(T) * ((size_t)3 * NDOF * PLANE + (size_t)4 * NDOF * NT);
}
__host__ __device__ constexpr int ycol(int hy) { return (hy & 1) ? ODD + (hy >> 1) : (hy >> 1); }
}  // namespace zp

// Element with lower face Fa (dy = 0) and upper face Fb (dy = 1), both after
// the x/z butterflies (index q = cx | cz << 1): the y butterfly, the sector
// product with B (in place, group by group) and the inverse y butterfly;
// returns the element's output faces G[0] (lower), G[1] (upper), still in
// x/z transform space and without the density.
template <int NDOF, int KIND, typename T>
__device__ __forceinline__ void pair_element(const T (&Fa)[4][NDOF], const T (&Fb)[4][NDOF],
                                             const Sector<T>& B, T (&G)[2][4][NDOF]) {
  T U[8][NDOF];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      const int lo = (q & 1) | ((q >> 1) << 2);      // chi with cy = 0
      U[lo][c] = Fa[q][c] + Fb[q][c];
      U[lo | 2][c] = Fa[q][c] - Fb[q][c];
    }
  // y[sig(chi, c)][c] = sum_c2 B[chi][c][c2] u[sig(chi, c2)][c2]: each chi maps
  // NDOF inputs to NDOF outputs on the same index set, so it runs in place
#pragma unroll
  for (int chi = 0; chi < 8; ++chi) {
    T in[NDOF];
#pragma unroll
    for (int c2 = 0; c2 < NDOF; ++c2) in[c2] = U[sig<3, NDOF>(chi, c2)][c2];
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      T acc = T(0);
#pragma unroll
      for (int c2 = 0; c2 < NDOF; ++c2)
        if (KIND != EK_SECTOR_HEX8 || ((hex8_mask(chi) >> (c * 3 + c2)) & 1u))
          acc += B.b[chi][c][c2] * in[c2];
      U[sig<3, NDOF>(chi, c)][c] = acc;
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      const int lo = (q & 1) | ((q >> 1) << 2);
      G[0][q][c] = U[lo][c] + U[lo | 2][c];
      G[1][q][c] = U[lo][c] - U[lo | 2][c];
    }
}

// the x and z butterflies of one face (q = dx | dz << 1 <-> cx | cz << 1)
template <int NDOF, typename T>
__device__ __forceinline__ void face_xz(T (&F)[4][NDOF]) {
#pragma unroll
  for (int c = 0; c < NDOF; ++c) {
    T t0 = F[0][c], t1 = F[1][c];
    F[0][c] = t0 + t1;
    F[1][c] = t0 - t1;
    t0 = F[2][c];
    t1 = F[3][c];
    F[2][c] = t0 + t1;
    F[3][c] = t0 - t1;
    t0 = F[0][c];
    t1 = F[2][c];
    F[0][c] = t0 + t1;
    F[2][c] = t0 - t1;
    t0 = F[1][c];
    t1 = F[3][c];
    F[1][c] = t0 + t1;
    F[3][c] = t0 - t1;
  }
}

// zc unused: blockIdx.z takes node planes [z nnz / gridDim.z, (z+1) nnz / gridDim.z)
template <int NDOF, typename T, typename S, int KIND, int MODE, int DOTK = -1, bool FLAT = false>
__global__ void __launch_bounds__(zp::NT, sizeof(T) == 8 ? 1 : 3) k_fine_zpair(ApplyArgs<T, S> a) {
  pdl_wait();
  pdl_trigger();
  using namespace zp;
  static_assert(32 % JY == 0, "the y shuffle needs warps made of whole rows of pairs");
  constexpr int SLOT = NDOF * PLANE;
  constexpr int NCP = ncopy<NDOF>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* us = reinterpret_cast<T*>(smem_raw);        // 3 node-plane slots [c][hx][PITCH]
  T* xch = us + 3 * SLOT;                         // x exchange [(face*2 + dz)*NDOF + c][NT]
  const Grid& g = a.g;
  const int tid = threadIdx.x;
  const int64_t pstride = (int64_t)g.nnx * g.nny * NDOF;
  const int64_t lstride = (int64_t)g.nex * g.ney;
  // work units: (node column, node plane), column-major; a CTA owns the
  // units [u0, u1) -- one column's z chunk (grid = columns x z chunks), or
  // with FLAT an equal share of all units over a 1-D grid, which may run
  // into the next column (a second segment; without FLAT the kernel
  // compiles to a single segment, without the loop's registers)
  const int gyn = (int)cdiv(g.nny, OY);
  int64_t u0, u1;
  if (FLAT) {
    const int64_t U = (int64_t)gyn * cdiv(g.nnx, OX) * g.nnz;
    u0 = (int64_t)blockIdx.x * U / gridDim.x;
    u1 = (int64_t)(blockIdx.x + 1) * U / gridDim.x;
  } else {
    const int64_t col = (int64_t)blockIdx.y * gyn + blockIdx.x;
    u0 = col * g.nnz + (int64_t)blockIdx.z * g.nnz / gridDim.z;
    u1 = col * g.nnz + (int64_t)(blockIdx.z + 1) * g.nnz / gridDim.z;
  }
  T dacc = T(0);
  do {
  const int col = (int)(u0 / g.nnz);
  const int zbeg = (int)(u0 - (int64_t)col * g.nnz);
  const int zend = (int)min((int64_t)g.nnz, zbeg + (u1 - u0));
  const int y0 = (col % gyn) * OY, x0 = (col / gyn) * OX;

  int goff[NCP], soff[NCP];
#pragma unroll
  for (int k = 0; k < NCP; ++k) {
    const int i = tid + k * NT;
    soff[k] = -1;
    goff[k] = 0;
    if (i < NDOF * PX * PY) {
      const int hx = i / (PY * NDOF), j = i % (PY * NDOF);
      const int hy = j / NDOF, c = j % NDOF;
      const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
      if (gx >= 0 && gx < g.nnx && gy >= 0 && gy < g.nny) {
        soff[k] = c * PLANE + hx * PITCH + ycol(hy);
        goff[k] = (gx * g.nny + gy) * NDOF + c;
      }
    }
  }
  for (int i = tid; i < 3 * SLOT; i += NT) us[i] = T(0);
  __syncthreads();
  auto load_plane = [&](int p, int slot) {
    if (p < 0 || p >= g.nnz) return;
    const T* src = a.u + p * pstride;
    T* dst = us + slot * SLOT;
#pragma unroll
    for (int k = 0; k < NCP; ++k)
      if (soff[k] >= 0) cp_async<sizeof(T)>(dst + soff[k], src + goff[k]);
  };

  // this thread's element pair and owned nodes
  const int exl = tid / JY, jy = tid % JY;
  const int ex = x0 - 1 + exl;
  const int eyA = y0 - 1 + 2 * jy;
  const bool xin = ex >= 0 && ex < g.nex;
  const bool vA = xin && eyA >= 0 && eyA < g.ney;
  const bool vB = xin && eyA + 1 < g.ney;
  const int64_t eoffA = (int64_t)ex * g.ney + eyA;
  auto load_rho = [&](int ez, bool v, int64_t eoff) -> T {
    return (v && ez >= 0 && ez < g.nez) ? load_scale<T, S>(a.scale, ez * lstride + eoff) : T(0);
  };
  const int row = exl * PITCH;
  const int cf0 = jy, cf1 = ODD + jy, cf2 = jy + 1;      // columns of faces y = 2jy, 2jy+1, 2jy+2
  const int nx = x0 - 1 + exl, ny0 = y0 - 1 + 2 * jy;
  const bool xown = exl >= 1 && nx < g.nnx;
  const bool own0 = xown && jy >= 1 && ny0 < g.nny;      // node (nx, ny0)
  const bool own1 = xown && ny0 + 1 < g.nny;             // node (nx, ny0 + 1)

  int s0 = 0, s1 = 1, s2 = 2;
  load_plane(zbeg - 1, s0);
  load_plane(zbeg, s1);
  cp_async_wait_all();
  __syncthreads();
  T rhoA = load_rho(zbeg - 1, vA, eoffA), rhoB = load_rho(zbeg - 1, vB, eoffA + 1);
  T acc[2][NDOF];
#pragma unroll
  for (int f = 0; f < 2; ++f)
#pragma unroll
    for (int c = 0; c < NDOF; ++c) acc[f][c] = T(0);

  for (int ez = zbeg - 1; ez < zend; ++ez) {
    if (ez + 1 < zend) load_plane(ez + 2, s2);
    const T rnA = load_rho(ez + 1, vA, eoffA), rnB = load_rho(ez + 1, vB, eoffA + 1);
    const bool owned = ez >= zbeg;
    const int64_t nid = ((int64_t)ez * g.nnx + nx) * g.nny + ny0;
    // node values of this layer's elements: O[face][q = dx | dz << 1][c]
    T O[3][4][NDOF];
    const bool lvalid = ez >= 0 && ez < g.nez;   // uniform over the CTA
    if (lvalid) {
      const T* p0 = us + s0 * SLOT + row;
      const T* p1 = us + s1 * SLOT + row;
      auto load_face = [&](int col, T (&F)[4][NDOF]) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int c = 0; c < NDOF; ++c)
            F[q][c] = ((q >> 1) ? p1 : p0)[c * PLANE + (q & 1) * PITCH + col];
        face_xz<NDOF, T>(F);
      };
      T Fa[4][NDOF], Fb[4][NDOF];
      load_face(cf0, Fa);
      load_face(cf1, Fb);
      T G[2][4][NDOF];
      pair_element<NDOF, KIND, T>(Fa, Fb, a.B, G);
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          O[0][q][c] = rhoA * G[0][q][c];
          O[1][q][c] = rhoA * G[1][q][c];
        }
      load_face(cf2, Fa);                        // face 2 (upper face of element B)
      pair_element<NDOF, KIND, T>(Fb, Fa, a.B, G);
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          O[1][q][c] = fma(rhoB, G[0][q][c], O[1][q][c]);
          O[2][q][c] = rhoB * G[1][q][c];
        }
#pragma unroll
      for (int f = 0; f < 3; ++f) face_xz<NDOF, T>(O[f]);
    } else {
#pragma unroll
      for (int f = 0; f < 3; ++f)
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int c = 0; c < NDOF; ++c) O[f][q][c] = T(0);
    }
    // y: face 2 of the previous pair (lane - 1) is this pair's face 0
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        const T v = __shfl_up_sync(0xffffffffu, O[2][q][c], 1);
        if (jy > 0) O[0][q][c] += v;
      }
    // x: the dx = 1 values of faces 0 and 1 go to the next element column
#pragma unroll
    for (int f = 0; f < 2; ++f)
#pragma unroll
      for (int dz = 0; dz < 2; ++dz)
#pragma unroll
        for (int c = 0; c < NDOF; ++c) xch[((f * 2 + dz) * NDOF + c) * NT + tid] = O[f][1 | (dz << 1)][c];
    // epilogue inputs of node plane ez (their latency overlaps the barrier)
    T bv[2][NDOF], dv[2][NDOF];
    uint8_t fx[2] = {0, 0};
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const bool o = owned && (f == 0 ? own0 : own1);
      if (o) fx[f] = a.fix[nid + f];
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        bv[f][c] = (o && MODE != AM_Y) ? a.b[(nid + f) * NDOF + c] : T(0);
        dv[f][c] = (o && MODE == AM_JACOBI) ? a.dinv[(nid + f) * NDOF + c] : T(0);
      }
    }
    __syncthreads();
    if (exl >= 1) {
#pragma unroll
      for (int f = 0; f < 2; ++f)
#pragma unroll
        for (int dz = 0; dz < 2; ++dz)
#pragma unroll
          for (int c = 0; c < NDOF; ++c)
            O[f][dz << 1][c] += xch[((f * 2 + dz) * NDOF + c) * NT + tid - JY];
    }
    // z: dz = 0 completes node plane ez, dz = 1 starts plane ez + 1
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const bool o = owned && (f == 0 ? own0 : own1);
      if (o) {
        const T* pu = us + s0 * SLOT + row + (f == 0 ? cf0 : cf1);
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          const T au = acc[f][c] + O[f][0][c];
          T out;
          if (MODE == AM_Y) out = au;
          else if (MODE == AM_RES) out = bv[f][c] - au;
          else out = pu[c * PLANE] + a.omega * dv[f][c] * (bv[f][c] - au);
          out = ((fx[f] >> c) & 1) ? T(0) : out;
          a.y[(nid + f) * NDOF + c] = out;
          if (DOTK == DOT_ALPHA) dacc = fma(pu[c * PLANE], out, dacc);
          else if (DOTK == DOT_RHO) dacc = fma(bv[f][c], out, dacc);
        }
      }
#pragma unroll
      for (int c = 0; c < NDOF; ++c) acc[f][c] = O[f][2][c];
    }
    rhoA = rnA;
    rhoB = rnB;
    cp_async_wait_all();
    __syncthreads();
    const int t = s0;
    s0 = s1; s1 = s2; s2 = t;
  }
  u0 += zend - zbeg;
  } while (FLAT && u0 < u1);
  if constexpr (DOTK >= 0) {
    __shared__ double sh[32];
    __shared__ int last;
    const double bs = block_sum((double)dacc, sh);
    const unsigned nblk = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    if (tid == 0) {
      a.part[bid] = bs;
      __threadfence();
      last = (atomicAdd(&a.pst->ticket, 1u) == nblk - 1);
    }
    __syncthreads();
    if (last) {
      __threadfence();
      const double tot = sum_partials(a.part, (int)nblk, sh);
      if (tid == 0) {
        pcg_dot_finish(a.pst, DOTK, tot);
        a.pst->ticket = 0;
      }
    }
  }
}

static int sm_count() {
  static const int n = [] {     // thread-safe one-time initialisation
    int dev = 0, v = 0;
    TG_CUDA(cudaGetDevice(&dev));
    TG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    return v;
  }();
  return n;
}

// z-streaming launch shape: (y columns, x columns, z chunks) and the chunk
// length; as many z chunks as fit in one wave of resident CTAs (4 per SM in
// FP32, 2 in FP64), so that no second partial wave doubles the kernel time
struct ZsShape {
  int gy, gx, chunks, zc;
  bool flat = false;         // paired kernel: 1-D grid over (column, plane) units
  int64_t ctas() const { return (int64_t)gy * gx * chunks; }
};
static ZsShape zstream_shape(const Grid& g, bool fp64) {
  ZsShape s;
  s.gy = (int)cdiv(g.nny, zs::OY);
  s.gx = (int)cdiv(g.nnx, zs::OX);
  const int target = sm_count() * (fp64 ? 2 : 4);
  const int cols = s.gx * s.gy;
  const int chunks = std::max(1, std::min(g.nnz, target / cols));
  s.zc = (int)cdiv(g.nnz, chunks);
  s.chunks = (int)cdiv(g.nnz, s.zc);
  return s;
}

// the paired-element kernel: every sector-form element product, FP32 and
// FP64 (in FP64 its shared faces and 1.10 instead of 1.26 evaluations per
// element cut the FP64-pipe work of the residual by a fifth)
template <typename T, int KIND> constexpr bool use_zpair() { return KIND != EK_DENSE; }
// its launch shape: 31 x 15 node columns, as many z chunks (balanced plane
// ranges) as fill one wave of resident CTAs (3 per SM in FP32, 1 in FP64)
static ZsShape zpair_shape(const Grid& g, bool fp64, bool flat_ok) {
  ZsShape s;
  s.gy = (int)cdiv(g.nny, zp::OY);
  s.gx = (int)cdiv(g.nnx, zp::OX);
  const int target = sm_count() * (fp64 ? 1 : 3);
  const int cols = s.gx * s.gy;
  s.chunks = std::max(1, std::min(g.nnz, target / cols));
  s.zc = (int)cdiv(g.nnz, s.chunks);
  s.flat = false;
  if (fp64 && flat_ok && (int64_t)cols * s.chunks < target) {
    // one CTA per SM: an equal share of the (column, plane) units each
    // instead of whole-column chunks that leave SMs idle
    const int64_t units = (int64_t)cols * g.nnz;
    s.gy = (int)std::min<int64_t>(target, units);
    s.gx = s.chunks = 1;
    s.flat = true;
  }
  return s;
}
// CTAs of the 3-D fine launch for (T, KIND) on g (fused dots need one
// partial-sum slot per CTA)
template <typename T, int KIND>
static int64_t fine3d_ctas(const Grid& g, bool flat64) {
  return use_zpair<T, KIND>() ? zpair_shape(g, sizeof(T) == 8, flat64).ctas()
                              : zstream_shape(g, sizeof(T) == 8).ctas();
}

template <int NDOF, typename T, typename S, int KIND, int MODE, int DOTK = -1>
static void launch_zstream(const ApplyArgs<T, S>& a, cudaStream_t st) {
  const int pk = std::is_same<T, double>::value ? PK_FINE_F64
                 : (std::is_same<S, float>::value ? PK_FINE_F32 : PK_FINE_BF16);
  if constexpr (use_zpair<T, KIND>()) {
    constexpr size_t smem = zp::smem<NDOF, T>();
    const ZsShape sh = zpair_shape(a.g, sizeof(T) == 8, a.flat64);
    if (DOTK >= 0 && sh.ctas() > RED_BLOCKS)
      throw Error{EINVAL_, "fused dot: more CTAs than partial-sum slots"};
    auto go = [&](auto kern) {
      set_smem_limit((const void*)kern, (int)smem);
      prof_begin(pk, st);
      launch_pdl(kern, dim3((unsigned)sh.gy, (unsigned)sh.gx, (unsigned)sh.chunks), dim3(zp::NT),
                 smem, st, a);
      prof_end(pk, st);
      TG_CHECK_LAUNCH();
    };
    if constexpr (sizeof(T) == 8) {
      if (sh.flat) {
        go(k_fine_zpair<NDOF, T, S, KIND, MODE, DOTK, true>);
        return;
      }
    }
    go(k_fine_zpair<NDOF, T, S, KIND, MODE, DOTK, false>);
    return;
  }
  constexpr size_t smem = zs::smem<NDOF, T, KIND>();
  auto kern = k_fine_zstream<NDOF, T, S, KIND, MODE, DOTK>;
  set_smem_limit((const void*)kern, (int)smem);
  const ZsShape sh = zstream_shape(a.g, sizeof(T) == 8);
  const int gy = sh.gy, gx = sh.gx, chunks = sh.chunks, zc = sh.zc;
  if (DOTK >= 0 && sh.ctas() > RED_BLOCKS)
    throw Error{EINVAL_, "fused dot: more CTAs than partial-sum slots"};
  prof_begin(pk, st);
  launch_pdl(kern, dim3((unsigned)gy, (unsigned)gx, (unsigned)chunks), dim3(zs::NT), smem, st, a,
             zc);
  prof_end(pk, st);
  TG_CHECK_LAUNCH();
}

template <int NDIM, int NDOF, typename T, typename S, int KIND, int MODE>
static void launch_apply(const ApplyArgs<T, S>& a, cudaStream_t st) {
  // the z-streaming kernel keeps 32-bit in-plane offsets
  if constexpr (NDIM == 3) {
    if ((int64_t)a.g.nnx * a.g.nny * NDOF < (int64_t(1) << 31)) {
      launch_zstream<NDOF, T, S, KIND, MODE>(a, st);
      return;
    }
  }
  using TL = Tile<NDIM>;
  constexpr size_t smem = apply_smem_v2<NDIM, NDOF, T, KIND>();
  auto kern = k_fine_apply<NDIM, NDOF, T, S, KIND, MODE>;
  set_smem_limit((const void*)kern, (int)smem);
  dim3 grid((unsigned)cdiv(a.g.nny, TL::Y), (unsigned)cdiv(a.g.nnx, TL::X),
            (unsigned)cdiv(a.g.nnz, TL::Z));
  const int pk = std::is_same<T, double>::value ? PK_FINE_F64
                 : (std::is_same<S, float>::value ? PK_FINE_F32 : PK_FINE_BF16);
  prof_begin(pk, st);
  launch_pdl(kern, grid, dim3(256), smem, st, a);
  prof_end(pk, st);
  TG_CHECK_LAUNCH();
}

template <int NDIM, int NDOF, typename T, typename S, int KIND>
static void dispatch_mode(const ApplyArgs<T, S>& a, int mode, cudaStream_t st) {
  if (mode == AM_Y) launch_apply<NDIM, NDOF, T, S, KIND, AM_Y>(a, st);
  else if (mode == AM_RES) launch_apply<NDIM, NDOF, T, S, KIND, AM_RES>(a, st);
  else launch_apply<NDIM, NDOF, T, S, KIND, AM_JACOBI>(a, st);
}

template <int NDIM, int NDOF, typename T, typename S>
static void dispatch_apply(const ApplyArgs<T, S>& a, int kind, int mode, cudaStream_t st) {
  if (kind == EK_SECTOR_HEX8 && NDIM == 3 && NDOF == 3)
    dispatch_mode<NDIM, NDOF, T, S, EK_SECTOR_HEX8>(a, mode, st);
  else if (kind != EK_DENSE)
    dispatch_mode<NDIM, NDOF, T, S, EK_SECTOR>(a, mode, st);
  else
    dispatch_mode<NDIM, NDOF, T, S, EK_DENSE>(a, mode, st);
}

template <typename T> static const T* ke_ptr(const FineOp& op);
template <> const double* ke_ptr<double>(const FineOp& op) { return op.KE64; }
template <> const float* ke_ptr<float>(const FineOp& op) { return op.KE32; }
template <typename T> static const Sector<T>& sec_ref(const FineOp& op);
template <> const Sector<double>& sec_ref<double>(const FineOp& op) { return op.B64; }
template <> const Sector<float>& sec_ref<float>(const FineOp& op) { return op.B32; }

template <typename T, typename S>
void fine_apply(const FineOp& op, const S* scale, const T* u, T* y, const T* b, const T* dinv,
                double omega, int mode, cudaStream_t st) {
  ApplyArgs<T, S> a;
  a.g = op.g; a.fix = op.fix; a.scale = scale; a.u = u; a.y = y; a.b = b; a.dinv = dinv;
  a.omega = (T)omega; a.KE = ke_ptr<T>(op); a.B = sec_ref<T>(op);
  a.part = nullptr; a.pst = nullptr; a.flat64 = op.flat64;
  const int key = op.g.ndim * 10 + op.g.ndof;
  switch (key) {
    case 33: dispatch_apply<3, 3, T, S>(a, op.kind, mode, st); break;
    case 31: dispatch_apply<3, 1, T, S>(a, op.kind, mode, st); break;
    case 22: dispatch_apply<2, 2, T, S>(a, op.kind, mode, st); break;
    case 21: dispatch_apply<2, 1, T, S>(a, op.kind, mode, st); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof) combination"};
  }
}

template <typename T, typename S>
void fine_apply_dot(const FineOp& op, const S* scale, const T* u, T* y, const T* b, const T* dinv,
                    double omega, int mode, double* part, PCGState* pst, int dot_op,
                    cudaStream_t st) {
  TG_REQUIRE((dot_op == DOT_ALPHA && mode == AM_Y) || (dot_op == DOT_RHO && mode == AM_JACOBI),
             "fused dot: DOT_ALPHA with AM_Y or DOT_RHO with AM_JACOBI");
  const bool zstream = op.g.ndim == 3 && op.g.ndof == 3 && op.kind == EK_SECTOR_HEX8 &&
                       (int64_t)op.g.nnx * op.g.nny * 3 < (int64_t(1) << 31) &&
                       fine3d_ctas<T, EK_SECTOR_HEX8>(op.g, op.flat64) <= RED_BLOCKS;
  if (!zstream) {   // other kernels (or more CTAs than partial slots): product, then dot
    fine_apply<T, S>(op, scale, u, y, b, dinv, omega, mode, st);
    dot<T, T>(op.g.ndofs(), dot_op == DOT_ALPHA ? u : b, y, part, pst, dot_op, st);
    return;
  }
  ApplyArgs<T, S> a;
  a.g = op.g; a.fix = op.fix; a.scale = scale; a.u = u; a.y = y; a.b = b; a.dinv = dinv;
  a.omega = (T)omega; a.KE = ke_ptr<T>(op); a.B = sec_ref<T>(op);
  a.part = part; a.pst = pst; a.flat64 = op.flat64;
  if (dot_op == DOT_ALPHA) launch_zstream<3, T, S, EK_SECTOR_HEX8, AM_Y, DOT_ALPHA>(a, st);
  else launch_zstream<3, T, S, EK_SECTOR_HEX8, AM_JACOBI, DOT_RHO>(a, st);
}
template void fine_apply_dot<float, float>(const FineOp&, const float*, const float*, float*,
                                           const float*, const float*, double, int, double*,
                                           PCGState*, int, cudaStream_t);
template void fine_apply_dot<float, __nv_bfloat16>(const FineOp&, const __nv_bfloat16*,
                                                   const float*, float*, const float*,
                                                   const float*, double, int, double*, PCGState*,
                                                   int, cudaStream_t);

template void fine_apply<double, double>(const FineOp&, const double*, const double*, double*,
                                         const double*, const double*, double, int, cudaStream_t);
template void fine_apply<float, float>(const FineOp&, const float*, const float*, float*,
                                       const float*, const float*, double, int, cudaStream_t);
template void fine_apply<float, __nv_bfloat16>(const FineOp&, const __nv_bfloat16*, const float*,
                                               float*, const float*, const float*, double, int,
                                               cudaStream_t);

// ---------------------------------------------------------------------------
// inverse diagonal
// ---------------------------------------------------------------------------
template <int NDIM, int NDOF, typename T, typename S>
__global__ void k_fine_dinv(Grid g, const uint8_t* fix, const S* scale, T* dinv, FineOp op) {
  pdl_wait();
  pdl_trigger();
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= g.nnodes()) return;
  const int y = (int)(n % g.nny);
  const int x = (int)((n / g.nny) % g.nnx);
  const int z = (int)(n / ((int64_t)g.nny * g.nnx));
  T acc[NDOF];   // in the operator's own precision (no FP64 work in the FP32 path)
#pragma unroll
  for (int c = 0; c < NDOF; ++c) acc[c] = T(0);
#pragma unroll
  for (int d = 0; d < (1 << NDIM); ++d) {
    const int ex = x - (d & 1), ey = y - ((d >> 1) & 1), ez = (NDIM == 3) ? z - ((d >> 2) & 1) : 0;
    if (ex < 0 || ex >= g.nex || ey < 0 || ey >= g.ney || ez < 0 || ez >= g.nez) continue;
    const T s = load_scale<T, S>(scale, g.elem(ex, ey, ez));
#pragma unroll
    for (int c = 0; c < NDOF; ++c) acc[c] = fma(s, (T)op.KEdiag[d * NDOF + c], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < NDOF; ++c)
    dinv[n * NDOF + c] = ((fix[n] >> c) & 1) ? T(0) : T(1) / acc[c];
}

template <typename T, typename S>
void fine_dinv(const FineOp& op, const S* scale, T* dinv, cudaStream_t st) {
  const int64_t nn = op.g.nnodes();
  const unsigned blocks = (unsigned)cdiv(nn, 256);
  const int key = op.g.ndim * 10 + op.g.ndof;
  switch (key) {
    case 33: launch_pdl(k_fine_dinv<3, 3, T, S>, dim3(blocks), dim3(256), 0, st, op.g, op.fix, scale, dinv, op); break;
    case 31: launch_pdl(k_fine_dinv<3, 1, T, S>, dim3(blocks), dim3(256), 0, st, op.g, op.fix, scale, dinv, op); break;
    case 22: launch_pdl(k_fine_dinv<2, 2, T, S>, dim3(blocks), dim3(256), 0, st, op.g, op.fix, scale, dinv, op); break;
    case 21: launch_pdl(k_fine_dinv<2, 1, T, S>, dim3(blocks), dim3(256), 0, st, op.g, op.fix, scale, dinv, op); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof) combination"};
  }
  TG_CHECK_LAUNCH();
}
template void fine_dinv<double, double>(const FineOp&, const double*, double*, cudaStream_t);
template void fine_dinv<float, float>(const FineOp&, const float*, float*, cudaStream_t);
template void fine_dinv<float, __nv_bfloat16>(const FineOp&, const __nv_bfloat16*, float*,
                                              cudaStream_t);

// ---------------------------------------------------------------------------
// compliance + sensitivity (FP64)
// ---------------------------------------------------------------------------
template <int NDIM, int NDOF, bool SECTOR>
__global__ void __launch_bounds__(RED_THREADS) k_compliance(Grid g, const double* __restrict__ xPhys,
                                                           const double* __restrict__ u,
                                                           const double* __restrict__ KE,
                                                           Sector<double> B, double eps,
                                                           double penal, double* dc,
                                                           double* partial,
                                                           const int8_t* __restrict__ flags,
                                                           int accumulate) {
  pdl_wait();
  pdl_trigger();
  constexpr int NC = 1 << NDIM;
  constexpr int NE = NC * NDOF;
  __shared__ double sh[32];
  double objp = 0.0;
  const int64_t nel = g.nel();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nel;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int ey = (int)(e % g.ney);
    const int ex = (int)((e / g.ney) % g.nex);
    const int ez = (int)(e / ((int64_t)g.ney * g.nex));
    if (flags && flags[e] == EL_OUTSIDE) {
      if (!accumulate) dc[e] = 0.0;
      continue;
    }
    double ue[NC][NDOF];
#pragma unroll
    for (int d = 0; d < NC; ++d) {
      const int64_t n = g.node(ex + (d & 1), ey + ((d >> 1) & 1), (NDIM == 3) ? ez + ((d >> 2) & 1) : 0);
#pragma unroll
      for (int c = 0; c < NDOF; ++c) ue[d][c] = __ldg(u + n * NDOF + c);
    }
    double ce = 0.0;
    if (SECTOR) {
      // u^T KE u = (H u)^T B (H u)
      wht<NDIM, NDOF, double>(ue);
#pragma unroll
      for (int chi = 0; chi < NC; ++chi)
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          double acc = 0.0;
#pragma unroll
          for (int c2 = 0; c2 < NDOF; ++c2)
            acc += B.b[chi][c][c2] * ue[sig<NDIM, NDOF>(chi, c2)][c2];
          ce += acc * ue[sig<NDIM, NDOF>(chi, c)][c];
        }
    } else {
      for (int i = 0; i < NE; ++i) {
        double acc = 0.0;
        for (int j = 0; j < NE; ++j) acc += __ldg(KE + i * NE + j) * ue[j / NDOF][j % NDOF];
        ce += acc * ue[i / NDOF][i % NDOF];
      }
    }
    const double xv = xPhys[e];
    double xp, xpm1;
    if (penal == 3.0) {
      xpm1 = xv * xv;
      xp = xpm1 * xv;
    } else {
      xp = pow(xv, penal);
      xpm1 = pow(xv, penal - 1.0);
    }
    objp += (eps + (1.0 - eps) * xp) * ce;
    const double dce = -(penal * (1.0 - eps) * xpm1) * ce;
    dc[e] = accumulate ? dc[e] + dce : dce;
  }
  const double s = block_sum(objp, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = accumulate ? partial[blockIdx.x] + s : s;
}

void fine_compliance(const FineOp& op, const double* xPhys, const double* u, double eps,
                     double penal, double* dc, double* partial, cudaStream_t st,
                     const int8_t* flags, bool accumulate) {
  const int64_t nel = op.g.nel();
  const unsigned blocks = red_blocks(nel);
  const int key = op.g.ndim * 10 + op.g.ndof;
#define TG_COMP(ND, NF)                                                                     \
  if (op.sector)                                                                            \
    launch_pdl(k_compliance<ND, NF, true>, dim3(blocks), dim3(RED_THREADS), 0, st, op.g, xPhys, u, op.KE64,      \
                                                              op.B64, eps, penal, dc, partial, flags, accumulate ? 1 : 0); \
  else                                                                                      \
    launch_pdl(k_compliance<ND, NF, false>, dim3(blocks), dim3(RED_THREADS), 0, st, op.g, xPhys, u, op.KE64,     \
                                                               op.B64, eps, penal, dc, partial, flags, accumulate ? 1 : 0);
  switch (key) {
    case 33: TG_COMP(3, 3) break;
    case 31: TG_COMP(3, 1) break;
    case 22: TG_COMP(2, 2) break;
    case 21: TG_COMP(2, 1) break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof) combination"};
  }
#undef TG_COMP
  TG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// adjoint sensitivity (FP64, dense element product)
// ---------------------------------------------------------------------------
template <int NDIM, int NDOF>
__global__ void __launch_bounds__(256) k_adjoint_sens(Grid g, const double* __restrict__ xPhys,
                                                     const double* __restrict__ u,
                                                     const double* __restrict__ v,
                                                     const double* __restrict__ KE, double eps,
                                                     double penal, double* __restrict__ dobj,
                                                     const int8_t* __restrict__ flags) {
  constexpr int NC = 1 << NDIM;
  constexpr int NE = NC * NDOF;
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  if (flags && flags[e] == EL_OUTSIDE) {
    dobj[e] = 0.0;
    return;
  }
  const int ey = (int)(e % g.ney);
  const int ex = (int)((e / g.ney) % g.nex);
  const int ez = (int)(e / ((int64_t)g.ney * g.nex));
  double ue[NE], ve[NE];
#pragma unroll
  for (int d = 0; d < NC; ++d) {
    const int64_t n = g.node(ex + (d & 1), ey + ((d >> 1) & 1), (NDIM == 3) ? ez + ((d >> 2) & 1) : 0);
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      ue[d * NDOF + c] = u[n * NDOF + c];
      ve[d * NDOF + c] = v[n * NDOF + c];
    }
  }
  double s = 0.0;
  for (int i = 0; i < NE; ++i) {
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < NE; ++j) t += __ldg(KE + i * NE + j) * ue[j];
    s += ve[i] * t;
  }
  const double xv = xPhys[e];
  const double dx = penal * (1.0 - eps) * ((penal == 3.0) ? xv * xv : pow(xv, penal - 1.0));
  dobj[e] = dx * s;
}

void fine_adjoint_sens(const FineOp& op, const double* xPhys, const double* u, const double* v,
                       double eps, double penal, double* dobj, cudaStream_t st,
                       const int8_t* flags) {
  const unsigned blocks = (unsigned)cdiv(op.g.nel(), 256);
  switch (op.g.ndim * 10 + op.g.ndof) {
    case 33: k_adjoint_sens<3, 3><<<blocks, 256, 0, st>>>(op.g, xPhys, u, v, op.KE64, eps, penal, dobj, flags); break;
    case 31: k_adjoint_sens<3, 1><<<blocks, 256, 0, st>>>(op.g, xPhys, u, v, op.KE64, eps, penal, dobj, flags); break;
    case 22: k_adjoint_sens<2, 2><<<blocks, 256, 0, st>>>(op.g, xPhys, u, v, op.KE64, eps, penal, dobj, flags); break;
    case 21: k_adjoint_sens<2, 1><<<blocks, 256, 0, st>>>(op.g, xPhys, u, v, op.KE64, eps, penal, dobj, flags); break;
    default: throw Error{EINVAL_, "unsupported (ndim, nnode_dof) combination"};
  }
  TG_CHECK_LAUNCH();
}

}  // namespace tg
