// Host-side launcher declarations shared by the library's translation units.
#pragma once
#include "tg_common.cuh"

namespace tg {

// Sector blocks of the element matrix.  With H the Walsh-Hadamard transform
// over the element's corner bits (d = dx | dy<<1 | dz<<2, y in index space),
// KE = H B H where B is block diagonal: block chi couples (sigma, c) with
// sigma = chi ^ (1<<c) for vector problems (ndof == ndim) and sigma = chi for
// scalar ones.  The 1/4^ndim normalisation is folded into B.
template <typename T> struct Sector {
  T b[8][3][3];
};

// Element-product kinds: dense KE, sector form with any block contents, and
// sector form with the zero pattern of the reference's hex8 elasticity
// blocks (45 of 72 entries non-zero; the host verifies the pattern).
enum ElemKind : int { EK_DENSE = 0, EK_SECTOR = 1, EK_SECTOR_HEX8 = 2 };
// bit (c*3 + c2) set: block chi, row c, column c2 is structurally non-zero
__host__ __device__ constexpr unsigned hex8_mask(int chi) {
  return chi == 0 || chi == 7 ? 0x1FFu
         : chi == 1 ? 0x1B0u : chi == 2 ? 0x145u : chi == 3 ? 0x11Bu
         : chi == 4 ? 0x01Bu : chi == 5 ? 0x155u : 0x1B1u;
}

// Fine-level (matrix-free) operator description.
struct FineOp {
  Grid g;
  const uint8_t* fix;       // [nnodes] fixed-DOF bits
  const double* KE64;       // [NE*NE] element matrix, corner-bit order (device)
  const float* KE32;        // same in FP32 (device)
  Sector<double> B64;
  Sector<float> B32;
  bool sector;              // use the sector path
  int kind;                 // element product: 0 dense, 1 sector, 2 sector with the hex8 zero pattern
  double KEdiag[24];        // diagonal of KE, corner-bit order
  // 3-D FP64 paired products over an equal share of (column, plane) units
  // per SM instead of whole-column chunks (the FP64 solver's contexts; the
  // mixed solver's FP64 residual leaves SMs to the hierarchy build beside it)
  bool flat64 = false;
};

enum ApplyMode : int { AM_Y = 0, AM_RES = 1, AM_JACOBI = 2 };

// y = M K(s) M u  (mode AM_Y);  y = b - A u  (AM_RES);
// y = u + omega * dinv * (b - A u)  (AM_JACOBI).  Fixed DOFs of y are 0.
template <typename T, typename S>
void fine_apply(const FineOp& op, const S* scale, const T* u, T* y, const T* b, const T* dinv,
                double omega, int mode, cudaStream_t st);

// dinv = 1/diag(A) on free DOFs, 0 on fixed DOFs
template <typename T, typename S>
void fine_dinv(const FineOp& op, const S* scale, T* dinv, cudaStream_t st);

// Element flag of padding elements (outside the user's grid, see ctx_init):
// zero stiffness, excluded from filter, volume, compliance and OC.
constexpr int8_t EL_OUTSIDE = 3;

// ce_e = u_e^T KE u_e ;  dc_e = -penal (1-eps) x^(penal-1) ce_e ;
// partial[b] = sum over the block's elements of simp(x_e) ce_e (padding
// elements, flag EL_OUTSIDE, contribute nothing and get dc = 0)
// (accumulate: dc and partial are added to, for a further load case)
// dobj_e = simp_dx(xPhys_e) * v_e^T KE u_e (FP64): the sensitivity of an
// objective with adjoint solution v (topology_optimization.py:473-500)
void fine_adjoint_sens(const FineOp& op, const double* xPhys, const double* u, const double* v,
                       double eps, double penal, double* dobj, cudaStream_t st,
                       const int8_t* flags = nullptr);
void fine_compliance(const FineOp& op, const double* xPhys, const double* u, double eps,
                     double penal, double* dc, double* partial, cudaStream_t st,
                     const int8_t* flags = nullptr, bool accumulate = false);

// ---------------------------------------------------------------------------
// assembled 3^ndim-point block stencils (coarse levels)
// layout: A[(dir * ndof + ci) * ndof + cj][node]   (structure of arrays, each
// array of stride g.slds(): nnodes rounded up to 32)
// ---------------------------------------------------------------------------
// Stencils are symmetric and stored half: the centre block and the 3^ndim/2
// upper direction blocks per node, [(dh*ndof+ci)*ndof+cj][node]
inline int stencil_half_dirs(int ndim) { return ndim == 3 ? 14 : 5; }
template <typename T>
void stencil_apply(const Grid& g, const T* A, const T* u, T* y, const T* b, const T* dinv,
                   double omega, int mode, cudaStream_t st);
// FP32 3-D sweeps on grids too large for the small-grid kernel stage their
// coefficients in shared memory by TMA (on by default); 0 selects the
// register-path kernel (same results)
void tune_set_stencil_tma(int on);
// 1 (and cleared) if a bounded wait of a TMA-fed stencil sweep ran out since
// the last call; synchronises st
int take_wait_error(cudaStream_t st);
// the tensor-core convolution's wait-error flag (read and cleared)
int take_conv_error(cudaStream_t st);
template <typename T>
void stencil_dinv(const Grid& g, const uint8_t* fix, const T* A, T* dinv, cudaStream_t st);

// level-1 stencil straight from element scale factors (exact masked Galerkin)
template <typename T>
void build_level1(const FineOp& op, const T* scale, const uint8_t* elem_touch_fixed,
                  const T* Q /* [nchild][NE][NE] */, const T* KE, const Grid& gc,
                  const uint8_t* fixc, T* Ac, cudaStream_t st);
// fine-level stencil from the element scale factors (fine grid = coarsest level)
void build_fine_stencil(const FineOp& op, const double* scale, double* A, cudaStream_t st);
// Galerkin product of an assembled stencil: Ac = M_c P^T A P M_c
template <typename T>
void build_galerkin(const Grid& gf, const T* Af, const Grid& gc, const uint8_t* fixc, T* Ac,
                    cudaStream_t st);

// full 3^ndim-direction layout [(d*ndof+ci)*ndof+cj][node] of a half-stored
// stencil (diagnostic export)
template <typename T>
void stencil_expand(const Grid& g, const T* Ah, double* Afull, cudaStream_t st);

// transfers (masked): bc = Mc P^T rf ;  xf += Mf P xc
template <typename T>
void restrict_(const Grid& gf, const Grid& gc, const uint8_t* fixc, const T* rf, T* bc,
               cudaStream_t st, const T* dinvc = nullptr, T* xc = nullptr, double omega = 0.0);
template <typename T>
void prolong_add(const Grid& gf, const Grid& gc, const uint8_t* fixf, const T* xc, T* xf,
                 cudaStream_t st);
// xf = Mf P xc (fixed DOFs 0)
template <typename T>
void prolong_set(const Grid& gf, const Grid& gc, const uint8_t* fixf, const T* xc, T* xf,
                 cudaStream_t st);

// The bottom of a V-cycle in one cooperative launch: restriction of the
// parent level's residual rp into the tail level (with its first smoothing
// step from zero), nsmooth - 1 Jacobi sweeps, the residual, restriction to
// the coarsest level, the coarsest solve (dense FP64 inverse), prolongation,
// nsmooth Jacobi sweeps, and prolongation of the tail level's iterate into
// the parent's xp -- phases separated by the cluster barrier of one
// thread-block cluster (up to 16 SMs), or by bounded grid barriers of a
// cooperative launch (bar->err set when one times out).  The tail level must
// use the small-grid stencil.
template <typename T> struct TailArgs {
  Grid gp, gt, gc;                         // parent, tail and coarsest grids
  const uint8_t *fixt, *fixc, *fixp;
  const T* rp;                             // parent residual
  T* xp;                                   // parent iterate (+= P x_t)
  const T* At;                             // tail stencil (half-stored)
  const T* dinvt;
  T *bt, *xt, *tt, *rt;                    // tail vectors
  T *bc, *xc;                              // coarsest vectors
  const double* Dc;                        // coarsest inverse
  const float* Dc32;                       // the same in FP32 (T = float; null: Dc)
  int64_t nc, ldc;
  double* part;                            // >= 8 * nc doubles
  T omega;
  int nsmooth;
  int cluster;                             // > 0: one thread-block cluster of at most this many CTAs
  int blocks;                              // cooperative launch: 0 one block per SM
  GridBar* bar;
};
template <typename T>
void coarse_tail(const TailArgs<T>& a, cudaStream_t st);
// the largest (node, DOF) row count of a tail level the fused kernel takes
constexpr int64_t TAIL_MAX_PAIRS = 65536;

// coarsest level: dense matrix (fixed DOFs -> identity) and its inverse
template <typename T>
void stencil_to_dense(const Grid& g, const uint8_t* fix, const T* A, double* D, int64_t n,
                      int64_t ld, cudaStream_t st);
// work: 32 * 32 + 2 * 32 * ld doubles (enough for pivot blocks up to 32)
void gj_inverse(double* D, int64_t n, int64_t ld, double* work, cudaStream_t st);
// the same in double-word FP32 arithmetic (about 48 significant bits; same
// work buffer): mixed-precision contexts, whose coarsest matrix holds FP32
// values and whose V-cycle runs in FP32
// lookahead: each step's update launch also forms the next step's panel
// (same values, ~half the launches, the panel chain off the critical path);
// work then needs two sets of 16*16 + 2*16*ld doubles (the 32*32 + 2*32*ld
// of gj_inverse suffice)
void gj_inverse_dw(double* D, int64_t n, int64_t ld, double* work, cudaStream_t st,
                   bool lookahead = true);
template <typename T>
void dense_apply(const double* Dinv, int64_t n, int64_t ld, const T* b, T* x,
                 double* work /* >= 8*n */, cudaStream_t st);
// the inverse stored in FP32 (mixed contexts' FP32 V-cycle)
void dense_apply(const float* Dinv, int64_t n, int64_t ld, const float* b, float* x,
                 double* work /* >= 8*n */, cudaStream_t st);

// ---------------------------------------------------------------------------
// design-variable kernels
// ---------------------------------------------------------------------------
struct FilterStencil {
  int R;                 // half width
  int nw;                // (2R+1)^ndim
  const double* w;       // [nw] weights, dz slowest, dx, dy fastest
  double* tmp;           // nel scratch for mode 1 (null: divide inside the stencil loop)
  int rex, rey, rez;     // element extents of the user's grid (smaller than the
                         // device grid when it is padded); taps beyond are skipped
};
// mode 0: y = (H x) / Hs ; mode 1: y = H (x / Hs) ; mode 2: y = H(x*d)/Hs/max(1e-3, x)
// mode 3: Hs = H 1 (x unused) ; mode 4: y = x (copy, used with the fused reductions)
void filter_apply(const Grid& ge, const FilterStencil& fs, const double* x, const double* d,
                  const double* Hs, double* y, int mode, cudaStream_t st);

void simp_scale(int64_t n, const double* x, double eps, double penal, double* s64, float* s32,
                __nv_bfloat16* s16, cudaStream_t st, const int8_t* flags = nullptr);
// copy between the user's grid numbering (rg) and the device grid (g, padded
// at the high end of each axis): per = values per node (nodes) or 1 (elements)
void embed_copy(const Grid& rg, const Grid& g, bool nodes, const double* src, double* dst,
                bool to_device_grid, cudaStream_t st);

// vector helpers
template <typename T>
void axpby(int64_t n, double a, const T* x, double b, T* y, cudaStream_t st);
void mask_vec_f64(int64_t nnodes, int ndof, const uint8_t* fix, double* v, cudaStream_t st);

}  // namespace tg
