/*
 * CPU restatement of the FP64 geometric-multigrid PCG for 3-D hex8
 * elasticity (test infrastructure and the CPU baseline of the benchmark;
 * never part of the GPU library).  OpenMP over nodes, FP64 throughout.
 *
 * It states on the host the same algorithm as oracle/gmg.py, with the fine
 * level matrix-free so that the 160x80x80 workload fits: the operator is
 * M K(s) M with K = sum_e s_e KE_e assembled from the reference element
 * matrix (elements/linear_elasticity_3d.py:65) in the reference numbering
 * (elements/trilinear_hexahedron.py:7-58: node (x, y, z) ->
 * (nelx+1)(nely+1) z + (nely+1) x + y, element (ex, ey, ez) ->
 * ez nelx nely + ex nely + ey, local corners (0,1,0) (1,1,0) (1,0,0) (0,0,0)
 * (0,1,1) (1,1,1) (1,0,1) (0,0,1)), M the 0/1 mask of free DOFs
 * (fem.py:208-237 restated on all DOFs).  Every coarse level is the
 * Galerkin product Pt^T A Pt of the trilinear interpolation from the
 * stride-2 nodes (gmg.py:148-189) with masks on both sides; since A is
 * element-assembled, so is Pt^T A Pt, and each level is built element by
 * element and applied as a 27-point block stencil.  The V-cycle and the PCG
 * driver live in oracle/cpu_gmg.py.
 *
 * Build: gcc -O3 -fopenmp -shared -fPIC oracle/cgmg.c -o oracle/libcgmg.so
 */
#include <omp.h>
#include <stdint.h>
#include <string.h>

static const int CX[8] = {0, 1, 1, 0, 0, 1, 1, 0};
static const int CY[8] = {1, 1, 0, 0, 1, 1, 0, 0};
static const int CZ[8] = {0, 0, 0, 0, 1, 1, 1, 1};

/* mode 0: y = M K M u;  1: y = b - M K M u;  2: y = u + omega dinv (b - M K M u)
 * fixn: per node, bit c set = DOF c fixed (u is masked here).  work: ndof
 * doubles.  K M u is formed element by element in 8 colour passes (elements
 * whose coordinates have the same parities share no node), so the scatter
 * into work needs no atomics; the epilogue then masks and combines. */
void hex8_apply(int nelx, int nely, int nelz, const double* KE, const double* s,
                const uint8_t* fixn, const double* u, double* y, const double* b,
                const double* dinv, double omega, int mode, double* work) {
  const int nnx = nelx + 1, nny = nely + 1, nnz = nelz + 1;
  const int64_t nnodes = (int64_t)nnx * nny * nnz;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < 3 * nnodes; ++i) work[i] = 0.0;
  for (int col = 0; col < 8; ++col) {
    const int pz = col >> 2, px = (col >> 1) & 1, py = col & 1;
    const int nzc = (nelz - pz + 1) / 2, nxc = (nelx - px + 1) / 2, nyc = (nely - py + 1) / 2;
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < nzc; ++iz)
      for (int ix = 0; ix < nxc; ++ix) {
        const int ez = pz + 2 * iz, ex = px + 2 * ix;
        for (int iy = 0; iy < nyc; ++iy) {
          const int ey = py + 2 * iy;
          const int64_t e = ((int64_t)ez * nelx + ex) * nely + ey;
          int64_t nd[8];
          double ue[24], ye[24];
          for (int j = 0; j < 8; ++j) {
            nd[j] = ((int64_t)(ez + CZ[j]) * nnx + (ex + CX[j])) * nny + (ey + CY[j]);
            const uint8_t fm = fixn[nd[j]];
            for (int c = 0; c < 3; ++c) ue[3 * j + c] = ((fm >> c) & 1) ? 0.0 : u[3 * nd[j] + c];
          }
          const double se = s[e];
          for (int i = 0; i < 24; ++i) {
            double t = 0.0;
            for (int j = 0; j < 24; ++j) t += KE[i * 24 + j] * ue[j];
            ye[i] = se * t;
          }
          for (int j = 0; j < 8; ++j)
            for (int c = 0; c < 3; ++c) work[3 * nd[j] + c] += ye[3 * j + c];
        }
      }
  }
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nnodes; ++n) {
    const uint8_t fn = fixn[n];
    for (int c = 0; c < 3; ++c) {
      const int64_t i = 3 * n + c;
      double out;
      if (mode == 0) out = work[i];
      else if (mode == 1) out = b[i] - work[i];
      else out = u[i] + omega * dinv[i] * (b[i] - work[i]);
      y[i] = ((fn >> c) & 1) ? 0.0 : out;
    }
  }
}

/* inverse diagonal of M K M (0 on fixed DOFs) */
void hex8_dinv(int nelx, int nely, int nelz, const double* KE, const double* s,
               const uint8_t* fixn, double* dinv) {
  const int nnx = nelx + 1, nny = nely + 1, nnz = nelz + 1;
  const int64_t nnodes = (int64_t)nnx * nny * nnz;
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nnodes; ++n) {
    const int yy = (int)(n % nny), xx = (int)((n / nny) % nnx), zz = (int)(n / ((int64_t)nny * nnx));
    double d[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 8; ++k) {
      const int ex = xx - CX[k], ey = yy - CY[k], ez = zz - CZ[k];
      if (ex < 0 || ex >= nelx || ey < 0 || ey >= nely || ez < 0 || ez >= nelz) continue;
      const int64_t e = ((int64_t)ez * nelx + ex) * nely + ey;
      for (int c = 0; c < 3; ++c) d[c] += s[e] * KE[(3 * k + c) * 24 + 3 * k + c];
    }
    for (int c = 0; c < 3; ++c) dinv[3 * n + c] = ((fixn[n] >> c) & 1) ? 0.0 : 1.0 / d[c];
  }
}

/* weight of the fine coordinate f in {0,1,2} from the coarse corner C in {0,2} */
static double w1(int f, int C) { return f == C ? 1.0 : (f == 1 ? 0.5 : 0.0); }

/* P_c[child][fine local dof][coarse local dof]: trilinear interpolation of a
 * child element's 8 nodes from its parent's 8 corners (node weights x I3) */
static void child_interp(double Pc[8][24][24]) {
  for (int ch = 0; ch < 8; ++ch) {
    memset(Pc[ch], 0, sizeof(Pc[ch]));
    for (int k = 0; k < 8; ++k) {
      const int fx = CX[ch] + CX[k], fy = CY[ch] + CY[k], fz = CZ[ch] + CZ[k];
      for (int K = 0; K < 8; ++K) {
        const double w = w1(fx, 2 * CX[K]) * w1(fy, 2 * CY[K]) * w1(fz, 2 * CZ[K]);
        for (int c = 0; c < 3; ++c) Pc[ch][3 * k + c][3 * K + c] = w;
      }
    }
  }
}

/* A += s P^T (m KE m) P for one child (m: 0/1 mask of the child's DOFs) */
static void child_product(const double* KE, const double* m, double s, const double P[24][24],
                          double* A) {
  double T[24][24];
  for (int i = 0; i < 24; ++i)
    for (int J = 0; J < 24; ++J) {
      double t = 0.0;
      for (int j = 0; j < 24; ++j) t += KE[i * 24 + j] * m[j] * P[j][J];
      T[i][J] = m[i] * t;
    }
  for (int I = 0; I < 24; ++I)
    for (int J = 0; J < 24; ++J) {
      double t = 0.0;
      for (int i = 0; i < 24; ++i) t += P[i][I] * T[i][J];
      A[I * 24 + J] += s * t;
    }
}

/* coarse mask on both sides of one coarse element matrix */
static void mask_coarse(double* A, const uint8_t* fixc, int cnx, int cny, int ex, int ey, int ez) {
  double mc[24];
  for (int K = 0; K < 8; ++K) {
    const int64_t N = ((int64_t)(ez + CZ[K]) * cnx + (ex + CX[K])) * cny + (ey + CY[K]);
    for (int c = 0; c < 3; ++c) mc[3 * K + c] = ((fixc[N] >> c) & 1) ? 0.0 : 1.0;
  }
  for (int I = 0; I < 24; ++I)
    for (int J = 0; J < 24; ++J) A[I * 24 + J] *= mc[I] * mc[J];
}

/* Coarse element matrices of level 1, Pt^T (M K M) Pt restricted to each
 * coarse element: ae[E*576 ...] for the (nelx/2, nely/2, nelz/2) coarse
 * elements.  fixn: fine node masks, fixc: coarse node masks (coarse DOF
 * fixed iff the coincident fine DOF is). */
void hex8_galerkin1(int nelx, int nely, int nelz, const double* KE, const double* s,
                    const uint8_t* fixn, const uint8_t* fixc, double* ae) {
  const int cx = nelx / 2, cy = nely / 2, cz = nelz / 2;
  const int nnx = nelx + 1, nny = nely + 1;
  const int64_t ncel = (int64_t)cx * cy * cz;
  double Pc[8][24][24];
  child_interp(Pc);
  /* children that touch no fixed DOF: A += s_e Q_c with Q_c = P_c^T KE P_c */
  double Q[8][576];
  double ones[24];
  for (int i = 0; i < 24; ++i) ones[i] = 1.0;
  for (int ch = 0; ch < 8; ++ch) {
    memset(Q[ch], 0, sizeof(Q[ch]));
    child_product(KE, ones, 1.0, Pc[ch], Q[ch]);
  }
#pragma omp parallel for schedule(static)
  for (int64_t E = 0; E < ncel; ++E) {
    const int ey = (int)(E % cy), ex = (int)((E / cy) % cx), ez = (int)(E / ((int64_t)cy * cx));
    double* A = ae + E * 576;
    memset(A, 0, sizeof(double) * 576);
    for (int ch = 0; ch < 8; ++ch) {
      const int fex = 2 * ex + CX[ch], fey = 2 * ey + CY[ch], fez = 2 * ez + CZ[ch];
      const int64_t e = ((int64_t)fez * nelx + fex) * nely + fey;
      double m[24];
      int masked = 0;
      for (int k = 0; k < 8; ++k) {
        const int64_t node = ((int64_t)(fez + CZ[k]) * nnx + (fex + CX[k])) * nny + (fey + CY[k]);
        for (int c = 0; c < 3; ++c) {
          m[3 * k + c] = ((fixn[node] >> c) & 1) ? 0.0 : 1.0;
          masked |= (fixn[node] >> c) & 1;
        }
      }
      if (masked) {
        child_product(KE, m, s[e], Pc[ch], A);
      } else {
        const double se = s[e];
        for (int i = 0; i < 576; ++i) A[i] += se * Q[ch][i];
      }
    }
    mask_coarse(A, fixc, cx + 1, cy + 1, ex, ey, ez);
  }
}

/* The next level's element matrices from this level's (ae_in: (nelx, nely,
 * nelz) elements, already masked on this level's DOFs): Galerkin product of
 * the trilinear interpolation, masked with the next level's fixc. */
void elem_galerkin(int nelx, int nely, int nelz, const double* ae_in, const uint8_t* fixc,
                   double* ae_out) {
  const int cx = nelx / 2, cy = nely / 2, cz = nelz / 2;
  const int64_t ncel = (int64_t)cx * cy * cz;
  double Pc[8][24][24];
  child_interp(Pc);
  double ones[24];
  for (int i = 0; i < 24; ++i) ones[i] = 1.0;
#pragma omp parallel for schedule(static)
  for (int64_t E = 0; E < ncel; ++E) {
    const int ey = (int)(E % cy), ex = (int)((E / cy) % cx), ez = (int)(E / ((int64_t)cy * cx));
    double* A = ae_out + E * 576;
    memset(A, 0, sizeof(double) * 576);
    for (int ch = 0; ch < 8; ++ch) {
      const int64_t e = ((int64_t)(2 * ez + CZ[ch]) * nelx + (2 * ex + CX[ch])) * nely +
                        (2 * ey + CY[ch]);
      child_product(ae_in + e * 576, ones, 1.0, Pc[ch], A);
    }
    mask_coarse(A, fixc, cx + 1, cy + 1, ex, ey, ez);
  }
}

/* 27-point stencil of 3x3 blocks, stencil[((d*3 + ci)*3 + cj)*nn + N] with
 * d = (dz+1)*9 + (dx+1)*3 + (dy+1) the direction to the neighbour, gathered
 * per node from its (up to 8) elements in a fixed order */
void elem_to_stencil(int nelx, int nely, int nelz, const double* ae, double* stencil) {
  const int nnx = nelx + 1, nny = nely + 1, nnz = nelz + 1;
  const int64_t nn = (int64_t)nnx * nny * nnz;
#pragma omp parallel for schedule(static)
  for (int64_t N = 0; N < nn; ++N) {
    const int yy = (int)(N % nny), xx = (int)((N / nny) % nnx), zz = (int)(N / ((int64_t)nny * nnx));
    for (int i = 0; i < 243; ++i) stencil[(int64_t)i * nn + N] = 0.0;
    for (int k = 0; k < 8; ++k) {
      const int ex = xx - CX[k], ey = yy - CY[k], ez = zz - CZ[k];
      if (ex < 0 || ex >= nelx || ey < 0 || ey >= nely || ez < 0 || ez >= nelz) continue;
      const double* A = ae + (((int64_t)ez * nelx + ex) * nely + ey) * 576;
      for (int j = 0; j < 8; ++j) {
        const int d = (CZ[j] - CZ[k] + 1) * 9 + (CX[j] - CX[k] + 1) * 3 + (CY[j] - CY[k] + 1);
        for (int ci = 0; ci < 3; ++ci)
          for (int cj = 0; cj < 3; ++cj)
            stencil[((int64_t)(d * 3 + ci) * 3 + cj) * nn + N] += A[(3 * k + ci) * 24 + 3 * j + cj];
      }
    }
  }
}

/* stencil operator: mode 0 y = A u, 1 y = b - A u, 2 y = u + omega dinv (b - A u) */
void stencil_apply(int nelx, int nely, int nelz, const double* S, const double* u, double* y,
                   const double* b, const double* dinv, double omega, int mode) {
  const int nnx = nelx + 1, nny = nely + 1, nnz = nelz + 1;
  const int64_t nn = (int64_t)nnx * nny * nnz;
#pragma omp parallel for schedule(static)
  for (int64_t N = 0; N < nn; ++N) {
    const int yy = (int)(N % nny), xx = (int)((N / nny) % nnx), zz = (int)(N / ((int64_t)nny * nnx));
    double acc[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < 27; ++d) {
      const int dy = d % 3 - 1, dx = (d / 3) % 3 - 1, dz = d / 9 - 1;
      const int X = xx + dx, Y = yy + dy, Z = zz + dz;
      if (X < 0 || X >= nnx || Y < 0 || Y >= nny || Z < 0 || Z >= nnz) continue;
      const int64_t M = ((int64_t)Z * nnx + X) * nny + Y;
      for (int ci = 0; ci < 3; ++ci)
        for (int cj = 0; cj < 3; ++cj)
          acc[ci] += S[((int64_t)(d * 3 + ci) * 3 + cj) * nn + N] * u[3 * M + cj];
    }
    for (int c = 0; c < 3; ++c) {
      const int64_t i = 3 * N + c;
      if (mode == 0) y[i] = acc[c];
      else if (mode == 1) y[i] = b[i] - acc[c];
      else y[i] = u[i] + omega * dinv[i] * (b[i] - acc[c]);
    }
  }
}

/* inverse diagonal of a stencil operator (0 where the diagonal is 0: fixed DOFs) */
void stencil_dinv(int nelx, int nely, int nelz, const double* S, double* dinv) {
  const int64_t nn = (int64_t)(nelx + 1) * (nely + 1) * (nelz + 1);
#pragma omp parallel for schedule(static)
  for (int64_t N = 0; N < nn; ++N)
    for (int c = 0; c < 3; ++c) {
      const double d = S[((int64_t)(13 * 3 + c) * 3 + c) * nn + N];
      dinv[3 * N + c] = d != 0.0 ? 1.0 / d : 0.0;
    }
}

/* 1-D weight of fine coordinate x from coarse coordinate X (stride 2) */
static double tw(int x, int X) {
  const int d = x - 2 * X;
  return d == 0 ? 1.0 : ((d == 1 || d == -1) ? 0.5 : 0.0);
}

/* x_f += Pt x_c (fine grid (nelx, nely, nelz), masks fixf / fixc) */
void prolong_add(int nelx, int nely, int nelz, const uint8_t* fixf, const uint8_t* fixc,
                 const double* xc, double* xf) {
  const int nnx = nelx + 1, nny = nely + 1, nnz = nelz + 1;
  const int cnx = nelx / 2 + 1, cny = nely / 2 + 1;
  const int64_t nn = (int64_t)nnx * nny * nnz;
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nn; ++n) {
    const int yy = (int)(n % nny), xx = (int)((n / nny) % nnx), zz = (int)(n / ((int64_t)nny * nnx));
    double acc[3] = {0.0, 0.0, 0.0};
    for (int Z = zz / 2; Z <= (zz + 1) / 2; ++Z)
      for (int X = xx / 2; X <= (xx + 1) / 2; ++X)
        for (int Y = yy / 2; Y <= (yy + 1) / 2; ++Y) {
          const double w = tw(xx, X) * tw(yy, Y) * tw(zz, Z);
          if (w == 0.0) continue;
          const int64_t N = ((int64_t)Z * cnx + X) * cny + Y;
          for (int c = 0; c < 3; ++c)
            if (!((fixc[N] >> c) & 1)) acc[c] += w * xc[3 * N + c];
        }
    for (int c = 0; c < 3; ++c)
      if (!((fixf[n] >> c) & 1)) xf[3 * n + c] += acc[c];
  }
}

/* b_c = Pt^T r_f */
void restrict_(int nelx, int nely, int nelz, const uint8_t* fixf, const uint8_t* fixc,
               const double* rf, double* bc) {
  const int nnx = nelx + 1, nny = nely + 1, nnz = nelz + 1;
  const int cnx = nelx / 2 + 1, cny = nely / 2 + 1, cnz = nelz / 2 + 1;
  const int64_t ncn = (int64_t)cnx * cny * cnz;
#pragma omp parallel for schedule(static)
  for (int64_t N = 0; N < ncn; ++N) {
    const int Y = (int)(N % cny), X = (int)((N / cny) % cnx), Z = (int)(N / ((int64_t)cny * cnx));
    double acc[3] = {0.0, 0.0, 0.0};
    for (int z = 2 * Z - 1; z <= 2 * Z + 1; ++z) {
      if (z < 0 || z >= nnz) continue;
      for (int x = 2 * X - 1; x <= 2 * X + 1; ++x) {
        if (x < 0 || x >= nnx) continue;
        for (int y = 2 * Y - 1; y <= 2 * Y + 1; ++y) {
          if (y < 0 || y >= nny) continue;
          const double w = tw(x, X) * tw(y, Y) * tw(z, Z);
          const int64_t n = ((int64_t)z * nnx + x) * nny + y;
          for (int c = 0; c < 3; ++c)
            if (!((fixf[n] >> c) & 1)) acc[c] += w * rf[3 * n + c];
        }
      }
    }
    for (int c = 0; c < 3; ++c) bc[3 * N + c] = ((fixc[N] >> c) & 1) ? 0.0 : acc[c];
  }
}

/* element compliances ce_e = u_e^T KE u_e (u masked) */
void hex8_ce(int nelx, int nely, int nelz, const double* KE, const double* u, double* ce) {
  const int nnx = nelx + 1, nny = nely + 1;
  const int64_t nel = (int64_t)nelx * nely * nelz;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nel; ++e) {
    const int ey = (int)(e % nely), ex = (int)((e / nely) % nelx), ez = (int)(e / ((int64_t)nely * nelx));
    double ue[24];
    for (int j = 0; j < 8; ++j) {
      const int64_t m = ((int64_t)(ez + CZ[j]) * nnx + (ex + CX[j])) * nny + (ey + CY[j]);
      for (int c = 0; c < 3; ++c) ue[3 * j + c] = u[3 * m + c];
    }
    double t = 0.0;
    for (int i = 0; i < 24; ++i) {
      double r = 0.0;
      for (int j = 0; j < 24; ++j) r += KE[i * 24 + j] * ue[j];
      t += ue[i] * r;
    }
    ce[e] = t;
  }
}

/* dot product in fixed chunks summed in order (reproducible for a fixed
 * thread count) */
double vec_dot(int64_t n, const double* a, const double* b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* y = a x + b y */
void vec_axpby(int64_t n, double a, const double* x, double b, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i] = a * x[i] + b * y[i];
}

/* y = a d .* x */
void vec_scale_mul(int64_t n, double a, const double* d, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i] = a * d[i] * x[i];
}

/* y = A x for a dense row-major n x n matrix (the coarsest inverse) */
void dense_matvec(int64_t n, const double* A, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double t = 0.0;
    for (int64_t j = 0; j < n; ++j) t += A[i * n + j] * x[j];
    y[i] = t;
  }
}

/* threads the OpenMP loops above use */
int cgmg_threads(void) { return omp_get_max_threads(); }
