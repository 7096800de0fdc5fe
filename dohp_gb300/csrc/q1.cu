// Q1-embedded preconditioning matrix on the device: symbolic CSR, numeric assembly, SpMV.
//
// The matrix is the one EllipJacobian (src/fs/tests/ellip.c:474-536) assembles: SPARSE quadrature (two
// Gauss points per GLL sub-interval, tensorquad.c:32-49) tiled into 2x2x2-point patches, Q1 basis on every
// GLL sub-cell (dEFSGetExplicitSparse_Tensor_Hex, efstopo.c:660-717: derivative with respect to the unit
// sub-cell coordinate), rows/columns mapped through E with Dirichlet rows/columns dropped
// (dFSMatSetValuesBlockedExpanded, fs.c:826-930 with negative global indices for Dirichlet nodes).
//
// Device layout: CSR over explicit scalar dofs with sorted columns. Assembly is owner-computes: each
// patch matrix is formed once (phase 1), then every row sums the patches that touch it in ascending
// (element, patch) order (phase 2) -- the same order in which MatSetValues(ADD) receives them, with no
// atomics, so the result is deterministic.
#include <algorithm>

#include "internal.h"

using namespace dgb;

dErr device_exclusive_scan(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s, int64_t *total);

namespace {

constexpr int MAXCOLS = 64;

__device__ __forceinline__ int64_t find_elem(const int32_t *xstart, int64_t nelem, int64_t x) {
  int64_t lo = 0, hi = nelem;  // largest e with xstart[e] <= x
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (xstart[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// visit the patches touching row r in ascending (element, patch) order:
// f(e, pidx, corner, px, py, pz, local node (a,b,c) of the patch origin)
template <typename F>
__device__ __forceinline__ void for_row_patches(int64_t r, const int32_t *et_ptr, const int32_t *et_idx, const int32_t *xstart,
                                                const int32_t *edeg, int64_t nelem, F f) {
  for (int32_t k = et_ptr[r]; k < et_ptr[r + 1]; k++) {
    const int64_t x = et_idx[k];
    const int64_t e = find_elem(xstart, nelem, x);
    const int px = edeg[3 * e], py = edeg[3 * e + 1], pz = edeg[3 * e + 2];
    const int loc = (int)(x - xstart[e]);
    const int a = loc / ((py + 1) * (pz + 1)), b = (loc / (pz + 1)) % (py + 1), c = loc % (pz + 1);
    for (int i = a - 1; i <= a; i++) {
      if (i < 0 || i >= px) continue;
      for (int j = b - 1; j <= b; j++) {
        if (j < 0 || j >= py) continue;
        for (int l = c - 1; l <= c; l++) {
          if (l < 0 || l >= pz) continue;
          const int corner = ((a - i) * 2 + (b - j)) * 2 + (c - l);
          f(e, (i * py + j) * pz + l, corner, px, py, pz, i, j, l);
        }
      }
    }
  }
}

__global__ void k_q1_symbolic(int64_t n, const int32_t *et_ptr, const int32_t *et_idx, const int32_t *xstart, const int32_t *edeg,
                              int64_t nelem, const int32_t *emap, const int32_t *rowptr, int32_t *counts, int32_t *cols,
                              int *overflow) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  int32_t set[MAXCOLS];
  int cnt = 0;
  for_row_patches(r, et_ptr, et_idx, xstart, edeg, nelem, [&](int64_t e, int, int, int, int py, int pz, int i, int j, int l) {
    for (int b = 0; b < 8; b++) {
      const int bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
      const int32_t col = emap[xstart[e] + ((i + bi) * (py + 1) + j + bj) * (pz + 1) + l + bk];
      if (col >= n) continue;
      int pos = cnt;
      while (pos > 0 && set[pos - 1] > col) pos--;
      if (pos > 0 && set[pos - 1] == col) continue;
      if (cnt == MAXCOLS) {
        *overflow = 1;
        continue;
      }
      for (int t = cnt; t > pos; t--) set[t] = set[t - 1];
      set[pos] = col;
      cnt++;
    }
  });
  if (!rowptr) {
    counts[r] = cnt;
  } else {
    for (int t = 0; t < cnt; t++) cols[rowptr[r] + t] = set[t];
  }
}

__device__ __forceinline__ double grf_eval_dev(const double *grf, const double x[3]) {
  const int nf = (int)grf[0];
  const double *w = grf + 3, *b = grf + 3 + 3 * nf;
  double s = 0;
  for (int f = 0; f < nf; f++) s += cos(w[3 * f] * x[0] + w[3 * f + 1] * x[1] + w[3 * f + 2] * x[2] + b[f]);
  return sqrt(2.0 * grf[1] / nf) * s;
}

__device__ __forceinline__ double inv3(const double a[9], double b[9]) {
  const double c0 = a[4] * a[8] - a[7] * a[5], c3 = -(a[3] * a[8] - a[6] * a[5]), c6 = a[3] * a[7] - a[6] * a[4];
  const double det = a[0] * c0 + a[1] * c3 + a[2] * c6, id = 1.0 / det;
  b[0] = id * c0;
  b[1] = -id * (a[1] * a[8] - a[7] * a[2]);
  b[2] = id * (a[1] * a[5] - a[4] * a[2]);
  b[3] = id * c3;
  b[4] = id * (a[0] * a[8] - a[6] * a[2]);
  b[5] = -id * (a[0] * a[5] - a[3] * a[2]);
  b[6] = id * c6;
  b[7] = -id * (a[0] * a[7] - a[6] * a[1]);
  b[8] = id * (a[0] * a[4] - a[3] * a[1]);
  return det;
}

// coordinates and Jacobian of the Q1 map at (s,t,u)
__device__ __forceinline__ void q1_map(const double *X, double s, double t, double u, double xo[3], double J[9]) {
  const double bs[2] = {0.5 * (1 - s), 0.5 * (1 + s)}, bt[2] = {0.5 * (1 - t), 0.5 * (1 + t)}, bu[2] = {0.5 * (1 - u), 0.5 * (1 + u)};
  for (int i = 0; i < 9; i++) J[i] = 0;
  xo[0] = xo[1] = xo[2] = 0;
  for (int v = 0; v < 8; v++) {
    const int a = v >> 2, b = (v >> 1) & 1, c = v & 1;
    const double da = a ? 0.5 : -0.5, db = b ? 0.5 : -0.5, dc = c ? 0.5 : -0.5;
    const double g0 = da * bt[b] * bu[c], g1 = bs[a] * db * bu[c], g2 = bs[a] * bt[b] * dc, ph = bs[a] * bt[b] * bu[c];
    for (int d = 0; d < 3; d++) {
      const double x = X[v * 3 + d];
      xo[d] += x * ph;
      J[d * 3 + 0] += x * g0;
      J[d * 3 + 1] += x * g1;
      J[d * 3 + 2] += x * g2;
    }
  }
}

struct SparseRules {
  double x[MAXP][2 * (MAXP - 1)], w[MAXP][2 * (MAXP - 1)];  // [p][2p points]
};

// Scalar patch matrices K[i][j] = sum_q w k dphi_i . dphi_j (EllipJacobian, ellip.c:474-536) and, for the
// p-Laplacian Jacobian (dref != NULL: the state's reference gradient at every SPARSE point, element-natural per element,
// 8 points per patch, elements back to back), the store of EllipPointwiseComputeStore (ellip.c:333-342) at the patch
// point with K[i][j] = sum_q dphi_i . (w eta dphi_j - w (s . dphi_j) s) (EllipPointwiseJacobian, ellip.c:369-377).
// Two phases for a chunk of elements whose SPARSE points are [t0, t0 + nt) (point index = pstart[e] * 8 +
// element-natural index):
//   k_q1_points: one thread per point: J^-1 and w det J (times k) at the point, and the p-Laplacian store from the
//                state's gradient mapped by that J^-1; every point is computed once;
//   k_q1_patchK: one 64-thread group per patch reads its 8 points (J^-1 at the reference's quirk index pidx*8+q when
//                quirk is set) and forms the 8 x 8 matrix.
// T is the arithmetic: double (the assembled preconditioner of FP64 solves) or float (FP32 / BF16 preconditioning).
template <typename T>
struct PointData {
  T *w, *ji, *st;  // [nt], [9][nt], [4][nt] (SoA over the chunk's points)
};

template <typename T>
__global__ void __launch_bounds__(256) k_q1_points(int64_t e0, int64_t e1, const int32_t *edeg, const int64_t *pstart, const double *coords,
                                                   const SparseRules *rules, const double *grf, const double *dref, double pe, double eps,
                                                   int64_t t0, int64_t nt, PointData<T> P) {
  const int64_t tl = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tl >= nt) return;
  const int64_t t = t0 + tl;
  int64_t lo = e0, hi = e1;  // element of point t: largest e with pstart[e] * 8 <= t
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (pstart[mid] * 8 <= t) lo = mid;
    else hi = mid;
  }
  const int64_t e = lo;
  const int px = edeg[3 * e], py = edeg[3 * e + 1], pz = edeg[3 * e + 2];
  const int a = (int)(t - pstart[e] * 8), Qy = 2 * py, Qz = 2 * pz;
  const int ai = a / (Qy * Qz), aj = (a / Qz) % Qy, ak = a % Qz;
  double xo[3], J[9], Ji[9];
  q1_map(coords + e * 24, rules->x[px][ai], rules->x[py][aj], rules->x[pz][ak], xo, J);
  const double det = inv3(J, Ji);
  double w = rules->w[px][ai] * rules->w[py][aj] * rules->w[pz][ak] * det;
  if (grf) w *= exp(grf_eval_dev(grf, xo));
  P.w[tl] = (T)w;
  for (int i = 0; i < 9; i++) P.ji[i * nt + tl] = (T)Ji[i];
  if (dref) {
    const double *dr = dref + t * 3;
    double Du[3];
    for (int c = 0; c < 3; c++) Du[c] = dr[0] * Ji[0 * 3 + c] + dr[1] * Ji[1 * 3 + c] + dr[2] * Ji[2 * 3 + c];
    const double gamma = 0.5 * (Du[0] * Du[0] + Du[1] * Du[1] + Du[2] * Du[2]);
    const double espg = eps * eps + gamma, eta = pow(espg, (pe - 2) / 2);
    const double sm = sqrt(-((pe - 2) / 2) * eta / espg);
    P.st[tl] = (T)eta;
    for (int c = 0; c < 3; c++) P.st[(1 + c) * nt + tl] = (T)(sm * Du[c]);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_q1_patchK(int64_t e0, int64_t e1, const int32_t *edeg, const int64_t *pstart, int quirk, bool plap,
                                                   int64_t p0, int64_t np, int64_t t0, int64_t nt, PointData<T> P, double *K) {
  __shared__ T sW[4][8], sDer[4][8][8][3], sSt[4][8][4];
  const int g = threadIdx.x >> 6, lt = threadIdx.x & 63;
  const int64_t gp = p0 + (int64_t)blockIdx.x * 4 + g;
  const bool active = gp < p0 + np;
  int64_t e = e0;
  int py = 1, pz = 1, pidx = 0;
  if (active) {
    int64_t lo = e0, hi = e1;
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (pstart[mid] <= gp) lo = mid;
      else hi = mid;
    }
    e = lo;
    py = edeg[3 * e + 1], pz = edeg[3 * e + 2];
    pidx = (int)(gp - pstart[e]);
  }
  const int pi = pidx / (py * pz), pj = (pidx / pz) % py, pk = pidx % pz;
  const int Qy = 2 * py, Qz = 2 * pz;
  const T I1[2][2] = {{(T)0.78867513459481287, (T)0.21132486540518713}, {(T)0.21132486540518713, (T)0.78867513459481287}};
  const T D1[2][2] = {{-1, 1}, {-1, 1}};
  const int64_t ebase = pstart[e] * 8 - t0;  // the element's first point in the chunk arrays
  if (active && lt < 8) {
    const int q = lt, qi = q >> 2, qj = (q >> 1) & 1, qk = q & 1;
    const int64_t a = ebase + ((2 * pi + qi) * Qy + 2 * pj + qj) * Qz + 2 * pk + qk;
    sW[g][q] = P.w[a];
    if (plap)
      for (int c = 0; c < 4; c++) sSt[g][q][c] = P.st[c * nt + a];
  }
  __syncthreads();
  if (active) {
    const int q = lt >> 3, b = lt & 7, qi = q >> 2, qj = (q >> 1) & 1, qk = q & 1, bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
    const T dX = D1[qi][bi] * I1[qj][bj] * I1[qk][bk], dY = I1[qi][bi] * D1[qj][bj] * I1[qk][bk], dZ = I1[qi][bi] * I1[qj][bj] * D1[qk][bk];
    // inverse Jacobian: the patch point's own, or the one at element-natural index pidx*8+q (efstopo.c:700)
    const int64_t aj = quirk ? ebase + pidx * 8 + q : ebase + ((2 * pi + qi) * Qy + 2 * pj + qj) * Qz + 2 * pk + qk;
    T Ji[9];
    for (int i = 0; i < 9; i++) Ji[i] = P.ji[i * nt + aj];
    for (int d = 0; d < 3; d++) sDer[g][q][b][d] = dX * Ji[0 * 3 + d] + dY * Ji[1 * 3 + d] + dZ * Ji[2 * 3 + d];
  }
  __syncthreads();
  if (active) {
    const int i = lt >> 3, j = lt & 7;
    T s = 0;
    for (int q = 0; q < 8; q++) {
      const T w = sW[g][q];
      T dv0, dv1, dv2;
      if (plap) {
        const T *st = sSt[g][q], *dj = sDer[g][q][j];
        const T dotw = (st[1] * dj[0] + st[2] * dj[1] + st[3] * dj[2]) * w, etaw = st[0] * w;
        dv0 = etaw * dj[0] - dotw * st[1];
        dv1 = etaw * dj[1] - dotw * st[2];
        dv2 = etaw * dj[2] - dotw * st[3];
      } else {
        dv0 = w * sDer[g][q][j][0], dv1 = w * sDer[g][q][j][1], dv2 = w * sDer[g][q][j][2];
      }
      s += sDer[g][q][i][0] * dv0 + sDer[g][q][i][1] * dv1 + sDer[g][q][i][2] * dv2;
    }
    K[gp * 64 + lt] = (double)s;
  }
}

// phase 2: each explicit row sums its patches in ascending (element, patch) order
__global__ void k_q1_rows(int64_t n, const int32_t *et_ptr, const int32_t *et_idx, const int32_t *xstart, const int32_t *edeg,
                          int64_t nelem, const int64_t *pstart, const int32_t *emap, const double *K, const int32_t *rowptr,
                          const int32_t *cols, double *vals) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t r0 = rowptr[r], r1 = rowptr[r + 1];
  for (int32_t t = r0; t < r1; t++) vals[t] = 0;
  for_row_patches(r, et_ptr, et_idx, xstart, edeg, nelem, [&](int64_t e, int pidx, int corner, int, int py, int pz, int i, int j, int l) {
    const double *Kp = K + (pstart[e] + pidx) * 64 + corner * 8;
    for (int b = 0; b < 8; b++) {
      const int bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
      const int32_t col = emap[xstart[e] + ((i + bi) * (py + 1) + j + bj) * (pz + 1) + l + bk];
      if (col >= n) continue;
      int lo = r0, hi = r1 - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cols[mid] < col) lo = mid + 1;
        else hi = mid;
      }
      vals[lo] += Kp[b];
    }
  });
}

// ElastJacobian patch matrices (elast.c:343-407 with ElastPointwiseJacobian at F = I, elast.c:269-280):
// K[i*3+fi][j*3+fj] = sum_q dphi_i . dv(fi), dv = w (lambda tr(eps) I + 2 mu eps), eps = sym(e_fj dphi_j^T).
// One 64-thread group per patch, thread (i, j) forms the 3 x 3 block; patches [p0, p0 + np) of the chunk.
__global__ void __launch_bounds__(256) k_q1_patch_elast(int64_t nelem, const int32_t *edeg, const int64_t *pstart, const double *coords,
                                                        const SparseRules *rules, int quirk, int64_t p0, int64_t np, double lam,
                                                        double mu, double *K) {
  __shared__ double sJ[4][8][9], sW[4][8], sDer[4][8][8][3];
  const int g = threadIdx.x >> 6, lt = threadIdx.x & 63;
  const int64_t gp = p0 + (int64_t)blockIdx.x * 4 + g;
  const bool active = gp < p0 + np;
  int64_t e = 0;
  int px = 1, py = 1, pz = 1, pidx = 0;
  if (active) {
    int64_t lo = 0, hi = nelem;
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (pstart[mid] <= gp) lo = mid;
      else hi = mid;
    }
    e = lo;
    px = edeg[3 * e], py = edeg[3 * e + 1], pz = edeg[3 * e + 2];
    pidx = (int)(gp - pstart[e]);
  }
  const int pi = pidx / (py * pz), pj = (pidx / pz) % py, pk = pidx % pz;
  const double I1[2][2] = {{0.78867513459481287, 0.21132486540518713}, {0.21132486540518713, 0.78867513459481287}};
  const double D1[2][2] = {{-1., 1.}, {-1., 1.}};
  if (active && lt < 8) {
    const int q = lt, qi = q >> 2, qj = (q >> 1) & 1, qk = q & 1;
    const double *X = coords + e * 24;
    const int ai = 2 * pi + qi, aj = 2 * pj + qj, ak = 2 * pk + qk;
    double xo[3], J[9], Ji[9];
    q1_map(X, rules->x[px][ai], rules->x[py][aj], rules->x[pz][ak], xo, J);
    const double det = inv3(J, Ji);
    sW[g][q] = rules->w[px][ai] * rules->w[py][aj] * rules->w[pz][ak] * det;
    if (quirk) {  // inverse Jacobian read at element-natural index pidx*8+q (efstopo.c:700)
      const int t = pidx * 8 + q, Qy = 2 * py, Qz = 2 * pz;
      const int ti = t / (Qy * Qz), tj = (t / Qz) % Qy, tk = t % Qz;
      q1_map(X, rules->x[px][ti], rules->x[py][tj], rules->x[pz][tk], xo, J);
      inv3(J, Ji);
    }
    for (int i = 0; i < 9; i++) sJ[g][q][i] = Ji[i];
  }
  __syncthreads();
  if (active) {
    const int q = lt >> 3, b = lt & 7, qi = q >> 2, qj = (q >> 1) & 1, qk = q & 1, bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
    const double dX = D1[qi][bi] * I1[qj][bj] * I1[qk][bk], dY = I1[qi][bi] * D1[qj][bj] * I1[qk][bk], dZ = I1[qi][bi] * I1[qj][bj] * D1[qk][bk];
    const double *Ji = sJ[g][q];
    for (int d = 0; d < 3; d++) sDer[g][q][b][d] = dX * Ji[0 * 3 + d] + dY * Ji[1 * 3 + d] + dZ * Ji[2 * 3 + d];
  }
  __syncthreads();
  if (!active) return;
  const int i = lt >> 3, j = lt & 7;
  double blk[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int q = 0; q < 8; q++) {
    const double w = sW[g][q], *Di = sDer[g][q][i], *Dj = sDer[g][q][j];
    for (int fj = 0; fj < 3; fj++) {
      double du[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int c = 0; c < 3; c++) du[fj * 3 + c] = Dj[c];
      const double dE[6] = {du[0], du[4], du[8], 0.5 * (du[1] + du[3]), 0.5 * (du[2] + du[6]), 0.5 * (du[5] + du[7])};
      const double tr = dE[0] + dE[1] + dE[2];
      double dS[6];
      for (int k = 0; k < 6; k++) dS[k] = lam * tr * (k < 3) + 2 * mu * dE[k];
      const double dv[9] = {dS[0] * w, dS[3] * w, dS[4] * w, dS[3] * w, dS[1] * w, dS[5] * w, dS[4] * w, dS[5] * w, dS[2] * w};
      for (int fi = 0; fi < 3; fi++) blk[fi][fj] += Di[0] * dv[fi * 3] + Di[1] * dv[fi * 3 + 1] + Di[2] * dv[fi * 3 + 2];
    }
  }
  double *Kp = K + (gp - p0) * 576;
  for (int fi = 0; fi < 3; fi++)
    for (int fj = 0; fj < 3; fj++) Kp[(i * 3 + fi) * 24 + j * 3 + fj] = blk[fi][fj];
}

// each node row adds the 3 x 3 blocks of its patches in [p0, p0 + np), in ascending (element, patch) order
__global__ void k_q1_rows_elast(int64_t n, const int32_t *et_ptr, const int32_t *et_idx, const int32_t *xstart, const int32_t *edeg,
                                int64_t nelem, const int64_t *pstart, const int32_t *emap, const double *K, int64_t p0, int64_t np,
                                const int32_t *srp, const int32_t *scol, const int32_t *rowptr, double *vals) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t s0 = srp[r], s1 = srp[r + 1], cnt = s1 - s0;
  for_row_patches(r, et_ptr, et_idx, xstart, edeg, nelem, [&](int64_t e, int pidx, int corner, int, int py, int pz, int i, int j, int l) {
    const int64_t gp = pstart[e] + pidx;
    if (gp < p0 || gp >= p0 + np) return;
    const double *Kp = K + (gp - p0) * 576;
    for (int b = 0; b < 8; b++) {
      const int bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
      const int32_t col = emap[xstart[e] + ((i + bi) * (py + 1) + j + bj) * (pz + 1) + l + bk];
      if (col >= n) continue;
      int lo = s0, hi = s1 - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (scol[mid] < col) lo = mid + 1;
        else hi = mid;
      }
      const int k = lo - s0;
      for (int fi = 0; fi < 3; fi++)
        for (int fj = 0; fj < 3; fj++) vals[rowptr[3 * r + fi] + 3 * k + fj] += Kp[(corner * 3 + fi) * 24 + b * 3 + fj];
    }
  });
  (void)cnt;
}

}  // namespace

// blocked pattern (bs = 3): node row r, component fi -> columns 3 c + fj for the node columns c of r
__global__ void k_expand_pattern(int64_t n, const int32_t *__restrict__ srp, const int32_t *__restrict__ scol,
                                 int32_t *__restrict__ rp, int32_t *__restrict__ col) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t s0 = srp[r], cnt = srp[r + 1] - s0;
  for (int fi = 0; fi < 3; fi++) {
    const int32_t base = 9 * s0 + fi * 3 * cnt;
    rp[3 * r + fi] = base;
    for (int k = 0; k < cnt; k++)
      for (int fj = 0; fj < 3; fj++) col[base + 3 * k + fj] = 3 * scol[s0 + k] + fj;
  }
  if (r == n - 1) rp[3 * n] = 9 * srp[n];
}

dErr q1_symbolic(_p_dFS *fs, _p_dMat *J) {
  if (fs->bs != 1 && fs->bs != 3) return set_error("Q1 matrix for block size %d not built", fs->bs);
  // rows and columns go through E as a node map (dFSMatSetValuesBlockedExpanded, fs.c:826-930), which needs
  // one closure node per expanded node: conforming spaces (the reference errors on p-nonconforming ones)
  if (!fs->boolean_e) return set_error("Q1-embedded matrix needs a conforming space (Boolean E)");
  const int64_t n = fs->n;
  J->nrows = n;
  CUCHK(cudaMalloc(&J->d_rowptr, (n + 1) * sizeof(int32_t)));
  int32_t *counts;
  int *d_over;
  CUCHK(cudaMalloc(&counts, std::max<int64_t>(n, 1) * sizeof(int32_t)));
  CUCHK(cudaMalloc(&d_over, sizeof(int)));
  CUCHK(cudaMemsetAsync(d_over, 0, sizeof(int), fs->stream));
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (n) {
    k_q1_symbolic<<<grid, 128, 0, fs->stream>>>(n, fs->d_et_ptr, fs->d_et_idx, fs->d_xstart, fs->d_edeg, fs->nelem, fs->d_emap,
                                                nullptr, counts, nullptr, d_over);
    CUCHK(cudaGetLastError());
  }
  int64_t nnz = 0;
  DCHK(device_exclusive_scan(counts, J->d_rowptr, n, fs->stream, &nnz));
  if (nnz > INT32_MAX) return set_error("Q1 matrix has %lld nonzeros, beyond 32-bit CSR", (long long)nnz);
  J->nnz = nnz;
  CUCHK(cudaMalloc(&J->d_col, std::max<int64_t>(nnz, 1) * sizeof(int32_t)));
  CUCHK(cudaMalloc(&J->d_val, std::max<int64_t>(nnz, 1) * sizeof(double)));
  if (n) {
    k_q1_symbolic<<<grid, 128, 0, fs->stream>>>(n, fs->d_et_ptr, fs->d_et_idx, fs->d_xstart, fs->d_edeg, fs->nelem, fs->d_emap,
                                                J->d_rowptr, counts, J->d_col, d_over);
    CUCHK(cudaGetLastError());
  }
  int over = 0;
  CUCHK(cudaMemcpyAsync(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost, fs->stream));
  CUCHK(cudaStreamSynchronize(fs->stream));
  cudaFree(counts);
  cudaFree(d_over);
  if (over) return set_error("Q1 row with more than %d columns", MAXCOLS);
  if (fs->bs == 3) {  // keep the node pattern, expand to the interleaved 3 x 3 blocked CSR
    J->bs = 3;
    J->snnz = J->nnz;
    J->d_srowptr = J->d_rowptr, J->d_scol = J->d_col;
    cudaFree(J->d_val);
    J->nrows = 3 * n;
    J->nnz = 9 * J->snnz;
    if (J->nnz > INT32_MAX) return set_error("blocked Q1 matrix has %lld nonzeros, beyond 32-bit CSR", (long long)J->nnz);
    CUCHK(cudaMalloc(&J->d_rowptr, (3 * n + 1) * sizeof(int32_t)));
    CUCHK(cudaMalloc(&J->d_col, std::max<int64_t>(J->nnz, 1) * sizeof(int32_t)));
    CUCHK(cudaMalloc(&J->d_val, std::max<int64_t>(J->nnz, 1) * sizeof(double)));
    if (n) {
      k_expand_pattern<<<(unsigned)((n + 127) / 128), 128, 0, fs->stream>>>(n, J->d_srowptr, J->d_scol, J->d_rowptr, J->d_col);
      CUCHK(cudaGetLastError());
    }
    CUCHK(cudaStreamSynchronize(fs->stream));
  }
  return 0;
}

template <typename T>
static dErr q1_patches_two_phase(_p_dFS *fs, const std::vector<int64_t> &pstart, const int64_t *d_pstart, const SparseRules *d_rules,
                                 const double *d_grf, int quirk, const double *dref, double pe, double eps, double *d_K) {
  // chunks of whole elements with at most kPts SPARSE points, so the point arrays stay near 1 GB
  constexpr int64_t kPts = 1 << 24;
  const int64_t npt = pstart[fs->nelem] * 8, cap = std::min<int64_t>(std::max<int64_t>(npt, 1), kPts);
  PointData<T> P;
  T *buf;
  CUCHK(cudaMalloc(&buf, (size_t)cap * 14 * sizeof(T)));
  P.w = buf, P.ji = buf + cap, P.st = buf + 10 * cap;
  dErr err = 0;
  for (int64_t e0 = 0; e0 < fs->nelem && !err;) {
    int64_t e1 = e0 + 1;
    while (e1 < fs->nelem && (pstart[e1 + 1] - pstart[e0]) * 8 <= cap) e1++;
    const int64_t t0 = pstart[e0] * 8, nt = (pstart[e1] - pstart[e0]) * 8;
    if (nt > cap) {
      err = set_error("Q1 assembly: one element has more SPARSE points than the chunk");
      break;
    }
    PointData<T> Pc = {P.w, P.ji, P.st};
    k_q1_points<T><<<(unsigned)((nt + 255) / 256), 256, 0, fs->stream>>>(e0, e1, fs->d_edeg, d_pstart, fs->d_coords, d_rules, d_grf, dref, pe,
                                                                          eps, t0, nt, Pc);
    if (cudaGetLastError() != cudaSuccess) err = set_error("k_q1_points launch failed");
    const int64_t p0 = pstart[e0], np = pstart[e1] - pstart[e0];
    if (!err && np) {
      k_q1_patchK<T><<<(unsigned)((np + 3) / 4), 256, 0, fs->stream>>>(e0, e1, fs->d_edeg, d_pstart, quirk, dref != nullptr, p0, np, t0, nt, Pc,
                                                                        d_K);
      if (cudaGetLastError() != cudaSuccess) err = set_error("k_q1_patchK launch failed");
    }
    e0 = e1;
  }
  CUCHK(cudaStreamSynchronize(fs->stream));
  cudaFree(buf);
  return err;
}

dErr q1_numeric(_p_dFS *fs, _p_dMat *J, const double *grf_host, int quirk, const double *dref, double pe, double eps, bool single) {
  std::vector<int64_t> pstart(fs->nelem + 1, 0);
  for (int64_t e = 0; e < fs->nelem; e++)
    pstart[e + 1] = pstart[e] + (int64_t)fs->edeg[3 * e] * fs->edeg[3 * e + 1] * fs->edeg[3 * e + 2];
  const int64_t np = pstart[fs->nelem];
  SparseRules h;
  for (int p = 1; p < MAXP; p++) rule_1d(dQUADRATURE_METHOD_SPARSE, 2 * p, h.x[p], h.w[p]);
  int64_t *d_pstart;
  SparseRules *d_rules;
  double *d_K, *d_grf = nullptr;
  CUCHK(cudaMalloc(&d_pstart, pstart.size() * sizeof(int64_t)));
  CUCHK(cudaMalloc(&d_rules, sizeof h));
  CUCHK(cudaMalloc(&d_K, std::max<int64_t>(np, 1) * 64 * sizeof(double)));
  CUCHK(cudaMemcpyAsync(d_pstart, pstart.data(), pstart.size() * sizeof(int64_t), cudaMemcpyHostToDevice, fs->stream));
  CUCHK(cudaMemcpyAsync(d_rules, &h, sizeof h, cudaMemcpyHostToDevice, fs->stream));
  if (grf_host) {
    const int nf = (int)grf_host[0];
    CUCHK(cudaMalloc(&d_grf, (3 + 4 * nf) * sizeof(double)));
    CUCHK(cudaMemcpyAsync(d_grf, grf_host, (3 + 4 * nf) * sizeof(double), cudaMemcpyHostToDevice, fs->stream));
  }
  if (np) {
    const dErr e = single ? q1_patches_two_phase<float>(fs, pstart, d_pstart, d_rules, d_grf, quirk, dref, pe, eps, d_K)
                          : q1_patches_two_phase<double>(fs, pstart, d_pstart, d_rules, d_grf, quirk, dref, pe, eps, d_K);
    if (e) {
      cudaFree(d_pstart);
      cudaFree(d_rules);
      cudaFree(d_K);
      cudaFree(d_grf);
      return e;
    }
  }
  if (fs->n) {
    k_q1_rows<<<(unsigned)((fs->n + 127) / 128), 128, 0, fs->stream>>>(fs->n, fs->d_et_ptr, fs->d_et_idx, fs->d_xstart, fs->d_edeg,
                                                                       fs->nelem, d_pstart, fs->d_emap, d_K, J->d_rowptr, J->d_col, J->d_val);
    CUCHK(cudaGetLastError());
  }
  CUCHK(cudaStreamSynchronize(fs->stream));
  cudaFree(d_pstart);
  cudaFree(d_rules);
  cudaFree(d_K);
  cudaFree(d_grf);
  J->sell_valid = false;
  return 0;
}

// blocked (bs = 3) elasticity assembly, in chunks of patches so the patch matrices stay within a few GB
dErr q1_numeric_elast(_p_dFS *fs, _p_dMat *J, double lam, double mu, int quirk) {
  std::vector<int64_t> pstart(fs->nelem + 1, 0);
  for (int64_t e = 0; e < fs->nelem; e++)
    pstart[e + 1] = pstart[e] + (int64_t)fs->edeg[3 * e] * fs->edeg[3 * e + 1] * fs->edeg[3 * e + 2];
  const int64_t np = pstart[fs->nelem], chunk = std::min<int64_t>(std::max<int64_t>(np, 1), 1 << 20);
  SparseRules h;
  for (int p = 1; p < MAXP; p++) rule_1d(dQUADRATURE_METHOD_SPARSE, 2 * p, h.x[p], h.w[p]);
  int64_t *d_pstart;
  SparseRules *d_rules;
  double *d_K;
  CUCHK(cudaMalloc(&d_pstart, pstart.size() * sizeof(int64_t)));
  CUCHK(cudaMalloc(&d_rules, sizeof h));
  CUCHK(cudaMalloc(&d_K, chunk * 576 * sizeof(double)));
  CUCHK(cudaMemcpyAsync(d_pstart, pstart.data(), pstart.size() * sizeof(int64_t), cudaMemcpyHostToDevice, fs->stream));
  CUCHK(cudaMemcpyAsync(d_rules, &h, sizeof h, cudaMemcpyHostToDevice, fs->stream));
  CUCHK(cudaMemsetAsync(J->d_val, 0, std::max<int64_t>(J->nnz, 1) * sizeof(double), fs->stream));
  for (int64_t p0 = 0; p0 < np; p0 += chunk) {
    const int64_t cnp = std::min(chunk, np - p0);
    k_q1_patch_elast<<<(unsigned)((cnp + 3) / 4), 256, 0, fs->stream>>>(fs->nelem, fs->d_edeg, d_pstart, fs->d_coords, d_rules, quirk,
                                                                        p0, cnp, lam, mu, d_K);
    CUCHK(cudaGetLastError());
    if (fs->n) {
      k_q1_rows_elast<<<(unsigned)((fs->n + 127) / 128), 128, 0, fs->stream>>>(fs->n, fs->d_et_ptr, fs->d_et_idx, fs->d_xstart, fs->d_edeg,
                                                                               fs->nelem, d_pstart, fs->d_emap, d_K, p0, cnp, J->d_srowptr,
                                                                               J->d_scol, J->d_rowptr, J->d_val);
      CUCHK(cudaGetLastError());
    }
  }
  CUCHK(cudaStreamSynchronize(fs->stream));
  cudaFree(d_pstart);
  cudaFree(d_rules);
  cudaFree(d_K);
  J->sell_valid = false;
  return 0;
}
