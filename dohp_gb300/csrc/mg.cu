// Geometric multigrid on the Q1-embedded lattice (dPC_MG_Q1): a V-cycle preconditioner for the Q1-embedded
// matrix of a scalar uniform-order space on a block mesh.
//
// The Q1-embedded matrix couples each GLL node with its lattice neighbours only (27-point stencil on the
// lattice of GLL nodes, (M p + 1) nodes per direction). The fine level is that matrix in lattice order, stored as
// 27 coefficient arrays (no column indices); Dirichlet nodes are masked rows. Coarse levels halve the lattice in
// every direction (L -> (L + 1) / 2, L odd) with trilinear prolongation P in index space and Galerkin operators
// P^T A P, which stay 27-point. Smoothing is the project's Chebyshev-Jacobi (the same polynomial as the
// single-level preconditioner, degree and [0.1, 1.1] lambda_max bounds from 20 power steps per level); the
// coarsest level (at most 9 nodes per direction) is solved exactly with a dense inverse built on the host. Pre-
// and post-smoothing use the same polynomial in D^-1 A, so the V-cycle is a symmetric fixed linear operator
// (usable inside CG as well as FGMRES). Deterministic: every kernel writes its own outputs, the eigenvalue
// estimates use the fixed-order reductions of the solver module.
//
// PETSc's PCMG / PCGAMG on the assembled Q1 matrix is what the reference's callers would select for this; the
// method here is the textbook geometric V-cycle (Trottenberg, Oosterlee, Schueller, Multigrid, 2001, ch. 2).
#include <algorithm>
#include <cmath>
#include <vector>

#include <type_traits>

#include "internal.h"

using namespace dgb;

dErr device_dot(int64_t n, const double *a, const double *b, double *part, double *out, cudaStream_t s);
dErr dot_part_alloc(double **part);

namespace {

inline unsigned nbk(int64_t n) { return (unsigned)std::max<int64_t>((n + 255) / 256, 1); }

__device__ __forceinline__ void lat_coord(int64_t i, int Ly, int Lz, int &x, int &y, int &z) {
  z = (int)(i % Lz);
  y = (int)((i / Lz) % Ly);
  x = (int)(i / ((int64_t)Ly * Lz));
}

// CSR (natural dof order, BS interleaved components per node) -> block stencil in lattice order:
// A[((s BS + ci) BS + cj) nl + node]; bad != 0 when a column is not a lattice neighbour
template <int BS>
__global__ void k_stencil_fill(int64_t nrows, const int32_t *__restrict__ rp, const int32_t *__restrict__ col, const double *__restrict__ val,
                               const int32_t *__restrict__ lat, int Ly, int Lz, int64_t nl, double *__restrict__ A, int *bad) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int64_t li = lat[r / BS];
  const int ci = (int)(r % BS);
  int ix, iy, iz;
  lat_coord(li, Ly, Lz, ix, iy, iz);
  for (int32_t k = rp[r]; k < rp[r + 1]; k++) {
    int jx, jy, jz;
    lat_coord(lat[col[k] / BS], Ly, Lz, jx, jy, jz);
    const int cj = col[k] % BS;
    const int dx = jx - ix, dy = jy - iy, dz = jz - iz;
    if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) {
      atomicExch(bad, 1);
      continue;
    }
    const int s = (dx + 1) * 9 + (dy + 1) * 3 + dz + 1;
    A[((int64_t)(s * BS + ci) * BS + cj) * nl + li] = val[k];
  }
}

template <int BS>
__device__ __forceinline__ double center(const double *A, int64_t n, int64_t i, int c) {
  return A[((int64_t)(13 * BS + c) * BS + c) * n + i];
}

template <int BS>
__global__ void k_dinv(int64_t n, const double *__restrict__ A, double *__restrict__ dinv) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * BS) return;
  const double a = center<BS>(A, n, t / BS, (int)(t % BS));
  dinv[t] = a != 0 ? 1.0 / a : 0.0;
}

// y = A x (27-point block stencil), or y = b - A x when b is given; one thread per (node, component)
template <int BS>
__global__ void k_stencil_mv(int Lx, int Ly, int Lz, const double *__restrict__ A, const double *__restrict__ x,
                             const double *__restrict__ b, double *__restrict__ y) {
  const int64_t n = (int64_t)Lx * Ly * Lz;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * BS) return;
  const int64_t i = t / BS;
  const int ci = (int)(t % BS);
  int ix, iy, iz;
  lat_coord(i, Ly, Lz, ix, iy, iz);
  double s = 0;
#pragma unroll
  for (int a = -1; a <= 1; a++)
#pragma unroll
    for (int c = -1; c <= 1; c++)
#pragma unroll
      for (int e = -1; e <= 1; e++) {
        const int jx = ix + a, jy = iy + c, jz = iz + e;
        if (jx < 0 || jx >= Lx || jy < 0 || jy >= Ly || jz < 0 || jz >= Lz) continue;
        const int st = (a + 1) * 9 + (c + 1) * 3 + e + 1;
        const int64_t j = i + ((int64_t)a * Ly + c) * Lz + e;
#pragma unroll
        for (int cj = 0; cj < BS; cj++) s += A[((int64_t)(st * BS + ci) * BS + cj) * n + i] * x[j * BS + cj];
      }
  y[t] = b ? b[t] - s : s;
}

// the symmetric half of a level's stencil: the centre and the 13 forward neighbours (stencil slots 13..26);
// A(i, i - o) is the transpose of A(i - o, i), which node i - o holds as a forward entry
template <int BS>
__global__ void k_sym_extract(int64_t n, const double *__restrict__ A, double *__restrict__ As) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 14 * BS * BS * n) return;
  As[t] = A[13 * BS * BS * n + t];
}

// row (i, ci) of A x from the symmetric half: forward entries of node i, transposed forward entries of the backward
// neighbours; about half the coefficient bytes of the full stencil. 32-bit lattice arithmetic (levels have fewer than
// 2^31 / BS nodes); interior nodes skip the bounds tests
template <int BS, typename T>
__device__ __forceinline__ T sym_row(int Lx, int Ly, int Lz, int i, int ci, int ix, int iy, int iz, const T *__restrict__ As,
                                     const T *__restrict__ x) {
  const int n = Lx * Ly * Lz, Lyz = Ly * Lz;
  T s = 0;
#pragma unroll
  for (int cj = 0; cj < BS; cj++) s += As[(ci * BS + cj) * (int64_t)n + i] * x[i * BS + cj];
  if (ix > 0 && ix < Lx - 1 && iy > 0 && iy < Ly - 1 && iz > 0 && iz < Lz - 1) {
#pragma unroll
    for (int h = 1; h < 14; h++) {
      const int st = 13 + h, a = st / 9 - 1, c = (st / 3) % 3 - 1, e = st % 3 - 1;
      const int o = a * Lyz + c * Lz + e;
#pragma unroll
      for (int cj = 0; cj < BS; cj++) s += As[((h * BS + ci) * BS + cj) * (int64_t)n + i] * x[(i + o) * BS + cj];
#pragma unroll
      for (int cj = 0; cj < BS; cj++) s += As[((h * BS + cj) * BS + ci) * (int64_t)n + (i - o)] * x[(i - o) * BS + cj];
    }
  } else {
#pragma unroll
    for (int h = 1; h < 14; h++) {
      const int st = 13 + h, a = st / 9 - 1, c = (st / 3) % 3 - 1, e = st % 3 - 1;
      const int o = a * Lyz + c * Lz + e;
      const int fx = ix + a, fy = iy + c, fz = iz + e, bx = ix - a, by = iy - c, bz = iz - e;
      if (fx >= 0 && fx < Lx && fy >= 0 && fy < Ly && fz >= 0 && fz < Lz)
#pragma unroll
        for (int cj = 0; cj < BS; cj++) s += As[((h * BS + ci) * BS + cj) * (int64_t)n + i] * x[(i + o) * BS + cj];
      if (bx >= 0 && bx < Lx && by >= 0 && by < Ly && bz >= 0 && bz < Lz)
#pragma unroll
        for (int cj = 0; cj < BS; cj++) s += As[((h * BS + cj) * BS + ci) * (int64_t)n + (i - o)] * x[(i - o) * BS + cj];
    }
  }
  return s;
}

// y = A x (or b - A x) from the symmetric half, one thread per (node, component) in lattice order
template <int BS, typename T>
__global__ void __launch_bounds__(256) k_stencil_mv_sym(int Lx, int Ly, int Lz, const T *__restrict__ As, const T *__restrict__ x,
                                                        const T *__restrict__ b, T *__restrict__ y) {
  const int n = Lx * Ly * Lz, Lyz = Ly * Lz;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * BS) return;
  const int i = t / BS, ci = t - i * BS;
  const int ix = i / Lyz, r = i - ix * Lyz, iy = r / Lz, iz = r - iy * Lz;
  const T s = sym_row<BS, T>(Lx, Ly, Lz, i, ci, ix, iy, iz, As, x);
  y[t] = b ? b[t] - s : s;
}

// the scalar FP32 form on 32 (z) x 8 (y) node tiles of one x plane (grid: z tiles, y tiles, Lx), 8 CTAs per SM:
// neighbour lines of the tile are shared in L1 and more loads are in flight per SM (257^3 lattice: 270 us
// against 345 us for the lattice-order form, the same bits)
__global__ void __launch_bounds__(256, 8) k_stencil_mv_sym_tile(int Lx, int Ly, int Lz, const float *__restrict__ As,
                                                                const float *__restrict__ x, const float *__restrict__ b,
                                                                float *__restrict__ y) {
  const int iz = blockIdx.x * 32 + threadIdx.x, iy = blockIdx.y * 8 + threadIdx.y, ix = blockIdx.z;
  if (iz >= Lz || iy >= Ly) return;
  const int i = (ix * Ly + iy) * Lz + iz;
  const float s = sym_row<1, float>(Lx, Ly, Lz, i, 0, ix, iy, iz, As, x);
  y[i] = b ? b[i] - s : s;
}

// Galerkin coarse operator: Ac(I, J) = sum_{i, j} P(i, I) Af(i, j) P(j, J) block by block, trilinear P in index
// space (the same for every component), coarse nodes whose fine node 2I is masked are masked (rows and
// columns); one thread per (coarse node, block entry)
template <int BS>
__global__ void k_galerkin(int Fx, int Fy, int Fz, int Cx, int Cy, int Cz, const double *__restrict__ Af, double *__restrict__ Ac) {
  const int64_t nc = (int64_t)Cx * Cy * Cz, nf = (int64_t)Fx * Fy * Fz;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nc * BS * BS) return;
  const int64_t I = t / (BS * BS);
  const int ci = (int)((t / BS) % BS), cj = (int)(t % BS);
  int Ix, Iy, Iz;
  lat_coord(I, Cy, Cz, Ix, Iy, Iz);
  auto fidx = [&](int x, int y, int z) { return ((int64_t)x * Fy + y) * Fz + z; };
  auto masked_c = [&](int x, int y, int z) { return center<BS>(Af, nf, fidx(2 * x, 2 * y, 2 * z), 0) == 0.0; };
  double acc[27];
#pragma unroll
  for (int s = 0; s < 27; s++) acc[s] = 0;
  if (!masked_c(Ix, Iy, Iz)) {
    for (int ux = -1; ux <= 1; ux++)
      for (int uy = -1; uy <= 1; uy++)
        for (int uz = -1; uz <= 1; uz++) {
          const int ix = 2 * Ix + ux, iy = 2 * Iy + uy, iz = 2 * Iz + uz;
          if (ix < 0 || ix >= Fx || iy < 0 || iy >= Fy || iz < 0 || iz >= Fz) continue;
          const double wi = (ux ? 0.5 : 1.0) * (uy ? 0.5 : 1.0) * (uz ? 0.5 : 1.0);
          const int64_t i = fidx(ix, iy, iz);
          for (int s = 0; s < 27; s++) {
            const double a = Af[((int64_t)(s * BS + ci) * BS + cj) * nf + i];
            if (a == 0.0) continue;
            const int jx = ix + s / 9 - 1, jy = iy + (s / 3) % 3 - 1, jz = iz + s % 3 - 1;
            // coarse parents of j per direction: even -> one (weight 1), odd -> two (weight 1/2)
            const int px0 = jx >> 1, px1 = (jx + 1) >> 1, py0 = jy >> 1, py1 = (jy + 1) >> 1, pz0 = jz >> 1, pz1 = (jz + 1) >> 1;
            const double wx = (jx & 1) ? 0.5 : 1.0, wy = (jy & 1) ? 0.5 : 1.0, wz = (jz & 1) ? 0.5 : 1.0;
            for (int qx = px0; qx <= px1; qx++)
              for (int qy = py0; qy <= py1; qy++)
                for (int qz = pz0; qz <= pz1; qz++) {
                  if (qx >= Cx || qy >= Cy || qz >= Cz || masked_c(qx, qy, qz)) continue;
                  const int dx = qx - Ix, dy = qy - Iy, dz = qz - Iz;
                  acc[(dx + 1) * 9 + (dy + 1) * 3 + dz + 1] += wi * a * wx * wy * wz;
                }
          }
        }
  }
#pragma unroll
  for (int s = 0; s < 27; s++) Ac[((int64_t)(s * BS + ci) * BS + cj) * nc + I] = acc[s];
}

// b_c = P^T r_f, per component
template <int BS, typename T>
__global__ void k_restrict_lat(int Fx, int Fy, int Fz, int Cx, int Cy, int Cz, const T *__restrict__ rf, T *__restrict__ bc) {
  const int64_t nc = (int64_t)Cx * Cy * Cz;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nc * BS) return;
  const int64_t I = t / BS;
  const int c = (int)(t % BS);
  int Ix, Iy, Iz;
  lat_coord(I, Cy, Cz, Ix, Iy, Iz);
  T s = 0;
  for (int ux = -1; ux <= 1; ux++)
    for (int uy = -1; uy <= 1; uy++)
      for (int uz = -1; uz <= 1; uz++) {
        const int ix = 2 * Ix + ux, iy = 2 * Iy + uy, iz = 2 * Iz + uz;
        if (ix < 0 || ix >= Fx || iy < 0 || iy >= Fy || iz < 0 || iz >= Fz) continue;
        s += (T)((ux ? 0.5 : 1.0) * (uy ? 0.5 : 1.0) * (uz ? 0.5 : 1.0)) * rf[(((int64_t)ix * Fy + iy) * Fz + iz) * BS + c];
      }
  bc[t] = s;
}

// x_f += P x_c on unmasked fine unknowns (masked coarse values are zero)
template <int BS, typename T>
__global__ void k_prolong_lat(int Fx, int Fy, int Fz, int Cy, int Cz, const T *__restrict__ dinvf, const T *__restrict__ xc,
                              T *__restrict__ xf) {
  const int64_t nf = (int64_t)Fx * Fy * Fz;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nf * BS || dinvf[t] == (T)0) return;
  const int64_t i = t / BS;
  const int c = (int)(t % BS);
  int ix, iy, iz;
  lat_coord(i, Fy, Fz, ix, iy, iz);
  T s = 0;
  for (int qx = ix >> 1; qx <= (ix + 1) >> 1; qx++)
    for (int qy = iy >> 1; qy <= (iy + 1) >> 1; qy++)
      for (int qz = iz >> 1; qz <= (iz + 1) >> 1; qz++)
        s += (T)(((ix & 1) ? 0.5 : 1.0) * ((iy & 1) ? 0.5 : 1.0) * ((iz & 1) ? 0.5 : 1.0)) * xc[(((int64_t)qx * Cy + qy) * Cz + qz) * BS + c];
  xf[t] += s;
}

template <typename T>
__global__ void k_cheb0(int64_t n, const T *dinv, const T *r, T inv_theta, T *d, T *z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T v = dinv[i] * r[i] * inv_theta;
  d[i] = v;
  z[i] = v;
}
template <typename T>
__global__ void k_chebk(int64_t n, const T *dinv, const T *r, const T *w, T c1, T c2, T *d, T *z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T v = c1 * d[i] + c2 * dinv[i] * (r[i] - w[i]);
  d[i] = v;
  z[i] += v;
}
template <typename T>
__global__ void k_add(int64_t n, const T *a, T *y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] += a[i];
}
__global__ void k_scale(int64_t n, const double *s, double *y) {  // y *= 1 / sqrt(*s)
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] /= sqrt(*s);
}
__global__ void k_mulv(int64_t n, const double *a, double *y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] *= a[i];
}
template <typename A, typename B>
__global__ void k_conv(int64_t n, const A *__restrict__ a, B *__restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (B)a[i];
}
// natural (node, component) FP64 <-> lattice (node, component) in the cycle's type
template <typename T>
__global__ void k_scatter(int64_t n, int bs, const int32_t *lat, const double *r, T *b) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n * bs) b[(int64_t)lat[t / bs] * bs + t % bs] = (T)r[t];
}
template <typename T>
__global__ void k_gather(int64_t n, int bs, const int32_t *lat, const T *x, double *z) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n * bs) z[t] = (double)x[(int64_t)lat[t / bs] * bs + t % bs];
}
// y = M x for the dense coarsest inverse (one block per row)
template <typename T>
__global__ void k_dense_mv(int64_t n, const T *__restrict__ M, const T *__restrict__ x, T *__restrict__ y) {
  __shared__ T red[256];
  const int64_t r = blockIdx.x;
  T s = 0;
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) s += M[r * n + j] * x[j];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) y[r] = red[0];
}

}  // namespace

struct MGLevel {
  int L[3];
  int64_t n = 0;  // lattice nodes (vectors hold n * bs values)
  double *A = nullptr, *dinv = nullptr;  // full 27-entry stencil (set-up only) and Jacobi
  double *As = nullptr;                   // symmetric half (14 entries) used by the cycle
  double *x = nullptr, *b = nullptr, *r = nullptr, *d = nullptr, *w = nullptr, *e = nullptr;
  double emin = 0, emax = 0;
  double *dense = nullptr;  // coarsest: dense inverse (masked rows and columns zero)
  // FP32 cycle (mixed-precision solvers): the same level in single precision
  float *As32 = nullptr, *dinv32 = nullptr, *dense32 = nullptr;
  float *x32 = nullptr, *b32 = nullptr, *r32 = nullptr, *d32 = nullptr, *w32 = nullptr, *e32 = nullptr;
};

struct MGData {
  std::vector<MGLevel> lev;
  int bs = 1;
  bool fp32 = false;
  int64_t n = 0;  // explicit nodes
  const int32_t *lat = nullptr;  // owned by the space (made once, reused by every rebuild)
  int degree = 3;
  double *part = nullptr, *s = nullptr;
};

static void mg_free(MGData *M) {
  if (!M) return;
  for (MGLevel &l : M->lev) {
    for (double *p : {l.A, l.As, l.dinv, l.x, l.b, l.r, l.d, l.w, l.e, l.dense}) cudaFree(p);
    for (float *p : {l.As32, l.dinv32, l.dense32, l.x32, l.b32, l.r32, l.d32, l.w32, l.e32}) cudaFree(p);
  }
  cudaFree(M->part);
  cudaFree(M->s);
  delete M;
}

void mg_destroy(void *m) { mg_free((MGData *)m); }

// the arrays of one level in the cycle's type
template <typename T>
struct LV {
  T *As, *dinv, *dense, *x, *b, *r, *d, *w, *e;
};
template <typename T>
static LV<T> view(MGLevel &l);
template <>
LV<double> view<double>(MGLevel &l) {
  return {l.As, l.dinv, l.dense, l.x, l.b, l.r, l.d, l.w, l.e};
}
template <>
LV<float> view<float>(MGLevel &l) {
  return {l.As32, l.dinv32, l.dense32, l.x32, l.b32, l.r32, l.d32, l.w32, l.e32};
}

// y = A x, or b - A x (the full stencil during set-up, the symmetric half afterwards)
static void stencil_mv(int bs, const MGLevel &l, const double *x, const double *b, double *y, cudaStream_t s) {
  const unsigned g = nbk(l.n * bs);
  if (l.As) {
    if (bs == 3) k_stencil_mv_sym<3, double><<<g, 256, 0, s>>>(l.L[0], l.L[1], l.L[2], l.As, x, b, y);
    else k_stencil_mv_sym<1, double><<<g, 256, 0, s>>>(l.L[0], l.L[1], l.L[2], l.As, x, b, y);
    return;
  }
  if (bs == 3) k_stencil_mv<3><<<g, 256, 0, s>>>(l.L[0], l.L[1], l.L[2], l.A, x, b, y);
  else k_stencil_mv<1><<<g, 256, 0, s>>>(l.L[0], l.L[1], l.L[2], l.A, x, b, y);
}

template <typename T>
static void stencil_mv_t(int bs, const MGLevel &l, const T *As, const T *x, const T *b, T *y, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value)
    if (bs == 1 && l.L[0] <= 65535) {
      const dim3 g((unsigned)(l.L[2] + 31) / 32, (unsigned)(l.L[1] + 7) / 8, (unsigned)l.L[0]);
      k_stencil_mv_sym_tile<<<g, dim3(32, 8), 0, s>>>(l.L[0], l.L[1], l.L[2], As, x, b, y);
      return;
    }
  const unsigned g = nbk(l.n * bs);
  if (bs == 3) k_stencil_mv_sym<3, T><<<g, 256, 0, s>>>(l.L[0], l.L[1], l.L[2], As, x, b, y);
  else k_stencil_mv_sym<1, T><<<g, 256, 0, s>>>(l.L[0], l.L[1], l.L[2], As, x, b, y);
}

// Chebyshev-Jacobi on one level from a zero guess: z = p(D^-1 A) D^-1 r
template <typename T>
static dErr level_cheb(MGData *M, MGLevel &l, const T *r, T *z, cudaStream_t s) {
  LV<T> v = view<T>(l);
  const int64_t nv = l.n * M->bs;
  const double theta = 0.5 * (l.emax + l.emin), delta = 0.5 * (l.emax - l.emin), sigma = theta / delta;
  double rho = 1.0 / sigma;
  k_cheb0<T><<<nbk(nv), 256, 0, s>>>(nv, v.dinv, r, (T)(1.0 / theta), v.d, z);
  for (int it = 1; it < M->degree; it++) {
    stencil_mv_t<T>(M->bs, l, v.As, z, nullptr, v.w, s);
    const double rho1 = 1.0 / (2.0 * sigma - rho);
    k_chebk<T><<<nbk(nv), 256, 0, s>>>(nv, v.dinv, r, v.w, (T)(rho1 * rho), (T)(2.0 * rho1 / delta), v.d, z);
    rho = rho1;
  }
  CUCHK(cudaGetLastError());
  return 0;
}

// x = V(b) on level k (b and x are the level's own arrays)
template <typename T>
static dErr vcycle(MGData *M, size_t k, cudaStream_t s) {
  MGLevel &l = M->lev[k];
  LV<T> v = view<T>(l);
  const int bs = M->bs;
  const int64_t nv = l.n * bs;
  if (k + 1 == M->lev.size()) {
    k_dense_mv<T><<<(unsigned)nv, 256, 0, s>>>(nv, v.dense, v.b, v.x);
    CUCHK(cudaGetLastError());
    return 0;
  }
  MGLevel &c = M->lev[k + 1];
  LV<T> cv = view<T>(c);
  DCHK(level_cheb<T>(M, l, v.b, v.x, s));             // pre-smooth
  stencil_mv_t<T>(bs, l, v.As, v.x, v.b, v.r, s);   // r = b - A x
  if (bs == 3) k_restrict_lat<3, T><<<nbk(c.n * 3), 256, 0, s>>>(l.L[0], l.L[1], l.L[2], c.L[0], c.L[1], c.L[2], v.r, cv.b);
  else k_restrict_lat<1, T><<<nbk(c.n), 256, 0, s>>>(l.L[0], l.L[1], l.L[2], c.L[0], c.L[1], c.L[2], v.r, cv.b);
  DCHK(vcycle<T>(M, k + 1, s));
  if (bs == 3) k_prolong_lat<3, T><<<nbk(nv), 256, 0, s>>>(l.L[0], l.L[1], l.L[2], c.L[1], c.L[2], v.dinv, cv.x, v.x);
  else k_prolong_lat<1, T><<<nbk(nv), 256, 0, s>>>(l.L[0], l.L[1], l.L[2], c.L[1], c.L[2], v.dinv, cv.x, v.x);
  stencil_mv_t<T>(bs, l, v.As, v.x, v.b, v.r, s);   // post-smooth: e = p(D^-1 A) D^-1 (b - A x), x += e
  DCHK(level_cheb<T>(M, l, v.r, v.e, s));
  k_add<T><<<nbk(nv), 256, 0, s>>>(nv, v.e, v.x);
  CUCHK(cudaGetLastError());
  return 0;
}

template <typename T>
static dErr apply_t(MGData *M, const double *r, double *z, cudaStream_t s) {
  MGLevel &f = M->lev[0];
  LV<T> v = view<T>(f);
  CUCHK(cudaMemsetAsync(v.b, 0, f.n * M->bs * sizeof(T), s));
  k_scatter<T><<<nbk(M->n * M->bs), 256, 0, s>>>(M->n, M->bs, M->lat, r, v.b);
  DCHK(vcycle<T>(M, 0, s));
  k_gather<T><<<nbk(M->n * M->bs), 256, 0, s>>>(M->n, M->bs, M->lat, v.x, z);
  CUCHK(cudaGetLastError());
  return 0;
}

dErr mg_apply(void *m, const double *r, double *z, cudaStream_t s) {
  Range range_("PCApply (Q1 multigrid V-cycle)");
  MGData *M = (MGData *)m;
  return M->fp32 ? apply_t<float>(M, r, z, s) : apply_t<double>(M, r, z, s);
}

// lambda_max(D^-1 A) by 20 power steps from a seeded vector (masked unknowns stay 0)
static dErr level_eig(MGData *M, MGLevel &l, cudaStream_t s) {
  const int64_t nv = l.n * M->bs;
  std::vector<double> h(nv);
  uint64_t st = 12345;
  for (int64_t i = 0; i < nv; i++) {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    h[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
  CUCHK(cudaMemcpyAsync(l.x, h.data(), nv * sizeof(double), cudaMemcpyHostToDevice, s));
  k_mulv<<<nbk(nv), 256, 0, s>>>(nv, l.dinv, l.x);  // zero on masked unknowns (dinv = 0 there)
  double lam = 1, nrm[2];
  for (int it = 0; it < 20; it++) {
    stencil_mv(M->bs, l, l.x, nullptr, l.w, s);
    k_mulv<<<nbk(nv), 256, 0, s>>>(nv, l.dinv, l.w);
    DCHK(device_dot(nv, l.w, l.w, M->part, M->s, s));
    DCHK(device_dot(nv, l.x, l.x, M->part, M->s + 1, s));
    CUCHK(cudaMemcpyAsync(nrm, M->s, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CUCHK(cudaStreamSynchronize(s));
    lam = sqrt(nrm[0] / nrm[1]);
    CUCHK(cudaMemcpyAsync(l.x, l.w, nv * sizeof(double), cudaMemcpyDeviceToDevice, s));
    k_scale<<<nbk(nv), 256, 0, s>>>(nv, M->s, l.x);
  }
  l.emax = 1.1 * lam;
  l.emin = 0.1 * lam;
  return 0;
}

// dense inverse of the coarsest operator on its unmasked unknowns (Gauss-Jordan with partial pivoting, host)
static dErr coarsest_dense(MGLevel &l, int bs, cudaStream_t s) {
  const int64_t n = l.n, nv = n * bs;
  std::vector<double> A(27 * bs * bs * n);
  CUCHK(cudaMemcpyAsync(A.data(), l.A, A.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUCHK(cudaStreamSynchronize(s));
  auto coef = [&](int st, int ci, int cj, int64_t i) { return A[((int64_t)(st * bs + ci) * bs + cj) * n + i]; };
  std::vector<int64_t> act, pos(nv, -1);
  for (int64_t i = 0; i < n; i++)
    if (coef(13, 0, 0, i) != 0)
      for (int c = 0; c < bs; c++) act.push_back(i * bs + c);
  const int64_t m = (int64_t)act.size();
  for (int64_t a = 0; a < m; a++) pos[act[a]] = a;
  std::vector<double> D(m * 2 * m, 0.0);  // [A | I]
  const int Ly = l.L[1], Lz = l.L[2];
  for (int64_t a = 0; a < m; a++) {
    const int64_t i = act[a] / bs;
    const int ci = (int)(act[a] % bs);
    const int ix = (int)(i / ((int64_t)Ly * Lz)), iy = (int)((i / Lz) % Ly), iz = (int)(i % Lz);
    for (int st = 0; st < 27; st++)
      for (int cj = 0; cj < bs; cj++) {
        const double v = coef(st, ci, cj, i);
        if (v == 0) continue;
        const int jx = ix + st / 9 - 1, jy = iy + (st / 3) % 3 - 1, jz = iz + st % 3 - 1;
        const int64_t j = (((int64_t)jx * Ly + jy) * Lz + jz) * bs + cj;
        if (pos[j] < 0) return set_error("multigrid coarsest level couples to a masked node");
        D[a * 2 * m + pos[j]] = v;
      }
    D[a * 2 * m + m + a] = 1.0;
  }
  for (int64_t c = 0; c < m; c++) {
    int64_t p = c;
    for (int64_t r = c + 1; r < m; r++)
      if (fabs(D[r * 2 * m + c]) > fabs(D[p * 2 * m + c])) p = r;
    if (D[p * 2 * m + c] == 0) return set_error("multigrid coarsest operator is singular");
    if (p != c)
      for (int64_t k = 0; k < 2 * m; k++) std::swap(D[p * 2 * m + k], D[c * 2 * m + k]);
    const double inv = 1.0 / D[c * 2 * m + c];
    for (int64_t k = 0; k < 2 * m; k++) D[c * 2 * m + k] *= inv;
    for (int64_t r = 0; r < m; r++) {
      if (r == c) continue;
      const double f = D[r * 2 * m + c];
      if (f == 0) continue;
      for (int64_t k = 0; k < 2 * m; k++) D[r * 2 * m + k] -= f * D[c * 2 * m + k];
    }
  }
  std::vector<double> Minv(nv * nv, 0.0);
  for (int64_t a = 0; a < m; a++)
    for (int64_t b = 0; b < m; b++) Minv[act[a] * nv + act[b]] = D[a * 2 * m + m + b];
  CUCHK(cudaMalloc(&l.dense, nv * nv * sizeof(double)));
  CUCHK(cudaMemcpy(l.dense, Minv.data(), nv * nv * sizeof(double), cudaMemcpyHostToDevice));
  return 0;
}

static dErr level_alloc(MGLevel &l, int bs) {
  l.n = (int64_t)l.L[0] * l.L[1] * l.L[2];
  const int64_t nv = l.n * bs;
  CUCHK(cudaMalloc(&l.A, 27 * bs * nv * sizeof(double)));
  CUCHK(cudaMemset(l.A, 0, 27 * bs * nv * sizeof(double)));
  for (double **p : {&l.dinv, &l.x, &l.b, &l.r, &l.d, &l.w, &l.e}) {
    CUCHK(cudaMalloc(p, nv * sizeof(double)));
    CUCHK(cudaMemset(*p, 0, nv * sizeof(double)));
  }
  return 0;
}

// lattice position of every explicit node of a uniform-order space on a block mesh: elements in x-major order,
// element (ex, ey, ez) local node (a, b, c) -> GLL lattice node (ex p + a, ey p + b, ez p + c) of the
// (M p + 1)-per-direction lattice L0; also used by the learned correction on the GLL lattice
dErr fs_gll_lattice(_p_dFS *fs, std::vector<int32_t> &lat, int L0[3]) {
  if (!fs->uniform) return set_error("the GLL lattice needs a uniform-order space");
  if (!fs->mesh->structured) return set_error("the GLL lattice needs a block mesh");
  const _p_dMesh *mesh = fs->mesh;
  const int p = fs->p, P = p + 1, My = mesh->ny - 1, Mz = mesh->nz - 1;
  L0[0] = (mesh->nx - 1) * p + 1, L0[1] = My * p + 1, L0[2] = Mz * p + 1;
  lat.assign(fs->n, -1);
  for (int64_t r = 0; r < fs->nelem; r++) {
    const int ex = (int)(r / ((int64_t)My * Mz)), ey = (int)((r / Mz) % My), ez = (int)(r % Mz);
    for (int a = 0; a < P; a++)
      for (int b = 0; b < P; b++)
        for (int c = 0; c < P; c++) {
          const int32_t d = fs->emap[fs->xstart[r] + (a * P + b) * P + c];
          if (d >= fs->n) continue;
          const int32_t L = (int32_t)((((int64_t)ex * p + a) * L0[1] + (ey * p + b)) * L0[2] + ez * p + c);
          if (lat[d] >= 0 && lat[d] != L) return set_error("dof %d sits at two lattice positions: the mesh is not a structured block", d);
          lat[d] = L;
        }
  }
  for (int64_t d = 0; d < fs->n; d++)
    if (lat[d] < 0) return set_error("dof %lld has no lattice position", (long long)d);
  return 0;
}

// the lattice map on the device, made once per space and kept on it (every Newton step rebuilds the hierarchy,
// not the map)
static dErr lattice_map(_p_dFS *fs) {
  if (fs->d_mg_lat) return 0;
  std::vector<int32_t> lat;
  int L0[3];
  DCHK(fs_gll_lattice(fs, lat, L0));
  CUCHK(cudaMalloc(&fs->d_mg_lat, std::max<int64_t>(fs->n, 1) * sizeof(int32_t)));
  CUCHK(cudaMemcpy(fs->d_mg_lat, lat.data(), fs->n * sizeof(int32_t), cudaMemcpyHostToDevice));
  return 0;
}

// build the hierarchy from the assembled Q1 matrix (scalar, or the interleaved 3 x 3 blocked elasticity matrix)
// of a uniform-order space on a block mesh
dErr mg_build(_p_dMat *J, int degree, bool fp32, void **out) {
  _p_dFS *fs = J->fs;
  const int bs = J->bs;
  if (bs != 1 && bs != 3) return set_error("Q1 multigrid: block size %d", bs);
  if (!fs->uniform) return set_error("Q1 multigrid needs a uniform-order space");
  if (!fs->mesh->structured) return set_error("Q1 multigrid needs a block mesh (its GLL lattice)");
  const _p_dMesh *mesh = fs->mesh;
  const int p = fs->p, Mx = mesh->nx - 1, My = mesh->ny - 1, Mz = mesh->nz - 1;
  const int L0[3] = {Mx * p + 1, My * p + 1, Mz * p + 1};
  for (int d = 0; d < 3; d++)
    if (L0[d] % 2 == 0 || L0[d] < 5) return set_error("Q1 multigrid needs an even number of GLL intervals (elements x degree) per direction");
  cudaStream_t s = fs->stream;
  MGData *M = new MGData();
  M->bs = bs;
  M->degree = std::max(2, degree);
  M->n = fs->n;
  dErr le = lattice_map(fs);
  if (le) {
    mg_free(M);
    return le;
  }
  M->lat = fs->d_mg_lat;
  DCHK(dot_part_alloc(&M->part));
  CUCHK(cudaMalloc(&M->s, 4 * sizeof(double)));
  // levels: halve until the coarsest is small enough for a dense inverse (9 nodes per direction for scalar
  // matrices, 5 for blocked ones)
  const int stop = bs == 1 ? 9 : 5;
  int L[3] = {L0[0], L0[1], L0[2]};
  for (;;) {
    MGLevel l;
    for (int d = 0; d < 3; d++) l.L[d] = L[d];
    dErr e = level_alloc(l, bs);
    M->lev.push_back(l);
    if (e) {
      mg_free(M);
      return e;
    }
    if (std::max(L[0], std::max(L[1], L[2])) <= stop || L[0] % 2 == 0 || L[1] % 2 == 0 || L[2] % 2 == 0) break;
    for (int d = 0; d < 3; d++) L[d] = (L[d] + 1) / 2;
  }
  if ((int64_t)M->lev.back().n * bs > 4096) {
    mg_free(M);
    return set_error("Q1 multigrid: the coarsest lattice is too large for a dense solve");
  }
  // fine operator from the CSR, then Galerkin coarse operators
  MGLevel &f = M->lev[0];
  int *bad;
  CUCHK(cudaMalloc(&bad, sizeof(int)));
  CUCHK(cudaMemsetAsync(bad, 0, sizeof(int), s));
  const int64_t nrows = fs->n * bs;
  if (bs == 3) k_stencil_fill<3><<<nbk(nrows), 256, 0, s>>>(nrows, J->d_rowptr, J->d_col, J->d_val, M->lat, f.L[1], f.L[2], f.n, f.A, bad);
  else k_stencil_fill<1><<<nbk(nrows), 256, 0, s>>>(nrows, J->d_rowptr, J->d_col, J->d_val, M->lat, f.L[1], f.L[2], f.n, f.A, bad);
  int hbad = 0;
  CUCHK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUCHK(cudaStreamSynchronize(s));
  cudaFree(bad);
  if (hbad) {
    mg_free(M);
    return set_error("Q1 matrix couples nodes that are not lattice neighbours");
  }
  for (size_t k = 0; k < M->lev.size(); k++) {
    MGLevel &l = M->lev[k];
    if (k > 0) {
      const MGLevel &fl = M->lev[k - 1];
      const int64_t nt = l.n * bs * bs;
      if (bs == 3) k_galerkin<3><<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(fl.L[0], fl.L[1], fl.L[2], l.L[0], l.L[1], l.L[2], fl.A, l.A);
      else k_galerkin<1><<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(fl.L[0], fl.L[1], fl.L[2], l.L[0], l.L[1], l.L[2], fl.A, l.A);
      CUCHK(cudaGetLastError());
    }
    if (bs == 3) k_dinv<3><<<nbk(l.n * 3), 256, 0, s>>>(l.n, l.A, l.dinv);
    else k_dinv<1><<<nbk(l.n), 256, 0, s>>>(l.n, l.A, l.dinv);
    CUCHK(cudaGetLastError());
    if (k + 1 < M->lev.size()) {  // the cycle runs on the symmetric half
      const int64_t ns = 14 * bs * bs * l.n;
      CUCHK(cudaMalloc(&l.As, ns * sizeof(double)));
      if (bs == 3) k_sym_extract<3><<<nbk(ns), 256, 0, s>>>(l.n, l.A, l.As);
      else k_sym_extract<1><<<nbk(ns), 256, 0, s>>>(l.n, l.A, l.As);
      CUCHK(cudaGetLastError());
    }
    dErr e = k + 1 < M->lev.size() ? level_eig(M, l, s) : coarsest_dense(l, bs, s);
    if (e) {
      mg_free(M);
      return e;
    }
  }
  CUCHK(cudaStreamSynchronize(s));
  for (MGLevel &l : M->lev) {  // the full stencils were needed for the Galerkin products and the dense solve only
    cudaFree(l.A);
    l.A = nullptr;
  }
  if (fp32) {  // the single-precision cycle: every cycle array rounded once
    M->fp32 = true;
    for (size_t k = 0; k < M->lev.size(); k++) {
      MGLevel &l = M->lev[k];
      const int64_t nv = l.n * bs;
      auto conv = [&](const double *a, float **b, int64_t cnt) -> dErr {
        CUCHK(cudaMalloc(b, std::max<int64_t>(cnt, 1) * sizeof(float)));
        if (a && cnt) k_conv<double, float><<<nbk(cnt), 256, 0, s>>>(cnt, a, *b);
        else CUCHK(cudaMemsetAsync(*b, 0, std::max<int64_t>(cnt, 1) * sizeof(float), s));
        CUCHK(cudaGetLastError());
        return 0;
      };
      dErr e = conv(l.dinv, &l.dinv32, nv);
      if (!e && l.As) e = conv(l.As, &l.As32, 14 * bs * nv);
      if (!e && l.dense) e = conv(l.dense, &l.dense32, nv * nv);
      for (float **p : {&l.x32, &l.b32, &l.r32, &l.d32, &l.w32, &l.e32})
        if (!e) e = conv(nullptr, p, nv);
      if (e) {
        mg_free(M);
        return e;
      }
    }
    CUCHK(cudaStreamSynchronize(s));
  }
  *out = M;
  return 0;
}
