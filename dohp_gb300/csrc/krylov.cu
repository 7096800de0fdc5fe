// Device linear algebra for the solvers: exclusive scan, CSR SpMV, deterministic dot products,
// Chebyshev-Jacobi smoothing on the Q1 matrix, preconditioned CG and FGMRES.
//
// PETSc KSPCG / KSPFGMRES / KSPCHEBYSHEV+PCJACOBI are the reference's solvers (not vendored); these are
// restatements of the textbook algorithms (Saad, Iterative Methods for Sparse Linear Systems, 2nd ed.:
// Alg. 6.18 CG, Alg. 9.6 FGMRES, Alg. 12.1 Chebyshev). Reductions use a fixed grid and a fixed-order tree
// so every run produces bitwise identical results.
#include <math.h>

#include <algorithm>
#include <vector>

#include "internal.h"

using namespace dgb;

dErr op_mult(_p_dOperator *op, const double *x, double *y);

namespace {

constexpr int RED_BLOCKS = 1024, RED_THREADS = 256;

__global__ void k_scan_block(const int32_t *in, int32_t *out, int64_t n, int64_t *block_sums) {
  __shared__ int64_t s[1024];
  const int64_t i = blockIdx.x * 1024LL + threadIdx.x;
  const int64_t v = i < n ? in[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int64_t t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = (int32_t)(s[threadIdx.x] - v);  // exclusive within block
  if (threadIdx.x == 1023) block_sums[blockIdx.x] = s[1023];
}

__global__ void k_scan_add(int32_t *out, int64_t n, const int64_t *block_offsets, int64_t total) {
  const int64_t i = blockIdx.x * 1024LL + threadIdx.x;
  if (i < n) out[i] += (int32_t)block_offsets[blockIdx.x];
  if (i == 0) out[n] = (int32_t)total;
}

template <typename T>
__global__ void k_spmv(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ col, const T *__restrict__ val,
                       const T *__restrict__ x, T *__restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  T s = 0;
  for (int32_t k = rp[i]; k < rp[i + 1]; k++) s += val[k] * x[col[k]];
  y[i] = s;
}

__global__ void k_dot_partial(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ part) {
  __shared__ double s[RED_THREADS];
  double acc = 0;
  for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n; i += (int64_t)RED_BLOCKS * RED_THREADS) acc += a[i] * b[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int off = RED_THREADS / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) s[threadIdx.x] += s[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void k_dot_final(const double *__restrict__ part, int nparts, double *__restrict__ out) {
  __shared__ double s[RED_BLOCKS];
  for (int i = threadIdx.x; i < RED_BLOCKS; i += blockDim.x) s[i] = i < nparts ? part[i] : 0.0;
  __syncthreads();
  for (int off = RED_BLOCKS / 2; off > 0; off >>= 1) {
    for (int i = threadIdx.x; i < off; i += blockDim.x) s[i] += s[i + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

__global__ void k_diag_inv(int64_t n, const int32_t *rp, const int32_t *col, const double *val, double *dinv) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0;
  for (int32_t k = rp[i]; k < rp[i + 1]; k++)
    if (col[k] == i) d = val[k];
  dinv[i] = d != 0 ? 1.0 / d : 0.0;
}

// y = a*x + b*y with optional device scalars: a = sa * (num ? *num / *den : 1)
__global__ void k_axpby(int64_t n, double sa, const double *num, const double *den, const double *x, double b, double *y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = num ? sa * (*num / *den) : sa;
  y[i] = a * x[i] + b * y[i];
}

// p = z + (num/den) p
__global__ void k_xpay_ratio(int64_t n, const double *z, const double *num, const double *den, double *p) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  p[i] = z[i] + (*num / *den) * p[i];
}

__global__ void k_cheb_first(int64_t n, const double *dinv, const double *r, double inv_theta, double *d, double *z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = dinv[i] * r[i] * inv_theta;
  d[i] = v;
  z[i] = v;
}

__global__ void k_cheb_step(int64_t n, const double *dinv, const double *r, const double *w, double c1, double c2, double *d, double *z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = c1 * d[i] + c2 * dinv[i] * (r[i] - w[i]);
  d[i] = v;
  z[i] += v;
}

__global__ void k_pointwise_mult(int64_t n, const double *a, const double *b, double *y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = a[i] * b[i];
}

inline unsigned nb(int64_t n, int t = 256) { return (unsigned)std::max<int64_t>((n + t - 1) / t, 1); }

}  // namespace

dErr device_exclusive_scan(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s, int64_t *total) {
  const int64_t nblk = std::max<int64_t>((n + 1023) / 1024, 1);
  int64_t *d_bs;
  CUCHK(cudaMalloc(&d_bs, nblk * sizeof(int64_t)));
  if (n) {
    k_scan_block<<<(unsigned)nblk, 1024, 0, s>>>(in, out, n, d_bs);
    CUCHK(cudaGetLastError());
  }
  std::vector<int64_t> h(nblk, 0);
  if (n) CUCHK(cudaMemcpyAsync(h.data(), d_bs, nblk * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  CUCHK(cudaStreamSynchronize(s));
  int64_t acc = 0;
  for (int64_t i = 0; i < nblk; i++) {
    const int64_t v = n ? h[i] : 0;
    h[i] = acc;
    acc += v;
  }
  CUCHK(cudaMemcpyAsync(d_bs, h.data(), nblk * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  k_scan_add<<<(unsigned)nblk, 1024, 0, s>>>(out, n, d_bs, acc);
  CUCHK(cudaGetLastError());
  CUCHK(cudaStreamSynchronize(s));
  cudaFree(d_bs);
  *total = acc;
  return 0;
}

dErr mat_mult(_p_dMat *J, const double *x, double *y, cudaStream_t s) {
  if (J->nrows == 0) return 0;
  k_spmv<double><<<nb(J->nrows), 256, 0, s>>>(J->nrows, J->d_rowptr, J->d_col, J->d_val, x, y);
  CUCHK(cudaGetLastError());
  return 0;
}

// deterministic dot product into a device scalar (uses `part` of RED_BLOCKS doubles)
dErr device_dot(int64_t n, const double *a, const double *b, double *part, double *out, cudaStream_t s) {
  k_dot_partial<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, a, b, part);
  k_dot_final<<<1, 1024, 0, s>>>(part, RED_BLOCKS, out);
  CUCHK(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------------------------------------------ KSP
struct _p_dKSP {
  dOperator op;
  dMat pmat;
  dKSPType type;
  dPCType pc;
  int cheb_degree = 3;
  int restart = 30;
  dPrecision pc_prec = dPREC_FP64;
  int64_t n = 0;
  double emin = 0, emax = 0;
  bool pc_ready = false;
  double *d_dinv = nullptr, *d_work = nullptr, *d_part = nullptr, *d_s = nullptr;
  std::vector<double *> V, Z;  // FGMRES bases
};

static dErr ksp_alloc(_p_dKSP *k) {
  if (k->d_work) return 0;
  CUCHK(cudaMalloc(&k->d_work, 8 * std::max<int64_t>(k->n, 1) * sizeof(double)));
  CUCHK(cudaMalloc(&k->d_part, RED_BLOCKS * sizeof(double)));
  CUCHK(cudaMalloc(&k->d_s, 64 * sizeof(double)));
  CUCHK(cudaMalloc(&k->d_dinv, std::max<int64_t>(k->n, 1) * sizeof(double)));
  return 0;
}

static dErr pc_setup(_p_dKSP *k) {
  if (k->pc_ready || k->pc == dPC_NONE) return 0;
  _p_dFS *fs = k->op->fs;
  cudaStream_t s = fs->stream;
  const int64_t n = k->n;
  if (!k->pmat) return set_error("preconditioner needs the Q1 matrix");
  k_diag_inv<<<nb(n), 256, 0, s>>>(n, k->pmat->d_rowptr, k->pmat->d_col, k->pmat->d_val, k->d_dinv);
  CUCHK(cudaGetLastError());
  if (k->pc == dPC_CHEBYSHEV_Q1) {  // lambda_max(D^-1 A_q1) by 20 power steps from a seeded vector
    std::vector<double> h(n);
    uint64_t st = 12345;
    for (int64_t i = 0; i < n; i++) {
      uint64_t z = (st += 0x9E3779B97F4A7C15ull);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      h[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
    double *z = k->d_work, *w = k->d_work + n;
    CUCHK(cudaMemcpyAsync(z, h.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    double lam = 1, nrm[2];
    for (int it = 0; it < 20; it++) {
      DCHK(mat_mult(k->pmat, z, w, s));
      k_pointwise_mult<<<nb(n), 256, 0, s>>>(n, w, k->d_dinv, w);
      DCHK(device_dot(n, w, w, k->d_part, k->d_s, s));
      DCHK(device_dot(n, z, z, k->d_part, k->d_s + 1, s));
      CUCHK(cudaMemcpyAsync(nrm, k->d_s, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
      CUCHK(cudaStreamSynchronize(s));
      const double nw = sqrt(nrm[0]), nz = sqrt(nrm[1]);
      lam = nw / nz;
      k_axpby<<<nb(n), 256, 0, s>>>(n, 1.0 / nw, nullptr, nullptr, w, 0.0, z);
    }
    k->emax = 1.1 * lam;
    k->emin = 0.1 * lam;
  }
  k->pc_ready = true;
  return 0;
}

// z = M^{-1} r
static dErr pc_apply(_p_dKSP *k, const double *r, double *z) {
  const int64_t n = k->n;
  cudaStream_t s = k->op->fs->stream;
  if (k->pc == dPC_NONE) {
    CUCHK(cudaMemcpyAsync(z, r, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return 0;
  }
  if (k->pc == dPC_JACOBI) {
    k_pointwise_mult<<<nb(n), 256, 0, s>>>(n, k->d_dinv, r, z);
    CUCHK(cudaGetLastError());
    return 0;
  }
  const double theta = 0.5 * (k->emax + k->emin), delta = 0.5 * (k->emax - k->emin), sigma = theta / delta;
  double rho = 1.0 / sigma;
  double *d = k->d_work + 6 * n, *w = k->d_work + 7 * n;
  k_cheb_first<<<nb(n), 256, 0, s>>>(n, k->d_dinv, r, 1.0 / theta, d, z);
  for (int it = 1; it < k->cheb_degree; it++) {
    DCHK(mat_mult(k->pmat, z, w, s));
    const double rho1 = 1.0 / (2.0 * sigma - rho);
    k_cheb_step<<<nb(n), 256, 0, s>>>(n, k->d_dinv, r, w, rho1 * rho, 2.0 * rho1 / delta, d, z);
    rho = rho1;
  }
  CUCHK(cudaGetLastError());
  return 0;
}

static dErr read_scalar(const double *d, double *h, cudaStream_t s) {
  CUCHK(cudaMemcpyAsync(h, d, sizeof(double), cudaMemcpyDeviceToHost, s));
  CUCHK(cudaStreamSynchronize(s));
  return 0;
}

static dErr cg_solve(_p_dKSP *k, const double *b, double *x, double rtol, int maxit, int *its, double *rnorm) {
  const int64_t n = k->n;
  cudaStream_t s = k->op->fs->stream;
  double *r = k->d_work, *z = k->d_work + n, *p = k->d_work + 2 * n, *q = k->d_work + 3 * n;
  double *S = k->d_s;  // S[0]=rz S[1]=pq S[2]=rr S[3]=bb S[4]=rz_new
  DCHK(op_mult(k->op, x, q));
  CUCHK(cudaMemcpyAsync(r, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  k_axpby<<<nb(n), 256, 0, s>>>(n, -1.0, nullptr, nullptr, q, 1.0, r);
  DCHK(device_dot(n, b, b, k->d_part, S + 3, s));
  DCHK(device_dot(n, r, r, k->d_part, S + 2, s));
  double bb, rr;
  DCHK(read_scalar(S + 3, &bb, s));
  DCHK(read_scalar(S + 2, &rr, s));
  const double bn = sqrt(bb) > 0 ? sqrt(bb) : 1.0;
  *its = 0;
  if (sqrt(rr) <= rtol * bn) {
    *rnorm = sqrt(rr) / bn;
    return 0;
  }
  DCHK(pc_apply(k, r, z));
  CUCHK(cudaMemcpyAsync(p, z, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  DCHK(device_dot(n, r, z, k->d_part, S, s));
  for (int it = 0; it < maxit; it++) {
    DCHK(op_mult(k->op, p, q));
    DCHK(device_dot(n, p, q, k->d_part, S + 1, s));
    k_axpby<<<nb(n), 256, 0, s>>>(n, 1.0, S, S + 1, p, 1.0, x);
    k_axpby<<<nb(n), 256, 0, s>>>(n, -1.0, S, S + 1, q, 1.0, r);
    DCHK(device_dot(n, r, r, k->d_part, S + 2, s));
    DCHK(read_scalar(S + 2, &rr, s));
    *its = it + 1;
    if (!(sqrt(rr) > rtol * bn)) break;
    DCHK(pc_apply(k, r, z));
    DCHK(device_dot(n, r, z, k->d_part, S + 4, s));
    k_xpay_ratio<<<nb(n), 256, 0, s>>>(n, z, S + 4, S, p);
    CUCHK(cudaMemcpyAsync(S, S + 4, sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  CUCHK(cudaGetLastError());
  *rnorm = sqrt(rr) / bn;
  if (!(sqrt(rr) <= rtol * bn)) return set_error("CG did not converge in %d iterations (relative residual %g)", maxit, *rnorm);
  return 0;
}

extern "C" {

dErr dKSPCreate(dOperator op, dMat pmat, dKSPType type, dPCType pc, dKSP *ksp) {
  if (!op || !ksp) return set_error("dKSPCreate: null argument");
  if (type != dKSP_CG) return set_error("KSP type %d not built yet", (int)type);
  _p_dKSP *k = new _p_dKSP();
  k->op = op;
  k->pmat = pmat;
  k->type = type;
  k->pc = pc;
  k->n = op->fs->n * op->fs->bs;
  *ksp = k;
  return 0;
}

dErr dKSPDestroy(dKSP *ksp) {
  if (!ksp || !*ksp) return 0;
  _p_dKSP *k = *ksp;
  cudaFree(k->d_dinv);
  cudaFree(k->d_work);
  cudaFree(k->d_part);
  cudaFree(k->d_s);
  delete k;
  *ksp = nullptr;
  return 0;
}

dErr dKSPSetOptions(dKSP ksp, dInt cheb_degree, dPrecision pc_precision, dInt restart) {
  if (!ksp) return set_error("null KSP");
  if (cheb_degree < 1) return set_error("Chebyshev degree must be >= 1");
  ksp->cheb_degree = cheb_degree;
  ksp->pc_prec = pc_precision;
  ksp->restart = restart;
  ksp->pc_ready = false;
  return 0;
}

dErr dKSPSolve(dKSP ksp, const dScalar *b, dScalar *x, dReal rtol, dInt maxit, dInt *its, dReal *rnorm) {
  if (!ksp) return set_error("null KSP");
  DCHK(ksp_alloc(ksp));
  DCHK(pc_setup(ksp));
  int it = 0;
  double rn = 0;
  dErr e = cg_solve(ksp, b, x, rtol, maxit, &it, &rn);
  if (its) *its = it;
  if (rnorm) *rnorm = rn;
  return e;
}

}  // extern "C"
