// Device linear algebra for the solvers: exclusive scan, sliced-ELL SpMV, deterministic dot products,
// Chebyshev-Jacobi smoothing on the Q1 matrix, preconditioned CG and FGMRES.
//
// PETSc KSPCG / KSPFGMRES / KSPCHEBYSHEV+PCJACOBI are the reference's solvers (not vendored); these are
// restatements of the textbook algorithms (Saad, Iterative Methods for Sparse Linear Systems, 2nd ed.:
// Alg. 6.18 CG, Alg. 9.6 FGMRES, Alg. 12.1 Chebyshev). Reductions use a fixed grid and a fixed-order tree
// so every run produces bitwise identical results.
#include <math.h>

#include <algorithm>
#include <vector>

#include <cuda_bf16.h>

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

__global__ void k_val_to_bf16(int64_t n, const double *__restrict__ a, __nv_bfloat16 *__restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16_rn((float)a[i]);
}

// Sliced ELL (SELL-32): rows in slices of 32, each slice stored column-major and padded to its longest row, so
// at step k the 32 lanes of a warp read 32 consecutive values and column indices. With the row-per-thread CSR
// loop each lane walks its own row and a warp touches 32 cache lines per step; on the 27-point Q1 rows that
// ran at 2.7 TB/s against 5.1-5.7 TB/s for this layout. Padding points at the row itself with value 0, so a
// row's sum runs over its CSR entries in CSR order plus exact zeros: the result equals the CSR loop's.
__device__ __forceinline__ double sell_val(double v) { return v; }
__device__ __forceinline__ float sell_val(float v) { return v; }
__device__ __forceinline__ float sell_val(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename V, typename T>
__global__ void k_sell(int64_t n, const int64_t *__restrict__ off, const int32_t *__restrict__ col, const V *__restrict__ val,
                       const T *__restrict__ x, T *__restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = off[i >> 5] + (i & 31), w = (off[(i >> 5) + 1] - off[i >> 5]) >> 5;
  T s = 0;
  for (int64_t k = 0; k < w; k++) s += sell_val(val[b + 32 * k]) * x[col[b + 32 * k]];
  y[i] = s;
}

// one thread per row of the padded slices (32 * nslices threads): the slice width is the warp's max row length
__global__ void k_sell_width(int64_t n, const int32_t *__restrict__ rp, int64_t nslices, int32_t *__restrict__ w) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 32 * nslices) return;  // whole warps only: 32 * nslices is a multiple of 32
  const int32_t len = i < n ? rp[i + 1] - rp[i] : 0;
  const int32_t m = __reduce_max_sync(0xffffffffu, len);
  if ((i & 31) == 0) w[i >> 5] = m;
}

// scatter CSR values (and, when scol is given, column indices) into the slices
__global__ void k_sell_fill(int64_t n, int64_t nslices, const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                            const double *__restrict__ val, const int64_t *__restrict__ off, int32_t *__restrict__ scol,
                            double *__restrict__ sval) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 32 * nslices) return;
  const int64_t b = off[i >> 5] + (i & 31), w = (off[(i >> 5) + 1] - off[i >> 5]) >> 5;
  const int32_t r0 = i < n ? rp[i] : 0, len = i < n ? rp[i + 1] - r0 : 0;
  const int32_t self = (int32_t)(i < n ? i : n - 1);
  for (int64_t k = 0; k < w; k++) {
    const bool in = k < len;
    if (scol) scol[b + 32 * k] = in ? col[r0 + k] : self;
    sval[b + 32 * k] = in ? val[r0 + k] : 0.0;
  }
}

// block partial of a . b, then the last block to finish (ticket counter) sums the partials in block order: one
// launch, deterministic for a given n (the grid depends on n only). part holds RED_BLOCKS partials followed by the
// ticket, which the last block resets to zero.
__device__ __forceinline__ void dot_finish(double acc, double *part, double *out) {
  __shared__ double s[RED_THREADS];
  __shared__ bool last;
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int off = RED_THREADS / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) s[threadIdx.x] += s[threadIdx.x + off];
    __syncthreads();
  }
  unsigned *ticket = reinterpret_cast<unsigned *>(part + RED_BLOCKS);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s[0];
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double a = 0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += RED_THREADS) a += ((volatile double *)part)[i];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int off = RED_THREADS / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) s[threadIdx.x] += s[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *out = s[0];
    *ticket = 0;
  }
}

__global__ void __launch_bounds__(RED_THREADS) k_dot1(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *part,
                                                     double *out) {
  double acc = 0;
  for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * RED_THREADS) acc += a[i] * b[i];
  dot_finish(acc, part, out);
}

// CG update fused with the residual norm: x += alpha p, r -= alpha q with alpha = rz / pq (S[4] / S[1]), out = r.r;
// S[0] takes rz for the next step's ratio (no other block of this launch reads S[0])
__global__ void __launch_bounds__(RED_THREADS) k_cg_update(int64_t n, double *S, const double *__restrict__ p,
                                                          const double *__restrict__ q, double *__restrict__ x, double *__restrict__ r,
                                                          double *part, double *out) {
  const double alpha = S[4] / S[1];
  if (blockIdx.x == 0 && threadIdx.x == 0) S[0] = S[4];
  double acc = 0;
  for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * RED_THREADS) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    acc += ri * ri;
  }
  dot_finish(acc, part, out);
}

static unsigned dot_grid(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(RED_BLOCKS, (n + RED_THREADS - 1) / RED_THREADS)); }

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

template <typename A, typename B>
__global__ void k_convert(int64_t n, const A *__restrict__ a, B *__restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (B)a[i];
}

template <typename T>
__global__ void k_cheb_first_t(int64_t n, const T *dinv, const T *r, T inv_theta, T *d, T *z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T v = dinv[i] * r[i] * inv_theta;
  d[i] = v;
  z[i] = v;
}

// one Chebyshev step with its matrix product fused: w_i = (A zin)_i (the sliced rows of k_sell, same order), then
// d_i = c1 d_i + c2 dinv_i (r_i - w_i) and zout_i = zin_i + d_i, the same arithmetic as a product followed by an
// elementwise step (zout must not alias zin: other rows still read zin)
template <typename V, typename T>
__global__ void k_sell_cheb(int64_t n, const int64_t *__restrict__ off, const int32_t *__restrict__ col, const V *__restrict__ val,
                            const T *__restrict__ dinv, const T *__restrict__ r, const T *__restrict__ zin, T c1, T c2,
                            T *__restrict__ d, T *__restrict__ zout) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = off[i >> 5] + (i & 31), w = (off[(i >> 5) + 1] - off[i >> 5]) >> 5;
  T s = 0;
  for (int64_t k = 0; k < w; k++) s += sell_val(val[b + 32 * k]) * zin[col[b + 32 * k]];
  const T v = c1 * d[i] + c2 * dinv[i] * (r[i] - s);
  d[i] = v;
  zout[i] = zin[i] + v;
}

// out[v] = <V_v, w> for v < nv (V row-major [nv][n]), fixed-order partials then a fixed-order tree
__global__ void k_mdot_partial(int64_t n, int nv, const double *__restrict__ V, const double *__restrict__ w, double *__restrict__ part) {
  __shared__ double s[RED_THREADS];
  const int v = blockIdx.y;
  const double *a = V + (int64_t)v * n;
  double acc = 0;
  for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n; i += (int64_t)RED_BLOCKS * RED_THREADS) acc += a[i] * w[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int off = RED_THREADS / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) s[threadIdx.x] += s[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(int64_t)v * RED_BLOCKS + blockIdx.x] = s[0];
}

__global__ void k_mdot_final(const double *__restrict__ part, double *__restrict__ out, double *__restrict__ acc) {
  __shared__ double s[RED_BLOCKS];
  const int v = blockIdx.x;
  for (int i = threadIdx.x; i < RED_BLOCKS; i += blockDim.x) s[i] = part[(int64_t)v * RED_BLOCKS + i];
  __syncthreads();
  for (int off = RED_BLOCKS / 2; off > 0; off >>= 1) {
    for (int i = threadIdx.x; i < off; i += blockDim.x) s[i] += s[i + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[v] = s[0];
    if (acc) acc[v] += s[0];
  }
}

// w += sign * sum_v c[v] V_v
__global__ void k_maxpy(int64_t n, int nv, double sign, const double *__restrict__ c, const double *__restrict__ V, double *__restrict__ w) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int v = 0; v < nv; v++) s += c[v] * V[(int64_t)v * n + i];
  w[i] += sign * s;
}

__global__ void k_scale_into(int64_t n, const double *__restrict__ a, const double *__restrict__ num, double inv, double *__restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = a[i] * inv;
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

// build the sliced-ELL copy of J's CSR (pattern once, values whenever an assembly has changed them)
dErr mat_sell(_p_dMat *J, cudaStream_t s) {
  if (J->sell_valid || J->nrows == 0) return 0;
  const int64_t n = J->nrows, ns = (n + 31) / 32;
  const bool pattern = !J->d_sell_off;
  if (pattern) {
    int32_t *d_w;
    CUCHK(cudaMalloc(&d_w, ns * sizeof(int32_t)));
    k_sell_width<<<nb(32 * ns), 256, 0, s>>>(n, J->d_rowptr, ns, d_w);
    CUCHK(cudaGetLastError());
    std::vector<int32_t> w(ns);
    CUCHK(cudaMemcpyAsync(w.data(), d_w, ns * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CUCHK(cudaStreamSynchronize(s));
    cudaFree(d_w);
    std::vector<int64_t> off(ns + 1, 0);
    for (int64_t i = 0; i < ns; i++) off[i + 1] = off[i] + 32 * (int64_t)w[i];
    J->sell_len = off[ns];
    CUCHK(cudaMalloc(&J->d_sell_off, (ns + 1) * sizeof(int64_t)));
    CUCHK(cudaMalloc(&J->d_sell_col, std::max<int64_t>(J->sell_len, 1) * sizeof(int32_t)));
    CUCHK(cudaMalloc(&J->d_sell_val, std::max<int64_t>(J->sell_len, 1) * sizeof(double)));
    CUCHK(cudaMemcpyAsync(J->d_sell_off, off.data(), (ns + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  }
  k_sell_fill<<<nb(32 * ns), 256, 0, s>>>(n, ns, J->d_rowptr, J->d_col, J->d_val, J->d_sell_off, pattern ? J->d_sell_col : nullptr,
                                          J->d_sell_val);
  CUCHK(cudaGetLastError());
  CUCHK(cudaStreamSynchronize(s));  // the host vector above must outlive its copy
  J->sell_valid = true;
  return 0;
}

dErr mat_mult(_p_dMat *J, const double *x, double *y, cudaStream_t s) {
  if (J->nrows == 0) return 0;
  DCHK(mat_sell(J, s));
  k_sell<double, double><<<nb(J->nrows), 256, 0, s>>>(J->nrows, J->d_sell_off, J->d_sell_col, J->d_sell_val, x, y);
  CUCHK(cudaGetLastError());
  return 0;
}

// deterministic dot product into a device scalar, one launch (part: RED_BLOCKS doubles and a zeroed ticket, see
// dot_part_alloc)
dErr device_dot(int64_t n, const double *a, const double *b, double *part, double *out, cudaStream_t s) {
  k_dot1<<<dot_grid(n), RED_THREADS, 0, s>>>(n, a, b, part, out);
  CUCHK(cudaGetLastError());
  return 0;
}

// workspace of device_dot: RED_BLOCKS partials and the ticket word, zeroed
dErr dot_part_alloc(double **part) {
  CUCHK(cudaMalloc(part, (RED_BLOCKS + 1) * sizeof(double)));
  CUCHK(cudaMemset(*part, 0, (RED_BLOCKS + 1) * sizeof(double)));
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
  dPrecision inner_prec = dPREC_FP64;  // precision of the operator applies inside an FGMRES cycle
  double *d_V = nullptr, *d_Z = nullptr, *d_h = nullptr;  // FGMRES bases [(m+1) x n], [m x n], coefficients
  double *d_trial = nullptr;  // FGMRES with a correction: saved iterate and residual, the plain trial's iterate [3 x n]
  float *d_w32 = nullptr, *d_dinv32 = nullptr, *d_val32 = nullptr;  // FP32 Chebyshev workspace
  __nv_bfloat16 *d_val16 = nullptr;                                // BF16 Q1 values
  // optional preconditioner correction applied after the Chebyshev step: z += corr(r) (learned correction,
  // FGMRES only), judged against the plain preconditioner by paired trial cycles (fgmres_solve)
  dErr (*correction)(void *ctx, const double *r, double *z) = nullptr;
  void *correction_ctx = nullptr;
  bool correction_on = false, plain_cycle = false;
  // 0: every preconditioner application; 1: first vector of each restart cycle (the true residual);
  // 2: adaptive -- a trial of each against a plain cycle, then the one that won by more
  int correction_policy = 2, active_policy = 0;
  int cycle_pos = 0;  // position of the vector being preconditioned within the FGMRES cycle
  int64_t pc_applies = 0, correction_rejects = 0;
  // optional per-iteration monitor (CG: after every iterate, with x and r)
  dErr (*monitor)(void *ctx, int it, const double *x, const double *r) = nullptr;
  void *monitor_ctx = nullptr;
  // shell form (a coupled system without a dOperator, e.g. Stokes): the operator and the preconditioner are
  // callbacks on vectors of length n, run on shell_stream
  dErr (*shell_mult)(void *ctx, const double *x, double *y) = nullptr;
  dErr (*shell_pc)(void *ctx, const double *r, double *z) = nullptr;
  void *shell_ctx = nullptr;
  cudaStream_t shell_stream = 0;
  void *mg = nullptr;  // dPC_MG_Q1 hierarchy (mg.cu)
};

dErr mg_build(_p_dMat *J, int degree, bool fp32, void **out);
dErr mg_apply(void *m, const double *r, double *z, cudaStream_t s);
void mg_destroy(void *m);

static cudaStream_t kstream(const _p_dKSP *k) { return k->shell_mult ? k->shell_stream : k->op->fs->stream; }
dErr op_mult_prec(_p_dOperator *op, const double *x, double *y, dPrecision prec);
static dErr kmult(_p_dKSP *k, const double *x, double *y, dPrecision prec) {
  return k->shell_mult ? k->shell_mult(k->shell_ctx, x, y) : op_mult_prec(k->op, x, y, prec);
}

// a KSP over a shell operator and preconditioner (FGMRES or CG)
dErr ksp_create_shell(int64_t n, cudaStream_t stream, dKSPType type, dErr (*mult)(void *, const double *, double *),
                      dErr (*pc)(void *, const double *, double *), void *ctx, int restart, dKSP *ksp) {
  if (!mult || !ksp) return set_error("null argument");
  _p_dKSP *k = new _p_dKSP();
  k->op = nullptr;
  k->pmat = nullptr;
  k->type = type;
  k->pc = dPC_NONE;
  k->n = n;
  k->restart = restart;
  k->shell_mult = mult;
  k->shell_pc = pc;
  k->shell_ctx = ctx;
  k->shell_stream = stream;
  *ksp = k;
  return 0;
}

dErr ksp_get_operator(dKSP ksp, dOperator *op) {
  if (!ksp || !op) return set_error("null argument");
  if (ksp->shell_mult) return set_error("this KSP runs a shell operator");
  *op = ksp->op;
  return 0;
}

dErr ksp_set_monitor(dKSP ksp, dErr (*fn)(void *, int, const double *, const double *), void *ctx) {
  if (!ksp) return set_error("null KSP");
  ksp->monitor = fn;
  ksp->monitor_ctx = ctx;
  return 0;
}

dErr ksp_set_correction(dKSP ksp, dErr (*fn)(void *, const double *, double *), void *ctx) {
  if (!ksp) return set_error("null KSP");
  if (fn && ksp->type != dKSP_FGMRES) return set_error("a learned correction needs FGMRES (it is not a fixed linear operator)");
  ksp->correction = fn;
  ksp->correction_ctx = ctx;
  return 0;
}

static dErr ksp_alloc(_p_dKSP *k) {
  if (k->d_work) return 0;
  CUCHK(cudaMalloc(&k->d_work, 8 * std::max<int64_t>(k->n, 1) * sizeof(double)));
  DCHK(dot_part_alloc(&k->d_part));
  CUCHK(cudaMalloc(&k->d_s, 64 * sizeof(double)));
  CUCHK(cudaMalloc(&k->d_dinv, std::max<int64_t>(k->n, 1) * sizeof(double)));
  return 0;
}

static dErr pc_setup(_p_dKSP *k) {
  if (k->pc_ready || k->pc == dPC_NONE) return 0;
  cudaStream_t s = kstream(k);
  const int64_t n = k->n;
  if (!k->pmat) return set_error("preconditioner needs the Q1 matrix");
  k_diag_inv<<<nb(n), 256, 0, s>>>(n, k->pmat->d_rowptr, k->pmat->d_col, k->pmat->d_val, k->d_dinv);
  CUCHK(cudaGetLastError());
  if (k->pc == dPC_MG_Q1) {
    mg_destroy(k->mg);
    k->mg = nullptr;
    // smoothing one degree below the single-level Chebyshev (2 at the default 3): measured at 64^3, p=4, the
    // same iteration count as degree 3 for 20 % less time per solve
    DCHK(mg_build(k->pmat, std::max(2, k->cheb_degree - 1), k->pc_prec != dPREC_FP64, &k->mg));
  }
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
// Chebyshev-Jacobi on the Q1 matrix in FP32 (values, vectors and arithmetic), FP64 in/out
static dErr pc_apply_fp32(_p_dKSP *k, const double *r, double *z) {
  _p_dMat *J = k->pmat;
  cudaStream_t s = kstream(k);
  DCHK(mat_sell(J, s));
  const int64_t n = k->n, nnz = J->sell_len;  // values converted in the sliced layout, padding included
  const bool bf = k->pc_prec == dPREC_BF16;
  if (!k->d_w32) {
    CUCHK(cudaMalloc(&k->d_w32, 5 * std::max<int64_t>(n, 1) * sizeof(float)));
    CUCHK(cudaMalloc(&k->d_dinv32, std::max<int64_t>(n, 1) * sizeof(float)));
    k_convert<double, float><<<nb(n), 256, 0, s>>>(n, k->d_dinv, k->d_dinv32);
  }
  if (!bf && !k->d_val32) {
    CUCHK(cudaMalloc(&k->d_val32, std::max<int64_t>(nnz, 1) * sizeof(float)));
    k_convert<double, float><<<nb(nnz), 256, 0, s>>>(nnz, J->d_sell_val, k->d_val32);
  }
  if (bf && !k->d_val16) {
    CUCHK(cudaMalloc(&k->d_val16, std::max<int64_t>(nnz, 1) * sizeof(__nv_bfloat16)));
    k_val_to_bf16<<<nb(nnz), 256, 0, s>>>(nnz, J->d_sell_val, k->d_val16);
  }
  float *r32 = k->d_w32, *z32 = r32 + n, *d32 = z32 + n, *w32 = d32 + n;
  k_convert<double, float><<<nb(n), 256, 0, s>>>(n, r, r32);
  const double theta = 0.5 * (k->emax + k->emin), delta = 0.5 * (k->emax - k->emin), sigma = theta / delta;
  double rho = 1.0 / sigma;
  // the iterate alternates between z32 and w32 (each step reads one and writes the other) and ends in z32
  float *zc = (k->cheb_degree - 1) % 2 == 0 ? z32 : w32;
  k_cheb_first_t<float><<<nb(n), 256, 0, s>>>(n, k->d_dinv32, r32, (float)(1.0 / theta), d32, zc);
  for (int it = 1; it < k->cheb_degree; it++) {
    const double rho1 = 1.0 / (2.0 * sigma - rho);
    float *zn = zc == z32 ? w32 : z32;
    if (bf)
      k_sell_cheb<__nv_bfloat16, float><<<nb(n), 256, 0, s>>>(n, J->d_sell_off, J->d_sell_col, k->d_val16, k->d_dinv32, r32, zc,
                                                              (float)(rho1 * rho), (float)(2.0 * rho1 / delta), d32, zn);
    else
      k_sell_cheb<float, float><<<nb(n), 256, 0, s>>>(n, J->d_sell_off, J->d_sell_col, k->d_val32, k->d_dinv32, r32, zc,
                                                      (float)(rho1 * rho), (float)(2.0 * rho1 / delta), d32, zn);
    zc = zn;
    rho = rho1;
  }
  k_convert<float, double><<<nb(n), 256, 0, s>>>(n, z32, z);
  CUCHK(cudaGetLastError());
  return 0;
}

static dErr pc_apply_plain(_p_dKSP *k, const double *r, double *z);

static dErr pc_apply(_p_dKSP *k, const double *r, double *z) {
  k->pc_applies++;
  if (k->shell_pc) return k->shell_pc(k->shell_ctx, r, z);
  DCHK(pc_apply_plain(k, r, z));
  if (k->correction && k->correction_on && !k->plain_cycle && (k->active_policy == 0 || k->cycle_pos == 0))
    DCHK(k->correction(k->correction_ctx, r, z));
  return 0;
}

static dErr pc_apply_plain(_p_dKSP *k, const double *r, double *z) {
  const int64_t n = k->n;
  cudaStream_t s = kstream(k);
  if (k->pc == dPC_MG_Q1) return mg_apply(k->mg, r, z, s);  // FP64 V-cycle, or FP32 for FP32 / BF16 preconditioning
  if (k->pc == dPC_CHEBYSHEV_Q1 && k->pc_prec != dPREC_FP64) return pc_apply_fp32(k, r, z);
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
  _p_dMat *J = k->pmat;
  DCHK(mat_sell(J, s));
  // the iterate alternates between z and w (each fused step reads one and writes the other) and ends in z
  double *zc = (k->cheb_degree - 1) % 2 == 0 ? z : w;
  k_cheb_first<<<nb(n), 256, 0, s>>>(n, k->d_dinv, r, 1.0 / theta, d, zc);
  for (int it = 1; it < k->cheb_degree; it++) {
    const double rho1 = 1.0 / (2.0 * sigma - rho);
    double *zn = zc == z ? w : z;
    if (n > 0)
      k_sell_cheb<double, double><<<nb(n), 256, 0, s>>>(n, J->d_sell_off, J->d_sell_col, J->d_sell_val, k->d_dinv, r, zc, rho1 * rho,
                                                        2.0 * rho1 / delta, d, zn);
    zc = zn;
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

// one CG step after the convergence test: z = M r, rz' = r.z, p = z + (rz'/rz) p, rz = rz', q = A p, pq = p.q,
// x += (rz/pq) p, r -= (rz/pq) q, rr = r.r (S[4] = rz, S[1] = pq, S[2] = rr; S[0] = the previous step's rz)
static dErr cg_step(_p_dKSP *k, double *x, double *r, double *z, double *p, double *q, double *S, bool first) {
  const int64_t n = k->n;
  cudaStream_t s = kstream(k);
  DCHK(pc_apply(k, r, z));
  DCHK(device_dot(n, r, z, k->d_part, S + 4, s));
  if (first) CUCHK(cudaMemcpyAsync(p, z, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  else k_xpay_ratio<<<nb(n), 256, 0, s>>>(n, z, S + 4, S, p);  // S[0]: the previous step's rz
  DCHK(kmult(k, p, q, dPREC_FP64));
  DCHK(device_dot(n, p, q, k->d_part, S + 1, s));
  k_cg_update<<<dot_grid(n), RED_THREADS, 0, s>>>(n, S, p, q, x, r, k->d_part, S + 2);
  CUCHK(cudaGetLastError());
  return 0;
}

// the convergence test of a device-looped CG: S[8] counts iterations; the loop continues while ||r|| > tol and fewer
// than maxit iterations were done (the host loop's test, on the device)
__global__ void k_cg_check(cudaGraphConditionalHandle h, double *S, double tol, double maxit) {
  S[8] += 1.0;
  cudaGraphSetConditional(h, (sqrt(S[2]) > tol && S[8] < maxit) ? 1u : 0u);
}

// Preconditioned CG (PETSc KSPCG). The first step runs eagerly (it makes the lazily allocated work arrays); the
// remaining steps run as one CUDA graph: a while-conditional node whose body is the step's launches (captured once per
// solve) followed by the convergence test on the device, so the whole solve costs one graph launch and one read of
// r.r. The graph is skipped with a monitor (host code per iterate), a learned correction, a shell operator or an
// operator on mixed orders / with its own launch form, which step eagerly with a host test per iteration.
static dErr cg_solve(_p_dKSP *k, const double *b, double *x, double rtol, int maxit, int *its, double *rnorm) {
  const int64_t n = k->n;
  cudaStream_t s = kstream(k);
  double *r = k->d_work, *z = k->d_work + n, *p = k->d_work + 2 * n, *q = k->d_work + 3 * n;
  double *S = k->d_s;  // S[0]=previous rz S[1]=pq S[2]=rr S[3]=bb S[4]=rz S[8]=iterations (device loop)
  DCHK(kmult(k, x, q, dPREC_FP64));
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
  if (k->monitor) DCHK(k->monitor(k->monitor_ctx, 0, x, r));
  // the operator's own launch forms for mixed orders (persistent kernel, its own graph) stay eager
  const bool graph = !k->monitor && !k->correction && !k->shell_mult && k->op->fs->uniform && k->op->launch == dLAUNCH_DEFAULT;
  DCHK(cg_step(k, x, r, z, p, q, S, true));
  if (k->monitor) DCHK(k->monitor(k->monitor_ctx, 1, x, r));
  DCHK(read_scalar(S + 2, &rr, s));
  *its = 1;
  if (!(sqrt(rr) > rtol * bn) || maxit <= 1) {
    *rnorm = sqrt(rr) / bn;
    return 0;
  }
  if (!graph) {
    for (int it = 1; it < maxit; it++) {
      DCHK(cg_step(k, x, r, z, p, q, S, false));
      if (k->monitor) DCHK(k->monitor(k->monitor_ctx, it + 1, x, r));
      DCHK(read_scalar(S + 2, &rr, s));
      *its = it + 1;
      if (!(sqrt(rr) > rtol * bn)) break;
    }
    *rnorm = sqrt(rr) / bn;
    return 0;
  }
  const double one = 1.0;
  CUCHK(cudaMemcpyAsync(S + 8, &one, sizeof one, cudaMemcpyHostToDevice, s));
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cs = nullptr;
  dErr err = 0;
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams cp = {};
  cudaGraphNode_t node;
  if (cudaGraphCreate(&g, 0) != cudaSuccess || cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
    err = set_error("CG graph: conditional handle creation failed");
  } else {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) != cudaSuccess) err = set_error("CG graph: conditional node creation failed");
  }
  const int64_t applies = k->pc_applies;  // the capture runs pc_apply's host bookkeeping once; the loop counts below
  if (!err) {  // the body: one step and the test, captured on a private stream (the legacy stream cannot be captured)
    _p_dFS *fs = k->op->fs;
    CUCHK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    fs->stream = cs;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaError_t ce = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      err = cg_step(k, x, r, z, p, q, S, false);
      if (!err) {
        k_cg_check<<<1, 1, 0, cs>>>(h, S, rtol * bn, (double)maxit);
        if (cudaGetLastError() != cudaSuccess) err = set_error("CG graph: test kernel launch failed");
      }
      ce = cudaStreamEndCapture(cs, &body);
    }
    fs->stream = s;
    if (!err && ce != cudaSuccess) err = set_error("CG graph capture failed: %s", cudaGetErrorString(ce));
  }
  if (!err && cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) err = set_error("CG graph instantiation failed");
  if (!err && cudaGraphLaunch(exec, s) != cudaSuccess) err = set_error("CG graph launch failed");
  double hs[9];
  if (!err && cudaMemcpyAsync(hs, S, sizeof hs, cudaMemcpyDeviceToHost, s) != cudaSuccess) err = set_error("CG: reading the result failed");
  if (!err && cudaStreamSynchronize(s) != cudaSuccess) err = set_error("CG graph execution failed");
  if (exec) cudaGraphExecDestroy(exec);
  if (g) cudaGraphDestroy(g);
  if (cs) cudaStreamDestroy(cs);
  if (err) return err;
  rr = hs[2];
  *its = (int)hs[8];
  k->pc_applies = applies + (*its - 1);  // one preconditioner application per iteration of the device loop
  *rnorm = sqrt(rr) / bn;
  return 0;
}

// Right-preconditioned FGMRES(m) (Saad Alg. 9.6) with classical Gram-Schmidt applied twice (CGS2) in FP64.
// Each cycle starts from the true residual b - A x computed with the FP64 operator; the operator applies
// inside a cycle and the preconditioner run in k->pc_prec (FP32 for the mixed-precision solver). The
// flexible (Z) basis makes the varying inner precision and a learned correction admissible.
//
// With a correction the plain preconditioner judges it: a trial runs one cycle with the plain preconditioner and one
// with the correction from the same iterate and keeps the iterate with the smaller true residual (both cycles count
// as iterations). Policy 2 (adaptive) tries the correction on every vector, then on the first vector of the cycle;
// policies 0 and 1 try theirs once. Afterwards the correction runs in the mode that beat its plain cycle by the larger
// margin, or is dropped for the rest of the solve if neither did; a later cycle with it that reduces the true residual
// by less than 1 % (or gives a non-finite one) drops it too.
static dErr fgmres_solve(_p_dKSP *k, const double *b, double *x, double rtol, int maxit, int *its, double *rnorm) {
  const int64_t n = k->n;
  const int m = std::max(1, k->restart);
  cudaStream_t s = kstream(k);
  if (!k->d_V) {
    CUCHK(cudaMalloc(&k->d_V, (size_t)(m + 1) * n * sizeof(double)));
    CUCHK(cudaMalloc(&k->d_Z, (size_t)m * n * sizeof(double)));
    CUCHK(cudaMalloc(&k->d_h, (size_t)(2 * (m + 2) + (m + 1) * RED_BLOCKS) * sizeof(double)));
  }
  if (k->correction && !k->d_trial) CUCHK(cudaMalloc(&k->d_trial, 3 * std::max<int64_t>(n, 1) * sizeof(double)));
  double *V = k->d_V, *Z = k->d_Z, *h1 = k->d_h, *h2 = k->d_h + (m + 2), *mpart = k->d_h + 2 * (m + 2);
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), yv(m), hcol(m + 2);
  double bb;
  DCHK(device_dot(n, b, b, k->d_part, k->d_s, s));
  DCHK(read_scalar(k->d_s, &bb, s));
  const double bn = sqrt(bb) > 0 ? sqrt(bb) : 1.0;
  int total = 0;
  // V0 = b - A x (FP64 operator) and its norm
  auto true_residual = [&](double &beta) -> dErr {
    DCHK(kmult(k, x, V, dPREC_FP64));
    k_axpby<<<nb(n), 256, 0, s>>>(n, 1.0, nullptr, nullptr, b, -1.0, V);
    double rr;
    DCHK(device_dot(n, V, V, k->d_part, k->d_s, s));
    DCHK(read_scalar(k->d_s, &rr, s));
    beta = sqrt(rr);
    return 0;
  };
  // one restart cycle from x, whose residual (norm beta) is in V0: Arnoldi with the preconditioner as set, x += Z y
  auto run_cycle = [&](double beta) -> dErr {
    k_scale_into<<<nb(n), 256, 0, s>>>(n, V, nullptr, 1.0 / beta, V);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m && total < maxit;) {
      double *w = V + (size_t)(j + 1) * n;
      k->cycle_pos = j;
      DCHK(pc_apply(k, V + (size_t)j * n, Z + (size_t)j * n));
      DCHK(kmult(k, Z + (size_t)j * n, w, k->pc_prec));
      const int nv = j + 1;
      k_mdot_partial<<<dim3(RED_BLOCKS, nv), RED_THREADS, 0, s>>>(n, nv, V, w, mpart);
      k_mdot_final<<<nv, 1024, 0, s>>>(mpart, h1, nullptr);
      k_maxpy<<<nb(n), 256, 0, s>>>(n, nv, -1.0, h1, V, w);
      k_mdot_partial<<<dim3(RED_BLOCKS, nv), RED_THREADS, 0, s>>>(n, nv, V, w, mpart);
      k_mdot_final<<<nv, 1024, 0, s>>>(mpart, h2, h1);
      k_maxpy<<<nb(n), 256, 0, s>>>(n, nv, -1.0, h2, V, w);
      DCHK(device_dot(n, w, w, k->d_part, h1 + nv, s));
      CUCHK(cudaMemcpyAsync(hcol.data(), h1, (nv + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
      CUCHK(cudaStreamSynchronize(s));
      const double hn = sqrt(hcol[nv]);
      if (hn > 0) k_scale_into<<<nb(n), 256, 0, s>>>(n, w, nullptr, 1.0 / hn, w);
      for (int i = 0; i < nv; i++) H[(size_t)i * m + j] = hcol[i];
      for (int i = 0; i < j; i++) {  // previous Givens rotations
        const double a = H[(size_t)i * m + j], c = H[(size_t)(i + 1) * m + j];
        H[(size_t)i * m + j] = cs[i] * a + sn[i] * c;
        H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
      }
      const double a = H[(size_t)j * m + j], r = hypot(a, hn);
      cs[j] = r > 0 ? a / r : 1.0;
      sn[j] = r > 0 ? hn / r : 0.0;
      H[(size_t)j * m + j] = r;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      total++;
      j++;
      if (!(fabs(g[j]) > rtol * bn) || hn == 0) break;
    }
    for (int i = j - 1; i >= 0; i--) {  // H y = g, upper triangular
      double t = g[i];
      for (int l = i + 1; l < j; l++) t -= H[(size_t)i * m + l] * yv[l];
      yv[i] = H[(size_t)i * m + i] != 0 ? t / H[(size_t)i * m + i] : 0.0;
    }
    CUCHK(cudaMemcpyAsync(h1, yv.data(), j * sizeof(double), cudaMemcpyHostToDevice, s));
    k_maxpy<<<nb(n), 256, 0, s>>>(n, j, 1.0, h1, Z, x);
    CUCHK(cudaStreamSynchronize(s));
    CUCHK(cudaGetLastError());
    return 0;
  };
  const int policy = k->correction_policy;
  const int ntrials = policy == 2 ? 2 : 1;  // policy 2: every vector, then the first vector
  double ratio[2] = {-1, -1};              // trial: corrected / plain true residual, per correction mode
  int trials = 0;
  double res = 0, prev = -1;
  k->correction_on = k->correction != nullptr;
  k->plain_cycle = false;
  for (;;) {
    double beta;
    DCHK(true_residual(beta));
    res = beta / bn;
    if (!(beta > rtol * bn) || total >= maxit) break;
    if (k->correction_on && trials == ntrials) {  // after the trials: a stagnating corrected cycle drops it
      if (prev > 0 && !(beta < 0.99 * prev)) {
        k->correction_on = false;
        k->correction_rejects++;
      }
    }
    prev = beta;
    if (k->correction_on && trials < ntrials) {
      const int mode = policy == 2 ? trials : policy;
      double *xs = k->d_trial, *rs = k->d_trial + n, *xp = k->d_trial + 2 * n;
      CUCHK(cudaMemcpyAsync(xs, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      CUCHK(cudaMemcpyAsync(rs, V, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      k->plain_cycle = true;  // the plain cycle
      DCHK(run_cycle(beta));
      double bp;
      DCHK(true_residual(bp));
      CUCHK(cudaMemcpyAsync(xp, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      double bc = bp;
      if (bp > rtol * bn && total < maxit) {  // the corrected cycle from the same iterate
        CUCHK(cudaMemcpyAsync(x, xs, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        CUCHK(cudaMemcpyAsync(V, rs, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        k->plain_cycle = false;
        k->active_policy = mode;
        DCHK(run_cycle(beta));
        DCHK(true_residual(bc));
        if (!(bc < bp)) CUCHK(cudaMemcpyAsync(x, xp, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        ratio[mode] = std::isfinite(bc) ? bc / bp : 1e300;
      }
      k->plain_cycle = false;
      if (++trials == ntrials) {  // the better mode, or no correction if none beat its plain cycle
        int best = -1;
        for (int q = 0; q < 2; q++)
          if (ratio[q] >= 0 && ratio[q] < 1.0 && (best < 0 || ratio[q] < ratio[best])) best = q;
        if (best < 0) {
          k->correction_on = false;
          k->correction_rejects++;
        } else {
          k->active_policy = best;
        }
      }
      prev = -1;  // the stagnation test applies to cycles after the trials
      continue;   // the next restart recomputes the true residual of the iterate kept
    }
    DCHK(run_cycle(beta));
  }
  k->plain_cycle = false;
  *its = total;
  *rnorm = res;
  return 0;
}

dPrecision ksp_pc_precision(dKSP ksp) { return ksp ? ksp->pc_prec : dPREC_FP64; }

extern "C" {

dErr dKSPCreate(dOperator op, dMat pmat, dKSPType type, dPCType pc, dKSP *ksp) {
  if (!op || !ksp) return set_error("dKSPCreate: null argument");
  if (type != dKSP_CG && type != dKSP_FGMRES) return set_error("KSP type %d not supported", (int)type);
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
  cudaFree(k->d_V);
  cudaFree(k->d_Z);
  cudaFree(k->d_h);
  cudaFree(k->d_trial);
  cudaFree(k->d_w32);
  cudaFree(k->d_dinv32);
  cudaFree(k->d_val32);
  cudaFree(k->d_val16);
  mg_destroy(k->mg);
  delete k;
  *ksp = nullptr;
  return 0;
}

dErr dKSPSetOptions(dKSP ksp, dInt cheb_degree, dPrecision pc_precision, dInt restart) {
  if (!ksp) return set_error("null KSP");
  if (cheb_degree < 1) return set_error("Chebyshev degree must be >= 1");
  ksp->cheb_degree = cheb_degree;
  ksp->pc_prec = pc_precision;
  if (restart < 1 || restart > 200) return set_error("restart %d out of range [1,200]", restart);
  if (ksp->restart != restart) {
    cudaFree(ksp->d_V);
    cudaFree(ksp->d_Z);
    cudaFree(ksp->d_h);
    ksp->d_V = ksp->d_Z = ksp->d_h = nullptr;
  }
  ksp->restart = restart;
  ksp->pc_ready = false;
  mg_destroy(ksp->mg);
  ksp->mg = nullptr;
  cudaFree(ksp->d_w32);
  cudaFree(ksp->d_dinv32);
  cudaFree(ksp->d_val32);
  cudaFree(ksp->d_val16);
  ksp->d_w32 = nullptr, ksp->d_dinv32 = nullptr, ksp->d_val32 = nullptr, ksp->d_val16 = nullptr;
  return 0;
}

dErr dKSPSetCorrectionPolicy(dKSP ksp, int policy) {
  if (!ksp) return set_error("null KSP");
  if (policy < 0 || policy > 2) return set_error("correction policy %d not in {0, 1, 2}", policy);
  ksp->correction_policy = policy;
  return 0;
}

dErr dKSPGetStats(dKSP ksp, int64_t *pc_applies, int64_t *correction_rejects, int *correction_active) {
  if (!ksp) return set_error("null KSP");
  if (pc_applies) *pc_applies = ksp->pc_applies;
  if (correction_rejects) *correction_rejects = ksp->correction_rejects;
  if (correction_active) *correction_active = ksp->correction_on;
  return 0;
}

dErr dKSPSetOperators(dKSP ksp, dOperator op, dMat pmat) {
  if (!ksp) return set_error("null KSP");
  if (ksp->shell_mult) return set_error("this KSP runs a shell operator (a coupled system); it takes no dOperator or dMat");
  if (op) {
    if (op->fs->n * op->fs->bs != ksp->n) return set_error("operator size differs from the KSP's");
    ksp->op = op;
  }
  if (pmat) {
    if (pmat->nrows != ksp->n) return set_error("matrix size differs from the KSP's");
    ksp->pmat = pmat;
  }
  ksp->pc_ready = false;
  cudaFree(ksp->d_w32);
  cudaFree(ksp->d_dinv32);
  cudaFree(ksp->d_val32);
  cudaFree(ksp->d_val16);
  ksp->d_w32 = nullptr, ksp->d_dinv32 = nullptr, ksp->d_val32 = nullptr, ksp->d_val16 = nullptr;
  return 0;
}

}  // extern "C"

// solve without treating the iteration limit as an error (inexact Newton steps); rnorm = ||b - A x|| / ||b||
dErr ksp_solve(dKSP ksp, const double *b, double *x, double rtol, int maxit, int *its, double *rnorm) {
  if (!ksp) return set_error("null KSP");
  DCHK(ksp_alloc(ksp));
  DCHK(pc_setup(ksp));
  int it = 0;
  double rn = 0;
  dErr e = ksp->type == dKSP_FGMRES ? fgmres_solve(ksp, b, x, rtol, maxit, &it, &rn) : cg_solve(ksp, b, x, rtol, maxit, &it, &rn);
  if (its) *its = it;
  if (rnorm) *rnorm = rn;
  return e;
}

// the KSP's preconditioner alone (set up on first use): z = M^-1 r, e.g. a block of a coupled preconditioner
dErr ksp_pc_only(dKSP ksp, const double *r, double *z) {
  if (!ksp) return set_error("null KSP");
  DCHK(ksp_alloc(ksp));
  DCHK(pc_setup(ksp));
  return pc_apply_plain(ksp, r, z);
}

extern "C" {

dErr dKSPSolve(dKSP ksp, const dScalar *b, dScalar *x, dReal rtol, dInt maxit, dInt *its, dReal *rnorm) {
  Range range_("KSPSolve");
  int it = 0;
  double rn = 0;
  DCHK(ksp_solve(ksp, b, x, rtol, maxit, &it, &rn));
  if (its) *its = it;
  if (rnorm) *rnorm = rn;
  if (!(rn <= rtol))
    return set_error("%s did not converge in %d iterations (relative residual %g)", ksp->type == dKSP_FGMRES ? "FGMRES" : "CG", it, rn);
  return 0;
}

}  // extern "C"
