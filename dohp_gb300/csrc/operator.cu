// Fused matrix-free operator apply (the hot path) and per-quadrature-point geometry.
//
// One apply = the iterator loop of EllipShellMatMult (src/fs/tests/ellip.c:442-472) / ElastShellMatMult
// (src/fs/tests/elast.c:311-341): gather the element's nodal values through E, GRAD (dEFSApply,
// src/jacobi/impls/tensor/efstopo.c:395-402), pointwise q-function, GRAD_TRANSPOSE (efstopo.c:404-418),
// then E^T. The element work is fused into one kernel that keeps the element in shared memory:
//   interpolate u to the Gauss points with three 1-D passes (B along x, y, z), take reference gradients
//   with the collocation derivative at the Gauss points (Dq = derivative of the Lagrange basis on the Gauss
//   points; exact because u restricted to the points is a degree-p polynomial in each direction), apply the
//   q-function with precomputed geometric factors, and run the transposes back to the nodes.
// Geometric factors are computed once per mesh (the reference recomputes them every apply,
// fsrulesetit.c:548-557): G = k w det(J) J^{-1} J^{-T} (6 values) for diffusion, {J^{-1}, w det J}
// (10 values) for elasticity, all FP64 (J^{-1} by cofactors and 1/det as dGeomInvert3, dohpgeom.h:57-79).
#include <stdio.h>

#include <mutex>

#include "element.cuh"

using namespace dgb;

dErr fs_restrict(_p_dFS *fs, const double *x, double *g, int add);
dErr fs_restrict32(_p_dFS *fs, const float *x, double *g, int add);
dErr tc_diffusion_apply(_p_dFS *fs, const double *x, const void *geo16, void **bops_cache, float *yexp, double *y);
dErr tc_check(_p_dFS *fs);

namespace {

__device__ int g_negative_jacobian;

// trilinear Jacobian of the Q1 coordinate map at reference point (s,t,u); X = [8][3] in tensor vertex order
__device__ __forceinline__ void q1_jacobian(const double *X, double s, double t, double u, double J[9]) {
  const double bs[2] = {0.5 * (1 - s), 0.5 * (1 + s)}, bt[2] = {0.5 * (1 - t), 0.5 * (1 + t)}, bu[2] = {0.5 * (1 - u), 0.5 * (1 + u)};
  const double dd[2] = {-0.5, 0.5};
  for (int i = 0; i < 9; i++) J[i] = 0;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const int a = v >> 2, b = (v >> 1) & 1, c = v & 1;
    const double g0 = dd[a] * bt[b] * bu[c], g1 = bs[a] * dd[b] * bu[c], g2 = bs[a] * bt[b] * dd[c];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double x = X[v * 3 + d];
      J[d * 3 + 0] += x * g0;
      J[d * 3 + 1] += x * g1;
      J[d * 3 + 2] += x * g2;
    }
  }
}

// cofactor inverse (same formula as dGeomInvert3)
__device__ __forceinline__ double invert3(const double a[9], double b[9]) {
  const double c0 = a[4] * a[8] - a[7] * a[5];
  const double c3 = -(a[3] * a[8] - a[6] * a[5]);
  const double c6 = a[3] * a[7] - a[6] * a[4];
  const double det = a[0] * c0 + a[1] * c3 + a[2] * c6;
  const double id = 1.0 / det;
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

struct RuleTab {
  double x[MAXP], w[MAXP];
};

// one thread per FAST quadrature point. mode 0: G (6, SoA per element), mode 1: {jinv(9), jw} (10, SoA)
__global__ void k_geometry(int64_t nelem, const int32_t *__restrict__ edeg, const int32_t *__restrict__ qoff,
                           const double *__restrict__ coords, const RuleTab *__restrict__ rules,
                           const double *__restrict__ kq, int mode, double *__restrict__ geo) {
  const int64_t e = blockIdx.x;
  if (e >= nelem) return;
  const int pa = edeg[3 * e], pb = edeg[3 * e + 1], pc = edeg[3 * e + 2];
  const int Qa = pa + 1, Qb = pb + 1, Qc = pc + 1, nq = Qa * Qb * Qc;
  const int64_t q0 = qoff[e];
  const double *X = coords + e * 24;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const int a = q / (Qb * Qc), b = (q / Qc) % Qb, c = q % Qc;
    double J[9], Ji[9];
    q1_jacobian(X, rules[pa].x[a], rules[pb].x[b], rules[pc].x[c], J);
    const double det = invert3(J, Ji);
    if (det < 0.) atomicExch(&g_negative_jacobian, 1);
    const double jw = rules[pa].w[a] * rules[pb].w[b] * rules[pc].w[c] * det;
    if (mode == 0) {
      const double s = jw * (kq ? kq[q0 + q] : 1.0);
      double G[6];
      G[0] = s * (Ji[0] * Ji[0] + Ji[1] * Ji[1] + Ji[2] * Ji[2]);
      G[1] = s * (Ji[0] * Ji[3] + Ji[1] * Ji[4] + Ji[2] * Ji[5]);
      G[2] = s * (Ji[0] * Ji[6] + Ji[1] * Ji[7] + Ji[2] * Ji[8]);
      G[3] = s * (Ji[3] * Ji[3] + Ji[4] * Ji[4] + Ji[5] * Ji[5]);
      G[4] = s * (Ji[3] * Ji[6] + Ji[4] * Ji[7] + Ji[5] * Ji[8]);
      G[5] = s * (Ji[6] * Ji[6] + Ji[7] * Ji[7] + Ji[8] * Ji[8]);
      for (int i = 0; i < 6; i++) geo[q0 * 6 + (int64_t)i * nq + q] = G[i];
    } else {
      for (int i = 0; i < 9; i++) geo[q0 * 10 + (int64_t)i * nq + q] = Ji[i];
      geo[q0 * 10 + 9LL * nq + q] = jw;
    }
  }
}

// ------------------------------------------------------------------------------------------ fused element apply
// Elements per block chosen so a 256-thread block has a few hundred outputs per pass.
template <int N>
struct Tile {
  static constexpr int EPB = N <= 2 ? 32 : N == 3 ? 16 : N == 4 ? 8 : N == 5 ? 4 : N <= 7 ? 2 : 1;
};
template <int N>
struct ETile {
  static constexpr int EPB = N <= 3 ? 8 : N == 4 ? 4 : N == 5 ? 2 : 1;
};

// y_exp = (B^T Dq^T) G (Dq B) E x for cap consecutive elements per block (uniform order, Boolean E)
template <int N, typename T, int KIND, typename GT = T, bool BF = false>
__global__ void __launch_bounds__(256) k_uniform(ElemArgs A, int64_t nelem, int cap) {
  extern __shared__ unsigned char raw[];
  const int64_t e0 = (int64_t)blockIdx.x * cap;
  const int ne = (int)min((int64_t)cap, nelem - e0);
  group_apply<N, T, KIND, GT, BF>(A, nullptr, e0, ne, cap, reinterpret_cast<T *>(raw));
}

template <int N, typename T, int KIND, typename GT = T, bool BF = false>
dErr launch_uniform(_p_dFS *fs, const double *x, const GT *geo, double lam, double mu, T *yexp, double *stash = nullptr,
                    const double *dcache = nullptr) {
  constexpr int cap = KIND == dOP_ELASTICITY ? ETile<N>::EPB : Tile<N>::EPB;
  ElemArgs A{};
  A.xstart = fs->d_xstart;
  A.qoff = fs->d_qoff;
  A.emap = fs->d_emap;
  A.n = fs->n;
  A.x = x;
  A.geo = geo;
  A.tab_all = fs->d_fast_tab;
  A.yexp = yexp;
  A.lam = lam;
  A.mu = mu;
  A.stash = stash;
  A.dcache = dcache;
  const size_t smem = (size_t)group_smem_elems(N, KIND, cap) * sizeof(T);
  CUCHK(cudaFuncSetAttribute(k_uniform<N, T, KIND, GT, BF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_uniform<N, T, KIND, GT, BF><<<(unsigned)((fs->nelem + cap - 1) / cap), 256, smem, fs->stream>>>(A, fs->nelem, cap);
  CUCHK(cudaGetLastError());
  return 0;
}

template <int N, typename T>
dErr launch_diffusion(_p_dFS *fs, const double *x, const T *geo, T *yexp) {
  return launch_uniform<N, T, dOP_DIFFUSION>(fs, x, geo, 0, 0, yexp);
}

template <int KIND>
dErr svk_launch(_p_dFS *fs, const double *x, const double *geo, double lam, double mu, double *yexp, double *stash,
                const double *dcache = nullptr) {
  switch (fs->p + 1) {
    case 2: return launch_uniform<2, double, KIND>(fs, x, geo, lam, mu, yexp, stash, dcache);
    case 3: return launch_uniform<3, double, KIND>(fs, x, geo, lam, mu, yexp, stash, dcache);
    case 4: return launch_uniform<4, double, KIND>(fs, x, geo, lam, mu, yexp, stash, dcache);
    case 5: return launch_uniform<5, double, KIND>(fs, x, geo, lam, mu, yexp, stash, dcache);
    case 6: return launch_uniform<6, double, KIND>(fs, x, geo, lam, mu, yexp, stash, dcache);
    case 7: return launch_uniform<7, double, KIND>(fs, x, geo, lam, mu, yexp, stash, dcache);
    case 8: return launch_uniform<8, double, KIND>(fs, x, geo, lam, mu, yexp, stash, dcache);
    case 9: return launch_uniform<9, double, KIND>(fs, x, geo, lam, mu, yexp, stash, dcache);
  }
  return ::dgb::set_error("degree %d not supported", fs->p);
}

template <int N>
dErr launch_diffusion_bf16(_p_dFS *fs, const double *x, const __nv_bfloat16 *geo, float *yexp) {
  return launch_uniform<N, float, dOP_DIFFUSION, __nv_bfloat16, true>(fs, x, geo, 0, 0, yexp);
}

template <int N, typename T>
dErr launch_elasticity(_p_dFS *fs, const double *x, const T *geo, T lam, T mu, T *yexp) {
  return launch_uniform<N, T, dOP_ELASTICITY>(fs, x, geo, (double)lam, (double)mu, yexp);
}

}  // namespace

// ----------------------------------------------------------------------------------------------------------
// geometric factors at the FAST points of every element into out (mode 0: 6 per point with coefficient kq,
// mode 1: {J^-1, w det J}, 10 per point); a negative Jacobian anywhere is an error
dErr geometry_fill(_p_dFS *fs, int mode, const double *kq, double *out) {
  RuleTab h[MAXP];
  for (int p = 1; p < MAXP; p++) gauss_rule(p + 1, h[p].x, h[p].w);
  RuleTab *d_rules;
  CUCHK(cudaMalloc(&d_rules, sizeof h));
  CUCHK(cudaMemcpyAsync(d_rules, h, sizeof h, cudaMemcpyHostToDevice, fs->stream));
  int zero = 0;
  CUCHK(cudaMemcpyToSymbolAsync(g_negative_jacobian, &zero, sizeof zero, 0, cudaMemcpyHostToDevice, fs->stream));
  k_geometry<<<(unsigned)fs->nelem, 128, 0, fs->stream>>>(fs->nelem, fs->d_edeg, fs->d_qoff, fs->d_coords, d_rules, kq, mode, out);
  CUCHK(cudaGetLastError());
  int neg = 0;
  CUCHK(cudaMemcpyFromSymbolAsync(&neg, g_negative_jacobian, sizeof neg, 0, cudaMemcpyDeviceToHost, fs->stream));
  CUCHK(cudaStreamSynchronize(fs->stream));
  cudaFree(d_rules);
  if (neg) return set_error("Negative Jacobian in the element geometry");
  return 0;
}

dErr op_compute_geometry(_p_dOperator *op) {
  _p_dFS *fs = op->fs;
  if (op->kind == dOP_PLAPLACE_JACOBIAN) {  // factors come from the stash (plap.cu)
    if (op->geo_valid) return 0;
    return set_error("p-Laplacian Jacobian has no stash: call dOperatorComputePLaplaceStash, dOperatorPLaplaceFunction "
                     "or dOperatorSetQuadratureData first");
  }
  const int mode = op->kind == dOP_ELASTICITY ? 1 : 0;
  const int ncomp = mode ? 10 : 6;
  if (op->geo_valid && op->geo_kind == mode) return 0;
  cudaFree(op->d_geo);
  op->d_geo = nullptr;
  CUCHK(cudaMalloc(&op->d_geo, (size_t)fs->nq * ncomp * sizeof(double)));
  DCHK(geometry_fill(fs, mode, op->kind == dOP_DIFFUSION ? op->d_k : nullptr, op->d_geo));
  if (op->d_geo32) {
    cudaFree(op->d_geo32);
    op->d_geo32 = nullptr;
  }
  if (op->d_geo16) {
    cudaFree(op->d_geo16);
    op->d_geo16 = nullptr;
  }
  if (op->d_geoff) {
    cudaFree(op->d_geoff);
    op->d_geoff = nullptr;
  }
  op->geo_valid = true;
  op->geo_kind = mode;
  return 0;
}

template <typename T>
dErr diffusion_apply_t(_p_dFS *fs, const double *x, const T *geo, T *yexp) {
  if (!fs->uniform) return set_error("fused uniform-order diffusion apply called on a space with per-element orders (hp spaces apply through the order-bucket launches)");
  switch (fs->p + 1) {
    case 2: return launch_diffusion<2, T>(fs, x, geo, yexp);
    case 3: return launch_diffusion<3, T>(fs, x, geo, yexp);
    case 4: return launch_diffusion<4, T>(fs, x, geo, yexp);
    case 5: return launch_diffusion<5, T>(fs, x, geo, yexp);
    case 6: return launch_diffusion<6, T>(fs, x, geo, yexp);
    case 7: return launch_diffusion<7, T>(fs, x, geo, yexp);
    case 8: return launch_diffusion<8, T>(fs, x, geo, yexp);
    case 9: return launch_diffusion<9, T>(fs, x, geo, yexp);
  }
  return set_error("degree %d not supported", fs->p);
}

template <typename T>
static dErr elasticity_apply_t(_p_dFS *fs, const double *x, const T *geo, T lam, T mu, T *yexp) {
  if (!fs->uniform) return set_error("fused elasticity apply needs a uniform-degree space (use the hp path)");
  switch (fs->p + 1) {
    case 2: return launch_elasticity<2, T>(fs, x, geo, lam, mu, yexp);
    case 3: return launch_elasticity<3, T>(fs, x, geo, lam, mu, yexp);
    case 4: return launch_elasticity<4, T>(fs, x, geo, lam, mu, yexp);
    case 5: return launch_elasticity<5, T>(fs, x, geo, lam, mu, yexp);
    case 6: return launch_elasticity<6, T>(fs, x, geo, lam, mu, yexp);
    case 7: return launch_elasticity<7, T>(fs, x, geo, lam, mu, yexp);
    case 8: return launch_elasticity<8, T>(fs, x, geo, lam, mu, yexp);
    case 9: return launch_elasticity<9, T>(fs, x, geo, lam, mu, yexp);
  }
  return set_error("degree %d not supported", fs->p);
}

dErr hp_mult_expanded(_p_dOperator *op, const double *x, double *yexp);

dErr op_mult_expanded(_p_dOperator *op, const double *x, double *yexp) {
  _p_dFS *fs = op->fs;
  if (!fs->uniform || op->launch != dLAUNCH_DEFAULT) return hp_mult_expanded(op, x, yexp);
  DCHK(op_compute_geometry(op));
  if (op->kind == dOP_DIFFUSION) return diffusion_apply_t<double>(fs, x, op->d_geo, yexp);
  if (op->kind == dOP_ELASTICITY && op->svk_state) return svk_launch<K_SVK_JAC>(fs, x, op->d_geo, op->lam, op->mu, yexp, op->d_svk);
  if (op->kind == dOP_ELASTICITY) return elasticity_apply_t<double>(fs, x, op->d_geo, op->lam, op->mu, yexp);
  if (op->kind == dOP_PLAPLACE_JACOBIAN) return diffusion_apply_t<double>(fs, x, op->d_geo, yexp);  // G from the stash
  return set_error("operator kind %d not built yet", (int)op->kind);
}

__global__ void k_to_float(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// FP32 element arithmetic (geometric factors rounded to FP32 once), FP64 input and FP64 restriction
static dErr op_mult_fp32(_p_dOperator *op, const double *x, double *y) {
  _p_dFS *fs = op->fs;
  if (op->kind != dOP_DIFFUSION && op->kind != dOP_ELASTICITY && op->kind != dOP_PLAPLACE_JACOBIAN)
    return set_error("FP32 apply for operator kind %d not built yet", (int)op->kind);
  if (op->svk_state) return set_error("FP32 St. Venant-Kirchhoff Jacobian not built (use FP64)");
  DCHK(op_compute_geometry(op));
  const int64_t ng = fs->nq * (op->kind == dOP_ELASTICITY ? 10 : 6);
  if (!op->d_geo32) {
    CUCHK(cudaMalloc(&op->d_geo32, ng * sizeof(float)));
    k_to_float<<<(unsigned)((ng + 255) / 256), 256, 0, fs->stream>>>(ng, op->d_geo, op->d_geo32);
    CUCHK(cudaGetLastError());
  }
  if (!op->d_y32) CUCHK(cudaMalloc(&op->d_y32, fs->nexp * fs->bs * sizeof(float)));
  if (op->kind == dOP_ELASTICITY)
    DCHK(elasticity_apply_t<float>(fs, x, op->d_geo32, (float)op->lam, (float)op->mu, op->d_y32));
  else
    DCHK(diffusion_apply_t<float>(fs, x, op->d_geo32, op->d_y32));
  return fs_restrict32(fs, op->d_y32, y, 0);
}

__global__ void k_to_bf16_geo(int64_t n, const double *__restrict__ a, __nv_bfloat16 *__restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16_rn((float)a[i]);
}

// BF16 storage (factors, inputs, basis tables), FP32 arithmetic; FP64 restriction
static dErr op_mult_bf16(_p_dOperator *op, const double *x, double *y) {
  _p_dFS *fs = op->fs;
  if (op->kind != dOP_DIFFUSION && op->kind != dOP_PLAPLACE_JACOBIAN)
    return set_error("BF16 apply for operator kind %d not built (scalar kinds only)", (int)op->kind);
  DCHK(op_compute_geometry(op));
  const int64_t ng = fs->nq * 6;
  if (!op->d_geo16) {
    CUCHK(cudaMalloc(&op->d_geo16, ng * sizeof(__nv_bfloat16)));
    k_to_bf16_geo<<<(unsigned)((ng + 255) / 256), 256, 0, fs->stream>>>(ng, op->d_geo, (__nv_bfloat16 *)op->d_geo16);
    CUCHK(cudaGetLastError());
  }
  if (!op->d_y32) CUCHK(cudaMalloc(&op->d_y32, fs->nexp * fs->bs * sizeof(float)));
  if (fs->bs == 1 && fs->boolean_e && fs->p >= 1 && fs->p <= 7) {
    // the contractions on the tensor cores (tc_apply.cu); the first apply of an operator is checked synchronously
    DCHK(tc_diffusion_apply(fs, x, op->d_geo16, &op->d_tcb, op->d_y32, y));
    if (!op->tc_checked) {
      DCHK(tc_check(fs));
      op->tc_checked = true;
    }
    return 0;
  }
  const __nv_bfloat16 *g = (const __nv_bfloat16 *)op->d_geo16;
  dErr e = 0;
  switch (fs->p + 1) {
    case 2: e = launch_diffusion_bf16<2>(fs, x, g, op->d_y32); break;
    case 3: e = launch_diffusion_bf16<3>(fs, x, g, op->d_y32); break;
    case 4: e = launch_diffusion_bf16<4>(fs, x, g, op->d_y32); break;
    case 5: e = launch_diffusion_bf16<5>(fs, x, g, op->d_y32); break;
    case 6: e = launch_diffusion_bf16<6>(fs, x, g, op->d_y32); break;
    case 7: e = launch_diffusion_bf16<7>(fs, x, g, op->d_y32); break;
    case 8: e = launch_diffusion_bf16<8>(fs, x, g, op->d_y32); break;
    case 9: e = launch_diffusion_bf16<9>(fs, x, g, op->d_y32); break;
    default: return set_error("degree %d not supported", fs->p);
  }
  if (e) return e;
  return fs_restrict32(fs, op->d_y32, y, 0);
}

__global__ void k_to_ff(int64_t n, const double *__restrict__ a, ff *__restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = ff(a[i]);
}

dErr fs_restrict_ff(_p_dFS *fs, const ff *x, double *g, int add);

// float-float element arithmetic (geometric factors split into float pairs once), FP64 input and restriction
static dErr op_mult_ff(_p_dOperator *op, const double *x, double *y) {
  _p_dFS *fs = op->fs;
  if (op->kind != dOP_DIFFUSION && op->kind != dOP_ELASTICITY && op->kind != dOP_PLAPLACE_JACOBIAN)
    return set_error("float-float apply for operator kind %d not built", (int)op->kind);
  if (op->svk_state) return set_error("float-float St. Venant-Kirchhoff Jacobian not built (use FP64)");
  DCHK(op_compute_geometry(op));
  const int64_t ng = fs->nq * (op->kind == dOP_ELASTICITY ? 10 : 6);
  if (!op->d_geoff) {
    CUCHK(cudaMalloc(&op->d_geoff, ng * sizeof(ff)));
    k_to_ff<<<(unsigned)((ng + 255) / 256), 256, 0, fs->stream>>>(ng, op->d_geo, (ff *)op->d_geoff);
    CUCHK(cudaGetLastError());
  }
  if (!op->d_yff) CUCHK(cudaMalloc(&op->d_yff, fs->nexp * fs->bs * sizeof(ff)));
  const ff *geo = (const ff *)op->d_geoff;
  ff *yexp = (ff *)op->d_yff;
  if (op->kind == dOP_ELASTICITY)
    DCHK(elasticity_apply_t<ff>(fs, x, geo, ff(op->lam), ff(op->mu), yexp));
  else
    DCHK(diffusion_apply_t<ff>(fs, x, geo, yexp));
  return fs_restrict_ff(fs, yexp, y, 0);
}

dErr hp_mult(_p_dOperator *op, const double *x, double *y);

dErr op_mult(_p_dOperator *op, const double *x, double *y) {
  _p_dFS *fs = op->fs;
  if (op->prec == dPREC_BF16 && (!fs->uniform || op->launch != dLAUNCH_DEFAULT))
    return set_error("BF16 apply needs a uniform-order space and the default launch");
  if (op->svk_state && (!fs->uniform || op->launch != dLAUNCH_DEFAULT))
    return set_error("St. Venant-Kirchhoff Jacobian needs a uniform-order space and the default launch");
  if (!fs->uniform || op->launch != dLAUNCH_DEFAULT) return hp_mult(op, x, y);
  if (op->prec == dPREC_FP32) return op_mult_fp32(op, x, y);
  if (op->prec == dPREC_FF) return op_mult_ff(op, x, y);
  if (op->prec == dPREC_BF16) return op_mult_bf16(op, x, y);
  if (!op->d_yexp) CUCHK(cudaMalloc(&op->d_yexp, fs->nexp * fs->bs * sizeof(double)));
  DCHK(op_mult_expanded(op, x, op->d_yexp));
  return fs_restrict(fs, op->d_yexp, y, 0);
}

// apply in a given precision regardless of the operator's default (used by the mixed-precision solvers)
dErr op_mult_prec(_p_dOperator *op, const double *x, double *y, dPrecision prec) {
  const dPrecision save = op->prec;
  op->prec = prec;
  const dErr e = op_mult(op, x, y);
  op->prec = save;
  return e;
}

// St. Venant-Kirchhoff state at g (ElastPointwiseComputeStore, elast.c:224-225) and, with y, the function
// (ElastFunction without body force, elast.c:282-309); g = NULL returns to F = I
static dErr svk_state(_p_dOperator *op, const double *g, double *y) {
  _p_dFS *fs = op->fs;
  if (op->kind != dOP_ELASTICITY) return set_error("St. Venant-Kirchhoff needs an elasticity operator");
  if (!g) {
    op->svk_state = false;
    return 0;
  }
  if (!fs->uniform) return set_error("St. Venant-Kirchhoff needs a uniform-order space");
  DCHK(op_compute_geometry(op));
  if (!op->d_svk) CUCHK(cudaMalloc(&op->d_svk, (size_t)fs->nq * 15 * sizeof(double)));
  if (!op->d_yexp) CUCHK(cudaMalloc(&op->d_yexp, fs->nexp * fs->bs * sizeof(double)));
  // the state is expanded dFS_INHOMOGENEOUS, as ElastFunction starts its iterator (elast.c:293): Dirichlet nodes take
  // the values committed with dFSInhomogeneousDirichletCommit (zero when none were)
  DCHK(svk_launch<K_SVK_FUNC>(fs, g, op->d_geo, op->lam, op->mu, op->d_yexp, op->d_svk, fs->nc > fs->n ? fs->d_dcache : nullptr));
  op->svk_state = true;
  if (y) DCHK(fs_restrict(fs, op->d_yexp, y, 0));
  return 0;
}

extern "C" dErr dOperatorElasticityState(dOperator op, const dScalar *g) {
  if (!op) return set_error("null operator");
  return svk_state(op, g, nullptr);
}

extern "C" dErr dOperatorElasticityFunction(dOperator op, const dScalar *g, dScalar *y) {
  if (!op || !g || !y) return set_error("null argument");
  return svk_state(op, g, y);
}

extern "C" dErr dOperatorMultExpanded(dOperator op, const dScalar *x, dScalar *yexp) {
  if (!op) return set_error("null operator");
  return op_mult_expanded(op, x, yexp);
}

// ----------------------------------------------------------------------------------------------------------
// Operator apply that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc or cudaFree while they run: applications that hand
// all device memory to their own pool or arena at start-up and account for every byte, and solver
// callbacks (a PETSc MatShell multiply inside a Krylov iteration) that run next to work on other
// streams, where a cudaMalloc or cudaFree may synchronize the whole device. dOperatorMultNoAlloc serves
// them. Its one temporary, the expanded element output (nexp*bs doubles), lives in the fixed-size
// file-scope device array below, which every GPU that loads this library holds until the process exits.
// In host code the array's name is only a host-side stand-in; its device address is looked up once per
// device with cudaGetSymbolAddress (with that device current) and passed to the kernels.
// Every call shares the array and overwrites all of the part it uses before reading it, so nothing has
// to be cleared between calls; calls that overlap on the GPU (different streams, or several host
// threads) race on it.
static constexpr int64_t kNoAllocScratchDoubles = 1 << 20;  // 8 MiB per device
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];
static std::mutex g_noalloc_mutex;
static double *g_noalloc_addr[128];  // device address of g_noalloc_scratch per device ordinal

static dErr noalloc_scratch(double **out) {
  int dev = -1;
  CUCHK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return set_error("dOperatorMultNoAlloc: device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    CUCHK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[dev] = (double *)p;
  }
  *out = g_noalloc_addr[dev];
  return 0;
}

extern "C" dErr dOperatorMultNoAlloc(dOperator op, const dScalar *x, dScalar *y) {
  if (!op) return set_error("null operator");
  _p_dFS *fs = op->fs;
  if (op->kind != dOP_DIFFUSION) return set_error("dOperatorMultNoAlloc: operator kind %d not supported", (int)op->kind);
  if (!fs->uniform) return set_error("dOperatorMultNoAlloc: uniform-order spaces only (this space has per-element orders)");
  if (op->prec != dPREC_FP64)
    return set_error("dOperatorMultNoAlloc: applies in FP64 only; the operator's precision is set to %d (dOperatorSetPrecision "
                     "dPREC_FP64 first, or use dOperatorMult)", (int)op->prec);
  if (!op->geo_valid || op->geo_kind != 0)
    return set_error("dOperatorMultNoAlloc: the operator's geometric factors do not exist yet; make one dOperatorMult "
                     "call at set-up time (where allocation is allowed) after the last dOperatorSetQuadratureData");
  const int64_t need = fs->nexp * fs->bs;
  if (need > kNoAllocScratchDoubles)
    return set_error("dOperatorMultNoAlloc: the space has %lld expanded values, more than the fixed scratch of %lld "
                     "doubles (8 MiB); use dOperatorMult for this space",
                     (long long)need, (long long)kNoAllocScratchDoubles);
  double *scratch = nullptr;
  DCHK(noalloc_scratch(&scratch));
  DCHK(diffusion_apply_t<double>(fs, x, op->d_geo, scratch));
  return fs_restrict(fs, scratch, y, 0);
}
