// p-Laplacian on the device: EllipPointwiseComputeStore, EllipPointwiseFunction and EllipPointwiseJacobian
// (src/fs/tests/ellip.c:333-377) for the operator path of EllipFunction / EllipShellMatMult / EllipJacobian
// (ellip.c:407-536), with lambda = 0 and the forcing left to the caller.
//
//   eta = (eps^2 + |Du|^2/2)^((p-2)/2),   s = sqrt(-eta') Du,   eta' = ((p-2)/2) eta / (eps^2 + |Du|^2/2)
//   function: Dv = w eta Du
//   Jacobian: Dv = w (eta I - s s^T) D(du)
//
// One kernel evaluates the state's gradient at the FAST points, forms the store, and writes the Jacobian's
// coefficient in reference coordinates, G = w J^-1 (eta I - s s^T) J^-T (6 per point, the layout of the
// diffusion kernel's factors), so that every Jacobian apply is the fused diffusion kernel with G (FP64 or
// FP32). With RES it also completes the function apply (transposed passes) into the expanded output.
// The Q1-embedded Jacobian (EllipJacobian on the SPARSE ruleset) takes the state's reference gradient at
// every SPARSE point from one batched dEFSApply GRAD and forms the store inside the Q1 patch kernel.
#include "internal.h"

using namespace dgb;

dErr fs_expand(_p_dFS *fs, const double *g, double *x, bool inhomogeneous, int add);
dErr fs_restrict(_p_dFS *fs, const double *x, double *g, int add);
dErr geometry_fill(_p_dFS *fs, int mode, const double *kq, double *out);
dErr q1_numeric(_p_dFS *fs, _p_dMat *J, const double *grf_host, int quirk, const double *dref, double pe, double eps, bool single);
dPrecision ksp_pc_precision(dKSP ksp);
dErr device_dot(int64_t n, const double *a, const double *b, double *part, double *out, cudaStream_t s);
dErr dot_part_alloc(double **part);
dErr ksp_solve(dKSP ksp, const double *b, double *x, double rtol, int maxit, int *its, double *rnorm);

namespace {

template <int N>
struct PTile {
  static constexpr int EPB = N <= 2 ? 32 : N == 3 ? 16 : N == 4 ? 8 : N == 5 ? 4 : N <= 7 ? 2 : 1;
};

// xexp: expanded state (Dirichlet values included); gbase: {J^-1, w det J} SoA per element;
// out: stash [nq][4] (may be NULL), G [6] SoA per element, and with RES the expanded function output
template <int N, bool RES>
__global__ void __launch_bounds__(256) k_plap_point(int64_t nelem, const double *__restrict__ xexp, const double *__restrict__ gbase,
                                                    const double *__restrict__ tab, double pe, double eps, double *__restrict__ stash,
                                                    double *__restrict__ G, double *__restrict__ yexp) {
  constexpr int N3 = N * N * N, NN = N * N, EPB = PTile<N>::EPB;
  __shared__ double sB[NN], sD[NN];
  __shared__ double S[4][EPB * N3];
  const int tid = threadIdx.x;
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  const int ne = (int)min((int64_t)EPB, nelem - e0);
  const int tot = ne * N3;
  for (int i = tid; i < NN; i += blockDim.x) {
    sB[i] = tab[i];
    sD[i] = tab[MAXP * MAXP + i];
  }
  for (int t = tid; t < tot; t += blockDim.x) S[0][t] = xexp[e0 * N3 + t];
  __syncthreads();
  for (int t = tid; t < tot; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, a = r / NN, jk = r - a * NN;
    const double *in = &S[0][el * N3 + jk];
    double s = 0;
#pragma unroll
    for (int i = 0; i < N; i++) s += sB[a * N + i] * in[i * NN];
    S[1][t] = s;
  }
  __syncthreads();
  for (int t = tid; t < tot; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, a = r / NN, b = (r / N) % N, k = r % N;
    const double *in = &S[1][el * N3 + a * NN + k];
    double s = 0;
#pragma unroll
    for (int j = 0; j < N; j++) s += sB[b * N + j] * in[j * N];
    S[0][t] = s;
  }
  __syncthreads();
  for (int t = tid; t < tot; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, ab = r / N, c = r % N;
    const double *in = &S[0][el * N3 + ab * N];
    double s = 0;
#pragma unroll
    for (int k = 0; k < N; k++) s += sB[c * N + k] * in[k];
    S[1][t] = s;
  }
  __syncthreads();
  for (int t = tid; t < tot; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, a = r / NN, b = (r / N) % N, c = r % N;
    const double *U = &S[1][el * N3];
    double g0 = 0, g1 = 0, g2 = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
      g0 += sD[a * N + i] * U[i * NN + b * N + c];
      g1 += sD[b * N + i] * U[a * NN + i * N + c];
      g2 += sD[c * N + i] * U[a * NN + b * N + i];
    }
    const int64_t e = e0 + el;
    const double *gb = gbase + e * 10 * N3 + r;
    double Ji[9];
#pragma unroll
    for (int i = 0; i < 9; i++) Ji[i] = gb[i * N3];
    const double w = gb[9 * N3];
    double Du[3];
#pragma unroll
    for (int k = 0; k < 3; k++) Du[k] = g0 * Ji[0 * 3 + k] + g1 * Ji[1 * 3 + k] + g2 * Ji[2 * 3 + k];
    const double gamma = 0.5 * (Du[0] * Du[0] + Du[1] * Du[1] + Du[2] * Du[2]);
    const double espg = eps * eps + gamma, eta = pow(espg, (pe - 2) / 2);
    const double sm = sqrt(-((pe - 2) / 2) * eta / espg);
    const double s0 = sm * Du[0], s1 = sm * Du[1], s2 = sm * Du[2];
    if (stash) {
      double *st = stash + (e * N3 + r) * 4;
      st[0] = eta, st[1] = s0, st[2] = s1, st[3] = s2;
    }
    // G = w (eta H - t t^T), H = J^-1 J^-T, t = J^-1 s
    double tt[3];
#pragma unroll
    for (int a2 = 0; a2 < 3; a2++) tt[a2] = Ji[a2 * 3 + 0] * s0 + Ji[a2 * 3 + 1] * s1 + Ji[a2 * 3 + 2] * s2;
    double *Gq = G + e * 6 * N3 + r;
    int o = 0;
#pragma unroll
    for (int a2 = 0; a2 < 3; a2++)
#pragma unroll
      for (int b2 = a2; b2 < 3; b2++) {
        const double h = Ji[a2 * 3 + 0] * Ji[b2 * 3 + 0] + Ji[a2 * 3 + 1] * Ji[b2 * 3 + 1] + Ji[a2 * 3 + 2] * Ji[b2 * 3 + 2];
        Gq[(o++) * N3] = w * (eta * h - tt[a2] * tt[b2]);
      }
    if (RES) {  // Dv = w eta Du, mapped back to reference directions
      const double etaw = eta * w;
      const double v0 = etaw * Du[0], v1 = etaw * Du[1], v2 = etaw * Du[2];
      S[0][t] = Ji[0] * v0 + Ji[1] * v1 + Ji[2] * v2;
      S[2][t] = Ji[3] * v0 + Ji[4] * v1 + Ji[5] * v2;
      S[3][t] = Ji[6] * v0 + Ji[7] * v1 + Ji[8] * v2;
    }
  }
  if (!RES) return;
  __syncthreads();
  for (int t = tid; t < tot; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, a = r / NN, b = (r / N) % N, c = r % N;
    const double *V0 = &S[0][el * N3], *V1 = &S[2][el * N3], *V2 = &S[3][el * N3];
    double s = 0;
#pragma unroll
    for (int i = 0; i < N; i++)
      s += sD[i * N + a] * V0[i * NN + b * N + c] + sD[i * N + b] * V1[a * NN + i * N + c] + sD[i * N + c] * V2[a * NN + b * N + i];
    S[1][t] = s;
  }
  __syncthreads();
  for (int t = tid; t < tot; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, ab = r / N, k = r % N;
    const double *in = &S[1][el * N3 + ab * N];
    double s = 0;
#pragma unroll
    for (int c = 0; c < N; c++) s += sB[c * N + k] * in[c];
    S[0][t] = s;
  }
  __syncthreads();
  for (int t = tid; t < tot; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, a = r / NN, j = (r / N) % N, k = r % N;
    const double *in = &S[0][el * N3 + a * NN + k];
    double s = 0;
#pragma unroll
    for (int b = 0; b < N; b++) s += sB[b * N + j] * in[b * N];
    S[1][t] = s;
  }
  __syncthreads();
  for (int t = tid; t < tot; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, i = r / NN, jk = r - i * NN;
    const double *in = &S[1][el * N3 + jk];
    double s = 0;
#pragma unroll
    for (int a = 0; a < N; a++) s += sB[a * N + i] * in[a * NN];
    yexp[e0 * N3 + t] = s;
  }
}

// G from a caller-supplied stash [nq][4] (dOperatorSetQuadratureData)
__global__ void k_plap_from_stash(int64_t nelem, int N3, const double *__restrict__ gbase, const double *__restrict__ stash,
                                  double *__restrict__ G) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nelem * N3) return;
  const int64_t e = t / N3;
  const int r = (int)(t - e * N3);
  const double *gb = gbase + e * 10 * N3 + r;
  double Ji[9];
  for (int i = 0; i < 9; i++) Ji[i] = gb[i * N3];
  const double w = gb[9 * N3];
  const double *st = stash + t * 4;
  double tt[3];
  for (int a = 0; a < 3; a++) tt[a] = Ji[a * 3 + 0] * st[1] + Ji[a * 3 + 1] * st[2] + Ji[a * 3 + 2] * st[3];
  double *Gq = G + e * 6 * N3 + r;
  int o = 0;
  for (int a = 0; a < 3; a++)
    for (int b = a; b < 3; b++) {
      const double h = Ji[a * 3 + 0] * Ji[b * 3 + 0] + Ji[a * 3 + 1] * Ji[b * 3 + 1] + Ji[a * 3 + 2] * Ji[b * 3 + 2];
      Gq[(o++) * N3] = w * (st[0] * h - tt[a] * tt[b]);
    }
}

// z = a x + b y
__global__ void k_waxpby(int64_t n, double a, const double *__restrict__ x, double b, const double *__restrict__ y,
                         double *__restrict__ z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) z[i] = a * x[i] + b * y[i];
}

dErr plap_prepare(_p_dOperator *op) {
  _p_dFS *fs = op->fs;
  if (op->kind != dOP_PLAPLACE_JACOBIAN) return set_error("operator is not a p-Laplacian Jacobian");
  if (fs->bs != 1) return set_error("p-Laplacian needs a scalar space");
  if (!fs->uniform) return set_error("p-Laplacian needs a uniform-order space");
  if (!op->d_gbase) {
    CUCHK(cudaMalloc(&op->d_gbase, (size_t)fs->nq * 10 * sizeof(double)));
    dErr e = geometry_fill(fs, 1, nullptr, op->d_gbase);
    if (e) {
      cudaFree(op->d_gbase);
      op->d_gbase = nullptr;
      return e;
    }
  }
  if (!op->d_geo || op->geo_kind != 2) {
    cudaFree(op->d_geo);
    op->d_geo = nullptr;
    CUCHK(cudaMalloc(&op->d_geo, (size_t)fs->nq * 6 * sizeof(double)));
    op->geo_valid = false;
    op->geo_kind = 2;
  }
  if (!op->d_stash) CUCHK(cudaMalloc(&op->d_stash, (size_t)fs->nq * 4 * sizeof(double)));
  if (op->d_geo32) {  // the FP32 copy of the factors is rebuilt on the next FP32 apply
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
  return 0;
}

template <int N>
dErr launch_point(_p_dOperator *op, const double *xexp, double pe, double eps, double *yexp) {
  constexpr int EPB = PTile<N>::EPB;
  _p_dFS *fs = op->fs;
  const unsigned grid = (unsigned)((fs->nelem + EPB - 1) / EPB);
  const double *tab = fs->d_fast_tab + (size_t)2 * (N - 2) * MAXP * MAXP;
  if (yexp)
    k_plap_point<N, true><<<grid, 256, 0, fs->stream>>>(fs->nelem, xexp, op->d_gbase, tab, pe, eps, op->d_stash, op->d_geo, yexp);
  else
    k_plap_point<N, false><<<grid, 256, 0, fs->stream>>>(fs->nelem, xexp, op->d_gbase, tab, pe, eps, op->d_stash, op->d_geo, nullptr);
  CUCHK(cudaGetLastError());
  return 0;
}

// store at the FAST points of the state g (dFS_INHOMOGENEOUS, as EllipFunction starts its iterator);
// with yexp also the function's element output
dErr plap_point(_p_dOperator *op, const double *g, double pe, double eps, double *yexp) {
  DCHK(plap_prepare(op));
  _p_dFS *fs = op->fs;
  // the store takes sqrt(-eta') (ellip.c:339), real only for 1 < p <= 2
  if (!(pe > 1 && pe <= 2)) return set_error("p-Laplacian exponent %g outside (1, 2]", pe);
  DCHK(fs_expand(fs, g, fs->d_scratch_exp, true, 0));
  dErr e = 0;
  switch (fs->p + 1) {
    case 2: e = launch_point<2>(op, fs->d_scratch_exp, pe, eps, yexp); break;
    case 3: e = launch_point<3>(op, fs->d_scratch_exp, pe, eps, yexp); break;
    case 4: e = launch_point<4>(op, fs->d_scratch_exp, pe, eps, yexp); break;
    case 5: e = launch_point<5>(op, fs->d_scratch_exp, pe, eps, yexp); break;
    case 6: e = launch_point<6>(op, fs->d_scratch_exp, pe, eps, yexp); break;
    case 7: e = launch_point<7>(op, fs->d_scratch_exp, pe, eps, yexp); break;
    case 8: e = launch_point<8>(op, fs->d_scratch_exp, pe, eps, yexp); break;
    case 9: e = launch_point<9>(op, fs->d_scratch_exp, pe, eps, yexp); break;
    default: return set_error("degree %d not supported", fs->p);
  }
  if (e) return e;
  op->param[0] = pe;
  op->param[1] = eps;
  op->geo_valid = true;
  return 0;
}

}  // namespace

dErr plap_set_stash(_p_dOperator *op, const double *stash) {
  if (!stash) return set_error("p-Laplacian Jacobian needs its stash");
  DCHK(plap_prepare(op));
  _p_dFS *fs = op->fs;
  CUCHK(cudaMemcpyAsync(op->d_stash, stash, fs->nq * 4 * sizeof(double), cudaMemcpyDeviceToDevice, fs->stream));
  const int N = fs->p + 1, N3 = N * N * N;
  k_plap_from_stash<<<(unsigned)((fs->nq + 255) / 256), 256, 0, fs->stream>>>(fs->nelem, N3, op->d_gbase, op->d_stash, op->d_geo);
  CUCHK(cudaGetLastError());
  op->geo_valid = true;
  return 0;
}

extern "C" {

dErr dOperatorComputePLaplaceStash(dOperator op, const dScalar *g, dReal p, dReal eps) {
  if (!op || !g) return set_error("null argument");
  return plap_point(op, g, p, eps, nullptr);
}

dErr dOperatorPLaplaceFunction(dOperator op, const dScalar *g, dReal p, dReal eps, dScalar *y) {
  if (!op || !g || !y) return set_error("null argument");
  _p_dFS *fs = op->fs;
  if (!op->d_yexp) CUCHK(cudaMalloc(&op->d_yexp, fs->nexp * fs->bs * sizeof(double)));
  DCHK(plap_point(op, g, p, eps, op->d_yexp));
  return fs_restrict(fs, op->d_yexp, y, 0);
}

dErr dOperatorGetQuadratureData(dOperator op, dReal *qdata) {
  if (!op || !qdata) return set_error("null argument");
  _p_dFS *fs = op->fs;
  if (op->kind == dOP_PLAPLACE_JACOBIAN) {
    if (!op->geo_valid || !op->d_stash) return set_error("p-Laplacian stash not computed yet");
    CUCHK(cudaMemcpyAsync(qdata, op->d_stash, fs->nq * 4 * sizeof(double), cudaMemcpyDeviceToDevice, fs->stream));
    return 0;
  }
  if (op->kind == dOP_DIFFUSION) {
    if (!op->d_k) return set_error("no coefficient set (k = 1)");
    CUCHK(cudaMemcpyAsync(qdata, op->d_k, fs->nq * sizeof(double), cudaMemcpyDeviceToDevice, fs->stream));
    return 0;
  }
  return set_error("operator kind %d has no quadrature data", (int)op->kind);
}

// the Q1-embedded p-Laplacian Jacobian at g; single: the patch matrices in FP32 arithmetic (the preconditioner of a
// solve whose preconditioning runs in FP32 or BF16), else FP64
static dErr assemble_q1_plap(dFS fs, dMat J, const dScalar *g, dReal p, dReal eps, int reference_quirk, bool single) {
  if (!fs || !J || !g) return set_error("null argument");
  if (fs->bs != 1 || !fs->uniform) return set_error("p-Laplacian Q1 assembly needs a scalar uniform-order space");
  if (!fs->jac) return set_error("dFS was created without a dJacobi");
  if (!(p > 1 && p <= 2)) return set_error("p-Laplacian exponent %g outside (1, 2]", p);
  const dInt deg[3] = {fs->p, fs->p, fs->p}, ro[3] = {2 * fs->p, 2 * fs->p, 2 * fs->p};
  dEFS sefs;
  DCHK(jacobi_efs(fs->jac, deg, dQUADRATURE_METHOD_SPARSE, ro, &sefs));
  const int64_t npts = fs->nelem * (int64_t)sefs->Q[0] * sefs->Q[1] * sefs->Q[2];
  double *dref;
  CUCHK(cudaMalloc(&dref, npts * 3 * sizeof(double)));
  dErr e = fs_expand(fs, g, fs->d_scratch_exp, true, 0);
  if (!e) e = dEFSApplyBatched(sefs, (dInt)fs->nelem, nullptr, 1, fs->d_scratch_exp, dref, dAPPLY_GRAD, INSERT_VALUES, fs->stream);
  if (!e) e = q1_numeric(fs, J, nullptr, reference_quirk, dref, p, eps, single);
  cudaFree(dref);
  return e;
}

dErr dFSAssembleQ1PLaplace(dFS fs, dMat J, const dScalar *g, dReal p, dReal eps, int reference_quirk) {
  Range range_("dQ1HexComputQuad (p-Laplacian)");
  return assemble_q1_plap(fs, J, g, p, eps, reference_quirk, false);
}

// Newton's method for N(u) = b (the SNES side of ellip.c: SNESSetFunction(EllipFunction),
// SNESSetJacobian(EllipJacobian), ellip.c:697-704) with a backtracking line search on ||F||:
// every step assembles the Q1 Jacobian at u, solves J du = -F with the caller's KSP (whose operator is op,
// the matrix-free Jacobian at u), and accepts u + lambda du once ||F|| drops by the Armijo factor.
dErr dPLaplaceNewtonSolve(dOperator op, dMat Jp, dKSP ksp, const dScalar *b, dScalar *u, dReal p, dReal eps,
                          const dNewtonOptions *opt, dInt *its, dReal *fnorm, dInt *lin_its) {
  Range range_("SNESSolve (p-Laplacian Newton)");
  if (!op || !Jp || !ksp || !b || !u || !opt) return set_error("null argument");
  _p_dFS *fs = op->fs;
  cudaStream_t s = fs->stream;
  const int64_t n = fs->n * fs->bs;
  const unsigned grid = (unsigned)((n + 255) / 256);
  DCHK(dKSPSetOperators(ksp, op, Jp));
  double *F, *du, *ut, *Ft, *part, *d_s;
  CUCHK(cudaMalloc(&F, 4 * std::max<int64_t>(n, 1) * sizeof(double)));
  du = F + n, ut = du + n, Ft = ut + n;
  DCHK(dot_part_alloc(&part));
  CUCHK(cudaMalloc(&d_s, sizeof(double)));
  auto residual = [&](const double *x, double *r, double *nrm) -> dErr {
    DCHK(dOperatorPLaplaceFunction(op, x, p, eps, r));
    k_waxpby<<<grid, 256, 0, s>>>(n, 1.0, r, -1.0, b, r);
    CUCHK(cudaGetLastError());
    DCHK(device_dot(n, r, r, part, d_s, s));
    double h;
    CUCHK(cudaMemcpyAsync(&h, d_s, sizeof h, cudaMemcpyDeviceToHost, s));
    CUCHK(cudaStreamSynchronize(s));
    *nrm = sqrt(h);
    return 0;
  };
  dErr err = 0;
  double fn = 0, fn0 = 0;
  int k = 0;
  err = residual(u, F, &fn);
  fn0 = fn;
  if (fnorm && !err) fnorm[0] = fn;
  for (; !err && k < opt->max_it && fn > opt->rtol * fn0 && fn > opt->atol; k++) {
    // the preconditioning matrix in the precision its preconditioner runs in (FP32 arithmetic for FP32 / BF16)
    err = assemble_q1_plap(fs, Jp, u, p, eps, opt->reference_quirk, ksp_pc_precision(ksp) != dPREC_FP64);
    if (!err) err = dKSPSetOperators(ksp, nullptr, Jp);
    if (err) break;
    k_waxpby<<<grid, 256, 0, s>>>(n, -1.0, F, 0.0, F, Ft);  // rhs = -F (Ft as scratch)
    CUCHK(cudaMemsetAsync(du, 0, n * sizeof(double), s));
    int li = 0;
    double rn = 0;
    // the stash of u is current: the last residual evaluation was at u. A solve that stops at lin_maxit
    // with some reduction still gives an (inexact) Newton direction.
    err = ksp_solve(ksp, Ft, du, opt->lin_rtol, opt->lin_maxit, &li, &rn);
    if (err) break;
    if (!(rn < 1)) {
      err = set_error("Newton step %d: linear solve made no progress (relative residual %g)", k, rn);
      break;
    }
    if (lin_its) lin_its[k] = li;
    double lam = 1, fnt = 0;
    int ls = 0;
    for (; ls < 12; ls++, lam *= 0.5) {
      k_waxpby<<<grid, 256, 0, s>>>(n, 1.0, u, lam, du, ut);
      err = residual(ut, Ft, &fnt);
      if (err || fnt < (1 - 1e-4 * lam) * fn) break;
    }
    if (err) break;
    if (ls == 12) {
      err = set_error("Newton line search failed at step %d (||F|| %g)", k, fn);
      break;
    }
    CUCHK(cudaMemcpyAsync(u, ut, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CUCHK(cudaMemcpyAsync(F, Ft, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    fn = fnt;
    if (fnorm) fnorm[k + 1] = fn;
  }
  CUCHK(cudaStreamSynchronize(s));
  cudaFree(F);
  cudaFree(part);
  cudaFree(d_s);
  if (its) *its = k;
  return err;
}

}  // extern "C"
