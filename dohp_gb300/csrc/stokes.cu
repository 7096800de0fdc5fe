// Mixed velocity-pressure (Stokes) operator and its block-preconditioned solve (src/fs/tests/stokes.c).
//
// Spaces: velocity u in the dFS fsu (bs 3, degree k, Dirichlet sets), pressure p in fsp (bs 1, degree k - codim,
// continuous, no boundary sets: StokesSetFromOptions, stokes.c:160-274) on the same mesh; every integral uses the
// velocity's FAST rule (k+1 Gauss points per direction), the pressure basis is evaluated at those points.
// Operator (MatMult_Nest_StokesCoupled stokes.c:541-577, StokesShellMatMult_All_IorA stokes.c:579-673):
//   A:  int eta Dv:Du + lambda div v div u, lambda = nu/(1 - 2 nu)  (StokesPointwiseJacobian_A, stokes.c:489-494)
//   Bt: -int p div v                                                 (StokesPointwiseJacobian_Bt, stokes.c:501-505)
//   B:  -int q div u                                                 (StokesPointwiseJacobian_B, stokes.c:496-499)
//   coupled [A Bt; B 0] without the penalty                          (StokesPointwiseJacobian, stokes.c:476-487)
// with Du the symmetric gradient in [00, 11, 22, 01, 02, 12] storage (dTensorSymCompress3, include/dohp.h:79-82).
// Rheology (StokesPointwiseComputeStore, stokes.c:447-453): eta = B (eps^2/2 + Du:Du/2)^((p-2)/2). The Newtonian
// case p = 2 is linear (eta = B). For p != 2, dStokesFunction evaluates the nonlinear function
// [eta(Du) Du - p I; -div u] (StokesPointwiseFunction stokes.c:460-474, the forcing moved into the caller's
// right-hand side) and keeps the store {eta, eta', Du} of its state at every point; the A and coupled applies are
// then the Jacobian at that state (StokesPointwiseJacobian(_A), stokes.c:476-494), eta Dv:Du + eta' (Dw:Du)(Dw:Dv).
// Before any function evaluation the state is zero (eta = B (eps^2/2)^((p-2)/2), no eta' term).
//
// One fused kernel per element group does all of it: velocity gather through E, B and Dq passes per component,
// pressure gather and three rectangular passes Bp (N x NP: the pressure's GLL basis at the velocity's Gauss
// points), the pointwise coupling with the geometric factors {J^-1, w det J}, the transposed passes, and the
// expanded outputs; the E^T restrictions of the two spaces follow.
//
// Solver (the reference's -pc_fieldsplit_type schur with a Q1-embedded velocity matrix and a viscosity-scaled
// pressure mass for the Schur complement, StokesGetMatrices / StokesJacobianAssemble_Velocity / _Pressure,
// stokes.c:367-505, 675-799): right-preconditioned FGMRES on the packed vector [u; p] with the block upper
// triangular preconditioner
//   z_p = -eta diag(M_p)^-1 r_p  (mean removed: the constant pressure is the null space with Dirichlet walls),
//   z_u = M_u (r_u - Bt z_p),
// A_q1 the blocked Q1-embedded matrix of the A block (the elasticity assembly with 2 mu = eta, lambda as A) and
// M_u one Q1 multigrid V-cycle on it (Chebyshev-Jacobi alone where the GLL lattice does not coarsen).
#include <algorithm>
#include <cmath>
#include <vector>

#include "element.cuh"

using namespace dgb;

dErr fs_restrict(_p_dFS *fs, const double *x, double *g, int add);
dErr fs_restrict_rows(_p_dFS *fs, const double *x, double *g, int64_t t0, int64_t t1, cudaStream_t s);
dErr geometry_fill(_p_dFS *fs, int mode, const double *kq, double *out);
dErr q1_numeric_elast(_p_dFS *fs, _p_dMat *J, double lam, double mu, int quirk);
dErr ksp_create_shell(int64_t n, cudaStream_t stream, dKSPType type, dErr (*mult)(void *, const double *, double *),
                      dErr (*pc)(void *, const double *, double *), void *ctx, int restart, dKSP *ksp);
dErr ksp_solve(dKSP ksp, const double *b, double *x, double rtol, int maxit, int *its, double *rnorm);
dErr ksp_pc_only(dKSP ksp, const double *r, double *z);
dErr device_dot(int64_t n, const double *a, const double *b, double *part, double *out, cudaStream_t s);
dErr dot_part_alloc(double **part);

namespace {

struct StokesArgs {
  ElemArgs U, P;     // velocity and pressure spaces (xstart, emap, n, x, yexp)
  const double *bp;  // Bp [N][NP]
  const double *geo; // velocity FAST geometry {J^-1 (9), w det J} per point, SoA per element
  double *store;     // {eta, eta', Du[6]} per velocity point, SoA per element; null: no state (eta constant)
  const double *udir;  // function mode: Dirichlet values of the velocity closure [(nc - n) * 3] (dFS_INHOMOGENEOUS)
  const double *fpq;   // pressure-integral mode: the integrand at the velocity's points
  double eta, lam;   // eta without a state
  double B, heps2, hexp;  // rheology: B, eps^2 / 2, (p - 2) / 2
};

constexpr int SM_A = 0, SM_BT = 1, SM_B = 2, SM_COUPLED = 3, SM_FUNCTION = 4, SM_PINT = 5;

// the velocity gather of the function: closure nodes beyond the explicit ones take the committed Dirichlet values
// (a uniform space: Boolean E through emap)
template <int N>
__device__ __forceinline__ void gather_inhomogeneous(const ElemArgs &A, const double *dir, int64_t first, int ne, int d, double *dst) {
  constexpr int N3 = N * N * N;
  for (int t = threadIdx.x; t < ne * N3; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3;
    const int32_t c = A.emap[A.xstart[first + el] + r];
    dst[t] = c < A.n ? A.x[(int64_t)c * 3 + d] : dir[(int64_t)(c - A.n) * 3 + d];
  }
}

// dColonSymScalar3 (include/dohp.h:77-78) on [00, 11, 22, 01, 02, 12] storage
__device__ __forceinline__ double colon_sym(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + 2 * (a[3] * b[3] + a[4] * b[4] + a[5] * b[5]);
}

// one rectangular pass along DIR of ne elements with input dims (D0, D1, D2): the DIR dimension goes from NP
// to N through Bp (TR false) or from N to NP through Bp^T (TR true)
template <int N, int NP, int D0, int D1, int D2, int DIR, bool TR>
__device__ __forceinline__ void rpass(const double *bp, const double *in, double *out, int ne) {
  constexpr int K = TR ? N : NP, M = TR ? NP : N;
  constexpr int O0 = DIR == 0 ? M : D0, O1 = DIR == 1 ? M : D1, O2 = DIR == 2 ? M : D2;
  constexpr int OUT = O0 * O1 * O2, IN = D0 * D1 * D2;
  for (int t = threadIdx.x; t < ne * OUT; t += blockDim.x) {
    const int el = t / OUT, r = t - el * OUT, i0 = r / (O1 * O2), i1 = (r / O2) % O1, i2 = r % O2;
    const int o = DIR == 0 ? i0 : DIR == 1 ? i1 : i2;
    const double *src = in + el * IN;
    double s = 0;
#pragma unroll
    for (int j = 0; j < K; j++) {
      const int j0 = DIR == 0 ? j : i0, j1 = DIR == 1 ? j : i1, j2 = DIR == 2 ? j : i2;
      s += (TR ? bp[j * NP + o] : bp[o * NP + j]) * src[(j0 * D1 + j1) * D2 + j2];
    }
    out[t] = s;
  }
}

template <int N, int NP>
__host__ __device__ constexpr int stokes_smem_elems(int cap) {
  return kTabElems + MAXP * MAXP + 12 * cap * N * N * N;
}

template <int N, int NP, int MODE>
__global__ void __launch_bounds__(256) k_stokes(StokesArgs S, int64_t nelem, int cap) {
  extern __shared__ double smem[];
  constexpr int N3 = N * N * N, P3 = NP * NP * NP;
  constexpr bool USE_U = MODE != SM_BT && MODE != SM_PINT, USE_P = MODE == SM_BT || MODE == SM_COUPLED || MODE == SM_FUNCTION;
  constexpr bool OUT_U = MODE != SM_B && MODE != SM_PINT;
  constexpr bool OUT_P = MODE == SM_B || MODE == SM_COUPLED || MODE == SM_FUNCTION || MODE == SM_PINT;
  const int64_t first = (int64_t)blockIdx.x * cap;
  const int ne = (int)min((int64_t)cap, nelem - first);
  double *tab = smem, *bp = smem + kTabElems, *buf = bp + MAXP * MAXP;
  const int L = cap * N3;
  double *S0 = buf, *S1 = buf + L, *G = buf + 2 * L, *Pq = buf + 11 * L;
  for (int i = threadIdx.x; i < N * NP; i += blockDim.x) bp[i] = S.bp[i];
  load_tables<N, double>(S.U.tab_all, tab);  // ends with a barrier
  if constexpr (USE_P) {
    gather<NP, double, 1>(S.P, S.P.x, nullptr, first, ne, 0, S0);
    __syncthreads();
    rpass<N, NP, NP, NP, NP, 0, false>(bp, S0, S1, ne);
    __syncthreads();
    rpass<N, NP, N, NP, NP, 1, false>(bp, S1, S0, ne);
    __syncthreads();
    rpass<N, NP, N, N, NP, 2, false>(bp, S0, Pq, ne);
    __syncthreads();
  }
  if constexpr (USE_U) {
    for (int d = 0; d < 3; d++) {
      if (MODE == SM_FUNCTION && S.udir)
        gather_inhomogeneous<N>(S.U, S.udir, first, ne, d, S0);
      else
        gather<N, double, 3>(S.U, S.U.x, nullptr, first, ne, d, S0);
      __syncthreads();
      interp3<N, double>(tab, S0, S1, ne);
      grad<N, double>(tab, S1, G + (d * 3 + 0) * L, G + (d * 3 + 1) * L, G + (d * 3 + 2) * L, ne);
    }
  }
  for (int t = threadIdx.x; t < ne * N3; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3;
    const double *gq = S.geo + (int64_t)S.U.qoff[first + el] * 10 + r;
    double Ji[9];
#pragma unroll
    for (int i = 0; i < 9; i++) Ji[i] = gq[i * N3];
    const double w = gq[9 * N3];
    double Du[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if constexpr (USE_U) {
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const double a0 = G[(d * 3 + 0) * L + t], a1 = G[(d * 3 + 1) * L + t], a2 = G[(d * 3 + 2) * L + t];
#pragma unroll
        for (int e = 0; e < 3; e++) Du[d * 3 + e] = a0 * Ji[0 * 3 + e] + a1 * Ji[1 * 3 + e] + a2 * Ji[2 * 3 + e];
      }
    }
    const double tr = Du[0] + Du[4] + Du[8];
    if constexpr (OUT_U) {
      const double p = USE_P ? Pq[t] : 0.0;
      const double lam = MODE == SM_A ? S.lam : 0.0;
      const double sd[6] = {Du[0], Du[4], Du[8], 0.5 * (Du[1] + Du[3]), 0.5 * (Du[2] + Du[6]), 0.5 * (Du[5] + Du[7])};
      double eta = MODE == SM_BT ? 0.0 : S.eta, dc = 0, sw[6] = {0, 0, 0, 0, 0, 0};
      if constexpr (MODE == SM_FUNCTION) {  // the store of this state
        if (S.store) {
          const double greg = S.heps2 + 0.5 * colon_sym(sd, sd);
          eta = S.B * pow(greg, S.hexp);
          double *st = S.store + (int64_t)S.U.qoff[first + el] * 8 + r;
          st[0] = eta;
          st[N3] = S.hexp * eta / greg;
#pragma unroll
          for (int i = 0; i < 6; i++) st[(2 + i) * N3] = sd[i];
        }
      } else if constexpr (MODE == SM_A || MODE == SM_COUPLED) {  // the Jacobian at the stored state
        if (S.store) {
          const double *st = S.store + (int64_t)S.U.qoff[first + el] * 8 + r;
          eta = st[0];
#pragma unroll
          for (int i = 0; i < 6; i++) sw[i] = st[(2 + i) * N3];
          dc = st[N3] * colon_sym(sw, sd);
        }
      }
      // Dv = w (eta Du_sym + eta' (Dw:Du) Dw + lam tr(Du) I - p I), symmetric
      const double diag = lam * tr - p;
      double Dv[9];
      Dv[0] = w * (eta * sd[0] + dc * sw[0] + diag);
      Dv[4] = w * (eta * sd[1] + dc * sw[1] + diag);
      Dv[8] = w * (eta * sd[2] + dc * sw[2] + diag);
      Dv[1] = Dv[3] = w * (eta * sd[3] + dc * sw[3]);
      Dv[2] = Dv[6] = w * (eta * sd[4] + dc * sw[4]);
      Dv[5] = Dv[7] = w * (eta * sd[5] + dc * sw[5]);
#pragma unroll
      for (int d = 0; d < 3; d++)
#pragma unroll
        for (int k = 0; k < 3; k++) G[(d * 3 + k) * L + t] = Dv[d * 3 + 0] * Ji[k * 3 + 0] + Dv[d * 3 + 1] * Ji[k * 3 + 1] + Dv[d * 3 + 2] * Ji[k * 3 + 2];
    }
    if constexpr (MODE == SM_PINT)
      Pq[t] = w * S.fpq[(int64_t)S.U.qoff[first + el] + r];
    else if constexpr (OUT_P)
      Pq[t] = -w * tr;
  }
  __syncthreads();
  if constexpr (OUT_U) {
    for (int d = 0; d < 3; d++)
      back<N, double, 3>(tab, G + (d * 3 + 0) * L, G + (d * 3 + 1) * L, G + (d * 3 + 2) * L, S0, S1, S.U, nullptr, first, ne, d,
                         (double *)S.U.yexp);
  }
  if constexpr (OUT_P) {
    rpass<N, NP, N, N, N, 2, true>(bp, Pq, S0, ne);
    __syncthreads();
    rpass<N, NP, N, N, NP, 1, true>(bp, S0, S1, ne);
    __syncthreads();
    rpass<N, NP, N, NP, NP, 0, true>(bp, S1, S0, ne);
    __syncthreads();
    double *yp = (double *)S.P.yexp;
    for (int t = threadIdx.x; t < ne * P3; t += blockDim.x) {
      const int el = t / P3, r = t - el * P3;
      yp[(int64_t)S.P.xstart[first + el] + r] = S0[t];
    }
  }
}

// diagonal of the pressure mass matrix on each element: sum_q w_q phi_i(x_q)^2, expanded layout
template <int N, int NP>
__global__ void k_pmass_diag(int64_t nelem, const int32_t *__restrict__ qoff, const int32_t *__restrict__ pxstart,
                             const double *__restrict__ geo, const double *__restrict__ bpg, double *__restrict__ dexp) {
  constexpr int N3 = N * N * N, P3 = NP * NP * NP;
  const int64_t e = blockIdx.x;
  if (e >= nelem) return;
  const double *w = geo + (int64_t)qoff[e] * 10 + 9 * N3;
  for (int r = threadIdx.x; r < P3; r += blockDim.x) {
    const int i0 = r / (NP * NP), i1 = (r / NP) % NP, i2 = r % NP;
    double s = 0;
    for (int q = 0; q < N3; q++) {
      const int a = q / (N * N), b = (q / N) % N, c = q % N;
      const double phi = bpg[a * NP + i0] * bpg[b * NP + i1] * bpg[c * NP + i2];
      s += w[q] * phi * phi;
    }
    dexp[(int64_t)pxstart[e] + r] = s;
  }
}

// z_p = -eta r_p / d (the Schur block)
__global__ void k_schur_diag(int64_t n, double eta, const double *__restrict__ d, const double *__restrict__ r, double *__restrict__ z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) z[i] = -eta * r[i] / d[i];
}
__global__ void k_sub_mean(int64_t n, const double *__restrict__ sum, double *__restrict__ z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) z[i] -= *sum / (double)n;
}
__global__ void k_rsub(int64_t n, const double *__restrict__ a, double *__restrict__ t) {  // t = a - t
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) t[i] = a[i] - t[i];
}
__global__ void k_axpby(int64_t n, double a, const double *x, double b, const double *y, double *w) {
  // w = a x + b y (w may alias x or y: each thread reads its own entries before writing)
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) w[i] = a * x[i] + b * y[i];
}
__global__ void k_fill(int64_t n, double v, double *__restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = v;
}

inline unsigned nblk(int64_t n) { return (unsigned)std::max<int64_t>((n + 255) / 256, 1); }

template <int N>
struct STile {
  static constexpr int EPB = N <= 3 ? 16 : N == 4 ? 8 : N == 5 ? 4 : 2;
};

template <int N, int NP, int MODE>
dErr launch_stokes_mode(const StokesArgs &S, int64_t nelem, cudaStream_t s) {
  constexpr int cap = STile<N>::EPB;
  const size_t smem = (size_t)stokes_smem_elems<N, NP>(cap) * sizeof(double);
  CUCHK(cudaFuncSetAttribute(k_stokes<N, NP, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_stokes<N, NP, MODE><<<(unsigned)((nelem + cap - 1) / cap), 256, smem, s>>>(S, nelem, cap);
  CUCHK(cudaGetLastError());
  return 0;
}

template <int N, int NP>
dErr launch_stokes_np(const StokesArgs &S, int mode, int64_t nelem, cudaStream_t s) {
  switch (mode) {
    case SM_A: return launch_stokes_mode<N, NP, SM_A>(S, nelem, s);
    case SM_BT: return launch_stokes_mode<N, NP, SM_BT>(S, nelem, s);
    case SM_B: return launch_stokes_mode<N, NP, SM_B>(S, nelem, s);
    case SM_COUPLED: return launch_stokes_mode<N, NP, SM_COUPLED>(S, nelem, s);
    case SM_FUNCTION: return launch_stokes_mode<N, NP, SM_FUNCTION>(S, nelem, s);
    case SM_PINT: return launch_stokes_mode<N, NP, SM_PINT>(S, nelem, s);
  }
  return set_error("Stokes mult mode %d", mode);
}

// velocity degree k = N - 1 in 2..6, pressure degree k - 1 or k - 2 (>= 1)
dErr launch_stokes(const StokesArgs &S, int N, int NP, int mode, int64_t nelem, cudaStream_t s) {
#define DGB_STOKES_CASE(a, b) \
  if (N == a && NP == b) return launch_stokes_np<a, b>(S, mode, nelem, s);
  DGB_STOKES_CASE(3, 2)
  DGB_STOKES_CASE(4, 3)
  DGB_STOKES_CASE(4, 2)
  DGB_STOKES_CASE(5, 4)
  DGB_STOKES_CASE(5, 3)
  DGB_STOKES_CASE(6, 5)
  DGB_STOKES_CASE(6, 4)
  DGB_STOKES_CASE(7, 6)
  DGB_STOKES_CASE(7, 5)
#undef DGB_STOKES_CASE
  return set_error("Stokes spaces of degrees %d / %d are not built (velocity 2..6, pressure codim 1 or 2)", N - 1, NP - 1);
}

dErr pmass_diag(int N, int NP, int64_t nelem, const int32_t *qoff, const int32_t *pxstart, const double *geo, const double *bp,
                double *dexp, cudaStream_t s) {
#define DGB_PM_CASE(a, b) \
  if (N == a && NP == b) {                                                                        \
    k_pmass_diag<a, b><<<(unsigned)std::max<int64_t>(nelem, 1), 64, 0, s>>>(nelem, qoff, pxstart, geo, bp, dexp); \
    CUCHK(cudaGetLastError());                                                                     \
    return 0;                                                                                      \
  }
  DGB_PM_CASE(3, 2)
  DGB_PM_CASE(4, 3)
  DGB_PM_CASE(4, 2)
  DGB_PM_CASE(5, 4)
  DGB_PM_CASE(5, 3)
  DGB_PM_CASE(6, 5)
  DGB_PM_CASE(6, 4)
  DGB_PM_CASE(7, 6)
  DGB_PM_CASE(7, 5)
#undef DGB_PM_CASE
  return set_error("Stokes spaces of degrees %d / %d are not built", N - 1, NP - 1);
}

}  // namespace

struct _p_dStokes {
  dFS fsu = nullptr, fsp = nullptr;
  double B = 1, eps = 1, p = 2, nu = 0, lam = 0;
  double eta0 = 1;              // viscosity at the zero state: the scale of the preconditioner's blocks
  double *d_store = nullptr;    // power law: {eta, eta', Du[6]} per velocity point at the last function's state
  bool have_state = false;
  int N = 0, NP = 0;
  int64_t nu3 = 0, np = 0;  // global sizes: velocity n*3, pressure n
  double *d_geo = nullptr, *d_bp = nullptr, *d_yu = nullptr, *d_yp = nullptr;
  double *d_mdiag = nullptr;  // diagonal of the pressure mass matrix (global)
  double *d_t = nullptr;      // velocity temporary
  double *d_part = nullptr, *d_s = nullptr;
  dOperator opu = nullptr;    // velocity elasticity-kind operator: carries the velocity block's KSP
  dMat Ap = nullptr;
  dKSP kspu = nullptr, ksp = nullptr;
  int restart = 30;
  double *d_pb = nullptr, *d_px = nullptr;  // packed [u; p] right-hand side and iterate of the solve
};

static dErr stokes_mult(_p_dStokes *S, int mode, const double *xu, const double *xp, double *yu, double *yp,
                        const double *fpq = nullptr) {
  _p_dFS *fu = S->fsu, *fp = S->fsp;
  cudaStream_t s = fu->stream;
  auto eargs = [](_p_dFS *fs, const double *x, double *yexp) {
    ElemArgs A{};
    A.xstart = fs->d_xstart;
    A.qoff = fs->d_qoff;
    A.emap = fs->d_emap;
    A.n = fs->n;
    A.x = x;
    A.tab_all = fs->d_fast_tab;
    A.yexp = yexp;
    return A;
  };
  StokesArgs A;
  A.U = eargs(fu, xu, S->d_yu);
  A.P = eargs(fp, xp, S->d_yp);
  A.bp = S->d_bp;
  A.geo = S->d_geo;
  A.store = nullptr;
  A.udir = mode == SM_FUNCTION && fu->nc > fu->n ? fu->d_dcache : nullptr;
  A.fpq = fpq;
  if (S->d_store && (mode == SM_FUNCTION || (S->have_state && (mode == SM_A || mode == SM_COUPLED)))) A.store = S->d_store;
  A.eta = S->eta0;
  A.lam = S->lam;
  A.B = S->B;
  A.heps2 = 0.5 * S->eps * S->eps;
  A.hexp = 0.5 * (S->p - 2);
  if (fu->nelem) DCHK(launch_stokes(A, S->N, S->NP, mode, fu->nelem, s));
  if (mode != SM_B && mode != SM_PINT) DCHK(fs_restrict(fu, S->d_yu, yu, 0));
  // the pressure restriction runs on the velocity space's stream, after the kernel that wrote d_yp, whatever
  // stream the pressure space carries
  if (mode == SM_B || mode == SM_COUPLED || mode == SM_FUNCTION || mode == SM_PINT)
    DCHK(fs_restrict_rows(fp, S->d_yp, yp, 0, fp->n, s));
  if (mode == SM_FUNCTION && S->d_store) S->have_state = true;
  return 0;
}

static dErr stokes_shell_mult(void *ctx, const double *x, double *y) {
  _p_dStokes *S = (_p_dStokes *)ctx;
  return stokes_mult(S, SM_COUPLED, x, x + S->nu3, y, y + S->nu3);
}

// block upper triangular preconditioner on the packed vector
static dErr stokes_shell_pc(void *ctx, const double *r, double *z) {
  _p_dStokes *S = (_p_dStokes *)ctx;
  cudaStream_t s = S->fsu->stream;
  const double *ru = r, *rp = r + S->nu3;
  double *zu = z, *zp = z + S->nu3;
  k_schur_diag<<<nblk(S->np), 256, 0, s>>>(S->np, S->eta0, S->d_mdiag, rp, zp);
  CUCHK(cudaGetLastError());
  // remove the constant (mean over the dofs): sum through a dot with the ones vector stored after d_t
  const double *ones = S->d_t + S->nu3;
  DCHK(device_dot(S->np, zp, ones, S->d_part, S->d_s, s));
  k_sub_mean<<<nblk(S->np), 256, 0, s>>>(S->np, S->d_s, zp);
  // t = r_u - Bt z_p, z_u = Cheb(A_q1) t
  double *t = S->d_t;
  DCHK(stokes_mult(S, SM_BT, nullptr, zp, t, nullptr));
  k_rsub<<<nblk(S->nu3), 256, 0, s>>>(S->nu3, ru, t);
  CUCHK(cudaGetLastError());
  return ksp_pc_only(S->kspu, t, zu);
}

extern "C" {

dErr dStokesCreate(dFS fsu, dFS fsp, const dReal rheo[4], dStokes *stk) {
  if (!fsu || !fsp || !stk) return set_error("null argument");
  if (!fsu->setup || !fsp->setup) return set_error("dFS not set up");
  if (fsu->bs != 3 || fsp->bs != 1) return set_error("Stokes needs a bs 3 velocity space and a bs 1 pressure space");
  if (fsu->nelem != fsp->nelem || fsu->mesh != fsp->mesh) return set_error("velocity and pressure spaces must share the mesh");
  if (!fsu->uniform || !fsp->uniform) return set_error("Stokes spaces of uniform degree only");
  if (fsp->dirichlet_mask) return set_error("the pressure space takes no Dirichlet sets (stokes.c:222)");
  _p_dStokes *S = new _p_dStokes();
  if (rheo) S->B = rheo[0], S->eps = rheo[1], S->p = rheo[2], S->nu = rheo[3];
  if (!(S->B > 0) || !(S->nu < 0.5) || !(S->p > 1) || (S->p != 2 && !(S->eps > 0))) {
    delete S;
    return set_error("Stokes rheology needs B > 0, p > 1, eps > 0 (p != 2) and nu < 1/2");
  }
  S->lam = S->nu / (1 - 2 * S->nu);  // StokesLambda (stokes.c:455-458)
  S->eta0 = S->p == 2 ? S->B : S->B * std::pow(0.5 * S->eps * S->eps, 0.5 * (S->p - 2));
  S->fsu = fsu, S->fsp = fsp;
  S->N = fsu->p + 1, S->NP = fsp->p + 1;
  if (!(S->NP == S->N - 1 || S->NP == S->N - 2) || S->NP < 2 || S->N > 7) {
    delete S;
    return set_error("Stokes spaces of degrees %d / %d are not built (velocity 2..6, pressure codim 1 or 2)", fsu->p, fsp->p);
  }
  S->nu3 = fsu->n * 3;
  S->np = fsp->n;
  cudaStream_t s = fsu->stream;
  // pressure GLL basis at the velocity's Gauss points
  {
    double x[MAXQ], w[MAXQ], gll[MAXP], lw[MAXP], val[MAXP], der[MAXP];
    gauss_rule(S->N, x, w);
    lobatto_rule(S->NP, gll, lw);
    std::vector<double> bp(S->N * S->NP);
    for (int a = 0; a < S->N; a++) {
      lagrange(S->NP, gll, x[a], val, der);
      for (int i = 0; i < S->NP; i++) bp[a * S->NP + i] = val[i];
    }
    CUCHK(cudaMalloc(&S->d_bp, bp.size() * sizeof(double)));
    CUCHK(cudaMemcpy(S->d_bp, bp.data(), bp.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  CUCHK(cudaMalloc(&S->d_geo, std::max<int64_t>(fsu->nq, 1) * 10 * sizeof(double)));
  DCHK(geometry_fill(fsu, 1, nullptr, S->d_geo));
  if (S->p != 2) CUCHK(cudaMalloc(&S->d_store, std::max<int64_t>(fsu->nq, 1) * 8 * sizeof(double)));
  CUCHK(cudaMalloc(&S->d_yu, std::max<int64_t>(fsu->nexp * 3, 1) * sizeof(double)));
  CUCHK(cudaMalloc(&S->d_yp, std::max<int64_t>(fsp->nexp, 1) * sizeof(double)));
  CUCHK(cudaMalloc(&S->d_mdiag, std::max<int64_t>(S->np, 1) * sizeof(double)));
  CUCHK(cudaMalloc(&S->d_t, (S->nu3 + std::max<int64_t>(S->np, 1)) * sizeof(double)));
  DCHK(dot_part_alloc(&S->d_part));
  CUCHK(cudaMalloc(&S->d_s, 8 * sizeof(double)));
  k_fill<<<nblk(S->np), 256, 0, s>>>(S->np, 1.0, S->d_t + S->nu3);  // ones vector for the pressure mean
  DCHK(pmass_diag(S->N, S->NP, fsu->nelem, fsu->d_qoff, fsp->d_xstart, S->d_geo, S->d_bp, S->d_yp, s));
  DCHK(fs_restrict_rows(fsp, S->d_yp, S->d_mdiag, 0, fsp->n, s));
  CUCHK(cudaStreamSynchronize(s));
  *stk = S;
  return 0;
}

dErr dStokesDestroy(dStokes *stk) {
  if (!stk || !*stk) return 0;
  _p_dStokes *S = *stk;
  for (double *p : {S->d_geo, S->d_bp, S->d_yu, S->d_yp, S->d_mdiag, S->d_t, S->d_part, S->d_s, S->d_pb, S->d_px, S->d_store})
    cudaFree(p);
  dKSPDestroy(&S->ksp);
  dKSPDestroy(&S->kspu);
  dMatDestroy(&S->Ap);
  dOperatorDestroy(&S->opu);
  delete S;
  *stk = nullptr;
  return 0;
}

dErr dStokesMult(dStokes stk, dStokesMultMode mode, const dScalar *xu, const dScalar *xp, dScalar *yu, dScalar *yp) {
  if (!stk) return set_error("null Stokes");
  const int m = (int)mode;
  if (m < SM_A || m > SM_COUPLED) return set_error("invalid Stokes mult mode %d", m);
  if ((m != SM_BT && !xu) || ((m == SM_BT || m == SM_COUPLED) && !xp) || (m != SM_B && !yu) || ((m == SM_B || m == SM_COUPLED) && !yp))
    return set_error("missing vector for Stokes mult mode %d", m);
  return stokes_mult(stk, m, xu, xp, yu, yp);
}

dErr dStokesFunction(dStokes stk, const dScalar *xu, const dScalar *xp, dScalar *yu, dScalar *yp) {
  if (!stk || !xu || !xp || !yu || !yp) return set_error("null argument");
  return stokes_mult(stk, SM_FUNCTION, xu, xp, yu, yp);
}

dErr dStokesIntegratePressure(dStokes stk, const dScalar *fq, dScalar *yp) {
  if (!stk || !fq || !yp) return set_error("null argument");
  return stokes_mult(stk, SM_PINT, nullptr, nullptr, nullptr, yp, fq);
}

}  // extern "C"

// the solver objects: the velocity block (one Q1 multigrid V-cycle or Chebyshev-Jacobi on the Q1-embedded A with
// 2 mu = eta0, lambda as A) and the FGMRES on the packed vector with the block preconditioner
static dErr stokes_solver_setup(_p_dStokes *S) {
  _p_dFS *fu = S->fsu;
  cudaStream_t s = fu->stream;
  if (!S->ksp) {
    DCHK(dFSCreateOperator(fu, dOP_ELASTICITY, nullptr, &S->opu));
    DCHK(dFSCreateMatrix(fu, &S->Ap));
    DCHK(q1_numeric_elast(fu, S->Ap, S->lam, 0.5 * S->eta0, 1));
    // the velocity block's approximate inverse: one Q1 multigrid V-cycle where the GLL lattice coarsens (an even
    // number of GLL intervals per direction), else the single-level Chebyshev-Jacobi
    const _p_dMesh *mesh = fu->mesh;
    const bool lattice = ((mesh->nx - 1) * fu->p) % 2 == 0 && ((mesh->ny - 1) * fu->p) % 2 == 0 && ((mesh->nz - 1) * fu->p) % 2 == 0 &&
                         (mesh->nx - 1) * fu->p >= 4 && (mesh->ny - 1) * fu->p >= 4 && (mesh->nz - 1) * fu->p >= 4;
    DCHK(dKSPCreate(S->opu, S->Ap, dKSP_CG, lattice ? dPC_MG_Q1 : dPC_CHEBYSHEV_Q1, &S->kspu));
    DCHK(ksp_create_shell(S->nu3 + S->np, s, dKSP_FGMRES, stokes_shell_mult, stokes_shell_pc, S, S->restart, &S->ksp));
  }
  if (!S->d_pb) {
    const int64_t n = S->nu3 + S->np;
    CUCHK(cudaMalloc(&S->d_pb, n * sizeof(double)));
    CUCHK(cudaMalloc(&S->d_px, n * sizeof(double)));
  }
  return 0;
}

extern "C" {

dErr dStokesSolve(dStokes stk, const dScalar *bu, const dScalar *bp, dScalar *xu, dScalar *xp, dReal rtol, dInt maxit, dInt *its,
                  dReal *rnorm) {
  Range range_("KSPSolve (Stokes)");
  if (!stk || !bu || !bp || !xu || !xp) return set_error("null argument");
  _p_dStokes *S = stk;
  cudaStream_t s = S->fsu->stream;
  DCHK(stokes_solver_setup(S));
  double *b = S->d_pb, *x = S->d_px;
  CUCHK(cudaMemcpyAsync(b, bu, S->nu3 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaMemcpyAsync(b + S->nu3, bp, S->np * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaMemcpyAsync(x, xu, S->nu3 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaMemcpyAsync(x + S->nu3, xp, S->np * sizeof(double), cudaMemcpyDeviceToDevice, s));
  int it = 0;
  double rn = 0;
  dErr e = ksp_solve(S->ksp, b, x, rtol, maxit, &it, &rn);
  if (!e) {  // the pressure is determined up to a constant: return the zero-mean one
    const double *ones = S->d_t + S->nu3;
    e = device_dot(S->np, x + S->nu3, ones, S->d_part, S->d_s, s);
    if (!e) k_sub_mean<<<nblk(S->np), 256, 0, s>>>(S->np, S->d_s, x + S->nu3);
  }
  if (!e) {
    CUCHK(cudaMemcpyAsync(xu, x, S->nu3 * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CUCHK(cudaMemcpyAsync(xp, x + S->nu3, S->np * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CUCHK(cudaStreamSynchronize(s));
  }
  if (e) return e;
  if (its) *its = it;
  if (rnorm) *rnorm = rn;
  if (!(rn <= rtol)) return set_error("Stokes FGMRES did not converge in %d iterations (relative residual %g)", it, rn);
  return 0;
}

// Newton for the power-law Stokes system N(x) = b (the SNES of stokes.c: StokesFunction / StokesJacobian,
// stokes.c:507-540, 675-740): each step solves J(x) dx = -F with the block-preconditioned FGMRES (the Jacobian at
// the store of the last function evaluation) and backtracks on ||F||.
dErr dStokesNewtonSolve(dStokes stk, const dScalar *bu, const dScalar *bp, dScalar *xu, dScalar *xp, const dNewtonOptions *opt,
                        dInt *its, dReal *fnorm, dInt *lin_its) {
  Range range_("SNESSolve (Stokes)");
  if (!stk || !bu || !bp || !xu || !xp || !opt) return set_error("null argument");
  _p_dStokes *S = stk;
  cudaStream_t s = S->fsu->stream;
  DCHK(stokes_solver_setup(S));
  const int64_t n = S->nu3 + S->np;
  const unsigned g = nblk(n);
  double *b = S->d_pb, *x = S->d_px, *block = nullptr;
  CUCHK(cudaMalloc(&block, 4 * n * sizeof(double)));
  double *F = block, *dx = F + n, *xt = dx + n, *Ft = xt + n;
  CUCHK(cudaMemcpyAsync(b, bu, S->nu3 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaMemcpyAsync(b + S->nu3, bp, S->np * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaMemcpyAsync(x, xu, S->nu3 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaMemcpyAsync(x + S->nu3, xp, S->np * sizeof(double), cudaMemcpyDeviceToDevice, s));
  auto residual = [&](const double *xx, double *r, double *nrm) -> dErr {  // r = N(xx) - b, keeps the store of xx
    DCHK(stokes_mult(S, SM_FUNCTION, xx, xx + S->nu3, r, r + S->nu3));
    k_axpby<<<g, 256, 0, s>>>(n, 1.0, r, -1.0, b, r);
    CUCHK(cudaGetLastError());
    DCHK(device_dot(n, r, r, S->d_part, S->d_s, s));
    double h = 0;
    CUCHK(cudaMemcpyAsync(&h, S->d_s, sizeof h, cudaMemcpyDeviceToHost, s));
    CUCHK(cudaStreamSynchronize(s));
    *nrm = std::sqrt(h);
    return 0;
  };
  double fn = 0, fn0 = 0;
  int k = 0;
  dErr err = residual(x, F, &fn);
  fn0 = fn;
  if (fnorm && !err) fnorm[0] = fn;
  for (; !err && k < opt->max_it && fn > opt->rtol * fn0 && fn > opt->atol; k++) {
    k_axpby<<<g, 256, 0, s>>>(n, -1.0, F, 0.0, F, Ft);  // rhs = -F (Ft as scratch)
    if (cudaMemsetAsync(dx, 0, n * sizeof(double), s) != cudaSuccess) {
      err = set_error("cudaMemsetAsync failed");
      break;
    }
    int li = 0;
    double rn = 0;
    err = ksp_solve(S->ksp, Ft, dx, opt->lin_rtol, opt->lin_maxit, &li, &rn);
    if (err) break;
    if (!(rn < 1)) {
      err = set_error("Stokes Newton step %d: linear solve made no progress (relative residual %g)", k, rn);
      break;
    }
    if (lin_its) lin_its[k] = li;
    double lam = 1, fnt = 0;
    int ls = 0;
    for (; ls < 12; ls++, lam *= 0.5) {
      k_axpby<<<g, 256, 0, s>>>(n, 1.0, x, lam, dx, xt);
      err = residual(xt, Ft, &fnt);
      if (err || fnt < (1 - 1e-4 * lam) * fn) break;
    }
    if (err) break;
    if (ls == 12) {
      err = set_error("Stokes Newton line search failed at step %d (||F|| %g)", k, fn);
      break;
    }
    std::swap(x, xt);  // the store is that of the accepted iterate, the last one evaluated
    std::swap(F, Ft);
    fn = fnt;
    if (fnorm) fnorm[k + 1] = fn;
  }
  if (!err) {  // the pressure is determined up to a constant: return the zero-mean one
    const double *ones = S->d_t + S->nu3;
    err = device_dot(S->np, x + S->nu3, ones, S->d_part, S->d_s, s);
    if (!err) k_sub_mean<<<nblk(S->np), 256, 0, s>>>(S->np, S->d_s, x + S->nu3);
  }
  if (!err && (cudaMemcpyAsync(xu, x, S->nu3 * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
               cudaMemcpyAsync(xp, x + S->nu3, S->np * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess))
    err = set_error("cudaMemcpyAsync failed");
  cudaStreamSynchronize(s);
  cudaFree(block);
  if (its) *its = k;
  return err;
}

}  // extern "C"
