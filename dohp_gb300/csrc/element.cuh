// Element kernel shared by the uniform-order and the hp operator applies (TensorMult_Hex and the
// EllipShellMatMult / ElastShellMatMult q-functions, inlinetmulthex.h:19-100, ellip.c:442-472,
// elast.c:227-341, restated as one fused pass per group of elements).
//
// Per element: gather the nodal values through E, interpolate to the Gauss points (B along x, y, z),
// collocation gradient at the Gauss points (Dq along x, y, z), pointwise q-function with precomputed
// geometric factors, transposed gradient, transposed interpolation, write the expanded output.
//
// Each 1-D contraction runs one thread per output value (N multiply-adds). An even-odd form (pairs of
// outputs from the centro-symmetry of B and Dq, about N^2/2 + 2N operations per line instead of N^2) was
// measured slower on GB300 in two forms: one thread per line leaves too few warps to hide the FP64 latency,
// and one thread per output pair (e/o values formed in a sub-pass) pays more in barriers and shared-memory
// round trips than the 16-30 % of FP64 operations it saves.
#pragma once

#include <cuda_bf16.h>

#include "ff.cuh"
#include "internal.h"

namespace dgb {

struct ElemArgs {
  const int32_t *xstart, *qoff;
  const int32_t *eptr, *ecol;  // E as weighted CSR (hp spaces), or NULL: Boolean E through emap
  const double *eval;
  const int32_t *emap;
  int64_t n;
  const double *x;
  const double *const *px;  // graph form: x read through this table when non-null
  const void *geo;
  const double *tab_all;
  void *yexp;
  double lam, mu;
  double *stash;  // St. Venant-Kirchhoff: {F (9), S (6)} per point, SoA per element
  const double *dcache;  // Dirichlet values of the closure nodes beyond n (inhomogeneous gather), or NULL: zero
};

// element kinds beyond the ABI's operator kinds: St. Venant-Kirchhoff function (writes the stash) and
// Jacobian at the stashed state (elast.c:224-280)
constexpr int K_SVK_FUNC = 100, K_SVK_JAC = 101;

// shared-memory table region: B and Dq (MAXP x MAXP each)
constexpr int kTabElems = 2 * MAXP * MAXP;
enum { M_B = 0, M_BT = 1, M_D = 2, M_DT = 3 };

// value rounded to BF16 and widened back (the BF16 apply stores inputs, tables and factors in BF16)
template <typename T>
__device__ __forceinline__ T bf16_round(double v) {
  return (T)__bfloat162float(__float2bfloat16_rn((float)v));
}

template <int N, typename T, bool BF = false>
__device__ __forceinline__ void load_tables(const double *tab_all, T *sm) {
  const double *tab = tab_all + (size_t)2 * (N - 2) * MAXP * MAXP;
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    sm[i] = BF ? bf16_round<T>(tab[i]) : (T)tab[i];
    sm[MAXP * MAXP + i] = BF ? bf16_round<T>(tab[MAXP * MAXP + i]) : (T)tab[MAXP * MAXP + i];
  }
  __syncthreads();
}

// one pass over all outputs of ne elements (blocks of N^3 values, back to back) along direction DIR
// (0: x, stride N*N; 1: y, stride N; 2: z, stride 1): out[..i..] = sum_j M[i][j] in[..j..]
template <int N, int MAT, int DIR, typename T>
__device__ __forceinline__ void pass(const T *sm, const T *in, T *out, int ne) {
  constexpr int NN = N * N, N3 = NN * N, ST = DIR == 0 ? NN : DIR == 1 ? N : 1;
  const T *M = MAT < 2 ? sm : sm + MAXP * MAXP;
  for (int t = threadIdx.x; t < ne * N3; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3;
    const int i = DIR == 0 ? r / NN : DIR == 1 ? (r / N) % N : r % N;
    const T *src = in + el * N3 + r - i * ST;
    T s = 0;
#pragma unroll
    for (int j = 0; j < N; j++) fma_acc(s, (MAT & 1) ? M[j * N + i] : M[i * N + j], src[j * ST]);
    out[t] = fin(s);
  }
}

__device__ __forceinline__ int64_t elem_id(const int32_t *els, int64_t first, int el) { return els ? els[el] : first + el; }

// gather one component of the element's nodes through E (closure nodes beyond n: A.dcache, or 0 when NULL)
template <int N, typename T, int BS, bool BF = false>
__device__ __forceinline__ void gather(const ElemArgs &A, const double *x, const int32_t *els, int64_t first, int ne, int d, T *dst) {
  constexpr int N3 = N * N * N;
  for (int t = threadIdx.x; t < ne * N3; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3;
    const int64_t row = A.xstart[elem_id(els, first, el)] + r;
    double v = 0;
    if (A.eptr) {
      for (int32_t k = A.eptr[row]; k < A.eptr[row + 1]; k++) {
        const int32_t c = A.ecol[k];
        if (c < A.n) v += A.eval[k] * x[(int64_t)c * BS + d];
        else if (A.dcache) v += A.eval[k] * A.dcache[(int64_t)(c - A.n) * BS + d];
      }
    } else {
      const int32_t c = A.emap[row];
      if (c < A.n) v = x[(int64_t)c * BS + d];
      else if (A.dcache) v = A.dcache[(int64_t)(c - A.n) * BS + d];
    }
    dst[t] = BF ? bf16_round<T>(v) : (T)v;
  }
}

// S0 (nodal) -> S1 (Gauss points), S0 as scratch
template <int N, typename T>
__device__ __forceinline__ void interp3(const T *sm, T *S0, T *S1, int ne) {
  pass<N, M_B, 0>(sm, S0, S1, ne);
  __syncthreads();
  pass<N, M_B, 1>(sm, S1, S0, ne);
  __syncthreads();
  pass<N, M_B, 2>(sm, S0, S1, ne);
  __syncthreads();
}

// reference gradient at the Gauss points of U (S1) -> G0, G1, G2 (collocation derivative Dq)
template <int N, typename T>
__device__ __forceinline__ void grad(const T *sm, const T *S1, T *G0, T *G1, T *G2, int ne) {
  constexpr int N3 = N * N * N, NN = N * N;
  const T *sD = sm + MAXP * MAXP;
  for (int t = threadIdx.x; t < ne * N3; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, a = r / NN, b = (r / N) % N, c = r % N;
    const T *U = &S1[el * N3];
    T g0 = 0, g1 = 0, g2 = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
      fma_acc(g0, sD[a * N + i], U[i * NN + b * N + c]);
      fma_acc(g1, sD[b * N + i], U[a * NN + i * N + c]);
      fma_acc(g2, sD[c * N + i], U[a * NN + b * N + i]);
    }
    G0[t] = fin(g0);
    G1[t] = fin(g1);
    G2[t] = fin(g2);
  }
  __syncthreads();
}

// transposed gradient (V0, V1, V2 -> S1), transposed interpolation, component d of the expanded output
template <int N, typename T, int BS>
__device__ __forceinline__ void back(const T *sm, const T *V0, const T *V1, const T *V2, T *S0, T *S1, const ElemArgs &A,
                                     const int32_t *els, int64_t first, int ne, int d, T *yexp) {
  constexpr int NN = N * N, N3 = NN * N;
  const T *sB = sm, *sD = sm + MAXP * MAXP;
  for (int t = threadIdx.x; t < ne * N3; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, a = r / NN, b = (r / N) % N, c = r % N;
    const T *v0 = &V0[el * N3], *v1 = &V1[el * N3], *v2 = &V2[el * N3];
    T s = 0;
#pragma unroll
    for (int i = 0; i < N; i++)
      dot3_acc(s, sD[i * N + a], v0[i * NN + b * N + c], sD[i * N + b], v1[a * NN + i * N + c], sD[i * N + c], v2[a * NN + b * N + i]);
    S1[t] = fin(s);
  }
  __syncthreads();
  pass<N, M_BT, 2>(sm, S1, S0, ne);
  __syncthreads();
  pass<N, M_BT, 1>(sm, S0, S1, ne);
  __syncthreads();
  for (int t = threadIdx.x; t < ne * N3; t += blockDim.x) {
    const int el = t / N3, r = t - el * N3, i = r / NN, jk = r - i * NN;
    const T *in = &S1[el * N3 + jk];
    T s = 0;
#pragma unroll
    for (int a = 0; a < N; a++) fma_acc(s, sB[a * N + i], in[a * NN]);
    yexp[((int64_t)A.xstart[elem_id(els, first, el)] + r) * BS + d] = fin(s);
  }
  __syncthreads();
}

// shared memory (in T) of one group of cap elements: tables + buffers
__host__ __device__ constexpr bool elastic_kind(int kind) { return kind == dOP_ELASTICITY || kind == K_SVK_FUNC || kind == K_SVK_JAC; }
__host__ __device__ constexpr int group_smem_elems(int N, int kind, int cap) {
  return kTabElems + (elastic_kind(kind) ? 11 : 5) * cap * N * N * N;
}

// apply the operator to ne (<= cap) elements: ids els[0..ne) or first..first+ne. T: arithmetic type;
// GT: storage type of the geometric factors; BF: inputs and basis tables rounded to BF16 (the BF16 apply:
// BF16 storage, FP32 arithmetic and accumulation)
template <int N, typename T, int KIND, typename GT = T, bool BF = false>
__device__ void group_apply(const ElemArgs &A, const int32_t *els, int64_t first, int ne, int cap, T *sm) {
  constexpr int N3 = N * N * N;
  T *buf = sm + kTabElems;
  const int L = cap * N3, tot = ne * N3;
  const double *x = A.px ? *A.px : A.x;
  T *yexp = (T *)A.yexp;
  load_tables<N, T, BF>(A.tab_all, sm);
  if constexpr (!elastic_kind(KIND)) {  // diffusion and the p-Laplacian Jacobian: G (6 per point)
    T *S0 = buf, *S1 = buf + L, *G0 = buf + 2 * L, *G1 = buf + 3 * L, *G2 = buf + 4 * L;
    gather<N, T, 1, BF>(A, x, els, first, ne, 0, S0);
    __syncthreads();
    interp3<N, T>(sm, S0, S1, ne);
    grad<N, T>(sm, S1, G0, G1, G2, ne);
    const GT *geo = (const GT *)A.geo;
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
      const int el = t / N3, r = t - el * N3;
      const GT *G = geo + (int64_t)A.qoff[elem_id(els, first, el)] * 6 + r;
      const T g0 = G0[t], g1 = G1[t], g2 = G2[t];
      const T a0 = (T)G[0], a1 = (T)G[N3], a2 = (T)G[2 * N3], a3 = (T)G[3 * N3], a4 = (T)G[4 * N3], a5 = (T)G[5 * N3];
      G0[t] = a0 * g0 + a1 * g1 + a2 * g2;
      G1[t] = a1 * g0 + a3 * g1 + a4 * g2;
      G2[t] = a2 * g0 + a4 * g1 + a5 * g2;
    }
    __syncthreads();
    back<N, T, 1>(sm, G0, G1, G2, S0, S1, A, els, first, ne, 0, yexp);
  } else {
    T *S0 = buf, *S1 = buf + L, *G = buf + 2 * L;  // G: [d][k][L]
    for (int d = 0; d < 3; d++) {
      gather<N, T, 3>(A, x, els, first, ne, d, S0);
      __syncthreads();
      interp3<N, T>(sm, S0, S1, ne);
      grad<N, T>(sm, S1, G + (d * 3 + 0) * L, G + (d * 3 + 1) * L, G + (d * 3 + 2) * L, ne);
    }
    const T *geo = (const T *)A.geo;
    const T lam = (T)A.lam, mu = (T)A.mu;
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
      const int el = t / N3, r = t - el * N3;
      const T *gq = geo + (int64_t)A.qoff[elem_id(els, first, el)] * 10 + r;
      T Ji[9];
#pragma unroll
      for (int i = 0; i < 9; i++) Ji[i] = gq[i * N3];
      const T w = gq[9 * N3];
      T Du[9];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const T a0 = G[(d * 3 + 0) * L + t], a1 = G[(d * 3 + 1) * L + t], a2 = G[(d * 3 + 2) * L + t];
#pragma unroll
        for (int e = 0; e < 3; e++) Du[d * 3 + e] = a0 * Ji[0 * 3 + e] + a1 * Ji[1 * 3 + e] + a2 * Ji[2 * 3 + e];
      }
      T S[9];
      if constexpr (KIND == dOP_ELASTICITY) {
        // ElastPointwiseJacobian at F = I (elast.c:269-280): eps = sym(grad u), dv = w (lambda tr(eps) I + 2 mu eps)
        const T e01 = (T)0.5 * (Du[1] + Du[3]), e02 = (T)0.5 * (Du[2] + Du[6]), e12 = (T)0.5 * (Du[5] + Du[7]);
        const T tr = Du[0] + Du[4] + Du[8];
        S[0] = w * (lam * tr + 2 * mu * Du[0]);
        S[4] = w * (lam * tr + 2 * mu * Du[4]);
        S[8] = w * (lam * tr + 2 * mu * Du[8]);
        S[1] = S[3] = w * (2 * mu * e01);
        S[2] = S[6] = w * (2 * mu * e02);
        S[5] = S[7] = w * (2 * mu * e12);
      } else {
        // St. Venant-Kirchhoff (elast.c:224-280): E = (F^T F - I)/2, S = lambda tr(E) I + 2 mu E (storage
        // [00, 11, 22, 01, 02, 12]); function Dv = w F S with F = I + Du, Jacobian Dv = w (F dS + dF S)
        double *st = A.stash + (int64_t)A.qoff[elem_id(els, first, el)] * 15 + r;
        T F[9], P6[6];
        auto dotcol = [](const T *a, const T *b, int i, int j) { return a[i] * b[j] + a[3 + i] * b[3 + j] + a[6 + i] * b[6 + j]; };
        auto pk2 = [&](const T *Fm, const T *dF, T *out) {  // dF == nullptr: S(F); else dS(F; dF)
          T E[6];
          const int ij[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
#pragma unroll
          for (int k = 0; k < 6; k++)
            E[k] = dF ? (T)0.5 * (dotcol(Fm, dF, ij[k][0], ij[k][1]) + dotcol(dF, Fm, ij[k][0], ij[k][1]))
                      : (T)0.5 * (dotcol(Fm, Fm, ij[k][0], ij[k][1]) - (k < 3 ? (T)1 : (T)0));
          const T trE = E[0] + E[1] + E[2];
#pragma unroll
          for (int k = 0; k < 6; k++) out[k] = lam * trE * (k < 3 ? (T)1 : (T)0) + 2 * mu * E[k];
        };
        auto gesy = [](T *C, const T *Am, const T *Sy, bool add) {
#pragma unroll
          for (int i = 0; i < 3; i++) {
            const T c0 = Am[i * 3 + 0] * Sy[0] + Am[i * 3 + 1] * Sy[3] + Am[i * 3 + 2] * Sy[4];
            const T c1 = Am[i * 3 + 0] * Sy[3] + Am[i * 3 + 1] * Sy[1] + Am[i * 3 + 2] * Sy[5];
            const T c2 = Am[i * 3 + 0] * Sy[4] + Am[i * 3 + 1] * Sy[5] + Am[i * 3 + 2] * Sy[2];
            C[i * 3 + 0] = add ? C[i * 3 + 0] + c0 : c0;
            C[i * 3 + 1] = add ? C[i * 3 + 1] + c1 : c1;
            C[i * 3 + 2] = add ? C[i * 3 + 2] + c2 : c2;
          }
        };
        if constexpr (KIND == K_SVK_FUNC) {
#pragma unroll
          for (int i = 0; i < 9; i++) F[i] = Du[i] + ((i % 4 == 0) ? (T)1 : (T)0);
          pk2(F, nullptr, P6);
          gesy(S, F, P6, false);
          if (A.stash) {
#pragma unroll
            for (int i = 0; i < 9; i++) st[i * N3] = F[i];
#pragma unroll
            for (int i = 0; i < 6; i++) st[(9 + i) * N3] = P6[i];
          }
        } else {
#pragma unroll
          for (int i = 0; i < 9; i++) F[i] = st[i * N3];
#pragma unroll
          for (int i = 0; i < 6; i++) P6[i] = st[(9 + i) * N3];
          T dS[6];
          pk2(F, Du, dS);
          gesy(S, F, dS, false);
          gesy(S, Du, P6, true);
        }
#pragma unroll
        for (int i = 0; i < 9; i++) S[i] *= w;
      }
#pragma unroll
      for (int d = 0; d < 3; d++)
#pragma unroll
        for (int k = 0; k < 3; k++) G[(d * 3 + k) * L + t] = S[d * 3 + 0] * Ji[k * 3 + 0] + S[d * 3 + 1] * Ji[k * 3 + 1] + S[d * 3 + 2] * Ji[k * 3 + 2];
    }
    __syncthreads();
    for (int d = 0; d < 3; d++)
      back<N, T, 3>(sm, G + (d * 3 + 0) * L, G + (d * 3 + 1) * L, G + (d * 3 + 2) * L, S0, S1, A, els, first, ne, d, yexp);
  }
}

}  // namespace dgb
