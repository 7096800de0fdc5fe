// BF16 tensor-core element apply (dPREC_BF16) for scalar diffusion-type operators on uniform-order spaces:
// the sum-factorized GRAD / q-function / GRAD_TRANSPOSE of EllipShellMatMult (src/fs/tests/ellip.c:442-472;
// TensorMult_Hex, src/jacobi/impls/tensor/inlinetmulthex.h:19-100) as six tcgen05 MMAs per group of elements, BF16
// operands from shared memory, FP32 accumulation in tensor memory (TMEM).
//
// Each 1-D contraction along a direction is a GEMM whose rows are the element's lines along that direction
// (n^2 lines per element, all lines of E elements stacked into 128-row tiles) and whose K index runs along the
// line. Contractions that share a direction are stacked: the K dimension holds several input blocks and the N
// dimension several output blocks of the same line, with a block matrix of the 1-D tables (B = Lagrange basis at the
// Gauss points, D = its derivative) as the B operand:
//   pass 1 (z):   [u]              -> [B u, D u]                     K = n,  N = 2n
//   pass 2 (y):   [P0 | P1]        -> [B P0, D P0, B P1]             K = 2n, N = 3n
//   pass 3 (x):   [Q0 | Q1 | Q2]   -> [D Q0, B Q1, B Q2] = grad u    K = 3n, N = 3n
//   q-function:   V = G grad u (G = w det J J^-1 k J^-T, 6 BF16 values per point), in registers
//   pass 4 (x^T): [V0 | V1 | V2]   -> [D^T V0, B^T V1, B^T V2]       K = 3n, N = 3n
//   pass 5 (y^T): [R0 | R1 | R2]   -> [B^T R0 + D^T R1, B^T R2]      K = 3n, N = 2n
//   pass 6 (z^T): [S0 | S1]        -> [B^T S0 + D^T S1] = y_e        K = 2n, N = n
// Between passes every thread reads its row (line) from TMEM (tcgen05.ld), rounds to BF16 and scatters the values
// into the next pass's A operand (the lines of the next direction). Shared-memory operands use the no-swizzle K-major
// layout of 8 x 16-byte core matrices (LBO = 128 B between core matrices along K, SBO = (K/8) * 128 B between 8-row
// groups). One thread issues the MMAs and commits them to an mbarrier; every wait is bounded and a timeout sets an
// error flag that the host reads (no trap). One CTA of 256 threads holds 256 TMEM columns (8 tiles x 32) for its
// lifetime and walks element groups in a grid-stride loop.
#include <cuda_bf16.h>
#include <stdint.h>

#include "internal.h"
#include "tcgen05.cuh"

using namespace dgb;

dErr fs_restrict32(_p_dFS *fs, const float *x, double *g, int add);

namespace {

constexpr int kTiles = 8;                  // 128-row tiles per element group
constexpr int kRows = 128 * kTiles;        // rows per group
constexpr int kA16Bytes = kRows * 16 * 2;  // A operand, K = 16 (passes 1, 2, 6)
constexpr int kA32Bytes = kRows * 32 * 2;  // A operand, K = 32 (passes 3, 4, 5)
constexpr int kBBytes = 6 * 32 * 32 * 2;   // B operands of the six passes, padded to N = K = 32
constexpr int kTmemCols = 256;
constexpr int kThreads = 256;
constexpr long long kWaitCycles = 4000000000LL;  // about 2 s at the maximum SM clock

__device__ int g_tc_error;  // 1: an mbarrier wait timed out

// byte offset of (row, k) in a K-major no-swizzle operand with kp columns (kp = 16 or 32) and 128-row tiles
__device__ __forceinline__ uint32_t aoff(int row, int k, int kp) {
  const int t = row >> 7, r = row & 127;
  return (uint32_t)(t * 128 * kp * 2 + (r >> 3) * (kp / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void st_bf16(unsigned char *base, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16 *>(base + off) = __float2bfloat16_rn(v);
}

struct TcArgs {
  int64_t nelem;
  int E;  // elements per group (E n^2 <= kRows)
  const int32_t *emap;
  int64_t n;  // explicit nodes (closure index >= n: homogeneous Dirichlet, 0)
  const double *x;
  const __nv_bfloat16 *geo;  // [nq][6] as 6 SoA planes per element (uniform order: element e at e * 6 n^3)
  const __nv_bfloat16 *bops;  // the six B operands in core-matrix layout, 32 x 32 each
  float *yexp;
};

// issue the MMAs of one pass (thread 0), commit, and let every thread wait for them; false on timeout
__device__ __forceinline__ bool run_pass(uint32_t tmem, uint32_t a_base, int kp, uint32_t b_base, int nout, int ntiles, uint64_t *bar,
                                         uint32_t &phase) {
  async_proxy_fence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x == 0) {
    const uint32_t id = idesc_bf16(nout);
    const uint32_t sbo = (uint32_t)(kp / 8) * 128;
    for (int t = 0; t < ntiles; t++)
      for (int s = 0; s < kp / 16; s++)
        mma_bf16(tmem + (uint32_t)(t * 32), sdesc(a_base + (uint32_t)(t * 128 * kp * 2 + s * 256), 128, sbo),
                 sdesc(b_base + (uint32_t)(s * 256), 128, 4 * 128), id, s > 0);
    mma_commit(bar);
  }
  const bool mine = mbar_wait(bar, phase, kWaitCycles, &g_tc_error);
  phase ^= 1u;
  const bool ok = __syncthreads_and(mine) != 0;  // every thread leaves with the same verdict
  tc_fence_after();
  return ok;
}

// this thread's row values of tile t from TMEM: ncol (16 or 32) columns
__device__ __forceinline__ void read_row(uint32_t tmem, int t, int ncol, float *v) {
  const uint32_t lane = (uint32_t)((threadIdx.x >> 5) & 3) * 32;
  const uint32_t addr = tmem + (lane << 16) + (uint32_t)(t * 32);
  tmem_ld16(addr, v);
  if (ncol > 16) tmem_ld16(addr + 16, v + 16);
  tmem_wait_ld();
}

template <int N>
__global__ void __launch_bounds__(kThreads, 1) k_tc_diffusion(TcArgs A) {
  constexpr int NN = N * N, N3 = NN * N;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *a16 = smem, *a32 = smem + kA16Bytes, *bsm = smem + kA16Bytes + kA32Bytes;
  uint64_t *bar = reinterpret_cast<uint64_t *>(bsm + kBBytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bsm + kBBytes + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
  // zero the operand buffers (finite values in every padding row and column), load the B operands
  for (int i = tid; i < (kA16Bytes + kA32Bytes) / 16; i += kThreads) reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
  for (int i = tid; i < kBBytes / 16; i += kThreads) reinterpret_cast<uint4 *>(bsm)[i] = reinterpret_cast<const uint4 *>(A.bops)[i];
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t A16 = smem_u32(a16), A32 = smem_u32(a32), Bs = smem_u32(bsm);
  uint32_t phase = 0;
  const int E = A.E, rows = E * NN, ntiles = (rows + 127) / 128;
  const int lg = warp & 3, tp = warp >> 2;  // TMEM lane group; tile parity of this warp
  bool ok = true;
  for (int64_t g0 = (int64_t)blockIdx.x * E; g0 < A.nelem && ok; g0 += (int64_t)gridDim.x * E) {
    const int ne = (int)min((int64_t)E, A.nelem - g0);
    // pass 1 input: rows (e, i, j) = z-lines, K = k; gathered nodal values (homogeneous Dirichlet)
    for (int t = tid; t < ne * N3; t += kThreads) {
      const int e = t / N3, r = t - e * N3, ij = r / N, k = r - ij * N;
      const int32_t c = A.emap[(g0 + e) * N3 + r];
      const double v = c < A.n ? A.x[c] : 0.0;
      st_bf16(a16, aoff(e * NN + ij, k, 16), (float)v);
    }
    if (!(ok = run_pass(tmem, A16, 16, Bs + 0 * 2048, 2 * N <= 16 ? 16 : 32, ntiles, bar, phase))) break;
    float v[32];
    // pass 1 -> 2: row (e,i,j) holds [B u, D u](k'); pass 2 rows (e, i, k'), K = b n + j
    for (int t = tp; t < ntiles; t += 2) {
      const int row = t * 128 + lg * 32 + (tid & 31);
      read_row(tmem, t, 2 * N <= 16 ? 16 : 32, v);
      if (row >= ne * NN) continue;
      const int e = row / NN, ij = row - e * NN, i = ij / N, j = ij - i * N;
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int k = 0; k < N; k++) st_bf16(a16, aoff(e * NN + i * N + k, b * N + j, 16), v[b * N + k]);
    }
    if (!(ok = run_pass(tmem, A16, 16, Bs + 1 * 2048, 32, ntiles, bar, phase))) break;
    // pass 2 -> 3: row (e,i,k) holds [Q0, Q1, Q2](j); pass 3 rows (e, j, k), K = b n + i
    for (int t = tp; t < ntiles; t += 2) {
      const int row = t * 128 + lg * 32 + (tid & 31);
      read_row(tmem, t, 32, v);
      if (row >= ne * NN) continue;
      const int e = row / NN, ik = row - e * NN, i = ik / N, k = ik - i * N;
#pragma unroll
      for (int b = 0; b < 3; b++)
#pragma unroll
        for (int j = 0; j < N; j++) st_bf16(a32, aoff(e * NN + j * N + k, b * N + i, 32), v[b * N + j]);
    }
    if (!(ok = run_pass(tmem, A32, 32, Bs + 2 * 2048, 32, ntiles, bar, phase))) break;
    // pass 3: row (e,j,k) holds the reference gradient (Gx, Gy, Gz)(i); q-function; pass 4 input on the same row
    for (int t = tp; t < ntiles; t += 2) {
      const int row = t * 128 + lg * 32 + (tid & 31);
      read_row(tmem, t, 32, v);
      if (row >= ne * NN) continue;
      const int e = row / NN, jk = row - e * NN;
      const __nv_bfloat16 *G = A.geo + (g0 + e) * 6 * N3 + jk;
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int q = i * NN;
        const float g0v = v[i], g1v = v[N + i], g2v = v[2 * N + i];
        const float a0 = __bfloat162float(G[q]), a1 = __bfloat162float(G[N3 + q]), a2 = __bfloat162float(G[2 * N3 + q]);
        const float a3 = __bfloat162float(G[3 * N3 + q]), a4 = __bfloat162float(G[4 * N3 + q]), a5 = __bfloat162float(G[5 * N3 + q]);
        st_bf16(a32, aoff(row, i, 32), a0 * g0v + a1 * g1v + a2 * g2v);
        st_bf16(a32, aoff(row, N + i, 32), a1 * g0v + a3 * g1v + a4 * g2v);
        st_bf16(a32, aoff(row, 2 * N + i, 32), a2 * g0v + a4 * g1v + a5 * g2v);
      }
    }
    if (!(ok = run_pass(tmem, A32, 32, Bs + 3 * 2048, 32, ntiles, bar, phase))) break;
    // pass 4 -> 5: row (e,j,k) holds [R0, R1, R2](i); pass 5 rows (e, i, k), K = b n + j
    for (int t = tp; t < ntiles; t += 2) {
      const int row = t * 128 + lg * 32 + (tid & 31);
      read_row(tmem, t, 32, v);
      if (row >= ne * NN) continue;
      const int e = row / NN, jk = row - e * NN, j = jk / N, k = jk - j * N;
#pragma unroll
      for (int b = 0; b < 3; b++)
#pragma unroll
        for (int i = 0; i < N; i++) st_bf16(a32, aoff(e * NN + i * N + k, b * N + j, 32), v[b * N + i]);
    }
    if (!(ok = run_pass(tmem, A32, 32, Bs + 4 * 2048, 2 * N <= 16 ? 16 : 32, ntiles, bar, phase))) break;
    // pass 5 -> 6: row (e,i,k) holds [S0, S1](j); pass 6 rows (e, i, j), K = b n + k
    for (int t = tp; t < ntiles; t += 2) {
      const int row = t * 128 + lg * 32 + (tid & 31);
      read_row(tmem, t, 2 * N <= 16 ? 16 : 32, v);
      if (row >= ne * NN) continue;
      const int e = row / NN, ik = row - e * NN, i = ik / N, k = ik - i * N;
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int j = 0; j < N; j++) st_bf16(a16, aoff(e * NN + i * N + j, b * N + k, 16), v[b * N + j]);
    }
    if (!(ok = run_pass(tmem, A16, 16, Bs + 5 * 2048, 16, ntiles, bar, phase))) break;
    // pass 6: row (e,i,j) holds y(k): the element's expanded output, FP32
    for (int t = tp; t < ntiles; t += 2) {
      const int row = t * 128 + lg * 32 + (tid & 31);
      read_row(tmem, t, 16, v);
      if (row >= ne * NN) continue;
      const int e = row / NN, ij = row - e * NN;
      float *y = A.yexp + (g0 + e) * N3 + ij * N;
#pragma unroll
      for (int k = 0; k < N; k++) y[k] = v[k];
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
  // every MMA this CTA issued has completed (each pass waited for its commit, or gave up after the timeout)
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// host: the six B operands (N x K, K-major, core-matrix layout, 32 x 32 BF16 each) from the 1-D tables
void build_bops(int n, const double *Bq, const double *Dq, std::vector<__nv_bfloat16> &out) {
  out.assign(6 * 32 * 32, __float2bfloat16(0.f));
  auto put = [&](int pass, int nrow, int kcol, double v) {
    const int off = (nrow >> 3) * 4 * 64 + (kcol >> 3) * 64 + (nrow & 7) * 8 + (kcol & 7);  // elements, SBO = 4 core matrices
    out[pass * 1024 + off] = __float2bfloat16((float)v);
  };
  auto B = [&](int q, int p) { return Bq[q * n + p]; };
  auto D = [&](int q, int p) { return Dq[q * n + p]; };
  for (int o = 0; o < n; o++)
    for (int i = 0; i < n; i++) {
      put(0, o, i, B(o, i));          // pass 1: [B u, D u]
      put(0, n + o, i, D(o, i));
      put(1, o, i, B(o, i));          // pass 2: [B P0, D P0, B P1]
      put(1, n + o, i, D(o, i));
      put(1, 2 * n + o, n + i, B(o, i));
      put(2, o, i, D(o, i));          // pass 3: [D Q0, B Q1, B Q2]
      put(2, n + o, n + i, B(o, i));
      put(2, 2 * n + o, 2 * n + i, B(o, i));
      put(3, o, i, D(i, o));          // pass 4: [D^T V0, B^T V1, B^T V2]
      put(3, n + o, n + i, B(i, o));
      put(3, 2 * n + o, 2 * n + i, B(i, o));
      put(4, o, i, B(i, o));          // pass 5: [B^T R0 + D^T R1, B^T R2]
      put(4, o, n + i, D(i, o));
      put(4, n + o, 2 * n + i, B(i, o));
      put(5, o, i, B(i, o));          // pass 6: B^T S0 + D^T S1
      put(5, o, n + i, D(i, o));
    }
}

template <int N>
dErr launch_tc(_p_dFS *fs, const double *x, const __nv_bfloat16 *geo, const __nv_bfloat16 *bops, float *yexp) {
  TcArgs A{};
  A.nelem = fs->nelem;
  A.E = kRows / (N * N);
  A.emap = fs->d_emap;
  A.n = fs->n;
  A.x = x;
  A.geo = geo;
  A.bops = bops;
  A.yexp = yexp;
  const size_t smem = (size_t)kA16Bytes + kA32Bytes + kBBytes + 64;
  CUCHK(cudaFuncSetAttribute(k_tc_diffusion<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int dev = 0, nsm = 0;
  CUCHK(cudaGetDevice(&dev));
  CUCHK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t groups = (fs->nelem + A.E - 1) / A.E;
  const int grid = (int)std::min<int64_t>(groups, 2LL * nsm);
  k_tc_diffusion<N><<<grid, kThreads, smem, fs->stream>>>(A);
  CUCHK(cudaGetLastError());
  return 0;
}

}  // namespace

// y = A x with BF16 tensor-core contractions (FP32 accumulation), BF16 geometric factors, FP64 restriction. geo16: the
// operator's BF16 factors [nq * 6]; tables: the FP64 1-D tables of degree p (B and D at the Gauss points, [n][n] each)
dErr tc_diffusion_apply(_p_dFS *fs, const double *x, const void *geo16, void **bops_cache, float *yexp, double *y) {
  if (!fs->uniform || fs->bs != 1 || !fs->boolean_e) return set_error("tensor-core apply: scalar uniform-order spaces");
  const int n = fs->p + 1;
  if (n < 2 || n > 8) return set_error("tensor-core apply: degree %d outside 1..7", fs->p);
  if (!*bops_cache) {
    Basis1D b;
    DCHK(make_basis(fs->p, dQUADRATURE_METHOD_FAST, &b));
    std::vector<__nv_bfloat16> h;
    build_bops(n, b.B, b.D, h);
    CUCHK(cudaMalloc(bops_cache, h.size() * sizeof(__nv_bfloat16)));
    CUCHK(cudaMemcpy(*bops_cache, h.data(), h.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice));
  }
  const __nv_bfloat16 *bops = (const __nv_bfloat16 *)*bops_cache;
  const __nv_bfloat16 *g = (const __nv_bfloat16 *)geo16;
  int zero = 0;
  CUCHK(cudaMemcpyToSymbolAsync(g_tc_error, &zero, sizeof zero, 0, cudaMemcpyHostToDevice, fs->stream));
  switch (n) {
    case 2: DCHK(launch_tc<2>(fs, x, g, bops, yexp)); break;
    case 3: DCHK(launch_tc<3>(fs, x, g, bops, yexp)); break;
    case 4: DCHK(launch_tc<4>(fs, x, g, bops, yexp)); break;
    case 5: DCHK(launch_tc<5>(fs, x, g, bops, yexp)); break;
    case 6: DCHK(launch_tc<6>(fs, x, g, bops, yexp)); break;
    case 7: DCHK(launch_tc<7>(fs, x, g, bops, yexp)); break;
    case 8: DCHK(launch_tc<8>(fs, x, g, bops, yexp)); break;
  }
  return fs_restrict32(fs, yexp, y, 0);
}

// the error flag of the last tensor-core apply (a bounded wait gave up); synchronizes the stream
dErr tc_check(_p_dFS *fs) {
  int err = 0;
  CUCHK(cudaMemcpyFromSymbolAsync(&err, g_tc_error, sizeof err, 0, cudaMemcpyDeviceToHost, fs->stream));
  CUCHK(cudaStreamSynchronize(fs->stream));
  if (err) return set_error("tensor-core apply: an mbarrier wait timed out");
  return 0;
}
