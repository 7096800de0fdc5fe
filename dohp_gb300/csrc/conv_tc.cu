// 3 x 3 x 3 convolutions of the learned correction's U-Net on the 5th-generation tensor cores (tcgen05): stride 1,
// zero padding, 16 or 32 input and output channels, BF16 operands, FP32 accumulation in tensor memory. The same
// kernel computes the data gradient of such a layer (the convolution with the kernel flipped in all three offsets
// and the channel roles swapped), with its weights packed the other way round; a second kernel (below) computes the
// layer's weight gradient as GEMMs over the output voxels.
//
// Implicit GEMM: an output tile of 4 (x) x 16 (y) x 16 (z) voxels is eight M = 128 tiles (16 y-rows x 8 z at one x);
// N = output channels; K = input channels, one MMA of K = 16 per tap and 16-channel step, 27 taps accumulated in TMEM.
// The input halo (6 x 18 x 18 voxels) is staged once per tile in shared memory, converted from the FP32 activations to
// BF16, as K-major no-swizzle core matrices: one plane per 8 channels, 16 bytes per voxel, z fastest. A tap's A
// operand is the same halo read at a shifted start address: 8 consecutive z voxels are one core matrix (16-byte rows),
// 8-row groups step by one y-row (SBO = 18 x 16 B), and channel planes step by LBO = the plane size. Every address an
// MMA reads lies inside the halo: x in [tx + a], y in [b, b + 15], z in [8 zh + c, 8 zh + c + 7] with tx <= 3 and
// a, b, c <= 2, zh <= 1.
//
// One thread issues the MMAs of a tile and commits them to an mbarrier; every wait is bounded by a clock limit,
// after which the kernel records an error that the host reads and frees its TMEM (no trap).
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>

#include "internal.h"
#include "tcgen05.cuh"

using namespace dgb;

namespace {

constexpr int TX = 4, TY = 16, TZ = 16;                 // output tile
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;    // input halo
constexpr int kHalo = HX * HY * HZ;                     // voxels
constexpr int kPlane = kHalo * 16;                      // bytes per 8-channel plane
constexpr int kMTiles = (TX * TY * TZ) / 128;           // 8
constexpr int kThreads = 256;
constexpr long long kWaitCycles = 4000000000LL;         // about 2 s at the maximum SM clock

__device__ int g_conv_error;  // 1: an mbarrier wait timed out

template <int CI, int CO>
struct ConvShape {
  static constexpr int a_bytes = CI / 8 * kPlane, w_bytes = 27 * CI * CO * 2, smem = a_bytes + w_bytes + 64;
  static constexpr int tmem = kMTiles * CO;  // 128 or 256 columns
};

struct ConvArgs {
  int B, dx, dy, dz;
  int ntx, nty, ntz;
  int64_t ntiles;
  const float *x;             // [B][CI][d]
  const __nv_bfloat16 *w;     // packed B operands [27][CI/16][2][CO][8]
  const float *bias;          // [CO] or null
  int relu, accumulate;
  float *y;                   // [B][CO][d]
};

template <int CI, int CO>
__global__ void __launch_bounds__(kThreads, 1) k_conv3_tc(ConvArgs A) {
  using S = ConvShape<CI, CO>;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *asm_ = smem, *wsm = smem + S::a_bytes;
  uint64_t *bar = reinterpret_cast<uint64_t *>(wsm + S::w_bytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(wsm + S::w_bytes + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < S::w_bytes / 16; i += kThreads) reinterpret_cast<uint4 *>(wsm)[i] = reinterpret_cast<const uint4 *>(A.w)[i];
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(S::tmem));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot, Abase = smem_u32(asm_), Wbase = smem_u32(wsm);
  const int64_t nv = (int64_t)A.dx * A.dy * A.dz;
  const int lg = warp & 3, half = warp >> 2;  // TMEM lane group; which four M-tiles this warp reads back
  uint32_t phase = 0;
  for (int64_t tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
    int64_t r = tile;
    const int tz = (int)(r % A.ntz);
    r /= A.ntz;
    const int ty = (int)(r % A.nty);
    r /= A.nty;
    const int tx = (int)(r % A.ntx);
    const int b = (int)(r / A.ntx);
    const int x0 = tx * TX, y0 = ty * TY, z0 = tz * TZ;
    // stage the halo: plane q holds channels 8q..8q+7 of every halo voxel as 8 BF16 values (zero outside the lattice);
    // each thread loads four items (32 independent loads) before it converts and stores them
    const float *xb = A.x + (int64_t)b * CI * nv;
    constexpr int kItems = CI / 8 * kHalo, kU = 4;
    for (int it0 = tid; it0 < kItems; it0 += kU * kThreads) {
      float v[kU][8];
      bool in[kU];
#pragma unroll
      for (int u = 0; u < kU; u++) {
        const int it = it0 + u * kThreads;
        const int q = it / kHalo, h = it - q * kHalo;
        const int hx = h / (HY * HZ), hy = (h / HZ) % HY, hz = h % HZ;
        const int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z0 + hz - 1;
        in[u] = it < kItems && gx >= 0 && gx < A.dx && gy >= 0 && gy < A.dy && gz >= 0 && gz < A.dz;
        const float *src = xb + (int64_t)q * 8 * nv + ((int64_t)gx * A.dy + gy) * A.dz + gz;
#pragma unroll
        for (int c = 0; c < 8; c++) v[u][c] = in[u] ? src[(int64_t)c * nv] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < kU; u++) {
        const int it = it0 + u * kThreads;
        if (it >= kItems) break;
        const int q = it / kHalo, h = it - q * kHalo;
        __nv_bfloat162 p0 = __floats2bfloat162_rn(v[u][0], v[u][1]), p1 = __floats2bfloat162_rn(v[u][2], v[u][3]);
        __nv_bfloat162 p2 = __floats2bfloat162_rn(v[u][4], v[u][5]), p3 = __floats2bfloat162_rn(v[u][6], v[u][7]);
        *reinterpret_cast<uint4 *>(asm_ + q * kPlane + h * 16) =
            make_uint4(*reinterpret_cast<uint32_t *>(&p0), *reinterpret_cast<uint32_t *>(&p1), *reinterpret_cast<uint32_t *>(&p2),
                       *reinterpret_cast<uint32_t *>(&p3));
      }
    }
    async_proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      const uint32_t id = idesc_bf16(CO);
#pragma unroll 1
      for (int mt = 0; mt < kMTiles; mt++) {
        const int mx = mt >> 1, zh = mt & 1;
#pragma unroll 1
        for (int tap = 0; tap < 27; tap++) {
          const int a = tap / 9, bb = (tap / 3) % 3, c = tap % 3;
          const uint32_t aoff = (uint32_t)((((mx + a) * HY + bb) * HZ + zh * 8 + c) * 16);
#pragma unroll
          for (int s = 0; s < CI / 16; s++)
            mma_bf16(tmem + (uint32_t)(mt * CO), sdesc(Abase + (uint32_t)(2 * s * kPlane) + aoff, kPlane, HZ * 16),
                     sdesc(Wbase + (uint32_t)((tap * (CI / 16) + s) * 2 * CO * 16), CO * 16, 128), id, (tap | s) != 0);
        }
      }
      mma_commit(bar);
    }
    const bool mine = mbar_wait(bar, phase, kWaitCycles, &g_conv_error);
    phase ^= 1u;
    if (!__syncthreads_and(mine)) break;  // every thread leaves with the same verdict
    tc_fence_after();
    // read back: row lg*32 + lane of M-tile mt is voxel (x0 + mt/2, y0 + row/8, z0 + 8 (mt%2) + row%8)
    const int row = lg * 32 + lane, oy = y0 + (row >> 3);
    float *yb = A.y + (int64_t)b * CO * nv;
#pragma unroll 1
    for (int k = 0; k < kMTiles / 2; k++) {
      const int mt = half * (kMTiles / 2) + k;
      const int ox = x0 + (mt >> 1), oz = z0 + (mt & 1) * 8 + (row & 7);
      float v[CO];
#pragma unroll
      for (int c0 = 0; c0 < CO; c0 += 16) tmem_ld16(tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(mt * CO + c0), v + c0);
      tmem_wait_ld();
      if (ox >= A.dx || oy >= A.dy || oz >= A.dz) continue;
      float *yo = yb + ((int64_t)ox * A.dy + oy) * A.dz + oz;
#pragma unroll
      for (int c = 0; c < CO; c++) {
        float o = v[c] + (A.bias ? A.bias[c] : 0.f);
        if (A.relu) o = fmaxf(o, 0.f);
        float *p = yo + (int64_t)c * nv;
        *p = A.accumulate ? *p + o : o;
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::tmem));
}

// B operands of a layer from W [co][ci][27] (BF16): element (n, k) of tap t, 16-channel step s at
// [((t (K/16) + s) 2 + (k%16)/8) N + n] 8 + k%8 with N x K = CO x CI (forward) or CI x CO with the taps flipped
// (t -> 26 - t: the data gradient)
__global__ void k_pack_conv(int ci, int co, int transpose, const __nv_bfloat16 *__restrict__ W, __nv_bfloat16 *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 27 * ci * co) return;
  const int t = i / (ci * co), rest = i % (ci * co), o = rest / ci, c = rest % ci;  // W[o][c][tap] read as (tap, o, c)
  const __nv_bfloat16 w = W[((size_t)o * ci + c) * 27 + t];
  int n, k, tap, K, N;
  if (!transpose) n = o, k = c, tap = t, K = ci, N = co;
  else n = c, k = o, tap = 26 - t, K = co, N = ci;
  out[((size_t)((tap * (K / 16) + k / 16) * 2 + (k % 16) / 8) * N + n) * 8 + k % 8] = w;
}

template <int CI, int CO>
dErr launch(const ConvArgs &A, cudaStream_t s) {
  using S = ConvShape<CI, CO>;
  CUCHK(cudaFuncSetAttribute(k_conv3_tc<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::smem));
  int dev = 0, nsm = 0;
  CUCHK(cudaGetDevice(&dev));
  CUCHK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int per_sm = S::smem <= 110 * 1024 ? 2 : 1;  // CTAs an SM holds by shared memory; their TMEM fits 512 columns
  const int grid = (int)std::min<int64_t>(A.ntiles, (int64_t)per_sm * nsm);
  k_conv3_tc<CI, CO><<<grid, kThreads, S::smem, s>>>(A);
  CUCHK(cudaGetLastError());
  return 0;
}


// ---------------------------------------------------------------------------------------------- weight gradient
// dW[co][ci][t] = sum_b sum_v gy[b][co][v] x[b][ci][v + (dx - 1, dy - 1, dz - 1)], t = (dx 3 + dy) 3 + dz, as GEMMs
// with K = the output voxels of a 2 (x) x 8 (y) x 16 (z) tile (one MMA per y-line pair of z-octets, K = 16):
//   A (M = 128 rows, 3 CI of them used): row dz CI + ci = x[ci] at the voxels shifted by dz along z, staged once per
//     tile for every (hx, hy) of the 4 x 10 halo as [z-octet][dz][ci][8 voxels] (the three z-shifted copies
//     interleaved, so the rows of one octet are 16 bytes apart: SBO = 128 B, LBO = 3 CI 16 B to the next z-octet);
//     rows 3 CI..127 read the next octets' values and land in accumulator rows that are never read;
//   B (N = CO rows): gy at the tile's voxels as [z-octet][co][8 voxels] (SBO = 128 B, LBO = CO 16 B);
//   D: one accumulator per (dx, dy) in TMEM (9 CO columns), summed over every tile the CTA takes; (dx, dy) moves the
//     A start address by whole octets.
// The CTA's sums go to partial[blockIdx.x][CO CI 27 + CO] (the bias gradient, sum of gy, on the CUDA cores in FP32),
// summed over CTAs in order afterwards (deterministic).
constexpr int WX = 2, WY = 8, WZ = 16;                  // output tile
constexpr int WHX = WX + 2, WHY = WY + 2, WOCT = WZ / 8;  // x halo, octets per z-line
constexpr int kWMMA = 9;                                 // accumulators (dx, dy)

template <int CI, int CO>
struct WShape {
  static constexpr int xoct = WHX * WHY * WOCT;                  // staged x octets
  static constexpr int x_bytes = xoct * 3 * CI * 16 + 2048;     // + the rows past the last octet that M = 128 reads
  static constexpr int g_bytes = WX * WY * WOCT * CO * 16;
  static constexpr int smem = x_bytes + g_bytes + 64;
  static constexpr int tmem = kWMMA * CO <= 256 ? 256 : 512;
};

struct WArgs {
  int B, dx, dy, dz;
  int ntx, nty, ntz;
  int64_t ntiles;
  const float *x, *gy;
  float *partial;
  int64_t np;  // CO CI 27 + CO
};

template <int CI, int CO>
__global__ void __launch_bounds__(kThreads, 1) k_conv3_wgrad_tc(WArgs A) {
  using S = WShape<CI, CO>;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *xs = smem, *gs = smem + S::x_bytes;
  uint64_t *bar = reinterpret_cast<uint64_t *>(gs + S::g_bytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(gs + S::g_bytes + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < S::x_bytes / 16; i += kThreads) reinterpret_cast<uint4 *>(xs)[i] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(S::tmem));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot, Xb = smem_u32(xs), Gb = smem_u32(gs);
  const int64_t nv = (int64_t)A.dx * A.dy * A.dz;
  float bsum[CO];  // this thread's share of the bias gradient, per output channel
#pragma unroll
  for (int c = 0; c < CO; c++) bsum[c] = 0.f;
  uint32_t phase = 0;
  bool ok = true, first = true;
  for (int64_t tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
    int64_t r = tile;
    const int tz = (int)(r % A.ntz);
    r /= A.ntz;
    const int ty = (int)(r % A.nty);
    r /= A.nty;
    const int tx = (int)(r % A.ntx);
    const int b = (int)(r / A.ntx);
    const int x0 = tx * WX, y0 = ty * WY, z0 = tz * WZ;
    // x: element e = ((((ci 3 + dz) WHX + hx) WHY + hy) WZ + z), z = 8 octet + k: x[ci][x0 + hx - 1][y0 + hy - 1][z0 + z + dz - 1]
    const float *xb = A.x + (int64_t)b * CI * nv;
    for (int e = tid; e < CI * 3 * WHX * WHY * WZ; e += kThreads) {
      const int z = e % WZ, hy = (e / WZ) % WHY, hx = (e / (WZ * WHY)) % WHX, dz = (e / (WZ * WHY * WHX)) % 3;
      const int ci = e / (WZ * WHY * WHX * 3);
      const int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z0 + z + dz - 1;
      float v = 0.f;
      if (gx >= 0 && gx < A.dx && gy >= 0 && gy < A.dy && gz >= 0 && gz < A.dz) v = xb[(int64_t)ci * nv + ((int64_t)gx * A.dy + gy) * A.dz + gz];
      const int oct = (hx * WHY + hy) * WOCT + (z >> 3);
      *reinterpret_cast<__nv_bfloat16 *>(xs + oct * (3 * CI * 16) + (dz * CI + ci) * 16 + (z & 7) * 2) = __float2bfloat16_rn(v);
    }
    // gy: element e = ((co WX + ox) WY + oy) WZ + z; the bias sums in FP32 (co is the same for a thread's elements of
    // one pass over e: kThreads is a multiple of WX WY WZ)
    const float *gb = A.gy + (int64_t)b * CO * nv;
#pragma unroll
    for (int co = 0; co < CO; co++)
      for (int e = tid; e < WX * WY * WZ; e += kThreads) {
        const int z = e % WZ, oy = (e / WZ) % WY, ox = e / (WZ * WY);
        const int gx = x0 + ox, gy = y0 + oy, gz = z0 + z;
        float v = 0.f;
        if (gx < A.dx && gy < A.dy && gz < A.dz) v = gb[(int64_t)co * nv + ((int64_t)gx * A.dy + gy) * A.dz + gz];
        bsum[co] += v;
        const int oct = (ox * WY + oy) * WOCT + (z >> 3);
        *reinterpret_cast<__nv_bfloat16 *>(gs + oct * (CO * 16) + co * 16 + (z & 7) * 2) = __float2bfloat16_rn(v);
      }
    async_proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      const uint32_t id = idesc_bf16(CO);
#pragma unroll 1
      for (int g = 0; g < kWMMA; g++) {
        const int ddx = g / 3, ddy = g % 3;
#pragma unroll 1
        for (int line = 0; line < WX * WY; line++) {
          const int ox = line / WY, oy = line % WY;
          const uint32_t aoff = (uint32_t)(((ox + ddx) * WHY + oy + ddy) * WOCT * (3 * CI * 16));
          const uint32_t boff = (uint32_t)(line * WOCT * (CO * 16));
          mma_bf16(tmem + (uint32_t)(g * CO), sdesc(Xb + aoff, 3 * CI * 16, 128), sdesc(Gb + boff, CO * 16, 128), id,
                   !(first && line == 0));
        }
      }
      mma_commit(bar);
    }
    first = false;
    const bool mine = mbar_wait(bar, phase, kWaitCycles, &g_conv_error);
    phase ^= 1u;
    if (!(ok = __syncthreads_and(mine) != 0)) break;
    tc_fence_after();
  }
  // the CTA's sums: accumulator row dz CI + ci (lanes 0..3 CI - 1), column (dx 3 + dy) CO + co
  float *pp = A.partial + (int64_t)blockIdx.x * A.np;
  if (ok && !first) {
    const int lg = warp & 3, half = warp >> 2;
    const int row = lg * 32 + lane;
#pragma unroll 1
    for (int g = half; g < kWMMA; g += 2) {
      float v[CO];
#pragma unroll
      for (int c0 = 0; c0 < CO; c0 += 16) tmem_ld16(tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(g * CO + c0), v + c0);
      tmem_wait_ld();
      if (row < 3 * CI) {
        const int dz = row / CI, ci = row % CI, t = g * 3 + dz;
#pragma unroll
        for (int co = 0; co < CO; co++) pp[((int64_t)co * CI + ci) * 27 + t] = v[co];
      }
    }
  } else {  // no tile (or a timed-out wait, which the host reads as an error): no contribution
    for (int i = tid; i < CO * CI * 27; i += kThreads) pp[i] = 0.f;
  }
  // bias: the threads' sums per channel, reduced in a fixed order (warp shuffles, then the warps in order)
  __shared__ float red[kThreads / 32][32];
#pragma unroll 1
  for (int co = 0; co < CO; co++) {
    float v = bsum[co];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][co] = v;
  }
  __syncthreads();
  if (tid < CO) {
    float v = 0.f;
    for (int w = 0; w < kThreads / 32; w++) v += red[w][tid];
    pp[(int64_t)CO * CI * 27 + tid] = v;
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::tmem));
}

template <int CI, int CO>
dErr launch_wgrad(WArgs &A, int64_t max_ctas, int *nchunks, cudaStream_t s) {
  using S = WShape<CI, CO>;
  CUCHK(cudaFuncSetAttribute(k_conv3_wgrad_tc<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::smem));
  int dev = 0, nsm = 0;
  CUCHK(cudaGetDevice(&dev));
  CUCHK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>({A.ntiles, (int64_t)nsm, max_ctas}));
  k_conv3_wgrad_tc<CI, CO><<<grid, kThreads, S::smem, s>>>(A);
  CUCHK(cudaGetLastError());
  *nchunks = grid;
  return 0;
}

}  // namespace

// the layer shapes the tensor-core path takes
bool conv_tc_supported(int ci, int co) { return (ci == 16 || ci == 32) && (co == 16 || co == 32); }

// packed B operands (27 ci co BF16 values) of a layer's weights W [co][ci][27], forward or for the data gradient
dErr conv_tc_pack(int ci, int co, bool transpose, const __nv_bfloat16 *W, __nv_bfloat16 *out, cudaStream_t s) {
  if (!conv_tc_supported(ci, co)) return set_error("tensor-core convolution: %d -> %d channels", ci, co);
  const int n = 27 * ci * co;
  k_pack_conv<<<(n + 255) / 256, 256, 0, s>>>(ci, co, transpose ? 1 : 0, W, out);
  CUCHK(cudaGetLastError());
  return 0;
}

// y (=, or += with accumulate) act(conv3(x) + bias), stride 1, zero padding; x [B][ci][d], y [B][co][d] FP32;
// wpack from conv_tc_pack (for the data gradient: ci and co are the gradient's input and output channels)
dErr conv_tc(int B, int ci, int co, const int d[3], const float *x, const __nv_bfloat16 *wpack, const float *bias, int relu,
             int accumulate, float *y, cudaStream_t s) {
  if (!conv_tc_supported(ci, co)) return set_error("tensor-core convolution: %d -> %d channels", ci, co);
  ConvArgs A{};
  A.B = B, A.dx = d[0], A.dy = d[1], A.dz = d[2];
  A.ntx = (d[0] + TX - 1) / TX, A.nty = (d[1] + TY - 1) / TY, A.ntz = (d[2] + TZ - 1) / TZ;
  A.ntiles = (int64_t)B * A.ntx * A.nty * A.ntz;
  A.x = x, A.w = wpack, A.bias = bias, A.relu = relu, A.accumulate = accumulate, A.y = y;
  if (ci == 16 && co == 16) return launch<16, 16>(A, s);
  if (ci == 16 && co == 32) return launch<16, 32>(A, s);
  if (ci == 32 && co == 16) return launch<32, 16>(A, s);
  return launch<32, 32>(A, s);
}

// weight and bias gradient partial sums of a stride-1 layer on the tensor cores: partial[c][co ci 27 + co] for
// c < *nchunks (at most max_chunks), to be summed over c in order; x [B][ci][d], gy [B][co][d] FP32
dErr conv_tc_wgrad(int B, int ci, int co, const int d[3], const float *x, const float *gy, float *partial, int64_t max_chunks,
                   int *nchunks, cudaStream_t s) {
  if (!conv_tc_supported(ci, co)) return set_error("tensor-core convolution: %d -> %d channels", ci, co);
  if (max_chunks < 1) return set_error("tensor-core weight gradient: no room for partial sums");
  WArgs A{};
  A.B = B, A.dx = d[0], A.dy = d[1], A.dz = d[2];
  A.ntx = (d[0] + WX - 1) / WX, A.nty = (d[1] + WY - 1) / WY, A.ntz = (d[2] + WZ - 1) / WZ;
  A.ntiles = (int64_t)B * A.ntx * A.nty * A.ntz;
  A.x = x, A.gy = gy, A.partial = partial, A.np = (int64_t)co * ci * 27 + co;
  if (ci == 16 && co == 16) return launch_wgrad<16, 16>(A, max_chunks, nchunks, s);
  if (ci == 16 && co == 32) return launch_wgrad<16, 32>(A, max_chunks, nchunks, s);
  if (ci == 32 && co == 16) return launch_wgrad<32, 16>(A, max_chunks, nchunks, s);
  return launch_wgrad<32, 32>(A, max_chunks, nchunks, s);
}

// 1 when a tensor-core convolution gave up waiting for its MMAs since the last call (the flag is cleared)
dErr conv_tc_check(cudaStream_t s) {
  int e = 0, zero = 0;
  CUCHK(cudaMemcpyFromSymbolAsync(&e, g_conv_error, sizeof e, 0, cudaMemcpyDeviceToHost, s));
  CUCHK(cudaMemcpyToSymbolAsync(g_conv_error, &zero, sizeof zero, 0, cudaMemcpyHostToDevice, s));
  CUCHK(cudaStreamSynchronize(s));
  if (e) return set_error("tensor-core convolution: an MMA wait timed out");
  return 0;
}
