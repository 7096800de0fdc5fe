// Learned coarse correction for the Q1-embedded Chebyshev-Jacobi preconditioner (no counterpart in the
// reference; the preconditioner it augments is the one EllipJacobian assembles, ellip.c:474-536).
//
// A 3-level 3-D convolutional U-Net (16/32/64 channels, 3x3x3 kernels, BF16 weights, FP32 accumulation) runs on one
// of two lattices. The vertex lattice (the coarsest level of the embedded Q1 hierarchy): input channels R r
// (R = P^T, normalised by its RMS over interior vertices) and log k at the vertices, output the error at the
// vertices, which P (trilinear interpolation of the vertex lattice onto every GLL node, element by element) carries
// back to the global dofs. Or the GLL-node lattice of the Q1-embedded matrix itself ((M p + 1) nodes per direction):
// R and P are then the injection of the explicit dofs, and the network is trained on windows of the lattice (the
// recorded pairs are cut to crop^3 windows at seeded origins that are multiples of 4, so the coarse levels of a
// window line up with those of the whole lattice) and applied to the whole lattice. FGMRES uses
// z = Chebyshev(r) + P N(R r).
//
// Training pairs (residual, error) come from the plain solver: a CG monitor records R r_k and x_k on the lattice
// (or its window); once the solve has converged, the targets are x* - x_k there. Training is plain minibatch Adam on
// the mean squared error over interior nodes, with hand-written forward and backward kernels: the stride-1
// convolutions of 16 / 32 channels with their data and weight gradients on the tcgen05 tensor cores (conv_tc.cu,
// BF16 operands, FP32 accumulation; dLearnedSetTensorCores), the other convolutions as direct FP32 convolutions on
// the CUDA cores; weight gradients summed in a fixed order (deterministic); activations FP32 in memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>

#include "internal.h"

using namespace dgb;

dErr device_dot(int64_t n, const double *a, const double *b, double *part, double *out, cudaStream_t s);
dErr ksp_set_monitor(dKSP ksp, dErr (*fn)(void *, int, const double *, const double *), void *ctx);
dErr ksp_set_correction(dKSP ksp, dErr (*fn)(void *, const double *, double *), void *ctx);
dErr ksp_solve(dKSP ksp, const double *b, double *x, double rtol, int maxit, int *its, double *rnorm);
dErr op_mult(_p_dOperator *op, const double *x, double *y);
dErr ksp_get_operator(dKSP ksp, dOperator *op);
dErr fs_gll_lattice(_p_dFS *fs, std::vector<int32_t> &lat, int L0[3]);
bool conv_tc_supported(int ci, int co);
dErr conv_tc_pack(int ci, int co, bool transpose, const __nv_bfloat16 *W, __nv_bfloat16 *out, cudaStream_t s);
dErr conv_tc(int B, int ci, int co, const int d[3], const float *x, const __nv_bfloat16 *wpack, const float *bias, int relu,
             int accumulate, float *y, cudaStream_t s);
dErr conv_tc_check(cudaStream_t s);
dErr conv_tc_wgrad(int B, int ci, int co, const int d[3], const float *x, const float *gy, float *partial, int64_t max_chunks,
                   int *nchunks, cudaStream_t s);

namespace {

struct Dims {
  int x, y, z;
  __host__ __device__ int64_t n() const { return (int64_t)x * y * z; }
};
Dims coarsen(Dims d) { return {(d.x - 1) / 2 + 1, (d.y - 1) / 2 + 1, (d.z - 1) / 2 + 1}; }

struct LayerDef {
  int ci, co, stride, level_in;  // level of the layer's input grid
};
enum { C1A, C1B, D1, C2A, D2, C3A, C3B, U2, C2B, U1, C1C, OUT, NLAYER };
// up blocks convolve on the coarse grid and then interpolate (U2: level 2 -> 1, U1: level 1 -> 0)
constexpr LayerDef kLayer[NLAYER] = {{2, 16, 1, 0},  {16, 16, 1, 0}, {16, 32, 2, 0}, {32, 32, 1, 1},
                                     {32, 64, 2, 1}, {64, 64, 1, 2}, {64, 64, 1, 2}, {64, 32, 1, 2},
                                     {32, 32, 1, 1}, {32, 16, 1, 1}, {16, 16, 1, 0}, {16, 1, 1, 0}};

// ------------------------------------------------------------------------------------------ kernels
__device__ __forceinline__ void vox(int64_t r, Dims d, int &i, int &j, int &k) {
  k = (int)(r % d.z);
  const int64_t q = r / d.z;
  j = (int)(q % d.y);
  i = (int)(q / d.y);
}

// a t-sized window of the lattice d: voxel v of the window at origin o[3] -> its index in the whole lattice
struct Win {
  Dims t, d;
  __device__ int64_t full(const int32_t *o, int64_t v) const {
    int i, j, k;
    vox(v, t, i, j, k);
    return ((int64_t)(o[0] + i) * d.y + o[1] + j) * d.z + o[2] + k;
  }
};

// y = act(conv(x) + bias) [+ skip]; x [B][Ci][di], W [Co][Ci][27] (bf16), y [B][Co][dout]
template <int CO_T>
__global__ void __launch_bounds__(128) k_conv_fwd(int B, int Ci, int Co, Dims di, Dims dout, int stride, const float *__restrict__ x,
                                                  const __nv_bfloat16 *__restrict__ W, const float *__restrict__ bias, int relu,
                                                  float *__restrict__ y) {
  constexpr int CK = 8;
  __shared__ float sW[CO_T][CK][27];
  const int64_t nvo = dout.n(), nvi = di.n();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = t < (int64_t)B * nvo;
  const int co0 = blockIdx.y * CO_T;
  const int64_t b = active ? t / nvo : 0, r = active ? t % nvo : 0;
  int ox, oy, oz;
  vox(r, dout, ox, oy, oz);
  float acc[CO_T];
#pragma unroll
  for (int c = 0; c < CO_T; c++) acc[c] = (co0 + c < Co) ? bias[co0 + c] : 0.f;
  for (int ci0 = 0; ci0 < Ci; ci0 += CK) {
    __syncthreads();
    for (int i = threadIdx.x; i < CO_T * CK * 27; i += blockDim.x) {
      const int c = i / (CK * 27), rr = i % (CK * 27), k = rr / 27, tap = rr % 27;
      sW[c][k][tap] = (co0 + c < Co && ci0 + k < Ci) ? __bfloat162float(W[((size_t)(co0 + c) * Ci + ci0 + k) * 27 + tap]) : 0.f;
    }
    __syncthreads();
    if (!active) continue;
    const int kmax = min(CK, Ci - ci0);
    for (int k = 0; k < kmax; k++) {
      const float *xc = x + ((size_t)b * Ci + ci0 + k) * nvi;
      float xv[27];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        const int ix = ox * stride + a - 1;
#pragma unroll
        for (int bb = 0; bb < 3; bb++) {
          const int iy = oy * stride + bb - 1;
#pragma unroll
          for (int cc = 0; cc < 3; cc++) {
            const int iz = oz * stride + cc - 1;
            const bool in = ix >= 0 && ix < di.x && iy >= 0 && iy < di.y && iz >= 0 && iz < di.z;
            xv[(a * 3 + bb) * 3 + cc] = in ? xc[((int64_t)ix * di.y + iy) * di.z + iz] : 0.f;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < CO_T; c++) {
        float s = acc[c];
#pragma unroll
        for (int tap = 0; tap < 27; tap++) s = fmaf(sW[c][k][tap], xv[tap], s);
        acc[c] = s;
      }
    }
  }
  if (!active) return;
#pragma unroll
  for (int c = 0; c < CO_T; c++) {
    if (co0 + c >= Co) break;
    const float v = relu ? fmaxf(acc[c], 0.f) : acc[c];
    y[((size_t)b * Co + co0 + c) * nvo + r] = v;
  }
}

// Register-blocked forms: a thread computes VZ consecutive outputs along z, so every weight read from
// shared memory feeds VZ multiply-adds and the 3 x 3 x ZW input window is shared by the VZ outputs.
constexpr int VZ = 4;
constexpr int64_t kQuadChunk = 4096;  // z-quads of output voxels per weight-gradient block

__device__ __forceinline__ void quad(int64_t r, Dims d, int nzq, int &ox, int &oy, int &oz0) {
  oz0 = (int)(r % nzq) * VZ;
  r /= nzq;
  oy = (int)(r % d.y);
  ox = (int)(r / d.y);
}

template <int S>
__device__ __forceinline__ void load_window(const float *__restrict__ xc, Dims di, int ox, int oy, int oz0,
                                            float (&w)[3][3][(VZ - 1) * S + 3]) {
  constexpr int ZW = (VZ - 1) * S + 3;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const int ix = ox * S + a - 1;
#pragma unroll
    for (int b = 0; b < 3; b++) {
      const int iy = oy * S + b - 1;
      const bool row = ix >= 0 && ix < di.x && iy >= 0 && iy < di.y;
      const float *xr = xc + ((int64_t)ix * di.y + iy) * di.z;
#pragma unroll
      for (int z = 0; z < ZW; z++) {
        const int iz = oz0 * S - 1 + z;
        w[a][b][z] = row && iz >= 0 && iz < di.z ? xr[iz] : 0.f;
      }
    }
  }
}

template <int CO_T, int S>
__global__ void __launch_bounds__(128) k_conv_fwd_rb(int B, int Ci, int Co, Dims di, Dims dout, const float *__restrict__ x,
                                                     const __nv_bfloat16 *__restrict__ W, const float *__restrict__ bias, int relu,
                                                     float *__restrict__ y) {
  constexpr int CK = 8, ZW = (VZ - 1) * S + 3;
  __shared__ float sW[CO_T][CK][27];
  const int nzq = (dout.z + VZ - 1) / VZ;
  const int64_t nq = (int64_t)dout.x * dout.y * nzq, nvo = dout.n(), nvi = di.n();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = t < (int64_t)B * nq;
  const int co0 = blockIdx.y * CO_T;
  const int64_t b = active ? t / nq : 0;
  int ox, oy, oz0;
  quad(active ? t % nq : 0, dout, nzq, ox, oy, oz0);
  float acc[CO_T][VZ];
#pragma unroll
  for (int c = 0; c < CO_T; c++)
#pragma unroll
    for (int v = 0; v < VZ; v++) acc[c][v] = (co0 + c < Co) ? bias[co0 + c] : 0.f;
  for (int ci0 = 0; ci0 < Ci; ci0 += CK) {
    __syncthreads();
    for (int i = threadIdx.x; i < CO_T * CK * 27; i += blockDim.x) {
      const int c = i / (CK * 27), rr = i % (CK * 27), k = rr / 27, tap = rr % 27;
      sW[c][k][tap] = (co0 + c < Co && ci0 + k < Ci) ? __bfloat162float(W[((size_t)(co0 + c) * Ci + ci0 + k) * 27 + tap]) : 0.f;
    }
    __syncthreads();
    if (!active) continue;
    const int kmax = min(CK, Ci - ci0);
    for (int k = 0; k < kmax; k++) {
      float xw[3][3][ZW];
      load_window<S>(x + ((size_t)b * Ci + ci0 + k) * nvi, di, ox, oy, oz0, xw);
#pragma unroll
      for (int c = 0; c < CO_T; c++)
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
          for (int bb = 0; bb < 3; bb++)
#pragma unroll
            for (int cc = 0; cc < 3; cc++) {
              const float w = sW[c][k][(a * 3 + bb) * 3 + cc];
#pragma unroll
              for (int v = 0; v < VZ; v++) acc[c][v] = fmaf(w, xw[a][bb][v * S + cc], acc[c][v]);
            }
    }
  }
  if (!active) return;
  float *yo = y + (size_t)b * Co * nvo + ((int64_t)ox * dout.y + oy) * dout.z + oz0;
#pragma unroll
  for (int c = 0; c < CO_T; c++) {
    if (co0 + c >= Co) break;
#pragma unroll
    for (int v = 0; v < VZ; v++)
      if (oz0 + v < dout.z) yo[(size_t)(co0 + c) * nvo + v] = relu ? fmaxf(acc[c][v], 0.f) : acc[c][v];
  }
}

// stride-2 data gradient, two z-outputs per thread (2m even, 2m + 1 odd) so that the z parity is the same across a
// warp: the even output takes tap cc = 1 of gy[.., m]; the odd one cc = 0 of gy[.., m + 1], then cc = 2 of gy[.., m]
// (taps in ascending order, as the adjoint of the forward convolution lists them)
template <int CI_T>
__global__ void __launch_bounds__(128) k_conv_bwd_data_s2(int B, int Ci, int Co, Dims di, Dims dout, const float *__restrict__ gy,
                                                          const __nv_bfloat16 *__restrict__ W, float *__restrict__ gx, int accumulate) {
  constexpr int CK = 8;
  __shared__ float sW[CK][CI_T][27];
  const int nzp = (di.z + 1) / 2;
  const int64_t np = (int64_t)di.x * di.y * nzp, nvo = dout.n(), nvi = di.n();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = t < (int64_t)B * np;
  const int ci0 = blockIdx.y * CI_T;
  const int64_t b = active ? t / np : 0, r = active ? t % np : 0;
  const int m = (int)(r % nzp), iy = (int)((r / nzp) % di.y), ix = (int)(r / ((int64_t)nzp * di.y));
  const bool odd_in = 2 * m + 1 < di.z, m1_in = m + 1 < dout.z;
  float ae[CI_T], ao[CI_T];
#pragma unroll
  for (int c = 0; c < CI_T; c++) ae[c] = ao[c] = 0.f;
  for (int co0 = 0; co0 < Co; co0 += CK) {
    __syncthreads();
    for (int i = threadIdx.x; i < CK * CI_T * 27; i += blockDim.x) {
      const int k = i / (CI_T * 27), rr = i % (CI_T * 27), c = rr / 27, tap = rr % 27;
      sW[k][c][tap] = (co0 + k < Co && ci0 + c < Ci) ? __bfloat162float(W[((size_t)(co0 + k) * Ci + ci0 + c) * 27 + tap]) : 0.f;
    }
    __syncthreads();
    if (!active) continue;
    const int kmax = min(CK, Co - co0);
    for (int k = 0; k < kmax; k++) {
      const float *gc = gy + ((size_t)b * Co + co0 + k) * nvo;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        const int nx = ix + 1 - a;
        if (nx < 0 || (nx & 1)) continue;
        const int vx = nx >> 1;
        if (vx >= dout.x) continue;
#pragma unroll
        for (int bb = 0; bb < 3; bb++) {
          const int ny = iy + 1 - bb;
          if (ny < 0 || (ny & 1)) continue;
          const int vy = ny >> 1;
          if (vy >= dout.y) continue;
          const float *gl = gc + ((int64_t)vx * dout.y + vy) * dout.z;
          const float g0 = gl[m], g1 = m1_in ? gl[m + 1] : 0.f;
          const int t0 = (a * 3 + bb) * 3;
#pragma unroll
          for (int c = 0; c < CI_T; c++) {
            ae[c] = fmaf(sW[k][c][t0 + 1], g0, ae[c]);
            if (m1_in) ao[c] = fmaf(sW[k][c][t0], g1, ao[c]);
            ao[c] = fmaf(sW[k][c][t0 + 2], g0, ao[c]);
          }
        }
      }
    }
  }
  if (!active) return;
#pragma unroll
  for (int c = 0; c < CI_T; c++) {
    if (ci0 + c >= Ci) break;
    float *o = gx + ((size_t)b * Ci + ci0 + c) * nvi + ((int64_t)ix * di.y + iy) * di.z + 2 * m;
    o[0] = accumulate ? o[0] + ae[c] : ae[c];
    if (odd_in) o[1] = accumulate ? o[1] + ao[c] : ao[c];
  }
}

// stride-1 data gradient: gx[ci][u] = sum_co sum_taps W[co][ci][t] gy[co][u + 1 - t] (flipped window of gy)
template <int CI_T>
__global__ void __launch_bounds__(128) k_conv_bwd_data_rb(int B, int Ci, int Co, Dims d, const float *__restrict__ gy,
                                                          const __nv_bfloat16 *__restrict__ W, float *__restrict__ gx, int accumulate) {
  constexpr int CK = 8, ZW = VZ + 2;
  __shared__ float sW[CK][CI_T][27];
  const int nzq = (d.z + VZ - 1) / VZ;
  const int64_t nq = (int64_t)d.x * d.y * nzq, nv = d.n();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = t < (int64_t)B * nq;
  const int ci0 = blockIdx.y * CI_T;
  const int64_t b = active ? t / nq : 0;
  int ix, iy, iz0;
  quad(active ? t % nq : 0, d, nzq, ix, iy, iz0);
  float acc[CI_T][VZ];
#pragma unroll
  for (int c = 0; c < CI_T; c++)
#pragma unroll
    for (int v = 0; v < VZ; v++) acc[c][v] = 0.f;
  for (int co0 = 0; co0 < Co; co0 += CK) {
    __syncthreads();
    for (int i = threadIdx.x; i < CK * CI_T * 27; i += blockDim.x) {
      const int k = i / (CI_T * 27), rr = i % (CI_T * 27), c = rr / 27, tap = rr % 27;
      sW[k][c][tap] = (co0 + k < Co && ci0 + c < Ci) ? __bfloat162float(W[((size_t)(co0 + k) * Ci + ci0 + c) * 27 + tap]) : 0.f;
    }
    __syncthreads();
    if (!active) continue;
    const int kmax = min(CK, Co - co0);
    for (int k = 0; k < kmax; k++) {
      float gw[3][3][ZW];  // gy at (ix - 1 + a', iy - 1 + b', iz0 - 1 + z')
      load_window<1>(gy + ((size_t)b * Co + co0 + k) * nv, d, ix, iy, iz0, gw);
#pragma unroll
      for (int c = 0; c < CI_T; c++)
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
          for (int bb = 0; bb < 3; bb++)
#pragma unroll
            for (int cc = 0; cc < 3; cc++) {
              const float w = sW[k][c][(a * 3 + bb) * 3 + cc];
#pragma unroll
              for (int v = 0; v < VZ; v++) acc[c][v] = fmaf(w, gw[2 - a][2 - bb][v + 2 - cc], acc[c][v]);
            }
    }
  }
  if (!active) return;
  float *go = gx + (size_t)b * Ci * nv + ((int64_t)ix * d.y + iy) * d.z + iz0;
#pragma unroll
  for (int c = 0; c < CI_T; c++) {
    if (ci0 + c >= Ci) break;
#pragma unroll
    for (int v = 0; v < VZ; v++)
      if (iz0 + v < d.z) {
        float *o = go + (size_t)(ci0 + c) * nv + v;
        *o = accumulate ? *o + acc[c][v] : acc[c][v];
      }
  }
}

// weight and bias gradient partial sums: CG output channels and one input channel per block, a chunk of
// output z-quads; partial layout [chunk][Co*Ci*27 + Co]
template <int CG, int S>
__global__ void __launch_bounds__(256) k_conv_bwd_weight_rb(int B, int Ci, int Co, Dims di, Dims dout, const float *__restrict__ x,
                                                            const float *__restrict__ gy, float *__restrict__ partial) {
  constexpr int ZW = (VZ - 1) * S + 3, NV = CG * 28;
  __shared__ float red[8][NV];
  const int pair = blockIdx.x, cg = pair / Ci, ci = pair % Ci, co0 = cg * CG;
  const int nzq = (dout.z + VZ - 1) / VZ;
  const int64_t nq = (int64_t)dout.x * dout.y * nzq, nvo = dout.n(), nvi = di.n(), total = (int64_t)B * nq;
  const int64_t q0 = blockIdx.y * kQuadChunk, q1 = min(total, q0 + kQuadChunk);
  float acc[CG][28];
#pragma unroll
  for (int c = 0; c < CG; c++)
#pragma unroll
    for (int i = 0; i < 28; i++) acc[c][i] = 0.f;
  for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    const int64_t b = q / nq;
    int ox, oy, oz0;
    quad(q % nq, dout, nzq, ox, oy, oz0);
    float g[CG][VZ];
    bool any = false;
#pragma unroll
    for (int c = 0; c < CG; c++) {
      const float *gr = gy + ((size_t)b * Co + co0 + c) * nvo + ((int64_t)ox * dout.y + oy) * dout.z + oz0;
#pragma unroll
      for (int v = 0; v < VZ; v++) {
        g[c][v] = oz0 + v < dout.z ? gr[v] : 0.f;
        any |= g[c][v] != 0.f;
      }
    }
    if (!any) continue;
    float xw[3][3][ZW];
    load_window<S>(x + ((size_t)b * Ci + ci) * nvi, di, ox, oy, oz0, xw);
#pragma unroll
    for (int c = 0; c < CG; c++) {
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int bb = 0; bb < 3; bb++)
#pragma unroll
          for (int cc = 0; cc < 3; cc++) {
            float s = acc[c][(a * 3 + bb) * 3 + cc];
#pragma unroll
            for (int v = 0; v < VZ; v++) s = fmaf(g[c][v], xw[a][bb][v * S + cc], s);
            acc[c][(a * 3 + bb) * 3 + cc] = s;
          }
#pragma unroll
      for (int v = 0; v < VZ; v++) acc[c][27] += g[c][v];
    }
  }
  // warp sums, then the 8 warp partials in order
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < CG; c++)
#pragma unroll
    for (int i = 0; i < 28; i++) {
      float v = acc[c][i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[wp][c * 28 + i] = v;
    }
  __syncthreads();
  if (threadIdx.x < NV) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
    const int c = threadIdx.x / 28, i = threadIdx.x % 28;
    const int64_t np = (int64_t)Co * Ci * 27 + Co;
    float *pp = partial + blockIdx.y * np;
    if (i < 27) pp[((int64_t)(co0 + c) * Ci + ci) * 27 + i] = s;
    else if (ci == 0) pp[(int64_t)Co * Ci * 27 + co0 + c] = s;
  }
}

// grad[p] = sum over chunks in order (deterministic)
__global__ void k_sum_chunks(int64_t np, int nchunk, const float *__restrict__ partial, float *__restrict__ grad) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= np) return;
  float s = 0.f;
  for (int c = 0; c < nchunk; c++) s += partial[(int64_t)c * np + p];
  grad[p] = s;
}

// trilinear interpolation between vertex-centred grids (align corners): fine point f sits at coarse position
// f (Lc - 1) / (Lf - 1), kept as the exact fraction num / den in integers (no FP64 on the way)
__device__ __forceinline__ float tent(int f, int Lf, int i, int Lc) {
  if (Lc == 1) return 1.f;
  const int den = Lf - 1, d = abs(f * (Lc - 1) - i * den);
  return d < den ? (float)(den - d) / (float)den : 0.f;
}

__device__ __forceinline__ void lohi(int f, int Lf, int Lc, int &lo, float &fr) {
  if (Lc == 1) {
    lo = 0, fr = 0.f;
    return;
  }
  const int num = f * (Lc - 1), den = Lf - 1;
  lo = min(num / den, Lc - 2);
  fr = (float)(num - lo * den) / (float)den;
}

// out[B][C][df] = interp(in[B][C][dc]); add: out += skip. One thread per fine voxel (z fastest across threads): the
// eight coarse neighbours and weights once, then every channel
__global__ void k_up_fwd(int B, int C, Dims dc, Dims df, const float *__restrict__ in, const float *__restrict__ skip,
                         float *__restrict__ out) {
  const int64_t nf = df.n(), nc = dc.n(), t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * nf) return;
  const int64_t b = t / nf, r = t % nf;
  int fx, fy, fz, lx, ly, lz;
  float ax, ay, az;
  vox(r, df, fx, fy, fz);
  lohi(fx, df.x, dc.x, lx, ax);
  lohi(fy, df.y, dc.y, ly, ay);
  lohi(fz, df.z, dc.z, lz, az);
  int64_t idx[8];
  float w[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int a = k >> 2, bb = (k >> 1) & 1, cc = k & 1;
    const int ix = min(lx + a, dc.x - 1), iy = min(ly + bb, dc.y - 1), iz = min(lz + cc, dc.z - 1);
    idx[k] = ((int64_t)ix * dc.y + iy) * dc.z + iz;
    w[k] = (a ? ax : 1.f - ax) * (bb ? ay : 1.f - ay) * (cc ? az : 1.f - az);
  }
  for (int c = 0; c < C; c++) {
    const float *cp = in + (b * C + c) * nc;
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += w[k] * cp[idx[k]];
    const int64_t o = (b * C + c) * nf + r;
    out[o] = skip ? s + skip[o] : s;
  }
}

// adjoint of the interpolation, as a gather over the fine points in each coarse point's support (at most 2 r + 1 per
// direction, r = (Lf - 1) / (Lc - 1) <= 3 for the halving lattices here); one thread per coarse voxel, the weights once,
// then every channel in the same summation order
__global__ void k_up_bwd(int B, int C, Dims dc, Dims df, const float *__restrict__ gf, float *__restrict__ gc) {
  const int64_t nc = dc.n(), nf = df.n(), t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * nc) return;
  const int64_t b = t / nc, r = t % nc;
  int cx, cy, cz;
  vox(r, dc, cx, cy, cz);
  constexpr int MS = 8;
  auto support = [](int i, int Lc, int Lf, int &f0, float *w) {  // fine points within one coarse spacing of i
    int f1;
    if (Lc == 1) {
      f0 = 0, f1 = Lf - 1;
    } else {
      f0 = i > 0 ? (i - 1) * (Lf - 1) / (Lc - 1) : 0;
      f1 = min(Lf - 1, ((i + 1) * (Lf - 1) + Lc - 2) / (Lc - 1));
    }
    const int n = min(f1 - f0 + 1, MS);
    for (int k = 0; k < MS; k++) w[k] = k < n ? tent(f0 + k, Lf, i, Lc) : 0.f;
    return n;
  };
  int x0, y0, z0;
  float wx[MS], wy[MS], wz[MS];
  const int nx = support(cx, dc.x, df.x, x0, wx), ny = support(cy, dc.y, df.y, y0, wy), nz = support(cz, dc.z, df.z, z0, wz);
  for (int c = 0; c < C; c++) {
    const float *g = gf + (b * C + c) * nf;
    float s = 0.f;
    for (int i = 0; i < nx; i++) {
      if (wx[i] == 0.f) continue;
      for (int j = 0; j < ny; j++) {
        if (wy[j] == 0.f) continue;
        const float *gr = g + ((int64_t)(x0 + i) * df.y + y0 + j) * df.z + z0;
        for (int k = 0; k < nz; k++)
          if (wz[k] != 0.f) s += wx[i] * wy[j] * wz[k] * gr[k];
      }
    }
    gc[(b * C + c) * nc + r] = s;
  }
}

__global__ void k_mask(int64_t n, const float *__restrict__ g, const float *__restrict__ act, float *__restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = act[i] > 0.f ? g[i] : 0.f;
}

__global__ void k_copy_f(int64_t n, const float *__restrict__ a, float *__restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

// MSE over interior lattice nodes (mask [B][nv], one per sample): grad = 2 (y - t) / count, block partial sums
// of (y - t)^2
__global__ void k_mse(int B, int64_t nv, const float *__restrict__ y, const float *__restrict__ tg, const uint8_t *__restrict__ mask,
                      float inv_count, float *__restrict__ grad, double *__restrict__ part) {
  __shared__ double red[256];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double l = 0;
  if (i < (int64_t)B * nv) {
    const bool in = mask[i];
    const float d = in ? y[i] - tg[i] : 0.f;
    grad[i] = 2.f * d * inv_count;
    l = (double)d * d;
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// partial sums of squares of the targets (zero at the masked nodes, where x* and x_k are gathered as zero)
__global__ void k_sumsq(int64_t total, const float *__restrict__ t, double *__restrict__ part) {
  __shared__ double red[256];
  double l = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    l += (double)t[i] * t[i];
  red[threadIdx.x] = l;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_adam(int64_t n, float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       float lr, float b1, float b2, float eps, float bc1, float bc2, __nv_bfloat16 *__restrict__ wb) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi, v[i] = vi;
  const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  w[i] = wi;
  wb[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(int64_t n, const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

// y = A x for a CSR matrix in FP64 (P: dofs x lattice, R = P^T: lattice x dofs)
__global__ void k_csr_mv(int64_t nrows, const int32_t *__restrict__ rp, const int32_t *__restrict__ col, const double *__restrict__ val,
                         const double *__restrict__ x, double *__restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nrows) return;
  double s = 0;
  for (int32_t k = rp[i]; k < rp[i + 1]; k++) s += val[k] * x[col[k]];
  y[i] = s;
}

// network input channel 0 = rc / rms(rc) (interior), channel 1 = log k; scale[0] = rms
__global__ void k_make_input(int64_t nv, const double *__restrict__ rc, const double *__restrict__ ss, double nint,
                             const uint8_t *__restrict__ mask, const float *__restrict__ logk, float *__restrict__ in,
                             double *__restrict__ scale) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const double s = sqrt(*ss / nint), inv = s > 0 ? 1.0 / s : 0.0;
  if (i == 0) *scale = s;
  if (i >= nv) return;
  in[i] = mask[i] ? (float)(rc[i] * inv) : 0.f;
  if (logk) in[nv + i] = logk[i];
}

// z += P (y * scale * ysc), non-finite values dropped and counted
__global__ void k_prolong_add(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ col, const double *__restrict__ val,
                              const float *__restrict__ y, const double *__restrict__ scale, double ysc, double *__restrict__ z,
                              int *__restrict__ bad) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int32_t k = rp[i]; k < rp[i + 1]; k++) s += val[k] * (double)y[col[k]];
  s *= *scale * ysc;
  if (!isfinite(s)) {
    atomicAdd(bad, 1);
    return;
  }
  z[i] += s;
}

// x at the lattice nodes (0 where the node is not an explicit dof)
__global__ void k_gather_vertices(int64_t nv, const int32_t *__restrict__ vdof, const double *__restrict__ x, double *__restrict__ xv) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nv) xv[i] = vdof[i] >= 0 ? x[vdof[i]] : 0.0;
}

// a window of a lattice array (FP32), and x at the nodes of a window (FP64, 0 where the node is not an explicit dof)
__global__ void k_crop_f(Win w, int o0, int o1, int o2, const float *__restrict__ full, float *__restrict__ out) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= w.t.n()) return;
  const int32_t o[3] = {o0, o1, o2};
  out[v] = full[w.full(o, v)];
}

__global__ void k_gather_crop(Win w, int o0, int o1, int o2, const int32_t *__restrict__ vdof, const double *__restrict__ x,
                              double *__restrict__ out) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= w.t.n()) return;
  const int32_t o[3] = {o0, o1, o2};
  const int32_t d = vdof[w.full(o, v)];
  out[v] = d >= 0 ? x[d] : 0.0;
}

// target = (x* - x_k) / scale_k on each pair's window (origins orig[p][3]; x* on the whole lattice)
__global__ void k_targets(Win w, int npairs, const int32_t *__restrict__ orig, const double *__restrict__ xstar,
                          const double *__restrict__ xk, const double *__restrict__ scale, float *__restrict__ tg) {
  const int64_t nt = w.t.n(), t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nt * npairs) return;
  const int64_t p = t / nt, v = t % nt;
  const double s = scale[p];
  tg[t] = s > 0 ? (float)((xstar[w.full(orig + 3 * p, v)] - xk[t]) / s) : 0.f;
}

// minibatch: in[b][0] = pair input, in[b][1] = log k of the pair's field on its window; tb[b] = target / ysc;
// bmask[b] = the interior mask on the window
__global__ void k_batch(int B, Win w, const int32_t *__restrict__ idx, const int32_t *__restrict__ pfield,
                        const int32_t *__restrict__ porig, const float *__restrict__ pin, const float *__restrict__ ptg,
                        const float *__restrict__ flogk, const uint8_t *__restrict__ mask, float inv_ysc, float *__restrict__ in,
                        float *__restrict__ tb, uint8_t *__restrict__ bmask) {
  const int64_t nt = w.t.n(), n0 = w.d.n(), t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * nt) return;
  const int64_t b = t / nt, v = t % nt;
  const int p = idx[b];
  const int64_t f = w.full(porig + 3 * p, v);
  in[(b * 2) * nt + v] = pin[(int64_t)p * nt + v];
  in[(b * 2 + 1) * nt + v] = flogk[(int64_t)pfield[p] * n0 + f];
  tb[t] = ptg[(int64_t)p * nt + v] * inv_ysc;
  bmask[t] = mask[f];
}

// the interior mask repeated for B samples
__global__ void k_bmask(int B, int64_t nv, const uint8_t *__restrict__ mask, uint8_t *__restrict__ bmask) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < (int64_t)B * nv) bmask[t] = mask[t % nv];
}

// seeded uniform values in [-1, 1) (splitmix64 of the index)
__global__ void k_uniform_noise(int64_t n, uint64_t seed, double *__restrict__ x) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  x[i] = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

__global__ void k_scale_d(int64_t n, const double *__restrict__ num, const double *__restrict__ den, double *__restrict__ x) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) x[i] *= sqrt(*num / *den);
}

// log k = g(x) at the vertex coordinates (random Fourier features, as dFSEvaluateLognormal)
__global__ void k_logk(int64_t nv, const double *__restrict__ xyz, const double *__restrict__ grf, float *__restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nv) return;
  if (!grf) {
    out[i] = 0.f;
    return;
  }
  const int nf = (int)grf[0];
  const double *w = grf + 3, *b = grf + 3 + 3 * nf, *x = xyz + 3 * i;
  double s = 0;
  for (int f = 0; f < nf; f++) s += cos(w[3 * f] * x[0] + w[3 * f + 1] * x[1] + w[3 * f + 2] * x[2] + b[f]);
  out[i] = (float)(sqrt(2.0 * grf[1] / nf) * s);
}

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------------------------------------ object
struct _p_dLearned {
  _p_dFS *fs = nullptr;
  int grid = dLEARNED_GRID_VERTEX;
  Dims d[3];                   // the lattice and its two coarse levels (inference)
  Dims dt[3];                  // the training window and its coarse levels (d when training on the whole lattice)
  const Dims *cur = nullptr;   // the dims the network runs on next (d or dt)
  int64_t nint = 0;            // interior (explicit dof) nodes of the lattice
  double lnorm = 1;            // nodes per sample the loss is averaged over (nint, or the window's size)
  // transfer between the global dofs and the lattice
  int32_t *Pp = nullptr, *Pc = nullptr, *Rp = nullptr, *Rc = nullptr, *vdof = nullptr;
  double *Pv = nullptr, *Rv = nullptr, *vxyz = nullptr;
  uint8_t *mask = nullptr;
  float *logk = nullptr;  // current field
  // parameters: per layer W [co][ci][27] then bias [co]
  int64_t woff[NLAYER], boff[NLAYER], nparam = 0;
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *wb = nullptr;
  // tensor-core convolutions (conv_tc.cu) for the stride-1 layers of 16 / 32 channels: packed B operands of the
  // forward convolution and of its data gradient per layer (-1: the layer runs on the CUDA cores)
  bool use_tc = true, tc_checked = false;
  __nv_bfloat16 *wtc = nullptr;
  int64_t tcf[16], tct[16];
  int64_t adam_t = 0;
  double ysc = 1.0;
  bool trained = false;
  // activations and gradients, each grown to the largest (batch, dims) requested so far
  float *act[16] = {};
  int64_t acap[16] = {};
  float *G1 = nullptr, *G2 = nullptr, *GZ = nullptr, *ga1 = nullptr, *ga2 = nullptr, *tb = nullptr, *partial = nullptr;
  int64_t gcap[6] = {}, partial_len = 0, bmcap = 0, lpcap = 0;
  uint8_t *bmask = nullptr;  // interior mask per sample of a batch
  double *lpart = nullptr;
  // correction workspace
  double *rc = nullptr, *ss = nullptr, *scale = nullptr, *dpart = nullptr;
  int *bad = nullptr;
  int64_t applies = 0, dropped = 0;
  // training pairs: input and target on a window (dt) of the lattice at origin porig[p][3], the field of each pair
  int maxpairs = 0, npairs = 0, nfields = 0, maxfields = 0;
  float *pin = nullptr, *ptg = nullptr, *flogk = nullptr;
  int32_t *pfield = nullptr, *porig = nullptr;
  std::vector<int32_t> h_pfield, h_porig;
  std::mt19937_64 wgen;  // window origins
  // collection in progress
  double *cxk = nullptr, *cscale = nullptr, *cxstar = nullptr;
  float *cin = nullptr;  // the whole lattice's input channel of the current iterate
  int cfirst = 0, ccount = 0, cevery = 1, cmax = 0;
};

namespace {

// activation slots
enum { X0, H1, A1, H2, A2, H3, H3B, A3, W2, S2, B2, W1, S1, B1, Y, NACT };

struct Shape {
  int c, level;
};
constexpr Shape kAct[NACT] = {{2, 0},  {16, 0}, {16, 0}, {32, 1}, {32, 1}, {64, 2}, {64, 2}, {64, 2},
                              {32, 2}, {32, 1}, {32, 1}, {16, 1}, {16, 0}, {16, 0}, {1, 0}};

// grow a device buffer to at least n elements (its contents are not kept)
template <typename T>
dErr grow(T **p, int64_t *cap, int64_t n) {
  if (n <= *cap) return 0;
  cudaFree(*p);
  *p = nullptr;
  CUCHK(cudaMalloc(p, std::max<int64_t>(n, 1) * sizeof(T)));
  *cap = n;
  return 0;
}

// buffers for a batch of B samples on the dims L->cur: the activations, and with grads the gradient buffers
dErr ensure_cap(_p_dLearned *L, int B, bool grads) {
  const Dims *d = L->cur;
  for (int i = 0; i < NACT; i++) DCHK(grow(&L->act[i], &L->acap[i], (int64_t)B * kAct[i].c * d[kAct[i].level].n()));
  if (!grads) return 0;
  int64_t gmax = 0;
  for (int i = 0; i < NACT; i++) gmax = std::max<int64_t>(gmax, (int64_t)kAct[i].c * d[kAct[i].level].n());
  DCHK(grow(&L->G1, &L->gcap[0], B * gmax));
  DCHK(grow(&L->G2, &L->gcap[1], B * gmax));
  DCHK(grow(&L->GZ, &L->gcap[2], B * gmax));
  DCHK(grow(&L->ga1, &L->gcap[3], (int64_t)B * 16 * d[0].n()));
  DCHK(grow(&L->ga2, &L->gcap[4], (int64_t)B * 32 * d[1].n()));
  DCHK(grow(&L->tb, &L->gcap[5], (int64_t)B * d[0].n()));
  DCHK(grow(&L->bmask, &L->bmcap, (int64_t)B * d[0].n()));
  DCHK(grow(&L->lpart, &L->lpcap, (int64_t)nblk((int64_t)B * d[0].n())));
  // weight-gradient partials: the largest chunk count times parameters over the layers, and room for one partial
  // per block of the grid-stride tensor-core weight-gradient kernel (up to two blocks per SM)
  int dev = 0, nsm = 0;
  CUCHK(cudaGetDevice(&dev));
  CUCHK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int64_t need = 0;
  for (int l = 0; l < NLAYER; l++) {
    const LayerDef &ld = kLayer[l];
    const Dims dout = ld.stride == 2 ? d[ld.level_in + 1] : d[ld.level_in];
    const int64_t nch = ((int64_t)B * dout.x * dout.y * ((dout.z + VZ - 1) / VZ) + kQuadChunk - 1) / kQuadChunk;
    need = std::max<int64_t>(need, std::max<int64_t>(nch, dout.n() > 0 ? 2 * nsm : 0) * ((int64_t)ld.co * ld.ci * 27 + ld.co));
  }
  DCHK(grow(&L->partial, &L->partial_len, need));
  return 0;
}

bool layer_tc(const _p_dLearned *L, int l) { return L->use_tc && L->tcf[l] >= 0; }

// the tensor-core layers' packed weights from the BF16 copies (after every change of the weights)
dErr repack_tc(_p_dLearned *L, cudaStream_t s) {
  for (int l = 0; l < NLAYER; l++) {
    if (L->tcf[l] < 0) continue;
    DCHK(conv_tc_pack(kLayer[l].ci, kLayer[l].co, false, L->wb + L->woff[l], L->wtc + L->tcf[l], s));
    DCHK(conv_tc_pack(kLayer[l].ci, kLayer[l].co, true, L->wb + L->woff[l], L->wtc + L->tct[l], s));
  }
  return 0;
}

// the first tensor-core convolutions of a network are checked synchronously for a timed-out MMA wait
dErr tc_first_check(_p_dLearned *L, cudaStream_t s) {
  if (L->tc_checked || !L->use_tc) return 0;
  L->tc_checked = true;
  return conv_tc_check(s);
}

dErr conv_fwd(_p_dLearned *L, int l, int B, const float *x, float *y, int relu, cudaStream_t s) {
  const LayerDef &ld = kLayer[l];
  const Dims di = L->cur[ld.level_in], dout = ld.stride == 2 ? L->cur[ld.level_in + 1] : di;
  const __nv_bfloat16 *W = L->wb + L->woff[l];
  const float *bias = L->w + L->boff[l];
  if (layer_tc(L, l)) {
    const int d3[3] = {di.x, di.y, di.z};
    return conv_tc(B, ld.ci, ld.co, d3, x, L->wtc + L->tcf[l], bias, relu, 0, y, s);
  }
  if (ld.co >= 16) {
    const int64_t nq = (int64_t)dout.x * dout.y * ((dout.z + VZ - 1) / VZ);
    dim3 grid(nblk((int64_t)B * nq, 128), (ld.co + 15) / 16);
    if (ld.stride == 1) k_conv_fwd_rb<16, 1><<<grid, 128, 0, s>>>(B, ld.ci, ld.co, di, dout, x, W, bias, relu, y);
    else k_conv_fwd_rb<16, 2><<<grid, 128, 0, s>>>(B, ld.ci, ld.co, di, dout, x, W, bias, relu, y);
  } else if (ld.stride == 1) {  // the one-channel output layer: register-blocked along z as the others
    const int64_t nq = (int64_t)dout.x * dout.y * ((dout.z + VZ - 1) / VZ);
    dim3 grid(nblk((int64_t)B * nq, 128), ld.co);
    k_conv_fwd_rb<1, 1><<<grid, 128, 0, s>>>(B, ld.ci, ld.co, di, dout, x, W, bias, relu, y);
  } else {
    dim3 grid(nblk((int64_t)B * dout.n(), 128), ld.co);
    k_conv_fwd<1><<<grid, 128, 0, s>>>(B, ld.ci, ld.co, di, dout, ld.stride, x, W, bias, relu, y);
  }
  CUCHK(cudaGetLastError());
  return 0;
}

// gx (=, or += with accumulate) = the data gradient of layer l for the output gradient gz
dErr conv_data(_p_dLearned *L, int l, int B, const float *gz, float *gx, int accumulate, cudaStream_t s) {
  const LayerDef &ld = kLayer[l];
  const Dims di = L->cur[ld.level_in], dout = ld.stride == 2 ? L->cur[ld.level_in + 1] : di;
  if (layer_tc(L, l)) {  // the convolution of gz with the flipped kernel, channels swapped
    const int d3[3] = {di.x, di.y, di.z};
    return conv_tc(B, ld.co, ld.ci, d3, gz, L->wtc + L->tct[l], nullptr, 0, accumulate, gx, s);
  }
  if (ld.stride == 1) {
    const int64_t nq = (int64_t)di.x * di.y * ((di.z + VZ - 1) / VZ);
    dim3 grid(nblk((int64_t)B * nq, 128), (ld.ci + 15) / 16);
    k_conv_bwd_data_rb<16><<<grid, 128, 0, s>>>(B, ld.ci, ld.co, di, gz, L->wb + L->woff[l], gx, accumulate);
  } else {
    const int64_t np = (int64_t)di.x * di.y * ((di.z + 1) / 2);
    dim3 grid(nblk((int64_t)B * np, 128), (ld.ci + 15) / 16);
    k_conv_bwd_data_s2<16><<<grid, 128, 0, s>>>(B, ld.ci, ld.co, di, dout, gz, L->wb + L->woff[l], gx, accumulate);
  }
  CUCHK(cudaGetLastError());
  return 0;
}

dErr conv_bwd(_p_dLearned *L, int l, int B, const float *x, const float *gz, float *gx, int accumulate, cudaStream_t s) {
  const LayerDef &ld = kLayer[l];
  const Dims di = L->cur[ld.level_in], dout = ld.stride == 2 ? L->cur[ld.level_in + 1] : di;
  const int64_t total = (int64_t)B * dout.x * dout.y * ((dout.z + VZ - 1) / VZ);
  int nch = (int)((total + kQuadChunk - 1) / kQuadChunk);
  const int64_t np = (int64_t)ld.co * ld.ci * 27 + ld.co;
  if ((int64_t)nch * np > L->partial_len) return set_error("learned correction: gradient workspace too small");
  if (layer_tc(L, l)) {  // per-CTA sums of the tensor-core weight gradient, then the same ordered sum over them
    const int d3[3] = {di.x, di.y, di.z};
    DCHK(conv_tc_wgrad(B, ld.ci, ld.co, d3, x, gz, L->partial, L->partial_len / np, &nch, s));
  } else if (ld.co % 2 == 0) {
    const dim3 grid(ld.co / 2 * ld.ci, nch);
    if (ld.stride == 1) k_conv_bwd_weight_rb<2, 1><<<grid, 256, 0, s>>>(B, ld.ci, ld.co, di, dout, x, gz, L->partial);
    else k_conv_bwd_weight_rb<2, 2><<<grid, 256, 0, s>>>(B, ld.ci, ld.co, di, dout, x, gz, L->partial);
  } else {
    const dim3 grid(ld.co * ld.ci, nch);
    if (ld.stride == 1) k_conv_bwd_weight_rb<1, 1><<<grid, 256, 0, s>>>(B, ld.ci, ld.co, di, dout, x, gz, L->partial);
    else k_conv_bwd_weight_rb<1, 2><<<grid, 256, 0, s>>>(B, ld.ci, ld.co, di, dout, x, gz, L->partial);
  }
  k_sum_chunks<<<nblk(np), 256, 0, s>>>(np, nch, L->partial, L->g + L->woff[l]);
  CUCHK(cudaGetLastError());
  return gx ? conv_data(L, l, B, gz, gx, accumulate, s) : 0;
}

dErr up_fwd(_p_dLearned *L, int B, int C, int lc, const float *in, const float *skip, float *out, cudaStream_t s) {
  const Dims dc = L->cur[lc], df = L->cur[lc - 1];
  k_up_fwd<<<nblk((int64_t)B * df.n()), 256, 0, s>>>(B, C, dc, df, in, skip, out);
  CUCHK(cudaGetLastError());
  return 0;
}

dErr up_bwd(_p_dLearned *L, int B, int C, int lc, const float *gf, float *gc, cudaStream_t s) {
  const Dims dc = L->cur[lc], df = L->cur[lc - 1];
  k_up_bwd<<<nblk((int64_t)B * dc.n()), 256, 0, s>>>(B, C, dc, df, gf, gc);
  CUCHK(cudaGetLastError());
  return 0;
}

dErr mask(int64_t n, const float *g, const float *act, float *out, cudaStream_t s) {
  k_mask<<<nblk(n), 256, 0, s>>>(n, g, act, out);
  CUCHK(cudaGetLastError());
  return 0;
}

// forward of a batch whose input is in act[X0]; output in act[Y]
dErr forward(_p_dLearned *L, int B, cudaStream_t s) {
  float **a = L->act;
  DCHK(conv_fwd(L, C1A, B, a[X0], a[H1], 1, s));
  DCHK(conv_fwd(L, C1B, B, a[H1], a[A1], 1, s));
  DCHK(conv_fwd(L, D1, B, a[A1], a[H2], 1, s));
  DCHK(conv_fwd(L, C2A, B, a[H2], a[A2], 1, s));
  DCHK(conv_fwd(L, D2, B, a[A2], a[H3], 1, s));
  DCHK(conv_fwd(L, C3A, B, a[H3], a[H3B], 1, s));
  DCHK(conv_fwd(L, C3B, B, a[H3B], a[A3], 1, s));
  DCHK(conv_fwd(L, U2, B, a[A3], a[W2], 1, s));
  DCHK(up_fwd(L, B, 32, 2, a[W2], a[A2], a[S2], s));  // s2 = up(w2) + a2
  DCHK(conv_fwd(L, C2B, B, a[S2], a[B2], 1, s));
  DCHK(conv_fwd(L, U1, B, a[B2], a[W1], 1, s));
  DCHK(up_fwd(L, B, 16, 1, a[W1], a[A1], a[S1], s));  // s1 = up(w1) + a1
  DCHK(conv_fwd(L, C1C, B, a[S1], a[B1], 1, s));
  DCHK(conv_fwd(L, OUT, B, a[B1], a[Y], 0, s));
  return tc_first_check(L, s);
}

// backward from dL/dy in G1 [B][1][n0]; parameter gradients into L->g
dErr backward(_p_dLearned *L, int B, cudaStream_t s) {
  float **a = L->act;
  const int64_t n0 = L->cur[0].n(), n1 = L->cur[1].n(), n2 = L->cur[2].n();
  float *G1 = L->G1, *G2 = L->G2, *GZ = L->GZ;
  DCHK(conv_bwd(L, OUT, B, a[B1], G1, G2, 0, s));  // dL/db1
  DCHK(mask((int64_t)B * 16 * n0, G2, a[B1], GZ, s));
  DCHK(conv_bwd(L, C1C, B, a[S1], GZ, G1, 0, s));  // dL/ds1 = dL/dv1 = dL/da1 (skip)
  k_copy_f<<<nblk((int64_t)B * 16 * n0), 256, 0, s>>>((int64_t)B * 16 * n0, G1, L->ga1);
  DCHK(up_bwd(L, B, 16, 1, G1, G2, s));  // dL/dw1 [16][n1]
  DCHK(mask((int64_t)B * 16 * n1, G2, a[W1], GZ, s));
  DCHK(conv_bwd(L, U1, B, a[B2], GZ, G1, 0, s));  // dL/db2
  DCHK(mask((int64_t)B * 32 * n1, G1, a[B2], GZ, s));
  DCHK(conv_bwd(L, C2B, B, a[S2], GZ, G1, 0, s));  // dL/ds2
  k_copy_f<<<nblk((int64_t)B * 32 * n1), 256, 0, s>>>((int64_t)B * 32 * n1, G1, L->ga2);
  DCHK(up_bwd(L, B, 32, 2, G1, G2, s));  // dL/dw2 [32][n2]
  DCHK(mask((int64_t)B * 32 * n2, G2, a[W2], GZ, s));
  DCHK(conv_bwd(L, U2, B, a[A3], GZ, G1, 0, s));  // dL/da3
  DCHK(mask((int64_t)B * 64 * n2, G1, a[A3], GZ, s));
  DCHK(conv_bwd(L, C3B, B, a[H3B], GZ, G1, 0, s));  // dL/dh3b
  DCHK(mask((int64_t)B * 64 * n2, G1, a[H3B], GZ, s));
  DCHK(conv_bwd(L, C3A, B, a[H3], GZ, G1, 0, s));  // dL/dh3
  DCHK(mask((int64_t)B * 64 * n2, G1, a[H3], GZ, s));
  DCHK(conv_bwd(L, D2, B, a[A2], GZ, L->ga2, 1, s));  // dL/da2 += down path
  DCHK(mask((int64_t)B * 32 * n1, L->ga2, a[A2], GZ, s));
  DCHK(conv_bwd(L, C2A, B, a[H2], GZ, G1, 0, s));  // dL/dh2
  DCHK(mask((int64_t)B * 32 * n1, G1, a[H2], GZ, s));
  DCHK(conv_bwd(L, D1, B, a[A1], GZ, L->ga1, 1, s));  // dL/da1 += down path
  DCHK(mask((int64_t)B * 16 * n0, L->ga1, a[A1], GZ, s));
  DCHK(conv_bwd(L, C1B, B, a[H1], GZ, G1, 0, s));  // dL/dh1
  DCHK(mask((int64_t)B * 16 * n0, G1, a[H1], GZ, s));
  DCHK(conv_bwd(L, C1A, B, a[X0], GZ, nullptr, 0, s));
  return 0;
}

// loss of act[Y] against L->tb; gradient into G1
dErr loss(_p_dLearned *L, int B, double *out, cudaStream_t s) {
  const int64_t n0 = L->cur[0].n(), tot = (int64_t)B * n0;
  const unsigned nb = nblk(tot);
  k_mse<<<nb, 256, 0, s>>>(B, n0, L->act[Y], L->tb, L->bmask, (float)(1.0 / ((double)B * L->lnorm)), L->G1, L->lpart);
  CUCHK(cudaGetLastError());
  if (out) {
    std::vector<double> h(nb);
    CUCHK(cudaMemcpyAsync(h.data(), L->lpart, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
    CUCHK(cudaStreamSynchronize(s));
    double t = 0;
    for (double v : h) t += v;
    *out = t / ((double)B * L->lnorm);
  }
  return 0;
}

dErr adam_step(_p_dLearned *L, double lr, cudaStream_t s) {
  L->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - powf(b1, (float)L->adam_t), bc2 = 1.f - powf(b2, (float)L->adam_t);
  k_adam<<<nblk(L->nparam), 256, 0, s>>>(L->nparam, L->w, L->g, L->m, L->v, (float)lr, b1, b2, 1e-8f, bc1, bc2, L->wb);
  CUCHK(cudaGetLastError());
  return repack_tc(L, s);
}

// the correction z += P N(R r); called by FGMRES after the Chebyshev step
dErr apply_correction(void *ctx, const double *r, double *z) {
  Range range_("LearnedCorrection");
  _p_dLearned *L = (_p_dLearned *)ctx;
  _p_dFS *fs = L->fs;
  cudaStream_t s = fs->stream;
  const int64_t n0 = L->d[0].n();
  L->cur = L->d;
  DCHK(ensure_cap(L, 1, false));
  k_csr_mv<<<nblk(n0), 256, 0, s>>>(n0, L->Rp, L->Rc, L->Rv, r, L->rc);
  DCHK(device_dot(n0, L->rc, L->rc, L->dpart, L->ss, s));
  k_make_input<<<nblk(n0), 256, 0, s>>>(n0, L->rc, L->ss, (double)L->nint, L->mask, L->logk, L->act[X0], L->scale);
  CUCHK(cudaGetLastError());
  DCHK(forward(L, 1, s));
  k_prolong_add<<<nblk(fs->n), 256, 0, s>>>(fs->n, L->Pp, L->Pc, L->Pv, L->act[Y], L->scale, L->ysc, z, L->bad);
  CUCHK(cudaGetLastError());
  L->applies++;
  return 0;
}

// CG monitor during pair collection: every cevery-th iterate, R r_k (normalised over the whole lattice) and x_k on a
// window of the lattice (the whole lattice when training on it), at a seeded origin that is a multiple of 4
dErr collect_monitor(void *ctx, int it, const double *x, const double *r) {
  _p_dLearned *L = (_p_dLearned *)ctx;
  if (it % L->cevery || L->ccount >= L->cmax) return 0;
  cudaStream_t s = L->fs->stream;
  const int64_t n0 = L->d[0].n(), nt = L->dt[0].n();
  const int p = L->cfirst + L->ccount;
  int32_t o[3];
  const int dd[3] = {L->d[0].x, L->d[0].y, L->d[0].z}, tt[3] = {L->dt[0].x, L->dt[0].y, L->dt[0].z};
  for (int c = 0; c < 3; c++) o[c] = 4 * (int32_t)(L->wgen() % (uint64_t)((dd[c] - tt[c]) / 4 + 1));
  const Win w{L->dt[0], L->d[0]};
  k_csr_mv<<<nblk(n0), 256, 0, s>>>(n0, L->Rp, L->Rc, L->Rv, r, L->rc);
  DCHK(device_dot(n0, L->rc, L->rc, L->dpart, L->ss, s));
  k_make_input<<<nblk(n0), 256, 0, s>>>(n0, L->rc, L->ss, (double)L->nint, L->mask, nullptr, L->cin, L->cscale + L->ccount);
  k_crop_f<<<nblk(nt), 256, 0, s>>>(w, o[0], o[1], o[2], L->cin, L->pin + (int64_t)p * nt);
  k_gather_crop<<<nblk(nt), 256, 0, s>>>(w, o[0], o[1], o[2], L->vdof, x, L->cxk + (int64_t)L->ccount * nt);
  CUCHK(cudaGetLastError());
  L->h_porig.insert(L->h_porig.end(), o, o + 3);
  L->ccount++;
  return 0;
}

}  // namespace

// ------------------------------------------------------------------------------------------ C ABI
extern "C" {

dErr dLearnedCreate(dFS fs, uint64_t seed, dLearned *out) { return dLearnedCreateOnGrid(fs, dLEARNED_GRID_VERTEX, 0, seed, out); }

dErr dLearnedCreateOnGrid(dFS fs, dLearnedGrid grid, dInt crop, uint64_t seed, dLearned *out) {
  if (!fs || !out) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  if (!fs->uniform || fs->bs != 1) return set_error("learned correction needs a scalar uniform-order space");
  if (grid != dLEARNED_GRID_VERTEX && grid != dLEARNED_GRID_GLL) return set_error("unknown lattice %d", (int)grid);
  if (grid == dLEARNED_GRID_VERTEX && crop) return set_error("the vertex lattice is trained whole (crop 0)");
  if (crop && (crop < 9 || crop % 4 != 1)) return set_error("training window %d: needs 4 m + 1 >= 9 nodes", crop);
  _p_dMesh *mesh = fs->mesh;
  const int p = fs->p, N = p + 1, N3 = N * N * N;
  const int64_t n = fs->n;
  std::vector<double> coords((size_t)fs->nelem * 24);
  CUCHK(cudaMemcpy(coords.data(), fs->d_coords, coords.size() * sizeof(double), cudaMemcpyDeviceToHost));
  double gll[MAXP], wgll[MAXP];
  lobatto_rule(N, gll, wgll);
  // the lattice: vdof (the explicit dof at each node, or -1), node coordinates, P (dofs x lattice) and R = P^T
  Dims d0;
  std::vector<int32_t> vdof, Pp, Pc;
  std::vector<double> Pv, vxyz;
  if (!mesh->structured) return set_error("learned correction needs a block mesh (its vertex or GLL lattice)");
  if (grid == dLEARNED_GRID_VERTEX) {
    d0 = {mesh->nx, mesh->ny, mesh->nz};
    if (std::min({d0.x, d0.y, d0.z}) < 5) return set_error("learned correction needs at least 4 elements per direction");
    const int64_t n0 = d0.n();
    // lattice index of every mesh vertex from its position (interior vertices move by less than half a cell)
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = 0; i < mesh->nv; i++)
      for (int c = 0; c < 3; c++) lo[c] = std::min(lo[c], mesh->vx[3 * i + c]), hi[c] = std::max(hi[c], mesh->vx[3 * i + c]);
    const int Ld[3] = {d0.x, d0.y, d0.z};
    auto lat = [&](const double *X, int c) { return (int)std::lround((X[c] - lo[c]) / (hi[c] - lo[c]) * (Ld[c] - 1)); };
    vxyz.assign((size_t)n0 * 3, 0.0);
    for (int64_t i = 0; i < mesh->nv; i++) {
      const double *X = &mesh->vx[3 * i];
      const int64_t li = ((int64_t)lat(X, 0) * d0.y + lat(X, 1)) * d0.z + lat(X, 2);
      for (int c = 0; c < 3; c++) vxyz[3 * li + c] = X[c];
    }
    // P: every explicit dof from its first occurrence in the expanded ordering; trilinear weights of the
    // element's corner vertices at the dof's GLL reference coordinates; Dirichlet vertices carry no value
    std::vector<int64_t> first(n, -1);
    for (int64_t x = 0; x < fs->nexp; x++) {
      const int32_t c = fs->emap[x];
      if (c < n && first[c] < 0) first[c] = x;
    }
    vdof.assign(n0, -1);
    std::vector<int64_t> corner_lat((size_t)fs->nelem * 8);
    for (int64_t e = 0; e < fs->nelem; e++)
      for (int v = 0; v < 8; v++) {
        const double *X = &coords[(size_t)e * 24 + 3 * v];
        corner_lat[e * 8 + v] = ((int64_t)lat(X, 0) * d0.y + lat(X, 1)) * d0.z + lat(X, 2);
        const int i = v >> 2, j = (v >> 1) & 1, k = v & 1;
        const int32_t c = fs->emap[e * N3 + ((i * p) * N + j * p) * N + k * p];
        if (c < n) vdof[corner_lat[e * 8 + v]] = c;
      }
    Pp.assign(n + 1, 0);
    Pc.reserve(n * 8), Pv.reserve(n * 8);
    for (int64_t d = 0; d < n; d++) {
      const int64_t x = first[d], e = x / N3;
      const int loc = (int)(x - e * N3), a = loc / (N * N), b = (loc / N) % N, c = loc % N;
      std::vector<std::pair<int64_t, double>> row;
      for (int v = 0; v < 8; v++) {
        const int i = v >> 2, j = (v >> 1) & 1, k = v & 1;
        const double w = (i ? 1 + gll[a] : 1 - gll[a]) * (j ? 1 + gll[b] : 1 - gll[b]) * (k ? 1 + gll[c] : 1 - gll[c]) / 8;
        const int64_t lt = corner_lat[e * 8 + v];
        if (w != 0 && vdof[lt] >= 0) row.push_back({lt, w});
      }
      std::sort(row.begin(), row.end());
      for (auto &q : row) Pc.push_back((int32_t)q.first), Pv.push_back(q.second);
      Pp[d + 1] = (int32_t)Pc.size();
    }
  } else {
    // the GLL nodes of the space (the lattice of the Q1-embedded matrix); P and R the injection of the explicit dofs
    std::vector<int32_t> lat;
    int L0[3];
    DCHK(fs_gll_lattice(fs, lat, L0));
    d0 = {L0[0], L0[1], L0[2]};
    if (std::min({d0.x, d0.y, d0.z}) < 9) return set_error("learned correction needs at least 9 GLL nodes per direction");
    const int64_t n0 = d0.n();
    vdof.assign(n0, -1);
    Pp.resize(n + 1), Pc.resize(n), Pv.assign(n, 1.0);
    for (int64_t d = 0; d < n; d++) vdof[lat[d]] = (int32_t)d, Pp[d] = (int32_t)d, Pc[d] = lat[d];
    Pp[n] = (int32_t)n;
    // node coordinates from each element's trilinear map at the GLL reference points
    vxyz.assign((size_t)n0 * 3, 0.0);
    const int My = mesh->ny - 1, Mz = mesh->nz - 1;
    for (int64_t e = 0; e < fs->nelem; e++) {
      const int ex = (int)(e / ((int64_t)My * Mz)), ey = (int)((e / Mz) % My), ez = (int)(e % Mz);
      for (int a = 0; a < N; a++)
        for (int b = 0; b < N; b++)
          for (int c = 0; c < N; c++) {
            const int64_t li = (((int64_t)ex * p + a) * d0.y + ey * p + b) * d0.z + ez * p + c;
            double X[3] = {0, 0, 0};
            for (int v = 0; v < 8; v++) {
              const int i = v >> 2, j = (v >> 1) & 1, k = v & 1;
              const double w = (i ? 1 + gll[a] : 1 - gll[a]) * (j ? 1 + gll[b] : 1 - gll[b]) * (k ? 1 + gll[c] : 1 - gll[c]) / 8;
              for (int q = 0; q < 3; q++) X[q] += w * coords[(size_t)e * 24 + 3 * v + q];
            }
            for (int q = 0; q < 3; q++) vxyz[3 * li + q] = X[q];
          }
    }
  }
  _p_dLearned *L = new _p_dLearned();
  L->fs = fs;
  L->grid = grid;
  L->use_tc = grid == dLEARNED_GRID_GLL;  // the whole-lattice forward at (M p + 1)^3 nodes is where the tensor cores pay
  L->d[0] = d0;
  L->d[1] = coarsen(L->d[0]);
  L->d[2] = coarsen(L->d[1]);
  L->dt[0] = crop ? Dims{std::min(crop, d0.x), std::min(crop, d0.y), std::min(crop, d0.z)} : d0;
  L->dt[1] = coarsen(L->dt[0]);
  L->dt[2] = coarsen(L->dt[1]);
  L->cur = L->d;
  L->wgen.seed(seed ^ 0x9E3779B97F4A7C15ull);
  const int64_t n0 = d0.n();
  // R = P^T with ascending dof order per lattice row
  std::vector<int32_t> Rp(n0 + 1, 0), Rc(Pc.size());
  std::vector<double> Rv(Pc.size());
  for (int32_t c : Pc) Rp[c + 1]++;
  for (int64_t i = 0; i < n0; i++) Rp[i + 1] += Rp[i];
  {
    std::vector<int32_t> pos(Rp.begin(), Rp.end() - 1);
    for (int64_t d = 0; d < n; d++)
      for (int32_t k = Pp[d]; k < Pp[d + 1]; k++) {
        Rc[pos[Pc[k]]] = (int32_t)d;
        Rv[pos[Pc[k]]++] = Pv[k];
      }
  }
  std::vector<uint8_t> msk(n0);
  for (int64_t i = 0; i < n0; i++) msk[i] = vdof[i] >= 0, L->nint += msk[i];
  L->lnorm = crop ? (double)L->dt[0].n() : (double)L->nint;
  auto up = [](auto **dst, const auto &src) -> dErr {
    CUCHK(cudaMalloc(dst, std::max<size_t>(src.size(), 1) * sizeof(src[0])));
    if (src.size()) CUCHK(cudaMemcpy(*dst, src.data(), src.size() * sizeof(src[0]), cudaMemcpyHostToDevice));
    return 0;
  };
  dErr err = 0;
  auto fail = [&](dErr e) {
    _p_dLearned *q = L;
    dLearnedDestroy(&q);
    return e;
  };
  if ((err = up(&L->Pp, Pp)) || (err = up(&L->Pc, Pc)) || (err = up(&L->Pv, Pv)) || (err = up(&L->Rp, Rp)) ||
      (err = up(&L->Rc, Rc)) || (err = up(&L->Rv, Rv)) || (err = up(&L->vdof, vdof)) || (err = up(&L->mask, msk)) ||
      (err = up(&L->vxyz, vxyz)))
    return fail(err);
  CUCHK(cudaMalloc(&L->logk, n0 * sizeof(float)));
  CUCHK(cudaMemset(L->logk, 0, n0 * sizeof(float)));
  CUCHK(cudaMalloc(&L->rc, n0 * sizeof(double)));
  CUCHK(cudaMalloc(&L->ss, 2 * sizeof(double)));
  CUCHK(cudaMalloc(&L->scale, sizeof(double)));
  CUCHK(cudaMalloc(&L->dpart, 1024 * sizeof(double)));
  CUCHK(cudaMalloc(&L->bad, sizeof(int)));
  CUCHK(cudaMemset(L->bad, 0, sizeof(int)));
  // parameters: He-uniform initialisation from a seeded generator, zero biases
  int64_t off = 0;
  for (int l = 0; l < NLAYER; l++) {
    L->woff[l] = off;
    off += (int64_t)kLayer[l].co * kLayer[l].ci * 27;
    L->boff[l] = off;
    off += kLayer[l].co;
  }
  L->nparam = off;
  std::vector<float> w(off, 0.f);
  std::mt19937_64 gen(seed);
  for (int l = 0; l < NLAYER; l++) {
    const double bound = std::sqrt(6.0 / (kLayer[l].ci * 27.0)) * (l == OUT ? 0.1 : 1.0);
    std::uniform_real_distribution<double> U(-bound, bound);
    for (int64_t i = L->woff[l]; i < L->boff[l]; i++) w[i] = (float)U(gen);
  }
  if ((err = up(&L->w, w))) return fail(err);
  for (float **q : {&L->g, &L->m, &L->v}) {
    CUCHK(cudaMalloc(q, off * sizeof(float)));
    CUCHK(cudaMemset(*q, 0, off * sizeof(float)));
  }
  CUCHK(cudaMalloc(&L->wb, off * sizeof(__nv_bfloat16)));
  k_to_bf16<<<nblk(off), 256>>>(off, L->w, L->wb);
  CUCHK(cudaGetLastError());
  int64_t toff = 0;
  for (int l = 0; l < NLAYER; l++) {
    const bool tc = kLayer[l].stride == 1 && conv_tc_supported(kLayer[l].ci, kLayer[l].co);
    L->tcf[l] = tc ? toff : -1;
    toff += tc ? 27LL * kLayer[l].ci * kLayer[l].co : 0;
    L->tct[l] = tc ? toff : -1;
    toff += tc ? 27LL * kLayer[l].ci * kLayer[l].co : 0;
  }
  CUCHK(cudaMalloc(&L->wtc, std::max<int64_t>(toff, 1) * sizeof(__nv_bfloat16)));
  if ((err = repack_tc(L, 0))) return fail(err);
  CUCHK(cudaDeviceSynchronize());
  *out = L;
  return 0;
}

dErr dLearnedDestroy(dLearned *net) {
  if (!net || !*net) return 0;
  _p_dLearned *L = *net;
  for (int i = 0; i < NACT; i++) cudaFree(L->act[i]);
  for (void *p : {(void *)L->Pp, (void *)L->Pc, (void *)L->Rp, (void *)L->Rc, (void *)L->vdof, (void *)L->Pv, (void *)L->Rv,
                  (void *)L->vxyz, (void *)L->mask, (void *)L->logk, (void *)L->w, (void *)L->g, (void *)L->m, (void *)L->v,
                  (void *)L->wb, (void *)L->G1, (void *)L->G2, (void *)L->GZ, (void *)L->ga1, (void *)L->ga2, (void *)L->tb,
                  (void *)L->partial, (void *)L->lpart, (void *)L->rc, (void *)L->ss, (void *)L->scale, (void *)L->dpart,
                  (void *)L->bad, (void *)L->pin, (void *)L->ptg, (void *)L->flogk, (void *)L->pfield, (void *)L->cxk,
                  (void *)L->cscale, (void *)L->cxstar, (void *)L->bmask, (void *)L->porig, (void *)L->cin, (void *)L->wtc})
    cudaFree(p);
  delete L;
  *net = nullptr;
  return 0;
}

dErr dLearnedGetSizes(dLearned L, dInt dims[3], int64_t *nparam, int64_t *npairs) {
  if (!L) return set_error("null network");
  if (dims) dims[0] = L->d[0].x, dims[1] = L->d[0].y, dims[2] = L->d[0].z;
  if (nparam) *nparam = L->nparam;
  if (npairs) *npairs = L->npairs;
  return 0;
}

dErr dLearnedSetField(dLearned L, const dReal *grf) {
  if (!L) return set_error("null network");
  const int64_t n0 = L->d[0].n();
  double *dg = nullptr;
  if (grf) {
    const int nf = (int)grf[0];
    CUCHK(cudaMalloc(&dg, (3 + 4 * nf) * sizeof(double)));
    CUCHK(cudaMemcpy(dg, grf, (3 + 4 * nf) * sizeof(double), cudaMemcpyHostToDevice));
  }
  k_logk<<<nblk(n0), 256, 0, L->fs->stream>>>(n0, L->vxyz, dg, L->logk);
  CUCHK(cudaGetLastError());
  CUCHK(cudaStreamSynchronize(L->fs->stream));
  cudaFree(dg);
  return 0;
}

dErr dLearnedGetWeights(dLearned L, float *w_host) {
  if (!L || !w_host) return set_error("null argument");
  CUCHK(cudaMemcpy(w_host, L->w, L->nparam * sizeof(float), cudaMemcpyDeviceToHost));
  return 0;
}

dErr dLearnedSetWeights(dLearned L, const float *w_host, dReal ysc) {
  if (!L || !w_host) return set_error("null argument");
  CUCHK(cudaMemcpy(L->w, w_host, L->nparam * sizeof(float), cudaMemcpyHostToDevice));
  k_to_bf16<<<nblk(L->nparam), 256>>>(L->nparam, L->w, L->wb);
  CUCHK(cudaGetLastError());
  DCHK(repack_tc(L, 0));
  CUCHK(cudaDeviceSynchronize());
  if (ysc > 0) L->ysc = ysc, L->trained = true;
  return 0;
}

// raw network on device arrays: in [B][2][lattice], out [B][1][lattice] (FP32)
dErr dLearnedForward(dLearned L, dInt B, const float *in, float *out) {
  if (!L || !in || !out || B < 1) return set_error("bad argument");
  cudaStream_t s = L->fs->stream;
  L->cur = L->d;
  DCHK(ensure_cap(L, B, false));
  const int64_t n0 = L->d[0].n();
  CUCHK(cudaMemcpyAsync(L->act[X0], in, (size_t)B * 2 * n0 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  DCHK(forward(L, B, s));
  CUCHK(cudaMemcpyAsync(out, L->act[Y], (size_t)B * n0 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaStreamSynchronize(s));
  return 0;
}

// loss (mean squared error over interior vertices) and its parameter gradient (device array [nparam])
dErr dLearnedLossGrad(dLearned L, dInt B, const float *in, const float *target, dReal *lossv, float *grad) {
  if (!L || !in || !target || B < 1) return set_error("bad argument");
  cudaStream_t s = L->fs->stream;
  L->cur = L->d;
  DCHK(ensure_cap(L, B, true));
  const int64_t n0 = L->d[0].n();
  CUCHK(cudaMemcpyAsync(L->act[X0], in, (size_t)B * 2 * n0 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaMemcpyAsync(L->tb, target, (size_t)B * n0 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  k_bmask<<<nblk((int64_t)B * n0), 256, 0, s>>>(B, n0, L->mask, L->bmask);
  CUCHK(cudaGetLastError());
  DCHK(forward(L, B, s));
  double lv = 0;
  DCHK(loss(L, B, &lv, s));
  DCHK(backward(L, B, s));
  if (grad) CUCHK(cudaMemcpyAsync(grad, L->g, L->nparam * sizeof(float), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaStreamSynchronize(s));
  if (lossv) *lossv = lv;
  return 0;
}

// run the plain solver (CG, its preconditioner as configured) on b and record up to max_pairs
// (residual, error) pairs from every `every`-th iterate; the current field (dLearnedSetField) is the
// pairs' log k channel
dErr dLearnedCollectPairs(dLearned L, dKSP ksp, const dScalar *b, dReal rtol, dInt maxit, dInt every, dInt max_pairs,
                          int rough_start, dInt *collected) {
  Range range_("LearnedCollectPairs");
  if (!L || !ksp || !b) return set_error("null argument");
  if (every < 1 || max_pairs < 1) return set_error("every and max_pairs must be positive");
  _p_dFS *fs = L->fs;
  cudaStream_t s = fs->stream;
  const int64_t n0 = L->d[0].n(), nt = L->dt[0].n();
  // grow the pair store (pairs on their windows, nt values each) and the field store (whole lattice)
  const int newmax = L->npairs + max_pairs;
  if (newmax > L->maxpairs) {
    float *pin, *ptg;
    int32_t *pf, *po;
    CUCHK(cudaMalloc(&pin, (size_t)newmax * nt * sizeof(float)));
    CUCHK(cudaMalloc(&ptg, (size_t)newmax * nt * sizeof(float)));
    CUCHK(cudaMalloc(&pf, (size_t)newmax * sizeof(int32_t)));
    CUCHK(cudaMalloc(&po, (size_t)newmax * 3 * sizeof(int32_t)));
    if (L->npairs) {
      CUCHK(cudaMemcpy(pin, L->pin, (size_t)L->npairs * nt * sizeof(float), cudaMemcpyDeviceToDevice));
      CUCHK(cudaMemcpy(ptg, L->ptg, (size_t)L->npairs * nt * sizeof(float), cudaMemcpyDeviceToDevice));
    }
    cudaFree(L->pin), cudaFree(L->ptg), cudaFree(L->pfield), cudaFree(L->porig);
    L->pin = pin, L->ptg = ptg, L->pfield = pf, L->porig = po, L->maxpairs = newmax;
  }
  if (L->nfields + 1 > L->maxfields) {
    const int nm = std::max(8, 2 * L->maxfields);
    float *fl;
    CUCHK(cudaMalloc(&fl, (size_t)nm * n0 * sizeof(float)));
    if (L->nfields) CUCHK(cudaMemcpy(fl, L->flogk, (size_t)L->nfields * n0 * sizeof(float), cudaMemcpyDeviceToDevice));
    cudaFree(L->flogk);
    L->flogk = fl, L->maxfields = nm;
  }
  CUCHK(cudaMemcpy(L->flogk + (int64_t)L->nfields * n0, L->logk, n0 * sizeof(float), cudaMemcpyDeviceToDevice));
  CUCHK(cudaMalloc(&L->cxk, (size_t)max_pairs * nt * sizeof(double)));
  CUCHK(cudaMalloc(&L->cscale, (size_t)max_pairs * sizeof(double)));
  CUCHK(cudaMalloc(&L->cxstar, (size_t)n0 * sizeof(double)));
  CUCHK(cudaMalloc(&L->cin, (size_t)n0 * sizeof(float)));
  L->cfirst = L->npairs, L->ccount = 0, L->cevery = every, L->cmax = max_pairs;
  L->h_porig.resize((size_t)L->npairs * 3);
  double *x;
  CUCHK(cudaMalloc(&x, std::max<int64_t>(fs->n, 1) * sizeof(double)));
  CUCHK(cudaMemsetAsync(x, 0, fs->n * sizeof(double), s));
  if (rough_start) {  // x0 = a xi, xi seeded noise, a such that ||A x0|| = ||b||: rough early residuals
    dOperator op;
    double *ax, *nrm;
    DCHK(ksp_get_operator(ksp, &op));
    CUCHK(cudaMalloc(&ax, std::max<int64_t>(fs->n, 1) * sizeof(double)));
    CUCHK(cudaMalloc(&nrm, 2 * sizeof(double)));
    k_uniform_noise<<<nblk(fs->n), 256, 0, s>>>(fs->n, 0x5EEDull + 7919ull * (uint64_t)L->nfields, x);
    DCHK(op_mult(op, x, ax));
    DCHK(device_dot(fs->n, b, b, L->dpart, nrm, s));
    DCHK(device_dot(fs->n, ax, ax, L->dpart, nrm + 1, s));
    k_scale_d<<<nblk(fs->n), 256, 0, s>>>(fs->n, nrm, nrm + 1, x);
    CUCHK(cudaGetLastError());
    CUCHK(cudaStreamSynchronize(s));
    cudaFree(ax);
    cudaFree(nrm);
  }
  int its = 0;
  double rn = 0;
  dErr err = ksp_set_monitor(ksp, collect_monitor, L);
  if (!err) err = ksp_solve(ksp, b, x, rtol, maxit, &its, &rn);
  ksp_set_monitor(ksp, nullptr, nullptr);
  if (!err && !(rn <= rtol)) err = set_error("plain solve reached only %g of %g while collecting pairs", rn, rtol);
  if (!err) {
    const int np = L->ccount;
    k_gather_vertices<<<nblk(n0), 256, 0, s>>>(n0, L->vdof, x, L->cxstar);
    L->h_pfield.resize(L->cfirst + np, L->nfields);
    if (L->cfirst + np) {
      CUCHK(cudaMemcpyAsync(L->pfield, L->h_pfield.data(), (L->cfirst + np) * sizeof(int32_t), cudaMemcpyHostToDevice, s));
      CUCHK(cudaMemcpyAsync(L->porig, L->h_porig.data(), (size_t)(L->cfirst + np) * 3 * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    }
    if (np)
      k_targets<<<nblk((int64_t)np * nt), 256, 0, s>>>(Win{L->dt[0], L->d[0]}, np, L->porig + 3 * L->cfirst, L->cxstar, L->cxk,
                                                       L->cscale, L->ptg + (int64_t)L->cfirst * nt);
    CUCHK(cudaStreamSynchronize(s));
    CUCHK(cudaGetLastError());
    L->npairs += np;
    L->nfields++;
    if (collected) *collected = np;
  }
  if (err) L->h_porig.resize((size_t)L->npairs * 3);
  cudaFree(x);
  cudaFree(L->cxk), cudaFree(L->cscale), cudaFree(L->cxstar), cudaFree(L->cin);
  L->cxk = L->cscale = L->cxstar = nullptr;
  L->cin = nullptr;
  return err;
}

// minibatch Adam on the collected pairs; losses[epochs] receives the mean loss of every epoch
dErr dLearnedTrain(dLearned L, dInt epochs, dInt batch, dReal lr, uint64_t seed, dReal *losses) {
  Range range_("LearnedTrain");
  if (!L) return set_error("null network");
  if (L->npairs < 1) return set_error("no training pairs collected");
  if (epochs < 1 || batch < 1) return set_error("epochs and batch must be positive");
  _p_dFS *fs = L->fs;
  cudaStream_t s = fs->stream;
  const int64_t nt = L->dt[0].n();
  const int B = std::min<int>(batch, L->npairs);
  L->cur = L->dt;
  DCHK(ensure_cap(L, B, true));
  // target scale: RMS of all targets over the nodes the loss averages over (fixed once, kept with the network)
  if (!L->trained) {
    k_sumsq<<<1024, 256, 0, s>>>((int64_t)L->npairs * nt, L->ptg, L->dpart);
    CUCHK(cudaGetLastError());
    std::vector<double> h(1024);
    CUCHK(cudaMemcpyAsync(h.data(), L->dpart, 1024 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CUCHK(cudaStreamSynchronize(s));
    double ss = 0;
    for (double v : h) ss += v;
    L->ysc = std::sqrt(ss / ((double)L->npairs * L->lnorm));
    if (!(L->ysc > 0)) L->ysc = 1;
  }
  int32_t *didx;
  CUCHK(cudaMalloc(&didx, B * sizeof(int32_t)));
  std::mt19937_64 gen(seed);
  std::vector<int32_t> perm(L->npairs);
  dErr err = 0;
  for (int ep = 0; ep < epochs && !err; ep++) {
    for (int i = 0; i < L->npairs; i++) perm[i] = i;
    std::shuffle(perm.begin(), perm.end(), gen);
    double tot = 0;
    int nb = 0;
    for (int i0 = 0; i0 + B <= L->npairs && !err; i0 += B, nb++) {
      CUCHK(cudaMemcpyAsync(didx, perm.data() + i0, B * sizeof(int32_t), cudaMemcpyHostToDevice, s));
      k_batch<<<nblk((int64_t)B * nt), 256, 0, s>>>(B, Win{L->dt[0], L->d[0]}, didx, L->pfield, L->porig, L->pin, L->ptg, L->flogk,
                                                    L->mask, (float)(1.0 / L->ysc), L->act[X0], L->tb, L->bmask);
      CUCHK(cudaGetLastError());
      DCHK(forward(L, B, s));
      double lv = 0;
      DCHK(loss(L, B, &lv, s));
      DCHK(backward(L, B, s));
      DCHK(adam_step(L, lr, s));
      tot += lv;
    }
    if (losses) losses[ep] = nb ? tot / nb : 0;
  }
  CUCHK(cudaStreamSynchronize(s));
  cudaFree(didx);
  if (!err && L->use_tc) err = conv_tc_check(s);
  L->trained = true;
  return err;
}

dErr dLearnedGetScale(dLearned L, dReal *ysc) {
  if (!L || !ysc) return set_error("null argument");
  *ysc = L->ysc;
  return 0;
}

// z += P N(R r) for a global residual r (device vectors)
dErr dLearnedApply(dLearned L, const dScalar *r, dScalar *z) {
  if (!L || !r || !z) return set_error("null argument");
  DCHK(apply_correction(L, r, z));
  CUCHK(cudaStreamSynchronize(L->fs->stream));
  return 0;
}

// restriction and prolongation on their own (device vectors): rc = R r [lattice], z += P c
dErr dLearnedRestrict(dLearned L, const dScalar *r, dScalar *rc) {
  if (!L || !r || !rc) return set_error("null argument");
  const int64_t n0 = L->d[0].n();
  k_csr_mv<<<nblk(n0), 256, 0, L->fs->stream>>>(n0, L->Rp, L->Rc, L->Rv, r, rc);
  CUCHK(cudaGetLastError());
  return 0;
}

dErr dLearnedProlong(dLearned L, const dScalar *c, dScalar *z) {
  if (!L || !c || !z) return set_error("null argument");
  k_csr_mv<<<nblk(L->fs->n), 256, 0, L->fs->stream>>>(L->fs->n, L->Pp, L->Pc, L->Pv, c, z);
  CUCHK(cudaGetLastError());
  return 0;
}

// FGMRES preconditioner z = Chebyshev(r) + P N(R r); NULL removes the correction
dErr dKSPSetLearnedCorrection(dKSP ksp, dLearned L) {
  if (!ksp) return set_error("null KSP");
  if (L && !L->trained) return set_error("the network has not been trained or loaded");
  return L ? ksp_set_correction(ksp, apply_correction, L) : ksp_set_correction(ksp, nullptr, nullptr);
}

// one convolution layer on device FP32 arrays: transpose 0: out = act(conv(in) + bias) (ReLU on every layer but the
// last), in [B][ci][dims] -> out [B][co][dims, halved for stride 2]; transpose 1: its data gradient, in [B][co][...]
// -> out [B][ci][dims]
dErr dLearnedLayerApply(dLearned L, dInt layer, dInt transpose, dInt B, const dInt dims[3], const float *in, float *out) {
  if (!L || !dims || !in || !out || B < 1) return set_error("bad argument");
  if (layer < 0 || layer >= NLAYER) return set_error("layer %d of %d", layer, NLAYER);
  const LayerDef &ld = kLayer[layer];
  Dims tmp[3] = {};
  tmp[ld.level_in] = {dims[0], dims[1], dims[2]};
  if (ld.level_in < 2) tmp[ld.level_in + 1] = coarsen(tmp[ld.level_in]);
  cudaStream_t s = L->fs->stream;
  L->cur = tmp;
  dErr e = transpose ? conv_data(L, layer, B, in, out, 0, s) : conv_fwd(L, layer, B, in, out, layer != OUT, s);
  L->cur = L->d;
  DCHK(e);
  CUCHK(cudaStreamSynchronize(s));
  return conv_tc_check(s);
}

// the weight and bias gradient of one layer for input x [B][ci][dims] and output gradient gy [B][co][dims'], into
// grad [co ci 27 + co] (device FP32)
dErr dLearnedLayerWeightGrad(dLearned L, dInt layer, dInt B, const dInt dims[3], const float *x, const float *gy, float *grad) {
  if (!L || !dims || !x || !gy || !grad || B < 1) return set_error("bad argument");
  if (layer < 0 || layer >= NLAYER) return set_error("layer %d of %d", layer, NLAYER);
  const LayerDef &ld = kLayer[layer];
  Dims tmp[3] = {};
  tmp[ld.level_in] = {dims[0], dims[1], dims[2]};
  if (ld.level_in < 2) tmp[ld.level_in + 1] = coarsen(tmp[ld.level_in]);
  cudaStream_t s = L->fs->stream;
  L->cur = tmp;
  dErr e = ensure_cap(L, B, true);
  if (!e) e = conv_bwd(L, layer, B, x, gy, nullptr, 0, s);
  L->cur = L->d;
  DCHK(e);
  const int64_t np = (int64_t)ld.co * ld.ci * 27 + ld.co;
  CUCHK(cudaMemcpyAsync(grad, L->g + L->woff[layer], np * sizeof(float), cudaMemcpyDeviceToDevice, s));
  CUCHK(cudaStreamSynchronize(s));
  return conv_tc_check(s);
}

dErr dLearnedSetTensorCores(dLearned L, int on) {
  if (!L) return set_error("null network");
  L->use_tc = on != 0;
  L->tc_checked = false;
  return 0;
}

// checkpoint file: "DGBUNET1", then (little-endian) uint32 format version 1, uint32 JSON length, int64 parameters,
// float64 target scale, int64 Adam steps, uint32 flags (1: Adam moments follow the weights), the JSON header (the
// same fields and the layer list, for readers), the FP32 weights, and with flag 1 the FP32 first and second moments
namespace {
constexpr char kMagic[8] = {'D', 'G', 'B', 'U', 'N', 'E', 'T', '1'};
struct CkptHead {
  uint32_t version, json_len;
  int64_t nparam;
  double ysc;
  int64_t adam_t;
  uint32_t flags;
};
}  // namespace

dErr dLearnedSave(dLearned L, const char *path, int with_moments) {
  if (!L || !path) return set_error("null argument");
  std::string js = "{\"format\": \"dohp_gb300 U-Net checkpoint\", \"version\": 1, \"nparam\": " + std::to_string(L->nparam) +
                   ", \"grid\": \"" + (L->grid == dLEARNED_GRID_GLL ? "gll" : "vertex") + "\", \"lattice\": [" +
                   std::to_string(L->d[0].x) + ", " + std::to_string(L->d[0].y) + ", " + std::to_string(L->d[0].z) +
                   "], \"layers\": [";
  const char *names[NLAYER] = {"C1A", "C1B", "D1", "C2A", "D2", "C3A", "C3B", "U2", "C2B", "U1", "C1C", "OUT"};
  for (int l = 0; l < NLAYER; l++)
    js += std::string(l ? ", " : "") + "[\"" + names[l] + "\", " + std::to_string(kLayer[l].ci) + ", " + std::to_string(kLayer[l].co) +
          ", " + std::to_string(kLayer[l].stride) + "]";
  js += "], \"weights\": \"per layer W[co][ci][27] then bias[co], float32 little-endian\"}";
  CkptHead h{1u, (uint32_t)js.size(), L->nparam, L->ysc, L->adam_t, with_moments ? 1u : 0u};
  std::vector<float> buf((size_t)L->nparam * (with_moments ? 3 : 1));
  CUCHK(cudaMemcpy(buf.data(), L->w, L->nparam * sizeof(float), cudaMemcpyDeviceToHost));
  if (with_moments) {
    CUCHK(cudaMemcpy(buf.data() + L->nparam, L->m, L->nparam * sizeof(float), cudaMemcpyDeviceToHost));
    CUCHK(cudaMemcpy(buf.data() + 2 * L->nparam, L->v, L->nparam * sizeof(float), cudaMemcpyDeviceToHost));
  }
  FILE *f = fopen(path, "wb");
  if (!f) return set_error("cannot open %s for writing", path);
  const bool ok = fwrite(kMagic, 1, 8, f) == 8 && fwrite(&h.version, 4, 1, f) == 1 && fwrite(&h.json_len, 4, 1, f) == 1 &&
                  fwrite(&h.nparam, 8, 1, f) == 1 && fwrite(&h.ysc, 8, 1, f) == 1 && fwrite(&h.adam_t, 8, 1, f) == 1 &&
                  fwrite(&h.flags, 4, 1, f) == 1 && fwrite(js.data(), 1, js.size(), f) == js.size() &&
                  fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
  if (fclose(f) != 0 || !ok) return set_error("writing %s failed", path);
  return 0;
}

dErr dLearnedLoad(dLearned L, const char *path) {
  if (!L || !path) return set_error("null argument");
  FILE *f = fopen(path, "rb");
  if (!f) return set_error("cannot open %s", path);
  char magic[8];
  CkptHead h{};
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, kMagic, 8) == 0 && fread(&h.version, 4, 1, f) == 1 && fread(&h.json_len, 4, 1, f) == 1 &&
            fread(&h.nparam, 8, 1, f) == 1 && fread(&h.ysc, 8, 1, f) == 1 && fread(&h.adam_t, 8, 1, f) == 1 && fread(&h.flags, 4, 1, f) == 1;
  if (!ok || h.version != 1) {
    fclose(f);
    return set_error("%s is not a U-Net checkpoint of format 1", path);
  }
  if (h.nparam != L->nparam) {
    fclose(f);
    return set_error("%s holds %lld parameters, the network has %lld", path, (long long)h.nparam, (long long)L->nparam);
  }
  const size_t count = (size_t)h.nparam * ((h.flags & 1u) ? 3 : 1);
  std::vector<float> buf(count);
  ok = fseek(f, (long)h.json_len, SEEK_CUR) == 0 && fread(buf.data(), sizeof(float), count, f) == count;
  fclose(f);
  if (!ok) return set_error("%s is truncated", path);
  CUCHK(cudaMemcpy(L->w, buf.data(), L->nparam * sizeof(float), cudaMemcpyHostToDevice));
  if (h.flags & 1u) {
    CUCHK(cudaMemcpy(L->m, buf.data() + L->nparam, L->nparam * sizeof(float), cudaMemcpyHostToDevice));
    CUCHK(cudaMemcpy(L->v, buf.data() + 2 * L->nparam, L->nparam * sizeof(float), cudaMemcpyHostToDevice));
    L->adam_t = h.adam_t;
  }
  k_to_bf16<<<nblk(L->nparam), 256>>>(L->nparam, L->w, L->wb);
  CUCHK(cudaGetLastError());
  DCHK(repack_tc(L, 0));
  CUCHK(cudaDeviceSynchronize());
  L->ysc = h.ysc;
  L->trained = true;
  return 0;
}

dErr dLearnedGetPair(dLearned L, dInt p, dInt window[3], dInt origin[3], float *input, float *target) {
  if (!L) return set_error("null network");
  if (p < 0 || p >= L->npairs) return set_error("pair %d of %d", p, L->npairs);
  const int64_t nt = L->dt[0].n();
  if (window) window[0] = L->dt[0].x, window[1] = L->dt[0].y, window[2] = L->dt[0].z;
  if (origin)
    for (int c = 0; c < 3; c++) origin[c] = L->h_porig[(size_t)p * 3 + c];
  if (input) CUCHK(cudaMemcpy(input, L->pin + (int64_t)p * nt, nt * sizeof(float), cudaMemcpyDeviceToHost));
  if (target) CUCHK(cudaMemcpy(target, L->ptg + (int64_t)p * nt, nt * sizeof(float), cudaMemcpyDeviceToHost));
  return 0;
}

dErr dLearnedGetStats(dLearned L, int64_t *applies, int64_t *dropped_values) {
  if (!L) return set_error("null network");
  int bad = 0;
  CUCHK(cudaMemcpy(&bad, L->bad, sizeof(int), cudaMemcpyDeviceToHost));
  if (applies) *applies = L->applies;
  if (dropped_values) *dropped_values = bad;
  return 0;
}

}  // extern "C"
