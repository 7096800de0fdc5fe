// dRulesetIterator, batched device form (src/fs/interface/fsrulesetit.c:234-643).
//
// The reference walks elements one at a time: GetPatchApplied evaluates coordinates (link 0: INTERP and
// GRAD of the Q1 coordinate space, dRuleComputePhysical) and the field (INTERP, GRAD mapped by J^-1) at the
// element's quadrature points, the caller's q-function fills v/dv, CommitPatchApplied integrates them back
// (INTERP_TRANSPOSE, GRAD_TRANSPOSE) into the expanded test vector, and Finish restricts it. Here one call of
// each step covers all elements: quadrature arrays are element-natural per element, elements back to back,
// and every evaluation is one batched dEFSApply launch per element order (one launch on a uniform-order
// space; on a mixed-order space the elements of each order triple form a bucket, and the launches read and
// write each element at its own expanded-node and quadrature-point offsets). FAST rules (one patch per
// element), and on uniform-order spaces the SPARSE rule (2 Gauss points in each GLL sub-interval, (2p)^3 points
// per element in tensor order: the p^3 patches of the reference's patch loop are the 2 x 2 x 2 blocks of it).
#include <algorithm>
#include <array>
#include <cmath>
#include <map>

#include "internal.h"

using namespace dgb;

dErr fs_expand(_p_dFS *fs, const double *g, double *x, bool inhomogeneous, int add);
dErr fs_restrict(_p_dFS *fs, const double *x, double *g, int add);
dErr efs_apply_list(dEFS efs, int64_t nelem, const int32_t *elist, const int32_t *ioff, const int32_t *ooff, const double *jinv,
                    int D, const double *in, double *out, dApplyMode amode, InsertMode imode, cudaStream_t stream);

namespace {
struct IterBucket {
  dEFS efs = nullptr, cefs = nullptr;  // field and coordinate element spaces on the same rule
  int64_t nel = 0;
  int32_t *d_elist = nullptr;  // the bucket's elements; null: every element, contiguous (uniform-order space)
};
}  // namespace

struct _p_dRulesetIterator {
  dFS fs;
  std::vector<IterBucket> buckets;
  int64_t nq = 0, nel = 0;
  double *xexp = nullptr, *yexp = nullptr;
  double *jw = nullptr, *x = nullptr, *dx = nullptr, *jinv = nullptr, *u = nullptr, *du = nullptr, *v = nullptr, *dv = nullptr;
  double *d_w = nullptr;  // rule weights: per element-natural point (uniform order) or per point (mixed orders)
  bool per_point_w = false;
  bool started = false, applied = false;
};

namespace {

// dRuleComputePhysical (src/jacobi/interface/jacobi.c:383-414): J^-1 by cofactors, jw = w det J, det < 0 is an error
__global__ void k_physical(int64_t ntot, int nq, bool per_point, const double *__restrict__ w, const double *__restrict__ dx,
                           double *__restrict__ jinv, double *__restrict__ jw, int *neg) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= ntot) return;
  const double *a = dx + t * 9;
  double *b = jinv + t * 9;
  const double c0 = a[4] * a[8] - a[7] * a[5], c3 = -(a[3] * a[8] - a[6] * a[5]), c6 = a[3] * a[7] - a[6] * a[4];
  const double det = a[0] * c0 + a[1] * c3 + a[2] * c6, id = 1.0 / det;
  b[0] = id * c0;
  b[1] = -id * (a[1] * a[8] - a[7] * a[2]);
  b[2] = id * (a[1] * a[5] - a[4] * a[2]);
  b[3] = id * c3;
  b[4] = id * (a[0] * a[8] - a[6] * a[2]);
  b[5] = -id * (a[0] * a[5] - a[3] * a[2]);
  b[6] = id * c6;
  b[7] = -id * (a[0] * a[7] - a[6] * a[1]);
  b[8] = id * (a[0] * a[4] - a[3] * a[1]);
  if (det < 0) atomicExch(neg, 1);
  jw[t] = (per_point ? w[t] : w[t % nq]) * det;
}

// dNormsUpdate (src/util/util.c:121-144) over all points: per block partial sums of |r| jw, r^2 jw, max |r| and
// of |grad r| jw, |grad r|^2 jw, max |grad r|
__global__ void k_norms(int64_t nq, int bs, const double *__restrict__ jw, const double *__restrict__ u, const double *__restrict__ du,
                        const double *__restrict__ uu, const double *__restrict__ duu, double *__restrict__ part) {
  __shared__ double red[6][256];
  double a[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nq; q += (int64_t)gridDim.x * blockDim.x) {
    const double w = jw[q];
    for (int i = 0; i < bs; i++) {
      if (uu) {
        const double r = uu[q * bs + i] - u[q * bs + i];
        a[0] += fabs(r) * w;
        a[1] += r * r * w;
        a[2] = fmax(a[2], fabs(r));
      }
      if (duu) {
        const double *e = duu + (q * bs + i) * 3, *g = du + (q * bs + i) * 3;
        const double d0 = e[0] - g[0], d1 = e[1] - g[1], d2 = e[2] - g[2];
        const double gr2 = d0 * d0 + d1 * d1 + d2 * d2, ga = sqrt(gr2);
        a[3] += ga * w;
        a[4] += gr2 * w;
        a[5] = fmax(a[5], ga);
      }
    }
  }
  for (int k = 0; k < 6; k++) red[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < 6; k++)
        red[k][threadIdx.x] = (k == 2 || k == 5) ? fmax(red[k][threadIdx.x], red[k][threadIdx.x + st]) : red[k][threadIdx.x] + red[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
}

}  // namespace

extern "C" {

dErr dRulesetIteratorCreate(dFS fs, dQuadratureMethod method, dRulesetIterator *it) {
  if (!fs || !it) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  if (method != dQUADRATURE_METHOD_FAST && method != dQUADRATURE_METHOD_SPARSE)
    return set_error("batched iterator supports FAST and SPARSE rules");
  if (method == dQUADRATURE_METHOD_SPARSE && !fs->uniform) return set_error("SPARSE batched iterator needs a uniform-order space");
  if (!fs->jac) return set_error("dFS was created without a dJacobi");
  _p_dRulesetIterator *I = new _p_dRulesetIterator();
  I->fs = fs;
  I->nel = fs->nelem;
  I->nq = fs->nq;  // FAST: (p+1)^3 points per element; SPARSE: set below from the rule
  std::map<std::array<int, 3>, std::vector<int32_t>> groups;  // order triple -> elements, ascending
  for (int64_t e = 0; e < fs->nelem; e++) groups[{fs->edeg[3 * e], fs->edeg[3 * e + 1], fs->edeg[3 * e + 2]}].push_back((int32_t)e);
  I->per_point_w = groups.size() > 1;
  std::vector<double> w(I->per_point_w ? std::max<int64_t>(fs->nq, 1) : 0);
  for (auto &kv : groups) {
    IterBucket B;
    const dInt deg[3] = {kv.first[0], kv.first[1], kv.first[2]}, one[3] = {1, 1, 1};
    const dInt ro[3] = {2 * deg[0], 2 * deg[1], 2 * deg[2]};
    dErr e = jacobi_efs(fs->jac, deg, method, ro, &B.efs);
    if (!e) e = jacobi_efs(fs->jac, one, method, ro, &B.cefs);
    if (e) {
      dRulesetIteratorDestroy(&I);
      return e;
    }
    B.nel = (int64_t)kv.second.size();
    const Basis1D *b = B.efs->b;
    const int Q = b[0].Q * b[1].Q * b[2].Q;
    if (method == dQUADRATURE_METHOD_SPARSE) I->nq = I->nel * Q;  // uniform: one bucket
    std::vector<double> wq(Q);
    for (int i = 0; i < b[0].Q; i++)
      for (int j = 0; j < b[1].Q; j++)
        for (int k = 0; k < b[2].Q; k++) wq[(i * b[1].Q + j) * b[2].Q + k] = b[0].w[i] * b[1].w[j] * b[2].w[k];
    if (I->per_point_w) {
      for (int32_t el : kv.second) std::copy(wq.begin(), wq.end(), w.begin() + fs->qoff[el]);
      CUCHK(cudaMalloc(&B.d_elist, B.nel * sizeof(int32_t)));
      CUCHK(cudaMemcpy(B.d_elist, kv.second.data(), B.nel * sizeof(int32_t), cudaMemcpyHostToDevice));
    } else {
      w = wq;
    }
    I->buckets.push_back(B);
  }
  const int bs = fs->bs;
  const int64_t nq = std::max<int64_t>(I->nq, 1);
  CUCHK(cudaMalloc(&I->xexp, fs->nexp * bs * sizeof(double)));
  CUCHK(cudaMalloc(&I->yexp, fs->nexp * bs * sizeof(double)));
  CUCHK(cudaMalloc(&I->jw, nq * sizeof(double)));
  CUCHK(cudaMalloc(&I->x, nq * 3 * sizeof(double)));
  CUCHK(cudaMalloc(&I->dx, nq * 9 * sizeof(double)));
  CUCHK(cudaMalloc(&I->jinv, nq * 9 * sizeof(double)));
  CUCHK(cudaMalloc(&I->u, nq * bs * sizeof(double)));
  CUCHK(cudaMalloc(&I->du, nq * bs * 3 * sizeof(double)));
  CUCHK(cudaMalloc(&I->v, nq * bs * sizeof(double)));
  CUCHK(cudaMalloc(&I->dv, nq * bs * 3 * sizeof(double)));
  CUCHK(cudaMalloc(&I->d_w, std::max<size_t>(w.size(), 1) * sizeof(double)));
  CUCHK(cudaMemcpy(I->d_w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice));
  *it = I;
  return 0;
}

dErr dRulesetIteratorDestroy(dRulesetIterator *it) {
  if (!it || !*it) return 0;
  _p_dRulesetIterator *I = *it;
  for (double *p : {I->xexp, I->yexp, I->jw, I->x, I->dx, I->jinv, I->u, I->du, I->v, I->dv, I->d_w}) cudaFree(p);
  for (IterBucket &B : I->buckets) cudaFree(B.d_elist);
  delete I;
  *it = nullptr;
  return 0;
}

dErr dRulesetIteratorStart(dRulesetIterator it, const dScalar *g, dFSHomogeneousMode hmode) {
  if (!it) return set_error("null iterator");
  _p_dFS *fs = it->fs;
  if (g) DCHK(fs_expand(fs, g, it->xexp, hmode == dFS_INHOMOGENEOUS, 0));
  else CUCHK(cudaMemsetAsync(it->xexp, 0, fs->nexp * fs->bs * sizeof(double), fs->stream));
  CUCHK(cudaMemsetAsync(it->yexp, 0, fs->nexp * fs->bs * sizeof(double), fs->stream));
  it->started = true;
  it->applied = false;
  return 0;
}

dErr dRulesetIteratorGetPatchApplied(dRulesetIterator it, int64_t *nq, const dReal **jw, const dScalar **x, const dScalar **dx,
                                     const dScalar **u, const dScalar **du, dScalar **v, dScalar **dv) {
  if (!it || !it->started) return set_error("dRulesetIteratorStart first");
  _p_dFS *fs = it->fs;
  cudaStream_t s = fs->stream;
  const int bs = fs->bs;
  const int Q = it->nel ? (int)(it->nq / it->nel) : 1;  // points per element when the order is uniform
  if (!it->applied && it->nq) {
    // link 0 (coordinates): INTERP and GRAD without mapping, then the physical map; coordinates are [nelem][8][3]
    for (const IterBucket &B : it->buckets) {
      const int32_t *qo = B.d_elist ? fs->d_qoff : nullptr;
      DCHK(efs_apply_list(B.cefs, B.nel, B.d_elist, nullptr, qo, nullptr, 3, fs->d_coords, it->x, dAPPLY_INTERP, INSERT_VALUES, s));
      DCHK(efs_apply_list(B.cefs, B.nel, B.d_elist, nullptr, qo, nullptr, 3, fs->d_coords, it->dx, dAPPLY_GRAD, INSERT_VALUES, s));
    }
    int *neg;
    CUCHK(cudaMalloc(&neg, sizeof(int)));
    CUCHK(cudaMemsetAsync(neg, 0, sizeof(int), s));
    k_physical<<<(unsigned)((it->nq + 255) / 256), 256, 0, s>>>(it->nq, Q, it->per_point_w, it->d_w, it->dx, it->jinv, it->jw, neg);
    CUCHK(cudaGetLastError());
    int hneg = 0;
    CUCHK(cudaMemcpyAsync(&hneg, neg, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUCHK(cudaStreamSynchronize(s));
    cudaFree(neg);
    if (hneg) return set_error("Negative Jacobian in the element geometry");
    // link 1 (field): INTERP and GRAD mapped to physical coordinates
    for (const IterBucket &B : it->buckets) {
      const int32_t *xo = B.d_elist ? fs->d_xstart : nullptr, *qo = B.d_elist ? fs->d_qoff : nullptr;
      DCHK(efs_apply_list(B.efs, B.nel, B.d_elist, xo, qo, nullptr, bs, it->xexp, it->u, dAPPLY_INTERP, INSERT_VALUES, s));
      DCHK(efs_apply_list(B.efs, B.nel, B.d_elist, xo, qo, it->jinv, bs, it->xexp, it->du, dAPPLY_GRAD, INSERT_VALUES, s));
    }
    CUCHK(cudaMemsetAsync(it->v, 0, it->nq * bs * sizeof(double), s));
    CUCHK(cudaMemsetAsync(it->dv, 0, it->nq * bs * 3 * sizeof(double), s));
  }
  it->applied = true;
  if (nq) *nq = it->nq;
  if (jw) *jw = it->jw;
  if (x) *x = it->x;
  if (dx) *dx = it->dx;
  if (u) *u = it->u;
  if (du) *du = it->du;
  if (v) *v = it->v;
  if (dv) *dv = it->dv;
  return 0;
}

dErr dRulesetIteratorCommitPatchApplied(dRulesetIterator it, InsertMode imode, int use_v, int use_dv) {
  if (!it || !it->applied) return set_error("dRulesetIteratorGetPatchApplied first");
  _p_dFS *fs = it->fs;
  if (!it->nq) return 0;
  for (const IterBucket &B : it->buckets) {  // every element is in one bucket: per-element INSERT is exact
    const int32_t *qo = B.d_elist ? fs->d_qoff : nullptr, *xo = B.d_elist ? fs->d_xstart : nullptr;
    InsertMode m = imode;
    if (use_v) {
      DCHK(efs_apply_list(B.efs, B.nel, B.d_elist, qo, xo, it->jinv, fs->bs, it->v, it->yexp, dAPPLY_INTERP_TRANSPOSE, m, fs->stream));
      m = ADD_VALUES;
    }
    if (use_dv)
      DCHK(efs_apply_list(B.efs, B.nel, B.d_elist, qo, xo, it->jinv, fs->bs, it->dv, it->yexp, dAPPLY_GRAD_TRANSPOSE, m, fs->stream));
  }
  return 0;
}

dErr dRulesetIteratorFinish(dRulesetIterator it, dScalar *y, InsertMode imode) {
  if (!it || !it->started) return set_error("dRulesetIteratorStart first");
  it->started = false;
  if (!y) return 0;
  return fs_restrict(it->fs, it->yexp, y, imode == ADD_VALUES);
}

// dNormsStart/Update/Finish (src/util/util.c:110-153) over all points of the last GetPatchApplied: errors of
// the field against exact values at the same points, uerr = {L1, L2, Linf} of u - exact_u and gerr = the same
// of |grad u - exact_du| (exact arrays on the device, [nq][bs] and [nq][bs][3]; either may be NULL)
dErr dRulesetIteratorErrorNorms(dRulesetIterator it, const dScalar *exact_u, const dScalar *exact_du, dReal uerr[3], dReal gerr[3]) {
  if (!it || !it->applied) return set_error("dRulesetIteratorGetPatchApplied first");
  cudaStream_t s = it->fs->stream;
  constexpr int NB = 512;
  double *part;
  CUCHK(cudaMalloc(&part, NB * 6 * sizeof(double)));
  k_norms<<<NB, 256, 0, s>>>(it->nq, it->fs->bs, it->jw, it->u, it->du, exact_u, exact_du, part);
  CUCHK(cudaGetLastError());
  std::vector<double> h(NB * 6);
  CUCHK(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUCHK(cudaStreamSynchronize(s));
  cudaFree(part);
  double a[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < NB; b++)
    for (int k = 0; k < 6; k++) a[k] = (k == 2 || k == 5) ? std::max(a[k], h[b * 6 + k]) : a[k] + h[b * 6 + k];
  if (uerr) uerr[0] = a[0], uerr[1] = std::sqrt(a[1]), uerr[2] = a[2];
  if (gerr) gerr[0] = a[3], gerr[1] = std::sqrt(a[4]), gerr[2] = a[5];
  return 0;
}

}  // extern "C"
