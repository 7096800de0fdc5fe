// Facet rules and boundary integrals on the weak boundary sets: a batched facet iterator.
//
// Rules follow dQuadratureGetFacetRules_Tensor_Private (src/jacobi/quadrature/impls/tensor/tensorquad.c:309-355):
// the tensor Gauss rule on the reference quad [-1,1]^2 is mapped onto side s of the reference hex by
// xi = R_s (X, Y, 0) + t_s (the side transforms of tensorquad.c:324-331) with the node map of
// dRuleGetNodeWeight_Transformed (tensorquad.c:224-242). The weak sets are the boundary sets registered with
// dFSBSTATUS_WEAK (the reference's weakFace set, src/fs/interface/fsbuild.c:87-90). The reference stops there: its
// quad rules have no node/weight accessor (src/jacobi/quadrature/impls/tensor/ruletopo.c:184) and no caller
// evaluates a facet integral. This file completes the path on the device:
//   Get:    per facet point the physical point and the outward area vector t_X x t_Y of the trilinear coordinate
//           map (tangents t_X, t_Y = J R_s[:,0], J R_s[:,1]), jw = w_X w_Y |t_X x t_Y|, the unit normal, and
//           the field u at the point from the element's face nodes (along the normal the GLL basis is 1 at the
//           end node and 0 at the others);
//   Commit: y_exp[i] += sum_q phi_i(xi_q) v_q over each facet's points, one block per element so the facets of
//           an element (edges and corners of the box) add into shared nodes in a fixed order;
//   Finish: the deterministic E^T restriction of the volume path.
// The 1-D GLL Lagrange values at the facet's Gauss points come from tables built on the host: evaluating them
// in the kernels put FP64 divisions on the (narrow) FP64 pipe and made a boundary cycle 4x slower. Start and
// Finish still touch the whole expanded vector (expand, zero, restrict), which dominates what is left.
#include <cmath>
#include <vector>

#include "internal.h"

using namespace dgb;

dErr fs_expand(_p_dFS *fs, const double *g, double *x, bool inhomogeneous, int add);
dErr fs_restrict(_p_dFS *fs, const double *x, double *g, int add);

namespace {

// xi = R (X, Y, 0) + t per hex side (tensorquad.c:324-331); the translation is the outward normal
constexpr double kSideR[6][3][3] = {
    {{1, 0, 0}, {0, 0, -1}, {0, 1, 0}},  {{0, 0, 1}, {1, 0, 0}, {0, 1, 0}},   {{-1, 0, 0}, {0, 0, 1}, {0, 1, 0}},
    {{0, 0, -1}, {-1, 0, 0}, {0, 1, 0}}, {{0, 1, 0}, {1, 0, 0}, {0, 0, -1}}, {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};
constexpr double kSideT[6][3] = {{0, -1, 0}, {1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, 0, -1}, {0, 0, 1}};

struct FacetTables {
  double gx[MAXP + 1][MAXP], gw[MAXP + 1][MAXP];  // n-point Gauss rule (the FAST rule of order 2(n-1))
  // L[0][n][a][i] = phi_i(+X_a), L[1][n][a][i] = phi_i(-X_a): the n GLL Lagrange functions at the n Gauss
  // points (a facet axis runs along +xi or -xi of its reference direction)
  double L[2][MAXP + 1][MAXP][MAXP];
  double R[6][3][3], t[6][3];
  int cx[6], cy[6], cn[6];  // reference direction of the facet's X, Y and normal axes
  int sx[6], sy[6];         // 0: the axis runs along +xi, 1: along -xi
};

struct FacetGeom {
  int P[3], cx, cy, cn, iN;
  int64_t stride[3], base;
};

__device__ __forceinline__ FacetGeom facet_geom(const FacetTables &T, int e, int s, const int32_t *edeg, const int32_t *xstart) {
  FacetGeom g;
  for (int c = 0; c < 3; c++) g.P[c] = edeg[3 * e + c] + 1;
  g.cx = T.cx[s], g.cy = T.cy[s], g.cn = T.cn[s];
  g.stride[0] = (int64_t)g.P[1] * g.P[2], g.stride[1] = g.P[2], g.stride[2] = 1;
  g.iN = T.t[s][g.cn] > 0 ? g.P[g.cn] - 1 : 0;
  g.base = xstart[e] + g.iN * g.stride[g.cn];
  return g;
}

// one thread per facet point
__global__ void k_facet_points(int64_t nq, int bs, const int32_t *__restrict__ qfacet, const int32_t *__restrict__ foff,
                               const int32_t *__restrict__ fel, const int32_t *__restrict__ fside, const int32_t *__restrict__ edeg,
                               const int32_t *__restrict__ xstart, const double *__restrict__ coords, const FacetTables *__restrict__ Tp,
                               const double *__restrict__ xexp, double *__restrict__ jw, double *__restrict__ x,
                               double *__restrict__ nrm, double *__restrict__ u) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const FacetTables &T = *Tp;
  const int f = qfacet[q], e = fel[f], s = fside[f];
  const FacetGeom G = facet_geom(T, e, s, edeg, xstart);
  const int nX = G.P[G.cx], nY = G.P[G.cy], loc = (int)(q - foff[f]), a = loc / nY, b = loc - a * nY;
  const double X = T.gx[nX][a], Y = T.gx[nY][b], w = T.gw[nX][a] * T.gw[nY][b];
  double xi[3];
  for (int c = 0; c < 3; c++) xi[c] = T.R[s][c][0] * X + T.R[s][c][1] * Y + T.t[s][c];
  // trilinear coordinate map; corner k in tensor order: bit 2 -> xi_0, bit 1 -> xi_1, bit 0 -> xi_2
  const double *C = coords + (int64_t)e * 24;
  double xp[3] = {0, 0, 0}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int k = 0; k < 8; k++) {
    const double s0 = (k & 4) ? 1.0 : -1.0, s1 = (k & 2) ? 1.0 : -1.0, s2 = (k & 1) ? 1.0 : -1.0;
    const double l0 = 0.5 * (1 + s0 * xi[0]), l1 = 0.5 * (1 + s1 * xi[1]), l2 = 0.5 * (1 + s2 * xi[2]);
    const double N = l0 * l1 * l2, d0 = 0.5 * s0 * l1 * l2, d1 = 0.5 * s1 * l0 * l2, d2 = 0.5 * s2 * l0 * l1;
    for (int d = 0; d < 3; d++) {
      const double v = C[3 * k + d];
      xp[d] += N * v;
      J[d][0] += d0 * v;
      J[d][1] += d1 * v;
      J[d][2] += d2 * v;
    }
  }
  double tx[3], ty[3];
  for (int d = 0; d < 3; d++) {
    tx[d] = J[d][0] * T.R[s][0][0] + J[d][1] * T.R[s][1][0] + J[d][2] * T.R[s][2][0];
    ty[d] = J[d][0] * T.R[s][0][1] + J[d][1] * T.R[s][1][1] + J[d][2] * T.R[s][2][1];
  }
  const double cr[3] = {tx[1] * ty[2] - tx[2] * ty[1], tx[2] * ty[0] - tx[0] * ty[2], tx[0] * ty[1] - tx[1] * ty[0]};
  const double ar = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
  jw[q] = w * ar;
  for (int d = 0; d < 3; d++) {
    x[3 * q + d] = xp[d];
    nrm[3 * q + d] = cr[d] / ar;
  }
  const double *LX = T.L[T.sx[s]][nX][a], *LY = T.L[T.sy[s]][nY][b];
  for (int c = 0; c < bs; c++) {
    double acc = 0;
    for (int i = 0; i < G.P[G.cx]; i++) {
      double r = 0;
      for (int j = 0; j < G.P[G.cy]; j++) r += LY[j] * xexp[(G.base + i * G.stride[G.cx] + j * G.stride[G.cy]) * bs + c];
      acc += LX[i] * r;
    }
    u[q * bs + c] = acc;
  }
}

// one block per element with weak facets; its facets in order, one thread per face node
__global__ void k_facet_commit(int bs, const int32_t *__restrict__ bfoff, const int32_t *__restrict__ foff, const int32_t *__restrict__ fel,
                               const int32_t *__restrict__ fside, const int32_t *__restrict__ edeg, const int32_t *__restrict__ xstart,
                               const FacetTables *__restrict__ Tp, const double *__restrict__ v, double *__restrict__ yexp) {
  const FacetTables &T = *Tp;
  for (int f = bfoff[blockIdx.x]; f < bfoff[blockIdx.x + 1]; f++) {
    const int e = fel[f], s = fside[f];
    const FacetGeom G = facet_geom(T, e, s, edeg, xstart);
    const int PX = G.P[G.cx], PY = G.P[G.cy];
    for (int t = threadIdx.x; t < PX * PY; t += blockDim.x) {
      const int i = t / PY, j = t - i * PY;
      double acc[3] = {0, 0, 0};
      for (int a = 0; a < PX; a++) {
        const double li = T.L[T.sx[s]][PX][a][i];
        for (int b = 0; b < PY; b++) {
          const double l = li * T.L[T.sy[s]][PY][b][j];
          const int64_t q = foff[f] + a * PY + b;
          for (int c = 0; c < bs; c++) acc[c] += l * v[q * bs + c];
        }
      }
      double *y = yexp + (G.base + i * G.stride[G.cx] + j * G.stride[G.cy]) * bs;
      for (int c = 0; c < bs; c++) y[c] += acc[c];
    }
    __syncthreads();
  }
}

}  // namespace

struct _p_dFacetIterator {
  dFS fs;
  int64_t nfacet = 0, nq = 0, nbel = 0;
  std::vector<int32_t> elem, side, qoff;
  int32_t *d_qfacet = nullptr, *d_foff = nullptr, *d_fel = nullptr, *d_fside = nullptr, *d_bfoff = nullptr;
  FacetTables *d_tab = nullptr;
  double *xexp = nullptr, *yexp = nullptr, *jw = nullptr, *x = nullptr, *nrm = nullptr, *u = nullptr, *v = nullptr;
  bool started = false, applied = false;
};

dErr dFSGetFacetRule(dInt side, dQuadratureMethod method, dInt order, dInt *nnodes, dReal *nodes, dReal *weights) {
  if (side < 0 || side > 5) return set_error("hex side %d out of range 0..5", side);
  if (method != dQUADRATURE_METHOD_FAST) return set_error("facet rules: FAST (Gauss) rules only");
  double x[MAXQ], w[MAXQ];
  if (order < 0 || order > 16) return set_error("facet rule order %d out of range 0..16", order);
  const int n = rule_1d(method, order, x, w);
  if (n <= 0) return set_error("no rule of order %d", order);
  if (nnodes) *nnodes = n * n;
  for (int a = 0; a < n; a++)
    for (int b = 0; b < n; b++) {
      const int i = a * n + b;
      if (nodes)
        for (int c = 0; c < 3; c++) nodes[3 * i + c] = kSideR[side][c][0] * x[a] + kSideR[side][c][1] * x[b] + kSideT[side][c];
      if (weights) weights[i] = w[a] * w[b];
    }
  return 0;
}

dErr dFacetIteratorCreate(dFS fs, dQuadratureMethod method, dFacetIterator *it) {
  if (!fs || !it) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  if (method != dQUADRATURE_METHOD_FAST) return set_error("facet iterator supports FAST rules");
  const _p_dMesh *m = fs->mesh;
  const int64_t R0 = m->nv + m->ne + m->nf;
  const int setbit[6] = {0, 0, 0, 0, 2, 1};  // generator face sets 0..3 -> 100, 4 -> 300, 5 -> 200
  _p_dFacetIterator *I = new _p_dFacetIterator();
  I->fs = fs;
  FacetTables T;
  for (int n = 1; n <= MAXP; n++) {
    double x[MAXQ], w[MAXQ], gll[MAXP], lw[MAXP], der[MAXP];
    rule_1d(dQUADRATURE_METHOD_FAST, 2 * (n - 1), x, w);
    for (int i = 0; i < n; i++) T.gx[n][i] = x[i], T.gw[n][i] = w[i];
    if (n >= 2) lobatto_rule(n, gll, lw);
    else gll[0] = 0;
    for (int a = 0; a < n; a++) {
      if (n >= 2) {
        lagrange(n, gll, x[a], T.L[0][n][a], der);
        lagrange(n, gll, -x[a], T.L[1][n][a], der);
      } else {
        T.L[0][n][a][0] = T.L[1][n][a][0] = 1.0;
      }
    }
  }
  for (int s = 0; s < 6; s++) {
    for (int c = 0; c < 3; c++) {
      for (int k = 0; k < 3; k++) T.R[s][c][k] = kSideR[s][c][k];
      T.t[s][c] = kSideT[s][c];
      if (kSideR[s][c][0] != 0) T.cx[s] = c, T.sx[s] = kSideR[s][c][0] < 0;
      if (kSideR[s][c][1] != 0) T.cy[s] = c, T.sy[s] = kSideR[s][c][1] < 0;
      if (kSideR[s][c][2] != 0) T.cn[s] = c;
    }
  }
  std::vector<int32_t> bfoff(1, 0), qfacet;
  I->qoff.push_back(0);
  for (int64_t r = 0; r < m->nr; r++) {
    bool any = false;
    for (int s = 0; s < 6; s++) {
      const int st = m->fset[m->adjind[m->adjoff[R0 + r] + s]];
      if (st < 0 || !((fs->weak_mask >> setbit[st]) & 1)) continue;
      const int nX = fs->edeg[3 * r + T.cx[s]] + 1, nY = fs->edeg[3 * r + T.cy[s]] + 1;
      I->elem.push_back((int32_t)r);
      I->side.push_back(s);
      qfacet.insert(qfacet.end(), (size_t)nX * nY, (int32_t)(I->elem.size() - 1));
      I->qoff.push_back(I->qoff.back() + nX * nY);
      any = true;
    }
    if (any) bfoff.push_back((int32_t)I->elem.size());
  }
  I->nfacet = (int64_t)I->elem.size();
  I->nq = I->qoff.back();
  I->nbel = (int64_t)bfoff.size() - 1;
  const int bs = fs->bs;
  auto up = [&](int32_t **d, const std::vector<int32_t> &h) -> dErr {
    CUCHK(cudaMalloc(d, std::max<size_t>(h.size(), 1) * sizeof(int32_t)));
    if (!h.empty()) CUCHK(cudaMemcpy(*d, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    return 0;
  };
  dErr e = up(&I->d_qfacet, qfacet);
  if (!e) e = up(&I->d_foff, I->qoff);
  if (!e) e = up(&I->d_fel, I->elem);
  if (!e) e = up(&I->d_fside, I->side);
  if (!e) e = up(&I->d_bfoff, bfoff);
  if (e) {
    dFacetIteratorDestroy(&I);
    return e;
  }
  const int64_t nq = std::max<int64_t>(I->nq, 1);
  CUCHK(cudaMalloc(&I->d_tab, sizeof(FacetTables)));
  CUCHK(cudaMemcpy(I->d_tab, &T, sizeof(FacetTables), cudaMemcpyHostToDevice));
  CUCHK(cudaMalloc(&I->xexp, fs->nexp * bs * sizeof(double)));
  CUCHK(cudaMalloc(&I->yexp, fs->nexp * bs * sizeof(double)));
  CUCHK(cudaMalloc(&I->jw, nq * sizeof(double)));
  CUCHK(cudaMalloc(&I->x, nq * 3 * sizeof(double)));
  CUCHK(cudaMalloc(&I->nrm, nq * 3 * sizeof(double)));
  CUCHK(cudaMalloc(&I->u, nq * bs * sizeof(double)));
  CUCHK(cudaMalloc(&I->v, nq * bs * sizeof(double)));
  *it = I;
  return 0;
}

dErr dFacetIteratorDestroy(dFacetIterator *it) {
  if (!it || !*it) return 0;
  _p_dFacetIterator *I = *it;
  for (int32_t *p : {I->d_qfacet, I->d_foff, I->d_fel, I->d_fside, I->d_bfoff}) cudaFree(p);
  for (double *p : {I->xexp, I->yexp, I->jw, I->x, I->nrm, I->u, I->v}) cudaFree(p);
  cudaFree(I->d_tab);
  delete I;
  *it = nullptr;
  return 0;
}

dErr dFacetIteratorGetFacets(dFacetIterator it, int64_t *nfacets, const dInt **elem, const dInt **side, const dInt **qoffset) {
  if (!it) return set_error("null iterator");
  if (nfacets) *nfacets = it->nfacet;
  if (elem) *elem = it->elem.data();
  if (side) *side = it->side.data();
  if (qoffset) *qoffset = it->qoff.data();
  return 0;
}

dErr dFacetIteratorStart(dFacetIterator it, const dScalar *g, dFSHomogeneousMode hmode) {
  if (!it) return set_error("null iterator");
  _p_dFS *fs = it->fs;
  if (g) DCHK(fs_expand(fs, g, it->xexp, hmode == dFS_INHOMOGENEOUS, 0));
  else CUCHK(cudaMemsetAsync(it->xexp, 0, fs->nexp * fs->bs * sizeof(double), fs->stream));
  CUCHK(cudaMemsetAsync(it->yexp, 0, fs->nexp * fs->bs * sizeof(double), fs->stream));
  it->started = true;
  it->applied = false;
  return 0;
}

dErr dFacetIteratorGetApplied(dFacetIterator it, int64_t *nq, const dReal **jw, const dReal **x, const dReal **normal,
                              const dScalar **u, dScalar **v) {
  if (!it || !it->started) return set_error("dFacetIteratorStart first");
  _p_dFS *fs = it->fs;
  cudaStream_t s = fs->stream;
  if (!it->applied) {
    if (it->nq) {
      k_facet_points<<<(unsigned)((it->nq + 127) / 128), 128, 0, s>>>(it->nq, fs->bs, it->d_qfacet, it->d_foff, it->d_fel, it->d_fside,
                                                                      fs->d_edeg, fs->d_xstart, fs->d_coords, it->d_tab, it->xexp,
                                                                      it->jw, it->x, it->nrm, it->u);
      CUCHK(cudaGetLastError());
      CUCHK(cudaMemsetAsync(it->v, 0, it->nq * fs->bs * sizeof(double), s));
    }
    it->applied = true;
  }
  if (nq) *nq = it->nq;
  if (jw) *jw = it->jw;
  if (x) *x = it->x;
  if (normal) *normal = it->nrm;
  if (u) *u = it->u;
  if (v) *v = it->v;
  return 0;
}

dErr dFacetIteratorCommit(dFacetIterator it, InsertMode imode) {
  if (!it || !it->applied) return set_error("dFacetIteratorGetApplied first");
  _p_dFS *fs = it->fs;
  if (imode == INSERT_VALUES) CUCHK(cudaMemsetAsync(it->yexp, 0, fs->nexp * fs->bs * sizeof(double), fs->stream));
  else if (imode != ADD_VALUES) return set_error("InsertMode %d not supported", (int)imode);
  if (it->nbel) {
    k_facet_commit<<<(unsigned)it->nbel, 128, 0, fs->stream>>>(fs->bs, it->d_bfoff, it->d_foff, it->d_fel, it->d_fside, fs->d_edeg,
                                                              fs->d_xstart, it->d_tab, it->v, it->yexp);
    CUCHK(cudaGetLastError());
  }
  return 0;
}

dErr dFacetIteratorFinish(dFacetIterator it, dScalar *y, InsertMode imode) {
  if (!it || !it->started) return set_error("dFacetIteratorStart first");
  it->started = false;
  if (!y) return 0;
  return fs_restrict(it->fs, it->yexp, y, imode == ADD_VALUES);
}
