// dRuleset and dRulesetIterator, batched device form (src/fs/interface/fsruleset.c, fsrulesetit.c:129-938).
//
// The reference walks elements one at a time: GetPatchApplied evaluates link 0 (the coordinate space: INTERP and
// GRAD of the Q1 coordinates, dRuleComputePhysical) and every further link (a field space added with
// dRulesetIteratorAddFS: INTERP, and GRAD mapped by J^-1) at the element's quadrature points, the caller's
// q-function fills v/dv, CommitPatchApplied integrates them back (INTERP_TRANSPOSE, GRAD_TRANSPOSE) into each
// link's expanded test vector, and Finish restricts those into the test vectors given at Start. Here one
// Start / GetPatchApplied / CommitPatchApplied / Finish cycle covers all elements: HasPatch is true once after
// Start and NextPatch ends the loop, so the reference's while loop runs its body once. Arrays are element-natural
// per element, elements back to back (element e's points start at the ruleset's point offset of e), and every
// evaluation is one batched dEFSApply launch per group of elements that share their rule and the link's basis
// orders (one launch per link on a uniform-order space). FAST and SPARSE rules on any space, each element with the
// rule of its own orders; the SPARSE rule has 2 Gauss points in each GLL sub-interval, (2p)^3 points per element in
// tensor order: the p^3 patches of the reference's patch loop are the 2 x 2 x 2 blocks of it (patch bases on
// uniform-order spaces). The stash (AddStash / GetStash,
// fsrulesetit.c:779-798) is device memory: elembytes per element and nodebytes per point, for all elements.
#include <stdarg.h>

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

struct _p_dRuleset {
  dFS fs = nullptr;  // the space whose degrees chose the rules (rule order 2p per direction, fsruleset.c:32-37)
  dQuadratureMethod method = dQUADRATURE_METHOD_FAST;
  int64_t nel = 0, nq = 0;
  std::vector<std::array<int, 3>> order;  // rule order per element
  std::vector<int32_t> qoff;              // first point of each element [nel+1]
  int32_t *d_qoff = nullptr;
  std::vector<double> w;                  // rule weight of every point
  double *d_w = nullptr;
  int refct = 1;
};

namespace {

struct IterBucket {
  dEFS efs = nullptr;
  int64_t nel = 0;
  int32_t *d_elist = nullptr;  // the bucket's elements; null: every element, contiguous (a single bucket)
};

struct ItLink {
  dFS fs = nullptr;
  int bs = 1;
  bool coords = false;  // link 0: the coordinate space
  std::vector<IterBucket> buckets;
  double *xexp = nullptr, *yexp = nullptr;
  double *u = nullptr, *du = nullptr, *v = nullptr, *dv = nullptr;
  const double *X = nullptr;  // trial vector of the current traversal (link 0: expanded coordinates)
  double *Y = nullptr;        // test vector restricted at Finish
  bool xinh = false;
  bool uvalid = false, duvalid = false;
};

void free_link(ItLink &L) {
  for (double *p : {L.xexp, L.yexp, L.u, L.du, L.v, L.dv}) cudaFree(p);
  for (IterBucket &B : L.buckets) cudaFree(B.d_elist);
  L = ItLink();
}

}  // namespace

struct _p_dRulesetIterator {
  _p_dRuleset *rset = nullptr;
  std::vector<ItLink> links;
  InsertMode imode = INSERT_VALUES;
  double *jinv = nullptr, *jw = nullptr;
  int64_t elembytes = 0, nodebytes = 0;
  unsigned char *stash_elem = nullptr, *stash_node = nullptr;
  bool started = false, has_patch = false, applied = false;
  // patch assembly arrays (SPARSE rules): per link, [nelem * npatches][...]
  std::vector<int32_t *> asm_rowcol;
  std::vector<double *> asm_interp, asm_deriv;
};

namespace {

void rset_release(_p_dRuleset *r) {
  if (!r || --r->refct > 0) return;
  cudaFree(r->d_qoff);
  cudaFree(r->d_w);
  delete r;
}

// dRuleComputePhysical (src/jacobi/interface/jacobi.c:383-414): J^-1 by cofactors, jw = w det J, det < 0 is an error
__global__ void k_physical(int64_t ntot, const double *__restrict__ w, const double *__restrict__ dx, double *__restrict__ jinv,
                           double *__restrict__ jw, int *neg) {
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
  jw[t] = w[t] * det;
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

// dEFSGetExplicitSparse_Tensor_Hex (efstopo.c:660-717) for every element of a uniform-order space at once: one
// thread per (element, patch, point); cjinv (element-natural, [nq][9]) read at the reference's index pidx*8+q
__global__ void k_patch_assembly(int64_t nelem, int px, int py, int pz, const int32_t *__restrict__ xstart, const double *__restrict__ cjinv,
                                 int Qe, int32_t *__restrict__ rowcol, double *__restrict__ interp, double *__restrict__ deriv) {
  const int npatch = px * py * pz;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nelem * npatch * 8) return;
  const int q = (int)(t & 7);
  const int64_t ep = t >> 3;
  const int64_t e = ep / npatch;
  const int pidx = (int)(ep - e * npatch);
  const int i = pidx / (py * pz), j = (pidx / pz) % py, k = pidx % pz;
  const double s1 = 0.78867513459481287, s0 = 0.21132486540518713;
  const double I1[2][2] = {{s1, s0}, {s0, s1}}, D1[2][2] = {{-1., 1.}, {-1., 1.}};
  const int ii = q >> 2, jj = (q >> 1) & 1, kk = q & 1;
  if (q == 0)
    for (int b = 0; b < 8; b++) {
      const int bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
      rowcol[ep * 8 + b] = xstart[e] + ((i + bi) * (py + 1) + j + bj) * (pz + 1) + k + bk;
    }
  double M[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (cjinv) {
    const double *c = cjinv + ((int64_t)e * Qe + pidx * 8 + q) * 9;
    for (int l = 0; l < 9; l++) M[l] = c[l];
  }
  for (int b = 0; b < 8; b++) {
    const int bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
    const int64_t off = (ep * 8 + q) * 8 + b;
    const double dX = D1[ii][bi] * I1[jj][bj] * I1[kk][bk], dY = I1[ii][bi] * D1[jj][bj] * I1[kk][bk], dZ = I1[ii][bi] * I1[jj][bj] * D1[kk][bk];
    interp[off] = I1[ii][bi] * I1[jj][bj] * I1[kk][bk];
    for (int l = 0; l < 3; l++) deriv[off * 3 + l] = dX * M[0 * 3 + l] + dY * M[1 * 3 + l] + dZ * M[2 * 3 + l];
  }
}

// buckets of a link: elements grouped by (the link's basis orders, the ruleset's rule orders)
dErr link_buckets(_p_dRuleset *R, ItLink &L) {
  _p_dFS *fs = L.fs;
  std::map<std::array<int, 6>, std::vector<int32_t>> groups;
  for (int64_t e = 0; e < R->nel; e++) {
    const std::array<int, 6> key = {L.coords ? 1 : fs->edeg[3 * e], L.coords ? 1 : fs->edeg[3 * e + 1], L.coords ? 1 : fs->edeg[3 * e + 2],
                                    R->order[e][0], R->order[e][1], R->order[e][2]};
    groups[key].push_back((int32_t)e);
  }
  for (auto &kv : groups) {
    IterBucket B;
    const dInt deg[3] = {kv.first[0], kv.first[1], kv.first[2]}, ro[3] = {kv.first[3], kv.first[4], kv.first[5]};
    DCHK(jacobi_efs(fs->jac, deg, R->method, ro, &B.efs));
    B.nel = (int64_t)kv.second.size();
    if (groups.size() > 1) {
      CUCHK(cudaMalloc(&B.d_elist, B.nel * sizeof(int32_t)));
      CUCHK(cudaMemcpy(B.d_elist, kv.second.data(), B.nel * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    L.buckets.push_back(B);
  }
  return 0;
}

dErr lazy(double **p, int64_t n) {
  if (!*p) CUCHK(cudaMalloc(p, std::max<int64_t>(n, 1) * sizeof(double)));
  return 0;
}

// per-element offsets: expanded nodes of the link (coordinates: 8 per element, contiguous) and ruleset points
inline const int32_t *node_off(const ItLink &L, const IterBucket &B) { return B.d_elist && !L.coords ? L.fs->d_xstart : nullptr; }
inline const int32_t *pt_off(const _p_dRuleset *R, const IterBucket &B) { return B.d_elist ? R->d_qoff : nullptr; }

dErr link_eval(_p_dRulesetIterator *it, ItLink &L, bool want_u, bool want_du, cudaStream_t s) {
  _p_dRuleset *R = it->rset;
  const double *xin = L.coords ? (L.X ? L.X : L.fs->d_coords) : L.xexp;
  const double *jinv = L.coords ? nullptr : it->jinv;
  if (want_u && !L.uvalid) {
    DCHK(lazy(&L.u, R->nq * L.bs));
    for (const IterBucket &B : L.buckets)
      DCHK(efs_apply_list(B.efs, B.nel, B.d_elist, node_off(L, B), pt_off(R, B), nullptr, L.bs, xin, L.u, dAPPLY_INTERP, INSERT_VALUES, s));
    L.uvalid = true;
  }
  if (want_du && !L.duvalid) {
    DCHK(lazy(&L.du, R->nq * L.bs * 3));
    for (const IterBucket &B : L.buckets)
      DCHK(efs_apply_list(B.efs, B.nel, B.d_elist, node_off(L, B), pt_off(R, B), jinv, L.bs, xin, L.du, dAPPLY_GRAD, INSERT_VALUES, s));
    L.duvalid = true;
  }
  return 0;
}

dErr iterator_add_link(_p_dRulesetIterator *it, dFS fs, bool coords) {
  if (!fs || !fs->setup) return set_error("dRulesetIteratorAddFS: dFS not set up");
  if (!fs->jac) return set_error("dRulesetIteratorAddFS: dFS was created without a dJacobi");
  if (fs->mesh != it->rset->fs->mesh) return set_error("dRulesetIteratorAddFS: the space lives on another mesh than the ruleset");
  if (it->started) return set_error("dRulesetIteratorAddFS: the iterator is in a traversal (Finish first)");
  ItLink L;
  L.fs = fs;
  L.bs = coords ? 3 : fs->bs;
  L.coords = coords;
  dErr e = link_buckets(it->rset, L);
  if (e) {
    free_link(L);
    return e;
  }
  it->links.push_back(L);
  return 0;
}

}  // namespace

extern "C" {

dErr dFSGetPreferredQuadratureRuleSet(dFS fs, dQuadratureMethod method, dRuleset *rset) {
  if (!fs || !rset) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  if (!fs->jac) return set_error("dFS was created without a dJacobi");
  if (method != dQUADRATURE_METHOD_FAST && method != dQUADRATURE_METHOD_SPARSE)
    return set_error("dFSGetPreferredQuadratureRuleSet: FAST and SPARSE rules");
  if (jacobi_quad_family(fs->jac, method) != dGAUSS_LEGENDRE)
    return set_error("dFSGetPreferredQuadratureRuleSet: the element loops use Gauss-Legendre rules (the dJacobi's quadrature "
                     "was set to another family)");
  _p_dRuleset *R = new _p_dRuleset();
  R->fs = fs;
  R->method = method;
  R->nel = fs->nelem;
  R->order.resize(R->nel);
  R->qoff.assign(R->nel + 1, 0);
  std::map<std::array<int, 3>, std::vector<double>> wtab;  // rule order -> weights in tensor order
  for (int64_t e = 0; e < R->nel; e++) {
    R->order[e] = {2 * fs->edeg[3 * e], 2 * fs->edeg[3 * e + 1], 2 * fs->edeg[3 * e + 2]};
    auto &W = wtab[R->order[e]];
    if (W.empty()) {
      _p_dRule *rule;
      const int o[3] = {R->order[e][0], R->order[e][1], R->order[e][2]};
      dErr err = jacobi_rule(fs->jac, method, o, &rule);
      if (err) {
        delete R;
        return err;
      }
      dInt n;
      dRuleGetSize(rule, nullptr, &n);
      W.resize(n);
      dRuleGetNodeWeight(rule, nullptr, W.data());
    }
    R->qoff[e + 1] = R->qoff[e] + (int32_t)W.size();
  }
  R->nq = R->qoff[R->nel];
  R->w.resize(std::max<int64_t>(R->nq, 1));
  for (int64_t e = 0; e < R->nel; e++) {
    const auto &W = wtab[R->order[e]];
    std::copy(W.begin(), W.end(), R->w.begin() + R->qoff[e]);
  }
  CUCHK(cudaMalloc(&R->d_qoff, R->qoff.size() * sizeof(int32_t)));
  CUCHK(cudaMemcpy(R->d_qoff, R->qoff.data(), R->qoff.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  CUCHK(cudaMalloc(&R->d_w, R->w.size() * sizeof(double)));
  CUCHK(cudaMemcpy(R->d_w, R->w.data(), R->w.size() * sizeof(double), cudaMemcpyHostToDevice));
  *rset = R;
  return 0;
}

dErr dRulesetGetSize(dRuleset rset, dInt *size) {
  if (!rset || !size) return set_error("null argument");
  *size = (dInt)rset->nel;
  return 0;
}

dErr dRulesetGetNumPoints(dRuleset rset, int64_t *nq, const dInt **qoffset) {
  if (!rset) return set_error("null ruleset");
  if (nq) *nq = rset->nq;
  if (qoffset) *qoffset = rset->qoff.data();
  return 0;
}

dErr dRulesetDestroy(dRuleset *rset) {
  if (!rset || !*rset) return 0;
  rset_release(*rset);
  *rset = nullptr;
  return 0;
}

dErr dFSGetCoordinateFS(dFS fs, dFS *cfs) {
  if (!fs || !cfs) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  if (!fs->coord_fs) {
    dFS c = nullptr;
    DCHK(dFSCreate(fs->mesh, fs->jac, &c));
    dErr e = dFSSetDegree(c, 1, nullptr);
    if (!e) e = dFSSetBlockSize(c, 3);
    if (!e) e = dFSSetStream(c, fs->stream);
    if (!e) e = dFSSetUp(c);
    if (e) {
      dFSDestroy(&c);
      return e;
    }
    fs->coord_fs = c;
  }
  *cfs = fs->coord_fs;
  return 0;
}

dErr dRulesetCreateIterator(dRuleset rset, dFS cfs, dRulesetIterator *iter) {
  if (!rset || !cfs || !iter) return set_error("null argument");
  if (cfs->bs != 3 || !cfs->uniform || cfs->p != 1) return set_error("dRulesetCreateIterator: the coordinate space must be Q1 with block size 3");
  _p_dRulesetIterator *I = new _p_dRulesetIterator();
  I->rset = rset;
  rset->refct++;
  dErr e = iterator_add_link(I, cfs, true);
  if (!e) e = lazy(&I->jinv, rset->nq * 9);
  if (!e) e = lazy(&I->jw, rset->nq);
  if (e) {
    dRulesetIteratorDestroy(&I);
    return e;
  }
  *iter = I;
  return 0;
}

dErr dRulesetIteratorAddFS(dRulesetIterator it, dFS fs) {
  if (!it) return set_error("null iterator");
  return iterator_add_link(it, fs, false);
}

dErr dRulesetIteratorSetMode(dRulesetIterator it, InsertMode imode) {
  if (!it) return set_error("null iterator");
  if (imode != INSERT_VALUES && imode != ADD_VALUES) return set_error("invalid insert mode %d", (int)imode);
  it->imode = imode;
  return 0;
}

dErr dRulesetIteratorAddStash(dRulesetIterator it, dInt elembytes, dInt nodebytes) {
  if (!it) return set_error("null iterator");
  if (elembytes < 0 || nodebytes < 0) return set_error("negative stash size");
  cudaFree(it->stash_elem);
  cudaFree(it->stash_node);
  it->stash_elem = it->stash_node = nullptr;
  it->elembytes = elembytes;
  it->nodebytes = nodebytes;
  return 0;
}

dErr dRulesetIteratorGetStash(dRulesetIterator it, void *elemstash, void *nodestash) {
  if (!it) return set_error("null iterator");
  if (!it->started) return set_error("dRulesetIteratorStart first");
  if (elemstash) *(void **)elemstash = it->stash_elem;
  if (nodestash) *(void **)nodestash = it->stash_node;
  return 0;
}

dErr dRulesetIteratorStart(dRulesetIterator it, const dScalar *X, ...) {
  Range range_("dRulesetIteratorStart");
  if (!it) return set_error("null iterator");
  va_list ap;
  va_start(ap, X);
  dErr err = 0;
  for (size_t i = 0; i < it->links.size() && !err; i++) {
    ItLink &L = it->links[i];
    _p_dFS *fs = L.fs;
    if (i) X = va_arg(ap, const dScalar *);
    int xmode = dFS_HOMOGENEOUS;
    if (X) xmode = va_arg(ap, int);
    double *Y = va_arg(ap, dScalar *);
    if (Y) (void)va_arg(ap, int);  // the test vector's homogeneous mode: restriction to the global space ignores it
    L.X = X;
    L.Y = Y;
    L.xinh = xmode == dFS_INHOMOGENEOUS;
    L.uvalid = L.duvalid = false;
    if (!L.coords) {
      const int64_t ne = fs->nexp * fs->bs;
      if ((err = lazy(&L.xexp, ne))) break;
      if (X) err = fs_expand(fs, X, L.xexp, L.xinh, 0);
      else if (cudaMemsetAsync(L.xexp, 0, ne * sizeof(double), fs->stream) != cudaSuccess) err = set_error("memset failed");
    }
    if (!err && Y) {
      const int64_t ne = fs->nexp * L.bs;
      if (!(err = lazy(&L.yexp, ne)) && cudaMemsetAsync(L.yexp, 0, ne * sizeof(double), fs->stream) != cudaSuccess)
        err = set_error("memset failed");
    }
  }
  va_end(ap);
  if (err) return err;
  _p_dRuleset *R = it->rset;
  if ((it->elembytes && !it->stash_elem) || (it->nodebytes && !it->stash_node)) {
    cudaStream_t s = it->links[0].fs->stream;
    if (it->elembytes) {
      CUCHK(cudaMalloc(&it->stash_elem, (size_t)it->elembytes * std::max<int64_t>(R->nel, 1)));
      CUCHK(cudaMemsetAsync(it->stash_elem, 0, (size_t)it->elembytes * std::max<int64_t>(R->nel, 1), s));
    }
    if (it->nodebytes) {
      CUCHK(cudaMalloc(&it->stash_node, (size_t)it->nodebytes * std::max<int64_t>(R->nq, 1)));
      CUCHK(cudaMemsetAsync(it->stash_node, 0, (size_t)it->nodebytes * std::max<int64_t>(R->nq, 1), s));
    }
  }
  it->started = true;
  it->has_patch = true;
  it->applied = false;
  return 0;
}

int dRulesetIteratorHasPatch(dRulesetIterator it) { return it && it->started && it->has_patch; }

dErr dRulesetIteratorNextPatch(dRulesetIterator it) {
  if (!it || !it->started) return set_error("dRulesetIteratorStart first");
  it->has_patch = false;
  return 0;
}

dErr dRulesetIteratorGetPatchApplied(dRulesetIterator it, dInt *Q, const dReal **jw, dScalar **u, dScalar **du, dScalar **v, dScalar **dv, ...) {
  if (!it || !it->started) return set_error("dRulesetIteratorStart first");
  _p_dRuleset *R = it->rset;
  if (R->nq > INT32_MAX) return set_error("more than 2^31 points: read the count from dRulesetGetNumPoints");
  cudaStream_t s = it->links[0].fs->stream;
  std::vector<std::array<dScalar **, 4>> out(it->links.size());
  va_list ap;
  va_start(ap, dv);
  for (size_t i = 0; i < it->links.size(); i++) {
    if (i) {
      u = va_arg(ap, dScalar **);
      du = va_arg(ap, dScalar **);
      v = va_arg(ap, dScalar **);
      dv = va_arg(ap, dScalar **);
    }
    out[i] = {u, du, v, dv};
  }
  va_end(ap);
  if (!it->applied && R->nq) {
    // link 0: coordinates, their reference gradient and the physical map
    ItLink &C = it->links[0];
    DCHK(link_eval(it, C, true, true, s));
    int *neg;
    CUCHK(cudaMalloc(&neg, sizeof(int)));
    CUCHK(cudaMemsetAsync(neg, 0, sizeof(int), s));
    k_physical<<<(unsigned)((R->nq + 255) / 256), 256, 0, s>>>(R->nq, R->d_w, C.du, it->jinv, it->jw, neg);
    CUCHK(cudaGetLastError());
    int hneg = 0;
    CUCHK(cudaMemcpyAsync(&hneg, neg, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUCHK(cudaStreamSynchronize(s));
    cudaFree(neg);
    if (hneg) return set_error("Negative Jacobian in the element geometry");
  }
  for (size_t i = 0; i < it->links.size(); i++) {
    ItLink &L = it->links[i];
    const bool want_u = out[i][0] != nullptr, want_du = out[i][1] != nullptr;
    if (R->nq) DCHK(link_eval(it, L, want_u, want_du, s));
    for (int k = 2; k < 4; k++) {
      if (!out[i][k]) continue;
      double **p = k == 2 ? &L.v : &L.dv;
      const int64_t n = R->nq * L.bs * (k == 2 ? 1 : 3);
      const bool fresh = *p == nullptr;
      DCHK(lazy(p, n));
      if (!it->applied || fresh) CUCHK(cudaMemsetAsync(*p, 0, std::max<int64_t>(n, 1) * sizeof(double), s));
    }
    if (out[i][0]) *out[i][0] = L.u;
    if (out[i][1]) *out[i][1] = L.du;
    if (out[i][2]) *out[i][2] = L.v;
    if (out[i][3]) *out[i][3] = L.dv;
  }
  it->applied = true;
  if (Q) *Q = (dInt)R->nq;
  if (jw) *jw = it->jw;
  return 0;
}

dErr dRulesetIteratorCommitPatchApplied(dRulesetIterator it, InsertMode imode, const dScalar *v, const dScalar *dv, ...) {
  if (!it || !it->applied) return set_error("dRulesetIteratorGetPatchApplied first");
  _p_dRuleset *R = it->rset;
  std::vector<std::array<const dScalar *, 2>> in(it->links.size());
  va_list ap;
  va_start(ap, dv);
  for (size_t i = 0; i < it->links.size(); i++) {
    if (i) {
      v = va_arg(ap, const dScalar *);
      dv = va_arg(ap, const dScalar *);
    }
    in[i] = {v, dv};
  }
  va_end(ap);
  for (size_t i = 0; i < it->links.size(); i++) {
    ItLink &L = it->links[i];
    if (!in[i][0] && !in[i][1]) continue;
    // the reference integrates the iterator's own test arrays (callers must not change the returned pointers,
    // fsrulesetit.c:617-625); anything else is an error here
    if ((in[i][0] && in[i][0] != L.v) || (in[i][1] && in[i][1] != L.dv))
      return set_error("dRulesetIteratorCommitPatchApplied: link %d: commit the v/dv arrays GetPatchApplied returned", (int)i);
    if (!L.yexp) return set_error("dRulesetIteratorCommitPatchApplied: link %d has no test vector (pass one to Start)", (int)i);
    if (!R->nq) continue;
    const double *jinv = L.coords ? nullptr : it->jinv;
    for (const IterBucket &B : L.buckets) {  // every element is in one bucket: per-element INSERT is exact
      InsertMode m = imode;
      if (in[i][0]) {
        DCHK(efs_apply_list(B.efs, B.nel, B.d_elist, pt_off(R, B), node_off(L, B), jinv, L.bs, L.v, L.yexp, dAPPLY_INTERP_TRANSPOSE, m,
                            L.fs->stream));
        m = ADD_VALUES;
      }
      if (in[i][1])
        DCHK(efs_apply_list(B.efs, B.nel, B.d_elist, pt_off(R, B), node_off(L, B), jinv, L.bs, L.dv, L.yexp, dAPPLY_GRAD_TRANSPOSE, m,
                            L.fs->stream));
    }
  }
  return 0;
}

dErr dRulesetIteratorGetPatchAssembly(dRulesetIterator it, dInt *P, const dInt **rowcol, const dReal **interp, const dReal **deriv, ...) {
  if (!it || !it->applied) return set_error("dRulesetIteratorGetPatchApplied first (it computes the element geometry)");
  _p_dRuleset *R = it->rset;
  if (R->method != dQUADRATURE_METHOD_SPARSE)
    return set_error("dRulesetIteratorGetPatchAssembly: SPARSE rulesets (the Q1 sub-cell bases of efstopo.c:660-717)");
  const size_t nl = it->links.size();
  it->asm_rowcol.resize(nl, nullptr);
  it->asm_interp.resize(nl, nullptr);
  it->asm_deriv.resize(nl, nullptr);
  va_list ap;
  va_start(ap, deriv);
  dErr err = 0;
  for (size_t i = 0; i < nl && !err; i++) {
    if (i) {
      P = va_arg(ap, dInt *);
      rowcol = va_arg(ap, const dInt **);
      interp = va_arg(ap, const dReal **);
      deriv = va_arg(ap, const dReal **);
    }
    if (!(P || rowcol || interp || deriv)) continue;
    ItLink &L = it->links[i];
    if (L.coords) {
      err = set_error("dRulesetIteratorGetPatchAssembly: the coordinate link has no patch bases here (pass NULL for link 0)");
      break;
    }
    if (!L.fs->uniform || !R->fs->uniform) {
      err = set_error("dRulesetIteratorGetPatchAssembly: link %d: patch bases need uniform-order spaces", (int)i);
      break;
    }
    const int px = L.fs->p, py = px, pz = px;
    const int sp = R->order[0][0] / 2;  // sub-intervals of the rule per direction
    if (px != sp) {
      err = set_error("dRulesetIteratorGetPatchAssembly: link %d has degree %d, the ruleset's patches are the sub-cells of degree %d", (int)i,
                      px, sp);
      break;
    }
    const int64_t np = R->nel * (int64_t)px * py * pz;
    if (!it->asm_rowcol[i]) {
      if (cudaMalloc(&it->asm_rowcol[i], std::max<int64_t>(np, 1) * 8 * sizeof(int32_t)) != cudaSuccess ||
          cudaMalloc(&it->asm_interp[i], std::max<int64_t>(np, 1) * 64 * sizeof(double)) != cudaSuccess ||
          cudaMalloc(&it->asm_deriv[i], std::max<int64_t>(np, 1) * 192 * sizeof(double)) != cudaSuccess) {
        err = set_error("dRulesetIteratorGetPatchAssembly: out of device memory");
        break;
      }
    }
    // the fields are mapped by the element's inverse Jacobians (fsrulesetit.c:673-681)
    const int Qe = (int)(R->nq / std::max<int64_t>(R->nel, 1));
    if (np) {
      k_patch_assembly<<<(unsigned)((np * 8 + 255) / 256), 256, 0, L.fs->stream>>>(R->nel, px, py, pz, L.fs->d_xstart, it->jinv, Qe,
                                                                                   it->asm_rowcol[i], it->asm_interp[i], it->asm_deriv[i]);
      if (cudaGetLastError() != cudaSuccess) err = set_error("k_patch_assembly launch failed");
    }
    if (P) *P = 8;
    if (rowcol) *rowcol = it->asm_rowcol[i];
    if (interp) *interp = it->asm_interp[i];
    if (deriv) *deriv = it->asm_deriv[i];
  }
  va_end(ap);
  return err;
}

dErr dRulesetIteratorFinish(dRulesetIterator it) {
  if (!it || !it->started) return set_error("dRulesetIteratorStart first");
  it->started = false;
  it->has_patch = false;
  for (ItLink &L : it->links) {
    if (!L.Y || L.coords) continue;
    DCHK(fs_restrict(L.fs, L.yexp, L.Y, it->imode == ADD_VALUES));
  }
  return 0;
}

dErr dRulesetIteratorDestroy(dRulesetIterator *it) {
  if (!it || !*it) return 0;
  _p_dRulesetIterator *I = *it;
  for (ItLink &L : I->links) free_link(L);
  cudaFree(I->jinv);
  cudaFree(I->jw);
  cudaFree(I->stash_elem);
  cudaFree(I->stash_node);
  for (auto p : I->asm_rowcol) cudaFree(p);
  for (auto p : I->asm_interp) cudaFree(p);
  for (auto p : I->asm_deriv) cudaFree(p);
  rset_release(I->rset);
  delete I;
  *it = nullptr;
  return 0;
}

// one field on its own preferred ruleset: dFSGetPreferredQuadratureRuleSet + dFSGetCoordinateFS + dRulesetCreateIterator
// + dRulesetIteratorAddFS (the ruleset is released with the iterator)
dErr dRulesetIteratorCreate(dFS fs, dQuadratureMethod method, dRulesetIterator *it) {
  if (!fs || !it) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  dRuleset R;
  dFS cfs;
  DCHK(dFSGetPreferredQuadratureRuleSet(fs, method, &R));
  dErr e = dFSGetCoordinateFS(fs, &cfs);
  if (!e) e = dRulesetCreateIterator(R, cfs, it);
  dRulesetDestroy(&R);
  if (!e) e = dRulesetIteratorAddFS(*it, fs);
  if (e) dRulesetIteratorDestroy(it);
  return e;
}

// dNormsStart/Update/Finish (src/util/util.c:110-153) over all points of the last GetPatchApplied for the first
// field link: errors against exact values at the same points, uerr = {L1, L2, Linf} of u - exact_u and gerr = the
// same of |grad u - exact_du| (exact arrays on the device, [nq][bs] and [nq][bs][3]; either may be NULL)
dErr dRulesetIteratorErrorNorms(dRulesetIterator it, const dScalar *exact_u, const dScalar *exact_du, dReal uerr[3], dReal gerr[3]) {
  if (!it || !it->applied) return set_error("dRulesetIteratorGetPatchApplied first");
  if (it->links.size() < 2) return set_error("dRulesetIteratorErrorNorms: the iterator has no field link");
  ItLink &L = it->links[1];
  cudaStream_t s = L.fs->stream;
  DCHK(link_eval(it, L, true, true, s));
  constexpr int NB = 512;
  double *part;
  CUCHK(cudaMalloc(&part, NB * 6 * sizeof(double)));
  k_norms<<<NB, 256, 0, s>>>(it->rset->nq, L.bs, it->jw, L.u, L.du, exact_u, exact_du, part);
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
