// C ABI entry points for dJacobi/dEFS, dOperator, dMat and the lognormal coefficient, plus the generic
// batched dEFSApply kernel (dEFSApply_Tensor_Hex, src/jacobi/impls/tensor/efstopo.c:368-423, on the device).
#include <math.h>
#include <string.h>

#include <algorithm>

#include "internal.h"

using namespace dgb;

dErr op_mult(_p_dOperator *op, const double *x, double *y);
dErr op_compute_geometry(_p_dOperator *op);
dErr q1_symbolic(_p_dFS *fs, _p_dMat *J);
dErr fs_restrict_rows(_p_dFS *fs, const double *x, double *g, int64_t t0, int64_t t1, cudaStream_t s);
dErr op_mult_expanded(_p_dOperator *op, const double *x, double *yexp);
dErr q1_numeric(_p_dFS *fs, _p_dMat *J, const double *grf_host, int quirk, const double *dref, double pe, double eps, bool single);
dErr q1_numeric_elast(_p_dFS *fs, _p_dMat *J, double lam, double mu, int quirk);
dErr plap_set_stash(_p_dOperator *op, const double *stash);
dErr mat_mult(_p_dMat *J, const double *x, double *y, cudaStream_t s);
void hp_plan_destroy(void *p);

namespace {

// Table layout on the device, per direction d: B[Q][P] then D[Q][P].
struct EFSDev {
  int P[3], Q[3];
  const double *B[3], *D[3];
};

// out[l,m,n,c] (+)= sum_{ijk} A0[l,i] A1[m,j] A2[n,k] in[i,j,k,c]; A given as [Q][P] (tr=0) or its transpose (tr=1)
__device__ void tmult(int D, const int P[3], const int Q[3], const double *const A[3], int tr, const double *in, double *t1,
                      double *t2, double *out, bool add) {
  // P = input sizes, Q = output sizes. tr=0: A[d] stored [Q][P]; tr=1: A[d] stored [P][Q] (the rule-by-basis
  // table read transposed, so rule values map back to the basis).
  const int p0 = P[0], p1 = P[1], p2 = P[2], q0 = Q[0], q1 = Q[1], q2 = Q[2];
  const int n1 = q0 * p1 * p2 * D;
  for (int t = threadIdx.x; t < n1; t += blockDim.x) {
    const int l = t / (p1 * p2 * D), rest = t % (p1 * p2 * D);
    double s = 0;
    for (int i = 0; i < p0; i++) s += (tr ? A[0][i * q0 + l] : A[0][l * p0 + i]) * in[i * p1 * p2 * D + rest];
    t1[t] = s;
  }
  __syncthreads();
  const int n2 = q0 * q1 * p2 * D;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    const int l = t / (q1 * p2 * D), m = (t / (p2 * D)) % q1, kc = t % (p2 * D);
    double s = 0;
    for (int j = 0; j < p1; j++) s += (tr ? A[1][j * q1 + m] : A[1][m * p1 + j]) * t1[(l * p1 + j) * p2 * D + kc];
    t2[t] = s;
  }
  __syncthreads();
  const int n3 = q0 * q1 * q2 * D;
  for (int t = threadIdx.x; t < n3; t += blockDim.x) {
    const int lm = t / (q2 * D), nn = (t / D) % q2, c = t % D;
    double s = 0;
    for (int k = 0; k < p2; k++) s += (tr ? A[2][k * q2 + nn] : A[2][nn * p2 + k]) * t2[(lm * p2 + k) * D + c];
    out[t] = add ? out[t] + s : s;
  }
  __syncthreads();
}

// one block per element; dynamic shared memory holds the element's input and temporaries. Elements are
// contiguous (element b at b * np nodes, b * nq points) unless an element list with node / point offsets is
// given (the elements of one order in a mixed-order space: elist[b] = e, ioff[e] / ooff[e] = the element's first
// input / output node or point)
// components [c0, c0 + Dk) of element b's values: value k of node (or point) i of a slice is global entry
// (base + i) D + c0 + k (with Dk = D the contiguous block of the element); elements too large for all D components in
// shared memory run one component per pass
__global__ void k_efs_apply(EFSDev f, int64_t nelem, const int32_t *elist, const int32_t *ioff, const int32_t *ooff,
                            const double *jinv, int D, int Dk, const double *in, double *out, int amode, int imode) {
  extern __shared__ double sm[];
  const int64_t b = blockIdx.x;
  if (b >= nelem) return;
  const int64_t e = elist ? elist[b] : b;
  const int P[3] = {f.P[0], f.P[1], f.P[2]}, Q[3] = {f.Q[0], f.Q[1], f.Q[2]};
  const int np = P[0] * P[1] * P[2], nq = Q[0] * Q[1] * Q[2];
  const bool fwd = amode == dAPPLY_INTERP || amode == dAPPLY_GRAD;
  const int64_t ib = ioff ? (int64_t)ioff[e] : e * (fwd ? np : nq), ob = ooff ? (int64_t)ooff[e] : e * (fwd ? nq : np);
  const int64_t qb = fwd ? ob : ib;  // first quadrature point of the element
  // generous scratch: each buffer holds max(P,Q)^3 * Dk
  const int m3 = max(max(P[0], Q[0]), max(max(P[1], Q[1]), max(P[2], Q[2])));
  const int buf = m3 * m3 * m3 * Dk;
  double *sin = sm, *t1 = sm + buf, *t2 = sm + 2 * buf, *g = sm + 3 * buf;  // g: 3 gradient buffers
  const bool add = imode == ADD_VALUES;
  const double *Jq = jinv ? jinv + qb * 9 : nullptr;
  auto gidx = [&](int64_t base, int t, int c0) { return (base + t / Dk) * D + c0 + t % Dk; };
  for (int c0 = 0; c0 < D; c0 += Dk) {
    if (fwd) {
      for (int t = threadIdx.x; t < np * Dk; t += blockDim.x) sin[t] = in[gidx(ib, t, c0)];
      __syncthreads();
      if (amode == dAPPLY_INTERP) {
        // write through shared then copy so that ADD semantics apply to global memory
        const double *A[3] = {f.B[0], f.B[1], f.B[2]};
        tmult(Dk, P, Q, A, 0, sin, t1, t2, g, false);
        for (int t = threadIdx.x; t < nq * Dk; t += blockDim.x) {
          double *o = out + gidx(ob, t, c0);
          *o = add ? *o + g[t] : g[t];
        }
      } else {
        for (int dir = 0; dir < 3; dir++) {
          const double *A[3] = {dir == 0 ? f.D[0] : f.B[0], dir == 1 ? f.D[1] : f.B[1], dir == 2 ? f.D[2] : f.B[2]};
          tmult(Dk, P, Q, A, 0, sin, t1, t2, g + dir * buf, false);
        }
        for (int t = threadIdx.x; t < nq * Dk; t += blockDim.x) {
          const int q = t / Dk;
          double *o = out + gidx(ob, t, c0) * 3;
          double gr[3] = {g[t], g[buf + t], g[2 * buf + t]};
          for (int c = 0; c < 3; c++) {
            double v = Jq ? gr[0] * Jq[q * 9 + 0 * 3 + c] + gr[1] * Jq[q * 9 + 1 * 3 + c] + gr[2] * Jq[q * 9 + 2 * 3 + c] : gr[c];
            o[c] = add ? o[c] + v : v;
          }
        }
      }
    } else {
      if (amode == dAPPLY_INTERP_TRANSPOSE) {
        for (int t = threadIdx.x; t < nq * Dk; t += blockDim.x) sin[t] = in[gidx(ib, t, c0)];
        __syncthreads();
        const double *A[3] = {f.B[0], f.B[1], f.B[2]};
        tmult(Dk, Q, P, A, 1, sin, t1, t2, g, false);
      } else {  // GRAD_TRANSPOSE: map with jinv^T then three transposed contractions accumulated
        for (int t = threadIdx.x; t < nq * Dk; t += blockDim.x) {
          const int q = t / Dk;
          const double *v = in + gidx(ib, t, c0) * 3;
          for (int dir = 0; dir < 3; dir++)
            g[dir * buf + t] = Jq ? v[0] * Jq[q * 9 + dir * 3 + 0] + v[1] * Jq[q * 9 + dir * 3 + 1] + v[2] * Jq[q * 9 + dir * 3 + 2] : v[dir];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < np * Dk; t += blockDim.x) sin[t] = 0;
        __syncthreads();
        for (int dir = 0; dir < 3; dir++) {
          const double *A[3] = {dir == 0 ? f.D[0] : f.B[0], dir == 1 ? f.D[1] : f.B[1], dir == 2 ? f.D[2] : f.B[2]};
          tmult(Dk, Q, P, A, 1, g + dir * buf, t1, t2, sin, true);
        }
      }
      const double *src = amode == dAPPLY_INTERP_TRANSPOSE ? g : sin;
      for (int t = threadIdx.x; t < np * Dk; t += blockDim.x) {
        double *o = out + gidx(ob, t, c0);
        *o = add ? *o + src[t] : src[t];
      }
    }
    __syncthreads();  // the next slice reuses the buffers
  }
}

// dEFSApply_Modal_All (src/jacobi/impls/modal/modaltopo.c:73-126) over nelem elements stored back to back: one
// block per element, one thread per output value summing over the modes (INTERP, GRAD) or the points
// (INTERP_TRANSPOSE) in the reference's order; tables interp [Q][P] and deriv [Q][P][3] in global memory (at most
// 18 modes: small and cached). Values [P][D] (modes) and [Q][D] (points), gradients [Q][D][3].
__global__ void k_modal_apply(int64_t nelem, int P, int Q, const double *interp, const double *deriv, int D,
                              const double *in, double *out, int amode, int imode) {
  const int64_t e = blockIdx.x;
  if (e >= nelem) return;
  const bool add = imode == ADD_VALUES;
  if (amode == dAPPLY_INTERP) {
    const double *u = in + e * P * D;
    double *v = out + e * Q * D;
    for (int t = threadIdx.x; t < Q * D; t += blockDim.x) {
      const int i = t / D, c = t % D;
      double s = 0;
      for (int j = 0; j < P; j++) s += interp[i * P + j] * u[j * D + c];
      v[t] = add ? v[t] + s : s;
    }
  } else if (amode == dAPPLY_INTERP_TRANSPOSE) {
    const double *u = in + e * Q * D;
    double *v = out + e * P * D;
    for (int t = threadIdx.x; t < P * D; t += blockDim.x) {
      const int j = t / D, c = t % D;
      double s = 0;
      for (int i = 0; i < Q; i++) s += interp[i * P + j] * u[i * D + c];
      v[t] = add ? v[t] + s : s;
    }
  } else {  // dAPPLY_GRAD
    const double *u = in + e * P * D;
    double *v = out + e * Q * D * 3;
    for (int t = threadIdx.x; t < Q * D * 3; t += blockDim.x) {
      const int i = t / (3 * D), c = (t / 3) % D, d = t % 3;
      double s = 0;
      for (int j = 0; j < P; j++) s += deriv[(i * P + j) * 3 + d] * u[j * D + c];
      v[t] = add ? v[t] + s : s;
    }
  }
}

}  // namespace

// the modal element's batched apply (dEFSApplyBatched on a modal dEFS); jinv is not used, as in the reference's
// modal apply
dErr efs_apply_modal(dEFS efs, int64_t nelem, int D, const double *in, double *out, dApplyMode amode, InsertMode imode,
                     cudaStream_t stream) {
  if (amode != dAPPLY_INTERP && amode != dAPPLY_INTERP_TRANSPOSE && amode != dAPPLY_GRAD)
    return set_error("modal dEFSApply: Apply-mode %d not implemented", (int)amode);
  if (imode != INSERT_VALUES && imode != ADD_VALUES) return set_error("InsertMode %d invalid", (int)imode);
  if (D < 1 || D > 4096) return set_error("dofs %d, must be in 1..4096", D);
  if (nelem < 0) return set_error("nelem %lld negative", (long long)nelem);
  if (nelem == 0) return 0;
  if (!in || !out) return set_error("null vector");
  if (!efs->d_tab) {
    CUCHK(cudaMalloc(&efs->d_tab, efs->h_tab.size() * sizeof(double)));
    CUCHK(cudaMemcpy(efs->d_tab, efs->h_tab.data(), efs->h_tab.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  const int P = efs->P[0], Q = efs->Q[0] * efs->Q[1] * efs->Q[2];
  k_modal_apply<<<(unsigned)nelem, 128, 0, stream>>>(nelem, P, Q, efs->d_tab, efs->d_tab + (size_t)Q * P, D, in, out,
                                                      (int)amode, (int)imode);
  CUCHK(cudaGetLastError());
  return 0;
}

// the batched apply over a list of elements with node / point offsets (dEFSApplyBatched: contiguous elements)
dErr efs_apply_list(dEFS efs, int64_t nelem, const int32_t *elist, const int32_t *ioff, const int32_t *ooff, const double *jinv,
                    int D, const double *in, double *out, dApplyMode amode, InsertMode imode, cudaStream_t stream) {
  if (!efs) return set_error("null EFS");
  if (efs->modal >= 0) return set_error("a modal element in a tensor element loop");
  if (amode < dAPPLY_INTERP || amode > dAPPLY_GRAD_TRANSPOSE) return set_error("invalid/unimplemented dApplyMode %d", (int)amode);
  if (imode != INSERT_VALUES && imode != ADD_VALUES) return set_error("InsertMode %d invalid", (int)imode);
  if (amode == dAPPLY_GRAD_TRANSPOSE && !jinv) return set_error("No Jinv, need a mapping");
  if (D < 1 || D > 3) return set_error("D = %d not supported", D);
  if (nelem <= 0) return 0;
  if (!efs->d_tab) {
    CUCHK(cudaMalloc(&efs->d_tab, efs->h_tab.size() * sizeof(double)));
    CUCHK(cudaMemcpy(efs->d_tab, efs->h_tab.data(), efs->h_tab.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  EFSDev f;
  const double *p = efs->d_tab;
  for (int d = 0; d < 3; d++) {
    f.P[d] = efs->P[d];
    f.Q[d] = efs->Q[d];
    f.B[d] = p;
    f.D[d] = p + efs->P[d] * efs->Q[d];
    p += 2 * efs->P[d] * efs->Q[d];
  }
  int m3 = 0;
  for (int d = 0; d < 3; d++) m3 = std::max(m3, std::max(f.P[d], f.Q[d]));
  // all D components at once when they fit in shared memory, else one component per pass
  const int Dk = 6ull * m3 * m3 * m3 * D * sizeof(double) <= 220 * 1024 ? D : 1;
  const size_t smem = 6ull * m3 * m3 * m3 * Dk * sizeof(double);
  if (smem > 220 * 1024) return set_error("element too large for the batched apply (%zu bytes of shared memory)", smem);
  CUCHK(cudaFuncSetAttribute(k_efs_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_efs_apply<<<(unsigned)nelem, 256, smem, stream>>>(f, nelem, elist, ioff, ooff, jinv, D, Dk, in, out, (int)amode, (int)imode);
  CUCHK(cudaGetLastError());
  return 0;
}

extern "C" {

dErr dJacobiCreate(dJacobi *jac) {
  if (!jac) return set_error("null argument");
  *jac = new _p_dJacobi();
  return 0;
}

dErr dJacobiDestroy(dJacobi *jac) {
  if (!jac || !*jac) return 0;
  for (auto &kv : (*jac)->efs) {
    cudaFree(kv.second->d_tab);
    delete kv.second;
  }
  jacobi_free_quadratures(*jac);
  delete *jac;
  *jac = nullptr;
  return 0;
}

dErr dJacobiGetEFSTensor(dJacobi jac, const dInt degree[3], dQuadratureMethod method, const dInt rule_order[3], dEFS *efs) {
  return jacobi_efs(jac, degree, method, rule_order, efs);
}

}  // extern "C"

dErr jacobi_efs(dJacobi jac, const dInt degree[3], dQuadratureMethod method, const dInt rule_order[3], dEFS *efs, int family) {
  if (!jac || !efs) return set_error("null argument");
  std::vector<int> key = {degree[0], degree[1], degree[2], (int)method, rule_order[0], rule_order[1], rule_order[2], family};
  auto it = jac->efs.find(key);
  if (it != jac->efs.end()) {
    *efs = it->second;
    return 0;
  }
  _p_dEFS *f = new _p_dEFS();
  f->method = method;
  std::vector<double> tab;
  for (int d = 0; d < 3; d++) {
    Basis1D &b = f->b[d];
    if (degree[d] < 1 || degree[d] + 1 > MAXP) {
      delete f;
      return set_error("basis degree %d out of range", degree[d]);
    }
    b.P = degree[d] + 1;
    b.Q = rule_1d(method, rule_order[d], b.x, b.w, family);
    if (b.Q < 1 || b.Q > MAXQ) {
      delete f;
      return set_error("rule size %d out of range", b.Q);
    }
    lobatto_rule(b.P, b.node, b.nodew);
    for (int i = 0; i < b.Q; i++) lagrange(b.P, b.node, b.x[i], b.B + i * b.P, b.D + i * b.P);
    f->P[d] = b.P;
    f->Q[d] = b.Q;
    tab.insert(tab.end(), b.B, b.B + b.P * b.Q);
    tab.insert(tab.end(), b.D, b.D + b.P * b.Q);
  }
  {
    const int ro[3] = {rule_order[0], rule_order[1], rule_order[2]};
    dErr e = jacobi_rule(jac, method, ro, &f->rule, family);
    if (e) {
      delete f;
      return e;
    }
  }
  f->h_tab = tab;  // uploaded on the first device use (host-only queries need no GPU)
  jac->efs[key] = f;
  *efs = f;
  return 0;
}

extern "C" {

dErr dEFSGetSizes(dEFS efs, dInt *dim, dInt *inodes, dInt *total) {
  if (!efs) return set_error("null EFS");
  if (dim) *dim = 3;
  if (efs->modal >= 0) {  // dEFSGetSizes_Modal_All (modaltopo.c:62-71): every mode is interior
    if (inodes) *inodes = efs->P[0];
    if (total) *total = efs->P[0];
    return 0;
  }
  if (inodes) *inodes = std::max(0, efs->P[0] - 2) * std::max(0, efs->P[1] - 2) * std::max(0, efs->P[2] - 2);
  if (total) *total = efs->P[0] * efs->P[1] * efs->P[2];
  return 0;
}

// dEFSGetTensorNodes_Tensor_Hex (efstopo.c:260-290): pointers to the element's own 1-D tables
dErr dEFSGetTensorNodes(dEFS efs, dInt *dim, dInt tsize[3], dReal *nodes[3], dReal *weight[3], const dReal *mscale[3],
                        const dReal *lscale[3]) {
  if (!efs) return set_error("null EFS");
  if (efs->modal >= 0) return set_error("dEFSGetTensorNodes: a modal element has no tensor nodes");
  if (mscale || lscale)
    return set_error("dEFSGetTensorNodes: the Q1 mass / Laplacian scalings (mscale, lscale) are not provided; pass NULL");
  if (dim) *dim = 3;
  for (int d = 0; d < 3; d++) {
    if (tsize) tsize[d] = efs->P[d];
    if (nodes) nodes[d] = efs->b[d].node;
    if (weight) weight[d] = efs->b[d].nodew;
  }
  return 0;
}

dErr dEFSGetTensorTables(dEFS efs, dInt P[3], dInt Q[3], dReal *basis_nodes, dReal *rule_points, dReal *rule_weights) {
  if (!efs) return set_error("null EFS");
  if (efs->modal >= 0) return set_error("dEFSGetTensorTables: a modal element has no tensor nodes");
  int op = 0, oq = 0;
  for (int d = 0; d < 3; d++) {
    if (P) P[d] = efs->P[d];
    if (Q) Q[d] = efs->Q[d];
    for (int i = 0; i < efs->P[d]; i++)
      if (basis_nodes) basis_nodes[op + i] = efs->b[d].node[i];
    for (int i = 0; i < efs->Q[d]; i++) {
      if (rule_points) rule_points[oq + i] = efs->b[d].x[i];
      if (rule_weights) rule_weights[oq + i] = efs->b[d].w[i];
    }
    op += efs->P[d];
    oq += efs->Q[d];
  }
  return 0;
}

dErr dEFSApplyBatched(dEFS efs, dInt nelem, const dReal *jinv, dInt D, const dScalar *in, dScalar *out, dApplyMode amode,
                      InsertMode imode, void *stream) {
  Range range_("dEFSApply");
  if (efs && efs->modal >= 0) return efs_apply_modal(efs, nelem, D, in, out, amode, imode, (cudaStream_t)stream);
  return efs_apply_list(efs, nelem, nullptr, nullptr, nullptr, jinv, D, in, out, amode, imode, (cudaStream_t)stream);
}

dErr dEFSApply(dEFS efs, const dReal *jinv, dInt D, const dScalar *in, dScalar *out, dApplyMode amode, InsertMode imode) {
  return dEFSApplyBatched(efs, 1, jinv, D, in, out, amode, imode, nullptr);
}

// ---------------------------------------------------------------- operator
dErr dFSCreateOperator(dFS fs, dOperatorKind kind, const dReal *param, dOperator *op) {
  if (!fs || !op) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  if ((kind == dOP_ELASTICITY) != (fs->bs == 3)) return set_error("operator kind %d does not match block size %d", (int)kind, fs->bs);
  _p_dOperator *o = new _p_dOperator();
  o->fs = fs;
  o->kind = kind;
  if (param)
    for (int i = 0; i < 2; i++) o->param[i] = param[i];
  if (kind == dOP_ELASTICITY) {  // ElastSetMaterial (src/fs/tests/elast.c:62-69)
    const double E0 = param ? param[0] : 1.0, nu = param ? param[1] : 0.3;
    o->lam = E0 * nu / ((1 + nu) * (1 - 2 * nu));
    o->mu = E0 / (2 * (1 + nu));
  }
  *op = o;
  return 0;
}

dErr dOperatorDestroy(dOperator *op) {
  if (!op || !*op) return 0;
  _p_dOperator *o = *op;
  cudaFree(o->d_geo);
  cudaFree(o->d_geo32);
  cudaFree(o->d_geo16);
  cudaFree(o->d_tcb);
  cudaFree(o->d_geoff);
  cudaFree(o->d_yff);
  cudaFree(o->d_k);
  cudaFree(o->d_stash);
  cudaFree(o->d_yexp);
  cudaFree(o->d_x32);
  cudaFree(o->d_y32);
  if (o->copy_stream) {
    cudaStreamDestroy((cudaStream_t)o->copy_stream);
    for (int k = 0; k < 4; k++) cudaEventDestroy((cudaEvent_t)o->copy_events[k]);
  }
  cudaFree(o->d_hx);
  cudaFree(o->d_hy);
  cudaFree(o->d_gbase);
  cudaFree(o->d_svk);
  hp_plan_destroy(o->hp_plan);
  delete o;
  *op = nullptr;
  return 0;
}

dErr dOperatorSetQuadratureData(dOperator op, const dReal *qdata) {
  if (!op) return set_error("null operator");
  _p_dFS *fs = op->fs;
  if (op->kind == dOP_DIFFUSION) {
    if (!qdata) {
      cudaFree(op->d_k);
      op->d_k = nullptr;
    } else {
      if (!op->d_k) CUCHK(cudaMalloc(&op->d_k, fs->nq * sizeof(double)));
      CUCHK(cudaMemcpyAsync(op->d_k, qdata, fs->nq * sizeof(double), cudaMemcpyDeviceToDevice, fs->stream));
    }
    op->geo_valid = false;
    return 0;
  }
  if (op->kind == dOP_PLAPLACE_JACOBIAN) return plap_set_stash(op, qdata);
  return set_error("operator kind %d takes no quadrature data", (int)op->kind);
}

dErr dOperatorSetPrecision(dOperator op, dPrecision prec) {
  if (!op) return set_error("null operator");
  if (prec != dPREC_FP64 && prec != dPREC_FP32 && prec != dPREC_BF16 && prec != dPREC_FF) return set_error("precision %d not supported", (int)prec);
  op->prec = prec;
  return 0;
}

dErr dOperatorMult(dOperator op, const dScalar *x, dScalar *y) {
  Range range_("EllipShellMult");
  if (!op) return set_error("null operator");
  return op_mult(op, x, y);
}

dErr dOperatorMultHost(dOperator op, const dScalar *x_host, dScalar *y_host) {
  Range range_("EllipShellMult (host vectors)");
  if (!op) return set_error("null operator");
  _p_dFS *fs = op->fs;
  const size_t bytes = fs->n * fs->bs * sizeof(double);
  if (!op->d_hx) {
    CUCHK(cudaMalloc(&op->d_hx, std::max<size_t>(bytes, 8)));
    CUCHK(cudaMalloc(&op->d_hy, std::max<size_t>(bytes, 8)));
  }
  const int64_t N = fs->n * fs->bs;
  const bool big = op->prec == dPREC_FP64 && !op->svk_state && N >= 4 * 65536;
  // page-locked input of a large FP64 apply: the element kernel reads it in place over the host link (the gather's
  // host reads overlap the kernel's FP64 arithmetic instead of a copy before it); otherwise one copy to the device
  const double *xd = op->d_hx;
  cudaPointerAttributes pa;
  if (big && cudaPointerGetAttributes(&pa, x_host) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
    xd = (const double *)pa.devicePointer;
  else
    CUCHK(cudaMemcpyAsync(op->d_hx, x_host, bytes, cudaMemcpyHostToDevice, fs->stream));
  cudaGetLastError();  // a pointer the runtime does not know leaves an error state behind
  if (!big) {
    DCHK(op_mult(op, op->d_hx, op->d_hy));
    CUCHK(cudaMemcpyAsync(y_host, op->d_hy, bytes, cudaMemcpyDeviceToHost, fs->stream));
    CUCHK(cudaStreamSynchronize(fs->stream));
    return 0;
  }
  // FP64: the element part, then the restriction in four row blocks; each block goes back to the host on a
  // second stream as soon as it is restricted, so the copy of one block overlaps the restriction of the next
  if (!op->copy_stream) {
    cudaStream_t cs;
    CUCHK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    op->copy_stream = cs;
    for (int k = 0; k < 4; k++) {
      cudaEvent_t ev;
      CUCHK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      op->copy_events[k] = ev;
    }
  }
  cudaStream_t cs = (cudaStream_t)op->copy_stream;
  if (!op->d_yexp) CUCHK(cudaMalloc(&op->d_yexp, fs->nexp * fs->bs * sizeof(double)));
  DCHK(op_mult_expanded(op, xd, op->d_yexp));
  for (int k = 0; k < 4; k++) {
    const int64_t t0 = N * k / 4, t1 = N * (k + 1) / 4;
    DCHK(fs_restrict_rows(fs, op->d_yexp, op->d_hy, t0, t1, fs->stream));
    CUCHK(cudaEventRecord((cudaEvent_t)op->copy_events[k], fs->stream));
    CUCHK(cudaStreamWaitEvent(cs, (cudaEvent_t)op->copy_events[k], 0));
    CUCHK(cudaMemcpyAsync(y_host + t0, op->d_hy + t0, (t1 - t0) * sizeof(double), cudaMemcpyDeviceToHost, cs));
  }
  CUCHK(cudaStreamSynchronize(cs));
  return 0;
}

// ---------------------------------------------------------------- Q1 matrix
dErr dFSCreateMatrix(dFS fs, dMat *J) {
  if (!fs || !J) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  _p_dMat *m = new _p_dMat();
  m->fs = fs;
  dErr e = q1_symbolic(fs, m);
  if (e) {
    delete m;
    return e;
  }
  *J = m;
  return 0;
}

dErr dMatDestroy(dMat *J) {
  if (!J || !*J) return 0;
  cudaFree((*J)->d_rowptr);
  cudaFree((*J)->d_col);
  cudaFree((*J)->d_val);
  cudaFree((*J)->d_srowptr);
  cudaFree((*J)->d_scol);
  cudaFree((*J)->d_sell_off);
  cudaFree((*J)->d_sell_col);
  cudaFree((*J)->d_sell_val);
  delete *J;
  *J = nullptr;
  return 0;
}

dErr dFSAssembleQ1(dFS fs, dMat J, dOperatorKind kind, const dReal *param, const dReal *grf, int reference_quirk) {
  Range range_("dQ1HexComputQuad");
  (void)param;
  if (!fs || !J) return set_error("null argument");
  if (kind == dOP_PLAPLACE_JACOBIAN) return set_error("the p-Laplacian Q1 matrix depends on the state: use dFSAssembleQ1PLaplace");
  if (kind == dOP_ELASTICITY) {  // ElastJacobian (elast.c:343-407) at F = I, Lame parameters as ElastSetMaterial
    if (fs->bs != 3 || J->bs != 3) return set_error("elasticity Q1 assembly needs block size 3");
    const double E0 = param ? param[0] : 1.0, nu = param ? param[1] : 0.3;
    return q1_numeric_elast(fs, J, E0 * nu / ((1 + nu) * (1 - 2 * nu)), E0 / (2 * (1 + nu)), reference_quirk);
  }
  if (kind != dOP_DIFFUSION) return set_error("Q1 assembly for operator kind %d not built yet", (int)kind);
  if (fs->bs != 1) return set_error("diffusion Q1 assembly needs block size 1");
  return q1_numeric(fs, J, grf, reference_quirk, nullptr, 0, 0, false);
}

dErr dMatGetCSR(dMat J, dInt *nrows, int64_t *nnz, const dInt **rowptr, const dInt **col, const dScalar **val) {
  if (!J) return set_error("null matrix");
  if (nrows) *nrows = (dInt)J->nrows;
  if (nnz) *nnz = J->nnz;
  if (rowptr) *rowptr = J->d_rowptr;
  if (col) *col = J->d_col;
  if (val) *val = J->d_val;
  return 0;
}

dErr dMatGetCSRHost(dMat J, dInt *rowptr, dInt *col, dScalar *val) {
  if (!J) return set_error("null matrix");
  cudaStream_t s = J->fs->stream;
  if (rowptr) CUCHK(cudaMemcpyAsync(rowptr, J->d_rowptr, (J->nrows + 1) * sizeof(dInt), cudaMemcpyDeviceToHost, s));
  if (col && J->nnz) CUCHK(cudaMemcpyAsync(col, J->d_col, J->nnz * sizeof(dInt), cudaMemcpyDeviceToHost, s));
  if (val && J->nnz) CUCHK(cudaMemcpyAsync(val, J->d_val, J->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUCHK(cudaStreamSynchronize(s));
  return 0;
}

}  // extern "C"

namespace {
// entries of a matrix set or added in the given order by one thread: the order a host loop over them would take, so
// repeated entries end as PETSc's MatSetValues leaves them (INSERT: the last wins; ADD: summed in order)
__global__ void k_set_entries(int64_t count, const int64_t *__restrict__ pos, const double *__restrict__ v, int add,
                              double *__restrict__ val) {
  if (blockIdx.x || threadIdx.x) return;
  for (int64_t i = 0; i < count; i++) val[pos[i]] = add ? val[pos[i]] + v[i] : v[i];
}
}  // namespace

extern "C" {

// dFSMatSetValuesBlockedExpanded (src/fs/interface/fs.c:826-930): an m x n block of values in expanded (element
// node) indices, v row-major [m bs][n bs] on the host, expanded through E into the explicit-dof matrix J (rows and
// columns of Dirichlet nodes dropped, as in the preconditioning matrix): each value becomes
// E[row][r] * (E[col][c] * v), columns expanded first as the reference does; every target must lie in J's pattern
// (the Q1-embedded sparsity), else an error. The values change on J's stream; a KSP built on J sees them after
// dKSPSetOperators, as after a PETSc MatAssembly.
dErr dFSMatSetValuesBlockedExpanded(dFS fs, dMat J, dInt m, const dInt idxm[], dInt n, const dInt idxn[], const dScalar v[],
                                    InsertMode imode) {
  if (!fs || !J || !idxm || !idxn || !v) return set_error("null argument");
  if (J->fs != fs) return set_error("the matrix belongs to another space");
  if (imode != INSERT_VALUES && imode != ADD_VALUES) return set_error("InsertMode %d invalid", (int)imode);
  if (m < 0 || n < 0) return set_error("negative block size");
  const int bs = fs->bs;
  if (J->nrows != fs->n * bs) return set_error("matrix rows %lld do not match the space (%lld)", (long long)J->nrows, (long long)fs->n * bs);
  if (J->h_rowptr.empty()) {
    J->h_rowptr.resize(J->nrows + 1);
    J->h_col.resize(J->nnz);
    CUCHK(cudaMemcpyAsync(J->h_rowptr.data(), J->d_rowptr, (J->nrows + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, fs->stream));
    if (J->nnz) CUCHK(cudaMemcpyAsync(J->h_col.data(), J->d_col, J->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, fs->stream));
    CUCHK(cudaStreamSynchronize(fs->stream));
  }
  // one expanded node's E row: (global node, weight) pairs
  auto erow = [&](int32_t e, std::vector<std::pair<int32_t, double>> &out) -> dErr {
    out.clear();
    if (e < 0 || e >= fs->nexp) return set_error("expanded index %d outside [0, %lld)", e, (long long)fs->nexp);
    if (fs->boolean_e) out.push_back({fs->emap[e], 1.0});
    else
      for (int32_t k = fs->eptr[e]; k < fs->eptr[e + 1]; k++) out.push_back({fs->ecol[k], fs->eval[k]});
    return 0;
  };
  std::vector<int64_t> pos;
  std::vector<double> val;
  std::vector<std::pair<int32_t, double>> er, ec;
  for (dInt i = 0; i < m; i++) {
    DCHK(erow(idxm[i], er));
    for (const auto &r : er) {
      if (r.first >= fs->n) continue;  // a Dirichlet node: no row of the preconditioning matrix
      for (int a = 0; a < bs; a++) {
        const int64_t row = (int64_t)r.first * bs + a;
        const int32_t *c0 = J->h_col.data() + J->h_rowptr[row], *c1 = J->h_col.data() + J->h_rowptr[row + 1];
        for (dInt j = 0; j < n; j++) {
          DCHK(erow(idxn[j], ec));
          for (const auto &c : ec) {
            if (c.first >= fs->n) continue;
            for (int b = 0; b < bs; b++) {
              const int32_t col = c.first * bs + b;
              const int32_t *hit = std::find(c0, c1, col);
              if (hit == c1) return set_error("entry (%lld, %d) is not in the matrix's sparsity pattern", (long long)row, col);
              pos.push_back(hit - J->h_col.data());
              val.push_back(r.second * (c.second * v[((int64_t)(i * bs + a) * n + j) * bs + b]));
            }
          }
        }
      }
    }
  }
  if (pos.empty()) return 0;
  int64_t *dpos;
  double *dval;
  CUCHK(cudaMallocAsync(&dpos, pos.size() * sizeof(int64_t), fs->stream));
  CUCHK(cudaMallocAsync(&dval, val.size() * sizeof(double), fs->stream));
  CUCHK(cudaMemcpyAsync(dpos, pos.data(), pos.size() * sizeof(int64_t), cudaMemcpyHostToDevice, fs->stream));
  CUCHK(cudaMemcpyAsync(dval, val.data(), val.size() * sizeof(double), cudaMemcpyHostToDevice, fs->stream));
  k_set_entries<<<1, 1, 0, fs->stream>>>((int64_t)pos.size(), dpos, dval, imode == ADD_VALUES, J->d_val);
  CUCHK(cudaGetLastError());
  CUCHK(cudaFreeAsync(dpos, fs->stream));
  CUCHK(cudaFreeAsync(dval, fs->stream));
  CUCHK(cudaStreamSynchronize(fs->stream));  // the host vectors above must outlive their copies
  J->sell_valid = false;
  return 0;
}

dErr dMatMult(dMat J, const dScalar *x, dScalar *y) {
  if (!J) return set_error("null matrix");
  return mat_mult(J, x, y, J->fs->stream);
}

// ---------------------------------------------------------------- lognormal coefficient
dErr dGRFCreate(dInt nf, dReal var, dReal ell, uint64_t seed, dReal *grf) {
  if (nf < 1 || !grf) return set_error("bad GRF arguments");
  const double twopi = 6.283185307179586476925286766559;
  uint64_t st = seed;
  auto next = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  grf[0] = nf, grf[1] = var, grf[2] = ell;
  for (int f = 0; f < nf; f++)
    for (int d = 0; d < 3; d++) {
      double u1 = next(), u2 = next();
      if (u1 < 1e-300) u1 = 1e-300;
      grf[3 + 3 * f + d] = sqrt(-2.0 * log(u1)) * cos(twopi * u2) / ell;  // Box-Muller
    }
  for (int f = 0; f < nf; f++) grf[3 + 3 * nf + f] = twopi * next();
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- quadrature-point fields
namespace {
struct GaussTab {
  double x[MAXP];
};
__global__ void k_qpt_coords(int64_t nelem, const int32_t *edeg, const int32_t *qoff, const double *coords, const GaussTab *gt,
                             const double *grf, double *xq, double *kq) {
  const int64_t e = blockIdx.x;
  if (e >= nelem) return;
  const int pa = edeg[3 * e], pb = edeg[3 * e + 1], pc = edeg[3 * e + 2], Qb = pb + 1, Qc = pc + 1, nq = (pa + 1) * Qb * Qc;
  const double *X = coords + e * 24;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const int a = q / (Qb * Qc), b = (q / Qc) % Qb, c = q % Qc;
    const double s = gt[pa].x[a], t = gt[pb].x[b], u = gt[pc].x[c];
    const double bs[2] = {0.5 * (1 - s), 0.5 * (1 + s)}, bt[2] = {0.5 * (1 - t), 0.5 * (1 + t)}, bu[2] = {0.5 * (1 - u), 0.5 * (1 + u)};
    double x[3] = {0, 0, 0};
    for (int v = 0; v < 8; v++) {
      const double ph = bs[v >> 2] * bt[(v >> 1) & 1] * bu[v & 1];
      for (int d = 0; d < 3; d++) x[d] += X[v * 3 + d] * ph;
    }
    const int64_t o = qoff[e] + q;
    if (xq)
      for (int d = 0; d < 3; d++) xq[o * 3 + d] = x[d];
    if (kq) {
      const int nf = (int)grf[0];
      const double *w = grf + 3, *bb = grf + 3 + 3 * nf;
      double g = 0;
      for (int f = 0; f < nf; f++) g += cos(w[3 * f] * x[0] + w[3 * f + 1] * x[1] + w[3 * f + 2] * x[2] + bb[f]);
      kq[o] = exp(sqrt(2.0 * grf[1] / nf) * g);
    }
  }
}

dErr qpt_fields(_p_dFS *fs, const double *grf_host, double *xq, double *kq) {
  GaussTab h[MAXP];
  for (int p = 1; p < MAXP; p++) {
    double w[MAXP];
    gauss_rule(p + 1, h[p].x, w);
  }
  GaussTab *d_gt;
  double *d_grf = nullptr;
  CUCHK(cudaMalloc(&d_gt, sizeof h));
  CUCHK(cudaMemcpyAsync(d_gt, h, sizeof h, cudaMemcpyHostToDevice, fs->stream));
  if (grf_host) {
    const int nf = (int)grf_host[0];
    CUCHK(cudaMalloc(&d_grf, (3 + 4 * nf) * sizeof(double)));
    CUCHK(cudaMemcpyAsync(d_grf, grf_host, (3 + 4 * nf) * sizeof(double), cudaMemcpyHostToDevice, fs->stream));
  }
  k_qpt_coords<<<(unsigned)fs->nelem, 128, 0, fs->stream>>>(fs->nelem, fs->d_edeg, fs->d_qoff, fs->d_coords, d_gt, d_grf, xq, kq);
  CUCHK(cudaGetLastError());
  CUCHK(cudaStreamSynchronize(fs->stream));
  cudaFree(d_gt);
  cudaFree(d_grf);
  return 0;
}
}  // namespace

extern "C" {

dErr dFSGetQuadratureCoordinates(dFS fs, dReal *xq) {
  if (!fs || !fs->setup) return set_error("dFS not set up");
  return qpt_fields(fs, nullptr, xq, nullptr);
}

dErr dFSEvaluateLognormal(dFS fs, const dReal *grf, dReal *kq) {
  if (!fs || !fs->setup) return set_error("dFS not set up");
  if (!grf) return set_error("null GRF");
  return qpt_fields(fs, grf, nullptr, kq);
}

}  // extern "C"
