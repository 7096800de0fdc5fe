// dJacobi quadrature, rules and explicit element bases on the host (src/jacobi/interface/jacobi.c,
// quadrature.c; src/jacobi/quadrature/impls/tensor/tensorquad.c; src/jacobi/impls/tensor/efstopo.c:660-717),
// the modal (P-discontinuous) element spaces of the modal dJacobi type (src/jacobi/impls/modal/modal.c),
// plus the vector constructors of a dFS.
//
// A dQuadrature is owned by its dJacobi (one per method, made on first request, as dJacobiGetQuadrature caches
// it); a dRule is a tensor Gauss (FAST), composite two-point (SPARSE) or Lobatto (SELF) rule on the reference
// hex, owned by its dQuadrature and shared by every caller that asks for the same orders. Arrays of handles
// returned by dQuadratureGetRules / dJacobiGetEFS are the caller's and are released with dFree, as in dohp.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include "internal.h"

using namespace dgb;

struct _p_dRule {
  dQuadratureMethod method;
  int family = dGAUSS_LEGENDRE;  // point family (dQuadratureTensorSetGaussFamily)
  // facet rules (dQuadratureGetFacetRules): side 0..5 of the hex, else -1; the 2-D rule's points (X, Y, 0) are mapped
  // by xi = R (X, Y, 0) + t (the reference's transformed rules, tensorquad.c:224-242)
  int facet = -1;
  double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, t[3] = {0, 0, 0};
  int order[3];  // polynomial order integrated exactly, per direction
  int Q[3];
  double x[3][MAXQ], w[3][MAXQ];
  int npatches = 0, patchsize = 0;  // patch tables (dRuleGetPatches), made on first request
  std::vector<int32_t> patchind;
  std::vector<double> patchweight;
};

struct _p_dQuadrature {
  dQuadratureMethod method;
  int family = dGAUSS_LEGENDRE;  // family of the rules made from now on
  std::map<std::vector<int>, _p_dRule *> rules;  // key {family, order x, y, z}
};

void jacobi_free_quadratures(dJacobi jac) {
  for (auto &q : jac->quad) {
    if (!q) continue;
    for (auto &kv : q->rules) delete kv.second;
    delete q;
    q = nullptr;
  }
}

dErr quad_rule(_p_dQuadrature *q, const int order[3], int family, _p_dRule **out);

// the rule of the given method, orders and family, owned by the dJacobi's quadrature (used for every dEFS's rule)
dErr jacobi_rule(dJacobi jac, dQuadratureMethod method, const int order[3], _p_dRule **out, int family) {
  dQuadrature q;
  DCHK(dJacobiGetQuadrature(jac, method, &q));
  return quad_rule(q, order, family, out);
}

// the family a dJacobi's quadrature of a method makes rules in (Gauss-Legendre before one exists)
int jacobi_quad_family(dJacobi jac, dQuadratureMethod method) {
  return jac && method >= 0 && method < 3 && jac->quad[method] ? jac->quad[method]->family : (int)dGAUSS_LEGENDRE;
}

dErr quad_rule(_p_dQuadrature *q, const int order[3], int family, _p_dRule **out) {
  std::vector<int> key = {family, order[0], order[1], order[2]};
  auto it = q->rules.find(key);
  if (it != q->rules.end()) {
    *out = it->second;
    return 0;
  }
  _p_dRule *r = new _p_dRule();
  r->method = q->method;
  r->family = family;
  for (int d = 0; d < 3; d++) {
    if (order[d] < 0 || order[d] > 2 * MAXQ) {
      delete r;
      return set_error("rule order %d out of range", order[d]);
    }
    r->order[d] = order[d];
    double x[64], w[64];
    const int n = rule_1d(q->method, order[d], x, w, family);
    if (n < 1 || n > MAXQ) {
      delete r;
      return set_error("rule of order %d has %d points (at most %d supported)", order[d], n, MAXQ);
    }
    r->Q[d] = n;
    std::copy(x, x + n, r->x[d]);
    std::copy(w, w + n, r->w[d]);
  }
  q->rules[key] = r;
  *out = r;
  return 0;
}

// the facet rule of a side and per-direction orders: a tensor rule on [-1,1]^2 (its third direction one point of
// weight 1 at 0), mapped by the side's rotation and translation (dQuadratureGetFacetRules_Tensor_Private,
// tensorquad.c:309-355: rotations and translations as the reference tabulates them; table as reference). The face
// rule's two orders are formed as the reference does, from the rows of the rotation (a direction's degree where
// the row is nonzero); for isotropic orders, the ones its callers pass, that is the order itself.
dErr quad_facet_rule(_p_dQuadrature *q, int facet, const int order[3], int family, _p_dRule **out) {
  static const double kR[6][3][3] = {{{1, 0, 0}, {0, 0, -1}, {0, 1, 0}},  {{0, 0, 1}, {1, 0, 0}, {0, 1, 0}},
                                     {{-1, 0, 0}, {0, 0, 1}, {0, 1, 0}},  {{0, 0, -1}, {-1, 0, 0}, {0, 1, 0}},
                                     {{0, 1, 0}, {1, 0, 0}, {0, 0, -1}},  {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};
  static const double kT[6][3] = {{0, -1, 0}, {1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, 0, -1}, {0, 0, 1}};
  if (facet < 0 || facet > 5) return set_error("facet %d of a hexahedron out of range 0..5", facet);
  int rot[2];
  for (int i = 0; i < 2; i++) {
    rot[i] = 0;
    for (int j = 0; j < 3; j++) rot[i] += kR[facet][i][j] != 0 ? order[j] : 0;
  }
  std::vector<int> key = {family, rot[0], rot[1], 0, 100 + facet};
  auto it = q->rules.find(key);
  if (it != q->rules.end()) {
    *out = it->second;
    return 0;
  }
  _p_dRule *r = new _p_dRule();
  r->method = q->method;
  r->family = family;
  r->facet = facet;
  for (int d = 0; d < 2; d++) {
    double x[64], w[64];
    const int n = rule_1d(q->method, rot[d], x, w, family);
    if (n < 1 || n > MAXQ) {
      delete r;
      return set_error("facet rule of order %d has %d points (at most %d supported)", rot[d], n, MAXQ);
    }
    r->order[d] = rot[d];
    r->Q[d] = n;
    std::copy(x, x + n, r->x[d]);
    std::copy(w, w + n, r->w[d]);
  }
  r->order[2] = 0, r->Q[2] = 1, r->x[2][0] = 0, r->w[2][0] = 1;
  for (int i = 0; i < 3; i++) {
    r->t[i] = kT[facet][i];
    for (int j = 0; j < 3; j++) r->R[i][j] = kR[facet][i][j];
  }
  q->rules[key] = r;
  *out = r;
  return 0;
}

namespace {

// dGeomInvert3 (include/dohpgeom.h:57-79): cofactor inverse and determinant
double invert3_host(const double a[9], double b[9]) {
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
  return det;
}

// Modal (P-discontinuous) hexahedral bases of the modal dJacobi (src/jacobi/impls/modal/modal.c:15-240). Every
// mode is a product of orthonormal Legendre polynomials sqrt(n + 1/2) P_n(t), one per direction; the modes of each
// order are listed by their degrees per direction in the reference's order (its order-3 set has 18 modes: the
// y^2 z and y z^2 products are not in it).
constexpr int kModalCount[4] = {1, 4, 10, 18};  // ModalPCount (modal.c:15-42), region
constexpr int kModalDegrees[18][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0}, {0, 2, 0},
                                      {0, 0, 2}, {1, 1, 0}, {0, 1, 1}, {1, 0, 1}, {3, 0, 0}, {0, 3, 0},
                                      {0, 0, 3}, {2, 1, 0}, {1, 2, 0}, {2, 0, 1}, {1, 0, 2}, {1, 1, 1}};

// sqrt(n + 1/2) P_n(t) and its derivative by Bonnet's recurrence (k+1) P_{k+1} = (2k+1) t P_k - k P_{k-1},
// P'_{k+1} = P'_{k-1} + (2k+1) P_k
void legendre_orthonormal(int n, double t, double *v, double *dv) {
  double p0 = 1, p1 = t, d0 = 0, d1 = 1;
  if (n == 0) p1 = 1, d1 = 0;
  for (int k = 1; k < n; k++) {
    const double p2 = ((2 * k + 1) * t * p1 - k * p0) / (k + 1), d2 = d0 + (2 * k + 1) * p1;
    p0 = p1, p1 = p2, d0 = d1, d1 = d2;
  }
  const double c = std::sqrt(n + 0.5);
  *v = c * p1;
  *dv = c * d1;
}

}  // namespace

// the modal element space of an order on a rule, cached in the dJacobi (key {-1, order, 0, method, rule orders,
// family}: tensor keys start with a degree >= 1); tables interp [nq][P] and deriv [nq][P][3] at the rule's points
dErr jacobi_efs_modal(dJacobi jac, int order, _p_dRule *rule, dEFS *efs) {
  if (order < 0 || order > 3) return set_error("modal basis: order %d for type region (orders 0..3)", order);
  std::vector<int> key = {-1, order, 0, (int)rule->method, rule->order[0], rule->order[1], rule->order[2], rule->family};
  auto it = jac->efs.find(key);
  if (it != jac->efs.end()) {
    *efs = it->second;
    return 0;
  }
  const int P = kModalCount[order], nq = rule->Q[0] * rule->Q[1] * rule->Q[2];
  std::vector<double> pts(3 * (size_t)nq);
  DCHK(dRuleGetNodeWeight(rule, pts.data(), nullptr));
  _p_dEFS *f = new _p_dEFS();
  f->modal = order;
  f->method = rule->method;
  f->rule = rule;
  f->P[0] = P, f->P[1] = f->P[2] = 1;
  for (int d = 0; d < 3; d++) f->Q[d] = rule->Q[d];
  f->h_tab.assign((size_t)nq * P * 4, 0.0);
  double *interp = f->h_tab.data(), *deriv = interp + (size_t)nq * P;
  for (int q = 0; q < nq; q++)
    for (int j = 0; j < P; j++) {
      double v[3], dv[3];
      for (int d = 0; d < 3; d++) legendre_orthonormal(kModalDegrees[j][d], pts[3 * q + d], &v[d], &dv[d]);
      interp[(size_t)q * P + j] = v[0] * v[1] * v[2];
      double *g = deriv + ((size_t)q * P + j) * 3;
      g[0] = dv[0] * v[1] * v[2];
      g[1] = v[0] * dv[1] * v[2];
      g[2] = v[0] * v[1] * dv[2];
    }
  jac->efs[key] = f;
  *efs = f;
  return 0;
}

extern "C" {

dErr dFree(void *ptr) {
  free(ptr);
  return 0;
}

dErr dJacobiGetQuadrature(dJacobi jac, dQuadratureMethod method, dQuadrature *quad) {
  if (!jac || !quad) return set_error("null argument");
  if (method != dQUADRATURE_METHOD_FAST && method != dQUADRATURE_METHOD_SPARSE && method != dQUADRATURE_METHOD_SELF)
    return set_error("invalid quadrature method %d", (int)method);
  if (!jac->quad[method]) {
    jac->quad[method] = new _p_dQuadrature();
    jac->quad[method]->method = method;
  }
  *quad = jac->quad[method];
  return 0;
}

dErr dQuadratureGetRules(dQuadrature quad, dInt n, const dEntTopology topo[], const dPolynomialOrder order[], dRule **rules) {
  if (!quad || !rules || (n > 0 && (!topo || !order))) return set_error("null argument");
  *rules = nullptr;
  dRule *arr = (dRule *)malloc(sizeof(dRule) * (size_t)std::max<dInt>(n, 1));
  if (!arr) return set_error("out of host memory");
  for (dInt i = 0; i < n; i++) {
    if (topo[i] != dTOPO_HEX) {
      free(arr);
      return set_error("dQuadratureGetRules: topology %d not supported (hexahedra only)", (int)topo[i]);
    }
    const int o[3] = {dPolynomialOrder1D(order[i], 0), dPolynomialOrder1D(order[i], 1), dPolynomialOrder1D(order[i], 2)};
    dErr e = quad_rule(quad, o, quad->family, &arr[i]);
    if (e) {
      free(arr);
      return e;
    }
  }
  *rules = arr;
  return 0;
}

dErr dQuadratureTensorSetGaussFamily(dQuadrature quad, dGaussFamily family) {
  if (!quad) return set_error("null quadrature");
  static const char *names[] = {"gauss", "lobatto", "radau"};
  if (family != dGAUSS_LEGENDRE && family != dGAUSS_LOBATTO) {
    if (family == dGAUSS_RADAU)
      return set_error("GaussFamily %s and dQuadratureMethod %d not supported", names[family], (int)quad->method);
    return set_error("invalid GaussFamily %d", (int)family);
  }
  quad->family = family;
  return 0;
}

dErr dQuadratureGetFacetRules(dQuadrature quad, dInt n, const dEntTopology topo[], const dInt facet[], const dPolynomialOrder order[],
                              dRule **rules) {
  if (!quad || !rules || (n > 0 && (!topo || !facet || !order))) return set_error("null argument");
  *rules = nullptr;
  dRule *arr = (dRule *)malloc(sizeof(dRule) * (size_t)std::max<dInt>(n, 1));
  if (!arr) return set_error("out of host memory");
  for (dInt i = 0; i < n; i++) {
    dErr e = 0;
    if (topo[i] != dTOPO_HEX) e = set_error("dQuadratureGetFacetRules: unsupported topology %d (hexahedra only)", (int)topo[i]);
    const int o[3] = {dPolynomialOrder1D(order[i], 0), dPolynomialOrder1D(order[i], 1), dPolynomialOrder1D(order[i], 2)};
    if (!e) e = quad_facet_rule(quad, facet[i], o, quad->family, &arr[i]);
    if (e) {
      free(arr);
      return e;
    }
  }
  *rules = arr;
  return 0;
}

dErr dRuleGetSize(dRule rule, dInt *dim, dInt *nnodes) {
  if (!rule) return set_error("null rule");
  if (dim) *dim = rule->facet >= 0 ? 2 : 3;
  if (nnodes) *nnodes = rule->Q[0] * rule->Q[1] * rule->Q[2];
  return 0;
}

dErr dRuleGetTensorNodeWeight(dRule rule, dInt *dim, dInt nnodes[3], const dReal *coord[3], const dReal *weight[3]) {
  if (!rule) return set_error("null rule");
  if (rule->facet >= 0) return set_error("dRuleGetTensorNodeWeight: a facet rule has no tensor form in the element's directions");
  if (dim) *dim = 3;
  for (int d = 0; d < 3; d++) {
    if (nnodes) nnodes[d] = rule->Q[d];
    if (coord) coord[d] = rule->x[d];
    if (weight) weight[d] = rule->w[d];
  }
  return 0;
}

dErr dRuleGetNodeWeight(dRule rule, dReal *coord, dReal *weight) {
  if (!rule) return set_error("null rule");
  const int *Q = rule->Q;
  for (int i = 0; i < Q[0]; i++)
    for (int j = 0; j < Q[1]; j++)
      for (int k = 0; k < Q[2]; k++) {
        const int q = (i * Q[1] + j) * Q[2] + k;
        const double X[3] = {rule->x[0][i], rule->x[1][j], rule->x[2][k]};
        if (coord) {
          if (rule->facet >= 0)  // dRuleGetNodeWeight_Transformed (tensorquad.c:224-242)
            for (int c = 0; c < 3; c++) coord[3 * q + c] = rule->R[c][0] * X[0] + rule->R[c][1] * X[1] + rule->R[c][2] * X[2] + rule->t[c];
          else
            coord[3 * q] = X[0], coord[3 * q + 1] = X[1], coord[3 * q + 2] = X[2];
        }
        if (weight) weight[q] = rule->w[0][i] * rule->w[1][j] * rule->w[2][k];
      }
  return 0;
}

// dRulePatchSetup_Tensor (tensorquad.c:120-169): SPARSE rules are tiled into 2 x 2 x 2 patches of points, other
// rules are one patch; ind = element-natural index of each patch point. The weights repeat the reference's z factor
// (the y rule's weight at the point's y index, tensorquad.c:159-161); nothing computes with them.
dErr dRuleGetPatches(dRule rule, dInt *npatches, dInt *patchsize, const dInt **ind, const dReal **weight) {
  if (!rule) return set_error("null rule");
  if (rule->patchind.empty()) {
    int N[3], P[3];
    const int *Q = rule->Q;
    for (int d = 0; d < 3; d++) {
      if (rule->method == dQUADRATURE_METHOD_SPARSE) {
        P[d] = Q[d] > 1 ? 2 : 1;
        N[d] = Q[d] / P[d];
        if (N[d] * P[d] != Q[d]) return set_error("sparse rule with an odd number of points %d", Q[d]);
      } else {
        N[d] = 1;
        P[d] = Q[d];
      }
    }
    rule->npatches = N[0] * N[1] * N[2];
    rule->patchsize = P[0] * P[1] * P[2];
    rule->patchind.resize((size_t)rule->npatches * rule->patchsize);
    rule->patchweight.resize(rule->patchind.size());
    for (int i = 0; i < N[0]; i++)
      for (int j = 0; j < N[1]; j++)
        for (int k = 0; k < N[2]; k++)
          for (int a = 0; a < P[0]; a++)
            for (int b = 0; b < P[1]; b++)
              for (int c = 0; c < P[2]; c++) {
                const int patch = (i * N[1] + j) * N[2] + k, pi = (a * P[1] + b) * P[2] + c;
                const int ie = i * P[0] + a, je = j * P[1] + b, ke = k * P[2] + c;
                rule->patchind[patch * rule->patchsize + pi] = (ie * Q[1] + je) * Q[2] + ke;
                rule->patchweight[patch * rule->patchsize + pi] = rule->w[0][ie] * rule->w[1][je] * rule->w[2][je];
              }
  }
  if (npatches) *npatches = rule->npatches;
  if (patchsize) *patchsize = rule->patchsize;
  if (ind) *ind = rule->patchind.data();
  if (weight) *weight = rule->patchweight.data();
  return 0;
}

dErr dRuleComputePhysical(dRule rule, const dScalar jac[], dReal jinv[], dReal jw[]) {
  if (!rule || !jinv || !jw) return set_error("null argument");
  const int n = rule->Q[0] * rule->Q[1] * rule->Q[2];
  DCHK(dRuleGetNodeWeight(rule, nullptr, jw));
  for (int i = 0; i < n; i++) {
    if (!jac) {
      for (int k = 0; k < 9; k++) jinv[9 * i + k] = (k % 4 == 0) ? 1.0 : 0.0;
      continue;
    }
    const double det = invert3_host(jac + 9 * i, jinv + 9 * i);
    if (det < 0.) return set_error("Negative Jacobian at node %d", i);
    jw[i] *= det;
  }
  return 0;
}

dErr dJacobiGetEFS(dJacobi jac, dInt n, const dEntTopology topo[], const dPolynomialOrder order[], const dRule rules[], dEFS **efs) {
  if (!jac || !efs || (n > 0 && (!topo || !order || !rules))) return set_error("null argument");
  *efs = nullptr;
  dEFS *arr = (dEFS *)malloc(sizeof(dEFS) * (size_t)std::max<dInt>(n, 1));
  if (!arr) return set_error("out of host memory");
  for (dInt i = 0; i < n; i++) {
    if (topo[i] != dTOPO_HEX) {
      free(arr);
      return set_error("dJacobiGetEFS: topology %d not supported (hexahedra only)", (int)topo[i]);
    }
    dErr e;
    if (jac->modal) {  // dJacobiGetEFS_Modal (modal.c:343-370): the total order of the degree
      e = jacobi_efs_modal(jac, dPolynomialOrderMax(order[i]), rules[i], &arr[i]);
    } else if (rules[i]->facet >= 0) {
      e = set_error("dJacobiGetEFS: tensor element spaces on facet rules are not built (dFacetIterator evaluates faces)");
    } else {
      const dInt deg[3] = {dPolynomialOrder1D(order[i], 0), dPolynomialOrder1D(order[i], 1), dPolynomialOrder1D(order[i], 2)};
      e = jacobi_efs(jac, deg, rules[i]->method, rules[i]->order, &arr[i], rules[i]->family);
    }
    if (e) {
      free(arr);
      return e;
    }
  }
  *efs = arr;
  return 0;
}

// dJacobiGetNodeCount (jacobi.c:254-264): interior and expanded node counts per entity. Tensor type
// (dJacobiGetNodeCount_Tensor, tensor.c:249-281): interior prod max(0, p_d - 1), expanded prod (p_d + 1) over the
// entity's directions (hexahedron 3, quadrilateral 2, line 1, point: 1 and 1). Modal type (modal.c:297-310): the
// modes of the total order, both counts (ModalPCount; regions only, as this library's modal spaces).
dErr dJacobiGetNodeCount(dJacobi jac, dInt count, const dEntTopology top[], const dPolynomialOrder deg[], dInt inode[], dInt xnode[]) {
  if (!jac || (count > 0 && (!top || !deg))) return set_error("null argument");
  for (dInt i = 0; i < count; i++) {
    if (jac->modal) {
      const int o = dPolynomialOrderMax(deg[i]);
      if (top[i] != dTOPO_HEX) return set_error("dJacobiGetNodeCount: modal bases on topology %d not built (hexahedra only)", (int)top[i]);
      if (o < 0 || o > 3) return set_error("Order %d for type region", o);
      if (inode) inode[i] = kModalCount[o];
      if (xnode) xnode[i] = kModalCount[o];
      continue;
    }
    int dims;
    switch (top[i]) {
      case dTOPO_HEX: dims = 3; break;
      case dTOPO_QUAD: dims = 2; break;
      case dTOPO_LINE: dims = 1; break;
      case dTOPO_POINT: dims = 0; break;
      default: return set_error("Topology %d not supported", (int)top[i]);
    }
    int ic = 1, xc = 1;
    for (int d = 0; d < dims; d++) {
      const int p = dPolynomialOrder1D(deg[i], d);
      ic *= std::max(0, p - 1);
      xc *= p + 1;
    }
    if (inode) inode[i] = ic;
    if (xnode) xnode[i] = xc;
  }
  return 0;
}

dErr dJacobiSetType(dJacobi jac, const char *type) {
  if (!jac || !type) return set_error("null argument");
  if (!strcmp(type, dJACOBI_TENSOR)) jac->modal = 0;
  else if (!strcmp(type, dJACOBI_MODAL)) jac->modal = 1;
  else return set_error("Unable to find requested dJacobi type %s", type);
  return 0;
}

dErr dJacobiGetType(dJacobi jac, const char **type) {
  if (!jac || !type) return set_error("null argument");
  *type = jac->modal ? dJACOBI_MODAL : dJACOBI_TENSOR;
  return 0;
}

// the reference's dJacobiModalSetFamily looks its implementation up under a name the modal type does not compose
// (modal.c:413-418 against 385), so it never reaches the check of dJacobiModalSetFamily_Modal (modal.c:273-281);
// here the check applies on a modal dJacobi
dErr dJacobiModalSetFamily(dJacobi jac, dJacobiModalFamily family) {
  if (!jac) return set_error("null dJacobi");
  if (!jac->modal) return 0;
  if (family != dJACOBI_MODAL_P_DISCONTINUOUS) return set_error("dJacobiModalSetFamily: only P-discontinuous");
  return 0;
}

// dEFSGetExplicit (jacobi.c:508-559): the basis and its (mapped) derivatives at the rule points; the reference's
// generic path applies INTERP and GRAD to each unit vector, the same numbers as the products formed here
dErr dEFSGetExplicit(dEFS efs, const dReal jinv[], dInt *Q, dInt *P, const dReal **basis, const dReal **deriv) {
  if (!efs || !Q || !P || !basis || !deriv) return set_error("null argument");
  const int nq = efs->Q[0] * efs->Q[1] * efs->Q[2], np = efs->P[0] * efs->P[1] * efs->P[2];
  double *B = (double *)malloc(sizeof(double) * (size_t)std::max(nq * np, 1));
  double *G = (double *)malloc(sizeof(double) * 3 * (size_t)std::max(nq * np, 1));
  if (!B || !G) {
    free(B);
    free(G);
    return set_error("out of host memory");
  }
  if (efs->modal >= 0) {  // dEFSApply_Modal_All ignores the mapping (modaltopo.c:73)
    std::copy(efs->h_tab.begin(), efs->h_tab.begin() + (size_t)nq * np, B);
    std::copy(efs->h_tab.begin() + (size_t)nq * np, efs->h_tab.begin() + (size_t)nq * np * 4, G);
  } else {
    const int *Pn = efs->P, *Qn = efs->Q;
    for (int q = 0; q < nq; q++) {
      const int a = q / (Qn[1] * Qn[2]), b = (q / Qn[2]) % Qn[1], c = q % Qn[2];
      for (int k = 0; k < np; k++) {
        const int ki = k / (Pn[1] * Pn[2]), kj = (k / Pn[2]) % Pn[1], kk = k % Pn[2];
        const double Bx = efs->b[0].B[a * Pn[0] + ki], By = efs->b[1].B[b * Pn[1] + kj], Bz = efs->b[2].B[c * Pn[2] + kk];
        const double Dx = efs->b[0].D[a * Pn[0] + ki], Dy = efs->b[1].D[b * Pn[1] + kj], Dz = efs->b[2].D[c * Pn[2] + kk];
        const double r[3] = {Dx * By * Bz, Bx * Dy * Bz, Bx * By * Dz};
        B[(size_t)q * np + k] = Bx * By * Bz;
        double *g = G + ((size_t)q * np + k) * 3;
        for (int e = 0; e < 3; e++)  // TensorRuleMapping (efstopo.c:557-590): sum_k r_k jinv[q][k][e]
          g[e] = jinv ? r[0] * jinv[q * 9 + e] + r[1] * jinv[q * 9 + 3 + e] + r[2] * jinv[q * 9 + 6 + e] : r[e];
      }
    }
  }
  *Q = nq;
  *P = np;
  *basis = B;
  *deriv = G;
  return 0;
}

dErr dEFSRestoreExplicit(dEFS efs, const dReal jinv[], dInt *Q, dInt *P, const dReal **basis, const dReal **deriv) {
  (void)jinv;
  if (!efs || !Q || !P || !basis || !deriv) return set_error("null argument");
  free((void *)*basis);
  free((void *)*deriv);
  *Q = *P = 0;
  *basis = *deriv = nullptr;
  return 0;
}

dErr dEFSGetRule(dEFS efs, dRule *rule) {
  if (!efs || !rule) return set_error("null argument");
  *rule = efs->rule;
  return 0;
}

// dEFSGetExplicitSparse (src/jacobi/interface/jacobi.c:592-609): Q1 bases on the GLL sub-cells of a SPARSE rule
// (dEFSGetExplicitSparse_Tensor_Hex, efstopo.c:660-717, when every patch has 8 points and the patches are the
// element's sub-cells) or else the element's own basis at each patch's points (dEFSGetExplicitSparse_Basic,
// jacobi.c:611-643). cjinv: inverse Jacobians of the element's points, read at index pidx*8+q on the sub-cell
// path and at qidx[qidx[pidx*Q+q]] on the basic path (both the reference's indexing).
dErr dEFSGetExplicitSparse(dEFS efs, dInt npatches, dInt Q, const dInt qidx[], const dReal cjinv[], dInt eoffset, dInt *P, dInt eidx[],
                           dReal interp[], dReal deriv[]) {
  if (!efs || !qidx || !P || !eidx || !interp || !deriv) return set_error("null argument");
  if (efs->modal >= 0) return set_error("dEFSGetExplicitSparse: not available for a modal element");  // jacobi.c:606
  if (npatches <= 0 || Q <= 0) return set_error("dEFSGetExplicitSparse: npatches and Q must be positive");
  const int px = efs->P[0] - 1, py = efs->P[1] - 1, pz = efs->P[2] - 1;
  static const double s1 = 0.78867513459481287, s0 = 0.21132486540518713;
  const double interp1[2][2] = {{s1, s0}, {s0, s1}}, deriv1[2][2] = {{-1., 1.}, {-1., 1.}};
  if (Q == 8 && px * py * pz == npatches) {
    *P = 8;
    for (int i = 0; i < px; i++)
      for (int j = 0; j < py; j++)
        for (int k = 0; k < pz; k++) {
          const int pidx = (i * py + j) * pz + k;
          for (int b = 0; b < 8; b++) {
            const int bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
            eidx[pidx * 8 + b] = eoffset + ((i + bi) * (py + 1) + j + bj) * (pz + 1) + k + bk;
          }
          for (int q = 0; q < 8; q++) {
            const int ii = q >> 2, jj = (q >> 1) & 1, kk = q & 1;
            if (qidx[pidx * Q + q] != ((i * 2 + ii) * py * 2 + (j * 2 + jj)) * pz * 2 + (k * 2 + kk))
              return set_error("dEFSGetExplicitSparse: unexpected qidx at patch %d point %d", pidx, q);
            double M[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
            if (cjinv) std::copy(cjinv + (pidx * 8 + q) * 9, cjinv + (pidx * 8 + q) * 9 + 9, M);
            for (int b = 0; b < 8; b++) {
              const int bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
              const int off = (pidx * Q + q) * 8 + b;
              const double dX = deriv1[ii][bi] * interp1[jj][bj] * interp1[kk][bk];
              const double dY = interp1[ii][bi] * deriv1[jj][bj] * interp1[kk][bk];
              const double dZ = interp1[ii][bi] * interp1[jj][bj] * deriv1[kk][bk];
              interp[off] = interp1[ii][bi] * interp1[jj][bj] * interp1[kk][bk];
              for (int l = 0; l < 3; l++) deriv[off * 3 + l] = dX * M[0 * 3 + l] + dY * M[1 * 3 + l] + dZ * M[2 * 3 + l];
            }
          }
        }
    return 0;
  }
  // the element's own basis, one row per patch point (through qidx into element-natural order)
  const int *Pn = efs->P, *Qn = efs->Q, eP = Pn[0] * Pn[1] * Pn[2], eQ = Qn[0] * Qn[1] * Qn[2];
  *P = eP;
  for (int pt = 0; pt < npatches; pt++) {
    for (int k = 0; k < eP; k++) eidx[pt * eP + k] = eoffset + k;
    for (int j = 0; j < Q; j++) {
      const int pq = pt * Q + j, eq = qidx[pq];
      if (eq < 0 || eq >= eQ) return set_error("dEFSGetExplicitSparse: qidx %d out of range", eq);
      const int a = eq / (Qn[1] * Qn[2]), b = (eq / Qn[2]) % Qn[1], c = eq % Qn[2];
      // the reference first reorders cjinv with ecjinv[i] = cjinv[qidx[i]] and then evaluates the element basis at
      // element point eq with ecjinv[eq] (jacobi.c:620-626): the point's inverse Jacobian is cjinv[qidx[eq]]
      double M[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
      if (cjinv) {
        const int src = qidx[eq];
        std::copy(cjinv + src * 9, cjinv + src * 9 + 9, M);
      }
      for (int k = 0; k < eP; k++) {
        const int ki = k / (Pn[1] * Pn[2]), kj = (k / Pn[2]) % Pn[1], kk = k % Pn[2];
        const double Bx = efs->b[0].B[a * Pn[0] + ki], By = efs->b[1].B[b * Pn[1] + kj], Bz = efs->b[2].B[c * Pn[2] + kk];
        const double Dx = efs->b[0].D[a * Pn[0] + ki], Dy = efs->b[1].D[b * Pn[1] + kj], Dz = efs->b[2].D[c * Pn[2] + kk];
        const double d0 = Dx * By * Bz, d1 = Bx * Dy * Bz, d2 = Bx * By * Dz;
        interp[pq * eP + k] = Bx * By * Bz;
        for (int l = 0; l < 3; l++) deriv[(pq * eP + k) * 3 + l] = d0 * M[0 * 3 + l] + d1 * M[1 * 3 + l] + d2 * M[2 * 3 + l];
      }
    }
  }
  return 0;
}

// dFSCreateExpandedVector / dFSCreateGlobalVector (include/dohpfs.h:77-78): zeroed device vectors of the space's
// expanded (nexp * bs) and global (n * bs) sizes; released with dVecDestroy
dErr dFSCreateExpandedVector(dFS fs, dScalar **x) {
  if (!fs || !x) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  const size_t bytes = (size_t)std::max<int64_t>(fs->nexp * fs->bs, 1) * sizeof(double);
  CUCHK(cudaMalloc(x, bytes));
  CUCHK(cudaMemsetAsync(*x, 0, bytes, fs->stream));
  return 0;
}

dErr dFSCreateGlobalVector(dFS fs, dScalar **x) {
  if (!fs || !x) return set_error("null argument");
  if (!fs->setup) return set_error("dFS not set up");
  const size_t bytes = (size_t)std::max<int64_t>(fs->n * fs->bs, 1) * sizeof(double);
  CUCHK(cudaMalloc(x, bytes));
  CUCHK(cudaMemsetAsync(*x, 0, bytes, fs->stream));
  return 0;
}

dErr dVecDestroy(dScalar **x) {
  if (!x || !*x) return 0;
  CUCHK(cudaFree(*x));
  *x = nullptr;
  return 0;
}

}  // extern "C"
