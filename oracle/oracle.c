/* CPU oracle for dohp's matrix-free hp-FEM operator path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the GPU product (dohp_gb300) is tested against. Only the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load this library. Each function restates the
 * algorithm of the dohp source lines it cites; comments name the file:line (relative to the dohp
 * project root). Written from the algorithm, not copied: loops, names and data layout are our own
 * except where the reference fixes a table or an ordering (those are marked "table as reference").
 */
#include "oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static char or_errbuf[512];
const char *or_last_error(void) { return or_errbuf; }
static int or_fail(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(or_errbuf, sizeof or_errbuf, fmt, ap);
  va_end(ap);
  return -1;
}
void or_free(void *p) { free(p); }

/* ----------------------------------------------------------------------------------------------
 * PRNG: splitmix64 (Steele, Lea, Flood 2014) -- used for seeded meshes and fields.
 * -------------------------------------------------------------------------------------------- */
uint64_t or_splitmix64(uint64_t *s)
{
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double or_uniform(uint64_t *s) { return (double)(or_splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

/* ----------------------------------------------------------------------------------------------
 * 1-D Gauss rules. The reference calls polylib zwgj/zwglj (src/jacobi/impls/tensor/polylib.c:182,272)
 * with alpha=beta=0; we compute the same Legendre nodes by Newton iteration on the three-term
 * recurrence (Golub & Welsch give the same roots), in long double, ascending order.
 * -------------------------------------------------------------------------------------------- */
static void legendre_pd(int n, long double x, long double *pn, long double *dpn, long double *pnm1)
{
  long double p0 = 1.0L, p1 = x;
  if (n == 0) { *pn = 1; *dpn = 0; *pnm1 = 0; return; }
  for (int k = 1; k < n; k++) {
    long double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
    p0 = p1; p1 = p2;
  }
  *pn = p1; *pnm1 = p0;
  *dpn = n * (x * p1 - p0) / (x * x - 1.0L);
}

void or_gauss(int n, double *x, double *w)
{
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < n; i++) {
    long double z = -cosl(pi * (i + 0.75L) / (n + 0.5L)), pn, dpn, pm;
    for (int it = 0; it < 100; it++) {
      legendre_pd(n, z, &pn, &dpn, &pm);
      long double dz = pn / dpn;
      z -= dz;
      if (fabsl(dz) < 1e-19L) break;
    }
    legendre_pd(n, z, &pn, &dpn, &pm);
    x[i] = (double)z;
    w[i] = (double)(2.0L / ((1.0L - z * z) * dpn * dpn));
  }
}

void or_lobatto(int n, double *x, double *w)
{
  const long double pi = 3.141592653589793238462643383279502884L;
  const int N = n - 1; /* polynomial degree */
  if (n == 1) { x[0] = 0; w[0] = 2; return; }
  for (int i = 0; i < n; i++) {
    long double z = -cosl(pi * i / N), pn = 0, dpn, pm = 0;
    if (i == 0 || i == N) {
      z = (i == 0) ? -1.0L : 1.0L;
    } else {
      for (int it = 0; it < 100; it++) { /* roots of (1-z^2) P'_N: Newton on z P_N - P_{N-1} */
        legendre_pd(N, z, &pn, &dpn, &pm);
        long double f = z * pn - pm, df = (N + 1) * pn;
        long double dz = f / df;
        z -= dz;
        if (fabsl(dz) < 1e-19L) break;
      }
    }
    if (i == 0 || i == N) { pn = (i == 0 && (N & 1)) ? -1.0L : 1.0L; }
    else legendre_pd(N, z, &pn, &dpn, &pm);
    x[i] = (double)z;
    w[i] = (double)(2.0L / (N * (N + 1) * pn * pn));
  }
}

/* Lagrange basis on nodes[P] evaluated (value, derivative) at t. */
static void lagrange_eval(int P, const double *nodes, double t, double *val, double *der)
{
  for (int j = 0; j < P; j++) {
    long double v = 1, d = 0;
    for (int m = 0; m < P; m++) {
      if (m == j) continue;
      long double inv = 1.0L / ((long double)nodes[j] - nodes[m]);
      d = d * (t - nodes[m]) * inv + v * inv;
      v = v * (t - nodes[m]) * inv;
    }
    val[j] = (double)v;
    der[j] = (double)d;
  }
}

/* TensorBasisCreate (src/jacobi/impls/tensor/tensor.c:22-109): GLL nodal basis with P nodes evaluated
 * at the Q rule points. deriv = interp * (collocation derivative) (tensor.c:54-62), which equals the
 * derivative of the Lagrange basis at the rule points. P==1 is the degenerate constant basis. */
int or_tensor_basis(int P, int Q, const double *rcoord, double *interp, double *deriv, double *node, double *weight)
{
  if (P <= 0) return or_fail("TensorBasis must be at least first order, given %d", P);
  if (P == 1) {
    for (int i = 0; i < Q; i++) { interp[i] = 1.0; deriv[i] = 0.0; }
    node[0] = 0.0; weight[0] = 2.0;
    return 0;
  }
  or_lobatto(P, node, weight);
  for (int i = 0; i < Q; i++) lagrange_eval(P, node, rcoord[i], interp + i * P, deriv + i * P);
  return 0;
}

/* TensorGetRule (src/jacobi/quadrature/impls/tensor/tensorquad.c:51-118) and the SPARSE two-point
 * composite rule two_point_private (tensorquad.c:32-49): 2 Gauss (or Lobatto) points in each GLL
 * sub-interval of the degree order/2 element, weight h/2. */
int or_rule_1d(int method, int family, int order, double *x, double *w)
{
  int size;
  if (!(0 <= order && order < 100)) return or_fail("rule order %d out of bounds", order);
  if (method == 1) { /* SPARSE */
    size = order > 0 ? order : 1;
    if (size == 1) { x[0] = 0; w[0] = 2; return 1; }
    {
      int nel = size / 2;
      double iv[101], unused[101];
      double x0 = family == 0 ? -0.57735026918962573 : -1.0, x1 = -x0;
      or_lobatto(nel + 1, iv, unused);
      for (int i = 0; i < nel; i++) {
        double h = iv[i + 1] - iv[i];
        x[2 * i + 0] = iv[i] + (x0 + 1) * h / 2.;
        x[2 * i + 1] = iv[i] + (x1 + 1) * h / 2.;
        w[2 * i + 0] = h / 2.;
        w[2 * i + 1] = h / 2.;
      }
      return size;
    }
  }
  if (method == 0) size = family == 0 ? 1 + order / 2 : 2 + order / 2; /* FAST */
  else if (method == 2) {                                               /* SELF */
    if (family != 1) return or_fail("SELF needs Lobatto");
    size = 1 + order / 2;
  } else return or_fail("quadrature method %d", method);
  if (size == 1) { x[0] = 0; w[0] = 2; return 1; }
  if (family == 0) or_gauss(size, x, w);
  else or_lobatto(size, x, w);
  return size;
}

/* dRulePatchSetup_Tensor (tensorquad.c:120-169). SPARSE tiles the element with 2x2x2 point patches,
 * other methods use one patch. The patch weight uses the y-direction weight index for z, exactly as
 * the reference (tensorquad.c:159-161); the weights are not consumed by any computation. */
int or_rule_patches(int method, const int Q[3], const double *w0, const double *w1, const double *w2,
                    int *patchsize, int *ind, double *weight)
{
  int N[3], P[3];

  for (int i = 0; i < 3; i++) {
    if (method == 1) {
      P[i] = Q[i] > 1 ? 2 : 1;
      N[i] = Q[i] / P[i];
      if (N[i] * P[i] != Q[i]) return or_fail("odd sparse rule size %d", Q[i]);
    } else { N[i] = 1; P[i] = Q[i]; }
  }
  const int NN = N[0] * N[1] * N[2], PP = P[0] * P[1] * P[2];
  for (int i = 0; i < N[0]; i++)
    for (int j = 0; j < N[1]; j++)
      for (int k = 0; k < N[2]; k++)
        for (int ii = 0; ii < P[0]; ii++)
          for (int jj = 0; jj < P[1]; jj++)
            for (int kk = 0; kk < P[2]; kk++) {
              int patch = (i * N[1] + j) * N[2] + k, pidx = (ii * P[1] + jj) * P[2] + kk;
              int ie = i * P[0] + ii, je = j * P[1] + jj, ke = k * P[2] + kk;
              ind[patch * PP + pidx] = (ie * Q[1] + je) * Q[2] + ke;
              weight[patch * PP + pidx] = w0[ie] * w1[je] * w2[je];
              (void)ke;
            }
  *patchsize = PP;
  return NN;
}

/* ----------------------------------------------------------------------------------------------
 * Element kernels
 * -------------------------------------------------------------------------------------------- */
/* TensorMult_Hex_nounroll (src/jacobi/impls/tensor/inlinetmulthex.h:19-100): three sum-factorized
 * stages, out[l,m,n,d] (+)= sum_{ijk} Az[n,k] Ay[m,j] Ax[l,i] in[i,j,k,d]. */
void or_tensor_mult_hex(int D, const int P[3], const int Q[3], const double *A[3], const double *in, double *out, int imode)
{
  const int JKD = P[1] * P[2] * D, KD = P[2] * D;
  double a[Q[0] * JKD], b[Q[0] * Q[1] * KD]; /* stack work arrays, as the reference (inlinetmulthex.h:21) */
  memset(a, 0, sizeof a);
  memset(b, 0, sizeof b);
  if (imode == OR_INSERT) memset(out, 0, sizeof(double) * Q[0] * Q[1] * Q[2] * D);
  for (int l = 0; l < Q[0]; l++)
    for (int i = 0; i < P[0]; i++) {
      const double c = A[0][l * P[0] + i];
      for (int t = 0; t < JKD; t++) a[l * JKD + t] += c * in[i * JKD + t];
    }
  for (int i = 0; i < Q[0]; i++)
    for (int l = 0; l < Q[1]; l++)
      for (int j = 0; j < P[1]; j++) {
        const double c = A[1][l * P[1] + j];
        for (int t = 0; t < KD; t++) b[(i * Q[1] + l) * KD + t] += c * a[i * JKD + j * KD + t];
      }
  for (int ij = 0; ij < Q[0] * Q[1]; ij++)
    for (int l = 0; l < Q[2]; l++)
      for (int d = 0; d < D; d++) {
        double s = 0;
        for (int k = 0; k < P[2]; k++) s += A[2][l * P[2] + k] * b[(ij * P[2] + k) * D + d];
        out[(ij * Q[2] + l) * D + d] += s;
      }
}

/* TensorRuleMapping / TensorRuleMappingTranspose / TensorRuleNoMapping (efstopo.c:518-623). */
static void rule_mapping(int Q, const double *jinv, int D, const double *in, double *out, int imode)
{
  for (int i = 0; i < Q; i++)
    for (int d = 0; d < D; d++)
      for (int e = 0; e < 3; e++) {
        double v;
        if (jinv) v = in[(0 * Q + i) * D + d] * jinv[i * 9 + 0 * 3 + e] + in[(1 * Q + i) * D + d] * jinv[i * 9 + 1 * 3 + e] + in[(2 * Q + i) * D + d] * jinv[i * 9 + 2 * 3 + e];
        else v = in[(e * Q + i) * D + d];
        if (imode == OR_INSERT) out[(i * D + d) * 3 + e] = v;
        else out[(i * D + d) * 3 + e] += v;
      }
}
static void rule_mapping_transpose(int Q, const double *jinv, int D, const double *in, double *out)
{
  for (int i = 0; i < Q; i++)
    for (int d = 0; d < D; d++)
      for (int e = 0; e < 3; e++)
        out[(e * Q + i) * D + d] = in[(i * D + d) * 3 + 0] * jinv[i * 9 + e * 3 + 0] + in[(i * D + d) * 3 + 1] * jinv[i * 9 + e * 3 + 1] + in[(i * D + d) * 3 + 2] * jinv[i * 9 + e * 3 + 2];
}

/* dEFSApply_Tensor_Hex (efstopo.c:368-423). interp/deriv are [Q][P] per direction; transposes are
 * formed here (the reference stores them explicitly, tensor.c:67-72). */
int or_efs_apply_hex(const int P[3], const int Q[3], const double *interp[3], const double *deriv[3],
                     const double *jinv, int D, const double *in, double *out, int amode, int imode)
{
  double itb[3][32 * 32], dtb[3][32 * 32], *it[3] = {itb[0], itb[1], itb[2]}, *dt[3] = {dtb[0], dtb[1], dtb[2]};
  const double *A[3];
  const int nq = Q[0] * Q[1] * Q[2];
  for (int d = 0; d < 3; d++) {
    for (int i = 0; i < Q[d]; i++)
      for (int j = 0; j < P[d]; j++) {
        it[d][j * Q[d] + i] = interp[d][i * P[d] + j];
        dt[d][j * Q[d] + i] = deriv[d][i * P[d] + j];
      }
  }
  int rc = 0;
  switch (amode) {
  case OR_INTERP:
    A[0] = interp[0]; A[1] = interp[1]; A[2] = interp[2];
    or_tensor_mult_hex(D, P, Q, A, in, out, imode);
    break;
  case OR_INTERP_TRANSPOSE:
    A[0] = it[0]; A[1] = it[1]; A[2] = it[2];
    or_tensor_mult_hex(D, Q, P, A, in, out, imode);
    break;
  case OR_GRAD: {
    double df[3 * nq * D];
    for (int g = 0; g < 3; g++) {
      for (int d = 0; d < 3; d++) A[d] = (d == g) ? deriv[d] : interp[d];
      or_tensor_mult_hex(D, P, Q, A, in, df + g * nq * D, OR_INSERT);
    }
    rule_mapping(nq, jinv, D, df, out, imode);
  } break;
  case OR_GRAD_TRANSPOSE: {
    double df[3 * nq * D];
    if (!jinv) { rc = or_fail("No Jinv, need a mapping"); break; }
    rule_mapping_transpose(nq, jinv, D, in, df);
    if (imode == OR_INSERT) memset(out, 0, sizeof(double) * P[0] * P[1] * P[2] * D);
    for (int g = 0; g < 3; g++) {
      for (int d = 0; d < 3; d++) A[d] = (d == g) ? dt[d] : it[d];
      or_tensor_mult_hex(D, Q, P, A, df + g * nq * D, out, OR_ADD);
    }
  } break;
  default: rc = or_fail("invalid dApplyMode %d", amode);
  }
  return rc;
}

/* dGeomInvert3 (include/dohpgeom.h:57-79): cofactor inverse of a row-major 3x3. */
void or_invert3(const double a[9], double b[9], double *det)
{
  const double c0 = a[4] * a[8] - a[7] * a[5];
  const double c3 = -(a[3] * a[8] - a[6] * a[5]);
  const double c6 = a[3] * a[7] - a[6] * a[4];
  const double dt = a[0] * c0 + a[1] * c3 + a[2] * c6;
  const double id = 1.0 / dt;
  b[0] = id * c0;
  b[1] = -id * (a[1] * a[8] - a[7] * a[2]);
  b[2] = id * (a[1] * a[5] - a[4] * a[2]);
  b[3] = id * c3;
  b[4] = id * (a[0] * a[8] - a[6] * a[2]);
  b[5] = -id * (a[0] * a[5] - a[3] * a[2]);
  b[6] = id * c6;
  b[7] = -id * (a[0] * a[7] - a[6] * a[1]);
  b[8] = id * (a[0] * a[4] - a[3] * a[1]);
  *det = dt;
}

/* dRuleComputePhysical (src/jacobi/interface/jacobi.c:383-414): jinv and jw = w * det J; error if det < 0 */
static int compute_physical(int nq, const double *w, const double *jac, double *jinv, double *jw)
{
  for (int i = 0; i < nq; i++) {
    double det;
    or_invert3(jac + 9 * i, jinv + 9 * i, &det);
    if (det < 0.) return or_fail("Negative Jacobian at node %d", i);
    jw[i] = w[i] * det;
  }
  return 0;
}

/* dEFSGetExplicitSparse_Tensor_Hex (efstopo.c:660-717): Q1 basis on each GLL sub-cell at the 2x2x2
 * patch points. interp1/deriv1 are the reference's constants (table as reference); the derivative is
 * with respect to the unit sub-cell coordinate (no 1/h_sub factor) and dXdx is read from cjinv at the
 * patch-natural index (pidx*8+pqidx), as the reference does. */
int or_explicit_sparse_hex(int px, int py, int pz, int npatches, int Q, const int *qidx, const double *cjinv,
                           int eoffset, int *P, int *eidx, double *interp, double *deriv)
{
  static const double i1[2][2] = {{0.78867513459481287, 0.21132486540518713}, {0.21132486540518713, 0.78867513459481287}};
  static const double d1[2][2] = {{-1., 1.}, {-1., 1.}};
  static const double eye[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (Q != 8 || px * py * pz != npatches) return or_fail("sparse explicit basis needs Q=8 patches");
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
          const int qi = q >> 2, qj = (q >> 1) & 1, qk = q & 1;
          const double *J = cjinv ? cjinv + (size_t)(pidx * 8 + q) * 9 : eye;
          if (qidx[pidx * Q + q] != ((i * 2 + qi) * py * 2 + (j * 2 + qj)) * pz * 2 + (k * 2 + qk)) return or_fail("Unexpected qidx");
          for (int b = 0; b < 8; b++) {
            const int bi = b >> 2, bj = (b >> 1) & 1, bk = b & 1;
            const size_t o = (size_t)(pidx * Q + q) * 8 + b;
            const double dX = d1[qi][bi] * i1[qj][bj] * i1[qk][bk];
            const double dY = i1[qi][bi] * d1[qj][bj] * i1[qk][bk];
            const double dZ = i1[qi][bi] * i1[qj][bj] * d1[qk][bk];
            interp[o] = i1[qi][bi] * i1[qj][bj] * i1[qk][bk];
            for (int e = 0; e < 3; e++) deriv[o * 3 + e] = dX * J[0 * 3 + e] + dY * J[1 * 3 + e] + dZ * J[2 * 3 + e];
          }
        }
      }
  return 0;
}


/* dEFSGetExplicitSparse_Basic (src/jacobi/interface/jacobi.c:611-643): dense explicit basis of the
 * element (dEFSGetExplicit, jacobi.c:508-559, via unit-vector applies) reordered to patch-natural
 * order, used when the rule's patches do not match the element's GLL sub-cells. */
static int explicit_sparse_basic(const int P3[3], const int Q3[3], const double *interp[3], const double *deriv[3],
                                 int npatches, int Q, const int *qidx, const double *cjinv, int eoffset,
                                 int *P, int *eidx, double *ointerp, double *oderiv)
{
  const int eP = P3[0] * P3[1] * P3[2], eQ = Q3[0] * Q3[1] * Q3[2];
  double *ecj = NULL, *tmp = calloc(eP, sizeof(double)), *bas = malloc(sizeof(double) * eP * eQ), *der = malloc(sizeof(double) * eP * eQ * 3);
  if (cjinv) {
    ecj = malloc(sizeof(double) * 9 * npatches * Q);
    for (int i = 0; i < npatches * Q; i++) memcpy(ecj + 9 * i, cjinv + 9 * qidx[i], 9 * sizeof(double));
  }
  for (int i = 0; i < eP; i++) {
    memset(tmp, 0, sizeof(double) * eP);
    tmp[i] = 1.;
    or_efs_apply_hex(P3, Q3, interp, deriv, ecj, 1, tmp, bas + (size_t)i * eQ, OR_INTERP, OR_INSERT);
    or_efs_apply_hex(P3, Q3, interp, deriv, ecj, 1, tmp, der + (size_t)i * eQ * 3, OR_GRAD, OR_INSERT);
  }
  *P = eP;
  for (int i = 0; i < npatches; i++) {
    for (int k = 0; k < eP; k++) eidx[i * eP + k] = eoffset + k;
    for (int j = 0; j < Q; j++) {
      const int pq = i * Q + j, eq = qidx[pq];
      for (int k = 0; k < eP; k++) {
        ointerp[(size_t)pq * eP + k] = bas[(size_t)k * eQ + eq];
        for (int l = 0; l < 3; l++) oderiv[((size_t)pq * eP + k) * 3 + l] = der[((size_t)k * eQ + eq) * 3 + l];
      }
    }
  }
  free(ecj); free(tmp); free(bas); free(der);
  return 0;
}

int or_explicit_sparse(const int P3[3], const int Q3[3], const double *interp[3], const double *deriv[3],
                       int npatches, int Q, const int *qidx, const double *cjinv, int eoffset,
                       int *P, int *eidx, double *ointerp, double *oderiv)
{
  const int px = P3[0] - 1, py = P3[1] - 1, pz = P3[2] - 1;
  if (Q != 8 || px * py * pz != npatches)
    return explicit_sparse_basic(P3, Q3, interp, deriv, npatches, Q, qidx, cjinv, eoffset, P, eidx, ointerp, oderiv);
  return or_explicit_sparse_hex(px, py, pz, npatches, Q, qidx, cjinv, eoffset, P, eidx, ointerp, oderiv);
}

/* ----------------------------------------------------------------------------------------------
 * Modal (P-discontinuous) element bases of the modal dJacobi (src/jacobi/impls/modal/modal.c,
 * modaltopo.c), hexahedra. The reference tabulates sympy-generated Gram-Schmidt polynomials; they are
 * products of orthonormal Legendre polynomials Lh_n(t) = sqrt(n + 1/2) P_n(t), one factor per direction,
 * evaluated here from the closed forms of P_0..P_3. The mode order is the reference's (table as reference,
 * modal.c:141-238): its order-3 set has 18 modes, without the y^2 z and y z^2 products.
 * -------------------------------------------------------------------------------------------- */
static const int modal_hex_exp[18][3] = {
  {0, 0, 0},                                                    /* order 0 */
  {1, 0, 0}, {0, 1, 0}, {0, 0, 1},                              /* order 1 */
  {2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {0, 1, 1}, {1, 0, 1}, /* order 2 */
  {3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {1, 2, 0}, {2, 0, 1}, {1, 0, 2}, {1, 1, 1} /* order 3 */
};

/* ModalPCount (modal.c:15-42), region case */
int or_modal_count(int order)
{
  static const int count[4] = {1, 4, 10, 18};
  if (order < 0 || order > 3) return or_fail("Order %d for type region", order);
  return count[order];
}

static void legendre_hat(int n, double t, double *v, double *d)
{
  double p, dp;
  switch (n) {
  case 0: p = 1; dp = 0; break;
  case 1: p = t; dp = 1; break;
  case 2: p = 1.5 * t * t - 0.5; dp = 3 * t; break;
  default: p = 2.5 * t * t * t - 1.5 * t; dp = 7.5 * t * t - 1.5; break;
  }
  *v = sqrt(n + 0.5) * p;
  *d = sqrt(n + 0.5) * dp;
}

/* dEFSModalSetUp (modal.c:45-240), hexahedra: interp [Q][P], deriv [Q][P][3] at the Q points rcoord [Q][3].
 * Returns P, or -1 for an unsupported order. */
int or_modal_basis(int order, int Q, const double *rcoord, double *interp, double *deriv)
{
  const int P = or_modal_count(order);
  if (P < 0) return -1;
  for (int i = 0; i < Q; i++) {
    for (int j = 0; j < P; j++) {
      double v[3], d[3];
      for (int k = 0; k < 3; k++) legendre_hat(modal_hex_exp[j][k], rcoord[3 * i + k], &v[k], &d[k]);
      interp[i * P + j] = v[0] * v[1] * v[2];
      deriv[(i * P + j) * 3 + 0] = d[0] * v[1] * v[2];
      deriv[(i * P + j) * 3 + 1] = v[0] * d[1] * v[2];
      deriv[(i * P + j) * 3 + 2] = v[0] * v[1] * d[2];
    }
  }
  return P;
}

/* dEFSApply_Modal_All (modaltopo.c:73-126): dense products with the tables; the mapping (jinv) is not used,
 * GRAD gives reference-coordinate derivatives [Q][D][3]; GRAD_TRANSPOSE is not implemented (an error). */
int or_modal_apply(int P, int Q, const double *interp, const double *deriv, int D, const double *in, double *out,
                   int amode, int imode)
{
  switch (amode) {
  case OR_INTERP:
    if (imode == OR_INSERT) memset(out, 0, sizeof(double) * Q * D);
    for (int i = 0; i < Q; i++)
      for (int j = 0; j < P; j++)
        for (int c = 0; c < D; c++) out[i * D + c] += interp[i * P + j] * in[j * D + c];
    return 0;
  case OR_INTERP_TRANSPOSE:
    if (imode == OR_INSERT) memset(out, 0, sizeof(double) * P * D);
    for (int i = 0; i < Q; i++)
      for (int j = 0; j < P; j++)
        for (int c = 0; c < D; c++) out[j * D + c] += interp[i * P + j] * in[i * D + c];
    return 0;
  case OR_GRAD:
    if (imode == OR_INSERT) memset(out, 0, sizeof(double) * Q * D * 3);
    for (int i = 0; i < Q; i++)
      for (int j = 0; j < P; j++)
        for (int c = 0; c < D; c++)
          for (int e = 0; e < 3; e++) out[(i * D + c) * 3 + e] += deriv[(i * P + j) * 3 + e] * in[j * D + c];
    return 0;
  default: return or_fail("Apply-mode not implemented");
  }
}

/* ----------------------------------------------------------------------------------------------
 * Structured block mesh: entity creation order of dMeshGenerateBlock (genblock.c:206-402),
 * adjacency in canonical side order (dMeshGetAdjacency, mesh.c:1074-1191) and orientation
 * permutations (dMeshAdjacencyPermutations_Private, mesh.c:1039-1072; dohpgeom.h:97-150).
 * -------------------------------------------------------------------------------------------- */
typedef struct { int x, y, z; } ordr;

struct or_fs {
  int nx, ny, nz, bs;
  int64_t nv, ne, nf, nr, nents;
  double *vx;              /* vertex coordinates */
  int64_t *econn, *fconn, *hconn;
  signed char *fset;       /* per entity: boundary face set 0..5 of genblock, or -1 */
  int32_t *adjoff, *adjind, *adjperm;
  ordr *deg;               /* per entity degree after propagation */
  int32_t *ordered, *goff, *gcoff, *inodes;
  int64_t n, nc, nexp;
  int32_t *xstart, *emap, *edeg;
  double *xexp;            /* expanded coordinates [nr][8][3] */
  int hp;                  /* 1: interpolation constraints on p-nonconforming entities (extension) */
  double gll[16][16];      /* GLL nodes per degree (index p) */
  /* constrained rows (hp): emap[r] = -2 - k refers to entries cptr[k]..cptr[k+1] */
  int64_t ncrow, ccap, nent, entcap;
  int64_t *cptr;
  int32_t *ccol;
  double *cval;
  /* E as CSR over expanded rows (built after the constraints) */
  int64_t *eptr;
  int32_t *ecol;
  double *eval;
  /* E^T as CSR over closure nodes, expanded rows ascending (made on the first threaded apply) */
  int64_t *tptr, *trow;
  double *tval;
};

/* Lagrange basis on the degree-p GLL nodes at t */
static void gll_lagrange(const or_fs *m, int p, double t, double *L)
{
  const double *x = m->gll[p];
  for (int j = 0; j <= p; j++) {
    long double v = 1;
    for (int k = 0; k <= p; k++)
      if (k != j) v *= ((long double)t - x[k]) / ((long double)x[j] - x[k]);
    L[j] = (double)v;
  }
}

typedef struct { int n; int32_t col[2048]; double w[2048]; } rowacc;
static void acc_add(rowacc *a, int32_t col, double w)
{
  for (int i = 0; i < a->n; i++)
    if (a->col[i] == col) { a->w[i] += w; return; }
  a->col[a->n] = col;
  a->w[a->n] = w;
  a->n++;
}

static int64_t VI(const or_fs *m, int i, int j, int k) { return ((int64_t)i * m->ny + j) * m->nz + k; }

/* face index helpers (creation order: z-normal, y-normal, x-normal families) */
static int64_t FZ(const or_fs *m, int i, int j, int k) { return ((int64_t)i * (m->ny - 1) + j) * m->nz + k; }
static int64_t FY(const or_fs *m, int i, int j, int k) { return (int64_t)(m->nx - 1) * (m->ny - 1) * m->nz + ((int64_t)i * m->ny + j) * (m->nz - 1) + k; }
static int64_t FX(const or_fs *m, int i, int j, int k) { return (int64_t)(m->nx - 1) * (m->ny - 1) * m->nz + (int64_t)(m->nx - 1) * m->ny * (m->nz - 1) + ((int64_t)i * (m->ny - 1) + j) * (m->nz - 1) + k; }
static int64_t EZ(const or_fs *m, int i, int j, int k) { return ((int64_t)i * m->ny + j) * (m->nz - 1) + k; }
static int64_t EY(const or_fs *m, int i, int j, int k) { return (int64_t)m->nx * m->ny * (m->nz - 1) + ((int64_t)i * (m->ny - 1) + j) * m->nz + k; }
static int64_t EX(const or_fs *m, int i, int j, int k) { return (int64_t)m->nx * m->ny * (m->nz - 1) + (int64_t)m->nx * (m->ny - 1) * m->nz + ((int64_t)i * m->ny + j) * m->nz + k; }

/* canonical hex faces and quad edges (table as reference, include/dohpgeom.h:19,26) */
static const int CN_HQ[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {0, 3, 2, 1}, {4, 5, 6, 7}};
static const int CN_QL[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};

static int build_mesh(or_fs *m, const double box[6], double perturb, uint64_t seed)
{
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  m->nv = (int64_t)nx * ny * nz;
  m->nr = (int64_t)(nx - 1) * (ny - 1) * (nz - 1);
  m->nf = (int64_t)(nx - 1) * (ny - 1) * nz + (int64_t)(nx - 1) * ny * (nz - 1) + (int64_t)nx * (ny - 1) * (nz - 1);
  m->ne = (int64_t)nx * ny * (nz - 1) + (int64_t)nx * (ny - 1) * nz + (int64_t)(nx - 1) * ny * nz;
  m->nents = m->nv + m->ne + m->nf + m->nr;
  m->vx = malloc(sizeof(double) * 3 * m->nv);
  m->econn = malloc(sizeof(int64_t) * 2 * m->ne);
  m->fconn = malloc(sizeof(int64_t) * 4 * m->nf);
  m->hconn = malloc(sizeof(int64_t) * 8 * m->nr);
  m->fset = malloc(m->nents);
  memset(m->fset, -1, m->nents);
  uint64_t st = seed;
  /* vertices (genblock.c:206-226), then a seeded perturbation of interior vertices */
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        int64_t I = VI(m, i, j, k);
        signed char f = -1;
        if (i == 0) f = 3; else if (i == nx - 1) f = 1; else if (j == 0) f = 0; else if (j == ny - 1) f = 2; else if (k == 0) f = 4; else if (k == nz - 1) f = 5;
        m->fset[I] = f;
        m->vx[3 * I + 0] = box[0] + (box[1] - box[0]) * (1. * i / (nx - 1));
        m->vx[3 * I + 1] = box[2] + (box[3] - box[2]) * (1. * j / (ny - 1));
        m->vx[3 * I + 2] = box[4] + (box[5] - box[4]) * (1. * k / (nz - 1));
        if (perturb != 0 && i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && k > 0 && k < nz - 1) {
          const double h[3] = {(box[1] - box[0]) / (nx - 1), (box[3] - box[2]) / (ny - 1), (box[5] - box[4]) / (nz - 1)};
          for (int d = 0; d < 3; d++) m->vx[3 * I + d] += perturb * h[d] * (2.0 * or_uniform(&st) - 1.0);
        }
      }
  /* regions (genblock.c:230-247) */
  for (int i = 0; i < nx - 1; i++)
    for (int j = 0; j < ny - 1; j++)
      for (int k = 0; k < nz - 1; k++) {
        int64_t r = ((int64_t)i * (ny - 1) + j) * (nz - 1) + k, *c = m->hconn + 8 * r;
        c[0] = VI(m, i, j, k); c[1] = VI(m, i + 1, j, k); c[2] = VI(m, i + 1, j + 1, k); c[3] = VI(m, i, j + 1, k);
        c[4] = VI(m, i, j, k + 1); c[5] = VI(m, i + 1, j, k + 1); c[6] = VI(m, i + 1, j + 1, k + 1); c[7] = VI(m, i, j + 1, k + 1);
      }
  /* faces (genblock.c:306-346) */
  const int64_t F0 = m->nv + m->ne, E0 = m->nv;
  for (int i = 0; i < nx - 1; i++)
    for (int j = 0; j < ny - 1; j++)
      for (int k = 0; k < nz; k++) {
        int64_t f = FZ(m, i, j, k), *c = m->fconn + 4 * f;
        if (k == 0) m->fset[F0 + f] = 4;
        if (k == nz - 1) m->fset[F0 + f] = 5;
        c[0] = VI(m, i, j, k); c[1] = VI(m, i + 1, j, k); c[2] = VI(m, i + 1, j + 1, k); c[3] = VI(m, i, j + 1, k);
      }
  for (int i = 0; i < nx - 1; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz - 1; k++) {
        int64_t f = FY(m, i, j, k), *c = m->fconn + 4 * f;
        if (j == 0) m->fset[F0 + f] = 0;
        if (j == ny - 1) m->fset[F0 + f] = 2;
        c[0] = VI(m, i, j, k); c[1] = VI(m, i + 1, j, k); c[2] = VI(m, i + 1, j, k + 1); c[3] = VI(m, i, j, k + 1);
      }
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny - 1; j++)
      for (int k = 0; k < nz - 1; k++) {
        int64_t f = FX(m, i, j, k), *c = m->fconn + 4 * f;
        if (i == 0) m->fset[F0 + f] = 3;
        if (i == nx - 1) m->fset[F0 + f] = 1;
        c[0] = VI(m, i, j, k); c[1] = VI(m, i, j + 1, k); c[2] = VI(m, i, j + 1, k + 1); c[3] = VI(m, i, j, k + 1);
      }
  /* edges (genblock.c:352-397), boundary-set assignment chains as the reference */
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz - 1; k++) {
        int64_t e = EZ(m, i, j, k);
        signed char f = -1;
        if (i == 0) f = 0; else if (i == nx - 1) f = 2; else if (j == 0) f = 3; else if (j == ny - 1) f = 1;
        m->fset[E0 + e] = f;
        m->econn[2 * e] = VI(m, i, j, k); m->econn[2 * e + 1] = VI(m, i, j, k + 1);
      }
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny - 1; j++)
      for (int k = 0; k < nz; k++) {
        int64_t e = EY(m, i, j, k);
        signed char f = -1;
        if (i == 0) f = 0; else if (i == nx - 1) f = 2; else if (k == 0) f = 4; else if (k == nz - 1) f = 5;
        m->fset[E0 + e] = f;
        m->econn[2 * e] = VI(m, i, j, k); m->econn[2 * e + 1] = VI(m, i, j + 1, k);
      }
  for (int i = 0; i < nx - 1; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        int64_t e = EX(m, i, j, k);
        signed char f = -1;
        if (j == 0) f = 3; else if (j == ny - 1) f = 1; else if (k == 0) f = 4; else if (k == nz - 1) f = 5;
        m->fset[E0 + e] = f;
        m->econn[2 * e] = VI(m, i, j, k); m->econn[2 * e + 1] = VI(m, i + 1, j, k);
      }
  return 0;
}

/* Adjacency with permutations. Entity index order = vertices, edges, faces, regions (MOAB handle order). */
static int build_adjacency(or_fs *m)
{
  static const int hq_perm[8][4] = {{0, 1, 2, 3}, {3, 0, 1, 2}, {2, 3, 0, 1}, {1, 2, 3, 0}, {0, 3, 2, 1}, {1, 0, 3, 2}, {2, 1, 0, 3}, {3, 2, 1, 0}};
  const int64_t E0 = m->nv, F0 = m->nv + m->ne, R0 = m->nv + m->ne + m->nf;
  const int64_t nadj = 2 * m->ne + 4 * m->nf + 6 * m->nr;
  m->adjoff = malloc(sizeof(int32_t) * (m->nents + 1));
  m->adjind = malloc(sizeof(int32_t) * nadj);
  m->adjperm = malloc(sizeof(int32_t) * nadj);
  int64_t a = 0;
  for (int64_t v = 0; v < m->nv; v++) m->adjoff[v] = (int32_t)a;
  for (int64_t e = 0; e < m->ne; e++) {
    m->adjoff[E0 + e] = (int32_t)a;
    for (int s = 0; s < 2; s++) { m->adjind[a] = (int32_t)m->econn[2 * e + s]; m->adjperm[a] = 0; a++; }
  }
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  for (int64_t f = 0; f < m->nf; f++) {
    m->adjoff[F0 + f] = (int32_t)a;
    int64_t ed[4];
    const int64_t nzf = (int64_t)(nx - 1) * (ny - 1) * nz, nyf = (int64_t)(nx - 1) * ny * (nz - 1);
    if (f < nzf) {
      int k = (int)(f % nz), j = (int)((f / nz) % (ny - 1)), i = (int)(f / nz / (ny - 1));
      ed[0] = EX(m, i, j, k); ed[1] = EY(m, i + 1, j, k); ed[2] = EX(m, i, j + 1, k); ed[3] = EY(m, i, j, k);
    } else if (f < nzf + nyf) {
      int64_t g = f - nzf;
      int k = (int)(g % (nz - 1)), j = (int)((g / (nz - 1)) % ny), i = (int)(g / (nz - 1) / ny);
      ed[0] = EX(m, i, j, k); ed[1] = EZ(m, i + 1, j, k); ed[2] = EX(m, i, j, k + 1); ed[3] = EZ(m, i, j, k);
    } else {
      int64_t g = f - nzf - nyf;
      int k = (int)(g % (nz - 1)), j = (int)((g / (nz - 1)) % (ny - 1)), i = (int)(g / (nz - 1) / (ny - 1));
      ed[0] = EY(m, i, j, k); ed[1] = EZ(m, i, j + 1, k); ed[2] = EY(m, i, j, k + 1); ed[3] = EZ(m, i, j, k);
    }
    const int64_t *fv = m->fconn + 4 * f;
    for (int s = 0; s < 4; s++) {
      const int64_t *ev = m->econn + 2 * ed[s];
      int perm = -1;
      if (ev[0] == fv[CN_QL[s][0]] && ev[1] == fv[CN_QL[s][1]]) perm = 0;
      else if (ev[1] == fv[CN_QL[s][0]] && ev[0] == fv[CN_QL[s][1]]) perm = 1;
      if (perm < 0) return or_fail("Edges cannot be matched (face %lld side %d)", (long long)f, s);
      m->adjind[a] = (int32_t)(E0 + ed[s]);
      m->adjperm[a] = perm;
      a++;
    }
  }
  for (int i = 0; i < nx - 1; i++)
    for (int j = 0; j < ny - 1; j++)
      for (int k = 0; k < nz - 1; k++) {
        int64_t r = ((int64_t)i * (ny - 1) + j) * (nz - 1) + k;
        m->adjoff[R0 + r] = (int32_t)a;
        const int64_t fs[6] = {FY(m, i, j, k), FX(m, i + 1, j, k), FY(m, i, j + 1, k), FX(m, i, j, k), FZ(m, i, j, k), FZ(m, i, j, k + 1)};
        const int64_t *rv = m->hconn + 8 * r;
        for (int s = 0; s < 6; s++) {
          const int64_t *fv = m->fconn + 4 * fs[s];
          int perm = -1;
          for (int p = 0; p < 8; p++) {
            if (fv[hq_perm[p][0]] == rv[CN_HQ[s][0]] && fv[hq_perm[p][1]] == rv[CN_HQ[s][1]]) {
              if (fv[hq_perm[p][2]] != rv[CN_HQ[s][2]] || fv[hq_perm[p][3]] != rv[CN_HQ[s][3]]) return or_fail("Faces cannot be matched");
              perm = p;
              break;
            }
          }
          if (perm < 0) return or_fail("Face (Quad) cannot be matched to region (Hex)");
          m->adjind[a] = (int32_t)(F0 + fs[s]);
          m->adjperm[a] = perm;
          a++;
        }
      }
  m->adjoff[m->nents] = (int32_t)a;
  return 0;
}

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }
static int dir_of(ordr o, int d) { return d == 0 ? o.x : d == 1 ? o.y : o.z; }

/* Degree tags (dMeshCreateRuleTagIsotropic, mesh.c:978-1023) and the min-rule propagation
 * dJacobiPropagateDown_Tensor (src/jacobi/impls/tensor/tensor.c:199-247); tables as reference. */
static int propagate_degree(or_fs *m, int degree, const int *elem_degree)
{
  static const int quadperm[4] = {0, 1, 0, 1};
  static const int hexperm[6][2] = {{0, 2}, {1, 2}, {0, 2}, {1, 2}, {1, 0}, {0, 1}};
  static const int orient[8][2] = {{0, 1}, {1, 0}, {0, 1}, {1, 0}, {1, 0}, {0, 1}, {1, 0}, {0, 1}};
  const int64_t E0 = m->nv, F0 = m->nv + m->ne, R0 = F0 + m->nf;
  int maxdeg = degree;
  if (elem_degree) { maxdeg = 0; for (int64_t r = 0; r < m->nr; r++) maxdeg = imax(maxdeg, elem_degree[r]); }
  m->deg = malloc(sizeof(ordr) * m->nents);
  for (int64_t v = 0; v < m->nv; v++) m->deg[v] = (ordr){0, 0, 0};
  for (int64_t e = 0; e < m->ne; e++) m->deg[E0 + e] = (ordr){maxdeg, 0, 0};
  for (int64_t f = 0; f < m->nf; f++) m->deg[F0 + f] = (ordr){maxdeg, maxdeg, 0};
  for (int64_t r = 0; r < m->nr; r++) {
    int p = elem_degree ? elem_degree[r] : degree;
    m->deg[R0 + r] = (ordr){p, p, p};
  }
  for (int64_t r = 0; r < m->nr; r++) {
    const int64_t e = R0 + r;
    for (int i = 0; i < 6; i++) {
      int ai = m->adjoff[e] + i, aind = m->adjind[ai], match = m->adjperm[ai];
      ordr o = m->deg[aind];
      m->deg[aind] = (ordr){imin(o.x, dir_of(m->deg[e], hexperm[i][orient[match][0]])), imin(o.y, dir_of(m->deg[e], hexperm[i][orient[match][1]])), 0};
    }
  }
  for (int64_t f = 0; f < m->nf; f++) {
    const int64_t e = F0 + f;
    for (int i = 0; i < 4; i++) {
      int ai = m->adjoff[e] + i, aind = m->adjind[ai];
      m->deg[aind] = (ordr){imin(m->deg[aind].x, dir_of(m->deg[e], quadperm[i])), 0, 0};
    }
  }
  for (int64_t e = 0; e < m->ne; e++) {
    for (int i = 0; i < 2; i++) m->deg[m->adjind[m->adjoff[E0 + e] + i]] = (ordr){0, 0, 0};
  }
  return 0;
}

/* dJacobiGetNodeCount_Tensor (tensor.c:249-281) */
static int interior_nodes(const or_fs *m, int64_t ent)
{
  const int64_t E0 = m->nv, F0 = m->nv + m->ne, R0 = F0 + m->nf;
  ordr o = m->deg[ent];
  if (ent < E0) return 1;
  if (ent < F0) return imax(0, o.x - 1);
  if (ent < R0) return imax(0, o.x - 1) * imax(0, o.y - 1);
  return imax(0, o.x - 1) * imax(0, o.y - 1) * imax(0, o.z - 1);
}

static int dGeomPermQuadIndex(int perm, const int dim[2], const int ij[2], int *ind)
{
  const int M = dim[0] - 2, N = dim[1] - 2, i = ij[0], j = ij[1];
  switch (perm) { /* dGeomPermQuadIndex (tensor.c:328-345), table as reference */
  case 0: *ind = i * N + j; break;
  case 1: *ind = (M - 1 - i) + j * M; break;
  case 2: *ind = (M - 1 - i) * N + (N - 1 - j); break;
  case 3: *ind = i + (N - 1 - j) * M; break;
  case 4: *ind = i + j * M; break;
  case 5: *ind = (M - 1 - i) * N + j; break;
  case 6: *ind = (M - 1 - i) + (N - 1 - j) * M; break;
  case 7: *ind = i * N + (N - 1 - j); break;
  default: return or_fail("Invalid permutation");
  }
  return 0;
}

/* dJacobiAddConstraints_Tensor for a HEX (tensor.c:360-468): one row of E per expanded node of the
 * element; the edge/face extraction and traversal tables are the reference's (table as reference). */
/* ---- interpolation constraints for p-nonconforming entities (extension; the reference errors,
 * src/jacobi/impls/tensor/tensor.c:417). An edge of degree q carries the polynomial through its GLL nodes
 * (vertex, q-1 interior dofs in the edge direction, vertex); a face of degree q carries the tensor
 * polynomial through its (q+1)^2 GLL grid in its own frame (u along fv0->fv1, v along fv0->fv3) whose
 * corner values are the vertices, boundary values the edge polynomials and interior values its dofs. */
static void edge_poly(const or_fs *m, int32_t edge, double t, double scale, rowacc *a)
{
  const int q = m->deg[edge].x;
  const int64_t *ev = m->econn + 2 * (edge - m->nv);
  double L[16];
  gll_lagrange(m, q, t, L);
  for (int k = 0; k <= q; k++) {
    const int32_t col = k == 0 ? m->gcoff[ev[0]] : k == q ? m->gcoff[ev[1]] : m->gcoff[edge] + (k - 1);
    acc_add(a, col, scale * L[k]);
  }
}

static void face_poly(const or_fs *m, int32_t face, double u, double v, rowacc *a)
{
  const int qu = m->deg[face].x, qv = m->deg[face].y;
  const int64_t *fv = m->fconn + 4 * (face - m->nv - m->ne);
  double Lu[16], Lv[16];
  gll_lagrange(m, qu, u, Lu);
  gll_lagrange(m, qv, v, Lv);
  for (int r = 0; r <= qu; r++)
    for (int c = 0; c <= qv; c++) {
      const double w = Lu[r] * Lv[c];
      const int bu = r == 0 || r == qu, bv = c == 0 || c == qv;
      if (bu && bv) {
        const int corner = r == 0 ? (c == 0 ? 0 : 3) : (c == 0 ? 1 : 2);
        acc_add(a, m->gcoff[fv[corner]], w);
      } else if (!bu && !bv) {
        acc_add(a, m->gcoff[face] + (r - 1) * (qv - 1) + (c - 1), w);
      } else {
        int side;
        double tau;
        if (c == 0) side = 0, tau = m->gll[qu][r];
        else if (r == qu) side = 1, tau = m->gll[qv][c];
        else if (c == qv) side = 2, tau = -m->gll[qu][r];
        else side = 3, tau = -m->gll[qv][c];
        const int32_t slot = m->adjoff[face] + side;
        edge_poly(m, m->adjind[slot], m->adjperm[slot] == 0 ? tau : -tau, w, a);
      }
    }
}

/* element-face traversal coordinates (s,t) -> face frame (u,v) for the 8 orientations of
 * dGeomPermQuadIndex (tensor.c:328-345) */
static void face_frame(int perm, double s, double t, double *u, double *v)
{
  switch (perm) {
  case 0: *u = s, *v = t; break;
  case 1: *u = t, *v = -s; break;
  case 2: *u = -s, *v = -t; break;
  case 3: *u = -t, *v = s; break;
  case 4: *u = t, *v = s; break;
  case 5: *u = -s, *v = t; break;
  case 6: *u = -t, *v = -s; break;
  default: *u = s, *v = -t; break;
  }
}

static int push_row(or_fs *m, int rw, const rowacc *a)
{
  if (m->ncrow + 1 >= m->ccap) {
    m->ccap = m->ccap ? 2 * m->ccap : 1024;
    m->cptr = realloc(m->cptr, sizeof(int64_t) * (m->ccap + 1));
  }
  if (m->ncrow == 0) m->cptr[0] = 0;
  for (int i = 0; i < a->n; i++) {
    if (fabs(a->w[i]) < 1e-14) continue; /* exact zeros of the Lagrange weights (node coincidences) */
    if (m->nent == m->entcap) {
      m->entcap = m->entcap ? 2 * m->entcap : 4096;
      m->ccol = realloc(m->ccol, sizeof(int32_t) * m->entcap);
      m->cval = realloc(m->cval, sizeof(double) * m->entcap);
    }
    m->ccol[m->nent] = a->col[i];
    m->cval[m->nent] = a->w[i];
    m->nent++;
  }
  m->cptr[m->ncrow + 1] = m->nent;
  m->emap[rw] = (int32_t)(-2 - m->ncrow);
  m->ncrow++;
  return 0;
}

static int add_constraints_hex(or_fs *m, int64_t r, int xs)
{
  static const struct { int f, e, o; } fe[12][2] = {
      {{0, 0, 0}, {4, 3, 1}}, {{1, 0, 0}, {4, 2, 1}}, {{2, 0, 0}, {4, 1, 1}}, {{3, 0, 0}, {4, 0, 1}},
      {{0, 2, 1}, {5, 0, 0}}, {{1, 2, 1}, {5, 1, 0}}, {{2, 2, 1}, {5, 2, 0}}, {{3, 2, 1}, {5, 3, 0}},
      {{0, 3, 1}, {3, 1, 0}}, {{0, 1, 0}, {1, 3, 1}}, {{1, 1, 0}, {2, 3, 1}}, {{2, 1, 0}, {3, 3, 1}}};
  static const int iperm[8][4] = {{0, 1, 2, 3}, {3, 0, 1, 2}, {2, 3, 0, 1}, {1, 2, 3, 0}, {3, 2, 1, 0}, {0, 3, 2, 1}, {1, 0, 3, 2}, {2, 1, 0, 3}};
  static const struct { int e, v; } ev_common[8][3] = {
      {{0, 0}, {3, 1}, {8, 0}}, {{0, 1}, {1, 0}, {9, 0}}, {{1, 1}, {2, 0}, {10, 0}}, {{2, 1}, {3, 0}, {11, 0}},
      {{4, 0}, {7, 1}, {8, 1}}, {{4, 1}, {5, 0}, {9, 1}}, {{5, 1}, {6, 0}, {10, 1}}, {{6, 1}, {7, 0}, {11, 1}}};
  static const int edge_flip[2][2] = {{0, 1}, {1, 0}};
  const int64_t ei = m->nv + m->ne + m->nf + r;
  const int32_t *aI = m->adjind, *aO = m->adjoff, *aP = m->adjperm, *is = m->gcoff;
  const int d0 = m->deg[ei].x + 1, d1 = m->deg[ei].y + 1, d2 = m->deg[ei].z + 1, d[3] = {d0, d1, d2};
  const int scan[3] = {d1 * d2, d2, 1};
  const int32_t *f = aI + aO[ei], *fP = aP + aO[ei];
  int e[12], eP[12], v[8];
  for (int i = 0; i < 12; i++) {
    int ef0 = fe[i][0].f, ef1 = fe[i][1].f;
    e[i] = aI[aO[f[ef0]] + iperm[fP[ef0]][fe[i][0].e]];
    if (e[i] != aI[aO[f[ef1]] + iperm[fP[ef1]][fe[i][1].e]]) return or_fail("faces don't agree about edge");
    eP[i] = aP[aO[f[ef0]] + iperm[fP[ef0]][fe[i][0].e]] ^ (((fP[ef0] >> 2) & 1) ^ fe[i][0].o);
    if (eP[i] != (aP[aO[f[ef1]] + iperm[fP[ef1]][fe[i][1].e]] ^ (((fP[ef1] >> 2) & 1) ^ fe[i][1].o))) return or_fail("orientations do not agree");
  }
  for (int i = 0; i < 8; i++) {
    int vv[3];
    for (int j = 0; j < 3; j++) {
      int E = ev_common[i][j].e;
      vv[j] = aI[aO[e[E]] + edge_flip[eP[E]][ev_common[i][j].v]];
    }
    if (vv[0] != vv[1] || vv[0] != vv[2]) return or_fail("edges don't agree about vertex");
    v[i] = vv[0];
  }
  int32_t *row = m->emap;
  {
    const int T[8][3] = {{0, 0, 0}, {d0 - 1, 0, 0}, {d0 - 1, d1 - 1, 0}, {0, d1 - 1, 0}, {0, 0, d2 - 1}, {d0 - 1, 0, d2 - 1}, {d0 - 1, d1 - 1, d2 - 1}, {0, d1 - 1, d2 - 1}};
    for (int i = 0; i < 8; i++) row[xs + (T[i][0] * d1 + T[i][1]) * d2 + T[i][2]] = is[v[i]];
  }
  {
    const struct { int start[3], incd, inci, end; } E[12] = {
        {{1, 0, 0}, 0, 1, d0 - 1}, {{d0 - 1, 1, 0}, 1, 1, d1 - 1}, {{d0 - 2, d1 - 1, 0}, 0, -1, 0}, {{0, d1 - 2, 0}, 1, -1, 0},
        {{1, 0, d2 - 1}, 0, 1, d0 - 1}, {{d0 - 1, 1, d2 - 1}, 1, 1, d1 - 1}, {{d0 - 2, d1 - 1, d2 - 1}, 0, -1, 0}, {{0, d1 - 2, d2 - 1}, 1, -1, 0},
        {{0, 0, 1}, 2, 1, d2 - 1}, {{d0 - 1, 0, 1}, 2, 1, d2 - 1}, {{d0 - 1, d1 - 1, 1}, 2, 1, d2 - 1}, {{0, d1 - 1, 1}, 2, 1, d2 - 1}};
    for (int i = 0; i < 12; i++) {
      const int *st = E[i].start, incd = E[i].incd, inci = E[i].inci, end = E[i].end;
      if (m->deg[e[i]].x != d[incd] - 1) {
        if (!m->hp) return or_fail("degree does not agree, p-nonconforming");
        /* extension: element edge nodes interpolate the lower-degree edge polynomial */
        for (int j = st[incd]; j != end; j += inci) {
          const int rw = xs + (st[0] * d1 + st[1]) * d2 + st[2] + (j - st[incd]) * scan[incd];
          const double tau = inci * m->gll[d[incd] - 1][j];
          rowacc *a = calloc(1, sizeof(rowacc));
          edge_poly(m, e[i], eP[i] == 0 ? tau : -tau, 1.0, a);
          if (push_row(m, rw, a)) { free(a); return -1; }
          free(a);
        }
        continue;
      }
      for (int j = st[incd]; j != end; j += inci) {
        int rw = xs + (st[0] * d1 + st[1]) * d2 + st[2] + (j - st[incd]) * scan[incd], col;
        if (eP[i] == 0) col = is[e[i]] + (j - st[incd]) / inci;
        else if (eP[i] == 1) col = is[e[i]] - (j - (end - inci)) / inci;
        else return or_fail("bad edge orientation");
        row[rw] = col;
      }
    }
  }
  {
    const struct { int start[3], incd[2], inc[2], end[2]; } F[6] = {
        {{1, 0, 1}, {0, 2}, {1, 1}, {d0 - 1, d2 - 1}}, {{d0 - 1, 1, 1}, {1, 2}, {1, 1}, {d1 - 1, d2 - 1}},
        {{d0 - 2, d1 - 1, 1}, {0, 2}, {-1, 1}, {0, d2 - 1}}, {{0, d1 - 2, 1}, {1, 2}, {-1, 1}, {0, d2 - 1}},
        {{1, 1, 0}, {1, 0}, {1, 1}, {d1 - 1, d0 - 1}}, {{1, 1, d2 - 1}, {0, 1}, {1, 1}, {d0 - 1, d1 - 1}}};
    for (int i = 0; i < 6; i++) {
      const int *st = F[i].start, *incd = F[i].incd, *inc = F[i].inc, *end = F[i].end;
      if (m->deg[f[i]].x != d[incd[0]] - 1 || m->deg[f[i]].y != d[incd[1]] - 1) {
        if (!m->hp) return or_fail("degree does not agree, p-nonconforming");
        /* extension: element face nodes interpolate the lower-degree face polynomial in the face's frame */
        for (int j = st[incd[0]]; j != end[0]; j += inc[0])
          for (int k = st[incd[1]]; k != end[1]; k += inc[1]) {
            const int rw = xs + (st[0] * d1 + st[1]) * d2 + st[2] + (j - st[incd[0]]) * scan[incd[0]] + (k - st[incd[1]]) * scan[incd[1]];
            const double s = inc[0] * m->gll[d[incd[0]] - 1][j], t = inc[1] * m->gll[d[incd[1]] - 1][k];
            double u, w;
            face_frame(fP[i], s, t, &u, &w);
            rowacc *a = calloc(1, sizeof(rowacc));
            face_poly(m, f[i], u, w, a);
            if (push_row(m, rw, a)) { free(a); return -1; }
            free(a);
          }
        continue;
      }
      for (int j = st[incd[0]]; j != end[0]; j += inc[0])
        for (int k = st[incd[1]]; k != end[1]; k += inc[1]) {
          const int dim[2] = {d[incd[0]], d[incd[1]]};
          int jk[2] = {(j - st[incd[0]]) / inc[0], (k - st[incd[1]]) / inc[1]}, fi = -1;
          if (dGeomPermQuadIndex(fP[i], dim, jk, &fi)) return -1;
          row[xs + (st[0] * d1 + st[1]) * d2 + st[2] + (j - st[incd[0]]) * scan[incd[0]] + (k - st[incd[1]]) * scan[incd[1]]] = is[f[i]] + fi;
        }
    }
  }
  for (int j = 1; j < d0 - 1; j++)
    for (int k = 1; k < d1 - 1; k++)
      for (int l = 1; l < d2 - 1; l++) row[xs + (j * d1 + k) * d2 + l] = is[ei] + ((j - 1) * (d1 - 2) + (k - 1)) * (d2 - 2) + (l - 1);
  return 0;
}

/* dFSBuildSpace_Cont (src/fs/impls/cont/cont.c:258-385) with natural ordering: explicit entities in
 * handle order, then Dirichlet entities (dMeshPopulateOrderedSet_Private cont.c:93-178, partition
 * fsbuild.c:55-95, offsets fsbuild.c:107-146, element offsets cont.c:371-376). */
/* expanded coordinates, tensor vertex order (dFSCreateGeometryFromMesh_Private fsgeom.c:146-156) */
static void expanded_coords(or_fs *m)
{
  static const int connidx[8] = {0, 4, 3, 7, 1, 5, 2, 6};
  for (int64_t r = 0; r < m->nr; r++)
    for (int i = 0; i < 8; i++)
      for (int d = 0; d < 3; d++) m->xexp[(r * 8 + i) * 3 + d] = m->vx[3 * m->hconn[8 * r + connidx[i]] + d];
}

static or_fs *fs_build(or_fs *m, int degree, const int *elem_degree, int dirichlet_mask);

or_fs *or_fs_create(int nx, int ny, int nz, const double box[6], double perturb, uint64_t seed,
                    int degree, const int *elem_degree, int bs, int dirichlet_mask)
{
  if (nx < 2 || ny < 2 || nz < 2) { or_fail("need at least 2 vertices per direction"); return NULL; }
  or_fs *m = calloc(1, sizeof(or_fs));
  m->nx = nx; m->ny = ny; m->nz = nz; m->bs = bs;
  m->hp = elem_degree != NULL;
  for (int p = 1; p < 16; p++) { double w[16]; or_lobatto(p + 1, m->gll[p], w); }
  if (build_mesh(m, box, perturb, seed) || build_adjacency(m)) { or_fs_destroy(m); return NULL; }
  return fs_build(m, degree, elem_degree, dirichlet_mask);
}

/* The space on a mesh with its adjacency (dFSBuildSpace: cont.c:93-385, fsbuild.c:55-146): degree propagation,
 * explicit / Dirichlet partition with natural ordering, E, expanded coordinates. Frees m on error. */
static or_fs *fs_build(or_fs *m, int degree, const int *elem_degree, int dirichlet_mask)
{
  if (propagate_degree(m, degree, elem_degree)) { or_fs_destroy(m); return NULL; }
  /* boundary face sets 0..3 -> 100 (walls), 5 -> 200 (top), 4 -> 300 (bottom) (genblock.c:409-421) */
  const int set_of_face[6] = {0, 0, 0, 0, 2, 1};
  m->ordered = malloc(sizeof(int32_t) * m->nents);
  m->goff = malloc(sizeof(int32_t) * m->nents);
  m->gcoff = malloc(sizeof(int32_t) * m->nents);
  m->inodes = malloc(sizeof(int32_t) * m->nents);
  unsigned char *dir = calloc(m->nents, 1);
  for (int64_t i = 0; i < m->nents; i++) {
    int fsid = m->fset[i];
    if (fsid >= 0 && (dirichlet_mask >> set_of_face[fsid] & 1)) dir[i] = 1;
    m->inodes[i] = interior_nodes(m, i);
  }
  int64_t c = 0;
  for (int64_t i = 0; i < m->nents; i++) if (!dir[i]) m->ordered[c++] = (int32_t)i;
  const int64_t nexplicit = c;
  for (int64_t i = 0; i < m->nents; i++) if (dir[i]) m->ordered[c++] = (int32_t)i;
  int64_t scan = 0;
  for (int64_t i = 0; i < m->nents; i++) m->goff[i] = -1;
  for (int64_t i = 0; i < nexplicit; i++) { m->goff[m->ordered[i]] = (int32_t)scan; scan += m->inodes[m->ordered[i]]; }
  m->n = scan;
  scan = 0;
  for (int64_t i = 0; i < m->nents; i++) { m->gcoff[m->ordered[i]] = (int32_t)scan; scan += m->inodes[m->ordered[i]]; }
  m->nc = scan;
  free(dir);
  /* elements (regions in creation order) */
  const int64_t R0 = m->nv + m->ne + m->nf;
  m->xstart = malloc(sizeof(int32_t) * (m->nr + 1));
  m->edeg = malloc(sizeof(int32_t) * 3 * m->nr);
  m->xstart[0] = 0;
  for (int64_t r = 0; r < m->nr; r++) {
    ordr o = m->deg[R0 + r];
    m->edeg[3 * r] = o.x; m->edeg[3 * r + 1] = o.y; m->edeg[3 * r + 2] = o.z;
    m->xstart[r + 1] = m->xstart[r] + (o.x + 1) * (o.y + 1) * (o.z + 1);
  }
  m->nexp = m->xstart[m->nr];
  m->emap = malloc(sizeof(int32_t) * m->nexp);
  for (int64_t i = 0; i < m->nexp; i++) m->emap[i] = -1;
  for (int64_t r = 0; r < m->nr; r++)
    if (add_constraints_hex(m, r, m->xstart[r])) { or_fs_destroy(m); return NULL; }
  for (int64_t i = 0; i < m->nexp; i++)
    if (m->emap[i] == -1) { or_fail("expanded node %lld has no constraint", (long long)i); or_fs_destroy(m); return NULL; }
  /* E as CSR: Boolean rows (1.0 at emap) and interpolation rows (columns ascending) */
  m->eptr = malloc(sizeof(int64_t) * (m->nexp + 1));
  {
    int64_t cnt = 0;
    for (int64_t i = 0; i < m->nexp; i++) cnt += m->emap[i] >= 0 ? 1 : m->cptr[-2 - m->emap[i] + 1] - m->cptr[-2 - m->emap[i]];
    m->ecol = malloc(sizeof(int32_t) * (cnt ? cnt : 1));
    m->eval = malloc(sizeof(double) * (cnt ? cnt : 1));
    int64_t o = 0;
    for (int64_t i = 0; i < m->nexp; i++) {
      m->eptr[i] = o;
      if (m->emap[i] >= 0) { m->ecol[o] = m->emap[i]; m->eval[o] = 1.0; o++; continue; }
      const int64_t k = -2 - m->emap[i], b = m->cptr[k], e2 = m->cptr[k + 1];
      for (int64_t t = b; t < e2; t++) { /* insertion by column */
        int64_t pos = o;
        while (pos > m->eptr[i] && m->ecol[pos - 1] > m->ccol[t]) { m->ecol[pos] = m->ecol[pos - 1]; m->eval[pos] = m->eval[pos - 1]; pos--; }
        m->ecol[pos] = m->ccol[t];
        m->eval[pos] = m->cval[t];
        o++;
      }
    }
    m->eptr[m->nexp] = o;
  }
  m->xexp = malloc(sizeof(double) * 24 * m->nr);
  expanded_coords(m);
  return m;
}

/* dMeshMorph (src/fs/mesh/interface/mesh.c): new vertex coordinates [nv][3] (same topology), e.g. the morph and
 * twist of ellip.c:173-181; the expanded coordinates follow */
void or_fs_set_vertex_coords(or_fs *m, const double *vx)
{
  memcpy(m->vx, vx, sizeof(double) * 3 * m->nv);
  expanded_coords(m);
}

/* dMeshGetAdjacency (mesh.c:1074-1191) for a mesh given by its entities: each canonical side of a face (CN_QL) is the
 * edge with the same two vertices, each side of a hexahedron (CN_HQ) the face with the same four, and the orientation
 * is the rotation / reflection that carries one onto the other (a search over all entities: small meshes only). */
static int build_adjacency_search(or_fs *m)
{
  static const int hq_perm[8][4] = {{0, 1, 2, 3}, {3, 0, 1, 2}, {2, 3, 0, 1}, {1, 2, 3, 0}, {0, 3, 2, 1}, {1, 0, 3, 2}, {2, 1, 0, 3}, {3, 2, 1, 0}};
  const int64_t E0 = m->nv, F0 = m->nv + m->ne, R0 = m->nv + m->ne + m->nf;
  const int64_t nadj = 2 * m->ne + 4 * m->nf + 6 * m->nr;
  m->adjoff = malloc(sizeof(int32_t) * (m->nents + 1));
  m->adjind = malloc(sizeof(int32_t) * nadj);
  m->adjperm = malloc(sizeof(int32_t) * nadj);
  int64_t a = 0;
  for (int64_t v = 0; v < m->nv; v++) m->adjoff[v] = 0;
  for (int64_t e = 0; e < m->ne; e++) {
    m->adjoff[E0 + e] = (int32_t)a;
    for (int s = 0; s < 2; s++) { m->adjind[a] = (int32_t)m->econn[2 * e + s]; m->adjperm[a] = 0; a++; }
  }
  for (int64_t f = 0; f < m->nf; f++) {
    m->adjoff[F0 + f] = (int32_t)a;
    const int64_t *fv = m->fconn + 4 * f;
    for (int s = 0; s < 4; s++) {
      const int64_t v0 = fv[CN_QL[s][0]], v1 = fv[CN_QL[s][1]];
      int64_t found = -1;
      int perm = 0;
      for (int64_t e = 0; e < m->ne && found < 0; e++) {
        const int64_t *ev = m->econn + 2 * e;
        if (ev[0] == v0 && ev[1] == v1) found = e, perm = 0;
        else if (ev[0] == v1 && ev[1] == v0) found = e, perm = 1;
      }
      if (found < 0) return or_fail("Edges cannot be matched (face %lld side %d)", (long long)f, s);
      m->adjind[a] = (int32_t)(E0 + found);
      m->adjperm[a] = perm;
      a++;
    }
  }
  for (int64_t r = 0; r < m->nr; r++) {
    m->adjoff[R0 + r] = (int32_t)a;
    const int64_t *rv = m->hconn + 8 * r;
    for (int s = 0; s < 6; s++) {
      int64_t found = -1;
      int perm = -1;
      for (int64_t f = 0; f < m->nf && found < 0; f++) {
        const int64_t *fv = m->fconn + 4 * f;
        for (int p = 0; p < 8; p++) {
          int same = 1;
          for (int c = 0; c < 4; c++) same = same && fv[hq_perm[p][c]] == rv[CN_HQ[s][c]];
          if (same) { found = f; perm = p; break; }
        }
      }
      if (found < 0) return or_fail("Face (Quad) cannot be matched to region (Hex) %lld side %d", (long long)r, s);
      m->adjind[a] = (int32_t)(F0 + found);
      m->adjperm[a] = perm;
      a++;
    }
  }
  m->adjoff[m->nents] = (int32_t)a;
  return 0;
}

or_fs *or_fs_create_conn(int nv, const double *vtx, int ne, const int *econn, int nf, const int *fconn, int nr,
                         const int *hconn, int degree, const int *elem_degree, int bs)
{
  or_fs *m = calloc(1, sizeof(or_fs));
  m->bs = bs;
  m->hp = elem_degree != NULL;
  for (int p = 1; p < 16; p++) { double w[16]; or_lobatto(p + 1, m->gll[p], w); }
  m->nv = nv; m->ne = ne; m->nf = nf; m->nr = nr;
  m->nents = m->nv + m->ne + m->nf + m->nr;
  m->vx = malloc(sizeof(double) * 3 * nv);
  memcpy(m->vx, vtx, sizeof(double) * 3 * nv);
  m->econn = malloc(sizeof(int64_t) * 2 * ne);
  m->fconn = malloc(sizeof(int64_t) * 4 * nf);
  m->hconn = malloc(sizeof(int64_t) * 8 * nr);
  for (int64_t i = 0; i < 2 * (int64_t)ne; i++) m->econn[i] = econn[i];
  for (int64_t i = 0; i < 4 * (int64_t)nf; i++) m->fconn[i] = fconn[i];
  for (int64_t i = 0; i < 8 * (int64_t)nr; i++) m->hconn[i] = hconn[i];
  m->fset = malloc(m->nents);
  memset(m->fset, -1, m->nents); /* no boundary sets */
  if (build_adjacency_search(m)) { or_fs_destroy(m); return NULL; }
  return fs_build(m, degree, elem_degree, 0);
}

const int32_t *or_fs_adjacency(const or_fs *m, const int32_t **adjind, const int32_t **adjperm)
{
  if (adjind) *adjind = m->adjind;
  if (adjperm) *adjperm = m->adjperm;
  return m->adjoff;
}

void or_fs_destroy(or_fs *m)
{
  if (!m) return;
  free(m->vx); free(m->econn); free(m->fconn); free(m->hconn); free(m->fset);
  free(m->adjoff); free(m->adjind); free(m->adjperm); free(m->deg);
  free(m->ordered); free(m->goff); free(m->gcoff); free(m->inodes);
  free(m->xstart); free(m->emap); free(m->edeg); free(m->xexp);
  free(m->cptr); free(m->ccol); free(m->cval); free(m->eptr); free(m->ecol); free(m->eval);
  free(m->tptr); free(m->trow); free(m->tval);
  free(m);
}

void or_fs_sizes(const or_fs *m, int64_t out[8])
{
  out[0] = m->nr; out[1] = m->n; out[2] = m->nc; out[3] = m->nexp; out[4] = m->bs;
  out[5] = m->nv; out[6] = m->ne; out[7] = m->nf;
}
const int32_t *or_fs_emap(const or_fs *m) { return m->emap; }
int64_t or_fs_ecsr(const or_fs *m, const int64_t **eptr, const int32_t **ecol, const double **eval)
{
  *eptr = m->eptr; *ecol = m->ecol; *eval = m->eval;
  return m->eptr[m->nexp];
}
const int32_t *or_fs_xstart(const or_fs *m) { return m->xstart; }
const int32_t *or_fs_elem_degree(const or_fs *m) { return m->edeg; }
const double *or_fs_coords_expanded(const or_fs *m) { return m->xexp; }
const double *or_fs_vertex_coords(const or_fs *m) { return m->vx; }
void or_fs_entity_info(const or_fs *m, int32_t *ordered, int32_t *goffset, int32_t *gcoffset, int32_t *inodes)
{
  if (ordered) memcpy(ordered, m->ordered, sizeof(int32_t) * m->nents);
  if (goffset) memcpy(goffset, m->goff, sizeof(int32_t) * m->nents);
  if (gcoffset) memcpy(gcoffset, m->gcoff, sizeof(int32_t) * m->nents);
  if (inodes) memcpy(inodes, m->inodes, sizeof(int32_t) * m->nents);
}

/* dFSGlobalToExpanded (fs.c:543-586): closure = [g, dirichlet values or 0]; x = E closure (MAIJ(bs)) */
void or_fs_global_to_expanded(const or_fs *m, const double *g, const double *dcache, double *x)
{
  const int bs = m->bs;
  for (int64_t r = 0; r < m->nexp; r++)
    for (int b = 0; b < bs; b++) {
      double v = 0;
      for (int64_t k = m->eptr[r]; k < m->eptr[r + 1]; k++) {
        const int64_t c = m->ecol[k];
        const double cv = c < m->n ? g[c * bs + b] : (dcache ? dcache[(c - m->n) * bs + b] : 0.0);
        v = (k == m->eptr[r]) ? m->eval[k] * cv : v + m->eval[k] * cv;
      }
      x[r * bs + b] = v;
    }
}

/* dFSExpandedToGlobal (fs.c:592-640): closure = E^T x (MatMultTranspose sums rows in order) */
void or_fs_expanded_to_global(const or_fs *m, const double *x, double *g, int add)
{
  const int bs = m->bs;
  double *cl = calloc((size_t)m->nc * bs, sizeof(double));
  for (int64_t r = 0; r < m->nexp; r++)
    for (int64_t k = m->eptr[r]; k < m->eptr[r + 1]; k++)
      for (int b = 0; b < bs; b++) cl[(int64_t)m->ecol[k] * bs + b] += m->eval[k] * x[r * bs + b];
  for (int64_t i = 0; i < m->n * bs; i++) g[i] = add ? g[i] + cl[i] : cl[i];
  free(cl);
}

/* The same expand and restrict with host threads: the reference runs one MPI rank per core, each expanding
 * and restricting its own partition; here rows of E (expand) and rows of E^T (restrict, each closure node's
 * terms summed in ascending expanded order, the order of the serial loop above) are split over threads, so
 * the results are bit-identical to the serial forms. */
static void fs_make_et(or_fs *m)
{
  if (m->tptr) return;
  const int64_t nnz = m->eptr[m->nexp];
  int64_t *ptr = calloc((size_t)m->nc + 1, sizeof(int64_t)), *row = malloc(sizeof(int64_t) * (nnz ? nnz : 1));
  double *val = malloc(sizeof(double) * (nnz ? nnz : 1));
  for (int64_t k = 0; k < nnz; k++) ptr[m->ecol[k] + 1]++;
  for (int64_t c = 0; c < m->nc; c++) ptr[c + 1] += ptr[c];
  int64_t *fill = malloc(sizeof(int64_t) * ((size_t)m->nc + 1));
  memcpy(fill, ptr, sizeof(int64_t) * ((size_t)m->nc + 1));
  for (int64_t r = 0; r < m->nexp; r++)
    for (int64_t k = m->eptr[r]; k < m->eptr[r + 1]; k++) {
      const int64_t at = fill[m->ecol[k]]++;
      row[at] = r;
      val[at] = m->eval[k];
    }
  free(fill);
  m->tptr = ptr, m->trow = row, m->tval = val;
}

static void fs_expand_par(const or_fs *m, const double *g, const double *dcache, double *x, int nthreads)
{
  const int bs = m->bs;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int64_t r = 0; r < m->nexp; r++)
    for (int b = 0; b < bs; b++) {
      double v = 0;
      for (int64_t k = m->eptr[r]; k < m->eptr[r + 1]; k++) {
        const int64_t c = m->ecol[k];
        const double cv = c < m->n ? g[c * bs + b] : (dcache ? dcache[(c - m->n) * bs + b] : 0.0);
        v = (k == m->eptr[r]) ? m->eval[k] * cv : v + m->eval[k] * cv;
      }
      x[r * bs + b] = v;
    }
  (void)nthreads;
}

static void fs_restrict_par(const or_fs *m, const double *x, double *g, int nthreads)
{
  const int bs = m->bs;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int64_t c = 0; c < m->n; c++)
    for (int b = 0; b < bs; b++) {
      double v = 0;
      for (int64_t k = m->tptr[c]; k < m->tptr[c + 1]; k++) v += m->tval[k] * x[m->trow[k] * bs + b];
      g[c * bs + b] = v;
    }
  (void)nthreads;
}

/* ----------------------------------------------------------------------------------------------
 * Operator apply (the iterator loop of EllipShellMatMult / ElastShellMatMult)
 * -------------------------------------------------------------------------------------------- */
typedef struct {
  int P, Q;
  double x[32], w[32], interp[32 * 11], deriv[32 * 11], cinterp[64], cderiv[64];
} basis1d;

static int basis_for(int method, int p, basis1d *b)
{
  double node[16], weight[16];
  b->P = p + 1;
  b->Q = or_rule_1d(method, 0, 2 * p, b->x, b->w); /* ruleset order 2p (fsruleset.c:32-37), Gauss family */
  if (b->Q < 0) return -1;
  if (or_tensor_basis(b->P, b->Q, b->x, b->interp, b->deriv, node, weight)) return -1;
  if (or_tensor_basis(2, b->Q, b->x, b->cinterp, b->cderiv, node, weight)) return -1;
  return 0;
}

int64_t or_fs_num_qpts(const or_fs *m, int32_t *qoffset)
{
  int64_t nq = 0;
  if (qoffset) qoffset[0] = 0;
  for (int64_t r = 0; r < m->nr; r++) {
    nq += (int64_t)(m->edeg[3 * r] + 1) * (m->edeg[3 * r + 1] + 1) * (m->edeg[3 * r + 2] + 1);
    if (qoffset) qoffset[r + 1] = (int32_t)nq;
  }
  return nq;
}

/* per-element geometry at FAST points: coordinate GRAD (no mapping) then dRuleComputePhysical */
static int element_geometry(const or_fs *m, int64_t r, const basis1d *b[3], double *xq, double *jinv, double *jw)
{
  const int P2[3] = {2, 2, 2}, Q[3] = {b[0]->Q, b[1]->Q, b[2]->Q}, nq = Q[0] * Q[1] * Q[2];
  const double *ci[3] = {b[0]->cinterp, b[1]->cinterp, b[2]->cinterp}, *cd[3] = {b[0]->cderiv, b[1]->cderiv, b[2]->cderiv};
  double *jac = malloc(sizeof(double) * 9 * nq), *w = malloc(sizeof(double) * nq);
  const double *xe = m->xexp + r * 24;
  if (xq) or_efs_apply_hex(P2, Q, ci, cd, NULL, 3, xe, xq, OR_INTERP, OR_INSERT);
  or_efs_apply_hex(P2, Q, ci, cd, NULL, 3, xe, jac, OR_GRAD, OR_INSERT);
  for (int i = 0; i < Q[0]; i++)
    for (int j = 0; j < Q[1]; j++)
      for (int k = 0; k < Q[2]; k++) w[(i * Q[1] + j) * Q[2] + k] = b[0]->w[i] * b[1]->w[j] * b[2]->w[k];
  int rc = compute_physical(nq, w, jac, jinv, jw);
  free(jac);
  free(w);
  return rc;
}

void or_fs_qpt_coords(const or_fs *m, double *xq)
{
  basis1d B[11];
  for (int p = 1; p <= 10; p++) basis_for(0, p, &B[p]);
  int64_t off = 0;
  for (int64_t r = 0; r < m->nr; r++) {
    const basis1d *b[3] = {&B[m->edeg[3 * r]], &B[m->edeg[3 * r + 1]], &B[m->edeg[3 * r + 2]]};
    const int P2[3] = {2, 2, 2}, Q[3] = {b[0]->Q, b[1]->Q, b[2]->Q};
    const double *ci[3] = {b[0]->cinterp, b[1]->cinterp, b[2]->cinterp}, *cd[3] = {b[0]->cderiv, b[1]->cderiv, b[2]->cderiv};
    or_efs_apply_hex(P2, Q, ci, cd, NULL, 3, m->xexp + r * 24, xq + off * 3, OR_INTERP, OR_INSERT);
    off += Q[0] * Q[1] * Q[2];
  }
}

/* the field of g (closure tail dcache: inhomogeneous Dirichlet values, NULL = 0) at the FAST points in
 * or_fs_qpt_coords order, as dRulesetIteratorGetPatchApplied yields it (fsrulesetit.c:517-589): u [nq][bs],
 * du [nq][bs][3] (physical gradient), jw [nq]; any output may be NULL. rule_deg > 0 takes the FAST rule of that
 * degree instead of the space's own (a second space on the first one's ruleset, as in a multi-field iterator). */
int or_fs_eval_points(const or_fs *m, int rule_deg, const double *g, const double *dcache, double *u, double *du, double *jw)
{
  const int bs = m->bs;
  double *xe = malloc(sizeof(double) * (size_t)m->nexp * bs);
  double *jinv = malloc(sizeof(double) * 9 * 1000), *w = malloc(sizeof(double) * 1000);
  double *tu = malloc(sizeof(double) * 1000 * bs), *tdu = malloc(sizeof(double) * 3000 * bs);
  or_fs_global_to_expanded(m, g, dcache, xe);
  int rc = 0;
  int64_t off = 0;
  for (int64_t r = 0; r < m->nr && !rc; r++) {
    basis1d B[3];
    double fi[3][16 * 16], fd[3][16 * 16], node[16], weight[16];
    const double *bi[3], *bd[3];
    int P[3], Q[3];
    for (int a = 0; a < 3 && !rc; a++) {
      if (basis_for(0, rule_deg > 0 ? rule_deg : m->edeg[3 * r + a], &B[a])) { rc = -1; break; }
      P[a] = m->edeg[3 * r + a] + 1, Q[a] = B[a].Q;
      if (rule_deg > 0) { /* the space's basis at the rule's points */
        if (or_tensor_basis(P[a], Q[a], B[a].x, fi[a], fd[a], node, weight)) { rc = -1; break; }
        bi[a] = fi[a], bd[a] = fd[a];
      } else {
        bi[a] = B[a].interp, bd[a] = B[a].deriv;
      }
    }
    if (rc) break;
    const basis1d *b[3] = {&B[0], &B[1], &B[2]};
    const int nq = Q[0] * Q[1] * Q[2];
    if ((rc = element_geometry(m, r, b, NULL, jinv, w))) break;
    const double *xr = xe + (int64_t)m->xstart[r] * bs;
    or_efs_apply_hex(P, Q, bi, bd, NULL, bs, xr, tu, OR_INTERP, OR_INSERT);
    or_efs_apply_hex(P, Q, bi, bd, jinv, bs, xr, tdu, OR_GRAD, OR_INSERT);
    if (u) memcpy(u + off * bs, tu, sizeof(double) * nq * bs);
    if (du) memcpy(du + off * bs * 3, tdu, sizeof(double) * nq * bs * 3);
    if (jw) memcpy(jw + off, w, sizeof(double) * nq);
    off += nq;
  }
  free(xe); free(jinv); free(w); free(tu); free(tdu);
  return rc ? or_fail("negative Jacobian or unsupported degree") : 0;
}

/* Pointwise q-functions: EllipPointwiseJacobian (ellip.c:369-377; p=2 gives eta=1, s=0) and
 * ElastPointwiseJacobian at F=I (elast.c:269-280: dS = lambda tr(dE) I + 2 mu dE, Dv = F dS + dF S). */
/* St. Venant-Kirchhoff pieces (elast.c:224-254): column dot, S = lambda tr(E) I + 2 mu E with the Green-Lagrange
 * strain E = (F^T F - I)/2 in compressed symmetric storage [00, 11, 22, 01, 02, 12], and C = A S */
static double dotcol(const double a[9], const double b[9], int i, int j)
{
  return a[0 * 3 + i] * b[0 * 3 + j] + a[1 * 3 + i] * b[1 * 3 + j] + a[2 * 3 + i] * b[2 * 3 + j];
}
static void svk_pk2(double lam, double mu, const double F[9], double S[6])
{
  double E[6], tr;
  E[0] = 0.5 * (dotcol(F, F, 0, 0) - 1);
  E[1] = 0.5 * (dotcol(F, F, 1, 1) - 1);
  E[2] = 0.5 * (dotcol(F, F, 2, 2) - 1);
  E[3] = 0.5 * dotcol(F, F, 0, 1);
  E[4] = 0.5 * dotcol(F, F, 0, 2);
  E[5] = 0.5 * dotcol(F, F, 1, 2);
  tr = E[0] + E[1] + E[2];
  for (int i = 0; i < 6; i++) S[i] = lam * tr * (i < 3) + 2 * mu * E[i];
}
static void svk_pk2_jac(double lam, double mu, const double F[9], const double dF[9], double dS[6])
{
  double dE[6], tr;
  dE[0] = 0.5 * (dotcol(F, dF, 0, 0) + dotcol(dF, F, 0, 0));
  dE[1] = 0.5 * (dotcol(F, dF, 1, 1) + dotcol(dF, F, 1, 1));
  dE[2] = 0.5 * (dotcol(F, dF, 2, 2) + dotcol(dF, F, 2, 2));
  dE[3] = 0.5 * (dotcol(F, dF, 0, 1) + dotcol(dF, F, 0, 1));
  dE[4] = 0.5 * (dotcol(F, dF, 0, 2) + dotcol(dF, F, 0, 2));
  dE[5] = 0.5 * (dotcol(F, dF, 1, 2) + dotcol(dF, F, 1, 2));
  tr = dE[0] + dE[1] + dE[2];
  for (int i = 0; i < 6; i++) dS[i] = lam * tr * (i < 3) + 2 * mu * dE[i];
}
static void mult_gesy3(double C[9], const double A[9], const double S[6], int add)
{
  for (int i = 0; i < 3; i++) {
    const double c0 = A[i * 3 + 0] * S[0] + A[i * 3 + 1] * S[3] + A[i * 3 + 2] * S[4];
    const double c1 = A[i * 3 + 0] * S[3] + A[i * 3 + 1] * S[1] + A[i * 3 + 2] * S[5];
    const double c2 = A[i * 3 + 0] * S[4] + A[i * 3 + 1] * S[5] + A[i * 3 + 2] * S[2];
    if (add) { C[i * 3 + 0] += c0; C[i * 3 + 1] += c1; C[i * 3 + 2] += c2; }
    else { C[i * 3 + 0] = c0; C[i * 3 + 1] = c1; C[i * 3 + 2] = c2; }
  }
}

static void qfunction(int kind, int D, const double *qd, const double *param, double w, const double *u, const double *du, double *v, double *dv)
{
  if (kind == 0) {
    const double k = qd ? qd[0] : 1.0;
    const double etaw = k * w;
    v[0] = -w * 0.0 * u[0];
    for (int i = 0; i < 3; i++) dv[i] = etaw * du[i];
  } else if (kind == 4) { /* ElastPointwiseFunction without body force (elast.c:256-266): Dv = w F S, F = I + Du */
    double F[9], S[6];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) F[i * 3 + j] = (i == j) + du[i * 3 + j];
    svk_pk2(param[0], param[1], F, S);
    mult_gesy3(dv, F, S, 0);
    for (int i = 0; i < 9; i++) dv[i] *= w;
    v[0] = v[1] = v[2] = 0;
  } else if (kind == 5) { /* ElastPointwiseJacobian at the stashed F (elast.c:268-280): Dv = w (F dS + dF S) */
    double S[6], dS[6];
    svk_pk2(param[0], param[1], qd, S);
    svk_pk2_jac(param[0], param[1], qd, du, dS);
    mult_gesy3(dv, qd, dS, 0);
    mult_gesy3(dv, du, S, 1);
    for (int i = 0; i < 9; i++) dv[i] *= w;
    v[0] = v[1] = v[2] = 0;
  } else if (kind == 6) { /* EllipPointwiseFunction (ellip.c:355-367) without forcing, lambda = 0: Dv = w eta Du */
    const double pe = param[0], eps = param[1];
    const double gamma = 0.5 * (du[0] * du[0] + du[1] * du[1] + du[2] * du[2]);
    const double etaw = pow(eps * eps + gamma, (pe - 2) / 2) * w;
    v[0] = 0;
    for (int i = 0; i < 3; i++) dv[i] = etaw * du[i];
  } else if (kind == 7) { /* EllipPointwiseFunction (ellip.c:355-367) with the Bratu term, param = {p, eps, lambda}:
                           v = -w lambda e^u, Dv = w eta Du (forcing added by the caller) */
    const double pe = param[0], eps = param[1], lam = param[2];
    const double gamma = 0.5 * (du[0] * du[0] + du[1] * du[1] + du[2] * du[2]);
    const double etaw = pow(eps * eps + gamma, (pe - 2) / 2) * w;
    v[0] = lam != 0 ? -w * lam * exp(u[0]) : 0; /* lambda_exp_u of EllipPointwiseComputeStore (ellip.c:341) */
    for (int i = 0; i < 3; i++) dv[i] = etaw * du[i];
  } else if (kind == 8) { /* EllipPointwiseJacobian (ellip.c:370-377) with the store [eta, sqrt(-eta') Du, lambda e^u]:
                           v = -w lambda e^u u, Dv = w (eta Du - (s . Du) s) */
    const double eta = qd[0], *s = qd + 1;
    const double dotw = (s[0] * du[0] + s[1] * du[1] + s[2] * du[2]) * w, etaw = eta * w;
    v[0] = -w * qd[4] * u[0];
    for (int i = 0; i < 3; i++) dv[i] = etaw * du[i] - dotw * s[i];
  } else if (kind == 3) { /* mass: the right-hand side b = int v f_h of src/fs/tests/ex1.c:399-430 */
    v[0] = w * u[0];
    dv[0] = dv[1] = dv[2] = 0;
  } else if (kind == 1) {
    const double eta = qd[0], *s = qd + 1;
    const double dotw = (s[0] * du[0] + s[1] * du[1] + s[2] * du[2]) * w, etaw = eta * w;
    v[0] = -w * 0.0 * u[0];
    for (int i = 0; i < 3; i++) dv[i] = etaw * du[i] - dotw * s[i];
  } else {
    const double lam = param[0], mu = param[1];
    double dE[6], dS[6], tr;
    (void)D;
    dE[0] = du[0]; dE[1] = du[4]; dE[2] = du[8];
    dE[3] = 0.5 * (du[1] + du[3]); dE[4] = 0.5 * (du[2] + du[6]); dE[5] = 0.5 * (du[5] + du[7]);
    tr = dE[0] + dE[1] + dE[2];
    for (int i = 0; i < 6; i++) dS[i] = lam * tr * (i < 3) + 2 * mu * dE[i];
    v[0] = v[1] = v[2] = 0;
    dv[0] = dS[0]; dv[1] = dS[3]; dv[2] = dS[4];
    dv[3] = dS[3]; dv[4] = dS[1]; dv[5] = dS[5];
    dv[6] = dS[4]; dv[7] = dS[5]; dv[8] = dS[2];
    for (int i = 0; i < 9; i++) dv[i] *= w;
  }
}

static int operator_eval(const or_fs *m, int kind, const double *qdata, const double *param, const double *g,
                         const double *dcache, const double *fq, double *y, int nthreads)
{
  const int bs = m->bs, D = bs;
  const int elastic = kind == 2 || kind == 4 || kind == 5;
  if (elastic != (bs == 3)) return or_fail("kind %d needs block size %d", kind, elastic ? 3 : 1);
  basis1d B[11];
  for (int p = 1; p <= 10; p++) if (basis_for(0, p, &B[p])) return -1;
  double *xexp = malloc(sizeof(double) * m->nexp * bs), *yexp = malloc(sizeof(double) * m->nexp * bs);
  int32_t *qoff = malloc(sizeof(int32_t) * (m->nr + 1));
  or_fs_num_qpts(m, qoff);
  if (nthreads < 1) nthreads = 1;
  fs_make_et((or_fs *)m);
  fs_expand_par(m, g, dcache, xexp, nthreads);
  int err = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    int maxq = 1000;
    double *xq = malloc(sizeof(double) * 3 * maxq), *jinv = malloc(sizeof(double) * 9 * maxq), *jw = malloc(sizeof(double) * maxq);
    double *u = malloc(sizeof(double) * D * maxq), *du = malloc(sizeof(double) * 3 * D * maxq);
    double *v = malloc(sizeof(double) * D * maxq), *dv = malloc(sizeof(double) * 3 * D * maxq);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int64_t r = 0; r < m->nr; r++) {
      const basis1d *b[3] = {&B[m->edeg[3 * r]], &B[m->edeg[3 * r + 1]], &B[m->edeg[3 * r + 2]]};
      const int P[3] = {b[0]->P, b[1]->P, b[2]->P}, Q[3] = {b[0]->Q, b[1]->Q, b[2]->Q}, nq = Q[0] * Q[1] * Q[2];
      const double *bi[3] = {b[0]->interp, b[1]->interp, b[2]->interp}, *bd[3] = {b[0]->deriv, b[1]->deriv, b[2]->deriv};
      if (element_geometry(m, r, b, xq, jinv, jw)) { err = 1; continue; }
      const double *xe = xexp + (int64_t)m->xstart[r] * bs;
      double *ye = yexp + (int64_t)m->xstart[r] * bs;
      or_efs_apply_hex(P, Q, bi, bd, jinv, D, xe, u, OR_INTERP, OR_INSERT);
      or_efs_apply_hex(P, Q, bi, bd, jinv, D, xe, du, OR_GRAD, OR_INSERT);
      for (int q = 0; q < nq; q++) {
        const double *qd = NULL;
        if (kind == 0 && qdata) qd = qdata + qoff[r] + q;
        if (kind == 1) qd = qdata + 4 * (int64_t)(qoff[r] + q);
        if (kind == 5) qd = qdata + 9 * (int64_t)(qoff[r] + q);
        if (kind == 8) qd = qdata + 5 * (int64_t)(qoff[r] + q);
        qfunction(kind, D, qd, param, jw[q], u + q * D, du + q * 3 * D, v + q * D, dv + q * 3 * D);
        if (fq) /* body force: the coefficient of v is -w f (ellip.c:362, elast.c:261) */
          for (int c = 0; c < D; c++) v[q * D + c] += -jw[q] * fq[(int64_t)(qoff[r] + q) * D + c];
      }
      or_efs_apply_hex(P, Q, bi, bd, jinv, D, v, ye, OR_INTERP_TRANSPOSE, OR_INSERT);
      or_efs_apply_hex(P, Q, bi, bd, jinv, D, dv, ye, OR_GRAD_TRANSPOSE, OR_ADD);
    }
    free(xq); free(jinv); free(jw); free(u); free(du); free(v); free(dv);
  }
  if (!err) fs_restrict_par(m, yexp, y, nthreads);
  free(xexp); free(yexp); free(qoff);
  return err ? or_fail("negative Jacobian") : 0;
}

int or_operator_apply(const or_fs *m, int kind, const double *qdata, const double *param,
                      const double *g, double *y, int nthreads)
{
  return operator_eval(m, kind, qdata, param, g, NULL, NULL, y, nthreads);
}

int or_operator_function(const or_fs *m, int kind, const double *param, const double *g, const double *dcache,
                         const double *fq, double *y, int nthreads)
{
  if (kind != 4 && kind != 6 && kind != 7)
    return or_fail("or_operator_function: kind 4 (St. Venant-Kirchhoff), 6 or 7 (p-Laplacian, 7 with the Bratu term)");
  return operator_eval(m, kind, NULL, param, g, dcache, fq, y, nthreads);
}

/* EllipPointwiseComputeStore (ellip.c:333-342) at the FAST points from the state g. */
/* EllipPointwiseComputeStore (ellip.c:333-342) at every FAST point; elements split over nthreads host threads
 * (each point's store depends only on its own element: the result does not depend on the thread count) */
int or_plap_stash_mt(const or_fs *m, double p, double eps, const double *g, double *stash, int nthreads)
{
  if (m->bs != 1) return or_fail("p-Laplacian is scalar");
  basis1d B[11];
  for (int k = 1; k <= 10; k++) if (basis_for(0, k, &B[k])) return -1;
  if (nthreads < 1) nthreads = 1;
  double *xexp = malloc(sizeof(double) * m->nexp);
  int32_t *qoff = malloc(sizeof(int32_t) * (m->nr + 1));
  or_fs_num_qpts(m, qoff);
  fs_expand_par(m, g, NULL, xexp, nthreads);
  int err = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    double *jinv = malloc(sizeof(double) * 9 * 1000), *jw = malloc(sizeof(double) * 1000), *du = malloc(sizeof(double) * 3000);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int64_t r = 0; r < m->nr; r++) {
      const basis1d *b[3] = {&B[m->edeg[3 * r]], &B[m->edeg[3 * r + 1]], &B[m->edeg[3 * r + 2]]};
      const int P[3] = {b[0]->P, b[1]->P, b[2]->P}, Q[3] = {b[0]->Q, b[1]->Q, b[2]->Q}, nq = Q[0] * Q[1] * Q[2];
      const double *bi[3] = {b[0]->interp, b[1]->interp, b[2]->interp}, *bd[3] = {b[0]->deriv, b[1]->deriv, b[2]->deriv};
      if (element_geometry(m, r, b, NULL, jinv, jw)) { err = 1; continue; }
      or_efs_apply_hex(P, Q, bi, bd, jinv, 1, xexp + m->xstart[r], du, OR_GRAD, OR_INSERT);
      for (int q = 0; q < nq; q++) {
        const double *Du = du + 3 * q;
        double gamma = 0.5 * (Du[0] * Du[0] + Du[1] * Du[1] + Du[2] * Du[2]);
        double espg = eps * eps + gamma, eta = pow(espg, (p - 2) / 2);
        double sm = sqrt(-((p - 2) / 2) * eta / espg);
        double *st = stash + 4 * ((int64_t)qoff[r] + q);
        st[0] = eta;
        for (int i = 0; i < 3; i++) st[1 + i] = sm * Du[i];
      }
    }
    free(jinv); free(jw); free(du);
  }
  free(xexp); free(qoff);
  return err ? -1 : 0;
}

int or_plap_stash(const or_fs *m, double p, double eps, const double *g, double *stash)
{
  return or_plap_stash_mt(m, p, eps, g, stash, 1);
}

int or_elast_state(const or_fs *m, const double *g, double *Fq)
{
  if (m->bs != 3) return or_fail("elasticity needs block size 3");
  basis1d B[11];
  for (int k = 1; k <= 10; k++) if (basis_for(0, k, &B[k])) return -1;
  double *xexp = malloc(sizeof(double) * m->nexp * 3);
  or_fs_global_to_expanded(m, g, NULL, xexp);
  double *jinv = malloc(sizeof(double) * 9 * 1000), *jw = malloc(sizeof(double) * 1000), *du = malloc(sizeof(double) * 9000);
  int64_t off = 0;
  for (int64_t r = 0; r < m->nr; r++) {
    const basis1d *b[3] = {&B[m->edeg[3 * r]], &B[m->edeg[3 * r + 1]], &B[m->edeg[3 * r + 2]]};
    const int P[3] = {b[0]->P, b[1]->P, b[2]->P}, Q[3] = {b[0]->Q, b[1]->Q, b[2]->Q}, nq = Q[0] * Q[1] * Q[2];
    const double *bi[3] = {b[0]->interp, b[1]->interp, b[2]->interp}, *bd[3] = {b[0]->deriv, b[1]->deriv, b[2]->deriv};
    if (element_geometry(m, r, b, NULL, jinv, jw)) { free(xexp); free(jinv); free(jw); free(du); return -1; }
    or_efs_apply_hex(P, Q, bi, bd, jinv, 3, xexp + (int64_t)m->xstart[r] * 3, du, OR_GRAD, OR_INSERT);
    for (int q = 0; q < nq; q++)
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Fq[9 * (off + q) + i * 3 + j] = (i == j) + du[q * 9 + i * 3 + j];
    off += nq;
  }
  free(xexp); free(jinv); free(jw); free(du);
  return 0;
}

/* ----------------------------------------------------------------------------------------------
 * Lognormal coefficient: random Fourier features of the squared-exponential kernel
 * -------------------------------------------------------------------------------------------- */
int or_grf_make(int nf, double var, double ell, uint64_t seed, double *grf)
{
  const double twopi = 6.283185307179586476925286766559;
  uint64_t st = seed;
  grf[0] = nf; grf[1] = var; grf[2] = ell;
  for (int f = 0; f < nf; f++)
    for (int d = 0; d < 3; d++) {
      double u1 = or_uniform(&st), u2 = or_uniform(&st);
      if (u1 < 1e-300) u1 = 1e-300;
      grf[3 + 3 * f + d] = sqrt(-2.0 * log(u1)) * cos(twopi * u2) / ell; /* Box-Muller, N(0, 1/ell^2) */
    }
  for (int f = 0; f < nf; f++) grf[3 + 3 * nf + f] = twopi * or_uniform(&st);
  return 0;
}
double or_grf_eval(const double *grf, const double x[3])
{
  const int nf = (int)grf[0];
  const double *w = grf + 3, *b = grf + 3 + 3 * nf;
  double s = 0;
  for (int f = 0; f < nf; f++) s += cos(w[3 * f] * x[0] + w[3 * f + 1] * x[1] + w[3 * f + 2] * x[2] + b[f]);
  return sqrt(2.0 * grf[1] / nf) * s;
}

/* ----------------------------------------------------------------------------------------------
 * Q1-embedded assembly (EllipJacobian ellip.c:474-536, ElastJacobian elast.c:343-407) into CSR via
 * dFSMatSetValuesBlockedExpanded (fs.c:826-930): rows/cols through E, Dirichlet (negative global
 * index) entries dropped, ADD in call order.
 * -------------------------------------------------------------------------------------------- */
typedef struct { int32_t n, cap; int32_t *col; double *val; } rowlist;

static void row_add(rowlist *rl, int32_t c, double v)
{
  for (int i = 0; i < rl->n; i++)
    if (rl->col[i] == c) { rl->val[i] += v; return; }
  if (rl->n == rl->cap) {
    rl->cap = rl->cap ? 2 * rl->cap : 32;
    rl->col = realloc(rl->col, sizeof(int32_t) * rl->cap);
    rl->val = realloc(rl->val, sizeof(double) * rl->cap);
  }
  rl->col[rl->n] = c;
  rl->val[rl->n] = v;
  rl->n++;
}

static int cmp_pair(const void *a, const void *b)
{
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

/* EllipJacobian (ellip.c:474-536) on the SPARSE ruleset: the state's gradient at every SPARSE point comes from
 * GetPatchApplied (element GRAD with the point's own inverse Jacobian, then patch order), the store from
 * EllipPointwiseComputeStore, and the patch matrix from EllipPointwiseJacobian with the Q1 patch bases. */
static int64_t q1_assemble(const or_fs *m, int kind, const double *param, const double *grf, int quirk,
                           const double *state, const double *sdcache, int32_t *rowptr, int32_t **colp, double **valp)
{
  const int bs = m->bs;
  if (kind == 1 && (!state || bs != 1)) return or_fail("p-Laplacian Q1 assembly needs a scalar space and the state");
  const int64_t nrows = m->n * bs;
  rowlist *rows = calloc(nrows, sizeof(rowlist));
  basis1d B[11];
  for (int p = 1; p <= 10; p++) if (basis_for(1, p, &B[p])) return -1;
  double *sexp = NULL;
  if (kind == 1) {
    sexp = malloc(sizeof(double) * m->nexp);
    or_fs_global_to_expanded(m, state, sdcache, sexp);
  }
  for (int64_t r = 0; r < m->nr; r++) {
    const basis1d *b[3] = {&B[m->edeg[3 * r]], &B[m->edeg[3 * r + 1]], &B[m->edeg[3 * r + 2]]};
    const int Q[3] = {b[0]->Q, b[1]->Q, b[2]->Q}, nq = Q[0] * Q[1] * Q[2];
    double *xq = malloc(sizeof(double) * 3 * nq), *cjinv = malloc(sizeof(double) * 9 * nq), *jwe = malloc(sizeof(double) * nq);
    if (element_geometry(m, r, b, xq, cjinv, jwe)) return -1;
    double *sdu = NULL;
    if (kind == 1) {
      const int P[3] = {b[0]->P, b[1]->P, b[2]->P};
      const double *bi[3] = {b[0]->interp, b[1]->interp, b[2]->interp}, *bd[3] = {b[0]->deriv, b[1]->deriv, b[2]->deriv};
      sdu = malloc(sizeof(double) * 3 * nq);
      or_efs_apply_hex(P, Q, bi, bd, cjinv, 1, sexp + m->xstart[r], sdu, OR_GRAD, OR_INSERT);
    }
    int *ind = malloc(sizeof(int) * nq), psz;
    double *pw = malloc(sizeof(double) * nq);
    const int np = or_rule_patches(1, Q, b[0]->w, b[1]->w, b[2]->w, &psz, ind, pw);
    int *eidx = malloc(sizeof(int) * np * 8), P;
    double *interp = malloc(sizeof(double) * np * 64), *deriv = malloc(sizeof(double) * np * 192);
    double *pjinv = NULL;
    if (!quirk) { /* patch-ordered jinv: the geometrically consistent variant */
      pjinv = malloc(sizeof(double) * 9 * nq);
      for (int i = 0; i < nq; i++) memcpy(pjinv + 9 * i, cjinv + 9 * ind[i], 9 * sizeof(double));
    }
    if (or_explicit_sparse_hex(m->edeg[3 * r], m->edeg[3 * r + 1], m->edeg[3 * r + 2], np, 8, ind, quirk ? cjinv : pjinv, m->xstart[r], &P, eidx, interp, deriv)) return -1;
    for (int pt = 0; pt < np; pt++) {
      double K[24][24];
      memset(K, 0, sizeof K);
      for (int q = 0; q < 8; q++) {
        const int eq = ind[pt * 8 + q];
        const double w = jwe[eq];
        const double *I = interp + (pt * 8 + q) * 8, *Dd = deriv + (pt * 8 + q) * 24;
        if (kind == 1) {
          const double *Du = sdu + 3 * eq, pe = param[0], eps = param[1];
          const double gamma = 0.5 * (Du[0] * Du[0] + Du[1] * Du[1] + Du[2] * Du[2]);
          const double espg = eps * eps + gamma, eta = pow(espg, (pe - 2) / 2);
          const double sm = sqrt(-((pe - 2) / 2) * eta / espg);
          const double st[4] = {eta, sm * Du[0], sm * Du[1], sm * Du[2]};
          for (int j = 0; j < 8; j++) {
            double v, dv[3], uu = I[j];
            qfunction(1, 1, st, param, w, &uu, Dd + 3 * j, &v, dv);
            for (int i = 0; i < 8; i++) K[i][j] += I[i] * v + Dd[3 * i] * dv[0] + Dd[3 * i + 1] * dv[1] + Dd[3 * i + 2] * dv[2];
          }
        } else if (bs == 1) {
          double qd = grf ? exp(or_grf_eval(grf, xq + 3 * eq)) : 1.0;
          for (int j = 0; j < 8; j++) {
            double v, dv[3], uu = I[j];
            qfunction(0, 1, &qd, param, w, &uu, Dd + 3 * j, &v, dv);
            for (int i = 0; i < 8; i++) K[i][j] += I[i] * v + Dd[3 * i] * dv[0] + Dd[3 * i + 1] * dv[1] + Dd[3 * i + 2] * dv[2];
          }
        } else {
          for (int j = 0; j < 8; j++)
            for (int fj = 0; fj < 3; fj++) {
              double uu[3] = {0, 0, 0}, duu[9] = {0}, v[3], dv[9];
              uu[fj] = I[j];
              for (int e = 0; e < 3; e++) duu[fj * 3 + e] = Dd[3 * j + e];
              qfunction(2, 3, NULL, param, w, uu, duu, v, dv);
              for (int i = 0; i < 8; i++)
                for (int fi = 0; fi < 3; fi++)
                  K[i * 3 + fi][j * 3 + fj] += I[i] * v[fi] + Dd[3 * i] * dv[fi * 3] + Dd[3 * i + 1] * dv[fi * 3 + 1] + Dd[3 * i + 2] * dv[fi * 3 + 2];
            }
        }
      }
      for (int i = 0; i < 8; i++) {
        const int32_t rn = m->emap[eidx[pt * 8 + i]];
        if (rn >= m->n) continue;
        for (int fi = 0; fi < bs; fi++)
          for (int j = 0; j < 8; j++) {
            const int32_t cn = m->emap[eidx[pt * 8 + j]];
            if (cn >= m->n) continue;
            for (int fj = 0; fj < bs; fj++) row_add(&rows[(int64_t)rn * bs + fi], cn * bs + fj, K[i * bs + fi][j * bs + fj]);
          }
      }
    }
    free(xq); free(cjinv); free(jwe); free(ind); free(pw); free(eidx); free(interp); free(deriv); free(pjinv); free(sdu);
  }
  free(sexp);
  int64_t nnz = 0;
  for (int64_t i = 0; i < nrows; i++) nnz += rows[i].n;
  int32_t *col = malloc(sizeof(int32_t) * (nnz ? nnz : 1));
  double *val = malloc(sizeof(double) * (nnz ? nnz : 1));
  int64_t o = 0;
  for (int64_t i = 0; i < nrows; i++) {
    rowptr[i] = (int32_t)o;
    int32_t *perm = malloc(sizeof(int32_t) * 2 * (rows[i].n ? rows[i].n : 1));
    for (int k = 0; k < rows[i].n; k++) { perm[2 * k] = rows[i].col[k]; perm[2 * k + 1] = k; }
    qsort(perm, rows[i].n, 2 * sizeof(int32_t), cmp_pair);
    for (int k = 0; k < rows[i].n; k++) { col[o] = perm[2 * k]; val[o] = rows[i].val[perm[2 * k + 1]]; o++; }
    free(perm); free(rows[i].col); free(rows[i].val);
  }
  rowptr[nrows] = (int32_t)o;
  free(rows);
  *colp = col;
  *valp = val;
  return nnz;
}

int64_t or_q1_assemble(const or_fs *m, int kind, const double *param, const double *grf, int quirk,
                       int32_t *rowptr, int32_t **colp, double **valp)
{
  if (kind == 1) return or_fail("p-Laplacian Q1 assembly needs the state: use or_q1_assemble_plap");
  return q1_assemble(m, kind, param, grf, quirk, NULL, NULL, rowptr, colp, valp);
}

int64_t or_q1_assemble_plap(const or_fs *m, double p, double eps, const double *g, int quirk,
                            int32_t *rowptr, int32_t **colp, double **valp)
{
  const double param[2] = {p, eps};
  return q1_assemble(m, 1, param, NULL, quirk, g, NULL, rowptr, colp, valp);
}

int64_t or_q1_assemble_plap_dir(const or_fs *m, double p, double eps, const double *g, const double *dcache, int quirk,
                                int32_t *rowptr, int32_t **colp, double **valp)
{
  const double param[2] = {p, eps};
  return q1_assemble(m, 1, param, NULL, quirk, g, dcache, rowptr, colp, valp);
}

/* ----------------------------------------------------------------------------------------------
 * Krylov + Chebyshev-Jacobi (replacements for PETSc KSPCG and KSPCHEBYSHEV/PCJACOBI)
 * -------------------------------------------------------------------------------------------- */
void or_csr_mult(int64_t nrows, const int32_t *rp, const int32_t *col, const double *val, const double *x, double *y)
{
  for (int64_t i = 0; i < nrows; i++) {
    double s = 0;
    for (int32_t k = rp[i]; k < rp[i + 1]; k++) s += val[k] * x[col[k]];
    y[i] = s;
  }
}

static double dot(int64_t n, const double *a, const double *b)
{
  double s = 0;
  for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* Chebyshev iteration (Saad, Iterative Methods, Alg. 12.1) on D^{-1} A with zero initial guess. */
static void cheb_apply(int64_t n, const int32_t *rp, const int32_t *col, const double *val, const double *dinv,
                       double emin, double emax, int degree, const double *r, double *z, double *w, double *d)
{
  const double theta = 0.5 * (emax + emin), delta = 0.5 * (emax - emin), sigma = theta / delta;
  double rho = 1.0 / sigma;
  for (int64_t i = 0; i < n; i++) { d[i] = dinv[i] * r[i] / theta; z[i] = d[i]; }
  for (int k = 1; k < degree; k++) {
    or_csr_mult(n, rp, col, val, z, w);
    const double rho1 = 1.0 / (2.0 * sigma - rho);
    for (int64_t i = 0; i < n; i++) {
      d[i] = rho1 * rho * d[i] + 2.0 * rho1 / delta * dinv[i] * (r[i] - w[i]);
      z[i] += d[i];
    }
    rho = rho1;
  }
}

int or_cg_solve(const or_fs *m, int kind, const double *qdata, const double *param,
                const int32_t *rp, const int32_t *col, const double *val, int cheb_degree,
                const double *b, double *x, double rtol, int maxit, double *rnorm, int nthreads)
{
  const int64_t n = m->n * m->bs;
  double *r = malloc(8 * n), *z = malloc(8 * n), *p = malloc(8 * n), *q = malloc(8 * n);
  double *dinv = malloc(8 * n), *w = malloc(8 * n), *d = malloc(8 * n);
  for (int64_t i = 0; i < n; i++) {
    dinv[i] = 0;
    for (int32_t k = rp[i]; k < rp[i + 1]; k++) if (col[k] == i) dinv[i] = 1.0 / val[k];
  }
  /* lambda_max(D^{-1} A) by 20 power steps from a seeded vector */
  uint64_t st = 12345;
  for (int64_t i = 0; i < n; i++) z[i] = or_uniform(&st) - 0.5;
  double lam = 1;
  for (int it = 0; it < 20; it++) {
    or_csr_mult(n, rp, col, val, z, w);
    for (int64_t i = 0; i < n; i++) w[i] *= dinv[i];
    double nw = sqrt(dot(n, w, w)), nz = sqrt(dot(n, z, z));
    lam = nw / nz;
    for (int64_t i = 0; i < n; i++) z[i] = w[i] / nw;
  }
  const double emax = 1.1 * lam, emin = 0.1 * lam;
  int its = -1;
  or_operator_apply(m, kind, qdata, param, x, q, nthreads);
  for (int64_t i = 0; i < n; i++) r[i] = b[i] - q[i];
  const double bn = sqrt(dot(n, b, b));
  double res = sqrt(dot(n, r, r));
  cheb_apply(n, rp, col, val, dinv, emin, emax, cheb_degree, r, z, w, d);
  memcpy(p, z, 8 * n);
  double rz = dot(n, r, z);
  for (int it = 0; it < maxit; it++) {
    if (res <= rtol * bn) { its = it; break; }
    or_operator_apply(m, kind, qdata, param, p, q, nthreads);
    const double alpha = rz / dot(n, p, q);
    for (int64_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    res = sqrt(dot(n, r, r));
    if (res <= rtol * bn) { its = it + 1; break; }
    cheb_apply(n, rp, col, val, dinv, emin, emax, cheb_degree, r, z, w, d);
    const double rz1 = dot(n, r, z), beta = rz1 / rz;
    rz = rz1;
    for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
  }
  if (rnorm) *rnorm = res / (bn > 0 ? bn : 1);
  free(r); free(z); free(p); free(q); free(dinv); free(w); free(d);
  return its;
}

/* ----------------------------------------------------------------------------------------------
 * Facet rules and boundary integrals over the faces of weak boundary sets
 * -------------------------------------------------------------------------------------------- */
/* The side transforms of dQuadratureGetFacetRules_Tensor_Private (tensorquad.c:324-331): a node (X, Y) of the
 * reference quad maps to xi = R (X, Y, 0) + t on side s of the reference hex (dRuleGetNodeWeight_Transformed,
 * tensorquad.c:224-242). The reference's quad rule has no node accessor (ruletopo.c:184), so the quad node order is
 * this restatement's convention: X slowest. */
static const double or_side_R[6][3][3] = {
  {{1, 0, 0}, {0, 0, -1}, {0, 1, 0}},  {{0, 0, 1}, {1, 0, 0}, {0, 1, 0}},   {{-1, 0, 0}, {0, 0, 1}, {0, 1, 0}},
  {{0, 0, -1}, {-1, 0, 0}, {0, 1, 0}}, {{0, 1, 0}, {1, 0, 0}, {0, 0, -1}}, {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};
static const double or_side_t[6][3] = {{0, -1, 0}, {1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, 0, -1}, {0, 0, 1}};

int or_facet_rule(int side, int method, int order, double *nodes, double *weights)
{
  double x[128], w[128];
  if (side < 0 || side > 5) return or_fail("side %d out of range", side);
  const int n = or_rule_1d(method, 0, order, x, w);
  if (n < 0) return -1;
  for (int a = 0; a < n; a++)
    for (int b = 0; b < n; b++) {
      const double ref[3] = {x[a], x[b], 0.0};
      for (int c = 0; c < 3; c++)
        nodes[3 * (a * n + b) + c] = or_side_R[side][c][0] * ref[0] + or_side_R[side][c][1] * ref[1] +
                                     or_side_R[side][c][2] * ref[2] + or_side_t[side][c];
      weights[a * n + b] = w[a] * w[b];
    }
  return n * n;
}

/* the faces of the weak sets (bit0 100 walls, bit1 200 top, bit2 300 bottom; generator face sets 0..3 -> 100,
 * 4 -> 300, 5 -> 200) as (region, side) pairs in region order, sides in the canonical order of the adjacency */
static int64_t facet_list(const or_fs *m, int weak_mask, int32_t *fel, int32_t *fside)
{
  static const int setbit[6] = {0, 0, 0, 0, 2, 1};
  const int64_t R0 = m->nv + m->ne + m->nf;
  int64_t nf = 0;
  for (int64_t r = 0; r < m->nr; r++)
    for (int s = 0; s < 6; s++) {
      const int st = m->fset[m->adjind[m->adjoff[R0 + r] + s]];
      if (st < 0 || !((weak_mask >> setbit[st]) & 1)) continue;
      if (fel) { fel[nf] = (int32_t)r; fside[nf] = s; }
      nf++;
    }
  return nf;
}

/* direction of the reference hex that the facet's X (k=0) or Y (k=1) axis runs along */
static int side_axis(int s, int k)
{
  for (int c = 0; c < 3; c++)
    if (or_side_R[s][c][k] != 0) return c;
  return -1;
}

int64_t or_facet_count(const or_fs *m, int weak_mask, int64_t *nfacets, int32_t *fel, int32_t *fside, int32_t *qoff)
{
  const int64_t nf = facet_list(m, weak_mask, NULL, NULL);
  int32_t *e = malloc(sizeof(int32_t) * (nf + 1)), *s = malloc(sizeof(int32_t) * (nf + 1));
  facet_list(m, weak_mask, e, s);
  int64_t nq = 0;
  if (qoff) qoff[0] = 0;
  for (int64_t f = 0; f < nf; f++) {
    const int r = e[f];
    nq += (int64_t)(m->edeg[3 * r + side_axis(s[f], 0)] + 1) * (m->edeg[3 * r + side_axis(s[f], 1)] + 1);
    if (fel) { fel[f] = e[f]; fside[f] = s[f]; }
    if (qoff) qoff[f + 1] = (int32_t)nq;
  }
  free(e); free(s);
  if (nfacets) *nfacets = nf;
  return nq;
}

/* for one facet point: reference point xi, 1-D Lagrange values of the field's GLL basis per direction (full
 * element: all P_c nodes, evaluated at xi_c by the TensorBasisCreate evaluation), area vector and physical point */
typedef struct { double xi[3], w, L[3][16], x[3], cr[3]; int P[3]; } facet_pt;

static int facet_point(const or_fs *m, int r, int s, int a, int b, facet_pt *fp)
{
  const int cx = side_axis(s, 0), cy = side_axis(s, 1);
  double gx[16], gwx[16], gy[16], gwy[16], node[16], weight[16], dd[16], ci[3][2], cd[3][2];
  for (int c = 0; c < 3; c++) fp->P[c] = m->edeg[3 * r + c] + 1;
  if (or_rule_1d(0, 0, 2 * (fp->P[cx] - 1), gx, gwx) < 0 || or_rule_1d(0, 0, 2 * (fp->P[cy] - 1), gy, gwy) < 0) return -1;
  const double ref[3] = {gx[a], gy[b], 0.0};
  for (int c = 0; c < 3; c++)
    fp->xi[c] = or_side_R[s][c][0] * ref[0] + or_side_R[s][c][1] * ref[1] + or_side_R[s][c][2] * ref[2] + or_side_t[s][c];
  fp->w = gwx[a] * gwy[b];
  for (int c = 0; c < 3; c++) {
    if (or_tensor_basis(fp->P[c], 1, &fp->xi[c], fp->L[c], dd, node, weight)) return -1;
    if (or_tensor_basis(2, 1, &fp->xi[c], ci[c], cd[c], node, weight)) return -1;
  }
  /* coordinate FS (Q1, tensor vertex order): x and J = dx/dxi */
  const double *X = m->xexp + (int64_t)r * 24;
  double J[3][3] = {{0}};
  for (int d = 0; d < 3; d++) fp->x[d] = 0;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) {
        const double *v = X + 3 * ((i * 2 + j) * 2 + k);
        for (int d = 0; d < 3; d++) {
          fp->x[d] += ci[0][i] * ci[1][j] * ci[2][k] * v[d];
          J[d][0] += cd[0][i] * ci[1][j] * ci[2][k] * v[d];
          J[d][1] += ci[0][i] * cd[1][j] * ci[2][k] * v[d];
          J[d][2] += ci[0][i] * ci[1][j] * cd[2][k] * v[d];
        }
      }
  double tx[3], ty[3];
  for (int d = 0; d < 3; d++) {
    tx[d] = ty[d] = 0;
    for (int c = 0; c < 3; c++) { tx[d] += J[d][c] * or_side_R[s][c][0]; ty[d] += J[d][c] * or_side_R[s][c][1]; }
  }
  fp->cr[0] = tx[1] * ty[2] - tx[2] * ty[1];
  fp->cr[1] = tx[2] * ty[0] - tx[0] * ty[2];
  fp->cr[2] = tx[0] * ty[1] - tx[1] * ty[0];
  return 0;
}

int or_facet_points(const or_fs *m, int weak_mask, const double *g, double *jw, double *x, double *nrm, double *u)
{
  int64_t nf;
  or_facet_count(m, weak_mask, &nf, NULL, NULL, NULL);
  int32_t *fel = malloc(sizeof(int32_t) * (nf + 1)), *fside = malloc(sizeof(int32_t) * (nf + 1)), *qoff = malloc(sizeof(int32_t) * (nf + 1));
  or_facet_count(m, weak_mask, &nf, fel, fside, qoff);
  const int bs = m->bs;
  double *xe = calloc((size_t)m->nexp * bs, sizeof(double));
  if (g) or_fs_global_to_expanded(m, g, NULL, xe);
  int rc = 0;
  for (int64_t f = 0; f < nf && !rc; f++) {
    const int r = fel[f], s = fside[f], nY = m->edeg[3 * r + side_axis(s, 1)] + 1;
    for (int64_t q = qoff[f]; q < qoff[f + 1] && !rc; q++) {
      facet_pt fp;
      const int loc = (int)(q - qoff[f]);
      if ((rc = facet_point(m, r, s, loc / nY, loc % nY, &fp))) break;
      const double ar = sqrt(fp.cr[0] * fp.cr[0] + fp.cr[1] * fp.cr[1] + fp.cr[2] * fp.cr[2]);
      jw[q] = fp.w * ar;
      for (int d = 0; d < 3; d++) { x[3 * q + d] = fp.x[d]; nrm[3 * q + d] = fp.cr[d] / ar; }
      for (int c = 0; c < bs; c++) { /* the whole element basis at the point */
        double acc = 0;
        for (int i = 0; i < fp.P[0]; i++)
          for (int j = 0; j < fp.P[1]; j++)
            for (int k = 0; k < fp.P[2]; k++)
              acc += fp.L[0][i] * fp.L[1][j] * fp.L[2][k] * xe[((int64_t)m->xstart[r] + (i * fp.P[1] + j) * fp.P[2] + k) * bs + c];
        u[q * bs + c] = acc;
      }
    }
  }
  free(fel); free(fside); free(qoff); free(xe);
  return rc;
}

int or_facet_commit(const or_fs *m, int weak_mask, const double *v, double *y, int add)
{
  int64_t nf;
  or_facet_count(m, weak_mask, &nf, NULL, NULL, NULL);
  int32_t *fel = malloc(sizeof(int32_t) * (nf + 1)), *fside = malloc(sizeof(int32_t) * (nf + 1)), *qoff = malloc(sizeof(int32_t) * (nf + 1));
  or_facet_count(m, weak_mask, &nf, fel, fside, qoff);
  const int bs = m->bs;
  double *ye = calloc((size_t)m->nexp * bs, sizeof(double));
  int rc = 0;
  for (int64_t f = 0; f < nf && !rc; f++) {
    const int r = fel[f], s = fside[f], nY = m->edeg[3 * r + side_axis(s, 1)] + 1;
    for (int64_t q = qoff[f]; q < qoff[f + 1]; q++) {
      facet_pt fp;
      const int loc = (int)(q - qoff[f]);
      if ((rc = facet_point(m, r, s, loc / nY, loc % nY, &fp))) break;
      for (int i = 0; i < fp.P[0]; i++)
        for (int j = 0; j < fp.P[1]; j++)
          for (int k = 0; k < fp.P[2]; k++) {
            const double phi = fp.L[0][i] * fp.L[1][j] * fp.L[2][k];
            for (int c = 0; c < bs; c++) ye[((int64_t)m->xstart[r] + (i * fp.P[1] + j) * fp.P[2] + k) * bs + c] += phi * v[q * bs + c];
          }
    }
  }
  if (!rc) or_fs_expanded_to_global(m, ye, y, add);
  free(fel); free(fside); free(qoff); free(ye);
  return rc;
}

/* ----------------------------------------------------------------------------------------------
 * Stokes (src/fs/tests/stokes.c, stokesimpl.h): velocity space (bs 3, degree k) and pressure space (bs 1,
 * degree k - codim, continuous, no Dirichlet sets) on the same mesh, the velocity's FAST rule (order 2k).
 * -------------------------------------------------------------------------------------------- */
/* include/dohp.h:77-82 */
static double colon_sym(const double a[6], const double b[6])
{
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + 2 * a[3] * b[3] + 2 * a[4] * b[4] + 2 * a[5] * b[5];
}
static void sym_compress(const double du[9], double s[6])
{
  s[0] = du[0]; s[1] = du[4]; s[2] = du[8];
  s[3] = (du[1] + du[3]) / 2; s[4] = (du[2] + du[6]) / 2; s[5] = (du[5] + du[7]) / 2;
}
static void sym_uncompress(const double s[6], double du[9])
{
  du[0] = s[0]; du[4] = s[1]; du[8] = s[2];
  du[1] = du[3] = s[3]; du[2] = du[6] = s[4]; du[5] = du[7] = s[5];
}

/* MatMult_Nest_StokesCoupled (stokes.c:541-577 with StokesPointwiseJacobian, stokes.c:476-487) and
 * StokesShellMatMult_All_IorA (stokes.c:579-673 with StokesPointwiseJacobian_A/_B/_Bt, stokes.c:489-505).
 * mode 0 A (with the penalty lambda = nu/(1-2nu), StokesLambda stokes.c:455-458), 1 Bt, 2 B, 3 coupled (lambda = 0).
 * The store (StokesPointwiseComputeStore stokes.c:447-453) is evaluated from the velocity state su (NULL: zero).
 * mode 4 is the nonlinear function of StokesFunction (stokes.c:507-540, StokesPointwiseFunction stokes.c:460-474)
 * without the forcing terms: Dv = w (eta(Du) Du - p I), q = -w div u, the store taken from xu itself (su unused). */
static int stokes_eval(const or_fs *fu, const or_fs *fp, int mode, const double rheo[4], const double *su, const double *sudir,
                       const double *xu, const double *udir, const double *xp, const double *fq, const double *fpq, double *yu,
                       double *yp)
{
  if (fu->bs != 3 || fp->bs != 1) return or_fail("Stokes needs a bs 3 velocity space and a bs 1 pressure space");
  if (fu->nr != fp->nr) return or_fail("velocity and pressure spaces are on different meshes");
  const double Bv = rheo[0], eps = rheo[1], pw = rheo[2], nu = rheo[3];
  const double lambda = mode == 0 ? nu / (1 - 2 * nu) : 0.0;
  if (mode < 0 || mode > 4) return or_fail("invalid Stokes mode");
  const int use_u = mode != 1, use_p = mode == 1 || mode == 3 || mode == 4;
  const int out_u = mode != 2, out_p = mode >= 2;
  double *xeu = calloc((size_t)fu->nexp * 3, sizeof(double)), *xep = calloc((size_t)fp->nexp, sizeof(double));
  double *seu = calloc((size_t)fu->nexp * 3, sizeof(double));
  double *yeu = calloc((size_t)fu->nexp * 3, sizeof(double)), *yep = calloc((size_t)fp->nexp, sizeof(double));
  if (use_u) or_fs_global_to_expanded(fu, xu, udir, xeu);
  if (use_p) or_fs_global_to_expanded(fp, xp, NULL, xep);
  if (mode == 4) memcpy(seu, xeu, sizeof(double) * (size_t)fu->nexp * 3); /* the function's state is its argument */
  else if (su) or_fs_global_to_expanded(fu, su, sudir, seu);
  double *jinv = malloc(sizeof(double) * 9 * 1000), *jw = malloc(sizeof(double) * 1000);
  double *du = malloc(sizeof(double) * 9000), *ds = malloc(sizeof(double) * 9000), *dv = malloc(sizeof(double) * 9000);
  double *pq = malloc(sizeof(double) * 1000), *qv = malloc(sizeof(double) * 1000), *vq = malloc(sizeof(double) * 3000);
  int rc = 0;
  int64_t qo = 0; /* offset of the element's first point in fq / fpq */
  for (int64_t r = 0; r < fu->nr && !rc; r++) {
    basis1d bu;
    if (basis_for(0, fu->edeg[3 * r], &bu)) { rc = -1; break; }
    const basis1d *b[3] = {&bu, &bu, &bu};
    const int P[3] = {bu.P, bu.P, bu.P}, Q[3] = {bu.Q, bu.Q, bu.Q}, nq = bu.Q * bu.Q * bu.Q;
    const int Pp1 = fp->edeg[3 * r] + 1, Pp[3] = {Pp1, Pp1, Pp1};
    double bpi[11 * 16], bpd[11 * 16], node[16], weight[16];
    if (or_tensor_basis(Pp1, bu.Q, bu.x, bpi, bpd, node, weight)) { rc = -1; break; }
    const double *bi[3] = {bu.interp, bu.interp, bu.interp}, *bd[3] = {bu.deriv, bu.deriv, bu.deriv};
    const double *pi3[3] = {bpi, bpi, bpi}, *pd3[3] = {bpd, bpd, bpd};
    if (element_geometry(fu, r, b, NULL, jinv, jw)) { rc = -1; break; }
    or_efs_apply_hex(P, Q, bi, bd, jinv, 3, xeu + (int64_t)fu->xstart[r] * 3, du, OR_GRAD, OR_INSERT);
    or_efs_apply_hex(P, Q, bi, bd, jinv, 3, seu + (int64_t)fu->xstart[r] * 3, ds, OR_GRAD, OR_INSERT);
    or_efs_apply_hex(Pp, Q, pi3, pd3, NULL, 1, xep + fp->xstart[r], pq, OR_INTERP, OR_INSERT);
    for (int q = 0; q < nq; q++) {
      double Du[6], Ds[6], Dv[6];
      sym_compress(du + 9 * q, Du);
      sym_compress(ds + 9 * q, Ds);
      const double greg = 0.5 * eps * eps + 0.5 * colon_sym(Ds, Ds);
      const double eta = Bv * pow(greg, 0.5 * (pw - 2)), deta = 0.5 * (pw - 2) * eta / greg;
      const double w = jw[q], tr = Du[0] + Du[1] + Du[2], dc = deta * colon_sym(Ds, Du), p = pq[q];
      for (int i = 0; i < 6; i++) {
        switch (mode) {
          case 0: Dv[i] = w * (eta * Du[i] + dc * Ds[i] + lambda * (i < 3) * tr); break;
          case 1: Dv[i] = i < 3 ? -w * p : 0; break;
          case 3: Dv[i] = w * (eta * Du[i] + dc * Ds[i] + lambda * (i < 3) * tr - p * (i < 3)); break;
          case 4: Dv[i] = w * (eta * Du[i] - p * (i < 3)); break;
          default: Dv[i] = 0;
        }
      }
      sym_uncompress(Dv, dv + 9 * q);
      /* StokesPointwiseFunction's forcing terms: v = -w fu, q = -w (div u + fp) */
      qv[q] = -w * (tr + (fpq ? fpq[qo + q] : 0.0));
      if (fq)
        for (int c = 0; c < 3; c++) vq[3 * q + c] = -w * fq[3 * (qo + q) + c];
    }
    if (out_u) or_efs_apply_hex(P, Q, bi, bd, jinv, 3, dv, yeu + (int64_t)fu->xstart[r] * 3, OR_GRAD_TRANSPOSE, OR_INSERT);
    if (out_u && fq) or_efs_apply_hex(P, Q, bi, bd, NULL, 3, vq, yeu + (int64_t)fu->xstart[r] * 3, OR_INTERP_TRANSPOSE, OR_ADD);
    if (out_p) or_efs_apply_hex(Pp, Q, pi3, pd3, NULL, 1, qv, yep + fp->xstart[r], OR_INTERP_TRANSPOSE, OR_INSERT);
    qo += nq;
  }
  if (!rc) {
    if (out_u) or_fs_expanded_to_global(fu, yeu, yu, 0);
    if (out_p) or_fs_expanded_to_global(fp, yep, yp, 0);
  }
  free(xeu); free(xep); free(seu); free(yeu); free(yep); free(jinv); free(jw); free(du); free(ds); free(dv); free(pq); free(qv);
  free(vq);
  return rc ? (rc == -1 ? -1 : or_fail("negative Jacobian")) : 0;
}

int or_stokes_apply(const or_fs *fu, const or_fs *fp, int mode, const double rheo[4], const double *su, const double *xu,
                    const double *xp, double *yu, double *yp)
{
  return stokes_eval(fu, fp, mode, rheo, su, NULL, xu, NULL, xp, NULL, NULL, yu, yp);
}

/* or_stokes_apply with a state that carries inhomogeneous Dirichlet values sudir ([nc - n][3]); x is expanded
 * homogeneously (MatMult_Nest_StokesCoupled, stokes.c:556) */
int or_stokes_apply_state(const or_fs *fu, const or_fs *fp, int mode, const double rheo[4], const double *su, const double *sudir,
                          const double *xu, const double *xp, double *yu, double *yp)
{
  if (mode == 4) return or_fail("the function takes its state from its argument (or_stokes_function)");
  return stokes_eval(fu, fp, mode, rheo, su, sudir, xu, NULL, xp, NULL, NULL, yu, yp);
}

/* StokesFunction (stokes.c:507-540) in full: inhomogeneous Dirichlet velocity values udir (closure tail, [nc - n][3],
 * NULL = 0; dFS_INHOMOGENEOUS expansion) and the forcing fq [nq][3], fpq [nq] at the velocity FAST points in
 * or_fs_qpt_coords order (NULL = 0) */
int or_stokes_function(const or_fs *fu, const or_fs *fp, const double rheo[4], const double *xu, const double *udir,
                       const double *xp, const double *fq, const double *fpq, double *yu, double *yp)
{
  return stokes_eval(fu, fp, 4, rheo, NULL, NULL, xu, udir, xp, fq, fpq, yu, yp);
}
