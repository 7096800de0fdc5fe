// 1-D GLL nodal bases and Gauss rules (host setup).
//
// Restates TensorBasisCreate (src/jacobi/impls/tensor/tensor.c:22-109) and TensorGetRule
// (src/jacobi/quadrature/impls/tensor/tensorquad.c:32-118): Legendre-Gauss points for FAST rules, two
// points per GLL sub-interval for SPARSE rules, Lagrange basis on GLL nodes evaluated at the rule points.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "internal.h"

namespace dgb {

static thread_local char g_err[1024];

dErr set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return 1;
}

// Legendre P_n and P_{n-1} at x by the three-term recurrence (long double)
static void legendre(int n, long double x, long double *pn, long double *pnm1) {
  long double a = 1.0L, b = x;
  if (n == 0) {
    *pn = 1;
    *pnm1 = 0;
    return;
  }
  for (int k = 1; k < n; k++) {
    long double c = ((2 * k + 1) * x * b - k * a) / (k + 1);
    a = b;
    b = c;
  }
  *pn = b;
  *pnm1 = a;
}

void gauss_rule(int n, double *x, double *w) {
  const long double pi = 3.141592653589793238462643383279502884L;
  if (n == 1) {
    x[0] = 0;
    w[0] = 2;
    return;
  }
  for (int i = 0; i < n; i++) {
    long double z = -cosl(pi * (4 * i + 3) / (4 * n + 2)), pn, pm, dp = 1;
    for (int it = 0; it < 64; it++) {
      legendre(n, z, &pn, &pm);
      dp = n * (z * pn - pm) / (z * z - 1);
      long double dz = pn / dp;
      z -= dz;
      if (fabsl(dz) < 1e-19L) break;
    }
    legendre(n, z, &pn, &pm);
    dp = n * (z * pn - pm) / (z * z - 1);
    x[i] = (double)z;
    w[i] = (double)(2 / ((1 - z * z) * dp * dp));
  }
}

void lobatto_rule(int n, double *x, double *w) {
  const long double pi = 3.141592653589793238462643383279502884L;
  const int N = n - 1;
  if (n == 1) {
    x[0] = 0;
    w[0] = 2;
    return;
  }
  for (int i = 0; i < n; i++) {
    long double z, pn, pm;
    if (i == 0 || i == N) {
      z = i == 0 ? -1.0L : 1.0L;
      pn = (i == 0 && (N % 2)) ? -1.0L : 1.0L;
    } else {
      z = -cosl(pi * i / N);
      for (int it = 0; it < 64; it++) {  // zeros of (1-z^2) P'_N
        legendre(N, z, &pn, &pm);
        long double dz = (z * pn - pm) / ((N + 1) * pn);
        z -= dz;
        if (fabsl(dz) < 1e-19L) break;
      }
      legendre(N, z, &pn, &pm);
    }
    x[i] = (double)z;
    w[i] = (double)(2.0L / (N * (N + 1) * pn * pn));
  }
}

void lagrange(int P, const double *nodes, double t, double *val, double *der) {
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

// family: dGAUSS_LEGENDRE or dGAUSS_LOBATTO (FAST and SPARSE rules; SELF rules are Lobatto); -1 for another
int rule_1d(dQuadratureMethod method, int order, double *x, double *w, int family) {
  if (family != dGAUSS_LEGENDRE && family != dGAUSS_LOBATTO) return -1;
  if (method == dQUADRATURE_METHOD_SPARSE) {
    int size = order > 0 ? order : 1;
    if (size == 1) {
      x[0] = 0;
      w[0] = 2;
      return 1;
    }
    int nel = size / 2;
    double iv[64], un[64];
    lobatto_rule(nel + 1, iv, un);
    // two points per GLL sub-interval: the Gauss pair +-1/sqrt(3), or the Lobatto pair (the interval's ends)
    const double g = family == dGAUSS_LEGENDRE ? 0.57735026918962573 : 1.0;
    for (int i = 0; i < nel; i++) {
      double h = iv[i + 1] - iv[i];
      x[2 * i] = iv[i] + (1 - g) * h / 2.;
      x[2 * i + 1] = iv[i] + (1 + g) * h / 2.;
      w[2 * i] = w[2 * i + 1] = h / 2.;
    }
    return size;
  }
  if (method == dQUADRATURE_METHOD_FAST) {
    if (family == dGAUSS_LOBATTO) {  // n Lobatto points integrate order 2n - 3 exactly
      int size = 2 + order / 2;
      lobatto_rule(size, x, w);
      return size;
    }
    int size = 1 + order / 2;
    gauss_rule(size, x, w);
    return size;
  }
  if (method == dQUADRATURE_METHOD_SELF) {
    int size = 1 + order / 2;
    lobatto_rule(size, x, w);
    return size;
  }
  return -1;
}

int make_basis(int p, dQuadratureMethod method, Basis1D *b) {
  if (p < 1 || p + 1 > MAXP) return set_error("basis degree %d out of range [1,%d]", p, MAXP - 1);
  b->P = p + 1;
  b->Q = rule_1d(method, 2 * p, b->x, b->w);
  if (b->Q < 1 || b->Q > MAXQ) return set_error("rule size %d out of range", b->Q);
  lobatto_rule(b->P, b->node, b->nodew);
  for (int i = 0; i < b->Q; i++) {
    lagrange(b->P, b->node, b->x[i], b->B + i * b->P, b->D + i * b->P);
    const double cn[2] = {-1.0, 1.0};
    lagrange(2, cn, b->x[i], b->cB + 2 * i, b->cD + 2 * i);
  }
  // collocation derivative at the rule points: Dq[i][j] = l_j'(x_i) for the Lagrange basis on the rule points
  for (int i = 0; i < b->Q; i++) {
    double val[MAXQ];
    lagrange(b->Q, b->x, b->x[i], val, b->Dq + i * b->Q);
  }
  return 0;
}

}  // namespace dgb

extern "C" const char *dGetLastError(void) { return dgb::g_err; }
