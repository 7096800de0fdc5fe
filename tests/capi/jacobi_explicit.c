/* A plain-C caller of the C ABI's host-side jacobi entry points, in the shape of the reference's explicit-basis test
 * program (src/jacobi/tests/ex3.c, TestExplicitBases): four hexahedral element spaces of a dJacobi type on the FAST
 * rules of one degree, each printed as its interpolation, gradient and mass matrices in the program's format.
 *
 *   jacobi_explicit tensor|modal gauss|lobatto <rule degree>
 *
 * tensor: basis degrees 1..4 per direction; modal: orders 0..3 (ex3.c's GetEFS). No GPU is needed. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dohp_gb300.h"

#define CHK(call)                                                 \
  do {                                                            \
    if ((call) != 0) {                                            \
      fprintf(stderr, "%s failed: %s\n", #call, dGetLastError()); \
      return 1;                                                   \
    }                                                             \
  } while (0)

static void print_matrix(dInt m, dInt n, const dReal *a) {
  for (dInt i = 0; i < m; i++)
    for (dInt j = 0; j < n; j++) printf("%+10.6f%s", a[i * n + j], j + 1 == n ? "\n" : " ");
}

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s tensor|modal gauss|lobatto <rule degree>\n", argv[0]);
    return 2;
  }
  const int modal = !strcmp(argv[1], "modal"), lobatto = !strcmp(argv[2], "lobatto"), rp = atoi(argv[3]);
  dJacobi jac;
  dQuadrature quad;
  dRule *rules;
  dEFS *efs;
  dEntTopology topo[4] = {dTOPO_HEX, dTOPO_HEX, dTOPO_HEX, dTOPO_HEX};
  dPolynomialOrder rdegree[4], bdegree[4];
  CHK(dJacobiCreate(&jac));
  CHK(dJacobiSetType(jac, modal ? dJACOBI_MODAL : dJACOBI_TENSOR));
  for (int i = 0; i < 4; i++) {
    rdegree[i] = modal ? dPolynomialOrderCreate(rp, 0, 0, 0) : dPolynomialOrderCreate(0, rp, rp, rp);
    bdegree[i] = modal ? dPolynomialOrderCreate(i, 0, 0, 0) : dPolynomialOrderCreate(0, i + 1, i + 1, i + 1);
  }
  CHK(dJacobiGetQuadrature(jac, dQUADRATURE_METHOD_FAST, &quad));
  if (lobatto) CHK(dQuadratureTensorSetGaussFamily(quad, dGAUSS_LOBATTO));
  CHK(dQuadratureGetRules(quad, 4, topo, rdegree, &rules));
  CHK(dJacobiGetEFS(jac, 4, topo, bdegree, rules, &efs));
  for (int i = 0; i < 4; i++) {
    dInt n, m, Q, P;
    const dReal *interp, *deriv;
    CHK(dRuleGetSize(rules[i], NULL, &n));
    CHK(dEFSGetSizes(efs[i], NULL, NULL, &m));
    dReal *coord = malloc(sizeof(dReal) * 3 * n), *weight = malloc(sizeof(dReal) * n), *mass = calloc((size_t)m * m, sizeof(dReal));
    if (!coord || !weight || !mass) return 1;
    CHK(dRuleGetNodeWeight(rules[i], coord, weight));
    CHK(dEFSGetExplicit(efs[i], NULL, &Q, &P, &interp, &deriv));
    if (Q != n || P != m) return 1;
    printf("Interpolation matrix of size (%d,%d)\n", Q, P);
    print_matrix(Q, P, interp);
    printf("Gradient matrix of size (%d,%d*3)\n", Q, P);
    print_matrix(Q, P * 3, deriv);
    for (dInt j = 0; j < Q; j++)
      for (dInt k = 0; k < P; k++)
        for (dInt l = 0; l < P; l++) mass[k * P + l] += interp[j * P + k] * weight[j] * interp[j * P + l];
    printf("Mass matrix of size (%d,%d)\n", P, P);
    print_matrix(P, P, mass);
    CHK(dEFSRestoreExplicit(efs[i], NULL, &Q, &P, &interp, &deriv));
    free(coord);
    free(weight);
    free(mass);
  }
  CHK(dFree(rules));
  CHK(dFree(efs));
  CHK(dJacobiDestroy(&jac));
  return 0;
}
