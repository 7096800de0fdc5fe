/* A plain-C caller of the C ABI (no Python, no PyTorch): the Poisson problem on an 8^3 perturbed hex mesh, degree 4,
 * homogeneous Dirichlet walls, a seeded right-hand side; the matrix-free operator (EllipShellMatMult), the
 * Q1-embedded preconditioning matrix (EllipJacobian), CG with Chebyshev(3)-Jacobi on it to rtol 1e-8, then the true
 * residual with the operator. The way a dohp caller would drive the library from C, with device vectors from the CUDA
 * runtime. Prints one line: "its=<n> rnorm=<r> true=<t>"; exits 0 only if the solve reached the tolerance. */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "dohp_gb300.h"

#define CHK(call)                                                   \
  do {                                                              \
    if ((call) != 0) {                                              \
      fprintf(stderr, "%s failed: %s\n", #call, dGetLastError());   \
      return 1;                                                     \
    }                                                               \
  } while (0)
#define CU(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      fprintf(stderr, "%s failed: %s\n", #call, cudaGetErrorString(e_));               \
      return 1;                                                                       \
    }                                                                                 \
  } while (0)

/* splitmix64: the seeded right-hand side */
static double uniform(uint64_t *state) {
  uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

int main(void) {
  const dInt npoints[3] = {9, 9, 9};
  const dReal box[6] = {0, 1, 0, 1, 0, 1};
  dMesh mesh;
  dJacobi jac;
  dFS fs;
  CHK(dMeshCreateBlock(npoints, box, 0.1, 1, &mesh));
  CHK(dJacobiCreate(&jac));
  CHK(dFSCreate(mesh, jac, &fs));
  CHK(dFSSetDegree(fs, 4, NULL));
  CHK(dFSSetBlockSize(fs, 1));
  CHK(dFSRegisterBoundary(fs, 100, dFSBSTATUS_DIRICHLET));
  CHK(dFSRegisterBoundary(fs, 200, dFSBSTATUS_DIRICHLET));
  CHK(dFSRegisterBoundary(fs, 300, dFSBSTATUS_DIRICHLET));
  CHK(dFSSetUp(fs));
  dInt n, nc, nexp, bs, nelem;
  CHK(dFSGetSizes(fs, &n, &nc, &nexp, &bs, &nelem));

  dOperator op;
  dMat J;
  dKSP ksp;
  CHK(dFSCreateOperator(fs, dOP_DIFFUSION, NULL, &op));
  CHK(dFSCreateMatrix(fs, &J));
  CHK(dFSAssembleQ1(fs, J, dOP_DIFFUSION, NULL, NULL, 1));
  CHK(dKSPCreate(op, J, dKSP_CG, dPC_CHEBYSHEV_Q1, &ksp));

  double *hb = (double *)malloc(sizeof(double) * n), *hr = (double *)malloc(sizeof(double) * n);
  uint64_t state = 2024;
  for (dInt i = 0; i < n; i++) hb[i] = uniform(&state);
  double *b, *x, *r;
  CU(cudaMalloc((void **)&b, sizeof(double) * n));
  CU(cudaMalloc((void **)&x, sizeof(double) * n));
  CU(cudaMalloc((void **)&r, sizeof(double) * n));
  CU(cudaMemcpy(b, hb, sizeof(double) * n, cudaMemcpyHostToDevice));
  CU(cudaMemset(x, 0, sizeof(double) * n));

  dInt its = 0;
  dReal rnorm = 0;
  CHK(dKSPSolve(ksp, b, x, 1e-8, 1000, &its, &rnorm));
  CHK(dOperatorMult(op, x, r));  /* the true residual b - A x, on the host */
  CU(cudaMemcpy(hr, r, sizeof(double) * n, cudaMemcpyDeviceToHost));
  double rr = 0, bb = 0;
  for (dInt i = 0; i < n; i++) rr += (hb[i] - hr[i]) * (hb[i] - hr[i]), bb += hb[i] * hb[i];
  const double t = sqrt(rr / bb);
  printf("n=%d its=%d rnorm=%.3e true=%.3e\n", (int)n, (int)its, rnorm, t);

  cudaFree(b), cudaFree(x), cudaFree(r), free(hb), free(hr);
  CHK(dKSPDestroy(&ksp));
  CHK(dMatDestroy(&J));
  CHK(dOperatorDestroy(&op));
  CHK(dFSDestroy(&fs));
  CHK(dJacobiDestroy(&jac));
  CHK(dMeshDestroy(&mesh));
  return rnorm <= 1e-8 && t <= 1.01e-8 ? 0 : 2;
}
