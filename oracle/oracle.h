/* CPU oracle for the matrix-free hp-FEM operator path of dohp.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it. The product
 * library (dohp_gb300) never links, loads or calls it.
 *
 * Every routine restates the algorithm of the reference source file:line it
 * cites (paths relative to the dohp project root). Plain C99, double precision.
 */
#ifndef DOHP_ORACLE_H
#define DOHP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- 1-D bases and rules (src/jacobi/impls/tensor/polylib.c, tensor.c) ---- */
void or_gauss(int n, double *x, double *w);   /* Gauss-Legendre, ascending (polylib zwgj, alpha=beta=0) */
void or_lobatto(int n, double *x, double *w); /* Gauss-Lobatto-Legendre, ascending (polylib zwglj) */
/* TensorBasisCreate (src/jacobi/impls/tensor/tensor.c:22-109): P GLL nodes, Q rule points.
 * interp/deriv are [Q][P] row-major; node/weight are the GLL nodes/weights. */
int or_tensor_basis(int P, int Q, const double *rcoord, double *interp, double *deriv, double *node, double *weight);
/* TensorGetRule (src/jacobi/quadrature/impls/tensor/tensorquad.c:51-118).
 * method: 0 FAST, 1 SPARSE, 2 SELF; family: 0 Gauss-Legendre, 1 Gauss-Lobatto.
 * Returns the rule size, or -1 on error. x/w need room for the size (<= 100). */
int or_rule_1d(int method, int family, int order, double *x, double *w);
/* dRulePatchSetup_Tensor (tensorquad.c:120-169): patch index/weight tables for a 3-D tensor rule
 * of sizes Q[3]; returns npatches, writes patchsize; ind/weight sized Q0*Q1*Q2. The weight table
 * keeps the reference's z-weight index (weight[jelem] for z). */
int or_rule_patches(int method, const int Q[3], const double *w0, const double *w1, const double *w2,
                    int *patchsize, int *ind, double *weight);

/* ---------------- element kernels (src/jacobi/impls/tensor/efstopo.c, inlinetmulthex.h) ---- */
#define OR_INTERP 40001
#define OR_INTERP_TRANSPOSE 40002
#define OR_GRAD 40003
#define OR_GRAD_TRANSPOSE 40004
#define OR_INSERT 1
#define OR_ADD 2
/* TensorMult_Hex_nounroll (inlinetmulthex.h:19-100) */
void or_tensor_mult_hex(int D, const int P[3], const int Q[3], const double *A[3], const double *in, double *out, int imode);
/* dEFSApply_Tensor_Hex (efstopo.c:368-423) for basis tables b (interp, deriv per direction). */
int or_efs_apply_hex(const int P[3], const int Q[3], const double *interp[3], const double *deriv[3],
                     const double *jinv, int D, const double *in, double *out, int amode, int imode);
/* dGeomInvert3 (include/dohpgeom.h:57-79) */
void or_invert3(const double a[9], double b[9], double *det);
/* Modal (P-discontinuous) hexahedral bases (src/jacobi/impls/modal/modal.c:15-240, modaltopo.c:73-126):
 * mode count of an order (0..3), tables interp [Q][P] / deriv [Q][P][3] at rcoord [Q][3] (returns P),
 * and the element apply (INTERP, INTERP_TRANSPOSE, GRAD; jinv unused, as the reference). */
int or_modal_count(int order);
int or_modal_basis(int order, int Q, const double *rcoord, double *interp, double *deriv);
int or_modal_apply(int P, int Q, const double *interp, const double *deriv, int D, const double *in, double *out,
                   int amode, int imode);
/* dEFSGetExplicitSparse_Tensor_Hex (efstopo.c:660-717); cjinv indexed as the reference does. */
int or_explicit_sparse_hex(int px, int py, int pz, int npatches, int Q, const int *qidx, const double *cjinv,
                           int eoffset, int *P, int *eidx, double *interp, double *deriv);

/* dEFSGetExplicitSparse for a tensor hex EFS: the Q1 sub-cell path when the patches match the GLL
 * sub-cells (efstopo.c:668-671), else the dense _Basic fallback (jacobi.c:611-643). */
int or_explicit_sparse(const int P3[3], const int Q3[3], const double *interp[3], const double *deriv[3],
                       int npatches, int Q, const int *qidx, const double *cjinv, int eoffset,
                       int *P, int *eidx, double *ointerp, double *oderiv);

/* ---------------- structured block mesh + function space ---------------- */
typedef struct or_fs or_fs;
/* Block mesh with nx*ny*nz vertices on box[6]={x0,x1,y0,y1,z0,z1} following the entity creation order of
 * dMeshGenerateBlock (src/fs/mesh/interface/genblock.c:206-402). Interior vertices are moved by
 * U[-perturb*h, perturb*h] per coordinate, drawn from splitmix64(seed) in vertex order.
 * elem_degree: NULL for uniform `degree`, else one isotropic degree per element (region order).
 * dirichlet_mask: bit0 = NEUMANN_SET 100 (walls), bit1 = 200 (top), bit2 = 300 (bottom).
 * Returns NULL on error (message via or_last_error). */
or_fs *or_fs_create(int nx, int ny, int nz, const double box[6], double perturb, uint64_t seed,
                    int degree, const int *elem_degree, int bs, int dirichlet_mask);
void or_fs_destroy(or_fs *fs);
/* The same space on a mesh given by its entities (vertices [nv][3], edges [ne][2], quadrilaterals [nf][4], hexahedra
 * [nr][8] in ITAPS order, each in creation order; the hand-built meshes of src/fs/tests/ex1.c, cunit.c, fsex4.c):
 * adjacency by vertex matching, no boundary sets. */
or_fs *or_fs_create_conn(int nv, const double *vtx, int ne, const int *econn, int nf, const int *fconn, int nr,
                         const int *hconn, int degree, const int *elem_degree, int bs);
/* adjoff [nents+1]; adjind / adjperm as dMeshGetAdjacency (mesh.c:1074-1191) */
const int32_t *or_fs_adjacency(const or_fs *fs, const int32_t **adjind, const int32_t **adjperm);
const char *or_last_error(void);
/* sizes: [0]=nelem [1]=n explicit nodes [2]=nc closure nodes [3]=nexp expanded nodes [4]=bs
 *        [5]=nverts [6]=nedges [7]=nfaces */
void or_fs_sizes(const or_fs *fs, int64_t out[8]);
const int32_t *or_fs_emap(const or_fs *fs);        /* expanded node -> closure node (one 1.0 per row of E); < -1 marks an interpolated row */
/* E as CSR (rows = expanded nodes, columns ascending); returns nnz. With per-element degrees, rows of element
 * nodes on lower-degree faces/edges interpolate that entity's polynomial (extension; the reference errors). */
int64_t or_fs_ecsr(const or_fs *fs, const int64_t **eptr, const int32_t **ecol, const double **eval);
const int32_t *or_fs_xstart(const or_fs *fs);      /* element offsets in expanded nodes, nelem+1 */
const int32_t *or_fs_elem_degree(const or_fs *fs); /* per element degree (x,y,z) triples */
const double *or_fs_coords_expanded(const or_fs *fs); /* [nelem][8][3] in tensor vertex order */
const double *or_fs_vertex_coords(const or_fs *fs);   /* [nverts][3] */
/* replace the vertex coordinates (same topology; a mesh morph), the expanded coordinates follow */
void or_fs_set_vertex_coords(or_fs *fs, const double *vx);
/* entity ordering (ordered set), per entity index arrays of length nents */
void or_fs_entity_info(const or_fs *fs, int32_t *ordered, int32_t *goffset, int32_t *gcoffset, int32_t *inodes);

/* dFSGlobalToExpanded (src/fs/interface/fs.c:543-586): g has n*bs, dcache (nc-n)*bs or NULL (zeros) */
void or_fs_global_to_expanded(const or_fs *fs, const double *g, const double *dcache, double *x);
/* dFSExpandedToGlobal (fs.c:592-640): closure = E^T x; g = explicit part (add=0 insert, 1 add) */
void or_fs_expanded_to_global(const or_fs *fs, const double *x, double *g, int add);

/* Matrix-free operator (EllipShellMatMult src/fs/tests/ellip.c:442-472 with p=2,
 * ElastShellMatMult src/fs/tests/elast.c:311-341 at F=I).
 * kind 0: scalar diffusion, dv = w det k du (k per FAST qpt, NULL -> 1)
 * kind 1: p-Laplacian Jacobian with stash [eta, sqrt_mdeta_Du[3]] per qpt (ellip.c:369-377)
 * kind 2: linear elasticity, lambda/mu in param[0..1] (elast.c:227-280 at F=I)
 * kind 3: mass, v = w u (the right-hand side of ex1.c:399-430 and of configuration 1)
 * kind 4: St. Venant-Kirchhoff function at the state g (ElastPointwiseFunction, elast.c:256-266, no body force)
 * kind 5: St. Venant-Kirchhoff Jacobian at the stashed deformation gradients qdata [nq][9] (elast.c:268-280)
 * kind 6: p-Laplacian function, param = {p, eps} (EllipPointwiseFunction, ellip.c:355-367, lambda = 0, no forcing)
 * kind 7: the same with the Bratu term, param = {p, eps, lambda}: v = -w lambda e^u (ellip.c:341, 363)
 * kind 8: p-Laplacian Jacobian with the Bratu term at the store qdata [nq][5] = {eta, sqrt(-eta') Du, lambda e^u}
 *         (EllipPointwiseJacobian, ellip.c:370-377)
 * nthreads: OpenMP threads over element ranges (the reference runs one MPI rank per core). */
int or_operator_apply(const or_fs *fs, int kind, const double *qdata, const double *param,
                      const double *g, double *y, int nthreads);
/* EllipFunction / ElastFunction (ellip.c:407-440, elast.c:282-309) in full: kind 6 or 4 at the state g expanded
 * dFS_INHOMOGENEOUS with the Dirichlet values dcache ([nc - n][bs], NULL = 0), the body force fq [nq][bs] at the
 * points of or_fs_qpt_coords (NULL = 0) entering as v = -w f */
int or_operator_function(const or_fs *fs, int kind, const double *param, const double *g, const double *dcache,
                         const double *fq, double *y, int nthreads);
/* Number of FAST quadrature points over all elements and per-element offsets (nelem+1). */
int64_t or_fs_num_qpts(const or_fs *fs, int32_t *qoffset);
/* Physical coordinates of FAST quadrature points [nq][3] (coordinate-FS INTERP). */
void or_fs_qpt_coords(const or_fs *fs, double *xq);
/* the field of g (+ Dirichlet values dcache, NULL = 0) at those points: u [nq][bs], physical du [nq][bs][3], jw [nq];
 * rule_deg > 0: at the FAST rule of that degree instead (the points of another space on the same mesh) */
int or_fs_eval_points(const or_fs *fs, int rule_deg, const double *g, const double *dcache, double *u, double *du, double *jw);
/* p-Laplacian residual stash (ellip.c:333-367) from the global state g (homogeneous Dirichlet):
 * writes [eta, sqrt_mdeta_Du[3]] per FAST qpt. */
int or_plap_stash(const or_fs *fs, double p, double eps, const double *g, double *stash);
int or_plap_stash_mt(const or_fs *m, double p, double eps, const double *g, double *stash, int nthreads);

/* Q1-embedded preconditioner assembly (EllipJacobian ellip.c:474-536 with the SPARSE rule, and the
 * elasticity analogue elast.c:343-407), into CSR over explicit scalar dofs (n*bs rows).
 * kcoef_fn: 0 -> k=1, 1 -> k from random Fourier features (or_grf_eval); quirk=1 reproduces
 * the reference's element-natural cjinv indexing (efstopo.c:700), 0 uses the patch point.
 * Returns nnz; rowptr has n*bs+1 entries (caller-allocated), col/val are malloc'd (free with or_free). */
int64_t or_q1_assemble(const or_fs *fs, int kind, const double *param, const double *grf, int quirk,
                       int32_t *rowptr, int32_t **col, double **val);
/* p-Laplacian Jacobian at the state g (homogeneous Dirichlet), exponent p, regularisation eps:
 * EllipJacobian (ellip.c:474-536), store at every SPARSE point (ellip.c:333-342). */
int64_t or_q1_assemble_plap(const or_fs *fs, double p, double eps, const double *g, int quirk,
                            int32_t *rowptr, int32_t **col, double **val);
/* the same at a state whose closure carries the Dirichlet values dcache [nc - n] (EllipJacobian's
 * dFS_INHOMOGENEOUS expansion) */
int64_t or_q1_assemble_plap_dir(const or_fs *fs, double p, double eps, const double *g, const double *dcache, int quirk,
                                int32_t *rowptr, int32_t **col, double **val);
void or_free(void *p);

/* ---------------- facet rules and boundary integrals ---------------- */
/* dQuadratureGetFacetRules_Tensor_Private (src/jacobi/quadrature/impls/tensor/tensorquad.c:309-355) with the node
 * map of dRuleGetNodeWeight_Transformed (tensorquad.c:224-242): the 1-D rule of `order` squared (X slowest) on side
 * `side` (0 y=-1, 1 x=+1, 2 y=+1, 3 x=-1, 4 z=-1, 5 z=+1). nodes [n][3], weights [n]; returns n or -1. */
int or_facet_rule(int side, int method, int order, double *nodes, double *weights);
/* faces of the weak sets (bit0 100, bit1 200, bit2 300) in (region, side) order; returns the number of FAST facet
 * points ((p+1)^2 per face); fel/fside [nfacets], qoff [nfacets+1] optional */
int64_t or_facet_count(const or_fs *fs, int weak_mask, int64_t *nfacets, int32_t *fel, int32_t *fside, int32_t *qoff);
/* per facet point: jw = w |t_X x t_Y|, physical x, outward unit normal, and the field of g (homogeneous
 * Dirichlet; NULL = 0) evaluated with the whole element basis at the point */
int or_facet_points(const or_fs *fs, int weak_mask, const double *g, double *jw, double *x, double *nrm, double *u);
/* y (+)= E^T sum_q phi(xi_q) v_q over the facet points (add = 0 insert, 1 add) */
int or_facet_commit(const or_fs *fs, int weak_mask, const double *v, double *y, int add);

/* ---------------- Stokes (src/fs/tests/stokes.c) ---------------- */
/* Coupled and block applies of the Stokes Jacobian on a velocity space fu (bs 3, degree k) and a pressure space fp
 * (bs 1, degree k - codim, no Dirichlet sets) of the same mesh, at the velocity FAST rule: mode 0 A (viscous block
 * with the penalty nu/(1-2nu)), 1 Bt (pressure -> velocity), 2 B (velocity -> pressure), 3 coupled [A Bt; B 0]
 * without penalty, 4 the nonlinear function [eta(Du) Du - p I; -div u] (the state is xu itself, forcing left to
 * the caller's right-hand side). rheo = {B, eps, p, nu}; the viscosity store of modes 0-3 comes from the velocity
 * state su (NULL: zero). */
int or_stokes_apply(const or_fs *fu, const or_fs *fp, int mode, const double rheo[4], const double *su, const double *xu,
                    const double *xp, double *yu, double *yp);
/* the full nonlinear function (mode 4 with the reference's forcing terms and inhomogeneous Dirichlet velocity
 * values): udir [nc - n][3] (NULL = 0), fq [nq][3] and fpq [nq] at the points of or_fs_qpt_coords (NULL = 0) */
int or_stokes_function(const or_fs *fu, const or_fs *fp, const double rheo[4], const double *xu, const double *udir,
                       const double *xp, const double *fq, const double *fpq, double *yu, double *yp);
/* modes 0-3 at a velocity state su whose closure carries the Dirichlet values sudir [nc - n][3] */
int or_stokes_apply_state(const or_fs *fu, const or_fs *fp, int mode, const double rheo[4], const double *su, const double *sudir,
                          const double *xu, const double *xp, double *yu, double *yp);

/* deformation gradient F = I + Du [nq][9] at every FAST point of the state g (bs = 3, homogeneous Dirichlet;
 * ElastPointwiseComputeStore, elast.c:224-225) */
int or_elast_state(const or_fs *fs, const double *g, double *Fq);

/* Lognormal coefficient field: g(x) = sqrt(2 var / nf) sum_f cos(w_f . x + b_f) (random Fourier
 * features of the squared-exponential kernel, Rahimi & Recht 2007). grf = [nf, var, ell, w(3nf), b(nf)] */
int or_grf_make(int nf, double var, double ell, uint64_t seed, double *grf);
double or_grf_eval(const double *grf, const double x[3]);

/* CSR helpers and Krylov (PETSc KSP replacements; no reference source) */
void or_csr_mult(int64_t nrows, const int32_t *rowptr, const int32_t *col, const double *val, const double *x, double *y);
/* Preconditioned CG on the matrix-free operator with a Chebyshev-Jacobi smoother on the Q1 CSR.
 * Returns iterations (negative on failure); rnorm receives the final relative residual. */
int or_cg_solve(const or_fs *fs, int kind, const double *qdata, const double *param,
                const int32_t *rowptr, const int32_t *col, const double *val, int cheb_degree,
                const double *b, double *x, double rtol, int maxit, double *rnorm, int nthreads);

uint64_t or_splitmix64(uint64_t *state);
double or_uniform(uint64_t *state);

#ifdef __cplusplus
}
#endif
#endif
