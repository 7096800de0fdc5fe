/* dohp_gb300: GB300-native matrix-free hp-FEM operator path with dohp's C API.
 *
 * Drop-in boundary for dohp callers (PETSc SNES/KSP shell operators and the dRulesetIterator element
 * loop). Every entry point returns dErr (0 = success); on failure dGetLastError() describes the error.
 * Vectors are plain device pointers (CUDA global memory) unless the name says Host. Each dFS owns one
 * CUDA stream (default: the legacy default stream); all work of a call is ordered on that stream.
 *
 * Layouts (as in dohp):
 *   global vector   : n explicit nodes x bs, node-major, components interleaved
 *   closure vector  : [global | Dirichlet nodes] x bs (VecDohp closure, src/vec/vecd.c:28-159)
 *   expanded vector : per element, (P0*P1*P2) nodes x bs, element-natural node order
 *                     ((i*P1 + j)*P2 + k, i along x slowest, k along z fastest)
 *
 * Reference locations are relative to the dohp project root.
 */
#ifndef DOHP_GB300_H
#define DOHP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int dErr;
typedef int32_t dInt;
typedef double dReal;
typedef double dScalar;

/* include/dohpjacobi.h:101-108 */
typedef enum {
  dAPPLY_INTERP = 40001,
  dAPPLY_INTERP_TRANSPOSE,
  dAPPLY_GRAD,
  dAPPLY_GRAD_TRANSPOSE,
  dAPPLY_SYMGRAD,
  dAPPLY_SYMGRAD_TRANSPOSE
} dApplyMode;
/* PETSc InsertMode values */
typedef enum { NOT_SET_VALUES = 0, INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
/* include/dohpfs.h:49 */
typedef enum { dFS_HOMOGENEOUS, dFS_INHOMOGENEOUS } dFSHomogeneousMode;
/* include/dohpjacobi.h:141-148 */
typedef enum { dQUADRATURE_METHOD_FAST, dQUADRATURE_METHOD_SPARSE, dQUADRATURE_METHOD_SELF } dQuadratureMethod;
/* include/dohpjacobi.h:223: point family of the tensor quadrature's rules (dQuadratureTensorSetGaussFamily) */
typedef enum { dGAUSS_LEGENDRE, dGAUSS_LOBATTO, dGAUSS_RADAU } dGaussFamily;
/* include/dohpjacobi.h:134-136, 211-217: dJacobi types and the families of the modal type */
#define dJACOBI_TENSOR "tensor"
#define dJACOBI_MODAL "modal"
typedef enum {
  dJACOBI_MODAL_P_CONFORMING,
  dJACOBI_MODAL_P_DISCONTINUOUS,
  dJACOBI_MODAL_Q_CONFORMING,
  dJACOBI_MODAL_Q_DISCONTINUOUS
} dJacobiModalFamily;
/* include/dohpfs.h:41-47: the reference's values (the low 16 bits hold a count of strongly enforced dofs, unused
 * here). DIRICHLET removes the set's nodes from the global space; WEAK puts its faces in the facet iterator. */
typedef enum {
  dFSBSTATUS_INTERIOR = 0,
  dFSBSTATUS_DIRICHLET = (0xffff + 1) << 0,
  dFSBSTATUS_WEAK = (0xffff + 1) << 1
} dFSBStatus;

/* include/dohptype.h:84-86: entity topologies (the element loop and the rules handle dTOPO_HEX) */
typedef enum {
  dTOPO_POINT, dTOPO_LINE, dTOPO_POLYGON, dTOPO_TRIANGLE, dTOPO_QUAD, dTOPO_POLYHEDRON, dTOPO_TET, dTOPO_HEX,
  dTOPO_PRISM, dTOPO_PYRAMID, dTOPO_SEPTAHEDRON, dTOPO_ALL
} dEntTopology;
/* include/dohpjacobi.h:51-81: a polynomial order in 3-D, four bytes {max, x, y, z}; a zero direction takes max */
typedef union {
  struct {
    unsigned char max, x, y, z;
  } s;
  int padding_;
} dPolynomialOrder;
static inline dPolynomialOrder dPolynomialOrderCreate(dInt max, dInt x, dInt y, dInt z) {
  dPolynomialOrder o;
  o.s.max = (unsigned char)max, o.s.x = (unsigned char)x, o.s.y = (unsigned char)y, o.s.z = (unsigned char)z;
  return o;
}
static inline dInt dPolynomialOrder1D(dPolynomialOrder o, dInt dir) {
  const dInt d = dir == 0 ? o.s.x : dir == 1 ? o.s.y : dir == 2 ? o.s.z : 0;
  return d ? d : o.s.max;
}
/* include/dohpjacobi.h:79-83: the total order (max, or x + y + z when larger) */
static inline dInt dPolynomialOrderMax(dPolynomialOrder o) {
  const dInt xyz = (dInt)o.s.x + o.s.y + o.s.z;
  return o.s.max > xyz ? (dInt)o.s.max : xyz;
}

typedef struct _p_dJacobi *dJacobi;
typedef struct _p_dQuadrature *dQuadrature;
typedef struct _p_dRule *dRule;
typedef struct _p_dEFS *dEFS;
typedef struct _p_dMesh *dMesh;
typedef struct _p_dFS *dFS;
typedef struct _p_dOperator *dOperator;
typedef struct _p_dMat *dMat;
typedef struct _p_dRulesetIterator *dRulesetIterator;
typedef struct _p_dKSP *dKSP;
typedef struct _p_dFacetIterator *dFacetIterator;
typedef struct _p_dStokes *dStokes;

/* Operator (pointwise q-function) kinds of the fused matrix-free apply */
typedef enum {
  dOP_DIFFUSION = 0,      /* EllipPointwiseJacobian with p=2 (src/fs/tests/ellip.c:369-377): dv = k w det(J) grad u */
  dOP_PLAPLACE_JACOBIAN = 1, /* EllipPointwiseJacobian with the residual stash (ellip.c:333-377) */
  dOP_ELASTICITY = 2      /* ElastPointwiseJacobian at F = I (src/fs/tests/elast.c:256-280), bs = 3 */
} dOperatorKind;
/* arithmetic of operator applies and of the Chebyshev-Jacobi preconditioner: FP64; FP32 (factors, inputs and
 * arithmetic in FP32); BF16 (geometric factors, inputs, basis tables and Q1 values stored in BF16, FP32
 * arithmetic and accumulation; scalar uniform-order operators); FF (float-float: each value a pair of FP32
 * words, unit roundoff ~2^-48, FP32 exponent range; the apply's arithmetic on the FP32 pipe with FP64-class
 * accuracy, FP64 input and restriction; operator applies only) */
typedef enum { dPREC_FP64 = 0, dPREC_FP32 = 1, dPREC_BF16 = 2, dPREC_FF = 3 } dPrecision;
/* Launch form of an operator apply: DEFAULT = one fused kernel for uniform-order spaces (per-order form for
 * hp spaces); PER_ORDER = one launch per order bucket; PERSISTENT = one launch over all buckets with a device
 * work counter; GRAPH = the persistent launch and the restriction replayed from a CUDA graph. */
typedef enum { dLAUNCH_DEFAULT = 0, dLAUNCH_PER_ORDER = 1, dLAUNCH_PERSISTENT = 2, dLAUNCH_GRAPH = 3 } dLaunchMode;

const char *dGetLastError(void);

/* ---------------------------------------------------------------- dJacobi / dEFS (src/jacobi) */
/* dJacobiCreate (src/jacobi/interface/jacobi.c) with the tensor (GLL nodal) type */
dErr dJacobiCreate(dJacobi *jac);
dErr dJacobiDestroy(dJacobi *jac);
/* dJacobiSetType / dJacobiGetType (src/jacobi/interface/jacobi.c:42-70): dJACOBI_TENSOR (the default: GLL nodal
 * tensor-product bases) or dJACOBI_MODAL (P-discontinuous modal bases of orders 0..3 on hexahedra,
 * src/jacobi/impls/modal/modal.c); another name is an error. The type decides what dJacobiGetEFS makes; element
 * spaces already made stay valid. A dFS needs the tensor type (its spaces are continuous). */
dErr dJacobiSetType(dJacobi jac, const char *type);
dErr dJacobiGetType(dJacobi jac, const char **type);
/* dJacobiModalSetFamily (modal.c:273-281, 413-418): only dJACOBI_MODAL_P_DISCONTINUOUS is built; another family is
 * an error on a modal dJacobi. On a tensor dJacobi the call does nothing, as the reference's PetscTryMethod. */
dErr dJacobiModalSetFamily(dJacobi jac, dJacobiModalFamily family);
/* dJacobiGetNodeCount (include/dohpjacobi.h:183, src/jacobi/interface/jacobi.c:254-264): per entity of topology top[i]
 * and degree deg[i], its interior nodes inode[i] and expanded nodes xnode[i] (either may be NULL). Tensor type:
 * prod max(0, p_d - 1) and prod (p_d + 1) over the entity's directions (tensor.c:249-281); modal type: the modes of
 * the total order for both (hexahedra). */
dErr dJacobiGetNodeCount(dJacobi jac, dInt count, const dEntTopology top[], const dPolynomialOrder deg[], dInt inode[], dInt xnode[]);
/* release an array the library allocated for the caller (dQuadratureGetRules, dJacobiGetEFS), as dohp's dFree */
dErr dFree(void *ptr);
/* dJacobiGetQuadrature (include/dohpjacobi.h:170, src/jacobi/interface/jacobi.c:268-285): the dJacobi's quadrature
 * for a method, made on first request and owned by the dJacobi */
dErr dJacobiGetQuadrature(dJacobi jac, dQuadratureMethod method, dQuadrature *quad);
/* dQuadratureGetRules (src/jacobi/interface/quadrature.c:17-29): *rules = a new array (dFree) of n rules integrating
 * order[i] exactly on the reference hex (tensorquad.c:51-118: FAST n = 1 + order/2 Gauss points, SPARSE two Gauss
 * points per GLL sub-interval, SELF Lobatto); the rules themselves are owned by the quadrature. Hexahedra only. */
dErr dQuadratureGetRules(dQuadrature quad, dInt n, const dEntTopology topo[], const dPolynomialOrder order[], dRule **rules);
/* dQuadratureTensorSetGaussFamily (tensorquad.c:446-462, rule sizes 51-118): the point family of the rules this
 * quadrature makes from now on. FAST: Gauss-Legendre (default, 1 + order/2 points) or Gauss-Lobatto (2 + order/2
 * points); SPARSE: two Gauss-Legendre or two Lobatto (end) points per GLL sub-interval; SELF rules are Lobatto for
 * either family. Radau is an error. Rules made before the call keep their family. The rulesets of a dFS are
 * Gauss-Legendre (dFSGetPreferredQuadratureRuleSet refuses a dJacobi whose quadrature was set otherwise). */
dErr dQuadratureTensorSetGaussFamily(dQuadrature quad, dGaussFamily family);
/* dRuleGetSize / dRuleGetNodeWeight / dRuleGetTensorNodeWeight (include/dohpjacobi.h:186-189): host arrays; nodes
 * [n][3] and weights [n] in tensor order (x slowest); the 1-D tables are owned by the rule */
dErr dRuleGetSize(dRule rule, dInt *dim, dInt *nnodes);
dErr dRuleGetNodeWeight(dRule rule, dReal *coord, dReal *weight);
dErr dRuleGetTensorNodeWeight(dRule rule, dInt *dim, dInt nnodes[3], const dReal *coord[3], const dReal *weight[3]);
/* dRuleGetPatches (src/jacobi/interface/jacobi.c:320-330, tensorquad.c:120-169): SPARSE rules tiled into 2 x 2 x 2 point
 * patches, other rules one patch; ind [npatches][patchsize] element-natural point indices; weights as the reference
 * tabulates them (its z factor is the y rule's weight at the y index; no computation uses them). Owned by the rule. */
dErr dRuleGetPatches(dRule rule, dInt *npatches, dInt *patchsize, const dInt **ind, const dReal **weight);
/* dRuleComputePhysical (src/jacobi/interface/jacobi.c:383-414): jinv [n][9] = jac^-1 (dGeomInvert3), jw [n] = w det jac;
 * jac NULL gives identities and the rule weights; a negative determinant is an error. Host arrays. */
dErr dRuleComputePhysical(dRule rule, const dScalar jac[], dReal jinv[], dReal jw[]);
/* dJacobiGetEFS (include/dohpjacobi.h:169): *efs = a new array (dFree) of n element spaces, basis degrees order[i] on
 * rules[i]; the dEFS objects are cached and owned by the dJacobi. Hexahedra only. */
dErr dJacobiGetEFS(dJacobi jac, dInt n, const dEntTopology topo[], const dPolynomialOrder order[], const dRule rules[], dEFS **efs);
/* the same for one hex from plain arrays (basis degree and rule order per direction) */
dErr dJacobiGetEFSTensor(dJacobi jac, const dInt degree[3], dQuadratureMethod method, const dInt rule_order[3], dEFS *efs);
/* dEFSGetRule (include/dohpjacobi.h:176) */
dErr dEFSGetRule(dEFS efs, dRule *rule);
/* dEFSGetExplicitSparse (include/dohpjacobi.h:181, src/jacobi/interface/jacobi.c:592-643): explicit bases of npatches
 * patches of Q points each (qidx [npatches][Q]: the patch points' element-natural indices, dRuleGetPatches): with 8
 * points per patch and the p_x p_y p_z GLL sub-cells as patches, the Q1 sub-cell bases of efstopo.c:660-717 (P = 8,
 * derivatives with respect to the unit sub-cell coordinate mapped by cjinv [pidx*8+q]), otherwise the element's own
 * basis at each patch point (P = nodes of the element, cjinv read at qidx[qidx[pidx*Q+q]] as jacobi.c:620-626 does).
 * cjinv NULL: reference coordinates. A modal element has no sparse form (an error, as jacobi.c:606).
 * Outputs (host): eidx [npatches][P] = eoffset + element node, interp [npatches][Q][P], deriv [npatches][Q][P][3]. */
dErr dEFSGetExplicitSparse(dEFS efs, dInt npatches, dInt Q, const dInt qidx[], const dReal cjinv[], dInt eoffset, dInt *P,
                           dInt eidx[], dReal interp[], dReal deriv[]);
/* dEFSGetExplicit / dEFSRestoreExplicit (include/dohpjacobi.h:179-180, src/jacobi/interface/jacobi.c:508-576): the
 * element basis at the rule points as host arrays *basis [Q][P] and *deriv [Q][P][3], the derivatives mapped by
 * jinv [Q][3][3] (NULL: reference coordinates; a modal basis ignores jinv, as its apply does). Restore releases
 * the arrays and zeroes the outputs. */
dErr dEFSGetExplicit(dEFS efs, const dReal jinv[], dInt *Q, dInt *P, const dReal **basis, const dReal **deriv);
dErr dEFSRestoreExplicit(dEFS efs, const dReal jinv[], dInt *Q, dInt *P, const dReal **basis, const dReal **deriv);
/* dEFSGetSizes (include/dohpjacobi.h:172): dim, interior nodes, total nodes (a modal basis: its modes for both) */
dErr dEFSGetSizes(dEFS efs, dInt *dim, dInt *inodes, dInt *total);
/* dEFSGetTensorNodes (include/dohpjacobi.h:174, src/jacobi/interface/jacobi.c:447-455, efstopo.c:260-290): dim (3),
 * the nodes per direction tsize[3], and pointers (owned by the element space) to its GLL nodes and their weights per
 * direction. mscale / lscale (the reference's tabulated Q1 mass and Laplacian scalings, which no reference caller
 * reads) are not provided: pass NULL (else an error). A modal element: an error, it has no nodes. */
dErr dEFSGetTensorNodes(dEFS efs, dInt *dim, dInt tsize[3], dReal *nodes[3], dReal *weight[3], const dReal *mscale[3],
                        const dReal *lscale[3]);
/* host copies of the basis nodes, rule points and rule weights, concatenated over the three directions (no reference
 * counterpart: the rule's side of dEFSGetTensorNodes and dRuleGetTensorNodeWeight in one call) */
dErr dEFSGetTensorTables(dEFS efs, dInt P[3], dInt Q[3], dReal *basis_nodes, dReal *rule_points, dReal *rule_weights);
/* dEFSApply (include/dohpjacobi.h:177, src/jacobi/impls/tensor/efstopo.c:368-423) for ONE element:
 * device pointers; jinv NULL means reference coordinates (efstopo.c:565-568). On a modal element
 * (src/jacobi/impls/modal/modaltopo.c:73-126): INTERP, INTERP_TRANSPOSE and GRAD (reference-coordinate
 * derivatives, jinv unused), GRAD_TRANSPOSE is an error; values are [P][D] per element for modes, D <= 4096. */
dErr dEFSApply(dEFS efs, const dReal *jinv, dInt D, const dScalar *in, dScalar *out, dApplyMode amode, InsertMode imode);
/* Batched dEFSApply over nelem elements stored back to back (element stride = the mode's in/out size),
 * jinv strided by 9*Q per element (or NULL). stream: cudaStream_t or NULL. */
dErr dEFSApplyBatched(dEFS efs, dInt nelem, const dReal *jinv, dInt D, const dScalar *in, dScalar *out,
                      dApplyMode amode, InsertMode imode, void *stream);

/* ---------------------------------------------------------------- dMesh (src/fs/mesh) */
/* dMeshGenerateBlock (src/fs/mesh/interface/genblock.c:145-521) with npoints vertices per direction on
 * box = {x0,x1,y0,y1,z0,z1}, followed by a seeded perturbation of interior vertices by
 * U[-perturb h, perturb h] per coordinate (splitmix64(seed), vertex order) in place of dMeshMorph. */
dErr dMeshCreateBlock(const dInt npoints[3], const dReal box[6], dReal perturb, uint64_t seed, dMesh *mesh);
/* A hexahedral mesh given by its entities, as a dohp caller builds one through iMesh (src/fs/tests/ex1.c:48-104,
 * cunit.c:76-136, fsex4.c:11-47): vertex coordinates vtx [nv][3], edges econn [ne][2], quadrilaterals fconn [nf][4] and
 * hexahedra hconn [nr][8] (ITAPS vertex order), each in creation order; entities are numbered vertices, edges, faces,
 * regions (dMeshGetAdjacency's toff). Every side of a hexahedron and of a face must be given. Adjacency and
 * orientations as dMeshGetAdjacency (src/fs/mesh/interface/mesh.c:1039-1191). Such a mesh has no boundary sets: a
 * dFS on it has no Dirichlet or weak sets (registering one is an error at dFSBuildSpace), and the block-lattice
 * parts (Q1 multigrid, learned correction) refuse it. DHM files hold its entities (dFSLoadDHM rebuilds it). */
dErr dMeshCreateFromConnectivity(dInt nv, const dReal *vtx, dInt ne, const dInt *econn, dInt nf, const dInt *fconn, dInt nr,
                                 const dInt *hconn, dMesh *mesh);
/* dMeshGetAdjacency (mesh.c:1074-1191, include/dohpmesh.h dMeshAdjacency): toff = the first entity of each type
 * (vertex, edge, face, region, end); adjoff [nents+1], adjind (edges: their 2 vertices; faces: 4 edges; regions:
 * 6 faces, canonical side order), adjperm (orientation of each side). Arrays owned by the mesh. */
dErr dMeshGetAdjacency(dMesh mesh, dInt toff[5], const dInt **adjoff, const dInt **adjind, const dInt **adjperm);
dErr dMeshDestroy(dMesh *mesh);
dErr dMeshGetNumEnts(dMesh mesh, dInt counts[4]); /* vertices, edges, faces, regions */

/* ---------------------------------------------------------------- dFS (src/fs/interface) */
dErr dFSCreate(dMesh mesh, dJacobi jac, dFS *fs);
dErr dFSDestroy(dFS *fs);
/* dFSSetDegree with an isotropic degree tag (dMeshCreateRuleTagIsotropic, mesh.c:978-1023); elem_degree
 * (host, one per region, may be NULL) gives per-element orders for hp spaces. */
dErr dFSSetDegree(dFS fs, dInt degree, const dInt *elem_degree);
dErr dFSSetBlockSize(dFS fs, dInt bs);
/* dFSRegisterBoundary (include/dohpfs.h): boundary set 100 (walls), 200 (top), 300 (bottom) */
dErr dFSRegisterBoundary(dFS fs, dInt setid, dFSBStatus status);
dErr dFSSetStream(dFS fs, void *stream);
/* dFSBuildSpace (src/fs/impls/cont/cont.c:258-385) with natural ordering: host maps only (no device) */
dErr dFSBuildSpace(dFS fs);
/* dFSSetFromOptions analogue: builds the space if needed and uploads maps and geometry to the device */
dErr dFSSetUp(dFS fs);
/* n explicit nodes, nc closure nodes, nexp expanded nodes, bs, nelem */
dErr dFSGetSizes(dFS fs, dInt *n, dInt *nc, dInt *nexp, dInt *bs, dInt *nelem);
/* host copies of the bit-exact maps: E (expanded node -> closure node) and element offsets */
dErr dFSGetExpandedMap(dFS fs, dInt *emap, dInt *xstart);
/* host copy of E as CSR (rows = expanded nodes, columns = closure nodes ascending, values); any output may
 * be NULL. With uniform degree every row is one 1.0 (the reference's Boolean E, cont.c:200-249). With
 * per-element degrees (dFSSetDegree elem_degree), element nodes on lower-degree faces/edges interpolate
 * that entity's polynomial (an extension: the reference errors on p-nonconforming entities, tensor.c:417). */
dErr dFSGetElementAssemblyMatrix(dFS fs, int64_t *nnz, dInt *rowptr, dInt *col, dReal *val);
/* host copy of per-element degrees (3 per element after propagation) */
dErr dFSGetElementDegrees(dFS fs, dInt *deg);
/* dFSCreateExpandedVector / dFSCreateGlobalVector (include/dohpfs.h:77-78): new zeroed device vectors of nexp*bs and
 * n*bs values (PETSc Vec -> device array), released with dVecDestroy */
dErr dFSCreateExpandedVector(dFS fs, dScalar **x);
dErr dFSCreateGlobalVector(dFS fs, dScalar **x);
dErr dVecDestroy(dScalar **x);
/* dFSGetGeometryVectorExpanded (src/fs/interface/fsgeom.c:216-227): device [nelem][8][3] */
dErr dFSGetGeometryVectorExpanded(dFS fs, const dReal **coords);
/* dFSInhomogeneousDirichletCommit (src/fs/interface/fs.c:527-541): cache the Dirichlet part of a closure vector */
dErr dFSInhomogeneousDirichletCommit(dFS fs, const dScalar *closure);
/* dFSGlobalToExpanded (fs.c:543-586) / dFSExpandedToGlobal (fs.c:592-640) on device vectors */
dErr dFSGlobalToExpanded(dFS fs, const dScalar *g, dScalar *x, dFSHomogeneousMode hmode, InsertMode imode);
dErr dFSExpandedToGlobal(dFS fs, const dScalar *x, dScalar *g, dFSHomogeneousMode hmode, InsertMode imode);
/* number of FAST quadrature points over all elements (rule order 2p, fsruleset.c:32-37) */
dErr dFSGetNumQuadraturePoints(dFS fs, int64_t *nq);
/* physical coordinates of the FAST quadrature points, device [nq][3] (caller-allocated) */
dErr dFSGetQuadratureCoordinates(dFS fs, dReal *xq);

/* ---------------------------------------------------------------- matrix-free operator (MatShell) */
/* The matrix-free Jacobian of EllipShellMatMult (src/fs/tests/ellip.c:442-472) or ElastShellMatMult
 * (src/fs/tests/elast.c:311-341) on global vectors with homogeneous Dirichlet conditions.
 * param: elasticity {E, nu} (Lame parameters as ElastSetMaterial, elast.c:62-69); unused otherwise. */
dErr dFSCreateOperator(dFS fs, dOperatorKind kind, const dReal *param, dOperator *op);
dErr dOperatorDestroy(dOperator *op);
/* per-quadrature-point data: dOP_DIFFUSION coefficient k [nq] (NULL: k = 1); dOP_PLAPLACE_JACOBIAN stash
 * [nq][4] = {eta, sqrt(-eta') du} (ellip.c:119-123). Device pointer, copied into the operator. */
dErr dOperatorSetQuadratureData(dOperator op, const dReal *qdata);
/* p-Laplacian stash from the state g (EllipPointwiseComputeStore, ellip.c:333-342), exponent p, eps: the store
 * [nq][4] at every FAST point and the Jacobian's coefficients, so that dOperatorMult then applies
 * EllipShellMatMult (ellip.c:442-472) at g. g is expanded dFS_INHOMOGENEOUS (as EllipFunction does). */
dErr dOperatorComputePLaplaceStash(dOperator op, const dScalar *g, dReal p, dReal eps);
/* EllipFunction (ellip.c:407-440) without the forcing term, lambda = 0: y = sum_e E^T B^T (w eta Du) at the
 * state g; also leaves the stash of g in place (the next dOperatorMult is the Jacobian at g). */
dErr dOperatorPLaplaceFunction(dOperator op, const dScalar *g, dReal p, dReal eps, dScalar *y);
/* St. Venant-Kirchhoff elasticity (dOP_ELASTICITY operators, uniform-order spaces, FP64): the state at g
 * (deformation gradient F = I + Du and second Piola-Kirchhoff stress S at every FAST point,
 * ElastPointwiseComputeStore elast.c:224-225; g expanded dFS_INHOMOGENEOUS as in dOperatorElasticityFunction), after which
 * dOperatorMult applies ElastShellMatMult at that state (ElastPointwiseJacobian, elast.c:268-280); g = NULL returns to
 * F = I (linear elasticity) */
dErr dOperatorElasticityState(dOperator op, const dScalar *g);
/* ElastFunction without body force (elast.c:282-309): y = sum_e E^T B^T (w F S) at g; also sets the state. g is expanded
 * dFS_INHOMOGENEOUS (elast.c:293): Dirichlet nodes take the values of dFSInhomogeneousDirichletCommit (zero without one);
 * the Jacobian applies at that state act on homogeneous increments (ElastShellMatMult, elast.c:322) */
dErr dOperatorElasticityFunction(dOperator op, const dScalar *g, dScalar *y);
/* copy out the per-point data: dOP_DIFFUSION coefficient [nq], dOP_PLAPLACE_JACOBIAN stash [nq][4] (device) */
dErr dOperatorGetQuadratureData(dOperator op, dReal *qdata);
dErr dOperatorSetPrecision(dOperator op, dPrecision prec);
dErr dOperatorSetLaunchMode(dOperator op, dLaunchMode mode);
/* measure tile shapes (elements per block x threads) per order bucket on the next apply; cache_path (may be
 * NULL) is a JSON file read before and written after tuning, keyed by device, kind, order and precision */
dErr dOperatorAutotune(dOperator op, const char *cache_path);
/* current tiles per order bucket (after the first apply): order, elements per block, threads per block */
dErr dOperatorGetTiles(dOperator op, dInt *nbuckets, dInt *order, dInt *cap, dInt *threads);
/* MatMult: y = A x, device vectors of n*bs entries */
dErr dOperatorMult(dOperator op, const dScalar *x, dScalar *y);
/* element part of MatMult: yexp = (per-element q-function apply) E x, expanded device vector of nexp*bs;
 * dFSExpandedToGlobal(yexp) then completes y = A x (the dRulesetIteratorCommitPatchApplied/Finish split) */
dErr dOperatorMultExpanded(dOperator op, const dScalar *x, dScalar *yexp);
/* MatMult that allocates nothing (no counterpart in the reference). For callers that cannot let a library
 * call cudaMalloc/cudaFree while they run: applications that give all device memory to their own pool or
 * arena, and solver callbacks running beside other streams, where cudaMalloc/cudaFree may synchronize
 * the device. Its temporary lives in a fixed 8 MiB device array per GPU (at most 1,048,576 expanded
 * values, nexp*bs); larger spaces are rejected with an error. dOP_DIFFUSION on uniform-order spaces only, and
 * always in FP64: an operator whose precision (dOperatorSetPrecision) is not dPREC_FP64 is refused. Requires one ordinary
 * dOperatorMult call first (after the last dOperatorSetQuadratureData), which builds the geometric factors.
 * The first call on a device looks up the array's device address; make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU race. */
dErr dOperatorMultNoAlloc(dOperator op, const dScalar *x, dScalar *y);
/* MatMult with host vectors: copies in, applies, copies out, synchronizes (end-to-end form) */
dErr dOperatorMultHost(dOperator op, const dScalar *x_host, dScalar *y_host);

/* ---------------------------------------------------------------- dRuleset / dRulesetIterator (batched device form) */
/* include/dohpfs.h:97-128, src/fs/interface/fsruleset.c, fsrulesetit.c. One Start / GetPatchApplied / CommitPatchApplied /
 * Finish cycle covers all elements at once on the device: dRulesetIteratorHasPatch is true once after Start and
 * dRulesetIteratorNextPatch ends the traversal, so the reference's loop
 *     while (dRulesetIteratorHasPatch(it)) { GetPatchApplied; q-function; CommitPatchApplied; NextPatch; }
 * runs its body once, over every point. Arrays are element-natural per element, elements back to back: element e's
 * points start at the ruleset's offset of e (dRulesetGetNumPoints; (p_x+1)(p_y+1)(p_z+1) points per element for FAST
 * rules, the layout of dFSGetNumQuadraturePoints). SPARSE rules (uniform-order spaces): (2p)^3 points per element in
 * tensor order; patch (a, b, c) of the reference's patch loop is the 2 x 2 x 2 block of points (2a..2a+1, 2b..2b+1,
 * 2c..2c+1). Link 0 is the coordinate space, links 1.. the spaces added with dRulesetIteratorAddFS, in order; varargs
 * repeat the per-link arguments for links 1.. exactly as in dohp. */
typedef struct _p_dRuleset *dRuleset;
/* dFSGetPreferredQuadratureRuleSet (include/dohpfs.h:97): the rules of the space's elements (order 2p per direction,
 * fsruleset.c:32-37), FAST or SPARSE, each element with the rule of its own orders; over all regions of the mesh */
dErr dFSGetPreferredQuadratureRuleSet(dFS fs, dQuadratureMethod method, dRuleset *rset);
dErr dRulesetGetSize(dRuleset rset, dInt *size);
/* total points and the host array of per-element point offsets [nelem+1] (owned by the ruleset) */
dErr dRulesetGetNumPoints(dRuleset rset, int64_t *nq, const dInt **qoffset);
dErr dRulesetDestroy(dRuleset *rset);
/* dFSGetCoordinateFS (src/fs/interface/fsgeom.c:176-204): the Q1, block size 3 space of vertex coordinates on the same mesh,
 * owned by fs; its expanded vector is dFSGetGeometryVectorExpanded's [nelem][8][3] */
dErr dFSGetCoordinateFS(dFS fs, dFS *cfs);
/* dFSGetNodalCoordinatesExpanded (src/fs/interface/fsgeom.c:17-58): the coordinates of every expanded node (each
 * element's trilinear map at its GLL nodes), coords [nexp][3]; dFSGetNodalCoordinatesGlobal (fsgeom.c:72-107): every
 * closure node's coordinates (the mean of its expanded copies), coords [nc][3]. coords is a device pointer when
 * on_device, else host memory. After dFSBuildSpace. */
dErr dFSGetNodalCoordinatesExpanded(dFS fs, dReal *coords, int on_device);
dErr dFSGetNodalCoordinatesGlobal(dFS fs, dReal *coords, int on_device);
/* dFSGetSubElementMeshSize / dFSGetSubElementMesh (src/fs/interface/fsgeom.c:257-285, cont.c:387-470): the Q1
 * sub-cell mesh of the space for visualization: p_x p_y p_z hexahedra per element (SPARSE patch order), their
 * vertices the closure nodes (nverts = nc), off [nelems+1], ind [nconn] in ITAPS hexahedron vertex order, topo all
 * dTOPO_HEX. Host arrays; needs a Boolean E (no hp constraint rows). */
dErr dFSGetSubElementMeshSize(dFS fs, dInt *nelems, dInt *nverts, dInt *nconn);
dErr dFSGetSubElementMesh(dFS fs, dInt nelems, dInt nconn, dEntTopology topo[], dInt off[], dInt ind[]);
/* dRulesetCreateIterator (fsrulesetit.c:129-150): link 0 = cfs (coordinates) */
dErr dRulesetCreateIterator(dRuleset rset, dFS cfs, dRulesetIterator *it);
/* dRulesetIteratorAddFS (fsrulesetit.c:161-181): one more field link (same mesh, any degrees on FAST rules) */
dErr dRulesetIteratorAddFS(dRulesetIterator it, dFS fs);
/* dRulesetIteratorSetMode (fsrulesetit.c:152-158): INSERT_VALUES (default) or ADD_VALUES for Finish's restriction */
dErr dRulesetIteratorSetMode(dRulesetIterator it, InsertMode imode);
/* dRulesetIteratorAddStash / GetStash (fsrulesetit.c:779-798): device memory of elembytes per element and nodebytes per
 * point (zeroed when made at the next Start, then kept across traversals); GetStash gives the start of each (element e's
 * point stash begins at its point offset times nodebytes) */
dErr dRulesetIteratorAddStash(dRulesetIterator it, dInt elembytes, dInt nodebytes);
dErr dRulesetIteratorGetStash(dRulesetIterator it, void *elemstash, void *nodestash);
/* dRulesetIteratorStart (fsrulesetit.c:234-303): per link (X, [xmode if X], Y, [ymode if Y]); link 0's X is the expanded
 * coordinate vector (NULL: the space's own geometry), the other links' X are global vectors expanded with xmode
 * (dFS_HOMOGENEOUS / dFS_INHOMOGENEOUS) or NULL (zero); Y are global test vectors filled at Finish, or NULL. Device pointers. */
dErr dRulesetIteratorStart(dRulesetIterator it, const dScalar *X, ...);
int dRulesetIteratorHasPatch(dRulesetIterator it);
dErr dRulesetIteratorNextPatch(dRulesetIterator it);
/* dRulesetIteratorGetPatchApplied (fsrulesetit.c:517-589): Q = points; jw [Q]; per link (u, du, v, dv): link 0 gives
 * u = x [Q][3] and du = dx [Q][3][3] (reference gradient of the coordinates), field links u [Q][bs] and du [Q][bs][3]
 * (physical gradient); v [Q][bs] and dv [Q][bs][3] are zeroed test arrays. NULL skips an output (and its work). */
dErr dRulesetIteratorGetPatchApplied(dRulesetIterator it, dInt *Q, const dReal **jw, dScalar **u, dScalar **du, dScalar **v,
                                     dScalar **dv, ...);
/* dRulesetIteratorCommitPatchApplied (fsrulesetit.c:595-643): per link (v, dv) as returned by GetPatchApplied or NULL;
 * integrates v (INTERP_TRANSPOSE) and dv (GRAD_TRANSPOSE) into the link's expanded test vector (imode per element) */
dErr dRulesetIteratorCommitPatchApplied(dRulesetIterator it, InsertMode imode, const dScalar *v, const dScalar *dv, ...);
/* dRulesetIteratorGetPatchAssembly (fsrulesetit.c:657-701), SPARSE rulesets on uniform-order spaces (an error on mixed
 * orders), after GetPatchApplied: per link (P, rowcol,
 * interp, deriv), NULL for link 0: the Q1 sub-cell bases of every patch of every element (dEFSGetExplicitSparse,
 * efstopo.c:660-717, the inverse Jacobian read at the reference's patch-natural index): P = 8, device arrays rowcol
 * [nelem*p^3][8] (expanded node indices), interp [nelem*p^3][8][8], deriv [nelem*p^3][8][8][3], patches element-major in
 * the reference's patch order, owned by the iterator */
dErr dRulesetIteratorGetPatchAssembly(dRulesetIterator it, dInt *P, const dInt **rowcol, const dReal **interp, const dReal **deriv,
                                      ...);
/* dRulesetIteratorFinish (fsrulesetit.c:309-322): restrict each link's expanded test vector into its Y */
dErr dRulesetIteratorFinish(dRulesetIterator it);
dErr dRulesetIteratorDestroy(dRulesetIterator *it);
/* one field on its own preferred ruleset: dFSGetPreferredQuadratureRuleSet + dFSGetCoordinateFS + dRulesetCreateIterator +
 * dRulesetIteratorAddFS(fs) (link 1 = fs) */
dErr dRulesetIteratorCreate(dFS fs, dQuadratureMethod method, dRulesetIterator *it);
/* dNormsStart/Update/Finish (src/util/util.c:110-153) over every point of the last GetPatchApplied, for link 1: uerr =
 * {L1, L2, Linf} of u - exact_u, gerr = the same of |grad u - exact_du| (device arrays [nq][bs], [nq][bs][3],
 * either may be NULL, e.g. exact values computed from the x that GetPatchApplied returned) */
dErr dRulesetIteratorErrorNorms(dRulesetIterator it, const dScalar *exact_u, const dScalar *exact_du, dReal uerr[3],
                                dReal gerr[3]);

/* ---------------------------------------------------------------- facet rules and boundary integrals */
/* dQuadratureGetFacetRules (include/dohpjacobi.h:210; src/jacobi/quadrature/impls/tensor/tensorquad.c:309-355) and
 * dRuleGetNodeWeight_Transformed (tensorquad.c:224-242) for one side of the reference hex: the tensor Gauss rule of
 * the given 1-D order on [-1,1]^2 (X slowest), mapped by xi = R_side (X, Y, 0) + t_side. Sides in the MOAB order
 * 0: y=-1, 1: x=+1, 2: y=+1, 3: x=-1, 4: z=-1, 5: z=+1; R_side's third column is the outward normal.
 * nodes [n][3], weights [n]; room for 81 nodes covers orders up to 16 (FAST). Host only. */
dErr dFSGetFacetRule(dInt side, dQuadratureMethod method, dInt order, dInt *nnodes, dReal *nodes, dReal *weights);
/* dQuadratureGetFacetRules (include/dohpjacobi.h:210, tensorquad.c:309-355) with the reference's arguments: *rules = a
 * new array (dFree) of n facet rules, facet[i] the side of the hex topo[i] (hexahedra only) in the order above, owned by
 * the quadrature: dRuleGetSize gives dim 2 and the face's points, dRuleGetNodeWeight the points on the side in
 * reference coordinates (as dFSGetFacetRule) with their face weights, dRuleGetPatches one patch (FAST) or the 2 x 2
 * blocks (SPARSE). The face orders come from the rows of the side's rotation as in the reference (the same for
 * isotropic orders). dRuleGetTensorNodeWeight and tensor element spaces (dJacobiGetEFS) are refused on them. */
dErr dQuadratureGetFacetRules(dQuadrature quad, dInt n, const dEntTopology topo[], const dInt facet[], const dPolynomialOrder order[],
                              dRule **rules);
/* Batched facet iterator over the faces of the sets registered with dFSBSTATUS_WEAK (the reference's weakFace set,
 * src/fs/interface/fsbuild.c:87-90), the boundary analogue of the dRulesetIterator: FAST rules (p+1 Gauss points
 * per face direction, order 2p as the volume rule), facets in (element, side) order, points X-major per facet.
 * Any space (uniform or per-element orders, bs 1 or 3). */
dErr dFacetIteratorCreate(dFS fs, dQuadratureMethod method, dFacetIterator *it);
dErr dFacetIteratorDestroy(dFacetIterator *it);
/* host arrays owned by the iterator: element and side of each facet, point offsets per facet [nfacets+1] */
dErr dFacetIteratorGetFacets(dFacetIterator it, int64_t *nfacets, const dInt **elem, const dInt **side, const dInt **qoffset);
dErr dFacetIteratorStart(dFacetIterator it, const dScalar *g, dFSHomogeneousMode hmode);
/* device pointers: jw[nq] = w_X w_Y |t_X x t_Y| (area weight), x[nq][3] physical points, normal[nq][3] outward unit
 * normals, u[nq][bs] the field of Start's g at the points; v[nq][bs] is the writable test array (zeroed) */
dErr dFacetIteratorGetApplied(dFacetIterator it, int64_t *nq, const dReal **jw, const dReal **x, const dReal **normal,
                              const dScalar **u, dScalar **v);
/* integrate v back: y_exp[i] (+)= sum_q phi_i(xi_q) v_q over the facet points (v carries the caller's jw) */
dErr dFacetIteratorCommit(dFacetIterator it, InsertMode imode);
/* restrict the expanded boundary vector into y (INSERT_VALUES overwrites, ADD_VALUES adds to a volume residual) */
dErr dFacetIteratorFinish(dFacetIterator it, dScalar *y, InsertMode imode);

/* ---------------------------------------------------------------- mixed velocity-pressure (Stokes) */
/* src/fs/tests/stokes.c: StokesMultMode (stokesimpl.h:34) plus the coupled MatMult_Nest_StokesCoupled */
typedef enum { dSTOKES_MULT_A = 0, dSTOKES_MULT_BT = 1, dSTOKES_MULT_B = 2, dSTOKES_MULT_COUPLED = 3 } dStokesMultMode;
/* StokesCreate / StokesSetFromOptions / StokesGetMatrices (stokes.c:102-130, 160-274, 367-445): fsu the velocity
 * space (bs 3, degree k in 2..6, Dirichlet sets), fsp the pressure space (bs 1, degree k-1 or k-2, no boundary sets)
 * on the same mesh; rheo = {B, eps, p, nu} (struct StokesRheology, stokesimpl.h:9-11; the reference's defaults
 * 1, 1, 2, 0; NULL takes them): viscosity eta = B (eps^2/2 + Du:Du/2)^((p-2)/2) (StokesPointwiseComputeStore,
 * stokes.c:447-453), p > 1; p = 2 is the linear (Newtonian) case. */
dErr dStokesCreate(dFS fsu, dFS fsp, const dReal rheo[4], dStokes *stk);
dErr dStokesDestroy(dStokes *stk);
/* y = [A Bt; B 0] x blocks (StokesShellMatMult_All_IorA stokes.c:579-673, MatMult_Nest_StokesCoupled 541-577):
 * A: xu -> yu (with the penalty nu/(1-2nu)); BT: xp -> yu; B: xu -> yp; COUPLED: (xu, xp) -> (yu, yp) without
 * the penalty. Device vectors; the unused ones may be NULL. With p != 2 the A and COUPLED blocks are the Jacobian
 * at the state of the last dStokesFunction (StokesPointwiseJacobian(_A), stokes.c:476-494; the zero state before
 * one). */
dErr dStokesMult(dStokes stk, dStokesMultMode mode, const dScalar *xu, const dScalar *xp, dScalar *yu, dScalar *yp);
/* StokesFunction (stokes.c:507-540, StokesPointwiseFunction 460-474) without the forcing, which the caller puts in
 * the right-hand side: yu = int eta(Du) Dv:Du - p div v, yp = -int q div u; keeps the store {eta, eta', Du} of
 * (xu, xp) as the state of the Jacobian applies. The velocity is expanded dFS_INHOMOGENEOUS, as StokesFunction
 * does: the Dirichlet nodes take the values committed to fsu by dFSInhomogeneousDirichletCommit (zero when none
 * were); the Jacobian applies act on homogeneous increments (MatMult_Nest_StokesCoupled, stokes.c:556). */
dErr dStokesFunction(dStokes stk, const dScalar *xu, const dScalar *xp, dScalar *yu, dScalar *yp);
/* yp = int q f over the velocity's FAST rule (the rule of the reference's Stokes iterator), f given at its points
 * in the dRulesetIterator order of fsu: the pressure forcing term int q fp of StokesPointwiseFunction as a
 * right-hand side */
dErr dStokesIntegratePressure(dStokes stk, const dScalar *fq, dScalar *yp);
/* the coupled system (the Jacobian at the current state) solved by FGMRES with the block upper triangular (Schur)
 * preconditioner: velocity block one Q1 multigrid V-cycle (Chebyshev-Jacobi where the GLL lattice does not
 * coarsen) on the Q1-embedded viscous matrix, Schur complement -diag(M_p)/eta (the viscosity-scaled pressure
 * mass, stokes.c:742-799), both at the zero-state viscosity; (xu, xp) is the initial guess and the result, xp
 * returned with zero mean */
dErr dStokesSolve(dStokes stk, const dScalar *bu, const dScalar *bp, dScalar *xu, dScalar *xp, dReal rtol, dInt maxit, dInt *its,
                  dReal *rnorm);

/* ---------------------------------------------------------------- Q1-embedded preconditioning matrix */
/* dFSCreateMatrix (src/fs/interface/fs.c:770-813) as a device CSR over explicit scalar dofs; the sparsity is
 * that of the Q1 sub-element grid (symbolic pass on the device). */
dErr dFSCreateMatrix(dFS fs, dMat *J);
dErr dMatDestroy(dMat *J);
/* EllipJacobian (src/fs/tests/ellip.c:474-536): SPARSE rule, Q1 sub-cell bases (efstopo.c:660-717),
 * dFSMatSetValuesBlockedExpanded (fs.c:826-930). kind/param as dFSCreateOperator; coefficient: k at the
 * SPARSE points (NULL: k = 1), reference_quirk = 1 reproduces the reference's inverse-Jacobian indexing. */
dErr dFSAssembleQ1(dFS fs, dMat J, dOperatorKind kind, const dReal *param, const dReal *grf, int reference_quirk);
/* EllipJacobian (ellip.c:474-536): the Q1-embedded p-Laplacian Jacobian at the state g (device vector),
 * store at every SPARSE point from the state's gradient there; scalar uniform-order spaces */
dErr dFSAssembleQ1PLaplace(dFS fs, dMat J, const dScalar *g, dReal p, dReal eps, int reference_quirk);
/* dFSMatSetValuesBlockedExpanded (src/fs/interface/fs.c:826-930): an element block of values in expanded indices
 * (host arrays; v row-major [m bs][n bs]) expanded through E into J's explicit-dof rows and columns (Dirichlet nodes
 * dropped), INSERT_VALUES or ADD_VALUES; targets outside J's Q1-embedded pattern are an error. A KSP on J sees the new
 * values after dKSPSetOperators. */
dErr dFSMatSetValuesBlockedExpanded(dFS fs, dMat J, dInt m, const dInt idxm[], dInt n, const dInt idxn[], const dScalar v[],
                                    InsertMode imode);
dErr dMatGetCSR(dMat J, dInt *nrows, int64_t *nnz, const dInt **rowptr, const dInt **col, const dScalar **val);
dErr dMatMult(dMat J, const dScalar *x, dScalar *y);
/* host copies of the CSR arrays (rowptr nrows+1, col nnz, val nnz) */
dErr dMatGetCSRHost(dMat J, dInt *rowptr, dInt *col, dScalar *val);

/* ---------------------------------------------------------------- Krylov (PETSc KSP replacement) */
typedef enum { dKSP_CG = 0, dKSP_FGMRES = 1 } dKSPType;
/* preconditioners on the Q1-embedded matrix: Jacobi; Chebyshev-Jacobi (degree from dKSPSetOptions); MG_Q1: geometric
 * V-cycle on the lattice of GLL nodes (scalar or 3 x 3 blocked matrices of uniform-order spaces on block meshes
 * with an even number of GLL intervals per direction; Chebyshev-Jacobi smoothing one degree below that degree,
 * at least 2; Galerkin coarse levels, exact coarsest solve; the cycle in FP64, or in FP32 when the
 * preconditioner precision of dKSPSetOptions is FP32 or BF16) */
typedef enum { dPC_NONE = 0, dPC_JACOBI = 1, dPC_CHEBYSHEV_Q1 = 2, dPC_MG_Q1 = 3 } dPCType;
dErr dKSPCreate(dOperator op, dMat pmat, dKSPType type, dPCType pc, dKSP *ksp);
dErr dKSPDestroy(dKSP *ksp);
/* Chebyshev-Jacobi degree on the Q1 matrix, inner precision, restart length */
dErr dKSPSetOptions(dKSP ksp, dInt cheb_degree, dPrecision pc_precision, dInt restart);
dErr dKSPSolve(dKSP ksp, const dScalar *b, dScalar *x, dReal rtol, dInt maxit, dInt *its, dReal *rnorm);
/* statistics: preconditioner applications, learned corrections dropped by the fallback, whether the
 * correction was still in use at the end of the last solve */
dErr dKSPGetStats(dKSP ksp, int64_t *pc_applies, int64_t *correction_rejects, int *correction_active);

/* ---------------------------------------------------------------- learned coarse correction */
/* No counterpart in the reference. A 3-level 3-D convolutional U-Net (16/32/64 channels, 3x3x3 kernels,
 * BF16 weights, FP32 accumulation) on the lattice of mesh vertices: z = Chebyshev(r) + P N(R r) inside
 * FGMRES, where R = P^T restricts the residual to the vertices, N maps [R r / rms, log k] to the error at
 * the vertices, and P interpolates trilinearly onto the GLL nodes. Scalar uniform-order spaces on block
 * meshes with at least 4 elements per direction. */
typedef struct _p_dLearned *dLearned;
dErr dLearnedCreate(dFS fs, uint64_t seed, dLearned *net);
/* the lattice the network runs on: the mesh vertices (R = P^T with P trilinear, as dLearnedCreate), or the GLL
 * nodes of the space, the lattice of the Q1-embedded matrix ((M p + 1) per direction; R and P the injection of the
 * explicit dofs). On the GLL lattice the network is trained on crop^3 windows of the recorded pairs (crop = 4 m + 1
 * >= 9, windows at origins that are multiples of 4, so that its coarse levels line up with those of the whole
 * lattice; 0: the whole lattice) and applied to the whole lattice. */
typedef enum { dLEARNED_GRID_VERTEX = 0, dLEARNED_GRID_GLL = 1 } dLearnedGrid;
dErr dLearnedCreateOnGrid(dFS fs, dLearnedGrid grid, dInt crop, uint64_t seed, dLearned *net);
dErr dLearnedDestroy(dLearned *net);
/* lattice dims (vertices or GLL nodes), parameter count, collected pairs */
dErr dLearnedGetSizes(dLearned net, dInt dims[3], int64_t *nparam, int64_t *npairs);
/* coefficient field of the next pairs / corrections: log k at the vertices from dGRFCreate data (NULL: k = 1) */
dErr dLearnedSetField(dLearned net, const dReal *grf);
/* run the plain solver (CG on ksp) on b to rtol and record every `every`-th (residual, error) pair; with
 * rough_start the solve starts from seeded noise scaled so that ||A x0|| = ||b|| (early residuals then carry
 * the rough components that FGMRES's Arnoldi vectors have), otherwise from zero */
dErr dLearnedCollectPairs(dLearned net, dKSP ksp, const dScalar *b, dReal rtol, dInt maxit, dInt every, dInt max_pairs,
                          int rough_start, dInt *collected);
/* Adam on the collected pairs (mean squared error over interior vertices); losses[epochs] (may be NULL) */
dErr dLearnedTrain(dLearned net, dInt epochs, dInt batch, dReal lr, uint64_t seed, dReal *losses);
/* z += P N(R r) */
dErr dLearnedApply(dLearned net, const dScalar *r, dScalar *z);
/* FGMRES preconditioner z = Chebyshev(r) + P N(R r) with the plain preconditioner as fallback; NULL removes it */
dErr dKSPSetLearnedCorrection(dKSP ksp, dLearned net);
/* where the correction is applied: 0 = every preconditioner application, 1 = only to the first vector of
 * each restart cycle (the true residual, the kind of input the network was trained on), 2 = adaptive
 * (default). The plain preconditioner judges it: a trial runs a plain cycle and a corrected cycle (policy 2: one
 * trial with each placement) from the same iterate and keeps the better iterate; the correction then runs in the
 * placement that beat the plain cycle by more, or is dropped when none did; a later corrected cycle that reduces
 * the true residual by less than 1 % drops it too */
dErr dKSPSetCorrectionPolicy(dKSP ksp, int policy);
/* the stride-1 convolutions of 16 / 32 channels (and their data and weight gradients) on the tcgen05 tensor
 * cores, with their operands rounded to BF16 (on = 1; the default on the GLL lattice), or every convolution on the
 * CUDA cores in FP32 (on = 0; the default on the vertex lattice) */
dErr dLearnedSetTensorCores(dLearned net, int on);
/* raw network (device FP32 arrays): in [B][2][lattice] -> out [B][1][lattice]; loss and parameter gradient */
dErr dLearnedForward(dLearned net, dInt B, const float *in, float *out);
dErr dLearnedLossGrad(dLearned net, dInt B, const float *in, const float *target, dReal *loss, float *grad);
/* one convolution layer (0..11 in the order C1A C1B D1 C2A D2 C3A C3B U2 C2B U1 C1C OUT) on device FP32 arrays:
 * transpose 0: out [B][co][dims'] = act(conv(in [B][ci][dims]) + bias) (dims' = dims, or halved for the stride-2
 * layers; ReLU on every layer but OUT); transpose 1: its data gradient, in [B][co][dims'] -> out [B][ci][dims] */
dErr dLearnedLayerApply(dLearned net, dInt layer, dInt transpose, dInt B, const dInt dims[3], const float *in, float *out);
/* that layer's weight and bias gradient for input x [B][ci][dims] and output gradient gy [B][co][dims'] into grad
 * [co ci 27 + co] (device FP32, W[co][ci][27] then bias[co]) */
dErr dLearnedLayerWeightGrad(dLearned net, dInt layer, dInt B, const dInt dims[3], const float *x, const float *gy, float *grad);
/* parameters (host FP32 [nparam], layer by layer: W[co][ci][27] then bias[co]); target scale */
dErr dLearnedGetWeights(dLearned net, float *w);
dErr dLearnedSetWeights(dLearned net, const float *w, dReal target_scale);
dErr dLearnedGetScale(dLearned net, dReal *target_scale);
/* checkpoint / resume: the weights and target scale (and with with_moments the Adam state, to continue training) in a
 * file with a JSON header; dLearnedLoad accepts a file of a network with the same layers and marks it trained */
dErr dLearnedSave(dLearned net, const char *path, int with_moments);
dErr dLearnedLoad(dLearned net, const char *path);
/* transfer operators on their own: rc = R r (lattice), z = P c (global) */
dErr dLearnedRestrict(dLearned net, const dScalar *r, dScalar *rc);
dErr dLearnedProlong(dLearned net, const dScalar *c, dScalar *z);
/* recorded pair p on its window: window dims, its origin on the lattice, and (host FP32 arrays of the window's size,
 * either may be NULL) the input channel R r_k / rms and the target (x* - x_k) / rms */
dErr dLearnedGetPair(dLearned net, dInt p, dInt window[3], dInt origin[3], float *input, float *target);
/* corrections applied and non-finite values dropped */
dErr dLearnedGetStats(dLearned net, int64_t *applies, int64_t *dropped_values);

/* ---------------------------------------------------------------- Newton (p-Laplacian) */
/* Newton-Krylov for N(u) = b with N the p-Laplacian function (dOperatorPLaplaceFunction): the SNES side of
 * ellip.c (SNESSetFunction/SNESSetJacobian, ellip.c:697-704; PETSc SNES is not part of this library).
 * Each step re-assembles the Q1 Jacobian into Jp at u (dFSAssembleQ1PLaplace), solves with ksp (operator
 * op = the matrix-free Jacobian at u; FGMRES with FP32 inner applies gives the mixed-precision form),
 * and backtracks on ||F||. fnorm receives max_it+1 residual norms, lin_its max_it iteration counts.
 * Reaching max_it is not an error (as SNES, the caller reads its and fnorm); a failed line search is. */
typedef struct {
  dInt max_it;
  dReal rtol, atol;   /* stop when ||F|| <= rtol ||F0|| or ||F|| <= atol */
  dReal lin_rtol;     /* linear solve tolerance per Newton step */
  dInt lin_maxit;
  int reference_quirk; /* Q1 assembly quirk (dFSAssembleQ1) */
} dNewtonOptions;
dErr dPLaplaceNewtonSolve(dOperator op, dMat Jp, dKSP ksp, const dScalar *b, dScalar *u, dReal p, dReal eps,
                          const dNewtonOptions *opt, dInt *its, dReal *fnorm, dInt *lin_its);
/* Newton-Krylov for the Stokes function N(x) = b (dStokesFunction; stokes.c's SNES with StokesFunction and
 * StokesJacobian, stokes.c:507-540, 675-740): each step solves the Jacobian at x with dStokesSolve's FGMRES and
 * block preconditioner to opt->lin_rtol and backtracks on ||F||; (xu, xp) is the initial guess and the result, xp
 * returned with zero mean. fnorm receives max_it+1 norms, lin_its max_it counts (reference_quirk is unused). */
dErr dStokesNewtonSolve(dStokes stk, const dScalar *bu, const dScalar *bp, dScalar *xu, dScalar *xp, const dNewtonOptions *opt,
                        dInt *its, dReal *fnorm, dInt *lin_its);
/* KSPSetOperators: new operator and/or preconditioning matrix (NULL keeps the current one); the
 * preconditioner is set up again on the next solve (a Newton step that re-assembled the Q1 matrix) */
dErr dKSPSetOperators(dKSP ksp, dOperator op, dMat pmat);

/* ---------------------------------------------------------------- DHM files (src/viewer/dhm.c, contviewdhm.c) */
/* HDF5 files with the reference's DHM group layout: /dohp/{type, mesh, fs, step}; committed types Units_type, Time_type,
 * BoundingBox_type, FS_type, Vec_type; one group per time step (000, 001, ...) with attribute "time"; one FS record per
 * space; one dataset [closure nodes][bs] per vector with attribute "meta". Written from the HDF5 file format
 * specification (version 2 superblock and object headers, compact links, contiguous data, lookup3 checksums). Against
 * the reference: strings are fixed-length (64 bytes), object and region references are path strings, and the mesh
 * (vertices, hexahedra, block extents, the space's degree and boundary-status tags) is stored in the file where the
 * reference names a MOAB file. The file is written when a write-mode viewer is destroyed. */
typedef struct _p_dViewer *dViewer;
/* PetscFileMode values */
typedef enum { dFILE_MODE_READ = 0, dFILE_MODE_WRITE = 1 } dFileMode;
/* PetscViewerCreate + PetscViewerSetType(PETSCVIEWERDHM) + FileSetMode + FileSetName; read mode parses the file */
dErr dViewerDHMOpen(const char *path, dFileMode mode, dViewer *viewer);
dErr dViewerDestroy(dViewer *viewer);
/* dViewerDHMSetTime / SetTimeUnits (dhm.c:339-360): a new time starts a new step group */
dErr dViewerDHMSetTime(dViewer viewer, dReal time);
dErr dViewerDHMSetTimeUnits(dViewer viewer, const char *units, dReal scale);
/* dViewerDHMGetSteps (dhm.c:525-553): number of steps and their times (times may be NULL; room for nsteps) */
dErr dViewerDHMGetSteps(dViewer viewer, dInt *nsteps, dReal *times);
/* dViewerDHMSetTimeStep (dhm.c:484-500): select a step (read mode: its time becomes the viewer's time) */
dErr dViewerDHMSetTimeStep(dViewer viewer, dInt step);
dErr dViewerDHMGetTime(dViewer viewer, dReal *time);
/* dFSView_Cont_DHM (contviewdhm.c:58-116): the space's mesh and its record /dohp/fs/<name> (host data; the space must be
 * built) */
dErr dFSViewDHM(dFS fs, const char *name, dViewer viewer);
/* VecView_Dohp_FSCont_DHM (contviewdhm.c:133-209): a closure vector ([global | Dirichlet] x bs, host or device pointer)
 * of a space written with dFSViewDHM, as dataset <name> of the current step */
dErr dVecViewDHM(dFS fs, const char *name, const dScalar *closure, int on_device, dViewer viewer);
/* VecDohpLoadIntoVector (contviewdhm.c:350-401): the closure vector <name> of the current step, scaled by its units */
dErr dVecLoadDHM(dViewer viewer, const char *name, dFS fs, dScalar *closure, int on_device);
/* dFSLoadIntoFS_Cont_DHM (contviewdhm.c:228-348): the mesh and the space recorded as <name>, built (dFSBuildSpace); the
 * caller owns both (dFSDestroy, dMeshDestroy) and calls dFSSetUp before device use */
dErr dFSLoadDHM(dViewer viewer, const char *name, dJacobi jac, dMesh *mesh, dFS *fs);
/* Jenkins' lookup3 hash, the checksum of HDF5 metadata blocks */
uint32_t dHDF5Checksum(const void *data, size_t len, uint32_t initval);

/* ---------------------------------------------------------------- lognormal coefficient */
/* g(x) = sqrt(2 var / nf) sum_f cos(w_f . x + b_f), random Fourier features of the squared-exponential
 * covariance (Rahimi & Recht 2007), w ~ N(0, I / ell^2), b ~ U[0, 2 pi), splitmix64(seed). grf is a host
 * array of 3 + 4 nf doubles; k = exp(g) is evaluated at the FAST points into kq (device [nq]). */
dErr dGRFCreate(dInt nf, dReal var, dReal ell, uint64_t seed, dReal *grf);
dErr dFSEvaluateLognormal(dFS fs, const dReal *grf, dReal *kq);

#ifdef __cplusplus
}
#endif
#endif
