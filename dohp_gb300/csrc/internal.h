// Internal declarations of dohp_gb300 (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/dohp_gb300.h"

namespace dgb {

dErr set_error(const char *fmt, ...);
#define DCHK(call)                                  \
  do {                                              \
    dErr _e = (call);                               \
    if (_e) return _e;                              \
  } while (0)
#define CUCHK(call)                                                                                  \
  do {                                                                                               \
    cudaError_t _c = (call);                                                                         \
    if (_c != cudaSuccess) return ::dgb::set_error("%s:%d CUDA error %s: %s", __FILE__, __LINE__,   \
                                                   cudaGetErrorName(_c), cudaGetErrorString(_c));    \
  } while (0)

// an NVTX range for the lifetime of the object (the phases a profiler shows: operator applies, assembly, solves,
// multigrid cycles, the learned correction); named after the reference's PETSc log events where it has one
struct Range {
  explicit Range(const char *name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range &) = delete;
  Range &operator=(const Range &) = delete;
};

constexpr int MAXP = 9;   // max nodes per direction (degree 8)
constexpr int MAXQ = 18;  // max rule points per direction (SPARSE rule of degree 8)

// ---------------------------------------------------------------- 1-D bases (basis.cu)
void gauss_rule(int n, double *x, double *w);
void lobatto_rule(int n, double *x, double *w);
// Lagrange basis on nodes[P] at t: values and derivatives
void lagrange(int P, const double *nodes, double t, double *val, double *der);
// 1-D rule of a method and order (tensorquad.c:51-118) in a point family (Gauss-Legendre unless given)
int rule_1d(dQuadratureMethod method, int order, double *x, double *w, int family = dGAUSS_LEGENDRE);
// 1-D tables for one basis degree p (P = p+1 GLL nodes) on a rule
struct Basis1D {
  int P = 0, Q = 0;
  double node[MAXP], nodew[MAXP], x[MAXQ], w[MAXQ];  // GLL nodes and their weights; rule points and weights
  double B[MAXQ * MAXP];   // interp [Q][P]
  double D[MAXQ * MAXP];   // deriv [Q][P]
  double Dq[MAXQ * MAXQ];  // collocation derivative at the rule points [Q][Q] (FAST: Q == P)
  double cB[MAXQ * 2], cD[MAXQ * 2];  // coordinate (P=2) basis on the same rule
};
int make_basis(int p, dQuadratureMethod method, Basis1D *b);

}  // namespace dgb

struct _p_dEFS {
  int P[3], Q[3];
  int modal = -1;  // >= 0: a modal (P-discontinuous) basis of this order, P[0] modes; h_tab = interp [nq][P], deriv [nq][P][3]
  dQuadratureMethod method;
  _p_dRule *rule = nullptr;  // the rule the basis is evaluated on (owned by the dJacobi's quadrature)
  dgb::Basis1D b[3];
  std::vector<double> h_tab;  // per direction B[Q][P], D[Q][P] packed
  double *d_tab = nullptr;      // device copy of h_tab, made on first use
};

struct _p_dJacobi {
  int modal = 0;  // dJacobiSetType: 0 tensor, 1 modal (what dJacobiGetEFS makes)
  std::map<std::vector<int>, _p_dEFS *> efs;
  _p_dQuadrature *quad[3] = {nullptr, nullptr, nullptr};  // per dQuadratureMethod, made on first request
};
void jacobi_free_quadratures(dJacobi jac);
// the dJacobi's rule / tensor element space of a method and orders in a point family (the dFS paths: Gauss-Legendre)
dErr jacobi_rule(dJacobi jac, dQuadratureMethod method, const int order[3], _p_dRule **out, int family = dGAUSS_LEGENDRE);
dErr jacobi_efs(dJacobi jac, const dInt degree[3], dQuadratureMethod method, const dInt rule_order[3], dEFS *efs,
                int family = dGAUSS_LEGENDRE);
int jacobi_quad_family(dJacobi jac, dQuadratureMethod method);  // the family dQuadratureTensorSetGaussFamily set

struct _p_dMesh {
  int nx, ny, nz;
  int64_t nv, ne, nf, nr, nents;
  std::vector<double> vx;                  // [nv][3]
  std::vector<int64_t> econn, fconn, hconn;  // [ne][2], [nf][4], [nr][8]
  std::vector<signed char> fset;           // generator face set per entity (0..5) or -1
  std::vector<int32_t> adjoff, adjind, adjperm;
  bool structured = true;  // a block (nx, ny, nz, lattice order); false: entities given by connectivity
};

struct _p_dFS {
  dMesh mesh = nullptr;
  dJacobi jac = nullptr;
  int bs = 1;
  int degree = 0;
  std::vector<int> elem_degree_in;
  int dirichlet_mask = 0;  // bit0 set 100 (walls), bit1 200 (top), bit2 300 (bottom)
  int weak_mask = 0;       // sets registered with dFSBSTATUS_WEAK, same bits
  bool built = false;  // host maps computed (dFSBuildSpace)
  bool setup = false;  // device arrays uploaded
  cudaStream_t stream = 0;
  // host results of the space build
  int64_t nelem = 0, n = 0, nc = 0, nexp = 0, nq = 0;
  std::vector<int32_t> xstart, emap, edeg, qoff;
  std::vector<int32_t> eptr, ecol;  // E as CSR (rows = expanded nodes); Boolean rows have one 1.0
  std::vector<double> eval;
  bool boolean_e = true;            // every row of E is a single 1.0 (emap holds it)
  bool uniform = true;
  int p = 0;  // uniform degree
  // device
  int32_t *d_emap = nullptr, *d_xstart = nullptr, *d_edeg = nullptr, *d_qoff = nullptr;
  int32_t *d_et_ptr = nullptr, *d_et_idx = nullptr;  // E^T over closure nodes (ascending expanded index)
  int32_t *d_eptr = nullptr, *d_ecol = nullptr;       // E as CSR (hp spaces only)
  double *d_eval = nullptr, *d_et_w = nullptr;        // E values and E^T weights (hp spaces only)
  void *d_et_wff = nullptr;                          // E^T weights as float pairs (hp spaces only)
  int32_t *d_mg_lat = nullptr;                       // Q1 multigrid: lattice position of each explicit node (made once)
  double *d_coords = nullptr;                        // [nelem][8][3]
  double *d_dcache = nullptr;                        // Dirichlet values [(nc-n)*bs]
  // per-degree basis tables on the device for FAST rules: [p] -> B, Dq (Q=P)
  double *d_fast_tab = nullptr;
  double *d_scratch_exp = nullptr;  // expanded-size scratch (nexp*bs)
  _p_dFS *coord_fs = nullptr;       // the Q1 coordinate space on the same mesh (dFSGetCoordinateFS), made on request
};

struct _p_dOperator {
  dFS fs;
  dOperatorKind kind;
  dPrecision prec = dPREC_FP64;
  double param[4] = {0, 0, 0, 0};
  double lam = 0, mu = 0;
  double *d_geo = nullptr;       // fp64 geometric factors per qpt
  float *d_geo32 = nullptr;      // fp32 copy
  void *d_geo16 = nullptr;       // bf16 copy (scalar kinds)
  void *d_tcb = nullptr;         // BF16 tensor-core apply: the six B operands (block tables of the 1-D bases)
  bool tc_checked = false;       // the first tensor-core apply was checked for a timed-out wait
  void *d_geoff = nullptr;       // float-float copy
  void *d_yff = nullptr;         // float-float expanded output
  double *d_k = nullptr;         // coefficient per qpt
  double *d_stash = nullptr;     // p-Laplacian stash [nq][4]
  double *d_gbase = nullptr;     // p-Laplacian: {J^-1, w det J} per qpt (10, SoA per element)
  double *d_svk = nullptr;       // St. Venant-Kirchhoff state: {F, S} per qpt (15, SoA per element)
  bool svk_state = false;        // elasticity Jacobian at that state instead of F = I
  double *d_yexp = nullptr;      // expanded output scratch
  float *d_x32 = nullptr, *d_y32 = nullptr;
  double *d_hx = nullptr, *d_hy = nullptr;  // device staging for the host-vector form
  void *copy_stream = nullptr;               // host-vector form: device-to-host copies beside the restriction
  void *copy_events[4] = {nullptr, nullptr, nullptr, nullptr};
  bool geo_valid = false;
  int geo_kind = -1;
  void *hp_plan = nullptr;  // order buckets, tiles, work list, graphs (hp.cu)
  dLaunchMode launch = dLAUNCH_DEFAULT;
  bool autotune = false;
  char tune_path[512] = "";
};

struct _p_dMat {
  dFS fs;
  int bs = 1;
  int64_t nrows = 0, nnz = 0;
  int32_t *d_rowptr = nullptr, *d_col = nullptr;
  double *d_val = nullptr;
  // bs > 1: the node (scalar) pattern the blocked CSR expands
  int64_t snnz = 0;
  int32_t *d_srowptr = nullptr, *d_scol = nullptr;
  // sliced-ELL copy the SpMV runs on (32-row slices, column-major, padded to the slice's longest row):
  // slice s holds entries [d_sell_off[s], d_sell_off[s+1]); built from the CSR on first use, values refreshed
  // after each numeric assembly (sell_valid false)
  int64_t sell_len = 0;
  int64_t *d_sell_off = nullptr;
  int32_t *d_sell_col = nullptr;
  double *d_sell_val = nullptr;
  bool sell_valid = false;
  // host copy of the CSR pattern (dFSMatSetValuesBlockedExpanded locates its entries on the host)
  std::vector<int32_t> h_rowptr, h_col;
};

dErr mat_sell(_p_dMat *J, cudaStream_t s);
