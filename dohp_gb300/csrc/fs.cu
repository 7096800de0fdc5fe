// dFS objects: space build upload, expand (E) / restrict (E^T) kernels, Dirichlet cache, geometry.
//
// Expand follows dFSGlobalToExpanded (src/fs/interface/fs.c:543-586): closure = [global | Dirichlet or 0],
// expanded = E closure. Restrict follows dFSExpandedToGlobal (fs.c:592-640): closure = E^T expanded, the
// explicit part lands in the global vector. E^T is stored as a CSR over closure nodes whose entries are the
// expanded indices in ascending order, so each global entry sums its element contributions in the same
// order as MatMultTranspose on E: deterministic, no atomics.
#include <string.h>

#include <algorithm>
#include <numeric>

#include "ff.cuh"
#include "internal.h"

using namespace dgb;

dErr fs_build_space(_p_dFS *fs);

namespace {

__global__ void k_expand(int64_t nexp, int bs, const int32_t *__restrict__ emap, int64_t n, const double *__restrict__ g,
                         const double *__restrict__ dcache, double *__restrict__ x, int add) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nexp * bs) return;
  const int64_t r = t / bs;
  const int b = (int)(t - r * bs);
  const int64_t c = emap[r];
  const double v = c < n ? g[c * bs + b] : (dcache ? dcache[(c - n) * bs + b] : 0.0);
  x[t] = add ? x[t] + v : v;
}

// one thread per explicit scalar dof: sum (in FP64) over its expanded copies in ascending order
template <typename TI>
__global__ void k_restrict(int64_t n, int bs, const int32_t *__restrict__ et_ptr, const int32_t *__restrict__ et_idx,
                           const TI *__restrict__ x, double *__restrict__ g, int add) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * bs) return;
  const int64_t c = t / bs;
  const int b = (int)(t - c * bs);
  double s = 0;
  for (int32_t k = et_ptr[c]; k < et_ptr[c + 1]; k++) s += (double)x[(int64_t)et_idx[k] * bs + b];
  g[t] = add ? g[t] + s : s;
}

// weighted forms for hp spaces (E with interpolation rows)
__global__ void k_expand_w(int64_t nexp, int bs, const int32_t *__restrict__ eptr, const int32_t *__restrict__ ecol,
                           const double *__restrict__ eval, int64_t n, const double *__restrict__ g,
                           const double *__restrict__ dcache, double *__restrict__ x, int add) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nexp * bs) return;
  const int64_t r = t / bs;
  const int b = (int)(t - r * bs);
  double v = 0;
  for (int32_t k = eptr[r]; k < eptr[r + 1]; k++) {
    const int64_t c = ecol[k];
    const double cv = c < n ? g[c * bs + b] : (dcache ? dcache[(c - n) * bs + b] : 0.0);
    v += eval[k] * cv;
  }
  x[t] = add ? x[t] + v : v;
}

template <typename TI>
__global__ void k_restrict_w(int64_t n, int bs, const int32_t *__restrict__ et_ptr, const int32_t *__restrict__ et_idx,
                             const double *__restrict__ et_w, const TI *__restrict__ x, double *__restrict__ g, int add) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * bs) return;
  const int64_t c = t / bs;
  const int b = (int)(t - c * bs);
  double s = 0;
  for (int32_t k = et_ptr[c]; k < et_ptr[c + 1]; k++) s += et_w[k] * (double)x[(int64_t)et_idx[k] * bs + b];
  g[t] = add ? g[t] + s : s;
}

// rows [t0, t1) of the restriction (one thread per explicit scalar dof), FP64, optionally weighted (hp)
__global__ void k_restrict_rows(int64_t t0, int64_t t1, int bs, const int32_t *__restrict__ et_ptr, const int32_t *__restrict__ et_idx,
                                const double *__restrict__ et_w, const double *__restrict__ x, double *__restrict__ g) {
  const int64_t t = t0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= t1) return;
  const int64_t c = t / bs;
  const int b = (int)(t - c * bs);
  double s = 0;
  if (et_w)
    for (int32_t k = et_ptr[c]; k < et_ptr[c + 1]; k++) s += et_w[k] * x[(int64_t)et_idx[k] * bs + b];
  else
    for (int32_t k = et_ptr[c]; k < et_ptr[c + 1]; k++) s += x[(int64_t)et_idx[k] * bs + b];
  g[t] = s;
}

}  // namespace

// a range of rows of the FP64 restriction (insert), on a given stream: the same sums, in the same order, as
// fs_restrict
dErr fs_restrict_rows(_p_dFS *fs, const double *x, double *g, int64_t t0, int64_t t1, cudaStream_t s) {
  if (t1 <= t0) return 0;
  k_restrict_rows<<<(unsigned)((t1 - t0 + 255) / 256), 256, 0, s>>>(t0, t1, fs->bs, fs->d_et_ptr, fs->d_et_idx,
                                                                     fs->boolean_e ? nullptr : fs->d_et_w, x, g);
  CUCHK(cudaGetLastError());
  return 0;
}

dErr fs_restrict(_p_dFS *fs, const double *x, double *g, int add) {
  const int64_t N = fs->n * fs->bs;
  if (N == 0) return 0;
  if (!fs->boolean_e) {
    k_restrict_w<double><<<(unsigned)((N + 255) / 256), 256, 0, fs->stream>>>(fs->n, fs->bs, fs->d_et_ptr, fs->d_et_idx, fs->d_et_w, x, g, add);
    CUCHK(cudaGetLastError());
    return 0;
  }
  k_restrict<double><<<(unsigned)((N + 255) / 256), 256, 0, fs->stream>>>(fs->n, fs->bs, fs->d_et_ptr, fs->d_et_idx, x, g, add);
  CUCHK(cudaGetLastError());
  return 0;
}

dErr fs_restrict32(_p_dFS *fs, const float *x, double *g, int add) {
  const int64_t N = fs->n * fs->bs;
  if (N == 0) return 0;
  if (!fs->boolean_e) {
    k_restrict_w<float><<<(unsigned)((N + 255) / 256), 256, 0, fs->stream>>>(fs->n, fs->bs, fs->d_et_ptr, fs->d_et_idx, fs->d_et_w, x, g, add);
    CUCHK(cudaGetLastError());
    return 0;
  }
  k_restrict<float><<<(unsigned)((N + 255) / 256), 256, 0, fs->stream>>>(fs->n, fs->bs, fs->d_et_ptr, fs->d_et_idx, x, g, add);
  CUCHK(cudaGetLastError());
  return 0;
}

// float-float restriction: the sums run in float-float on the FP32 pipe and each result is widened to FP64
// once (widening every expanded value instead made the restriction 3.4x slower than the FP64 one)
__global__ void k_restrict_ffsum(int64_t n, int bs, const int32_t *__restrict__ et_ptr, const int32_t *__restrict__ et_idx,
                                 const ff *__restrict__ w, const ff *__restrict__ x, double *const *py, double *__restrict__ g, int add) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * bs) return;
  const int64_t c = t / bs;
  const int b = (int)(t - c * bs);
  ff s = 0;
  for (int32_t k = et_ptr[c]; k < et_ptr[c + 1]; k++) {
    const ff v = x[(int64_t)et_idx[k] * bs + b];
    if (w) fma_acc(s, w[k], v);
    else s = s + v;
  }
  s = fin(s);
  double *out = py ? *py : g;
  const double r = (double)s;
  out[t] = add ? out[t] + r : r;
}

dErr fs_restrict_ff_to(_p_dFS *fs, const ff *x, double *const *py, double *g, int add, cudaStream_t s) {
  const int64_t N = fs->n * fs->bs;
  if (N == 0) return 0;
  k_restrict_ffsum<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(fs->n, fs->bs, fs->d_et_ptr, fs->d_et_idx,
                                                                fs->boolean_e ? nullptr : (const ff *)fs->d_et_wff, x, py, g, add);
  CUCHK(cudaGetLastError());
  return 0;
}

dErr fs_restrict_ff(_p_dFS *fs, const ff *x, double *g, int add) { return fs_restrict_ff_to(fs, x, nullptr, g, add, fs->stream); }

dErr fs_expand(_p_dFS *fs, const double *g, double *x, bool inhomogeneous, int add) {
  const int64_t N = fs->nexp * fs->bs;
  if (!fs->boolean_e) {
    k_expand_w<<<(unsigned)((N + 255) / 256), 256, 0, fs->stream>>>(fs->nexp, fs->bs, fs->d_eptr, fs->d_ecol, fs->d_eval, fs->n, g,
                                                                    inhomogeneous ? fs->d_dcache : nullptr, x, add);
    CUCHK(cudaGetLastError());
    return 0;
  }
  k_expand<<<(unsigned)((N + 255) / 256), 256, 0, fs->stream>>>(fs->nexp, fs->bs, fs->d_emap, fs->n, g,
                                                                inhomogeneous ? fs->d_dcache : nullptr, x, add);
  CUCHK(cudaGetLastError());
  return 0;
}

static void fs_free_device(_p_dFS *fs) {
  cudaFree(fs->d_emap);
  cudaFree(fs->d_xstart);
  cudaFree(fs->d_edeg);
  cudaFree(fs->d_qoff);
  cudaFree(fs->d_et_ptr);
  cudaFree(fs->d_et_idx);
  cudaFree(fs->d_coords);
  cudaFree(fs->d_dcache);
  cudaFree(fs->d_fast_tab);
  cudaFree(fs->d_scratch_exp);
  cudaFree(fs->d_eptr);
  cudaFree(fs->d_ecol);
  cudaFree(fs->d_eval);
  cudaFree(fs->d_et_w);
  cudaFree(fs->d_et_wff);
  cudaFree(fs->d_mg_lat);
  fs->d_et_wff = nullptr;
  fs->d_mg_lat = nullptr;
  fs->d_eptr = fs->d_ecol = nullptr;
  fs->d_eval = fs->d_et_w = nullptr;
  fs->d_emap = fs->d_xstart = fs->d_edeg = fs->d_qoff = fs->d_et_ptr = fs->d_et_idx = nullptr;
  fs->d_coords = fs->d_dcache = fs->d_fast_tab = fs->d_scratch_exp = nullptr;
}

template <typename T>
static dErr upload(T **d, const T *h, size_t count) {
  CUCHK(cudaMalloc((void **)d, std::max<size_t>(count, 1) * sizeof(T)));
  if (count) CUCHK(cudaMemcpy(*d, h, count * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

extern "C" {

dErr dFSCreate(dMesh mesh, dJacobi jac, dFS *fs) {
  if (!mesh || !fs) return set_error("dFSCreate: null argument");
  if (jac && jac->modal) return set_error("dFSCreate: a dFS needs a tensor dJacobi (modal element spaces are discontinuous)");
  _p_dFS *f = new _p_dFS();
  f->mesh = mesh;
  f->jac = jac;
  *fs = f;
  return 0;
}

dErr dFSDestroy(dFS *fs) {
  if (!fs || !*fs) return 0;
  if ((*fs)->coord_fs) dFSDestroy(&(*fs)->coord_fs);
  fs_free_device(*fs);
  delete *fs;
  *fs = nullptr;
  return 0;
}

dErr dFSSetDegree(dFS fs, dInt degree, const dInt *elem_degree) {
  if (!fs) return set_error("null dFS");
  if (fs->setup) return set_error("dFSSetDegree after dFSSetUp");
  fs->degree = degree;
  fs->elem_degree_in.clear();
  if (elem_degree) fs->elem_degree_in.assign(elem_degree, elem_degree + fs->mesh->nr);
  return 0;
}

dErr dFSSetBlockSize(dFS fs, dInt bs) {
  if (!fs) return set_error("null dFS");
  if (bs != 1 && bs != 3) return set_error("block size %d not supported (1 or 3)", bs);
  fs->bs = bs;
  return 0;
}

dErr dFSRegisterBoundary(dFS fs, dInt setid, dFSBStatus status) {
  if (!fs) return set_error("null dFS");
  const int bit = setid == 100 ? 0 : setid == 200 ? 1 : setid == 300 ? 2 : -1;
  if (bit < 0) return set_error("unknown boundary set %d (block meshes have 100, 200, 300)", setid);
  if (status & ~(dFSBSTATUS_DIRICHLET | dFSBSTATUS_WEAK | 0xffff)) return set_error("unknown boundary status %#x", (unsigned)status);
  if (status & dFSBSTATUS_DIRICHLET) fs->dirichlet_mask |= 1 << bit;
  else fs->dirichlet_mask &= ~(1 << bit);
  if (status & dFSBSTATUS_WEAK) fs->weak_mask |= 1 << bit;
  else fs->weak_mask &= ~(1 << bit);
  return 0;
}

dErr dFSSetStream(dFS fs, void *stream) {
  if (!fs) return set_error("null dFS");
  fs->stream = (cudaStream_t)stream;
  return 0;
}

dErr dFSBuildSpace(dFS fs) {
  if (!fs) return set_error("null dFS");
  if (fs->built) return 0;
  if (fs->jac && fs->jac->modal) return set_error("dFSBuildSpace: a dFS needs a tensor dJacobi (modal element spaces are discontinuous)");
  DCHK(fs_build_space(fs));
  fs->built = true;
  return 0;
}

dErr dFSSetUp(dFS fs) {
  if (!fs) return set_error("null dFS");
  if (fs->setup) return 0;
  DCHK(dFSBuildSpace(fs));
  const _p_dMesh *m = fs->mesh;
  // E^T over closure nodes, ascending expanded index (counting sort over the row-ordered E): each closure
  // node sums its contributions in MatMultTranspose order
  const int64_t enz = (int64_t)fs->ecol.size();
  std::vector<int32_t> ptr(fs->nc + 1, 0), idx(enz);
  std::vector<double> wts(enz);
  for (int64_t k = 0; k < enz; k++) ptr[fs->ecol[k] + 1]++;
  for (int64_t c = 0; c < fs->nc; c++) ptr[c + 1] += ptr[c];
  {
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int64_t r = 0; r < fs->nexp; r++)
      for (int32_t k = fs->eptr[r]; k < fs->eptr[r + 1]; k++) {
        const int32_t pos = fill[fs->ecol[k]]++;
        idx[pos] = (int32_t)r;
        wts[pos] = fs->eval[k];
      }
  }
  if (!fs->boolean_e) {
    DCHK(upload(&fs->d_eptr, fs->eptr.data(), fs->eptr.size()));
    DCHK(upload(&fs->d_ecol, fs->ecol.data(), fs->ecol.size()));
    DCHK(upload(&fs->d_eval, fs->eval.data(), fs->eval.size()));
    DCHK(upload(&fs->d_et_w, wts.data(), wts.size()));
    std::vector<ff> wff(wts.begin(), wts.end());  // for the float-float restriction
    ff *dwff = nullptr;
    DCHK(upload(&dwff, wff.data(), wff.size()));
    fs->d_et_wff = dwff;
  }
  // expanded coordinates in tensor vertex order (dFSCreateGeometryFromMesh_Private, fsgeom.c:146-156)
  static const int kConn[8] = {0, 4, 3, 7, 1, 5, 2, 6};
  std::vector<double> coords(24 * fs->nelem);
  for (int64_t r = 0; r < fs->nelem; r++)
    for (int i = 0; i < 8; i++)
      for (int d = 0; d < 3; d++) coords[(r * 8 + i) * 3 + d] = m->vx[3 * m->hconn[8 * r + kConn[i]] + d];
  DCHK(upload(&fs->d_emap, fs->emap.data(), fs->emap.size()));
  DCHK(upload(&fs->d_xstart, fs->xstart.data(), fs->xstart.size()));
  DCHK(upload(&fs->d_edeg, fs->edeg.data(), fs->edeg.size()));
  DCHK(upload(&fs->d_qoff, fs->qoff.data(), fs->qoff.size()));
  DCHK(upload(&fs->d_et_ptr, ptr.data(), ptr.size()));
  DCHK(upload(&fs->d_et_idx, idx.data(), idx.size()));
  DCHK(upload(&fs->d_coords, coords.data(), coords.size()));
  CUCHK(cudaMalloc(&fs->d_dcache, std::max<int64_t>((fs->nc - fs->n) * fs->bs, 1) * sizeof(double)));
  CUCHK(cudaMemset(fs->d_dcache, 0, std::max<int64_t>((fs->nc - fs->n) * fs->bs, 1) * sizeof(double)));
  // FAST-rule basis tables for every degree present: [p-1][B (P*P) | Dq (P*P)] padded to MAXP^2 each
  std::vector<double> tab(2 * (MAXP - 1) * MAXP * MAXP, 0.0);
  for (int p = 1; p < MAXP; p++) {
    Basis1D b;
    DCHK(make_basis(p, dQUADRATURE_METHOD_FAST, &b));
    double *B = &tab[(2 * (p - 1)) * MAXP * MAXP], *Dq = B + MAXP * MAXP;
    for (int i = 0; i < b.Q * b.P; i++) B[i] = b.B[i];
    for (int i = 0; i < b.Q * b.Q; i++) Dq[i] = b.Dq[i];
  }
  DCHK(upload(&fs->d_fast_tab, tab.data(), tab.size()));
  CUCHK(cudaMalloc(&fs->d_scratch_exp, fs->nexp * fs->bs * sizeof(double)));
  fs->setup = true;
  return 0;
}

dErr dFSGetSizes(dFS fs, dInt *n, dInt *nc, dInt *nexp, dInt *bs, dInt *nelem) {
  if (!fs || !fs->built) return set_error("dFS space not built");
  if (n) *n = (dInt)fs->n;
  if (nc) *nc = (dInt)fs->nc;
  if (nexp) *nexp = (dInt)fs->nexp;
  if (bs) *bs = fs->bs;
  if (nelem) *nelem = (dInt)fs->nelem;
  return 0;
}

dErr dFSGetExpandedMap(dFS fs, dInt *emap, dInt *xstart) {
  if (!fs || !fs->built) return set_error("dFS space not built");
  if (emap) memcpy(emap, fs->emap.data(), fs->emap.size() * sizeof(dInt));
  if (xstart) memcpy(xstart, fs->xstart.data(), fs->xstart.size() * sizeof(dInt));
  return 0;
}

dErr dFSGetElementDegrees(dFS fs, dInt *deg) {
  if (!fs || !fs->built) return set_error("dFS space not built");
  memcpy(deg, fs->edeg.data(), fs->edeg.size() * sizeof(dInt));
  return 0;
}

dErr dFSGetGeometryVectorExpanded(dFS fs, const dReal **coords) {
  if (!fs || !fs->setup) return set_error("dFS not set up");
  *coords = fs->d_coords;
  return 0;
}

dErr dFSInhomogeneousDirichletCommit(dFS fs, const dScalar *closure) {
  if (!fs || !fs->setup) return set_error("dFS not set up");
  const int64_t nd = (fs->nc - fs->n) * fs->bs;
  if (nd) CUCHK(cudaMemcpyAsync(fs->d_dcache, closure + fs->n * fs->bs, nd * sizeof(double), cudaMemcpyDeviceToDevice, fs->stream));
  return 0;
}

dErr dFSGlobalToExpanded(dFS fs, const dScalar *g, dScalar *x, dFSHomogeneousMode hmode, InsertMode imode) {
  if (!fs || !fs->setup) return set_error("dFS not set up");
  if (imode != INSERT_VALUES && imode != ADD_VALUES) return set_error("InsertMode %d not supported", (int)imode);
  return fs_expand(fs, g, x, hmode == dFS_INHOMOGENEOUS, imode == ADD_VALUES);
}

dErr dFSExpandedToGlobal(dFS fs, const dScalar *x, dScalar *g, dFSHomogeneousMode hmode, InsertMode imode) {
  (void)hmode;  // only matters for rotated coordinates (fs.c:631), which this path does not support
  if (!fs || !fs->setup) return set_error("dFS not set up");
  if (imode != INSERT_VALUES && imode != ADD_VALUES) return set_error("InsertMode %d not supported", (int)imode);
  return fs_restrict(fs, x, g, imode == ADD_VALUES);
}

dErr dFSGetNumQuadraturePoints(dFS fs, int64_t *nq) {
  if (!fs || !fs->built) return set_error("dFS space not built");
  *nq = fs->nq;
  return 0;
}

}  // extern "C"
