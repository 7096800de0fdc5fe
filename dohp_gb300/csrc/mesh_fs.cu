// Block mesh, adjacency and function-space build (host setup; results uploaded to the device).
//
//  * entity creation order and boundary sets of dMeshGenerateBlock (src/fs/mesh/interface/genblock.c:206-421)
//  * canonical downward adjacency + orientation permutations (dMeshGetAdjacency, mesh.c:1039-1191;
//    dGeomOrientFindPerm_HexQuad/_QuadLine, include/dohpgeom.h:97-150)
//  * min-rule degree propagation (dJacobiPropagateDown_Tensor, src/jacobi/impls/tensor/tensor.c:199-247)
//  * partition explicit/Dirichlet and natural ordering (fsbuild.c:55-146, cont.c:93-178, cont.c:293-385)
//  * the element assembly map E (dJacobiAddConstraints_Tensor, tensor.c:360-468)
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <map>

#include "internal.h"

using namespace dgb;

namespace {

struct Ord {
  int x, y, z;
};

inline int64_t vidx(const _p_dMesh *m, int i, int j, int k) { return ((int64_t)i * m->ny + j) * m->nz + k; }
// face/edge families in creation order: z-normal, y-normal, x-normal faces; z-, y-, x-directed edges
inline int64_t nzf(const _p_dMesh *m) { return (int64_t)(m->nx - 1) * (m->ny - 1) * m->nz; }
inline int64_t nyf(const _p_dMesh *m) { return (int64_t)(m->nx - 1) * m->ny * (m->nz - 1); }
inline int64_t fz(const _p_dMesh *m, int i, int j, int k) { return ((int64_t)i * (m->ny - 1) + j) * m->nz + k; }
inline int64_t fy(const _p_dMesh *m, int i, int j, int k) { return nzf(m) + ((int64_t)i * m->ny + j) * (m->nz - 1) + k; }
inline int64_t fx(const _p_dMesh *m, int i, int j, int k) { return nzf(m) + nyf(m) + ((int64_t)i * (m->ny - 1) + j) * (m->nz - 1) + k; }
inline int64_t nze(const _p_dMesh *m) { return (int64_t)m->nx * m->ny * (m->nz - 1); }
inline int64_t nye(const _p_dMesh *m) { return (int64_t)m->nx * (m->ny - 1) * m->nz; }
inline int64_t ez(const _p_dMesh *m, int i, int j, int k) { return ((int64_t)i * m->ny + j) * (m->nz - 1) + k; }
inline int64_t ey(const _p_dMesh *m, int i, int j, int k) { return nze(m) + ((int64_t)i * (m->ny - 1) + j) * m->nz + k; }
inline int64_t ex(const _p_dMesh *m, int i, int j, int k) { return nze(m) + nye(m) + ((int64_t)i * m->ny + j) * m->nz + k; }

// canonical sides of a hex (faces) and a quad (edges); tables as in include/dohpgeom.h:19,26
const int kHexFace[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {0, 3, 2, 1}, {4, 5, 6, 7}};
const int kQuadEdge[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
// quad rotations/reflections in the order of dGeomOrientFindPerm_HexQuad (dohpgeom.h:100)
const int kQuadPerm[8][4] = {{0, 1, 2, 3}, {3, 0, 1, 2}, {2, 3, 0, 1}, {1, 2, 3, 0}, {0, 3, 2, 1}, {1, 0, 3, 2}, {2, 1, 0, 3}, {3, 2, 1, 0}};

uint64_t splitmix(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double unif(uint64_t *s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

dErr mesh_build(_p_dMesh *m, const double box[6], double perturb, uint64_t seed) {
  const int NX = m->nx, NY = m->ny, NZ = m->nz;
  m->nv = (int64_t)NX * NY * NZ;
  m->nr = (int64_t)(NX - 1) * (NY - 1) * (NZ - 1);
  m->nf = nzf(m) + nyf(m) + (int64_t)NX * (NY - 1) * (NZ - 1);
  m->ne = nze(m) + nye(m) + (int64_t)(NX - 1) * NY * NZ;
  m->nents = m->nv + m->ne + m->nf + m->nr;
  m->vx.assign(3 * m->nv, 0.0);
  m->econn.assign(2 * m->ne, 0);
  m->fconn.assign(4 * m->nf, 0);
  m->hconn.assign(8 * m->nr, 0);
  m->fset.assign(m->nents, -1);
  const double h[3] = {(box[1] - box[0]) / (NX - 1), (box[3] - box[2]) / (NY - 1), (box[5] - box[4]) / (NZ - 1)};
  uint64_t st = seed;
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY; j++)
      for (int k = 0; k < NZ; k++) {
        const int64_t v = vidx(m, i, j, k);
        signed char s = -1;  // genblock vertex set chain (genblock.c:212-218)
        if (i == 0) s = 3;
        else if (i == NX - 1) s = 1;
        else if (j == 0) s = 0;
        else if (j == NY - 1) s = 2;
        else if (k == 0) s = 4;
        else if (k == NZ - 1) s = 5;
        m->fset[v] = s;
        double *x = &m->vx[3 * v];
        x[0] = box[0] + (box[1] - box[0]) * (1. * i / (NX - 1));
        x[1] = box[2] + (box[3] - box[2]) * (1. * j / (NY - 1));
        x[2] = box[4] + (box[5] - box[4]) * (1. * k / (NZ - 1));
        const bool interior = i > 0 && i < NX - 1 && j > 0 && j < NY - 1 && k > 0 && k < NZ - 1;
        if (perturb != 0 && interior)
          for (int d = 0; d < 3; d++) x[d] += perturb * h[d] * (2.0 * unif(&st) - 1.0);
      }
  for (int i = 0; i < NX - 1; i++)
    for (int j = 0; j < NY - 1; j++)
      for (int k = 0; k < NZ - 1; k++) {
        int64_t *c = &m->hconn[8 * (((int64_t)i * (NY - 1) + j) * (NZ - 1) + k)];
        const int di[8] = {0, 1, 1, 0, 0, 1, 1, 0}, dj[8] = {0, 0, 1, 1, 0, 0, 1, 1}, dk[8] = {0, 0, 0, 0, 1, 1, 1, 1};
        for (int t = 0; t < 8; t++) c[t] = vidx(m, i + di[t], j + dj[t], k + dk[t]);
      }
  const int64_t F0 = m->nv + m->ne, E0 = m->nv;
  auto setf = [&](int64_t f, int a0, int a1, int a2, int b0, int b1, int b2, int c0, int c1, int c2, int d0, int d1, int d2) {
    int64_t *c = &m->fconn[4 * f];
    c[0] = vidx(m, a0, a1, a2);
    c[1] = vidx(m, b0, b1, b2);
    c[2] = vidx(m, c0, c1, c2);
    c[3] = vidx(m, d0, d1, d2);
  };
  for (int i = 0; i < NX - 1; i++)
    for (int j = 0; j < NY - 1; j++)
      for (int k = 0; k < NZ; k++) {
        const int64_t f = fz(m, i, j, k);
        if (k == 0) m->fset[F0 + f] = 4;
        if (k == NZ - 1) m->fset[F0 + f] = 5;
        setf(f, i, j, k, i + 1, j, k, i + 1, j + 1, k, i, j + 1, k);
      }
  for (int i = 0; i < NX - 1; i++)
    for (int j = 0; j < NY; j++)
      for (int k = 0; k < NZ - 1; k++) {
        const int64_t f = fy(m, i, j, k);
        if (j == 0) m->fset[F0 + f] = 0;
        if (j == NY - 1) m->fset[F0 + f] = 2;
        setf(f, i, j, k, i + 1, j, k, i + 1, j, k + 1, i, j, k + 1);
      }
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY - 1; j++)
      for (int k = 0; k < NZ - 1; k++) {
        const int64_t f = fx(m, i, j, k);
        if (i == 0) m->fset[F0 + f] = 3;
        if (i == NX - 1) m->fset[F0 + f] = 1;
        setf(f, i, j, k, i, j + 1, k, i, j + 1, k + 1, i, j, k + 1);
      }
  auto sete = [&](int64_t e, int64_t a, int64_t b, signed char s) {
    m->econn[2 * e] = a;
    m->econn[2 * e + 1] = b;
    m->fset[E0 + e] = s;
  };
  for (int i = 0; i < NX; i++)  // edge set chains as genblock.c:356-393
    for (int j = 0; j < NY; j++)
      for (int k = 0; k < NZ - 1; k++) {
        signed char s = -1;
        if (i == 0) s = 0;
        else if (i == NX - 1) s = 2;
        else if (j == 0) s = 3;
        else if (j == NY - 1) s = 1;
        sete(ez(m, i, j, k), vidx(m, i, j, k), vidx(m, i, j, k + 1), s);
      }
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY - 1; j++)
      for (int k = 0; k < NZ; k++) {
        signed char s = -1;
        if (i == 0) s = 0;
        else if (i == NX - 1) s = 2;
        else if (k == 0) s = 4;
        else if (k == NZ - 1) s = 5;
        sete(ey(m, i, j, k), vidx(m, i, j, k), vidx(m, i, j + 1, k), s);
      }
  for (int i = 0; i < NX - 1; i++)
    for (int j = 0; j < NY; j++)
      for (int k = 0; k < NZ; k++) {
        signed char s = -1;
        if (j == 0) s = 3;
        else if (j == NY - 1) s = 1;
        else if (k == 0) s = 4;
        else if (k == NZ - 1) s = 5;
        sete(ex(m, i, j, k), vidx(m, i, j, k), vidx(m, i + 1, j, k), s);
      }
  return 0;
}

dErr mesh_adjacency(_p_dMesh *m) {
  const int NX = m->nx, NY = m->ny, NZ = m->nz;
  const int64_t E0 = m->nv, F0 = m->nv + m->ne, R0 = F0 + m->nf;
  m->adjoff.assign(m->nents + 1, 0);
  m->adjind.assign(2 * m->ne + 4 * m->nf + 6 * m->nr, 0);
  m->adjperm.assign(m->adjind.size(), 0);
  int64_t a = 0;
  for (int64_t e = 0; e < m->ne; e++) {
    m->adjoff[E0 + e] = (int32_t)a;
    m->adjind[a++] = (int32_t)m->econn[2 * e];
    m->adjind[a++] = (int32_t)m->econn[2 * e + 1];
  }
  for (int64_t f = 0; f < m->nf; f++) {
    m->adjoff[F0 + f] = (int32_t)a;
    int64_t ed[4];
    if (f < nzf(m)) {
      const int k = (int)(f % NZ), j = (int)((f / NZ) % (NY - 1)), i = (int)(f / NZ / (NY - 1));
      ed[0] = ex(m, i, j, k), ed[1] = ey(m, i + 1, j, k), ed[2] = ex(m, i, j + 1, k), ed[3] = ey(m, i, j, k);
    } else if (f < nzf(m) + nyf(m)) {
      const int64_t g = f - nzf(m);
      const int k = (int)(g % (NZ - 1)), j = (int)((g / (NZ - 1)) % NY), i = (int)(g / (NZ - 1) / NY);
      ed[0] = ex(m, i, j, k), ed[1] = ez(m, i + 1, j, k), ed[2] = ex(m, i, j, k + 1), ed[3] = ez(m, i, j, k);
    } else {
      const int64_t g = f - nzf(m) - nyf(m);
      const int k = (int)(g % (NZ - 1)), j = (int)((g / (NZ - 1)) % (NY - 1)), i = (int)(g / (NZ - 1) / (NY - 1));
      ed[0] = ey(m, i, j, k), ed[1] = ez(m, i, j + 1, k), ed[2] = ey(m, i, j, k + 1), ed[3] = ez(m, i, j, k);
    }
    const int64_t *fv = &m->fconn[4 * f];
    for (int s = 0; s < 4; s++) {
      const int64_t *ev = &m->econn[2 * ed[s]];
      int perm;
      if (ev[0] == fv[kQuadEdge[s][0]] && ev[1] == fv[kQuadEdge[s][1]]) perm = 0;
      else if (ev[1] == fv[kQuadEdge[s][0]] && ev[0] == fv[kQuadEdge[s][1]]) perm = 1;
      else return set_error("edge %lld does not match side %d of face %lld", (long long)ed[s], s, (long long)f);
      m->adjind[a] = (int32_t)(E0 + ed[s]);
      m->adjperm[a++] = perm;
    }
  }
  for (int i = 0; i < NX - 1; i++)
    for (int j = 0; j < NY - 1; j++)
      for (int k = 0; k < NZ - 1; k++) {
        const int64_t r = ((int64_t)i * (NY - 1) + j) * (NZ - 1) + k;
        m->adjoff[R0 + r] = (int32_t)a;
        const int64_t side[6] = {fy(m, i, j, k), fx(m, i + 1, j, k), fy(m, i, j + 1, k), fx(m, i, j, k), fz(m, i, j, k), fz(m, i, j, k + 1)};
        const int64_t *rv = &m->hconn[8 * r];
        for (int s = 0; s < 6; s++) {
          const int64_t *fv = &m->fconn[4 * side[s]];
          int perm = -1;
          for (int t = 0; t < 8 && perm < 0; t++)
            if (fv[kQuadPerm[t][0]] == rv[kHexFace[s][0]] && fv[kQuadPerm[t][1]] == rv[kHexFace[s][1]]) {
              if (fv[kQuadPerm[t][2]] != rv[kHexFace[s][2]] || fv[kQuadPerm[t][3]] != rv[kHexFace[s][3]])
                return set_error("face %lld only partly matches side %d of region %lld", (long long)side[s], s, (long long)r);
              perm = t;
            }
          if (perm < 0) return set_error("face %lld does not match side %d of region %lld", (long long)side[s], s, (long long)r);
          m->adjind[a] = (int32_t)(F0 + side[s]);
          m->adjperm[a++] = perm;
        }
      }
  m->adjoff[m->nents] = (int32_t)a;
  return 0;
}

// dMeshGetAdjacency (mesh.c:1074-1191) for a mesh given by its entities: the same canonical sides and orientation
// permutations as the block form above, each side's edge or face found by its vertices
dErr mesh_adjacency_general(_p_dMesh *m) {
  const int64_t E0 = m->nv, F0 = m->nv + m->ne, R0 = F0 + m->nf;
  std::map<std::pair<int64_t, int64_t>, int64_t> edge_of;  // sorted vertex pair -> edge
  for (int64_t e = 0; e < m->ne; e++) {
    const int64_t a = m->econn[2 * e], b = m->econn[2 * e + 1];
    if (a == b) return set_error("edge %lld has one vertex twice", (long long)e);
    if (!edge_of.emplace(std::make_pair(std::min(a, b), std::max(a, b)), e).second)
      return set_error("edge %lld repeats another edge", (long long)e);
  }
  std::map<std::array<int64_t, 4>, int64_t> face_of;  // sorted vertex quadruple -> face
  for (int64_t f = 0; f < m->nf; f++) {
    std::array<int64_t, 4> k = {m->fconn[4 * f], m->fconn[4 * f + 1], m->fconn[4 * f + 2], m->fconn[4 * f + 3]};
    std::sort(k.begin(), k.end());
    if (!face_of.emplace(k, f).second) return set_error("face %lld repeats another face", (long long)f);
  }
  m->adjoff.assign(m->nents + 1, 0);
  m->adjind.assign(2 * m->ne + 4 * m->nf + 6 * m->nr, 0);
  m->adjperm.assign(m->adjind.size(), 0);
  int64_t a = 0;
  for (int64_t e = 0; e < m->ne; e++) {
    m->adjoff[E0 + e] = (int32_t)a;
    m->adjind[a++] = (int32_t)m->econn[2 * e];
    m->adjind[a++] = (int32_t)m->econn[2 * e + 1];
  }
  for (int64_t f = 0; f < m->nf; f++) {
    m->adjoff[F0 + f] = (int32_t)a;
    const int64_t *fv = &m->fconn[4 * f];
    for (int s = 0; s < 4; s++) {
      const int64_t v0 = fv[kQuadEdge[s][0]], v1 = fv[kQuadEdge[s][1]];
      auto it = edge_of.find(std::make_pair(std::min(v0, v1), std::max(v0, v1)));
      if (it == edge_of.end()) return set_error("no edge on side %d of face %lld", s, (long long)f);
      m->adjind[a] = (int32_t)(E0 + it->second);
      m->adjperm[a++] = m->econn[2 * it->second] == v0 ? 0 : 1;
    }
  }
  for (int64_t r = 0; r < m->nr; r++) {
    m->adjoff[R0 + r] = (int32_t)a;
    const int64_t *rv = &m->hconn[8 * r];
    for (int s = 0; s < 6; s++) {
      std::array<int64_t, 4> k = {rv[kHexFace[s][0]], rv[kHexFace[s][1]], rv[kHexFace[s][2]], rv[kHexFace[s][3]]};
      std::sort(k.begin(), k.end());
      auto it = face_of.find(k);
      if (it == face_of.end()) return set_error("no face on side %d of region %lld", s, (long long)r);
      const int64_t *fv = &m->fconn[4 * it->second];
      int perm = -1;
      for (int t = 0; t < 8 && perm < 0; t++) {
        bool match = true;
        for (int c = 0; c < 4; c++) match = match && fv[kQuadPerm[t][c]] == rv[kHexFace[s][c]];
        if (match) perm = t;
      }
      if (perm < 0) return set_error("face %lld is not a rotation or reflection of side %d of region %lld", (long long)it->second, s, (long long)r);
      m->adjind[a] = (int32_t)(F0 + it->second);
      m->adjperm[a++] = perm;
    }
  }
  m->adjoff[m->nents] = (int32_t)a;
  return 0;
}

inline int dirv(const Ord &o, int d) { return d == 0 ? o.x : d == 1 ? o.y : o.z; }

// index into the interior of a face with orientation perm (dGeomPermQuadIndex, tensor.c:328-345)
inline int perm_quad_index(int perm, int M, int N, int i, int j) {
  switch (perm) {
    case 0: return i * N + j;
    case 1: return (M - 1 - i) + j * M;
    case 2: return (M - 1 - i) * N + (N - 1 - j);
    case 3: return i + (N - 1 - j) * M;
    case 4: return i + j * M;
    case 5: return (M - 1 - i) * N + j;
    case 6: return (M - 1 - i) + (N - 1 - j) * M;
    default: return i * N + (N - 1 - j);
  }
}

}  // namespace

// Interpolation rows for p-nonconforming entities (extension of dJacobiAddConstraints_Tensor, which
// errors at tensor.c:417). An edge of degree q carries the polynomial through its q+1 GLL nodes (vertex,
// q-1 interior dofs in the edge direction, vertex); a face of degree q the tensor polynomial through its
// (q+1)^2 GLL grid in its own frame (u along fv0->fv1, v along fv0->fv3): corners are the vertices, the
// boundary the edge polynomials, the interior its dofs. An element node on a lower-degree edge or face
// takes that polynomial's value at the node; rows keep their columns ascending, weights |w| < 1e-14 (exact
// zeros of the Lagrange weights at coinciding nodes) are dropped.
struct HpRows {
  double gll[MAXP + 1][MAXP + 1];
  std::vector<int64_t> row;                 // expanded row of each constrained row
  std::vector<int64_t> ptr{0};              // entries of constrained row k: ptr[k]..ptr[k+1]
  std::vector<int32_t> col;
  std::vector<double> w;
};

struct Acc {
  int n = 0;
  int32_t c[2048];
  double w[2048];
  void add(int32_t col, double v) {
    for (int i = 0; i < n; i++)
      if (c[i] == col) {
        w[i] += v;
        return;
      }
    c[n] = col;
    w[n] = v;
    n++;
  }
};

static void gll_weights(const HpRows &h, int q, double t, double *L) {
  for (int j = 0; j <= q; j++) {
    long double v = 1;
    for (int k = 0; k <= q; k++)
      if (k != j) v *= ((long double)t - h.gll[q][k]) / ((long double)h.gll[q][j] - h.gll[q][k]);
    L[j] = (double)v;
  }
}

static void edge_value(const _p_dMesh *m, const std::vector<Ord> &deg, const std::vector<int32_t> &loff, const HpRows &h,
                       int32_t edge, double t, double scale, Acc &a) {
  const int q = deg[edge].x;
  const int64_t *ev = &m->econn[2 * (edge - m->nv)];
  double L[MAXP + 1];
  gll_weights(h, q, t, L);
  for (int k = 0; k <= q; k++) a.add(k == 0 ? loff[ev[0]] : k == q ? loff[ev[1]] : loff[edge] + (k - 1), scale * L[k]);
}

static void face_value(const _p_dMesh *m, const std::vector<Ord> &deg, const std::vector<int32_t> &loff, const HpRows &h,
                       int32_t face, double u, double v, Acc &a) {
  const int qu = deg[face].x, qv = deg[face].y;
  const int64_t *fv = &m->fconn[4 * (face - m->nv - m->ne)];
  double Lu[MAXP + 1], Lv[MAXP + 1];
  gll_weights(h, qu, u, Lu);
  gll_weights(h, qv, v, Lv);
  for (int r = 0; r <= qu; r++)
    for (int c = 0; c <= qv; c++) {
      const double w = Lu[r] * Lv[c];
      const bool bu = r == 0 || r == qu, bv = c == 0 || c == qv;
      if (bu && bv) {
        a.add(loff[fv[r == 0 ? (c == 0 ? 0 : 3) : (c == 0 ? 1 : 2)]], w);
      } else if (!bu && !bv) {
        a.add(loff[face] + (r - 1) * (qv - 1) + (c - 1), w);
      } else {
        int side;
        double tau;
        if (c == 0) side = 0, tau = h.gll[qu][r];
        else if (r == qu) side = 1, tau = h.gll[qv][c];
        else if (c == qv) side = 2, tau = -h.gll[qu][r];
        else side = 3, tau = -h.gll[qv][c];
        const int32_t slot = m->adjoff[face] + side;
        edge_value(m, deg, loff, h, m->adjind[slot], m->adjperm[slot] == 0 ? tau : -tau, w, a);
      }
    }
}

static void push_hp_row(HpRows &h, int64_t row, Acc &a) {
  // ascending columns
  for (int i = 1; i < a.n; i++)
    for (int j = i; j > 0 && a.c[j - 1] > a.c[j]; j--) {
      std::swap(a.c[j - 1], a.c[j]);
      std::swap(a.w[j - 1], a.w[j]);
    }
  h.row.push_back(row);
  for (int i = 0; i < a.n; i++)
    if (fabs(a.w[i]) >= 1e-14) {
      h.col.push_back(a.c[i]);
      h.w.push_back(a.w[i]);
    }
  h.ptr.push_back((int64_t)h.col.size());
}

// element-face traversal coordinates (s,t) to the face frame (u,v) for the 8 orientations of
// dGeomPermQuadIndex (tensor.c:328-345)
static void face_frame(int perm, double s, double t, double &u, double &v) {
  switch (perm) {
    case 0: u = s, v = t; break;
    case 1: u = t, v = -s; break;
    case 2: u = -s, v = -t; break;
    case 3: u = -t, v = s; break;
    case 4: u = t, v = s; break;
    case 5: u = -s, v = t; break;
    case 6: u = -t, v = -s; break;
    default: u = s, v = -t; break;
  }
}

// E rows of one hex (tensor.c:360-468). loff: closure offset of every entity. hp: interpolation rows for
// lower-degree edges/faces (NULL: error as the reference).
static dErr fill_element_map(const _p_dMesh *m, const std::vector<Ord> &deg, const std::vector<int32_t> &loff,
                             int64_t r, int32_t xs, int32_t *row, HpRows *hp) {
  // which face/edge-of-face pairs meet at each hex edge, with edge orientation (tensor.c:380-383)
  static const int FE[12][2][3] = {{{0, 0, 0}, {4, 3, 1}}, {{1, 0, 0}, {4, 2, 1}}, {{2, 0, 0}, {4, 1, 1}}, {{3, 0, 0}, {4, 0, 1}},
                                   {{0, 2, 1}, {5, 0, 0}}, {{1, 2, 1}, {5, 1, 0}}, {{2, 2, 1}, {5, 2, 0}}, {{3, 2, 1}, {5, 3, 0}},
                                   {{0, 3, 1}, {3, 1, 0}}, {{0, 1, 0}, {1, 3, 1}}, {{1, 1, 0}, {2, 3, 1}}, {{2, 1, 0}, {3, 3, 1}}};
  static const int IPERM[8][4] = {{0, 1, 2, 3}, {3, 0, 1, 2}, {2, 3, 0, 1}, {1, 2, 3, 0}, {3, 2, 1, 0}, {0, 3, 2, 1}, {1, 0, 3, 2}, {2, 1, 0, 3}};
  static const int EV[8][3][2] = {{{0, 0}, {3, 1}, {8, 0}}, {{0, 1}, {1, 0}, {9, 0}}, {{1, 1}, {2, 0}, {10, 0}}, {{2, 1}, {3, 0}, {11, 0}},
                                  {{4, 0}, {7, 1}, {8, 1}}, {{4, 1}, {5, 0}, {9, 1}}, {{5, 1}, {6, 0}, {10, 1}}, {{6, 1}, {7, 0}, {11, 1}}};
  const int32_t *aI = m->adjind.data(), *aO = m->adjoff.data(), *aP = m->adjperm.data();
  const int64_t ei = m->nv + m->ne + m->nf + r;
  const int d0 = deg[ei].x + 1, d1 = deg[ei].y + 1, d2 = deg[ei].z + 1, d[3] = {d0, d1, d2}, scan[3] = {d1 * d2, d2, 1};
  const int32_t *f = aI + aO[ei], *fP = aP + aO[ei];
  int e[12], eP[12], v[8];
  for (int i = 0; i < 12; i++) {
    int ent[2], ori[2];
    for (int s = 0; s < 2; s++) {
      const int fa = FE[i][s][0], slot = aO[f[fa]] + IPERM[fP[fa]][FE[i][s][1]];
      ent[s] = aI[slot];
      ori[s] = aP[slot] ^ (((fP[fa] >> 2) & 1) ^ FE[i][s][2]);
    }
    if (ent[0] != ent[1]) return set_error("faces disagree about edge %d of region %lld", i, (long long)r);
    if (ori[0] != ori[1]) return set_error("edge orientations disagree on region %lld", (long long)r);
    e[i] = ent[0];
    eP[i] = ori[0];
  }
  for (int i = 0; i < 8; i++) {
    int vv[3];
    for (int s = 0; s < 3; s++) {
      const int E = EV[i][s][0], end = EV[i][s][1];
      vv[s] = aI[aO[e[E]] + (eP[E] ? 1 - end : end)];
    }
    if (vv[0] != vv[1] || vv[0] != vv[2]) return set_error("edges disagree about vertex %d of region %lld", i, (long long)r);
    v[i] = vv[0];
  }
  auto at = [&](int a, int b, int c) -> int32_t & { return row[xs + (a * d1 + b) * d2 + c]; };
  const int T[8][3] = {{0, 0, 0}, {d0 - 1, 0, 0}, {d0 - 1, d1 - 1, 0}, {0, d1 - 1, 0}, {0, 0, d2 - 1}, {d0 - 1, 0, d2 - 1}, {d0 - 1, d1 - 1, d2 - 1}, {0, d1 - 1, d2 - 1}};
  for (int i = 0; i < 8; i++) at(T[i][0], T[i][1], T[i][2]) = loff[v[i]];
  // hex edge traversal: start node, varying direction, step, end (tensor.c:413-416)
  const int ES[12][6] = {{1, 0, 0, 0, 1, d0 - 1},          {d0 - 1, 1, 0, 1, 1, d1 - 1},          {d0 - 2, d1 - 1, 0, 0, -1, 0},
                         {0, d1 - 2, 0, 1, -1, 0},          {1, 0, d2 - 1, 0, 1, d0 - 1},          {d0 - 1, 1, d2 - 1, 1, 1, d1 - 1},
                         {d0 - 2, d1 - 1, d2 - 1, 0, -1, 0}, {0, d1 - 2, d2 - 1, 1, -1, 0},        {0, 0, 1, 2, 1, d2 - 1},
                         {d0 - 1, 0, 1, 2, 1, d2 - 1},      {d0 - 1, d1 - 1, 1, 2, 1, d2 - 1},    {0, d1 - 1, 1, 2, 1, d2 - 1}};
  for (int i = 0; i < 12; i++) {
    const int *s = ES[i], dir = s[3], inc = s[4], end = s[5];
    if (deg[e[i]].x != d[dir] - 1) {
      if (!hp) return set_error("degree does not agree, p-nonconforming (region %lld edge %d)", (long long)r, i);
      for (int j = s[dir]; j != end; j += inc) {
        const int64_t rw = xs + (s[0] * d1 + s[1]) * d2 + s[2] + (j - s[dir]) * scan[dir];
        const double tau = inc * hp->gll[d[dir] - 1][j];
        Acc a;
        edge_value(m, deg, loff, *hp, e[i], eP[i] == 0 ? tau : -tau, 1.0, a);
        row[rw] = -2;
        push_hp_row(*hp, rw, a);
      }
      continue;
    }
    for (int j = s[dir]; j != end; j += inc) {
      const int t = (j - s[dir]) / inc, ne = d[dir] - 2;
      const int32_t col = eP[i] == 0 ? loff[e[i]] + t : loff[e[i]] + (ne - 1 - t);
      row[xs + (s[0] * d1 + s[1]) * d2 + s[2] + (j - s[dir]) * scan[dir]] = col;
    }
  }
  // hex face traversal: start node, two varying directions, steps, ends (tensor.c:432-436)
  const int FS[6][9] = {{1, 0, 1, 0, 2, 1, 1, d0 - 1, d2 - 1},     {d0 - 1, 1, 1, 1, 2, 1, 1, d1 - 1, d2 - 1},
                        {d0 - 2, d1 - 1, 1, 0, 2, -1, 1, 0, d2 - 1}, {0, d1 - 2, 1, 1, 2, -1, 1, 0, d2 - 1},
                        {1, 1, 0, 1, 0, 1, 1, d1 - 1, d0 - 1},     {1, 1, d2 - 1, 0, 1, 1, 1, d0 - 1, d1 - 1}};
  for (int i = 0; i < 6; i++) {
    const int *s = FS[i], da = s[3], db = s[4], ia = s[5], ib = s[6];
    const int M = d[da] - 2, N = d[db] - 2;
    if (deg[f[i]].x != d[da] - 1 || deg[f[i]].y != d[db] - 1) {
      if (!hp) return set_error("degree does not agree, p-nonconforming (region %lld face %d)", (long long)r, i);
      for (int j = s[da]; j != s[7]; j += ia)
        for (int k = s[db]; k != s[8]; k += ib) {
          const int64_t rw = xs + (s[0] * d1 + s[1]) * d2 + s[2] + (j - s[da]) * scan[da] + (k - s[db]) * scan[db];
          double u, v;
          face_frame(fP[i], ia * hp->gll[d[da] - 1][j], ib * hp->gll[d[db] - 1][k], u, v);
          Acc a;
          face_value(m, deg, loff, *hp, f[i], u, v, a);
          row[rw] = -2;
          push_hp_row(*hp, rw, a);
        }
      continue;
    }
    for (int j = s[da]; j != s[7]; j += ia)
      for (int k = s[db]; k != s[8]; k += ib) {
        const int fi = perm_quad_index(fP[i], M, N, (j - s[da]) / ia, (k - s[db]) / ib);
        row[xs + (s[0] * d1 + s[1]) * d2 + s[2] + (j - s[da]) * scan[da] + (k - s[db]) * scan[db]] = loff[f[i]] + fi;
      }
  }
  for (int a = 1; a < d0 - 1; a++)
    for (int b = 1; b < d1 - 1; b++)
      for (int c = 1; c < d2 - 1; c++) at(a, b, c) = loff[ei] + ((a - 1) * (d1 - 2) + (b - 1)) * (d2 - 2) + (c - 1);
  return 0;
}

dErr fs_build_space(_p_dFS *fs) {
  const _p_dMesh *m = fs->mesh;
  const int64_t E0 = m->nv, F0 = m->nv + m->ne, R0 = F0 + m->nf;
  int maxdeg = fs->degree;
  const bool per_elem = !fs->elem_degree_in.empty();
  if (per_elem) {
    if ((int64_t)fs->elem_degree_in.size() != m->nr) return set_error("elem_degree has %zu entries, mesh has %lld regions", fs->elem_degree_in.size(), (long long)m->nr);
    maxdeg = *std::max_element(fs->elem_degree_in.begin(), fs->elem_degree_in.end());
  }
  if (maxdeg < 1 || maxdeg > MAXP - 1) return set_error("degree %d out of range [1,%d]", maxdeg, MAXP - 1);
  if (!m->structured && (fs->dirichlet_mask || fs->weak_mask))
    return set_error("boundary sets are those of the block generator: a mesh from connectivity has none");
  // isotropic degree tag then min-rule propagation (tables as tensor.c:201-204)
  std::vector<Ord> deg(m->nents);
  for (int64_t v = 0; v < m->nv; v++) deg[v] = {0, 0, 0};
  for (int64_t e = 0; e < m->ne; e++) deg[E0 + e] = {maxdeg, 0, 0};
  for (int64_t f = 0; f < m->nf; f++) deg[F0 + f] = {maxdeg, maxdeg, 0};
  for (int64_t r = 0; r < m->nr; r++) {
    const int p = per_elem ? fs->elem_degree_in[r] : fs->degree;
    if (p < 1 || p > MAXP - 1) return set_error("element %lld degree %d out of range", (long long)r, p);
    deg[R0 + r] = {p, p, p};
  }
  static const int HEXAXIS[6][2] = {{0, 2}, {1, 2}, {0, 2}, {1, 2}, {1, 0}, {0, 1}};
  static const int ORIENT[8][2] = {{0, 1}, {1, 0}, {0, 1}, {1, 0}, {1, 0}, {0, 1}, {1, 0}, {0, 1}};
  static const int QUADAXIS[4] = {0, 1, 0, 1};
  for (int64_t r = 0; r < m->nr; r++) {
    const int64_t e = R0 + r;
    for (int i = 0; i < 6; i++) {
      const int ai = m->adjoff[e] + i, f = m->adjind[ai], t = m->adjperm[ai];
      deg[f] = {std::min(deg[f].x, dirv(deg[e], HEXAXIS[i][ORIENT[t][0]])), std::min(deg[f].y, dirv(deg[e], HEXAXIS[i][ORIENT[t][1]])), 0};
    }
  }
  for (int64_t f = 0; f < m->nf; f++)
    for (int i = 0; i < 4; i++) {
      const int ed = m->adjind[m->adjoff[F0 + f] + i];
      deg[ed] = {std::min(deg[ed].x, dirv(deg[F0 + f], QUADAXIS[i])), 0, 0};
    }
  // explicit / Dirichlet partition (sets 0..3 -> 100, 5 -> 200, 4 -> 300) and natural ordering
  const int setbit[6] = {0, 0, 0, 0, 2, 1};
  std::vector<int32_t> inodes(m->nents), loff(m->nents);
  std::vector<char> isdir(m->nents);
  for (int64_t i = 0; i < m->nents; i++) {
    const int s = m->fset[i];
    isdir[i] = s >= 0 && ((fs->dirichlet_mask >> setbit[s]) & 1);
    const Ord o = deg[i];
    if (i < E0) inodes[i] = 1;
    else if (i < F0) inodes[i] = std::max(0, o.x - 1);
    else if (i < R0) inodes[i] = std::max(0, o.x - 1) * std::max(0, o.y - 1);
    else inodes[i] = std::max(0, o.x - 1) * std::max(0, o.y - 1) * std::max(0, o.z - 1);
  }
  int64_t scan = 0;
  for (int pass = 0; pass < 2; pass++)
    for (int64_t i = 0; i < m->nents; i++)
      if (isdir[i] == pass) {
        loff[i] = (int32_t)scan;
        scan += inodes[i];
      }
  fs->nc = scan;
  fs->n = 0;
  for (int64_t i = 0; i < m->nents; i++)
    if (!isdir[i]) fs->n += inodes[i];
  if (fs->nc > INT32_MAX / 4) return set_error("space too large for 32-bit indices");
  // elements, expanded offsets, E
  fs->nelem = m->nr;
  fs->xstart.assign(m->nr + 1, 0);
  fs->edeg.assign(3 * m->nr, 0);
  fs->qoff.assign(m->nr + 1, 0);
  fs->uniform = true;
  fs->p = deg[R0].x;
  {  // expanded nodes (and Gauss points) times the block size are indexed in 32 bits
    int64_t ne = 0;
    for (int64_t r = 0; r < m->nr; r++) {
      const Ord o = deg[R0 + r];
      ne += (int64_t)(o.x + 1) * (o.y + 1) * (o.z + 1);
    }
    if (ne * std::max(fs->bs, 1) > INT32_MAX)
      return set_error("space too large for 32-bit indices: %lld expanded values", (long long)(ne * std::max(fs->bs, 1)));
  }
  for (int64_t r = 0; r < m->nr; r++) {
    const Ord o = deg[R0 + r];
    fs->edeg[3 * r] = o.x, fs->edeg[3 * r + 1] = o.y, fs->edeg[3 * r + 2] = o.z;
    if (o.x != fs->p || o.y != fs->p || o.z != fs->p) fs->uniform = false;
    fs->xstart[r + 1] = fs->xstart[r] + (o.x + 1) * (o.y + 1) * (o.z + 1);
    fs->qoff[r + 1] = fs->qoff[r] + (o.x + 1) * (o.y + 1) * (o.z + 1);  // FAST rule: p+1 Gauss points per direction
  }
  fs->nexp = fs->xstart[m->nr];
  fs->nq = fs->qoff[m->nr];
  fs->emap.assign(fs->nexp, -1);
  HpRows hp;
  for (int q = 1; q <= MAXP; q++) {
    double w[MAXP + 1];
    lobatto_rule(q + 1, hp.gll[q], w);
  }
  for (int64_t r = 0; r < m->nr; r++) DCHK(fill_element_map(m, deg, loff, r, fs->xstart[r], fs->emap.data(), per_elem ? &hp : nullptr));
  for (int64_t i = 0; i < fs->nexp; i++)
    if (fs->emap[i] == -1) return set_error("expanded node %lld has no constraint", (long long)i);
  // E as CSR over expanded rows
  fs->boolean_e = hp.row.empty();
  fs->eptr.assign(fs->nexp + 1, 0);
  {
    std::vector<int64_t> which(fs->nexp, -1);
    for (size_t k = 0; k < hp.row.size(); k++) which[hp.row[k]] = (int64_t)k;
    int64_t nnz = 0;
    for (int64_t i = 0; i < fs->nexp; i++) nnz += which[i] < 0 ? 1 : hp.ptr[which[i] + 1] - hp.ptr[which[i]];
    if (nnz > INT32_MAX) return set_error("E has too many entries");
    fs->ecol.resize(nnz);
    fs->eval.resize(nnz);
    int64_t o = 0;
    for (int64_t i = 0; i < fs->nexp; i++) {
      fs->eptr[i] = (int32_t)o;
      if (which[i] < 0) {
        fs->ecol[o] = fs->emap[i];
        fs->eval[o] = 1.0;
        o++;
      } else {
        for (int64_t t = hp.ptr[which[i]]; t < hp.ptr[which[i] + 1]; t++, o++) fs->ecol[o] = hp.col[t], fs->eval[o] = hp.w[t];
      }
    }
    fs->eptr[fs->nexp] = (int32_t)o;
  }
  return 0;
}

// ---------------------------------------------------------------------------------------------------- C ABI
extern "C" {

dErr dMeshCreateBlock(const dInt npoints[3], const dReal box[6], dReal perturb, uint64_t seed, dMesh *mesh) {
  if (!mesh || !npoints || !box) return set_error("dMeshCreateBlock: null argument");
  *mesh = nullptr;
  if (npoints[0] < 2 || npoints[1] < 2 || npoints[2] < 2) return set_error("need at least 2 vertices per direction");
  if ((double)npoints[0] * npoints[1] * npoints[2] > 2e8) return set_error("mesh too large");
  _p_dMesh *m = new _p_dMesh();
  m->nx = npoints[0], m->ny = npoints[1], m->nz = npoints[2];
  dErr e = mesh_build(m, box, perturb, seed);
  if (!e) e = mesh_adjacency(m);
  if (e) {
    delete m;
    return e;
  }
  *mesh = m;
  return 0;
}

dErr dMeshCreateFromConnectivity(dInt nv, const dReal *vtx, dInt ne, const dInt *econn, dInt nf, const dInt *fconn, dInt nr,
                                 const dInt *hconn, dMesh *mesh) {
  if (!mesh || !vtx || (ne && !econn) || (nf && !fconn) || !hconn) return set_error("dMeshCreateFromConnectivity: null argument");
  *mesh = nullptr;
  if (nv < 8 || ne < 12 || nf < 6 || nr < 1) return set_error("dMeshCreateFromConnectivity: a hexahedral mesh needs its vertices, edges, faces and regions");
  const struct { dInt n, k; const dInt *c; } lists[3] = {{ne, 2, econn}, {nf, 4, fconn}, {nr, 8, hconn}};
  for (const auto &l : lists)
    for (int64_t i = 0; i < (int64_t)l.n * l.k; i++)
      if (l.c[i] < 0 || l.c[i] >= nv) return set_error("dMeshCreateFromConnectivity: vertex %d out of range [0,%d)", l.c[i], nv);
  _p_dMesh *m = new _p_dMesh();
  m->structured = false;
  m->nx = m->ny = m->nz = 0;
  m->nv = nv, m->ne = ne, m->nf = nf, m->nr = nr;
  m->nents = (int64_t)nv + ne + nf + nr;
  m->vx.assign(vtx, vtx + 3 * (size_t)nv);
  m->econn.assign(econn, econn + 2 * (size_t)ne);
  m->fconn.assign(fconn, fconn + 4 * (size_t)nf);
  m->hconn.assign(hconn, hconn + 8 * (size_t)nr);
  m->fset.assign(m->nents, -1);  // no boundary sets
  dErr e = mesh_adjacency_general(m);
  if (e) {
    delete m;
    return e;
  }
  *mesh = m;
  return 0;
}

dErr dMeshGetAdjacency(dMesh m, dInt toff[5], const dInt **adjoff, const dInt **adjind, const dInt **adjperm) {
  if (!m) return set_error("null mesh");
  if (toff) toff[0] = 0, toff[1] = (dInt)m->nv, toff[2] = (dInt)(m->nv + m->ne), toff[3] = (dInt)(m->nv + m->ne + m->nf), toff[4] = (dInt)m->nents;
  if (adjoff) *adjoff = m->adjoff.data();
  if (adjind) *adjind = m->adjind.data();
  if (adjperm) *adjperm = m->adjperm.data();
  return 0;
}

dErr dMeshDestroy(dMesh *mesh) {
  if (mesh && *mesh) {
    delete *mesh;
    *mesh = nullptr;
  }
  return 0;
}

dErr dMeshGetNumEnts(dMesh m, dInt counts[4]) {
  if (!m) return set_error("null mesh");
  counts[0] = (dInt)m->nv, counts[1] = (dInt)m->ne, counts[2] = (dInt)m->nf, counts[3] = (dInt)m->nr;
  return 0;
}

}  // extern "C"

namespace {

// the coordinates of every expanded node: the element's trilinear map (its 8 vertices in tensor order, as the
// coordinate space holds them, fsgeom.c:151) at its GLL nodes, [nexp][3] (dFSGetNodalCoordinatesExpanded,
// fsgeom.c:17-58, which applies the coordinate space's INTERP on the Lobatto nodes of each element's degree)
void nodal_coordinates_expanded(const _p_dFS *fs, std::vector<double> &out) {
  static const int kConn[8] = {0, 4, 3, 7, 1, 5, 2, 6};
  const _p_dMesh *m = fs->mesh;
  out.assign(3 * (size_t)fs->nexp, 0.0);
  for (int64_t r = 0; r < fs->nelem; r++) {
    const int P[3] = {fs->edeg[3 * r] + 1, fs->edeg[3 * r + 1] + 1, fs->edeg[3 * r + 2] + 1};
    double node[3][MAXP], w[MAXP];
    for (int d = 0; d < 3; d++) lobatto_rule(P[d], node[d], w);
    double X[8][3];
    for (int v = 0; v < 8; v++)
      for (int c = 0; c < 3; c++) X[v][c] = m->vx[3 * m->hconn[8 * r + kConn[v]] + c];
    int64_t row = fs->xstart[r];
    for (int a = 0; a < P[0]; a++)
      for (int b = 0; b < P[1]; b++)
        for (int cc = 0; cc < P[2]; cc++, row++) {
          const double t[3] = {node[0][a], node[1][b], node[2][cc]};
          double L[3][2];
          for (int d = 0; d < 3; d++) L[d][0] = 0.5 * (1 - t[d]), L[d][1] = 0.5 * (1 + t[d]);
          for (int c = 0; c < 3; c++) {
            double s = 0;
            for (int v = 0; v < 8; v++) s += L[0][v >> 2] * L[1][(v >> 1) & 1] * L[2][v & 1] * X[v][c];
            out[3 * row + c] = s;
          }
        }
  }
}

dErr copy_out(const std::vector<double> &h, dReal *coords, int on_device) {
  if (on_device) CUCHK(cudaMemcpy(coords, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
  else std::copy(h.begin(), h.end(), coords);
  return 0;
}

}  // namespace

extern "C" {

dErr dFSGetNodalCoordinatesExpanded(dFS fs, dReal *coords, int on_device) {
  if (!fs || !coords) return set_error("null argument");
  if (!fs->built) return set_error("dFS space not built");
  std::vector<double> h;
  nodal_coordinates_expanded(fs, h);
  return copy_out(h, coords, on_device);
}

// dFSGetNodalCoordinatesGlobal (fsgeom.c:72-107): every closure node's coordinates, the mean over its expanded
// copies (E^T of the expanded coordinates over E^T of ones); rows of E that interpolate (hp constraints) are not
// nodes of the closure and are skipped
dErr dFSGetNodalCoordinatesGlobal(dFS fs, dReal *coords, int on_device) {
  if (!fs || !coords) return set_error("null argument");
  if (!fs->built) return set_error("dFS space not built");
  std::vector<double> x, g(3 * (size_t)fs->nc, 0.0), count(fs->nc, 0.0);
  nodal_coordinates_expanded(fs, x);
  for (int64_t row = 0; row < fs->nexp; row++) {
    const int32_t c = fs->emap[row];
    if (c < 0) continue;
    count[c] += 1;
    for (int d = 0; d < 3; d++) g[3 * (size_t)c + d] += x[3 * row + d];
  }
  for (int64_t c = 0; c < fs->nc; c++)
    for (int d = 0; d < 3; d++) g[3 * c + d] /= count[c];
  return copy_out(g, coords, on_device);
}

// dFSGetSubElementMeshSize_Cont (cont.c:387-415): px py pz hexahedral sub-cells per element, the closure nodes as
// vertices, 8 vertices per sub-cell
dErr dFSGetSubElementMeshSize(dFS fs, dInt *nelems, dInt *nverts, dInt *nconn) {
  if (!fs || !nelems || !nverts || !nconn) return set_error("null argument");
  if (!fs->built) return set_error("dFS space not built");
  int64_t nsub = 0;
  for (int64_t r = 0; r < fs->nelem; r++) nsub += (int64_t)fs->edeg[3 * r] * fs->edeg[3 * r + 1] * fs->edeg[3 * r + 2];
  if (8 * nsub > INT32_MAX) return set_error("sub-element mesh too large for 32-bit sizes");
  *nelems = (dInt)nsub;
  *nverts = (dInt)fs->nc;
  *nconn = (dInt)(8 * nsub);
  return 0;
}

// dFSGetSubElementMesh_Cont (cont.c:417-470): the sub-cells of each element in its SPARSE patch order (x-major), each
// as 8 closure nodes in ITAPS hexahedron order (the tensor corners {0,4,6,2,1,5,7,3}); E must be Boolean there
dErr dFSGetSubElementMesh(dFS fs, dInt nelems, dInt nconn, dEntTopology topo[], dInt off[], dInt ind[]) {
  if (!fs || !topo || !off || !ind) return set_error("null argument");
  dInt ns, nv, nc;
  DCHK(dFSGetSubElementMeshSize(fs, &ns, &nv, &nc));
  if (nelems < ns || nconn < nc) return set_error("Insufficient preallocation for the sub-element mesh (%d, %d needed)", ns, nc);
  static const int kItapsToTensor[8] = {0, 4, 6, 2, 1, 5, 7, 3};
  int64_t sub = 0, subc = 0;
  for (int64_t r = 0; r < fs->nelem; r++) {
    const int px = fs->edeg[3 * r], py = fs->edeg[3 * r + 1], pz = fs->edeg[3 * r + 2];
    for (int i = 0; i < px; i++)
      for (int j = 0; j < py; j++)
        for (int k = 0; k < pz; k++, sub++) {
          topo[sub] = dTOPO_HEX;
          off[sub] = (dInt)subc;
          for (int v = 0; v < 8; v++, subc++) {
            const int t = kItapsToTensor[v], bi = t >> 2, bj = (t >> 1) & 1, bk = t & 1;
            const int64_t row = fs->xstart[r] + ((int64_t)(i + bi) * (py + 1) + j + bj) * (pz + 1) + k + bk;
            if (fs->emap[row] < 0) return set_error("Element assembly matrix is not boolean (row %lld)", (long long)row);
            ind[subc] = fs->emap[row];
          }
        }
  }
  off[sub] = (dInt)subc;
  return 0;
}

}  // extern "C"

extern "C" dErr dFSGetElementAssemblyMatrix(dFS fs, int64_t *nnz, dInt *rowptr, dInt *col, dReal *val) {
  if (!fs || !fs->built) return set_error("dFS space not built");
  if (nnz) *nnz = (int64_t)fs->ecol.size();
  if (rowptr) memcpy(rowptr, fs->eptr.data(), fs->eptr.size() * sizeof(dInt));
  if (col) memcpy(col, fs->ecol.data(), fs->ecol.size() * sizeof(dInt));
  if (val) memcpy(val, fs->eval.data(), fs->eval.size() * sizeof(double));
  return 0;
}
