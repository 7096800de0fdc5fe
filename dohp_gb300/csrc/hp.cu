// hp (mixed-order) operator apply.
//
// Elements are bucketed by order (p = 1..8, isotropic). Each element gathers its nodal values through the
// interpolation-constrained E (CSR rows of weights; Boolean rows for conforming nodes), runs the same
// sum-factorized element kernel as the uniform path for its order (interpolate to Gauss points, collocation
// gradient, q-function, transposes; see operator.cu), and writes its expanded output; the weighted E^T
// restriction sums contributions per closure node in ascending expanded order (deterministic).
// Launch forms:
//   dLAUNCH_PER_ORDER : one launch per order bucket (plain)
//   dLAUNCH_PERSISTENT: one launch over all buckets; blocks take (bucket, element group) work items from a
//                       device counter in descending order cost; each item is processed by exactly one block,
//                       so results are bitwise identical to the per-order form
//   dLAUNCH_GRAPH     : the persistent launch and the restriction replayed from a CUDA graph; x and y are
//                       passed through a small device pointer table so one graph serves every call
// Tile sizes (elements per block, threads per block) come from a measured autotuner per (kind, order,
// precision), optionally persisted as JSON.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <sstream>

#include "element.cuh"

using namespace dgb;

dErr op_compute_geometry(_p_dOperator *op);
dErr fs_restrict(_p_dFS *fs, const double *x, double *g, int add);
dErr fs_restrict32(_p_dFS *fs, const float *x, double *g, int add);
dErr fs_restrict_ff(_p_dFS *fs, const ff *x, double *g, int add);
dErr fs_restrict_ff_to(_p_dFS *fs, const ff *x, double *const *py, double *g, int add, cudaStream_t s);

namespace {

using HpArgs = ElemArgs;

template <int N, typename T, int KIND>
__global__ void __launch_bounds__(256) k_hp_bucket(HpArgs A, const int32_t *__restrict__ elist, int64_t count, int cap) {
  extern __shared__ unsigned char raw[];
  const int64_t g0 = (int64_t)blockIdx.x * cap;
  const int ne = (int)min((int64_t)cap, count - g0);
  group_apply<N, T, KIND>(A, elist + g0, 0, ne, cap, reinterpret_cast<T *>(raw));
}

// work item: x = nodes per direction, y = first element in elist, z = elements, w = group capacity
template <typename T, int KIND>
__global__ void __launch_bounds__(256) k_hp_persistent(HpArgs A, const int32_t *__restrict__ elist, const int4 *__restrict__ work,
                                                       int nwork, int *counter) {
  extern __shared__ unsigned char raw[];
  __shared__ int item;
  T *sm = reinterpret_cast<T *>(raw);
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = item;
    __syncthreads();
    if (it >= nwork) break;
    const int4 w = work[it];
    switch (w.x) {
      case 2: group_apply<2, T, KIND>(A, elist + w.y, 0, w.z, w.w, sm); break;
      case 3: group_apply<3, T, KIND>(A, elist + w.y, 0, w.z, w.w, sm); break;
      case 4: group_apply<4, T, KIND>(A, elist + w.y, 0, w.z, w.w, sm); break;
      case 5: group_apply<5, T, KIND>(A, elist + w.y, 0, w.z, w.w, sm); break;
      case 6: group_apply<6, T, KIND>(A, elist + w.y, 0, w.z, w.w, sm); break;
      case 7: group_apply<7, T, KIND>(A, elist + w.y, 0, w.z, w.w, sm); break;
      case 8: group_apply<8, T, KIND>(A, elist + w.y, 0, w.z, w.w, sm); break;
      case 9: group_apply<9, T, KIND>(A, elist + w.y, 0, w.z, w.w, sm); break;
    }
    __syncthreads();
  }
}

// weighted E^T restriction reading the output pointer through the table (graph form)
template <typename TI>
__global__ void k_restrict_table(int64_t n, int bs, const int32_t *__restrict__ et_ptr, const int32_t *__restrict__ et_idx,
                                 const double *__restrict__ et_w, const TI *__restrict__ x, double *const *py) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * bs) return;
  const int64_t c = t / bs;
  const int b = (int)(t - c * bs);
  double s = 0;
  for (int32_t k = et_ptr[c]; k < et_ptr[c + 1]; k++) s += (et_w ? et_w[k] : 1.0) * (double)x[(int64_t)et_idx[k] * bs + b];
  (*py)[t] = s;
}

int default_cap(int N, int kind) {
  if (kind == dOP_ELASTICITY) return N <= 3 ? 8 : N == 4 ? 4 : N == 5 ? 2 : 1;
  return N <= 2 ? 32 : N == 3 ? 16 : N == 4 ? 8 : N == 5 ? 4 : N <= 7 ? 2 : 1;
}

template <int N, typename T, int KIND>
dErr launch_bucket(const HpArgs &A, const int32_t *elist, int64_t count, int cap, int threads, cudaStream_t s) {
  if (count == 0) return 0;
  const size_t smem = (size_t)group_smem_elems(N, KIND, cap) * sizeof(T);
  CUCHK(cudaFuncSetAttribute(k_hp_bucket<N, T, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_hp_bucket<N, T, KIND><<<(unsigned)((count + cap - 1) / cap), threads, smem, s>>>(A, elist, count, cap);
  CUCHK(cudaGetLastError());
  return 0;
}

template <typename T, int KIND>
dErr launch_bucket_n(int N, const HpArgs &A, const int32_t *elist, int64_t count, int cap, int threads, cudaStream_t s) {
  switch (N) {
    case 2: return launch_bucket<2, T, KIND>(A, elist, count, cap, threads, s);
    case 3: return launch_bucket<3, T, KIND>(A, elist, count, cap, threads, s);
    case 4: return launch_bucket<4, T, KIND>(A, elist, count, cap, threads, s);
    case 5: return launch_bucket<5, T, KIND>(A, elist, count, cap, threads, s);
    case 6: return launch_bucket<6, T, KIND>(A, elist, count, cap, threads, s);
    case 7: return launch_bucket<7, T, KIND>(A, elist, count, cap, threads, s);
    case 8: return launch_bucket<8, T, KIND>(A, elist, count, cap, threads, s);
    case 9: return launch_bucket<9, T, KIND>(A, elist, count, cap, threads, s);
  }
  return set_error("order %d out of range", N - 1);
}

}  // namespace

// ---------------------------------------------------------------------------------------------------- plan
struct HpPlan {
  int nb = 0;
  int N[MAXP], cap[MAXP], threads[MAXP];
  int64_t first[MAXP], count[MAXP];
  int32_t *d_elist = nullptr;
  int4 *d_work = nullptr;
  int nwork = 0;
  int *d_counter = nullptr;
  size_t persistent_smem[2] = {0, 0};  // per precision (0: fp64, 1: fp32)
  int persistent_blocks = 0;
  bool tuned = false;
  // graph form
  const double **d_ptrs = nullptr;  // [x, y]
  cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};  // per precision (fp64, fp32, float-float)
};

static void plan_free(HpPlan *p) {
  if (!p) return;
  cudaFree(p->d_elist);
  cudaFree(p->d_work);
  cudaFree(p->d_counter);
  cudaFree((void *)p->d_ptrs);
  for (int i = 0; i < 3; i++)
    if (p->exec[i]) cudaGraphExecDestroy(p->exec[i]);
  delete p;
}

void hp_plan_destroy(void *p) { plan_free((HpPlan *)p); }

static dErr plan_work(HpPlan *P, int kind, cudaStream_t s) {
  std::vector<int4> work;
  for (int b = 0; b < P->nb; b++)
    for (int64_t g = 0; g < P->count[b]; g += P->cap[b])
      work.push_back(make_int4(P->N[b], (int)(P->first[b] + g), (int)std::min<int64_t>(P->cap[b], P->count[b] - g), P->cap[b]));
  P->nwork = (int)work.size();
  cudaFree(P->d_work);
  CUCHK(cudaMalloc(&P->d_work, std::max<size_t>(work.size(), 1) * sizeof(int4)));
  CUCHK(cudaMemcpyAsync(P->d_work, work.data(), work.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  for (int pr = 0; pr < 2; pr++) {
    size_t mx = 0;
    for (int b = 0; b < P->nb; b++) mx = std::max(mx, (size_t)group_smem_elems(P->N[b], kind, P->cap[b]) * (pr ? 4 : 8));
    P->persistent_smem[pr] = mx;
  }
  CUCHK(cudaStreamSynchronize(s));
  return 0;
}

static dErr plan_build(_p_dOperator *op) {
  _p_dFS *fs = op->fs;
  HpPlan *P = new HpPlan();
  std::vector<std::vector<int32_t>> by(MAXP + 1);
  for (int64_t e = 0; e < fs->nelem; e++) {
    const int px = fs->edeg[3 * e];
    if (fs->edeg[3 * e + 1] != px || fs->edeg[3 * e + 2] != px) {
      delete P;
      return set_error("hp apply needs isotropic element orders");
    }
    by[px + 1].push_back((int32_t)e);
  }
  std::vector<int32_t> elist;
  for (int N = MAXP; N >= 2; N--)  // descending cost first (load balance of the persistent form)
    if (!by[N].empty()) {
      const int b = P->nb++;
      P->N[b] = N;
      P->first[b] = (int64_t)elist.size();
      P->count[b] = (int64_t)by[N].size();
      P->cap[b] = default_cap(N, op->kind);
      P->threads[b] = 256;
      elist.insert(elist.end(), by[N].begin(), by[N].end());
    }
  CUCHK(cudaMalloc(&P->d_elist, std::max<size_t>(elist.size(), 1) * sizeof(int32_t)));
  CUCHK(cudaMemcpy(P->d_elist, elist.data(), elist.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  CUCHK(cudaMalloc(&P->d_counter, sizeof(int)));
  CUCHK(cudaMalloc((void **)&P->d_ptrs, 2 * sizeof(double *)));
  int dev, sms;
  CUCHK(cudaGetDevice(&dev));
  CUCHK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  P->persistent_blocks = sms;
  DCHK(plan_work(P, op->kind, fs->stream));
  op->hp_plan = P;
  return 0;
}

// geometric factors in the apply's storage type (FP32 rounding or float-float split), once per geometry
template <typename T>
__global__ void k_geo_to(int64_t n, const double *__restrict__ a, T *__restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = T(a[i]);
}

// precision index: 0 FP64, 1 FP32, 2 float-float
static int prec_index(const _p_dOperator *op) { return op->prec == dPREC_FP32 ? 1 : op->prec == dPREC_FF ? 2 : 0; }

static HpArgs make_args(_p_dOperator *op, const double *x, int pi, void *yexp, const double *const *px) {
  _p_dFS *fs = op->fs;
  HpArgs A{};
  A.xstart = fs->d_xstart;
  A.qoff = fs->d_qoff;
  A.eptr = fs->d_eptr;
  A.ecol = fs->d_ecol;
  A.eval = fs->d_eval;
  A.emap = fs->d_emap;
  A.stash = nullptr;
  A.n = fs->n;
  A.x = x;
  A.px = px;
  A.geo = pi == 1 ? (const void *)op->d_geo32 : pi == 2 ? (const void *)op->d_geoff : (const void *)op->d_geo;
  A.tab_all = fs->d_fast_tab;
  A.yexp = yexp;
  A.lam = op->lam;
  A.mu = op->mu;
  return A;
}

template <typename T>
static dErr run_per_order(_p_dOperator *op, const HpArgs &A) {
  HpPlan *P = (HpPlan *)op->hp_plan;
  for (int b = 0; b < P->nb; b++) {
    const int32_t *el = P->d_elist + P->first[b];
    if (op->kind == dOP_ELASTICITY) DCHK((launch_bucket_n<T, dOP_ELASTICITY>(P->N[b], A, el, P->count[b], P->cap[b], P->threads[b], op->fs->stream)));
    else DCHK((launch_bucket_n<T, dOP_DIFFUSION>(P->N[b], A, el, P->count[b], P->cap[b], P->threads[b], op->fs->stream)));
  }
  return 0;
}

// shared-memory attribute and grid of the persistent kernel (outside any stream capture)
template <typename T>
static dErr prepare_persistent(_p_dOperator *op, int *grid) {
  HpPlan *P = (HpPlan *)op->hp_plan;
  const size_t smem = P->persistent_smem[sizeof(T) == 4];
  int per = 1;
  if (op->kind == dOP_ELASTICITY) {
    CUCHK(cudaFuncSetAttribute(k_hp_persistent<T, dOP_ELASTICITY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUCHK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_hp_persistent<T, dOP_ELASTICITY>, 256, smem));
  } else {
    CUCHK(cudaFuncSetAttribute(k_hp_persistent<T, dOP_DIFFUSION>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUCHK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_hp_persistent<T, dOP_DIFFUSION>, 256, smem));
  }
  *grid = P->persistent_blocks * std::max(per, 1);
  return 0;
}

template <typename T>
static dErr run_persistent(_p_dOperator *op, const HpArgs &A, cudaStream_t s, int grid) {
  HpPlan *P = (HpPlan *)op->hp_plan;
  const size_t smem = P->persistent_smem[sizeof(T) == 4];
  CUCHK(cudaMemsetAsync(P->d_counter, 0, sizeof(int), s));
  if (op->kind == dOP_ELASTICITY)
    k_hp_persistent<T, dOP_ELASTICITY><<<grid, 256, smem, s>>>(A, P->d_elist, P->d_work, P->nwork, P->d_counter);
  else
    k_hp_persistent<T, dOP_DIFFUSION><<<grid, 256, smem, s>>>(A, P->d_elist, P->d_work, P->nwork, P->d_counter);
  CUCHK(cudaGetLastError());
  return 0;
}

// Measured tile choice per bucket: capacity in {c/2, c, 2c} x threads {128, 256}, 3 timed launches each.
template <typename T>
static dErr autotune(_p_dOperator *op, const HpArgs &A) {
  HpPlan *P = (HpPlan *)op->hp_plan;
  cudaStream_t s = op->fs->stream;
  cudaEvent_t e0, e1;
  CUCHK(cudaEventCreate(&e0));
  CUCHK(cudaEventCreate(&e1));
  for (int b = 0; b < P->nb; b++) {
    const int base = default_cap(P->N[b], op->kind);
    int best_cap = base, best_thr = 256;
    float best = 1e30f;
    const int caps[3] = {std::max(1, base / 2), base, base * 2};
    for (int ci = 0; ci < 3; ci++)
      for (int thr : {128, 256}) {
        const int cap = caps[ci];
        if ((size_t)group_smem_elems(P->N[b], op->kind, cap) * sizeof(T) > 160 * 1024) continue;
        const int32_t *el = P->d_elist + P->first[b];
        auto go = [&]() -> dErr {
          if (op->kind == dOP_ELASTICITY) return launch_bucket_n<T, dOP_ELASTICITY>(P->N[b], A, el, P->count[b], cap, thr, s);
          return launch_bucket_n<T, dOP_DIFFUSION>(P->N[b], A, el, P->count[b], cap, thr, s);
        };
        DCHK(go());
        CUCHK(cudaEventRecord(e0, s));
        for (int r = 0; r < 3; r++) DCHK(go());
        CUCHK(cudaEventRecord(e1, s));
        CUCHK(cudaEventSynchronize(e1));
        float ms;
        CUCHK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) best = ms, best_cap = cap, best_thr = thr;
      }
    P->cap[b] = best_cap;
    P->threads[b] = best_thr;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  P->tuned = true;
  for (int i = 0; i < 3; i++)
    if (P->exec[i]) cudaGraphExecDestroy(P->exec[i]), P->exec[i] = nullptr;
  return plan_work(P, op->kind, s);
}

static std::string tune_key(_p_dOperator *op, int N, int pi) {
  char name[256] = "gpu";
  int dev;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) snprintf(name, sizeof name, "%s", prop.name);
  for (char *c = name; *c; c++)
    if (*c == ' ' || *c == '"') *c = '_';
  std::ostringstream k;
  k << name << ":kind" << (int)op->kind << ":N" << N << ":" << (pi == 1 ? "fp32" : pi == 2 ? "ff" : "fp64");
  return k.str();
}

// JSON cache: {"key": [cap, threads], ...}
static void tune_load(_p_dOperator *op, const char *path, int pi) {
  std::ifstream f(path);
  if (!f) return;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string js = ss.str();
  HpPlan *P = (HpPlan *)op->hp_plan;
  int found = 0;
  for (int b = 0; b < P->nb; b++) {
    const std::string key = "\"" + tune_key(op, P->N[b], pi) + "\"";
    const size_t at = js.find(key);
    if (at == std::string::npos) continue;
    int cap, thr;
    if (sscanf(js.c_str() + at + key.size(), " : [%d , %d]", &cap, &thr) == 2 || sscanf(js.c_str() + at + key.size(), ": [%d, %d]", &cap, &thr) == 2) {
      if (cap >= 1 && cap <= 64 && (thr == 128 || thr == 256)) P->cap[b] = cap, P->threads[b] = thr, found++;
    }
  }
  if (found == P->nb) P->tuned = true;
}

static void tune_save(_p_dOperator *op, const char *path, int pi) {
  HpPlan *P = (HpPlan *)op->hp_plan;
  std::string js;
  {
    std::ifstream f(path);
    if (f) {
      std::stringstream ss;
      ss << f.rdbuf();
      js = ss.str();
    }
  }
  std::ostringstream o;
  o << "{\n";
  bool firstk = true;
  // keep other keys from the existing file
  size_t pos = 0;
  while ((pos = js.find('"', pos)) != std::string::npos) {
    const size_t end = js.find('"', pos + 1);
    if (end == std::string::npos) break;
    const std::string key = js.substr(pos + 1, end - pos - 1);
    const size_t lb = js.find('[', end), rb = js.find(']', end);
    if (lb == std::string::npos || rb == std::string::npos) break;
    bool ours = false;
    for (int b = 0; b < P->nb; b++) ours |= key == tune_key(op, P->N[b], pi);
    if (!ours) {
      o << (firstk ? "" : ",\n") << " \"" << key << "\": " << js.substr(lb, rb - lb + 1);
      firstk = false;
    }
    pos = rb + 1;
  }
  for (int b = 0; b < P->nb; b++) {
    o << (firstk ? "" : ",\n") << " \"" << tune_key(op, P->N[b], pi) << "\": [" << P->cap[b] << ", " << P->threads[b] << "]";
    firstk = false;
  }
  o << "\n}\n";
  std::ofstream f(path);
  f << o.str();
}

// y = A x for hp spaces (any E) in the operator's launch form and precision
dErr hp_mult(_p_dOperator *op, const double *x, double *y);

// element part only (FP64): yexp = element kernels in the per-order or persistent form, no restriction
dErr hp_mult_expanded(_p_dOperator *op, const double *x, double *yexp) {
  if (op->prec != dPREC_FP64) return set_error("expanded-output form is FP64 only");
  if (!op->hp_plan) {  // run one full apply to build the plan, geometry and tiles
    double *tmp;
    CUCHK(cudaMalloc(&tmp, std::max<int64_t>(op->fs->n * op->fs->bs, 1) * sizeof(double)));
    const dLaunchMode save = op->launch;
    if (op->launch == dLAUNCH_GRAPH) op->launch = dLAUNCH_PERSISTENT;
    const dErr e = hp_mult(op, x, tmp);
    op->launch = save;
    CUCHK(cudaStreamSynchronize(op->fs->stream));
    cudaFree(tmp);
    if (e) return e;
  }
  const HpArgs A = make_args(op, x, false, yexp, nullptr);
  if (op->launch == dLAUNCH_PER_ORDER || op->launch == dLAUNCH_DEFAULT) return run_per_order<double>(op, A);
  int grid = 0;
  DCHK(prepare_persistent<double>(op, &grid));
  return run_persistent<double>(op, A, op->fs->stream, grid);
}

dErr hp_mult(_p_dOperator *op, const double *x, double *y) {
  _p_dFS *fs = op->fs;
  if (op->kind == dOP_PLAPLACE_JACOBIAN) return set_error("hp apply for the p-Laplacian Jacobian not built yet");
  if (fs->boolean_e) {  // uniform-order spaces also run here when the caller asks for the hp forms
    if (!fs->d_eptr) {
      std::vector<int32_t> p(fs->nexp + 1);
      for (int64_t i = 0; i <= fs->nexp; i++) p[i] = (int32_t)i;
      std::vector<double> w(fs->nexp, 1.0);
      CUCHK(cudaMalloc(&fs->d_eptr, p.size() * sizeof(int32_t)));
      CUCHK(cudaMalloc(&fs->d_eval, w.size() * sizeof(double)));
      CUCHK(cudaMalloc(&fs->d_ecol, fs->nexp * sizeof(int32_t)));
      CUCHK(cudaMemcpy(fs->d_eptr, p.data(), p.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
      CUCHK(cudaMemcpy(fs->d_eval, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice));
      CUCHK(cudaMemcpy(fs->d_ecol, fs->d_emap, fs->nexp * sizeof(int32_t), cudaMemcpyDeviceToDevice));
    }
  }
  DCHK(op_compute_geometry(op));
  const int pi = prec_index(op);
  if (pi && !(pi == 1 ? op->d_geo32 : op->d_geoff)) {  // factors rounded to FP32 / split into float pairs once
    const int64_t ng = fs->nq * (op->kind == dOP_ELASTICITY ? 10 : 6);
    const unsigned g = (unsigned)std::max<int64_t>((ng + 255) / 256, 1);
    if (pi == 1) {
      CUCHK(cudaMalloc(&op->d_geo32, std::max<int64_t>(ng, 1) * sizeof(float)));
      k_geo_to<float><<<g, 256, 0, fs->stream>>>(ng, op->d_geo, (float *)op->d_geo32);
    } else {
      CUCHK(cudaMalloc(&op->d_geoff, std::max<int64_t>(ng, 1) * sizeof(ff)));
      k_geo_to<ff><<<g, 256, 0, fs->stream>>>(ng, op->d_geo, (ff *)op->d_geoff);
    }
    CUCHK(cudaGetLastError());
  }
  if (!op->hp_plan) {
    DCHK(plan_build(op));
    if (op->tune_path[0]) tune_load(op, op->tune_path, pi);
  }
  HpPlan *P = (HpPlan *)op->hp_plan;
  void *yexp;
  if (pi == 1) {
    if (!op->d_y32) CUCHK(cudaMalloc(&op->d_y32, fs->nexp * fs->bs * sizeof(float)));
    yexp = op->d_y32;
  } else if (pi == 2) {
    if (!op->d_yff) CUCHK(cudaMalloc(&op->d_yff, fs->nexp * fs->bs * sizeof(ff)));
    yexp = op->d_yff;
  } else {
    if (!op->d_yexp) CUCHK(cudaMalloc(&op->d_yexp, fs->nexp * fs->bs * sizeof(double)));
    yexp = op->d_yexp;
  }
  if (op->autotune && !P->tuned) {
    const HpArgs A = make_args(op, x, pi, yexp, nullptr);
    if (pi == 1) DCHK(autotune<float>(op, A));
    else if (pi == 2) DCHK(autotune<ff>(op, A));
    else DCHK(autotune<double>(op, A));
    if (op->tune_path[0]) tune_save(op, op->tune_path, pi);
  }
  cudaStream_t s = fs->stream;
  auto persistent = [&](const HpArgs &A, cudaStream_t st, int grid) -> dErr {
    return pi == 1 ? run_persistent<float>(op, A, st, grid) : pi == 2 ? run_persistent<ff>(op, A, st, grid) : run_persistent<double>(op, A, st, grid);
  };
  int grid = 0;
  if (op->launch == dLAUNCH_PERSISTENT || op->launch == dLAUNCH_GRAPH)
    DCHK(pi == 1 ? prepare_persistent<float>(op, &grid) : pi == 2 ? prepare_persistent<ff>(op, &grid) : prepare_persistent<double>(op, &grid));
  if (op->launch == dLAUNCH_GRAPH) {
    const double *ptrs[2] = {x, y};
    CUCHK(cudaMemcpyAsync((void *)P->d_ptrs, ptrs, sizeof ptrs, cudaMemcpyHostToDevice, s));
    cudaGraphExec_t &ex = P->exec[pi];
    if (!ex) {
      // capture on a private stream (the legacy default stream cannot be captured); the graph is then
      // launched on the operator's stream, ordered after the pointer-table copy above
      cudaStream_t cs;
      CUCHK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t g;
      CUCHK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      const HpArgs A = make_args(op, nullptr, pi, yexp, P->d_ptrs);
      dErr e = persistent(A, cs, grid);
      const int64_t N = fs->n * fs->bs;
      if (!e && N) {
        const int32_t *eti = fs->d_et_idx;
        const double *etw = fs->boolean_e ? nullptr : fs->d_et_w;
        const unsigned nbk = (unsigned)((N + 255) / 256);
        double *const *py = (double *const *)(P->d_ptrs + 1);
        if (pi == 1) k_restrict_table<float><<<nbk, 256, 0, cs>>>(fs->n, fs->bs, fs->d_et_ptr, eti, etw, (const float *)yexp, py);
        else if (pi == 2) e = fs_restrict_ff_to(fs, (const ff *)yexp, py, nullptr, 0, cs);
        else k_restrict_table<double><<<nbk, 256, 0, cs>>>(fs->n, fs->bs, fs->d_et_ptr, eti, etw, (const double *)yexp, py);
      }
      cudaError_t ce = cudaStreamEndCapture(cs, &g);
      cudaStreamDestroy(cs);
      if (e) return e;
      CUCHK(ce);
      CUCHK(cudaGraphInstantiate(&ex, g, 0));
      CUCHK(cudaGraphDestroy(g));
    }
    CUCHK(cudaGraphLaunch(ex, s));
    return 0;
  }
  const HpArgs A = make_args(op, x, pi, yexp, nullptr);
  if (op->launch == dLAUNCH_PERSISTENT) DCHK(persistent(A, s, grid));
  else DCHK(pi == 1 ? run_per_order<float>(op, A) : pi == 2 ? run_per_order<ff>(op, A) : run_per_order<double>(op, A));
  if (pi == 1) return fs_restrict32(fs, (const float *)yexp, y, 0);
  if (pi == 2) return fs_restrict_ff(fs, (const ff *)yexp, y, 0);
  return fs_restrict(fs, (const double *)yexp, y, 0);
}

extern "C" {

dErr dOperatorSetLaunchMode(dOperator op, dLaunchMode mode) {
  if (!op) return set_error("null operator");
  if (mode < dLAUNCH_DEFAULT || mode > dLAUNCH_GRAPH) return set_error("launch mode %d invalid", (int)mode);
  op->launch = mode;
  return 0;
}

dErr dOperatorAutotune(dOperator op, const char *cache_path) {
  if (!op) return set_error("null operator");
  op->autotune = true;
  op->tune_path[0] = 0;
  if (cache_path) snprintf(op->tune_path, sizeof op->tune_path, "%s", cache_path);
  if (op->hp_plan) {
    ((HpPlan *)op->hp_plan)->tuned = false;
    if (op->tune_path[0]) tune_load(op, op->tune_path, op->prec == dPREC_FP32);
  }
  return 0;
}

dErr dOperatorGetTiles(dOperator op, dInt *nbuckets, dInt *order, dInt *cap, dInt *threads) {
  if (!op) return set_error("null operator");
  HpPlan *P = (HpPlan *)op->hp_plan;
  if (!P) {
    if (nbuckets) *nbuckets = 0;
    return 0;
  }
  if (nbuckets) *nbuckets = P->nb;
  for (int b = 0; b < P->nb; b++) {
    if (order) order[b] = P->N[b] - 1;
    if (cap) cap[b] = P->cap[b];
    if (threads) threads[b] = P->threads[b];
  }
  return 0;
}

}  // extern "C"
