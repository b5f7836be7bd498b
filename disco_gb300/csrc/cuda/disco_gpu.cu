// C-ABI entry points of the GB300 RK substep cycle.  The per-module
// instances live in disco_gpu_euler.cu / disco_gpu_mhd.cu.
#include "instance.cuh"
#include "disco_gpu_debug.h"
#include "disco_gpu_noalloc.h"
#include "disco_gpu_batch.h"
#include "disco_gpu_report.h"
#include "disco_gpu_diag.h"
#include "disco_gpu_mlp.h"
#include "mlp_train.cuh"

#include <cmath>
#include <nvtx3/nvToolsExt.h>

std::atomic<long long> g_launches{0};

// A named NVTX range over one C-ABI call (header-only NVTX3: a no-op unless
// a profiler is attached), so that a timeline shows the host's calls --
// getmindt, timestep, run, the batch's steps, training -- around the
// kernels they launch.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};
long long disco_gpu_launch_count(void) { return g_launches.load(); }

namespace disco_impl {
InstanceBase* make_euler_double(const disco_host_domain* dom, int* rc);
InstanceBase* make_euler_float(const disco_host_domain* dom, int* rc);
InstanceBase* make_mhd_double(const disco_host_domain* dom, int* rc);
InstanceBase* make_mhd_float(const disco_host_domain* dom, int* rc);
InstanceBase* make_grmhd_double(const disco_host_domain* dom, int* rc);
}
using namespace disco_impl;


struct disco_gpu {
  InstanceBase* impl;
};

// A batch: members of one module, precision and launch sequence form
// groups at create (multi_plan.cuh); the other members run their own launch
// sequences.  A step is one graph launch, captured per piph parity with a
// fork/join: one branch per sub-group, each sub-group a share of a group
// advanced by the multi-instance stage kernels (one launch per stage over
// all its members), and one branch per member that runs its own sequence.
// The split -- sub-groups per group, from kSplitCand, 0 meaning that every
// member runs its own sequence -- trades launches against concurrency
// between the stages of different sub-groups.  It is chosen by timing each
// candidate on two of the batch's first steps (real steps: the split does
// not change what is computed).
constexpr int kSplitCand[] = {1, 2, 4, 8, 16, 0};
constexpr int kSplitN = 6, kTuneReps = 2;
struct BatchSplit {
  bool built = false;
  std::vector<MultiPlanBase*> plans;
  std::vector<cudaStream_t> st;        // one per plan
  std::vector<int> lead;               // the member that counts a plan's launches
  std::vector<int> solo;               // members on their own sequences
  std::vector<cudaEvent_t> join;       // one per branch
  cudaGraphExec_t g[2] = {nullptr, nullptr};
  std::vector<long long> per;          // launches per step, per member
  void drop_graphs() {
    for (auto& x : g) if (x) { cudaGraphExecDestroy(x); x = nullptr; }
  }
  void release() {
    drop_graphs();
    for (auto p : plans) delete p;
    for (auto s : st) if (s) cudaStreamDestroy(s);
    for (auto e : join) if (e) cudaEventDestroy(e);
    plans.clear(); st.clear(); join.clear(); lead.clear(); solo.clear();
    built = false;
  }
};
struct disco_batch {
  std::vector<InstanceBase*> m;
  std::vector<std::vector<int>> groups;   // member indices of each group (two or more)
  std::vector<int> ungrouped;             // members no group takes
  BatchSplit sets[kSplitN];
  cudaStream_t root = nullptr;
  cudaEvent_t fork = nullptr;
  int parity = 0;
  int split_i = -1;                       // the split in force (-1: timing the candidates)
  int ctas = 8;                           // blocks per SM of the stage kernels (capped by residency)
  int tune_i = 0;
  double tune_ms[kSplitN] = {0, 0, 0, 0, 0, 0};
  void* flush = nullptr;
  size_t flush_size = 0;
  ~disco_batch() {
    for (auto& x : sets) x.release();
    if (fork) cudaEventDestroy(fork);
    if (root) cudaStreamDestroy(root);
    if (flush) cudaFree(flush);
  }
};

// The plans and streams of split candidate ci (outside any capture).
static int batch_split_build(disco_batch* b, int ci) {
  BatchSplit& x = b->sets[ci];
  if (x.built) return 0;
  const int split = kSplitCand[ci];
  x.solo = b->ungrouped;
  for (auto& grp : b->groups) {
    if (split == 0) {
      x.solo.insert(x.solo.end(), grp.begin(), grp.end());
      continue;
    }
    // min(split, size) sub-groups, balanced by cells: largest member first,
    // each to the sub-group with the fewest cells so far
    const int k = std::min<int>(split, (int)grp.size());
    std::vector<int> order = grp;
    std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return b->m[u]->N > b->m[v]->N; });
    std::vector<std::vector<int>> sub(k);
    std::vector<long> load(k, 0);
    for (int i : order) {
      const int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      sub[s].push_back(i);
      load[s] += b->m[i]->N;
    }
    for (auto& v : sub) {
      std::sort(v.begin(), v.end());
      MultiPlanBase* p = b->m[v[0]]->new_multi_plan();
      if (!p) { disco_set_error("disco_batch: a grouped member has no multi-instance plan"); return DISCO_E_STATE; }
      for (size_t t = 1; t < v.size(); ++t) p->add(b->m[v[t]]);
      x.plans.push_back(p);
      x.lead.push_back(v[0]);
      int rc = p->prepare();
      if (rc) return rc;
      cudaStream_t s;
      CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
      x.st.push_back(s);
    }
  }
  std::sort(x.solo.begin(), x.solo.end());
  x.join.assign(x.plans.size() + x.solo.size(), nullptr);
  for (auto& e : x.join) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  x.built = true;
  return 0;
}

static int batch_build(disco_batch* b, int ci, int par) {
  BatchSplit& x = b->sets[ci];
  long long before = g_launches.load();
  CK(cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal));
  CK(cudaEventRecord(b->fork, b->root));
  x.per.assign(b->m.size(), 0);
  size_t br = 0;
  for (size_t p = 0; p < x.plans.size(); ++p, ++br) {
    long long l0 = g_launches.load();
    CK(cudaStreamWaitEvent(x.st[p], b->fork, 0));
    int rc = x.plans[p]->launch_step(par, x.st[p], b->ctas, nullptr);
    if (rc) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(b->root, &g);
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    CK(cudaEventRecord(x.join[br], x.st[p]));
    CK(cudaStreamWaitEvent(b->root, x.join[br], 0));
    x.per[x.lead[p]] += g_launches.load() - l0;
  }
  for (int i : x.solo) {
    long long l0 = g_launches.load();
    CK(cudaStreamWaitEvent(b->m[i]->stream(), b->fork, 0));
    b->m[i]->launch_step(par);
    CK(cudaEventRecord(x.join[br], b->m[i]->stream()));
    CK(cudaStreamWaitEvent(b->root, x.join[br], 0));
    x.per[i] += g_launches.load() - l0;
    ++br;
  }
  cudaGraph_t g;
  CK(cudaStreamEndCapture(b->root, &g));
  g_launches -= g_launches.load() - before;   // counted on each replay
  cudaError_t e = cudaGraphInstantiate(&x.g[par], g, 0);
  cudaGraphDestroy(g);
  CK(e);
  CK(cudaGraphUpload(x.g[par], b->root));
  return 0;
}

static int batch_steps(disco_batch* b, int nsteps, size_t flush_bytes, double* ms) {
  if (flush_bytes > b->flush_size) {
    if (b->flush) cudaFree(b->flush);
    b->flush = nullptr; b->flush_size = 0;
    CK(cudaMalloc(&b->flush, flush_bytes));
    b->flush_size = flush_bytes;
  }
  std::vector<cudaEvent_t> ev(ms ? 2 * (size_t)nsteps : 0);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  cudaEvent_t te[2] = {nullptr, nullptr};
  if (b->split_i < 0)
    for (auto& e : te) CK(cudaEventCreate(&e));
  std::vector<long long> launched(b->m.size(), 0);
  for (int s = 0; s < nsteps; ++s) {
    const bool tuning = b->split_i < 0;
    const int ci = tuning ? b->tune_i / kTuneReps : b->split_i;
    int rc = batch_split_build(b, ci);
    if (rc) return rc;
    BatchSplit& x = b->sets[ci];
    if (!x.g[b->parity]) { rc = batch_build(b, ci, b->parity); if (rc) return rc; }
    for (size_t i = 0; i < b->m.size(); ++i) launched[i] += x.per[i];
    if (ms && flush_bytes) CK(cudaMemsetAsync(b->flush, s & 0xff, flush_bytes, b->root));
    if (ms) CK(cudaEventRecord(ev[2 * s], b->root));
    if (tuning) CK(cudaEventRecord(te[0], b->root));
    CK(cudaGraphLaunch(x.g[b->parity], b->root));
    if (tuning) CK(cudaEventRecord(te[1], b->root));
    if (ms) CK(cudaEventRecord(ev[2 * s + 1], b->root));
    b->parity ^= 1;
    if (tuning) {
      float t;
      CK(cudaEventSynchronize(te[1]));
      CK(cudaEventElapsedTime(&t, te[0], te[1]));
      if (b->tune_i % kTuneReps == 0 || t < b->tune_ms[ci]) b->tune_ms[ci] = t;
      if (++b->tune_i == kSplitN * kTuneReps) {
        int best = 0;
        for (int c = 1; c < kSplitN; ++c)
          if (b->tune_ms[c] < b->tune_ms[best]) best = c;
        b->split_i = best;
        for (int c = 0; c < kSplitN; ++c)
          if (c != best) b->sets[c].release();
      }
    }
  }
  for (auto e : te) if (e) cudaEventDestroy(e);
  CK(cudaStreamSynchronize(b->root));
  if (ms) {
    double tot = 0;
    for (int s = 0; s < nsteps; ++s) {
      float t;
      CK(cudaEventElapsedTime(&t, ev[2 * s], ev[2 * s + 1]));
      tot += t;
    }
    *ms = tot;
    for (auto e : ev) cudaEventDestroy(e);
  }
  for (size_t i = 0; i < b->m.size(); ++i) {
    int rc = b->m[i]->after_external_steps(nsteps, launched[i]);
    if (rc) return rc;
  }
  return 0;
}

// The cons2prim MLP: FP32 masters with Adam moments and gradient, BF16
// copies, the standardisation, the harvested training pairs and the batch
// buffers of training.
struct disco_mlp {
  cudaStream_t st = nullptr;
  float *p = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr, *loss = nullptr;
  disco::bf16 *W1b = nullptr, *W2b = nullptr, *W3b = nullptr;
  float norm[DISCO_MLP_NORM];
  float *X = nullptr, *Y = nullptr;
  long cap = 0, held = 0;
  unsigned long long* count = nullptr;
  disco::MlpBatch bt{};
  long bcap = 0;
  long long step = 0;
  double warm_floor = 0.0, warm_ratio = 1.0;
  ~disco_mlp() {
    for (void* q : {(void*)p, (void*)m1, (void*)m2, (void*)grad, (void*)loss, (void*)W1b, (void*)W2b, (void*)W3b,
                    (void*)X, (void*)Y, (void*)count})
      if (q) cudaFree(q);
    free_batch();
    if (st) cudaStreamDestroy(st);
  }
  void free_batch() {
    for (void* q : {(void*)bt.X, (void*)bt.dY, (void*)bt.H1, (void*)bt.H2, (void*)bt.Z1, (void*)bt.Z2})
      if (q) cudaFree(q);
    bt = disco::MlpBatch{};
    bcap = 0;
  }
  int ensure_batch(long B) {
    if (B <= bcap) return 0;
    free_batch();
    const long n = (B + 63) / 64 * 64;
    CK(cudaMalloc(&bt.X, sizeof(disco::bf16) * n * 16));
    CK(cudaMalloc(&bt.dY, sizeof(disco::bf16) * n * 16));
    CK(cudaMalloc(&bt.H1, sizeof(disco::bf16) * n * 64));
    CK(cudaMalloc(&bt.H2, sizeof(disco::bf16) * n * 64));
    CK(cudaMalloc(&bt.Z1, sizeof(disco::bf16) * n * 64));
    CK(cudaMalloc(&bt.Z2, sizeof(disco::bf16) * n * 64));
    bcap = n;
    return 0;
  }
  disco::MlpDev view() const {
    disco::MlpDev v;
    v.W1b = W1b; v.W2b = W2b; v.W3b = W3b; v.params = p;
    constexpr int F = DISCO_MLP_FEATURES;
    for (int q = 0; q < F; ++q) { v.xm[q] = norm[q]; v.xs[q] = norm[F + q]; }
    for (int q = 0; q < 2; ++q) { v.ym[q] = norm[2 * F + q]; v.ys[q] = norm[2 * F + 2 + q]; }
    v.warm_floor = warm_floor;
    v.warm_ratio = warm_ratio;
    return v;
  }
  int refresh_bf16() {
    disco::k_mlp_bf16<<<16, 256, 0, st>>>(p, W1b, W2b, W3b);
    ++g_launches;
    CK(cudaGetLastError());
    return 0;
  }
  // forward + backward over a batch: grad (mean over the batch) and the
  // summed loss, on the stream
  int fwd_bwd(const float* Xd, const float* Yd, long n, int B, unsigned long long seed) {
    int rc = ensure_batch(B);
    if (rc) return rc;
    CK(cudaMemsetAsync(grad, 0, sizeof(float) * DISCO_MLP_PARAMS, st));
    CK(cudaMemsetAsync(loss, 0, sizeof(float), st));
    const disco::MlpDev v = view();
    disco::k_mlp_fwdbwd<<<(B + 63) / 64, 128, 0, st>>>(v, Xd, Yd, n, B, seed, bt, loss);
    disco::k_mlp_wgrad<<<(B + disco::kWgSamples - 1) / disco::kWgSamples, 320, 0, st>>>(bt, B, grad);
    g_launches += 2;
    CK(cudaGetLastError());
    return 0;
  }
};

static unsigned long long mlp_splitmix(unsigned long long& x) {
  unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

extern "C" {

int disco_mlp_create(unsigned long long seed, long capacity, disco_mlp** out) {
  if (!out || capacity < 0) { disco_set_error("disco_mlp_create: bad argument"); return DISCO_E_ARG; }
  disco_mlp* m = new disco_mlp();
  auto fail = [&](int rc) { delete m; return rc; };
  if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) != cudaSuccess) {
    disco_set_error("disco_mlp_create: no stream");
    return fail(DISCO_E_CUDA);
  }
  const size_t np = DISCO_MLP_PARAMS;
  if (cudaMalloc(&m->p, 4 * np) || cudaMalloc(&m->m1, 4 * np) || cudaMalloc(&m->m2, 4 * np) ||
      cudaMalloc(&m->grad, 4 * np) || cudaMalloc(&m->loss, 4) || cudaMalloc(&m->W1b, 2 * 64 * 16) ||
      cudaMalloc(&m->W2b, 2 * 64 * 64) || cudaMalloc(&m->W3b, 2 * 16 * 64) || cudaMalloc(&m->count, 8) ||
      cudaMalloc(&m->X, 4 * (size_t)std::max(capacity, 1L) * DISCO_MLP_FEATURES) ||
      cudaMalloc(&m->Y, 4 * (size_t)std::max(capacity, 1L) * DISCO_MLP_OUTPUTS)) {
    disco_set_error("disco_mlp_create: device allocation failed");
    return fail(DISCO_E_NOMEM);
  }
  m->cap = capacity;
  // Xavier-uniform weights, zero biases (inputs 8..15 of W1 and rows 2..7
  // of W3 stay zero)
  std::vector<float> h(np, 0.f);
  unsigned long long s = seed;
  auto fill = [&](int off, int nout, int nin, int ld, int fan_in, int fan_out) {
    const double a = sqrt(6.0 / (double)(fan_in + fan_out));
    for (int o = 0; o < nout; ++o)
      for (int i = 0; i < nin; ++i) {
        const double u = (double)(mlp_splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
        h[off + o * ld + i] = (float)((2.0 * u - 1.0) * a);
      }
  };
  fill(disco::kOffW1, 64, DISCO_MLP_FEATURES, 16, DISCO_MLP_FEATURES, 64);
  fill(disco::kOffW2, 64, 64, 64, 64, 64);
  fill(disco::kOffW3, DISCO_MLP_OUTPUTS, 64, 64, 64, DISCO_MLP_OUTPUTS);
  constexpr int F = DISCO_MLP_FEATURES;
  for (int q = 0; q < F; ++q) { m->norm[q] = 0.f; m->norm[F + q] = 1.f; }
  for (int q = 0; q < 2; ++q) { m->norm[2 * F + q] = 0.f; m->norm[2 * F + 2 + q] = 1.f; }
  if (cudaMemcpy(m->p, h.data(), 4 * np, cudaMemcpyHostToDevice) || cudaMemset(m->m1, 0, 4 * np) ||
      cudaMemset(m->m2, 0, 4 * np) || cudaMemset(m->count, 0, 8)) {
    disco_set_error("disco_mlp_create: upload failed");
    return fail(DISCO_E_CUDA);
  }
  int rc = m->refresh_bf16();
  if (!rc && cudaStreamSynchronize(m->st) != cudaSuccess) rc = DISCO_E_CUDA;
  if (rc) return fail(rc);
  *out = m;
  return 0;
}

void disco_mlp_free(disco_mlp* m) { delete m; }

int disco_mlp_harvest(disco_mlp* m, disco_gpu* g, int stride, int steps, long* count) {
  if (!m || !g || stride < 1 || steps < 0) { disco_set_error("disco_mlp_harvest: bad argument"); return DISCO_E_ARG; }
  CK(cudaStreamSynchronize(m->st));
  const disco::MlpDev v = m->view();
  disco::C2PRecord rec{m->X, m->Y, m->cap, m->count, stride};
  int rc = g->impl->harvest(&v, &rec, steps);
  if (rc) return rc;
  unsigned long long c = 0;
  CK(cudaMemcpy(&c, m->count, 8, cudaMemcpyDeviceToHost));
  m->held = (long)std::min<unsigned long long>(c, (unsigned long long)m->cap);
  if (count) *count = m->held;
  return 0;
}

int disco_mlp_pairs(disco_mlp* m, long first, long n, float* X, float* Y) {
  if (!m || first < 0 || n < 0 || first + n > m->held) { disco_set_error("disco_mlp_pairs: bad range"); return DISCO_E_ARG; }
  if (X) CK(cudaMemcpy(X, m->X + first * DISCO_MLP_FEATURES, 4 * (size_t)n * DISCO_MLP_FEATURES, cudaMemcpyDeviceToHost));
  if (Y) CK(cudaMemcpy(Y, m->Y + first * DISCO_MLP_OUTPUTS, 4 * (size_t)n * DISCO_MLP_OUTPUTS, cudaMemcpyDeviceToHost));
  return 0;
}

int disco_mlp_fit_norm(disco_mlp* m) {
  if (!m || m->held < 2) { disco_set_error("disco_mlp_fit_norm: fewer than two pairs held"); return DISCO_E_STATE; }
  const long n = m->held;
  std::vector<float> X((size_t)n * DISCO_MLP_FEATURES), Y((size_t)n * DISCO_MLP_OUTPUTS);
  int rc = disco_mlp_pairs(m, 0, n, X.data(), Y.data());
  if (rc) return rc;
  auto stats = [&](const std::vector<float>& a, int dim, int q, float* mean, float* sd) {
    double s = 0, s2 = 0;
    for (long i = 0; i < n; ++i) s += a[(size_t)i * dim + q];
    const double mu = s / n;
    for (long i = 0; i < n; ++i) { const double d = a[(size_t)i * dim + q] - mu; s2 += d * d; }
    const double sdv = sqrt(s2 / n);
    *mean = (float)mu;
    *sd = (float)(sdv > 1e-6 ? sdv : 1.0);
  };
  constexpr int F = DISCO_MLP_FEATURES;
  for (int q = 0; q < F; ++q) stats(X, F, q, &m->norm[q], &m->norm[F + q]);
  for (int q = 0; q < 2; ++q) stats(Y, 2, q, &m->norm[2 * F + q], &m->norm[2 * F + 2 + q]);
  return 0;
}

int disco_mlp_train(disco_mlp* m, int steps, int batch, float lr, unsigned long long seed, float* loss_first,
                    float* loss_last) {
  if (!m || steps < 0 || batch < 16 || !(lr > 0.f)) { disco_set_error("disco_mlp_train: bad argument"); return DISCO_E_ARG; }
  if (m->held < 1) { disco_set_error("disco_mlp_train: no training pairs held"); return DISCO_E_STATE; }
  NvtxRange r("disco_mlp_train");
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int k = 0; k < steps; ++k) {
    const unsigned long long sd = seed + (unsigned long long)m->step * (unsigned long long)batch;
    int rc = m->fwd_bwd(m->X, m->Y, m->held, batch, sd == ~0ull ? sd - 1 : sd);
    if (rc) return rc;
    if (k == 0 && loss_first) {
      CK(cudaMemcpyAsync(loss_first, m->loss, 4, cudaMemcpyDeviceToHost, m->st));
      CK(cudaStreamSynchronize(m->st));
      *loss_first /= (float)(batch * DISCO_MLP_OUTPUTS);
    }
    ++m->step;
    const float bc1 = 1.f - powf(b1, (float)m->step), bc2 = 1.f - powf(b2, (float)m->step);
    disco::k_mlp_adam<<<(DISCO_MLP_PARAMS + 255) / 256, 256, 0, m->st>>>(m->p, m->m1, m->m2, m->grad, lr, b1, b2,
                                                                         eps, bc1, bc2);
    ++g_launches;
    rc = m->refresh_bf16();
    if (rc) return rc;
  }
  if (loss_last) {
    CK(cudaMemcpyAsync(loss_last, m->loss, 4, cudaMemcpyDeviceToHost, m->st));
    CK(cudaStreamSynchronize(m->st));
    *loss_last /= (float)(batch * DISCO_MLP_OUTPUTS);
  }
  CK(cudaStreamSynchronize(m->st));
  CK(cudaGetLastError());
  return 0;
}

int disco_mlp_grad(disco_mlp* m, const float* X, const float* Y, int n, float* loss, float* grad) {
  if (!m || !X || !Y || n < 1 || !grad) { disco_set_error("disco_mlp_grad: bad argument"); return DISCO_E_ARG; }
  float *dX = nullptr, *dY = nullptr;
  int rc = 0;
  if (cudaMalloc(&dX, 4 * (size_t)n * DISCO_MLP_FEATURES) != cudaSuccess ||
      cudaMalloc(&dY, 4 * (size_t)n * DISCO_MLP_OUTPUTS) != cudaSuccess) {
    if (dX) cudaFree(dX);
    disco_set_error("disco_mlp_grad: device allocation failed");
    return DISCO_E_NOMEM;
  }
  if (cudaMemcpy(dX, X, 4 * (size_t)n * DISCO_MLP_FEATURES, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dY, Y, 4 * (size_t)n * DISCO_MLP_OUTPUTS, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = DISCO_E_CUDA;
  }
  if (!rc) rc = m->fwd_bwd(dX, dY, n, n, ~0ull);
  if (!rc) {
    if (cudaMemcpyAsync(grad, m->grad, 4 * DISCO_MLP_PARAMS, cudaMemcpyDeviceToHost, m->st) != cudaSuccess ||
        (loss && cudaMemcpyAsync(loss, m->loss, 4, cudaMemcpyDeviceToHost, m->st) != cudaSuccess) ||
        cudaStreamSynchronize(m->st) != cudaSuccess)
      rc = DISCO_E_CUDA;
  }
  cudaFree(dX);
  cudaFree(dY);
  if (rc == DISCO_E_CUDA) disco_set_error("disco_mlp_grad: CUDA error");
  return rc;
}

int disco_mlp_predict(disco_mlp* m, const float* X, long n, float* Y) {
  if (!m || !X || !Y || n < 0) { disco_set_error("disco_mlp_predict: bad argument"); return DISCO_E_ARG; }
  if (n == 0) return 0;
  float *dX = nullptr, *dY = nullptr;
  if (cudaMalloc(&dX, 4 * (size_t)n * DISCO_MLP_FEATURES) != cudaSuccess ||
      cudaMalloc(&dY, 4 * (size_t)n * DISCO_MLP_OUTPUTS) != cudaSuccess) {
    if (dX) cudaFree(dX);
    disco_set_error("disco_mlp_predict: device allocation failed");
    return DISCO_E_NOMEM;
  }
  cudaError_t e = cudaMemcpyAsync(dX, X, 4 * (size_t)n * DISCO_MLP_FEATURES, cudaMemcpyHostToDevice, m->st);
  if (e == cudaSuccess) {
    disco::k_mlp_predict<<<(unsigned)((n + 127) / 128), 128, 0, m->st>>>(m->view(), dX, n, dY);
    ++g_launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(Y, dY, 4 * (size_t)n * DISCO_MLP_OUTPUTS, cudaMemcpyDeviceToHost, m->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
  cudaFree(dX);
  cudaFree(dY);
  CK(e);
  return 0;
}

int disco_mlp_params(disco_mlp* m, float* get, const float* set, float* norm_get, const float* norm_set) {
  if (!m) { disco_set_error("disco_mlp_params: null model"); return DISCO_E_ARG; }
  CK(cudaStreamSynchronize(m->st));
  if (get) CK(cudaMemcpy(get, m->p, 4 * DISCO_MLP_PARAMS, cudaMemcpyDeviceToHost));
  if (norm_get) memcpy(norm_get, m->norm, sizeof m->norm);
  if (norm_set) memcpy(m->norm, norm_set, sizeof m->norm);
  if (set) {
    CK(cudaMemcpy(m->p, set, 4 * DISCO_MLP_PARAMS, cudaMemcpyHostToDevice));
    int rc = m->refresh_bf16();
    if (rc) return rc;
    CK(cudaStreamSynchronize(m->st));
  }
  return 0;
}

int disco_mlp_set_gate(disco_mlp* m, double floor, double ratio) {
  if (!m || !(floor >= 0.0) || !(ratio > 0.0 && ratio <= 1.0)) {
    disco_set_error("disco_mlp_set_gate: bad argument");
    return DISCO_E_ARG;
  }
  m->warm_floor = floor;
  m->warm_ratio = ratio;
  return 0;
}

int disco_gpu_attach_guess(disco_gpu* g, disco_mlp* m) {
  if (!g) { disco_set_error("disco_gpu_attach_guess: null instance"); return DISCO_E_ARG; }
  if (!m) return g->impl->attach_guess(nullptr);
  CK(cudaStreamSynchronize(m->st));
  const disco::MlpDev v = m->view();
  return g->impl->attach_guess(&v);
}

int disco_gpu_c2p_stats(disco_gpu* g, long long out[4], int reset) {
  if (!g || !out) { disco_set_error("disco_gpu_c2p_stats: bad argument"); return DISCO_E_ARG; }
  return g->impl->c2p_stats(out, reset);
}

int disco_gpu_create(const disco_host_domain* dom, int precision, disco_gpu** out) {
  if (!dom || !out) { disco_set_error("disco_gpu_create: null argument"); return DISCO_E_ARG; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    disco_set_error("disco_gpu_create: no CUDA device");
    return DISCO_E_NODEV;
  }
  int rc = 0;
  InstanceBase* impl;
  if (dom->mod.hydro == DISCO_HYDRO_EULER) {
    impl = precision ? make_euler_float(dom, &rc) : make_euler_double(dom, &rc);
  } else if (dom->mod.hydro == DISCO_HYDRO_GRMHD) {
    if (precision) {
      disco_set_error("disco_gpu_create: GRMHD runs on the FP64 path only (precision 0)");
      return DISCO_E_MODULE;
    }
    impl = make_grmhd_double(dom, &rc);
  } else {
    impl = precision ? make_mhd_float(dom, &rc) : make_mhd_double(dom, &rc);
  }
  if (!impl) return rc ? rc : DISCO_E_CUDA;
  *out = new disco_gpu{impl};
  return 0;
}

int disco_gpu_report(disco_gpu* g, double* out, int nout) {
  if (!g || !out || nout < 0) { disco_set_error("disco_gpu_report: bad argument"); return DISCO_E_ARG; }
  return g->impl->report(out, nout);
}

int disco_gpu_sink_accum(disco_gpu* g, double* out, int max_bodies, int reset) {
  if (!g || max_bodies < 0) { disco_set_error("disco_gpu_sink_accum: bad argument"); return DISCO_E_ARG; }
  return g->impl->sink_accum(out, max_bodies, reset);
}

int disco_gpu_diag_count(disco_gpu* g) {
  if (!g) { disco_set_error("disco_gpu_diag_count: null argument"); return DISCO_E_ARG; }
  return g->impl->diag(0, nullptr, -1, nullptr, nullptr, 0.0);
}

int disco_gpu_diag_download(disco_gpu* g, double* Qrz, long long len, double* t_avg) {
  if (!g || (Qrz && len < 0)) { disco_set_error("disco_gpu_diag_download: bad argument"); return DISCO_E_ARG; }
  return g->impl->diag(0, Qrz, Qrz ? len : -1, t_avg, nullptr, 0.0);
}

int disco_gpu_diag_upload(disco_gpu* g, const double* Qrz, long long len, double t_avg) {
  if (!g) { disco_set_error("disco_gpu_diag_upload: null argument"); return DISCO_E_ARG; }
  return g->impl->diag(Qrz ? 1 : 2, nullptr, len, nullptr, Qrz, t_avg);
}

int disco_gpu_getmindt(disco_gpu* g, double* dt) {
  if (!g || !dt) { disco_set_error("null argument"); return DISCO_E_ARG; }
  NvtxRange r("disco_gpu_getmindt");
  return g->impl->getmindt(dt);
}
int disco_gpu_timestep(disco_gpu* g, double dt) {
  if (!g) { disco_set_error("null argument"); return DISCO_E_ARG; }
  if (!(dt > 0.0)) { disco_set_error("timestep: dt must be positive"); return DISCO_E_ARG; }
  NvtxRange r("disco_gpu_timestep");
  return g->impl->timestep(dt);
}
int disco_gpu_run(disco_gpu* g, int nsteps, double t_end) {
  if (!g || nsteps < 0) { disco_set_error("bad argument"); return DISCO_E_ARG; }
  NvtxRange r("disco_gpu_run");
  return g->impl->run(nsteps, t_end);
}
int disco_gpu_download(disco_gpu* g, disco_state_view* v) {
  if (!g || !v) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->download(v);
}
int disco_gpu_upload(disco_gpu* g, const disco_state_view* v) {
  if (!g || !v) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->upload(v);
}
int disco_gpu_run_timed(disco_gpu* g, int nsteps, double t_end, size_t flush_bytes, double* ms) {
  if (!g || nsteps < 0 || !ms) { disco_set_error("bad argument"); return DISCO_E_ARG; }
  return g->impl->run_timed(nsteps, t_end, flush_bytes, ms);
}
int disco_gpu_profile(disco_gpu* g, int nsteps, disco_kernel_time* out, int max_out, int* n_out) {
  if (!g || !out || !n_out || nsteps < 0) { disco_set_error("bad argument"); return DISCO_E_ARG; }
  return g->impl->profile(nsteps, out, max_out, n_out);
}
int disco_gpu_planets(disco_gpu* g, disco_planet* out, int max, int* n) {
  if (!g || !n || (max > 0 && !out) || max < 0) { disco_set_error("disco_gpu_planets: bad argument"); return DISCO_E_ARG; }
  return g->impl->planets(out, max, n);
}
int disco_gpu_status(disco_gpu* g, disco_gpu_errs* e) {
  if (!g || !e) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->status(e);
}
int disco_gpu_debug_ct(disco_gpu* g, int stage, double* E, double* B, double* Ephi, double* Phi) {
  if (!g || stage < 0 || stage > 4) { disco_set_error("bad argument"); return DISCO_E_ARG; }
  return g->impl->debug_ct(stage, E, B, Ephi, Phi);
}
int disco_gpu_debug_faces(disco_gpu* g, int dim, int* npair, long* nface, int* fIndex, int* L, int* R,
                          int* LRtype, double* phic, double* dA) {
  if (!g) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->debug_faces(dim, npair, nface, fIndex, L, R, LRtype, phic, dA);
}
int disco_gpu_debug_grad(disco_gpu* g, double* gradp, double* gradr, double* gradz) {
  if (!g) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->debug_grad(gradp, gradr, gradz);
}
int disco_gpu_debug_sweep(disco_gpu* g, int on) {
  if (!g) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->set_sweep(on);
}
int disco_gpu_divb(disco_gpu* g, double* div, double* scale) {
  if (!g) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->divb(div, scale);
}
int disco_gpu_debug_convert(const double* in, const float* fin, long n, float* f_int, float* f_hw,
                            double* d_int, double* d_hw) {
  if (!in || !fin || n < 0 || !f_int || !f_hw || !d_int || !d_hw) {
    disco_set_error("disco_gpu_debug_convert: bad argument");
    return DISCO_E_ARG;
  }
  if (n == 0) return 0;
  const size_t nb = (size_t)n;
  double *din = nullptr, *dd_int = nullptr, *dd_hw = nullptr;
  float *dfin = nullptr, *df_int = nullptr, *df_hw = nullptr;
  int rc = 0;
  cudaError_t e = cudaSuccess;
  if ((e = cudaMalloc(&din, nb * 8)) == cudaSuccess && (e = cudaMalloc(&dd_int, nb * 8)) == cudaSuccess &&
      (e = cudaMalloc(&dd_hw, nb * 8)) == cudaSuccess && (e = cudaMalloc(&dfin, nb * 4)) == cudaSuccess &&
      (e = cudaMalloc(&df_int, nb * 4)) == cudaSuccess && (e = cudaMalloc(&df_hw, nb * 4)) == cudaSuccess &&
      (e = cudaMemcpy(din, in, nb * 8, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = cudaMemcpy(dfin, fin, nb * 4, cudaMemcpyHostToDevice)) == cudaSuccess) {
    const int grid = (int)std::min<long>((n + 255) / 256, 152L * 8);
    disco::k_convert_check<<<grid, 256>>>(din, n, df_int, df_hw, dfin, dd_int, dd_hw);
    ++g_launches;
    if ((e = cudaGetLastError()) == cudaSuccess && (e = cudaDeviceSynchronize()) == cudaSuccess &&
        (e = cudaMemcpy(f_int, df_int, nb * 4, cudaMemcpyDeviceToHost)) == cudaSuccess &&
        (e = cudaMemcpy(f_hw, df_hw, nb * 4, cudaMemcpyDeviceToHost)) == cudaSuccess &&
        (e = cudaMemcpy(d_int, dd_int, nb * 8, cudaMemcpyDeviceToHost)) == cudaSuccess)
      e = cudaMemcpy(d_hw, dd_hw, nb * 8, cudaMemcpyDeviceToHost);
  }
  if (e != cudaSuccess) {
    char b[160];
    snprintf(b, sizeof b, "disco_gpu_debug_convert: CUDA %s", cudaGetErrorString(e));
    disco_set_error(b);
    rc = DISCO_E_CUDA;
  }
  cudaFree(din); cudaFree(dd_int); cudaFree(dd_hw); cudaFree(dfin); cudaFree(df_int); cudaFree(df_hw);
  return rc;
}
int disco_gpu_getmindt_noalloc(disco_gpu* g, double* dt) {
  if (!g || !dt) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->getmindt_noalloc(dt);
}
int disco_batch_create(disco_gpu* const* members, int n, disco_batch** out) {
  return disco_batch_create_flags(members, n, 0, out);
}
int disco_batch_create_flags(disco_gpu* const* members, int n, int flags, disco_batch** out) {
  if (!members || n <= 0 || !out || (flags & ~DISCO_BATCH_NO_GROUPS)) {
    disco_set_error("disco_batch_create: bad argument");
    return DISCO_E_ARG;
  }
  int par = -1;
  for (int i = 0; i < n; ++i) {
    if (!members[i]) { disco_set_error("disco_batch_create: null member"); return DISCO_E_ARG; }
    int p = members[i]->impl->cur_parity();
    if (par >= 0 && p != par) {
      disco_set_error("disco_batch_create: members have taken different step counts (parity)");
      return DISCO_E_STATE;
    }
    par = p;
  }
  disco_batch* b = new disco_batch();
  for (int i = 0; i < n; ++i) b->m.push_back(members[i]->impl);
  b->parity = par;
  // groups: members of one type and launch sequence, in member order (a
  // probe plan per group decides who joins)
  std::vector<MultiPlanBase*> probe;
  for (int i = 0; i < n; ++i) {
    InstanceBase* x = b->m[i];
    bool placed = false;
    for (size_t p = 0; p < probe.size() && !placed; ++p)
      if (probe[p]->accepts(x)) { probe[p]->add(x); b->groups[p].push_back(i); placed = true; }
    if (placed) continue;
    MultiPlanBase* p = (flags & DISCO_BATCH_NO_GROUPS) ? nullptr : x->new_multi_plan();
    if (p) { probe.push_back(p); b->groups.push_back({i}); }
    else b->ungrouped.push_back(i);
  }
  for (auto p : probe) delete p;
  for (size_t g = 0; g < b->groups.size();) {   // a group of one is a member of its own
    if (b->groups[g].size() > 1) { ++g; continue; }
    b->ungrouped.push_back(b->groups[g][0]);
    b->groups.erase(b->groups.begin() + g);
  }
  std::sort(b->ungrouped.begin(), b->ungrouped.end());
  if (b->groups.empty()) b->split_i = kSplitN - 1;   // nothing to split: every member on its own
  if (cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    delete b;
    disco_set_error("disco_batch_create: stream/event creation failed");
    return DISCO_E_CUDA;
  }
  *out = b;
  return 0;
}
int disco_batch_run(disco_batch* b, int nsteps) {
  if (!b || nsteps < 0) { disco_set_error("bad argument"); return DISCO_E_ARG; }
  NvtxRange r("disco_batch_run");
  return batch_steps(b, nsteps, 0, nullptr);
}
int disco_batch_run_timed(disco_batch* b, int nsteps, size_t flush_bytes, double* ms) {
  if (!b || nsteps < 0 || !ms) { disco_set_error("bad argument"); return DISCO_E_ARG; }
  return batch_steps(b, nsteps, flush_bytes, ms);
}
int disco_batch_profile(disco_batch* b, int nsteps, disco_kernel_time* out, int max_out, int* n_out) {
  if (!b || nsteps < 0 || !out || !n_out || max_out < 0) { disco_set_error("disco_batch_profile: bad argument"); return DISCO_E_ARG; }
  // the sub-groups' stages launched one by one on their streams, each
  // bracketed by events; members on their own sequences step untimed
  const int ci = b->split_i >= 0 ? b->split_i : 0;
  int rc = batch_split_build(b, ci);
  if (rc) return rc;
  BatchSplit& x = b->sets[ci];
  std::vector<KTimer> kt(x.plans.size());
  for (size_t p = 0; p < x.plans.size(); ++p) { kt[p].on = true; kt[p].st = x.st[p]; }
  for (int s = 0; s < nsteps; ++s) {
    for (size_t p = 0; p < x.plans.size(); ++p) {
      rc = x.plans[p]->launch_step(b->parity, x.st[p], b->ctas, &kt[p]);
      if (rc) return rc;
    }
    for (int i : x.solo) b->m[i]->launch_step(b->parity);
    b->parity ^= 1;
  }
  CK(cudaDeviceSynchronize());
  std::vector<std::string> names;
  std::vector<long long> cnt;
  std::vector<double> ms;
  for (auto& k : kt)
    for (auto& r : k.recs) {
      float t = 0;
      cudaEventElapsedTime(&t, r.a, r.b);
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
      size_t i = 0;
      for (; i < names.size(); ++i) if (names[i] == r.name) break;
      if (i == names.size()) { names.push_back(r.name); cnt.push_back(0); ms.push_back(0); }
      cnt[i] += 1;
      ms[i] += t;
    }
  int k = 0;
  for (size_t i = 0; i < names.size() && k < max_out; ++i, ++k) {
    snprintf(out[k].name, sizeof out[k].name, "%s", names[i].c_str());
    out[k].launches = cnt[i];
    out[k].ms = ms[i];
  }
  *n_out = k;
  for (auto* m : b->m) {
    rc = m->after_external_steps(nsteps, 0);
    if (rc) return rc;
  }
  return 0;
}
int disco_batch_set_grid(disco_batch* b, int ctas_per_sm) {
  if (!b || ctas_per_sm < 1 || ctas_per_sm > 64) { disco_set_error("disco_batch_set_grid: bad argument"); return DISCO_E_ARG; }
  b->ctas = ctas_per_sm;
  for (auto& x : b->sets) x.drop_graphs();
  return 0;
}
int disco_batch_set_split(disco_batch* b, int split) {
  if (!b) { disco_set_error("disco_batch_set_split: null batch"); return DISCO_E_ARG; }
  if (split == -1) {
    if (b->groups.empty()) return 0;
    b->split_i = -1;
    b->tune_i = 0;
    return 0;
  }
  for (int c = 0; c < kSplitN; ++c)
    if (kSplitCand[c] == split) {
      b->split_i = b->groups.empty() ? kSplitN - 1 : c;
      return 0;
    }
  disco_set_error("disco_batch_set_split: split must be -1, 0, 1, 2, 4, 8 or 16");
  return DISCO_E_ARG;
}
int disco_batch_info(const disco_batch* b, int* groups, int* grouped, int* split, int* ctas_per_sm,
                     double* tune_ms) {
  if (!b) { disco_set_error("disco_batch_info: null batch"); return DISCO_E_ARG; }
  if (groups) *groups = (int)b->groups.size();
  if (grouped) {
    int k = 0;
    for (auto& g : b->groups) k += (int)g.size();
    *grouped = k;
  }
  if (split) *split = b->split_i >= 0 ? kSplitCand[b->split_i] : -1;
  if (ctas_per_sm) *ctas_per_sm = b->ctas;
  if (tune_ms)
    for (int c = 0; c < kSplitN; ++c) tune_ms[c] = b->tune_i > c * kTuneReps ? b->tune_ms[c] : -1.0;
  return 0;
}
void disco_batch_free(disco_batch* b) { delete b; }

double disco_gpu_time(disco_gpu* g) { return g ? g->impl->time() : 0.0; }
long disco_gpu_num_cells(disco_gpu* g) { return g ? g->impl->N : 0; }
long disco_gpu_num_real_cells(disco_gpu* g) { return g ? g->impl->Nreal : 0; }
void disco_gpu_free(disco_gpu* g) {
  if (!g) return;
  delete g->impl;
  delete g;
}

}  // extern "C"
