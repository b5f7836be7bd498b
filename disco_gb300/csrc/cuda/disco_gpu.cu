// C-ABI entry points of the GB300 RK substep cycle.  The per-module
// instances live in disco_gpu_euler.cu / disco_gpu_mhd.cu.
#include "instance.cuh"
#include "disco_gpu_debug.h"
#include "disco_gpu_noalloc.h"
#include "disco_gpu_batch.h"
#include "disco_gpu_report.h"
#include "disco_gpu_diag.h"

std::atomic<long long> g_launches{0};
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

// A batch: one graph per piph parity, built by stream capture with a
// fork/join over the members' own streams, so the captured graph has one
// branch per member.
struct disco_batch {
  std::vector<InstanceBase*> m;
  cudaStream_t root = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  long long nodes = 0;          // kernel launches per graph
  std::vector<long long> per;   // per member
  int parity = 0;
  void* flush = nullptr;
  size_t flush_size = 0;
  ~disco_batch() {
    for (auto& g : graph) if (g) cudaGraphExecDestroy(g);
    for (auto e : join) if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (root) cudaStreamDestroy(root);
    if (flush) cudaFree(flush);
  }
};

static int batch_build(disco_batch* b, int par) {
  long long before = g_launches.load();
  CK(cudaStreamBeginCapture(b->root, cudaStreamCaptureModeThreadLocal));
  CK(cudaEventRecord(b->fork, b->root));
  b->per.assign(b->m.size(), 0);
  for (size_t i = 0; i < b->m.size(); ++i) {
    long long l0 = g_launches.load();
    CK(cudaStreamWaitEvent(b->m[i]->stream(), b->fork, 0));
    b->m[i]->launch_step(par);
    CK(cudaEventRecord(b->join[i], b->m[i]->stream()));
    CK(cudaStreamWaitEvent(b->root, b->join[i], 0));
    b->per[i] = g_launches.load() - l0;
  }
  cudaGraph_t g;
  CK(cudaStreamEndCapture(b->root, &g));
  b->nodes = g_launches.load() - before;
  g_launches -= b->nodes;   // counted on each replay
  CK(cudaGraphInstantiate(&b->graph[par], g, 0));
  cudaGraphDestroy(g);
  return 0;
}

static int batch_steps(disco_batch* b, int nsteps, size_t flush_bytes, double* ms) {
  for (int p = 0; p < 2; ++p)
    if (!b->graph[p]) { int rc = batch_build(b, p); if (rc) return rc; }
  if (flush_bytes > b->flush_size) {
    if (b->flush) cudaFree(b->flush);
    b->flush = nullptr; b->flush_size = 0;
    CK(cudaMalloc(&b->flush, flush_bytes));
    b->flush_size = flush_bytes;
  }
  std::vector<cudaEvent_t> ev(ms ? 2 * (size_t)nsteps : 0);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  for (int s = 0; s < nsteps; ++s) {
    if (ms && flush_bytes) CK(cudaMemsetAsync(b->flush, s & 0xff, flush_bytes, b->root));
    if (ms) CK(cudaEventRecord(ev[2 * s], b->root));
    CK(cudaGraphLaunch(b->graph[b->parity], b->root));
    if (ms) CK(cudaEventRecord(ev[2 * s + 1], b->root));
    b->parity ^= 1;
  }
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
    int rc = b->m[i]->after_external_steps(nsteps, b->per[i] * nsteps);
    if (rc) return rc;
  }
  return 0;
}

extern "C" {

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
  return g->impl->getmindt(dt);
}
int disco_gpu_timestep(disco_gpu* g, double dt) {
  if (!g) { disco_set_error("null argument"); return DISCO_E_ARG; }
  if (!(dt > 0.0)) { disco_set_error("timestep: dt must be positive"); return DISCO_E_ARG; }
  return g->impl->timestep(dt);
}
int disco_gpu_run(disco_gpu* g, int nsteps, double t_end) {
  if (!g || nsteps < 0) { disco_set_error("bad argument"); return DISCO_E_ARG; }
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
  if (!members || n <= 0 || !out) { disco_set_error("disco_batch_create: bad argument"); return DISCO_E_ARG; }
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
  b->join.assign(n, nullptr);
  if (cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    delete b;
    disco_set_error("disco_batch_create: stream/event creation failed");
    return DISCO_E_CUDA;
  }
  for (int i = 0; i < n; ++i)
    if (cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) != cudaSuccess) {
      delete b;
      disco_set_error("disco_batch_create: event creation failed");
      return DISCO_E_CUDA;
    }
  *out = b;
  return 0;
}
int disco_batch_run(disco_batch* b, int nsteps) {
  if (!b || nsteps < 0) { disco_set_error("bad argument"); return DISCO_E_ARG; }
  return batch_steps(b, nsteps, 0, nullptr);
}
int disco_batch_run_timed(disco_batch* b, int nsteps, size_t flush_bytes, double* ms) {
  if (!b || nsteps < 0 || !ms) { disco_set_error("bad argument"); return DISCO_E_ARG; }
  return batch_steps(b, nsteps, flush_bytes, ms);
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
