// C-ABI entry points of the GB300 RK substep cycle.  The per-module
// instances live in disco_gpu_euler.cu / disco_gpu_mhd.cu.
#include "instance.cuh"
#include "disco_gpu_debug.h"
#include "disco_gpu_noalloc.h"

std::atomic<long long> g_launches{0};
long long disco_gpu_launch_count(void) { return g_launches.load(); }

namespace disco_impl {
InstanceBase* make_euler_double(const disco_host_domain* dom, int* rc);
InstanceBase* make_euler_float(const disco_host_domain* dom, int* rc);
InstanceBase* make_mhd_double(const disco_host_domain* dom, int* rc);
InstanceBase* make_mhd_float(const disco_host_domain* dom, int* rc);
}
using namespace disco_impl;


struct disco_gpu {
  InstanceBase* impl;
};

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
  if (dom->mod.hydro == DISCO_HYDRO_EULER)
    impl = precision ? make_euler_float(dom, &rc) : make_euler_double(dom, &rc);
  else
    impl = precision ? make_mhd_float(dom, &rc) : make_mhd_double(dom, &rc);
  if (!impl) return rc ? rc : DISCO_E_CUDA;
  *out = new disco_gpu{impl};
  return 0;
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
int disco_gpu_getmindt_noalloc(disco_gpu* g, double* dt) {
  if (!g || !dt) { disco_set_error("null argument"); return DISCO_E_ARG; }
  return g->impl->getmindt_noalloc(dt);
}
double disco_gpu_time(disco_gpu* g) { return g ? g->impl->time() : 0.0; }
long disco_gpu_num_cells(disco_gpu* g) { return g ? g->impl->N : 0; }
long disco_gpu_num_real_cells(disco_gpu* g) { return g ? g->impl->Nreal : 0; }
void disco_gpu_free(disco_gpu* g) {
  if (!g) return;
  delete g->impl;
  delete g;
}

}  // extern "C"
