// Device instance of one domain: owns the device arrays and launches the
// kernels of kernels.cuh / ct_kernels.cuh in onestep.c order.  Included by
// one translation unit per hydro module.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "disco_gpu.h"
#include "../host/disco_host_internal.h"
#include "kernels.cuh"
#include "ct_kernels.cuh"
#include "noalloc.cuh"
#include "report.cuh"
#include "diag.cuh"
#include "checks.cuh"
#include "mlp_c2p.cuh"
#include "phi_sweep.cuh"
#include "../plugins/bc_plugins.h"

using namespace disco;

extern std::atomic<long long> g_launches;

#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      char b_[256];                                                            \
      snprintf(b_, sizeof b_, "CUDA %s at %s:%d", cudaGetErrorString(e_),      \
               __FILE__, __LINE__);                                            \
      disco_set_error(b_);                                                     \
      return DISCO_E_CUDA;                                                     \
    }                                                                          \
  } while (0)

namespace disco_impl {

struct InstanceBase;
struct KTimer;

// A group of instances of one hydro module and precision whose steps launch
// the same kernel sequence, advanced together by the persistent stage
// kernels of multi.cuh: each stage is one launch over every member's tiles.
struct MultiPlanBase {
  virtual ~MultiPlanBase() {}
  // x has this group's type and launch sequence (and may join it)
  virtual bool accepts(InstanceBase* x) const = 0;
  virtual void add(InstanceBase* x) = 0;
  virtual int size() const = 0;
  // device member tables and work lists, from the members as they are now
  virtual int prepare() = 0;
  // one full step of every member from piph parity par, on stream st, each
  // stage kernel a grid of at most ctas_per_sm blocks per SM (and at most
  // as many as are resident at once); kt, when given, times each stage
  virtual int launch_step(int par, cudaStream_t st, int ctas_per_sm, KTimer* kt) = 0;
};

struct InstanceBase {
  virtual ~InstanceBase() {}
  virtual int getmindt(double* dt) = 0;
  virtual int timestep(double dt) = 0;
  virtual int run(int n, double t_end) = 0;
  virtual int download(disco_state_view* v) = 0;
  virtual int upload(const disco_state_view* v) = 0;
  virtual int status(disco_gpu_errs* e) = 0;
  virtual int run_timed(int n, double t_end, size_t flush_bytes, double* ms) = 0;
  virtual int profile(int n, disco_kernel_time* out, int maxo, int* nout) = 0;
  virtual double time() = 0;
  virtual int debug_ct(int stage, double* E, double* B, double* Ephi, double* Phi) = 0;
  virtual int debug_faces(int dim, int* npair_out, long* nface_out, int* fIndex, int* L, int* Rr,
                          int* LRtype, double* phic, double* dA) = 0;
  virtual int debug_grad(double* gp, double* gr, double* gz) = 0;
  virtual int divb(double* div, double* scale) = 0;
  virtual int planets(disco_planet* out, int max, int* n) = 0;
  virtual int set_sweep(int on) = 0;
  // GRMHD cons2prim with a learned starting point (mlp.cuh): attach (null
  // detaches), harvest training pairs, read / reset the iteration counters
  virtual int attach_guess(const MlpDev* m) = 0;
  virtual int harvest(const MlpDev* m, const C2PRecord* rec, int steps) = 0;
  virtual int c2p_stats(long long* out, int reset) = 0;
  virtual int getmindt_noalloc(double* dt) = 0;
  virtual int sink_accum(double* out, int max_bodies, int reset) = 0;
  virtual int report(double* out, int nout) = 0;
  virtual int diag(int op, double* Qrz, long long n, double* t_avg, const double* set, double set_t) = 0;
  // batch support: launch one full step (getmindt + timestep) from piph
  // parity `par` on the instance's stream, then account for nsteps steps
  // taken outside the instance's own run()
  virtual void launch_step(int par) = 0;
  virtual int cur_parity() const = 0;
  virtual cudaStream_t stream() const = 0;
  virtual int after_external_steps(int nsteps, long long nodes) = 0;
  // a new group holding this instance alone, or null if its launch sequence
  // has stages the multi-instance kernels do not cover
  virtual MultiPlanBase* new_multi_plan() { return nullptr; }
  long N = 0, Nreal = 0;
};

template <class Phys, typename R, int NQ>
struct MultiPlan;

// The dynamic shared-memory limit is an attribute of the kernel function,
// shared by every instance in the process: only ever raise it, so a smaller
// instance created later cannot lower the limit a larger one relies on.
template <typename K>
static cudaError_t raise_smem_limit(K* kernel, size_t bytes) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kernel);
  if (e != cudaSuccess) return e;
  if ((size_t)a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename T>
static int dalloc(T** p, size_t n, std::vector<void*>& keep) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    disco_set_error("cudaMalloc failed");
    return DISCO_E_NOMEM;
  }
  keep.push_back((void*)*p);
  return 0;
}

struct KTimer {
  bool on = false;
  cudaStream_t st = nullptr;
  struct Rec { const char* name; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  cudaEvent_t cur_a = nullptr;
  void begin() {
    if (!on) return;
    cudaEventCreate(&cur_a);
    cudaEventRecord(cur_a, st);
  }
  void end(const char* name) {
    if (!on) return;
    cudaEvent_t b;
    cudaEventCreate(&b);
    cudaEventRecord(b, st);
    recs.push_back({name, cur_a, b});
  }
};

#define LAUNCH(NAME, ...)            \
  do {                               \
    kt.begin();                      \
    __VA_ARGS__;                     \
    kt.end(NAME);                    \
    ++g_launches;                    \
  } while (0)

template <class Phys, typename R, int NQ>
struct Instance : InstanceBase {
  KTimer kt;
  void* flush_buf = nullptr;
  size_t flush_size = 0;
  DevParams P{};
  DevState<R> S{};
  CtStateT<R> C{};
  bool ct = false;
  std::vector<void*> keep;
  cudaStream_t st = nullptr;
  int Nr = 0, Nz = 0, nring = 0, npair[2] = {0, 0};
  int maxNf[2] = {0, 0};
  std::vector<int> face_off_h[2];   // host copy of face_off
  double* piph_buf[2] = {nullptr, nullptr};
  int parity = 0;  // which piph buffer is current
  int planets_id = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  size_t edge_smem = 0;
  long nev = 0;   // edge-walk events per substep (cache size)
  int maxring = 0;
  int graph_nodes = 0;
  double host_t = 0;
  std::vector<double> ring_Om_h;   // ring frames (host copy)

  // FP64 staging of the primitives for download / upload on the mixed path
  // (NQ N doubles), allocated at the first transfer and kept: a per-call
  // allocation and release of this size cost more than the copy itself
  double* stage64 = nullptr;
  double* staging() {
    if (!stage64 && cudaMalloc(&stage64, sizeof(double) * NQ * N) != cudaSuccess) {
      cudaGetLastError();
      stage64 = nullptr;
    }
    return stage64;
  }

  ~Instance() override {
    if (stage64) cudaFree(stage64);
    if (flush_buf) cudaFree(flush_buf);
    for (int i = 0; i < 2; ++i)
      if (graph[i]) cudaGraphExecDestroy(graph[i]);
    if (st) cudaStreamDestroy(st);
    for (void* p : keep) cudaFree(p);
  }

  int blocks(long n, int b = 256) const { return (int)((n + b - 1) / b); }
  // k_ct_flip: LRtype bytes (padded to 16) + the flagged-face list (Nf + 1 ints)
  size_t flip_smem(int d) const { return (size_t)((maxNf[d] + 15) & ~15) + 4 * ((size_t)maxNf[d] + 1); }

  void set_piph(int par) {
    S.piph = piph_buf[par];
    S.piph_out = piph_buf[par ^ 1];
  }

  int device = 0;   // the device current at create: the instance's memory and stream live there
  int create(const disco_host_domain* dom) {
    const disco_params& p = dom->par;
    CK(cudaGetDevice(&device));
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    Nr = dom->Nr; Nz = dom->Nz; nring = Nr * Nz;
    N = dom->Ncell;
    // cell-component indices q*N + c are int32: NQ*N must stay below 2^31
    // (face-component indices use 64-bit products)
    if ((long long)N * dom->num_q >= 0x7fffffffLL) {
      disco_set_error("too many cells for int32 cell-component indexing (num_q * Ncell >= 2^31)");
      return DISCO_E_ARG;
    }
    // ---- parameters (set*Params pushes, domain.c:259-270)
    P.Nr = Nr; P.Nz = Nz; P.NgRa = dom->NgRa; P.NgRb = dom->NgRb; P.NgZa = dom->NgZa; P.NgZb = dom->NgZb;
    P.Ncell = N; P.num_q = dom->num_q; P.num_c = dom->mod.num_c; P.phi_max = dom->phi_max;
    P.gamma_law = p.Adiabatic_Index; P.rho_floor = p.Density_Floor; P.p_floor = p.Pressure_Floor;
    P.explicit_viscosity = p.viscosity; P.mach = p.Disk_Mach;
    P.include_viscosity = p.visc_flag; P.isothermal = p.isothermal_flag; P.alpha_flag = p.alpha_flag;
    P.polar_sources = dom->mod.hydro == DISCO_HYDRO_EULER ? (p.NoBC_Rmin == 1) : (dom->NgRa == 0);
    P.riemann_solver = p.Riemann_Solver; P.mesh_motion = p.Mesh_Motion;
    P.PLM = p.PLM; P.CFL = p.CFL; P.maxDT = p.maxDT;
    P.meshOmChoice = p.Exact_Mesh_Omega; P.enOmChoice = p.Energy_Omega; P.cs2Choice = p.Cs2_Profile;
    P.Omega0 = p.RotOmega; P.om_M = p.metricPar2; P.om_r1 = p.initPar2; P.om_H0 = p.initPar4;
    P.eps = p.grav_eps;
    P.rot_flag = p.RotFrame; P.rot_omega = p.RotOmega; P.rot_d = p.RotD;
    P.grav2D = p.grav2D;
    P.polar_r = P.polar_p = (p.NoBC_Rmin == 1);    // planet.c:13-18 (cylindrical)
    {
      const double rp0 = dom->r_jph[1], rm0 = dom->r_jph[0];   // r_jph[0], r_jph[-1]
      P.geom_bd_r = dom->NgRa == 0 && !(rp0 < 0.0 || fabs(rm0) > 1.0e-10 * rp0);
    }
    P.Npl = dom->Npl;
    P.initial_id = dom->mod.initial; P.boundary_id = dom->mod.boundary;
    double icp[8] = {p.initPar1, p.initPar2, p.initPar3, p.initPar4, p.initPar5, p.initPar6, p.initPar7, p.initPar8};
    for (int i = 0; i < 8; ++i) P.ic[i] = icp[i];
    for (int i = 0; i < 4; ++i) P.ic_aux[i] = dom->ic_aux[i];
    P.t_end = 0.0;
    if ((long)nring >= (1L << 24) || Nr >= (1 << 16)) {
      disco_set_error("grid too large for the ring index arithmetic (Nr*Nz < 2^24, Nr < 2^16)");
      return DISCO_E_ARG;
    }
    P.mul_nr = ((1ull << 40) + (unsigned long long)Nr - 1) / (unsigned long long)Nr;
    P.mul_nr1 = Nr > 1 ? ((1ull << 40) + (unsigned long long)(Nr - 1) - 1) / (unsigned long long)(Nr - 1) : 0;
    P.f.gamma_law = (float)P.gamma_law; P.f.rho_floor = (float)P.rho_floor; P.f.p_floor = (float)P.p_floor;
    P.f.explicit_viscosity = (float)P.explicit_viscosity; P.f.mach = (float)P.mach; P.f.PLM = (float)P.PLM;
    P.f.Omega0 = (float)P.Omega0; P.f.om_M = (float)P.om_M; P.f.om_r1 = (float)P.om_r1;
    P.f.om_H0 = (float)P.om_H0; P.f.eps = (float)P.eps;
    planets_id = dom->mod.planets;
    if (!Phys::MHD && P.riemann_solver == SOLVER_HLLD) {
      disco_set_error("Riemann_Solver = HLLD with a hydro module (riemann.c:19-22)");
      return DISCO_E_MODULE;
    }
    if (p.sinkType < 0 || p.sinkType > 3 || (p.nozzleType != 0 && p.nozzleType != 1)) {
      disco_set_error("Sink_Type 0-3 and Nozzle_Type 0-1 are the sink.c source terms");
      return DISCO_E_MODULE;
    }
    P.sink_type = p.sinkType;
    P.nozzle_type = p.nozzleType;
    P.sink_bodies = dom->Npl;
    if (p.sinkNumber > 0 && p.sinkNumber < dom->Npl) P.sink_bodies = p.sinkNumber;   // sink.c:163
    {
      const double sp[5] = {p.sinkPar1, p.sinkPar2, p.sinkPar3, p.sinkPar4, p.sinkPar5};
      const double np[4] = {p.nozzlePar1, p.nozzlePar2, p.nozzlePar3, p.nozzlePar4};
      for (int i = 0; i < 5; ++i) P.sink_par[i] = sp[i];
      for (int i = 0; i < 4; ++i) P.nozzle_par[i] = np[i];
    }
    P.cool_type = p.coolType;
    P.cool_beta = p.coolPar1;
    P.damp_type[0] = p.dampInnerType; P.damp_type[1] = p.dampOuterType;
    P.damp_type[2] = p.dampUpperType; P.damp_type[3] = p.dampLowerType;
    P.damp_len[0] = p.dampLenInner; P.damp_len[1] = p.dampLenOuter;
    P.damp_len[2] = p.dampLenUpper; P.damp_len[3] = p.dampLenLower;
    P.damp_time[0] = p.dampTimeInner; P.damp_time[1] = p.dampTimeOuter;
    P.damp_time[2] = p.dampTimeUpper; P.damp_time[3] = p.dampTimeLower;
    P.dom_rmin = p.rmin; P.dom_rmax = p.rmax; P.dom_zmax = p.zmax;
    P.twoD = dom->Nz == 1;
    // the extra-sources variant of the update: cooling, damping, sinks, nozzle
    P.cool_damp = (p.coolType == 1 || p.coolType == 2) ||
                  p.dampInnerType > 0 || p.dampOuterType > 0 || p.dampUpperType > 0 || p.dampLowerType > 0 ||
                  p.sinkType != 0 || p.nozzleType != 0;
    if (P.cool_damp && Phys::GR) {
      disco_set_error("cooling/damping/sinks are built for the Newtonian modules");
      return DISCO_E_MODULE;
    }
    if (p.Timestep != 0 && p.Timestep != 3) {
      // Timestep 1 runs forward Euler and then the RK2 pair as well
      // (timestep.c:29-49: the RK2 branch is the else of the RK3 test),
      // blending against the state before the Euler step
      disco_set_error("Timestep 0 (RK2) and 3 (RK3) are built");
      return DISCO_E_MODULE;
    }
    rk3 = p.Timestep == 3;
    ct = Phys::MHD && !Phys::GR && dom->mod.ct_mode == 2 && p.CT;
    P.gr_M = p.metricPar2;
    P.gr_kerr = dom->mod.metric == DISCO_METRIC_KERR_KS_RPZ ? 1 : 0;
    P.gr_a = P.gr_kerr ? p.metricPar3 : 0.0;
    if constexpr (Phys::GR) {
      // the GRMHD module as built: FP64, HLL, cell-centred B (CT_MODE 0), a
      // static mesh, adiabatic, no viscosity, no rotating frame, no planets
      const char* why = nullptr;
      if (kMix<R>) why = "GRMHD runs on the FP64 path only (precision 0)";
      else if (P.riemann_solver != SOLVER_HLL) why = "GRMHD is built with the HLL solver only (Riemann_Solver 0)";
      else if (dom->mod.ct_mode != 0) why = "GRMHD is built with cell-centred B only (CT_MODE 0)";
      else if (P.mesh_motion != 0) why = "GRMHD is built on a static mesh only (Mesh_Motion 0)";
      else if (P.isothermal) why = "GRMHD is built for the adiabatic equation of state only";
      else if (P.include_viscosity || P.rot_flag) why = "GRMHD with viscosity or a rotating frame is not built";
      else if (dom->mod.planets != 0) why = "GRMHD takes PLANETS=none";
      else if (P.gr_M <= 0.0) why = "GRMHD needs Metric_Par2 (the black-hole mass) > 0";
      else if (P.gr_kerr && !(fabs(P.gr_a) < P.gr_M)) why = "kerr_ks_rpz needs |Metric_Par3| (the spin) < Metric_Par2";
      if (why) {
        disco_set_error(why);
        return DISCO_E_MODULE;
      }
    }
    if (Phys::MHD && !Phys::GR) {
      if (!ct) {
        disco_set_error("MHD is built with constrained transport only (CT_MODE 2, Constrained_Transport 1)");
        return DISCO_E_MODULE;
      }
      const bool hll_hllc = P.riemann_solver == SOLVER_HLL || P.riemann_solver == SOLVER_HLLC;
      if (P.riemann_solver != SOLVER_HLLD && !(hll_hllc && !kMix<R>)) {
        disco_set_error("MHD is built with HLLD (Riemann_Solver 2), and with HLL / HLLC (0, 1) on the "
                        "FP64 path");
        return DISCO_E_MODULE;
      }
      if (dom->NgRa == 0 || dom->NgRb == 0 || (dom->Nz > 1 && (dom->NgZa == 0 || dom->NgZb == 0))) {
        disco_set_error("MHD with coordinate (NoBC) boundaries is not built");
        return DISCO_E_MODULE;
      }
      if (dom->Nz <= 1) {
        disco_set_error("MHD with CT_MODE 2 needs Num_Z > 1");
        return DISCO_E_MODULE;
      }
    }
    n_bc_ops = disco_bc_plugin_ops(dom->mod.boundary, bc_ops);
    if (n_bc_ops < 0) {
      disco_set_error("BOUNDARY plugin not built");
      return DISCO_E_MODULE;
    }
    for (int o = 0; o < n_bc_ops; ++o) {   // the source rings of the copies must be real rings
      const int dim = bc_ops[o].side < 2 ? 1 : 2, side = bc_ops[o].side & 1;
      const int ng = dim == 1 ? (side ? dom->NgRb : dom->NgRa) : (side ? dom->NgZb : dom->NgZa);
      const int nreal = dim == 1 ? dom->Nr - dom->NgRa - dom->NgRb : dom->Nz - dom->NgZa - dom->NgZb;
      const int need = bc_ops[o].op == DISCO_BCOP_ZEROGRAD ? 1 : ng;
      const bool copy = bc_ops[o].op >= DISCO_BCOP_ZEROGRAD && bc_ops[o].op <= DISCO_BCOP_NOSLIP;
      if (copy && ng > 0 && nreal < need) {
        disco_set_error("boundary copy needs more real rings than the domain has");
        return DISCO_E_ARG;
      }
    }

    for (int jk = 0; jk < nring; ++jk) maxring = std::max(maxring, dom->Np[jk]);
    if ((maxring + 1) * 8 > 48 * 1024)
      CK(raise_smem_limit(k_wcell_avg<R>, (size_t)(maxring + 1) * 8));
    // ---- index arrays
    std::vector<int> ring_off(nring + 1), cell_ring(N);
    for (int jk = 0; jk <= nring; ++jk) ring_off[jk] = (int)dom->ring_off[jk];
    for (int jk = 0; jk < nring; ++jk)
      for (int c = ring_off[jk]; c < ring_off[jk + 1]; ++c) cell_ring[c] = jk;
    Nreal = 0;
    for (int k = dom->NgZa; k < Nz - dom->NgZb; ++k)
      for (int j = dom->NgRa; j < Nr - dom->NgRb; ++j) Nreal += dom->Np[j + Nr * k];

    int rc;
    int *d_ring_off, *d_cell_ring;
    double *d_r, *d_z;
#define A(ptr, n) do { if ((rc = dalloc(ptr, (size_t)(n), keep))) return rc; } while (0)
    A(&d_ring_off, nring + 1); A(&d_cell_ring, N); A(&d_r, Nr + 1); A(&d_z, Nz + 1);
    CK(cudaMemcpy(d_ring_off, ring_off.data(), sizeof(int) * (nring + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_cell_ring, cell_ring.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_r, dom->r_jph, sizeof(double) * (Nr + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_z, dom->z_kph, sizeof(double) * (Nz + 1), cudaMemcpyHostToDevice));
    S.N = (int)N; S.cell_ring = d_cell_ring; S.ring_off = d_ring_off; S.r_jph = d_r; S.z_kph = d_z;
    A(&S.ring_rc, nring); A(&S.ring_r23, nring);
    A(&S.ring_rc_r, nring); A(&S.ring_r1_r, nring); A(&S.ring_vol_r, nring); A(&S.ring_dA_r, nring);
    A(&S.ring_r23_r, nring); A(&S.ring_zc_r, nring);
    A(&S.ring_Om, nring); A(&S.ring_Om_r, nring); A(&S.ring_Lsh, nring);
    A(&S.ring_gL_r, nring); A(&S.ring_gR_r, nring); A(&S.ring_cfl, 3 * (size_t)nring);
    for (int d = 0; d < 2; ++d) { A(&S.ring_At_r[d], nring); A(&S.ring_dl_r[d], nring); }
    A(&piph_buf[0], N); A(&piph_buf[1], N);
    A(&S.dphi, N); A(&S.wiph, N);
    if (kMix<R>) {
      A(&S.dphi_r, N);
    } else {
      S.dphi_r = (R*)S.dphi;
    }
    A(&S.prim, (size_t)NQ * N); A(&S.cons, (size_t)NQ * N);
    if (kMix<R>) A(&S.RKdU, (size_t)NQ * N);
    else A(&S.RKcons, (size_t)NQ * N);
    A(&S.gradp, (size_t)NQ * N); A(&S.gradr, (size_t)NQ * N); A(&S.gradz, (size_t)NQ * N);
    A(&S.fphi, (size_t)NQ * N);
    A(&S.anchor, nring);
    CK(cudaMemset(S.gradr, 0, sizeof(R) * NQ * N));
    CK(cudaMemset(S.gradz, 0, sizeof(R) * NQ * N));
    CK(cudaMemset(S.wiph, 0, sizeof(double) * N));
    // faces per dimension
    for (int d = 0; d < 2; ++d) {
      int dim = d + 1;
      int np = 0;
      if (dim == 1 && Nr > 1) np = (Nr - 1) * Nz;
      if (dim == 2 && Nz > 1) np = Nr * (Nz - 1);
      npair[d] = np;
      std::vector<int> off(np + 1, 0);
      int mx = 0;
      for (int pr = 0; pr < np; ++pr) {
        int L, Rr;
        if (dim == 1) { int j = pr % (Nr - 1), k = pr / (Nr - 1); L = j + Nr * k; Rr = j + 1 + Nr * k; }
        else { int j = pr % Nr, k = pr / Nr; L = j + Nr * k; Rr = j + Nr * (k + 1); }
        int nf = dom->Np[L] + dom->Np[Rr];
        off[pr + 1] = off[pr] + nf;
        if (nf > mx) mx = nf;
      }
      maxNf[d] = mx;
      int nf = off[np];
      S.nf[d] = nf;
      int* d_off;
      A(&d_off, np + 1);
      CK(cudaMemcpy(d_off, off.data(), sizeof(int) * (np + 1), cudaMemcpyHostToDevice));
      S.face_off[d] = d_off;
      face_off_h[d] = off;
      A(&S.fL[d], nf); A(&S.fR[d], nf); A(&S.fLR[d], nf); A(&S.fphic[d], nf); A(&S.fdA[d], nf);
      A(&S.fdpL[d], nf); A(&S.fdpR[d], nf);
      A(&S.pdxL[d], np); A(&S.pdxR[d], np); A(&S.pdxs[d], np); A(&S.prad[d], np);
      A(&S.pidxs[d], np); A(&S.pdA[d], np); A(&S.pdOm[d], np); A(&S.pcX[d], np);
      A(&S.fflux[d], (size_t)NQ * nf);
      A(&S.run_up_s[d], N); A(&S.run_up_e[d], N); A(&S.run_dn_s[d], N); A(&S.run_dn_e[d], N);
      A(&S.nb_up[d], N); A(&S.nb_dn[d], N);
      if (ct) {
        A(&S.fErz[d], nf); A(&S.fBrz[d], nf); A(&S.fEphi[d], nf);
        A(&S.ffrL[d], nf); A(&S.ffrR[d], nf); A(&S.fdp1[d], nf); A(&S.fdp2[d], nf);
      }
      C.last_pair[d] = np - 1;
      if (np > 0 && mx * 13 + 64 > 48 * 1024) {
        CK(raise_smem_limit(k_faces<R>, (size_t)mx * 13 + 64));
      }
    }
    A(&S.fslope, (size_t)NQ * std::max(S.nf[0], S.nf[1]));
    {   // chunks of kTileCells consecutive cells of each ring
      std::vector<int> cr, ci;
      for (int jk = 0; jk < nring; ++jk)
        for (int i0 = 0; i0 < dom->Np[jk]; i0 += kTileCells) { cr.push_back(jk); ci.push_back(i0); }
      int *d_cr, *d_ci;
      A(&d_cr, cr.size()); A(&d_ci, ci.size());
      CK(cudaMemcpy(d_cr, cr.data(), sizeof(int) * cr.size(), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(d_ci, ci.data(), sizeof(int) * ci.size(), cudaMemcpyHostToDevice));
      S.chunk_ring = d_cr; S.chunk_i0 = d_ci; S.nchunk = (int)cr.size();
    }
    {   // ghost cells filled by the boundary plugin (fixed.c: r ghosts;
        // fixed3d.c: r and z ghosts), as chunks of kTileCells cells per ring
      // a periodic dimension's ghosts come from the ring copy instead
      // (R_Periodic, Z_Periodic: onestep.c:166-172 skips that dimension's
      // boundary_trans)
      std::vector<int> gr, gi;
      for (int jk = 0; jk < nring; ++jk) {
        int k = jk / Nr, j = jk - k * Nr;
        bool rghost = (j < P.NgRa) || (j >= Nr - P.NgRb);
        bool zghost = (k < P.NgZa) || (k >= Nz - P.NgZb);
        bool rfill = rghost && Nr > 1 && !p.R_Periodic, zfill = zghost && Nz > 1 && !p.Z_Periodic;
        bool fill = P.boundary_id == 0 ? rfill : P.boundary_id == 1 ? (rfill || zfill) : false;
        if (!fill) continue;
        for (int i0 = 0; i0 < dom->Np[jk]; i0 += kTileCells) { gr.push_back(jk); gi.push_back(i0); }
      }
      int *d_gr = nullptr, *d_gi = nullptr;
      if (!gr.empty()) {
        A(&d_gr, gr.size()); A(&d_gi, gi.size());
        CK(cudaMemcpy(d_gr, gr.data(), sizeof(int) * gr.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_gi, gi.data(), sizeof(int) * gi.size(), cudaMemcpyHostToDevice));
      }
      S.ghost_ring = d_gr; S.ghost_i0 = d_gi; S.nghost = (int)gr.size();
      // horizon3d / horizon: the rings the plugin excises, when a pass
      // that excises runs at all (main.c:53-61: r when Nr > 1 and not
      // R_Periodic; horizon.c also after the z pass, when Nz > 1 and not
      // Z_Periodic)
      std::vector<int> hr;
      std::vector<unsigned char> hx(nring, 0);
      bool hor = false, cut = false, rpass = Nr > 1 && !p.R_Periodic, zpass = Nz > 1 && !p.Z_Periodic;
      for (int o = 0; o < n_bc_ops; ++o)
        if (bc_ops[o].op == DISCO_BCOP_HORIZON) {
          const bool zop = bc_ops[o].side >= 2;
          if ((zop && zpass) || (!zop && rpass)) { hor = true; cut = bc_ops[o].arg == 1; }
        }
      if (hor)
        for (int jk = 0; jk < nring; ++jk) {
          const int k = jk / Nr, j = jk - k * Nr;
          const double *rj = dom->r_jph + 1, *zk = dom->z_kph + 1;
          if (cut ? disco_bc_horizon_cut_ring(rj, zk, Nz, j, k) : disco_bc_horizon_ring(rj, zk, j, k)) {
            hr.push_back(jk);
            hx[jk] = 1;
          }
        }
      S.hor_rings = nullptr; S.ring_excised = nullptr; S.nhor = (int)hr.size();
      // horizon_bin: the candidate rings of its two holes, for each pass
      // that runs, and the per-cell flag its cut-outs set
      std::vector<int> hl;
      bool holes = false;
      for (int o = 0; o < n_bc_ops; ++o)
        if (bc_ops[o].op == DISCO_BCOP_HOLES) {
          const bool zop = bc_ops[o].side >= 2;
          holes = holes || (zop && zpass) || (!zop && rpass);
        }
      if (holes)
        for (int h = 0; h < 2; ++h)
          for (int jk = 0; jk < nring; ++jk) {
            const int k = jk / Nr, j = jk - k * Nr;
            double rc, zc;
            if (disco_bc_hole_ring(dom->r_jph + 1, dom->z_kph + 1, Nr, Nz, j, k, h, &rc, &zc))
              hl.push_back(2 * jk + h);
          }
      S.hole_list = nullptr; S.cell_excised = nullptr; S.nhole = (int)hl.size();
      if (holes) {
        unsigned char* d_cx;
        A(&d_cx, (size_t)N);
        CK(cudaMemset(d_cx, 0, (size_t)N));
        S.cell_excised = d_cx;
        if (!hl.empty()) {
          int* d_hl;
          A(&d_hl, hl.size());
          CK(cudaMemcpy(d_hl, hl.data(), sizeof(int) * hl.size(), cudaMemcpyHostToDevice));
          S.hole_list = d_hl;
        }
      }
      if (!hr.empty()) {
        int* d_hr;
        unsigned char* d_hx;
        A(&d_hr, hr.size()); A(&d_hx, (size_t)nring);
        CK(cudaMemcpy(d_hr, hr.data(), sizeof(int) * hr.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_hx, hx.data(), (size_t)nring, cudaMemcpyHostToDevice));
        S.hor_rings = d_hr; S.ring_excised = d_hx;
      }
      S.ghost_tab = nullptr;
      if (S.nghost > 0 && (P.initial_id == 1 || P.initial_id == 2 || P.initial_id == 5)) {   // axisymmetric
        double* tab = nullptr;
        A(&tab, (size_t)nring * NQ);
        k_ghost_tab<R, NQ><<<(int)blocks(nring, 128), 128, 0, st>>>(P, nring, tab, S.r_jph, S.z_kph);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        S.ghost_tab = tab;
      }
    }
    {   // periodic ghost rings and their sources, r then z (exchange.c)
      std::vector<int> dst, src;
      for (int dim = 1; dim <= 2; ++dim) {
        for (int k = 0; k < Nz; ++k)
          for (int j = 0; j < Nr; ++j) {
            const int s = disco_periodic_source(dom, dim, j, k);
            if (s < 0) continue;
            dst.push_back(j + Nr * k);
            src.push_back(s);
          }
        n_pcopy[dim - 1] = (int)dst.size() - (dim == 2 ? n_pcopy[0] : 0);
      }
      if (!dst.empty()) {
        A(&pc_dst, dst.size()); A(&pc_src, src.size());
        CK(cudaMemcpy(pc_dst, dst.data(), sizeof(int) * dst.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(pc_src, src.data(), sizeof(int) * src.size(), cudaMemcpyHostToDevice));
      }
    }
    A(&S.planets, MAX_PL); A(&S.scal, SC_COUNT); A(&S.errs, 1);
    sink_on = P.sink_type != 0 && P.sink_bodies > 0;
    if (sink_on) {
      A(&S.sink_acc, 2 * MAX_PL * kSinkAcc);
      A(&S.sink_part, (size_t)blocks(N) * MAX_PL * kSinkAcc);
      CK(cudaMemset(S.sink_acc, 0, sizeof(double) * 2 * MAX_PL * kSinkAcc));
    }
    diag_id = dom->mod.analysis;
    diag_n = diag_count(diag_id);
    if (diag_id == DISCO_DIAG_MHDMRI && NQ < 8) {
      disco_set_error("ANALYSIS=diag_mhdmri reads magnetic fields: MHD or GRMHD modules only");
      return DISCO_E_MODULE;
    }
    if (diag_id == DISCO_DIAG_GRMHDMRI && !Phys::GR) {
      disco_set_error("ANALYSIS=diag_grmhdmri reads the metric: GRMHD module only");
      return DISCO_E_MODULE;
    }
    if (diag_n) {
      A(&diag_Qrz, (size_t)nring * diag_n);
      CK(cudaMemset(diag_Qrz, 0, sizeof(double) * nring * diag_n));
    }
    S.ct = ct ? 1 : 0;
    if (ct) {
      A(&S.Eraw, (size_t)8 * N); A(&S.Braw, (size_t)8 * N);
      A(&C.Phi, (size_t)5 * N); A(&C.RKPhi, (size_t)5 * N); A(&C.Efin, (size_t)4 * N);
      A(&C.Ephi, (size_t)4 * N); A(&C.errs, 1);
      CK(cudaMemset(S.Eraw, 0, sizeof(R) * 8 * N)); CK(cudaMemset(S.Braw, 0, sizeof(R) * 8 * N));
      CK(cudaMemset(C.Phi, 0, sizeof(double) * 5 * N)); CK(cudaMemset(C.RKPhi, 0, sizeof(double) * 5 * N));
      CK(cudaMemset(C.Ephi, 0, sizeof(R) * 4 * N)); CK(cudaMemset(C.errs, 0, 8));
      if (std::max(maxNf[0], maxNf[1]) > 64 * 256) {
        disco_set_error("CT flip repair handles at most 16384 faces per ring pair");
        return DISCO_E_ARG;
      }
      for (int d = 0; d < 2; ++d)
        if (flip_smem(d) > 48 * 1024)
          CK(raise_smem_limit(k_ct_flip<R>, flip_smem(d)));
      edge_smem = (size_t)4 * maxring * 8;
      // edge-walk event cache: one event per cell of each quad's four rings
      {
        std::vector<int> qoff((size_t)(Nr - 1) * (Nz - 1) + 1, 0);
        long tot = 0;
        for (int k = 0; k + 1 < Nz; ++k)
          for (int j = 0; j + 1 < Nr; ++j) {
            int qd = j + (Nr - 1) * k;
            qoff[qd] = (int)tot;
            tot += dom->Np[j + Nr * k] + dom->Np[j + 1 + Nr * k] + dom->Np[j + Nr * (k + 1)] +
                   dom->Np[j + 1 + Nr * (k + 1)];
          }
        qoff.back() = (int)tot;
        nev = tot;
        size_t need = (size_t)tot * (sizeof(int4) + 1 + sizeof(R));
        size_t fr = 0, tt = 0;
        cudaMemGetInfo(&fr, &tt);
        A(&C.ev_ok, 1);
        CK(cudaMemset(C.ev_ok, 0, sizeof(int)));
        // kept only where it leaves room (8 GB) for the rest of the run
        if (tot < 0x7fffffffL && fr > need + ((size_t)8 << 30)) {
          int* d_q;
          A(&d_q, qoff.size());
          CK(cudaMemcpy(d_q, qoff.data(), sizeof(int) * qoff.size(), cudaMemcpyHostToDevice));
          C.quad_ev_off = d_q;
          A(&C.ev_cid, tot); A(&C.ev_flag, tot); A(&C.ev_dl, tot);
        }
      }
      if (edge_smem > 48 * 1024)
        CK(raise_smem_limit(k_ct_edge<R>, edge_smem));
    }
#undef A
    std::vector<DevPlanet> pl(MAX_PL);
    for (int i = 0; i < dom->Npl && i < MAX_PL; ++i) {
      pl[i].r = dom->planets[i].r; pl[i].phi = dom->planets[i].phi; pl[i].M = dom->planets[i].M;
      pl[i].omega = dom->planets[i].omega; pl[i].vr = dom->planets[i].vr;
      pl[i].eps = dom->planets[i].eps; pl[i].type = dom->planets[i].type;
    }
    CK(cudaMemcpy(S.planets, pl.data(), sizeof(DevPlanet) * MAX_PL, cudaMemcpyHostToDevice));
    // report.c's mass ratio and the softening behind its torque cut radii
    report_q = dom->Npl > 1 ? dom->planets[1].M / dom->planets[0].M : 0.0;
    report_soft = p.sinkPar3;
    double scal[SC_COUNT] = {0, dom->t, 0, 0};
    unsigned long long inf = 0x7ff0000000000000ull;
    memcpy(&scal[SC_MIN], &inf, 8);
    CK(cudaMemcpy(S.scal, scal, sizeof scal, cudaMemcpyHostToDevice));
    CK(cudaMemset(S.errs, 0, sizeof(DevErrs)));
    host_t = dom->t;

    // ring frames of the mixed path (0 on the FP64 path): the ring mean of
    // the initial omega of the real rings, the nearest real ring's for ghosts
    ring_Om_h.assign(nring, 0.0);
    if (kMix<R>) {
      const int NgRa = dom->NgRa, NgRb = dom->NgRb, NgZa = dom->NgZa, NgZb = dom->NgZb;
      for (int jk = 0; jk < nring; ++jk) {
        int j = jk % Nr, k = jk / Nr;
        int jr = std::min(std::max(j, NgRa), Nr - NgRb - 1);
        int kr = std::min(std::max(k, NgZa), Nz - NgZb - 1);
        int src = jr + Nr * kr;
        double sum = 0;
        for (long c = dom->ring_off[src]; c < dom->ring_off[src + 1]; ++c)
          sum += dom->prim[(long)UPP * N + c];
        long np_ = dom->ring_off[src + 1] - dom->ring_off[src];
        ring_Om_h[jk] = np_ > 0 ? sum / (double)np_ : 0.0;
      }
      // a periodic ghost ring takes its source ring's frame (r, then z)
      for (int dim = 1; dim <= 2; ++dim)
        for (int jk = 0; jk < nring; ++jk) {
          const int s = disco_periodic_source(dom, dim, jk % Nr, jk / Nr);
          if (s >= 0) ring_Om_h[jk] = ring_Om_h[s];
        }
    }
    CK(cudaMemcpy(S.ring_Om, ring_Om_h.data(), sizeof(double) * nring, cudaMemcpyHostToDevice));
    LAUNCH("ring_geom", (k_ring_geom<R><<<blocks(nring), 256, 0, st>>>(P, S, nring)));
    for (int d = 0; d < 2; ++d)
      if (npair[d]) LAUNCH("pair_geom", (k_pair_geom<R><<<blocks(npair[d]), 256, 0, st>>>(P, S, d + 1, npair[d])));
    // ---- state upload + set-up kernels (setupCells, domain.c:283-385)
    CK(cudaMemcpy(piph_buf[0], dom->piph, sizeof(double) * N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(S.dphi, dom->dphi, sizeof(double) * N, cudaMemcpyHostToDevice));
    sync_dphi_r();
    parity = 0;
    set_piph(0);
    double* d_prim0;
    CK(cudaMalloc(&d_prim0, sizeof(double) * NQ * N));
    CK(cudaMemcpy(d_prim0, dom->prim, sizeof(double) * NQ * N, cudaMemcpyHostToDevice));
    // a restarted domain carries its face fluxes: setupCells then skips
    // set_B_fields and runs prim2cons + cons2prim on the file's primitives
    // (domain.c:211-238)
    const bool phi_in = ct && dom->Phi && dom->num_faces == 5;
    k_init_cells<Phys, R, NQ><<<blocks(N), 256, 0, st>>>(P, S, d_prim0, (ct && !phi_in) ? 0 : 1);
    ++g_launches;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    cudaFree(d_prim0);
    if (phi_in) {
      CK(cudaMemcpy(C.Phi, dom->Phi, sizeof(double) * 5 * N, cudaMemcpyHostToDevice));
    } else if (ct) {   // set_B_fields (bfields.c:13-86), then cons2prim (domain.c:365-382)
      launch_faces();
      LAUNCH("ct_init", (k_ct_init_phi0<R><<<blocks(N), 256, 0, st>>>(P, S, C)));
      for (int d = 0; d < 2; ++d)
        if (npair[d]) LAUNCH("ct_init", (k_ct_init_face_phi<R><<<blocks(S.nf[d]), 256, 0, st>>>(P, S, C, d + 1)));
      LAUNCH("ct_b2c", (k_ct_b2c<R, NQ><<<blocks(N), 256, 0, st>>>(P, S, C, 0)));
      LAUNCH("c2p", (k_c2p<Phys, R, NQ><<<blocks(N), 256, 0, st>>>(P, S)));
    }
    launch_boundary();
    launch_wcell();
    launch_faces();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    // the staged phi sweep of the mixed path (not with explicit viscosity,
    // whose phi fluxes read the transverse gradients of plm_trans)
    if (kMix<R> && !P.include_viscosity) {
      sweep = make_sweep_tmap(&tm_prim, (const float*)S.prim, (unsigned long long)NQ * N) == 0 &&
              make_sweep_tmap(&tm_dphi, (const float*)S.dphi_r, (unsigned long long)N) == 0;
      sweep_ok = sweep;
    }
    return 0;
  }
  bool sweep_ok = false;   // the tensor maps exist
  // test access: the staged sweep on (1) or the separate plm_phi / flux_phi
  // kernels (0); returns the setting in force
  int set_sweep(int on) override {
    sweep = on && sweep_ok;
    sweep_no_copies = sweep && on == 2;
    for (int i = 0; i < 2; ++i)
      if (graph[i]) { cudaGraphExecDestroy(graph[i]); graph[i] = nullptr; }
    return sweep ? 1 : 0;
  }
  bool sweep = false;   // k_phi_sweep in place of k_plm_phi + k_flux_phi
  bool sweep_no_copies = false;   // debug: the sweep issues no copies (its waits run out)
  CUtensorMap tm_prim{}, tm_dphi{};

  // ---- launch helpers -----------------------------------------------------
  void sync_dphi_r() {
    if (kMix<R>) LAUNCH("dphi_r", (k_dphi_r<R><<<blocks(N), 256, 0, st>>>(S)));
  }
  void launch_wcell() {
    if (kMix<R> && P.mesh_motion == 3) {
      LAUNCH("wcell_ring", (k_wcell_ring<R><<<nring, 256, 0, st>>>(P, S)));
      return;
    }
    LAUNCH("wcell", (k_wcell<R, NQ><<<blocks(N), 256, 0, st>>>(P, S)));
    if (P.mesh_motion == 3)
      LAUNCH("wcell_avg", (k_wcell_avg<R><<<nring, 64, (maxring + 1) * sizeof(double), st>>>(P, S)));
  }
  disco_bc_op bc_ops[DISCO_BC_MAX_OPS];
  int n_bc_ops = 0;
  // R_Periodic / Z_Periodic: the ghost rings of that dimension take their
  // source rings' cells (k_periodic_copy)
  int n_pcopy[2] = {0, 0};
  int* pc_dst = nullptr;
  int* pc_src = nullptr;
  void launch_periodic(int dim) {
    const int n = n_pcopy[dim - 1];
    if (!n) return;
    const int o = dim == 1 ? 0 : n_pcopy[0];
    LAUNCH("periodic", (k_periodic_copy<R, NQ><<<n, kTileCells, 0, st>>>(P, S, ct ? C.Phi : nullptr,
                                                                       ct ? C.RKPhi : nullptr, pc_dst + o,
                                                                       pc_src + o)));
  }
  // onestep.c:166-172: exchangeData(r); boundary_trans(r) unless
  // R_Periodic; exchangeData(z); boundary_trans(z) unless Z_Periodic
  void launch_boundary() {
    if (n_bc_ops > 0) {   // plugins written as boundary_functions.c primitives
      launch_periodic(1);
      bool z_started = false;
      for (int o = 0; o < n_bc_ops; ++o) {
        const disco_bc_op& b = bc_ops[o];
        const int dim = b.side < 2 ? 1 : 2, side = b.side & 1;
        if (dim == 2 && !z_started) { launch_periodic(2); z_started = true; }
        if ((dim == 1 && Nr <= 1) || (dim == 2 && Nz <= 1)) continue;
        if ((dim == 1 && n_pcopy[0]) || (dim == 2 && n_pcopy[1])) continue;
        if (b.op == DISCO_BCOP_HOLES) {
          if (S.nhole) LAUNCH("boundary", (k_bc_holes<R, NQ><<<S.nhole, 128, 0, st>>>(P, S)));
          continue;
        }
        if (b.op == DISCO_BCOP_HORIZON) {   // every excised ring, ghosts or not
          if (S.nhor) LAUNCH("boundary", (k_bc_horizon<R, NQ><<<S.nhor, 128, 0, st>>>(P, S, b.arg ? 3 : 0)));
          continue;
        }
        const int ng = dim == 1 ? (side ? P.NgRb : P.NgRa) : (side ? P.NgZb : P.NgZa);
        if (ng == 0) continue;
        const int per_layer = dim == 1 ? Nz : Nr, n = dim == 1 ? Nr : Nz;
        if (b.op <= DISCO_BCOP_FIXED_PHI || b.op == DISCO_BCOP_FIXED_MEAN) {
          const int mode = b.op == DISCO_BCOP_FIXED_MEAN ? 3 : b.op;
          LAUNCH("boundary", (k_bc_init<R, NQ><<<ng * per_layer, 128, 0, st>>>(P, S, dim, side, mode, b.arg,
                                                                               b.pa, b.pb)));
        } else {
          const int mode = b.op - DISCO_BCOP_ZEROGRAD;   // 0 zerograd, 1 reflect, 2 noslip
          for (int l = 0; l < ng; ++l) {   // from the real domain outward
            const int layer = side ? n - ng + l : ng - 1 - l;
            LAUNCH("boundary", (k_bc_copy<R, NQ><<<blocks(per_layer, 64), 64, 0, st>>>(P, S, dim, side, layer,
                                                                                       mode, b.arg)));
          }
        }
      }
      if (!z_started) launch_periodic(2);
      return;
    }
    // fixed / fixed3d fill the non-periodic ghosts in one kernel: after the
    // r copy (its corners then come from the z boundary, as boundary_trans
    // dimension 2 rewrites them) and before the z copy (which rewrites the
    // corners from the source layers)
    launch_periodic(1);
    if (S.nghost > 0)
      LAUNCH("boundary", (k_boundary<R, NQ><<<S.nghost, kTileCells, 0, st>>>(P, S)));
    launch_periodic(2);
  }
  void launch_faces() {
    if (npair[0] == 0 && npair[1] == 0) return;
    LAUNCH("anchor", (k_anchor<R><<<blocks((long)nring * 32), 256, 0, st>>>(P, S, nring)));
    for (int d = 0; d < 2; ++d) {
      if (!npair[d]) continue;
      size_t sm = (size_t)maxNf[d] * 13 + 64;
      LAUNCH(d == 0 ? "faces_r" : "faces_z", (k_faces<R><<<npair[d], 256, sm, st>>>(P, S, d + 1)));
    }
  }
  // plm_trans per dimension: face slopes, then the per-cell gather
  void launch_plm_trans() {
    for (int d = 0; d < 2; ++d) {
      if (!npair[d]) continue;
      dim3 grid(npair[d], (maxNf[d] + 256 * kSlopeFaces - 1) / (256 * kSlopeFaces));
      LAUNCH(d == 0 ? "plm_slopes_r" : "plm_slopes_z",
             (k_plm_slopes<R, NQ><<<grid, 256, 0, st>>>(P, S, d + 1)));
      LAUNCH(d == 0 ? "plm_trans_r" : "plm_trans_z",
             (k_plm_trans<R, NQ><<<dim3(S.nchunk, plm_groups<NQ>()), kTileCells, 0, st>>>(P, S, d + 1)));
    }
  }
  void launch_mindt() {
    LAUNCH("mindt", (k_mindt<Phys, R, NQ><<<blocks(N), 256, 0, st>>>(P, S)));
    LAUNCH("dt_finalize", (k_dt_finalize<<<1, 1, 0, st>>>(P, S.scal)));
  }
  // The ring pairs of the flux sweep across dimension d + 1: jcount x kcount
  // rings from (jmin, kmin); false if there are none (misc.c:464-500; with
  // CT one more layer across the other dimension)
  bool trans_range(int d, int* jmin_o, int* jcount_o, int* kmin_o, int* kcount_o) const {
    if (!npair[d]) return false;
    const int dim = d + 1;
    int jmin, jmax, kmin, kmax;
    if (dim == 1) {
      jmin = P.NgRa == 0 ? 0 : P.NgRa - 1;
      jmax = P.NgRb == 0 ? Nr - 1 : Nr - P.NgRb;
      if (ct) { kmin = P.NgZa == 0 ? 0 : P.NgZa - 1; kmax = P.NgZb == 0 ? Nz : Nz - P.NgZb + 1; }
      else { kmin = P.NgZa; kmax = Nz - P.NgZb; }
    } else {
      if (ct) { jmin = P.NgRa == 0 ? 0 : P.NgRa - 1; jmax = P.NgRb == 0 ? Nr : Nr - P.NgRb + 1; }
      else { jmin = P.NgRa; jmax = Nr - P.NgRb; }
      kmin = P.NgZa == 0 ? 0 : P.NgZa - 1;
      kmax = P.NgZb == 0 ? Nz - 1 : Nz - P.NgZb;
    }
    *jmin_o = jmin; *jcount_o = jmax - jmin; *kmin_o = kmin; *kcount_o = kmax - kmin;
    return *jcount_o > 0 && *kcount_o > 0;
  }
  void launch_trans_fluxes(double fac) {
    for (int d = 0; d < 2; ++d) {
      const int dim = d + 1;
      int jmin, jc, kmin, kc;
      if (!trans_range(d, &jmin, &jc, &kmin, &kc)) continue;
      dim3 grid(jc * kc, (maxNf[d] + 255) / 256);
      LAUNCH(dim == 1 ? "flux_r" : "flux_z",
             (k_flux_trans<Phys, R, NQ><<<grid, 256, 0, st>>>(P, S, dim, jmin, jc, kmin, fac)));
    }
  }
  // one onestep (onestep.c:86-186); mid marks a substep that is neither the
  // first nor the last (RK3's second)
  void substep(double RK, double fac, int first, int mid = 0) {
    if (first) launch_wcell();
    if constexpr (kMix<R>) {
      if (sweep) {   // plm_phi and the phi fluxes from one staged pass
        LAUNCH("phi_sweep", (k_phi_sweep<Phys, R, NQ><<<S.nchunk, kTileCells, 0, st>>>(P, S, fac, tm_prim, tm_dphi,
                                                                                    sweep_no_copies ? 1 : 0)));
        launch_plm_trans();
      }
    }
    if (!sweep) {
      LAUNCH("plm_phi", (k_plm_phi<R, NQ><<<blocks(N), 256, 0, st>>>(P, S)));
      launch_plm_trans();
      LAUNCH("flux_phi", (k_flux_phi<Phys, R, NQ><<<blocks(N), 256, 0, st>>>(P, S, fac)));
    }
    launch_trans_fluxes(fac);
    if (ct) {   // avg_Efields, subtract_advective_B_fluxes, update_B_fluxes (onestep.c:261-265)
      LAUNCH("ct_gather", (k_ct_gather<R><<<blocks(N), 256, 0, st>>>(P, S, C)));
      LAUNCH("ct_avg", (k_ct_avg<R><<<blocks(N), 256, 0, st>>>(P, S, C)));
      LAUNCH("ct_bflux", (k_ct_bflux<R><<<blocks(N), 256, 0, st>>>(P, S, C, fac, RK, first)));
      if (Nz > 1) {
        // first substep: replay the events the last walk recorded (same
        // positions) or walk if there are none; second substep: walk and
        // record them for the next step
        const int mode = C.ev_cid ? (first ? 1 : 2) : 0;
        LAUNCH("ct_edge", (k_ct_edge<R><<<(Nr - 1) * (Nz - 1), 512, edge_smem, st>>>(P, S, C, fac, mode)));
        if (C.ev_cid && first)
          LAUNCH("ct_edge_replay", (k_ct_edge_replay<R><<<(int)((nev + 255) / 256), 256, 0, st>>>(P, S, C, fac, nev)));
        if (C.ev_cid && !first) LAUNCH("ct_edge_flag", (k_set_flag<<<1, 1, 0, st>>>(C.ev_ok, 1)));
      }
    }
    if (sink_on) {   // the sink bodies' accumulators, from the state add_source sees
      LAUNCH("sink_acc", (k_sink_acc<Phys, R, NQ><<<blocks(N), 256, 0, st>>>(P, S, fac)));
      LAUNCH("sink_final", (k_sink_final<<<1, MAX_PL * kSinkAcc, 0, st>>>(S.sink_acc, S.sink_part, (int)blocks(N),
                                                                            RK, first, P.sink_bodies)));
    }
    {
      // GRMHD with a learned starting point: calc_prim is its own pass below
      const int c2p = (ct || mlp_on || rec_on.X) ? 0 : 1;
      const dim3 g((unsigned)blocks(N));
      if (P.cool_damp && mid) LAUNCH("update", (k_update<Phys, R, NQ, true, true><<<g, 256, 0, st>>>(P, S, RK, fac, first, c2p)));
      else if (P.cool_damp)   LAUNCH("update", (k_update<Phys, R, NQ, true, false><<<g, 256, 0, st>>>(P, S, RK, fac, first, c2p)));
      else if (mid)           LAUNCH("update", (k_update<Phys, R, NQ, false, true><<<g, 256, 0, st>>>(P, S, RK, fac, first, c2p)));
      else                    LAUNCH("update", (k_update<Phys, R, NQ, false, false><<<g, 256, 0, st>>>(P, S, RK, fac, first, c2p)));
    }
    if (first) {
      parity ^= 1;
      set_piph(parity);
      LAUNCH("after_first", (k_after_first<<<1, 1, 0, st>>>(P, S.scal, S.planets, planets_id, S.errs)));
    }
    if constexpr (Phys::GR)
      if (mlp_on || rec_on.X)
        LAUNCH("c2p_guess", (k_c2p_guess<Phys, R, NQ><<<blocks(N), 256, 0, st>>>(P, S, mlp, rec_on.X ? 0 : 1,
                                                                                 rec_on)));
    if (ct) {   // flips (first substep), B_faces_to_cells, calc_prim (onestep.c:270-296)
      if (first)
        for (int d = 0; d < 2; ++d)
          if (npair[d]) LAUNCH("ct_flip", (k_ct_flip<R><<<npair[d], 256, flip_smem(d), st>>>(P, S, C, d + 1)));
      LAUNCH("ct_b2c_c2p", (k_ct_b2c_c2p<Phys, R, NQ><<<blocks(N), 256, 0, st>>>(P, S, C)));
    }
    launch_boundary();
    if (first) launch_faces();
  }
  // add_diagnostics (analysis.c:52-108) with the ANALYSIS plugin
  int diag_id = -1, diag_n = 0;
  double* diag_Qrz = nullptr;
  void launch_diag() {
    switch (diag_id) {
      case 0: LAUNCH("diag", (k_diag<R, NQ, 0><<<nring, kDiagBlock, 0, st>>>(P, S, diag_Qrz))); break;
      case 1: LAUNCH("diag", (k_diag<R, NQ, 1><<<nring, kDiagBlock, 0, st>>>(P, S, diag_Qrz))); break;
      case 2: LAUNCH("diag", (k_diag<R, NQ, 2><<<nring, kDiagBlock, 0, st>>>(P, S, diag_Qrz))); break;
      case 3: LAUNCH("diag", (k_diag<R, NQ, 3><<<nring, kDiagBlock, 0, st>>>(P, S, diag_Qrz))); break;
      case 4:
        if constexpr (NQ >= 8)
          LAUNCH("diag", (k_diag<R, NQ, 4><<<nring, kDiagBlock, 0, st>>>(P, S, diag_Qrz)));
        break;
      case 5:
        if constexpr (Phys::GR)
          LAUNCH("diag", (k_diag<R, NQ, 5><<<nring, kDiagBlock, 0, st>>>(P, S, diag_Qrz)));
        break;
      default: break;
    }
  }
  // timestep.c:7-54: Timestep 0 (RK2) or 3 (RK3), then add_diagnostics (:51)
  int rk3 = 0;
  void step_kernels() {
    if (rk3) {
      substep(0.0, 1.0, 1);
      substep(0.75, 0.25, 0, 1);
      substep(1. / 3., 2. / 3., 0);
    } else {
      substep(0.0, 1.0, 1);
      substep(0.5, 0.5, 0);
    }
    launch_diag();
  }
  // Ring diagnostics: Qrz [Nr*Nz][n] and t_avg, as analysis.c keeps them
  // op 0: read (Qrz may be null); op 1: replace with `set` and set_t
  // (restart); op 2: zero (zero_diagnostics, analysis.c:9-27)
  int diag(int op, double* Qrz, long long n, double* t_avg, const double* set, double set_t) override {
    if (!diag_n) return 0;
    const size_t tot = (size_t)nring * diag_n;
    if (op == 1 || op == 2) {
      if (op == 1) {
        if (!set || n != (long long)tot) { disco_set_error("disco_gpu_diag_upload: size mismatch"); return DISCO_E_ARG; }
        CK(cudaMemcpyAsync(diag_Qrz, set, sizeof(double) * tot, cudaMemcpyHostToDevice, st));
      } else {
        set_t = 0.0;
        CK(cudaMemsetAsync(diag_Qrz, 0, sizeof(double) * tot, st));
      }
      CK(cudaMemcpyAsync(&S.scal[SC_TAVG], &set_t, sizeof(double), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
      return diag_n;
    }
    if (Qrz && n >= 0) {
      if (n < (long long)tot) { disco_set_error("disco_gpu_diag_download: buffer too small"); return DISCO_E_ARG; }
      CK(cudaMemcpyAsync(Qrz, diag_Qrz, sizeof(double) * tot, cudaMemcpyDeviceToHost, st));
    }
    if (t_avg) CK(cudaMemcpyAsync(t_avg, &S.scal[SC_TAVG], sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return diag_n;
  }

  int getmindt(double* dt) override {
    P.t_end = 0.0;
    launch_mindt();
    CK(cudaMemcpyAsync(dt, &S.scal[SC_DT], sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    return 0;
  }
  int timestep(double dt) override {
    double slot[1] = {0};
    float dtf = (float)dt;
    memcpy(slot, &dtf, sizeof dtf);
    CK(cudaMemcpyAsync(&S.scal[SC_DT], &dt, sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(&S.scal[SC_DTF], slot, sizeof(double), cudaMemcpyHostToDevice, st));
    step_kernels();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    host_t += dt;
    return 0;
  }
  int build_graph(int par, double t_end) {
    // capture one full step starting from piph parity `par`
    int save = parity;
    parity = par;
    set_piph(par);
    P.t_end = t_end;
    long long before = g_launches.load();
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    launch_mindt();
    step_kernels();
    cudaGraph_t g;
    CK(cudaStreamEndCapture(st, &g));
    graph_nodes = (int)(g_launches.load() - before);
    g_launches -= graph_nodes;  // counted again on each replay
    CK(cudaGraphInstantiate(&graph[par], g, 0));
    cudaGraphDestroy(g);
    parity = save;
    set_piph(save);
    return 0;
  }
  double graph_t_end = -1.0;
  int run(int n, double t_end) override {
    if (graph_t_end != t_end) {
      for (int i = 0; i < 2; ++i) if (graph[i]) { cudaGraphExecDestroy(graph[i]); graph[i] = nullptr; }
      graph_t_end = t_end;
    }
    for (int i = 0; i < 2; ++i)
      if (!graph[i]) { int rc = build_graph(i, t_end); if (rc) return rc; }
    for (int s = 0; s < n; ++s) {
      CK(cudaGraphLaunch(graph[parity], st));
      g_launches += graph_nodes;
      parity ^= 1;
    }
    set_piph(parity);
    P.t_end = 0.0;
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    double sc[SC_COUNT];
    CK(cudaMemcpy(sc, S.scal, sizeof sc, cudaMemcpyDeviceToHost));
    host_t = sc[SC_T];
    return 0;
  }
  int run_timed(int n, double t_end, size_t flush_bytes, double* ms) override {
    if (graph_t_end != t_end) {
      for (int i = 0; i < 2; ++i) if (graph[i]) { cudaGraphExecDestroy(graph[i]); graph[i] = nullptr; }
      graph_t_end = t_end;
    }
    for (int i = 0; i < 2; ++i)
      if (!graph[i]) { int rc = build_graph(i, t_end); if (rc) return rc; }
    if (flush_bytes > flush_size) {
      if (flush_buf) cudaFree(flush_buf);
      flush_buf = nullptr; flush_size = 0;
      CK(cudaMalloc(&flush_buf, flush_bytes));
      flush_size = flush_bytes;
    }
    std::vector<cudaEvent_t> ev(2 * (size_t)n);
    for (auto& e : ev) CK(cudaEventCreate(&e));
    for (int s = 0; s < n; ++s) {
      if (flush_bytes) CK(cudaMemsetAsync(flush_buf, s & 0xff, flush_bytes, st));
      CK(cudaEventRecord(ev[2 * s], st));
      CK(cudaGraphLaunch(graph[parity], st));
      CK(cudaEventRecord(ev[2 * s + 1], st));
      g_launches += graph_nodes;
      parity ^= 1;
    }
    set_piph(parity);
    CK(cudaStreamSynchronize(st));
    double tot = 0;
    for (int s = 0; s < n; ++s) {
      float t;
      CK(cudaEventElapsedTime(&t, ev[2 * s], ev[2 * s + 1]));
      tot += t;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    *ms = tot;
    double sc[SC_COUNT];
    CK(cudaMemcpy(sc, S.scal, sizeof sc, cudaMemcpyDeviceToHost));
    host_t = sc[SC_T];
    return 0;
  }
  int profile(int n, disco_kernel_time* out, int maxo, int* nout) override {
    kt.on = true;
    kt.st = st;
    kt.recs.clear();
    for (int s = 0; s < n; ++s) {
      P.t_end = 0.0;
      launch_mindt();
      step_kernels();
    }
    kt.on = false;
    CK(cudaStreamSynchronize(st));
    std::vector<std::string> names;
    std::vector<long long> cnt;
    std::vector<double> ms;
    for (auto& r : kt.recs) {
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
    kt.recs.clear();
    int k = 0;
    for (size_t i = 0; i < names.size() && k < maxo; ++i, ++k) {
      snprintf(out[k].name, sizeof out[k].name, "%s", names[i].c_str());
      out[k].launches = cnt[i];
      out[k].ms = ms[i];
    }
    *nout = k;
    double sc[SC_COUNT];
    CK(cudaMemcpy(sc, S.scal, sizeof sc, cudaMemcpyDeviceToHost));
    host_t = sc[SC_T];
    return 0;
  }
  int debug_ct(int stage, double* E, double* B, double* Ephi, double* Phi) override {
    if (!ct) { disco_set_error("debug_ct: not a CT instance"); return DISCO_E_STATE; }
    if (C.ev_ok) CK(cudaMemsetAsync(C.ev_ok, 0, sizeof(int), st));
    P.t_end = 0.0;
    launch_mindt();
    const double RK = 0.0, fac = 1.0;
    const int first = 1;
    launch_wcell();
    LAUNCH("plm_phi", (k_plm_phi<R, NQ><<<blocks(N), 256, 0, st>>>(P, S)));
    launch_plm_trans();
    LAUNCH("flux_phi", (k_flux_phi<Phys, R, NQ><<<blocks(N), 256, 0, st>>>(P, S, fac)));
    if (stage >= 1) {
      launch_trans_fluxes(fac);
      LAUNCH("ct_gather", (k_ct_gather<R><<<blocks(N), 256, 0, st>>>(P, S, C)));
    }
    if (stage >= 2) LAUNCH("ct_avg", (k_ct_avg<R><<<blocks(N), 256, 0, st>>>(P, S, C)));
    if (stage >= 3) LAUNCH("ct_bflux", (k_ct_bflux<R><<<blocks(N), 256, 0, st>>>(P, S, C, fac, RK, first)));
    if (stage >= 4 && Nz > 1)
      LAUNCH("ct_edge", (k_ct_edge<R><<<(Nr - 1) * (Nz - 1), 512, edge_smem, st>>>(P, S, C, fac, 0)));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    auto fetch = [&](double* dst, const R* src, size_t n) -> int {
      std::vector<R> t(n);
      CK(cudaMemcpy(t.data(), src, sizeof(R) * n, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n; ++i) dst[i] = (double)t[i];
      return 0;
    };
    int rc2 = 0;
    if (stage == 2) {
      if (E) {
        std::vector<double> t((size_t)4 * N);
        if ((rc2 = fetch(t.data(), C.Efin, (size_t)4 * N))) return rc2;
        const int slot[4] = {0, 1, 4, 5};
        for (int q = 0; q < 4; ++q) memcpy(E + (size_t)slot[q] * N, t.data() + (size_t)q * N, sizeof(double) * N);
      }
    } else {
      if (E && (rc2 = fetch(E, S.Eraw, (size_t)8 * N))) return rc2;
      if (B && (rc2 = fetch(B, S.Braw, (size_t)8 * N))) return rc2;
    }
    if (Ephi && (rc2 = fetch(Ephi, C.Ephi, (size_t)4 * N))) return rc2;
    if (Phi) CK(cudaMemcpy(Phi, C.Phi, sizeof(double) * 5 * N, cudaMemcpyDeviceToHost));
    return 0;
  }
  int planets(disco_planet* out, int max, int* n) override {
    std::vector<DevPlanet> pl(MAX_PL);
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(pl.data(), S.planets, sizeof(DevPlanet) * MAX_PL, cudaMemcpyDeviceToHost));
    *n = P.Npl;
    for (int i = 0; i < P.Npl && i < max && i < MAX_PL; ++i) {
      out[i].r = pl[i].r; out[i].phi = pl[i].phi; out[i].M = pl[i].M; out[i].omega = pl[i].omega;
      out[i].vr = pl[i].vr; out[i].eps = pl[i].eps; out[i].type = pl[i].type;
    }
    return 0;
  }

  // ---- learned starting point of the GRMHD cons2prim ----------------------
  MlpDev mlp{};
  bool mlp_on = false;
  int attach_guess(const MlpDev* m) override {
    if (!Phys::GR) {
      disco_set_error("a cons2prim guess is built for the GRMHD module only");
      return DISCO_E_MODULE;
    }
    mlp_on = m != nullptr;
    if (m) mlp = *m;
    for (int i = 0; i < 2; ++i)   // the step graphs bake the calc_prim launches in
      if (graph[i]) { cudaGraphExecDestroy(graph[i]); graph[i] = nullptr; }
    return 0;
  }
  // steps of (getmindt, timestep) from the reference's start, every
  // cons2prim recording training pairs into rec
  C2PRecord rec_on{};
  int harvest(const MlpDev* m, const C2PRecord* rec, int steps) override {
    if constexpr (Phys::GR) {
      const MlpDev keep = mlp;
      mlp = *m;
      rec_on = *rec;
      int rc = 0;
      for (int s = 0; s < steps && !rc; ++s) {
        double dt;
        rc = getmindt(&dt);
        if (!rc) rc = timestep(dt);
      }
      rec_on = C2PRecord{};
      mlp = keep;
      return rc;
    } else {
      (void)m; (void)rec; (void)steps;
      disco_set_error("harvest: cons2prim pairs come from the GRMHD module only");
      return DISCO_E_MODULE;
    }
  }
  // out = {calls, summed k_converge, summed iterations, calls started from the guess}
  int c2p_stats(long long* out, int reset) override {
    DevErrs h;
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(&h, S.errs, sizeof h, cudaMemcpyDeviceToHost));
    out[0] = (long long)h.c2p_calls; out[1] = (long long)h.c2p_kconv;
    out[2] = (long long)h.c2p_iters; out[3] = (long long)h.c2p_guessed;
    if (reset) {
      h.c2p_calls = h.c2p_kconv = h.c2p_iters = h.c2p_guessed = 0;
      CK(cudaMemcpy(S.errs, &h, sizeof h, cudaMemcpyHostToDevice));
    }
    return 0;
  }

  // Face tables of one dimension as the device holds them (test access).
  int debug_faces(int dim, int* npair_out, long* nface_out, int* fIndex, int* L, int* Rr,
                  int* LRtype, double* phic, double* dA) override {
    if (dim != 1 && dim != 2) { disco_set_error("debug_faces: dim must be 1 or 2"); return DISCO_E_ARG; }
    const int d = dim - 1;
    CK(cudaStreamSynchronize(st));
    if (npair_out) *npair_out = npair[d];
    if (nface_out) *nface_out = npair[d] ? S.nf[d] : 0;
    if (!npair[d]) return 0;
    const size_t nf = (size_t)S.nf[d];
    if (fIndex) CK(cudaMemcpy(fIndex, S.face_off[d], sizeof(int) * (npair[d] + 1), cudaMemcpyDeviceToHost));
    if (L) CK(cudaMemcpy(L, S.fL[d], sizeof(int) * nf, cudaMemcpyDeviceToHost));
    if (Rr) CK(cudaMemcpy(Rr, S.fR[d], sizeof(int) * nf, cudaMemcpyDeviceToHost));
    if (LRtype) {
      std::vector<signed char> t(nf);
      CK(cudaMemcpy(t.data(), S.fLR[d], nf, cudaMemcpyDeviceToHost));
      for (size_t f = 0; f < nf; ++f) LRtype[f] = t[f];
    }
    if (phic) CK(cudaMemcpy(phic, S.fphic[d], sizeof(double) * nf, cudaMemcpyDeviceToHost));
    if (dA) {
      std::vector<R> t(nf);
      CK(cudaMemcpy(t.data(), S.fdA[d], sizeof(R) * nf, cudaMemcpyDeviceToHost));
      for (size_t f = 0; f < nf; ++f) dA[f] = (double)t[f];
    }
    return 0;
  }
  // plm_phi and plm_trans (onestep.c:104-130) on the current state, then the
  // gradients widened to FP64 (test access; the state is not changed).
  int debug_grad(double* gp, double* gr, double* gz) override {
    LAUNCH("plm_phi", (k_plm_phi<R, NQ><<<blocks(N), 256, 0, st>>>(P, S)));
    launch_plm_trans();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    const size_t n = (size_t)NQ * N;
    std::vector<R> t(n);
    const R* src[3] = {S.gradp, S.gradr, S.gradz};
    double* dst[3] = {gp, gr, gz};
    for (int a = 0; a < 3; ++a) {
      if (!dst[a]) continue;
      CK(cudaMemcpy(t.data(), src[a], sizeof(R) * n, cudaMemcpyDeviceToHost));
      for (size_t x = 0; x < n; ++x) dst[a][x] = (double)t[x];
    }
    return 0;
  }
  // Per-cell divergence of the face fluxes of B (constrained transport only).
  int divb(double* div, double* scale) override {
    if (!ct) { disco_set_error("divb: the instance does not evolve face fluxes (no constrained transport)"); return DISCO_E_STATE; }
    double *d_div = nullptr, *d_sc = nullptr;
    if (cudaMalloc(&d_div, sizeof(double) * N) != cudaSuccess ||
        cudaMalloc(&d_sc, sizeof(double) * N) != cudaSuccess) {
      if (d_div) cudaFree(d_div);
      disco_set_error("divb: no device memory for the per-cell result");
      return DISCO_E_NOMEM;
    }
    k_divb<R><<<blocks(N), 256, 0, st>>>(P, S, C, d_div, d_sc);
    ++g_launches;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && div) e = cudaMemcpyAsync(div, d_div, sizeof(double) * N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && scale) e = cudaMemcpyAsync(scale, d_sc, sizeof(double) * N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_div);
    cudaFree(d_sc);
    CK(e);
    return 0;
  }
  // grid of the primitive conversion kernels: a few waves over the SMs
  unsigned prim_grid() const {
    long want = ((long)NQ * N + 255) / 256;
    return (unsigned)std::min<long>(std::max<long>(want, 1), 152L * 16);
  }
  int download(disco_state_view* v) override {
    CK(cudaStreamSynchronize(st));
    if (v->piph) CK(cudaMemcpy(v->piph, S.piph, sizeof(double) * N, cudaMemcpyDeviceToHost));
    if (v->dphi) CK(cudaMemcpy(v->dphi, S.dphi, sizeof(double) * N, cudaMemcpyDeviceToHost));
    if (v->wiph) CK(cudaMemcpy(v->wiph, S.wiph, sizeof(double) * N, cudaMemcpyDeviceToHost));
    if (v->cons) CK(cudaMemcpy(v->cons, S.cons, sizeof(double) * NQ * N, cudaMemcpyDeviceToHost));
    if (v->Phi && ct) CK(cudaMemcpy(v->Phi, C.Phi, sizeof(double) * 5 * N, cudaMemcpyDeviceToHost));
    if (v->prim) {
      if (sizeof(R) == sizeof(double)) {
        CK(cudaMemcpy(v->prim, S.prim, sizeof(double) * NQ * N, cudaMemcpyDeviceToHost));
      } else {   // widened (and back to the lab frame) on the device, then one copy
        double* stage = staging();
        if (!stage) {
          disco_set_error("download: no device memory for the FP64 staging copy");
          return DISCO_E_NOMEM;
        }
        k_prim_out<R, NQ><<<prim_grid(), 256, 0, st>>>(S, stage);
        CK(cudaMemcpyAsync(v->prim, stage, sizeof(double) * NQ * N, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
      }
    }
    double sc[SC_COUNT];
    CK(cudaMemcpy(sc, S.scal, sizeof sc, cudaMemcpyDeviceToHost));
    v->t = sc[SC_T];
    return 0;
  }
  int upload(const disco_state_view* v) override {
    CK(cudaStreamSynchronize(st));
    if (v->piph) CK(cudaMemcpy((void*)S.piph, v->piph, sizeof(double) * N, cudaMemcpyHostToDevice));
    if (v->dphi) CK(cudaMemcpy(S.dphi, v->dphi, sizeof(double) * N, cudaMemcpyHostToDevice));
    if (v->wiph) CK(cudaMemcpy(S.wiph, v->wiph, sizeof(double) * N, cudaMemcpyHostToDevice));
    if (v->cons) CK(cudaMemcpy(S.cons, v->cons, sizeof(double) * NQ * N, cudaMemcpyHostToDevice));
    if (v->Phi && ct) CK(cudaMemcpy(C.Phi, v->Phi, sizeof(double) * 5 * N, cudaMemcpyHostToDevice));
    if (v->prim) {
      if (sizeof(R) == sizeof(double)) {
        CK(cudaMemcpy(S.prim, v->prim, sizeof(double) * NQ * N, cudaMemcpyHostToDevice));
      } else {   // one copy of the FP64 view, converted (into the ring frame) on the device
        double* stage = staging();
        if (!stage) {
          disco_set_error("upload: no device memory for the FP64 staging copy");
          return DISCO_E_NOMEM;
        }
        CK(cudaMemcpyAsync(stage, v->prim, sizeof(double) * NQ * N, cudaMemcpyHostToDevice, st));
        k_prim_in<R, NQ><<<prim_grid(), 256, 0, st>>>(S, stage);
        CK(cudaStreamSynchronize(st));
      }
    }
    if (v->dphi) sync_dphi_r();
    if (ct && C.ev_ok) CK(cudaMemsetAsync(C.ev_ok, 0, sizeof(int), st));   // positions changed
    if (v->piph || v->dphi) launch_faces();
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    return 0;
  }
  int status(disco_gpu_errs* e) override {
    DevErrs h;
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(&h, S.errs, sizeof h, cudaMemcpyDeviceToHost));
    e->nan_cells = (long long)h.nan_cells;
    e->rho_floor_hits = (long long)h.rho_floor_hits;
    e->p_floor_hits = (long long)h.p_floor_hits;
    e->face_errors = (long long)h.face_errors;
    e->steps = (long long)h.steps;
    e->c2p_no_converge = (long long)h.c2p_no_converge;
    e->async_timeouts = (long long)h.async_timeouts;
    if (ct) {
      unsigned long long ce = 0;
      CK(cudaMemcpy(&ce, C.errs, 8, cudaMemcpyDeviceToHost));
      e->face_errors += (long long)ce;
    }
    return 0;
  }
  double time() override { return host_t; }

  void launch_step(int par) override {
    int save = parity;
    parity = par;
    set_piph(par);
    P.t_end = 0.0;
    launch_mindt();
    step_kernels();
    parity = save;
    set_piph(save);
  }
  int cur_parity() const override { return parity; }
  bool sink_on = false;
  // the sink bodies' accumulators (report.c:81-100): out[b * kSinkAcc + q]
  // for the first min(bodies, max_bodies) bodies; reset zeroes them and
  // their RK copy, as report() does after printing
  int sink_accum(double* out, int max_bodies, int reset) override {
    if (!sink_on) return 0;
    const int nb = std::min(P.sink_bodies, max_bodies);
    CK(cudaStreamSynchronize(st));
    if (out && nb > 0) CK(cudaMemcpy(out, S.sink_acc, sizeof(double) * nb * kSinkAcc, cudaMemcpyDeviceToHost));
    if (reset) CK(cudaMemset(S.sink_acc, 0, sizeof(double) * 2 * MAX_PL * kSinkAcc));
    return nb;
  }
  MultiPlanBase* new_multi_plan() override;
  cudaStream_t stream() const override { return st; }
  int after_external_steps(int nsteps, long long nodes) override {
    g_launches += nodes;
    parity ^= (nsteps & 1);
    set_piph(parity);
    double sc[SC_COUNT];
    CK(cudaMemcpyAsync(sc, S.scal, sizeof sc, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    host_t = sc[SC_T];
    return 0;
  }

  // report.c as a device reduction: out = {t, q, Mass, Torque, Torque2,
  // Torque1_cut[0], Torque2_cut[0], ..., Torque1_cut[4], Torque2_cut[4]}
  double report_q = 0.0, report_soft = 0.0;
  double* report_part = nullptr;
  int report(double* out, int nout) override {
    const int nb = (int)blocks(N, kReportBlock);
    if (!report_part) {
      int rc = dalloc(&report_part, (size_t)nb * kReportSums + kReportSums, keep);
      if (rc) return rc;
    }
    k_report_blocks<R, NQ><<<nb, kReportBlock, 0, st>>>(P, S, report_soft, report_part);
    k_report_final<<<1, 32, 0, st>>>(report_part, nb, report_part + (size_t)nb * kReportSums);
    g_launches += 2;
    CK(cudaGetLastError());
    double sums[kReportSums], sc[SC_COUNT];
    CK(cudaMemcpyAsync(sums, report_part + (size_t)nb * kReportSums, sizeof sums, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(sc, S.scal, sizeof sc, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double all[2 + kReportSums];
    all[0] = sc[SC_T];
    all[1] = report_q;
    all[2] = sums[0]; all[3] = sums[1]; all[4] = sums[2];
    for (int n = 0; n < 5; ++n) { all[5 + 2 * n] = sums[3 + n]; all[6 + 2 * n] = sums[8 + n]; }
    const int m = std::min(nout, 2 + kReportSums);
    for (int i = 0; i < m; ++i) out[i] = all[i];
    return m;
  }
  // CFL dt with partial minima in the library's static scratch array: no
  // device allocation, no write to the instance (disco_gpu_noalloc.h).  The
  // work runs on the instance's device (the one current at create); the
  // caller's current device is switched to it for the call and restored.
  int getmindt_noalloc(double* dt) override {
    long nb = blocks(N, kNoallocBlock);
    if (N > DISCO_NOALLOC_MAX_CELLS || nb > kNoallocMaxBlocks) {
      disco_set_error("getmindt_noalloc: instance larger than the static scratch (DISCO_NOALLOC_MAX_CELLS)");
      return DISCO_E_ARG;
    }
    int cur = 0;
    CK(cudaGetDevice(&cur));
    if (cur != device) CK(cudaSetDevice(device));
    int rc = getmindt_noalloc_on_device(dt);
    if (cur != device) {
      cudaError_t e = cudaSetDevice(cur);
      if (!rc && e != cudaSuccess) CK(e);
    }
    return rc;
  }
  int getmindt_noalloc_on_device(double* dt) {
    long nb = blocks(N, kNoallocBlock);
    unsigned long long* part = noalloc_scratch(device);
    if (!part) { disco_set_error("getmindt_noalloc: scratch symbol not available"); return DISCO_E_CUDA; }
    DevParams Pn = P;
    Pn.t_end = 0.0;
    k_mindt_blocks<Phys, R, NQ><<<(int)nb, kNoallocBlock, 0, st>>>(Pn, S, part);
    k_mindt_final<<<1, 1024, 0, st>>>(Pn, part, (int)nb);
    g_launches += 2;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dt, part + kNoallocMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
  }
};

}  // namespace disco_impl

#include "multi_plan.cuh"

namespace disco_impl {

template <class Phys, typename R, int NQ>
InstanceBase* make_instance(const disco_host_domain* dom, int* rc) {
  auto* x = new Instance<Phys, R, NQ>();
  *rc = x->create(dom);
  if (*rc) { delete x; return nullptr; }
  return x;
}

}  // namespace disco_impl
