// Host side of the multi-instance step (multi.cuh): a group of instances of
// one hydro module and precision whose steps launch the same kernel
// sequence.  prepare() builds, on the device, two member tables (one per
// piph parity) and the work lists of every stage -- for each member the
// blocks it launches on its own, as (member, block x, block y) items --
// and launch_step() issues the step as one launch per stage, in the order
// Instance::launch_step issues the members' own kernels.
//
// The group takes the sequence of an instance without constrained
// transport, boundary plugins, the staged phi sweep, a learned cons2prim
// start, sinks, the nozzle or periodic ghosts; such instances stay outside (a batch gives them their own graph
// branch).  Included by instance.cuh after the Instance template.
#pragma once
#include "multi.cuh"

namespace disco_impl {

template <class Phys, typename R, int NQ>
struct MultiPlan : MultiPlanBase {
  using Inst = Instance<Phys, R, NQ>;
  struct List {
    long off = 0;
    int n = 0;
  };
  std::vector<Inst*> m;
  MultiMember<R>* tab[2] = {nullptr, nullptr};   // device: members at piph parity 0 / 1
  MultiTile* tiles = nullptr;                     // device: every work list
  List cells, rings, anchor, bnd, faces[2], slopes[2], trans[2], flux[2];
  size_t smem_faces[2] = {0, 0}, smem_avg = 0;
  int nsm = 0;

  explicit MultiPlan(Inst* first) { m.push_back(first); }
  ~MultiPlan() override {
    for (auto& t : tab)
      if (t) cudaFree(t);
    if (tiles) cudaFree(tiles);
  }

  static bool covered(const Inst* x) {
    return !x->ct && x->n_bc_ops == 0 && !x->sweep && !x->mlp_on && !x->rec_on.X && !x->sink_on &&
           x->P.nozzle_type == 0 && !x->n_pcopy[0] && !x->n_pcopy[1];
  }
  bool accepts(InstanceBase* b) const override {
    auto* x = dynamic_cast<Inst*>(b);
    if (!x || !covered(x)) return false;
    const Inst* a = m[0];
    return x->device == a->device && x->rk3 == a->rk3 && x->P.cool_damp == a->P.cool_damp &&
           (x->P.mesh_motion == 3) == (a->P.mesh_motion == 3) && x->diag_id == a->diag_id;
  }
  void add(InstanceBase* b) override { m.push_back(static_cast<Inst*>(b)); }
  int size() const override { return (int)m.size(); }

  int prepare() override {
    const int n = (int)m.size();
    std::vector<MultiMember<R>> h[2];
    std::vector<MultiTile> all;
    auto put = [&](List& l, auto&& fill) {
      l.off = (long)all.size();
      for (int i = 0; i < n; ++i) fill(i, m[i]);
      l.n = (int)((long)all.size() - l.off);
    };
    auto grid = [&](int i, long nx, long ny) {
      for (long y = 0; y < ny; ++y)
        for (long x = 0; x < nx; ++x) all.push_back(MultiTile{i, (int)x, (int)y, 0});
    };
    // the (x, y) tiles of a face kernel whose y blocks cover the faces of
    // pair(x) by `per` faces each: only those that hold a face (the
    // member's own grid also has blocks past a short pair's last face,
    // which return at once)
    auto face_tiles = [&](int i, const Inst* x, int d, long nx, auto&& pair_of, int per) {
      const std::vector<int>& fo = x->face_off_h[d];
      for (long bx = 0; bx < nx; ++bx) {
        const int pr = pair_of(bx);
        const int nf = fo[pr + 1] - fo[pr];
        for (int by = 0; by * per < nf; ++by) all.push_back(MultiTile{i, (int)bx, by, 0});
      }
    };
    for (int par = 0; par < 2; ++par)
      for (int i = 0; i < n; ++i) {
        const Inst* x = m[i];
        MultiMember<R> mm;
        memset(&mm, 0, sizeof mm);
        mm.P = x->P;
        mm.P.t_end = 0.0;
        mm.S = x->S;
        mm.S.piph = x->piph_buf[par];
        mm.S.piph_out = x->piph_buf[par ^ 1];
        for (int d = 0; d < 2; ++d) {
          int kc = 0;
          if (!x->trans_range(d, &mm.fr[d][0], &mm.fr[d][1], &mm.fr[d][2], &kc)) mm.fr[d][1] = 0;
        }
        mm.planets_id = x->planets_id;
        mm.qrz = x->diag_Qrz;
        h[par].push_back(mm);
      }
    put(cells, [&](int i, const Inst* x) { grid(i, x->blocks(x->N), 1); });
    put(rings, [&](int i, const Inst* x) { grid(i, x->nring, 1); });
    put(anchor, [&](int i, const Inst* x) {
      if (x->npair[0] || x->npair[1]) grid(i, x->blocks((long)x->nring * 32), 1);
    });
    put(bnd, [&](int i, const Inst* x) { grid(i, x->S.nghost, 1); });
    for (int d = 0; d < 2; ++d) {
      put(faces[d], [&](int i, const Inst* x) { grid(i, x->npair[d], 1); });
      put(slopes[d], [&](int i, const Inst* x) {
        if (x->npair[d]) face_tiles(i, x, d, x->npair[d], [](long bx) { return (int)bx; }, 256 * kSlopeFaces);
      });
      put(trans[d], [&](int i, const Inst* x) {
        if (x->npair[d]) grid(i, x->S.nchunk, plm_groups<NQ>());
      });
      put(flux[d], [&](int i, const Inst* x) {
        int jmin, jc, kmin, kc;
        if (!x->trans_range(d, &jmin, &jc, &kmin, &kc)) return;
        const int Nr = x->Nr;
        face_tiles(i, x, d, (long)jc * kc, [&](long bx) {   // the pair of k_flux_trans_body
          const int pj = jmin + (int)(bx % jc), pk = kmin + (int)(bx / jc);
          return d == 0 ? pj + (Nr - 1) * pk : pj + Nr * pk;
        }, 256);
      });
      smem_faces[d] = 0;
      for (const Inst* x : m)
        if (x->npair[d]) smem_faces[d] = std::max(smem_faces[d], (size_t)x->maxNf[d] * 13 + 64);
    }
    smem_avg = 0;
    for (const Inst* x : m) smem_avg = std::max(smem_avg, (size_t)(x->maxring + 1) * sizeof(double));
    CK(cudaSetDevice(m[0]->device));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, m[0]->device));
    for (int par = 0; par < 2; ++par) {
      if (tab[par]) cudaFree(tab[par]);
      tab[par] = nullptr;
      CK(cudaMalloc(&tab[par], sizeof(MultiMember<R>) * n));
      CK(cudaMemcpy(tab[par], h[par].data(), sizeof(MultiMember<R>) * n, cudaMemcpyHostToDevice));
    }
    if (tiles) cudaFree(tiles);
    tiles = nullptr;
    CK(cudaMalloc(&tiles, sizeof(MultiTile) * std::max<size_t>(all.size(), 1)));
    CK(cudaMemcpy(tiles, all.data(), sizeof(MultiTile) * all.size(), cudaMemcpyHostToDevice));
    const size_t fmax = std::max(smem_faces[0], smem_faces[1]);
    if (fmax > 48 * 1024) CK(raise_smem_limit(km_faces<R>, fmax));
    if (smem_avg > 48 * 1024) CK(raise_smem_limit(km_wcell_avg<R>, smem_avg));
    occ.clear();
    query = true;   // the dry pass: resident blocks of every stage kernel
    launch_step(0, nullptr, 1, nullptr);
    launch_step(1, nullptr, 1, nullptr);
    query = false;
    return 0;
  }

  // resident blocks per SM of each stage kernel at its block size and
  // dynamic shared memory, queried once by a dry pass of launch_step in
  // prepare (never during a stream capture)
  std::vector<std::pair<const void*, int>> occ;
  bool query = false;
  int occupancy(const void* fn, int threads, size_t smem) {
    for (auto& o : occ)
      if (o.first == fn) return o.second;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess) nb = 1;
    nb = std::max(nb, 1);
    occ.push_back({fn, nb});
    return nb;
  }

  int launch_step(int par, cudaStream_t st, int ctas_per_sm, KTimer* kt) override {
    const int n = (int)m.size();
    const MultiMember<R>* A = tab[par];       // before the first substep's update
    const MultiMember<R>* B = tab[par ^ 1];   // after it
    long long nl = 0;
    // one stage: a grid of min(items, min(ctas_per_sm, resident) x SMs)
    // blocks over the list
#define DISCO_ML(NAME, LIST, THREADS, SMEM, KERNEL, ...)                                                  \
  do {                                                                                                   \
    if ((LIST).n > 0) {                                                                                  \
      auto kfn_ = KERNEL;                                                                                \
      const int occ_ = occupancy((const void*)kfn_, (THREADS), (SMEM));                                  \
      if (!query) {                                                                                      \
        const long cap_ = (long)std::min(std::max(ctas_per_sm, 1), occ_) * nsm;                          \
        if (kt) kt->begin();                                                                             \
        kfn_<<<(unsigned)std::min<long>((LIST).n, cap_), (THREADS), (SMEM), st>>>(__VA_ARGS__);         \
        if (kt) kt->end(NAME);                                                                           \
        ++nl;                                                                                            \
      }                                                                                                  \
    }                                                                                                    \
  } while (0)
#define DISCO_MLA(NAME, LIST, THREADS, SMEM, KERNEL, T, a0, a1, i0, i1) \
  DISCO_ML(NAME, LIST, THREADS, SMEM, KERNEL, T, tiles + (LIST).off, (LIST).n, a0, a1, i0, i1)
#define DISCO_M1(NAME, KERNEL, T)                            \
  do {                                                       \
    if (!query) {                                            \
      if (kt) kt->begin();                                   \
      KERNEL<<<(unsigned)((n + 63) / 64), 64, 0, st>>>(T, n); \
      if (kt) kt->end(NAME);                                 \
      ++nl;                                                  \
    }                                                        \
  } while (0)
    DISCO_MLA("mindt", cells, 256, 0, (km_mindt<Phys, R, NQ>), A, 0.0, 0.0, 0, 0);
    DISCO_M1("dt_finalize", km_dt_finalize<R>, A);
    auto substep = [&](double RK, double fac, int first, int mid) {
      const MultiMember<R>* T = first ? A : B;
      if (first) {
        if (kMix<R> && m[0]->P.mesh_motion == 3) {
          DISCO_MLA("wcell_ring", rings, 256, 0, km_wcell_ring<R>, T, 0.0, 0.0, 0, 0);
        } else {
          DISCO_MLA("wcell", cells, 256, 0, (km_wcell<R, NQ>), T, 0.0, 0.0, 0, 0);
          if (m[0]->P.mesh_motion == 3)
            DISCO_MLA("wcell_avg", rings, 64, smem_avg, km_wcell_avg<R>, T, 0.0, 0.0, 0, 0);
        }
      }
      DISCO_MLA("plm_phi", cells, 256, 0, (km_plm_phi<R, NQ>), T, 0.0, 0.0, 0, 0);
      for (int d = 0; d < 2; ++d) {
        DISCO_MLA(d ? "plm_slopes_z" : "plm_slopes_r", slopes[d], 256, 0, (km_plm_slopes<R, NQ>), T, 0.0, 0.0, d + 1, 0);
        DISCO_MLA(d ? "plm_trans_z" : "plm_trans_r", trans[d], kTileCells, 0, (km_plm_trans<R, NQ>), T, 0.0, 0.0, d + 1, 0);
      }
      DISCO_MLA("flux_phi", cells, 256, 0, (km_flux_phi<Phys, R, NQ>), T, fac, 0.0, 0, 0);
      for (int d = 0; d < 2; ++d)
        DISCO_MLA(d ? "flux_z" : "flux_r", flux[d], 256, 0, (km_flux_trans<Phys, R, NQ>), T, fac, 0.0, d + 1, 0);
      const bool cd = m[0]->P.cool_damp;
      const MultiTile* tc = tiles + cells.off;
      if (cd && mid) DISCO_ML("update", cells, 256, 0, (km_update<Phys, R, NQ, true, true>), T, tc, cells.n, RK, fac, first, 1);
      else if (cd)   DISCO_ML("update", cells, 256, 0, (km_update<Phys, R, NQ, true, false>), T, tc, cells.n, RK, fac, first, 1);
      else if (mid)  DISCO_ML("update", cells, 256, 0, (km_update<Phys, R, NQ, false, true>), T, tc, cells.n, RK, fac, first, 1);
      else           DISCO_ML("update", cells, 256, 0, (km_update<Phys, R, NQ, false, false>), T, tc, cells.n, RK, fac, first, 1);
      if (first) {
        DISCO_M1("after_first", km_after_first<R>, A);
        T = B;
      }
      DISCO_MLA("boundary", bnd, kTileCells, 0, (km_boundary<R, NQ>), T, 0.0, 0.0, 0, 0);
      if (first) {
        DISCO_MLA("anchor", anchor, 256, 0, km_anchor<R>, T, 0.0, 0.0, 0, 0);
        for (int d = 0; d < 2; ++d)
          DISCO_MLA(d ? "faces_z" : "faces_r", faces[d], 256, smem_faces[d], km_faces<R>, T, 0.0, 0.0, d + 1, 0);
      }
    };
    if (m[0]->rk3) {
      substep(0.0, 1.0, 1, 0);
      substep(0.75, 0.25, 0, 1);
      substep(1. / 3., 2. / 3., 0, 0);
    } else {
      substep(0.0, 1.0, 1, 0);
      substep(0.5, 0.5, 0, 0);
    }
    const MultiTile* tr = tiles + rings.off;
    switch (m[0]->diag_id) {   // add_diagnostics (analysis.c:52-108)
      case 0: DISCO_ML("diag", rings, kDiagBlock, 0, (km_diag<R, NQ, 0>), B, tr, rings.n); break;
      case 1: DISCO_ML("diag", rings, kDiagBlock, 0, (km_diag<R, NQ, 1>), B, tr, rings.n); break;
      case 2: DISCO_ML("diag", rings, kDiagBlock, 0, (km_diag<R, NQ, 2>), B, tr, rings.n); break;
      case 3: DISCO_ML("diag", rings, kDiagBlock, 0, (km_diag<R, NQ, 3>), B, tr, rings.n); break;
      case 4:
        if constexpr (NQ >= 8) DISCO_ML("diag", rings, kDiagBlock, 0, (km_diag<R, NQ, 4>), B, tr, rings.n);
        break;
      case 5:
        if constexpr (Phys::GR) DISCO_ML("diag", rings, kDiagBlock, 0, (km_diag<R, NQ, 5>), B, tr, rings.n);
        break;
      default: break;
    }
#undef DISCO_M1
#undef DISCO_MLA
#undef DISCO_ML
    g_launches += nl;
    CK(cudaGetLastError());
    return 0;
  }
};

template <class Phys, typename R, int NQ>
MultiPlanBase* Instance<Phys, R, NQ>::new_multi_plan() {
  return MultiPlan<Phys, R, NQ>::covered(this) ? new MultiPlan<Phys, R, NQ>(this) : nullptr;
}

}  // namespace disco_impl
