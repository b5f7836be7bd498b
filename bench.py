#!/usr/bin/env python
"""Benchmark of the GB300 RK substep cycle: zone-updates/s on one GB300.

A "step" is one full RK2 timestep (timestep.c:7 -> two onestep() substeps)
of every interior cell, preceded by the CFL reduction (getmindt).  The metric
is zone-updates/s = interior cells x steps / seconds.  The chosen path is the
mixed-precision one (FP32 reconstruction, Riemann fluxes and sources; FP64
positions, face geometry, conserved accumulation, dt); the plain FP64 path is
measured beside it, with the relative L1 error of the chosen path against it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host CPU (the C
restatement in oracle/, pinned bit-for-bit to the reference build).
Under torchrun (N>1) every rank advances an independent replica (the domain
is not decomposed across GPUs); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "mhd_disk3d": {"dir": "configs/cfg2_mhd_disk",
                   "desc": "3D Newtonian MHD Keplerian disk, Nr=256 x Nz=64 on r in [1,4], "
                           "z in [-0.5,0.5], HLLD + constrained transport, PLM 1.5, RK2, "
                           "isothermal c_s=0.05 v_K, beta=400 vertical field",
                   # bounded CPU samples: same physics at reduced resolution
                   "cpu_sample": {"Num_R": 64, "Num_Z": 16},
                   "ref_sample": {"Num_R": 32, "Num_Z": 8},
                   # reference arm: tiles of 64 rings x 2 layers of the full
                   # grid (Nr, Nz, r range, z range), one per host core
                   "ref_tiles": {"grid": (256, 64, 1.0, 4.0, -0.5, 0.5), "tile": (64, 2)},
                   "cells_full": 22004544},
    # the circumbinary MHD disk at full size: 134 M cells (about 136 GB on the
    # mixed path, 228 GB on the FP64 path, measured one after the other)
    "cbd_large": {"dir": "configs/cfg5_cbd_mhd",
                  "desc": "3D circumbinary MHD disk, Nr=512 x Nz=128 on r in [0.8,8], z in [-1,1], "
                          "equal-mass binary at a = 1 (Planets/cm.c), Sigma ~ 1/r with a cavity "
                          "inside r = 2, h/r = 0.1, toroidal field at beta = 100, HLLD + CT, RK2",
                  "cpu_sample": {"Num_R": 64, "Num_Z": 16},
                  "ref_sample": {"Num_R": 32, "Num_Z": 8}},
    # the same disk at 64 x 16 rings (1.4 M cells, 0.4 GB of state, still
    # larger than L2): the small case for full ncu captures
    "mhd_disk3d_small": {"dir": "configs/cfg2_mhd_disk",
                         "desc": "3D Newtonian MHD Keplerian disk at Nr=64 x Nz=16 (profiling case)",
                         "overrides": {"Num_R": 64, "Num_Z": 16},
                         "cpu_sample": {"Num_R": 32, "Num_Z": 8},
                         "ref_sample": {"Num_R": 32, "Num_Z": 8}},
    # the same disk at 128 x 32 rings (about 1.9 M cells, 0.8 GB of state,
    # well above L2): the case for DRAM-traffic captures of single kernels
    "mhd_disk3d_medium": {"dir": "configs/cfg2_mhd_disk",
                          "desc": "3D Newtonian MHD Keplerian disk at Nr=128 x Nz=32 (profiling case)",
                          "overrides": {"Num_R": 128, "Num_Z": 32},
                          "cpu_sample": {"Num_R": 32, "Num_Z": 8},
                          "ref_sample": {"Num_R": 32, "Num_Z": 8}},
    # GRMHD Fishbone-Moncrief torus around a Kerr black hole (a = 0.9):
    # 192 x 96 rings on r in [2, 40], z in [-20, 20], Np capped at 1024,
    # 11.9 M cells, FP64
    "grmhd_torus": {"dir": "configs/cfg4_grmhd_torus",
                    "desc": "3D GRMHD Fishbone-Moncrief torus (r_in 6, r_pk 12, gamma 4/3, loop field at "
                            "beta 100, 4% pressure noise) around a Kerr black hole a=0.9 in Kerr-Schild "
                            "cylindrical coordinates, Nr=192 on r in [2,40], Nz=96 on z in [-20,20], "
                            "Np capped at 1024, HLL, cell-centred B, Noble 2D cons2prim, PLM 1.5, RK2, FP64",
                    "precisions": (0,),
                    "cpu_sample": None, "ref_sample": None},
    # 64 independent planet-disk runs in one graph launch per step: Nr drawn
    # from U{64..512} and the planet mass ratio log-uniform in [1e-5, 1e-3]
    # by splitmix64 seeded 0..63
    "planet_batch": {"dir": "configs/cfg3_planet_disk",
                     "desc": "64 independent 2D locally isothermal disk + planet runs (alpha 1e-3, "
                             "h/r 0.05, r in [0.4,2.5], Nr ~ U{64..512}, q ~ logU[1e-5,1e-3]), "
                             "one CUDA graph per step",
                     "batch": 64,
                     "cpu_sample": {"Num_R": 128},
                     "ref_sample": {"Num_R": 64}},
    # the same disks at survey resolution: 256 members with Nr ~ U{16..64}
    # (a few thousand cells each), where a member's own step is bound by
    # its launches rather than its cells
    "planet_batch_small": {"dir": "configs/cfg3_planet_disk",
                           "desc": "256 independent 2D locally isothermal disk + planet runs (alpha 1e-3, "
                                   "h/r 0.05, r in [0.4,2.5], Nr ~ U{16..64}, q ~ logU[1e-5,1e-3]), "
                                   "one CUDA graph per step",
                           "batch": 256, "nr_range": (16, 64),
                           "cpu_sample": {"Num_R": 32},
                           "ref_sample": {"Num_R": 32}},
    # GRMHD (FP64 only): thin disk around a Schwarzschild black hole in
    # Kerr-Schild cylindrical coordinates, about 4.9 M cells
    "grmhd_disk": {"dir": "configs/cfg4_grmhd_disk",
                   "desc": "3D GRMHD thin disk around a Schwarzschild black hole (Kerr-Schild "
                           "cylindrical metric, M = 1), Nr=128 x Nz=32 on r in [6,12], z in [-1,1], "
                           "HLL, cell-centred B, Noble 2D cons2prim, PLM 1.5, RK2, FP64",
                   "overrides": {"Num_R": 128, "Num_Z": 32},
                   "precisions": (0,),
                   "cpu_sample": None, "ref_sample": None},
    "vortex2d": {"dir": "configs/cfg1_vortex",
                 "desc": "2D cylindrical Newtonian hydro, Gaussian isentropic vortex, "
                         "Nr=128 on r in [0.5,3], HLLC, PLM 1.5, RK2, CFL 0.5",
                 "cpu_sample": {}, "ref_sample": {}},
}
DEFAULT_WORKLOAD = "mhd_disk3d"
L2_BYTES = 126 * 1024 * 1024


# profile entry (one per launch site) -> kernel function
KERNEL_FUNCTION = {"flux_r": "flux_trans", "flux_z": "flux_trans",
                   "plm_slopes_r": "plm_slopes", "plm_slopes_z": "plm_slopes",
                   "plm_trans_r": "plm_trans", "plm_trans_z": "plm_trans",
                   "faces_r": "faces", "faces_z": "faces", "dt_finalize": "mindt"}
# kernel function -> its symbol in disco_gb300/csrc/cuda
KERNEL_SYMBOL = {"flux_trans": "k_flux_trans", "plm_slopes": "k_plm_slopes", "plm_trans": "k_plm_trans",
                 "faces": "k_faces", "update": "k_update", "flux_phi": "k_flux_phi", "plm_phi": "k_plm_phi",
                 "ct_gather": "k_ct_gather", "ct_avg": "k_ct_avg", "ct_bflux": "k_ct_bflux",
                 "ct_edge": "k_ct_edge", "ct_edge_replay": "k_ct_edge_replay", "ct_flip": "k_ct_flip",
                 "ct_b2c_c2p": "k_ct_b2c_c2p", "mindt": "k_mindt", "diag": "k_diag",
                 "boundary": "k_boundary", "anchor": "k_anchor", "wcell": "k_wcell",
                 "wcell_ring": "k_wcell_ring", "wcell_avg": "k_wcell_avg", "after_first": "k_after_first",
                 "ct_edge_flag": "k_set_flag", "phi_sweep": "k_phi_sweep", "sink_acc": "k_sink_acc",
                 "sink_final": "k_sink_final", "c2p_guess": "k_c2p_guess"}


def _traffic(func: str, alg_bytes: float, workload: str):
    """DRAM bytes per launch of kernel function `func`: the ratio of measured
    to algorithmic bytes from a committed ncu summary of the same workload
    family and precision (a line `traffic_ratio <func> <ratio>` in
    profiles/<func>_<workload>*_dram.md, captured on a case larger than L2
    but a few GB at most), times this launch's algorithmic bytes -- the
    kernel's traffic grows in proportion to the cells and faces it
    processes.  (None, None) when no capture of this workload exists.
    Returns (bytes, source)."""
    import glob
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", f"{func}_{workload}*_dram.md"))):
        for ln in open(path):
            parts = ln.split()
            if len(parts) == 3 and parts[0] == "traffic_ratio" and parts[1] == func:
                return (float(parts[2]) * alg_bytes,
                        "ncu dram__bytes_read.sum + dram__bytes_write.sum over algorithmic bytes on a "
                        f"smaller case, scaled to one full launch ({os.path.relpath(path, ROOT)})")
    return None, None


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def wait_first(self, timeout=3.0):
        t0 = time.time()
        while self.proc is not None and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.02)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def kernel_bytes(name: str, N: int, nf: dict, nq: int, sw: int, ct: bool) -> float:
    """Algorithmic (compulsory) HBM bytes of one launch of each kernel: every
    array element the kernel must read or write, moved once (neighbour and
    face re-reads are assumed served on chip).  N = cells incl. ghosts,
    nf[d] = faces of dimension d ("r", "z"), sw = bytes of a reconstruction
    value (4 mixed, 8 FP64), index = 4 bytes, positions/conserved = 8 bytes."""
    ix, f8 = 4, 8
    nfa = nf["r"] + nf["z"]
    c = 1 if ct else 0
    if name == "plm_phi":
        return N * (2 * nq * sw + sw)
    if name.startswith("plm_slopes"):   # per face: indices, offsets, slopes out
        d = name[-1]
        return N * 2 * nq * sw + nf[d] * (2 * ix + 2 * sw + nq * sw)
    if name.startswith("plm_trans"):    # per cell: runs, gradient out; per face: slopes, area
        d = name[-1]
        return N * (nq * sw + sw + 4 * ix) + nf[d] * (nq * sw + sw)
    if name in ("flux_phi", "phi_sweep"):
        # the staged sweep (plm_phi + flux_phi from one stage) reads the
        # primitives and widths once and writes the gradients it forms: the
        # same compulsory bytes as flux_phi alone
        return N * (3 * nq * sw + sw + 2 * f8 + c * 16 * sw)
    if name in ("flux_r", "flux_z"):
        d = name[-1]
        return N * 3 * nq * sw + nf[d] * (2 * ix + f8 + 3 * sw + nq * sw + c * 3 * sw)
    if name == "ct_gather":
        return N * (36 * sw + 4 * ix) + nfa * 5 * sw
    if name == "ct_avg":
        return N * (20 * sw + f8 + 4 * ix) + nfa * 2 * sw
    if name == "ct_bflux":   # incl. the RK adjustment of Phi (RKPhi read or written)
        return N * (4 * sw + 15 * f8 + 4 * ix)
    if name == "ct_edge":
        return N * (f8 + 4 * sw + 10 * f8)
    if name == "ct_flip":
        return N * f8 + nfa * (1 + 2 * ix)
    if name == "ct_b2c":
        return N * (5 * f8 + 3 * f8 + sw + 4 * ix) + nfa * (sw + 1 + 2 * ix)
    if name == "c2p":
        return N * (nq * f8 + nq * sw + sw + f8)
    if name == "ct_b2c_c2p":
        return kernel_bytes("ct_b2c", N, nf, nq, sw, ct) + kernel_bytes("c2p", N, nf, nq, sw, ct)
    if name == "update":
        return N * (2 * nq * f8 + 3 * nq * sw + 5 * f8 + sw + 8 * ix) + nfa * nq * sw
    if name in ("faces_r", "faces_z"):
        d = name[-1]
        return N * (2 * f8 + 4 * ix) + nf[d] * (2 * ix + 1 + f8 + 3 * sw + c * 4 * sw)
    if name == "mindt":
        return N * (nq * sw + 2 * f8 + sw)
    if name in ("wcell_ring", "wcell", "wcell_avg"):
        return N * (sw + f8)
    if name == "boundary":
        return N * 2 * f8
    if name == "diag":   # ring diagnostics: five primitives and the position of each cell
        return N * (5 * sw + 2 * f8)
    if name == "anchor":
        return N * f8
    return 0.0


def splitmix64(x: int):
    """The splitmix64 generator (Steele, Lea, Flood 2014): returns
    (next state, 64-bit output)."""
    M = (1 << 64) - 1
    x = (x + 0x9E3779B97F4A7C15) & M
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return x, z ^ (z >> 31)


def batch_members(n: int, nr_range=(64, 512)):
    """(Num_R, Mass_Ratio) of batch member i, drawn from splitmix64 seeded i."""
    out = []
    lo, hi = nr_range
    for i in range(n):
        st, a = splitmix64(i)
        st, b = splitmix64(st)
        nr = lo + a % (hi - lo + 1)
        q = 10.0 ** (-5.0 + 2.0 * (b / 2.0 ** 64))
        out.append({"Num_R": int(nr), "Mass_Ratio": float(q)})
    return out


def measure_batch(args, wl):
    """The batch workload: both precisions as one Batch each, same members."""
    import torch
    import disco_gb300 as dg
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    cfg = os.path.join(ROOT, wl["dir"])
    par, mk = os.path.join(cfg, "in.par"), os.path.join(cfg, "Makefile_opt.in")
    mem = batch_members(wl["batch"], wl.get("nr_range", (64, 512)))
    res, sets, batches = {}, {}, {}
    for prec in (1, 0):
        doms = [dg.Domain(par, mk, precision=prec, overrides=m) for m in mem]
        b = dg.Batch(doms)
        sets[prec], batches[prec] = doms, b
        cells = sum(d.num_real_cells for d in doms)
        N = sum(d.num_cells for d in doms)
        nq = doms[0].host.num_q
        sw = 4 if prec else 8
        state_bytes = N * nq * (4 * 8 + 4 * sw)
        flush = 2 * L2_BYTES if state_bytes < 4 * L2_BYTES else 0
        b.run(args.warmup)
        tune_steps = 0
        while b.info()["split"] < 0:   # the split autotuner's steps: more warm-up
            b.run(1)
            tune_steps += 1
        torch.cuda.synchronize()
        clk = ClockSampler(dev) if prec == 1 else None
        if clk:
            clk.start()
            clk.wait_first()
        l0 = dg.lib().disco_gpu_launch_count()
        ms = b.run_timed(args.steps, flush_bytes=flush)
        launches = dg.lib().disco_gpu_launch_count() - l0
        if clk:
            time.sleep(0.25)
        clocks = clk.stop() if clk else None
        res[prec] = {"ms": ms, "cells": cells, "N": N, "nq": nq, "sw": sw, "flush": flush,
                     "launches": launches, "clocks": clocks,
                     "value": cells * args.steps / (ms / 1e3),
                     "batch": {**b.info(), "autotune_warmup_steps": tune_steps,
                               "launches_per_step": launches / args.steps}}
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import cell_radius, grouped_rel_l1
    worst, worst128, per_member = {}, {}, []
    for m, d1, d0 in zip(mem, sets[1], sets[0]):
        s1, s0 = d1.state(), d0.state()
        h = d0.host
        real = h.real_mask()
        r = cell_radius(h.Np, h.r_jph, h.Nr, h.Nz)[real]
        e = grouped_rel_l1(s1["cons"][:, real], s0["cons"][:, real], r, 5)
        per_member.append([m["Num_R"], max(e.values())])
        for k, v in e.items():
            worst[k] = max(worst.get(k, 0.0), v)
            if m["Num_R"] >= 128:
                worst128[k] = max(worst128.get(k, 0.0), v)
    res["l1_err"] = {"max_over_quantities": max(worst.values()), "per_quantity": worst,
                     "max_over_quantities_Nr_ge_128": max(worst128.values()) if worst128 else None,
                     "per_member_Nr_and_max": sorted(per_member),
                     "note": "maximum over the batch members of the per-member error"}
    # the same members with one graph branch each (no multi-instance groups)
    nb = dg.Batch(sets[1], groups=False)
    nb.run(args.warmup)
    l0 = dg.lib().disco_gpu_launch_count()
    nms = nb.run_timed(args.steps, flush_bytes=res[1]["flush"])
    res[1]["batch"]["branch_per_member"] = {
        "ms_per_step": nms / args.steps, "launches_per_step": (dg.lib().disco_gpu_launch_count() - l0) / args.steps,
        "value": res[1]["cells"] * args.steps / (nms / 1e3)}
    nb.close()
    res[1]["batch"]["stages"] = batches[1].profile(2)
    # per-kernel profile of the largest member (its own stream, no graph)
    big = max(range(len(mem)), key=lambda i: sets[1][i].num_cells)
    res["profile"] = sets[1][big].profile(3)
    hb = sets[1][big].host
    Np = hb.Np.reshape(hb.Nz, hb.Nr)
    res["profiled"] = {"N": sets[1][big].num_cells,
                       "nf": {"r": int((Np[:, :-1] + Np[:, 1:]).sum()) if hb.Nr > 1 else 0,
                              "z": int((Np[:-1, :] + Np[1:, :]).sum()) if hb.Nz > 1 else 0},
                       "member": big, "Num_R": mem[big]["Num_R"]}
    # e2e: upload every member's state from pinned host memory, K x (one batch
    # step, read every member's time to the host), download every member
    doms = sets[1]
    pins = []
    for d in doms:
        st = d.state()
        pin = {k: torch.empty(st[k].shape, dtype=torch.float64, pin_memory=True).numpy()
               for k in ("piph", "dphi", "wiph", "prim", "cons")}
        for k in pin:
            pin[k][...] = st[k]
        pins.append(pin)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for d, pin in zip(doms, pins):
        d.upload(**pin)
    for _ in range(args.steps):
        batches[1].run(1)
        [d.t for d in doms]
    outs = [d.state() for d in doms]
    t1 = time.perf_counter()
    up = sum(pin[k].nbytes for pin in pins for k in pin)
    down = sum(o[k].nbytes for o in outs for k in ("piph", "dphi", "wiph", "prim", "cons"))
    res["e2e"] = {"value": res[1]["cells"] * args.steps / (t1 - t0), "unit": "zone-updates/s",
                  "h2d_bytes_per_step": int(up / args.steps),
                  "d2h_bytes_per_step": int(down / args.steps + 8 * len(doms)),
                  "timed": "upload of every member's state, K x (batch step, members' times "
                           "to host), download of every member"}
    for bb in batches.values():
        bb.close()
    for ds in sets.values():
        for d in ds:
            d.close()
    return res


def measure_learned_c2p(args, wl, steps=None, warmup=None):
    """GRMHD torus: the Newton cons2prim started from the previous
    primitives (the reference's start) against the learned starting point,
    both from the same state.  One domain: W warm-up steps, its state saved;
    training pairs recorded by the running torus's own cons2prim solves
    (every 8th real cell, four steps) and the MLP trained on the GPU; then
    the saved state restored and K timed steps with the plain start, restored
    again and K timed steps with the learned start attached.  Reports for
    both the mean iteration at first convergence (k_converge), the mean
    iterations per call, the calls that did not converge and the throughput,
    and the relative L1 difference of the two final states."""
    import torch
    import disco_gb300 as dg
    K = steps or args.steps
    W = warmup or args.warmup
    cfg = os.path.join(ROOT, wl["dir"])
    d = dg.Domain(os.path.join(cfg, "in.par"), os.path.join(cfg, "Makefile_opt.in"), precision=0,
                  overrides=wl.get("overrides"))
    cells = d.num_real_cells
    d.run(W)
    torch.cuda.synchronize()
    keys = ("piph", "dphi", "wiph", "prim", "cons")
    s0 = d.state()
    saved = {k: s0[k].copy() for k in keys}
    m = dg.Mlp(seed=1, capacity=1 << 21)
    t0 = time.perf_counter()
    held = m.harvest(d, stride=8, steps=4)
    t1 = time.perf_counter()
    m.fit_norm()
    l0, l1 = m.train(2000, batch=8192, lr=2e-3, seed=5)
    t2 = time.perf_counter()

    def arm(guess, ratio=1.0):
        d.upload(**saved)
        m.set_gate(0.0, ratio)
        d.attach_guess(m if guess else None)
        st0 = d.status()
        d.c2p_stats(reset=True)
        ms = d.run_timed(K)
        sc = d.c2p_stats(reset=True)
        st1 = d.status()
        sc["nan_cells"] = st1["nan_cells"] - st0["nan_cells"]
        return ms, sc, st1["c2p_no_converge"] - st0["c2p_no_converge"], d.state()["cons"]

    ms_plain, sp, ncp, up = arm(False)
    ms_learned, sl, ncl, ul = arm(True)
    gated = arm(True, 1e-2)
    d.attach_guess(None)
    real = d.host.real_mask()

    def rdiff(u):
        # over the cells finite in both states (the non-finite ones are
        # counted per arm: nan_cells)
        ok = real & np.isfinite(u).all(0) & np.isfinite(up).all(0)
        return max(float(np.abs(u[q, ok] - up[q, ok]).sum() / max(np.abs(up[q, ok]).sum(), 1e-300))
                   for q in range(up.shape[0]))
    diff = rdiff(ul)
    d.close()
    m.close()

    def mean(s, k):
        return s[k] / s["calls"] if s["calls"] else None
    kp, kl = mean(sp, "kconv"), mean(sl, "kconv")
    ms_g, sg, ncg, ug = gated
    return {"cells": cells, "steps": K,
            "plain": {"zone_updates_per_s": cells * K / (ms_plain / 1e3), "ms_per_step": ms_plain / K,
                      "mean_k_converge": kp, "mean_iterations": mean(sp, "iters"), "calls": sp["calls"],
                      "no_converge": ncp, "nan_cells": sp["nan_cells"]},
            "learned": {"zone_updates_per_s": cells * K / (ms_learned / 1e3), "ms_per_step": ms_learned / K,
                        "mean_k_converge": kl, "mean_iterations": mean(sl, "iters"), "calls": sl["calls"],
                        "no_converge": ncl, "nan_cells": sl["nan_cells"],
                        "guess_used_fraction": sl["guessed"] / sl["calls"] if sl["calls"] else None},
            "k_converge_ratio_plain_over_learned": (kp / kl) if kp and kl else None,
            "final_state_rel_l1_learned_vs_plain": diff,
            "learned_gate_1e-2": {"zone_updates_per_s": cells * K / (ms_g / 1e3), "ms_per_step": ms_g / K,
                                  "mean_k_converge": mean(sg, "kconv"), "mean_iterations": mean(sg, "iters"),
                                  "no_converge": ncg, "nan_cells": sg["nan_cells"],
                                  "guess_used_fraction": sg["guessed"] / sg["calls"] if sg["calls"] else None,
                                  "final_state_rel_l1_vs_plain": rdiff(ug),
                                  "gate": "learned start taken where its residual is below 1e-2 of the "
                                          "previous primitives'"},
            "training": {"pairs": held, "harvest_s": t1 - t0, "train_s": t2 - t1, "steps": 2000, "batch": 8192,
                         "loss_first": l0, "loss_last": l1},
            "k_converge_definition": ("Newton iteration at which the relative change of eta first falls "
                                      "below 1e-12 (the 10 polishing iterations that follow are not counted; "
                                      "0 for a call that never converged; a learned start that did not "
                                      "converge adds its iterations to the fallback solve's)")}


def measure_ours(args, wl, rank):
    """One domain at a time (the large workloads do not fit twice in HBM):
    the mixed path first -- timing, per-kernel profile, its state kept on the
    host, e2e through the C ABI -- then the FP64 path on the same input, and
    the mixed path's error against it."""
    import torch
    import disco_gb300 as dg
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    cfg = os.path.join(ROOT, wl["dir"])
    par, mk = os.path.join(cfg, "in.par"), os.path.join(cfg, "Makefile_opt.in")
    res = {}
    saved = {}
    precs = wl.get("precisions", (1, 0))
    chosen = precs[0]   # the path the line reports; the other one checks its error
    res["chosen"] = chosen
    for prec in precs:
        d = dg.Domain(par, mk, precision=prec, overrides=wl.get("overrides"))
        cells = d.num_real_cells
        N = d.num_cells
        nq = d.host.num_q
        sw = 4 if prec else 8
        state_bytes = N * nq * (4 * 8 + 4 * sw)
        flush = 2 * L2_BYTES if state_bytes < 4 * L2_BYTES else 0
        d.run(args.warmup)
        torch.cuda.synchronize()
        clk = ClockSampler(dev) if prec == chosen else None
        if clk:
            clk.start()
            clk.wait_first()
        l0 = dg.lib().disco_gpu_launch_count()
        ms = d.run_timed(args.steps, flush_bytes=flush)
        launches = dg.lib().disco_gpu_launch_count() - l0
        if clk:
            time.sleep(0.25)
        clocks = clk.stop() if clk else None
        res[prec] = {"ms": ms, "cells": cells, "N": N, "nq": nq, "sw": sw, "flush": flush,
                     "launches": launches, "clocks": clocks,
                     "value": cells * args.steps / (ms / 1e3)}
        st = d.state()
        saved[prec] = {"cons": st["cons"]}
        if prec == 0:
            saved["host"] = d.host
        if prec == chosen:
            # per-kernel breakdown (events around each launch), then e2e
            # through the C ABI with host buffers: upload from pinned host
            # memory, K x (getmindt -> dt to host, timestep(dt) -> dt to
            # device), download
            res["profile"] = d.profile(3)
            # report.c's domain sums as a device reduction (disco_gpu_report):
            # host-timed calls, each including its result's copy to the host
            d.report()
            t0 = time.perf_counter()
            for _ in range(10):
                d.report()
            rms = (time.perf_counter() - t0) / 10 * 1e3
            res["report"] = {"ms_per_call": rms, "cells_per_s": cells / (rms / 1e3)}
            # the whole state: with constrained transport the face fluxes Phi too
            keys = ("piph", "dphi", "wiph", "prim", "cons") + (("Phi",) if "Phi" in st else ())
            pin = {k: torch.empty(st[k].shape, dtype=torch.float64, pin_memory=True).numpy()
                   for k in keys}
            for k in pin:
                pin[k][...] = st[k]
            del st
            # the download lands in pinned host buffers as well.  One untimed
            # round trip through both sets of buffers first, as a running
            # program reuses its transfer buffers: the first device write to
            # fresh pinned pages costs up to several times the copy itself
            # (54 against 26 ms for the same download measured back to back)
            pout = {k: torch.empty(pin[k].shape, dtype=torch.float64, pin_memory=True).numpy()
                    for k in pin}
            d.upload(**pin)
            d.state(out=pout)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d.upload(**pin)
            tu = time.perf_counter()
            for _ in range(args.steps):
                d.timestep(d.getmindt())
            torch.cuda.synchronize()   # the last step's kernels count as steps
            ts = time.perf_counter()
            out = d.state(out=pout)
            t1 = time.perf_counter()
            up = sum(pin[k].nbytes for k in pin)
            down = sum(out[k].nbytes for k in keys)
            res["e2e"] = {"value": cells * args.steps / (t1 - t0), "unit": "zone-updates/s",
                          "h2d_bytes_per_step": int(up / args.steps + 8),
                          "d2h_bytes_per_step": int(down / args.steps + 8),
                          "timed": "upload of the full state, K x (getmindt, timestep), download",
                          "phases_ms": {"upload": (tu - t0) * 1e3, "steps": (ts - tu) * 1e3,
                                        "download": (t1 - ts) * 1e3}}
            del out, pin
        d.close()
        del d
    if len(precs) < 2:
        return res
    # accuracy of the chosen path against plain FP64 after the same steps
    h = saved["host"]
    real = h.real_mask()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import cell_radius, component_norms, grouped_rel_l1
    r = cell_radius(h.Np, h.r_jph, h.Nr, h.Nz)[real]
    num_c = 8 if h.num_q >= 8 else 5
    c1, c0 = saved[1]["cons"], saved[0]["cons"]
    grp = grouped_rel_l1(c1[:, real], c0[:, real], r, num_c)
    comp = component_norms(c1[:, real], c0[:, real])
    res["l1_err"] = {"max_over_quantities": max(grp.values()), "per_quantity": grp,
                     "per_component": comp["l1"], "linf_per_component": comp["linf"]}
    return res


def _sample_domain(wl, key):
    import disco_gb300 as dg
    cfg = os.path.join(ROOT, wl["dir"])
    p = dg.read_params(os.path.join(cfg, "in.par"))
    for k, v in wl[key].items():
        setattr(p, k, v)
    return dg.HostDomain(p, dg.read_modules(os.path.join(cfg, "Makefile_opt.in")))


def cpu_baseline(wl, target_s=12.0):
    """The reference on one host core, on a bounded sample of the workload:
    the unmodified reference binary on one tile of the full grid (3 steps
    after 1 warm-up) where it was built; else the oracle (plain-C
    restatement, bit-exact with the reference build), single thread, on the
    same configuration at the resolution in wl["cpu_sample"], for as many
    steps as fit in about target_s seconds."""
    exe = os.path.join(ROOT, "oracle", "_ref", os.path.basename(wl["dir"]), "disco_ref")
    if wl.get("ref_tiles") is not None and os.path.exists(exe):
        class _A:
            steps, warmup = 3, 1
        v, cells, sec, sample, nt = run_reference_binary(_A, wl, exe, 1)
        return {"value": v, "unit": "zone-updates/s", "cores": 1, "kind": "reference", "sample": sample}
    from oracle.port import PortDomain
    h = _sample_domain(wl, "cpu_sample")
    o = PortDomain(h)
    cells = o.num_real
    t0 = time.perf_counter()
    o.step()
    one = time.perf_counter() - t0
    n = max(1, int(target_s / max(one, 1e-6)))
    t0 = time.perf_counter()
    o.run(n)
    dt = time.perf_counter() - t0
    res = ", ".join(f"{k}={v}" for k, v in wl["cpu_sample"].items()) or "full resolution"
    return {"value": cells * n / dt, "unit": "zone-updates/s", "cores": 1, "kind": "port",
            "sample": f"{n} RK2 steps of the same configuration at {res} ({cells} cells), 1 thread"}


def _ref_worker(wl_name, warmup, steps, q):
    wl = WORKLOADS[wl_name]
    from oracle.port import PortDomain
    h = _sample_domain(wl, "ref_sample")
    o = PortDomain(h)
    o.run(warmup)
    t0 = time.perf_counter()
    o.run(steps)
    q.put((o.num_real, time.perf_counter() - t0))


def _ref_tiles(wl, ncores):
    """Tiles of the workload's full grid for the reference arm: (in.par
    overrides, description) per host core.  A tile is a block of whole rings
    of the full-resolution grid -- its radial and vertical bounds are the
    full grid's ring edges, so every ring keeps its Np and every cell its
    size and initial state -- bounded by the configured boundary plugin at
    the tile edges, as the reference's own domain decomposition
    (mpisetup.c, gridsetup.c) cuts the grid, without the halo exchange."""
    t = wl.get("ref_tiles")
    if t is None:
        return None
    Nr, Nz, rmin, rmax, zmin, zmax = t["grid"]
    tr, tz = t["tile"]
    na, nb = Nr // tr, Nz // tz
    dr, dz = (rmax - rmin) / Nr, (zmax - zmin) / Nz
    nslab = max(1, (ncores + na - 1) // na)     # vertical positions sampled
    step = max(1, nb // nslab)
    out = []
    for i in range(ncores):
        a = i % na
        b = ((i // na) * step + step // 2) % nb
        ov = {"Num_R": tr, "R_Min": rmin + a * tr * dr, "R_Max": rmin + (a + 1) * tr * dr,
              "Num_Z": tz, "Z_Min": zmin + b * tz * dz, "Z_Max": zmin + (b + 1) * tz * dz}
        out.append((ov, f"rings {a * tr}..{(a + 1) * tr - 1}, layers {b * tz}..{(b + 1) * tz - 1}"))
    return out


def run_reference_binary(args, wl, exe, ncores):
    """The unmodified reference (built from its own sources by
    oracle/ref/Makefile) on tiles of the full grid, one process per host
    core, all running at once: each process does W untimed warm-up steps and
    K timed steps of its tile (getmindt + timestep, the reference's main
    loop), timed by the harness with clock_gettime."""
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import patch_par
    base = open(os.path.join(ROOT, wl["dir"], "in.par")).read()
    tiles = _ref_tiles(wl, ncores)
    procs = []
    tmp = tempfile.mkdtemp(prefix="disco_refarm_")
    for i, (ov, _) in enumerate(tiles):
        td = os.path.join(tmp, f"t{i}")
        os.makedirs(td)
        with open(os.path.join(td, "in.par"), "w") as f:
            f.write(patch_par(base, ov))
        procs.append(subprocess.Popen([exe, "time", str(args.steps), str(args.warmup)], cwd=td,
                                      stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True))
    res = []
    for p in procs:
        _, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"reference tile run failed ({p.returncode}): {err[-400:]}")
        line = [ln for ln in err.splitlines() if ln.startswith("{")][-1]
        res.append(json.loads(line))
    cells = sum(r["cells"] for r in res)
    sec = max(r["seconds"] for r in res)
    v = cells * args.steps / sec
    t = wl["ref_tiles"]
    sample = (f"{len(tiles)} tiles of the full {t['grid'][0]}x{t['grid'][1]} grid at full resolution "
              f"({t['tile'][0]} rings x {t['tile'][1]} layers each, {cells} cells in all, "
              f"{cells / wl['cells_full']:.3f} of the grid), one process per host core, "
              f"{args.steps} RK2 steps after {args.warmup} warm-up; the unmodified reference built "
              "from its own sources (oracle/ref/Makefile), serial build, clock_gettime around the step loop")
    return v, cells, sec, sample, len(tiles)


def run_reference(args, wl, rank, world):
    """The reference's own CPU implementation of the path on the host cores:
    the unmodified reference binary on tiles of the full grid (one process
    per core) where it was built, else the C restatement (bit-exact with the
    reference build) as independent replicas on a bounded sample."""
    if rank != 0:
        return
    ncores = max(1, min(os.cpu_count() or 1, 16))
    exe = os.path.join(ROOT, "oracle", "_ref", os.path.basename(wl["dir"]), "disco_ref")
    if wl.get("ref_tiles") is not None and not os.path.exists(exe):
        from oracle.build_oracle import build_ref
        build_ref(configs=[wl["dir"]])
    if wl.get("ref_tiles") is not None and os.path.exists(exe):
        v, cells, sec, sample, nt = run_reference_binary(args, wl, exe, ncores)
        line = {"metric": "zone-updates/s", "value": v, "unit": "zone-updates/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "impl": "reference",
                "config": {"workload": wl["desc"], "cells_timed": cells, "tiles": nt,
                           "same_grid": "tiles of the full-resolution grid"},
                "cpu_baseline": {"value": v, "unit": "zone-updates/s", "cores": nt, "kind": "reference",
                                 "sample": sample},
                "e2e": {"value": v, "unit": "zone-updates/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if wl.get("ref_sample") is None:
        print(json.dumps({"impl": "reference",
                          "unavailable": "the C restatement of the reference covers the Newtonian "
                                         "modules only; the reference's GRMHD build runs only where "
                                         "its sources are"}), flush=True)
        return
    import multiprocessing as mp
    from oracle.build_oracle import build_port
    build_port()
    ncores = max(1, min(os.cpu_count() or 1, 64))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_ref_worker, args=(args.workload, args.warmup, args.steps, q))
             for _ in range(ncores)]
    for p in procs:
        p.start()
    out = [q.get() for _ in procs]
    for p in procs:
        p.join()
    cells = out[0][0]
    sec = max(o[1] for o in out)
    v = ncores * cells * args.steps / sec
    res = ", ".join(f"{k}={v2}" for k, v2 in wl["ref_sample"].items()) or "full resolution"
    sample = (f"{ncores} independent replicas (one per host core) of the same configuration at "
              f"{res} ({cells} cells each), {args.steps} RK2 steps after {args.warmup} warm-up; "
              "C restatement pinned bit-for-bit to the reference build (the reference sources "
              "are not on this host)")
    line = {"metric": "zone-updates/s", "value": v, "unit": "zone-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": wl["desc"], "cells_per_replica": cells, "replicas": ncores},
            "cpu_baseline": {"value": v, "unit": "zone-updates/s", "cores": ncores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "zone-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=list(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    wl = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        run_reference(args, wl, rank, world)
        return

    import torch
    import __graft_entry__
    __graft_entry__.build()
    pg = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        pg = dist
        dist.barrier()
    res = measure_batch(args, wl) if wl.get("batch") else measure_ours(args, wl, rank)
    if wl["dir"].endswith("cfg4_grmhd_torus"):
        res["learned_c2p"] = measure_learned_c2p(args, wl)
    ch = res.get("chosen", 1)
    ms = res[ch]["ms"]
    if pg is not None:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
        pg.barrier()
    if rank != 0:
        if pg is not None:
            pg.destroy_process_group()
        return
    cells = res[ch]["cells"]
    value = world * cells * args.steps / (ms / 1e3)
    hbm, peak_kind = _peaks()
    # dominant kernel of the chosen path, from the per-launch CUDA-event profile
    N, nq, sw = res[ch]["N"], res[ch]["nq"], res[ch]["sw"]
    import disco_gb300 as dg  # noqa: F401
    from disco_gb300.api import Domain  # noqa: F401
    nf = {"r": 0, "z": 0}
    if "profiled" in res:   # batch: the profile is of its largest member
        N, nf = res["profiled"]["N"], res["profiled"]["nf"]
    else:
        hp = dg.read_params(os.path.join(ROOT, wl["dir"], "in.par"))
        for k, v in (wl.get("overrides") or {}).items():
            setattr(hp, k, v)
        hd = dg.HostDomain(hp,
                           dg.read_modules(os.path.join(ROOT, wl["dir"], "Makefile_opt.in")))
        Np = hd.Np.reshape(hd.Nz, hd.Nr)
        if hd.Nr > 1:
            nf["r"] = int((Np[:, :-1] + Np[:, 1:]).sum())
        if hd.Nz > 1:
            nf["z"] = int((Np[:-1, :] + Np[1:, :]).sum())
    ct = nq >= 8 and "precisions" not in wl   # the GRMHD workload has cell-centred B
    # per kernel FUNCTION: the r and z launches of one kernel (flux_r and
    # flux_z are both k_flux_trans) count together
    funcs = {}
    for name, launches, ms_tot in res["profile"]:
        f = KERNEL_FUNCTION.get(name, name)
        e = funcs.setdefault(f, {"launches": 0, "ms": 0.0, "bytes": 0.0})
        e["launches"] += launches
        e["ms"] += ms_tot
        e["bytes"] += kernel_bytes(name, N, nf, nq, sw, ct) * launches
    tot_prof = sum(e["ms"] for e in funcs.values())
    top_name, top = max(funcs.items(), key=lambda kv: kv[1]["ms"])
    top_bytes = top["bytes"] / top["launches"]
    top_avg_s = top["ms"] / top["launches"] / 1e3
    achieved = top_bytes / top_avg_s / 1e9
    traffic, traffic_src = _traffic(top_name, top_bytes, args.workload)
    # fused-RK2 compulsory bytes per zone-update: NQ (6 s_W + 4 s_U) + 6 x 8
    # (the RK copy of the state is one s_W write and one s_W read: the mixed
    # path keeps the first substep's increment in R), plus 25 x 8 for the
    # face fluxes Phi / RK_Phi of constrained transport
    bz = nq * (6 * sw + 4 * 8) + 6 * 8 + (200 if ct else 0)
    whole = {"algorithmic_bytes_per_zone_update": bz, "achieved_GBps": bz * value / 1e9,
             "frac_of_hbm": bz * value / 1e9 / hbm}
    symbols = KERNEL_SYMBOL
    roof = {"bound": "hbm", "kernel": symbols.get(top_name, top_name), "achieved": achieved,
            "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "peak_kind": peak_kind,
            "traffic": traffic, "traffic_source": traffic_src,
            "algorithmic_bytes_per_launch": top_bytes, "launches_per_step": top["launches"] / 3,
            "share_of_step": top["ms"] / tot_prof,
            "step": {"algorithmic_bytes_per_zone_update": bz, "achieved": whole["achieved_GBps"],
                     "frac": whole["frac_of_hbm"]}}
    line = {
        "metric": "zone-updates/s", "value": value, "unit": "zone-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 reconstruction/fluxes, f64 positions/accumulation" if ch == 1 else "f64",
        "data": "synthetic",
        "config": {"workload": wl["desc"], "cells": cells, "precision": "mixed" if ch == 1 else "fp64",
                   **({"members": wl["batch"], "profiled_member": res["profiled"]}
                      if "profiled" in res else {}),
                   "l2": "flushed between steps" if res[ch]["flush"] else "inputs larger than L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": roof,
        "step_hbm": whole,
        "kernels": {symbols.get(f, f): {"ms_per_step": e["ms"] / 3, "launches_per_step": e["launches"] / 3,
                                              "GBps": e["bytes"] / (e["ms"] / 1e3) / 1e9 if e["ms"] > 0 else None}
                    for f, e in sorted(funcs.items(), key=lambda kv: -kv[1]["ms"])},
        "e2e": res["e2e"],
        **({"report_reduction": res["report"]} if "report" in res else {}),
        **({"learned_c2p": res["learned_c2p"]} if "learned_c2p" in res else {}),
        **({"batch": {"mixed": res[1]["batch"], "fp64": res[0]["batch"]}}
           if "profiled" in res else {}),
        "gpu_launches": int(res[ch]["launches"]),
        "clocks": res[ch]["clocks"],
    }
    if ch == 1 and 0 in res:
        line["fp64"] = {"value": world * res[0]["cells"] * args.steps / (res[0]["ms"] / 1e3),
                        "ms_per_step": res[0]["ms"] / args.steps}
    if "l1_err" in res:
        line["l1_err_vs_fp64"] = res["l1_err"]
        line["l1_err_definition"] = ("sum over interior cells of |U_chosen - U_fp64| / sum |U_fp64| per "
                                     "physical quantity (mass, energy, momentum vector, B vector, passive; "
                                     "vectors through the norm of the difference), per conserved component, "
                                     "and max |U_chosen - U_fp64| / max |U_fp64| per component (Linf), "
                                     "after warmup+steps RK2 steps from the same initial state, each path "
                                     "with its own FP64 CFL dt")
    if world == 1 and not args.no_cpu_baseline:
        if wl.get("cpu_sample") is None:
            line["cpu_baseline"] = {"value": None, "unit": "zone-updates/s", "cores": 0, "kind": None,
                                    "sample": None,
                                    "unavailable": "the C restatement covers the Newtonian modules only; "
                                                   "GRMHD parity is pinned to the reference build's fixtures"}
        else:
            line["cpu_baseline"] = cpu_baseline(wl)
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
