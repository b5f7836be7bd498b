"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference sources are compiled (unmodified, read in place) together with
the harness main by oracle/ref/Makefile into oracle/_ref/<config>/disco_ref;
each case below runs that binary on a small in.par and stores its output as
a compressed .npz.  Run from the repository root:

    python tests/golden/make_golden.py [REFERENCE_DIR [CASE ...]]

The GPU tests compare the device path against these files, so they can run
where the reference sources are not available.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from dumpio import read_dump  # noqa: E402

# name -> (config dir, in.par overrides, number of steps)
CASES = {
    "cfg1_n24": ("configs/cfg1_vortex", {"Num_R": 24}, 10),
    "cfg2_n12": ("configs/cfg2_mhd_disk", {"Num_R": 12, "Num_Z": 6}, 5),
    # the circumbinary MHD disk (binary about its centre of mass, cavity,
    # toroidal field, seeded density perturbations) at 16 x 8 rings
    "cfg5_n16": ("configs/cfg5_cbd_mhd", {"Num_R": 16, "Num_Z": 8}, 5),
    # solver / mesh-motion variants of the vortex: HLL on a static mesh, and
    # HLLC with the exact Keplerian mesh rotation and a different PLM theta
    "cfg1_hll_static": ("configs/cfg1_vortex", {"Num_R": 24, "Riemann_Solver": 0, "Mesh_Motion": 0}, 10),
    "cfg1_exact_mesh": ("configs/cfg1_vortex", {"Num_R": 24, "Mesh_Motion": 4, "Exact_Mesh_Omega": 2,
                                                 "PLM": 1.0}, 10),
    # rotating frame with an off-centre axis and a Keplerian energy frame;
    # HLLC with the small-radius HLL switch
    "cfg1_rotframe": ("configs/cfg1_vortex", {"Num_R": 24, "RotFrame": 1, "RotOmega": 0.3, "RotD": 0.1,
                                               "Energy_Omega": 2, "Riemann_Solver": 3}, 10),
    # one instance of the planet-disk batch: alpha viscosity, locally
    # isothermal, a planet on a circular orbit
    "cfg3_n24": ("configs/cfg3_planet_disk", {"Num_R": 24}, 10),
    # zero-gradient ghosts (Boundary/zerograd.c) on the vortex, in 3D so the
    # z passes run too; outflow ghosts (Boundary/outflow3d.c) on the planet disk
    "cfg1_zerograd": ("configs/cfg1_vortex_zerograd", {"Num_R": 16, "Num_Z": 2}, 10),
    "cfg3_outflow": ("configs/cfg3_planet_disk_outflow", {"Num_R": 24}, 10),
    # the other ghost-ring plugins (Boundary/*.c), each on the 3D vortex;
    # polar3d and tube leave the inner ghost rings alone (they are meant for
    # a domain without them), so their cases have none (NoBC_Rmin): with
    # stale inner ghosts the reference run stalls (polar3d) or goes
    # non-finite (tube) within six steps
    **{f"bc_{b}": ("configs/cfg1_vortex_zerograd",
                   {"Num_R": 12, "Num_Z": 2,
                    **({"NoBC_Rmin": 1} if b in ("polar3d", "polar", "tube") else {})}, 6,
                   {"BOUNDARY": b})
       for b in ("zerograd_omk", "zerograd_omIN", "accrete3d", "fixRrefZ", "polar3d", "fixed_gap",
                 "tube", "surfaceGravBox", "flowthrough", "polar")},
    # Boundary/horizon3d.c on the 2D vortex (r from 0.5): boundary_fixed_horizon
    # resets the rings within R_HOR = 1 of the origin to initial() at every
    # r boundary pass and drops them from the CFL minimum; fixed outer ghosts
    "bc_horizon3d": ("configs/cfg1_vortex", {"Num_R": 24}, 10, {"BOUNDARY": "horizon3d"}),
    # Boundary/horizon.c on the same disk: its own cut (0.7 of 2M, M = 1) with
    # arithmetic-mean positions, after both the r and the z boundary pass
    "bc_horizon": ("configs/cfg1_vortex", {"Num_R": 24}, 10, {"BOUNDARY": "horizon"}),
    # Boundary/horizon_bin.c: two holes of radius 0.8 at x = +-5 (its fixed
    # M = 1, a = 10, q = 1), cell by cell; the vortex out to r = 6 reaches them
    # (no inner ghost rings: the plugin never fills them)
    "bc_horizon_bin": ("configs/cfg1_vortex", {"Num_R": 48, "R_Max": 6.0, "NoBC_Rmin": 1}, 10,
                       {"BOUNDARY": "horizon_bin"}),
    # the MHD disk with the HLL and HLLC solvers (Riemann_Solver 0, 1):
    # mhd.c's vel (fast magnetosonic bounds) and getUstar, with CT
    "cfg2_hll": ("configs/cfg2_mhd_disk", {"Num_R": 12, "Num_Z": 6, "Riemann_Solver": 0}, 5),
    "cfg2_hllc": ("configs/cfg2_mhd_disk", {"Num_R": 12, "Num_Z": 6, "Riemann_Solver": 1}, 5),
    # third-order Runge-Kutta (Timestep 3, timestep.c:35-42) on the vortex,
    # the MHD disk and the viscous planet disk
    "cfg1_rk3": ("configs/cfg1_vortex", {"Num_R": 24, "Timestep": 3}, 10),
    "cfg2_rk3": ("configs/cfg2_mhd_disk", {"Num_R": 12, "Num_Z": 6, "Timestep": 3}, 5),
    "cfg3_rk3": ("configs/cfg3_planet_disk", {"Num_R": 24, "Timestep": 3}, 10),
    # the planet disk with beta cooling relaxing its energy to the
    # sound-speed profile and inner / outer damping towards the initial state
    # (sink.c:274-427); locally isothermal as the disks here are (cooling
    # then acts on the conserved energy), the adiabatic disk goes non-finite
    # within six steps even without these terms
    "cfg3_cooldamp": ("configs/cfg3_planet_disk",
                      {"Num_R": 24, "Cool_Type": 2, "Cool_Par1": 0.5,
                       "DampInner_Type": 2, "DampInner_Time": 1.0, "DampInner_Len": 0.3,
                       "DampOuter_Type": 1, "DampOuter_Time": 2.0, "DampOuter_Len": 0.5}, 10),
    # GRMHD thin disk around a Schwarzschild black hole (Kerr-Schild
    # cylindrical metric, HLL, cell-centred B) at 12 x 4 rings
    "cfg4_n12": ("configs/cfg4_grmhd_disk", {"Num_R": 12, "Num_Z": 4}, 5),
    # the same disk with the GRMHD ring diagnostics (Diagnostics/diag_grmhdmri.c)
    "cfg4_diag": ("configs/cfg4_grmhd_disk", {"Num_R": 12, "Num_Z": 4}, 5, {"ANALYSIS": "diag_grmhdmri"}),
    # the Fishbone-Moncrief torus around a Kerr black hole (a = 0.9, Kerr-Schild
    # cylindrical): the torus body at 16 x 4 rings, and the whole domain
    # (atmosphere down to r = 2) at 24 x 12 rings; the reference's own
    # Hydro/grmhd.c evaluated on the repository's Kerr metric plugin
    "cfg4t_body": ("configs/cfg4_grmhd_torus", {"Num_R": 16, "Num_Z": 4, "R_Min": 8.0, "R_Max": 16.0,
                                                "Z_Min": -2.0, "Z_Max": 2.0}, 5),
    "cfg4t_n24": ("configs/cfg4_grmhd_torus", {"Num_R": 24, "Num_Z": 12}, 5),
    # accreting sinks and the gas nozzle (sink.c:105-247) on the planet disk
    # (dt is about 0.5 here, so the accretion rate Sink_Par1 x omega_p stays
    # well below 1 per step; the central body has omega 0 and accretes
    # nothing): polynomial sinks (Sink_Type 1) with delta 0.5, an
    # exponential sink (Sink_Type 2) with delta 0, and the nozzle
    # (Nozzle_Type 1) feeding gas at r = 1.5
    "cfg3_sink": ("configs/cfg3_planet_disk",
                  {"Num_R": 24, "Sink_Type": 1, "Sink_Number": 0, "Sink_Par1": 0.2, "Sink_Par2": 0.5,
                   "Sink_Par3": 0.15, "Sink_Par4": 2.0, "Sink_Par5": 2.0}, 10),
    "cfg3_sink_exp": ("configs/cfg3_planet_disk",
                      {"Num_R": 24, "Sink_Type": 2, "Sink_Number": 0, "Sink_Par1": 0.2, "Sink_Par2": 0.0,
                       "Sink_Par3": 0.1, "Sink_Par4": 2.0, "Sink_Par5": 1.0}, 10),
    # the MHD disk (HLLD + CT) with zero-gradient and outflow ghosts: the
    # boundary primitives copy the ghost rings' primitives, B included, and
    # leave the CT face fluxes to the CT update, as with fixed ghosts
    "cfg2_outflow": ("configs/cfg2_mhd_disk", {"Num_R": 12, "Num_Z": 6}, 5, {"BOUNDARY": "outflow3d"}),
    "cfg2_zerograd": ("configs/cfg2_mhd_disk", {"Num_R": 12, "Num_Z": 6}, 5, {"BOUNDARY": "zerograd"}),
    # the GRMHD disk with outflow and zero-gradient ghosts
    "cfg4_outflow": ("configs/cfg4_grmhd_disk", {"Num_R": 12, "Num_Z": 4}, 5, {"BOUNDARY": "outflow3d"}),
    "cfg4_zerograd": ("configs/cfg4_grmhd_disk", {"Num_R": 12, "Num_Z": 4}, 5, {"BOUNDARY": "zerograd"}),
    "cfg3_nozzle": ("configs/cfg3_planet_disk",
                    {"Num_R": 24, "Nozzle_Type": 1, "Nozzle_Par1": 1.5, "Nozzle_Par2": 0.5,
                     "Nozzle_Par3": 0.8, "Nozzle_Par4": 20.0}, 10),
}


def patch_par(text: str, overrides: dict) -> str:
    for k, v in overrides.items():
        pat = re.compile(rf"^{re.escape(k)}\b.*$", re.M)
        line = f"{k}\t{v}"
        text, n = pat.subn(line, text)
        if n == 0:
            text += f"\n{line}\n"
    return text


def build_ref(cfg: str, ref: str) -> str:
    subprocess.run(["make", "-s", "-f", "oracle/ref/Makefile", f"CFG={cfg}", f"REF={ref}"],
                   cwd=ROOT, check=True)
    return os.path.join(ROOT, "oracle", "_ref", os.path.basename(cfg), "disco_ref")


def patch_mk(text: str, overrides: dict) -> str:
    for k, v in overrides.items():
        text, n = re.subn(rf"(?m)^{k}\s*=.*$", f"{k} = {v}", text)
        if n == 0:
            text += f"\n{k} = {v}\n"
    return text


def case_config(name: str):
    """(config dir, in.par overrides, steps, Makefile_opt.in text); a case
    with module overrides gets a generated config dir under oracle/_ref."""
    cfg, over, nsteps = CASES[name][:3]
    mk = open(os.path.join(ROOT, cfg, "Makefile_opt.in")).read()
    if len(CASES[name]) > 3:
        mk = patch_mk(mk, CASES[name][3])
        gen = os.path.join("oracle", "_ref", "cfgs", name)
        os.makedirs(os.path.join(ROOT, gen), exist_ok=True)
        with open(os.path.join(ROOT, gen, "Makefile_opt.in"), "w") as f:
            f.write(mk)
        with open(os.path.join(ROOT, cfg, "in.par")) as f, open(os.path.join(ROOT, gen, "in.par"), "w") as g:
            g.write(f.read())
        return gen, over, nsteps, mk, cfg
    return cfg, over, nsteps, mk, cfg


def run_case(name: str, ref: str) -> None:
    gcfg, over, nsteps, mk_text, cfg = case_config(name)
    exe = build_ref(gcfg, ref)
    with open(os.path.join(ROOT, cfg, "in.par")) as f:
        par = patch_par(f.read(), over)
    with tempfile.TemporaryDirectory() as td:
        with open(os.path.join(td, "in.par"), "w") as f:
            f.write(par)
        for mode, args in (("init", ["init", "init.bin"]), ("grad", ["grad", "grad.bin"]),
                           ("run", ["run", str(nsteps), "run.bin"])):
            subprocess.run([exe, *args], cwd=td, check=True, capture_output=True)
        ini = read_dump(os.path.join(td, "init.bin"))
        grd = read_dump(os.path.join(td, "grad.bin"))
        run = read_dump(os.path.join(td, "run.bin"))
        # report.c's line for the final state (printed with 7 significant
        # digits; its "%.7le%le" leaves no space after q, so split on the
        # exponent form every field has)
        line = open(os.path.join(td, "report.dat")).read().strip().splitlines()[-1]
        rep = np.array([float(v) for v in
                        re.findall(r"[-+]?\d\.\d+e[-+]\d{2}(?:\d(?!\.))?", line)])
        # analysis.c's ring diagnostics accumulated over the run
        raw = open(os.path.join(td, "diag.bin"), "rb").read()
        nq, nring = np.frombuffer(raw[:8], dtype="<i4")
        dg = np.frombuffer(raw[8:], dtype="<f8")
        diag_tavg, diag_Qrz = dg[0], dg[1:1 + nq * nring].reshape(nring, nq)
        # the bodies and their sink accumulators before report() zeroed them
        praw = open(os.path.join(td, "planets.bin"), "rb").read()
        npl = int(np.frombuffer(praw[:4], dtype="<i4")[0])
        planets = np.frombuffer(praw[4:], dtype="<f8")[:14 * npl].reshape(npl, 14)
    out = {"par_text": np.array(par), "nsteps": nsteps, "cfg": np.array(cfg), "report": rep,
           "mk_text": np.array(mk_text),
           "diag_tavg": diag_tavg, "diag_Qrz": diag_Qrz, "planets": planets,
           "Np": ini["Np"], "r_jph": ini["r_jph"], "z_kph": ini["z_kph"], "real": ini["real"],
           "init_piph": ini["piph"], "init_dphi": ini["dphi"], "init_prim": ini["prim"],
           "init_cons": ini["cons"], "init_wiph": ini["wiph"],
           "grad_gradp": grd["gradp"], "grad_gradr": grd["gradr"], "grad_gradz": grd["gradz"],
           "run_piph": run["piph"], "run_dphi": run["dphi"], "run_wiph": run["wiph"],
           "run_prim": run["prim"], "run_cons": run["cons"], "run_t": run["t"],
           "init_Phi": ini["Phi"], "run_Phi": run["Phi"]}
    for key in ("r", "z"):
        fc = grd.get(f"faces_{key}")
        if fc is None:
            continue
        out[f"faces_{key}_fIndex"] = fc["fIndex"]
        out[f"faces_{key}_L"] = fc["L"]
        out[f"faces_{key}_R"] = fc["R"]
        out[f"faces_{key}_LRtype"] = fc["LRtype"]
        out[f"faces_{key}_phic"] = fc["cm"][:, 1]
        out[f"faces_{key}_dA"] = fc["dA"]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"wrote {name}.npz")


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    from oracle.build_oracle import reference_dir
    ref = sys.argv[1] if len(sys.argv) > 1 else reference_dir()
    if not ref:
        raise SystemExit("reference sources not found: pass REFERENCE_DIR or set DISCO_REFERENCE")
    names = sys.argv[2:] or list(CASES)
    for n in names:
        run_case(n, ref)
