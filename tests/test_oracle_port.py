"""Pin the CPU oracle (oracle/port, a plain-C restatement of the hot path)
against the reference: bit-for-bit equal to the golden fixture made by the
reference binary, and -- where the reference sources are present -- to a
fresh reference run at another size."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from helpers import ROOT, load_golden, mk_path, write_par


def _port_run(par_path, mk, nsteps):
    import disco_gb300 as dg
    from oracle.port import PortDomain
    h = dg.HostDomain(dg.read_params(par_path), dg.read_modules(mk))
    d = PortDomain(h)
    d.run(nsteps)
    return h, d.state()


def _port_domain(g):
    import disco_gb300 as dg
    from oracle.port import PortDomain
    h = dg.HostDomain(dg.read_params(write_par(g["par_text"])), dg.read_modules(mk_path(g)))
    d = PortDomain(h)
    d.run(int(g["nsteps"]))
    return d


BC_CASES = [f"bc_{b}" for b in ("zerograd_omk", "zerograd_omIN", "accrete3d", "fixRrefZ", "polar3d",
                                 "fixed_gap", "tube", "surfaceGravBox", "flowthrough", "polar",
                                 "horizon3d", "horizon", "horizon_bin")]
SINK_CASES = ["cfg3_sink", "cfg3_sink_exp", "cfg3_nozzle"]
HYDRO_CASES = ["cfg1_n24", "cfg1_hll_static", "cfg1_exact_mesh", "cfg1_rotframe", "cfg3_n24",
               "cfg1_zerograd", "cfg3_outflow", "cfg1_rk3", "cfg3_rk3", "cfg3_cooldamp"] + BC_CASES + SINK_CASES


@pytest.mark.parametrize("name", HYDRO_CASES)
def test_port_bit_exact_vs_golden(name):
    """Hydro cases: HLLC vortex, HLL on a static mesh, exact Keplerian mesh
    rotation, rotating frame with a Keplerian energy frame (HLLC with the
    centre switch), the planet disk with alpha viscosity, and the
    zero-gradient / outflow ghost variants."""
    g = load_golden(name)
    h, s = _port_run(write_par(g["par_text"]), mk_path(g), int(g["nsteps"]))
    real = g["real"].astype(bool)
    assert s["t"] == float(g["run_t"])
    assert np.array_equal(s["piph"], g["run_piph"])
    assert np.array_equal(s["dphi"], g["run_dphi"])
    assert np.array_equal(s["cons"][:, real], g["run_cons"][:, real])
    assert np.array_equal(s["prim"], g["run_prim"]) or np.array_equal(s["prim"][:, real], g["run_prim"][:, real])


@pytest.mark.parametrize("name", SINK_CASES)
def test_port_sink_accumulators_vs_golden(name):
    """sink_src's per-body accumulators (gravL, dM, accL, Ls, kin, therm,
    linXmom, linYmom) after the fixture's steps equal the reference's, which
    the harness dumps before report() zeroes them: bit for bit, the
    restatement summing in the reference's cell order."""
    g = load_golden(name)
    d = _port_domain(g)
    ref = np.asarray(g["planets"])[:, 6:14]
    got = d.sink_accum(ref.shape[0])
    assert np.array_equal(got, ref), (got, ref)
    if name != "cfg3_nozzle":
        assert np.abs(ref[1]).max() > 0   # the planet accretes


def _ref_dir():
    from oracle.build_oracle import reference_dir
    return reference_dir()


REF = _ref_dir()


@pytest.mark.skipif(REF is None, reason="reference sources not present")
def test_port_bit_exact_vs_reference_binary():
    sys_path_golden = os.path.join(ROOT, "tests", "golden")
    import sys
    sys.path.insert(0, sys_path_golden)
    from make_golden import build_ref, patch_par
    from dumpio import read_dump
    exe = build_ref("configs/cfg1_vortex", REF)
    par = patch_par(open(os.path.join(ROOT, "configs/cfg1_vortex/in.par")).read(),
                    {"Num_R": 40, "PLM": 1.2, "Riemann_Solver": 0})
    td = tempfile.mkdtemp()
    with open(os.path.join(td, "in.par"), "w") as f:
        f.write(par)
    subprocess.run([exe, "run", "7", "out.bin"], cwd=td, check=True, capture_output=True)
    ref = read_dump(os.path.join(td, "out.bin"))
    h, s = _port_run(os.path.join(td, "in.par"), os.path.join(ROOT, "configs/cfg1_vortex/Makefile_opt.in"), 7)
    real = ref["real"].astype(bool)
    assert np.array_equal(s["piph"], ref["piph"])
    assert np.array_equal(s["cons"][:, real], ref["cons"][:, real])
    shutil.rmtree(td)


@pytest.mark.parametrize("name", ["cfg2_n12", "cfg2_rk3", "cfg2_outflow", "cfg2_zerograd", "cfg2_hll",
                                  "cfg2_hllc"])
def test_port_mhd_ct_bit_exact_vs_golden(name):
    """3D MHD disk with constrained transport (HLLD; HLL and HLLC with
    mhd.c's vel and getUstar; RK2 and RK3, fixed, outflow and zero-gradient
    ghosts): the oracle equals the reference bit for bit (conserved
    variables, face fluxes, positions)."""
    g = load_golden(name)
    h, s = _port_run(write_par(g["par_text"]), mk_path(g), int(g["nsteps"]))
    real = g["real"].astype(bool)
    assert s["t"] == float(g["run_t"])
    assert np.array_equal(s["piph"], g["run_piph"])
    assert np.array_equal(s["cons"][:, real], g["run_cons"][:, real])
    assert np.array_equal(s["prim"][:, real], g["run_prim"][:, real])


def test_port_circumbinary_vs_golden():
    """3D circumbinary MHD disk (toroidal field, binary about its centre of
    mass): time, positions and face tables are exact; the conserved state
    and face fluxes agree with the reference to a few ulps in a few hundred
    cells (relative L1 below 1e-15)."""
    from helpers import rel_l1
    g = load_golden("cfg5_n16")
    h, s = _port_run(write_par(g["par_text"]), os.path.join(ROOT, str(g["cfg"]), "Makefile_opt.in"),
                     int(g["nsteps"]))
    real = g["real"].astype(bool)
    assert s["t"] == float(g["run_t"])
    assert np.array_equal(s["piph"], g["run_piph"])
    for q in range(s["cons"].shape[0]):
        assert rel_l1(s["cons"][q, real], g["run_cons"][q, real]) < 1e-15, q



# report.c's line: t, q, then 8 per-body sink accumulators per body (zero
# here), then Mass, Torque, Torque2 and the five (Torque1_cut, Torque2_cut)
def _ref_report(g, npl):
    rep = g["report"]
    tail = rep[2 + 8 * npl:]
    keys = ["Mass", "Torque", "Torque2"] + [f"Torque{i}_cut{n}" for n in range(5) for i in (1, 2)]
    out = {"t": rep[0], "q": rep[1]}
    out.update(dict(zip(keys, tail)))
    assert np.all(rep[2:2 + 8 * npl] == 0.0)   # no sinks: the accumulators stay zero
    return out


@pytest.mark.parametrize("name,npl", [("cfg3_n24", 2), ("cfg2_n12", 1)])
def test_port_report_vs_reference(name, npl):
    """The restated report sums equal the reference's report line to its
    7 printed significant digits."""
    import disco_gb300 as dg
    from oracle.port import PortDomain
    g = load_golden(name)
    h = dg.HostDomain(dg.read_params(write_par(g["par_text"])),
                      dg.read_modules(os.path.join(ROOT, str(g["cfg"]), "Makefile_opt.in")))
    d = PortDomain(h)
    d.run(int(g["nsteps"]))
    mine = d.report()
    ref = _ref_report(g, npl)
    for k, v in ref.items():
        assert abs(mine[k] - v) <= 6e-7 * abs(v) + 1e-300, (k, mine[k], v)


@pytest.mark.parametrize("name", HYDRO_CASES + ["cfg2_n12", "cfg5_n16"])
def test_port_diagnostics_vs_reference(name):
    """analysis.c's ring accumulators after the fixture's steps: bit for bit
    where the state is (every case but the circumbinary disk, whose state
    carries a few ulps)."""
    from helpers import rel_l1
    g = load_golden(name)
    dg = _port_domain(g).diagnostics()
    assert dg["t_avg"] == float(g["diag_tavg"])
    if name == "cfg5_n16":
        for q in range(g["diag_Qrz"].shape[1]):
            assert rel_l1(dg["Qrz"][:, q], g["diag_Qrz"][:, q]) < 1e-14, q
    else:
        assert np.array_equal(dg["Qrz"], g["diag_Qrz"])


FACE_CASES = ["cfg1_n24", "cfg2_n12", "cfg5_n16", "cfg3_n24", "cfg1_zerograd"] + BC_CASES


@pytest.mark.parametrize("name", FACE_CASES)
def test_port_faces_and_gradients_bit_exact_vs_golden(name):
    """The restatement's face tables (faces_alt.c) and PLM gradients
    (plm.c) of the initial state equal the reference's, bit for bit: the
    checker the device's face and gradient tests rest on."""
    import disco_gb300 as dg
    from oracle.port import PortDomain
    g = load_golden(name)
    h = dg.HostDomain(dg.read_params(write_par(g["par_text"])), dg.read_modules(mk_path(g)))
    o = PortDomain(h)
    for key, dim in (("r", 1), ("z", 2)):
        if f"faces_{key}_L" not in g:
            continue
        f = o.faces(dim)
        for k in ("fIndex", "L", "R", "LRtype", "phic", "dA"):
            assert np.array_equal(f[k], g[f"faces_{key}_{k}"]), (key, k)
    gr = o.gradients()
    for k in ("gradp", "gradr", "gradz"):
        assert np.array_equal(gr[k], g[f"grad_{k}"]), k
