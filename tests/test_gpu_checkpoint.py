"""Checkpoint of a running device domain (disco_gpu_checkpoint) and restart
from it (disco_host_restart + disco_gpu_create), on the MHD disk with
constrained transport and the planet disk.

The file holds the device state as the reference's output() writes it
(h5out.c:366-620): primitives, face fluxes and phases per cell, the moved
planets, and the ring diagnostics divided by their accumulation time, which
the checkpoint then zeroes (h5out.c:389, :610).  A restart rebuilds the
conserved state from the primitives (prim2cons + cons2prim,
domain.c:211-238), so a restarted run follows the uninterrupted one to the
rounding of that round trip: within 1e-12 per physical quantity on the FP64
path, 1e-6 on the mixed path, after further steps.  With Isothermal the
conserved energy is carried along but never read back (the pressure comes
from the sound-speed profile), so a restart recomputes it from the
primitives, as the reference's does; energy is compared on the adiabatic
vortex.  (An adiabatic run of the MHD disk hits the pressure floor, whose
floored pressure is what the file holds: its energy cannot survive the
restart, in the reference as here, so it makes no restart test.)"""
import os

import numpy as np
import pytest

import h5spec
from helpers import ROOT, cell_radius, grouped_rel_l1

pytestmark = pytest.mark.gpu

CASES = {"mhd": ("configs/cfg2_mhd_disk", {"Num_R": 16, "Num_Z": 8, "noiseType": 0}),
         "vortex": ("configs/cfg1_vortex", {"noiseType": 0}),
         "grmhd": ("configs/cfg4_grmhd_disk", {"Num_R": 16, "Num_Z": 4, "noiseType": 0}),
         "planets": ("configs/cfg3_planet_disk", {"Num_R": 32, "noiseType": 0})}


def _close(err, tol, isothermal):
    keys = [k for k in err if not (isothermal and k == "energy")]
    return all(err[k] < tol for k in keys)


def _domain(name, precision, restart=None):
    import disco_gb300 as dg
    cfg, over = CASES[name]
    par, mk = os.path.join(ROOT, cfg, "in.par"), os.path.join(ROOT, cfg, "Makefile_opt.in")
    return dg.Domain(par, mk, precision=precision, overrides=over, restart=restart)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", list(CASES))
def test_checkpoint_then_restart_continues_the_run(name, precision, tmp_path):
    if name == "grmhd" and precision:
        pytest.skip("GRMHD runs on the FP64 path only")
    d = _domain(name, precision)
    for _ in range(4):
        d.timestep(d.getmindt())
    s = d.state()
    diag = d.diagnostics()
    planets = d.planets()
    path = str(tmp_path / "checkpoint_0001.h5")
    d.checkpoint(path)

    # the file: the downloaded state, the planets, the averaged diagnostics
    f = h5spec.File(path)
    h = d.host
    nq, nf = h.num_q, h.num_faces
    cells = f.dataset("Data/Cells")
    assert cells.shape == (h.Ncell, nq + nf + 1)
    assert np.array_equal(cells[:, :nq].T, s["prim"])
    if nf:
        assert np.array_equal(cells[:, nq:nq + nf].T, s["Phi"])
    assert np.array_equal(cells[:, -1], s["piph"])
    assert f.dataset("Grid/T").tolist() == [s["t"]]
    pl = f.dataset("Data/Planets")
    for i, b in enumerate(planets):
        assert pl[i].tolist() == [b["M"], b["vr"], b["omega"], b["r"], b["phi"], b["eps"], float(b["type"])]
    n = diag["Qrz"].shape[1]
    if n:
        want = (diag["Qrz"] / diag["t_avg"]).reshape(h.Nz, h.Nr, n)
        assert np.array_equal(f.dataset("Data/Diagnostics"), want)
        after = d.diagnostics()
        assert after["t_avg"] == 0.0 and not after["Qrz"].any()

    # the restarted domain starts from the file's state
    r = _domain(name, precision, restart=path)
    s0 = r.state()
    assert s0["t"] == s["t"]
    assert np.array_equal(s0["piph"], s["piph"]) and np.array_equal(s0["dphi"], s["dphi"])
    if nf:
        assert np.array_equal(s0["Phi"], s["Phi"])
    real = h.real_mask()
    rad, nc = cell_radius(h.Np, h.r_jph, h.Nr, h.Nz)[real], d.modules.num_c
    tol = 1e-12 if precision == 0 else 1e-6
    iso = bool(d.params.isothermal_flag)
    err = grouped_rel_l1(s0["cons"][:, real], s["cons"][:, real], rad, nc)
    assert _close(err, tol, iso), err
    assert r.planets() == [{**b, "type": 0} for b in planets]

    # both continue with the same steps
    for _ in range(4):
        dt = d.getmindt()
        d.timestep(dt)
        r.timestep(dt)
    a, b = d.state(), r.state()
    assert a["t"] == b["t"]
    # the cells move with the flow, which differs at rounding: phases agree
    # to that rounding (compared modulo the period)
    pmax = d.params.phimax
    dp = np.abs((a["piph"] - b["piph"] + .5 * pmax) % pmax - .5 * pmax)
    assert dp.max() < (1e-10 if precision == 0 else 1e-6), dp.max()
    err = grouped_rel_l1(b["cons"][:, real], a["cons"][:, real], rad, nc)
    assert _close(err, tol, iso), err
    if precision == 0:   # every primitive on the FP64 path
        for q in range(nq):
            e = np.abs(b["prim"][q, real] - a["prim"][q, real]).sum() / max(np.abs(a["prim"][q, real]).sum(), 1e-300)
            assert e < 1e-11, (q, e)
    assert d.status()["nan_cells"] == 0 and r.status()["nan_cells"] == 0
