"""Ring diagnostics that timestep() accumulates (analysis.c:52-108 with the
configuration's Diagnostics/ plugin, called at timestep.c:51), against the
reference's own accumulators after the fixture's steps.

Bar: plain FP64 path within 1e-11 relative L1 per diagnostic over the rings
(the planet cases' torque columns carry the last-bit differences of FP64
cos/sin between CUDA and glibc; everything else sits at 1e-15), t_avg within
1e-12; the mixed path within the state's mixed bound (velocity-linear
fluxes judged against the orbital flux, as the state's vectors are judged
through their norm)."""
import numpy as np
import pytest

from helpers import rel_l1
from test_gpu_parity import CASES, FP64_ONLY, MIXED_BOUND, _domain

pytestmark = pytest.mark.gpu


def _ring_radius(g):
    rj = g["r_jph"]   # r_jph[-1 .. Nr-1]
    rp, rm = rj[1:], rj[:-1]
    r = 2.0 * (rp * rp + rp * rm + rm * rm) / (3.0 * (rp + rm))
    nz = g["diag_Qrz"].shape[0] // len(r)
    return np.tile(r, nz)


def _gross_torque(g, host):
    """Per ring, 2 pi r * (time-integrated mean density) * r * <|f_phi|>:
    the torque density with |f_phi| in place of f_phi.  <|f_phi|> is the
    azimuthal mean of the second body's |f_phi| on the ring (independent of
    where the body is on its circular orbit), from planet.c's point-mass
    force; the body's radius, mass and softening as set up."""
    h = host._ptr.contents
    if h.Npl < 2:
        return None
    pl = h.planets[1]
    r = _ring_radius(g)
    zk = g["z_kph"]
    zc = np.repeat(0.5 * (zk[1:] + zk[:-1]), len(r) // (len(zk) - 1))
    if h.par.grav2D == 1:
        zc = 0.0 * zc
    dl = np.linspace(-np.pi, np.pi, 2048, endpoint=False)[None, :]
    rr, zz = r[:, None], zc[:, None]
    d2 = (rr - pl.r) ** 2 + 4.0 * rr * pl.r * np.sin(0.5 * dl) ** 2 + zz * zz
    fphi = pl.M * pl.r * np.abs(np.sin(dl)) / (d2 + pl.eps ** 2) ** 1.5
    return np.abs(2.0 * np.pi * r * g["diag_Qrz"][:, 0] * r * fphi.mean(axis=1))


def _mixed_errors(a, b, g, host):
    """Relative L1 per diagnostic.  diag_euler's columns that are linear in
    v_r or v_z (the mass fluxes 2 pi r rho v_r, 2 pi r rho v_z and the
    angular-momentum flux 2 pi r rho r^2 Omega v_r) are judged against the
    same flux with the azimuthal velocity r Omega in place of v_r or v_z,
    as the state's vector quantities are judged through their norm: in a
    disk v_r is a small fraction of the orbital speed.  The torque density
    (2 pi r rho r f_phi) is judged against its gross value with |f_phi|: a
    ring's net torque is the residual of terms of both signs set by the
    small density perturbation, which FP32 primitives resolve to about
    1e-7 of the density itself."""
    r = _ring_radius(g)
    scale = {}
    if b.shape[1] == 8:
        scale = {1: np.abs(b[:, 6]) / r, 2: np.abs(b[:, 6]) / r, 4: np.abs(b[:, 6] * r * b[:, 5])}
        gross = _gross_torque(g, host)
        if gross is not None:
            scale[3] = gross
    out = {}
    for q in range(b.shape[1]):
        den = np.abs(b[:, q]).sum() + (scale[q].sum() if q in scale else 0.0)
        out[q] = float(np.abs(a[:, q] - b[:, q]).sum() / (den if den > 0 else 1.0))
    return out


# The 24-ring planet disks, whose state is held to 3e-6 (FP32 and FP64 take
# different minmod branches in a few cells at that resolution): their ring
# means of density and pressure, ghost rings included, sit at 2.9e-6 and
# 3.2e-6 after ten steps.
DIAG_MIXED_BOUND = {"cfg3_n24": 4e-6, "cfg3_outflow": 4e-6, "cfg3_rk3": 4e-6, "cfg3_cooldamp": 4e-6,
                    # the MHD disk's RK3 run, whose dt collapses after one step
                    # (see the state's bound): its ring mean of Omega sits at 7.8e-6
                    "cfg2_rk3": 1.5e-5}


def _run(d, n):
    for _ in range(n):
        d.timestep(d.getmindt())
    return d.diagnostics()


@pytest.mark.parametrize("name", list(CASES))
def test_diagnostics_match_reference_fp64(name):
    d, g = _domain(name)
    dg = _run(d, int(g["nsteps"]))
    ref_q, ref_t = g["diag_Qrz"], float(g["diag_tavg"])
    assert dg["Qrz"].shape == ref_q.shape
    assert abs(dg["t_avg"] - ref_t) <= 1e-12 * abs(ref_t)
    for q in range(ref_q.shape[1]):
        e = rel_l1(dg["Qrz"][:, q], ref_q[:, q])
        assert e < 1e-11, (q, e)
    d.close()


@pytest.mark.parametrize("name", list(CASES))
def test_diagnostics_mixed_precision(name):
    if name in FP64_ONLY:
        pytest.skip("FP64-only module")
    d, g = _domain(name, precision=1)
    dg = _run(d, int(g["nsteps"]))
    errs = _mixed_errors(dg["Qrz"], g["diag_Qrz"], g, d.host)
    bound = DIAG_MIXED_BOUND.get(name, MIXED_BOUND.get(name, 1e-6))
    bad = {q: e for q, e in errs.items() if not e < bound}
    assert not bad, bad
    d.close()


@pytest.mark.parametrize("name", ["cfg1_n24", "cfg3_n24", "cfg5_n16"])
def test_diagnostics_graph_equals_stepwise(name):
    """The accumulation captured in the step graph (disco_gpu_run) gives
    the same accumulators as the getmindt/timestep loop."""
    d1, g = _domain(name)
    d2, _ = _domain(name)
    n = int(g["nsteps"])
    a = _run(d1, n)
    d2.run(n)
    b = d2.diagnostics()
    if name.startswith("cfg5"):   # MHD: FP64 atomics in the EMF sums
        assert rel_l1(b["Qrz"], a["Qrz"]) < 1e-13
    else:
        assert np.array_equal(a["Qrz"], b["Qrz"])
    assert a["t_avg"] == b["t_avg"]
    d1.close(); d2.close()


def test_diagnostics_zero_and_restart():
    """zero_diagnostics and the restart upload: the accumulators are
    replaced, and later steps add to the uploaded values."""
    d, g = _domain("cfg1_n24")
    d.run(2)
    a = d.diagnostics()
    assert a["t_avg"] > 0 and np.abs(a["Qrz"]).sum() > 0
    d.set_diagnostics()
    z = d.diagnostics()
    assert z["t_avg"] == 0.0 and not z["Qrz"].any()
    d.set_diagnostics(a["Qrz"], a["t_avg"])
    b = d.diagnostics()
    assert np.array_equal(a["Qrz"], b["Qrz"]) and b["t_avg"] == a["t_avg"]
    # one more step from the restored accumulators equals one more step
    # of an uninterrupted run
    d2, _ = _domain("cfg1_n24")
    d2.run(3)
    d.run(1)
    assert np.array_equal(d.diagnostics()["Qrz"], d2.diagnostics()["Qrz"])
    with pytest.raises(Exception):
        d.set_diagnostics(np.zeros(3), 0.0)
    d.close(); d2.close()
