"""Failure detection by host injection: bad conserved values uploaded
through disco_gpu_upload are caught by the device's health counters
(disco_gpu_status), the kernels never trap, and every call returns 0.

Counters: nan_cells (non-finite primitives after cons2prim), rho_floor_hits
and p_floor_hits (euler.c:107,123 and their GRMHD forms), c2p_no_converge
(the Noble 2D iteration stopped at its cap of 30, grmhd.c:959-968, where the
reference prints and continues)."""
import numpy as np
import pytest

from test_gpu_parity import _domain

pytestmark = pytest.mark.gpu


def _real_cell(g, frac=0.5):
    real = np.flatnonzero(g["real"].astype(bool))
    return int(real[int(frac * (len(real) - 1))])


@pytest.mark.parametrize("precision", [0, 1])
def test_uploaded_nan_is_counted(precision):
    d, g = _domain("cfg1_n24", precision)
    assert d.status()["nan_cells"] == 0
    s = d.state()
    cons = s["cons"].copy()
    c = _real_cell(g)
    cons[1, c] = np.nan          # energy of one real cell
    d.upload(cons=cons)
    d.timestep(d.getmindt())
    st = d.status()
    assert st["nan_cells"] >= 1
    p = d.state()["prim"]
    assert not np.all(np.isfinite(p[:, c]))
    d.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_density_and_pressure_floors_are_counted(precision):
    """A negative mass and a negative energy in two real cells: after the
    step their primitives sit on the floors and both counters fire."""
    import disco_gb300 as dg
    from helpers import load_golden, mk_path, write_par
    g = load_golden("cfg1_n24")
    d = dg.Domain(write_par(g["par_text"]), mk_path(g, "configs/cfg1_vortex"), precision=precision,
                  overrides={"Density_Floor": 1e-4, "Pressure_Floor": 1e-4})
    s = d.state()
    cons = s["cons"].copy()
    a, b = _real_cell(g, 0.3), _real_cell(g, 0.7)
    cons[0, a] = -10.0 * abs(cons[0, a])
    cons[1, b] = -10.0 * abs(cons[1, b])
    d.upload(cons=cons)
    d.timestep(d.getmindt())
    st = d.status()
    assert st["rho_floor_hits"] >= 1
    assert st["p_floor_hits"] >= 1
    p = d.state()["prim"]
    assert p[0, a] == pytest.approx(1e-4, rel=1e-6)
    assert np.all(np.isfinite(p[:, a])) and np.all(np.isfinite(p[:, b]))
    d.close()


def test_grmhd_newton_cap_is_counted():
    """GRMHD: one real cell given a momentum 100 times its own (far beyond
    what its energy allows) drives the Noble 2D iteration to its cap of 30;
    the counter fires and the recovered primitives stay finite."""
    d, g = _domain("cfg4_n12", 0)
    s = d.state()
    cons = s["cons"].copy()
    c = _real_cell(g)
    for q in (2, 3, 4):
        cons[q, c] *= 100.0
    d.upload(cons=cons)
    d.timestep(d.getmindt())
    st = d.status()
    assert st["c2p_no_converge"] >= 1
    p = d.state()["prim"]
    assert np.all(np.isfinite(p[:, c]))
    d.close()


def test_sweep_wait_timeout_is_counted():
    """The staged phi sweep's waits on its tensor copies are bounded (about
    a second of SM clock).  With the copies withheld (a debug mode of
    disco_gpu_debug_sweep) no wait can complete: every block counts the
    timeout, waits once more (bounded) and returns, the call returns 0, and
    the context stays usable -- the domain steps on with the copies back,
    and so does a new one."""
    d, g = _domain("cfg1_n24", 1)
    assert d.set_sweep(True)
    assert d.status()["async_timeouts"] == 0
    assert d.set_sweep(2)
    d.timestep(d.getmindt())
    assert d.status()["async_timeouts"] >= 1
    n0 = d.status()["async_timeouts"]
    assert d.set_sweep(True)
    d.timestep(d.getmindt())
    assert d.status()["async_timeouts"] == n0
    d.close()
    e, _ = _domain("cfg1_n24", 1)
    e.run(2)
    assert np.isfinite(e.state()["cons"]).all() and e.status()["async_timeouts"] == 0
    e.close()
