"""disco_gpu_report (report.c's domain sums as a device reduction) against
the C restatement after the same steps, and against the reference's own
report line (printed with 7 significant digits)."""
import os

import numpy as np
import pytest

from helpers import ROOT, load_golden, write_par

pytestmark = pytest.mark.gpu

CASES = [("cfg3_n24", "configs/cfg3_planet_disk", 2), ("cfg2_n12", "configs/cfg2_mhd_disk", 1)]


def _runs(name, cfg, precision):
    import disco_gb300 as dg
    from oracle.port import PortDomain
    g = load_golden(name)
    par, mk = write_par(g["par_text"]), os.path.join(ROOT, cfg, "Makefile_opt.in")
    d = dg.Domain(par, mk, precision=precision)
    n = int(g["nsteps"])
    for _ in range(n):
        d.timestep(d.getmindt())
    mine = d.report()
    d.close()
    p = PortDomain(dg.HostDomain(dg.read_params(par), dg.read_modules(mk)))
    p.run(n)
    return g, mine, p.report()


@pytest.mark.parametrize("name,cfg,npl", CASES)
def test_report_fp64_vs_restatement(name, cfg, npl):
    """FP64 path: the same sums as the serial restatement to summation-order
    rounding; the reference's printed values to their 7 digits."""
    g, mine, port = _runs(name, cfg, 0)
    # t to 1e-12: the planet disk's FP64 cos/sin/pow may differ from glibc
    # in the last bit, which reaches dt
    assert abs(mine["t"] - port["t"]) <= 1e-12 * port["t"] and mine["q"] == port["q"]
    for k, v in port.items():
        assert abs(mine[k] - v) <= 1e-12 * abs(v) + 1e-18, (k, mine[k], v)
    rep = g["report"]
    assert abs(mine["Mass"] - rep[2 + 8 * npl]) <= 6e-7 * abs(rep[2 + 8 * npl])
    assert abs(mine["Torque"] - rep[3 + 8 * npl]) <= 6e-7 * abs(rep[3 + 8 * npl]) + 1e-300


@pytest.mark.parametrize("name,cfg,npl", CASES)
def test_report_mixed_mass(name, cfg, npl):
    """Mixed path: the gas mass from the FP32 primitives within 1e-6."""
    g, mine, port = _runs(name, cfg, 1)
    assert abs(mine["Mass"] - port["Mass"]) <= 1e-6 * abs(port["Mass"])
