"""disco_gpu_upload / disco_gpu_download (the restart path): a state taken
from one instance and uploaded into a fresh one continues as the original
does."""
import os

import numpy as np
import pytest

from helpers import ROOT, cell_radius, grouped_rel_l1, load_golden, rel_l1, write_par

pytestmark = pytest.mark.gpu


def _pair(name, cfg, precision):
    import disco_gb300 as dg
    g = load_golden(name)
    mk = os.path.join(ROOT, cfg, "Makefile_opt.in")
    return (dg.Domain(write_par(g["par_text"]), mk, precision=precision),
            dg.Domain(write_par(g["par_text"]), mk, precision=precision), g)


def test_upload_continues_fp64_vortex():
    """FP64 path: the uploaded instance takes bit-identical steps."""
    d1, d2, g = _pair("cfg1_n24", "configs/cfg1_vortex", 0)
    for _ in range(3):
        d1.timestep(d1.getmindt())
    s = d1.state()
    d2.upload(**{k: s[k] for k in ("piph", "dphi", "wiph", "prim", "cons")})
    s2 = d2.state()
    for k in ("piph", "dphi", "prim", "cons"):
        assert np.array_equal(s[k], s2[k]), k
    for _ in range(3):
        d1.timestep(d1.getmindt())
        d2.timestep(d2.getmindt())
    a, b = d1.state(), d2.state()
    assert np.array_equal(a["cons"], b["cons"])
    assert np.array_equal(a["piph"], b["piph"])
    d1.close(); d2.close()


def test_upload_continues_mixed_mhd_disk():
    """Mixed path with constrained transport (face fluxes Phi included):
    the primitives cross the C ABI in FP64 with the lab-frame omega, are
    converted on the device, and the continuation stays within rounding of
    the original run."""
    d1, d2, g = _pair("cfg2_n12", "configs/cfg2_mhd_disk", 1)
    for _ in range(2):
        d1.timestep(d1.getmindt())
    s = d1.state()
    d2.upload(**{k: s[k] for k in ("piph", "dphi", "wiph", "prim", "cons", "Phi")})
    s2 = d2.state()
    real = g["real"].astype(bool)
    assert np.array_equal(s["cons"], s2["cons"])
    assert np.array_equal(s["Phi"], s2["Phi"])
    for q in range(s["prim"].shape[0]):
        assert rel_l1(s2["prim"][q, real], s["prim"][q, real]) < 1e-12, q
    for _ in range(3):
        d1.timestep(d1.getmindt())
        d2.timestep(d2.getmindt())
    a, b = d1.state(), d2.state()
    h = d1.host
    r = cell_radius(h.Np, h.r_jph, h.Nr, h.Nz)[real]
    for k, e in grouped_rel_l1(b["cons"][:, real], a["cons"][:, real], r, 8).items():
        assert e < 1e-9, (k, e)
    d1.close(); d2.close()
