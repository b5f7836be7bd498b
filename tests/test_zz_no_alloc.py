"""disco_gpu_getmindt_noalloc (include/disco_gpu_noalloc.h) against the
existing entry point disco_gpu_getmindt: the same dt, bit for bit, on two
calls in a row (the static scratch carries nothing from one call to the
next), for both precisions and both hydro modules.  Named to be collected
last, so it also runs after every other GPU test has used the device."""
import os
import struct

import pytest

from helpers import ROOT, load_golden, write_par

pytestmark = pytest.mark.gpu

CASES = {"cfg1_n24": "configs/cfg1_vortex", "cfg2_n12": "configs/cfg2_mhd_disk"}


def _bits(x: float) -> bytes:
    return struct.pack("<d", x)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", list(CASES))
def test_noalloc_dt_equals_getmindt(name, precision):
    import disco_gb300 as dg
    g = load_golden(name)
    d = dg.Domain(write_par(g["par_text"]), os.path.join(ROOT, CASES[name], "Makefile_opt.in"),
                  precision=precision)
    try:
        for _ in range(2):
            a1 = d.getmindt_noalloc()
            a2 = d.getmindt_noalloc()
            ref = d.getmindt()
            assert a1 > 0.0
            assert _bits(a1) == _bits(ref) and _bits(a2) == _bits(ref), (a1, a2, ref)
            d.timestep(ref)
    finally:
        d.close()


def test_noalloc_leaves_the_instance_unchanged():
    """The no-allocation call writes nothing into the instance: a step after
    it is identical to a step without it."""
    import numpy as np
    import disco_gb300 as dg
    g = load_golden("cfg1_n24")
    mk = os.path.join(ROOT, CASES["cfg1_n24"], "Makefile_opt.in")
    par = write_par(g["par_text"])
    d1 = dg.Domain(par, mk, precision=0)
    d2 = dg.Domain(par, mk, precision=0)
    try:
        dt = d1.getmindt()
        d2.getmindt_noalloc()
        assert _bits(d2.getmindt()) == _bits(dt)
        d1.timestep(dt)
        d2.timestep(dt)
        s1, s2 = d1.state(), d2.state()
        for k in ("cons", "prim", "piph", "dphi"):
            assert np.array_equal(s1[k], s2[k]), k
    finally:
        d1.close()
        d2.close()
