"""Periodic r / z ghosts on the device (k_periodic_copy) against the
oracle's restatement of the one-rank wrap-around exchange (exchange.c:
173-279; the serial reference never refreshes periodic ghosts, so there is
no reference run to pin them to): the FP64 path within 1e-12 per physical
quantity with bit-exact face tables, the mixed path within 1e-6; and every
periodic ghost ring holds exactly its source ring's cells."""
import os

import numpy as np
import pytest

from helpers import ROOT, cell_radius, grouped_rel_l1
from test_periodic import CASES, ghost_pairs, ring

pytestmark = pytest.mark.gpu


def _pair(name, precision):
    import disco_gb300 as dg
    from oracle.port import PortDomain
    cfg, over = CASES[name]
    par, mk = os.path.join(ROOT, cfg, "in.par"), os.path.join(ROOT, cfg, "Makefile_opt.in")
    d = dg.Domain(par, mk, precision=precision, overrides=over)
    o = PortDomain(d.host)
    return d, o


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", list(CASES))
def test_periodic_ghosts_match_restatement(name, precision):
    d, o = _pair(name, precision)
    n = 6
    for _ in range(n):
        if precision == 0:   # the device's own dt
            d.timestep(d.getmindt())
            o.step()
        else:                # the mixed path takes the restatement's dt: one clock
            d.timestep(o.step())
    s, so = d.state(), o.state()
    h = d.host
    real = h.real_mask()
    r = cell_radius(h.Np, h.r_jph, h.Nr, h.Nz)[real]
    num_c = 8 if h.num_q >= 8 else 5
    bar = 1e-12 if precision == 0 else 1e-6
    assert abs(s["t"] - so["t"]) <= 1e-12 * so["t"]
    for k, e in grouped_rel_l1(s["cons"][:, real], so["cons"][:, real], r, num_c).items():
        assert e < bar, (k, e)
    if precision == 0:
        assert np.max(np.abs(s["piph"] - so["piph"])) < 1e-12 * 2 * np.pi
        for dim in (1, 2):
            fd, fo = d.faces(dim), o.faces(dim)
            for k in ("fIndex", "L", "R", "LRtype"):
                assert np.array_equal(fd[k], fo[k]), (dim, k)
    off = np.concatenate([[0], np.cumsum(h.Np)])
    for g, src in ghost_pairs(h, name):
        for k in ("cons", "prim", "piph"):
            assert np.array_equal(ring(s[k], off, g), ring(s[k], off, src)), (g, src, k)
    st = d.status()
    assert st["nan_cells"] == 0 and st["face_errors"] == 0
    d.close()
