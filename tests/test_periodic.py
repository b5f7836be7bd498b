"""Periodic r / z ghosts (R_Periodic, Z_Periodic) on the host set-up and the
oracle restatement.  The reference fills them only through exchangeData on
an MPI cartesian communicator with wrap-around (exchange.c:173-279); its
serial build never refreshes them, so these cases are pinned to the
restatement of that exchange, not to a reference run."""
import numpy as np
import pytest

from helpers import ROOT

CASES = {
    "z": ("configs/cfg1_vortex", {"Num_R": 24, "Num_Z": 4, "Z_Periodic": 1}),
    "rz": ("configs/cfg1_vortex", {"Num_R": 24, "Num_Z": 4, "R_Periodic": 1, "Z_Periodic": 1}),
    "z_zerograd": ("configs/cfg1_vortex_zerograd", {"Num_R": 16, "Num_Z": 4, "Z_Periodic": 1}),
    "z_mhd": ("configs/cfg2_mhd_disk", {"Num_R": 12, "Num_Z": 6, "Z_Periodic": 1}),
}


def host(name):
    import os
    import disco_gb300 as dg
    cfg, over = CASES[name]
    p = dg.read_params(os.path.join(ROOT, cfg, "in.par"))
    for k, v in over.items():
        setattr(p, k, v)
    return dg.HostDomain(p, dg.read_modules(os.path.join(ROOT, cfg, "Makefile_opt.in")))


def ghost_pairs(h, name):
    """(ghost ring, source ring) of every periodic dimension, r then z."""
    over = CASES[name][1]
    Nr, Nz, out = h.Nr, h.Nz, []
    if over.get("R_Periodic") and Nr > 1:
        n = Nr - h.NgRa - h.NgRb
        for k in range(Nz):
            out += [(j + Nr * k, j + n + Nr * k) for j in range(h.NgRa)]
            out += [(j + Nr * k, j - n + Nr * k) for j in range(Nr - h.NgRb, Nr)]
    if over.get("Z_Periodic") and Nz > 1:
        n = Nz - h.NgZa - h.NgZb
        for j in range(Nr):
            out += [(j + Nr * k, j + Nr * (k + n)) for k in range(h.NgZa)]
            out += [(j + Nr * k, j + Nr * (k - n)) for k in range(Nz - h.NgZb, Nz)]
    return out


def ring(a, off, jk):
    return a[..., off[jk]:off[jk + 1]]


@pytest.mark.parametrize("name", list(CASES))
def test_host_ghost_rings_take_their_sources(name):
    """Set-up: a periodic ghost ring has its source ring's Np, positions and
    initial primitives (the first exchange, main.c:53-61)."""
    h = host(name)
    off = np.concatenate([[0], np.cumsum(h.Np)])
    pairs = ghost_pairs(h, name)
    assert pairs
    for g, s in pairs:
        assert h.Np[g] == h.Np[s]
        assert np.array_equal(ring(h.piph, off, g), ring(h.piph, off, s))
        assert np.array_equal(ring(h.prim, off, g), ring(h.prim, off, s))


@pytest.mark.parametrize("name", list(CASES))
def test_restatement_ghosts_equal_sources_after_steps(name):
    """The restatement after five steps: every periodic ghost ring holds its
    source ring's cells exactly, and the state stays finite."""
    from oracle.port import PortDomain
    h = host(name)
    o = PortDomain(h)
    o.run(5)
    s = o.state()
    off = np.concatenate([[0], np.cumsum(h.Np)])
    assert np.isfinite(s["cons"]).all()
    for g, src in ghost_pairs(h, name):
        for k in ("cons", "prim", "piph", "dphi"):
            assert np.array_equal(ring(s[k], off, g), ring(s[k], off, src)), (g, src, k)
