"""Batched instances (include/disco_gpu_batch.h): a batch step is one graph
launch whose branches are the members' own steps, so every member must end
exactly where it ends when run on its own."""
import os

import numpy as np
import pytest

from helpers import ROOT, load_golden, rel_l1, write_par

pytestmark = pytest.mark.gpu

MEMBERS = [("cfg1_n24", 0), ("cfg3_n24", 0), ("cfg3_n24", 1), ("cfg2_n12", 0), ("cfg1_hll_static", 1)]


def _make(name, precision):
    import disco_gb300 as dg
    g = load_golden(name)
    return dg.Domain(write_par(g["par_text"]), os.path.join(ROOT, str(g["cfg"]), "Makefile_opt.in"),
                     precision=precision)


def test_batch_equals_members_run_alone():
    import disco_gb300 as dg
    solo = [_make(n, p) for n, p in MEMBERS]
    batch_members = [_make(n, p) for n, p in MEMBERS]
    nsteps = 5
    for d in solo:
        d.run(nsteps)
    b = dg.Batch(batch_members)
    b.run(2)
    b.run(nsteps - 2)          # odd then even parity: both captured graphs used
    for (name, prec), d1, d2 in zip(MEMBERS, solo, batch_members):
        s1, s2 = d1.state(), d2.state()
        if name.startswith("cfg2"):   # edge-EMF FP64 atomics: equal to rounding
            real = d1.host.real_mask()
            assert abs(s1["t"] - s2["t"]) <= 1e-13 * abs(s1["t"]), name
            assert np.max(np.abs(s1["piph"] - s2["piph"])) < 1e-12, name
            for q in range(s1["cons"].shape[0]):
                assert rel_l1(s1["cons"][q, real], s2["cons"][q, real]) < 1e-13, (name, q)
        else:
            assert s1["t"] == s2["t"], name
            assert np.array_equal(s1["piph"], s2["piph"]), name
            assert np.array_equal(s1["cons"], s2["cons"]), (name, prec)
        st = d2.status()
        assert st["nan_cells"] == 0 and st["face_errors"] == 0 and st["steps"] == nsteps
    # members stay usable on their own after the batch
    batch_members[0].timestep(batch_members[0].getmindt())
    b.close()
    for d in solo + batch_members:
        d.close()


def test_batch_rejects_members_at_different_parity():
    import disco_gb300 as dg
    a, c = _make("cfg1_n24", 0), _make("cfg1_n24", 0)
    a.run(1)
    with pytest.raises(dg.DiscoError):
        dg.Batch([a, c])
    a.close()
    c.close()


def test_later_smaller_instance_keeps_larger_one_steppable():
    """Kernel shared-memory limits are per function: creating a smaller
    instance after a larger one must not break the larger one's launches
    (both face merges here need more than the default 48 KB)."""
    import disco_gb300 as dg
    cfg = os.path.join(ROOT, "configs", "cfg1_vortex")
    par, mk = os.path.join(cfg, "in.par"), os.path.join(cfg, "Makefile_opt.in")
    big = dg.Domain(par, mk, precision=0, overrides={"Num_R": 400})
    mid = dg.Domain(par, mk, precision=0, overrides={"Num_R": 300})
    big.timestep(big.getmindt())
    mid.timestep(mid.getmindt())
    assert big.status()["face_errors"] == 0 and mid.status()["face_errors"] == 0
    big.close()
    mid.close()
