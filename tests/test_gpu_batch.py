"""Batched instances (include/disco_gpu_batch.h): a batch step is one graph
launch whose branches are the members' own steps, so every member must end
exactly where it ends when run on its own."""
import os

import numpy as np
import pytest

from helpers import ROOT, cell_radius, grouped_rel_l1, load_golden, rel_l1, write_par

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


# (golden case, precision, Num_R): the groups that form are the FP64 and
# mixed planet disks (RK2), the mixed planet disks (RK3), the FP64 disks with
# cooling and damping, the FP64 vortices (moving and static mesh, HLLC and
# HLL in one group), and the GRMHD members (two thin disks and the Kerr
# torus: one module, one launch sequence); the mixed vortex (staged phi
# sweep) and the outflow disk (boundary plugin) run their own launch
# sequences
GROUPED = [("cfg3_n24", 0, 24), ("cfg3_n24", 0, 40), ("cfg3_n24", 1, 24), ("cfg3_n24", 1, 40),
           ("cfg3_rk3", 1, 24), ("cfg3_rk3", 1, 32), ("cfg3_cooldamp", 0, 24), ("cfg3_cooldamp", 0, 28),
           ("cfg1_n24", 0, 24), ("cfg1_hll_static", 0, 32), ("cfg4_diag", 0, 12), ("cfg4_diag", 0, 16),
           ("cfg1_n24", 1, 24), ("cfg3_outflow", 0, 24), ("cfg4t_n24", 0, 24)]
N_GROUPS, N_GROUPED = 6, 13


def _make_nr(name, precision, nr):
    import disco_gb300 as dg
    g = load_golden(name)
    return dg.Domain(write_par(g["par_text"]), os.path.join(ROOT, str(g["cfg"]), "Makefile_opt.in"),
                     precision=precision, overrides={"Num_R": nr})


def _same(d1, d2, tag):
    """FP64 members: bit for bit.  Mixed members: the FP32 units are built
    with multiply-add contraction on, and the compiler may contract a body
    differently inside a multi-instance kernel than inside its own kernel,
    so they agree to FP32 rounding: within 1e-9 relative L1 per physical
    quantity (vectors through their norm), positions within 1e-9 of a turn,
    time exactly.  An isothermal run's energy is the exception: its
    pressure comes from the sound-speed profile, so the energy never feeds
    back, and FP32 rounding differences in its own flux accumulate there
    undamped (1.4e-7 after 13 steps of the planet disk, with mass,
    momentum and passive scalar exactly equal); it is held to the mixed
    path's 1e-6."""
    s1, s2 = d1.state(), d2.state()
    assert s1["t"] == s2["t"], tag
    if tag[1] == 0:
        assert np.array_equal(s1["piph"], s2["piph"]), tag
        for k in ("cons", "prim"):
            assert np.array_equal(s1[k], s2[k]), (tag, k)
        q1, q2 = d1.diagnostics(), d2.diagnostics()
        assert np.array_equal(q1["Qrz"], q2["Qrz"]), tag
    else:
        h = d1.host
        real = h.real_mask()
        r = cell_radius(h.Np, h.r_jph, h.Nr, h.Nz)[real]
        e = grouped_rel_l1(s2["cons"][:, real], s1["cons"][:, real], r, 8 if h.num_q >= 8 else 5)
        print(tag, "relative L1 per quantity", e)
        iso = bool(d1.params.isothermal_flag)
        for k, v in e.items():
            assert v < (1e-6 if (iso and k == "energy") else 1e-9), (tag, k, e)
        dp = np.abs((s1["piph"] - s2["piph"] + np.pi) % (2 * np.pi) - np.pi)
        assert dp.max() < 1e-9 * 2 * np.pi, tag
    st = d2.status()
    assert st["nan_cells"] == 0 and st["face_errors"] == 0, tag


@pytest.mark.parametrize("split", [1, 4, -1])
def test_grouped_members_equal_members_run_alone(split):
    """Members advanced by the multi-instance stage kernels end where they
    end alone (bit for bit on the FP64 path), in one sub-group per group, in
    four, and under the split autotuner (twelve timed steps of the
    candidates, then the choice), with the grid capped at 3 blocks per SM."""
    import disco_gb300 as dg
    nsteps = 13
    solo = [_make_nr(*m) for m in GROUPED]
    for d in solo:
        d.run(nsteps)
    mem = [_make_nr(*m) for m in GROUPED]
    nb = dg.Batch(mem, groups=False)
    assert nb.info()["groups"] == 0
    nb.close()
    b = dg.Batch(mem)
    info = b.info()
    assert info["groups"] == N_GROUPS and info["grouped_members"] == N_GROUPED, info
    b.set_grid(3)
    b.set_split(split)
    b.run(4)
    b.run(nsteps - 4)
    info = b.info()
    print(info)
    if split >= 0:
        assert info["split"] == split
    else:
        assert info["split"] in (0, 1, 2, 4, 8, 16)
        assert all(v > 0 for v in info["tune_ms"].values()), info
    for m, d1, d2 in zip(GROUPED, solo, mem):
        _same(d1, d2, m)
        assert d2.status()["steps"] == nsteps
    # the per-stage profile steps the members too: still where alone ends
    prof = b.profile(2)
    assert {"update", "flux_r", "mindt"} <= {p[0] for p in prof}, prof
    for d in solo:
        d.run(2)
    for m, d1, d2 in zip(GROUPED, solo, mem):
        _same(d1, d2, m)
    b.close()
    for d in solo + mem:
        d.close()
