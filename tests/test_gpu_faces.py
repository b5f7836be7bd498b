"""Integer face tables, PLM gradients, face fluxes of B and div B on the
device against the reference's fixtures (tests/golden, made by the
unmodified reference build) and the CPU oracle.

Bars: on the plain FP64 path the face tables (fIndex, L, R, LRtype, and the
FP64 centroid phi and area) equal the reference bit for bit; the mixed path
keeps the integer tables bit-exact too.  Gradients of the initial state and
the face fluxes Phi after the steps are within 1e-12 relative L1 (FP64).
Constrained transport keeps the divergence of every cell's face fluxes at
its initial value to roundoff away from the inner radial boundary (FP64
roundoff on the plain path, the FP32 rounding of the edge EMFs on the mixed
path), and next to that boundary the device reproduces the reference's own
change."""
import numpy as np
import pytest

from helpers import divb_from_faces, load_golden, rel_l1
from test_gpu_parity import CASES, FP64_ONLY, _domain

pytestmark = pytest.mark.gpu

INT_KEYS = ("fIndex", "L", "R", "LRtype")
CT_CASES = [n for n in CASES if n.startswith(("cfg2", "cfg5"))]
# cases whose oracle restatement exists (Newtonian hydro and MHD)
PORT_CASES = [n for n in CASES if n not in FP64_ONLY]


def _fixture_faces(g, key):
    return {k: g[f"faces_{key}_{k}"] for k in (*INT_KEYS, "phic", "dA")}


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", list(CASES))
def test_face_tables_match_reference(name, precision):
    """The device's sheared faces of the initial state (k_anchor + the merge
    path of k_faces) against the reference's setup_faces output."""
    if precision and name in FP64_ONLY:
        pytest.skip("FP64-only module")
    d, g = _domain(name, precision)
    for key, dim in (("r", 1), ("z", 2)):
        if f"faces_{key}_L" not in g:
            assert len(d.faces(dim)["L"]) == 0
            continue
        ref = _fixture_faces(g, key)
        dev = d.faces(dim)
        for k in INT_KEYS:
            assert np.array_equal(dev[k], ref[k]), (key, k)
        if precision == 0:
            assert np.array_equal(dev["phic"], ref["phic"]), key
            assert np.array_equal(dev["dA"], ref["dA"]), key
        else:
            # the mixed path forms the face from FP32 offsets of FP64 positions
            dp = np.abs((dev["phic"] - ref["phic"] + np.pi) % (2 * np.pi) - np.pi)
            assert dp.max() < 1e-6, key
            assert rel_l1(dev["dA"], ref["dA"]) < 1e-6, key
    d.close()


@pytest.mark.parametrize("name", PORT_CASES)
def test_face_tables_after_steps_match_oracle(name):
    """After the fixture's steps (cells moved, faces rebuilt every step) the
    device's face tables equal the oracle's, built from its own positions
    (the oracle equals the reference bit for bit)."""
    import disco_gb300 as dg
    from oracle.port import PortDomain
    d, g = _domain(name)
    n = int(g["nsteps"])
    d.run(n)
    h = dg.HostDomain(d.params, d.modules)
    o = PortDomain(h)
    o.run(n)
    for key, dim in (("r", 1), ("z", 2)):
        dev, ref = d.faces(dim), o.faces(dim)
        for k in INT_KEYS:
            assert np.array_equal(dev[k], ref[k]), (key, k)
        # positions can differ from the oracle's in the last bits where FP64
        # transcendentals (the planet disk's gravity and alpha scale height,
        # the exact mesh rotation) differ from glibc's -- within 1e-12 of a
        # turn, the bar of the position check.  Each of a face's two phi
        # edges may move by that angle, which changes its area by at most
        # the angle times the face's extent across phi (r dz for an r face,
        # r dr for a z face): the area bar, for the largest extent
        if len(ref["dA"]) == 0:   # a 2D domain has no z faces
            continue
        atol_phi = 1e-12 * 2 * np.pi
        assert np.allclose(dev["phic"], ref["phic"], rtol=0, atol=atol_phi), key
        rj, zk = np.asarray(h.r_jph, dtype=float), np.asarray(h.z_kph, dtype=float)
        ext = np.abs(rj).max() * max(np.diff(rj).max(initial=0.0), np.diff(zk).max(initial=0.0))
        assert np.max(np.abs(dev["dA"] - ref["dA"])) <= 2 * atol_phi * ext, key
    d.close()


@pytest.mark.parametrize("name", list(CASES))
def test_gradients_match_reference(name):
    """plm_phi and plm_trans of the initial state (plm.c:6-232) against the
    reference's gradients (the fixture's grad_* arrays), FP64 path."""
    d, g = _domain(name)
    gr = d.gradients()
    real = g["real"].astype(bool)
    keys = ("gradp", "gradr", "gradz")
    for q in range(g["grad_gradp"].shape[0]):
        # a gradient that vanishes analytically (the z-gradient of a
        # z-uniform passive scalar) holds rounding noise of order 1e-163 in
        # the reference: each is judged against the component's gradients
        # in all three directions together
        scale = sum(np.abs(g[f"grad_{k}"][q, real]).sum() for k in keys)
        for k in keys:
            ref = g[f"grad_{k}"]
            num = np.abs(gr[k][q, real] - ref[q, real]).sum()
            assert num <= 1e-12 * scale, (k, q, num, scale)
    d.close()


@pytest.mark.parametrize("name", CT_CASES)
def test_face_fluxes_match_reference(name):
    """The face fluxes of B (Phi[5] per cell, bfields.c) initially and after
    the steps, against the reference's, FP64 path."""
    d, g = _domain(name)
    real = g["real"].astype(bool)
    s0 = d.state()
    for q in range(5):
        assert rel_l1(s0["Phi"][q, real], g["init_Phi"][q, real]) < 1e-14, q
    for _ in range(int(g["nsteps"])):
        d.timestep(d.getmindt())
    s = d.state()
    for q in range(5):
        ref = g["run_Phi"][q, real]
        if np.abs(ref).sum() == 0:
            assert np.abs(s["Phi"][q, real]).sum() == 0, q
        else:
            assert rel_l1(s["Phi"][q, real], ref) < 1e-12, q
    d.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", CT_CASES)
def test_divb_stays_at_roundoff(name, precision):
    """div B as the net face flux of each cell.  The device kernel agrees
    with the same sum formed on the host from the device's Phi and face
    tables.  After the steps, every real cell's divergence differs from its
    initial value by roundoff (relative to the flux through the cell),
    except next to the inner radial boundary: there the reference's own
    scheme changes div B (by up to 1e-4 of the cell's flux after five
    steps, spreading one ring inward per step), and the device reproduces
    the oracle's per-cell change there (the oracle equals the reference bit
    for bit)."""
    import disco_gb300 as dg
    from oracle.port import PortDomain
    if precision and name in FP64_ONLY:
        pytest.skip("FP64 path only")
    d, g = _domain(name, precision)
    h = d.host
    real = g["real"].astype(bool)
    n = int(g["nsteps"])
    div0, sc0 = d.divb()
    for _ in range(n):
        d.timestep(d.getmindt())
    div1, sc1 = d.divb()
    s = d.state()
    faces = {"r": d.faces(1), "z": d.faces(2)}
    host = divb_from_faces(s["Phi"], h.Np, faces)
    ev = real & (sc1 > 0) & (sc0 > 0)
    assert ev.sum() > 0.5 * real.sum()
    assert np.max(np.abs(host[ev] - div1[ev]) / sc1[ev]) < 1e-14
    change = (div1 - div0)[ev] / sc1[ev]
    # the oracle's change per cell, from its own Phi and faces
    o = PortDomain(dg.HostDomain(d.params, d.modules))
    so = o.state()
    fo = {"r": o.faces(1), "z": o.faces(2)}
    od0 = divb_from_faces(so["Phi"], h.Np, fo)
    o.run(n)
    so = o.state()
    fo = {"r": o.faces(1), "z": o.faces(2)}
    od1 = divb_from_faces(so["Phi"], h.Np, fo)
    ochange = (od1 - od0)[ev] / sc1[ev]
    tol = 1e-12 if precision == 0 else 1e-6
    assert np.max(np.abs(change - ochange)) < tol
    jk = np.repeat(np.arange(h.Nr * h.Nz), h.Np)
    away = (jk % h.Nr >= h.NgRa + 3)[ev]
    # the mixed path adds FP32 edge EMFs (times dl dt) to FP64 face fluxes:
    # its divergence is held to FP32 rounding of those increments
    assert np.abs(change[away]).max() < (1e-13 if precision == 0 else 1e-7), np.abs(change[away]).max()
    d.close()
