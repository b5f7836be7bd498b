"""Host C set-up (grid, ring phases, initial state, in.par reader) against
the reference's own output -- no GPU needed."""
import ctypes
import ctypes.util
import os

import numpy as np
import pytest

from helpers import ROOT, load_golden, write_par


def _dg():
    import disco_gb300 as dg
    return dg


def test_grid_and_phases_bit_exact():
    dg = _dg()
    g = load_golden("cfg1_n24")
    p = dg.read_params(write_par(g["par_text"]))
    m = dg.read_modules(os.path.join(ROOT, "configs/cfg1_vortex/Makefile_opt.in"))
    h = dg.HostDomain(p, m)
    assert np.array_equal(h.Np, g["Np"])
    assert np.array_equal(h.r_jph, g["r_jph"])
    assert np.array_equal(h.z_kph, g["z_kph"])
    assert np.array_equal(h.piph, g["init_piph"])
    assert np.array_equal(h.dphi, g["init_dphi"])
    real = g["real"].astype(bool)
    assert np.array_equal(h.real_mask(), real)
    # initial() prims vs the reference's prims after its prim2cons/cons2prim
    assert np.max(np.abs(h.prim[:, real] - g["init_prim"][:, real])) < 1e-14


def test_grmhd_disk_initial_state_bit_exact():
    """GRMHD disk (Kerr-Schild metric module, gr_disk initial condition):
    grid and phases equal the reference build's, initial primitives to
    rounding."""
    dg = _dg()
    g = load_golden("cfg4_n12")
    p = dg.read_params(write_par(g["par_text"]))
    m = dg.read_modules(os.path.join(ROOT, "configs/cfg4_grmhd_disk/Makefile_opt.in"))
    assert (m.hydro, m.metric, m.frame, m.ct_mode) == (2, 0, 0, 0)
    h = dg.HostDomain(p, m)
    assert np.array_equal(h.Np, g["Np"])
    assert np.array_equal(h.piph, g["init_piph"])
    real = g["real"].astype(bool)
    # initial() prims vs the reference's prims after its prim2cons and the
    # Newton cons2prim seeded with them
    assert np.max(np.abs(h.prim[:, real] - g["init_prim"][:, real])) < 1e-14


@pytest.mark.parametrize("name", ["cfg4t_body", "cfg4t_n24"])
def test_grmhd_torus_initial_state(name):
    """Fishbone-Moncrief torus on the Kerr metric (kerr_ks_rpz, fm_torus):
    grid and phases equal the reference build's, and so do the initial
    primitives with the 4 % pressure noise drawn from the same rand()
    stream, to the rounding of the reference's prim2cons / Newton
    cons2prim round trip."""
    dg = _dg()
    g = load_golden(name)
    p = dg.read_params(write_par(g["par_text"]))
    m = dg.read_modules(os.path.join(ROOT, "configs/cfg4_grmhd_torus/Makefile_opt.in"))
    assert (m.hydro, m.metric, m.initial) == (2, 1, 5)
    h = dg.HostDomain(p, m)
    assert np.array_equal(h.Np, g["Np"])
    assert np.array_equal(h.piph, g["init_piph"])
    real = g["real"].astype(bool)
    # the reference's initial primitives are those of its prim2cons + Newton
    # cons2prim round trip, which floors the torus-edge cells whose initial
    # density is below Density_Floor; those are compared on the device
    floor = float(p.Density_Floor)
    ok = real & (g["init_prim"][0] > 10 * floor) & (h.prim[0] > 10 * floor)
    assert ok.sum() > 0.3 * real.sum()
    for q in range(h.prim.shape[0]):
        ref = g["init_prim"][q, ok]
        scale = np.abs(ref).max()
        assert np.max(np.abs(h.prim[q, ok] - ref)) <= 1e-12 * max(scale, 1e-300), q


def test_grmhd_unbuilt_metric_rejected(tmp_path):
    """A metric other than schw_ks_rpz / kerr_ks_rpz is refused at module
    selection."""
    dg = _dg()
    src = open(os.path.join(ROOT, "configs/cfg4_grmhd_disk/Makefile_opt.in")).read()
    mk = tmp_path / "Makefile_opt.in"
    mk.write_text(src.replace("schw_ks_rpz", "schw_sc_rpz"))
    with pytest.raises(dg.DiscoError):
        dg.read_modules(str(mk))


def test_rand_restatement_matches_libc():
    """The restated glibc rand() stream equals the C library's (where the
    host C library is glibc)."""
    dg = _dg()
    libc_path = ctypes.util.find_library("c")
    libc = ctypes.CDLL(libc_path)
    try:
        libc.gnu_get_libc_version
    except AttributeError:
        pytest.skip("host C library is not glibc")
    n = 5000
    out = (ctypes.c_int * n)()
    L = dg.lib()
    L.disco_rand_sequence.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.disco_rand_sequence(314159, n, out)
    libc.srand(314159)
    ref = [libc.rand() for _ in range(n)]
    assert list(out) == ref


def test_cell_count_full_vortex_config():
    """72,398 interior cells for the 2D vortex configuration (Np from the
    outer-edge radius, gridsetup.c:132-139)."""
    dg = _dg()
    p = dg.read_params(os.path.join(ROOT, "configs/cfg1_vortex/in.par"))
    m = dg.read_modules(os.path.join(ROOT, "configs/cfg1_vortex/Makefile_opt.in"))
    h = dg.HostDomain(p, m)
    assert int(h.Np[h.NgRa:h.Nr - h.NgRb].sum()) == 72398
    assert h.Np[h.NgRa:h.Nr - h.NgRb].min() == 167 and h.Np[h.NgRa:h.Nr - h.NgRb].max() == 965


def test_readvar_semantics(tmp_path):
    """readpar.c:6-42: first matching line wins, value after any of
    '\\t :=>_', absent keys read as 0 and are counted, x2pi scalings."""
    dg = _dg()
    f = tmp_path / "in.par"
    f.write_text("//comment\nNum_R = 12\nNum_R 99\naspect =>_ 2.5\naspect_x 7\nPhi_Max 1.0\n"
                 "P_Times_2pi 1\nT_End 3\nT_Times_2pi 1\nR_Min\t0.25 // trailing\n")
    p = dg.read_params(str(f))
    assert p.Num_R == 12
    assert p.aspect == 2.5
    assert p.phimax == 2.0 * np.pi
    assert p.t_max == 6.0 * np.pi
    assert p.rmin == 0.25
    assert p.Num_Z == 0 and p.read_errors > 50


def test_missing_files_and_modules_fail_loudly(tmp_path):
    dg = _dg()
    with pytest.raises(dg.DiscoError):
        dg.read_params(str(tmp_path / "nope.par"))
    mk = tmp_path / "Makefile_opt.in"
    mk.write_text("INITIAL = vortex_gauss\nHYDRO = grmhd2\nGEOMETRY = cylindrical\n"
                  "BOUNDARY = fixed\nPLANETS = none\nNUM_C = 5\nNUM_N = 1\nCT_MODE = 0\n")
    with pytest.raises(dg.DiscoError, match="HYDRO=grmhd2"):
        dg.read_modules(str(mk))


BOUNDARY_PLUGINS = ["fixed", "fixed3d", "outflow3d", "zerograd", "zerograd_omk", "zerograd_omIN",
                    "accrete3d", "fixRrefZ", "polar3d", "fixed_gap", "tube", "surfaceGravBox",
                    "flowthrough", "polar", "horizon3d", "horizon", "horizon_bin"]
ANALYSIS_PLUGINS = ["diag_euler", "diag_disk2d", "diag_cb", "diag_bl", "diag_mhdmri", "diag_grmhdmri"]


def _mk(tmp_path, **kw):
    keys = {"INITIAL": "vortex_gauss", "HYDRO": "euler", "GEOMETRY": "cylindrical", "BOUNDARY": "fixed",
            "PLANETS": "none", "ANALYSIS": "diag_euler", "NUM_C": 5, "NUM_N": 1, "CT_MODE": 0}
    keys.update(kw)
    p = tmp_path / "Makefile_opt.in"
    p.write_text("".join(f"{k} = {v}\n" for k, v in keys.items() if v is not None))
    return str(p)


def test_boundary_and_analysis_plugins_select(tmp_path):
    """Every built BOUNDARY and ANALYSIS plugin name maps to its id, in the
    order of disco_boundary_id / disco_analysis_id; a missing ANALYSIS key
    selects none (the reference build requires one: no accumulators)."""
    dg = _dg()
    for i, b in enumerate(BOUNDARY_PLUGINS):
        m = dg.read_modules(_mk(tmp_path, BOUNDARY=b))
        assert m.boundary == i and m.boundary_name.decode() == b
    for i, a in enumerate(ANALYSIS_PLUGINS):
        m = dg.read_modules(_mk(tmp_path, ANALYSIS=a))
        assert m.analysis == i and m.analysis_name.decode() == a
    assert dg.read_modules(_mk(tmp_path, ANALYSIS=None)).analysis == -1


@pytest.mark.parametrize("key,name", [("BOUNDARY", "wedge"), ("BOUNDARY", "inflow"),
                                      ("ANALYSIS", "diag_nonexistent")])
def test_unbuilt_plugins_fail_loudly(tmp_path, key, name):
    dg = _dg()
    with pytest.raises(dg.DiscoError, match=f"{key}={name} not built"):
        dg.read_modules(_mk(tmp_path, **{key: name}))


@pytest.mark.parametrize("plugin", ["polar", "horizon", "horizon_bin"])
def test_frame_free_plugins_with_rotating_frame_rejected(tmp_path, plugin):
    """Boundary/polar.c and horizon.c fill cells without subtract_omega; with
    RotFrame that differs from the built fill, so the set-up refuses it."""
    dg = _dg()
    p = dg.read_params(os.path.join(ROOT, "configs/cfg1_vortex/in.par"))
    m = dg.read_modules(_mk(tmp_path, BOUNDARY=plugin))
    dg.HostDomain(p, m)   # without RotFrame: built
    p.RotFrame = 1
    with pytest.raises(dg.DiscoError, match=f"{plugin} with RotFrame"):
        dg.HostDomain(p, m)


def test_cooling_damping_keys_read(tmp_path):
    """Cool_* and Damp*_* keys (readpar.c:155-174) land in disco_params."""
    dg = _dg()
    src = open(os.path.join(ROOT, "configs/cfg3_planet_disk/in.par")).read()
    import re
    src = re.sub(r"(?m)^Timestep\s.*$", "Timestep 3", src)   # readvar takes a key's first line
    extra = ("\nCool_Type 2\nCool_Par1 0.5\nDampInner_Type 2\nDampInner_Time 1.0\nDampInner_Len 0.3\n"
             "DampOuter_Type 1\nDampOuter_Time 2.0\nDampOuter_Len 0.5\n")
    p = dg.read_params(write_par(src + extra))
    assert (p.coolType, p.coolPar1) == (2, 0.5)
    assert (p.dampInnerType, p.dampTimeInner, p.dampLenInner) == (2, 1.0, 0.3)
    assert (p.dampOuterType, p.dampTimeOuter, p.dampLenOuter) == (1, 2.0, 0.5)
    assert p.Timestep == 3
