"""Checkpoint file and restart (disco_host_checkpoint / disco_host_restart)
against the reference's layout: Output/h5out.c output() (:366-620) with
writeOpts (:98-166) and writePars (:168-364), and Restart/h5in.c restart()
(:100-354) with setupCells' restart branch (domain.c:139-238).

No HDF5 library exists on either machine, so the files are read by two
independent readers of the specification: the library's own (restart) and
tests/h5spec.py, which verifies every checksum and structural field."""
import ctypes as C
import os

import numpy as np
import pytest

import h5spec
from helpers import ROOT

CFGS = {"euler": "configs/cfg1_vortex", "mhd": "configs/cfg2_mhd_disk",
        "planets": "configs/cfg3_planet_disk"}
SMALL = {"euler": {}, "mhd": {"Num_R": 12, "Num_Z": 6}, "planets": {"Num_R": 24}}


def _pm(name, **over):
    import disco_gb300.api as api
    cfg = os.path.join(ROOT, CFGS[name])
    p = api.read_params(os.path.join(cfg, "in.par"))
    m = api.read_modules(os.path.join(cfg, "Makefile_opt.in"))
    for k, v in {**SMALL[name], **over}.items():
        setattr(p, k, v)
    return p, m


def _host(name, **over):
    import disco_gb300.api as api
    p, m = _pm(name, **over)
    return api.HostDomain(p, m), p, m


def test_lookup3_published_vectors():
    """The checker's checksum against the values published with lookup3.c."""
    assert h5spec.lookup3(b"") == 0xDEADBEEF
    assert h5spec.lookup3(b"", 0xDEADBEEF) == 0xBD5B7DDE
    assert h5spec.lookup3(b"Four score and seven years ago") == 0x17770551
    assert h5spec.lookup3(b"Four score and seven years ago", 1) == 0xCD628161


# writePars' datasets: (name, DiscoParams field, is_int), h5out.c:168-364
PARS = [("Num_R", "Num_R", 1), ("Num_Z", "Num_Z", 1), ("aspect", "aspect", 0),
        ("Num_Reports", "NumRepts", 1), ("Num_Snapshots", "NumSnaps", 1),
        ("Num_Checkpoints", "NumChecks", 1), ("T_Start", "t_min", 0), ("T_End", "t_max", 0),
        ("R_Min", "rmin", 0), ("R_Max", "rmax", 0), ("Z_Min", "zmin", 0), ("Z_Max", "zmax", 0),
        ("Phi_Max", "phimax", 0), ("Use_Logtime", "Out_LogTime", 1), ("Log_Zoning", "LogZoning", 1),
        ("R_Periodic", "R_Periodic", 1), ("Z_Periodic", "Z_Periodic", 1),
        ("NoBC_Rmin", "NoBC_Rmin", 1), ("NoBC_Rmax", "NoBC_Rmax", 1), ("NoBC_Zmin", "NoBC_Zmin", 1),
        ("NoBC_Zmax", "NoBC_Zmax", 1), ("Log_Radius", "LogRadius", 0),
        ("Max_Aspect_Short", "MaxShort", 0), ("Max_Aspect_Long", "MaxLong", 0), ("CFL", "CFL", 0),
        ("PLM", "PLM", 0), ("Max_DT", "maxDT", 0), ("Adiabatic_Index", "Adiabatic_Index", 0),
        ("Isothermal", "isothermal_flag", 1), ("Cs2_Profile", "Cs2_Profile", 1), ("Cs2_Par", "Cs2_Par", 0),
        ("Density_Floor", "Density_Floor", 0), ("Pressure_Floor", "Pressure_Floor", 0),
        ("Mesh_Motion", "Mesh_Motion", 1), ("Riemann_Solver", "Riemann_Solver", 1),
        ("Initial_Regrid", "Initial_Regrid", 1), ("Restart", "restart_flag", 1),
        ("Exact_Mesh_Omega", "Exact_Mesh_Omega", 1), ("Exact_Mesh_Omega_Par", "Exact_Mesh_Omega_Par", 0),
        ("Energy_Omega", "Energy_Omega", 1), ("Energy_Omega_Par", "Energy_Omega_Par", 0),
        ("RotFrame", "RotFrame", 1), ("RotOmega", "RotOmega", 0), ("RotD", "RotD", 0),
        ("Use_Viscosity", "visc_flag", 1), ("Viscosity", "viscosity", 0), ("Use_As_Alpha", "alpha_flag", 1),
        ("Include_Atmos", "include_atmos", 1), ("Mach_Number", "Disk_Mach", 0),
        ("Mass_Ratio", "Mass_Ratio", 0), ("Eccentricity", "Eccentricity", 0),
        ("Drift_Rate", "Drift_Rate", 0), ("Drift_Exp", "Drift_Exp", 0),
        ("Constrained_Transport", "CT", 1)] + \
       [(f"Metric_Par{i}", f"metricPar{i}", int(i == 0)) for i in range(5)] + \
       [(f"Init_Par{i}", f"initPar{i}", int(i == 0)) for i in range(9)] + \
       [("Noise_Type", "noiseType", 1), ("Noise_Abs", "noiseAbs", 0), ("Noise_Rel", "noiseRel", 0),
        ("Sink_Type", "sinkType", 1)] + [(f"Sink_Par{i}", f"sinkPar{i}", 0) for i in range(1, 6)] + \
       [("Nozzle_Type", "nozzleType", 1)] + [(f"Nozzle_Par{i}", f"nozzlePar{i}", 0) for i in range(1, 5)] + \
       [("Cool_Type", "coolType", 1)] + [(f"Cool_Par{i}", f"coolPar{i}", 0) for i in range(1, 5)] + \
       [("Softening", "grav_eps", 0)]


def _id_phi0(h):
    """Id_phi0 as h5out.c:536-546 forms it: the first cell of largest cos(phi)
    (phi at the cell centre), starting from phi = pi and Id = 0."""
    out = np.zeros(h.Nr * h.Nz, dtype=np.int32)
    for jk in range(h.Nr * h.Nz):
        c0 = h.ring_off[jk]
        phi0, ident = np.pi, 0
        for i in range(h.Np[jk]):
            phi = h.piph[c0 + i] - .5 * h.dphi[c0 + i]
            if np.cos(phi0) < np.cos(phi):
                phi0, ident = phi, c0 + i
        out[jk] = ident
    return out


@pytest.mark.parametrize("name", list(CFGS))
def test_host_checkpoint_layout(name, tmp_path):
    h, p, m = _host(name)
    path = str(tmp_path / "checkpoint_0000.h5")
    h.checkpoint(path)
    f = h5spec.File(path)
    assert f.keys("/") == ["Data", "GIT_VERSION", "Grid", "Opts", "Pars"]
    assert all(f.is_group(g) for g in ("Grid", "Data", "Opts", "Pars"))
    assert f.keys("Grid") == ["Id_phi0", "Index", "Np", "T", "r_jph", "z_kph"]
    assert f.keys("Data") == ["Cells", "Diagnostics", "Planets"]
    nq, nf = h.num_q, h.num_faces
    assert nf == (5 if name == "mhd" else 0)
    cells = f.dataset("Data/Cells")
    assert cells.dtype == np.float64 and cells.shape == (h.Ncell, nq + nf + 1)
    assert np.array_equal(cells[:, :nq].T, h.prim)
    assert np.array_equal(cells[:, nq:nq + nf], np.zeros((h.Ncell, nf)))
    assert np.array_equal(cells[:, -1], h.piph)
    for key, want in (("Index", h.ring_off[:-1]), ("Np", h.Np), ("Id_phi0", _id_phi0(h))):
        a = f.dataset("Grid/" + key)
        assert a.dtype == np.int32 and a.shape == (h.Nz, h.Nr)
        assert np.array_equal(a.ravel(), want), key
    assert np.array_equal(f.dataset("Grid/r_jph"), h.r_jph)
    assert np.array_equal(f.dataset("Grid/z_kph"), h.z_kph)
    assert f.dataset("Grid/T").tolist() == [h.t]
    pl = f.dataset("Data/Planets")
    assert pl.shape == (h.Npl, 7)
    for i, b in enumerate(h.planets):
        assert pl[i].tolist() == [b["M"], b["vr"], b["omega"], b["r"], b["phi"], b["eps"], float(b["type"])]
    assert f.dataset("Data/Diagnostics").shape == (h.Nz, h.Nr, 0)
    assert f.dataset("GIT_VERSION")[0] == "disco_gb300"
    names = {"INITIAL": m.initial_name, "HYDRO": m.hydro_name, "BOUNDARY": m.boundary_name,
             "PLANETS": m.planets_name, "GEOMETRY": m.geometry_name, "HLLD": m.hlld_name}
    for k, v in names.items():
        assert f.dataset("Opts/" + k)[0] == v.decode(), k
    assert f.dataset("Opts/HYDRO")[0] == ("euler" if name == "planets" else name)
    for k, v in (("NUM_C", m.num_c), ("NUM_N", m.num_n), ("CT_MODE", m.ct_mode)):
        assert f.dataset("Opts/" + k).tolist() == [v]
    assert sorted(n for n, _, _ in PARS) == f.keys("Pars")
    for key, field, is_int in PARS:
        a = f.dataset("Pars/" + key)
        assert a.shape == (1,) and a.dtype == (np.int32 if is_int else np.float64), key
        assert a[0] == getattr(p, field), key


@pytest.mark.parametrize("name", list(CFGS))
def test_restart_reads_the_checkpoint_back(name, tmp_path):
    """Without noise, a restart reproduces the host domain bit for bit;
    the grid comes from the file even when in.par names another size
    (h5in.c:135-157)."""
    import disco_gb300.api as api
    h, p, m = _host(name, noiseType=0)
    path = str(tmp_path / "ck.h5")
    h.checkpoint(path)
    p2, _ = _pm(name, noiseType=0, Num_R=p.Num_R + 4)
    r = api.HostDomain(p2, m, restart=path)
    assert (r.Nr, r.Nz, r.Ncell) == (h.Nr, h.Nz, h.Ncell)
    assert r.params.Num_R == p.Num_R and r.params.Num_Z == p.Num_Z
    for k in ("Np", "ring_off", "r_jph", "z_kph", "piph", "dphi", "prim"):
        assert np.array_equal(getattr(r, k), getattr(h, k)), k
    assert r.t == h.t and r.planets == h.planets
    if h.num_faces:
        assert np.array_equal(r.Phi, np.zeros((h.num_faces, h.Ncell)))
    else:
        assert r.Phi is None
    # a checkpoint of the restarted domain is the same file content
    path2 = str(tmp_path / "ck2.h5")
    r.checkpoint(path2)
    f1, f2 = h5spec.File(path), h5spec.File(path2)
    for ds in ("Data/Cells", "Grid/Index", "Grid/Np", "Grid/r_jph", "Grid/T", "Data/Planets"):
        assert np.array_equal(f1.dataset(ds), f2.dataset(ds)), ds


def test_restart_draws_noise_after_the_phases(tmp_path):
    """setupCells adds Noise_Type's noise on a restart too (domain.c:204),
    drawing from rand() where in.par's grid left it -- the same draws as the
    initial set-up's.  With only absolute noise on prim[2], prim[3]
    (noise.c, type 1), the restart therefore adds exactly the set-up's
    perturbation a second time."""
    import disco_gb300.api as api
    p0, m = _pm("mhd", noiseType=0)
    clean = api.HostDomain(p0, m)
    h, p, _ = _host("mhd", noiseType=1, noiseRel=0.0, noiseAbs=1e-3)
    path = str(tmp_path / "ck.h5")
    h.checkpoint(path)
    r = api.HostDomain(p, m, restart=path)
    real = h.real_mask()
    first = h.prim - clean.prim
    second = r.prim - h.prim
    assert np.abs(first[2:4][:, real]).max() > 1e-4
    np.testing.assert_allclose(second[2:4][:, real], first[2:4][:, real], rtol=0, atol=1e-15)
    for q in (0, 1, 4, 5, 6, 7, 8):
        assert np.array_equal(r.prim[q], h.prim[q]), q
    assert np.array_equal(r.prim[:, ~real], h.prim[:, ~real])


def test_restart_rejects_bad_files(tmp_path):
    import disco_gb300.api as api
    h, p, m = _host("mhd", noiseType=0)
    path = str(tmp_path / "ck.h5")
    h.checkpoint(path)
    raw = bytearray(open(path, "rb").read())
    with pytest.raises(api.DiscoError, match="cannot open"):
        api.HostDomain(p, m, restart=str(tmp_path / "missing.h5"))
    # a flipped byte in the superblock, and one in an object header
    for where in (20, 100):
        bad = bytearray(raw)
        bad[where] ^= 0x40
        bp = str(tmp_path / f"bad{where}.h5")
        open(bp, "wb").write(bad)
        with pytest.raises(api.DiscoError):
            api.HostDomain(p, m, restart=bp)
    # truncated
    tp = str(tmp_path / "trunc.h5")
    open(tp, "wb").write(raw[:len(raw) // 2])
    with pytest.raises(api.DiscoError):
        api.HostDomain(p, m, restart=tp)
    # an MHD checkpoint read with the euler modules: NUM_Q + NUM_FACES + 1
    # differs (h5in.c:322)
    pe, me = _pm("euler", noiseType=0)
    with pytest.raises(api.DiscoError, match="columns"):
        api.HostDomain(pe, me, restart=path)


def test_restart_survives_any_flipped_byte(tmp_path):
    """The reader checks every offset, size and checksum it takes from the
    file: a checkpoint with one byte flipped anywhere in its metadata (every
    byte of the superblock and root header, every fifth byte of the rest of
    the first 8 KB and of the last 16 KB, where the headers, the global heap
    and the parameter tables lie) or in its data either restarts or raises
    DiscoError -- it never crashes the process or reads out of bounds."""
    import disco_gb300.api as api
    h, p, m = _host("mhd", noiseType=0)
    path = str(tmp_path / "ck.h5")
    h.checkpoint(path)
    raw = bytearray(open(path, "rb").read())
    n = len(raw)
    where = [*range(0, 2048), *range(2048, 8192, 5), *range(n - 16384, n, 5),
             *range(8192, n - 16384, 4099)]
    bp = str(tmp_path / "bad.h5")
    errors = 0
    for w in where:
        bad = bytearray(raw)
        bad[w] ^= 0xff
        open(bp, "wb").write(bad)
        try:
            api.HostDomain(p, m, restart=bp)
        except api.DiscoError:
            errors += 1
    # the superblock's 48 bytes end in a checksum over the first 44: a flip
    # of any of them is caught
    assert errors >= 48


def test_checkpoint_abi_symbols():
    """The checkpoint entry points are exported with the header's names."""
    import disco_gb300.api as api
    L = api.lib()
    for s in ("disco_gpu_checkpoint", "disco_host_checkpoint", "disco_host_restart"):
        assert hasattr(L, s)
    hdr = open(os.path.join(ROOT, "include", "disco_gpu_checkpoint.h")).read()
    assert all(s in hdr for s in ("disco_gpu_checkpoint", "disco_host_checkpoint", "disco_host_restart"))
    assert C.sizeof(api.DiscoHostDomain) > 0
