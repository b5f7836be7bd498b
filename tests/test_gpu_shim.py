"""The reference's own harness (init, getmindt/timestep loop, dump,
report()) driven through the reference-side binding gb300_shim.c: the hot
path runs in libdisco_gb300 on the GPU and the synced struct domain gives
the reference's dump and report line.  Compared with the fixtures the
unmodified reference wrote: state at 1e-12 (FP64 path), positions bit-exact,
face fluxes Phi (constrained transport) and the point masses through the
report line."""
import os
import re
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from helpers import ROOT, load_golden, rel_l1

pytestmark = pytest.mark.gpu


def _ref():
    from oracle.build_oracle import reference_dir
    return reference_dir()


CASES = {"cfg1_n24": "configs/cfg1_vortex", "cfg2_n12": "configs/cfg2_mhd_disk",
         "cfg3_n24": "configs/cfg3_planet_disk"}


def _run_harness(exe, td, par_text, makefile_opt, nsteps, out="out.bin"):
    with open(os.path.join(td, "in.par"), "w") as f:
        f.write(par_text)
    shutil.copy(makefile_opt, os.path.join(td, "Makefile_opt.in"))
    r = subprocess.run([exe, "run", str(nsteps), out], cwd=td, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.skipif(_ref() is None, reason="reference sources not present")
def test_restart_on_the_shim_continues_the_reference_run():
    """Half the vortex run, its checkpoint through gb300_output, then the
    reference's main loop with Restart 1 from that file (input.h5) for the
    other half: the final state equals the unmodified reference's
    uninterrupted run (the fixture) within 1e-12, the time exactly."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from dumpio import read_dump
    from disco_gb300 import build
    build.build()
    name, cfg = "cfg1_n24", CASES["cfg1_n24"]
    subprocess.run(["make", "-s", "-f", "oracle/ref/Makefile", f"CFG={cfg}", f"REF={_ref()}", "gb300"],
                   cwd=ROOT, check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", os.path.basename(cfg), "disco_ref_gb300")
    g = load_golden(name)
    n = int(g["nsteps"])
    par = str(g["par_text"])
    mk = os.path.join(ROOT, cfg, "Makefile_opt.in")
    td1, td2 = tempfile.mkdtemp(prefix="disco_shim_"), tempfile.mkdtemp(prefix="disco_shim_")
    _run_harness(exe, td1, par, mk, n // 2)
    shutil.copy(os.path.join(td1, "checkpoint_gb300.h5"), os.path.join(td2, "input.h5"))
    par2 = re.sub(r"^Restart\s+\d+", "Restart\t1", par, flags=re.M)
    assert par2 != par
    _run_harness(exe, td2, par2, mk, n - n // 2)
    out = read_dump(os.path.join(td2, "out.bin"))
    real = g["real"].astype(bool)
    assert abs(out["t"] - float(g["run_t"])) <= 1e-14 * abs(float(g["run_t"]))
    assert np.max(np.abs(out["piph"] - g["run_piph"])) < 1e-12 * 2 * np.pi
    for q in range(out["cons"].shape[0]):
        assert rel_l1(out["cons"][q, real], g["run_cons"][q, real]) < 1e-11, q
        assert rel_l1(out["prim"][q, real], g["run_prim"][q, real]) < 1e-11, q
    shutil.rmtree(td1)
    shutil.rmtree(td2)


@pytest.mark.skipif(_ref() is None, reason="reference sources not present")
@pytest.mark.parametrize("name", list(CASES))
def test_reference_harness_on_the_shim(name):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from dumpio import read_dump
    from disco_gb300 import build
    build.build()
    cfg = CASES[name]
    subprocess.run(["make", "-s", "-f", "oracle/ref/Makefile", f"CFG={cfg}", f"REF={_ref()}", "gb300"],
                   cwd=ROOT, check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", os.path.basename(cfg), "disco_ref_gb300")
    g = load_golden(name)
    td = tempfile.mkdtemp(prefix="disco_shim_")
    with open(os.path.join(td, "in.par"), "w") as f:
        f.write(str(g["par_text"]))
    shutil.copy(os.path.join(ROOT, cfg, "Makefile_opt.in"), os.path.join(td, "Makefile_opt.in"))
    n = int(g["nsteps"])
    r = subprocess.run([exe, "run", str(n), "out.bin"], cwd=td, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    out = read_dump(os.path.join(td, "out.bin"))
    real = g["real"].astype(bool)
    assert abs(out["t"] - float(g["run_t"])) <= 1e-12 * abs(float(g["run_t"]))
    assert np.max(np.abs(out["piph"] - g["run_piph"])) < 1e-12 * 2 * np.pi
    for q in range(out["cons"].shape[0]):
        assert rel_l1(out["cons"][q, real], g["run_cons"][q, real]) < 1e-11, q
        assert rel_l1(out["prim"][q, real], g["run_prim"][q, real]) < 1e-11, q
    for q in range(out["Phi"].shape[0]):
        ref = g["run_Phi"][q, real]
        if np.abs(ref).sum() > 0:
            assert rel_l1(out["Phi"][q, real], ref) < 1e-11, q
    # report() of the reference on the synced domain (planets included)
    line = open(os.path.join(td, "report.dat")).read().strip().splitlines()[-1]
    rep = np.array([float(v) for v in re.findall(r"[-+]?\d\.\d+e[-+]\d{2}(?:\d(?!\.))?", line)])
    assert rep.shape == g["report"].shape
    assert np.allclose(rep, g["report"], rtol=2e-6, atol=1e-30)
    # the shim's gb300_output in place of output(): the checkpoint file of
    # the same final state, read by the specification reader
    import h5spec
    f = h5spec.File(os.path.join(td, "checkpoint_gb300.h5"))
    cells = f.dataset("Data/Cells")
    nq, nf = out["prim"].shape[0], out["Phi"].shape[0]
    assert cells.shape == (out["prim"].shape[1], nq + nf + 1)
    assert np.array_equal(cells[:, :nq].T, out["prim"])
    assert np.array_equal(cells[:, nq:nq + nf].T, out["Phi"])
    assert np.array_equal(cells[:, -1], out["piph"])
    assert f.dataset("Grid/T").tolist() == [out["t"]]
    shutil.rmtree(td)
