"""The reference-side binding (disco_gb300/csrc/shim/gb300_shim.c) compiled
against the reference's own paul.h and objects: the reference's getmindt
and timestep are renamed out of misc.c / timestep.c, the shim defines them
on libdisco_gb300, and the reference harness links (oracle/ref/Makefile,
target gb300).  Runs where the reference sources are (DISCO_REFERENCE or the
staged copy in baseline/_ref/src); the run itself is tests/test_gpu_shim.py."""
import os
import subprocess

import pytest

from helpers import ROOT


def _ref():
    from oracle.build_oracle import reference_dir
    return reference_dir()


@pytest.mark.skipif(_ref() is None, reason="reference sources not present")
@pytest.mark.parametrize("cfg", ["configs/cfg1_vortex", "configs/cfg2_mhd_disk"])
def test_shim_builds_against_the_reference(cfg):
    from disco_gb300 import build
    build.build()
    subprocess.run(["make", "-s", "-f", "oracle/ref/Makefile", f"CFG={cfg}", f"REF={_ref()}", "gb300"],
                   cwd=ROOT, check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", os.path.basename(cfg), "disco_ref_gb300")
    nm = subprocess.run(["nm", exe], capture_output=True, text=True, check=True).stdout
    syms = {ln.split()[-1]: ln.split()[-2] for ln in nm.splitlines() if len(ln.split()) >= 2}
    # the main loop's two calls resolve to the shim; the reference's own
    # definitions are still there under other names
    for s in ("getmindt", "timestep", "gb300_init", "gb300_sync_to_host",
              "disco_reference_getmindt", "disco_reference_timestep"):
        assert syms.get(s) == "T", s
    dyn = subprocess.run(["nm", "-D", exe], capture_output=True, text=True, check=True).stdout
    for s in ("disco_gpu_create", "disco_gpu_getmindt", "disco_gpu_timestep", "disco_gpu_download",
              "disco_gpu_planets"):
        assert s in dyn, s
