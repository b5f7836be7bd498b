"""The C-ABI library loads and exports every symbol include/*.h declares;
without a GPU the device entry points fail with an error code (no CPU
fallback)."""
import ctypes
import glob
import os
import re

import pytest

from helpers import ROOT, write_par


def _declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(disco_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_exports_every_declared_symbol():
    import disco_gb300 as dg
    L = dg.lib()
    names = _declared_functions()
    assert "disco_gpu_timestep" in names and "disco_gpu_getmindt" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert L.disco_abi_version() == 1


def test_python_signatures_cover_header():
    import disco_gb300.api as api
    names = set(_declared_functions())
    assert names <= set(api.SIGNATURES), names - set(api.SIGNATURES)


def test_create_without_gpu_is_an_error():
    import disco_gb300 as dg
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(dg.DiscoError, match="no CUDA device"):
        dg.Domain(os.path.join(ROOT, "configs/cfg1_vortex/in.par"),
                  os.path.join(ROOT, "configs/cfg1_vortex/Makefile_opt.in"))
