"""The mixed path's staged azimuthal sweep (k_phi_sweep: plm_phi and the
phi-face fluxes of a ring chunk from one tensor-memory-accelerator stage)
against the separate plm_phi and flux_phi kernels: the same arithmetic on
the same values, so the states after the steps agree bit for bit on the
hydro cases.  With constrained transport the edge EMFs are summed with FP64
atomics in no fixed order; on the mixed path those last-bit differences
pass through FP32 arithmetic, so two runs of either kernel set agree to
a few 1e-9 relative L1 per physical quantity after five steps (vectors
through their norm; the magnetic field, 2.3e-8 on the MHD disk, the
most), and 1e-7 is the bar there.  No bounded wait on the copies ran
out."""
import numpy as np
import pytest

from helpers import cell_radius, grouped_rel_l1
from test_gpu_parity import _domain

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cfg1_n24", "cfg1_rotframe", "cfg2_n12", "cfg5_n16", "bc_polar3d"])
def test_staged_sweep_equals_separate_kernels(name):
    a, g = _domain(name, 1)
    b, _ = _domain(name, 1)
    assert a.set_sweep(True)
    assert not b.set_sweep(False)
    n = int(g["nsteps"])
    for _ in range(n):
        dt = a.getmindt()
        a.timestep(dt)
        b.timestep(dt)
    sa, sb = a.state(), b.state()
    if name.startswith(("cfg2", "cfg5")):
        h = a.host
        real = h.real_mask()
        r = cell_radius(h.Np, h.r_jph, h.Nr, h.Nz)[real]
        e = grouped_rel_l1(sa["cons"][:, real], sb["cons"][:, real], r, 8)   # MHD: B is a vector too
        assert max(e.values()) < 1e-7, e
    else:
        assert np.array_equal(sa["cons"], sb["cons"])
        assert np.array_equal(sa["piph"], sb["piph"])
    assert a.status()["async_timeouts"] == 0
    a.close(); b.close()


def test_staged_sweep_not_used_with_viscosity():
    """The planet disk has explicit viscosity, whose phi fluxes read the
    transverse gradients: it keeps the separate kernels."""
    d, _ = _domain("cfg3_n24", 1)
    assert not d.set_sweep(True)
    d.close()
