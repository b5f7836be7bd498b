"""Accreting sinks and the gas nozzle (sink.c:105-247): the sink bodies'
accumulators (gravL, dM, accL, Ls, kin, therm, linXmom, linYmom) after the
fixture's steps against the reference's own values, which its harness
dumps before report() zeroes them.  The device sums each substep's
contributions by a fixed tree over blocks, the reference cell by cell: the
FP64 path agrees to 1e-12 of each accumulator's largest magnitude over the
bodies, the mixed path (FP32 primitives) to 2e-5.  The conserved state of
these cases is checked with the other parity cases."""
import numpy as np
import pytest

from test_gpu_parity import _domain

pytestmark = pytest.mark.gpu

CASES = ["cfg3_sink", "cfg3_sink_exp", "cfg3_nozzle"]
KEYS = ("gravL", "dM", "accL", "Ls", "kin", "therm", "linXmom", "linYmom")


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", CASES)
def test_sink_accumulators_match_reference(name, precision):
    d, g = _domain(name, precision)
    n = int(g["nsteps"])
    for _ in range(n):
        d.timestep(d.getmindt())
    ref = np.asarray(g["planets"])[:, 6:14]
    acc = d.sink_accum()
    if name == "cfg3_nozzle":
        assert acc == []   # no sinks: nothing accumulated, nothing returned
        d.close()
        return
    got = np.array([[a[k] for k in KEYS] for a in acc])
    assert got.shape == ref.shape
    tol = 1e-12 if precision == 0 else 2e-5
    for j, k in enumerate(KEYS):
        scale = np.abs(ref[:, j]).max()
        assert np.abs(got[:, j] - ref[:, j]).max() <= tol * scale, (k, got[:, j], ref[:, j])
    # reset zeroes them (report.c:91-108) and the next step accumulates anew
    d.sink_accum(reset=True)
    assert all(v == 0.0 for a in d.sink_accum() for v in a.values())
    d.timestep(d.getmindt())
    assert d.sink_accum()[1]["dM"] > 0
    st = d.status()
    assert st["nan_cells"] == 0
    d.close()
