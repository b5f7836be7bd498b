"""Small cases of single kernels for profiling (ncu) with the library's own
API, for kernels the benchmark workloads do not isolate:

    python -m disco_gb300.profile_cases mlp        # k_mlp_fwdbwd, k_mlp_wgrad
    python -m disco_gb300.profile_cases phi_sweep  # k_phi_sweep
    python -m disco_gb300.profile_cases flux_trans # k_flux_trans (HLLD + CT)
    python -m disco_gb300.profile_cases all        # mlp and phi_sweep

mlp: the MLP gradient (forward + backward and the weight gradient, BF16
tensor-core kernels) over 262,144 random (feature, target) rows.
phi_sweep: the staged azimuthal sweep of the mixed path on the 2D vortex at
Num_R = 1024 (4.6 M cells, 0.4 GB of sweep inputs and outputs: larger than
L2), two RK2 steps (four launches).  flux_trans: two RK2 steps of the 3D
MHD disk at Num_R = 128, Num_Z = 32 on the mixed path (2.9 M cells; eight
launches, r and z).  Each case prints one line and exits 0.
"""
import os
import sys

import numpy as np

from . import api as dg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def mlp() -> None:
    rng = np.random.default_rng(0)
    m = dg.Mlp(seed=1, capacity=16)
    n = 1 << 18
    X = rng.standard_normal((n, 10)).astype(np.float32)
    Y = rng.standard_normal((n, 2)).astype(np.float32)
    loss, _ = m.grad(X, Y)
    m.close()
    print("mlp: rows", n, "loss", loss)


def phi_sweep() -> None:
    cfg = os.path.join(ROOT, "configs", "cfg1_vortex")
    d = dg.Domain(os.path.join(cfg, "in.par"), os.path.join(cfg, "Makefile_opt.in"), precision=1,
                  overrides={"Num_R": 1024})
    if not d.set_sweep(True):
        raise RuntimeError("the staged sweep does not apply")
    cells = d.num_cells
    d.run(2)
    st = d.status()
    d.close()
    if st["async_timeouts"]:
        raise RuntimeError("a staged-sweep wait ran out")
    print("phi_sweep: cells", cells, "steps 2")


def flux_trans() -> None:
    cfg = os.path.join(ROOT, "configs", "cfg2_mhd_disk")
    d = dg.Domain(os.path.join(cfg, "in.par"), os.path.join(cfg, "Makefile_opt.in"), precision=1,
                  overrides={"Num_R": 128, "Num_Z": 32})
    cells = d.num_cells
    d.run(2)
    st = d.status()
    d.close()
    if st["nan_cells"] or st["face_errors"]:
        raise RuntimeError(f"unexpected health counters {st}")
    print("flux_trans: cells", cells, "steps 2")


CASES = {"mlp": mlp, "phi_sweep": phi_sweep, "flux_trans": flux_trans}


def main(argv) -> int:
    names = argv[1:] or ["all"]
    for name in names:
        picked = {"mlp": mlp, "phi_sweep": phi_sweep} if name == "all" else {name: CASES[name]}
        for case in picked.values():
            case()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
