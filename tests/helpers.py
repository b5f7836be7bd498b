"""Shared helpers for the tests: fixture loading and error norms."""
from __future__ import annotations

import os
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def load_golden(name: str) -> dict:
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return {k: g[k] for k in g.files}


def write_par(text: str) -> str:
    td = tempfile.mkdtemp(prefix="disco_par_")
    p = os.path.join(td, "in.par")
    with open(p, "w") as f:
        f.write(str(text))
    return p


def mk_path(g, cfg=None) -> str:
    """Makefile_opt.in of a fixture: its own module text when it carries one
    (cases that swap a module of a configuration), else the configuration's."""
    if "mk_text" in g:
        td = tempfile.mkdtemp(prefix="disco_mk_")
        p = os.path.join(td, "Makefile_opt.in")
        with open(p, "w") as f:
            f.write(str(g["mk_text"]))
        return p
    return os.path.join(ROOT, str(cfg if cfg is not None else g["cfg"]), "Makefile_opt.in")


def rel_l1(a: np.ndarray, b: np.ndarray) -> float:
    """sum |a - b| / sum |b| (relative L1 error of a against b)."""
    den = np.abs(b).sum()
    return float(np.abs(a - b).sum() / (den if den > 0 else 1.0))


def real_mask(Np, Nr, Nz, NgRa, NgRb, NgZa, NgZb):
    jk = np.repeat(np.arange(Nr * Nz), Np)
    j, k = jk % Nr, jk // Nr
    return (j >= NgRa) & (j < Nr - NgRb) & (k >= NgZa) & (k < Nz - NgZb)


def cell_radius(Np, r_jph, Nr, Nz):
    """Centroid radius of every cell (ring-major order)."""
    rp, rm = r_jph[1:], r_jph[:-1]
    rc = 2.0 * (rp * rp + rp * rm + rm * rm) / (3.0 * (rp + rm))
    jk = np.repeat(np.arange(Nr * Nz), Np)
    return rc[jk % Nr]


def grouped_rel_l1(a, b, r, num_c):
    """Relative L1 error of a conserved state a against b per physical
    quantity: mass, energy, momentum vector (S_r, L/r, S_z), magnetic field
    vector and passive scalar; vector quantities are compared through the
    Euclidean norm of the difference over the norm of the reference vector,
    so a near-zero component (radial momentum of a Keplerian disk) is
    measured against the flow it belongs to."""
    out = {"mass": rel_l1(a[0], b[0]), "energy": rel_l1(a[1], b[1])}
    def vec(x):
        return np.stack([x[2], x[3] / r, x[4]])
    da, db = vec(a) - vec(b), vec(b)
    out["momentum"] = float(np.sqrt((da ** 2).sum(0)).sum() / np.sqrt((db ** 2).sum(0)).sum())
    if num_c == 8:
        ba, bb = a[5:8], b[5:8]
        out["magnetic"] = float(np.sqrt(((ba - bb) ** 2).sum(0)).sum() / np.sqrt((bb ** 2).sum(0)).sum())
    if a.shape[0] > num_c:
        out["passive"] = rel_l1(a[num_c], b[num_c])
    return out
