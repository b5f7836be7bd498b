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


def divb_from_faces(Phi, Np, faces):
    """Net outward face flux of B per cell (the sum of
    Python/discopy/geom.py:370-520, calcDivB) from the face fluxes Phi
    [5, N] and face tables {"r": ..., "z": ...} (L, R, LRtype per face): a
    face's flux lives in L.Phi[2] / L.Phi[4] (LRtype 0) or R.Phi[1] /
    R.Phi[3] (bfields.c:52-76)."""
    N = Phi.shape[1]
    off = np.concatenate([[0], np.cumsum(Np)])
    div = np.zeros(N)
    for jk in range(len(Np)):
        a, b = off[jk], off[jk + 1]
        div[a:b] += Phi[0, a:b] - np.roll(Phi[0, a:b], 1)
    for key, up, dn in (("r", 2, 1), ("z", 4, 3)):
        f = faces.get(key)
        if f is None or len(f["L"]) == 0:
            continue
        L, R = f["L"].astype(np.int64), f["R"].astype(np.int64)
        flux = np.where(f["LRtype"] == 0, Phi[up, L], Phi[dn, R])
        np.add.at(div, L, flux)
        np.add.at(div, R, -flux)
    return div


def component_norms(a, b):
    """Per conserved component q of a [nq, n] against b: the relative L1
    error sum|a-b| / sum|b| and the relative Linf error max|a-b| / max|b|
    (each 0 where b is identically zero and a equals it)."""
    out = {"l1": {}, "linf": {}}
    for q in range(b.shape[0]):
        d = np.abs(a[q] - b[q])
        s1, m1 = np.abs(b[q]).sum(), np.abs(b[q]).max() if b.shape[1] else 0.0
        out["l1"][q] = float(d.sum() / s1) if s1 > 0 else float(d.sum())
        out["linf"][q] = float(d.max() / m1) if m1 > 0 else float(d.max() if d.size else 0.0)
    return out
