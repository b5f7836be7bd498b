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


def rel_l1(a: np.ndarray, b: np.ndarray) -> float:
    """sum |a - b| / sum |b| (relative L1 error of a against b)."""
    den = np.abs(b).sum()
    return float(np.abs(a - b).sum() / (den if den > 0 else 1.0))


def real_mask(Np, Nr, Nz, NgRa, NgRb, NgZa, NgZb):
    jk = np.repeat(np.arange(Nr * Nz), Np)
    j, k = jk % Nr, jk // Nr
    return (j >= NgRa) & (j < Nr - NgRb) & (k >= NgZa) & (k < Nz - NgZb)
