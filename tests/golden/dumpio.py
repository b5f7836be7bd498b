"""Reader for the raw state dumps written by the reference harness
(oracle/ref/harness_main.c: write_state / write_faces)."""
from __future__ import annotations

import numpy as np

MAGIC = 0x4F435344


class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf
        self.o = 0

    def i(self, n=None):
        k = 1 if n is None else n
        a = np.frombuffer(self.b, dtype="<i4", count=k, offset=self.o)
        self.o += 4 * k
        return int(a[0]) if n is None else a.copy()

    def d(self, n=None):
        k = 1 if n is None else n
        a = np.frombuffer(self.b, dtype="<f8", count=k, offset=self.o)
        self.o += 8 * k
        return float(a[0]) if n is None else a.copy()


def read_dump(path: str) -> dict:
    with open(path, "rb") as f:
        r = _Reader(f.read())
    assert r.i() == MAGIC, "not a state dump"
    r.i()  # version
    out = {}
    for k in ("Nr", "Nz", "NgRa", "NgRb", "NgZa", "NgZb", "num_q", "num_faces", "N", "with_grad"):
        out[k] = r.i()
    out["t"] = r.d()
    out["phi_max"] = r.d()
    Nr, Nz, N, nq, nf = out["Nr"], out["Nz"], out["N"], out["num_q"], out["num_faces"]
    out["Np"] = r.i(Nr * Nz)
    out["r_jph"] = r.d(Nr + 1)
    out["z_kph"] = r.d(Nz + 1)
    out["piph"] = r.d(N)
    out["dphi"] = r.d(N)
    out["wiph"] = r.d(N)
    out["real"] = r.i(N)
    out["prim"] = r.d(nq * N).reshape(nq, N)
    out["cons"] = r.d(nq * N).reshape(nq, N)
    out["Phi"] = r.d(nf * N).reshape(nf, N) if nf else np.zeros((0, N))
    if out["with_grad"]:
        out["gradp"] = r.d(nq * N).reshape(nq, N)
        out["gradr"] = r.d(nq * N).reshape(nq, N)
        out["gradz"] = r.d(nq * N).reshape(nq, N)
        off = np.concatenate([[0], np.cumsum(out["Np"])])
        for _ in range(2):
            dim = r.i()
            if dim == 0:
                continue
            NN = r.i()
            fI = r.i(NN + 1)
            Nf = int(fI[-1])
            ints = r.i(5 * Nf).reshape(Nf, 5)
            dbl = r.d(8 * Nf).reshape(Nf, 8)
            key = "r" if dim == 1 else "z"
            out[f"faces_{key}"] = {
                "fIndex": fI,
                "L": off[ints[:, 0]] + ints[:, 1],
                "R": off[ints[:, 2]] + ints[:, 3],
                "LRtype": ints[:, 4],
                "cm": dbl[:, 0:3], "dphi": dbl[:, 3], "dA": dbl[:, 4], "dl": dbl[:, 5],
                "dxL": dbl[:, 6], "dxR": dbl[:, 7],
            }
    return out
