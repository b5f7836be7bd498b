"""CHECKER INFRASTRUCTURE (oracle): ctypes binding of oracle/port/disco_port.c.

Runs the plain-C restatement of the reference hot path on a domain produced
by the product's host set-up (itself checked bit-for-bit against the
reference)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build_oracle import build_port

_L = None
_dp = C.POINTER(C.c_double)


def _lib():
    global _L
    if _L is None:
        L = C.CDLL(build_port())
        L.disco_port_create.restype = C.c_void_p
        L.disco_port_create.argtypes = [C.c_void_p]
        L.disco_port_run.argtypes = [C.c_void_p, C.c_int]
        L.disco_port_step.restype = C.c_double
        L.disco_port_step.argtypes = [C.c_void_p]
        L.disco_port_state.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.disco_port_num_real.restype = C.c_long
        L.disco_port_num_real.argtypes = [C.c_void_p]
        L.disco_port_free.argtypes = [C.c_void_p]
        L.disco_port_phi.argtypes = [C.c_void_p, _dp]
        L.disco_port_report.argtypes = [C.c_void_p, _dp]
        L.disco_port_diag.argtypes = [C.c_void_p, _dp, _dp]
        L.disco_port_sink_accum.argtypes = [C.c_void_p, _dp, C.c_int]
        _ip = C.POINTER(C.c_int)
        L.disco_port_faces.restype = C.c_long
        L.disco_port_faces.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip, _ip, _dp, _dp]
        L.disco_port_grad.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.disco_port_debug_ct.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]
        _L = L
    return _L


class PortDomain:
    def __init__(self, host):
        """host: disco_gb300.HostDomain"""
        self.host = host
        self._d = _lib().disco_port_create(C.cast(host._ptr, C.c_void_p))
        if not self._d:
            raise RuntimeError("oracle port: unsupported module combination")

    def run(self, n: int) -> None:
        _lib().disco_port_run(self._d, int(n))

    def step(self) -> float:
        return _lib().disco_port_step(self._d)

    @property
    def num_real(self) -> int:
        return _lib().disco_port_num_real(self._d)

    def state(self) -> dict:
        N, nq = self.host.Ncell, self.host.num_q
        s = {"piph": np.empty(N), "dphi": np.empty(N), "prim": np.empty((nq, N)),
             "cons": np.empty((nq, N))}
        t = C.c_double()
        _lib().disco_port_state(self._d, *(s[k].ctypes.data_as(_dp) for k in ("piph", "dphi", "prim", "cons")),
                                C.byref(t))
        s["t"] = t.value
        if self.host.num_q == 9:
            s["Phi"] = np.empty((5, N))
            _lib().disco_port_phi(self._d, s["Phi"].ctypes.data_as(_dp))
        return s

    REPORT_KEYS = ("t", "q", "Mass", "Torque", "Torque2") + tuple(
        f"Torque{i}_cut{n}" for n in range(5) for i in (1, 2))

    def report(self) -> dict:
        """report.c's domain sums (the restatement, serial reference order)."""
        out = np.empty(len(self.REPORT_KEYS))
        _lib().disco_port_report(self._d, out.ctypes.data_as(_dp))
        return dict(zip(self.REPORT_KEYS, out.tolist()))

    def sink_accum(self, nbody: int) -> np.ndarray:
        """The sink accumulators of the first nbody bodies, [nbody, 8]:
        gravL, dM, accL, Ls, kin, therm, linXmom, linYmom."""
        out = np.zeros((nbody, 8))
        _lib().disco_port_sink_accum(self._d, out.ctypes.data_as(_dp), int(nbody))
        return out

    def diagnostics(self) -> dict:
        """analysis.c's ring accumulators: Qrz [Nr*Nz, n] and t_avg."""
        n = _lib().disco_port_diag(self._d, None, None)
        q = np.zeros((self.host.Nr * self.host.Nz, n))
        t = C.c_double()
        _lib().disco_port_diag(self._d, q.ctypes.data_as(_dp), C.byref(t))
        return {"Qrz": q, "t_avg": t.value}

    def faces(self, dim: int) -> dict:
        """The face tables built from the current positions (faces_alt.c),
        in the layout of disco_gb300.Domain.faces."""
        h = self.host
        ntr = (h.Nr - 1) * h.Nz if dim == 1 else h.Nr * (h.Nz - 1)
        nf = _lib().disco_port_faces(self._d, int(dim), None, None, None, None, None, None)
        out = {"fIndex": np.zeros(max(ntr, 0) + 1, np.int32)}
        for k in ("L", "R", "LRtype"):
            out[k] = np.zeros(nf, np.int32)
        for k in ("phic", "dA"):
            out[k] = np.zeros(nf)
        if nf:
            ip = C.POINTER(C.c_int)
            _lib().disco_port_faces(self._d, int(dim), *(out[k].ctypes.data_as(ip) for k in ("fIndex", "L", "R", "LRtype")),
                                    *(out[k].ctypes.data_as(_dp) for k in ("phic", "dA")))
        return out

    def gradients(self) -> dict:
        """plm_phi + plm_trans on the current state (gradp, gradr, gradz)."""
        shp = (self.host.num_q, self.host.Ncell)
        out = {k: np.zeros(shp) for k in ("gradp", "gradr", "gradz")}
        _lib().disco_port_grad(self._d, *(out[k].ctypes.data_as(_dp) for k in ("gradp", "gradr", "gradz")))
        return out

    def __del__(self):
        if getattr(self, "_d", None):
            _lib().disco_port_free(self._d)
            self._d = None
