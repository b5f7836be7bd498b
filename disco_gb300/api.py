"""Python view of the C ABI in include/disco_gpu.h (ctypes).

This mirrors the reference's driver loop (main.c:27-89): parameters come from
in.par (readpar.c) and module names from Makefile_opt.in; `getmindt()` and
`timestep(dt)` replace the reference's getmindt/timestep hooks.  All compute
runs in the native library; if it cannot be loaded or finds no GPU the calls
raise -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class DiscoParams(C.Structure):
    _fields_ = [
        ("t_min", C.c_double), ("t_max", C.c_double),
        ("Num_R", C.c_int), ("Num_Z", C.c_int),
        ("aspect", C.c_double),
        ("rmin", C.c_double), ("rmax", C.c_double), ("zmin", C.c_double), ("zmax", C.c_double),
        ("phimax", C.c_double),
        ("NoBC_Rmin", C.c_int), ("NoBC_Rmax", C.c_int), ("NoBC_Zmin", C.c_int), ("NoBC_Zmax", C.c_int),
        ("LogZoning", C.c_int), ("R_Periodic", C.c_int), ("Z_Periodic", C.c_int),
        ("LogRadius", C.c_double),
        ("Mesh_Motion", C.c_int), ("Riemann_Solver", C.c_int), ("Timestep", C.c_int),
        ("CFL", C.c_double), ("PLM", C.c_double), ("maxDT", C.c_double),
        ("Density_Floor", C.c_double), ("Pressure_Floor", C.c_double),
        ("Exact_Mesh_Omega", C.c_int), ("Exact_Mesh_Omega_Par", C.c_double),
        ("Energy_Omega", C.c_int), ("Energy_Omega_Par", C.c_double),
        ("RotFrame", C.c_int), ("RotOmega", C.c_double), ("RotD", C.c_double),
        ("Adiabatic_Index", C.c_double),
        ("visc_flag", C.c_int), ("viscosity", C.c_double),
        ("alpha_flag", C.c_int),
        ("isothermal_flag", C.c_int),
        ("Cs2_Profile", C.c_int), ("Cs2_Par", C.c_double),
        ("Disk_Mach", C.c_double), ("Mass_Ratio", C.c_double),
        ("grav2D", C.c_int),
        ("CT", C.c_int),
        ("metricPar0", C.c_int), ("metricPar1", C.c_double), ("metricPar2", C.c_double),
        ("metricPar3", C.c_double), ("metricPar4", C.c_double),
        ("initPar0", C.c_int), ("initPar1", C.c_double), ("initPar2", C.c_double),
        ("initPar3", C.c_double), ("initPar4", C.c_double), ("initPar5", C.c_double),
        ("initPar6", C.c_double), ("initPar7", C.c_double), ("initPar8", C.c_double),
        ("noiseType", C.c_int), ("noiseAbs", C.c_double), ("noiseRel", C.c_double),
        ("sinkType", C.c_int), ("nozzleType", C.c_int), ("coolType", C.c_int),
        ("dampInnerType", C.c_int), ("dampOuterType", C.c_int),
        ("dampUpperType", C.c_int), ("dampLowerType", C.c_int),
        ("grav_eps", C.c_double),
        ("read_errors", C.c_int),
        ("sinkPar3", C.c_double),
        ("coolPar1", C.c_double), ("coolPar2", C.c_double), ("coolPar3", C.c_double), ("coolPar4", C.c_double),
        ("dampTimeInner", C.c_double), ("dampLenInner", C.c_double), ("dampTimeOuter", C.c_double),
        ("dampLenOuter", C.c_double), ("dampTimeUpper", C.c_double), ("dampLenUpper", C.c_double),
        ("dampTimeLower", C.c_double), ("dampLenLower", C.c_double),
        ("maxNp", C.c_int),
        ("sinkNumber", C.c_int),
        ("sinkPar1", C.c_double), ("sinkPar2", C.c_double), ("sinkPar4", C.c_double), ("sinkPar5", C.c_double),
        ("nozzlePar1", C.c_double), ("nozzlePar2", C.c_double), ("nozzlePar3", C.c_double),
        ("nozzlePar4", C.c_double),
        ("NumRepts", C.c_int), ("NumSnaps", C.c_int), ("NumChecks", C.c_int),
        ("Out_LogTime", C.c_int), ("Initial_Regrid", C.c_int), ("restart_flag", C.c_int),
        ("include_atmos", C.c_int),
        ("MaxShort", C.c_double), ("MaxLong", C.c_double), ("Eccentricity", C.c_double),
        ("Drift_Rate", C.c_double), ("Drift_Exp", C.c_double),
    ]


class DiscoModules(C.Structure):
    _fields_ = [
        ("hydro", C.c_int), ("initial", C.c_int), ("boundary", C.c_int), ("planets", C.c_int),
        ("num_c", C.c_int), ("num_n", C.c_int), ("ct_mode", C.c_int),
        ("initial_name", C.c_char * 64), ("hydro_name", C.c_char * 64),
        ("boundary_name", C.c_char * 64), ("planets_name", C.c_char * 64),
        ("metric", C.c_int), ("frame", C.c_int),
        ("metric_name", C.c_char * 64), ("frame_name", C.c_char * 64),
        ("analysis", C.c_int), ("analysis_name", C.c_char * 64),
        ("geometry_name", C.c_char * 64), ("output_name", C.c_char * 64),
        ("restart_name", C.c_char * 64), ("hlld_name", C.c_char * 64),
    ]


class DiscoPlanet(C.Structure):
    _fields_ = [("r", C.c_double), ("phi", C.c_double), ("M", C.c_double),
                ("omega", C.c_double), ("vr", C.c_double), ("eps", C.c_double),
                ("type", C.c_int)]


class DiscoHostDomain(C.Structure):
    _fields_ = [
        ("par", DiscoParams), ("mod", DiscoModules),
        ("Nr", C.c_int), ("Nz", C.c_int), ("NgRa", C.c_int), ("NgRb", C.c_int),
        ("NgZa", C.c_int), ("NgZb", C.c_int),
        ("num_q", C.c_int), ("num_faces", C.c_int),
        ("Ncell", C.c_long),
        ("Np", C.POINTER(C.c_int)), ("ring_off", C.POINTER(C.c_long)),
        ("r_jph", C.POINTER(C.c_double)), ("z_kph", C.POINTER(C.c_double)),
        ("phi_max", C.c_double), ("t", C.c_double),
        ("piph", C.POINTER(C.c_double)), ("dphi", C.POINTER(C.c_double)),
        ("prim", C.POINTER(C.c_double)),
        ("Npl", C.c_int),
        ("planets", DiscoPlanet * 4),
        ("ic_aux", C.c_double * 4),
        ("Phi", C.POINTER(C.c_double)),
    ]


class DiscoStateView(C.Structure):
    _fields_ = [("piph", C.POINTER(C.c_double)), ("dphi", C.POINTER(C.c_double)),
                ("wiph", C.POINTER(C.c_double)), ("prim", C.POINTER(C.c_double)),
                ("cons", C.POINTER(C.c_double)), ("Phi", C.POINTER(C.c_double)),
                ("t", C.c_double)]


class DiscoKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_longlong), ("ms", C.c_double)]


class DiscoGpuErrs(C.Structure):
    _fields_ = [("nan_cells", C.c_longlong), ("rho_floor_hits", C.c_longlong),
                ("p_floor_hits", C.c_longlong), ("face_errors", C.c_longlong),
                ("steps", C.c_longlong), ("c2p_no_converge", C.c_longlong),
                ("async_timeouts", C.c_longlong)]


# Every symbol include/*.h declares, with its ctypes signature.
_P = C.c_void_p
SIGNATURES = {
    "disco_params_read": (C.c_int, [C.c_char_p, C.POINTER(DiscoParams)]),
    "disco_modules_read": (C.c_int, [C.c_char_p, C.POINTER(DiscoModules)]),
    "disco_host_setup": (C.c_int, [C.POINTER(DiscoParams), C.POINTER(DiscoModules),
                                   C.POINTER(C.POINTER(DiscoHostDomain))]),
    "disco_host_free": (None, [C.POINTER(DiscoHostDomain)]),
    "disco_host_restart": (C.c_int, [C.POINTER(DiscoParams), C.POINTER(DiscoModules), C.c_char_p,
                                     C.POINTER(C.POINTER(DiscoHostDomain))]),
    "disco_host_checkpoint": (C.c_int, [C.POINTER(DiscoHostDomain), C.c_char_p]),
    "disco_gpu_checkpoint": (C.c_int, [_P, C.POINTER(DiscoHostDomain), C.c_char_p]),
    "disco_gpu_create": (C.c_int, [C.POINTER(DiscoHostDomain), C.c_int, C.POINTER(_P)]),
    "disco_gpu_getmindt": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "disco_gpu_timestep": (C.c_int, [_P, C.c_double]),
    "disco_gpu_run": (C.c_int, [_P, C.c_int, C.c_double]),
    "disco_gpu_download": (C.c_int, [_P, C.POINTER(DiscoStateView)]),
    "disco_gpu_upload": (C.c_int, [_P, C.POINTER(DiscoStateView)]),
    "disco_gpu_status": (C.c_int, [_P, C.POINTER(DiscoGpuErrs)]),
    "disco_gpu_planets": (C.c_int, [_P, C.POINTER(DiscoPlanet), C.c_int, C.POINTER(C.c_int)]),
    "disco_gpu_run_timed": (C.c_int, [_P, C.c_int, C.c_double, C.c_size_t, C.POINTER(C.c_double)]),
    "disco_gpu_profile": (C.c_int, [_P, C.c_int, C.POINTER(DiscoKernelTime), C.c_int,
                                    C.POINTER(C.c_int)]),
    "disco_gpu_debug_ct": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "disco_gpu_debug_faces": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_long),
                                        C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "disco_gpu_debug_grad": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]),
    "disco_gpu_debug_convert": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_long,
                                          C.POINTER(C.c_float), C.POINTER(C.c_float),
                                          C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "disco_gpu_divb": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "disco_gpu_debug_sweep": (C.c_int, [_P, C.c_int]),
    "disco_gpu_getmindt_noalloc": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "disco_mlp_create": (C.c_int, [C.c_ulonglong, C.c_long, C.POINTER(_P)]),
    "disco_mlp_free": (None, [_P]),
    "disco_mlp_harvest": (C.c_int, [_P, _P, C.c_int, C.c_int, C.POINTER(C.c_long)]),
    "disco_mlp_pairs": (C.c_int, [_P, C.c_long, C.c_long, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "disco_mlp_fit_norm": (C.c_int, [_P]),
    "disco_mlp_train": (C.c_int, [_P, C.c_int, C.c_int, C.c_float, C.c_ulonglong, C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)]),
    "disco_mlp_grad": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float),
                                 C.POINTER(C.c_float)]),
    "disco_mlp_predict": (C.c_int, [_P, C.POINTER(C.c_float), C.c_long, C.POINTER(C.c_float)]),
    "disco_mlp_params": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(C.c_float)]),
    "disco_gpu_attach_guess": (C.c_int, [_P, _P]),
    "disco_mlp_set_gate": (C.c_int, [_P, C.c_double, C.c_double]),
    "disco_gpu_c2p_stats": (C.c_int, [_P, C.POINTER(C.c_longlong), C.c_int]),
    "disco_gpu_report": (C.c_int, [_P, C.POINTER(C.c_double), C.c_int]),
    "disco_gpu_diag_count": (C.c_int, [_P]),
    "disco_gpu_sink_accum": (C.c_int, [_P, C.POINTER(C.c_double), C.c_int, C.c_int]),
    "disco_gpu_diag_download": (C.c_int, [_P, C.POINTER(C.c_double), C.c_longlong, C.POINTER(C.c_double)]),
    "disco_gpu_diag_upload": (C.c_int, [_P, C.POINTER(C.c_double), C.c_longlong, C.c_double]),
    "disco_batch_create": (C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(_P)]),
    "disco_batch_create_flags": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int, C.POINTER(_P)]),
    "disco_batch_run": (C.c_int, [_P, C.c_int]),
    "disco_batch_run_timed": (C.c_int, [_P, C.c_int, C.c_size_t, C.POINTER(C.c_double)]),
    "disco_batch_free": (None, [_P]),
    "disco_batch_set_grid": (C.c_int, [_P, C.c_int]),
    "disco_batch_profile": (C.c_int, [_P, C.c_int, C.POINTER(DiscoKernelTime), C.c_int, C.POINTER(C.c_int)]),
    "disco_batch_set_split": (C.c_int, [_P, C.c_int]),
    "disco_batch_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "disco_gpu_time": (C.c_double, [_P]),
    "disco_gpu_num_cells": (C.c_long, [_P]),
    "disco_gpu_num_real_cells": (C.c_long, [_P]),
    "disco_gpu_free": (None, [_P]),
    "disco_gpu_launch_count": (C.c_longlong, []),
    "disco_last_error": (C.c_char_p, []),
    "disco_abi_version": (C.c_int, []),
}


def lib(build_if_missing: bool = True) -> C.CDLL:
    """Load libdisco_gb300.so (building it first if needed)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"native library missing: {path}")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class DiscoError(RuntimeError):
    pass


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = lib().disco_last_error().decode(errors="replace")
        raise DiscoError(f"{what} failed ({rc}): {msg}")


def read_params(in_par: str) -> DiscoParams:
    p = DiscoParams()
    _check(lib().disco_params_read(in_par.encode(), C.byref(p)), "disco_params_read")
    return p


def read_modules(makefile_opt: str) -> DiscoModules:
    m = DiscoModules()
    _check(lib().disco_modules_read(makefile_opt.encode(), C.byref(m)), "disco_modules_read")
    return m


class HostDomain:
    """Host-side grid + initial state (disco_host_setup), no GPU needed; with
    `restart` the grid and state of that checkpoint file (disco_host_restart)."""

    def __init__(self, params: DiscoParams, modules: DiscoModules, restart: str | None = None):
        ptr = C.POINTER(DiscoHostDomain)()
        if restart is None:
            _check(lib().disco_host_setup(C.byref(params), C.byref(modules), C.byref(ptr)),
                   "disco_host_setup")
        else:
            _check(lib().disco_host_restart(C.byref(params), C.byref(modules), restart.encode(),
                                            C.byref(ptr)), "disco_host_restart")
        self._ptr = ptr
        d = ptr.contents
        self.Nr, self.Nz = d.Nr, d.Nz
        self.NgRa, self.NgRb, self.NgZa, self.NgZb = d.NgRa, d.NgRb, d.NgZa, d.NgZb
        self.num_q = d.num_q
        self.Ncell = d.Ncell
        self.phi_max = d.phi_max
        self.t = d.t
        n = self.Ncell
        self.Np = np.ctypeslib.as_array(d.Np, (self.Nr * self.Nz,)).copy()
        self.ring_off = np.ctypeslib.as_array(d.ring_off, (self.Nr * self.Nz + 1,)).copy()
        self.r_jph = np.ctypeslib.as_array(d.r_jph, (self.Nr + 1,)).copy()
        self.z_kph = np.ctypeslib.as_array(d.z_kph, (self.Nz + 1,)).copy()
        self.piph = np.ctypeslib.as_array(d.piph, (n,)).copy()
        self.dphi = np.ctypeslib.as_array(d.dphi, (n,)).copy()
        self.prim = np.ctypeslib.as_array(d.prim, (self.num_q * n,)).copy().reshape(self.num_q, n)
        self.num_faces = d.num_faces
        self.Phi = (np.ctypeslib.as_array(d.Phi, (self.num_faces * n,)).copy().reshape(self.num_faces, n)
                    if d.Phi else None)
        self.Npl = d.Npl
        self.planets = [{k: getattr(d.planets[i], k) for k, _ in DiscoPlanet._fields_} for i in range(d.Npl)]
        self.params = d.par

    def checkpoint(self, path: str) -> None:
        """The checkpoint file of this host state (disco_host_checkpoint)."""
        _check(lib().disco_host_checkpoint(self._ptr, path.encode()), "disco_host_checkpoint")

    def real_mask(self) -> np.ndarray:
        jk = np.repeat(np.arange(self.Nr * self.Nz), self.Np)
        j, k = jk % self.Nr, jk // self.Nr
        return ((j >= self.NgRa) & (j < self.Nr - self.NgRb) &
                (k >= self.NgZa) & (k < self.Nz - self.NgZb))

    def __del__(self):
        if getattr(self, "_ptr", None) is not None and _lib is not None:
            _lib.disco_host_free(self._ptr)
            self._ptr = None


class Domain:
    """A domain resident on the GPU: the reference's getmindt/timestep pair."""

    def __init__(self, in_par: str, makefile_opt: str, precision: int = 0,
                 overrides: dict | None = None, restart: str | None = None):
        self.params = read_params(in_par)
        for k, v in (overrides or {}).items():
            setattr(self.params, k, v)
        self.modules = read_modules(makefile_opt)
        self.host = HostDomain(self.params, self.modules, restart=restart)
        g = C.c_void_p()
        _check(lib().disco_gpu_create(self.host._ptr, int(precision), C.byref(g)), "disco_gpu_create")
        self._g = g
        self.precision = precision

    # -- the reference's hot-path entry points -----------------------------
    def getmindt(self) -> float:
        dt = C.c_double()
        _check(lib().disco_gpu_getmindt(self._g, C.byref(dt)), "disco_gpu_getmindt")
        return dt.value

    def getmindt_noalloc(self) -> float:
        """getmindt through the no-allocation entry point (static scratch)."""
        dt = C.c_double()
        _check(lib().disco_gpu_getmindt_noalloc(self._g, C.byref(dt)), "disco_gpu_getmindt_noalloc")
        return dt.value

    REPORT_KEYS = ("t", "q", "Mass", "Torque", "Torque2") + tuple(
        f"Torque{i}_cut{n}" for n in range(5) for i in (1, 2))

    def report(self) -> dict:
        """report.c's domain sums from the device state (disco_gpu_report)."""
        out = (C.c_double * len(self.REPORT_KEYS))()
        rc = lib().disco_gpu_report(self._g, out, len(out))
        _check(rc if rc < 0 else 0, "disco_gpu_report")
        return {k: out[i] for i, k in enumerate(self.REPORT_KEYS)}

    SINK_KEYS = ("gravL", "dM", "accL", "Ls", "kin", "therm", "linXmom", "linYmom")

    def sink_accum(self, reset: bool = False) -> list:
        """The sink bodies' accumulators (disco_gpu_sink_accum): one dict per
        sink body, keys SINK_KEYS; reset zeroes them after the read."""
        out = (C.c_double * (8 * 4))()
        n = lib().disco_gpu_sink_accum(self._g, out, 4, int(reset))
        _check(n if n < 0 else 0, "disco_gpu_sink_accum")
        return [{k: out[8 * b + i] for i, k in enumerate(self.SINK_KEYS)} for b in range(n)]

    def diagnostics(self) -> dict:
        """analysis.c's ring diagnostics as timestep() accumulated them:
        Qrz [Nr*Nz, n] (ring jk = k*Nr + j) and t_avg (disco_gpu_diag_download).
        Qrz / t_avg is what the reference's output step writes."""
        n = lib().disco_gpu_diag_count(self._g)
        _check(n if n < 0 else 0, "disco_gpu_diag_count")
        nring = self.host.Nr * self.host.Nz
        q = np.zeros((nring, n), dtype=np.float64)
        t = C.c_double(0.0)
        rc = lib().disco_gpu_diag_download(self._g, q.ctypes.data_as(C.POINTER(C.c_double)), q.size,
                                           C.byref(t))
        _check(rc if rc < 0 else 0, "disco_gpu_diag_download")
        return {"Qrz": q, "t_avg": t.value}

    def set_diagnostics(self, Qrz=None, t_avg: float = 0.0) -> None:
        """Replace the accumulators (restart), or zero them when Qrz is None
        (zero_diagnostics)."""
        if Qrz is None:
            rc = lib().disco_gpu_diag_upload(self._g, None, 0, 0.0)
        else:
            a = np.ascontiguousarray(Qrz, dtype=np.float64)
            rc = lib().disco_gpu_diag_upload(self._g, a.ctypes.data_as(C.POINTER(C.c_double)), a.size,
                                             float(t_avg))
        _check(rc if rc < 0 else 0, "disco_gpu_diag_upload")

    def faces(self, dim: int) -> dict:
        """The device's sheared-face tables of dimension dim (1 = r, 2 = z):
        fIndex [npair+1] and per face L, R (global cell ids), LRtype, phic
        (cm[1]) and dA (disco_gpu_debug_faces)."""
        npair, nface = C.c_int(), C.c_long()
        _check(lib().disco_gpu_debug_faces(self._g, int(dim), C.byref(npair), C.byref(nface),
                                           None, None, None, None, None, None), "disco_gpu_debug_faces")
        out = {"fIndex": np.zeros(npair.value + 1, np.int32)}
        for k in ("L", "R", "LRtype"):
            out[k] = np.zeros(nface.value, np.int32)
        for k in ("phic", "dA"):
            out[k] = np.zeros(nface.value, np.float64)
        if npair.value == 0:
            return out
        ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
        _check(lib().disco_gpu_debug_faces(self._g, int(dim), C.byref(npair), C.byref(nface),
                                           *(out[k].ctypes.data_as(ip) for k in ("fIndex", "L", "R", "LRtype")),
                                           *(out[k].ctypes.data_as(dp) for k in ("phic", "dA"))),
               "disco_gpu_debug_faces")
        return out

    def gradients(self) -> dict:
        """plm_phi + plm_trans on the current state: gradp, gradr, gradz
        [num_q, Ncell] (disco_gpu_debug_grad)."""
        shp = (self.host.num_q, self.num_cells)
        out = {k: np.zeros(shp) for k in ("gradp", "gradr", "gradz")}
        dp = C.POINTER(C.c_double)
        _check(lib().disco_gpu_debug_grad(self._g, *(out[k].ctypes.data_as(dp) for k in ("gradp", "gradr", "gradz"))),
               "disco_gpu_debug_grad")
        return out

    def set_sweep(self, on: bool) -> bool:
        """Staged phi sweep (True) or separate plm_phi / flux_phi kernels;
        returns the setting in force (disco_gpu_debug_sweep)."""
        rc = lib().disco_gpu_debug_sweep(self._g, int(on))   # 2: copies withheld (timeout test)
        _check(rc if rc < 0 else 0, "disco_gpu_debug_sweep")
        return bool(rc)

    def divb(self) -> tuple:
        """(div, scale) per cell: net outward face flux of B and the sum of
        the absolute face fluxes (disco_gpu_divb); scale < 0 marks cells
        that are not evaluated."""
        n = self.num_cells
        div, sc = np.zeros(n), np.zeros(n)
        dp = C.POINTER(C.c_double)
        _check(lib().disco_gpu_divb(self._g, div.ctypes.data_as(dp), sc.ctypes.data_as(dp)), "disco_gpu_divb")
        return div, sc

    def attach_guess(self, mlp) -> None:
        """Start the GRMHD cons2prim from mlp's guess (None: from the previous
        primitives only)."""
        _check(lib().disco_gpu_attach_guess(self._g, None if mlp is None else mlp._m), "disco_gpu_attach_guess")

    def c2p_stats(self, reset: bool = False) -> dict:
        """Newton cons2prim counters: calls, summed k_converge, summed
        iterations, calls started from the guess."""
        out = (C.c_longlong * 4)()
        _check(lib().disco_gpu_c2p_stats(self._g, out, int(reset)), "disco_gpu_c2p_stats")
        return {"calls": out[0], "kconv": out[1], "iters": out[2], "guessed": out[3]}

    def timestep(self, dt: float) -> None:
        _check(lib().disco_gpu_timestep(self._g, float(dt)), "disco_gpu_timestep")

    def run(self, nsteps: int, t_end: float = 0.0) -> None:
        _check(lib().disco_gpu_run(self._g, int(nsteps), float(t_end)), "disco_gpu_run")

    def run_timed(self, nsteps: int, t_end: float = 0.0, flush_bytes: int = 0) -> float:
        """Run n steps; returns summed device milliseconds (CUDA events)."""
        ms = C.c_double()
        _check(lib().disco_gpu_run_timed(self._g, int(nsteps), float(t_end), int(flush_bytes),
                                         C.byref(ms)), "disco_gpu_run_timed")
        return ms.value

    def profile(self, nsteps: int) -> list:
        """Per-kernel (name, launches, ms) over n steps launched without graphs."""
        out = (DiscoKernelTime * 64)()
        n = C.c_int()
        _check(lib().disco_gpu_profile(self._g, int(nsteps), out, 64, C.byref(n)), "disco_gpu_profile")
        return [(out[i].name.decode(), out[i].launches, out[i].ms) for i in range(n.value)]

    @property
    def t(self) -> float:
        return lib().disco_gpu_time(self._g)

    @property
    def num_cells(self) -> int:
        return lib().disco_gpu_num_cells(self._g)

    @property
    def num_real_cells(self) -> int:
        return lib().disco_gpu_num_real_cells(self._g)

    def checkpoint(self, path: str) -> None:
        """Write the checkpoint file of the device state (disco_gpu_checkpoint):
        the layout of the reference's h5out.c output(); the ring diagnostics
        are averaged into the file and zeroed, as output() does."""
        _check(lib().disco_gpu_checkpoint(self._g, self.host._ptr, path.encode()), "disco_gpu_checkpoint")

    def state(self, out: dict | None = None) -> dict:
        """Download the state.  `out` may hold preallocated C-contiguous
        float64 arrays (e.g. in pinned memory) for any of the keys, of the
        shapes this method would allocate; they are filled in place."""
        n = self.num_cells
        q = self.host.num_q
        out = dict(out or {})
        shapes = {"piph": (n,), "dphi": (n,), "wiph": (n,), "prim": (q, n), "cons": (q, n)}
        if self.host.num_q >= 8:
            shapes["Phi"] = (5, n)
        for k, shp in shapes.items():
            if k not in out:
                out[k] = np.zeros(shp) if k == "Phi" else np.empty(shp)
            a = out[k]
            if a.shape != shp or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError(f"state(out): {k} must be C-contiguous float64 of shape {shp}")
        v = DiscoStateView()
        dp = C.POINTER(C.c_double)
        for k in ("piph", "dphi", "wiph", "prim", "cons", "Phi"):
            if k in out:
                setattr(v, k, out[k].ctypes.data_as(dp))
        _check(lib().disco_gpu_download(self._g, C.byref(v)), "disco_gpu_download")
        out["t"] = v.t
        return out

    def upload(self, **arrays) -> None:
        v = DiscoStateView()
        dp = C.POINTER(C.c_double)
        keep = []
        for k in ("piph", "dphi", "wiph", "prim", "cons", "Phi"):
            if k in arrays:
                a = np.ascontiguousarray(arrays[k], dtype=np.float64)
                keep.append(a)
                setattr(v, k, a.ctypes.data_as(dp))
        _check(lib().disco_gpu_upload(self._g, C.byref(v)), "disco_gpu_upload")

    def planets(self) -> list:
        """The point masses as the device has advanced them."""
        out = (DiscoPlanet * 4)()
        n = C.c_int()
        _check(lib().disco_gpu_planets(self._g, out, 4, C.byref(n)), "disco_gpu_planets")
        return [{k: getattr(out[i], k) for k, _ in DiscoPlanet._fields_} for i in range(min(n.value, 4))]

    def status(self) -> dict:
        e = DiscoGpuErrs()
        _check(lib().disco_gpu_status(self._g, C.byref(e)), "disco_gpu_status")
        return {k: getattr(e, k) for k, _ in DiscoGpuErrs._fields_}

    def close(self) -> None:
        if getattr(self, "_g", None):
            lib().disco_gpu_free(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


MLP_FEATURES, MLP_OUTPUTS, MLP_PARAMS, MLP_NORM = 10, 2, 5768, 24


class Mlp:
    """The learned starting point of the GRMHD Newton cons2prim
    (include/disco_gpu_mlp.h): a 2 x 64 MLP trained and evaluated by the
    library's BF16 tensor-core kernels."""

    def __init__(self, seed: int = 1, capacity: int = 1 << 21):
        m = C.c_void_p()
        _check(lib().disco_mlp_create(int(seed), int(capacity), C.byref(m)), "disco_mlp_create")
        self._m = m

    def harvest(self, dom: "Domain", stride: int = 1, steps: int = 1) -> int:
        """Advance dom by `steps` steps from the reference's start, recording
        a training pair for every stride-th real cell at every cons2prim;
        returns the pairs held."""
        n = C.c_long()
        _check(lib().disco_mlp_harvest(self._m, dom._g, int(stride), int(steps), C.byref(n)), "disco_mlp_harvest")
        return n.value

    def pairs(self, first: int, n: int) -> tuple:
        X = np.zeros((n, MLP_FEATURES), np.float32)
        Y = np.zeros((n, MLP_OUTPUTS), np.float32)
        fp = C.POINTER(C.c_float)
        _check(lib().disco_mlp_pairs(self._m, int(first), int(n), X.ctypes.data_as(fp), Y.ctypes.data_as(fp)),
               "disco_mlp_pairs")
        return X, Y

    def fit_norm(self) -> None:
        _check(lib().disco_mlp_fit_norm(self._m), "disco_mlp_fit_norm")

    def train(self, steps: int, batch: int = 4096, lr: float = 1e-3, seed: int = 7) -> tuple:
        """steps of Adam; returns (loss of the first batch, of the last)."""
        a, b = C.c_float(), C.c_float()
        _check(lib().disco_mlp_train(self._m, int(steps), int(batch), float(lr), int(seed), C.byref(a), C.byref(b)),
               "disco_mlp_train")
        return a.value, b.value

    def grad(self, X: np.ndarray, Y: np.ndarray) -> tuple:
        """(summed squared error, gradient of its mean) over given pairs."""
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = C.c_float()
        fp = C.POINTER(C.c_float)
        _check(lib().disco_mlp_grad(self._m, X.ctypes.data_as(fp), Y.ctypes.data_as(fp), len(X), C.byref(loss),
                                    g.ctypes.data_as(fp)), "disco_mlp_grad")
        return loss.value, g

    def set_gate(self, floor: float = 0.0, ratio: float = 1.0) -> None:
        """cons2prim takes the model's start where the previous primitives'
        residual is above floor and the model's is below ratio times it
        (used at the next attach)."""
        _check(lib().disco_mlp_set_gate(self._m, float(floor), float(ratio)), "disco_mlp_set_gate")

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((len(X), MLP_OUTPUTS), np.float32)
        fp = C.POINTER(C.c_float)
        _check(lib().disco_mlp_predict(self._m, X.ctypes.data_as(fp), len(X), Y.ctypes.data_as(fp)),
               "disco_mlp_predict")
        return Y

    def params(self) -> tuple:
        p = np.zeros(MLP_PARAMS, np.float32)
        nm = np.zeros(MLP_NORM, np.float32)
        fp = C.POINTER(C.c_float)
        _check(lib().disco_mlp_params(self._m, p.ctypes.data_as(fp), None, nm.ctypes.data_as(fp), None),
               "disco_mlp_params")
        return p, nm

    def set_params(self, p=None, norm=None) -> None:
        fp = C.POINTER(C.c_float)
        pa = None if p is None else np.ascontiguousarray(p, np.float32)
        na = None if norm is None else np.ascontiguousarray(norm, np.float32)
        _check(lib().disco_mlp_params(self._m, None, None if pa is None else pa.ctypes.data_as(fp), None,
                                      None if na is None else na.ctypes.data_as(fp)), "disco_mlp_params")

    def close(self) -> None:
        if getattr(self, "_m", None) is not None and self._m.value:
            lib().disco_mlp_free(self._m)
            self._m = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def convert_check(x: np.ndarray, y: np.ndarray) -> dict:
    """The mixed path's integer-pipe conversions beside the hardware's, on
    the device: f_int / f_hw from the float64 array x, d_int / d_hw from the
    float32 array y (same length)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float32)
    if x.shape != y.shape:
        raise ValueError("convert_check: x and y must have the same length")
    n = x.size
    out = {"f_int": np.zeros(n, np.float32), "f_hw": np.zeros(n, np.float32),
           "d_int": np.zeros(n, np.float64), "d_hw": np.zeros(n, np.float64)}
    fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
    _check(lib().disco_gpu_debug_convert(x.ctypes.data_as(dp), y.ctypes.data_as(fp), n,
                                         out["f_int"].ctypes.data_as(fp), out["f_hw"].ctypes.data_as(fp),
                                         out["d_int"].ctypes.data_as(dp), out["d_hw"].ctypes.data_as(dp)),
           "disco_gpu_debug_convert")
    return out


class Batch:
    """Independent domains advanced together (disco_gpu_batch.h): each step is
    one CUDA-graph launch, every member using its own CFL dt; members of one
    module, precision and launch sequence are advanced by multi-instance
    stage kernels.  The members stay usable on their own (state(), status())."""

    def __init__(self, members: list, groups: bool = True):
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m._g.value for m in self.members])
        b = C.c_void_p()
        _check(lib().disco_batch_create_flags(arr, len(self.members), 0 if groups else 1, C.byref(b)),
               "disco_batch_create")
        self._b = b

    @property
    def num_real_cells(self) -> int:
        return sum(m.num_real_cells for m in self.members)

    def run(self, nsteps: int) -> None:
        _check(lib().disco_batch_run(self._b, int(nsteps)), "disco_batch_run")

    def run_timed(self, nsteps: int, flush_bytes: int = 0) -> float:
        ms = C.c_double()
        _check(lib().disco_batch_run_timed(self._b, int(nsteps), int(flush_bytes), C.byref(ms)),
               "disco_batch_run_timed")
        return ms.value

    def set_grid(self, ctas_per_sm: int) -> None:
        """At most this many blocks per SM in the multi-instance stage kernels."""
        _check(lib().disco_batch_set_grid(self._b, int(ctas_per_sm)), "disco_batch_set_grid")

    def set_split(self, split: int) -> None:
        """Sub-groups per group (0: every member on its own sequence; -1:
        choose by timing the candidates)."""
        _check(lib().disco_batch_set_split(self._b, int(split)), "disco_batch_set_split")

    def profile(self, nsteps: int) -> list:
        """Per stage of the groups: (name, launches, summed ms) over nsteps
        steps launched without the graph (disco_batch_profile)."""
        out = (DiscoKernelTime * 64)()
        n = C.c_int()
        _check(lib().disco_batch_profile(self._b, int(nsteps), out, 64, C.byref(n)), "disco_batch_profile")
        return [(out[i].name.decode(), out[i].launches, out[i].ms) for i in range(n.value)]

    def info(self) -> dict:
        g, k, sp, c = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        t = (C.c_double * 6)()
        _check(lib().disco_batch_info(self._b, C.byref(g), C.byref(k), C.byref(sp), C.byref(c), t),
               "disco_batch_info")
        return {"groups": g.value, "grouped_members": k.value, "split": sp.value, "ctas_per_sm": c.value,
                "tune_ms": {n: t[i] for i, n in enumerate((1, 2, 4, 8, 16, 0))}}

    def close(self) -> None:
        if getattr(self, "_b", None) is not None and self._b.value:
            lib().disco_batch_free(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
