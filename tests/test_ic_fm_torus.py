"""The Fishbone-Moncrief torus initial condition in Kerr-Schild cylindrical
coordinates (disco_gb300/csrc/plugins/ic_fm_torus.h), checked on the CPU
through its defining properties: ell = u^t u_phi is the same constant in
every torus cell and equals the circular-orbit value at r_pk; the motion is
purely azimuthal (u^r = u^z = 0); rho peaks at 1 at the pressure maximum and
vanishes at the inner edge; the field is divergence-free and normalised to
max P / max(B^2/2) = beta."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PL = os.path.join(ROOT, "disco_gb300", "csrc", "plugins")

_SRC = r'''
#include "%s/ic_fm_torus.h"
static struct disco_ic_fm P;
void setup(double M, double a, double rin, double rpk, double beta, double acut, double gam) {
   P.gam = gam; P.M = M; P.a = a; P.rin = rin; P.rpk = rpk; P.beta = beta; P.acut = acut;
   P.rho_atm = 1e-6; P.cs2_atm = 1e-8;
   disco_ic_fm_setup(&P);
}
double get(int i) { double v[4] = {P.ell, P.F_in, P.hpk1, P.bscale}; return v[i]; }
void eval(double r, double z, double *prim) { double x[3] = {r, 0.3, z}; disco_ic_fm_eval(&P, prim, x, 8, 9); }
void g3(double r, double z, double *out) {
   double x[3] = {r, 0.0, z};
   disco_kerr_3p1(x, P.M, P.a, out, out + 1, out + 4, out + 13);
}
'''

GAM, M, A, RIN, RPK, BETA, ACUT = 4.0 / 3.0, 1.0, 0.9, 6.0, 12.0, 100.0, 0.2


@pytest.fixture(scope="module")
def fm():
    td = tempfile.mkdtemp(prefix="disco_fm_")
    src = os.path.join(td, "fm.c")
    with open(src, "w") as f:
        f.write(_SRC % PL)
    so = os.path.join(td, "fm.so")
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", src, "-o", so, "-lm"],
                   check=True)
    L = C.CDLL(so)
    L.setup.argtypes = [C.c_double] * 7
    L.get.restype = C.c_double
    L.get.argtypes = [C.c_int]
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    L.eval.argtypes = [C.c_double, C.c_double, dp]
    L.g3.argtypes = [C.c_double, C.c_double, dp]
    L.setup(M, A, RIN, RPK, BETA, ACUT, GAM)

    class F:
        def prim(self, r, z):
            p = np.zeros(9); L.eval(r, z, p); return p

        def metric(self, r, z):
            o = np.zeros(22); L.g3(r, z, o)
            return o[0], o[1:4], o[4:13].reshape(3, 3), o[13:22].reshape(3, 3)
        ell = L.get(0)
        bscale = L.get(3)
    return F()


def _four_velocity(fm, r, z, p):
    al, be, gam, igam = fm.metric(r, z)
    u = np.array([p[2], p[3] * r * r, p[4]])     # u_r, u_phi, u_z
    W = np.sqrt(1.0 + u @ igam @ u)
    ut = W / al
    ui = igam @ u - W * be / al                 # u^i = gamma^ij u_j - W beta^i / alpha
    return ut, ui, u


def test_constant_angular_momentum_and_azimuthal_motion(fm):
    n = 0
    for r in np.linspace(7.0, 30.0, 24):
        for z in np.linspace(-8.0, 8.0, 17):
            p = fm.prim(r, z)
            if p[8] != 1.0:
                continue
            n += 1
            ut, ui, u = _four_velocity(fm, r, z, p)
            assert ut * u[1] == pytest.approx(fm.ell, rel=1e-10)
            assert abs(ui[0]) < 1e-12 and abs(ui[2]) < 1e-12
            assert ui[1] > 0.0
    assert n > 100


def test_density_peak_and_inner_edge(fm):
    rpk_cyl = np.sqrt(RPK ** 2 + A ** 2)
    assert fm.prim(rpk_cyl, 0.0)[0] == pytest.approx(1.0, rel=1e-12)
    for dr in (-0.3, 0.3):
        assert fm.prim(rpk_cyl + dr, 0.0)[0] < 1.0
    assert fm.prim(rpk_cyl, 0.5)[0] < 1.0
    rin_cyl = np.sqrt(RIN ** 2 + A ** 2)
    assert fm.prim(rin_cyl - 0.01, 0.0)[0] == 1e-6       # atmosphere inside r_in
    assert fm.prim(rin_cyl + 0.05, 0.0)[0] < 1e-3
    # the atmosphere is at rest for the normal observer
    p = fm.prim(3.0, 15.0)
    assert p[0] == 1e-6 and p[1] == pytest.approx(1e-14) and not np.any(p[2:5])


def test_field_divergence_free_and_normalised(fm):
    assert fm.bscale > 0
    h = 1e-3
    worst, scale = 0.0, 0.0
    for r in np.linspace(9.0, 20.0, 12):
        for z in np.linspace(-3.0, 3.0, 9):
            def rb(rr, zz):
                p = fm.prim(rr, zz)
                return rr * p[5], rr * p[7]
            d = (rb(r + h, z)[0] - rb(r - h, z)[0]) / (2 * h) + (rb(r, z + h)[1] - rb(r, z - h)[1]) / (2 * h)
            worst = max(worst, abs(d))
            scale = max(scale, abs(rb(r, z)[0]) + abs(rb(r, z)[1]))
    assert worst < 1e-3 * scale
    # max P / max (B^2 / 2) = beta on a lattice
    pmax, pmag = 0.0, 0.0
    for r in np.linspace(6.5, 40.0, 120):
        for z in np.linspace(-12.0, 12.0, 97):
            p = fm.prim(r, z)
            if p[8] != 1.0:
                continue
            al, be, gam, igam = fm.metric(r, z)
            B = al * np.array([p[5], 0.0, p[7]])
            pmax = max(pmax, p[1])
            pmag = max(pmag, 0.5 * B @ gam @ B)
    assert pmax / pmag == pytest.approx(BETA, rel=0.1)
