"""The Kerr-Schild cylindrical metric (disco_gb300/csrc/plugins/
metric_kerr.h) checked on the CPU: its derivatives against centred finite
differences of the metric itself, the 3+1 pieces against the 4-metric
(lapse, shift and spatial metric reassemble g_mu,nu; gamma^ij inverts
gamma_ij), det g = -r^2, and the a = 0 case against the reference's
Schwarzschild Kerr-Schild formulas (Hydro/Metric/schw_ks_rpz.c)."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "disco_gb300", "csrc", "plugins", "metric_kerr.h")

_SRC = r'''
#include "%s"
void g4(const double *x, double M, double a, double *g) {
   double al, be[3], gam[9];
   disco_kerr_3p1(x, M, a, &al, be, gam, 0);
   double bd[3] = {0, 0, 0};
   for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) bd[i] += gam[3*i + j]*be[j];
   double b2 = bd[0]*be[0] + bd[1]*be[1] + bd[2]*be[2];
   g[0] = -al*al + b2;
   for(int i = 0; i < 3; i++) { g[i + 1] = bd[i]; g[4*(i + 1)] = bd[i]; }
   for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) g[4*(i + 1) + j + 1] = gam[3*i + j];
}
void p3(const double *x, double M, double a, double *out) {
   disco_kerr_3p1(x, M, a, out, out + 1, out + 4, out + 13);
}
void dg(const double *x, double M, double a, int i, double *out) { disco_kerr_der_g(x, M, a, i, out); }
void da(const double *x, double M, double a, double *out) { disco_kerr_der_lapse(x, M, a, out); }
void db(const double *x, double M, double a, double *out) { disco_kerr_der_shift(x, M, a, out); }
'''


@pytest.fixture(scope="module")
def kerr():
    td = tempfile.mkdtemp(prefix="disco_kerr_")
    src = os.path.join(td, "k.c")
    with open(src, "w") as f:
        f.write(_SRC % HDR)
    so = os.path.join(td, "k.so")
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", src, "-o", so, "-lm"],
                   check=True)
    L = C.CDLL(so)
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    for n in ("g4", "p3", "da", "db"):
        getattr(L, n).argtypes = [dp, C.c_double, C.c_double, dp]
    L.dg.argtypes = [dp, C.c_double, C.c_double, C.c_int, dp]

    class K:
        def g(self, x, M, a):
            o = np.zeros(16); L.g4(np.asarray(x, float), M, a, o); return o.reshape(4, 4)

        def p3(self, x, M, a):
            o = np.zeros(22); L.p3(np.asarray(x, float), M, a, o)
            return o[0], o[1:4], o[4:13].reshape(3, 3), o[13:22].reshape(3, 3)

        def dg(self, x, M, a, i):
            o = np.zeros(16); L.dg(np.asarray(x, float), M, a, i, o); return o.reshape(4, 4)

        def da(self, x, M, a):
            o = np.zeros(4); L.da(np.asarray(x, float), M, a, o); return o

        def db(self, x, M, a):
            o = np.zeros(12); L.db(np.asarray(x, float), M, a, o); return o.reshape(4, 3)
    return K()


POINTS = [(3.0, 0.4, 0.0), (2.0, 0.0, 1.5), (7.5, 2.0, -3.0), (12.0, 5.0, 0.7), (25.0, 0.1, 18.0)]


@pytest.mark.parametrize("a", [0.0, 0.5, 0.9])
@pytest.mark.parametrize("x", POINTS)
def test_metric_is_kerr_schild(kerr, x, a):
    M = 1.0
    g = kerr.g(x, M, a)
    r, z = x[0], x[2]
    # null-vector form: g = eta + H l l with l_t = 1, so g_tt + 1 = H and
    # the t row gives l; eta = diag(-1, 1, r^2, 1)
    H = g[0, 0] + 1.0
    l = g[0] / H
    l[0] = 1.0
    eta = np.diag([-1.0, 1.0, r * r, 1.0])
    assert np.allclose(g, eta + H * np.outer(l, l), rtol=1e-13, atol=1e-13)
    # l is null with respect to both eta and g
    ieta = np.diag([-1.0, 1.0, 1.0 / (r * r), 1.0])
    assert abs(l @ ieta @ l) < 1e-13
    # sqrt(-g) = r
    assert np.linalg.det(g) == pytest.approx(-r * r, rel=1e-12)
    # R solves its quartic; at large distance the metric tends to flat
    al, be, gam, igam = kerr.p3(x, M, a)
    assert np.allclose(gam @ igam, np.eye(3), atol=1e-12)
    assert 0.0 < al < 1.0


@pytest.mark.parametrize("a", [0.0, 0.9])
@pytest.mark.parametrize("x", POINTS)
def test_derivatives_match_finite_differences(kerr, x, a):
    M = 1.0
    x = np.asarray(x, float)
    for i, ax in ((1, 0), (3, 2)):
        h = 1e-5 * max(1.0, abs(x[ax]))
        xp, xm = x.copy(), x.copy()
        xp[ax] += h
        xm[ax] -= h
        fd = (kerr.g(xp, M, a) - kerr.g(xm, M, a)) / (2 * h)
        assert np.allclose(kerr.dg(x, M, a, i), fd, rtol=1e-6, atol=1e-8), i
        fda = (kerr.p3(xp, M, a)[0] - kerr.p3(xm, M, a)[0]) / (2 * h)
        assert kerr.da(x, M, a)[i] == pytest.approx(fda, rel=1e-6, abs=1e-9)
        fdb = (kerr.p3(xp, M, a)[1] - kerr.p3(xm, M, a)[1]) / (2 * h)
        assert np.allclose(kerr.db(x, M, a)[i], fdb, rtol=1e-6, atol=1e-9)
    for i in (0, 2):   # Killing directions
        assert not np.any(kerr.dg(x, M, a, i))
        assert kerr.da(x, M, a)[i] == 0.0
        assert not np.any(kerr.db(x, M, a)[i])


@pytest.mark.parametrize("x", POINTS)
def test_zero_spin_is_the_references_schwarzschild(kerr, x):
    """a = 0 against the formulas of schw_ks_rpz.c (metric_lapse :20,
    metric_shift :26, metric_gam :39, metric_der_g :93)."""
    M = 1.0
    r, _, z = x
    R = np.hypot(r, z)
    H = 2 * M / R
    st, ct = r / R, z / R
    al, be, gam, igam = kerr.p3(x, M, 0.0)
    assert al == pytest.approx(1 / np.sqrt(1 + H), rel=1e-14)
    assert np.allclose(be, [2 * M * r / R ** 2 / (1 + H), 0, 2 * M * z / R ** 2 / (1 + H)], rtol=1e-14)
    ref = np.array([[1 + H * st * st, 0, H * st * ct], [0, r * r, 0], [H * st * ct, 0, 1 + H * ct * ct]])
    assert np.allclose(gam, ref, rtol=1e-14, atol=1e-15)
    d = kerr.dg(x, M, 0.0, 1)
    MoR2, MoR3 = M / R ** 2, M / R ** 3
    assert d[0, 0] == pytest.approx(-2 * MoR2 * st, rel=1e-12)
    assert d[1, 1] == pytest.approx(2 * MoR3 * r * (2 - 3 * st * st), rel=1e-12)
    assert d[2, 2] == pytest.approx(2 * r, rel=1e-14)
