"""ctypes wrapper of oracle/_ref/libref_kat.so: the reference's own
constraint and projector arithmetic (built from the reference's sources by
oracle/ref/Makefile). Test infrastructure: used by tests/golden/make_ref_golden.py
to write the committed vectors and by tests/test_ref_pin.py when the library
is present."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(os.path.dirname(HERE), "_ref", "libref_kat.so")
_lib = None


def available() -> bool:
    """True when the reference checkout is here (its library can be built)."""
    return subprocess.run(["make", "-s", "-C", HERE, "available"], capture_output=True).returncode == 0


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P, I, D, LL = C.c_void_p, C.c_int, C.c_double, C.c_longlong
        L.ref_rest.argtypes = [P, D, D, P, P, P, P, P]
        L.ref_eval.argtypes = [P, P, D, D, P, P, P, P]
        L.ref_project_combined.argtypes = [P, P, P, D, D, D, I, P, P, P]
        L.ref_project_single.argtypes = [I, P, P, P, D, D, D, I, P, P]
        L.ref_project_collision.argtypes = [P, P, P, P, D, D, D, D, I, P, P]
        L.ref_gs_steps.argtypes = [LL, P, P, LL, P, P, P, P, P, D, D, I, I, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _c(a, dt=np.float64):
    return np.ascontiguousarray(a, dt)


def rest(X4, E, nu):
    X4 = _c(X4)
    Q = np.zeros(9)
    out = np.zeros(4)
    lib().ref_rest(_p(X4), E, nu, _p(Q), _p(out[0:]), _p(out[1:]), _p(out[2:]), _p(out[3:]))
    return Q, out  # out = vol, alpha_dev, alpha_hyd, gamma


def evaluate(X4, x4, E, nu):
    X4, x4 = _c(X4), _c(x4)
    c = np.zeros(2)
    gd, gh = np.zeros(12), np.zeros(12)
    lib().ref_eval(_p(X4), _p(x4), E, nu, _p(c[0:]), _p(c[1:]), _p(gd), _p(gh))
    return c, gd, gh


def project_combined(X4, x4, m4, E, nu, dt, nproj):
    X4, x4, m4 = _c(X4), _c(x4), _c(m4)
    dx, lam, xo = np.zeros((nproj, 12)), np.zeros((nproj, 2)), np.zeros(12)
    lib().ref_project_combined(_p(X4), _p(x4), _p(m4), E, nu, dt, nproj, _p(dx), _p(lam), _p(xo))
    return dx, lam, xo


def project_single(which, X4, x4, m4, E, nu, dt, nproj):
    X4, x4, m4 = _c(X4), _c(x4), _c(m4)
    dx, xo = np.zeros((nproj, 12)), np.zeros(12)
    lib().ref_project_single(which, _p(X4), _p(x4), _p(m4), E, nu, dt, nproj, _p(dx), _p(xo))
    return dx, xo


def project_collision(x3, m3, p, n, u, v, w, dt, nproj):
    x3, m3, p, n = _c(x3), _c(m3), _c(p), _c(n)
    dx, xo = np.zeros((nproj, 9)), np.zeros(9)
    lib().ref_project_collision(_p(x3), _p(m3), _p(p), _p(n), u, v, w, dt, nproj, _p(dx), _p(xo))
    return dx, xo


def gs_steps(X, tets, E, nu, rho, fixed, dt, g, num_iter, nsteps, x0=None):
    X, tets = _c(X), _c(tets, np.int32)
    T, V = tets.shape[0], X.shape[0]
    E, nu, rho = (_c(np.broadcast_to(a, (T,))) for a in (E, nu, rho))
    fixed = _c(fixed, np.uint8)
    x0 = None if x0 is None else _c(x0)
    xo, lam = np.zeros((V, 3)), np.zeros((T, 2))
    lib().ref_gs_steps(V, _p(X), _p(x0), T, _p(tets), _p(E), _p(nu), _p(rho), _p(fixed), dt, g, num_iter, nsteps,
                       _p(xo), _p(lam))
    return xo, lam
