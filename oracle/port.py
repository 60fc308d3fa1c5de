"""ctypes binding of the C port in ``d2q9_port.c`` -- TEST INFRASTRUCTURE ONLY.

Loaded by the tests as a second checker and by ``bench.py`` as the timed
CPU baseline.  The shared object is built by ``make -C oracle`` (called from
``__graft_entry__.build()``) into ``oracle/_build/``.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_d2q9.so")

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P, I64, I, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        for suf in ("f64", "f32"):
            getattr(L, "oracle_equilibrium_" + suf).argtypes = [P, P, P, P, I64, I64, I]
            getattr(L, "oracle_collide_" + suf).argtypes = [P, I64, I64, D, I]
            getattr(L, "oracle_stream_periodic_" + suf).argtypes = [P, P, I, I, I]
            getattr(L, "oracle_stream_bb_" + suf).argtypes = [P, P, I, I, D, I]
            getattr(L, "oracle_cavity_run_" + suf).argtypes = [P, P, I, I, D, D, I, I]
            getattr(L, "oracle_cavity_run_" + suf).restype = I
            getattr(L, "oracle_periodic_run_" + suf).argtypes = [P, P, I, I, D, I, I]
            getattr(L, "oracle_periodic_run_" + suf).restype = I
        L.oracle_max_threads.restype = I
        L.oracle_mass_momentum_f64.argtypes = [P, I64, P]
        _lib = L
    return _lib


def _suf(a):
    if a.dtype == np.float64:
        return "f64"
    if a.dtype == np.float32:
        return "f32"
    raise TypeError("oracle port supports float32/float64, got %s" % a.dtype)


def _p(a):
    assert a.flags.c_contiguous
    return a.ctypes.data


def max_threads():
    return lib().oracle_max_threads()


def collide(f2d, omega, nthreads=1):
    getattr(lib(), "oracle_collide_" + _suf(f2d))(_p(f2d), f2d.shape[1], f2d.shape[1], omega, nthreads)


def equilibrium(rho, ux, uy, f2d, nthreads=1):
    n = rho.size
    getattr(lib(), "oracle_equilibrium_" + _suf(f2d))(_p(rho), _p(ux), _p(uy), _p(f2d), n, f2d.shape[1], nthreads)


def stream(f, nthreads=1):
    g = f.copy()
    getattr(lib(), "oracle_stream_periodic_" + _suf(f))(_p(g), _p(f), f.shape[1], f.shape[2], nthreads)


def stream_and_bounce_back(f, u0=0.1, nthreads=1):
    g = f.copy()
    getattr(lib(), "oracle_stream_bb_" + _suf(f))(_p(g), _p(f), f.shape[1], f.shape[2], u0, nthreads)


def cavity_run(f, omega, u0, nsteps, nthreads=0, scratch=None):
    """Run ``nsteps`` cavity steps in place on ``f``; returns ``f``."""
    b = np.empty_like(f) if scratch is None else scratch
    which = getattr(lib(), "oracle_cavity_run_" + _suf(f))(_p(f), _p(b), f.shape[1], f.shape[2],
                                                           omega, u0, nsteps, nthreads)
    if which == 1:
        f[...] = b
    return f


def run_raw(a, b, boundary, omega, u0, nsteps, nthreads=0):
    """``nsteps`` steps ping-ponging between ``a`` and ``b`` without copies;
    returns the buffer that holds the result."""
    L = lib()
    if boundary == "cavity":
        which = getattr(L, "oracle_cavity_run_" + _suf(a))(_p(a), _p(b), a.shape[1], a.shape[2], omega, u0,
                                                           nsteps, nthreads)
    else:
        which = getattr(L, "oracle_periodic_run_" + _suf(a))(_p(a), _p(b), a.shape[1], a.shape[2], omega,
                                                             nsteps, nthreads)
    return b if which == 1 else a


def periodic_run(f, omega, nsteps, nthreads=0):
    b = np.empty_like(f)
    which = getattr(lib(), "oracle_periodic_run_" + _suf(f))(_p(f), _p(b), f.shape[1], f.shape[2],
                                                             omega, nsteps, nthreads)
    if which == 1:
        f[...] = b
    return f


def mass_momentum(f):
    out = np.zeros(3)
    f = np.ascontiguousarray(f, dtype=np.float64)
    lib().oracle_mass_momentum_f64(_p(f), f[0].size, _p(out))
    return out
