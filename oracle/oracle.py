"""ctypes front end of the CPU oracle (liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The engine never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

import sys
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from qdng_gb300 import abi  # noqa: E402  (data layouts only)

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


# Builds of the same source: the parity oracle ("", -O2, IEEE arithmetic)
# and two timed CPU baselines ("o3": -O3 -funroll-loops; "fast": also
# -ffast-math, QDng's configure default for optimised builds).
VARIANTS = {"": "liborc.so", "o3": "liborc_o3.so", "fast": "liborc_fast.so"}


def build(force=False, variant=""):
    """Compile the oracle libraries with the committed Makefile (g++, OpenMP)."""
    so = os.path.join(_HERE, VARIANTS[variant])
    src = os.path.join(_HERE, "qdng_oracle.cpp")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, VARIANTS[variant]])
    return so


def use_variant(variant):
    """Load a timed-baseline build instead of the parity oracle (before the
    first call; bench.py's CPU legs only)."""
    global _LIB, _VARIANT
    if _LIB is not None and _VARIANT != variant:
        raise RuntimeError("the oracle library is already loaded")
    _VARIANT = variant


_VARIANT = ""


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(build(variant=_VARIANT))
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        L.orc_last_error.restype = C.c_char_p
        L.orc_num_threads.argtypes = [C.c_int]
        L.orc_fft1.argtypes = [C.c_int, dp, C.c_int]
        L.orc_fftn.argtypes = [C.POINTER(abi.Grid), dp, C.c_int]
        L.orc_system_create.restype = vp
        L.orc_system_create.argtypes = [C.POINTER(abi.HPlanDesc)]
        L.orc_system_destroy.argtypes = [vp]
        L.orc_erange.argtypes = [vp, dp, dp]
        L.orc_h_apply.argtypes = [vp, dp, dp, C.c_long]
        L.orc_observables.argtypes = [vp, dp, dp, C.c_long, dp]
        L.orc_eigen_lanczos.argtypes = [vp, dp, C.c_int, dp, dp, C.POINTER(C.c_int), dp]
        L.orc_eigen_ac.argtypes = [vp, dp, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, dp,
                                   C.POINTER(C.c_int), dp, dp]
        for f, args in (("orc_expec_position", [vp, dp, C.c_int, C.c_double]),
                        ("orc_expec_momentum", [vp, dp, C.c_int, C.c_double]),
                        ("orc_expec_kinetic", [vp, dp]),
                        ("orc_expec_grid", [vp, dp, C.c_int]),
                        ("orc_expec_projection", [vp, dp, dp, C.c_int])):
            getattr(L, f).argtypes = args
            getattr(L, f).restype = C.c_double
        L.orc_prop_create.restype = vp
        L.orc_prop_create.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_double, C.c_int, C.c_int]
        L.orc_prop_destroy.argtypes = [vp]
        L.orc_prop_info.argtypes = [vp, dp]
        L.orc_prop_coeffs.argtypes = [vp, dp, C.c_int]
        L.orc_prop_apply.argtypes = [vp, dp, C.c_long]
        L.orc_propagate.argtypes = [vp, dp, dp, C.c_long, C.c_int, dp, C.POINTER(C.c_int)]
        L.orc_eigen_imag.argtypes = [vp, dp, C.c_int, C.c_int, C.c_double, C.c_int, dp, dp, dp,
                                     C.POINTER(C.c_int)]
        L.orc_bessel.argtypes = [C.c_int, C.c_int, C.c_double, dp]
        _LIB = L
    return _LIB


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def threads(n=0):
    return lib().orc_num_threads(n)


def fft1(x, sign):
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    lib().orc_fft1(a.size, _dp(a), sign)
    return a


def fftn(grid, x, sign):
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    g = grid.to_c()
    lib().orc_fftn(C.byref(g), _dp(a), sign)
    return a


def bessel(kind, n, x):
    out = np.zeros(n)
    z = lib().orc_bessel(kind, n, x, _dp(out))
    return out, z


class System:
    """Oracle copy of an HPlan (operators.HPlan)."""

    def __init__(self, hplan):
        self.hplan = hplan
        self.S = hplan.nstates
        self.npts = hplan.npts
        self.h = lib().orc_system_create(C.byref(hplan.desc))

    def __del__(self):
        if getattr(self, "h", None) and _LIB is not None:
            _LIB.orc_system_destroy(self.h)
            self.h = None

    def erange(self):
        a, b = np.zeros(2), np.zeros(2)
        lib().orc_erange(self.h, _dp(a), _dp(b))
        return complex(a[0], a[1]), complex(b[0], b[1])

    def h_apply(self, psi, step=0):
        x = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1)
        out = np.zeros_like(x)
        lib().orc_h_apply(self.h, _dp(x), _dp(out), step)
        return out

    def observables(self, psi, psi0=None, step=0):
        x = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1)
        out = np.zeros(4 + self.S)
        p0 = np.ascontiguousarray(psi0, dtype=np.complex128).reshape(-1) if psi0 is not None else None
        lib().orc_observables(self.h, _dp(x), _dp(p0) if p0 is not None else None, step, _dp(out))
        return dict(norm2=out[0], pops=out[1:1 + self.S], energy=out[1 + self.S],
                    autocorr=complex(out[2 + self.S], out[3 + self.S]))

    # expectation filters, Re <psi|O|psi> / <psi|psi> (FiltersList.cpp:289-308, ProgPropa.cpp:260,276)
    def _x(self, psi):
        return np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1)

    def expec_position(self, psi, dim=-1, scale=1.0):
        return lib().orc_expec_position(self.h, _dp(self._x(psi)), dim, scale)

    def expec_momentum(self, psi, dim=-1, factor=1.0):
        return lib().orc_expec_momentum(self.h, _dp(self._x(psi)), dim, factor)

    def expec_kinetic(self, psi):
        return lib().orc_expec_kinetic(self.h, _dp(self._x(psi)))

    def expec_grid(self, psi, grid):
        return lib().orc_expec_grid(self.h, _dp(self._x(psi)), grid)

    def expec_projection(self, psi, funcs):
        f = np.ascontiguousarray(np.stack([self._x(v) for v in funcs]))
        return lib().orc_expec_projection(self.h, _dp(self._x(psi)), _dp(f), len(funcs))


class Propagator:
    def __init__(self, system, name, params="", dt=1.0, imaginary_time=False, backward=False):
        self.system = system
        self.h = lib().orc_prop_create(system.h, name.encode(), params.encode(), dt,
                                       int(imaginary_time), int(backward))
        if not self.h:
            raise ValueError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _LIB is not None:
            _LIB.orc_prop_destroy(self.h)
            self.h = None

    def info(self):
        o = np.zeros(6)
        lib().orc_prop_info(self.h, _dp(o))
        return dict(order=int(o[0]), scaling=o[1], offset=complex(o[2], o[3]), exponent=complex(o[4], o[5]))

    def coeffs(self):
        n = lib().orc_prop_coeffs(self.h, None, 0)
        o = np.zeros(max(n, 1))
        lib().orc_prop_coeffs(self.h, _dp(o), n)
        return o[:n]

    def apply(self, psi, step):
        """In place on a complex128 array; returns the terms used."""
        assert psi.dtype == np.complex128 and psi.flags.c_contiguous
        t = lib().orc_prop_apply(self.h, _dp(psi), step)
        if t < 0:
            raise ValueError(lib().orc_last_error().decode())
        return t

    def propagate(self, psi, psi0, nsteps, start=0):
        """ProgPropa loop: report then step. Returns (obs array [nsteps, 4+S], terms)."""
        S = self.system.S
        obs = np.zeros((nsteps, 4 + S))
        terms = np.zeros(nsteps, dtype=np.int32)
        rc = lib().orc_propagate(self.h, _dp(psi), _dp(psi0), start, nsteps, _dp(obs),
                                 terms.ctypes.data_as(C.POINTER(C.c_int)))
        if rc < 0:
            raise ValueError(lib().orc_last_error().decode())
        return obs, terms

    def eigen_autocorr(self, psi_init, nsteps, tol=1.0, width=-1, win=True, max_nef=64):
        """ProgEigen::AutoCorrEF: (energies, efs [k x size], spectrum, peaks found)."""
        n = self.system.S * self.system.npts
        x = np.ascontiguousarray(psi_init, dtype=np.complex128).reshape(-1)
        e = np.zeros(max(max_nef, 1))
        efs = np.zeros((max(max_nef, 1), n), dtype=np.complex128)
        spec = np.zeros(nsteps, dtype=np.complex128)
        nef = C.c_int(0)
        rc = lib().orc_eigen_ac(self.h, _dp(x), nsteps, tol, width, int(win), max_nef, _dp(e), C.byref(nef),
                                _dp(efs), _dp(spec))
        if rc < 0:
            raise ValueError(lib().orc_last_error().decode())
        k = min(nef.value, max_nef)
        return e[:k], efs[:k], spec, nef.value

    def eigen_lanczos(self, psi_init, max_nef=64):
        """ProgEigen::LanczosEF + DiagBasis: (e_raw, e_diag, efs, basis size)."""
        n = self.system.S * self.system.npts
        x = np.ascontiguousarray(psi_init, dtype=np.complex128).reshape(-1)
        er, ed = np.zeros(max(max_nef, 1)), np.zeros(max(max_nef, 1))
        efs = np.zeros((max(max_nef, 1), n), dtype=np.complex128)
        nef = C.c_int(0)
        lib().orc_eigen_lanczos(self.h, _dp(x), max_nef, _dp(er), _dp(ed), C.byref(nef), _dp(efs))
        k = min(nef.value, max_nef)
        return er[:k], ed[:k], efs[:k], nef.value

    def eigen_imag(self, psi_init, nef, maxsteps, conv, diag=True):
        n = self.system.npts * self.system.S
        efs = np.zeros((nef, n), dtype=np.complex128)
        e_raw, e_diag = np.zeros(nef), np.zeros(nef)
        steps = np.zeros(nef, dtype=np.int32)
        x = np.ascontiguousarray(psi_init, dtype=np.complex128).reshape(-1)
        rc = lib().orc_eigen_imag(self.h, _dp(x), nef, maxsteps, conv, int(diag), _dp(efs),
                                  _dp(e_raw), _dp(e_diag), steps.ctypes.data_as(C.POINTER(C.c_int)))
        if rc < 0:
            raise ValueError(lib().orc_last_error().decode())
        return efs, e_raw, e_diag, steps
