"""Python front end of the engine's C ABI (used by tests, smoke and bench).

Mirrors the QDng call pattern: a plan is the device image of the operator
tree (Init(WaveFunction*)), a Propagator mirrors OCheby / OGSPO / OSIL /
OArnoldi (Init, Apply) and observables mirror Reporter::Analyze.
"""
import atexit
import ctypes as C

import numpy as np

from . import abi
from ._lib import QDGError, check, load

PRECISIONS = {"fp64": abi.PREC_FP64, "mixed": abi.PREC_MIXED, "df64": abi.PREC_DF64}

# At interpreter exit the CUDA runtime may already be torn down; handles are
# then left to process teardown instead of being released one by one.
_exiting = [False]
atexit.register(lambda: _exiting.__setitem__(0, True))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Plan:
    def __init__(self, hplan, precision="fp64"):
        self.lib = load()
        self.hplan = hplan
        self.S = hplan.nstates
        self.npts = hplan.npts
        self.precision = precision
        h = C.c_void_p()
        check(self.lib.qdg_plan_create(C.byref(hplan.desc), PRECISIONS[precision], C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) and not _exiting[0]:
            self.lib.qdg_plan_destroy(self.h)
        self.h = None

    __del__ = close

    def erange(self):
        a, b = np.zeros(2), np.zeros(2)
        check(self.lib.qdg_plan_erange(self.h, _dp(a), _dp(b)))
        return complex(a[0], a[1]), complex(b[0], b[1])

    def synchronize(self):
        check(self.lib.qdg_plan_synchronize(self.h))

    def set_stream(self, cuda_stream_ptr):
        check(self.lib.qdg_plan_set_stream(self.h, C.c_void_p(cuda_stream_ptr)))

    def profile(self, on=True):
        check(self.lib.qdg_profile_enable(self.h, int(on)))

    def profile_read(self):
        ms = np.zeros(8)
        n = np.zeros(8, dtype=np.int64)
        check(self.lib.qdg_profile_read(self.h, _dp(ms), n.ctypes.data_as(C.POINTER(C.c_int64))))
        return ms, n

    def inject_barrier_stall(self):
        """Failure-path test aid: the next persistent step kernel's grid
        barrier cannot complete, so the step returns QDG_ETIMEOUT."""
        check(self.lib.qdg_plan_inject_barrier_stall(self.h))

    def wavefunction(self, psi=None):
        w = WaveFunction(self)
        if psi is not None:
            w.upload(psi)
        return w

    def h_apply(self, win, wout, step=0):
        check(self.lib.qdg_h_apply(self.h, win.h, wout.h, step))

    def observables(self, psi, psi0=None, step=0):
        o = abi.Observables()
        check(self.lib.qdg_observables_compute(self.h, psi.h, psi0.h if psi0 is not None else None, step,
                                               C.byref(o)))
        return dict(norm2=o.norm2, pops=np.array(o.pops[:self.S]), energy=o.energy,
                    autocorr=complex(o.autocorr_re, o.autocorr_im))

    # expectation filters (FiltersList expec/expeconly), each Re <psi|O|psi> / <psi|psi>
    def expec_position(self, psi, dim=-1, scale=1.0):
        v = C.c_double()
        check(self.lib.qdg_expec_position(self.h, psi.h, dim, scale, C.byref(v)))
        return v.value

    def expec_momentum(self, psi, dim=-1, factor=1.0):
        v = C.c_double()
        check(self.lib.qdg_expec_momentum(self.h, psi.h, dim, factor, C.byref(v)))
        return v.value

    def expec_kinetic(self, psi):
        v = C.c_double()
        check(self.lib.qdg_expec_kinetic(self.h, psi.h, C.byref(v)))
        return v.value

    def expec_grid(self, psi, grid):
        v = C.c_double()
        check(self.lib.qdg_expec_grid(self.h, psi.h, grid, C.byref(v)))
        return v.value

    def expec_projection(self, psi, funcs):
        fs = [np.ascontiguousarray(f, dtype=np.complex128).reshape(-1) for f in funcs]
        ptrs = (C.POINTER(C.c_double) * max(1, len(fs)))(*[_dp(f) for f in fs])
        v = C.c_double()
        check(self.lib.qdg_expec_projection(self.h, psi.h, ptrs, len(fs), C.byref(v)))
        return v.value


class WaveFunction:
    def __init__(self, plan):
        self.plan = plan
        self.lib = plan.lib
        h = C.c_void_p()
        check(self.lib.qdg_wf_create(plan.h, C.byref(h)))
        self.h = h
        self.size = plan.S * plan.npts

    def close(self):
        if getattr(self, "h", None) and not _exiting[0]:
            self.lib.qdg_wf_destroy(self.h)
        self.h = None

    __del__ = close

    def upload(self, psi):
        a = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1)
        assert a.size == self.size
        check(self.lib.qdg_wf_upload(self.h, _dp(a)))

    def download(self):
        out = np.empty(self.size, dtype=np.complex128)
        check(self.lib.qdg_wf_download(self.h, _dp(out)))
        return out

    def copy_from(self, other):
        check(self.lib.qdg_wf_copy(self.h, other.h))


class Propagator:
    """OCheby / OGSPO / OSIL / OArnoldi on the device."""

    def __init__(self, plan, name, params="", dt=1.0, imaginary_time=False, backward=False):
        self.plan = plan
        self.lib = plan.lib
        h = C.c_void_p()
        check(self.lib.qdg_prop_create(plan.h, name.encode(), params.encode(), dt, int(imaginary_time),
                                       int(backward), C.byref(h)))
        self.h = h
        check(self.lib.qdg_prop_init(self.h))

    def close(self):
        if getattr(self, "h", None) and not _exiting[0]:
            self.lib.qdg_prop_destroy(self.h)
        self.h = None

    __del__ = close

    def info(self):
        i = abi.PropInfo()
        check(self.lib.qdg_prop_get_info(self.h, C.byref(i)))
        return dict(kind=i.kind, order=i.order, scaling=i.scaling, offset=complex(i.offset_re, i.offset_im),
                    exponent=complex(i.exponent_re, i.exponent_im))

    def coeffs(self):
        n = self.info()["order"]
        out = np.zeros(max(1, n))
        check(self.lib.qdg_prop_get_coeffs(self.h, _dp(out), n))
        return out[:n]

    def apply(self, wf, step):
        used = C.c_int32(0)
        check(self.lib.qdg_prop_apply(self.h, wf.h, step, C.byref(used)))
        return used.value

    def apply_host(self, scratch, psi, step):
        """The drop-in call: psi is a host complex128 array updated in place."""
        assert psi.dtype == np.complex128 and psi.flags.c_contiguous
        used = C.c_int32(0)
        check(self.lib.qdg_prop_apply_host(self.h, scratch.h, _dp(psi), step, C.byref(used)))
        return used.value

    def apply_host_states(self, scratch, states, step):
        """The drop-in call with one host block per state (QDng's WFMultistate
        layout): each complex128 array is updated in place."""
        for a in states:
            assert a.dtype == np.complex128 and a.flags.c_contiguous
        ptrs = (C.POINTER(C.c_double) * len(states))(*[_dp(a) for a in states])
        used = C.c_int32(0)
        check(self.lib.qdg_prop_apply_host_states(self.h, scratch.h, ptrs, step, C.byref(used)))
        return used.value

    def phase_times(self):
        """ns spent by one block (block 0, or QDG_TRACE_BLOCK) of the persistent step kernel
        while profiling, over the terms after the first: gathering and finishing phi
        (gather), the shared-memory FFTs (fft), the norm reduction and grid barrier
        (barrier), and the rest of the term (other: batch setup, the sum of the block
        partials, the series cut)."""
        ns = np.zeros(4)
        check(self.lib.qdg_prop_phase_times(self.h, _dp(ns)))
        other = max(0.0, ns[2] - ns[0] - ns[1] - ns[3]) if ns[2] > 0 else 0.0
        return dict(gather=ns[0], fft=ns[1], barrier=ns[3], other=other)

    def eigen_imag(self, psi_init, nef, maxsteps, conv, diag=True):
        """ProgEigen::ImagTimeEF (+ DiagBasis): returns (efs [nef x size],
        e_raw, e_diag, steps), the layout of the oracle's eigen_imag."""
        n = self.plan.S * self.plan.npts
        efs = np.zeros((nef, n), dtype=np.complex128)
        e_raw, e_diag = np.zeros(nef), np.zeros(nef)
        steps = np.zeros(nef, dtype=np.int32)
        x = np.ascontiguousarray(psi_init, dtype=np.complex128).reshape(-1)
        check(self.lib.qdg_eigen_imag(self.h, _dp(x), nef, maxsteps, conv, int(diag), _dp(efs), _dp(e_raw),
                                      _dp(e_diag), steps.ctypes.data_as(C.c_void_p)))
        return efs, e_raw, e_diag, steps

    def eigen_autocorr(self, psi_init, nsteps, tol=1.0, width=-1, win=True, max_nef=64, want_efs=True):
        """ProgEigen::AutoCorrEF: (energies, efs [k x size] or None, spectrum [nsteps],
        number of peaks found)."""
        n = self.plan.S * self.plan.npts
        x = np.ascontiguousarray(psi_init, dtype=np.complex128).reshape(-1)
        e = np.zeros(max(max_nef, 1))
        efs = np.zeros((max(max_nef, 1), n), dtype=np.complex128) if want_efs else None
        spec = np.zeros(nsteps, dtype=np.complex128)
        nef = C.c_int32(0)
        check(self.lib.qdg_eigen_autocorr(self.h, _dp(x), nsteps, tol, width, int(win), max_nef, _dp(e), C.byref(nef),
                                          _dp(efs) if efs is not None else None, _dp(spec)))
        k = min(nef.value, max_nef)
        return e[:k], (efs[:k] if efs is not None else None), spec, nef.value

    def eigen_lanczos(self, psi_init, max_nef=64, want_efs=True):
        """ProgEigen::LanczosEF + DiagBasis: (e_raw, e_diag, efs or None, basis size)."""
        n = self.plan.S * self.plan.npts
        x = np.ascontiguousarray(psi_init, dtype=np.complex128).reshape(-1)
        er, ed = np.zeros(max(max_nef, 1)), np.zeros(max(max_nef, 1))
        efs = np.zeros((max(max_nef, 1), n), dtype=np.complex128) if want_efs else None
        nef = C.c_int32(0)
        check(self.lib.qdg_eigen_lanczos(self.h, _dp(x), max_nef, _dp(er), _dp(ed), C.byref(nef),
                                         _dp(efs) if efs is not None else None))
        k = min(nef.value, max_nef)
        return er[:k], ed[:k], (efs[:k] if efs is not None else None), nef.value

    def run(self, wf, step0, nsteps):
        tot = C.c_int64(0)
        check(self.lib.qdg_prop_run(self.h, wf.h, step0, nsteps, C.byref(tot)))
        return tot.value

    def propagate(self, wf, psi0_wf, nsteps, start=0):
        """ProgPropa loop with the Reporter on the device: report then step."""
        rows, terms = [], []
        for i in range(nsteps):
            step = start + i
            o = self.plan.observables(wf, psi0_wf, step)
            rows.append([o["norm2"], *o["pops"], o["energy"], o["autocorr"].real, o["autocorr"].imag])
            terms.append(self.apply(wf, step))
        return np.array(rows), np.array(terms)


class Ensemble:
    """Batched independent wavepackets (qdg_ensemble_*): one persistent launch.

    members: dicts with keys grid (operators.GridSystem), mass, V, and
    optionally mu and laser (GridDipole x field)."""

    def __init__(self, members, dt, params="", precision="mixed"):
        self.lib = load()
        self.members = members
        self._keep = []
        arr = (abi.EnsembleMember * len(members))()
        self.sizes = []
        for i, m in enumerate(members):
            g = m["grid"]
            e = arr[i]
            e.grid = g.to_c()
            for d, mass in enumerate(np.atleast_1d(m["mass"])):
                e.mass[d] = float(mass)
            V = np.ascontiguousarray(m["V"], dtype=np.float64).reshape(-1)
            self._keep.append(V)
            e.potential = V.ctypes.data_as(C.POINTER(C.c_double))
            if m.get("mu") is not None and m.get("laser") is not None:
                mu = np.ascontiguousarray(m["mu"], dtype=np.float64).reshape(-1)
                las = np.ascontiguousarray(m["laser"], dtype=np.float64).reshape(-1)
                self._keep += [mu, las]
                e.dipole = mu.ctypes.data_as(C.POINTER(C.c_double))
                e.laser = las.ctypes.data_as(C.POINTER(C.c_double))
                e.laser_nt = las.size
            self.sizes.append(g.npts)
        h = C.c_void_p()
        check(self.lib.qdg_ensemble_create(arr, len(members), dt, params.encode(), PRECISIONS[precision],
                                           C.byref(h)))
        self.h = h
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])

    def close(self):
        if getattr(self, "h", None) and not _exiting[0]:
            self.lib.qdg_ensemble_destroy(self.h)
        self.h = None

    __del__ = close

    def upload(self, psis):
        a = np.ascontiguousarray(np.concatenate([np.asarray(p, dtype=np.complex128).reshape(-1) for p in psis]))
        check(self.lib.qdg_ensemble_upload(self.h, _dp(a)))

    def download(self):
        out = np.empty(int(self.offsets[-1]), dtype=np.complex128)
        check(self.lib.qdg_ensemble_download(self.h, _dp(out)))
        return [out[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.sizes))]

    def run(self, step0, nsteps):
        t = C.c_int64(0)
        check(self.lib.qdg_ensemble_run(self.h, step0, nsteps, C.byref(t)))
        return t.value

    def timeline(self):
        """(start, end) in ns of every member in the last run, and the block that ran it."""
        n = len(self.members)
        se = np.zeros(2 * n, dtype=np.int64)
        blk = np.zeros(n, dtype=np.int32)
        check(self.lib.qdg_ensemble_timeline(self.h, se.ctypes.data_as(C.c_void_p), blk.ctypes.data_as(C.c_void_p)))
        return se.reshape(-1, 2), blk

    def info(self, i):
        inf = abi.PropInfo()
        check(self.lib.qdg_ensemble_member_info(self.h, i, C.byref(inf)))
        return dict(order=inf.order, scaling=inf.scaling, offset=complex(inf.offset_re, inf.offset_im))


def kernel_launches():
    return load().qdg_kernel_launches()


PASS_MODES = ["kinetic", "kin_acc", "h_apply", "cheby_first", "cheby_term", "gspo_kin", "cheby_step"]

__all__ = ["Plan", "WaveFunction", "Propagator", "Ensemble", "QDGError", "kernel_launches", "PASS_MODES"]
