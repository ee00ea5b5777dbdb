"""Which propagators a mixed-precision plan runs in FP32 and which on its
FP64 copy: imaginary-time Chebyshev, the Krylov propagators (by default) and
Chebyshev on one 512-2048-point line must equal the FP64 plan's results;
real-time Chebyshev on other grids and the FP32 Krylov basis
(krylov_fp32=1) are FP32 and stay within their stated errors."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from qdng_gb300 import build, engine
    build.build()
    return engine


def _run(eng, hp, psi, prec, name, params, imag, nsteps, dt):
    plan = eng.Plan(hp, prec)
    P = eng.Propagator(plan, name, params, dt=dt, imaginary_time=imag, backward=imag)
    w, w0 = plan.wavefunction(psi), plan.wavefunction(psi)
    rows, terms = P.propagate(w, w0, nsteps)
    return rows, terms, w.download()


@pytest.mark.parametrize("name,params,imag", [("Cheby", "", True), ("SIL", "order=16", False),
                                              ("Arnoldi", "order=16", False), ("SIL", "order=16", True)])
def test_fp64_copy_forms_equal_fp64(eng, name, params, imag):
    hp, psi, _ = cases.cfg5_double_well(n=48)
    a = _run(eng, hp, psi, "fp64", name, params, imag, 5, 20.0)
    b = _run(eng, hp, psi, "mixed", name, params, imag, 5, 20.0)
    assert list(a[1]) == list(b[1])
    assert np.abs(a[2] - b[2]).max() <= 1e-13 * np.abs(a[2]).max()


def test_krylov_fp32_basis_is_close(eng):
    hp, psi, _ = cases.cfg5_double_well(n=48)
    a = _run(eng, hp, psi, "fp64", "SIL", "order=16", False, 10, 20.0)
    b = _run(eng, hp, psi, "mixed", "SIL", "order=16 krylov_fp32=1", False, 10, 20.0)
    ac_a, ac_b = a[0][:, 3] + 1j * a[0][:, 4], b[0][:, 3] + 1j * b[0][:, 4]
    err = np.abs(ac_a - ac_b).max() / a[0][0, 0]
    assert 0 < err < 1e-4


def test_mixed_line_runs_binary64(eng):
    """A single 1024-point line in the mixed form takes the binary64 cluster
    step (the FP32 line kernels are slower there): same terms and wave
    function as the FP64 plan; cluster=1 keeps the FP32 radix kernel, whose
    error stays at the FP32 level."""
    hp, psi, run = cases.cfg1_morse()
    a = _run(eng, hp, psi, "fp64", "Cheby", "", False, 20, run["dt"])
    b = _run(eng, hp, psi, "mixed", "Cheby", "", False, 20, run["dt"])
    assert list(a[1]) == list(b[1])
    assert np.abs(a[2] - b[2]).max() <= 1e-13 * np.abs(a[2]).max()
    c = _run(eng, hp, psi, "mixed", "Cheby", "cluster=1", False, 20, run["dt"])
    err = np.abs(a[2] - c[2]).max() / np.abs(a[2]).max()
    assert 1e-12 < err < 1e-3
