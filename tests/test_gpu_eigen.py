"""Imaginary-time eigenstates on the GPU (ProgEigen::ImagTimeEF with
OProjection and DiagBasis) against the oracle and QDng's TGE goldens."""
import numpy as np
import pytest

from oracle import oracle as O
from qdng_gb300 import operators as op
from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from qdng_gb300 import build, engine
    build.build()
    return engine


@pytest.mark.parametrize("method", ["Cheby", "SIL", "Arnoldi"])
def test_tge_eigen_matches_oracle_and_golden(eng, fixtures, golden, method):
    hp, psi, run = cases.tge(fixtures, method)
    S = O.System(hp)
    Q = O.Propagator(S, run["name"], run["params"], dt=run["dt"], imaginary_time=True, backward=True)
    efs_o, raw_o, diag_o, steps_o = Q.eigen_imag(psi, run["nef"], run["steps"], run["conv"], diag=True)
    plan = eng.Plan(hp, "fp64")
    P = eng.Propagator(plan, run["name"], run["params"], dt=run["dt"], imaginary_time=True, backward=True)
    efs, raw, diag, steps = P.eigen_imag(psi, run["nef"], run["steps"], run["conv"], diag=True)
    assert list(steps) == list(steps_o)
    np.testing.assert_allclose(raw, raw_o, rtol=1e-10)
    np.testing.assert_allclose(diag, diag_o, rtol=1e-10)
    # the diagonalised basis: same functions up to a phase
    dx = np.prod(hp.grid.dx)
    for i in range(run["nef"]):
        ov = abs(np.vdot(efs_o[i], efs[i])) * dx
        assert abs(ov - 1) < 1e-8, (i, ov)
    for i, txt in golden["tge_imag"]:
        dec = len(txt.split(".")[1])
        assert abs(diag[i] - float(txt)) < 1.5 * 10 ** (-dec), (method, i, diag[i], txt)


def _oscillator(n=32):
    """Anisotropic 2-D oscillator on [-4,4]^2: well separated levels, so the
    relaxation converges fast and the step counts are not rounding sensitive."""
    g = op.GridSystem([n, n], [-4.0, -4.0], [4.0, 4.0])
    X, Y = g.mesh()
    V = 0.5 * 0.04 * X ** 2 + 0.5 * 0.09 * Y ** 2 + 0.002 * X ** 3
    hp = op.HPlan(g, op.Sum([op.GridNablaSq([300.0, 300.0]), op.GridPotential(V)]))
    psi = (np.exp(-((X - 0.4) ** 2 + (Y - 0.3) ** 2)) * (1 + 0.3 * X + 0.2 * Y + 0.1 * X * Y)).reshape(-1)
    return hp, psi.astype(np.complex128)


def test_oscillator_eigen_fp64_matches_oracle(eng):
    hp, psi = _oscillator()
    nef, maxsteps, conv = 4, 400, 1e-10
    S = O.System(hp)
    Q = O.Propagator(S, "Cheby", "", dt=5.0, imaginary_time=True, backward=True)
    _, raw_o, diag_o, steps_o = Q.eigen_imag(psi, nef, maxsteps, conv, diag=True)
    plan = eng.Plan(hp, "fp64")
    P = eng.Propagator(plan, "Cheby", "", dt=5.0, imaginary_time=True, backward=True)
    _, raw, diag, steps = P.eigen_imag(psi, nef, maxsteps, conv, diag=True)
    assert max(steps_o) < maxsteps  # converged
    np.testing.assert_allclose(raw, raw_o, rtol=1e-9)
    np.testing.assert_allclose(diag, diag_o, rtol=1e-10)


def test_double_well_eigen_on_mixed_plan(eng):
    """The eigen-relaxation system of the benchmark set (2-D double well
    0.002 (x^2 - 4)^2 + 0.01 y^2, m = 1836, dt = 20) on a 64 x 64 grid,
    4 states, on a mixed plan.  The imaginary-time Chebyshev series reaches
    the low states through cancellations of terms ~1/sqrt(2 pi R) down to
    e^{-R(1-X)}, far below FP32 resolution, so a mixed plan runs it on an
    FP64 copy: the energies equal the FP64 plan's."""
    hp, psi, run = cases.cfg5_double_well(n=64)
    nef, maxsteps, conv = 4, 300, 1e-7
    out = {}
    for prec in ("fp64", "mixed"):
        plan = eng.Plan(hp, prec)
        P = eng.Propagator(plan, "Cheby", "", dt=run["dt"], imaginary_time=True, backward=True)
        out[prec] = P.eigen_imag(psi, nef, maxsteps, conv, diag=True)
    assert list(out["mixed"][3]) == list(out["fp64"][3])
    np.testing.assert_allclose(out["mixed"][2], out["fp64"][2], rtol=1e-13)


@pytest.mark.parametrize("method", ["Cheby", "SIL"])
def test_tge_autocorr_matches_oracle_and_golden(eng, fixtures, golden, method):
    """ProgEigen::AutoCorrEF on the GPU (2048 stored steps, autocorrelation,
    Hann window, FFT, peaks, time integration) against the oracle: the same
    peaks, spectrum to 1e-10, energies to 1e-10, eigenfunctions to 1e-9;
    and QDng's TGE-ac golden energies."""
    hp, psi, run = cases.tge(fixtures, method)
    S = O.System(hp)
    Qi = O.Propagator(S, run["name"], run["params"], dt=run["dt"], imaginary_time=True, backward=True)
    efs, _, _, _ = Qi.eigen_imag(psi, run["nef"], run["steps"], run["conv"], diag=True)
    lc = cases._normalize(hp, efs[:6].sum(axis=0))
    Q = O.Propagator(S, run["name"], run["params"], dt=run["dt"])
    e_o, ef_o, spec_o, npk_o = Q.eigen_autocorr(lc, 2048)
    plan = eng.Plan(hp, "fp64")
    P = eng.Propagator(plan, run["name"], run["params"], dt=run["dt"])
    e, ef, spec, npk = P.eigen_autocorr(lc, 2048)
    assert npk == npk_o >= 6
    assert np.abs(spec - spec_o).max() <= 1e-10 * np.abs(spec_o).max()
    np.testing.assert_allclose(e, e_o, rtol=1e-10)
    dx = np.prod(hp.grid.dx)
    for i in range(len(e)):
        assert np.abs(ef[i] - ef_o[i]).max() <= 1e-9 * np.abs(ef_o[i]).max(), i
    for i, txt in golden["tge_ac"]:
        dec = len(txt.split(".")[1])
        assert abs(e[i] - float(txt)) < 1.5 * 10 ** (-dec), (method, i, e[i], txt)


def test_autocorr_2d_double_well(eng):
    """A 2-D superposition (48^2 double well), 512 steps, windowed peaks with
    width 8: engine and oracle find the same peaks and energies."""
    hp, psi, run = cases.cfg5_double_well(n=48)
    S = O.System(hp)
    Q = O.Propagator(S, "Cheby", "", dt=20.0)
    plan = eng.Plan(hp, "fp64")
    P = eng.Propagator(plan, "Cheby", "", dt=20.0)
    e_o, _, _, npk_o = Q.eigen_autocorr(psi, 512, tol=2.0, width=8, max_nef=12)
    e, _, _, npk = P.eigen_autocorr(psi, 512, tol=2.0, width=8, max_nef=12)
    assert npk == npk_o and npk > 0
    np.testing.assert_allclose(e, e_o, rtol=1e-9)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lanczos_matches_oracle(eng, fixtures, precision):
    """ProgEigen::LanczosEF on the GPU (the Arnoldi propagator's basis build,
    Ritz pairs, DiagBasis) against the oracle (a mixed plan builds the Krylov
    basis on its binary64 copy).  Fifteen modified Gram-Schmidt vectors lose
    orthogonality, and the Ritz values of two binary64 implementations part
    at 1e-7 relative for the upper ones (the low ones to 1e-9): the basis
    size, the six lowest Ritz values to 1e-8, all to 1e-6, DiagBasis equal to
    the Ritz values, and the three lowest functions to 1e-6 up to sign."""
    hp, psi, run = cases.tge(fixtures, "Arnoldi")
    S = O.System(hp)
    Qi = O.Propagator(S, "Cheby", "", dt=5.0, imaginary_time=True, backward=True)
    efs, _, _, _ = Qi.eigen_imag(psi, run["nef"], run["steps"], run["conv"], diag=True)
    lc = cases._normalize(hp, efs[:6].sum(axis=0))
    Q = O.Propagator(S, "Arnoldi", run["params"], dt=run["dt"])
    er_o, ed_o, ef_o, nb_o = Q.eigen_lanczos(lc)
    plan = eng.Plan(hp, precision)
    P = eng.Propagator(plan, "Arnoldi", run["params"], dt=run["dt"])
    er, ed, ef, nb = P.eigen_lanczos(lc)
    assert nb == nb_o
    np.testing.assert_allclose(er[:6], er_o[:6], rtol=1e-8)
    np.testing.assert_allclose(er, er_o, rtol=1e-6)
    np.testing.assert_allclose(ed, er, rtol=1e-12, atol=1e-15)
    for i in range(3):
        s = np.sign(np.vdot(ef_o[i], ef[i]).real)
        assert np.abs(s * ef[i] - ef_o[i]).max() <= 1e-6 * np.abs(ef_o[i]).max(), i
