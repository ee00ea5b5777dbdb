"""Imaginary-time eigenstates on the GPU (ProgEigen::ImagTimeEF with
OProjection and DiagBasis) against the oracle and QDng's TGE goldens."""
import numpy as np
import pytest

from oracle import oracle as O
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


def test_double_well_eigen_fp64_and_mixed(eng):
    """BASELINE's eigen-relaxation system (2-D double well, m = 1836) on a
    64 x 64 grid, 4 states: FP64 against the oracle, mixed against FP64."""
    hp, psi, run = cases.cfg5_double_well(n=64)
    nef, maxsteps, conv = 4, 300, 1e-7
    S = O.System(hp)
    Q = O.Propagator(S, "Cheby", "", dt=run["dt"], imaginary_time=True, backward=True)
    _, raw_o, diag_o, steps_o = Q.eigen_imag(psi, nef, maxsteps, conv, diag=True)
    out = {}
    for prec in ("fp64", "mixed"):
        plan = eng.Plan(hp, prec)
        P = eng.Propagator(plan, "Cheby", "", dt=run["dt"], imaginary_time=True, backward=True)
        out[prec] = P.eigen_imag(psi, nef, maxsteps, conv, diag=True)
    _, raw, diag, steps = out["fp64"]
    assert list(steps) == list(steps_o)
    np.testing.assert_allclose(diag, diag_o, rtol=1e-10)
    # mixed: FP32 H phi (spectral range ~2 hartree, unit roundoff 6e-8), so
    # the energies carry ~1e-7 hartree; the lowest splittings here are 4e-8
    # (tunnelling pair) and 3e-3 hartree
    err = np.abs(out["mixed"][2] - diag_o)
    print("mixed eigenenergy errors (hartree):", err)
    assert err.max() < 1e-6
