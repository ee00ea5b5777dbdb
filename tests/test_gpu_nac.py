"""OGridNAC (first-derivative non-adiabatic coupling) and non-hermitian
Multistate matrices on the GPU against the oracle.  Tolerances as in the
other parity tests: H psi to 1e-13 (FP64) and 5e-5 (mixed), propagated norm
and autocorrelation to 1e-12 (FP64)."""
import numpy as np
import pytest

from oracle import oracle as O
from qdng_gb300 import operators as op
from qdng_gb300._lib import QDGError
from tests import cases

pytestmark = pytest.mark.gpu

CASES = [(1, 96, True), (1, 96, False), (2, 32, True), (2, 24, False)]


@pytest.fixture(scope="module")
def eng():
    from qdng_gb300 import build, engine
    build.build()
    return engine


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.mark.parametrize("nd,n,paired", CASES)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 5e-5)])
def test_nac_h_apply(eng, nd, n, paired, precision, tol):
    hp, _, _, _, _ = cases.nac_two_state(n=n, nd=nd, paired=paired)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(hp.size) + 1j * rng.standard_normal(hp.size)
    ref = O.System(hp).h_apply(x)
    plan = eng.Plan(hp, precision)
    a, b = plan.wavefunction(x), plan.wavefunction()
    plan.h_apply(a, b)
    assert rel(b.download(), ref) < tol


@pytest.mark.parametrize("nd,n,paired", CASES)
def test_nac_energy_range(eng, nd, n, paired):
    hp, _, _, _, _ = cases.nac_two_state(n=n, nd=nd, paired=paired)
    e1, e2 = eng.Plan(hp, "fp64").erange()
    o1, o2 = O.System(hp).erange()
    assert abs(e1 - o1) <= 1e-13 * abs(o1) and abs(e2 - o2) <= 1e-13 * abs(o1)


@pytest.mark.parametrize("nd,n", [(1, 128), (2, 32)])
@pytest.mark.parametrize("name", ["Cheby", "SIL"])
def test_nac_propagation_parity(eng, nd, n, name):
    hp, psi, run, _, _ = cases.nac_two_state(n=n, nd=nd, paired=True)
    params = "order=12" if name == "SIL" else ""
    S = O.System(hp)
    Q = O.Propagator(S, name, params, dt=run["dt"])
    x = psi.copy()
    obs_o, terms_o = Q.propagate(x, psi.copy(), 20)
    plan = eng.Plan(hp, "fp64")
    P = eng.Propagator(plan, name, params, dt=run["dt"])
    w, w0 = plan.wavefunction(psi), plan.wavefunction(psi)
    obs_g, terms_g = P.propagate(w, w0, 20)
    assert list(terms_o) == list(terms_g)
    assert np.abs(obs_g[:, 0] - obs_o[:, 0]).max() <= 1e-12 * np.abs(obs_o[:, 0]).max()
    ac_o = obs_o[:, 4] + 1j * obs_o[:, 5]
    ac_g = obs_g[:, 4] + 1j * obs_g[:, 5]
    assert np.abs(ac_g - ac_o).max() <= 1e-12 * np.abs(ac_o).max()
    assert obs_o[-1, 2] > 1e-8  # population reached state 1 through the coupling
    assert rel(w.download(), x) < 1e-10


def test_nac_rejected_in_gspo(eng):
    g = op.GridSystem([64], [-6.0], [6.0])
    X = g.axes()[0]
    f = 0.5 * np.exp(-X ** 2)
    hp = op.HPlan(g, members=[
        op.DMultistate({(0, 0): op.GridNablaSq([2000.0]), (1, 1): op.GridNablaSq([2000.0])}),
        op.DMultistate({(0, 0): op.GridPotential(X ** 2), (1, 1): op.GridPotential(X ** 2),
                        (0, 1): op.GridNAC([f], mass=2000.0)})])
    plan = eng.Plan(hp, "fp64")
    with pytest.raises(QDGError):
        P = eng.Propagator(plan, "GSPO", "", dt=5.0)
        w = plan.wavefunction(np.ones(hp.size, dtype=np.complex128))
        P.apply(w, 0)
