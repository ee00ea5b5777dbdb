"""The kinetic operators without a k-space table on the device: OGridNablaSq
with method="HOFD" (finite differences, QDng's neighbour rule), OGridHOFD
(finite differences along each dimension) and OGridGMat (the G-matrix),
against the oracle, which reproduces QDng's TGP-Expec-HOFD and TGP-Gmat
goldens (tests/test_oracle_golden.py)."""
import numpy as np
import pytest

from oracle import oracle as O
from qdng_gb300 import operators as op
from tests import cases
from tests.test_gpu_parity import _assert_parity, _run_both, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from qdng_gb300 import build, engine
    build.build()
    return engine


def _packet(g, k=(1.5, -1.0, 0.5)):
    Q = g.mesh()
    e = sum(-(Q[d] - 0.3 * d) ** 2 for d in range(g.ndims))
    ph = sum(k[d] * Q[d] for d in range(g.ndims))
    psi = (np.exp(e) * np.exp(1j * ph)).reshape(-1).astype(np.complex128)
    return psi / np.sqrt((np.abs(psi) ** 2).sum() * np.prod(g.dx))


def _gmat_2d(kind="grid"):
    g = op.GridSystem([32, 24], [-4.0, -3.0], [4.0, 3.5])
    X, Y = g.mesh()
    if kind == "grid":
        G = op.GridGMat(2, gmat={(0, 0): (1 / 900.0) * (1 + 0.2 * np.tanh(Y)),
                                 (1, 0): (1 / 4000.0) * np.exp(-X ** 2),
                                 (1, 1): (1 / 1200.0) * (1 + 0.1 * X ** 2 / 16)})
    elif kind == "const":
        G = op.GridGMat(2, G=[1 / 900.0, -1 / 5000.0, 1 / 1200.0])
    else:  # element sources mixed, one dropped
        G = op.GridGMat(2, gmat={(1, 1): (1 / 1200.0) * (1 + 0.1 * Y ** 2 / 9)}, G=[1 / 900.0, 0.0, 0.0],
                        Gdef="cxg")
    V = op.GridPotential(0.01 * (X ** 2 + Y ** 2))
    return g, op.HPlan(g, op.Sum([G, V]))


def _fd(shape, order=8, pbc=False, states=1):
    g = op.GridSystem(list(shape), [-4.0, -3.0, -2.5][:len(shape)], [4.0, 3.5, 3.0][:len(shape)])
    Q = g.mesh()
    T = op.GridNablaSq([900.0, 1200.0, 1500.0][:len(shape)], method="HOFD", order=order, pbc=pbc)
    V = op.GridPotential(0.01 * sum(q ** 2 for q in Q))
    if states == 1:
        return g, op.HPlan(g, op.Sum([T, V]))
    T2 = op.GridNablaSq([600.0, 800.0, 1000.0][:len(shape)], method="HOFD", order=order, pbc=pbc)
    return g, op.HPlan(g, op.Multistate({(0, 0): op.Sum([T, V]), (1, 1): op.Sum([T2, V]),
                                         (0, 1): op.GridPotential(0.02 * np.exp(-Q[0] ** 2))}))


def _h_parity(eng, hp, psi, precision="fp64"):
    S = O.System(hp)
    want = S.h_apply(psi)
    plan = eng.Plan(hp, precision)
    w, o = plan.wavefunction(psi), plan.wavefunction()
    plan.h_apply(w, o)
    got = o.download()
    a = plan.erange()
    b = S.erange()
    return rel(got, want), a, b


@pytest.mark.parametrize("kinetic", ["FFT", "HOFD", "GMAT"])
def test_tgp_expec_kinetic_forms_parity(eng, fixtures, kinetic):
    """TGP-Expec-SP / -HOFD / Gmat for 200 steps: norm and autocorrelation
    per step within 1e-12, the same series orders, and the filterpost <T>."""
    hp, psi, run = cases.tgp_expec_lc(fixtures, kinetic)
    res = _run_both(eng, hp, psi, run, 200)
    _assert_parity(hp, *res)
    x, xg = res[2], res[5]
    S = O.System(hp)
    plan = eng.Plan(hp, "fp64")
    w = plan.wavefunction(xg)
    assert abs(plan.expec_kinetic(w) - S.expec_kinetic(x)) <= 1e-12 * abs(S.expec_kinetic(x))


@pytest.mark.parametrize("shape,pbc,states", [((64,), False, 1), ((64,), True, 1), ((32, 24), False, 1),
                                              ((16, 12, 10), False, 1), ((32, 24), False, 2)],
                         ids=["1d", "1d-pbc", "2d", "3d", "2d-two-states"])
@pytest.mark.parametrize("order", [2, 8, 16])
def test_hofd_h_apply(eng, shape, pbc, states, order):
    """One H application and the energy range: QDng's neighbour rule on one
    to three dimensions, periodic on one, two states with their own masses."""
    g, hp = _fd(shape, order, pbc, states)
    psi = np.tile(_packet(g), hp.nstates)
    psi = psi + 0.05 * np.random.default_rng(3).normal(size=psi.size)
    r, a, b = _h_parity(eng, hp, psi)
    assert r <= 1e-13, r
    assert abs(a[0] - b[0]) <= 1e-14 * abs(b[0]) and abs(a[1] - b[1]) <= 1e-14 * max(1.0, abs(b[1]))


@pytest.mark.parametrize("kind", ["grid", "const", "mixed-sources"])
def test_gmat_h_apply(eng, kind):
    g, hp = _gmat_2d(kind)
    psi = _packet(g)
    r, a, b = _h_parity(eng, hp, psi)
    assert r <= 1e-13, r
    assert abs(a[0] - b[0]) <= 1e-14 * abs(b[0]) and abs(a[1] - b[1]) <= 1e-14 * max(1.0, abs(b[1]))


@pytest.mark.parametrize("case", ["hofd-2d", "hofd-2d-two-states", "gmat-2d"])
def test_kinetic_forms_propagation(eng, case):
    """Chebyshev (graph path) and Arnoldi steps on 2-D grids within 1e-12;
    the mixed form within 1e-5 of the oracle."""
    if case == "gmat-2d":
        g, hp = _gmat_2d("grid")
    else:
        g, hp = _fd((32, 24), 8, False, 2 if "two" in case else 1)
    psi = np.tile(_packet(g), hp.nstates) / np.sqrt(hp.nstates)
    run = dict(name="Cheby", params="", dt=5.0)
    _assert_parity(hp, *_run_both(eng, hp, psi, run, 20))
    _assert_parity(hp, *_run_both(eng, hp, psi, dict(name="Arnoldi", params="order=16 conv=1e-30", dt=5.0), 10),
                   rtol=1e-11, check_terms=False)
    obs_o, _, x, obs_g, _, xg = _run_both(eng, hp, psi, run, 20, precision="mixed")
    assert np.abs(obs_g[:, 0] - obs_o[:, 0]).max() <= 1e-5
    assert rel(xg, x) <= 1e-4


@pytest.mark.parametrize("case", ["hofd-3d", "gmat-2d"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_kinetic_expectation(eng, case, precision):
    """<T> by the direct operator (no k-space Parseval) in binary64 in every
    precision form, to 1e-12 of the oracle."""
    if case == "gmat-2d":
        g, hp = _gmat_2d("grid")
    else:
        g, hp = _fd((16, 12, 10), 8, False, 1)
    psi = _packet(g)
    S = O.System(hp)
    plan = eng.Plan(hp, precision)
    w = plan.wavefunction(psi)
    want = S.expec_kinetic(psi)
    assert abs(plan.expec_kinetic(w) - want) <= 1e-12 * abs(want)


def test_kinetic_forms_rejected(eng):
    g = op.GridSystem([64], [-5.0], [5.0])
    hofd = op.GridNablaSq([100.0], method="HOFD")
    plan = eng.Plan(op.HPlan(g, members=[hofd, op.GridPotential(np.zeros(64))]), "fp64")
    with pytest.raises(Exception) as e:
        eng.Propagator(plan, "GSPO", "", dt=1.0)
    assert "diagonal representation" in str(e.value)
    gm = op.GridGMat(1, G=[0.01])
    plan = eng.Plan(op.HPlan(g, members=[gm, op.GridPotential(np.zeros(64))]), "fp64")
    with pytest.raises(Exception):
        eng.Propagator(plan, "GSPO", "", dt=1.0)
    with pytest.raises(Exception):  # one kinetic form per plan
        eng.Plan(op.HPlan(g, op.Sum([hofd, op.GridNablaSq([100.0])])), "fp64")
    with pytest.raises(Exception):
        op.GridNablaSq([100.0], method="HOFD", order=7)


@pytest.mark.parametrize("shape,deriv,dim,pbc,mass", [
    ((64,), 1, -1, False, None), ((64,), 2, -1, True, [500.0]), ((32, 24), 2, -1, False, [300.0, 900.0]),
    ((32, 24), 1, 1, True, None), ((16, 12, 10), 2, 2, False, [100.0, 200.0, 400.0])],
    ids=["1d-d1", "1d-d2-pbc", "2d-d2-mass", "2d-d1-dim1-pbc", "3d-d2-dim2"])
def test_gridhofd_h_apply(eng, shape, deriv, dim, pbc, mass):
    """OGridHOFD: each dimension's (or one dimension's) lines with zero or
    periodic ends, first or second derivative, the mass factor of the last
    dimension; H psi and the energy range against the oracle."""
    g = op.GridSystem(list(shape), [-4.0, -3.0, -2.5][:len(shape)], [4.0, 3.5, 3.0][:len(shape)])
    Q = g.mesh()
    hp = op.HPlan(g, op.Sum([op.GridHOFD(deriv=deriv, order=8, dim=dim, pbc=pbc, mass=mass),
                             op.GridPotential(0.02 * sum(q ** 2 for q in Q))]))
    psi = _packet(g) + 0.05 * np.random.default_rng(4).normal(size=g.npts)
    r, a, b = _h_parity(eng, hp, psi)
    assert r <= 1e-13, r
    assert abs(a[0] - b[0]) <= 1e-14 * abs(b[0]) and abs(a[1] - b[1]) <= 1e-14 * max(1.0, abs(b[1]))


def test_gridhofd_propagation(eng):
    """A two-dimensional packet under GridHOFD (second derivative, masses)
    plus a potential: Chebyshev and SIL steps against the oracle."""
    g = op.GridSystem([32, 24], [-4.0, -3.0], [4.0, 3.5])
    X, Y = g.mesh()
    hp = op.HPlan(g, op.Sum([op.GridHOFD(deriv=2, order=8, mass=[900.0, 900.0]),
                             op.GridPotential(0.01 * (X ** 2 + Y ** 2))]))
    psi = _packet(g)
    _assert_parity(hp, *_run_both(eng, hp, psi, dict(name="Cheby", params="", dt=5.0), 20))
    _assert_parity(hp, *_run_both(eng, hp, psi, dict(name="SIL", params="order=12", dt=5.0), 10),
                   rtol=1e-11, check_terms=False)
