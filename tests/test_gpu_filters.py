"""The engine's negative imaginary potential (OGobbler with nip) and the
expectation filters against the oracle, which reproduces QDng's TGP-NIP-Cheby
and TGP-Expec goldens (tests/test_oracle_golden.py)."""
import numpy as np
import pytest

from oracle import oracle as O
from qdng_gb300 import abi, operators as op
from tests import cases
from tests.test_gpu_parity import _assert_parity, _run_both, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from qdng_gb300 import build, engine
    build.build()
    return engine


def _nip_2d(n=64, states=1):
    """A 2-D (or two-state) packet running into Gobbler absorbers at both
    ends of x, with a real Gobbler step along y."""
    g = op.GridSystem([n, n // 2], [-6.0, -4.0], [6.0, 4.0])
    X, Y = g.mesh()
    T = op.GridNablaSq([900.0, 1200.0])
    nip = op.Gobbler(rp={0: 3.5}, order=6, gain=0.05, nip=True)
    step = op.Gobbler(lp={1: 2.5}, order=10, gain=0.02)
    V = op.GridPotential(0.01 * Y ** 2)
    if states == 1:
        hp = op.HPlan(g, op.Sum([T, nip, step, V]))
    else:
        hp = op.HPlan(g, op.Multistate({(0, 0): op.Sum([T, nip, V]), (1, 1): op.Sum([T, step, V]),
                                        (0, 1): op.GridPotential(0.01 * np.exp(-X ** 2))}))
    psi = np.exp(-(X - 1.0) ** 2 - Y ** 2 + 3.0j * X).astype(np.complex128)
    psi = np.tile(psi.reshape(-1), hp.nstates) / np.sqrt(hp.nstates)
    return hp, psi / np.sqrt((np.abs(psi) ** 2).sum() * np.prod(g.dx))


def test_tgp_nip_cheby_parity(eng, fixtures):
    """The TGP-NIP-Cheby Hamiltonian (T, Gobbler nip, Gobbler step) for 300
    steps: the complex offset switches the series cut off (OCheby.cpp:181), so
    every step runs the full order; norm and autocorrelation within 1e-12."""
    hp, psi, run = cases.tgp_nip(fixtures)
    _assert_parity(hp, *_run_both(eng, hp, psi, run, 300))


@pytest.mark.parametrize("states", [1, 2])
def test_nip_2d_parity(eng, states):
    hp, psi = _nip_2d(states=states)
    run = dict(name="Cheby", params="", dt=5.0)
    _assert_parity(hp, *_run_both(eng, hp, psi, run, 40))


def test_nip_arnoldi_and_graph_path(eng):
    hp, psi = _nip_2d()
    _assert_parity(hp, *_run_both(eng, hp, psi, dict(name="Arnoldi", params="order=16 conv=1e-30", dt=5.0), 20),
                   rtol=1e-11, check_terms=False)
    _assert_parity(hp, *_run_both(eng, hp, psi, dict(name="Cheby", params="path=graph", dt=5.0), 20))


def test_gspo_rejects_gobbler(eng):
    g = op.GridSystem([64], [-5.0], [5.0])
    hp = op.HPlan(g, members=[op.GridNablaSq([100.0]), op.Gobbler(rp={0: 3.0}, gain=0.1, nip=True)])
    plan = eng.Plan(hp, "fp64")
    with pytest.raises(Exception) as e:
        eng.Propagator(plan, "GSPO", "", dt=1.0)
    assert "ODSpace" in str(e.value)


def _filter_cases():
    rng = np.random.default_rng(5)
    out = []
    g1 = op.GridSystem([128], [1.8897], [6.1104])
    x = g1.axes()[0]
    hp1 = op.HPlan(g1, op.Sum([op.GridNablaSq([1763.2]), op.GridPotential(0.1 * (x - 3) ** 2)]))
    out.append((hp1, np.exp(-(x - 3.2) ** 2 / 0.1 + 2.0j * x).astype(np.complex128)))
    hp2, psi2 = _nip_2d(states=2)
    out.append((hp2, psi2 * np.exp(1j * rng.normal(size=psi2.size) * 0.1)))
    g3 = op.GridSystem([16, 12, 10], [-3.0, -2.0, -2.5], [3.0, 2.5, 2.0])
    Q = g3.mesh()
    hp3 = op.HPlan(g3, op.Sum([op.GridNablaSq([100.0, 200.0, 300.0]), op.GridPotential(0.1 * Q[0] ** 2)]))
    out.append((hp3, (np.exp(-Q[0] ** 2 - Q[1] ** 2 - Q[2] ** 2) * np.exp(1j * (Q[0] - 2 * Q[2]))).reshape(-1)
                .astype(np.complex128)))
    return out


@pytest.mark.parametrize("case", [0, 1, 2], ids=["1d", "2d-two-states", "3d"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_filters_match_oracle(eng, case, precision):
    """Position and momentum per dimension and summed, kinetic, a potential
    grid and a projection: the engine (per-line transforms, Parseval) against
    the oracle (QDng's N-dimensional apply and scalar product) to 1e-12; the
    filters compute in binary64 in every precision form."""
    hp, psi = _filter_cases()[case]
    S = O.System(hp)
    plan = eng.Plan(hp, precision)
    w = plan.wavefunction(psi)
    nd = hp.grid.ndims
    pairs = []
    for d in list(range(nd)) + [-1]:
        pairs.append((plan.expec_position(w, d, 1.0), S.expec_position(psi, d, 1.0)))
        pairs.append((plan.expec_momentum(w, d, 1.0), S.expec_momentum(psi, d, 1.0)))
    pairs.append((plan.expec_kinetic(w), S.expec_kinetic(psi)))
    pairs.append((plan.expec_grid(w, 0), S.expec_grid(psi, 0)))
    rng = np.random.default_rng(7)
    funcs = [psi * np.exp(1j * k) + 0.1 * (rng.normal(size=psi.size) + 1j * rng.normal(size=psi.size))
             for k in range(3)]
    pairs.append((plan.expec_projection(w, funcs), S.expec_projection(psi, funcs)))
    for i, (a, b) in enumerate(pairs):
        assert abs(a - b) <= 1e-12 * max(1.0, abs(b)), (i, a, b)


def test_filters_reject_bad_arguments(eng):
    hp, psi = _filter_cases()[0]
    plan = eng.Plan(hp, "fp64")
    w = plan.wavefunction(psi)
    with pytest.raises(Exception):
        plan.expec_position(w, 3, 1.0)
    with pytest.raises(Exception):
        plan.expec_grid(w, 7)
