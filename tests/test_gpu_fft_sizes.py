"""Grid lengths with prime factors above 5 (FFTW takes any N,
src/fft/fft.cpp:98-122): their transforms add direct-DFT stages of the prime
radix and the plan runs on the graph path.  Engine against the oracle, whose
transform is checked against numpy for such lengths
(tests/test_oracle_golden.py::test_fft_matches_numpy)."""
import numpy as np
import pytest

from oracle import oracle as O
from qdng_gb300 import operators as op
from tests import cases
from tests.test_gpu_parity import _assert_parity, _run_both

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from qdng_gb300 import build, engine
    build.build()
    return engine


def _system(shape, states=1):
    g = op.GridSystem(list(shape), [-4.0, -3.0, -2.5][:len(shape)], [4.0, 3.5, 3.0][:len(shape)])
    Q = g.mesh()
    T = op.GridNablaSq([900.0, 1200.0, 1500.0][:len(shape)])
    V = 0.02 * sum(q ** 2 for q in Q)
    if states == 1:
        hp = op.HPlan(g, op.Sum([T, op.GridPotential(V)]))
    else:
        hp = op.HPlan(g, op.Multistate({(0, 0): op.Sum([T, op.GridPotential(V)]),
                                        (1, 1): op.Sum([T, op.GridPotential(V + 0.05)]),
                                        (0, 1): op.GridPotential(0.01 * np.exp(-Q[0] ** 2))}))
    e = sum(-(Q[d] - 0.4) ** 2 for d in range(g.ndims))
    psi = (np.exp(e) * np.exp(1.3j * Q[0])).reshape(-1).astype(np.complex128)
    psi = np.tile(psi, hp.nstates)
    return hp, psi / np.sqrt((np.abs(psi) ** 2).sum() * np.prod(g.dx))


@pytest.mark.parametrize("shape,states", [((97,), 1), ((7,), 1), ((28, 21), 2), ((14, 11, 13), 1)],
                         ids=["1d-prime97", "1d-7", "2d-28x21-two-states", "3d-14x11x13"])
def test_prime_lengths_cheby_parity(eng, shape, states):
    hp, psi = _system(shape, states)
    _assert_parity(hp, *_run_both(eng, hp, psi, dict(name="Cheby", params="", dt=5.0), 20))


@pytest.mark.parametrize("shape", [(97,), (28, 21)], ids=["1d-prime97", "2d-28x21"])
def test_prime_lengths_gspo_and_sil(eng, shape):
    hp, psi = _system(shape)
    g = hp.grid
    Q = g.mesh()
    hg = op.HPlan(g, members=[op.GridNablaSq([900.0, 1200.0][:len(shape)]),
                              op.GridPotential(0.02 * sum(q ** 2 for q in Q))])
    _assert_parity(hg, *_run_both(eng, hg, psi, dict(name="GSPO", params="", dt=5.0), 20))
    _assert_parity(hp, *_run_both(eng, hp, psi, dict(name="SIL", params="order=12", dt=5.0), 10),
                   rtol=1e-11, check_terms=False)


def test_prime_lengths_filters(eng):
    """Momentum and kinetic energy by the per-line spectral sums on 28 x 21."""
    hp, psi = _system((28, 21), 2)
    S = O.System(hp)
    plan = eng.Plan(hp, "fp64")
    w = plan.wavefunction(psi)
    for d in (0, 1, -1):
        a, b = plan.expec_momentum(w, d, 1.0), S.expec_momentum(psi, d, 1.0)
        assert abs(a - b) <= 1e-12 * max(1.0, abs(b)), (d, a, b)
    a, b = plan.expec_kinetic(w), S.expec_kinetic(psi)
    assert abs(a - b) <= 1e-12 * abs(b)


def test_prime_lengths_mixed(eng):
    hp, psi = _system((28, 21), 2)
    obs_o, _, x, obs_g, _, xg = _run_both(eng, hp, psi, dict(name="Cheby", params="", dt=5.0), 20, precision="mixed")
    assert np.abs(obs_g[:, 0] - obs_o[:, 0]).max() <= 1e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ensemble_members_of_prime_lengths(eng, precision):
    """Ensemble members whose lines have prime factors above 5 (1-D 97 and
    154 points, 2-D 21 x 14) next to a 256-point member, in one launch:
    binary64 against each member's oracle propagation to 1e-12, the mixed
    form to 1e-5."""
    from oracle import oracle as O
    from tests.test_gpu_parity import rel
    rng = np.random.default_rng(13)
    ens = [cases.cfg4_member(rng, 1, n, nt=4) for n in (97, 154, 256)]
    m2 = cases.cfg4_member(rng, 2, 14, nt=4)
    g = op.GridSystem([21, 14], [1.0, -3.0], [10.0, 3.0])
    X, Y = g.mesh()
    p = m2["params"]
    psi = np.exp(-(X - p["re"] - 0.1) ** 2 / 0.02 - Y ** 2 / 2.0).astype(np.complex128).reshape(-1)
    ens.append(dict(grid=g, mass=[1728.0, 1728.0],
                    V=(p["D"] * (1 - np.exp(-p["a"] * (X - p["re"]))) ** 2 + 0.005 * Y ** 2).reshape(-1),
                    mu=(X * np.exp(-X / 4)).reshape(-1), laser=m2["laser"],
                    psi=psi / np.sqrt((np.abs(psi) ** 2).sum() * np.prod(g.dx))))
    E = eng.Ensemble(ens, dt=10.0, precision=precision)
    E.upload([m["psi"] for m in ens])
    E.run(0, 2)
    out = E.download()
    for i, m in enumerate(ens):
        Pm = O.Propagator(O.System(cases.member_hplan(m)), "Cheby", "", dt=10.0)
        x = m["psi"].copy()
        Pm.apply(x, 0)
        Pm.apply(x, 1)
        assert rel(out[i], x) < (1e-12 if precision == "fp64" else 1e-5), (m["grid"].n, rel(out[i], x))
