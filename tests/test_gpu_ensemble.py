"""Batched ensemble on the GPU against the oracle, member by member."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases

pytestmark = pytest.mark.gpu


def small_ensemble(nt=16, seed=7):
    rng = np.random.default_rng(seed)
    specs = [(1, 256), (1, 384), (1, 512), (2, 64), (1, 256), (2, 96), (1, 768), (2, 48)]
    return [cases.cfg4_member(rng, k, s, nt=nt) for k, s in specs]


def oracle_run(mem, nsteps, dt=10.0):
    S = O.System(cases.member_hplan(mem))
    P = O.Propagator(S, "Cheby", "", dt=dt)
    x = mem["psi"].copy()
    terms = [P.apply(x, s) for s in range(nsteps)]
    return x, P.info()["order"], terms


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-5)])
def test_ensemble_matches_oracle(precision, tol):
    from qdng_gb300 import build, engine
    build.build()
    ens = small_ensemble()
    E = engine.Ensemble(ens, dt=10.0, params="", precision=precision)
    E.upload([m["psi"] for m in ens])
    nsteps = 4
    E.run(0, nsteps)
    out = E.download()
    for i, m in enumerate(ens):
        ref, order, _ = oracle_run(m, nsteps)
        assert E.info(i)["order"] == order
        err = np.abs(out[i] - ref).max() / np.abs(ref).max()
        assert err < tol, (i, m["grid"].n, err)


def test_ensemble_two_runs_continue_the_clock():
    """run(0, 2) then run(2, 2) equals run(0, 4): the field is indexed by the clock step."""
    from qdng_gb300 import engine
    ens = small_ensemble()[:3]
    A = engine.Ensemble(ens, dt=10.0, precision="fp64")
    B = engine.Ensemble(ens, dt=10.0, precision="fp64")
    A.upload([m["psi"] for m in ens])
    B.upload([m["psi"] for m in ens])
    A.run(0, 2)
    A.run(2, 2)
    B.run(0, 4)
    for a, b in zip(A.download(), B.download()):
        assert np.array_equal(a, b)
