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


# FP64: the engine's series is the oracle's, so psi agrees to rounding.
# Mixed: phi and H phi are FP32 (unit roundoff 6e-8) and a rounding error
# made at one term is carried by the recurrence into every later term, so the
# error grows with the series length (50 to 250 terms per step here); the
# FP64 accumulator and reductions keep it from growing further.
TOLS = {"fp64": dict(psi=1e-12, obs=1e-12), "mixed": dict(psi=1e-4, obs=1e-4)}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ensemble_matches_oracle(precision):
    from qdng_gb300 import build, engine
    build.build()
    tol = TOLS[precision]
    ens = small_ensemble()
    E = engine.Ensemble(ens, dt=10.0, params="", precision=precision)
    E.upload([m["psi"] for m in ens])
    nsteps = 4
    E.run(0, nsteps)
    out = E.download()
    rows = []
    for i, m in enumerate(ens):
        ref, order, terms = oracle_run(m, nsteps)
        assert E.info(i)["order"] == order
        p0 = m["psi"]
        ac, ac_ref = np.vdot(p0, out[i]), np.vdot(p0, ref)
        n, n_ref = np.vdot(out[i], out[i]).real, np.vdot(ref, ref).real
        rows.append((i, m["grid"].n, sum(terms), np.abs(out[i] - ref).max() / np.abs(ref).max(),
                     abs(ac - ac_ref) / abs(ac_ref), abs(n - n_ref) / n_ref))
    for r in rows:
        print("member %d grid %s terms %d psi %.3g autocorrelation %.3g norm %.3g" % r)
    for r in rows:
        assert r[3] < tol["psi"] and r[4] < tol["obs"] and r[5] < tol["obs"], r


def test_ensemble_long_lines_both_paths():
    """Long 1-D members: in FP64 a 2048-point line stays in shared memory for
    the whole step and a 4096-point line goes through the global-memory path;
    one step of each (about 6000 series terms for 4096 points) against the
    oracle."""
    from qdng_gb300 import engine
    rng = np.random.default_rng(11)
    ens = [cases.cfg4_member(rng, 1, 4096, nt=4), cases.cfg4_member(rng, 1, 2048, nt=4)]
    E = engine.Ensemble(ens, dt=10.0, precision="fp64")
    E.upload([m["psi"] for m in ens])
    E.run(0, 1)
    out = E.download()
    for i, m in enumerate(ens):
        ref, order, _ = oracle_run(m, 1)
        err = np.abs(out[i] - ref).max() / np.abs(ref).max()
        assert err < 1e-12, (i, err)


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
