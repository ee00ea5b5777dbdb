"""Failure paths of the device code, exercised without faulting the GPU.

The persistent step kernel's grid barriers spin with an iteration limit.
The plan's barrier is preset so that no arrival completes it: every block
waits out its limit, raises the error flag and leaves; the step reports
QDG_ETIMEOUT, and the next step on the same plan (from a restored psi)
matches the oracle.  A NaN planted in psi reports QDG_ENONFINITE.
"""
import numpy as np
import pytest

from oracle import oracle as O
from qdng_gb300 import abi
from tests import cases
from tests.test_gpu_parity import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from qdng_gb300 import build, engine
    build.build()
    return engine


@pytest.mark.parametrize("case,precision", [("2d", "fp64"), ("2d", "mixed"), ("1d", "fp64")])
def test_barrier_timeout_then_recovery(eng, fixtures, case, precision):
    if case == "2d":
        hp, psi, run = cases.cfg2_two_state(n=64)
    else:
        hp, psi, run = cases.tgplms(fixtures)
    plan = eng.Plan(hp, precision)
    P = eng.Propagator(plan, run["name"], run["params"], dt=run["dt"])
    w = plan.wavefunction(psi)
    plan.inject_barrier_stall()
    with pytest.raises(eng.QDGError) as e:
        P.apply(w, 0)
    assert e.value.status == abi.QDG_ETIMEOUT
    # the barrier is reset: the next step from the restored psi is a normal
    # one, bit for bit the step of a propagator that never stalled
    w.upload(psi)
    terms = P.apply(w, 0)
    P2 = eng.Propagator(plan, run["name"], run["params"], dt=run["dt"])
    w2 = plan.wavefunction(psi)
    assert terms == P2.apply(w2, 0)
    assert np.array_equal(w.download(), w2.download())
    if precision == "fp64":  # and the oracle's step
        Q = O.Propagator(O.System(hp), run["name"], run["params"], dt=run["dt"])
        x = psi.copy()
        assert terms == Q.apply(x, 0)
        assert rel(w.download(), x) < 1e-12
