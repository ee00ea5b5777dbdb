"""The oracle's OGridNAC (first-derivative non-adiabatic coupling) and the
non-hermitian Multistate rule, against an independent numpy restatement
and against analytic derivatives."""
import numpy as np

from oracle import oracle as O
from qdng_gb300 import operators as op
from tests import cases


def _ddx(g, d, x):
    """d/dx_d by FFT on QDng's periodic grid: k = 2 pi m / (L + dx), with the
    Nyquist entry of an even line taken as -N/2 (Kspace::Init1Dddx)."""
    n = g.n[d]
    L = g.xmax[d] - g.xmin[d] + g.dx[d]
    m = np.arange(n)
    m = np.where(m < (n + 1) // 2, m, m - n).astype(np.float64)
    kk = 2 * np.pi / L * m
    a = x.reshape(g.n[::-1])
    ax = g.ndims - 1 - d
    shape = [1] * g.ndims
    shape[ax] = n
    return np.fft.ifft(1j * kk.reshape(shape) * np.fft.fft(a, axis=ax), axis=ax).reshape(-1)


def _nac(g, f, mass, sign, x):
    c = 0.5 * sign / mass
    return sum(c * (f[d] * _ddx(g, d, x) + _ddx(g, d, f[d] * x)) for d in range(g.ndims))


def _diag_blocks(g, nd):
    if nd == 1:
        X = g.axes()[0]
        V0, V1 = 0.5 * 0.01 * X ** 2, 0.5 * 0.01 * (X - 1.0) ** 2 + 0.02
        T = op.GridNablaSq([2000.0])
    else:
        X, Y = g.mesh()
        V0 = 0.5 * 0.01 * (X ** 2 + Y ** 2)
        V1 = 0.5 * 0.01 * ((X - 1.0) ** 2 + Y ** 2) + 0.02
        T = op.GridNablaSq([2000.0, 2000.0])
    return op.Sum([T, op.GridPotential(V0)]), op.Sum([T, op.GridPotential(V1)])


def _h_ref(hp, nd, f, mass, psi, paired):
    """H psi of the nac_two_state systems: the oracle's diagonal blocks plus
    the coupling written out with numpy."""
    g = hp.grid
    d0, d1 = _diag_blocks(g, nd)
    out = O.System(op.HPlan(g, op.Multistate({(0, 0): d0, (1, 1): d1}))).h_apply(psi)
    n = g.npts
    m = 1.0 if mass is None else mass
    out[:n] += _nac(g, f, m, 1.0, psi[n:])
    out[n:] += _nac(g, f, m, -1.0 if paired else 1.0, psi[:n])
    return out


def test_nac_h_apply_matches_numpy():
    rng = np.random.default_rng(5)
    for nd, n in ((1, 96), (2, 24)):
        for paired in (True, False):
            hp, _, _, f, mass = cases.nac_two_state(n=n, nd=nd, paired=paired)
            assert hp.nonhermitian == paired
            x = rng.standard_normal(hp.size) + 1j * rng.standard_normal(hp.size)
            got = O.System(hp).h_apply(x)
            want = _h_ref(hp, nd, f, mass, x, paired)
            assert np.abs(got - want).max() / np.abs(want).max() < 1e-12, (nd, paired)


def test_nac_plane_wave_is_analytic():
    """Constant f and a plane wave on the periodic grid: the derivative is
    exact, so NAC psi = sign f (i k) psi / mass."""
    g = op.GridSystem([64], [0.0], [63.0 / 64.0 * 2 * np.pi])
    x = g.axes()[0]
    L = g.xmax[0] - g.xmin[0] + g.dx[0]
    kk = 2 * np.pi * 5 / L
    psi = np.exp(1j * kk * x)
    f = np.full(64, 0.3)
    hp = op.HPlan(g, op.Multistate({(0, 1): op.GridNAC([f], mass=2.0, sign=-1.0),
                                    (1, 1): op.GridPotential(np.zeros(64))}))
    out = O.System(hp).h_apply(np.concatenate([np.zeros(64), psi]))
    np.testing.assert_allclose(out[:64], -0.3 * 1j * kk * psi / 2.0, atol=1e-13)


def test_nac_energy_range():
    """OGridNAC::Emax = sum_d max f_d * pi / mass / dx_0, Emin = 0; the
    Multistate range is the extreme eigenvalue of the |E_ij| matrix."""
    hp, _, _, f, mass = cases.nac_two_state(n=64, nd=1, paired=True)
    emax, emin = O.System(hp).erange()
    g = hp.grid
    Tm = np.pi ** 2 / 2 / (2000.0 * g.dx[0] ** 2)
    X = g.axes()[0]
    d0 = Tm + (0.5 * 0.01 * X ** 2).max()
    d1 = Tm + (0.5 * 0.01 * (X - 1.0) ** 2 + 0.02).max()
    e01 = f[0].max() * np.pi / mass / g.dx[0]
    want = np.linalg.eigvalsh(np.array([[d0, e01], [e01, d1]]))[-1]
    assert abs(emax.real - want) < 1e-12 * want
    v0min, v1min = (0.5 * 0.01 * X ** 2).min(), (0.5 * 0.01 * (X - 1.0) ** 2 + 0.02).min()
    assert abs(emin.real - min(v0min, v1min)) < 1e-15  # the NAC element's Emin is 0


def test_nac_paired_hamiltonian_is_hermitian_and_conserves_norm():
    hp, psi, run, f, mass = cases.nac_two_state(n=128, nd=1, paired=True)
    S = O.System(hp)
    rng = np.random.default_rng(1)
    a = rng.standard_normal(hp.size) + 1j * rng.standard_normal(hp.size)
    b = rng.standard_normal(hp.size) + 1j * rng.standard_normal(hp.size)
    lhs, rhs = np.vdot(a, S.h_apply(b)), np.vdot(S.h_apply(a), b)
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
    P = O.Propagator(S, "Cheby", "", dt=run["dt"])
    x = psi.copy()
    n0 = np.vdot(x, x).real
    for i in range(20):
        P.apply(x, i)
    n = hp.npts
    assert abs(np.vdot(x, x).real - n0) < 1e-8 * n0  # series cut at prec = 1e-10 per step
    assert np.vdot(x[n:], x[n:]).real > 1e-8 * n0  # the coupling moved population
