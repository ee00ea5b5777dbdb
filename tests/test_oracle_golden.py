"""Pin the CPU oracle against QDng's own goldens (tests/checktests.sh).

The reference prints the last propagation line as
    step  time  norm  [pop_i ...]  energy  <psi(t)|psi0>
with 6 decimals for populations and 8 for energy and autocorrelation
(Reporter.cpp:96-141); the eigen tests grep the leading digits of
energy.dat.  Agreement here is to the printed digits (half a unit in the
last printed place), which is all the reference's goldens carry.
"""
import numpy as np
import pytest

from oracle import oracle as O
from qdng_gb300 import operators as op
from tests import cases


def _last_line(hp, psi, run, step_count=None):
    S = O.System(hp)
    P = O.Propagator(S, run["name"], run["params"], dt=run["dt"])
    psi0 = psi.copy()
    x = psi.copy()
    n = step_count or run["steps"]
    obs, terms = P.propagate(x, psi0, n)
    return obs[-1], terms


def _check(golden_line, obs_row, nstates):
    vals = golden_line["values"]
    # vals: step, time, norm, [pops], energy, autocorr
    norm = obs_row[0]
    assert abs(norm - vals[2]) <= 0.5e-6
    k = 3
    if nstates > 1:
        for s in range(nstates):
            assert abs(obs_row[1 + s] - vals[k]) <= 0.5e-6, (s, obs_row[1 + s], vals[k])
            k += 1
    e = obs_row[1 + nstates]
    assert abs(e - vals[k]) <= 0.5e-8 + 1e-12, (e, vals[k])
    ac = complex(obs_row[2 + nstates], obs_row[3 + nstates])
    gre, gim = vals[k + 1]
    assert abs(ac.real - gre) <= 0.5e-8 + 1e-12 and abs(ac.imag - gim) <= 0.5e-8 + 1e-12, (ac, gre, gim)


def test_fft_matches_numpy():
    rng = np.random.default_rng(1)
    # 2^a 3^b 5^c and lengths with other prime factors (FFTW takes any N):
    # 7, 11 x 13, the primes 97 and 257 (above the radix buffers of 64)
    for n in [1, 2, 3, 5, 8, 9, 12, 64, 96, 128, 384, 1024, 1536, 3072, 4096, 7, 28, 143, 97, 257, 2 * 3 * 7 * 11]:
        x = rng.normal(size=n) + 1j * rng.normal(size=n)
        ref = np.fft.fft(x)
        sc = np.abs(ref).max()
        assert np.abs(O.fft1(x, -1) - ref).max() <= 1e-14 * sc, n
        assert np.abs(O.fft1(x, +1) - np.fft.ifft(x) * n).max() <= 1e-14 * sc


def test_fftn_matches_numpy():
    from qdng_gb300 import operators as op
    rng = np.random.default_rng(2)
    g = op.GridSystem([8, 6, 4], [0, 0, 0], [1, 1, 1])
    x = rng.normal(size=g.npts) + 1j * rng.normal(size=g.npts)
    ref = np.fft.fftn(x.reshape(4, 6, 8)).reshape(-1)
    assert np.abs(O.fftn(g, x, -1) - ref).max() <= 1e-13 * np.abs(ref).max()


def test_fft_sine_analytic():
    """FFTnTest-style known answer (src/tests/FFTnTest.cpp:27-125): a pure
    sine of k cycles has |F| = N/2 at bins k and N-k and 0 elsewhere."""
    for n, k in [(4, 1), (6, 2), (8, 3), (9, 2)]:
        x = np.sin(2 * np.pi * k * np.arange(n) / n).astype(np.complex128)
        F = np.abs(O.fft1(x, -1))
        expect = np.zeros(n)
        expect[k] = expect[n - k] = n / 2
        assert np.abs(F - expect).max() < 1e-10   # LOOSE_EPS (src/tests/defs.h)


def test_bessel_against_amos():
    """Cheby coefficients: J_n (ZBESJ) and e^-x I_n (ZBESI) vs SciPy's AMOS."""
    special = pytest.importorskip("scipy.special")
    for x in [0.5, 9.65, 11.39, 41.98, 185.96]:
        N = int(20 * x) + 50
        j, _ = O.bessel(0, N, x)
        i, _ = O.bessel(1, N, x)
        rj = special.jv(np.arange(N), x)
        ri = special.ive(np.arange(N), x)
        assert np.abs(j - rj).max() <= 5e-15 * max(1.0, np.abs(rj).max() * 10)
        m = ri > 1e-250
        assert (np.abs(i[m] - ri[m]) / ri[m]).max() < 1e-12


def test_nablasq_sine_eigenvalue():
    """OGridNablaSqTest-style known answer (src/tests/OGridNablaSqTest.cpp:76-139):
    on a periodic grid, sin(2 pi x/(L+dx)) is an eigenfunction of -1/(2m) d2/dx2
    with eigenvalue (2 pi/(L+dx))^2/(2m)."""
    from qdng_gb300 import operators as op
    for n in [8, 9]:
        g = op.GridSystem([n], [0.0], [1.0])
        dx = g.dx[0]
        x = g.axes()[0]
        kk = 2 * np.pi / (1.0 + dx)
        psi = np.sin(kk * x).astype(np.complex128)
        hp = op.HPlan(g, op.GridNablaSq([1.0]))
        Hpsi = O.System(hp).h_apply(psi)
        assert np.abs(Hpsi - 0.5 * kk ** 2 * psi).max() < 1e-10


def test_tgp_expec(fixtures, golden):
    hp, psi, run = cases.tgp_expec(fixtures)
    obs, terms = _last_line(hp, psi, run)
    _check(golden["propagation"]["TGP-Expec"], obs, 1)


def _expec_row(S, hp, x, V, fixtures=None):
    """The filterpost columns of the golden expec lines: GridMomentum,
    GridPosition, [Projection on ef_0..3], T, V."""
    row = [S.expec_momentum(x), S.expec_position(x)]
    if fixtures is not None:
        row.append(S.expec_projection(x, [fixtures[f"GridPot0_ef_{k}"] for k in range(4)]))
    row += [S.expec_kinetic(x), S.expec_grid(x, hp.grid_of(V))]
    return row


def _check_expec(golden_line, row):
    """Each value to the digits printed before the golden's [0-9]* wildcard."""
    for got, (txt, want) in zip(row, zip(golden_line["text"].split()[1:], golden_line["values"][1:])):
        mant = txt.split("[")[0].split("e")[0]
        digits = len(mant.split(".")[1]) if "." in mant else 0
        exp = int(txt.split("e")[1]) if "e" in txt else 0
        tol = 10.0 ** (exp - digits)
        assert abs(got - want) <= tol, (got, want, tol)


def test_tgp_expec_filters(fixtures, golden):
    """TGP-Expec's filterpost line after 1000 steps: <p>, <x>, the projection
    on the four eigenfunctions, <T>, <V>, each renormalised by <psi|psi>."""
    hp, psi, run = cases.tgp_expec(fixtures)
    S = O.System(hp)
    P = O.Propagator(S, run["name"], run["params"], dt=run["dt"])
    x = psi.copy()
    P.propagate(x, psi.copy(), run["steps"])
    V = hp  # the potential is the Sum's GridPotential
    row = [S.expec_momentum(x), S.expec_position(x),
           S.expec_projection(x, [fixtures[f"GridPot0_ef_{k}"] for k in range(4)]),
           S.expec_kinetic(x), S.expec_grid(x, 0)]
    _check_expec(golden["expec"]["TGP-Expec"], row)


@pytest.mark.parametrize("kinetic,name", [("FFT", "TGP-Expec-SP"), ("HOFD", "TGP-Expec-HOFD"),
                                          ("GMAT", "TGP-Gmat")])
def test_tgp_expec_kinetic_forms(fixtures, golden, kinetic, name):
    """One packet under three kinetic operators: GridNablaSq by FFT, by 8th
    order finite differences (OGridNablaSq method=HOFD) and the G-matrix
    (OGridGMat with G = 1/m): the Reporter line after 999 steps and the
    filterpost line (<p>, <x>, projection, <T>, <V>) against QDng."""
    hp, psi, run = cases.tgp_expec_lc(fixtures, kinetic)
    S = O.System(hp)
    P = O.Propagator(S, run["name"], run["params"], dt=run["dt"])
    x = psi.copy()
    obs, terms = P.propagate(x, psi.copy(), run["steps"])
    _check(golden["propagation"][name], obs[-1], 1)
    _check_expec(golden["expec"][name], _expec_row(S, hp, x, run["V"], fixtures))


def test_fd_weights_and_stencil():
    """The finite-difference weights (closed form) reproduce QDng's table
    values (HOFD.h cfd tables: order 2 {1, -2}, order 4 {-1/12, 4/3, -5/2}),
    and the 1-D HOFD stencil follows QDng's boundary rule: neighbours above
    the grid are dropped, those below it wrap to the top end."""
    n = 16
    g = op.GridSystem([n], [0.0], [float(n - 1)])
    for order, w in [(2, [1.0, -2.0]), (4, [-1 / 12, 4 / 3, -2.5])]:
        hp = op.HPlan(g, op.GridNablaSq([0.5], method="HOFD", order=order))
        S = O.System(hp)
        o2 = order // 2
        for i in [0, 1, n // 2, n - 1]:
            e = np.zeros(n, complex)
            e[i] = 1.0
            col = S.h_apply(e)  # column i of -1/(2m) D2 with m = 1/2, dx = 1: -D2
            want = np.zeros(n)
            want[i] += -w[o2]
            for k in range(1, o2 + 1):
                # point i feeds the point below it (i - k, if on the grid) through
                # that point's upper neighbour, and the point above (i + k) through
                # its lower neighbour, which wraps around
                if i - k >= 0:
                    want[i - k] += -w[o2 - k]
                want[(i + k) % n] += -w[o2 - k]
            assert np.allclose(col.real, want, rtol=0, atol=1e-13), (order, i, col.real, want)


def test_tgp_nip_cheby(fixtures, golden):
    """TGP-NIP-Cheby: a negative imaginary potential (Gobbler nip) absorbs the
    wave packet (norm 0.0959 after 999 steps); Reporter line and filterpost
    line (<p>, <x>, <T>, <V> of the nip-free Gobbler) against QDng."""
    hp, psi, run = cases.tgp_nip(fixtures)
    S = O.System(hp)
    emax, emin = S.erange()
    assert emin.imag == -0.02 and emax.real > 0
    P = O.Propagator(S, run["name"], run["params"], dt=run["dt"])
    x = psi.copy()
    obs, terms = P.propagate(x, psi.copy(), run["steps"])
    _check(golden["propagation"]["TGP-NIP-Cheby"], obs[-1], 1)
    _check_expec(golden["expec"]["TGP-NIP-Cheby"], _expec_row(S, hp, x, run["V"]))


def test_tgpms_cheby(fixtures, golden):
    hp, psi, run = cases.tgpms(fixtures)
    obs, _ = _last_line(hp, psi, run)
    _check(golden["propagation"]["TGPMS-Cheby"], obs, 2)


def test_tgpms_gspo(fixtures, golden):
    hp, psi, run = cases.tgpms(fixtures, gspo=True)
    obs, _ = _last_line(hp, psi, run)
    _check(golden["propagation"]["TGPMS-GSPO"], obs, 2)


def test_tgplms_cheby(fixtures, golden):
    hp, psi, run = cases.tgplms(fixtures)
    obs, _ = _last_line(hp, psi, run)
    _check(golden["propagation"]["TGPLMS-Cheby"], obs, 2)


def test_tgplms_sil(fixtures, golden):
    hp, psi, run = cases.tgplms(fixtures, sil=True)
    obs, _ = _last_line(hp, psi, run)
    _check(golden["propagation"]["TGPLMS-SIL"], obs, 2)


def test_tgpl_ir_pulse_cheby(fixtures, golden):
    hp, psi, run = cases.tgpl_ir_pulse(fixtures)
    obs, _ = _last_line(hp, psi, run)
    _check(golden["propagation"]["TGPL-IR-Pulse-Cheby"], obs, 1)


def test_tgpl_ir_pulse_gspo(fixtures, golden):
    hp, psi, run = cases.tgpl_ir_pulse(fixtures, gspo=True)
    obs, _ = _last_line(hp, psi, run)
    _check(golden["propagation"]["TGPL-IR-Pulse-GSPO"], obs, 1)


def test_tge_initial(fixtures, golden):
    hp, psi, run = cases.tge(fixtures, "Cheby")
    o = O.System(hp).observables(psi)
    n0, e0 = golden["tge_initial"]
    assert f"{np.sqrt(o['norm2']):.6e}" == n0
    assert f"{o['energy']:.6e}" == e0


@pytest.mark.parametrize("method", ["Cheby", "GSPO", "SIL", "Arnoldi"])
def test_tge_imag(fixtures, golden, method):
    hp, psi, run = cases.tge(fixtures, method)
    S = O.System(hp)
    P = O.Propagator(S, run["name"], run["params"], dt=run["dt"], imaginary_time=True, backward=True)
    _, e_raw, e_diag, steps = P.eigen_imag(psi, run["nef"], run["steps"], run["conv"], diag=True)
    for i, txt in golden["tge_imag"]:
        # energy.dat lines start with the grepped digits (ProgEigen WriteEnergyFile)
        dec = len(txt.split(".")[1])
        got = f"{e_diag[i]:.{dec + 3}f}"
        assert got.startswith(txt) or abs(e_diag[i] - float(txt)) < 1.5 * 10 ** (-dec), (method, i, e_diag[i], txt)


@pytest.mark.parametrize("method", ["Cheby", "SIL", "Arnoldi"])
def test_tge_autocorr(fixtures, golden, method):
    """TGE-<method>-ac: the normalised sum of the first six imaginary-time
    eigenfunctions propagated for 2048 steps of dt = 5; AutoCorrEF (Hann
    window, PeakFinder tol 1) must find the golden energies (energy.dat of
    the reference, 6 digits, raw energies: diag is off for ac)."""
    hp, psi, run = cases.tge(fixtures, method)
    S = O.System(hp)
    Pi = O.Propagator(S, run["name"], run["params"], dt=run["dt"], imaginary_time=True, backward=True)
    efs, _, _, _ = Pi.eigen_imag(psi, run["nef"], run["steps"], run["conv"], diag=True)
    lc = cases._normalize(hp, efs[:6].sum(axis=0))
    P = O.Propagator(S, run["name"], run["params"], dt=run["dt"])
    e, ef, spec, npk = P.eigen_autocorr(lc, 2048)
    assert npk >= 6
    for i, txt in golden["tge_ac"]:
        dec = len(txt.split(".")[1])
        assert abs(e[i] - float(txt)) < 1.5 * 10 ** (-dec), (method, i, e[i], txt)


def test_lanczos_eigen_driver(fixtures, golden):
    """ProgEigen::LanczosEF with the TGE Arnoldi propagator (order 15) on the
    normalised sum of six imaginary-time eigenfunctions: the Ritz values
    approach the golden eigenenergies (the ground state to the golden's
    digits, the others to the accuracy of the relaxed functions), and
    DiagBasis leaves them (the Ritz functions are H-orthogonal)."""
    hp, psi, run = cases.tge(fixtures, "Arnoldi")
    S = O.System(hp)
    Pi = O.Propagator(S, "Cheby", "", dt=5.0, imaginary_time=True, backward=True)
    efs, _, _, _ = Pi.eigen_imag(psi, run["nef"], run["steps"], run["conv"], diag=True)
    lc = cases._normalize(hp, efs[:6].sum(axis=0))
    P = O.Propagator(S, "Arnoldi", run["params"], dt=run["dt"])
    er, ed, ef, nb = P.eigen_lanczos(lc)
    assert nb == 15
    np.testing.assert_allclose(ed, er, rtol=1e-12, atol=1e-15)
    gold = [float(t) for _, t in golden["tge_imag"][:6]]
    assert abs(er[0] - gold[0]) < 1.5e-7
    np.testing.assert_allclose(er[:6], gold, rtol=2e-3)


@pytest.mark.parametrize("pbc", [False, True])
def test_gridhofd_derivatives(pbc):
    """OGridHOFD on a periodic function: first and second derivatives of
    order 8 agree with the analytic ones away from the ends (everywhere with
    pbc); the zero boundary drops the neighbours beyond the ends."""
    n = 64
    L = 2 * np.pi
    g = op.GridSystem([n], [0.0], [L * (n - 1) / n])  # dx = L / n: sin(3 x) is periodic on the grid
    x = g.axes()[0]
    f = np.sin(3 * x).astype(np.complex128)
    inner = slice(8, n - 8) if not pbc else slice(0, n)
    for deriv, want in [(1, 3 * np.cos(3 * x)), (2, -9 * np.sin(3 * x))]:
        S = O.System(op.HPlan(g, op.GridHOFD(deriv=deriv, order=8, pbc=pbc)))
        got = S.h_apply(f).real
        assert np.abs(got[inner] - want[inner]).max() < 1e-6, (deriv, np.abs(got[inner] - want[inner]).max())
    # zero boundary: the first point's second derivative lacks the neighbours below
    S = O.System(op.HPlan(g, op.GridHOFD(deriv=2, order=2, pbc=pbc)))
    e = np.zeros(n, complex)
    e[n - 1] = 1.0
    col = S.h_apply(e).real * g.dx[0] ** 2
    assert col[0] == (1.0 if pbc else 0.0) and col[n - 2] == 1.0 and col[n - 1] == -2.0


def test_gridhofd_mass_factor_and_erange():
    """With masses the factor is -1/(2 m) of the last dimension for both
    dimensions (OGridHOFD.cpp:74-91); Emax follows the per-dimension masses
    (OGridHOFD.cpp:97-111)."""
    g = op.GridSystem([32, 24], [-3.0, -2.0], [3.0, 2.0])
    rng = np.random.default_rng(2)
    psi = rng.normal(size=g.npts) + 1j * rng.normal(size=g.npts)
    a = O.System(op.HPlan(g, op.GridHOFD(deriv=2, order=4, mass=[100.0, 400.0]))).h_apply(psi)
    b = O.System(op.HPlan(g, op.GridHOFD(deriv=2, order=4))).h_apply(psi)
    assert np.allclose(a, b * (-1.0 / 800.0), rtol=1e-13, atol=0)
    emax, emin = O.System(op.HPlan(g, op.GridHOFD(deriv=2, order=4, mass=[100.0, 400.0]))).erange()
    dx = g.dx
    assert abs(emax - np.pi ** 2 / 2 * (1 / (100 * dx[0] ** 2) + 1 / (400 * dx[1] ** 2))) < 1e-12 * abs(emax)
    emax, emin = O.System(op.HPlan(g, op.GridHOFD(deriv=1, order=4, dim=1))).erange()
    assert emax == 1j * np.pi / dx[0] and emin == -1j * np.pi / dx[0]
