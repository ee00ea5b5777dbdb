"""Test systems: QDng's own integration-test inputs (tests/*.qdi.in) rebuilt
from the committed fixtures, and the seeded synthetic workloads.

Each builder returns (HPlan, psi0 [normalised, complex128], dict of run settings).
"""
import numpy as np

from qdng_gb300 import operators as op


def mgh_grid(fx):
    n, xmin, xmax = fx["GridPot0_grid"]
    return op.GridSystem([int(n)], [xmin], [xmax])


def _normalize(hp, psi):
    dx = np.prod(hp.grid.dx)
    return psi / np.sqrt((np.abs(psi) ** 2).sum() * dx)


def tgp_expec(fx):
    """tests/TGP-Expec.qdi.in: Cheby, Sum(T, V0), ef_0, dt=20, 1000 steps."""
    g = mgh_grid(fx)
    hp = op.HPlan(g, op.Sum([op.GridNablaSq([1763.2]), op.GridPotential(fx["GridPot0"])]))
    psi = _normalize(hp, fx["GridPot0_ef_0"].astype(np.complex128))
    return hp, psi, dict(name="Cheby", params="prec=1e-12", dt=20.0, steps=1000)


def tgp_expec_lc(fx, kinetic="FFT"):
    """tests/TGP-Expec-SP.qdi.in (kinetic="FFT"), TGP-Expec-HOFD.qdi.in ("HOFD":
    GridNablaSq method=HOFD order=8, prec 1e-10) and TGP-Gmat.qdi.in ("GMAT":
    GridGMat dims=1 with the GridGM_00 grid): Cheby, dt=20, 1000 steps, from the
    normalised linear combination of GridPot0_ef_0..3 (ChainLoader.cpp:257-284
    adds each function twice; the normalisation removes the factor)."""
    g = mgh_grid(fx)
    if kinetic == "GMAT":
        T = op.GridGMat(1, gmat={(0, 0): fx["GridGM_00"]})
    elif kinetic == "HOFD":
        T = op.GridNablaSq([1763.2], method="HOFD", order=8)
    else:
        T = op.GridNablaSq([1763.2])
    V = op.GridPotential(fx["GridPot0"])
    hp = op.HPlan(g, op.Sum([T, V]))
    psi = sum(2.0 * fx[f"GridPot0_ef_{k}"].astype(np.complex128) for k in range(4))
    prec = "1e-10" if kinetic == "HOFD" else "1e-12"
    return hp, _normalize(hp, psi), dict(name="Cheby", params=f"prec={prec}", dt=20.0, steps=1000, V=V)


def tgp_nip(fx):
    """tests/TGP-NIP-Cheby.qdi.in: Cheby, Sum(T, Gobbler nip rp0=5.5 order 5 gain 0.02,
    Gobbler lp0=2 order 20 gain 0.3 (key V)), ef_0, dt=10, 1000 steps."""
    g = mgh_grid(fx)
    V = op.Gobbler(dims=1, lp={0: 2.0}, order=20, gain=0.3, nip=False)
    hp = op.HPlan(g, op.Sum([op.GridNablaSq([1763.2]),
                             op.Gobbler(dims=1, rp={0: 5.5}, order=5, gain=0.02, nip=True), V]))
    psi = _normalize(hp, fx["GridPot0_ef_0"].astype(np.complex128))
    return hp, psi, dict(name="Cheby", params="", dt=10.0, steps=1000, V=V)


def tgpms(fx, gspo=False):
    """tests/TGPMS-Cheby.qdi.in / TGPMS-GSPO.qdi.in: two uncoupled states."""
    g = mgh_grid(fx)
    T = op.GridNablaSq([1763.2])
    V0, V1 = op.GridPotential(fx["GridPot0"]), op.GridPotential(fx["GridPot1"])
    if gspo:
        hp = op.HPlan(g, members=[op.DMultistate({(0, 0): T, (1, 1): op.GridNablaSq([1763.2])}),
                                  op.DMultistate({(0, 0): V0, (1, 1): V1})])
        run = dict(name="GSPO", params="", dt=2.0, steps=3000)
    else:
        hp = op.HPlan(g, op.Multistate({(0, 0): op.Sum([T, V0]), (1, 1): op.Sum([T, V1])}))
        run = dict(name="Cheby", params="prec=1e-12", dt=10.0, steps=1000)
    ef = fx["GridPot0_ef_0"].astype(np.complex128)
    psi = _normalize(hp, np.concatenate([ef, ef]))
    return hp, psi, run


def tgpl_ir_pulse(fx, gspo=False):
    """tests/TGPL-IR-Pulse-{Cheby,GSPO}.qdi.in: laser-driven single state."""
    g = mgh_grid(fx)
    T = op.GridNablaSq([1763.2])
    V = op.GridPotential(fx["GridPot0"])
    D = op.GridDipole(fx["GridDip0"], fx["GridLaser_w0p00713"])
    if gspo:
        hp = op.HPlan(g, members=[T, V, D])
        run = dict(name="GSPO", params="", dt=10.0, steps=6750)
    else:
        hp = op.HPlan(g, op.Sum([T, V, D]))
        run = dict(name="Cheby", params="prec=1e-12", dt=10.0, steps=6750)
    psi = _normalize(hp, fx["GridPot0_ef_0"].astype(np.complex128))
    return hp, psi, run


def tgplms(fx, sil=False):
    """tests/TGPLMS-{Cheby,SIL}.qdi.in: two states coupled by a dipole x field."""
    g = mgh_grid(fx)
    T = op.GridNablaSq([1763.2])
    H = op.Multistate({(0, 0): op.Sum([T, op.GridPotential(fx["GridPot0"])]),
                       (1, 1): op.Sum([T, op.GridPotential(fx["GridPot1"])]),
                       (1, 0): op.GridDipole(fx["GridDip01"], fx["GridLaser_w0p176"])})
    hp = op.HPlan(g, H)
    ef = fx["GridPot0_ef_0"].astype(np.complex128)
    psi = _normalize(hp, np.concatenate([ef, np.zeros_like(ef)]))
    run = dict(name="SIL", params="order=20", dt=1.0, steps=400) if sil else \
        dict(name="Cheby", params="prec=1e-12", dt=1.0, steps=400)
    return hp, psi, run


def tge(fx, method):
    """tests/TGE-<method>.qdi.in imaginary-time part: Sum(T, V0) on GridGauss, dt=5."""
    g = mgh_grid(fx)
    T, V = op.GridNablaSq([1763.2]), op.GridPotential(fx["GridPot0"])
    if method == "GSPO":
        hp = op.HPlan(g, members=[T, V])
        params = ""
    else:
        hp = op.HPlan(g, op.Sum([T, V]))
        params = {"Cheby": "", "SIL": "order=25", "Arnoldi": "order=15"}[method]
    psi = _normalize(hp, fx["GridGauss"].astype(np.complex128))
    return hp, psi, dict(name=method, params=params, dt=5.0, steps=1000, nef=10, conv=1e-5)


# ---------------------------------------------------------------- synthetic
def cfg1_morse(n=1024):
    """1-D Morse, 1024 points on [1,10], m=1728, D=0.1, a=1, re=2, Gaussian at 2.3 (sigma 0.2), dt=10."""
    g = op.GridSystem([n], [1.0], [10.0])
    x = g.axes()[0]
    V = 0.1 * (1 - np.exp(-(x - 2.0))) ** 2
    hp = op.HPlan(g, op.Sum([op.GridNablaSq([1728.0]), op.GridPotential(V)]))
    psi = _normalize(hp, np.exp(-(x - 2.3) ** 2 / (2 * 0.2 ** 2)).astype(np.complex128))
    return hp, psi, dict(name="Cheby", params="", dt=10.0, steps=2000)


def cfg2_two_state(n=256, gspo=False):
    """2-D two-state diabatic model on [-4,4]^2, masses (1836, 3672), k=0.02, dt=5."""
    g = op.GridSystem([n, n], [-4.0, -4.0], [4.0, 4.0])
    X, Y = g.mesh()
    k = 0.02
    V1 = 0.5 * k * (X ** 2 + Y ** 2)
    V2 = 0.5 * k * ((X - 1.0) ** 2 + Y ** 2) + 0.05
    V12 = 0.01 * np.exp(-(X - 0.5) ** 2 - Y ** 2)
    m = [1836.0, 3672.0]
    if gspo:
        hp = op.HPlan(g, members=[
            op.DMultistate({(0, 0): op.GridNablaSq(m), (1, 1): op.GridNablaSq(m)}),
            op.DMultistate({(0, 0): op.GridPotential(V1), (1, 1): op.GridPotential(V2),
                            (0, 1): op.GridPotential(V12)})])
        run = dict(name="GSPO", params="", dt=5.0, steps=4000)
    else:
        T = op.GridNablaSq(m)
        hp = op.HPlan(g, op.Multistate({(0, 0): op.Sum([T, op.GridPotential(V1)]),
                                        (1, 1): op.Sum([T, op.GridPotential(V2)]),
                                        (0, 1): op.GridPotential(V12)}))
        run = dict(name="Cheby", params="", dt=5.0, steps=4000)
    sig = [(mm * np.sqrt(k)) ** -0.5 for mm in m]
    g1 = np.exp(-(X - 0.3) ** 2 / (2 * sig[0] ** 2) - Y ** 2 / (2 * sig[1] ** 2))
    psi = np.concatenate([g1.reshape(-1), np.zeros(g.npts)]).astype(np.complex128)
    return hp, _normalize(hp, psi), run


def cfg3_anharmonic(n=128, seed=3):
    """3-D anharmonic oscillator on [-6,6]^3, m=1836, k=(0.01,0.015,0.02), +0.001 q0 q1 q2, dt=10."""
    g = op.GridSystem([n] * 3, [-6.0] * 3, [6.0] * 3)
    Q = g.mesh()
    kk = [0.01, 0.015, 0.02]
    V = sum(0.5 * kk[i] * Q[i] ** 2 for i in range(3)) + 0.001 * Q[0] * Q[1] * Q[2]
    hp = op.HPlan(g, op.Sum([op.GridNablaSq([1836.0] * 3), op.GridPotential(V)]))
    off = np.random.default_rng(seed).uniform(-0.5, 0.5, size=3)
    sig = [(1836.0 * np.sqrt(k)) ** -0.5 for k in kk]
    psi = np.exp(-sum((Q[i] - off[i]) ** 2 / (2 * sig[i] ** 2) for i in range(3)))
    return hp, _normalize(hp, psi.reshape(-1).astype(np.complex128)), dict(name="Cheby", params="", dt=10.0,
                                                                          steps=1000)


def cfg5_double_well(n=128):
    """2-D double well V=0.002(x^2-4)^2+0.01y^2 on [-5,5]^2, m=1836."""
    g = op.GridSystem([n, n], [-5.0, -5.0], [5.0, 5.0])
    X, Y = g.mesh()
    V = 0.002 * (X ** 2 - 4) ** 2 + 0.01 * Y ** 2
    hp = op.HPlan(g, op.Sum([op.GridNablaSq([1836.0, 1836.0]), op.GridPotential(V)]))
    psi = np.exp(-((X - 2.0) ** 2 + Y ** 2) / 0.5).reshape(-1).astype(np.complex128)
    return hp, _normalize(hp, psi), dict(name="Cheby", params="", dt=20.0, steps=2000)


def superposition(hp, funcs):
    """Normalised equal-weight superposition of the given wave functions
    (the start of the double-well Krylov propagation: its 8 relaxed states)."""
    return _normalize(hp, np.sum(np.asarray(funcs, dtype=np.complex128), axis=0))


def nac_two_state(n=128, nd=1, paired=True):
    """Two adiabatic harmonic states coupled by a first-derivative NAC
    (OGridNAC, the Handbook's Multistate example: m0.1 with sign +1 and m1.0
    with sign -1, which makes the matrix non-hermitian in QDng's sense and H
    itself hermitian).  paired=False gives m0.1 alone (hermitian copy).
    Returns (HPlan, psi0, run settings, coupling grids, NAC mass)."""
    m = 2000.0
    k = 0.01
    if nd == 1:
        g = op.GridSystem([n], [-6.0], [6.0])
        X = g.axes()[0]
        V0 = 0.5 * k * X ** 2
        V1 = 0.5 * k * (X - 1.0) ** 2 + 0.02
        f = [0.5 * np.exp(-X ** 2)]
        T = op.GridNablaSq([m])
        nac_mass = m
        psi = np.exp(-(X + 0.5) ** 2 / (2 * (m * np.sqrt(k)) ** -1.0))
    else:
        g = op.GridSystem([n, n], [-5.0, -5.0], [5.0, 5.0])
        X, Y = g.mesh()
        V0 = 0.5 * k * (X ** 2 + Y ** 2)
        V1 = 0.5 * k * ((X - 1.0) ** 2 + Y ** 2) + 0.02
        # N-D: the reduced mass is folded into the coupling data (mass = 1)
        f = [0.5 * np.exp(-X ** 2 - Y ** 2) / m, 0.2 * np.exp(-(X - 0.5) ** 2 - Y ** 2) / m]
        T = op.GridNablaSq([m, m])
        nac_mass = None
        sig = (m * np.sqrt(k)) ** -0.5
        psi = np.exp(-((X + 0.5) ** 2 + Y ** 2) / (2 * sig ** 2))
    el = {(0, 0): op.Sum([T, op.GridPotential(V0)]), (1, 1): op.Sum([T, op.GridPotential(V1)]),
          (0, 1): op.GridNAC(f, mass=nac_mass, sign=1.0)}
    if paired:
        el[(1, 0)] = op.GridNAC(f, mass=nac_mass, sign=-1.0)
    hp = op.HPlan(g, op.Multistate(el))
    psi = np.concatenate([psi.reshape(-1), np.zeros(g.npts)]).astype(np.complex128)
    f = [fd.reshape(-1) for fd in f]
    return hp, _normalize(hp, psi), dict(name="Cheby", params="", dt=10.0, steps=200), f, nac_mass


# ----------------------------------------------------------------- ensemble
ENS_1D_SIZES = [256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096]
ENS_2D_SIDES = [64, 96, 128, 192, 256]


def cfg4_member(rng, kind, size, nt=5000, dt=10.0):
    """One laser-driven Morse member of the 512-member ensemble; 2-D members add a
    harmonic y mode.  Box x in [1,10] (y in [-3,3]), mass 1728, dt 10."""
    D = rng.uniform(0.05, 0.2)
    a = rng.uniform(0.7, 1.3)
    re = rng.uniform(1.5, 2.5)
    E0 = rng.uniform(0.001, 0.02)
    w = rng.uniform(0.005, 0.02)
    m = 1728.0
    if kind == 1:
        g = op.GridSystem([size], [1.0], [10.0])
        x = g.axes()[0]
        V = D * (1 - np.exp(-a * (x - re))) ** 2
        mu = x * np.exp(-x / 4)
        sig = (m * a * np.sqrt(2 * D / m)) ** -0.5
        psi = np.exp(-(x - re - 0.1) ** 2 / (2 * sig ** 2)).astype(np.complex128)
        mass = [m]
    else:
        g = op.GridSystem([size, size], [1.0, -3.0], [10.0, 3.0])
        X, Y = g.mesh()
        ky = 0.01
        V = D * (1 - np.exp(-a * (X - re))) ** 2 + 0.5 * ky * Y ** 2
        mu = X * np.exp(-X / 4)
        sig = (m * a * np.sqrt(2 * D / m)) ** -0.5
        sy = (m * np.sqrt(ky / m)) ** -0.5
        psi = np.exp(-(X - re - 0.1) ** 2 / (2 * sig ** 2) - Y ** 2 / (2 * sy ** 2)).astype(np.complex128)
        mass = [m, m]
    T = nt * dt
    t = np.arange(nt) * dt
    laser = E0 * np.sin(np.pi * t / T) ** 2 * np.cos(w * t)
    psi = psi.reshape(-1)
    psi /= np.sqrt((np.abs(psi) ** 2).sum() * np.prod(g.dx))
    return dict(grid=g, mass=mass, V=V.reshape(-1), mu=mu.reshape(-1), laser=laser, psi=psi,
                params=dict(D=D, a=a, re=re, E0=E0, w=w))


def cfg4_ensemble(n=512, seed=4, frac_2d=0.25, sizes_1d=ENS_1D_SIZES, sides_2d=ENS_2D_SIDES, nt=5000):
    """The seeded 512-member ensemble; 1-D/2-D split and sizes drawn uniformly."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        if rng.uniform() < frac_2d:
            out.append(cfg4_member(rng, 2, int(rng.choice(sides_2d)), nt))
        else:
            out.append(cfg4_member(rng, 1, int(rng.choice(sizes_1d)), nt))
    return out


def member_hplan(mem):
    """The member as a QDng operator tree: Sum(GridNablaSq, GridPotential, GridDipole)."""
    return op.HPlan(mem["grid"], op.Sum([op.GridNablaSq(mem["mass"]), op.GridPotential(mem["V"]),
                                         op.GridDipole(mem["mu"], mem["laser"])]))


def lpt_partition(costs, nparts):
    """Largest-processing-time-first assignment of independent members to ranks
    (the package's, qdng_gb300.sharding)."""
    from qdng_gb300.sharding import lpt_partition as lpt
    return lpt(costs, nparts)
