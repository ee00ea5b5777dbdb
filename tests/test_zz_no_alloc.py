"""qdg_h_apply_noalloc: H psi for callers that cannot allocate device memory.

Frameworks whose memory pool owns all device memory, or plug-ins that must
not change the process's allocation state, cannot let a library call
cudaMalloc.  This entry
point takes device arrays the caller owns and keeps its own scratch in a
static device array of the library, so it must give the same H psi as the
plan-based qdg_h_apply.  Collected last so that a failure here comes after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from qdng_gb300 import abi, operators as op

pytestmark = pytest.mark.gpu


def _case_2d():
    g = op.GridSystem([64, 48], [-4.0, -3.0], [4.0, 3.5])
    X, Y = g.mesh()
    V1 = 0.01 * (X ** 2 + Y ** 2)
    V2 = 0.01 * ((X - 1) ** 2 + Y ** 2) + 0.05
    mu = 0.3 * X * np.exp(-0.1 * Y ** 2)
    laser = 0.02 * np.sin(0.3 * np.arange(16))
    T = op.GridNablaSq([1836.0, 3672.0])
    hp = op.HPlan(g, op.Multistate({(0, 0): op.Sum([T, op.GridPotential(V1)]),
                                    (1, 1): op.Sum([T, op.GridPotential(V2)]),
                                    (0, 1): op.GridDipole(mu, laser)}))
    return hp


def _case_1d():
    g = op.GridSystem([384], [1.0], [10.0])
    x = g.axes()[0]
    return op.HPlan(g, op.Sum([op.GridNablaSq([1728.0]), op.GridPotential(0.1 * (1 - np.exp(-(x - 2))) ** 2)]))


def _case_3d():
    g = op.GridSystem([16, 8, 12], [-4.0, -3.0, -5.0], [4.0, 3.0, 5.0])
    Q = g.mesh()
    V = 0.01 * Q[0] ** 2 + 0.02 * Q[1] ** 2 + 0.015 * Q[2] ** 2 + 0.001 * Q[0] * Q[1] * Q[2]
    return op.HPlan(g, op.Sum([op.GridNablaSq([1836.0, 900.0, 2000.0]), op.GridPotential(V)]))


def _case_prime_lengths():
    """Lines of 28 and 21 points (prime factors 7 and 3, 7): direct-DFT stages."""
    g = op.GridSystem([28, 21], [-4.0, -3.0], [4.0, 3.5])
    X, Y = g.mesh()
    return op.HPlan(g, op.Sum([op.GridNablaSq([900.0, 1200.0]), op.GridPotential(0.02 * (X ** 2 + Y ** 2))]))


def _case_three_states(nonhermitian=False):
    """Three states with off-diagonal potentials and a dipole coupling; with
    nonhermitian=True the (j, i) elements are not mirrored."""
    g = op.GridSystem([48, 40], [-4.0, -4.0], [4.0, 4.0])
    X, Y = g.mesh()
    T = op.GridNablaSq([1500.0, 2500.0])
    mu = 0.2 * X * np.exp(-0.1 * Y ** 2)
    laser = 0.03 * np.cos(0.2 * np.arange(10))
    el = {(0, 0): op.Sum([T, op.GridPotential(0.01 * (X ** 2 + Y ** 2))]),
          (1, 1): op.Sum([T, op.GridPotential(0.01 * ((X - 1) ** 2 + Y ** 2) + 0.02)]),
          (2, 2): op.Sum([T, op.GridPotential(0.012 * (X ** 2 + (Y - 0.5) ** 2) + 0.04)]),
          (0, 1): op.GridPotential(0.005 * np.exp(-X ** 2 - Y ** 2)),
          (1, 2): op.GridDipole(mu, laser),
          (0, 2): op.GridPotential(0.002 * np.exp(-(X - 0.5) ** 2))}
    if nonhermitian:
        el[(1, 0)] = op.GridPotential(0.003 * np.exp(-(Y - 0.3) ** 2))
    return op.HPlan(g, op.Multistate(el, nonhermitian=nonhermitian))


def _noalloc_apply(lib, hp, psi, step, torch):
    dev = torch.device("cuda")
    grids = torch.from_numpy(np.ascontiguousarray(hp.grid_data)).to(dev)
    lasers = torch.from_numpy(np.ascontiguousarray(hp.laser_data)).to(dev)
    x = torch.from_numpy(np.ascontiguousarray(psi).view(np.float64)).to(dev)
    y = torch.empty_like(x)
    d = abi.HPlanDesc()
    C.pointer(d)[0] = hp.desc
    d.grid_data = C.cast(C.c_void_p(grids.data_ptr()), C.POINTER(C.c_double))
    d.laser_data = C.cast(C.c_void_p(lasers.data_ptr()), C.POINTER(C.c_double))
    stream = torch.cuda.current_stream()
    rc = lib.qdg_h_apply_noalloc(C.byref(d), C.cast(C.c_void_p(x.data_ptr()), C.POINTER(C.c_double)),
                                 C.cast(C.c_void_p(y.data_ptr()), C.POINTER(C.c_double)), step,
                                 C.c_void_p(stream.cuda_stream))
    assert rc == abi.QDG_OK, lib.qdg_last_error().decode()
    torch.cuda.synchronize()
    return y.cpu().numpy().view(np.complex128).copy()


@pytest.mark.parametrize("builder", [_case_2d, _case_1d, _case_3d, _case_three_states,
                                     lambda: _case_three_states(nonhermitian=True), _case_prime_lengths],
                         ids=["2d", "1d", "3d", "three-states", "three-states-nonhermitian", "prime-lengths"])
def test_noalloc_matches_plan_h_apply(builder):
    torch = pytest.importorskip("torch")
    from qdng_gb300 import build, engine
    from qdng_gb300._lib import load
    build.build()
    lib = load()
    hp = builder()
    plan = engine.Plan(hp, "fp64")
    rng = np.random.default_rng(11)
    # calls in a row with different inputs and field steps, including steps
    # before the first and past the last field sample (the field is zero there)
    nt = hp.desc.laser_nt
    for call, step in enumerate([3, 7, -1, max(nt, 1)]):
        psi = rng.normal(size=hp.size) + 1j * rng.normal(size=hp.size)
        a, b = plan.wavefunction(psi), plan.wavefunction()
        plan.h_apply(a, b, step)
        ref = b.download()
        got = _noalloc_apply(lib, hp, psi, step, torch)
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < 1e-13, (call, err)


def test_noalloc_rejects_oversized_problem():
    torch = pytest.importorskip("torch")
    from qdng_gb300._lib import load
    lib = load()
    g = op.GridSystem([256, 256, 64], [-1.0] * 3, [1.0] * 3)  # 3 x 4M complex128 of scratch > 8 MiB
    hp = op.HPlan(g, op.GridNablaSq([1.0, 1.0, 1.0]))
    x = torch.zeros(hp.size * 2, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    rc = lib.qdg_h_apply_noalloc(C.byref(hp.desc), C.cast(C.c_void_p(x.data_ptr()), C.POINTER(C.c_double)),
                                 C.cast(C.c_void_p(y.data_ptr()), C.POINTER(C.c_double)), 0, None)
    assert rc == abi.QDG_EINVAL
    assert "scratch" in lib.qdg_last_error().decode()


@pytest.mark.parametrize("kinetic", ["HOFD", "GMAT"])
def test_noalloc_rejects_table_free_kinetic(kinetic):
    """Finite-difference (method HOFD) and G-matrix kinetic operators need a
    plan's buffers: the no-alloc entry refuses them instead of applying an
    FFT kinetic in their place."""
    torch = pytest.importorskip("torch")
    from qdng_gb300._lib import load
    lib = load()
    g = op.GridSystem([64], [-1.0], [1.0])
    T = op.GridNablaSq([1.0], method="HOFD") if kinetic == "HOFD" else op.GridGMat(1, G=[1.0])
    hp = op.HPlan(g, op.Sum([T, op.GridPotential(np.zeros(64))]))
    x = torch.zeros(hp.size * 2, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    rc = lib.qdg_h_apply_noalloc(C.byref(hp.desc), C.cast(C.c_void_p(x.data_ptr()), C.POINTER(C.c_double)),
                                 C.cast(C.c_void_p(y.data_ptr()), C.POINTER(C.c_double)), 0, None)
    assert rc == abi.QDG_EUNSUPPORTED
