"""CPU checks of the drop-in boundary: libqdg.so builds for sm_103a, loads
without a GPU, exports every function include/qdg.h declares, and the ctypes
layouts match the C structs; host-side tree flattening of operators.py."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from qdng_gb300 import abi, operators as op

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "qdg.h")


@pytest.fixture(scope="module")
def lib():
    from qdng_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_exports_every_header_symbol(lib):
    names = abi.header_symbols(HEADER)
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    declared = {n for n, _, _ in abi.SIGNATURES}
    assert set(names) == declared


def test_abi_version(lib):
    assert lib.qdg_abi_version() == 3


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "qdg.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(qdg_grid), sizeof(qdg_hterm),'
                   ' sizeof(qdg_hplan_desc), sizeof(qdg_observables), sizeof(qdg_prop_info),'
                   ' offsetof(qdg_hterm, mass), offsetof(qdg_hplan_desc, laser_data));'
                   ' printf("%zu %zu\\n", offsetof(qdg_hterm, sign), offsetof(qdg_hplan_desc, nonhermitian));'
                   ' printf("%zu %zu\\n", sizeof(qdg_ensemble_member), offsetof(qdg_ensemble_member, laser_nt));'
                   ' return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    want = [C.sizeof(abi.Grid), C.sizeof(abi.HTerm), C.sizeof(abi.HPlanDesc), C.sizeof(abi.Observables),
            C.sizeof(abi.PropInfo), abi.HTerm.mass.offset, abi.HPlanDesc.laser_data.offset,
            abi.HTerm.sign.offset, abi.HPlanDesc.nonhermitian.offset,
            C.sizeof(abi.EnsembleMember), abi.EnsembleMember.laser_nt.offset]
    assert got == want


def test_status_without_gpu_is_an_error_not_a_crash(lib):
    """No device here: plan creation must fail with a status, never fall back to the CPU."""
    g = op.GridSystem([16], [0.0], [1.0])
    hp = op.HPlan(g, op.Sum([op.GridNablaSq([1.0]), op.GridPotential(np.linspace(0, 1, 16))]))
    h = C.c_void_p()
    rc = lib.qdg_plan_create(C.byref(hp.desc), 0, C.byref(h))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    assert rc == abi.QDG_ECUDA
    assert lib.qdg_last_error().decode()


def test_multistate_flattening():
    g = op.GridSystem([8, 4], [0, 0], [1, 1])
    V = np.arange(32.0)
    T = op.GridNablaSq([2.0, 3.0])
    D = op.GridDipole(V, np.ones(5))
    hp = op.HPlan(g, op.Multistate({(0, 0): op.Sum([T, op.GridPotential(V)]), (1, 1): T, (1, 0): D}))
    kinds = [(t.kind, t.row, t.col) for t in hp.terms]
    assert kinds == [(abi.TERM_KINETIC, 0, 0), (abi.TERM_POTENTIAL, 0, 0), (abi.TERM_DIPOLE, 1, 0),
                     (abi.TERM_KINETIC, 1, 1)]
    assert hp.nstates == 2 and hp.ngrids == 2 and hp.nlasers == 1 and hp.laser_nt == 5
    assert list(hp.terms[0].mass)[:2] == [2.0, 3.0]


def test_gspo_members_set_groups():
    g = op.GridSystem([8], [0], [1])
    hp = op.HPlan(g, members=[op.GridNablaSq([1.0]), op.GridPotential(np.zeros(8)),
                              op.GridDipole(np.ones(8), np.zeros(3))])
    assert [t.group for t in hp.terms] == [0, 1, 2]


def test_reference_parameter_errors():
    with pytest.raises(op.EParamProblem):
        op.GridNablaSq([0.0])            # "Zero mass defined" (OGridNablaSq.cpp:47-48)
    with pytest.raises(op.EParamProblem):
        op.GridSystem([0], [0], [1])     # "Zero points grid defined"
    with pytest.raises(op.EParamProblem):
        op.GridSystem([4], [1], [1])     # "Zero length grid defined"
    g = op.GridSystem([8], [0], [1])
    with pytest.raises(op.EIncompatible):
        op.HPlan(g, op.GridPotential(np.zeros(9)))


def test_potential_setzero_offset_scale():
    v = op.GridPotential(np.array([3.0, 1.0, 2.0]), setzero=True, offset=0.5, scale=2.0).values
    assert np.allclose(v, (np.array([3.0, 1.0, 2.0]) - 1.0 + 0.5) * 2.0)   # OGridPotential.cpp:56-76


def test_nac_flattening_and_nonhermitian_flag():
    """GridNAC takes one grid slot per dimension; elements at both (0,1) and
    (1,0) make the Multistate non-hermitian (OMultistate.cpp:52-53)."""
    g = op.GridSystem([8, 4], [0.0, 0.0], [1.0, 1.0])
    f0, f1 = np.ones(32), 2 * np.ones(32)
    V = op.GridPotential(np.zeros(32))
    hp = op.HPlan(g, op.Multistate({(0, 0): V, (1, 1): V, (0, 1): op.GridNAC([f0, f1], mass=5.0, sign=-1)}))
    t = [x for x in hp.terms if x.kind == abi.TERM_NAC][0]
    assert (t.row, t.col, t.sign, t.mass[0]) == (0, 1, -1.0, 1.0)  # N-D: mass folded into f
    np.testing.assert_array_equal(hp.grid_data[t.grid * 32:(t.grid + 2) * 32], np.concatenate([f0, f1]))
    assert hp.desc.nonhermitian == 0
    hp2 = op.HPlan(g, op.Multistate({(0, 0): V, (1, 1): V, (0, 1): op.GridNAC([f0, f1]),
                                     (1, 0): op.GridNAC([f0, f1], sign=-1)}))
    assert hp2.desc.nonhermitian == 1
    g1 = op.GridSystem([8], [0.0], [1.0])
    hp3 = op.HPlan(g1, op.Multistate({(0, 1): op.GridNAC([np.ones(8)], mass=5.0)}, nonhermitian=True))
    t3 = hp3.terms[0]
    assert t3.mass[0] == 5.0 and hp3.desc.nonhermitian == 1
