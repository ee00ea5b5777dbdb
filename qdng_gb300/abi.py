"""ctypes mirror of include/qdg.h (data layouts only; loading libqdg.so lives in _lib.py).

Every structure here matches the C declaration field for field; the
reference classes each one replaces are cited in include/qdg.h.
"""
import ctypes as C

QDG_MAX_DIMS = 4
QDG_MAX_STATES = 64

QDG_OK = 0
QDG_EINVAL = 1
QDG_ENONFINITE = 2
QDG_ETIMEOUT = 3
QDG_ECUDA = 4
QDG_ENOMEM = 5
QDG_EUNSUPPORTED = 6
QDG_ENOTCONVERGED = 7

STATUS_NAMES = {
    0: "QDG_OK", 1: "QDG_EINVAL", 2: "QDG_ENONFINITE", 3: "QDG_ETIMEOUT",
    4: "QDG_ECUDA", 5: "QDG_ENOMEM", 6: "QDG_EUNSUPPORTED", 7: "QDG_ENOTCONVERGED",
}

TERM_KINETIC = 1
TERM_POTENTIAL = 2
TERM_DIPOLE = 3
TERM_NAC = 4
TERM_GOBBLER = 5
TERM_GMAT = 6
TERM_HOFD = 7

PREC_FP64 = 0
PREC_MIXED = 1
PREC_DF64 = 2


class Grid(C.Structure):
    _fields_ = [
        ("ndims", C.c_int32),
        ("n", C.c_int32 * QDG_MAX_DIMS),
        ("xmin", C.c_double * QDG_MAX_DIMS),
        ("xmax", C.c_double * QDG_MAX_DIMS),
    ]


class HTerm(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("row", C.c_int32),
        ("col", C.c_int32),
        ("grid", C.c_int32),
        ("laser", C.c_int32),
        ("group", C.c_int32),
        ("mass", C.c_double * QDG_MAX_DIMS),
        ("sign", C.c_double),
        ("fd_order", C.c_int32),
        ("flags", C.c_int32),
    ]


class HPlanDesc(C.Structure):
    _fields_ = [
        ("grid", Grid),
        ("nstates", C.c_int32),
        ("nterms", C.c_int32),
        ("terms", C.POINTER(HTerm)),
        ("ngrids", C.c_int32),
        ("grid_data", C.POINTER(C.c_double)),
        ("nlasers", C.c_int32),
        ("laser_nt", C.c_int32),
        ("laser_data", C.POINTER(C.c_double)),
        ("nonhermitian", C.c_int32),
    ]


class Observables(C.Structure):
    _fields_ = [
        ("norm2", C.c_double),
        ("pops", C.c_double * QDG_MAX_STATES),
        ("energy", C.c_double),
        ("autocorr_re", C.c_double),
        ("autocorr_im", C.c_double),
    ]


class PropInfo(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("order", C.c_int32),
        ("scaling", C.c_double),
        ("offset_re", C.c_double),
        ("offset_im", C.c_double),
        ("exponent_re", C.c_double),
        ("exponent_im", C.c_double),
    ]


class EnsembleMember(C.Structure):
    _fields_ = [
        ("grid", Grid),
        ("mass", C.c_double * QDG_MAX_DIMS),
        ("potential", C.POINTER(C.c_double)),
        ("dipole", C.POINTER(C.c_double)),
        ("laser", C.POINTER(C.c_double)),
        ("laser_nt", C.c_int32),
    ]


# Every symbol include/qdg.h declares: (name, restype, argtypes).
_vp = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_dp = C.POINTER(C.c_double)
SIGNATURES = [
    ("qdg_last_error", C.c_char_p, []),
    ("qdg_abi_version", _i32, []),
    ("qdg_plan_create", _i32, [C.POINTER(HPlanDesc), _i32, C.POINTER(_vp)]),
    ("qdg_plan_destroy", _i32, [_vp]),
    ("qdg_plan_erange", _i32, [_vp, _dp, _dp]),
    ("qdg_plan_set_stream", _i32, [_vp, _vp]),
    ("qdg_plan_synchronize", _i32, [_vp]),
    ("qdg_wf_create", _i32, [_vp, C.POINTER(_vp)]),
    ("qdg_wf_destroy", _i32, [_vp]),
    ("qdg_wf_upload", _i32, [_vp, _dp]),
    ("qdg_wf_download", _i32, [_vp, _dp]),
    ("qdg_wf_copy", _i32, [_vp, _vp]),
    ("qdg_h_apply", _i32, [_vp, _vp, _vp, _i64]),
    ("qdg_observables_compute", _i32, [_vp, _vp, _vp, _i64, C.POINTER(Observables)]),
    ("qdg_eigen_autocorr", _i32, [_vp, C.POINTER(C.c_double), _i32, C.c_double, _i32, _i32, _i32,
                                  C.POINTER(C.c_double), C.POINTER(_i32), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]),
    ("qdg_eigen_lanczos", _i32, [_vp, C.POINTER(C.c_double), _i32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(_i32), C.POINTER(C.c_double)]),
    ("qdg_expec_position", _i32, [_vp, _vp, _i32, C.c_double, C.POINTER(C.c_double)]),
    ("qdg_expec_momentum", _i32, [_vp, _vp, _i32, C.c_double, C.POINTER(C.c_double)]),
    ("qdg_expec_kinetic", _i32, [_vp, _vp, C.POINTER(C.c_double)]),
    ("qdg_expec_grid", _i32, [_vp, _vp, _i32, C.POINTER(C.c_double)]),
    ("qdg_expec_projection", _i32, [_vp, _vp, C.POINTER(C.POINTER(C.c_double)), _i32, C.POINTER(C.c_double)]),
    ("qdg_prop_create", _i32, [_vp, C.c_char_p, C.c_char_p, C.c_double, _i32, _i32, C.POINTER(_vp)]),
    ("qdg_prop_destroy", _i32, [_vp]),
    ("qdg_prop_init", _i32, [_vp]),
    ("qdg_prop_get_info", _i32, [_vp, C.POINTER(PropInfo)]),
    ("qdg_prop_get_coeffs", _i32, [_vp, _dp, _i32]),
    ("qdg_prop_apply", _i32, [_vp, _vp, _i64, C.POINTER(_i32)]),
    ("qdg_prop_apply_host", _i32, [_vp, _vp, _dp, _i64, C.POINTER(_i32)]),
    ("qdg_prop_apply_host_states", _i32, [_vp, _vp, C.POINTER(_dp), _i64, C.POINTER(_i32)]),
    ("qdg_prop_run", _i32, [_vp, _vp, _i64, _i32, C.POINTER(_i64)]),
    ("qdg_ensemble_timeline", _i32, [_vp, _vp, _vp]),
    ("qdg_eigen_imag", _i32, [_vp, _vp, _i32, _i32, C.c_double, _i32, _vp, _vp, _vp, _vp]),
    ("qdg_kernel_launches", _i64, []),
    ("qdg_profile_enable", _i32, [_vp, _i32]),
    ("qdg_profile_read", _i32, [_vp, _dp, C.POINTER(_i64)]),
    ("qdg_prop_phase_times", _i32, [_vp, _dp]),
    ("qdg_plan_inject_barrier_stall", _i32, [_vp]),
    ("qdg_h_apply_noalloc", _i32, [C.POINTER(HPlanDesc), _dp, _dp, _i64, _vp]),
    ("qdg_fft_schedule_set", _i32, [_i32, _i32, _i32, C.POINTER(_i32), _i32, _i32]),
    ("qdg_fft_schedule_get", _i32, [_i32, _i32, _i32, C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_i32)]),
    ("qdg_fft_schedule_reset", _i32, [_i32]),
    ("qdg_ensemble_create", _i32, [C.POINTER(EnsembleMember), _i32, C.c_double, C.c_char_p, _i32, C.POINTER(_vp)]),
    ("qdg_ensemble_destroy", _i32, [_vp]),
    ("qdg_ensemble_upload", _i32, [_vp, _dp]),
    ("qdg_ensemble_download", _i32, [_vp, _dp]),
    ("qdg_ensemble_run", _i32, [_vp, _i64, _i32, C.POINTER(_i64)]),
    ("qdg_ensemble_member_info", _i32, [_vp, _i32, C.POINTER(PropInfo)]),
]


def header_symbols(path):
    """Names of the functions declared in a qdg header (for the export test)."""
    import re
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qdg_[a-z0-9_]+)\s*\(", text)))
