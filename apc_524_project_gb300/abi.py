"""ctypes view of the C ABI in include/emoo.h.

The native library (libemoo.so, built in-tree by build_native.py) is the only
compute path: loading fails loudly when it is missing, there is no fallback.
"""
import ctypes as C
import os

NDIM = 3
NCHAR = 64
NSPEC = 32
NWAVE = 32

OK = 0
ERR_ARG = -1
ERR_OOM = -2
ERR_NOT_CONVERGED = -3
ERR_FIXED_OVERFLOW = -4
ERR_BOUNDS = -5
ERR_CUDA = -6
ERR_INPUT = -7
ERR_STATE = -8
ERR_UNSUPPORTED = -9

FP64 = 0
MIXED = 1

# field IDs (reference Grid / Poisson_Solver)
EX, EY, EZ, BX, BY, BZ, JX, JY, JZ, RHO, BX_TM1, BY_TM1, BZ_TM1 = range(13)
PHI1, AX1, AY1, AZ1, PHI2, AX2, AY2, AZ2 = range(13, 21)
NFIELDS = 21
FIELD_NAMES = ["Ex", "Ey", "Ez", "Bx", "By", "Bz", "Jx", "Jy", "Jz", "rho", "Bx_tm1", "By_tm1", "Bz_tm1",
               "phi1", "Ax1", "Ay1", "Az1", "phi2", "Ax2", "Ay2", "Az2"]
SEND_EB = -1
SEND_JRHO = -2


class InputInfo(C.Structure):
    """Binary twin of the reference's Input_Info_t (src/IO/input.hpp:15-126)."""

    _fields_ = [
        ("nCell", C.c_int * NDIM),
        ("nProc", C.c_int * NDIM),
        ("nt", C.c_int),
        ("restart", C.c_int),
        ("debug", C.c_int),
        ("relativity", C.c_int),
        ("electrostatic", C.c_int),
        ("nspecies", C.c_int),
        ("nstep_fields", C.c_int),
        ("nstep_parts", C.c_int),
        ("nstep_restart", C.c_int),
        ("nstep_sort", C.c_int),
        ("which_fields", C.c_int),
        ("output_pCount", C.c_int),
        ("nwaves", C.c_int),
        ("inSide", C.c_int * NWAVE),
        ("inPolE", C.c_int * NWAVE),
        ("isTestParticle", C.c_int * NSPEC),
        ("nparticles_tot", C.c_int64),
        ("nparticles_domain", C.c_int64),
        ("t0", C.c_double),
        ("dens_phys", C.c_double),
        ("super_ratio", C.c_double),
        ("mass_ratio", C.c_double * NSPEC),
        ("charge_ratio", C.c_double * NSPEC),
        ("dens_frac", C.c_double * NSPEC),
        ("temp", C.c_double * NSPEC),
        ("peakamps", C.c_double * NWAVE),
        ("omegas", C.c_double * NWAVE),
        ("phases", C.c_double * NWAVE),
        ("invWidths", C.c_double * NWAVE),
        ("delays", C.c_double * NWAVE),
        ("E0", C.c_double * NDIM),
        ("B0", C.c_double * NDIM),
        ("bound_phi", C.c_double * (2 * NDIM)),
        ("bound_Ax", C.c_double * (2 * NDIM)),
        ("bound_Ay", C.c_double * (2 * NDIM)),
        ("bound_Az", C.c_double * (2 * NDIM)),
        ("xyz0", C.c_double * NDIM),
        ("Lxyz", C.c_double * NDIM),
        ("distname", C.c_char * NCHAR),
        ("parts_init", C.c_char * NCHAR),
        ("fields_init", C.c_char * NCHAR),
        ("parts_bound", (C.c_char * NCHAR) * (2 * NDIM)),
        ("fields_bound", (C.c_char * NCHAR) * (2 * NDIM)),
    ]


class Opts(C.Structure):
    _fields_ = [
        ("precision", C.c_int),
        ("device", C.c_int),
        ("dt", C.c_double),
        ("capacity", C.c_int64),
        ("track_ids", C.c_int),
        ("deposit_rho", C.c_int),
        ("history_every", C.c_int),
        ("rho_background", C.c_double),
        ("rho_background_xmin", C.c_double),
        ("policy", C.c_int),
        ("poisson_solver", C.c_int),
        ("poisson_rtol", C.c_double),
    ]


class GenParams(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("species", C.c_int),
        ("relativistic_gamma", C.c_int),
        ("x0", C.c_double * 3),
        ("L", C.c_double * 3),
        ("vth", C.c_double * 3),
        ("vdrift", C.c_double * 3),
        ("dens_amp", C.c_double),
        ("dens_k", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("launches", C.c_int64),
        ("timed_launches", C.c_int64),
        ("timed_ms", C.c_double),
        ("ad_cell_mismatch", C.c_int64),
    ]


AD_FORWARD, AD_TANGENT, AD_ADJOINT = 0, 1, 2
AD_OBJ_FIELD, AD_OBJ_KINETIC = 0, 1
FIELDS_RHO, FIELDS_E, FIELDS_J, FIELDS_B, FIELDS_ALL = 0, 1, 2, 3, 4
POLICY_REFERENCE, POLICY_CORRECTED = 0, 1
POISSON_JACOBI, POISSON_MULTIGRID = 0, 1
NCOEF = 16


class AdSpec(C.Structure):
    _fields_ = [
        ("nsteps", C.c_int),
        ("checkpoint_every", C.c_int),
        ("slab_lo", C.c_int),
        ("slab_hi", C.c_int),
        ("objective", C.c_int),
        ("species", C.c_int),
    ]


class WaveShape(C.Structure):
    """emoo_wave_shape: transverse Gaussian spot and sine-series envelope of
    one injected wave."""

    _fields_ = [
        ("waist", C.c_double),
        ("center", C.c_double * 2),
        ("t_start", C.c_double),
        ("window", C.c_double),
        ("ncoef", C.c_int),
        ("coef", C.c_double * NCOEF),
    ]


class RestartDesc(C.Structure):
    _fields_ = [
        ("precision", C.c_int),
        ("n", C.c_int * 3),
        ("nspec", C.c_int),
        ("has_ids", C.c_int),
        ("np", C.c_int64),
        ("count", C.c_int64 * NSPEC),
        ("t", C.c_double),
        ("step_index", C.c_int64),
        ("nhist_rows", C.c_int64),
    ]


class AdResult(C.Structure):
    _fields_ = [
        ("objective", C.c_double),
        ("tangent", C.c_double),
        ("forward_ms", C.c_double),
        ("recompute_ms", C.c_double),
        ("reverse_ms", C.c_double),
    ]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I = C.POINTER(C.c_int)

# name -> (restype, argtypes); every symbol include/emoo.h declares
PROTOTYPES = {
    "emoo_default_opts": (C.c_int, [C.POINTER(Opts)]),
    "emoo_strerror": (C.c_char_p, [C.c_int]),
    "emoo_create": (C.c_int, [C.POINTER(InputInfo), C.POINTER(Opts), C.POINTER(_P)]),
    "emoo_destroy": (C.c_int, [_P]),
    "emoo_load_particles": (C.c_int, [_P, C.c_int, C.c_int64, _D, _D, _D, _D, _D, _D, _D, _I64]),
    "emoo_generate_host": (C.c_int, [C.POINTER(GenParams), C.c_int64, C.c_int64, _D, _D, _D, _D, _D, _D, _D]),
    "emoo_load_generated": (C.c_int, [_P, C.POINTER(GenParams), C.c_int64]),
    "emoo_num_particles": (C.c_int, [_P, C.c_int, _I64]),
    "emoo_get_particles": (C.c_int, [_P, C.c_int, C.c_int64, _D, _D, _D, _D, _D, _D, _D, _I64, _I64]),
    "emoo_get_particle_fields": (C.c_int, [_P, C.c_int, C.c_int64, _D, _D, _D, _D, _D, _D, _I64]),
    "emoo_get_field": (C.c_int, [_P, C.c_int, _D]),
    "emoo_set_field": (C.c_int, [_P, C.c_int, _D]),
    "emoo_cell_id": (C.c_int, [_P, C.c_double, C.c_double, C.c_double, _I]),
    "emoo_init_fields": (C.c_int, [_P, _I]),
    "emoo_poisson_init": (C.c_int, [_P, _I]),
    "emoo_sort": (C.c_int, [_P]),
    "emoo_interpolate": (C.c_int, [_P]),
    "emoo_push": (C.c_int, [_P]),
    "emoo_apply_particle_bc": (C.c_int, [_P, _I64]),
    "emoo_deposit": (C.c_int, [_P, C.c_int]),
    "emoo_execute_bc": (C.c_int, [_P, C.c_int]),
    "emoo_evolve_fields": (C.c_int, [_P, C.c_int]),
    "emoo_step": (C.c_int, [_P, C.c_int, _I64]),
    "emoo_history": (C.c_int, [_P, _D]),
    "emoo_history_rows": (C.c_int, [_P, C.c_int, _D, _I]),
    "emoo_gauss_residual": (C.c_int, [_P, _D]),
    "emoo_time": (C.c_int, [_P, _D, _D]),
    "emoo_check": (C.c_int, [_P]),
    "emoo_perturb": (C.c_int, [_P, C.c_uint64, C.c_double]),
    "emoo_read_input": (C.c_int, [C.c_char_p, C.POINTER(InputInfo)]),
    "emoo_parse_input": (C.c_int, [C.c_char_p, C.POINTER(InputInfo)]),
    "emoo_input_message": (C.c_char_p, []),
    "emoo_process_info": (C.c_int, [C.POINTER(InputInfo)]),
    "emoo_set_particles": (C.c_int, [_P, C.c_int, C.c_int64, _D, _D, _D, _D, _D, _D, _D]),
    "emoo_attach_particles": (C.c_int, [_P, C.c_int, C.c_int64, _D, _D, _D, _D, _D, _D, _D]),
    "emoo_detach_particles": (C.c_int, [_P]),
    "emoo_get_stream": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "emoo_set_profiling": (C.c_int, [_P, C.c_int]),
    "emoo_get_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "emoo_sort_permutation_noalloc": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_void_p]),
    "emoo_set_waves": (C.c_int, [_P, C.c_int, _D, _D]),
    "emoo_set_wave_shape": (C.c_int, [_P, C.c_int, C.POINTER(WaveShape)]),
    "emoo_ad_nparams": (C.c_int, [_P]),
    "emoo_write_fields": (C.c_int, [_P, C.c_char_p, C.c_int]),
    "emoo_write_restart": (C.c_int, [_P, C.c_char_p]),
    "emoo_read_restart": (C.c_int, [_P, C.c_char_p]),
    "emoo_restart_info": (C.c_int, [C.c_char_p, C.POINTER(RestartDesc)]),
    "emoo_ad_run": (C.c_int, [_P, C.POINTER(AdSpec), C.c_int, _D, _D, C.POINTER(AdResult), _D, _D]),
}

NOALLOC_SORT_MAX = 1048576

_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libemoo.so")


class EmooError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = _strerror(status)
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


def _strerror(status):
    try:
        return lib().emoo_strerror(status).decode()
    except Exception:  # library not loadable: plain code
        return f"status {status}"


def lib():
    """Loads libemoo.so (raises if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"native library not built: {LIB_PATH} (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status, what=""):
    if status != OK:
        raise EmooError(status, what)
    return status
