"""ctypes binding of libgbmg.so (the C ABI declared in include/gbmg.h).

The library is loaded from the package's own _build directory; importing this
module never falls back to anything else.  If the library is missing it is
built with fortrancfd_gb300.build (nvcc, sm_103a), and a failed build raises.
"""
import ctypes as C
import os
import threading

from . import build as _build

GBMG_OK = 0
GBMG_NOT_CONVERGED = 1
GBMG_DIVERGED = 2
GBMG_INVALID_ARG = 3
GBMG_CUDA_ERROR = 4
GBMG_NO_DEVICE = 5
GBMG_OUT_OF_MEMORY = 6
GBMG_STATE_ERROR = 7

GBMG_PREC_FP64 = 0
GBMG_PREC_MIXED = 1
GBMG_STOP_RELATIVE = 0
GBMG_STOP_RMS = 1
GBMG_STOP_INCREMENT = 2
GBMG_MEM_HOST = 0
GBMG_MEM_DEVICE = 1

# Every symbol include/gbmg.h declares (checked by the tests).
EXPORTS = (
    "gbmg_default_params", "gbmg_create", "gbmg_destroy", "gbmg_set_rho", "gbmg_set_phi",
    "gbmg_set_coef", "gbmg_solve", "gbmg_project", "gbmg_divergence", "gbmg_residual",
    "gbmg_div_stats", "gbmg_level_coef", "gbmg_level_dims", "gbmg_kernel_launches",
    "gbmg_strerror", "gbmg_last_error", "gbmg_set_profiling", "gbmg_profile", "gbmg_adjoint",
    "gbmg_div_stats_noalloc", "gbmg_set_split", "gbmg_project_split",
    "gbmg_ls_create", "gbmg_ls_destroy", "gbmg_ls_advect", "gbmg_ls_redistance",
    "gbmg_ls_kernel_launches", "gbmg_ls_last_error",
    "gbmg_ns_ab_step", "gbmg_ns_ab_predict", "gbmg_ns_velbc", "gbmg_ns_curvature",
    "gbmg_ns_rho_mu", "gbmg_ns_bc", "gbmg_ns_mass_correct", "gbmg_ns_vof_advect", "gbmg_ns_ibm",
)

PROF_CLASSES = ("smooth_fine", "smooth_coarse", "restrict_fine", "restrict_coarse",
                "prolong_fine", "prolong_coarse", "coarse_solve", "residual", "vector", "setup",
                "certify", "momentum")


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]


class Params(C.Structure):
    _fields_ = [("precision", C.c_int32), ("nu1", C.c_int32), ("nu2", C.c_int32),
                ("levels", C.c_int32), ("coarse_max", C.c_int32), ("max_cycles", C.c_int32),
                ("krylov", C.c_int32), ("use_graph", C.c_int32), ("remove_rhs_mean", C.c_int32),
                ("certify", C.c_int32), ("device", C.c_int32), ("stream", C.c_void_p),
                ("stop_rule", C.c_int32), ("zero_wall_faces", C.c_int32),
                ("inner_cycles", C.c_int32), ("split_restarts", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("status", C.c_int32), ("cycles", C.c_int32), ("levels", C.c_int32),
                ("coarse_n", C.c_int32), ("rel_residual", C.c_double),
                ("rms_residual", C.c_double), ("res0", C.c_double), ("ms", C.c_double),
                ("bytes", C.c_double), ("increment", C.c_double), ("device_loop", C.c_int32),
                ("restarts", C.c_int32)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Field(C.Structure):
    _fields_ = [("data", C.c_void_p), ("sy", C.c_int64), ("sz", C.c_int64)]


class NSParams(C.Structure):
    _fields_ = [("ghost", C.c_int32), ("bc", C.c_int32 * 6), ("iterations", C.c_int32),
                ("adv_scheme", C.c_int32),
                ("dt", C.c_double), ("re", C.c_double), ("fr", C.c_double), ("we", C.c_double),
                ("mu_12", C.c_double), ("gx", C.c_double), ("gy", C.c_double),
                ("gz", C.c_double), ("btn_g", C.c_double), ("btn_sf", C.c_double),
                ("p_tol", C.c_double)]


NS_FIELDS = ("u", "v", "w", "u_old", "v_old", "w_old", "su", "sv", "sw", "su_old", "sv_old",
             "sw_old", "rho", "mu", "delta", "phi", "nrm_x", "nrm_y", "nrm_z", "curv", "p")


class NSFields(C.Structure):
    _fields_ = [(name, Field) for name in NS_FIELDS]


class NSStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("cycles", C.c_int32), ("max_rel_residual", C.c_double),
                ("linf", C.c_double), ("l2f", C.c_double), ("ms", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None
_lock = threading.Lock()


def library_path():
    return _build.SO


def load(build_if_missing: bool = True):
    """Load libgbmg.so, building it first when it is missing or stale."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        so = _build.SO
        if build_if_missing:
            so = _build.build()
        if not os.path.exists(so):
            raise RuntimeError(f"libgbmg.so not found at {so}; build it with fortrancfd_gb300.build")
        L = C.CDLL(so)
        H = C.c_void_p
        P = C.POINTER
        L.gbmg_default_params.argtypes = [P(Params)]
        L.gbmg_default_params.restype = None
        L.gbmg_create.argtypes = [P(Grid), P(Params), P(H)]
        L.gbmg_destroy.argtypes = [H]
        L.gbmg_set_rho.argtypes = [H, Field, C.c_int]
        L.gbmg_set_phi.argtypes = [H, Field, C.c_double, C.c_double, C.c_double, C.c_int]
        L.gbmg_set_coef.argtypes = [H, Field, Field, Field, C.c_int]
        L.gbmg_solve.argtypes = [H, Field, Field, C.c_double, C.c_int, P(Stats)]
        L.gbmg_project.argtypes = [H, Field, Field, Field, Field, C.c_double, C.c_double, C.c_int,
                                   P(Stats)]
        L.gbmg_divergence.argtypes = [H, Field, Field, Field, C.c_double, Field, C.c_int]
        L.gbmg_residual.argtypes = [H, Field, Field, Field, P(C.c_double), C.c_int]
        L.gbmg_div_stats.argtypes = [H, Field, Field, Field, P(C.c_double), P(C.c_double), C.c_int]
        L.gbmg_level_coef.argtypes = [H, C.c_int, Field, Field, Field, C.c_int]
        L.gbmg_level_dims.argtypes = [H, P(C.c_int32), P(C.c_int32), C.c_int32]
        L.gbmg_kernel_launches.argtypes = [H]
        L.gbmg_kernel_launches.restype = C.c_int64
        L.gbmg_strerror.argtypes = [C.c_int]
        L.gbmg_strerror.restype = C.c_char_p
        L.gbmg_last_error.argtypes = [H]
        L.gbmg_last_error.restype = C.c_char_p
        L.gbmg_set_profiling.argtypes = [H, C.c_int]
        L.gbmg_adjoint.argtypes = [H, Field, Field, Field, C.c_double, C.c_double, C.c_double,
                                   Field, Field, C.c_int]
        L.gbmg_profile.argtypes = [H, P(C.c_double), P(C.c_int64), C.c_int32]
        L.gbmg_set_split.argtypes = [H, Field, C.c_double, C.c_int]
        L.gbmg_project_split.argtypes = [H, Field, Field, Field, Field, Field, C.c_double,
                                         C.c_double, C.c_int, P(Stats)]
        L.gbmg_div_stats_noalloc.argtypes = [P(Grid), Field, Field, Field, P(C.c_double),
                                             P(C.c_double), C.c_int, C.c_void_p, C.c_char_p,
                                             C.c_size_t]
        L.gbmg_ls_create.argtypes = [P(Grid), C.c_int, C.c_void_p, P(H)]
        L.gbmg_ls_destroy.argtypes = [H]
        L.gbmg_ls_advect.argtypes = [H, Field, Field, Field, Field, C.c_double, C.c_int, C.c_int]
        L.gbmg_ls_kernel_launches.argtypes = [H]
        L.gbmg_ls_kernel_launches.restype = C.c_int64
        L.gbmg_ls_last_error.argtypes = [H]
        L.gbmg_ls_last_error.restype = C.c_char_p
        L.gbmg_ls_redistance.argtypes = [H, Field, C.c_double, C.c_double, C.c_double, C.c_int,
                                         C.c_int, C.c_int, P(C.c_int32), P(C.c_double)]
        L.gbmg_ns_ab_step.argtypes = [H, P(NSParams), P(NSFields), C.c_int, P(NSStats)]
        L.gbmg_ns_ab_predict.argtypes = [H, P(NSParams), P(NSFields), C.c_int]
        L.gbmg_ns_velbc.argtypes = [H, P(NSParams), Field, Field, Field, C.c_int]
        L.gbmg_ns_curvature.argtypes = [H, P(NSParams), Field, Field, Field, Field, Field, C.c_int]
        L.gbmg_ns_rho_mu.argtypes = [H, P(NSParams), Field, C.c_double, C.c_double, Field, Field,
                                     Field, C.c_int]
        L.gbmg_ns_bc.argtypes = [H, P(NSParams), Field, C.c_int]
        L.gbmg_ns_mass_correct.argtypes = [H, P(NSParams), Field, C.c_double, C.c_double,
                                           C.c_double, C.c_int, C.c_int, P(C.c_double)]
        L.gbmg_ns_vof_advect.argtypes = [H, P(NSParams), Field, Field, Field, Field, Field, Field,
                                         C.c_int]
        L.gbmg_ns_ibm.argtypes = [H, P(NSParams), Field, C.c_double, Field, Field, Field, C.c_int]
        for name in ("gbmg_ls_create", "gbmg_ls_destroy", "gbmg_ls_advect", "gbmg_ls_redistance",
                     "gbmg_ns_ab_step", "gbmg_ns_ab_predict", "gbmg_ns_velbc",
                     "gbmg_ns_curvature", "gbmg_ns_rho_mu", "gbmg_ns_bc",
                     "gbmg_ns_mass_correct", "gbmg_ns_vof_advect", "gbmg_ns_ibm"):
            getattr(L, name).restype = C.c_int
        for name in ("gbmg_create", "gbmg_destroy", "gbmg_set_rho", "gbmg_set_phi",
                     "gbmg_set_coef", "gbmg_solve", "gbmg_project", "gbmg_divergence",
                     "gbmg_residual", "gbmg_div_stats", "gbmg_level_coef", "gbmg_level_dims",
                     "gbmg_set_profiling", "gbmg_profile", "gbmg_adjoint",
                     "gbmg_div_stats_noalloc", "gbmg_set_split", "gbmg_project_split"):
            getattr(L, name).restype = C.c_int
        _lib = L
        return _lib
