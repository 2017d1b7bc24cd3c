"""ctypes loader for the in-tree CUDA library libdeft_gb300.so.

There is no CPU fallback: if the library is missing or cannot initialise a
GPU, every call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdeft_gb300.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NAN, ERR_LINESEARCH, ERR_MAXITER, ERR_NOMEM, ERR_TIMEOUT = 1, 2, 3, 4, 5, 6, 7
TERM_HS, TERM_IDEAL, TERM_MU, TERM_VEXT, TERM_MASK, TERM_VEFF, TERM_SAFT = 1, 2, 4, 8, 16, 32, 64
NTERMS = 6
LS_SECANT, LS_QUADRATIC_REF, LS_NEW_API = 0, 1, 2
PC_NONE, PC_FUNCTIONAL, PC_DENSITY, PC_STRUCTURE = 0, 1, 2, 3
HS_WB_NOTENSOR, HS_RF, HS_WB_MARK2, HS_WB_TENSOR, HS_TARAZONA = 0, 1, 2, 3, 4
CONTACT_GSIGMA_S, CONTACT_GSIGMA_A, CONTACT_GROSS, CONTACT_YUWU, CONTACT_YUWU_S = 0, 1, 2, 3, 4

# Every symbol include/deft_gb300.h declares.
EXPORTS = (
    "deft_strerror", "deft_last_error",
    "deft_ctx_create", "deft_ctx_destroy", "deft_ctx_sync", "deft_ctx_stream",
    "deft_grid_create", "deft_grid_create_dx", "deft_grid_destroy", "deft_grid_info",
    "deft_grid_fft", "deft_grid_ifft",
    "deft_grid_profile", "deft_grid_profile_count", "deft_grid_profile_entry",
    "deft_grid_set_tiles", "deft_grid_get_tiles", "deft_grid_graphs", "deft_tuning_set",
    "deft_tuning_clear",
    "deft_fmt_create", "deft_fmt_destroy", "deft_fmt_set_params", "deft_fmt_set_vext",
    "deft_fmt_set_mask", "deft_fmt_energy", "deft_fmt_energy_grad", "deft_fmt_energy_grad_pgrad",
    "deft_fmt_weighted", "deft_fmt_contact", "deft_fmt_set_saft",
    "deft_fmt_hessian_vector", "deft_fmt_precondition",
    "deft_find_chemical_potential", "deft_bulk_density",
    "deft_fmt_energy_grad_noalloc", "deft_noalloc_scratch_bytes",
    "deft_cg_create", "deft_cg_destroy", "deft_cg_set_params", "deft_cg_set_x", "deft_cg_get_x", "deft_cg_x_device",
    "deft_cg_step", "deft_cg_solve", "deft_cg_solve_device", "deft_cg_checkpoint", "deft_cg_restore", "deft_cg_set_log", "deft_batch_solve",
    "deft_batch_solve_device", "deft_batch_device_times",
    "deft_fno_create", "deft_fno_destroy", "deft_fno_param_count", "deft_fno_get_params",
    "deft_fno_set_params", "deft_fno_eval", "deft_fno_adam", "deft_fno_train_step",
    "deft_fno_warm_start", "deft_fno_initial_density", "deft_fno_launches",
)


class DeftError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"deft_gb300 status {status}: {msg}")
        self.status = status


PRECISION_FP64, PRECISION_MIXED = 0, 1


class FmtParams(ctypes.Structure):
    _fields_ = [("R", ctypes.c_double), ("kT", ctypes.c_double), ("mu", ctypes.c_double),
                ("terms", ctypes.c_int), ("precision", ctypes.c_int), ("functional", ctypes.c_int)]


class CgParams(ctypes.Structure):
    _fields_ = [("linesearch", ctypes.c_int), ("gtol", ctypes.c_double), ("maxiter", ctypes.c_int),
                ("step", ctypes.c_double), ("precision", ctypes.c_double),
                ("refine_rel", ctypes.c_double), ("preconditioned", ctypes.c_int),
                ("refine_abs", ctypes.c_double), ("relative_precision", ctypes.c_double),
                ("miniter", ctypes.c_int), ("device_loops", ctypes.c_int)]


class CgStatus(ctypes.Structure):
    _fields_ = [("iter", ctypes.c_int), ("evals", ctypes.c_int), ("energy", ctypes.c_double),
                ("gnorm", ctypes.c_double), ("converged", ctypes.c_int), ("status", ctypes.c_int),
                ("evals_fp64", ctypes.c_int), ("hvps", ctypes.c_int), ("stage", ctypes.c_int)]


class BatchProblem(ctypes.Structure):
    _fields_ = [("lat", ctypes.c_double * 9), ("N", ctypes.c_int * 3), ("R", ctypes.c_double),
                ("kT", ctypes.c_double), ("mu", ctypes.c_double), ("terms", ctypes.c_int),
                ("precision", ctypes.c_int), ("mask", ctypes.c_void_p), ("V", ctypes.c_void_p),
                ("n_init", ctypes.c_void_p), ("n_out", ctypes.c_void_p),
                ("functional", ctypes.c_int)]


class BatchParams(ctypes.Structure):
    _fields_ = [("workers", ctypes.c_int), ("cg", CgParams)]


_lib = None
_vp = ctypes.c_void_p
_dp = ctypes.c_void_p  # data pointers are passed as raw addresses
_pp = ctypes.POINTER(ctypes.c_void_p)


def load():
    """Load the library (building it first if it is absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import _build
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "deft_strerror": (ctypes.c_char_p, [ctypes.c_int]),
        "deft_last_error": (ctypes.c_char_p, []),
        "deft_ctx_create": (ctypes.c_int, [ctypes.c_int, _pp]),
        "deft_ctx_destroy": (ctypes.c_int, [_vp]),
        "deft_ctx_sync": (ctypes.c_int, [_vp]),
        "deft_ctx_stream": (_vp, [_vp]),
        "deft_grid_create": (ctypes.c_int, [_vp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _pp]),
        "deft_grid_create_dx": (ctypes.c_int, [_vp, _dp, ctypes.c_double, _pp]),
        "deft_grid_destroy": (ctypes.c_int, [_vp]),
        "deft_grid_info": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp]),
        "deft_grid_fft": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int]),
        "deft_grid_ifft": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int]),
        "deft_grid_profile": (ctypes.c_int, [_vp, ctypes.c_int]),
        "deft_grid_profile_count": (ctypes.c_int, [_vp]),
        "deft_grid_profile_entry": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                                   _dp, _dp]),
        "deft_grid_set_tiles": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
        "deft_grid_get_tiles": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
        "deft_grid_graphs": (ctypes.c_int, [_vp, ctypes.c_int]),
        "deft_tuning_set": (ctypes.c_int, [_dp, ctypes.c_int, _dp, _dp]),
        "deft_tuning_clear": (ctypes.c_int, []),
        "deft_fmt_create": (ctypes.c_int, [_vp, ctypes.POINTER(FmtParams), _pp]),
        "deft_fmt_destroy": (ctypes.c_int, [_vp]),
        "deft_fmt_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(FmtParams)]),
        "deft_fmt_set_vext": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
        "deft_fmt_set_mask": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
        "deft_fmt_energy": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp, _dp]),
        "deft_fmt_energy_grad": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp, _dp, _dp]),
        "deft_fmt_energy_grad_pgrad": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp, _dp, _dp, _dp]),
        "deft_fmt_weighted": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp]),
        "deft_fmt_contact": (ctypes.c_int, [_vp, _dp, ctypes.c_int, ctypes.c_int, _dp]),
        "deft_fmt_set_saft": (ctypes.c_int, [_vp, _dp]),
        "deft_fmt_hessian_vector": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int, _dp]),
        "deft_fmt_precondition": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int, _dp, _dp]),
        "deft_find_chemical_potential": (ctypes.c_int, [ctypes.c_double, ctypes.c_double,
                                                        ctypes.c_double, _dp]),
        "deft_bulk_density": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_int, _dp]),
        "deft_fmt_energy_grad_noalloc": (ctypes.c_int, [_dp, ctypes.c_int, ctypes.c_int,
                                                         ctypes.c_int, ctypes.POINTER(FmtParams),
                                                         _dp, _dp, _dp, _dp, _dp, _dp, _vp]),
        "deft_noalloc_scratch_bytes": (ctypes.c_size_t, []),
        "deft_cg_create": (ctypes.c_int, [_vp, ctypes.POINTER(CgParams), _pp]),
        "deft_cg_destroy": (ctypes.c_int, [_vp]),
        "deft_cg_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(CgParams)]),
        "deft_cg_set_x": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
        "deft_cg_get_x": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
        "deft_cg_x_device": (_vp, [_vp]),
        "deft_cg_step": (ctypes.c_int, [_vp, ctypes.POINTER(CgStatus)]),
        "deft_cg_solve": (ctypes.c_int, [_vp, ctypes.POINTER(CgStatus)]),
        "deft_cg_solve_device": (ctypes.c_int, [_vp, ctypes.POINTER(CgStatus)]),
        "deft_cg_checkpoint": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "deft_cg_restore": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "deft_cg_set_log": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "deft_fno_create": (ctypes.c_int, [ctypes.c_int] * 5 + [ctypes.c_ulonglong, _pp]),
        "deft_fno_destroy": (ctypes.c_int, [_vp]),
        "deft_fno_param_count": (ctypes.c_size_t, [_vp]),
        "deft_fno_get_params": (ctypes.c_int, [_vp, _dp]),
        "deft_fno_set_params": (ctypes.c_int, [_vp, _dp]),
        "deft_fno_eval": (ctypes.c_int, [_vp, _dp, ctypes.c_float, _dp, ctypes.c_int, _dp, _dp,
                                         _dp]),
        "deft_fno_adam": (ctypes.c_int, [_vp, ctypes.c_float]),
        "deft_fno_launches": (ctypes.c_longlong, [_vp]),
        "deft_fno_train_step": (ctypes.c_int, [_vp, _dp, ctypes.c_float, _dp, ctypes.c_int,
                                               ctypes.c_float, _dp]),
        "deft_fno_warm_start": (ctypes.c_int, [_vp, _dp, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, _dp]),
        "deft_fno_initial_density": (ctypes.c_int, [_vp, _vp, _dp, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_double, _dp, _dp,
                                                    _dp, _dp]),
        "deft_batch_solve": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(BatchProblem),
                                            ctypes.POINTER(BatchParams), ctypes.POINTER(CgStatus)]),
        "deft_batch_device_times": (ctypes.c_int, [_dp]),
        "deft_batch_solve_device": (ctypes.c_int, [ctypes.c_int, ctypes.c_int,
                                                   ctypes.POINTER(BatchProblem),
                                                   ctypes.POINTER(CgParams),
                                                   ctypes.POINTER(CgStatus)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status):
    if status != OK:
        msg = load().deft_last_error().decode(errors="replace")
        raise DeftError(status, msg)
    return status
