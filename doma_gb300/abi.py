"""ctypes mirror of include/doma_gb300.h and the loader of the native library.

The native library (``doma_gb300/_lib/libdoma_gb300.so``) is the product: CUDA
kernels for sm_103a plus the C ABI.  This module only binds it.  There is no
fallback: if the library is missing or a call needs a GPU that is not there,
the call fails loudly.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_DIR = PKG_DIR / "_lib"
LIB_PATH = LIB_DIR / "libdoma_gb300.so"

DOMA_OK = 0
DOMA_NOT_CONVERGED = 1
DOMA_BAD_INPUT = 2
DOMA_CUDA_ERROR = 3
DOMA_DEVICE_WAIT_TIMEOUT = 4
DOMA_NO_DEVICE = 5
DOMA_NUMERIC_ERROR = 6

STATUS_NAMES = {
    0: "DOMA_OK",
    1: "DOMA_NOT_CONVERGED",
    2: "DOMA_BAD_INPUT",
    3: "DOMA_CUDA_ERROR",
    4: "DOMA_DEVICE_WAIT_TIMEOUT",
    5: "DOMA_NO_DEVICE",
    6: "DOMA_NUMERIC_ERROR",
}

DOMA_SCHEME_DD = 0
DOMA_SCHEME_TW_DD = 1
DOMA_PREC_FP64 = 0
DOMA_PREC_FP32 = 1
DOMA_ITER_GAUSS_SEIDEL = 0
DOMA_ITER_MULTIGROUP = 1
DOMA_CONV_AUTO = 0
DOMA_CONV_MMA = 1
DOMA_CONV_TENSOR_MEMORY = 2
ABI_VERSION = 2

_dp = ctypes.POINTER(ctypes.c_double)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_fp = ctypes.POINTER(ctypes.c_float)
_u8p = ctypes.POINTER(ctypes.c_uint8)


class DomaProblem(ctypes.Structure):
    _fields_ = [
        ("num_dims", ctypes.c_uint32),
        ("nx", ctypes.c_uint32),
        ("ny", ctypes.c_uint32),
        ("nz", ctypes.c_uint32),
        ("dx", _dp),
        ("dy", _dp),
        ("dz", _dp),
        ("num_groups", ctypes.c_uint32),
        ("num_materials", ctypes.c_uint32),
        ("cell_material", _u32p),
        ("total", _dp),
        ("scatter", _dp),
        ("source", _dp),
        ("has_fission", _u8p),
        ("chi_p", _dp),
        ("nu_sigma_f", _dp),
        ("num_polar", ctypes.c_uint32),
        ("num_azimuthal", ctypes.c_uint32),
    ]


class DomaTransient(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("num_steps", ctypes.c_uint32),
        ("num_d_groups", ctypes.c_uint32),
        ("inv_v", ctypes.POINTER(ctypes.c_double)),
        ("d_groups", ctypes.POINTER(ctypes.c_uint32)),
        ("chi_d", ctypes.POINTER(ctypes.c_double)),
        ("beta", ctypes.POINTER(ctypes.c_double)),
        ("lambda_", ctypes.POINTER(ctypes.c_double)),
        ("step_type", ctypes.POINTER(ctypes.c_uint32)),
        ("step_insert", ctypes.POINTER(ctypes.c_double)),
        ("step_remove", ctypes.POINTER(ctypes.c_double)),
        ("step_source", ctypes.POINTER(ctypes.c_double)),
    ]


DOMA_STEP_NONE = 0
DOMA_STEP_BOTH = 1
DOMA_STEP_INSERT = 2
DOMA_STEP_REMOVE = 3

# int (*doma_step_callback)(void *user, uint32_t step, double t, const double *phi,
#                           const double *dnps)
StepCallback = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_double,
                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double))


class DomaOptions(ctypes.Structure):
    _fields_ = [
        ("scheme", ctypes.c_uint32),
        ("theta", ctypes.c_double),
        ("precision", ctypes.c_uint32),
        ("fs_tol", ctypes.c_double),
        ("fs_max_it", ctypes.c_uint32),
        ("mg_tol", ctypes.c_double),
        ("mg_max_it", ctypes.c_uint32),
        ("verbose", ctypes.c_uint32),
        ("tile_x", ctypes.c_uint32),
        ("tile_y", ctypes.c_uint32),
        ("tile_z", ctypes.c_uint32),
        ("iteration", ctypes.c_uint32),
    ]


class DomaReport(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_uint32),
        ("mg_iterations", ctypes.c_uint32),
        ("si_iterations", ctypes.c_uint64),
        ("updates", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
        ("mg_residual", ctypes.c_double),
        ("si_residual", ctypes.c_double),
        ("solve_ms", ctypes.c_double),
        ("si_counts", _u32p),
        ("si_counts_capacity", ctypes.c_size_t),
        ("si_counts_len", ctypes.c_size_t),
    ]


# Every entry point declared in include/doma_gb300.h: name -> (restype, argtypes).
class DomaAccelOptions(ctypes.Structure):
    _fields_ = [("first", ctypes.c_uint32), ("interval", ctypes.c_uint32),
                ("max_corrections", ctypes.c_uint32), ("guard", ctypes.c_uint32)]


class DomaAccelStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint32), ("corrections_accepted", ctypes.c_uint32),
                ("corrections_rejected", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("error", ctypes.c_double), ("solve_ms", ctypes.c_double)]


SIGNATURES = {
    "doma_default_options": (None, [ctypes.POINTER(DomaOptions)]),
    "doma_last_error": (ctypes.c_char_p, []),
    "doma_abi_version": (ctypes.c_uint32, []),
    "doma_quadrature": (
        ctypes.c_int,
        [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _dp, _dp, _dp, _dp, _u32p],
    ),
    "doma_solver_create": (
        ctypes.c_int,
        [ctypes.POINTER(DomaProblem), ctypes.POINTER(DomaOptions), ctypes.POINTER(ctypes.c_void_p)],
    ),
    "doma_solver_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "doma_solver_solve_fixed_source": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DomaReport)]),
    "doma_solver_solve_eigenvalue": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double,
                                                    ctypes.POINTER(DomaReport), _dp]),
    "doma_solver_solve_transient": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DomaTransient),
                                                   StepCallback, ctypes.c_void_p,
                                                   ctypes.POINTER(DomaReport)]),
    "doma_solver_get_scalar_flux": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_size_t]),
    "doma_solver_source_iterations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]),
    "doma_solver_sweeps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]),
    "doma_solver_describe": (
        ctypes.c_int,
        [ctypes.c_void_p, _u32p, _u32p, ctypes.POINTER(ctypes.c_uint64)],
    ),
    "doma_solver_destroy": (None, [ctypes.c_void_p]),
    "doma_batch_create": (
        ctypes.c_int,
        [ctypes.POINTER(DomaProblem), ctypes.c_size_t, ctypes.POINTER(DomaOptions),
         ctypes.POINTER(ctypes.c_void_p)],
    ),
    "doma_batch_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "doma_batch_tune": (ctypes.c_int, [ctypes.c_void_p, _u32p]),
    "doma_batch_tiles": (ctypes.c_int, [ctypes.c_void_p, _u32p, ctypes.c_size_t]),
    "doma_batch_tune_report": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float),
                                              ctypes.POINTER(ctypes.c_float), _u32p]),
    "doma_batch_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DomaReport), ctypes.c_size_t]),
    "doma_batch_get_scalar_flux": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, _dp, ctypes.c_size_t]),
    "doma_batch_destroy": (None, [ctypes.c_void_p]),
    "doma_sweep_noalloc": (
        ctypes.c_int,
        [ctypes.POINTER(DomaProblem), ctypes.c_uint32, ctypes.c_double, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    ),
    "doma_batch_begin": (ctypes.c_int, [ctypes.c_void_p]),
    "doma_batch_iterate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, _u32p]),
    "doma_batch_state": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p),
         ctypes.POINTER(ctypes.c_void_p)],
    ),
    "doma_batch_reports": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DomaReport), ctypes.c_size_t]),
    "doma_batch_set_increment": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "doma_solver_set_accelerator": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(DomaAccelOptions)]),
    "doma_solver_set_reference": (
        ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_size_t, ctypes.c_double]),
    "doma_solver_accel_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DomaAccelStats)]),
    "doma_unet_create": (ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    "doma_unet_destroy": (None, [ctypes.c_void_p]),
    "doma_unet_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "doma_unet_num_params": (ctypes.c_size_t, [ctypes.c_void_p]),
    "doma_unet_get_params": (ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.c_size_t]),
    "doma_unet_set_params": (ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.c_size_t]),
    "doma_unet_get_grads": (ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.c_size_t]),
    "doma_unet_forward": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_uint32] * 4,
    ),
    "doma_unet_backward": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_uint32] * 4,
    ),
    "doma_unet_backward_weighted": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_uint32] * 4,
    ),
    "doma_unet_last_loss": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "doma_unet_adam": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_float] * 4),
    "doma_conv3_forward": (
        ctypes.c_int,
        [ctypes.c_void_p] + [ctypes.c_uint32] * 5 + [ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.c_uint32, ctypes.c_uint32,
                                                      ctypes.c_void_p, ctypes.c_uint32,
                                                      ctypes.c_void_p],
    ),
    "doma_conv3_wgrad": (
        ctypes.c_int,
        [ctypes.c_void_p] + [ctypes.c_uint32] * 5 + [ctypes.c_void_p, ctypes.c_uint32,
                                                      ctypes.c_void_p, ctypes.c_uint32,
                                                      ctypes.c_void_p],
    ),
    "doma_conv_wait_error": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
}

_LIB = None


class DomaError(RuntimeError):
    def __init__(self, status: int, where: str, message: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} {message}".strip())


def load_library(path: os.PathLike | str | None = None) -> ctypes.CDLL:
    """Load the native library and bind every declared symbol (raises if absent)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"native library {p} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)"
        )
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.doma_abi_version() != ABI_VERSION:
        raise RuntimeError("doma_gb300 ABI version mismatch")
    if path is None:
        _LIB = lib
    return lib


def last_error(lib: ctypes.CDLL | None = None) -> str:
    lib = lib or load_library()
    msg = lib.doma_last_error()
    return msg.decode() if msg else ""


def check(status: int, where: str, lib: ctypes.CDLL | None = None, allow=(DOMA_OK,)) -> int:
    if status not in allow:
        raise DomaError(status, where, last_error(lib))
    return status
