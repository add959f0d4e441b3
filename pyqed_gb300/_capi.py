"""ctypes binding of the C ABI declared in ``include/lindblad_gb300.h``.

This is the binding a maintainer of the reference would add beside
``pyqed/oqs.py``: plain pointers and sizes, device memory held by torch
tensors, status codes turned into ``LindbladError``.  The library is loaded
from the package tree (``pyqed_gb300/_lib``); if it is missing the product
path raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_lib", "liblindblad_gb300.so")

# status codes
LGB_OK = 0
LGB_ERR_INVALID_ARG = 1
LGB_ERR_UNSUPPORTED = 2
LGB_ERR_CUDA = 3
LGB_ERR_NONFINITE = 4
LGB_ERR_TIMEOUT = 5
LGB_ERR_NO_DEVICE = 6
LGB_ERR_STATE = 7
LGB_ERR_TOO_LARGE = 8
LGB_ERR_CHECK = 9
NOALLOC_MAX_DIM, NOALLOC_MAX_COPS, NOALLOC_MAX_EOPS = 64, 4, 4

# precisions
PREC = {"fp64": 0, "fp32": 1, "3xtf32": 2, "3xbf16": 3}
PREC_NAME = {v: k for k, v in PREC.items()}
# collapse-operator storage
COPS_NONE, COPS_DENSE, COPS_DIAG = 0, 1, 2
# schedules
SCHED = {"auto": 0, "cta": 1, "gemm": 2}
SCHED_NAME = {v: k for k, v in SCHED.items()}

# Every symbol include/lindblad_gb300.h declares.
EXPORTS = [
    "lgb_get_version", "lgb_status_string", "lgb_plan_create", "lgb_plan_destroy",
    "lgb_plan_set_operators", "lgb_plan_propagate", "lgb_plan_errors", "lgb_plan_check_stats",
    "lgb_plan_get_info",
    "lgb_propagate_noalloc", "lgb_plan_adjoint", "lgb_plan_set_option",
    "lgb_redfield_tensor", "lgb_redfield_tensor_batch", "lgb_redfield_max_dim", "lgb_redfield_create", "lgb_redfield_destroy",
    "lgb_redfield_set", "lgb_redfield_propagate", "lgb_redfield_errors",
    "lgb_heom_max_dim", "lgb_heom_max_levels_on_chip", "lgb_heom_create", "lgb_heom_destroy",
    "lgb_heom_layout", "lgb_heom_set", "lgb_heom_propagate", "lgb_heom_errors",
    "lgb_spectral_sum", "lgb_spectral_2t",
]
# tuning options (lgb_option_t)
OPT = {"tc_pairs": 1, "gemm_waves": 2, "test_stall": 3, "check": 4, "gemm_ksplit": 5,
       "graph_steps": 6, "gemm_persist": 7}
FLAG_ADJOINT = 1
HEOM_DOUBLE_FIRST = 1
HEOM_DIAG_SZ = 2


class LindbladError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = _status_text(status)
        super().__init__("%s: %s (status %d)" % (what, msg, status) if what else msg)


class Problem(ctypes.Structure):
    _fields_ = [
        ("n_inst", ctypes.c_int32), ("n_cops", ctypes.c_int32), ("cops_kind", ctypes.c_int32),
        ("n_eops", ctypes.c_int32), ("n_drive", ctypes.c_int32), ("nt", ctypes.c_int32),
        ("obs_t0", ctypes.c_int32), ("store_every", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("schedule", ctypes.c_int32),
        ("drive_shared", ctypes.c_int32), ("flags", ctypes.c_int32), ("dt", ctypes.c_double),
        ("checkpoint_every", ctypes.c_int32), ("reserved", ctypes.c_int32),
    ]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("schedule", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("smem_bytes", ctypes.c_int32), ("launches_per_propagate", ctypes.c_int32),
        ("workspace_bytes", ctypes.c_int64), ("flops_per_step", ctypes.c_int64),
        ("persistent_instances", ctypes.c_int32), ("reserved", ctypes.c_int32),
    ]


class RedfieldProblem(ctypes.Structure):
    _fields_ = [
        ("n_inst", ctypes.c_int32), ("n_eops", ctypes.c_int32), ("nt", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("store_every", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("dt", ctypes.c_double),
    ]


class HeomProblem(ctypes.Structure):
    _fields_ = [
        ("n_inst", ctypes.c_int32), ("n_eops", ctypes.c_int32), ("nt", ctypes.c_int32),
        ("nado", ctypes.c_int32), ("precision", ctypes.c_int32), ("flags", ctypes.c_int32),
        ("dt", ctypes.c_double),
    ]


_lib = None


def _status_text(status):
    try:
        return lib().lgb_status_string(status).decode()
    except Exception:  # library not loadable: still produce a message
        return "status %d" % status


def lib():
    """Load (once) and return the CUDA library; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError(
            "pyqed_gb300 CUDA library not found at %s; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python -m pyqed_gb300.build`" % LIBPATH)
    L = ctypes.CDLL(LIBPATH)
    vp, i32, dp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p
    L.lgb_get_version.restype = ctypes.c_int
    L.lgb_get_version.argtypes = []
    L.lgb_status_string.restype = ctypes.c_char_p
    L.lgb_status_string.argtypes = [ctypes.c_int]
    L.lgb_plan_create.restype = ctypes.c_int
    L.lgb_plan_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Problem),
                                  ctypes.POINTER(i32)]
    L.lgb_plan_destroy.restype = ctypes.c_int
    L.lgb_plan_destroy.argtypes = [vp]
    L.lgb_plan_set_operators.restype = ctypes.c_int
    L.lgb_plan_set_operators.argtypes = [vp, dp, dp, dp, dp, vp]
    L.lgb_plan_propagate.restype = ctypes.c_int
    L.lgb_plan_propagate.argtypes = [vp, dp, dp, dp, dp, dp, vp]
    L.lgb_plan_errors.restype = ctypes.c_int
    L.lgb_plan_errors.argtypes = [vp, ctypes.POINTER(i32)]
    L.lgb_plan_check_stats.restype = ctypes.c_int
    L.lgb_plan_check_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.lgb_plan_get_info.restype = ctypes.c_int
    L.lgb_plan_get_info.argtypes = [vp, ctypes.POINTER(PlanInfo)]
    L.lgb_redfield_tensor.restype = ctypes.c_int
    L.lgb_redfield_tensor.argtypes = [i32, i32, dp, dp, dp, dp, vp]
    L.lgb_redfield_tensor_batch.restype = ctypes.c_int
    L.lgb_redfield_tensor_batch.argtypes = [i32, ctypes.POINTER(i32), i32, dp, dp, dp, dp, vp]
    L.lgb_redfield_max_dim.restype = ctypes.c_int
    L.lgb_redfield_max_dim.argtypes = [i32]
    L.lgb_redfield_create.restype = ctypes.c_int
    L.lgb_redfield_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(RedfieldProblem),
                                      ctypes.POINTER(i32)]
    L.lgb_redfield_destroy.restype = ctypes.c_int
    L.lgb_redfield_destroy.argtypes = [vp]
    L.lgb_redfield_set.restype = ctypes.c_int
    L.lgb_redfield_set.argtypes = [vp, dp, dp, vp]
    L.lgb_redfield_propagate.restype = ctypes.c_int
    L.lgb_redfield_propagate.argtypes = [vp, dp, dp, dp, dp, vp]
    L.lgb_redfield_errors.restype = ctypes.c_int
    L.lgb_redfield_errors.argtypes = [vp, ctypes.POINTER(i32)]
    L.lgb_heom_max_dim.restype = ctypes.c_int
    L.lgb_heom_max_dim.argtypes = [i32]
    L.lgb_heom_max_levels_on_chip.restype = ctypes.c_int
    L.lgb_heom_max_levels_on_chip.argtypes = [i32, i32]
    L.lgb_heom_create.restype = ctypes.c_int
    L.lgb_heom_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(HeomProblem), ctypes.POINTER(i32)]
    L.lgb_heom_destroy.restype = ctypes.c_int
    L.lgb_heom_destroy.argtypes = [vp]
    L.lgb_heom_layout.restype = ctypes.c_int
    L.lgb_heom_layout.argtypes = [vp, ctypes.POINTER(i32)]
    L.lgb_heom_set.restype = ctypes.c_int
    L.lgb_heom_set.argtypes = [vp, dp, dp, dp, dp, vp]
    L.lgb_heom_propagate.restype = ctypes.c_int
    L.lgb_heom_propagate.argtypes = [vp, dp, dp, dp, dp, vp]
    L.lgb_heom_errors.restype = ctypes.c_int
    L.lgb_heom_errors.argtypes = [vp, ctypes.POINTER(i32)]
    L.lgb_spectral_sum.restype = ctypes.c_int
    L.lgb_spectral_sum.argtypes = [i32, i32, i32, i32, dp, dp, dp, dp, vp]
    L.lgb_spectral_2t.restype = ctypes.c_int
    L.lgb_spectral_2t.argtypes = [i32, i32, i32, dp, dp, dp, dp, dp, vp]
    L.lgb_plan_set_option.restype = ctypes.c_int
    L.lgb_plan_set_option.argtypes = [vp, i32, i32]
    L.lgb_plan_adjoint.restype = ctypes.c_int
    L.lgb_plan_adjoint.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, vp]
    L.lgb_propagate_noalloc.restype = ctypes.c_int
    L.lgb_propagate_noalloc.argtypes = [dp, i32, dp, i32, i32, dp, i32, dp, i32, ctypes.c_double,
                                        i32, dp, dp, dp, vp]
    _lib = L
    return L


def check(status, what=""):
    if status != LGB_OK:
        raise LindbladError(status, what)
