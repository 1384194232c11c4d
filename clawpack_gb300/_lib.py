"""ctypes binding of libgclaw.so (the CUDA step) and of the C structs in
include/gclaw.h.

The library must exist: there is no CPU fallback.  ``lib()`` raises
``RuntimeError`` when ``libgclaw.so`` has not been built
(``python -c "import __graft_entry__ as g; g.build()"``).  The environment
variable GCLAW_LIBRARY, if set, names another build of the same sources to
load instead (for example one compiled with different tile shapes).
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgclaw.so")
# Same sources built with -fmad=false (bit-for-bit comparison with the oracle).
STRICT_LIB_PATH = os.path.join(HERE, "libgclaw_strict.so")

RP_ACOUSTICS_2D = 1
RP_SHALLOW_ROE_WITH_EFIX_2D = 2
RP_EULER_4WAVE_2D = 3
RP_VC_ACOUSTICS_2D = 4
RP_SHALLOW_BATHYMETRY_FWAVE_2D = 5

PREC_FP64 = 0
PREC_FP32_BULK = 1

OK = 0
ERR_ARG = -1
ERR_CUDA = -2
ERR_UNSUPPORTED = -4
ERR_WORKSPACE = -5
ERR_TOO_LARGE = -6
NOALLOC_MAX_BLOCKS = 131072
NONPHYSICAL = 2
CFL_FIXED_DT = 3
MAX_STEPS = 4

MAX_WAVES = 4


class GclawSolver(ctypes.Structure):
    _fields_ = [
        ("rp", ctypes.c_int),
        ("mx", ctypes.c_int),
        ("my", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("bc_lower", ctypes.c_int * 2),
        ("bc_upper", ctypes.c_int * 2),
        ("mthlim", ctypes.c_int * MAX_WAVES),
        ("order", ctypes.c_int),
        ("transverse_waves", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("problem_data", ctypes.c_double * 8),
        ("aux", ctypes.c_void_p),
        ("aux_bc_lower", ctypes.c_int * 2),
        ("aux_bc_upper", ctypes.c_int * 2),
        ("capa", ctypes.c_int),
    ]


class GclawBatchProblem(ctypes.Structure):
    _fields_ = [
        ("mx", ctypes.c_int),
        ("my", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("q_offset", ctypes.c_longlong),
    ]


class GclawCtrl(ctypes.Structure):
    _fields_ = [
        ("t", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("t_start", ctypes.c_double),
        ("t_end", ctypes.c_double),
        ("cfl_max", ctypes.c_double),
        ("cfl_desired", ctypes.c_double),
        ("dt_max", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("cflmax", ctypes.c_double),
        ("dtmin", ctypes.c_double),
        ("dtmax", ctypes.c_double),
        ("smax_bits", ctypes.c_ulonglong * 2),
        ("parity", ctypes.c_int),
        ("numsteps", ctypes.c_int),
        ("attempts", ctypes.c_int),
        ("max_steps", ctypes.c_int),
        ("max_accepted", ctypes.c_int),
        ("dt_variable", ctypes.c_int),
        ("done", ctypes.c_int),
        ("status", ctypes.c_int),
        ("blocks_done", ctypes.c_uint),
        ("flags", ctypes.c_uint),
    ]


CTRL_BYTES = ctypes.sizeof(GclawCtrl)

# include/gclaw3.h: the unsplit 3D step
RP3_ACOUSTICS_3D = 1
RP3_EULER_3D = 2


class GclawSolver3(ctypes.Structure):
    _fields_ = [
        ("rp", ctypes.c_int),
        ("mx", ctypes.c_int),
        ("my", ctypes.c_int),
        ("mz", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("dz", ctypes.c_double),
        ("bc_lower", ctypes.c_int * 3),
        ("bc_upper", ctypes.c_int * 3),
        ("mthlim", ctypes.c_int * MAX_WAVES),
        ("order", ctypes.c_int),
        ("transverse_waves", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("problem_data", ctypes.c_double * 8),
    ]

# (restype, argtypes) of the C entry points.
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_SZ = ctypes.c_size_t
_SP = ctypes.POINTER(GclawSolver)
_SP3 = ctypes.POINTER(GclawSolver3)
# Every symbol include/gclaw.h and include/gclaw3.h declare.
SIGNATURES = {
    "gclaw_version": (ctypes.c_char_p, []),
    "gclaw_strerror": (ctypes.c_char_p, [_I]),
    "gclaw_rp_shape": (_I, [_I, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "gclaw_check": (_I, [_SP]),
    "gclaw_ctrl_init": (_I, [_P, _D, _D, _D, _D, _D, _D, _I, _I, _I, _P]),
    "gclaw_step2": (_I, [_SP, _P, _P, _D, _P, ctypes.POINTER(_D), _P]),
    "gclaw_step": (_I, [_SP, _P, _P, _D, _P, _P]),
    "gclaw_advance": (_I, [_SP, _P, _P, _P, _I, _P]),
    "gclaw_step_workspace_bytes": (_SZ, [_SP]),
    "gclaw_step_host": (_I, [_SP, _P, _P, _D, _P, _SZ, ctypes.POINTER(_D), _P]),
    "gclaw_evolve_workspace_bytes": (_SZ, [_SP]),
    "gclaw_step2_noalloc": (_I, [_SP, _P, _P, _D, ctypes.POINTER(_D), _P]),
    "gclaw_adjoint_step": (_I, [_SP, _P, _P, _P, _D, _P]),
    "gclaw_fp32_kernel": (_I, [_I]),
    "gclaw_fp64_kernel": (_I, [_I]),
    "gclaw_split_kernel": (_I, [_I]),
    "gclaw_rcp_fp64": (_I, [_P, _P, ctypes.c_longlong, _P]),
    "gclaw_step_split": (_I, [_SP, _P, _P, _P, _D, _P, _P]),
    "gclaw_advance_split": (_I, [_SP, _P, _P, _P, _P, _I, _P]),
    "gclaw_batch_table_bytes": (_SZ, [_I]),
    "gclaw_batch_prepare": (_I, [_SP, _P, _I, _P, _SZ, ctypes.POINTER(_I), _P]),
    "gclaw_batch_ctrl_init": (_I, [_P, _I, _P, _D, _D, _D, _D, _D, _I, _I, _I, _P]),
    "gclaw_batch_advance": (_I, [_SP, _P, _I, _I, _P, _P, _P, _I, _P]),
    "gclaw_evolve_host": (_I, [_SP, _P, _P, _D, _D, _D, _I, _D, _D, _D, _I, _P, _SZ, _I,
                               ctypes.POINTER(GclawCtrl), _P]),
    "gclaw3_rp_shape": (_I, [_I, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "gclaw3_check": (_I, [_SP3]),
    "gclaw3_workspace_bytes": (_SZ, [_SP3]),
    "gclaw3_step": (_I, [_SP3, _P, _P, _D, _P, _P, _P]),
    "gclaw3_advance": (_I, [_SP3, _P, _P, _P, _P, _I, _P]),
    "gclaw3_step_split": (_I, [_SP3, _P, _P, _P, _D, _P, _P, _P]),
    "gclaw3_advance_split": (_I, [_SP3, _P, _P, _P, _P, _P, _I, _P]),
    "gclaw3_split_kernel": (_I, [_I]),
    "gclaw3_unsplit_kernel": (_I, [_I]),
}

_libs = {}


def lib(strict=False):
    """Load libgclaw.so (or its -fmad=false twin) once and attach the C
    signatures."""
    path = STRICT_LIB_PATH if strict else os.environ.get("GCLAW_LIBRARY", LIB_PATH)
    L = _libs.get(path)
    if L is None:
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: the CUDA extension has not been built. "
                "Run: python -c 'import __graft_entry__ as g; g.build()'")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _libs[path] = L
    return L


class GclawError(RuntimeError):
    def __init__(self, status, where=""):
        msg = lib().gclaw_strerror(status).decode()
        super().__init__(f"{where}: {msg} (status {status})" if where else f"{msg} ({status})")
        self.status = status


def check(status, where=""):
    if status != OK:
        raise GclawError(status, where)
    return status
