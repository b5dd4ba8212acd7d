"""ctypes binding of the CUDA library (the C ABI of ``include/fteik_gb300.h``).

This is the only way the Python layer reaches the GPU: every compute call goes
through these entry points, which run hand-written sm_103a kernels. There is no
CPU fallback: if the library is missing, or no CUDA device is present, the
calls raise.
"""

import ctypes
import os
import threading

from . import _build

_D = ctypes.c_double
_I = ctypes.c_int
_LL = ctypes.c_longlong
_SZ = ctypes.c_size_t
_P = ctypes.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "fteik_version": (ctypes.c_char_p, []),
    "fteik_last_error": (ctypes.c_char_p, []),
    "fteik_slowness": (_I, [_P, _LL, _P, _P, _P]),
    "fteik_kernel_timing": (_I, [_I]),
    "fteik_set_option": (_I, [ctypes.c_char_p, _LL]),
    "fteik_last_sweep_ms": (_I, [ctypes.POINTER(ctypes.c_float)]),
    "fteik_fp64_peak": (_I, [_P, _I, _I, ctypes.POINTER(ctypes.c_double), _P]),
    "fteik_sqrt_rn": (_I, [_P, _LL, _P, _P]),
    "fteik_div_rn": (_I, [_P, _LL, _D, _P, _P]),
    "fteik_recip_rn": (_I, [_P, _LL, _P, _P]),
    "fteik3d_workspace_bytes": (_SZ, [_I, _I, _I, _I, _I]),
    "fteik3d_solve": (_I, [_P, _I, _I, _I, _D, _D, _D, _P, _I, _I, _I, _P, _P, _P, _P, _SZ, _LL, _P]),
    "fteik3d_solve_async": (_I, [_P, _I, _I, _I, _D, _D, _D, _P, _I, _I, _I, _P, _P, _P, _P, _SZ, _LL, _P]),
    "fteik_workspace_status": (_I, [_P, _P]),
    "fteik3d_solve_noalloc": (_I, [_P, _I, _I, _I, _D, _D, _D, _P, _I, _I, _I, _P, _P, _P, _LL, _P]),
    "fteik3d_adjoint_workspace_bytes": (_SZ, [_I, _I, _I, _I]),
    "fteik_get_option": (_I, [ctypes.c_char_p, ctypes.POINTER(_LL)]),
    "fteik3d_batch_workspace_bytes": (_SZ, [_I, _P, _P, _I]),
    "fteik3d_solve_batch": (
        _I, [_I, _P, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _SZ, _LL, _P]
    ),
    "fteik3d_autotune": (
        _I,
        [_P, _I, _I, _I, _D, _D, _D, _P, _I, _I, _P, _P, _P, _P, _SZ, _LL, _P, _P, _P],
    ),
    "fteik3d_batch_autotune": (
        _I, [_I, _P, _P, _P, _P, _P, _I, _P, _P, _P, _P, _SZ, _LL, _P, _P, _P]
    ),
    "fteik_clear_tuning": (_I, []),
    "fteik_last_sweep_kernel": (ctypes.c_char_p, []),
    "fteik3d_tape_bytes": (_SZ, [_I, _I, _I, _I, _I, _I]),
    "fteik3d_solve_tape": (
        _I, [_P, _I, _I, _I, _D, _D, _D, _P, _I, _I, _P, _P, _P, _SZ, _I, _P, _SZ, _LL, _P]
    ),
    "fteik3d_adjoint": (
        _I,
        [_P, _I, _I, _I, _D, _D, _D, _I, _I, _P, _I, _P, _SZ, _P, _P, _P, _P, _P, _I, _P, _I,
         _P, _P, _SZ, _LL, _P],
    ),
    "fteik3d_adjoint_part": (
        _I,
        [_P, _I, _I, _I, _D, _D, _D, _I, _I, _I, _I, _P, _I, _P, _SZ, _P, _P, _P, _P, _P, _I,
         _P, _I, _P, _P, _SZ, _LL, _P],
    ),
    "fteik_resample": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "fteik_correlate1d": (_I, [_I, _P, _P, _I, _P, _I, _P, _P]),
    "fteik2d_workspace_bytes": (_SZ, [_I, _I, _I, _I]),
    "fteik2d_solve": (_I, [_P, _I, _I, _D, _D, _P, _I, _I, _I, _P, _P, _P, _P, _SZ, _P]),
    "fteik2d_chain_stats": (_I, [_P, ctypes.POINTER(ctypes.c_ulonglong),
                                 ctypes.POINTER(ctypes.c_ulonglong), _P]),
    "fteik_interp3d": (_I, [_P, _I, _P, _I, _P, _I, _P, _LL, _P, _I, _D, _P, _P]),
    "fteik_interp2d": (_I, [_P, _I, _P, _I, _P, _LL, _P, _I, _D, _P, _P]),
    "fteik_vinterp3d": (_I, [_P, _I, _P, _I, _P, _I, _P, _LL, _P, _P, _I, _P, _P, _D, _P, _P]),
    "fteik_vinterp2d": (_I, [_P, _I, _P, _I, _P, _LL, _P, _P, _I, _P, _P, _D, _P, _P]),
    "fteik_ray3d": (_I, [_P, _I, _P, _I, _P, _I, _P, _LL, _P, _P, _I, _P, _D, _I, _I, _P, _P, _P, _P]),
    "fteik_ray2d": (_I, [_P, _I, _P, _I, _P, _LL, _P, _P, _I, _P, _D, _I, _I, _P, _P, _P, _P]),
    "fteik_ray_pack": (_I, [_I, _P, _I, _I, _P, _P, _P, _P]),
}

OK = 0
SOURCE_OUT_OF_BOUND = 1
END_POINT_OUT_OF_BOUND = 2
MAX_STEP_REACHED = 3
DEVICE_WAIT_TIMEOUT = 4
INVALID_ARGUMENT = 5
CUDA_ERROR = 6
WORKSPACE_TOO_SMALL = 7
TAPE_OVERFLOW = 8

_lock = threading.Lock()
_lib = None


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library and bind its symbols."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(
                "fteik_gb300 CUDA library not built (expected %s); run "
                "fteikpy_gb300.build()" % path
            )
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc, what=""):
    """Map a C-ABI status code to the reference's exceptions."""
    if rc == OK:
        return
    if rc == SOURCE_OUT_OF_BOUND:
        raise ValueError("source out of bound")
    if rc == END_POINT_OUT_OF_BOUND:
        raise ValueError("end point out of bound")
    if rc == MAX_STEP_REACHED:
        raise RuntimeError("maximum number of steps reached")
    if rc == DEVICE_WAIT_TIMEOUT:
        raise RuntimeError(f"{what}: a device-side dependency wait timed out")
    if rc == INVALID_ARGUMENT:
        raise ValueError(f"{what}: invalid argument")
    if rc == WORKSPACE_TOO_SMALL:
        raise RuntimeError(f"{what}: workspace too small")
    if rc == TAPE_OVERFLOW:
        raise RuntimeError(f"{what}: the adjoint's tape overflowed")
    err = load().fteik_last_error().decode()
    raise RuntimeError(f"{what}: CUDA error {err}")
