"""ctypes binding of liblbgb.so (the C ABI declared in include/lbgb.h).

The library is loaded on first use.  There is no fallback: if it has not been
built, every operator raises ``LBGBUnavailable``.
"""

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbgb.so")

# storage codes
F32, F64, F16DEV, BF16DEV, F32DEV = 0, 1, 2, 3, 4
# boundary codes
PERIODIC, CAVITY, CAVITY_LADD = 0, 1, 2
# lbgb_collide_ex flags
COLLIDE_KEEP_MASS = 1
# return codes
OK, EINVAL, EDTYPE, ECUDA, EWORKSPACE, ETIMEOUT, EUNSUPPORTED = 0, -1, -2, -3, -4, -5, -6

STORAGE_CODES = {"f32": F32, "f64": F64, "f16dev": F16DEV, "bf16dev": BF16DEV, "f32dev": F32DEV}
BOUNDARY_CODES = {"periodic": PERIODIC, "cavity": CAVITY, "cavity-ladd": CAVITY_LADD}


class LBGBError(RuntimeError):
    """A CUDA-side failure reported by liblbgb."""


class LBGBTimeout(LBGBError):
    """A bounded device-side wait of liblbgb gave up."""


class LBGBUnavailable(RuntimeError):
    """liblbgb.so is not built or cannot be loaded."""


_lock = threading.Lock()
_lib = None

_P, _I, _I64, _D, _SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_size_t

# name -> (restype, argtypes); must match include/lbgb.h
SIGNATURES = {
    "lbgb_version": (_I, []),
    "lbgb_last_error": (_I, [ctypes.c_char_p, _SZ]),
    "lbgb_equilibrium": (_I, [_P, _P, _P, _P, _I64, _I64, _I, _P]),
    "lbgb_collide": (_I, [_P, _I64, _I64, _I, _D, _P]),
    "lbgb_collide_ex": (_I, [_P, _I64, _I64, _I, _D, _I, _P]),
    "lbgb_stream_periodic": (_I, [_P, _P, _I, _I, _I, _P]),
    "lbgb_stream_bounce_back": (_I, [_P, _P, _I, _I, _D, _I, _P]),
    "lbgb_stream_inplace_workspace_bytes": (_SZ, [_I, _I, _I]),
    "lbgb_stream_periodic_inplace": (_I, [_P, _I, _I, _I, _P, _SZ, _P]),
    "lbgb_stream_bounce_back_inplace": (_I, [_P, _I, _I, _D, _I, _P, _SZ, _P]),
    "lbgb_step_fused": (_I, [_P, _P, _I, _I, _I, _D, _D, _I, _P]),
    "lbgb_copy_rows": (_I, [_P, _P, _I, _I, _I, _I, _I, _P]),
    "lbgb_step_fused_rows": (_I, [_P, _P, _I, _I, _I, _I, _I, ctypes.c_double, ctypes.c_double, _I, _P]),
    "lbgb_run_fused": (_I, [_P, _P, _I, _I, _I, _D, _D, _I, _I, ctypes.POINTER(_I), _P]),
    "lbgb_steps_per_launch": (_I, [_I, _I, _I, _I]),
    "lbgb_run_fused_sr": (_I, [_P, _P, _I, _I, _I, _D, _D, _I, _I, ctypes.c_uint, _P, ctypes.POINTER(_I), _P]),
    "lbgb_macroscopic": (_I, [_P, _P, _P, _P, _I64, _I64, _I, _P]),
    "lbgb_mass_momentum_workspace_bytes": (_SZ, []),
    "lbgb_mass_momentum": (_I, [_P, _I64, _I64, _I, _P, _P, _SZ, _P]),
    "lbgb_mass_momentum_noalloc": (_I, [_P, _I64, _I64, _I, _P, _P]),
    "lbgb_convert": (_I, [_P, _I, _I64, _P, _I, _I64, _I64, _P]),
    "lbgb_batch_step": (_I, [_P, _P, ctypes.c_longlong, _P, _I, _P, ctypes.c_longlong, _I, _I, _I, _I, _I, _I, _P]),
    "lbgb_batch_shear_amplitude": (_I, [_P, ctypes.c_longlong, _P, _I, _I, _P, _P, _P]),
    "lbgb_batch_velocity_change": (_I, [_P, ctypes.c_longlong, _P, _I, _I, _P, ctypes.c_longlong, _P, _P, _P]),
    "lbgb_row_fft_amplitude": (_I, [_P, _I, _I, _I, _I, _P, _P]),
    "lbgb_wall_bounce_back": (_I, [_P, _I, _I, ctypes.c_double, _I, _I, _I, _P]),
    "lbgb_solid_bounce_back": (_I, [_P, _P, _I, _I, _I, _I, _P]),
    "lbgb_pressure_periodic": (_I, [_P, _I, _I, ctypes.c_double, ctypes.c_double, _I, _P]),
    "lbgb_chapman_enskog": (_I, [_P, _P, _P, _P, _I, _I, ctypes.c_double, ctypes.c_double, _I, _I, _I, _P]),
    "lbgb_gemm_bf16": (_I, [_I, _I, _I, _P, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong, _P,
                            ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong, _P, ctypes.c_longlong,
                            ctypes.c_longlong, ctypes.c_longlong, _I, ctypes.c_float, ctypes.c_float, _I, _I, _P]),
    "lbgb_gemm_bf16_bias_act": (_I, [_I, _I, _I, _P, ctypes.c_longlong, ctypes.c_longlong, _P, ctypes.c_longlong,
                                     _P, ctypes.c_longlong, ctypes.c_float, ctypes.c_float, _P, ctypes.c_longlong,
                                     _I, _P, _P]),
    "lbgb_gemm_status": (_I, [_I]),
    "lbgb_fno_to_bf16": (_I, [_P, _P, ctypes.c_longlong, _P]),
    "lbgb_fno_bias_act": (_I, [_P, _P, _P, _P, _P, _I, ctypes.c_longlong, _I, _P]),
    "lbgb_fno_gelu_back": (_I, [_P, _P, _P, _P, ctypes.c_longlong, _P]),
    "lbgb_fno_row_sum": (_I, [_P, _P, _P, _I, ctypes.c_longlong, _P]),
    "lbgb_fno_mix": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "lbgb_fno_mix_back": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "lbgb_fno_mse": (_I, [_P, _P, _P, _P, _I, ctypes.c_longlong, _P]),
    "lbgb_fno_mse_weighted": (_I, [_P, _P, _P, ctypes.c_longlong, _P, _P, _I, ctypes.c_longlong, _P]),
    "lbgb_fno_adam": (_I, [_P, _P, _P, _P, _P, ctypes.c_longlong, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                           ctypes.c_float, _I, ctypes.c_float, _P]),
    "lbgb_fno_sum_splits": (_I, [_P, _P, _I, ctypes.c_longlong, ctypes.c_float, _P]),
    "lbgb_set_tuning": (_I, [_I, ctypes.c_longlong]),
    "lbgb_get_tuning": (ctypes.c_longlong, [_I]),
    "lbgb_device_status": (_I, [_I]),
}

TUNE_KERNEL, TUNE_STAGES, TUNE_WAIT_LIMIT, TUNE_PIPE_MIN_CELLS, TUNE_TEST_STALL_PRODUCER, TUNE_TWO_STEP = 0, 1, 2, 3, 4, 5
KERNELS = {"auto": 0, "register": 1, "pipelined": 2}
NOALLOC_MAX_CELLS = 268435456
DIAG_CHUNKS = 64  # LBGB_DIAG_CHUNKS: partials per instance of the batch diagnostics


def load(path=LIB_PATH):
    """Load (once) and return the ctypes handle of liblbgb.so."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise LBGBUnavailable(
                    "liblbgb.so is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"` "
                    "or `python -m latticeboltzmann_gb300._build`" % path)
            try:
                handle = ctypes.CDLL(path)
            except OSError as e:
                raise LBGBUnavailable("cannot load %s: %s" % (path, e)) from e
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().lbgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, what=""):
    """Translate a liblbgb return code into the matching Python exception."""
    if rc == OK:
        return
    msg = last_error() or what
    if rc == EINVAL:
        raise ValueError(msg)
    if rc == EDTYPE:
        raise TypeError(msg)
    if rc == ETIMEOUT:
        raise LBGBTimeout(msg)
    raise LBGBError("%s (code %d)" % (msg, rc))


def call(name, *args):
    check(getattr(load(), name)(*args), name)


def set_tuning(key, value):
    call("lbgb_set_tuning", key, int(value))


def get_tuning(key):
    return load().lbgb_get_tuning(key)


def device_status(reset=True):
    """Synchronize and raise LBGBTimeout if a bounded device-side wait of the
    pipelined step kernels gave up (their output is then incomplete)."""
    check(load().lbgb_device_status(1 if reset else 0), "lbgb_device_status")


def gemm_status(reset=True):
    """Synchronize and raise LBGBTimeout if a bounded wait of the tensor-core
    GEMM gave up (its output is then incomplete)."""
    check(load().lbgb_gemm_status(1 if reset else 0), "lbgb_gemm_status")


def all_status(reset=True):
    """Both status words: call at a point that synchronizes anyway."""
    device_status(reset)
    gemm_status(reset)
