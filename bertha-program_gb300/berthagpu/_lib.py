"""ctypes binding of libberthagpu.so (the C ABI of include/bertha_gpu.h).

The library is the only compute path: if it is missing or fails to load,
every call raises BerthaGPUError.  There is no CPU fallback.
"""
import ctypes
import os

from .build import LIB

BG_OK, BG_ERR_ARG, BG_ERR_CAPACITY, BG_ERR_CUDA, BG_ERR_STATE = 0, 1, 2, 3, 4
HMLT = {"NORL": 0, "BARE": 1, "DHFR": 2, "DHFP": 3, "DHFB": 4, "DHFQ": 5}
SHAPE = {"NOSYMM": 0, "PLANAR": 0, "GENERAL": 0, "DIATOM": 1, "LINEAR": 1, "ATOMIC": 2}
FLAG_NO_RACAH1 = 1
FLAG_GAUNT = 2
PREC = {"fp64": 0, "df32": 1, "auto": 2, "tc32": 3}
MAX_L = 3

_CODES = {1: "invalid argument", 2: "capacity exceeded", 3: "CUDA error", 4: "context unusable"}


class BerthaGPUError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"{_CODES.get(code, 'error')} ({code}): {msg}")
        self.code = code


_L = None


def lib():
    global _L
    if _L is None:
        if not os.path.exists(LIB):
            raise BerthaGPUError(BG_ERR_STATE, f"{LIB} not built (run build())")
        L = ctypes.CDLL(LIB)
        P, i, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
        L.bertha_gpu_init.argtypes = [ctypes.POINTER(P), i, P, P, P, i, P, i, i, i, i]
        L.bertha_gpu_dims.argtypes = [P, P, P]
        L.bertha_gpu_set_precision.argtypes = [P, i]
        L.bertha_gpu_set_screening.argtypes = [P, ctypes.c_double]
        L.bertha_gpu_set_list_limits.argtypes = [P, ll, ll]
        L.bertha_gpu_clmfast.argtypes = [P, P, i, i, P, P, i]
        L.bertha_gpu_clmfast_device.argtypes = [P, P, i, i, P, P, i, P]
        L.bertha_gpu_brtfast.argtypes = [P, P, i, i, P, i]
        L.bertha_gpu_brtfast_device.argtypes = [P, P, i, i, P, i, P]
        L.bertha_gpu_oneel.argtypes = [P, P, P, P, P, P, i]
        L.bertha_gpu_oneel_device.argtypes = [P, P, P, P, P, P, i, P]
        L.bertha_gpu_quartets.argtypes = [P, P, ll, i, i, P, i, P, P, i, P]
        L.bertha_gpu_quartets_noalloc.argtypes = [P, P, ll, i, i, P, i, P, P, i, P]
        L.bertha_gpu_quartets_segments.argtypes = [P, P, i, P, P, i, i, P, i, P, P, i, P]
        L.bertha_gpu_shells.argtypes = [P, P, P, P, P]
        L.bertha_gpu_layout.argtypes = [P, P]
        L.bertha_gpu_launches.argtypes = [P]
        L.bertha_gpu_launches.restype = ll
        L.bertha_gpu_last_error.argtypes = [P]
        L.bertha_gpu_last_error.restype = ctypes.c_char_p
        L.bertha_gpu_free.argtypes = [P]
        L.bertha_gpu_free.restype = None
        L.bertha_gpu_auto_stats.argtypes = [P, P, P, P]
        L.bertha_gpu_batch_auto_stats.argtypes = [P, P, P, P]
        L.bertha_gpu_kernel_stats.argtypes = [P, P, P]
        L.bertha_gpu_breit_kernel_stats.argtypes = [P, P, P]
        L.bertha_gpu_tuning_record.argtypes = [P, i, i, P, P, P]
        L.bertha_gpu_batch_kernel_stats.argtypes = [P, P, P]
        L.bertha_gpu_set_error_budget.argtypes = [P, ctypes.c_double]
        L.bertha_gpu_batch_set_error_budget.argtypes = [P, ctypes.c_double]
        L.bertha_gpu_device_status.argtypes = [P]
        L.bertha_gpu_batch_create.argtypes = [ctypes.POINTER(P), i, P, P, P]
        L.bertha_gpu_batch_set_precision.argtypes = [P, i]
        L.bertha_gpu_batch_clmfast_device.argtypes = [P, P, i, P, P, P]
        L.bertha_gpu_batch_quartets.argtypes = [P]
        L.bertha_gpu_batch_quartets.restype = ll
        L.bertha_gpu_batch_launches.argtypes = [P]
        L.bertha_gpu_batch_launches.restype = ll
        L.bertha_gpu_batch_last_error.argtypes = [P]
        L.bertha_gpu_batch_last_error.restype = ctypes.c_char_p
        L.bertha_gpu_batch_free.argtypes = [P]
        L.bertha_gpu_batch_free.restype = None
        _L = L
    return _L


EXPORTED = [
    "bertha_gpu_init", "bertha_gpu_set_screening", "bertha_gpu_set_precision",
    "bertha_gpu_set_list_limits",
    "bertha_gpu_dims", "bertha_gpu_clmfast",
    "bertha_gpu_clmfast_device", "bertha_gpu_brtfast", "bertha_gpu_brtfast_device",
    "bertha_gpu_oneel", "bertha_gpu_oneel_device",
    "bertha_gpu_quartets", "bertha_gpu_quartets_noalloc", "bertha_gpu_quartets_segments",
    "bertha_gpu_shells",
    "bertha_gpu_layout", "bertha_gpu_launches", "bertha_gpu_last_error",
    "bertha_gpu_free",
    "bertha_gpu_batch_create", "bertha_gpu_batch_set_precision",
    "bertha_gpu_batch_clmfast_device", "bertha_gpu_batch_quartets",
    "bertha_gpu_batch_launches", "bertha_gpu_batch_last_error", "bertha_gpu_batch_free",
    "bertha_gpu_auto_stats", "bertha_gpu_batch_auto_stats",
    "bertha_gpu_kernel_stats", "bertha_gpu_batch_kernel_stats", "bertha_gpu_breit_kernel_stats",
    "bertha_gpu_tuning_record",
    "bertha_gpu_set_error_budget", "bertha_gpu_batch_set_error_budget",
    "bertha_gpu_device_status",
]


def device_status():
    """Tensor-core kernel status since the last call (synchronises): 0 when
    every quartet was digested (see bertha_gpu_device_status)."""
    v = ctypes.c_int()
    check(lib().bertha_gpu_device_status(ctypes.byref(v)))
    return v.value


def check(rc, ctx=None):
    if rc != BG_OK:
        msg = lib().bertha_gpu_last_error(ctx)
        raise BerthaGPUError(rc, msg.decode() if msg else "")


def check_batch(rc, batch=None):
    if rc != BG_OK:
        msg = lib().bertha_gpu_batch_last_error(batch)
        raise BerthaGPUError(rc, msg.decode() if msg else "")
