"""ctypes binding of libgbmie.so (include/gbmie.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, every entry point raises.  Device buffers are torch tensors; their
data pointers are passed straight to the C ABI, and calls are issued on
torch's current CUDA stream.
"""
import ctypes
import os
import threading

import torch

from . import build as _build

GBMIE_OK = 0
GBMIE_ERR_INVALID = 1
GBMIE_ERR_NMAX = 2
GBMIE_ERR_TIMEOUT = 4
GBMIE_PLAIN_FP64 = 0
GBMIE_MIXED = 1
GRID_X = 0
GRID_RADIUS = 1
PSD_LOGNORM = 0
PSD_POWER4 = 1
PSD_WEIGHTS = 2
NSCALAR = 14
NNL = 9

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_D = ctypes.c_double

# name -> (restype, argtypes); every symbol declared in include/gbmie.h
SIGNATURES = {
    "gbmie_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
    "gbmie_ctx_destroy": (ctypes.c_int, [_P]),
    "gbmie_ctx_set_stream": (ctypes.c_int, [_P, _P]),
    "gbmie_ctx_synchronize": (ctypes.c_int, [_P]),
    "gbmie_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "gbmie_last_error": (ctypes.c_char_p, [_P]),
    "gbmie_launch_count": (_I64, [_P]),
    "gbmie_ctx_set_timing": (ctypes.c_int, [_P, ctypes.c_int]),
    "gbmie_ctx_kernel_times": (ctypes.c_int, [_P, _I32, _P, _P, _P, ctypes.POINTER(_I32)]),
    "gbmie_nmax": (ctypes.c_int, [_P, _D, ctypes.POINTER(_I32)]),
    "gbmie_layout": (ctypes.c_int, [_P, _I64, _P, _P, ctypes.POINTER(_I64)]),
    "gbmie_coeffs": (ctypes.c_int, [_P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "gbmie_pitau": (ctypes.c_int, [_P, _I32, _P, _I32, _P, _P]),
    "gbmie_s12": (ctypes.c_int, [_P, _I64, _P, _P, _P, _I32, _P, _P, _P]),
    "gbmie_size_range": (ctypes.c_int, [_P, _I64, _P, _D, _D, _I32, _P, _P, _P, _P]),
    "gbmie_s12_pt": (ctypes.c_int, [_P, _I64, _P, _P, _P, _I32, _I32, _P, _P, _P, _P]),
    "gbmie_s12_noalloc": (ctypes.c_int, [_P, _I64, _P, _P, _P, _I32, _I32, _P, _P, _P]),
    "gbmie_table_plan_create": (ctypes.c_int, [_P, _P, ctypes.POINTER(_P), ctypes.POINTER(_I64)]),
    "gbmie_table_plan_destroy": (ctypes.c_int, [_P]),
    "gbmie_table_run": (ctypes.c_int, [_P, _P, _P]),
    "gbmie_table_run_graph": (ctypes.c_int, [_P, _P, _P]),
    "gbmie_table_plan_autotune": (ctypes.c_int, [_P, _P, _P]),
    "gbmie_table_plan_tuning": (ctypes.c_int, [_P, _P]),
    "gbmie_table_plan_set_tuning": (ctypes.c_int, [_P, _P]),
    "gbmie_table_plan_set_wait_limit": (ctypes.c_int, [_P, _I64]),
    "gbmie_table_plan_set_dn_fp64": (ctypes.c_int, [_P, _I32]),
    "gbmie_gsf": (ctypes.c_int, [_P, _I32, _I32, _P, _P, _I32, _P, _P, _I32]),
    "gbmie_band_average": (ctypes.c_int, [_P, _I32, _I32, _I32, _I32, _P, _P, _I32, _P, _P, _P]),
    "gbmie_measure_fp64_peak": (ctypes.c_int, [_P, ctypes.POINTER(_D)]),
}

_lib = None
_lock = threading.Lock()


class GbmieError(RuntimeError):
    """A failure reported by the CUDA library."""


class DeviceTimeout(GbmieError):
    """A device-side wait ran out of tries (GBMIE_ERR_TIMEOUT): the kernel gave
    up and returned; the context stays usable."""


def library_path():
    return _build.LIB


def load():
    """Load libgbmie.so (building it from csrc/ if it is absent or stale)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            if not os.path.exists(path):
                raise GbmieError("libgbmie.so is missing and could not be built")
            lib = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name, None)
                if fn is None:   # tests/test_abi.py enforces the full export list
                    continue
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


class Context:
    """One gbmie_ctx on one CUDA device (issued on torch's current stream)."""

    def __init__(self, device=0):
        if not torch.cuda.is_available():
            raise GbmieError("geosmie_gb300 needs a CUDA device (no CPU fallback)")
        self.lib = load()
        self.device = torch.device("cuda", device)
        with torch.cuda.device(self.device):
            h = _P()
            st = self.lib.gbmie_ctx_create(device, ctypes.byref(h))
            if st != GBMIE_OK:
                raise GbmieError("gbmie_ctx_create failed: %s" % self.lib.gbmie_status_string(st).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbmie_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bind_stream(self):
        s = torch.cuda.current_stream(self.device)
        self.lib.gbmie_ctx_set_stream(self.h, _P(s.cuda_stream))

    def check(self, st, what):
        if st == GBMIE_OK:
            return
        msg = "%s: %s (%s)" % (what, self.lib.gbmie_status_string(st).decode(),
                               (self.lib.gbmie_last_error(self.h) or b"").decode())
        if st in (GBMIE_ERR_INVALID, GBMIE_ERR_NMAX):
            raise ValueError(msg)
        if st == GBMIE_ERR_TIMEOUT:
            raise DeviceTimeout(msg)
        raise GbmieError(msg)

    def call(self, name, *args):
        self.bind_stream()
        st = getattr(self.lib, name)(self.h, *args)
        self.check(st, name)

    def sync(self):
        self.check(self.lib.gbmie_ctx_synchronize(self.h), "gbmie_ctx_synchronize")

    def launches(self):
        return int(self.lib.gbmie_launch_count(self.h))

    def set_timing(self, enable):
        self.check(self.lib.gbmie_ctx_set_timing(self.h, int(enable)), "gbmie_ctx_set_timing")

    def kernel_times(self):
        """{kernel name: (launches, total device ms)} since timing was enabled."""
        cap = 64
        names = (ctypes.c_char_p * cap)()
        launches = (ctypes.c_int64 * cap)()
        ms = (ctypes.c_double * cap)()
        n = _I32()
        self.bind_stream()
        self.check(self.lib.gbmie_ctx_kernel_times(self.h, cap, names, launches, ms, ctypes.byref(n)),
                   "gbmie_ctx_kernel_times")
        return {names[i].decode(): (int(launches[i]), float(ms[i])) for i in range(n.value)}


_ctx = {}


def context(device=0):
    """Process-wide context per device."""
    c = _ctx.get(device)
    if c is None:
        c = Context(device)
        _ctx[device] = c
    return c


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return _P(t.data_ptr())
