"""ctypes binding of libnbody_cuda.so (the C ABI declared in include/nbody.h).

Device arrays are passed as torch CUDA tensors (float64, contiguous); torch is only the
allocator and stream provider here. There is no CPU fallback: if the library is missing the
import-time load raises.
"""

from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libnbody_cuda.so")

NB_OK = 0
STATUS_NAMES = {0: "NB_OK", 1: "NB_ERR_INVALID_ARG", 2: "NB_ERR_CUDA", 3: "NB_ERR_OOM",
                4: "NB_ERR_POOL_OVERFLOW", 5: "NB_ERR_DEPTH_OVERFLOW", 6: "NB_ERR_STACK_OVERFLOW",
                7: "NB_ERR_TIMEOUT", 8: "NB_ERR_UNSUPPORTED", 9: "NB_ERR_NOT_BUILT"}

NB_F64, NB_F64_IEEE, NB_F32C = 0, 1, 2
PRECISIONS = {"f64": NB_F64, "f64_ieee": NB_F64_IEEE, "f32c": NB_F32C}

_vp = C.c_void_p
_u32 = C.c_uint32
_d = C.c_double
_i = C.c_int


class NBodyError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# name -> (restype, argtypes); every function returns nb_status (int) unless stated.
SIGNATURES = {
    "nb_ctx_create": [_i, C.POINTER(_vp)],
    "nb_ctx_destroy": [_vp],
    "nb_sync": [_vp, _vp],
    "nb_naive_accel": [_vp] + [_vp] * 7 + [_u32, _d, _d, _i, _i, _vp],
    "nb_naive_accel_range": [_vp] + [_vp] * 7 + [_u32, _u32, _u32, _d, _d, _i, _vp],
    "nb_leapfrog_kick_drift": [_vp] + [_vp] * 12 + [_u32, _d, _vp],
    "nb_leapfrog_kick": [_vp] + [_vp] * 9 + [_u32, _d, _vp],
    "nb_leapfrog_kick_kick_drift": [_vp] + [_vp] * 12 + [_u32, _d, _vp],
    "nb_energy": [_vp] + [_vp] * 7 + [_u32, _d, _vp, _vp],
    "nb_aabb": [_vp] + [_vp] * 3 + [_u32, _vp, _vp],
}
STRING_FUNCS = ("nb_last_error_string", "nb_version")

_lib = None


def load() -> C.CDLL:
    """Loads the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not found: run n-body-simulation_gb300/build.py first")
        L = C.CDLL(LIB_PATH)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = argtypes
        for name in STRING_FUNCS:
            getattr(L, name).restype = C.c_char_p
            getattr(L, name).argtypes = []
        _lib = L
    return _lib


def check(status: int):
    if status != NB_OK:
        raise NBodyError(status, load().nb_last_error_string().decode())


def ptr(t) -> int:
    """Device pointer of a contiguous torch CUDA tensor (or None -> NULL)."""
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous(), "expected a contiguous CUDA tensor"
    return t.data_ptr()


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class Context:
    """Owns an nb_ctx (device id, scratch memory, device error word)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = _vp()
        check(self.lib.nb_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nb_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self, stream=None):
        check(self.lib.nb_sync(self.handle, stream_ptr(stream)))

    # -- naive -----------------------------------------------------------------------------
    def naive_accel(self, m, x, y, z, ax, ay, az, G, eps2, precision="f64", block_size=0,
                    stream=None):
        n = m.numel()
        check(self.lib.nb_naive_accel(self.handle, ptr(m), ptr(x), ptr(y), ptr(z), ptr(ax),
                                      ptr(ay), ptr(az), n, G, eps2, PRECISIONS[precision],
                                      block_size, stream_ptr(stream)))

    def naive_accel_range(self, m, x, y, z, ax, ay, az, i_begin, i_end, G, eps2,
                          precision="f64", stream=None):
        n = m.numel()
        check(self.lib.nb_naive_accel_range(self.handle, ptr(m), ptr(x), ptr(y), ptr(z), ptr(ax),
                                            ptr(ay), ptr(az), n, i_begin, i_end, G, eps2,
                                            PRECISIONS[precision], stream_ptr(stream)))

    # -- integration -------------------------------------------------------------------------
    def kick_drift(self, vh, v, p, a, dt, stream=None):
        n = v[0].numel()
        check(self.lib.nb_leapfrog_kick_drift(self.handle, *map(ptr, vh), *map(ptr, v),
                                              *map(ptr, p), *map(ptr, a), n, dt,
                                              stream_ptr(stream)))

    def kick(self, v, vh, a, dt, stream=None):
        n = v[0].numel()
        check(self.lib.nb_leapfrog_kick(self.handle, *map(ptr, v), *map(ptr, vh), *map(ptr, a), n,
                                        dt, stream_ptr(stream)))

    def kick_kick_drift(self, v, vh, p, a, dt, stream=None):
        n = v[0].numel()
        check(self.lib.nb_leapfrog_kick_kick_drift(self.handle, *map(ptr, v), *map(ptr, vh),
                                                   *map(ptr, p), *map(ptr, a), n, dt,
                                                   stream_ptr(stream)))

    def energy(self, m, x, y, z, vx, vy, vz, G, out, stream=None):
        check(self.lib.nb_energy(self.handle, ptr(m), ptr(x), ptr(y), ptr(z), ptr(vx), ptr(vy),
                                 ptr(vz), m.numel(), G, ptr(out), stream_ptr(stream)))

    def aabb(self, x, y, z, out, stream=None):
        check(self.lib.nb_aabb(self.handle, ptr(x), ptr(y), ptr(z), x.numel(), ptr(out),
                               stream_ptr(stream)))
