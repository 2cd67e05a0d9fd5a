"""Loads libhtr_gb300.so and exposes its C ABI to Python.

The product path is the CUDA library only: if the library is missing or no
sm_103 device is usable, the calls fail with an HtrError; there is no CPU
fallback.
"""
import ctypes as C
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhtr_gb300.so")

EXTRA_PROTOTYPES = {}

_lib = None


class htr_step_params(C.Structure):
    _fields_ = [("scheme", C.c_int), ("vorticityScale", C.c_double), ("cfl", C.c_double),
                ("deltaTime", C.c_double), ("explicitChemistry", C.c_int)]


SCHEMES = {"Hybrid": 0, "TENO": 1, "TENOA": 2, "TENOLAD": 3, "SkewSymmetric": 4}


def lib():
    """The loaded CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise abi.HtrError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        l = C.CDLL(LIB_PATH)
        abi.bind(l)
        l.htr_rk3_step.argtypes = [C.POINTER(abi.htr_fluid_view), abi.htr_rect3, abi.htr_rect3,
                                   C.POINTER(htr_step_params), C.c_void_p, C.POINTER(C.c_double),
                                   C.c_void_p, C.c_void_p]
        l.htr_rk3_step.restype = C.c_int
        for name, args in EXTRA_PROTOTYPES.items():
            fn = getattr(l, name, None)
            if fn is not None:
                fn.argtypes = args
                fn.restype = C.c_int
        _lib = l
    return _lib


def stream_handle(stream=None):
    """cudaStream_t of a torch stream (default: the current stream)."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def load_mixture(eos, struct):
    l = lib()
    h = C.c_void_p()
    abi.check(l, l.htr_load_mixture(eos, C.byref(struct), C.sizeof(struct), C.byref(h)),
              "htr_load_mixture")
    return h


def rk3_step(fluid, mixh, scheme="Hybrid", vorticity_scale=1.0, cfl=0.0, dt=0.0,
             chemistry=True, stream=None, interior=None, status_dev=None):
    """One SSP-RK3 step of a periodic device grid; returns the dt used."""
    l = lib()
    p = htr_step_params(SCHEMES[scheme], vorticity_scale, cfl, dt, 1 if chemistry else 0)
    v = fluid.view()
    used = C.c_double(0.0)
    inner = fluid.interior() if interior is None else interior
    st = l.htr_rk3_step(C.byref(v), inner, fluid.bounds(), C.byref(p), mixh, C.byref(used),
                        status_dev, stream_handle(stream))
    abi.check(l, st, "htr_rk3_step")
    return used.value
