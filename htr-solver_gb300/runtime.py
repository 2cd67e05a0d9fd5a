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
                ("deltaTime", C.c_double), ("explicitChemistry", C.c_int), ("implicitChemistry", C.c_int)]


SCHEMES = {"Hybrid": 0, "TENO": 1, "TENOA": 2, "TENOLAD": 3, "SkewSymmetric": 4}


class htr_bc_params(C.Structure):
    _fields_ = [("type", C.c_int * 6), ("P", C.c_double * 6), ("LengthScale", C.c_double * 6),
                ("plane", abi.htr_rect3 * 6), ("sensor", abi.htr_rect3 * 3)]


BC_TYPES = {"Periodic": 0, "NSCBC_Inflow": 1, "NSCBC_Outflow": 2, "IsothermalWall": 3, "AdiabaticWall": 4}


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
        l.htr_rk3_workspace_bytes.argtypes = [abi.htr_rect3, C.c_void_p]
        l.htr_rk3_workspace_bytes.restype = C.c_size_t
        l.htr_rk3_step_ws.argtypes = [C.POINTER(abi.htr_fluid_view), abi.htr_rect3, abi.htr_rect3,
                                      C.POINTER(htr_step_params), C.c_void_p, C.c_void_p, C.c_size_t,
                                      C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
        l.htr_rk3_step_ws.restype = C.c_int
        l.htr_rk3_step_static.argtypes = [C.POINTER(abi.htr_fluid_view), abi.htr_rect3, abi.htr_rect3,
                                          C.POINTER(htr_step_params), C.c_void_p, C.POINTER(C.c_double),
                                          C.c_void_p, C.c_void_p]
        l.htr_rk3_step_static.restype = C.c_int
        l.htr_rk3_step_bc_ws.argtypes = [C.POINTER(abi.htr_fluid_view), abi.htr_rect3, abi.htr_rect3,
                                         C.POINTER(htr_step_params), C.POINTER(htr_bc_params), C.c_void_p,
                                         C.c_void_p, C.c_size_t, C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
        l.htr_rk3_step_bc_ws.restype = C.c_int
        l.htr_rk3_step_cells_ws.argtypes = [C.POINTER(abi.htr_fluid_view), abi.htr_rect3, abi.htr_rect3,
                                            C.POINTER(htr_step_params), C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_size_t, C.c_void_p, C.c_void_p]
        l.htr_rk3_step_cells_ws.restype = C.c_int
        l.htr_rk3_static_scratch_bytes.argtypes = []
        l.htr_rk3_static_scratch_bytes.restype = C.c_size_t
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


class Workspace:
    """Device workspace of the fused step (grown on demand, 256-byte aligned)."""

    def __init__(self):
        self.buf = None
        self.nbytes = 0

    def get(self, nbytes, device):
        import torch
        dev = torch.device(device)
        if dev.type == "cuda" and dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        if self.buf is None or self.nbytes < nbytes or self.buf.device != dev:
            self.buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
            self.nbytes = nbytes
        addr = self.buf.data_ptr()
        return (addr + 255) // 256 * 256


_workspace = Workspace()


def workspace_bytes(fluid, mixh, interior=None):
    inner = fluid.interior() if interior is None else interior
    return lib().htr_rk3_workspace_bytes(inner, mixh)


def rk3_step(fluid, mixh, scheme="Hybrid", vorticity_scale=1.0, cfl=0.0, dt=0.0,
             chemistry=True, stream=None, interior=None, status_dev=None, fused=True,
             workspace=None, implicit=False):
    """One SSP-RK3 step of a device grid; returns the dt used.

    fused=True runs htr_rk3_step_ws (fused stage pipeline, periodic grids) on
    `workspace` (a Workspace, default: one cached per process); fused=False
    runs htr_rk3_step, the composition of the per-task entry points.
    implicit=True advances the chemistry with the implicit solver
    (Integrator.implicitChemistry) instead of explicit sources."""
    l = lib()
    p = htr_step_params(SCHEMES[scheme], vorticity_scale, cfl, dt, 1 if chemistry else 0, 1 if implicit else 0)
    v = fluid.view()
    used = C.c_double(0.0)
    inner = fluid.interior() if interior is None else interior
    if fused:
        nb = l.htr_rk3_workspace_bytes(inner, mixh)
        ws = (workspace or _workspace).get(nb, fluid.device)
        st = l.htr_rk3_step_ws(C.byref(v), inner, fluid.bounds(), C.byref(p), mixh, C.c_void_p(ws), nb,
                               C.byref(used), status_dev, stream_handle(stream))
        abi.check(l, st, "htr_rk3_step_ws")
    else:
        st = l.htr_rk3_step(C.byref(v), inner, fluid.bounds(), C.byref(p), mixh, C.byref(used),
                            status_dev, stream_handle(stream))
        abi.check(l, st, "htr_rk3_step")
    return used.value


def rk3_step_cells(fluid, mixh, dt_cell, scheme="Hybrid", vorticity_scale=1.0, chemistry=True, stream=None,
                   status_dev=None, workspace=None, implicit=False):
    """One SSP-RK3 step of a device grid of packed independent instances,
    each cell advancing by its own step size dt_cell (a device float64 tensor
    of one value per cell, shaped like the grid, x fastest):
    htr_rk3_step_cells_ws."""
    l = lib()
    if dt_cell.dtype.itemsize != 8 or not dt_cell.is_contiguous() or dt_cell.numel() != fluid.ncells:
        raise abi.HtrError("dt_cell must be a contiguous float64 tensor with one value per cell")
    p = htr_step_params(SCHEMES[scheme], vorticity_scale, 0.0, 0.0, 1 if chemistry else 0, 1 if implicit else 0)
    v = fluid.view()
    inner = fluid.interior()
    nb = l.htr_rk3_workspace_bytes(inner, mixh)
    ws = (workspace or _workspace).get(nb, fluid.device)
    st = l.htr_rk3_step_cells_ws(C.byref(v), inner, fluid.bounds(), C.byref(p), mixh, C.c_void_p(dt_cell.data_ptr()),
                                 C.c_void_p(ws), nb, status_dev, stream_handle(stream))
    abi.check(l, st, "htr_rk3_step_cells_ws")


def stable_dt(fluid, mixh, cfl=0.8, chemistry=True, stream=None):
    """Step size of a device grid: cfl / max spectral radius
    (src/prometeo_cfl.hpp:55-190), and with chemistry at most half the fastest
    chemical time scale rho_i / |w_i| of the species that carry at least 0.1 %
    of the mass (explicit chemistry stays stable)."""
    import torch
    l = lib()
    v = fluid.view()
    s = stream_handle(stream)
    out = torch.zeros(1, dtype=torch.float64, device=fluid.device)
    abi.check(l, l.htr_CalculateMaxSpectralRadius(C.byref(v), fluid.interior(), mixh,
                                                  C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)), s),
              "htr_CalculateMaxSpectralRadius")
    st = stream if stream is not None else torch.cuda.current_stream()
    st.synchronize()
    dt = cfl / out.item()
    if chemistry and fluid.nspec > 1:
        abi.check(l, l.htr_InitializeTimeDerivatives(C.byref(v), fluid.bounds(), 0, mixh, s), "init")
        abi.check(l, l.htr_AddChemistrySources(C.byref(v), fluid.interior(), mixh, s), "chem")
        st.synchronize()
        ns = fluid.nspec
        w = fluid["Conserved_t"][..., :ns].abs()
        rhoi = fluid["Conserved"][..., :ns]
        rho = fluid["rho"][..., None]
        sig = rhoi > 1e-3 * rho
        tau = torch.where(sig, rhoi / w.clamp_min(1e-300), torch.full_like(rhoi, float("inf"))).min().item()
        dt = min(dt, 0.5 * tau)
    return dt
