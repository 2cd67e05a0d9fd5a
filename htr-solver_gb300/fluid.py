"""Field storage for one HTR grid instance, host (numpy) or device (torch).

Arrays are shaped (Nz, Ny, Nx[, ncomp]) so that x is the fastest index and
vector components are contiguous per point: the reference's default Legion
layout for Fluid_columns (src/prometeo_types.h:49-114).  Grid point
(x, y, z) is element [z, y, x]; the view passed over the C ABI carries the
address of point (0,0,0) and byte strides.
"""
import numpy as np

from . import abi

_NP_DTYPES = {"float64": np.float64, "int32": np.int32, "bool": np.bool_}


def ncomp(spec, nspec):
    if spec == "nSpec":
        return nspec
    if spec == "nEq":
        return nspec + 4
    return int(spec)


def field_shape(name, shape, nspec):
    for n, _dt, comp in abi.FIELD_SPECS:
        if n == name:
            c = ncomp(comp, nspec)
            return tuple(shape) + ((c,) if c > 1 or comp in ("nSpec", "nEq", 3) else ())
    raise KeyError(name)


class Fluid:
    """One grid's fields.  `shape` is (Nx, Ny, Nz) including ghost layers."""

    def __init__(self, shape, nspec, device=None, fields=None):
        self.nx, self.ny, self.nz = (int(s) for s in shape)
        self.nspec = int(nspec)
        self.neq = self.nspec + 4
        self.device = device
        self.arrays = {}
        self.meta = {}
        names = abi.FIELD_NAMES if fields is None else fields
        for name, dt, comp in abi.FIELD_SPECS:
            if name not in names:
                continue
            shp = field_shape(name, (self.nz, self.ny, self.nx), self.nspec)
            if device is None:
                self.arrays[name] = np.zeros(shp, dtype=_NP_DTYPES[dt])
            else:
                import torch
                tdt = {"float64": torch.float64, "int32": torch.int32, "bool": torch.bool}[dt]
                self.arrays[name] = torch.zeros(shp, dtype=tdt, device=device)

    @property
    def shape(self):
        return (self.nx, self.ny, self.nz)

    @property
    def ncells(self):
        return self.nx * self.ny * self.nz

    def __getitem__(self, name):
        return self.arrays[name]

    def __setitem__(self, name, value):
        a = self.arrays[name]
        if self.device is None:
            a[...] = value
        else:
            import torch
            if isinstance(value, np.ndarray):
                value = torch.from_numpy(np.ascontiguousarray(value))
            a.copy_(value.to(a.device) if hasattr(value, "to") else value)

    def view(self):
        """htr_fluid_view over these arrays (null for absent fields)."""
        v = abi.htr_fluid_view()
        for name, a in self.arrays.items():
            f = getattr(v, name)
            if self.device is None:
                f.base = a.ctypes.data
                st = a.strides
                f.stride[0], f.stride[1], f.stride[2] = st[2], st[1], st[0]
            else:
                f.base = a.data_ptr()
                es = a.element_size()
                st = a.stride()
                f.stride[0], f.stride[1], f.stride[2] = st[2] * es, st[1] * es, st[0] * es
        return v

    def to_device(self, device, fields=None):
        import torch
        out = Fluid(self.shape, self.nspec, device=device, fields=list(self.arrays))
        for name, a in self.arrays.items():
            if fields is None or name in fields:
                out.arrays[name].copy_(torch.from_numpy(np.ascontiguousarray(a)))
        return out

    def to_host(self, fields=None):
        out = Fluid(self.shape, self.nspec, device=None, fields=list(self.arrays))
        for name, a in self.arrays.items():
            if fields is None or name in fields:
                out.arrays[name][...] = a.detach().cpu().numpy() if self.device else a
        return out

    def copy(self):
        """Deep copy on the same device (host arrays or device tensors)."""
        out = Fluid(self.shape, self.nspec, device=self.device, fields=list(self.arrays))
        for name, a in self.arrays.items():
            if self.device is None:
                out.arrays[name][...] = a
            else:
                out.arrays[name].copy_(a)
        out.meta = dict(self.meta)
        return out

    def interior(self, bnum=(0, 0, 0)):
        bx, by, bz = bnum
        return abi.rect((bx, by, bz), (self.nx - 1 - bx, self.ny - 1 - by, self.nz - 1 - bz))

    def bounds(self):
        return abi.rect((0, 0, 0), (self.nx - 1, self.ny - 1, self.nz - 1))
