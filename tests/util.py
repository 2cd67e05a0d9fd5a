"""Shared helpers of the test suite: seeded states, CPU oracle runs, error metrics."""
import ctypes as C

import numpy as np

from htr_gb300 import abi, workloads  # noqa: F401  (re-exported for tests)

import oracle

# Relative error bound of the RHS path against the CPU oracle (FP64): per
# conserved component, max |gpu - cpu| / max |cpu| over the grid.
RHS_REL_TOL = 1e-11


def rel_err(a, b):
    """Per-component max |a-b| / max |b| over all cells (last axis = components)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.ndim == 3:
        a, b = a[..., None], b[..., None]
    d = np.abs(a - b).reshape(-1, a.shape[-1]).max(axis=0)
    s = np.abs(b).reshape(-1, b.shape[-1]).max(axis=0)
    return d / np.maximum(s, 1e-300)


def make_state(lib, kind, n, seed=0):
    """Seeded state built (properties + conserved) by `lib`; returns fluid, mixture handle, struct."""
    if kind == "tg":
        fl = workloads.taylor_green(shape=n, seed=seed)
    else:
        fl = workloads.air_box(shape=n, seed=seed)
    eos = fl.meta["eos"]
    m = workloads.make_mixture_struct(lib, eos, fl.meta["mix"])
    h = oracle.load_mixture(lib, eos, m)
    workloads.derive_state(lib, fl, h)
    return fl, h, m


def call(lib, name, *args):
    st = getattr(lib, name)(*args)
    abi.check(lib, st, name)


def struct_diff(a, b, prefix=""):
    """Field-wise differences of two ctypes structures (padding ignored)."""
    out = []
    if hasattr(a, "_fields_"):
        for name, _ in type(a)._fields_:
            out += struct_diff(getattr(a, name), getattr(b, name), prefix + "." + name)
    elif hasattr(a, "_length_") and not isinstance(a, (bytes, str)):
        for i in range(len(a)):
            out += struct_diff(a[i], b[i], f"{prefix}[{i}]")
    elif a != b and not (a != a and b != b):
        out.append((prefix, a, b))
    return out
