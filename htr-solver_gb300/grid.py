"""Stretched Cartesian grids with boundary layers: HTR's grid set-up.

  node positions  InitializeNodeGrid / transform_uniform_to_nonuniform
                  (src/prometeo_grid.rg:100-221): Uniform, Cosine, Tanh,
                  TanhMinus, TanhPlus, Sinh, SinhMinus, SinhPlus
  cell centres    InitializeCellCenters (src/prometeo_grid.rg:228-320):
                  midpoints of the nodes; a staggered boundary point sits on
                  the boundary node, a collocated one half a cell outside
  ghost layers    one per non-periodic direction (src/prometeo.rg:713-718)
  node types      InitializeOperators + CorrectGhostOperators
                  (src/prometeo_metric.rg:130-291)
  metrics         htr_InitializeMetric + htr_CorrectGhostMetric{X,Y,Z}
                  (InitializeMetric, src/prometeo_metric.rg:347-378)

A grid is a product of three 1-D axes, so coordinates and node types are
built per axis and broadcast.  Boundary-condition types are the reference's
FlowBC names (config_schema.lua).
"""
import ctypes as C
import math

import numpy as np

from . import abi

PERIODIC = "Periodic"
STAGGERED = {"Dirichlet", "AdiabaticWall", "IsothermalWall", "SuctionAndBlowingWall"}
COLLOCATED = {"NSCBC_Inflow", "NSCBC_Outflow", "NSCBC_FarField", "IncomingShock", "RecycleRescaling"}

# node types (src/prometeo_metric_coeffs.h:54-66)
STD, L_S, LP1_S, LP2_S, RM3_S, RM2_S, RM1_S, R_S, L_C, LP1_C, RM2_C, RM1_C, R_C = range(13)


def _lerp(xi, alpha, beta, a, b):
    return (b - a) / (beta - alpha) * (xi - alpha) + a


def _transform(x, xmin, xmax, kind, s):
    """Map a uniform sample to the stretched one (prometeo_grid.rg:137-203)."""
    if kind == "Uniform":
        return x
    if kind == "Cosine":
        t = _lerp(x, xmin, xmax, -1.0, 1.0)
        return _lerp(-1.0 * math.cos(math.pi * (t + 1.0) / 2.0), -1.0, 1.0, xmin, xmax)
    table = {"TanhMinus": (-1.0, 0.0, math.tanh), "TanhPlus": (0.0, 1.0, math.tanh), "Tanh": (-1.0, 1.0, math.tanh),
             "SinhMinus": (0.0, 1.0, math.sinh), "SinhPlus": (-1.0, 0.0, math.sinh), "Sinh": (-1.0, 1.0, math.sinh)}
    if kind not in table:
        raise ValueError(f"grid type {kind}")
    lo, hi, f = table[kind]
    t = _lerp(x, xmin, xmax, lo, hi)
    return _lerp(f(s * t) / f(s), lo, hi, xmin, xmax)


def nodes(origin, width, num, kind="Uniform", stretching=1.0):
    """num + 1 node positions of one axis."""
    dx = (origin + width - origin) / num
    return np.array([_transform(origin + float(c) * dx, origin, origin + width, kind, stretching)
                     for c in range(num + 1)])


def bnum(bc_left):
    return 0 if bc_left == PERIODIC else 1


def centers(node, num, left, right):
    """Cell-centre coordinates of one axis including its ghost points."""
    b = bnum(left)
    n = num + 2 * b
    out = np.empty(n)
    for c in range(n):
        if c < b:
            out[c] = node[c] if left in STAGGERED else 1.5 * node[c] - 0.5 * node[c + 1]
        elif c >= num + b:
            out[c] = node[c - 1] if right in STAGGERED else 1.5 * node[c - 1] - 0.5 * node[c - 2]
        else:
            i = c - b
            out[c] = 0.5 * (node[i + 1] + node[i])
    return out


def node_types(n, num, left, right):
    """Node type of every point of one axis (CorrectGhostOperators): the left
    side is set first, the right side after it (it wins on short axes)."""
    t = np.full(n, STD, dtype=np.int32)
    if left == PERIODIC:
        return t
    b = bnum(left)
    neg = lambda c: c < b
    pos = lambda c: c >= num + b
    ls, lc = left in STAGGERED, left in COLLOCATED
    rs, rc = right in STAGGERED, right in COLLOCATED
    for c in range(n):
        cm1, cm2 = (c - 1) % n, (c - 2) % n
        cp1, cp2, cp3 = (c + 1) % n, (c + 2) % n, (c + 3) % n
        if neg(c):
            t[c] = L_S if ls else (L_C if lc else t[c])
        elif neg(cm1):
            t[c] = LP1_S if ls else (LP1_C if lc else t[c])
        elif neg(cm2):
            if ls:
                t[c] = LP2_S
        if pos(c):
            t[c] = R_S if rs else (R_C if rc else t[c])
        elif pos(cp1):
            t[c] = RM1_S if rs else (RM1_C if rc else t[c])
        elif pos(cp2):
            t[c] = RM2_S if rs else (RM2_C if rc else t[c])
        elif pos(cp3):
            if rs:
                t[c] = RM3_S
    return t


class Grid:
    """A stretched Cartesian grid: per-axis centres and node types.

    num[d]        interior cells of axis d
    width[d]      domain width; origin[d] its start
    bc[d]         (left, right) FlowBC types of axis d
    kind[d]       (grid type, stretching) of axis d
    """

    def __init__(self, num, width, bc, kind=(("Uniform", 1.0),) * 3, origin=(0.0, 0.0, 0.0)):
        self.num = tuple(int(n) for n in num)
        self.width = tuple(float(w) for w in width)
        self.origin = tuple(float(o) for o in origin)
        self.bc = tuple(tuple(b) for b in bc)
        for left, right in self.bc:
            if (left == PERIODIC) != (right == PERIODIC):
                raise ValueError("a periodic axis is periodic on both sides")
        self.bnum = tuple(bnum(b[0]) for b in self.bc)
        self.shape = tuple(n + 2 * b for n, b in zip(self.num, self.bnum))
        self.node = [nodes(o, w, n, k, s) for o, w, n, (k, s) in zip(self.origin, self.width, self.num, kind)]
        self.center = [centers(nd, n, *b) for nd, n, b in zip(self.node, self.num, self.bc)]
        self.ntype = [node_types(s, n, *b) for s, n, b in zip(self.shape, self.num, self.bc)]

    def center_coordinates(self):
        """(Nz, Ny, Nx, 3) cell-centre coordinates."""
        nx, ny, nz = self.shape
        cc = np.empty((nz, ny, nx, 3))
        cc[..., 0] = self.center[0][None, None, :]
        cc[..., 1] = self.center[1][None, :, None]
        cc[..., 2] = self.center[2][:, None, None]
        return cc

    def fill(self, fl, lib, stream=None):
        """Node types and metrics of Fluid `fl` (host or device) through `lib`."""
        fl["nType_x"] = np.broadcast_to(self.ntype[0][None, None, :], (fl.nz, fl.ny, fl.nx)).copy()
        fl["nType_y"] = np.broadcast_to(self.ntype[1][None, :, None], (fl.nz, fl.ny, fl.nx)).copy()
        fl["nType_z"] = np.broadcast_to(self.ntype[2][:, None, None], (fl.nz, fl.ny, fl.nx)).copy()
        cc = self.center_coordinates()
        if fl.device is not None:
            import torch
            cc = torch.from_numpy(cc).to(fl["rho"].device)
        f = field_of(cc)
        v = fl.view()
        allr = fl.bounds()
        w = (C.c_double * 3)(*self.width)
        abi.check(lib, lib.htr_InitializeMetric(C.byref(v), f, allr, allr, w, stream), "InitializeMetric")
        for d in "XYZ":
            abi.check(lib, getattr(lib, f"htr_CorrectGhostMetric{d}")(C.byref(v), f, allr, stream),
                      f"CorrectGhostMetric{d}")
        if fl.device is not None:
            import torch
            torch.cuda.synchronize()  # set-up only: the coordinates are released after this
        return fl


def field_of(a):
    """htr_field over an (Nz, Ny, Nx[, c]) numpy array or torch tensor."""
    f = abi.htr_field()
    if isinstance(a, np.ndarray):
        f.base = a.ctypes.data
        st = a.strides
        f.stride[0], f.stride[1], f.stride[2] = st[2], st[1], st[0]
    else:
        es = a.element_size()
        st = a.stride()
        f.base = a.data_ptr()
        f.stride[0], f.stride[1], f.stride[2] = st[2] * es, st[1] * es, st[0] * es
    return f
