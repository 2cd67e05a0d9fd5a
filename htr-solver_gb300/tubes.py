"""Batched 1-D shock tubes: seeded instances, packing into one strip, stepping.

A shock tube is a 1-D grid of L interior cells on [0, 1] with one staggered
Dirichlet ghost node at each end (HTR's node types for a Dirichlet boundary,
src/prometeo_metric.rg:196-264: L_S, Lp1_S, Lp2_S, Std..., Rm3_S, Rm2_S,
Rm1_S, R_S) and a single periodic cell in y and z.  The batched form packs
many tubes end to end into one strip (nx = sum(L_i + 2), ny = nz = 1).  The
boundary node types keep every stencil inside its own tube, the ghost nodes
keep their imposed state, and the one-cell y/z directions contribute nothing,
so one fused RK3 step of the strip advances every tube exactly as a separate
step of each tube would (same arithmetic per cell).

Instances follow the batched configuration of the benchmark: lengths
U{128..8192}, single-species gas (gamma 1.4) or 5-species air with
probability 1/2, seeded left/right states with pressure ratio 2-100,
density ratio 1-10, temperatures 300-3000 K, gas at rest.
"""
import math

import ctypes as C

import numpy as np

from . import abi
from .fluid import Fluid

RGAS = 8.3144598
W_AIR = np.array([2 * 14.0067e-3, 2 * 15.9994e-3, 30.00610e-3, 14.0067e-3, 15.9994e-3])
X_AIR = np.array([0.79, 0.21, 0.0, 0.0, 0.0])
# CFL number of a shock tube's own step size: at 0.8 the first SSP-RK3 step
# of the strongest seeded tubes (pressure ratio up to 100) already drives
# the reference's Newton solve for T to NaN in some short air tubes; 0.4
# keeps every seeded tube well behaved.
TUBE_CFL = 0.4

AIR_REF = dict(PRef=101325.0, TRef=300.0, LRef=1.0, XiRef=(0.79, 0.21, 0.0, 0.0, 0.0))
GAS_R = 287.15
GAS_PARAMS = dict(gasConstant=GAS_R, gamma=1.4, prandtl=0.71, viscosityModel=abi.HTR_VISC_CONSTANT,
                  p0=1.8e-5, p1=0.0, p2=0.0)

# Node types (src/prometeo_metric_coeffs.h:54-66)
STD, L_S, LP1_S, LP2_S, RM3_S, RM2_S, RM1_S, R_S = 0, 1, 2, 3, 4, 5, 6, 7

# The rows of the reference's stencil tables used by a staggered Dirichlet
# tube (src/prometeo_metric_coeffs.cc: offsets, Recon_Plus, Coeffs_Plus,
# Grad); they define the grid metric of such a tube.
_Z6 = [0.0] * 6
_STD_R = [[0.0, -1 / 6, 5 / 6, 2 / 6, 0.0, 0.0], [0.0, 0.0, 2 / 6, 5 / 6, -1 / 6, 0.0],
          [2 / 6, -7 / 6, 11 / 6, 0.0, 0.0, 0.0], [0.0, 0.0, 3 / 12, 13 / 12, -5 / 12, 1 / 12]]
_STD_W = [9 / 20, 6 / 20, 1 / 20, 4 / 20]
NODE = {
    STD: dict(off=(-2, -1, 1, 2, 3), rp=_STD_R, cp=_STD_W, grad=(0.5, 0.5)),
    L_S: dict(off=(0, 0, 1, 1, 1), rp=[[0, 0, 1.0, 0, 0, 0]] * 4, cp=_STD_W, grad=(0.0, 2.0)),
    LP1_S: dict(off=(-1, -1, 1, 2, 3), rp=[[0.0, -2 / 4, 5 / 4, 1 / 4, 0.0, 0.0], _STD_R[1], _Z6, _STD_R[3]],
                cp=[2 / 4, 1 / 4, 0.0, 1 / 4], grad=(1.0, 0.5)),
    LP2_S: dict(off=(-2, -1, 1, 2, 3), rp=[_STD_R[0], _STD_R[1], [1.0, -2.0, 2.0, 0.0, 0.0, 0.0], _STD_R[3]],
                cp=[47 / 100, 27 / 100, 10 / 100, 16 / 100], grad=(0.5, 0.5)),
    RM3_S: dict(off=(-2, -1, 1, 2, 3), rp=[_STD_R[0], _STD_R[1], _STD_R[2], [0.0, 0.0, 2 / 9, 11 / 9, -7 / 9, 3 / 9]],
                cp=[39 / 100, 27 / 100, 4 / 100, 30 / 100], grad=(0.5, 0.5)),
    RM2_S: dict(off=(-2, -1, 1, 2, 2), rp=[_STD_R[0], [0.0, 0.0, 1 / 4, 5 / 4, -2 / 4, 0.0], _STD_R[2], _Z6],
                cp=[7 / 16, 8 / 16, 1 / 16, 0.0], grad=(0.5, 0.5)),
    RM1_S: dict(off=(-1, -1, 1, 1, 1), rp=[[0, 0, 0, 1.0, 0, 0]] * 4, cp=_STD_W, grad=(0.5, 1.0)),
    R_S: dict(off=(-1, -1, 0, 0, 0), rp=[_Z6] * 4, cp=[0.0] * 4, grad=(2.0, 0.0)),
}


def node_types(L):
    """x node types of a tube with L interior cells (L >= 6) and its 2 ghosts."""
    t = np.full(L + 2, STD, dtype=np.int32)
    t[0], t[1], t[2] = L_S, LP1_S, LP2_S
    t[-4], t[-3], t[-2], t[-1] = RM3_S, RM2_S, RM1_S, R_S
    return t


def metric_1d(L, width=1.0):
    """Euler, diffusion and staggered x metrics of a uniform tube with staggered
    ghosts on the boundary faces (src/prometeo_metric.cc:73-110,
    src/prometeo_metric.hpp:142-170, ghost corrections :186-255)."""
    dx = width / L
    x = np.concatenate([[0.0], (np.arange(L) + 0.5) * dx, [width]])
    t = node_types(L)
    n = L + 2

    def recon(p):
        nd = NODE[int(t[p])]
        o = nd["off"]
        pts = [x[min(max(p + o[0], 0), n - 1)], x[min(max(p + o[1], 0), n - 1)], x[p],
               x[min(max(p + o[2], 0), n - 1)], x[min(max(p + o[3], 0), n - 1)], x[min(max(p + o[4], 0), n - 1)]]
        return sum(pts[j] * sum(nd["rp"][k][j] * nd["cp"][k] for k in range(4)) for j in range(6))

    # face coordinates x_{p+1/2}: standard nodes vectorised, boundary nodes one by one
    xf = np.empty(n)
    w = np.array([sum(NODE[STD]["rp"][k][j] * NODE[STD]["cp"][k] for k in range(4)) for j in range(6)])
    i = np.arange(3, n - 4)
    xf[i] = (x[i - 2] * w[0] + x[i - 1] * w[1] + x[i] * w[2] + x[i + 1] * w[3] + x[i + 2] * w[4] +
             x[i + 3] * w[5])
    for p in list(range(0, 3)) + list(range(n - 4, n)):
        xf[p] = recon(p)
    xm0 = recon(0 + NODE[int(t[0])]["off"][1])
    dxf = np.diff(np.concatenate([[xm0], xf]))
    m_e = np.divide(1.0, dxf, out=np.zeros(n), where=dxf != 0)
    # collocated (getDeriv) and staggered metrics
    m_d = np.empty(n)
    m_d[i] = 1.0 / (0.5 * (x[i] - x[i - 1]) + 0.5 * (x[i + 1] - x[i]))
    for p in list(range(0, 3)) + list(range(n - 4, n)):
        nd = NODE[int(t[p])]
        pm1 = min(max(p + nd["off"][1], 0), n - 1)
        pp1 = min(max(p + nd["off"][2], 0), n - 1)
        m_d[p] = 1.0 / (nd["grad"][0] * (x[p] - x[pm1]) + nd["grad"][1] * (x[pp1] - x[p]))
    m_s = np.empty(n)
    m_s[:-1] = 1.0 / np.diff(x)
    m_s[-1] = 1.0 / dx
    m_e[0] = 1.0 / (-8.0 / 3.0 * x[0] + 3.0 * x[1] - 1.0 / 3.0 * x[2])
    m_e[-1] = 1.0 / (8.0 / 3.0 * x[-1] - 3.0 * x[-2] + 1.0 / 3.0 * x[-3])
    return m_e, m_d, m_s


def instances(n, seed=0, length=(128, 8192), air_fraction=0.5, rng=None):
    """Seeded tube descriptors: dict(L, eos, left=(p, T), right=(p, T))."""
    rng = rng or np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        L = int(rng.integers(length[0], length[1] + 1))
        eos = abi.HTR_EOS_AIRMIX if rng.uniform() < air_fraction else abi.HTR_EOS_CONSTPROPMIX
        while True:
            TL, TR = rng.uniform(300.0, 3000.0, size=2)
            rp = math.exp(rng.uniform(math.log(2.0), math.log(100.0)))
            rr = rp * TR / TL  # rho_L / rho_R of an ideal gas of one composition
            if 1.0 <= rr <= 10.0:
                break
        pL = 101325.0 * math.exp(rng.uniform(math.log(0.5), math.log(5.0)))
        out.append(dict(L=L, eos=eos, left=(pL, TL), right=(pL / rp, TR)))
    return out


def tube_fluid(inst):
    """Host Fluid of one tube (L + 2 cells in x, ghosts included)."""
    L = inst["L"]
    nspec = 5 if inst["eos"] == abi.HTR_EOS_AIRMIX else 1
    fl = Fluid((L + 2, 1, 1), nspec)
    xs = np.concatenate([[0.0], (np.arange(L) + 0.5) / L, [1.0]])
    left = xs < 0.5
    (pL, TL), (pR, TR) = inst["left"], inst["right"]
    p = np.where(left, pL, pR)
    T = np.where(left, TL, TR)
    if nspec == 5:
        fl["pressure"] = (p / AIR_REF["PRef"]).reshape(1, 1, -1)
        fl["temperature"] = (T / AIR_REF["TRef"]).reshape(1, 1, -1)
        fl["MolarFracs"] = np.broadcast_to(X_AIR, fl["MolarFracs"].shape)
    else:
        fl["pressure"] = p.reshape(1, 1, -1)
        fl["temperature"] = T.reshape(1, 1, -1)
        fl["MolarFracs"] = 1.0
    fl["velocity"] = 0.0
    fl["nType_x"] = node_types(L).reshape(1, 1, -1)
    m_e, m_d, m_s = metric_1d(L)  # LRef = 1 m: the same in nondimensional units
    fl["dcsi_e"] = m_e.reshape(1, 1, -1)
    fl["dcsi_d"] = m_d.reshape(1, 1, -1)
    fl["dcsi_s"] = m_s.reshape(1, 1, -1)
    for name in ("deta", "dzet"):
        for suf in ("_e", "_d", "_s"):
            fl[name + suf] = 1.0
    fl.meta = dict(workload="shock_tube", eos=inst["eos"], L=L, bnum=(1, 0, 0),
                   mix=(AIR_REF if nspec == 5 else GAS_PARAMS), vorticityScale=1.0)
    return fl


def _tube_arrays(inst):
    """Per-cell x arrays of one tube: node type, metrics, p, T (model units)."""
    L = inst["L"]
    m_e, m_d, m_s = metric_1d(L)
    xs = np.concatenate([[0.0], (np.arange(L) + 0.5) / L, [1.0]])
    left = xs < 0.5
    (pL, TL), (pR, TR) = inst["left"], inst["right"]
    p = np.where(left, pL, pR)
    T = np.where(left, TL, TR)
    if inst["eos"] == abi.HTR_EOS_AIRMIX:
        p = p / AIR_REF["PRef"]
        T = T / AIR_REF["TRef"]
    return node_types(L), m_e, m_d, m_s, p, T


def build_strip(insts):
    """The strip of `insts` (one mixture) built directly; equals
    pack([tube_fluid(i) for i in insts]).  Returns (strip, x offsets)."""
    assert len({i["eos"] for i in insts}) == 1
    air = insts[0]["eos"] == abi.HTR_EOS_AIRMIX
    parts = [_tube_arrays(i) for i in insts]
    offs = np.cumsum([0] + [len(pt[0]) for pt in parts])
    n = int(offs[-1])
    strip = Fluid((n, 1, 1), 5 if air else 1)
    cat = lambda k: np.concatenate([pt[k] for pt in parts]).reshape(1, 1, -1)
    strip["nType_x"] = cat(0)
    strip["dcsi_e"], strip["dcsi_d"], strip["dcsi_s"] = cat(1), cat(2), cat(3)
    strip["pressure"], strip["temperature"] = cat(4), cat(5)
    if air:
        strip["MolarFracs"] = np.broadcast_to(X_AIR, strip["MolarFracs"].shape)
    else:
        strip["MolarFracs"] = 1.0
    strip["velocity"] = 0.0
    for name in ("deta", "dzet"):
        for suf in ("_e", "_d", "_s"):
            strip[name + suf] = 1.0
    strip.meta = dict(workload="shock_tube_strip", eos=insts[0]["eos"], bnum=(0, 0, 0), tubes=len(insts),
                      mix=(AIR_REF if air else GAS_PARAMS), vorticityScale=1.0)
    return strip, offs[:-1]


def tube_view(strip_view, off, L):
    """htr_fluid_view of one tube inside a strip (bases shifted by `off` cells),
    with its bounds and interior rectangles in tube coordinates."""
    import ctypes as C
    v = abi.htr_fluid_view()
    C.memmove(C.byref(v), C.byref(strip_view), C.sizeof(v))
    for name, _ in abi.htr_fluid_view._fields_:
        f = getattr(v, name)
        if f.base:
            f.base = f.base + off * f.stride[0]
    return v, abi.rect((0, 0, 0), (L + 1, 0, 0)), abi.rect((1, 0, 0), (L, 0, 0))


def pack(fluids):
    """One strip holding the given tubes (same mixture) end to end; returns the
    strip and the x offset of each tube."""
    assert len({f.nspec for f in fluids}) == 1
    offs = np.cumsum([0] + [f.nx for f in fluids])
    strip = Fluid((int(offs[-1]), 1, 1), fluids[0].nspec)
    for name in strip.arrays:
        strip.arrays[name][...] = np.concatenate([f.arrays[name] for f in fluids], axis=2)
    strip.meta = dict(fluids[0].meta)
    strip.meta.update(workload="shock_tube_strip", bnum=(0, 0, 0), tubes=len(fluids))
    return strip, offs[:-1]


def cell_dt(offs, widths, dts):
    """Step size of every cell of a strip (ghost nodes included): the dt of
    the tube the cell belongs to.  widths[k] = cells of tube k with its two
    ghosts."""
    n = int(offs[-1] + widths[-1])
    out = np.empty(n)
    for o, w, d in zip(offs, widths, dts):
        out[int(o):int(o) + int(w)] = d
    return out


def strip_dts(strip_dev, offs, widths, gh, cfl=TUBE_CFL, chemistry=False, lib=None):
    """Each tube's own step size (CFL `cfl` over its own spectral radius;
    with chemistry also at most half its fastest chemical time scale), as one
    run of the reference computes it per simulation
    (src/prometeo.rg:1153-1172).  Device strip in, list of floats out."""
    import torch

    from . import runtime
    from .fluid import Fluid
    l = lib or runtime.lib()
    dts = []
    for o, w in zip(offs, widths):
        L = int(w) - 2
        v, fb, inner = tube_view(strip_dev.view(), int(o), L)
        out = torch.zeros(1, dtype=torch.float64, device=strip_dev.device)
        abi.check(l, l.htr_CalculateMaxSpectralRadius(C.byref(v), inner, gh, C.cast(C.c_void_p(out.data_ptr()),
                                                                                    C.POINTER(C.c_double)),
                                                      runtime.stream_handle()), "spectral radius")
        dts.append(out)
    torch.cuda.synchronize()
    dts = [cfl / d.item() for d in dts]
    if chemistry:
        v = strip_dev.view()
        abi.check(l, l.htr_InitializeTimeDerivatives(C.byref(v), strip_dev.bounds(), 0, gh, runtime.stream_handle()),
                  "init")
        abi.check(l, l.htr_AddChemistrySources(C.byref(v), strip_dev.interior(), gh, runtime.stream_handle()),
                  "chem")
        torch.cuda.synchronize()
        ns = strip_dev.nspec
        w_ = strip_dev["Conserved_t"][0, 0, :, :ns].abs()
        rhoi = strip_dev["Conserved"][0, 0, :, :ns]
        sig = rhoi > 1e-3 * strip_dev["rho"][0, 0, :, None]
        tau = torch.where(sig, rhoi / w_.clamp_min(1e-300), torch.full_like(rhoi, float("inf"))).min(dim=1).values
        tau = tau.cpu().numpy()
        dts = [min(d, 0.5 * float(tau[int(o) + 1:int(o) + int(w) - 1].min())) for d, o, w in zip(dts, offs, widths)]
    return dts


def unpack(strip, offs, lengths):
    """Views of each tube's cells in a host strip: list of dict name -> array."""
    out = []
    for o, L in zip(offs, lengths):
        out.append({k: a[:, :, o:o + L + 2] for k, a in strip.arrays.items()})
    return out
