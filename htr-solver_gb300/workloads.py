"""Seeded synthetic initial states for the RHS workloads.

No dataset is involved: every workload is built from seeded random smooth
fields (numpy PCG64).  Generators fill the primitive variables (pressure,
temperature, MolarFracs, velocity), node types and grid metrics of a
`Fluid`; `derive_state` then completes the state the way HTR does after an
initialisation (UpdatePropertiesFromPrimitive followed by
UpdateConservedFromPrimitive, src/prometeo.rg:428-478) through any library
that exports the C ABI.

Workloads:
  taylor_green   3-D periodic 32^3 box, single-species calorically perfect
                 gas (gamma 1.4, Pr 0.71, power-law viscosity), Taylor-Green
                 vortex at Mach 0.1 (form of src/prometeo_init.rg:134-158)
                 with +-1 % seeded perturbations on rho, u, v, w, p.
  air_box        3-D periodic box of 5-species air: T in 300-8000 K from
                 smooth random modes, p in 0.1-10 bar (log-uniform modes),
                 Dirichlet(1)-distributed mass fractions varying smoothly in
                 space, velocities of local Mach 0.5-3 built from random
                 solenoidal plus compressive modes.
  vortex2d       2-D periodic isentropic vortex on a uniform stream.
(1-D shock tubes: see tubes.py.)
"""
import math

import numpy as np

from . import abi
from .fluid import Fluid

TWO_PI = 6.28318530718  # domain width used by HTR's periodic solver tests


def _centers(n, width=TWO_PI):
    dx = width / n
    return (np.arange(n) + 0.5) * dx, dx


def _uniform_metrics(fl, dx, dy, dz):
    for name, d in (("dcsi", dx), ("deta", dy), ("dzet", dz)):
        for suf in ("_e", "_d", "_s"):
            fl[name + suf] = 1.0 / d


def _smooth(rng, X, Y, Z, kmax=3, nmodes=6):
    """Smooth periodic random field normalised to [0, 1]."""
    f = np.zeros(np.broadcast(X, Y, Z).shape)
    for _ in range(nmodes):
        k = rng.integers(-kmax, kmax + 1, size=3)
        if not k.any():
            k[0] = 1
        amp = rng.uniform(0.5, 1.0) / math.sqrt(float(k @ k))
        ph = rng.uniform(0, 2 * math.pi)
        f = f + amp * np.cos(k[0] * X + k[1] * Y + k[2] * Z + ph)
    lo, hi = f.min(), f.max()
    return (f - lo) / (hi - lo) if hi > lo else np.zeros_like(f)


def constpropmix_params(visc_ref=1.0e-3):
    """Mixture of the Taylor-Green workload: (R, gamma, Pr, power law)."""
    gamma = 1.4
    T0 = 1.0 / gamma  # rho = 1, p = 1/gamma, R = 1
    return dict(gasConstant=1.0, gamma=gamma, prandtl=0.71,
                viscosityModel=abi.HTR_VISC_POWERLAW, p0=T0, p1=visc_ref, p2=0.0)


AIR_REF = dict(PRef=101325.0, TRef=300.0, LRef=1.0, XiRef=(0.79, 0.21, 0.0, 0.0, 0.0))


def taylor_green(n=32, seed=0, shape=None, device=None):
    """Config: 32^3 periodic Taylor-Green + 1 % perturbations (ConstPropMix)."""
    nx, ny, nz = shape if shape is not None else (n, n, n)
    rng = np.random.Generator(np.random.PCG64(seed))
    xc, dx = _centers(nx)
    yc, dy = _centers(ny)
    zc, dz = _centers(nz)
    Z, Y, X = np.meshgrid(zc, yc, xc, indexing="ij")
    gamma, R, rho0, V0 = 1.4, 1.0, 1.0, 0.1
    p0 = 1.0 / gamma
    u = V0 * np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -V0 * np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(u)
    p = p0 + rho0 * V0 * V0 / 16.0 * (np.cos(2 * Z) + 2.0) * (np.cos(2 * X) + np.cos(2 * Y))
    pert = lambda: rng.uniform(-0.01, 0.01, size=u.shape)
    rho = rho0 * (1.0 + pert())
    p = p * (1.0 + pert())
    u = u + V0 * pert()
    v = v + V0 * pert()
    w = w + V0 * pert()
    fl = Fluid((nx, ny, nz), 1)
    fl["pressure"] = p
    fl["temperature"] = p / (rho * R)
    fl["MolarFracs"] = 1.0
    fl["velocity"] = np.stack([u, v, w], axis=-1)
    _uniform_metrics(fl, dx, dy, dz)
    fl.meta = dict(workload="taylor_green", eos=abi.HTR_EOS_CONSTPROPMIX, seed=seed,
                   mix=constpropmix_params(), periodic=(True, True, True), bnum=(0, 0, 0),
                   vorticityScale=1.0, cfl=0.8)
    return fl


def air_box(n=256, seed=0, shape=None, mach=(0.5, 3.0), T=(300.0, 8000.0), p_bar=(0.1, 10.0)):
    """Config: periodic box of 5-species reacting air (AirMix)."""
    nx, ny, nz = shape if shape is not None else (n, n, n)
    rng = np.random.Generator(np.random.PCG64(seed))
    xc, dx = _centers(nx)
    yc, dy = _centers(ny)
    zc, dz = _centers(nz)
    Z, Y, X = np.meshgrid(zc, yc, xc, indexing="ij")
    ref = AIR_REF
    Tk = T[0] + (T[1] - T[0]) * _smooth(rng, X, Y, Z)
    lp = math.log10(p_bar[0] * 1e5) + (math.log10(p_bar[1] / p_bar[0])) * _smooth(rng, X, Y, Z)
    Pa = 10.0 ** lp
    # Dirichlet(1) marginals that vary smoothly: exponential transforms of
    # smooth uniforms, normalised.
    W = np.array([2 * 14.0067e-3, 2 * 15.9994e-3, 14.0067e-3 + 15.9994e-3, 14.0067e-3, 15.9994e-3])
    e = np.stack([-np.log1p(-0.999 * _smooth(rng, X, Y, Z)) for _ in range(5)], axis=-1)
    Yi = e / e.sum(axis=-1, keepdims=True)
    Yi = np.maximum(Yi, 1e-12)
    Yi = Yi / Yi.sum(axis=-1, keepdims=True)
    Xi = (Yi / W) / (Yi / W).sum(axis=-1, keepdims=True)
    MixW = (Xi * W).sum(axis=-1)
    # velocity: solenoidal (curl of a random vector potential) + compressive
    # (gradient of a random scalar potential) modes, unit RMS
    usol = np.zeros(X.shape + (3,))
    ucmp = np.zeros(X.shape + (3,))
    for _ in range(8):
        k = rng.integers(-3, 4, size=3)
        if not k.any():
            k[2] = 1
        a = rng.normal(size=3)
        ph = rng.uniform(0, 2 * math.pi)
        c = np.cos(k[0] * X + k[1] * Y + k[2] * Z + ph)[..., None]
        usol += np.cross(k, a) * c / float(k @ k)
        b = rng.normal()
        ph = rng.uniform(0, 2 * math.pi)
        c = np.cos(k[0] * X + k[1] * Y + k[2] * Z + ph)[..., None]
        ucmp += b * k * c / float(k @ k)
    uraw = usol / np.sqrt((usol ** 2).sum(-1).mean()) + ucmp / np.sqrt((ucmp ** 2).sum(-1).mean())
    uraw /= np.sqrt((uraw ** 2).sum(-1)).max()
    # frozen speed of sound estimate (gamma 1.4) for the Mach scaling
    a = np.sqrt(1.4 * 8.3144598 / MixW * Tk)
    M = mach[0] + (mach[1] - mach[0]) * _smooth(rng, X, Y, Z)
    vel = uraw * (M * a)[..., None]
    # nondimensionalise (src/Mixtures/MultiComponent.inl:438-487)
    XiRef = np.array(ref["XiRef"])
    XiRef = np.where(XiRef > 0, XiRef, 1e-60)
    MixWRef = float((XiRef * W).sum())
    rhoRef = ref["PRef"] * MixWRef / (8.3144598 * ref["TRef"])
    uRef = math.sqrt(ref["PRef"] / rhoRef)
    fl = Fluid((nx, ny, nz), 5)
    fl["pressure"] = Pa / ref["PRef"]
    fl["temperature"] = Tk / ref["TRef"]
    fl["MolarFracs"] = Xi
    fl["velocity"] = vel / uRef
    _uniform_metrics(fl, dx, dy, dz)
    fl.meta = dict(workload="air_box", eos=abi.HTR_EOS_AIRMIX, seed=seed, mix=dict(ref),
                   periodic=(True, True, True), bnum=(0, 0, 0), vorticityScale=1.0, cfl=0.8)
    return fl


def vortex2d(n=128, seed=0, shape=None, strength=None, mach=None, width=10.0):
    """2-D periodic isentropic vortex advected by a uniform stream (single-
    species gas, gamma 1.4, R 1, Pr 0.71, constant viscosity 1e-4): the
    vortex-advection case of the served mix (seeded strength in 0.1-5 and
    stream Mach number in 0.3-2 unless given).  nz = 1."""
    nx, ny = shape if shape is not None else (n, n)
    rng = np.random.Generator(np.random.PCG64(seed))
    beta = strength if strength is not None else rng.uniform(0.1, 5.0)
    M = mach if mach is not None else rng.uniform(0.3, 2.0)
    gamma = 1.4
    xc, dx = _centers(nx, width)
    yc, dy = _centers(ny, width)
    Y, X = np.meshgrid(yc, xc, indexing="ij")
    r2 = (X - 0.5 * width) ** 2 + (Y - 0.5 * width) ** 2
    f = np.exp(0.5 * (1.0 - r2))
    u = M + beta / (2 * math.pi) * -(Y - 0.5 * width) * f
    v = beta / (2 * math.pi) * (X - 0.5 * width) * f
    T = 1.0 - (gamma - 1.0) * beta * beta / (8.0 * gamma * math.pi ** 2) * f * f
    rho = T ** (1.0 / (gamma - 1.0))
    p = rho * T / gamma  # free stream: rho 1, a 1
    fl = Fluid((nx, ny, 1), 1)
    fl["pressure"] = p[None]
    fl["temperature"] = (p / rho)[None]
    fl["MolarFracs"] = 1.0
    fl["velocity"] = np.stack([u, v, np.zeros_like(u)], axis=-1)[None]
    _uniform_metrics(fl, dx, dy, 1.0)
    fl.meta = dict(workload="vortex2d", eos=abi.HTR_EOS_CONSTPROPMIX, seed=seed,
                   mix=dict(gasConstant=1.0, gamma=gamma, prandtl=0.71, viscosityModel=abi.HTR_VISC_CONSTANT,
                            p0=1e-4, p1=0.0, p2=0.0),
                   periodic=(True, True, True), bnum=(0, 0, 0), vorticityScale=1.0, cfl=0.8,
                   strength=beta, mach=M)
    return fl


def make_mixture_struct(lib, eos, params):
    """Build the reference-compatible mixture struct with `lib`'s builder."""
    import ctypes as C
    if eos == abi.HTR_EOS_CONSTPROPMIX:
        m = abi.htr_constpropmix_t()
        st = lib.htr_constpropmix_init(params["gasConstant"], params["gamma"], params["prandtl"],
                                       params["viscosityModel"], params["p0"], params["p1"],
                                       params["p2"], C.byref(m))
    else:
        m = abi.htr_airmix_t()
        xi = (C.c_double * 5)(*params["XiRef"])
        st = lib.htr_airmix_init(params["PRef"], params["TRef"], params["LRef"], xi, C.byref(m))
    abi.check(lib, st, "mixture init")
    return m


def derive_state(lib, fl, mixh, stream=None):
    """Properties then conserved variables from primitives over the whole grid."""
    import ctypes as C
    v = fl.view()
    r = fl.bounds()
    abi.check(lib, lib.htr_UpdatePropertiesFromPrimitive(C.byref(v), r, mixh, stream),
              "UpdatePropertiesFromPrimitive")
    abi.check(lib, lib.htr_UpdateConservedFromPrimitive(C.byref(v), r, mixh, stream),
              "UpdateConservedFromPrimitive")
