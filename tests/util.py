"""Shared helpers of the test suite: seeded states, CPU oracle runs, error metrics."""
import ctypes as C
import json
import os

import numpy as np

from htr_gb300 import abi, workloads  # noqa: F401  (re-exported for tests)

import oracle

# The parity bar, element by element: the reference's own regression rule
# (solverTests/testAll.py:22-26, |new - ref| <= max(tol |ref|, floor)) with
# tol = 1e-11, ten times tighter than the reference's 1e-10.
RHS_REL_TOL = 1e-11

# Absolute floor of each field: 1e-12 of the largest |ref| of the compared
# component over the grid (the reference's absolute floor of 1e-12 for its
# O(1) nondimensional fields, in units of the component's own scale).  It
# only matters where a value is itself at the level of cancellation: a
# momentum component crossing zero (the step adds fluxes of the component's
# full magnitude to it), a trace species, a right-hand side whose flux
# differences cancel.  Measured on a GB300, the worst such element needs
# 1.0e-13 of its component's largest value (momentum after a restart
# continuation), below this floor by ten.
FLOOR_REL = {}
FLOOR_REL_STATE = 1e-12


def floor_for(name):
    return FLOOR_REL.get(name, FLOOR_REL_STATE)


def rel_err(a, b):
    """Per-component max |a-b| / max |b| over all cells (last axis =
    components): the normwise figure, reported beside the pointwise bar."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.ndim == 3:
        a, b = a[..., None], b[..., None]
    d = np.abs(a - b).reshape(-1, a.shape[-1]).max(axis=0)
    s = np.abs(b).reshape(-1, b.shape[-1]).max(axis=0)
    return d / np.maximum(s, 1e-300)


def pointwise(got, want, name="", tol=RHS_REL_TOL, floor_rel=None):
    """Element-wise check |got - want| <= max(tol |want|, floor_c), floor_c =
    floor_rel * max |want| of component c.  Returns (ratio, info): ratio is
    the largest |got - want| / max(tol |want|, floor_c) (<= 1 passes), info
    describes the worst element, the normwise error and the floor that the
    comparison would need at `tol` (as a fraction of the component's max)."""
    a = np.asarray(got, dtype=np.float64)
    b = np.asarray(want, dtype=np.float64)
    if a.shape != b.shape:
        raise ValueError(f"{name}: shapes {a.shape} and {b.shape}")
    if a.ndim == 3:
        a, b = a[..., None], b[..., None]
    a2 = a.reshape(-1, a.shape[-1])
    b2 = b.reshape(-1, b.shape[-1])
    fr = floor_for(name) if floor_rel is None else floor_rel
    scale = np.abs(b2).max(axis=0)
    floor = np.maximum(fr * scale, 1e-300)
    d = np.abs(a2 - b2)
    bound = np.maximum(tol * np.abs(b2), floor[None, :])
    both_nan = np.isnan(a2) & np.isnan(b2)
    r = np.where(both_nan, 0.0, d / bound)
    r = np.where(np.isnan(r), np.inf, r)
    k = int(np.argmax(r))
    cell, comp = divmod(k, a2.shape[1])
    over = d > tol * np.abs(b2)
    need = np.where(over, d, 0.0).max(axis=0) / np.maximum(scale, 1e-300)
    info = dict(test=os.environ.get("PYTEST_CURRENT_TEST", ""), field=name, ratio=float(r.max()), cell=int(cell),
                comp=int(comp),
                got=float(a2[cell, comp]), want=float(b2[cell, comp]),
                normwise=float(rel_err(a, b).max()), floor_needed=float(need.max()), floor_rel=fr)
    log = os.environ.get("HTR_PARITY_LOG")
    if log:
        with open(log, "a") as f:
            f.write(json.dumps(info) + "\n")
    return info["ratio"], info


def log_record(**rec):
    """Append a record to the parity log named by HTR_PARITY_LOG, if set."""
    log = os.environ.get("HTR_PARITY_LOG")
    if log:
        rec.setdefault("test", os.environ.get("PYTEST_CURRENT_TEST", ""))
        with open(log, "a") as f:
            f.write(json.dumps(rec) + "\n")


def check(got, want, name="", tol=RHS_REL_TOL, floor_rel=None):
    """Assert the pointwise bar (see `pointwise`) for one field."""
    ratio, info = pointwise(got, want, name, tol, floor_rel)
    assert ratio <= 1.0, f"{name}: pointwise bar exceeded {info}"
    return info


def check_fields(got, want, names, tol=RHS_REL_TOL):
    """`check` for every field of `names` of two Fluid objects."""
    for n in names:
        check(got[n], want[n], n, tol)


# The reference's Newton solve for T from the internal energy
# (src/Mixtures/MultiComponent.inl:188-209) stops when the next correction
# |f / dfdT| falls below 1e-8 (nondimensional temperature) and returns the
# iterate without applying it: its T lies within about 1e-8 of the root.
NEWTON_TOL = 1e-8


def check_state_after_step(got, want, names, max_flip_fraction=5e-6):
    """The state after a step: the pointwise bar everywhere except in cells
    where the two temperatures differ beyond it -- cells where rounding put
    the last Newton correction of one side on the other side of the
    reference's tolerance, so one side stopped an iteration later.  Those
    cells must be rare (at most max_flip_fraction of the cells, and at least
    4 allowed), their temperatures within 2 x 1e-8 of each other, and every
    other field there within 20 x 1e-8 / T relative (the fields that follow
    T move in proportion).  Conserved is checked without exception.  On the
    256^3 air box 13 to 16 of the 16.8 M cells (about 1e-6) flipped across
    builds that differ only in rounding; the count bound leaves 5 times
    that, the temperature bound is the tolerance itself (measured: 1.00006e-8)."""
    T_got = np.asarray(got["temperature"], dtype=np.float64)
    T_want = np.asarray(want["temperature"], dtype=np.float64)
    scale = np.abs(T_want).max()
    bar = np.maximum(RHS_REL_TOL * np.abs(T_want), FLOOR_REL_STATE * scale)
    dT = np.abs(T_got - T_want)
    flip = dT > bar
    nflip = int(flip.sum())
    log_record(newton_flip_cells=nflip, cells=int(flip.size), max_dT=float(dT.max()))
    assert nflip <= max(4, max_flip_fraction * flip.size), f"{nflip} cells with temperatures beyond the bar"
    assert float(dT.max()) <= 2 * NEWTON_TOL, f"temperature difference {dT.max():.3e} beyond 2 x the Newton tolerance"
    rel_flip = 20 * NEWTON_TOL / np.maximum(np.abs(T_want), 1e-300)
    for n in names:
        a = np.asarray(got[n], dtype=np.float64)
        b = np.asarray(want[n], dtype=np.float64)
        if n == "Conserved" or nflip == 0:
            check(a, b, n)
            continue
        keep = ~flip
        ka, kb = (a[keep], b[keep]) if a.ndim == 3 else (a[keep, :], b[keep, :])
        ratio, info = pointwise(ka.reshape(-1, 1 if a.ndim == 3 else a.shape[-1]),
                                kb.reshape(-1, 1 if a.ndim == 3 else a.shape[-1]), n)
        assert ratio <= 1.0, f"{n}: pointwise bar exceeded outside the Newton-tolerance cells {info}"
        fa, fb = (a[flip], b[flip]) if a.ndim == 3 else (a[flip, :], b[flip, :])
        lim = rel_flip[flip] if a.ndim == 3 else rel_flip[flip][:, None]
        assert np.all(np.abs(fa - fb) <= lim * np.abs(fb) + FLOOR_REL_STATE * np.abs(b).max()), n


def ulp_spread(run, fl, fields, perturb=("Conserved", "Conserved_t")):
    """The spread of an algorithm's own results under rounding-level changes
    of its inputs: `run` (an oracle computation, in place on a host Fluid) on
    `fl` and on copies with each field of `perturb` moved by one ulp
    (np.nextafter towards +inf).  Returns (the unperturbed result, {field:
    per-component largest |change|})."""
    base = fl.copy()
    run(base)
    spread = {}
    for name in perturb:
        f = fl.copy()
        f[name] = np.nextafter(fl[name], np.inf)
        run(f)
        for out in fields:
            a, b = np.asarray(f[out], dtype=np.float64), np.asarray(base[out], dtype=np.float64)
            if a.ndim == 3:
                a, b = a[..., None], b[..., None]
            d = np.abs(a - b).reshape(-1, a.shape[-1]).max(axis=0)
            spread[out] = np.maximum(spread.get(out, 0.0), d)
    return base, spread


def check_within_spread(got, want, name, spread, k=10.0, tol=RHS_REL_TOL):
    """`check` with the absolute floor raised, per component, to k times the
    reference algorithm's own one-ulp spread (ulp_spread): for adaptive
    solvers whose step sequence, and so whose result at the level of their
    error tolerance, changes with the rounding of their inputs.  Logs the
    ratio of the largest difference to the spread."""
    a = np.asarray(got, dtype=np.float64)
    b = np.asarray(want, dtype=np.float64)
    if a.ndim == 3:
        a, b = a[..., None], b[..., None]
    a2, b2 = a.reshape(-1, a.shape[-1]), b.reshape(-1, b.shape[-1])
    scale = np.abs(b2).max(axis=0)
    floor = np.maximum(np.maximum(FLOOR_REL_STATE * scale, k * np.asarray(spread)), 1e-300)
    d = np.abs(a2 - b2)
    r = d / np.maximum(tol * np.abs(b2), floor[None, :])
    dmax = d.max(axis=0)
    info = dict(field=name, ratio=float(r.max()), max_abs_diff=float(dmax.max()),
                spread=[float(x) for x in np.atleast_1d(spread)],
                diff_over_spread=float((dmax / np.maximum(np.asarray(spread), 1e-300)).max()), k=k)
    log_record(spread_check=info)
    assert r.max() <= 1.0, f"{name}: beyond {k} x the reference's own one-ulp spread {info}"
    return info


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


def make_air_state(lib, shape, seed=0, T=(300.0, 3000.0), dissociation=1e-2, mach=(0.3, 1.5)):
    """Five-species air near the composition of air (molar fractions N2 0.78,
    O2 0.21, NO, N and O `dissociation`, 1/2, 1/2 of it, varied smoothly by
    +-10 %), T and velocities from the seeded air-box generator, p 0.5-2 bar.

    The reference's implicit Rosenbrock solver (src/Utils/math_utils.hpp:196-441)
    returns NaN for many cells of the air-box workload's Dirichlet-random
    compositions (atoms at low temperature) once the chemical step exceeds
    about 1e-6: its first trial step takes the whole interval, a non-finite
    error estimate makes the step size NaN, and nothing resets it.  Its
    implicit-chemistry tests therefore run on this composition, where the
    solver converges over whole CFL steps."""
    fl = workloads.air_box(shape=shape, seed=seed, T=T, mach=mach, p_bar=(0.5, 2.0))
    X = fl["MolarFracs"].copy()
    base = np.array([0.78, 0.21, dissociation, dissociation / 2, dissociation / 2])
    X = base * (1 + 0.1 * (X - X.mean(axis=(0, 1, 2))))
    fl["MolarFracs"] = X / X.sum(axis=-1, keepdims=True)
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
