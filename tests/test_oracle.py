"""The CPU oracle port against the reference's own CPU task code.

The reference is compiled from its sources (oracle/ref/Makefile) only where
those sources exist; elsewhere these tests skip and the port is pinned by the
golden vectors of tests/golden/ instead (test_golden.py).  Here every task
of the RHS path and one full SSP-RK3 step must agree bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests import util

CASES = {"tg": (12, 10, 8), "air": (10, 8, 6)}


def _ref(eos):
    lib = oracle.ref_lib(eos)
    if lib is None:
        pytest.skip("reference CPU build not present on this machine")
    return lib


def _pair(kind):
    eos = 1 if kind == "tg" else 2
    ref = _ref(eos)
    port = oracle.port_lib()
    fr, hr, mr = util.make_state(ref, kind, CASES[kind], seed=7)
    fp, hp, mp = util.make_state(port, kind, CASES[kind], seed=7)
    return ref, port, (fr, hr, mr), (fp, hp, mp)


def _eq(a, b, name):
    assert np.array_equal(a[name], b[name]), f"{name}: max rel {util.rel_err(a[name], b[name]).max()}"


@pytest.mark.parametrize("kind", ["tg", "air"])
def test_mixture_builders_match(kind):
    ref, port, (fr, hr, mr), (fp, hp, mp) = _pair(kind)
    # compare field by field (padding and members the reference leaves
    # unset for the chosen viscosity law are not compared)
    skip = {".constantVisc", ".sutherlandSRef", ".sutherlandTempRef", ".sutherlandViscRef"}
    diffs = [d for d in util.struct_diff(mp, mr) if not (kind == "tg" and d[0] in skip)]
    assert not diffs, diffs[:5]


@pytest.mark.parametrize("kind", ["tg", "air"])
def test_state_derivation(kind):
    ref, port, (fr, hr, mr), (fp, hp, mp) = _pair(kind)
    for name in ("rho", "mu", "lam", "Di", "SoS", "MassFracs", "Conserved"):
        _eq(fp, fr, name)


@pytest.mark.parametrize("kind", ["tg", "air"])
def test_sensors(kind):
    ref, port, (fr, hr, mr), (fp, hp, mp) = _pair(kind)
    oracle.update_sensors(ref, fr, hr, 1.0)
    oracle.update_sensors(port, fp, hp, 1.0)
    for name in ("DucrosSensor", "shockSensorX", "shockSensorY", "shockSensorZ"):
        _eq(fp, fr, name)


@pytest.mark.parametrize("kind", ["tg", "air"])
@pytest.mark.parametrize("task", ["Hybrid", "TENO", "TENOA", "TENOLAD", "SkewSymmetric", "Diffusion",
                                  "Chem"])
def test_task(kind, task):
    ref, port, (fr, hr, mr), (fp, hp, mp) = _pair(kind)
    oracle.update_sensors(ref, fr, hr, 1.0)
    oracle.update_sensors(port, fp, hp, 1.0)
    rk = (C.c_double * 2)(0.75, 0.25)
    for d in ("X", "Y", "Z") if task != "Chem" else ("",):
        for lib, fl, h in ((ref, fr, hr), (port, fp, hp)):
            fl["Conserved_t"] = 0.0
            fl["Conserved_old"] = fl["Conserved"] * 1.0001
            v = fl.view()
            if task == "Chem":
                util.call(lib, "htr_AddChemistrySources", C.byref(v), fl.interior(), h, None)
            elif task == "SkewSymmetric":
                util.call(lib, f"htr_UpdateUsingSkewSymmetricEulerFlux{d}", C.byref(v), fl.interior(),
                          fl.bounds(), h, None)
            elif task == "Diffusion":
                util.call(lib, f"htr_UpdateUsingDiffusionFlux{d}", C.byref(v), fl.interior(), fl.bounds(), h,
                          None)
            else:
                util.call(lib, f"htr_UpdateUsing{task}EulerFlux{d}", C.byref(v), fl.interior(), fl.bounds(),
                          rk, 1e-3, h, None)
        _eq(fp, fr, "Conserved_t")


@pytest.mark.parametrize("kind", ["tg", "air"])
def test_rk3_step(kind):
    ref, port, (fr, hr, mr), (fp, hp, mp) = _pair(kind)
    dtr = oracle.spectral_dt(ref, fr, hr, 0.8)
    dtp = oracle.spectral_dt(port, fp, hp, 0.8)
    assert dtr == dtp
    dt = 1e-9 if kind == "air" else dtr
    oracle.step(ref, fr, hr, dt=dt, chemistry=(kind == "air"))
    oracle.step(port, fp, hp, dt=dt, chemistry=(kind == "air"))
    for name in ("Conserved", "temperature", "pressure", "Conserved_t", "rho", "mu", "Di",
                 "shockSensorX", "shockSensorY", "shockSensorZ"):
        _eq(fp, fr, name)


def test_implicit_chemistry():
    ref, port, (fr, hr, mr), (fp, hp, mp) = _pair("air")
    for lib, fl, h in ((ref, fr, hr), (port, fp, hp)):
        fl["Conserved_t"] = 0.0
        v = fl.view()
        st = C.c_int(0)
        util.call(lib, "htr_UpdateChemistry", C.byref(v), fl.interior(), 1e-8, h, C.byref(st), None)
    for name in ("Conserved", "temperature", "Conserved_t_old"):
        _eq(fp, fr, name)


@pytest.mark.parametrize("scheme", ["Hybrid", "TENOLAD"])
def test_implicit_chemistry_step(scheme):
    """One SSP-RK3 step through the implicit-chemistry branch of the driver
    (src/prometeo.rg:1360-1398, src/prometeo_rk.rg:59-112) on near-air
    compositions at 300-3000 K, at a step size far above the explicit
    chemical limit: the port equals the reference's compiled tasks bit for
    bit."""
    ref = _ref(2)
    port = oracle.port_lib()
    fr, hr, _ = util.make_air_state(ref, CASES["air"], seed=7)
    fp, hp, _ = util.make_air_state(port, CASES["air"], seed=7)
    dt = oracle.spectral_dt(ref, fr, hr, 0.08)
    start = fp["Conserved"].copy()
    oracle.step(ref, fr, hr, scheme=scheme, dt=dt, implicit=True)
    oracle.step(port, fp, hp, scheme=scheme, dt=dt, implicit=True)
    for name in ("Conserved", "temperature", "pressure", "Conserved_t", "Conserved_t_old", "rho", "mu", "Di",
                 "MolarFracs"):
        _eq(fp, fr, name)
    assert np.all(np.isfinite(fp["Conserved"])) and not np.array_equal(fp["Conserved"], start)
