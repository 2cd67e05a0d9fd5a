"""Generates tests/golden/*.npz from the reference's own CPU task code.

Run where the reference sources are available (the reference oracle is built
by oracle/build.py into oracle/_ref/):

    python tests/golden/make_golden.py

Each fixture holds one seeded periodic state (every field of the view) and
the outputs of every RHS-path task computed by the compiled reference on
that state.  The test suite replays the same tasks with the CPU port and the
CUDA library and compares.
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()

import oracle  # noqa: E402
from tests import util  # noqa: E402

CASES = {"tg": dict(shape=(8, 6, 5), seed=21, eos=1), "air": dict(shape=(6, 5, 4), seed=22, eos=2)}
EULER = ["Hybrid", "TENO", "TENOA", "TENOLAD", "SkewSymmetric"]
RK = (0.75, 0.25)
DT_FLUX = 2e-3


def fields_of(fl):
    return {f"in/{k}": np.array(v) for k, v in fl.arrays.items()}


def run_tasks(lib, fl, h):
    """Apply every task to copies of `fl`; returns {key: array}."""
    out = {}
    rk = (C.c_double * 2)(*RK)
    for scheme in EULER:
        for d in "XYZ":
            f = fl.copy()
            f["Conserved_t"] = 0.0
            v = f.view()
            if scheme == "SkewSymmetric":
                util.call(lib, f"htr_UpdateUsingSkewSymmetricEulerFlux{d}", C.byref(v), f.interior(),
                          f.bounds(), h, None)
            else:
                util.call(lib, f"htr_UpdateUsing{scheme}EulerFlux{d}", C.byref(v), f.interior(), f.bounds(),
                          rk, DT_FLUX, h, None)
            out[f"out/euler_{scheme}_{d}"] = f["Conserved_t"].copy()
    for d in "XYZ":
        f = fl.copy()
        f["Conserved_t"] = 0.0
        v = f.view()
        util.call(lib, f"htr_UpdateUsingDiffusionFlux{d}", C.byref(v), f.interior(), f.bounds(), h, None)
        out[f"out/diffusion_{d}"] = f["Conserved_t"].copy()
    f = fl.copy()
    f["Conserved_t"] = 0.0
    v = f.view()
    util.call(lib, "htr_AddChemistrySources", C.byref(v), f.interior(), h, None)
    out["out/chem"] = f["Conserved_t"].copy()
    # properties from primitives
    f = fl.copy()
    for k in ("rho", "mu", "lam", "Di", "SoS", "MassFracs"):
        f[k] = 0.0
    v = f.view()
    util.call(lib, "htr_UpdatePropertiesFromPrimitive", C.byref(v), f.bounds(), h, None)
    for k in ("rho", "mu", "lam", "Di", "SoS", "MassFracs"):
        out[f"out/props_{k}"] = f[k].copy()
    # primitives from conserved with a perturbed temperature guess
    f = fl.copy()
    f["temperature"] = fl["temperature"] * 1.01
    v = f.view()
    util.call(lib, "htr_UpdatePrimitiveFromConserved", C.byref(v), f.bounds(), h, None)
    for k in ("temperature", "pressure", "MolarFracs", "velocity"):
        out[f"out/prim_{k}"] = f[k].copy()
    # spectral radius
    f = fl.copy()
    v = f.view()
    r = C.c_double()
    util.call(lib, "htr_CalculateMaxSpectralRadius", C.byref(v), f.interior(), h, C.byref(r), None)
    out["out/spectral_radius"] = np.array(r.value)
    return out


def make(kind):
    cfg = CASES[kind]
    ref = oracle.ref_lib(cfg["eos"])
    if ref is None:
        raise SystemExit("reference oracle not built (needs the reference sources)")
    fl, h, m = util.make_state(ref, kind, cfg["shape"], seed=cfg["seed"])
    rng = np.random.default_rng(cfg["seed"])
    fl["Conserved_old"] = fl["Conserved"] * (1 + 1e-3 * rng.standard_normal(fl["Conserved"].shape))
    oracle.update_sensors(ref, fl, h, 1.0)
    data = fields_of(fl)
    data.update(run_tasks(ref, fl, h))
    # one SSP-RK3 step from this state
    f = fl.copy()
    chem = kind == "air"
    dt = 1e-9 if chem else 0.05
    oracle.step(ref, f, h, dt=dt, chemistry=chem)
    for k in ("Conserved", "temperature", "pressure", "shockSensorX", "shockSensorY", "shockSensorZ"):
        data[f"out/step_{k}"] = f[k].copy()
    # implicit chemistry over 1e-8
    if chem:
        f = fl.copy()
        f["Conserved_t"] = 0.0
        v = f.view()
        st = C.c_int(0)
        util.call(ref, "htr_UpdateChemistry", C.byref(v), f.interior(), 1e-8, h, C.byref(st), None)
        for k in ("Conserved", "temperature"):
            data[f"out/implicit_{k}"] = f[k].copy()
    meta = dict(kind=kind, shape=cfg["shape"], seed=cfg["seed"], eos=cfg["eos"], rk=RK, dt_flux=DT_FLUX,
                step_dt=dt, mix=fl.meta["mix"])
    data["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, f"{kind}.npz")
    np.savez_compressed(path, **data)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    for k in CASES:
        make(k)
