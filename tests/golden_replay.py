"""Replays the golden fixtures (tests/golden/*.npz, made by the compiled
reference) through any library that exports the C ABI."""
import ctypes as C
import json
import os

import numpy as np

from htr_gb300 import abi, workloads
from htr_gb300.fluid import Fluid

from tests import util

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EULER = ["Hybrid", "TENO", "TENOA", "TENOLAD", "SkewSymmetric"]


def load(kind):
    z = np.load(os.path.join(GOLDEN, f"{kind}.npz"))
    meta = json.loads(str(z["meta"]))
    nspec = 1 if meta["eos"] == abi.HTR_EOS_CONSTPROPMIX else 5
    fl = Fluid(meta["shape"], nspec)
    for k in z.files:
        if k.startswith("in/"):
            fl[k[3:]] = z[k]
    fl.meta = dict(eos=meta["eos"], mix=meta["mix"])
    return fl, {k[4:]: z[k] for k in z.files if k.startswith("out/")}, meta


def replay(lib, kind, load_mix, device=None, sync=lambda: None, stream=None):
    """Run every task of the fixture with `lib`; returns {key: array} like the fixture."""
    base, _, meta = load(kind)
    struct = workloads.make_mixture_struct(lib, meta["eos"], meta["mix"])
    h = load_mix(meta["eos"], struct)
    rk = (C.c_double * 2)(*meta["rk"])
    out = {}

    def fresh(**zero):
        f = base.copy()
        for k, val in zero.items():
            f[k] = val
        return f.to_device(device) if device else f

    def back(f, keys):
        sync()
        h_ = f.to_host(keys) if device else f
        return {k: np.array(h_[k]) for k in keys}

    for scheme in EULER:
        for d in "XYZ":
            f = fresh(Conserved_t=0.0)
            v = f.view()
            if scheme == "SkewSymmetric":
                util.call(lib, f"htr_UpdateUsingSkewSymmetricEulerFlux{d}", C.byref(v), f.interior(), f.bounds(),
                          h, stream)
            else:
                util.call(lib, f"htr_UpdateUsing{scheme}EulerFlux{d}", C.byref(v), f.interior(), f.bounds(), rk,
                          meta["dt_flux"], h, stream)
            out[f"euler_{scheme}_{d}"] = back(f, ["Conserved_t"])["Conserved_t"]
    for d in "XYZ":
        f = fresh(Conserved_t=0.0)
        v = f.view()
        util.call(lib, f"htr_UpdateUsingDiffusionFlux{d}", C.byref(v), f.interior(), f.bounds(), h, stream)
        out[f"diffusion_{d}"] = back(f, ["Conserved_t"])["Conserved_t"]
    f = fresh(Conserved_t=0.0)
    v = f.view()
    util.call(lib, "htr_AddChemistrySources", C.byref(v), f.interior(), h, stream)
    out["chem"] = back(f, ["Conserved_t"])["Conserved_t"]
    props = ("rho", "mu", "lam", "Di", "SoS", "MassFracs")
    f = fresh(**{k: 0.0 for k in props})
    v = f.view()
    util.call(lib, "htr_UpdatePropertiesFromPrimitive", C.byref(v), f.bounds(), h, stream)
    for k, a in back(f, props).items():
        out[f"props_{k}"] = a
    f = fresh(temperature=base["temperature"] * 1.01)
    v = f.view()
    util.call(lib, "htr_UpdatePrimitiveFromConserved", C.byref(v), f.bounds(), h, stream)
    for k, a in back(f, ("temperature", "pressure", "MolarFracs", "velocity")).items():
        out[f"prim_{k}"] = a
    # sensors from the fixture's pre-sensor state
    f = fresh(DucrosSensor=0.0, shockSensorX=False, shockSensorY=False, shockSensorZ=False)
    v = f.view()
    r = f.bounds()
    util.call(lib, "htr_UpdateDucrosSensor", C.byref(v), r, r, 1.0, stream)
    for d in "XYZ":
        util.call(lib, f"htr_UpdateShockSensor{d}", C.byref(v), r, r, h, stream)
    for k, a in back(f, ("DucrosSensor", "shockSensorX", "shockSensorY", "shockSensorZ")).items():
        out[f"sensor_{k}"] = a
    return out, base, h, meta
