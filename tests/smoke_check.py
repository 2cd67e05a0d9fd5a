"""Small invocations of the hot path on cuda:0 checked against the CPU oracle:
one hybrid RHS evaluation of a periodic box, and one fused SSP-RK3 step of a
boundary-layer grid (metrics on the device, TENO-LAD, NSCBC and wall rules)."""
import ctypes as C

import numpy as np


def run():
    import torch

    from htr_gb300 import runtime

    import oracle
    from tests import util

    port = oracle.port_lib()
    fl, h, m = util.make_state(port, "tg", (12, 10, 8), seed=1)
    host = fl.copy()
    oracle.update_sensors(port, host, h, 1.0)
    oracle.update_derivatives(port, host, h, 1, 0.01, "Hybrid", chemistry=False)
    gh = runtime.load_mixture(fl.meta["eos"], m)
    dev = fl.to_device("cuda:0")
    gpu = runtime.lib()
    v = dev.view()
    r = dev.bounds()
    s = runtime.stream_handle()
    util.call(gpu, "htr_UpdateDucrosSensor", C.byref(v), r, r, 1.0, s)
    for d in "XYZ":
        util.call(gpu, f"htr_UpdateShockSensor{d}", C.byref(v), r, r, gh, s)
    util.call(gpu, "htr_InitializeTimeDerivatives", C.byref(v), r, 0, gh, s)
    rk = (C.c_double * 2)(1.0, 0.0)
    for d in "ZYX":
        util.call(gpu, f"htr_UpdateUsingHybridEulerFlux{d}", C.byref(v), r, r, rk, 0.01, gh, s)
    for d in "ZYX":
        util.call(gpu, f"htr_UpdateUsingDiffusionFlux{d}", C.byref(v), r, r, gh, s)
    torch.cuda.synchronize()
    out = dev.to_host()
    for d in "XYZ":
        assert np.array_equal(out[f"shockSensor{d}"], host[f"shockSensor{d}"]), d
    err = util.check(out["Conserved_t"], host["Conserved_t"], "Conserved_t")["ratio"]

    # boundary layer: the device metrics equal the port's; one fused step
    # equals the oracle's step within the RHS tolerance
    from htr_gb300 import wall, workloads
    bl = wall.boundary_layer(num=(12, 8, 4), seed=2)
    g = bl.meta["grid"]
    g.fill(bl, port)
    mb = workloads.make_mixture_struct(port, bl.meta["eos"], bl.meta["mix"])
    hb = oracle.load_mixture(port, bl.meta["eos"], mb)
    workloads.derive_state(port, bl, hb)
    dev = bl.to_device("cuda:0")
    g.fill(dev, gpu)
    torch.cuda.synchronize()
    met = dev.to_host()
    for name in ("dcsi_e", "deta_e", "deta_d", "deta_s"):
        assert np.array_equal(met[name], bl[name]), name
    bc = bl.meta["bc"]
    dt = wall.BoundaryRun(port, bl, hb, bc).spectral_dt(0.8)
    oracle.boundary_layer_step(port, bl, hb, dt, bc["xNeg"][1]["P"], bc["xPos"][1]["P"],
                               (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"]))
    wall.FusedBoundaryRun(dev, runtime.load_mixture(bl.meta["eos"], mb), bc).step(dt)
    torch.cuda.synchronize()
    err2 = util.check(dev.to_host()["Conserved"], bl["Conserved"], "Conserved")["ratio"]
    print(f"smoke ok: pointwise error / bound {err:.3e} (hybrid RHS), {err2:.3e} (boundary-layer step)")


if __name__ == "__main__":
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__
    __graft_entry__.load_package()
    run()
