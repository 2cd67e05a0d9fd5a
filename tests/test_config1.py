"""The plain small configuration: a 32^3 periodic Taylor-Green box of a
calorically perfect gas (gamma 1.4, Pr 0.71, power-law viscosity) with +-1 %
seeded perturbations, hybrid scheme with the Ducros / TENO-A sensor, viscous
diffusion, one SSP-RK3 step at CFL 0.8.

CPU: the port's step equals the reference's compiled tasks' step bit for bit
(where the reference sources exist).  GPU (-m gpu): the task composition and
the fused pipeline against the port's step: sensors bit for bit, every state
field within the pointwise bar of util.check.
"""
import numpy as np
import pytest

from htr_gb300 import runtime, workloads

import oracle
from tests import util

FIELDS = ("Conserved", "temperature", "pressure", "velocity", "rho", "mu", "lam", "SoS")


def _tg(lib):
    fl = workloads.taylor_green(32, seed=0)
    m = workloads.make_mixture_struct(lib, fl.meta["eos"], fl.meta["mix"])
    h = oracle.load_mixture(lib, fl.meta["eos"], m)
    workloads.derive_state(lib, fl, h)
    return fl, h, m


def test_config1_port_matches_reference():
    ref = oracle.ref_lib(1)
    if ref is None:
        pytest.skip("reference CPU build not present on this machine")
    port = oracle.port_lib()
    a, ha, _ = _tg(port)
    b, hb, _ = _tg(ref)
    dta = oracle.step(port, a, ha, scheme="Hybrid", cfl=0.8, chemistry=False)
    dtb = oracle.step(ref, b, hb, scheme="Hybrid", cfl=0.8, chemistry=False)
    assert dta == dtb
    for name in a.arrays:
        assert np.array_equal(a[name], b[name]), name


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [False, True])
def test_config1_gpu_step(fused):
    import torch
    port = oracle.port_lib()
    host, h, m = _tg(port)
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    dt = oracle.step(port, host, h, scheme="Hybrid", cfl=0.8, chemistry=False)
    runtime.rk3_step(dev, gh, scheme="Hybrid", dt=dt, chemistry=False, fused=fused)
    torch.cuda.synchronize()
    out = dev.to_host()
    for d in "XYZ":
        assert np.array_equal(out[f"shockSensor{d}"], host[f"shockSensor{d}"]), d
    util.check_fields(out, host, FIELDS)
