"""htr_rk3_step_static: the fused step on the library's fixed device scratch.

Two consecutive steps must equal, bit for bit, the same two steps of
htr_rk3_step_ws on a caller workspace; the calls must not change the device
memory in use; a grid whose workspace exceeds the scratch is rejected before
any launch.  (Kept in the last-collected file of the suite.)"""
import ctypes as C

import numpy as np
import pytest

from htr_gb300 import abi, runtime

import oracle
from tests import util

pytestmark = pytest.mark.gpu

CASES = {"tg": ((16, 12, 10), 0.05, False), "air": ((12, 10, 8), 1e-9, True)}


def _static_step(dev, gh, dt, chem):
    l = runtime.lib()
    p = runtime.htr_step_params(runtime.SCHEMES["Hybrid"], 1.0, 0.0, dt, 1 if chem else 0)
    v = dev.view()
    used = C.c_double(0.0)
    return l.htr_rk3_step_static(C.byref(v), dev.interior(), dev.bounds(), C.byref(p), gh, C.byref(used),
                                 None, runtime.stream_handle())


@pytest.mark.parametrize("kind", sorted(CASES))
def test_static_scratch_equals_workspace_path(kind):
    import torch
    shape, dt, chem = CASES[kind]
    fl, h, m = util.make_state(oracle.port_lib(), kind, shape, seed=3)
    gh = runtime.load_mixture(fl.meta["eos"], m)
    a = fl.to_device("cuda")
    b = fl.to_device("cuda")
    assert runtime.workspace_bytes(a, gh) <= runtime.lib().htr_rk3_static_scratch_bytes()
    for _ in range(2):
        runtime.rk3_step(a, gh, dt=dt, chemistry=chem, fused=True)
        abi.check(runtime.lib(), _static_step(b, gh, dt, chem), "htr_rk3_step_static")
        torch.cuda.synchronize()
        ha, hb = a.to_host(), b.to_host()
        for name in ha.arrays:
            assert np.array_equal(ha[name], hb[name], equal_nan=True), name


def test_static_scratch_allocates_nothing():
    import torch
    shape, dt, chem = CASES["air"]
    fl, h, m = util.make_state(oracle.port_lib(), "air", shape, seed=4)
    gh = runtime.load_mixture(fl.meta["eos"], m)
    dev = fl.to_device("cuda")
    abi.check(runtime.lib(), _static_step(dev, gh, dt, chem), "first call")
    torch.cuda.synchronize()
    before_torch = torch.cuda.memory_allocated()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        abi.check(runtime.lib(), _static_step(dev, gh, dt, chem), "htr_rk3_step_static")
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert torch.cuda.memory_allocated() == before_torch
    assert free_after == free_before


def test_static_scratch_rejects_oversize():
    fl = util.workloads.air_box(48, seed=5)
    m = util.workloads.make_mixture_struct(oracle.port_lib(), fl.meta["eos"], fl.meta["mix"])
    gh = runtime.load_mixture(fl.meta["eos"], m)
    dev = fl.to_device("cuda")
    assert runtime.workspace_bytes(dev, gh) > runtime.lib().htr_rk3_static_scratch_bytes()
    assert _static_step(dev, gh, 1e-9, True) == abi.HTR_ERR_UNSUPPORTED
