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


def _measure_in_this_process():
    """Free device memory around the first two static steps of a process
    that has loaded its mixture (htr_load_mixture is the set-up point that
    loads the scratch's module).  One step through the caller-workspace
    entry point runs first: under CUDA's lazy module loading the first launch
    of each kernel in a process loads that kernel's module, whichever entry
    point launches it."""
    import torch
    shape, dt, chem = CASES["air"]
    fl, h, m = util.make_state(oracle.port_lib(), "air", shape, seed=4)
    dev = fl.to_device("cuda")
    gh = runtime.load_mixture(fl.meta["eos"], m)
    warm = dev.copy()
    ws = runtime.Workspace()
    runtime.rk3_step(warm, gh, dt=dt, chemistry=chem, fused=True, workspace=ws)
    torch.cuda.synchronize()
    before_torch = torch.cuda.memory_allocated()
    free_before, _ = torch.cuda.mem_get_info()
    for k in range(2):
        abi.check(runtime.lib(), _static_step(dev, gh, dt, chem), f"htr_rk3_step_static call {k}")
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    return before_torch, torch.cuda.memory_allocated(), free_before, free_after


def test_static_scratch_allocates_nothing():
    """In a fresh process (where the scratch's module is not yet loaded) and
    in this one: once the mixture is loaded, the first static steps change
    neither torch's allocations nor the device's free memory."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, json; sys.path.insert(0, %r); import __graft_entry__ as g; g.load_package(); "
            "from tests import test_zz_no_alloc as t; print(json.dumps(t._measure_in_this_process()))" % root)
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    fresh = json.loads(r.stdout.strip().splitlines()[-1])
    for bt, at, fb, fa in (fresh, _measure_in_this_process()):
        assert at == bt
        assert fa == fb


def test_static_scratch_rejects_oversize():
    fl = util.workloads.air_box(48, seed=5)
    m = util.workloads.make_mixture_struct(oracle.port_lib(), fl.meta["eos"], fl.meta["mix"])
    gh = runtime.load_mixture(fl.meta["eos"], m)
    dev = fl.to_device("cuda")
    assert runtime.workspace_bytes(dev, gh) > runtime.lib().htr_rk3_static_scratch_bytes()
    assert _static_step(dev, gh, 1e-9, True) == abi.HTR_ERR_UNSUPPORTED
