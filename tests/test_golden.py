"""Golden vectors made by the compiled reference (tests/golden/make_golden.py).

CPU: the oracle port replays every task of both fixtures; on x86-64 (the
host the fixtures were made on) the results are bit-identical, elsewhere the
host libm may differ in the last bit of exp/log/pow, so 1e-13 relative.
GPU: the CUDA library replays them; sensors bit-exact, single-species Euler
fluxes bit-exact, the rest within the pointwise bar of util.check.
"""
import platform

import numpy as np
import pytest

import oracle
from tests import golden_replay, util

KINDS = ["tg", "air"]
EXACT_HOST = platform.machine() in ("x86_64", "AMD64")


def _cmp(got, want, key, exact, tol):
    if want.dtype == np.bool_:
        assert np.array_equal(got, want), f"{key}: {(got != want).sum()} flags differ"
    elif exact:
        assert np.array_equal(got, want), util.pointwise(got, want, _field(key))[1]
    else:
        ratio, info = util.pointwise(got, want, _field(key), tol)
        assert ratio <= 1.0, (key, info)


def _field(key):
    """Field name of a fixture key (for its pointwise floor)."""
    if key.startswith(("euler_", "diffusion_", "chem")):
        return "Conserved_t"
    return key.split("_", 1)[1] if "_" in key else key


@pytest.mark.parametrize("kind", KINDS)
def test_fixture_pins_port(kind):
    port = oracle.port_lib()
    got, base, _, _ = golden_replay.replay(port, kind, lambda eos, s: oracle.load_mixture(port, eos, s))
    _, want, _ = golden_replay.load(kind)
    for key, a in got.items():
        wkey = key.replace("sensor_", "") if key.startswith("sensor_") else key
        ref = want.get(wkey, base[wkey] if wkey in base.arrays else None)
        _cmp(a, ref, key, EXACT_HOST, 1e-13)


@pytest.mark.parametrize("kind", KINDS)
def test_fixture_step_and_implicit_chemistry(kind):
    import ctypes as C
    port = oracle.port_lib()
    fl, want, meta = golden_replay.load(kind)
    s = util.workloads.make_mixture_struct(port, meta["eos"], meta["mix"])
    h = oracle.load_mixture(port, meta["eos"], s)
    f = fl.copy()
    oracle.step(port, f, h, dt=meta["step_dt"], chemistry=(kind == "air"))
    for k in ("Conserved", "temperature", "pressure", "shockSensorX", "shockSensorY", "shockSensorZ"):
        _cmp(f[k], want[f"step_{k}"], k, EXACT_HOST, 1e-12)
    if kind == "air":
        f = fl.copy()
        f["Conserved_t"] = 0.0
        v = f.view()
        st = C.c_int(0)
        util.call(port, "htr_UpdateChemistry", C.byref(v), f.interior(), 1e-8, h, C.byref(st), None)
        for k in ("Conserved", "temperature"):
            _cmp(f[k], want[f"implicit_{k}"], k, EXACT_HOST, 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", KINDS)
def test_fixture_pins_gpu(kind):
    import torch

    from htr_gb300 import runtime
    gpu = runtime.lib()
    got, base, _, _ = golden_replay.replay(gpu, kind, runtime.load_mixture, device="cuda",
                                           sync=torch.cuda.synchronize, stream=runtime.stream_handle())
    _, want, _ = golden_replay.load(kind)
    for key, a in got.items():
        wkey = key.replace("sensor_", "") if key.startswith("sensor_") else key
        ref = want.get(wkey, base[wkey] if wkey in base.arrays else None)
        exact = key.startswith("sensor_") or (kind == "tg" and key.startswith("euler_"))
        _cmp(a, ref, key, exact, util.RHS_REL_TOL)
