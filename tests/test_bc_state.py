"""Boundary-condition state updates of the boundary points.

CPU: the oracle port against the reference's compiled SetNSCBC_InflowBCTask
and SetNSCBC_OutflowBCTask (bit for bit, where the reference sources exist),
and the Regent-defined wall and NSCBC time-derivative updates against their
definitions written in numpy (src/prometeo_bc.rg:1207-1263, 1794-1810).
GPU (-m gpu): the CUDA library against the port (bit for bit for the copies
and the time derivatives; <= 1e-11 for the pressure and the outflow
primitive recovery).
"""
import ctypes as C

import numpy as np
import pytest

from htr_gb300 import abi, runtime

import oracle
from tests import util


def _state(lib, kind, seed=9, shape=(9, 8, 7)):
    fl, h, m = util.make_state(lib, kind, shape, seed=seed)
    rng = np.random.default_rng(seed)
    ns = fl.nspec
    X = rng.uniform(0.1, 1.0, size=fl["MolarFracs_profile"].shape)
    fl["MolarFracs_profile"] = X / X.sum(axis=-1, keepdims=True) if ns > 1 else 1.0
    fl["temperature_profile"] = fl["temperature"] * rng.uniform(0.9, 1.1, size=fl["temperature"].shape)
    up = fl["velocity"] * rng.uniform(0.5, 1.5, size=fl["velocity"].shape)
    up[0, 0, 0, 0] = 50.0 * fl["SoS"][0, 0, 0]  # one supersonic inflow point
    fl["velocity_profile"] = up
    fl["velocity_old_NSCBC"] = fl["velocity"] * 0.9
    fl["temperature_old_NSCBC"] = fl["temperature"] * 1.01
    return fl, h, m


def _plane(fl, d, pos):
    lo = [0, 0, 0]
    hi = [fl.nx - 1, fl.ny - 1, fl.nz - 1]
    lo[d] = hi[d] = pos
    return abi.rect(tuple(lo), tuple(hi))


@pytest.mark.parametrize("kind", ["tg", "air"])
@pytest.mark.parametrize("d", [0, 1, 2])
@pytest.mark.parametrize("which", ["inflow", "outflow"])
def test_port_matches_reference(kind, d, which):
    eos = 1 if kind == "tg" else 2
    ref = oracle.ref_lib(eos)
    if ref is None:
        pytest.skip("reference CPU build not present on this machine")
    port = oracle.port_lib()
    outs = []
    for lib in (ref, port):
        fl, h, _ = _state(lib, kind)
        v = fl.view()
        bc = _plane(fl, d, 0)
        if which == "inflow":
            st = getattr(lib, f"htr_SetNSCBC_InflowBC{'XYZ'[d]}")(C.byref(v), bc, h, 0.77, None)
        else:
            st = lib.htr_SetNSCBC_OutflowBC(C.byref(v), bc, h, None, None)
        abi.check(lib, st, which)
        outs.append(fl)
    for name in ("pressure", "temperature", "MolarFracs", "velocity"):
        assert np.array_equal(outs[0][name], outs[1][name]), name


@pytest.mark.parametrize("side", range(6))
@pytest.mark.parametrize("iso", [True, False])
def test_port_wall_state(side, iso):
    port = oracle.port_lib()
    fl, h, _ = _state(port, "air")
    ref = fl.copy()
    d, pos = side // 2, (0 if side % 2 == 0 else [fl.nx, fl.ny, fl.nz][side // 2] - 1)
    step = 1 if side % 2 == 0 else -1
    v = fl.view()
    fn = port.htr_SetIsothermalWallBC if iso else port.htr_SetAdiabaticWallBC
    abi.check(port, fn(C.byref(v), _plane(fl, d, pos), side, h, None), "wall")
    sl = [slice(None)] * 3
    sl[2 - d] = pos
    si = list(sl)
    si[2 - d] = pos + step
    sl, si = tuple(sl), tuple(si)
    assert np.array_equal(fl["MolarFracs"][sl], ref["MolarFracs"][si])
    assert np.array_equal(fl["pressure"][sl], ref["pressure"][si])
    assert np.array_equal(fl["temperature"][sl], ref["temperature_profile"][sl] if iso else ref["temperature"][si])
    assert np.all(fl["velocity"][sl] == 0.0)


def test_port_nscbc_time_derivatives():
    port = oracle.port_lib()
    fl, h, _ = _state(port, "air")
    ref = fl.copy()
    v = fl.view()
    bc = _plane(fl, 0, 0)
    abi.check(port, port.htr_UpdateNSCBCGhostCellTimeDerivatives(C.byref(v), bc, 0.125, None), "dt")
    s = (slice(None), slice(None), 0)
    assert np.array_equal(fl["dudtBoundary"][s], (ref["velocity"][s] - ref["velocity_old_NSCBC"][s]) / 0.125)
    assert np.array_equal(fl["dTdtBoundary"][s], (ref["temperature"][s] - ref["temperature_old_NSCBC"][s]) / 0.125)
    assert np.array_equal(fl["velocity_old_NSCBC"][s], ref["velocity"][s])
    assert np.array_equal(fl["temperature_old_NSCBC"][s], ref["temperature"][s])


def _gpu_vs_port(kind, call):
    import torch
    port = oracle.port_lib()
    host, hp, m = _state(port, kind)
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    call(port, host, hp, None)
    call(runtime.lib(), dev, gh, runtime.stream_handle())
    torch.cuda.synchronize()
    return host, dev.to_host()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tg", "air"])
@pytest.mark.parametrize("d", [0, 1, 2])
def test_gpu_inflow_outflow_state(kind, d):
    def inflow(lib, fl, h, s):
        v = fl.view()
        abi.check(lib, getattr(lib, f"htr_SetNSCBC_InflowBC{'XYZ'[d]}")(C.byref(v), _plane(fl, d, 0), h, 0.77, s), "in")

    def outflow(lib, fl, h, s):
        v = fl.view()
        abi.check(lib, lib.htr_SetNSCBC_OutflowBC(C.byref(v), _plane(fl, d, 1), h, None, s), "out")

    for call in (inflow, outflow):
        host, out = _gpu_vs_port(kind, call)
        util.check_fields(out, host, ("temperature", "MolarFracs", "velocity", "pressure"))


@pytest.mark.gpu
@pytest.mark.parametrize("side", range(6))
def test_gpu_wall_state_and_time_derivatives(side):
    def walls(lib, fl, h, s):
        v = fl.view()
        d = side // 2
        pos = 0 if side % 2 == 0 else [fl.nx, fl.ny, fl.nz][d] - 1
        abi.check(lib, lib.htr_SetIsothermalWallBC(C.byref(v), _plane(fl, d, pos), side, h, s), "wall")
        abi.check(lib, lib.htr_UpdateNSCBCGhostCellTimeDerivatives(C.byref(v), fl.bounds(), 0.25, s), "dt")

    host, out = _gpu_vs_port("air", walls)
    for name in ("MolarFracs", "pressure", "temperature", "velocity", "dudtBoundary", "dTdtBoundary",
                 "velocity_old_NSCBC", "temperature_old_NSCBC"):
        assert np.array_equal(out[name], host[name]), name
