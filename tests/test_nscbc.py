"""NSCBC boundary terms (inflow / outflow, both sides of each direction) and
the maximum Mach number.

CPU: the oracle port against the reference's own compiled tasks, bit for bit
(skips where the reference sources are absent).  GPU (-m gpu): the CUDA
library against the port, within the pointwise bar of util.check.

States: seeded boxes of both mixtures whose boundary planes carry the
collocated node types of a characteristic boundary in the tested direction
(L_C, Lp1_C ... Rm2_C, Rm1_C, R_C; src/prometeo_metric.rg:196-264), random
imposed-inflow time derivatives and a random Conserved_t to add to.
"""
import ctypes as C

import numpy as np
import pytest

from htr_gb300 import abi, runtime, workloads

import oracle
from tests import util

L_C, LP1_C, RM2_C, RM1_C, R_C = 8, 9, 10, 11, 12
SIDES = [("XNeg", 0, True), ("XPos", 0, False), ("YNeg", 1, True), ("YPos", 1, False),
         ("ZNeg", 2, True), ("ZPos", 2, False)]


def _state(lib, kind, d, seed=5, shape=(10, 9, 8)):
    fl, h, m = util.make_state(lib, kind, shape, seed=seed)
    nt = fl[f"nType_{'xyz'[d]}"]
    n = shape[d]
    idx = [slice(None)] * 3
    for pos, t in ((0, L_C), (1, LP1_C), (n - 3, RM2_C), (n - 2, RM1_C), (n - 1, R_C)):
        idx[2 - d] = pos
        nt[tuple(idx)] = t
    rng = np.random.default_rng(seed + d)
    fl["dudtBoundary"] = rng.standard_normal(fl["dudtBoundary"].shape)
    fl["dTdtBoundary"] = rng.standard_normal(fl["dTdtBoundary"].shape)
    fl["Conserved_t"] = rng.standard_normal(fl["Conserved_t"].shape)
    # a subsonic state at the boundaries (the supersonic branch is also exercised below)
    return fl, h, m


def _plane(fl, d, minus):
    lo = [0, 0, 0]
    hi = [fl.nx - 1, fl.ny - 1, fl.nz - 1]
    pos = 0 if minus else hi[d]
    lo[d] = hi[d] = pos
    return abi.rect(tuple(lo), tuple(hi))


def _run(lib, fl, h, side, d, minus, kind_bc, stream=None):
    v = fl.view()
    bc = _plane(fl, d, minus)
    if kind_bc == "in":
        st = getattr(lib, f"htr_UpdateUsingFluxNSCBCInflow{side}")(C.byref(v), bc, h, stream)
    else:
        st = getattr(lib, f"htr_UpdateUsingFluxNSCBCOutflow{side}")(C.byref(v), bc, fl.bounds(), h, 0.7, 1.3,
                                                                     0.9, stream)
    abi.check(lib, st, f"nscbc {kind_bc} {side}")


@pytest.mark.parametrize("kind", ["tg", "air"])
@pytest.mark.parametrize("side,d,minus", SIDES)
@pytest.mark.parametrize("kind_bc", ["in", "out"])
def test_port_matches_reference(kind, side, d, minus, kind_bc):
    eos = 1 if kind == "tg" else 2
    ref = oracle.ref_lib(eos)
    if ref is None:
        pytest.skip("reference CPU build not present on this machine")
    port = oracle.port_lib()
    fr, hr, _ = _state(ref, kind, d)
    fp, hp, _ = _state(port, kind, d)
    for name in fr.arrays:
        assert np.array_equal(fr[name], fp[name]), name
    _run(ref, fr, hr, side, d, minus, kind_bc)
    _run(port, fp, hp, side, d, minus, kind_bc)
    assert np.array_equal(fr["Conserved_t"], fp["Conserved_t"])
    assert not np.array_equal(fr["Conserved_t"], _state(port, kind, d)[0]["Conserved_t"])


def test_supersonic_inlet_zeroes_the_rhs():
    port = oracle.port_lib()
    fl, h, _ = _state(port, "tg", 0)
    fl["velocity"][..., 0] = 10.0 * fl["SoS"]  # supersonic towards +x at the x- inlet
    _run(port, fl, h, "XNeg", 0, True, "in")
    assert np.all(fl["Conserved_t"][:, :, 0] == 0.0)


def test_max_mach_number():
    port = oracle.port_lib()
    fl, h, _ = _state(port, "air", 0)
    for d in range(3):
        out = C.c_double(0.0)
        v = fl.view()
        abi.check(port, port.htr_CalculateMaxMachNumber(C.byref(v), fl.interior(), d, C.byref(out), None), "mach")
        assert out.value == np.max(np.abs(fl["velocity"][..., d]) / fl["SoS"])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tg", "air"])
@pytest.mark.parametrize("side,d,minus", SIDES)
@pytest.mark.parametrize("kind_bc", ["in", "out"])
def test_gpu_matches_port(kind, side, d, minus, kind_bc):
    import torch
    port = oracle.port_lib()
    host, hp, m = _state(port, kind, d)
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    _run(port, host, hp, side, d, minus, kind_bc)
    _run(runtime.lib(), dev, gh, side, d, minus, kind_bc, runtime.stream_handle())
    torch.cuda.synchronize()
    util.check(dev.to_host()["Conserved_t"], host["Conserved_t"], "Conserved_t")


@pytest.mark.gpu
def test_gpu_max_mach_number():
    import torch
    port = oracle.port_lib()
    host, hp, m = _state(port, "air", 0)
    dev = host.to_device("cuda")
    for d in range(3):
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        v = dev.view()
        abi.check(runtime.lib(), runtime.lib().htr_CalculateMaxMachNumber(
            C.byref(v), dev.interior(), d, C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)),
            runtime.stream_handle()), "mach")
        torch.cuda.synchronize()
        assert out.item() == np.max(np.abs(host["velocity"][..., d]) / host["SoS"])
