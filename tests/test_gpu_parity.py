"""GPU parity: every RHS-path entry point of the CUDA library against the CPU
oracle on identical seeded inputs.

Bars (stated per check):
* shock sensors (booleans) and the Ducros value: bit-exact;
* Euler fluxes of the single-species gas: bit-exact (every operation on that
  path is correctly rounded on both sides, TENO powers included);
* everything else: per-component max relative error <= 1e-11
  (util.RHS_REL_TOL), the bar of the spec for the RHS after one RK3 step.
"""
import ctypes as C

import numpy as np
import pytest

from htr_gb300 import abi, runtime, workloads

import oracle
from tests import util

pytestmark = pytest.mark.gpu

CASES = {"tg": (16, 12, 10), "air": (12, 10, 8)}


@pytest.fixture(scope="module")
def port():
    return oracle.port_lib()


@pytest.fixture(scope="module")
def gpu():
    return runtime.lib()


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request, port):
    kind = request.param
    fl, h, m = util.make_state(port, kind, CASES[kind], seed=11)
    rng = np.random.default_rng(5)
    fl["Conserved_old"] = fl["Conserved"] * (1 + 1e-3 * rng.standard_normal(fl["Conserved"].shape))
    fl["Conserved_t"] = 0.01 * rng.standard_normal(fl["Conserved_t"].shape)
    eos = fl.meta["eos"]
    gh = runtime.load_mixture(eos, m)
    return kind, fl, h, gh


def _run_both(port, gpu, fl, h, gh, name, build_args):
    import torch
    host = fl.copy()
    dev = fl.to_device("cuda")
    vh, vd = host.view(), dev.view()
    util.call(port, name, *build_args(C.byref(vh), host, h, None))
    util.call(gpu, name, *build_args(C.byref(vd), dev, gh, runtime.stream_handle()))
    torch.cuda.synchronize()
    return host, dev.to_host()


@pytest.mark.parametrize("d", "XYZ")
@pytest.mark.parametrize("scheme", ["Hybrid", "TENO", "TENOA", "TENOLAD", "SkewSymmetric"])
def test_euler_flux(port, gpu, case, scheme, d):
    kind, fl, h, gh = case
    # sensors from the oracle so both sides see the same flags
    oracle.update_sensors(port, fl, h, 1.0)
    rk = (C.c_double * 2)(0.75, 0.25)
    if scheme == "SkewSymmetric":
        name = f"htr_UpdateUsingSkewSymmetricEulerFlux{d}"
        args = lambda v, f, m, s: (v, f.interior(), f.bounds(), m, s)
    else:
        name = f"htr_UpdateUsing{scheme}EulerFlux{d}"
        args = lambda v, f, m, s: (v, f.interior(), f.bounds(), rk, 2e-3, m, s)
    host, dev = _run_both(port, gpu, fl, h, gh, name, args)
    if kind == "tg":
        assert np.array_equal(dev["Conserved_t"], host["Conserved_t"]), \
            f"max rel err {util.rel_err(dev['Conserved_t'], host['Conserved_t']).max()}"
    else:
        err = util.rel_err(dev["Conserved_t"], host["Conserved_t"])
        assert err.max() <= util.RHS_REL_TOL, err


@pytest.mark.parametrize("d", "XYZ")
def test_diffusion_flux(port, gpu, case, d):
    kind, fl, h, gh = case
    name = f"htr_UpdateUsingDiffusionFlux{d}"
    host, dev = _run_both(port, gpu, fl, h, gh, name, lambda v, f, m, s: (v, f.interior(), f.bounds(), m, s))
    err = util.rel_err(dev["Conserved_t"], host["Conserved_t"])
    assert err.max() <= util.RHS_REL_TOL, err


def test_sensors_bit_exact(port, gpu, case):
    import torch
    kind, fl, h, gh = case
    host = fl.copy()
    dev = fl.to_device("cuda")
    oracle.update_sensors(port, host, h, 1.0)
    vd = dev.view()
    r = dev.bounds()
    s = runtime.stream_handle()
    util.call(gpu, "htr_UpdateDucrosSensor", C.byref(vd), r, r, 1.0, s)
    for d in "XYZ":
        util.call(gpu, f"htr_UpdateShockSensor{d}", C.byref(vd), r, r, gh, s)
    torch.cuda.synchronize()
    out = dev.to_host()
    assert np.array_equal(out["DucrosSensor"], host["DucrosSensor"])
    for d in "XYZ":
        a, b = out[f"shockSensor{d}"], host[f"shockSensor{d}"]
        assert np.array_equal(a, b), f"{(a != b).sum()} of {a.size} sensor{d} flags differ"


@pytest.mark.parametrize("kind,n,mach", [("air", 40, (0.5, 3.0)), ("air", 32, (2.0, 6.0)), ("tg", 40, None)])
def test_sensors_bit_exact_large(port, gpu, kind, n, mach):
    """Shock sensors on larger seeded grids (tens of thousands of cells per
    direction, strong compressions for the Mach 2-6 case): every boolean and
    the Ducros value equal the oracle's."""
    import torch
    if kind == "air":
        fl = workloads.air_box(n, seed=21, mach=mach)
    else:
        fl = workloads.taylor_green(n, seed=21)
    m = workloads.make_mixture_struct(port, fl.meta["eos"], fl.meta["mix"])
    h = oracle.load_mixture(port, fl.meta["eos"], m)
    workloads.derive_state(port, fl, h)
    gh = runtime.load_mixture(fl.meta["eos"], m)
    host = fl.copy()
    dev = fl.to_device("cuda")
    oracle.update_sensors(port, host, h, 1.0)
    vd = dev.view()
    r = dev.bounds()
    s = runtime.stream_handle()
    util.call(gpu, "htr_UpdateDucrosSensor", C.byref(vd), r, r, 1.0, s)
    for d in "XYZ":
        util.call(gpu, f"htr_UpdateShockSensor{d}", C.byref(vd), r, r, gh, s)
    torch.cuda.synchronize()
    out = dev.to_host()
    assert np.array_equal(out["DucrosSensor"], host["DucrosSensor"])
    for d in "XYZ":
        a, b = out[f"shockSensor{d}"], host[f"shockSensor{d}"]
        assert np.array_equal(a, b), f"{(a != b).sum()} of {a.size} sensor{d} flags differ"
        assert 0 < b.sum() <= b.size


def test_chemistry_sources(port, gpu, case):
    kind, fl, h, gh = case
    host, dev = _run_both(port, gpu, fl, h, gh, "htr_AddChemistrySources",
                          lambda v, f, m, s: (v, f.interior(), m, s))
    err = util.rel_err(dev["Conserved_t"], host["Conserved_t"])
    assert err.max() <= util.RHS_REL_TOL, err


def test_properties(port, gpu, case):
    kind, fl, h, gh = case
    host, dev = _run_both(port, gpu, fl, h, gh, "htr_UpdatePropertiesFromPrimitive",
                          lambda v, f, m, s: (v, f.bounds(), m, s))
    for name in ("rho", "mu", "lam", "Di", "SoS", "MassFracs"):
        err = util.rel_err(dev[name], host[name])
        assert err.max() <= util.RHS_REL_TOL, (name, err)


def test_conserved_and_primitive(port, gpu, case):
    kind, fl, h, gh = case
    host, dev = _run_both(port, gpu, fl, h, gh, "htr_UpdateConservedFromPrimitive",
                          lambda v, f, m, s: (v, f.bounds(), m, s))
    err = util.rel_err(dev["Conserved"], host["Conserved"])
    assert err.max() <= util.RHS_REL_TOL, err
    # perturb the temperature guess, then recover primitives with Newton
    fl2 = fl.copy()
    fl2["temperature"] = fl["temperature"] * 1.01
    host, dev = _run_both(port, gpu, fl2, h, gh, "htr_UpdatePrimitiveFromConserved",
                          lambda v, f, m, s: (v, f.bounds(), m, s))
    for name in ("temperature", "pressure", "MolarFracs", "velocity"):
        err = util.rel_err(dev[name], host[name])
        assert err.max() <= util.RHS_REL_TOL, (name, err)


def test_spectral_radius(port, gpu, case):
    import torch
    kind, fl, h, gh = case
    r_cpu = C.c_double()
    vh = fl.view()
    util.call(port, "htr_CalculateMaxSpectralRadius", C.byref(vh), fl.interior(), h, C.byref(r_cpu), None)
    dev = fl.to_device("cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    vd = dev.view()
    util.call(gpu, "htr_CalculateMaxSpectralRadius", C.byref(vd), dev.interior(), gh,
              C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)), runtime.stream_handle())
    torch.cuda.synchronize()
    assert abs(out.item() - r_cpu.value) <= util.RHS_REL_TOL * r_cpu.value


@pytest.mark.parametrize("fused", [False, True], ids=["tasks", "fused"])
@pytest.mark.parametrize("scheme", ["Hybrid", "TENO", "TENOA", "TENOLAD", "SkewSymmetric"])
def test_rk3_step(port, gpu, case, scheme, fused):
    """One full SSP-RK3 step on the device against the oracle driver: the
    composition of the task entry points (htr_rk3_step) and the fused stage
    pipeline (htr_rk3_step_ws), every Euler scheme."""
    import torch
    kind, fl, h, gh = case
    host = fl.copy()
    dev = fl.to_device("cuda")
    chem = kind == "air"
    dt = 1e-9 if chem else 0.05
    oracle.step(port, host, h, scheme=scheme, dt=dt, chemistry=chem)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    runtime.rk3_step(dev, gh, scheme=scheme, dt=dt, chemistry=chem, fused=fused,
                     status_dev=C.c_void_p(status.data_ptr()))
    torch.cuda.synchronize()
    assert status.item() == 0
    out = dev.to_host()
    for name in ("Conserved", "temperature", "pressure", "Conserved_t", "MolarFracs", "velocity",
                 "rho", "mu", "lam", "Di", "SoS", "MassFracs"):
        err = util.rel_err(out[name], host[name])
        assert err.max() <= util.RHS_REL_TOL, (name, err.max())
    if scheme == "Hybrid":
        for d in "XYZ":
            assert np.array_equal(out[f"shockSensor{d}"], host[f"shockSensor{d}"])


def test_fused_step_rejects_bad_workspace(gpu, case):
    """htr_rk3_step_ws checks the workspace size and the periodic-grid
    requirement on the host, before any launch."""
    kind, fl, h, gh = case
    dev = fl.to_device("cuda")
    v = dev.view()
    p = runtime.htr_step_params(0, 1.0, 0.0, 1e-9, 0)
    used = C.c_double(0.0)
    nb = gpu.htr_rk3_workspace_bytes(dev.interior(), gh)
    assert nb > 0
    st = gpu.htr_rk3_step_ws(C.byref(v), dev.interior(), dev.bounds(), C.byref(p), gh, None, nb,
                             C.byref(used), None, runtime.stream_handle())
    assert st == abi.HTR_ERR_ARGUMENT
    import torch
    buf = torch.empty(nb, dtype=torch.uint8, device="cuda")
    st = gpu.htr_rk3_step_ws(C.byref(v), dev.interior(), dev.bounds(), C.byref(p), gh,
                             C.c_void_p(buf.data_ptr()), nb - 8, C.byref(used), None, runtime.stream_handle())
    assert st == abi.HTR_ERR_ARGUMENT
    inner = dev.interior()
    inner.hi[0] -= 1
    st = gpu.htr_rk3_step_ws(C.byref(v), inner, dev.bounds(), C.byref(p), gh,
                             C.c_void_p(buf.data_ptr()), nb, C.byref(used), None, runtime.stream_handle())
    assert st == abi.HTR_ERR_UNSUPPORTED
