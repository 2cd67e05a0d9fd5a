"""GPU parity: every RHS-path entry point of the CUDA library against the CPU
oracle on identical seeded inputs.

Bars (stated per check):
* shock sensors (booleans) and the Ducros value: bit-exact;
* Euler fluxes of the single-species gas: bit-exact (every operation on that
  path is correctly rounded on both sides, TENO powers included);
* everything else: the pointwise bar of util.check, element by element
  |gpu - cpu| <= max(1e-11 |cpu|, floor) (the reference's own regression
  rule, solverTests/testAll.py:22-26, at a ten times tighter tolerance).
"""
import ctypes as C

import numpy as np
import pytest

from htr_gb300 import abi, runtime, workloads

import oracle
from tests import util

pytestmark = pytest.mark.gpu

CASES = {"tg": (16, 12, 10), "air": (12, 10, 8)}
# state fields compared after a step
STEP_FIELDS = ("Conserved", "temperature", "pressure", "Conserved_t", "MolarFracs", "velocity",
               "rho", "mu", "lam", "Di", "SoS", "MassFracs")


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
            util.pointwise(dev["Conserved_t"], host["Conserved_t"], "Conserved_t")[1]
    else:
        util.check(dev["Conserved_t"], host["Conserved_t"], "Conserved_t")


@pytest.mark.parametrize("d", "XYZ")
def test_diffusion_flux(port, gpu, case, d):
    kind, fl, h, gh = case
    name = f"htr_UpdateUsingDiffusionFlux{d}"
    host, dev = _run_both(port, gpu, fl, h, gh, name, lambda v, f, m, s: (v, f.interior(), f.bounds(), m, s))
    util.check(dev["Conserved_t"], host["Conserved_t"], "Conserved_t")


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
        # both outcomes occur (these grids hold 12-50 % false flags)
        assert 0 < b.sum() < b.size


def test_chemistry_sources(port, gpu, case):
    kind, fl, h, gh = case
    host, dev = _run_both(port, gpu, fl, h, gh, "htr_AddChemistrySources",
                          lambda v, f, m, s: (v, f.interior(), m, s))
    util.check(dev["Conserved_t"], host["Conserved_t"], "Conserved_t")


@pytest.mark.parametrize("state,dt", [("dirichlet", 1e-7), ("air", 1e-6), ("air", 1e-4), ("air", 3e-3)])
def test_update_chemistry_seeded(port, gpu, state, dt):
    """Implicit Rosenbrock chemistry (UpdateChemistryTask, src/prometeo_chem.cc:31-68,
    src/prometeo_chem.hpp:53-93, src/Utils/math_utils.hpp:196-441) with the
    transport RHS of the state frozen in Conserved_t, over chemical steps
    from non-stiff to stiff: on the air-box workload's state (T 300-8000 K,
    p 0.1-10 bar, Dirichlet compositions) at the small step where the
    reference's solver still converges everywhere, and on near-air
    compositions (util.make_air_state) up to whole CFL steps; status 0.

    Bar: the solver adapts its steps to an absolute error of 1e-10, and a
    one-ulp change of its inputs alone moves the reference's own result (and
    the intermediate temperature it leaves behind) by up to ~700 times the
    pointwise bar; Conserved, Conserved_t_old and temperature must lie
    within the pointwise bar or 10 times that measured spread
    (util.check_within_spread)."""
    import torch
    if state == "dirichlet":
        fl, h, m = util.make_state(port, "air", (12, 10, 8), seed=11)
    else:
        fl, h, m = util.make_air_state(port, (12, 10, 8), seed=12)
    oracle.update_sensors(port, fl, h, 1.0)
    fl["Conserved_old"] = fl["Conserved"]
    oracle.update_derivatives(port, fl, h, 1, dt, chemistry=False)
    gh = runtime.load_mixture(fl.meta["eos"], m)

    def solve(f):
        st = C.c_int(0)
        v = f.view()
        util.call(port, "htr_UpdateChemistry", C.byref(v), f.interior(), dt, h, C.byref(st), None)
        assert st.value == 0

    fields = ("Conserved", "Conserved_t_old", "temperature")
    host, spread = util.ulp_spread(solve, fl, fields)
    assert np.all(np.isfinite(host["Conserved"]))
    dev = fl.to_device("cuda")
    sd = torch.zeros(1, dtype=torch.int32, device="cuda")
    vd = dev.view()
    util.call(gpu, "htr_UpdateChemistry", C.byref(vd), dev.interior(), dt, gh,
              C.cast(C.c_void_p(sd.data_ptr()), C.POINTER(C.c_int)), runtime.stream_handle())
    torch.cuda.synchronize()
    assert sd.item() == 0
    out = dev.to_host()
    # the step changed the state (the comparison is not of an idle solve)
    assert not np.array_equal(host["Conserved"], fl["Conserved"])
    for name in fields:
        util.check_within_spread(out[name], host[name], name, spread[name])


@pytest.mark.parametrize("fused", [False, True], ids=["tasks", "fused"])
@pytest.mark.parametrize("scheme,cfl", [("Hybrid", 0.3), ("TENOLAD", 0.08)])
def test_implicit_chemistry_step(port, gpu, scheme, cfl, fused):
    """One SSP-RK3 step with Integrator.implicitChemistry (src/prometeo.rg:1360-1398,
    src/prometeo_rk.rg:59-112) on near-air compositions at a CFL step far
    above the explicit chemical limit: the task composition (htr_rk3_step)
    and the fused pipeline (htr_rk3_step_ws) against the oracle driver's
    implicit branch on the port; sensors bit for bit, status 0, every state
    field within the pointwise bar or 10 times the spread that one-ulp input
    changes cause in the oracle's own step (the chemistry solve's adaptive
    steps, see test_update_chemistry_seeded)."""
    import torch
    host, h, m = util.make_air_state(port, (12, 10, 8), seed=5)
    gh = runtime.load_mixture(host.meta["eos"], m)
    dev = host.to_device("cuda")
    dt = oracle.spectral_dt(port, host, h, cfl)
    fields = STEP_FIELDS + ("Conserved_t_old",)
    ref, spread = util.ulp_spread(lambda f: oracle.step(port, f, h, scheme=scheme, dt=dt, implicit=True),
                                  host, fields)
    assert np.all(np.isfinite(ref["Conserved"]))
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    runtime.rk3_step(dev, gh, scheme=scheme, dt=dt, fused=fused, implicit=True,
                     status_dev=C.c_void_p(status.data_ptr()))
    torch.cuda.synchronize()
    assert status.item() == 0
    out = dev.to_host()
    for name in fields:
        util.check_within_spread(out[name], ref[name], name, spread[name])
    if scheme == "Hybrid":
        for d in "XYZ":
            assert np.array_equal(out[f"shockSensor{d}"], ref[f"shockSensor{d}"])


def test_properties(port, gpu, case):
    kind, fl, h, gh = case
    host, dev = _run_both(port, gpu, fl, h, gh, "htr_UpdatePropertiesFromPrimitive",
                          lambda v, f, m, s: (v, f.bounds(), m, s))
    util.check_fields(dev, host, ("rho", "mu", "lam", "Di", "SoS", "MassFracs"))


def test_conserved_and_primitive(port, gpu, case):
    kind, fl, h, gh = case
    host, dev = _run_both(port, gpu, fl, h, gh, "htr_UpdateConservedFromPrimitive",
                          lambda v, f, m, s: (v, f.bounds(), m, s))
    util.check(dev["Conserved"], host["Conserved"], "Conserved")
    # perturb the temperature guess, then recover primitives with Newton
    fl2 = fl.copy()
    fl2["temperature"] = fl["temperature"] * 1.01
    host, dev = _run_both(port, gpu, fl2, h, gh, "htr_UpdatePrimitiveFromConserved",
                          lambda v, f, m, s: (v, f.bounds(), m, s))
    util.check_fields(dev, host, ("temperature", "pressure", "MolarFracs", "velocity"))


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
    util.check_fields(out, host, STEP_FIELDS)
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


@pytest.mark.parametrize("fused", [False, True], ids=["tasks", "fused"])
def test_step_with_pure_nitrogen_cells(port, gpu, fused):
    """Cells of nearly pure N2 (every other species at a mole fraction of
    1e-30) beside air.  The double-float transport properties keep the FP64
    routine for cells where fewer than two species have a mole fraction of
    1e-20 (their diffusion partner sums underflow in float range): the
    properties of the prepared state, pure cells included, within the
    pointwise bar of the oracle.  Then one step through the task path and
    the fused pipeline, every field within the bar, except the species
    diffusivities of cells whose second most abundant species has a mole
    fraction below 1e-6: there the dominant species' diffusivity is a mean
    over trace mole fractions of 1e-20 and less, which no bar on the state
    pins (a one-ulp change of the state moves the reference's own value by
    up to 2e-10 relative).  (Exact zeros are outside the reference's domain:
    its diffusivity of the one species present is 0/0 there.)"""
    import torch
    fl, h, m = util.make_air_state(port, (12, 10, 8), seed=23)
    X = fl["MolarFracs"].copy()
    pure = np.zeros(X.shape[:3], dtype=bool)
    # eight of twelve cells along x: the middle ones stay nearly pure
    # through the first stage (their stencils see only nitrogen)
    pure[:, :, 2:10] = True
    X[pure] = np.array([1.0, 1e-30, 1e-30, 1e-30, 1e-30])
    fl["MolarFracs"] = X
    workloads.derive_state(port, fl, h)
    assert np.all(fl["MassFracs"][pure][:, 1:] < 1e-29)
    gh = runtime.load_mixture(fl.meta["eos"], m)
    host, dev = _run_both(port, gpu, fl, h, gh, "htr_UpdatePropertiesFromPrimitive",
                          lambda v, f, mm, s: (v, f.bounds(), mm, s))
    util.check_fields(dev, host, ("rho", "mu", "lam", "Di", "SoS", "MassFracs"))
    host = fl.copy()
    oracle.step(port, host, h, dt=1e-9, chemistry=True)
    dv = fl.to_device("cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    runtime.rk3_step(dv, gh, dt=1e-9, chemistry=True, fused=fused, status_dev=C.c_void_p(status.data_ptr()))
    torch.cuda.synchronize()
    assert status.item() == 0
    out = dv.to_host()
    util.check_fields(out, host, tuple(f for f in STEP_FIELDS if f != "Di"))
    second = np.sort(host["MolarFracs"], axis=-1)[..., -2]
    mixed = second >= 1e-6
    assert 0 < mixed.sum() < mixed.size
    util.check(out["Di"][mixed], host["Di"][mixed], "Di")
