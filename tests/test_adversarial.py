"""Decisions at the margins of the single-precision filters, and the
positivity limiter.

The kernels decide TENO stencil selections, shock sensors and the cut-off
exponents of TENO-LAD and of the sensor first in single precision and run
the reference's exact double-precision expression only inside a safety
margin of the cut-off (see tests/adversarial.py).  These grids put many
decisions inside those margins, on both sides of the cut-off.

CPU: the grids really land there (numpy restatement of the quotients), and
  the oracle port equals the compiled reference on them bit for bit (where
  the reference is built).
GPU: shock sensors and single-species TENO / TENO-LAD Euler fluxes equal the
  port bit for bit, and htr_decision_counters shows that the exact path ran
  for at least as many decisions as the design puts inside the margins;
  a multi-species TENO flux with a time step large enough that the predicted
  partial densities go negative blends with the first-order flux
  (src/prometeo_rhs.inl:710-758), the counters show the blends, and the flux
  meets the pointwise bar against the port.
"""
import ctypes as C

import numpy as np
import pytest

from htr_gb300 import abi, runtime, workloads

import oracle
from tests import adversarial as A
from tests import util

SENSOR_SHAPE = (24, 16, 16)
TENO_SHAPE = (32, 16, 16)
PHI_CUT = A.bisect(lambda x: A.sensor_cut_argument(x) - 6.5, 0.0, 1.0)  # cut-off 1e-6


def _tg_state(lib, shape):
    fl = workloads.taylor_green(shape=shape, seed=3)
    m = workloads.make_mixture_struct(lib, fl.meta["eos"], fl.meta["mix"])
    h = oracle.load_mixture(lib, fl.meta["eos"], m)
    return fl, h, m


def sensor_grid(lib):
    """Taylor-Green state whose rho (Conserved[0]) and Ducros value are the
    adversarial sensor field (the shock sensor reads only those, the node
    types and the bounds)."""
    fl, h, m = _tg_state(lib, SENSOR_SHAPE)
    workloads.derive_state(lib, fl, h)
    rho, phi, q_near, cut_near = A.sensor_field(*SENSOR_SHAPE, PHI_CUT)
    c = fl["Conserved"].copy()
    c[..., 0] = rho
    fl["Conserved"] = c
    fl["DucrosSensor"] = phi
    return fl, h, m, q_near, cut_near


def entropy_wave_grid(lib, rho):
    """Single-species entropy wave: the given density, uniform pressure 1/gamma
    and velocity (0.3, 0, 0); properties and conserved variables derived."""
    nz, ny, nx = rho.shape
    fl, h, m = _tg_state(lib, (nx, ny, nz))
    p = 1.0 / 1.4
    fl["pressure"] = p
    fl["temperature"] = p / rho
    vel = np.zeros(rho.shape + (3,))
    vel[..., 0] = 0.3
    fl["velocity"] = vel
    workloads.derive_state(lib, fl, h)
    fl["Conserved_old"] = fl["Conserved"]
    fl["Conserved_t"] = 0.0
    return fl, h, m


def limiter_grid(lib, shape=(24, 8, 8)):
    """Five-species air with one species nearly absent in half of the box (X
    of N 1e-14 for x < nx/2) and a uniform stream of Mach ~2 along x."""
    fl = workloads.air_box(shape=shape, seed=17, mach=(1.5, 2.5))
    x = fl["MolarFracs"].copy()
    x[:, :, : shape[0] // 2, 3] = 1e-14
    x /= x.sum(axis=-1, keepdims=True)
    fl["MolarFracs"] = x
    vel = fl["velocity"].copy()
    vel[..., 0] = np.abs(vel[..., 0]) + 1.0
    fl["velocity"] = vel
    m = workloads.make_mixture_struct(lib, fl.meta["eos"], fl.meta["mix"])
    h = oracle.load_mixture(lib, fl.meta["eos"], m)
    workloads.derive_state(lib, fl, h)
    fl["Conserved_old"] = fl["Conserved"]
    fl["Conserved_t"] = 0.0
    return fl, h, m


# ---------------------------------------------------------------------------
# CPU
# ---------------------------------------------------------------------------
def test_design_lands_in_the_margins():
    """Enough decisions of each kind lie inside the filter margins, and the
    sensor grid holds both outcomes among them."""
    rho, phi, q_near, cut_near = A.sensor_field(*SENSOR_SHAPE, PHI_CUT)
    assert q_near >= 40 and cut_near >= 1000, (q_near, cut_near)
    _, near = A.teno_lad_field(*TENO_SHAPE)
    assert near >= 100, near
    cut = float(A.sensor_cut(PHI_CUT))
    outcomes = set()
    for pen in rho.reshape(-1, SENSOR_SHAPE[0])[: SENSOR_SHAPE[1] * SENSOR_SHAPE[2] // 2]:
        q = A.quotients(A.window(pen, SENSOR_SHAPE[0] // 4 - 1), 1e-8)[0]
        if np.abs(q.min() / cut - 1) < 5e-5:
            outcomes.add(bool(q.min() > cut))
    assert outcomes == {True, False}


def test_port_matches_reference_on_margin_grids():
    """The oracle port and the compiled reference agree bit for bit on the
    adversarial grids: sensors, TENO and TENO-LAD fluxes, and the limiter
    case (the port pins the GPU below)."""
    ref = oracle.ref_lib(abi.HTR_EOS_CONSTPROPMIX)
    ref_air = oracle.ref_lib(abi.HTR_EOS_AIRMIX)
    if ref is None or ref_air is None:
        pytest.skip("the compiled reference is not built here")
    port = oracle.port_lib()
    fl, h, m, _, _ = sensor_grid(port)
    hr = oracle.load_mixture(ref, abi.HTR_EOS_CONSTPROPMIX, m)
    a, b = fl.copy(), fl.copy()
    r = fl.bounds()
    va, vb = a.view(), b.view()
    util.call(port, "htr_UpdateShockSensorX", C.byref(va), r, r, h, None)
    util.call(ref, "htr_UpdateShockSensorX", C.byref(vb), r, r, hr, None)
    assert np.array_equal(a["shockSensorX"], b["shockSensorX"])
    rk = (C.c_double * 2)(0.0, 1.0)
    for scheme, rho in (("TENO", A.teno_field(*TENO_SHAPE)), ("TENOLAD", A.teno_lad_field(*TENO_SHAPE)[0])):
        fl, h, m = entropy_wave_grid(port, rho)
        hr = oracle.load_mixture(ref, abi.HTR_EOS_CONSTPROPMIX, m)
        a, b = fl.copy(), fl.copy()
        va, vb = a.view(), b.view()
        util.call(port, f"htr_UpdateUsing{scheme}EulerFluxX", C.byref(va), a.bounds(), a.bounds(), rk, 1e-3, h, None)
        util.call(ref, f"htr_UpdateUsing{scheme}EulerFluxX", C.byref(vb), b.bounds(), b.bounds(), rk, 1e-3, hr, None)
        assert np.array_equal(a["Conserved_t"], b["Conserved_t"]), scheme
    fl, h, m = limiter_grid(port)
    hr = oracle.load_mixture(ref_air, abi.HTR_EOS_AIRMIX, m)
    a, b = fl.copy(), fl.copy()
    va, vb = a.view(), b.view()
    dt = _limiter_dt(fl)
    util.call(port, "htr_UpdateUsingTENOEulerFluxX", C.byref(va), a.bounds(), a.bounds(), rk, dt, h, None)
    util.call(ref_air, "htr_UpdateUsingTENOEulerFluxX", C.byref(vb), b.bounds(), b.bounds(), rk, dt, hr, None)
    assert np.array_equal(a["Conserved_t"], b["Conserved_t"])


def _limiter_dt(fl):
    """A limiter deltaTime of about three convective cell times: the
    predicted partial densities rho_i - dt (m_e[p] + m_e[p+1]) F_i of cells
    that the stream empties go negative."""
    dx = 1.0 / fl["dcsi_e"].max()
    return 3.0 * dx / np.abs(fl["velocity"][..., 0]).max()


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _counts(gpu, enable):
    c = (C.c_ulonglong * abi.HTR_DECISION_COUNTERS)()
    abi.check(gpu, gpu.htr_decision_counters(enable, c), "htr_decision_counters")
    return dict(zip(abi.DECISION_COUNTERS, list(c)))


@pytest.fixture
def counting():
    gpu = runtime.lib()
    _counts(gpu, 1)
    yield gpu
    _counts(gpu, 0)


@pytest.mark.gpu
def test_gpu_sensor_at_the_margins(counting):
    import torch
    gpu = counting
    port = oracle.port_lib()
    fl, h, m, q_near, cut_near = sensor_grid(port)
    host = fl.copy()
    r = fl.bounds()
    vh = host.view()
    util.call(port, "htr_UpdateShockSensorX", C.byref(vh), r, r, h, None)
    dev = fl.to_device("cuda")
    gh = runtime.load_mixture(fl.meta["eos"], m)
    vd = dev.view()
    _counts(gpu, 1)
    util.call(gpu, "htr_UpdateShockSensorX", C.byref(vd), r, r, gh, runtime.stream_handle())
    torch.cuda.synchronize()
    n = _counts(gpu, 1)
    util.log_record(counters=n, predicted_sensor_exact=q_near, predicted_cut_exact=cut_near)
    out = dev.to_host()
    a, b = out["shockSensorX"], host["shockSensorX"]
    assert np.array_equal(a, b), f"{(a != b).sum()} flags differ"
    assert 0 < b.sum() < b.size
    assert n["sensor_exact"] >= q_near, (n, q_near)
    assert n["cut_exact"] >= cut_near, (n, cut_near)
    assert n["sensor_filtered"] > 0 and n["cut_filtered"] > 0, n


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["TENO", "TENOLAD"])
def test_gpu_teno_at_the_margins(counting, scheme):
    """Single-species TENO / TENO-LAD Euler fluxes are bit-exact, so any
    selection flag that differed would show in Conserved_t."""
    import torch
    gpu = counting
    port = oracle.port_lib()
    if scheme == "TENO":
        rho, near = A.teno_field(*TENO_SHAPE), 1
    else:
        rho, near = A.teno_lad_field(*TENO_SHAPE)
    fl, h, m = entropy_wave_grid(port, rho)
    rk = (C.c_double * 2)(0.0, 1.0)
    host = fl.copy()
    vh = host.view()
    name = f"htr_UpdateUsing{scheme}EulerFluxX"
    util.call(port, name, C.byref(vh), fl.bounds(), fl.bounds(), rk, 1e-3, h, None)
    dev = fl.to_device("cuda")
    gh = runtime.load_mixture(fl.meta["eos"], m)
    vd = dev.view()
    _counts(gpu, 1)
    util.call(gpu, name, C.byref(vd), fl.bounds(), fl.bounds(), rk, 1e-3, gh, runtime.stream_handle())
    torch.cuda.synchronize()
    n = _counts(gpu, 1)
    util.log_record(counters=n, predicted_exact=near)
    out = dev.to_host()
    assert np.array_equal(out["Conserved_t"], host["Conserved_t"]), \
        util.pointwise(out["Conserved_t"], host["Conserved_t"], "Conserved_t")[1]
    assert n["teno_exact"] >= near, n
    assert n["teno_filtered"] > 0, n


@pytest.mark.gpu
def test_gpu_positivity_limiter(counting):
    import torch
    gpu = counting
    port = oracle.port_lib()
    fl, h, m = limiter_grid(port)
    dt = _limiter_dt(fl)
    rk = (C.c_double * 2)(0.0, 1.0)
    host = fl.copy()
    vh = host.view()
    util.call(port, "htr_UpdateUsingTENOEulerFluxX", C.byref(vh), fl.bounds(), fl.bounds(), rk, dt, h, None)
    # the same call with a vanishing step never blends: the blended fluxes differ
    calm = fl.copy()
    vc = calm.view()
    util.call(port, "htr_UpdateUsingTENOEulerFluxX", C.byref(vc), fl.bounds(), fl.bounds(), rk, 1e-30, h, None)
    assert not np.array_equal(calm["Conserved_t"], host["Conserved_t"])
    dev = fl.to_device("cuda")
    gh = runtime.load_mixture(fl.meta["eos"], m)
    vd = dev.view()
    _counts(gpu, 1)
    util.call(gpu, "htr_UpdateUsingTENOEulerFluxX", C.byref(vd), fl.bounds(), fl.bounds(), rk, dt, gh,
              runtime.stream_handle())
    torch.cuda.synchronize()
    n = _counts(gpu, 1)
    util.log_record(counters=n)
    assert n["limiter_blend"] > 0, n
    util.check(dev.to_host()["Conserved_t"], host["Conserved_t"], "Conserved_t")
