"""Known answers of the reference's own unit tests on this path.

The expected values are the ones the reference's unit tests assert, with the
tolerances those tests use:

* unitTests/mixTest/mixTest.rg:87-171 and its ConstPropMix.json / AirMix.json
  (mixture at 750 K, 1 atm; every property within 1e-3 relative,
  mixTest.rg:759-900);
* unitTests/chemTest/chemTest.rg:40-49, 115-145 (AirMix at 5000 K, 1 atm:
  explicit production rates and one implicit Rosenbrock step of
  dt = 1e-6 uRef/LRef, within 1e-5 relative).

The CPU oracle is checked here without a GPU; the same states run through the
CUDA library under `-m gpu`.  Both go through the task entry points
(UpdatePropertiesFromPrimitive, UpdateConservedFromPrimitive,
AddChemistrySources, UpdateChemistry) on a 2x2x2 uniform grid.
"""
import ctypes as C
import math

import numpy as np
import pytest

from htr_gb300 import abi, runtime
from htr_gb300.fluid import Fluid

import oracle
from tests import util

RGAS = 8.3144598
W_AIR = np.array([2 * 14.0067e-3, 2 * 15.9994e-3, 30.00610e-3, 14.0067e-3, 15.9994e-3])

# mixTest.rg:88-117 (ConstPropMix.json: R 287.15, gamma 1.4, Pr 0.71, constant mu 5e-3)
CP_T, CP_P, CP_R = 750.0, 101325.0, 287.15
CP_EXPECT = dict(rho=CP_P / (CP_R * CP_T), mu=5.0e-3, lam=1.005025e+03 * 5.0e-3 / 0.71,
                 sos=math.sqrt(1.4 * CP_R * CP_T))

# mixTest.rg:119-167 (AirMix.json: XiRef N2 0.78 / O2 0.22, TRef 300 K, PRef 1 atm)
AIR_T, AIR_P = 750.0, 101325.0
AIR_Y = np.full(5, 0.2)
AIR_EXPECT = dict(
    MixW=2.135186e-02,
    X=np.array([1.524403e-01, 1.334541e-01, 1.423168e-01, 3.048806e-01, 2.669082e-01]),
    mu=3.723077e-05, lam=6.736994e-02, sos=6.567317e+02,
    Di=np.array([1.192983e-04, 1.174019e-04, 1.162986e-04, 1.820668e-04, 1.882347e-04]),
    prod=np.array([3.413124e+07, 2.664566e+04, -3.578332e+07, -1.742776e+07, 1.905320e+07]),
)
MIXTEST_REF = dict(PRef=101325.0, TRef=300.0, LRef=1.0, XiRef=(0.78, 0.22, 0.0, 0.0, 0.0))

# chemTest.rg:40-57
CH_T, CH_P = 5000.0, 101325.0
CH_Y = np.array([0.78, 0.22, 1.0e-60, 1.0e-60, 1.0e-60])
CH_EPROD = np.array([-1.658328e-01, -1.445940e+03, 1.332770e-54, 1.658328e-01, 1.445940e+03])
CH_CRES = np.array([5.460212e-02, 1.296359e-02, 2.994386e-04, 1.502734e-05, 2.321006e-03,
                    0.0, 0.0, 0.0, 3.141423e+05])
CH_MIXWREF = 1.0 / (0.78 / 28.0134e-3 + 0.22 / (2 * 15.999e-3))
CHEMTEST_REF = dict(PRef=101325.0, TRef=300.0, LRef=1.0,
                    XiRef=(CH_MIXWREF * 0.78 / 28.0134e-3, CH_MIXWREF * 0.22 / (2 * 15.999e-3), 0.0, 0.0, 0.0))


def _refs(ref):
    xi = np.where(np.array(ref["XiRef"]) > 0, np.array(ref["XiRef"]), 0.0)
    MixWRef = float((xi * W_AIR).sum())
    rhoRef = ref["PRef"] * MixWRef / (RGAS * ref["TRef"])
    return dict(MixWRef=MixWRef, rhoRef=rhoRef, eRef=ref["PRef"] / rhoRef,
                uRef=math.sqrt(ref["PRef"] / rhoRef), muRef=math.sqrt(ref["PRef"] * rhoRef) * ref["LRef"],
                lamRef=math.sqrt(ref["PRef"] * rhoRef) * ref["LRef"] * RGAS / MixWRef,
                DiRef=math.sqrt(ref["PRef"] / rhoRef) * ref["LRef"],
                wiRef=math.sqrt(ref["PRef"] * rhoRef) / ref["LRef"])


def _uniform(nspec, T, P, X):
    fl = Fluid((2, 2, 2), nspec)
    fl["temperature"] = T
    fl["pressure"] = P
    fl["MolarFracs"] = np.broadcast_to(np.asarray(X, dtype=np.float64), fl["MolarFracs"].shape)
    return fl


def _run(lib, fl, mixh, device, chem_dt=None):
    """Properties, conserved, chemistry sources (and one implicit step) with `lib`."""
    f = fl.to_device(device) if device else fl
    s = runtime.stream_handle() if device else None
    v = f.view()
    r = f.bounds()
    util.call(lib, "htr_UpdatePropertiesFromPrimitive", C.byref(v), r, mixh, s)
    util.call(lib, "htr_UpdateConservedFromPrimitive", C.byref(v), r, mixh, s)
    util.call(lib, "htr_InitializeTimeDerivatives", C.byref(v), r, 0, mixh, s)
    util.call(lib, "htr_AddChemistrySources", C.byref(v), r, mixh, s)
    out = {"props": None}
    if device:
        import torch
        torch.cuda.synchronize()
    out["props"] = f.to_host() if device else f.copy()
    if chem_dt is not None:
        # as chemTest.rg:115-127: the implicit step starts from Conserved_t
        # holding the explicit production rates
        if device:
            import torch
            st = torch.zeros(1, dtype=torch.int32, device=device)
            util.call(lib, "htr_UpdateChemistry", C.byref(v), r, chem_dt, mixh,
                      C.cast(C.c_void_p(st.data_ptr()), C.POINTER(C.c_int)), s)
            torch.cuda.synchronize()
            assert st.item() == 0
            out["chem"] = f.to_host()
        else:
            st = C.c_int(0)
            util.call(lib, "htr_UpdateChemistry", C.byref(v), r, chem_dt, mixh, C.byref(st), None)
            assert st.value == 0
            out["chem"] = f.copy()
    return out


def _close(a, b, tol):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    err = np.abs(a - b) / np.where(b != 0, np.abs(b), 1.0)
    assert err.max() < tol, (a, b, err.max())


def _mixture(lib, eos, params):
    m = util.workloads.make_mixture_struct(lib, eos, params)
    return m, oracle.load_mixture(lib, eos, m)


def check_constpropmix(lib, device=None):
    params = dict(gasConstant=CP_R, gamma=1.4, prandtl=0.71, viscosityModel=abi.HTR_VISC_CONSTANT,
                  p0=5.0e-3, p1=0.0, p2=0.0)
    m, h = _mixture(oracle.port_lib(), abi.HTR_EOS_CONSTPROPMIX, params)
    if device:
        h = runtime.load_mixture(abi.HTR_EOS_CONSTPROPMIX, m)
    out = _run(lib, _uniform(1, CP_T, CP_P, [1.0]), h, device)["props"]
    _close(out["rho"], CP_EXPECT["rho"], 1e-3)
    _close(out["mu"], CP_EXPECT["mu"], 1e-3)
    _close(out["lam"], CP_EXPECT["lam"], 1e-3)
    _close(out["SoS"], CP_EXPECT["sos"], 1e-3)


def check_airmix(lib, device=None):
    m, h = _mixture(oracle.port_lib(), abi.HTR_EOS_AIRMIX, MIXTEST_REF)
    if device:
        h = runtime.load_mixture(abi.HTR_EOS_AIRMIX, m)
    R = _refs(MIXTEST_REF)
    # molar fractions of Y = 0.2 each, exactly as the mixture converts them
    X = (AIR_Y / W_AIR) / (AIR_Y / W_AIR).sum()
    out = _run(lib, _uniform(5, AIR_T / MIXTEST_REF["TRef"], AIR_P / MIXTEST_REF["PRef"], X), h, device)["props"]
    _close(X, AIR_EXPECT["X"], 1e-3)
    _close(out["MassFracs"][0, 0, 0], AIR_Y, 1e-3)
    _close(out["rho"] * R["rhoRef"], AIR_P * AIR_EXPECT["MixW"] / (RGAS * AIR_T), 1e-3)
    _close(out["mu"] * R["muRef"], AIR_EXPECT["mu"], 1e-3)
    _close(out["lam"] * R["lamRef"], AIR_EXPECT["lam"], 1e-3)
    _close(out["SoS"] * R["uRef"], AIR_EXPECT["sos"], 1e-3)
    _close(out["Di"][0, 0, 0] * R["DiRef"], AIR_EXPECT["Di"], 1e-3)
    _close(out["Conserved_t"][0, 0, 0, :5] * R["wiRef"], AIR_EXPECT["prod"], 1e-3)


def check_chemistry(lib, device=None):
    m, h = _mixture(oracle.port_lib(), abi.HTR_EOS_AIRMIX, CHEMTEST_REF)
    if device:
        h = runtime.load_mixture(abi.HTR_EOS_AIRMIX, m)
    R = _refs(CHEMTEST_REF)
    X = (CH_Y / W_AIR) / (CH_Y / W_AIR).sum()
    dt = 1e-6 * R["uRef"] / CHEMTEST_REF["LRef"]
    res = _run(lib, _uniform(5, CH_T / CHEMTEST_REF["TRef"], CH_P / CHEMTEST_REF["PRef"], X), h, device,
               chem_dt=dt)
    prod = res["props"]["Conserved_t"][0, 0, 0, :5] * R["wiRef"]
    for i in range(5):
        if abs(CH_EPROD[i]) > 1e-40:
            _close(prod[i], CH_EPROD[i], 1e-5)
    C_ = res["chem"]["Conserved"][0, 0, 0]
    got = np.concatenate([C_[:8] * R["rhoRef"], [C_[8] * R["rhoRef"] * R["eRef"]]])
    for i in range(9):
        if CH_CRES[i] != 0.0:
            _close(got[i], CH_CRES[i], 1e-5)
        else:
            assert abs(got[i]) < 1e-12


def test_oracle_constpropmix_mixtest():
    check_constpropmix(oracle.port_lib())


def test_oracle_airmix_mixtest():
    check_airmix(oracle.port_lib())


def test_oracle_chemtest():
    check_chemistry(oracle.port_lib())


@pytest.mark.gpu
def test_gpu_constpropmix_mixtest():
    check_constpropmix(runtime.lib(), "cuda")


@pytest.mark.gpu
def test_gpu_airmix_mixtest():
    check_airmix(runtime.lib(), "cuda")


@pytest.mark.gpu
def test_gpu_chemtest():
    check_chemistry(runtime.lib(), "cuda")
