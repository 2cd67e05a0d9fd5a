"""The hot path at the benchmark's full sizes.

Point by point against the CPU oracle (the port on all host cores, about 20
s per step): one fused SSP-RK3 step of the 256^3 periodic box of 5-species
reacting air (hybrid scheme, diffusion, explicit chemistry) and one fused
step of the 512 x 192 x 128 TENO-LAD boundary layer, from the same state:
Conserved within the pointwise bar of util.check everywhere, the primitive
and property fields too except in the rare cells where the two sides'
Newton solves for T stop one iteration apart at the reference's tolerance
(util.check_state_after_step).

Size-independent properties of the same grids:

- conservation: on a periodic uniform grid every face flux enters its two
  cells with opposite signs, so one RHS evaluation (hybrid Euler flux with
  its sensors, diffusion, chemistry sources) sums to zero over the grid in
  the total mass, the momentum and the total energy, up to rounding
  (chemistry only moves mass between species; the total energy includes
  the formation enthalpies);
- translation: rolling every input field by a periodic shift rolls the
  state after one fused RK3 step by the same shift, bit for bit (every face
  and cell is computed from its own stencil, wherever it falls in the
  tiles and in the TENO queue);
- determinism: the same step run twice gives the same bits.
"""
import ctypes as C

import pytest

N = 256
SHIFT = (7, 3, 5)  # cells in z, y, x


@pytest.fixture(scope="module")
def box():
    import torch

    from htr_gb300 import runtime, workloads
    fl = workloads.air_box(N, seed=1234)
    lib = runtime.lib()
    m = workloads.make_mixture_struct(lib, fl.meta["eos"], fl.meta["mix"])
    gh = runtime.load_mixture(fl.meta["eos"], m)
    dev = fl.to_device("cuda:0")
    del fl
    workloads.derive_state(lib, dev, gh, runtime.stream_handle())
    torch.cuda.synchronize()
    return dev, gh


def _port():
    import os

    import oracle
    port = oracle.port_lib()
    port.htr_oracle_set_threads(os.cpu_count() or 1)
    return port


STATE = ("Conserved", "temperature", "pressure", "velocity", "MolarFracs", "MassFracs", "rho", "mu", "lam", "Di",
         "SoS")


@pytest.mark.gpu
def test_fullsize_step_matches_the_oracle(box):
    """One fused SSP-RK3 step of the 256^3 benchmark box at the benchmark's
    step size against the oracle driver's step on the port, from the same
    (device-derived) state: sensors bit for bit, every state field within
    the pointwise bar."""
    import numpy as np
    import torch

    import oracle
    from htr_gb300 import abi, runtime, workloads
    from tests import util
    base, gh = box
    dev = base.copy()
    dt = runtime.stable_dt(dev, gh, cfl=0.8, chemistry=True)
    host = base.to_host()
    port = _port()
    eos = abi.HTR_EOS_AIRMIX
    hp = oracle.load_mixture(port, eos, workloads.make_mixture_struct(port, eos, workloads.AIR_REF))
    runtime.rk3_step(dev, gh, dt=dt, chemistry=True)
    oracle.step(port, host, hp, scheme="Hybrid", dt=dt, chemistry=True)
    torch.cuda.synchronize()
    out = dev.to_host()
    for d in "XYZ":
        a, b = out[f"shockSensor{d}"], host[f"shockSensor{d}"]
        assert np.array_equal(a, b), f"{(a != b).sum()} sensor{d} flags differ"
        assert 0 < b.sum() < b.size
    for name in STATE:
        ratio, info = util.pointwise(out[name], host[name], name)
        print(f"{name}: pointwise error / bound {ratio:.3e}, normwise {info['normwise']:.3e}")
    util.check_state_after_step(out, host, STATE)


@pytest.mark.gpu
def test_boundary_layer_fullsize_step_matches_the_oracle():
    """One fused step of the 512 x 192 x 128 TENO-LAD boundary layer (config
    3: NSCBC inflow/outflow in x, isothermal wall and outflow in y, periodic
    z, explicit chemistry) against the oracle's boundary-layer step on the
    port, from the same state: every state field within the pointwise bar."""
    import torch

    import oracle
    from htr_gb300 import runtime, wall, workloads
    from tests import util
    lib = runtime.lib()
    host = wall.boundary_layer(num=(512, 192, 128), seed=77)
    g, bc = host.meta["grid"], host.meta["bc"]
    m = workloads.make_mixture_struct(lib, host.meta["eos"], host.meta["mix"])
    gh = runtime.load_mixture(host.meta["eos"], m)
    dev = host.to_device("cuda:0")
    g.fill(dev, lib)
    workloads.derive_state(lib, dev, gh, runtime.stream_handle())
    mach = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    dt = wall.BoundaryRun(lib, dev, gh, bc, stream=runtime.stream_handle(), max_mach_buffer=mach).spectral_dt(0.8)
    torch.cuda.synchronize()
    ref = dev.to_host()
    ref.meta = dict(host.meta)
    del host
    port = _port()
    hp = oracle.load_mixture(port, ref.meta["eos"], workloads.make_mixture_struct(port, ref.meta["eos"],
                                                                                  ref.meta["mix"]))
    wall.FusedBoundaryRun(dev, gh, bc).step(dt)
    oracle.boundary_layer_step(port, ref, hp, dt, bc["xNeg"][1]["P"], bc["xPos"][1]["P"],
                               (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"]))
    torch.cuda.synchronize()
    out = dev.to_host()
    for name in STATE + ("dudtBoundary", "dTdtBoundary"):
        ratio, info = util.pointwise(out[name], ref[name], name)
        print(f"{name}: pointwise error / bound {ratio:.3e}, normwise {info['normwise']:.3e}")
    util.check_state_after_step(out, ref, STATE + ("dudtBoundary", "dTdtBoundary"))


@pytest.mark.gpu
def test_rhs_conserves_mass_momentum_energy(box):
    import torch

    from htr_gb300 import abi, runtime
    base, gh = box
    dev = base.copy()
    lib = runtime.lib()
    v = dev.view()
    r = dev.bounds()
    s = runtime.stream_handle()
    rk = (C.c_double * 2)(1.0, 0.0)

    def call(name, *args):
        abi.check(lib, getattr(lib, name)(*args), name)

    call("htr_InitializeTemporaries", C.byref(v), r, gh, s)  # Conserved_old for the limiter
    call("htr_UpdateDucrosSensor", C.byref(v), r, r, 1.0, s)
    for d in "XYZ":
        call(f"htr_UpdateShockSensor{d}", C.byref(v), r, r, gh, s)
    call("htr_InitializeTimeDerivatives", C.byref(v), r, 0, gh, s)
    for d in "ZYX":
        call(f"htr_UpdateUsingHybridEulerFlux{d}", C.byref(v), r, r, rk, 1e-9, gh, s)
    for d in "ZYX":
        call(f"htr_UpdateUsingDiffusionFlux{d}", C.byref(v), r, r, gh, s)
    call("htr_AddChemistrySources", C.byref(v), r, gh, s)
    torch.cuda.synchronize()
    ct = dev["Conserved_t"]
    assert torch.isfinite(ct).all()
    nsp = dev.nspec
    checks = {"mass": (ct[..., :nsp].sum(), ct[..., :nsp].abs().sum())}
    for k, name in enumerate(("momentum x", "momentum y", "momentum z", "energy")):
        c = ct[..., nsp + k]
        checks[name] = (c.sum(), c.abs().sum())
    for name, (total, scale) in checks.items():
        rel = abs(total.item()) / scale.item()
        print(f"{name}: |sum| / sum|.| = {rel:.3e}")
        assert scale.item() > 0 and rel <= 1e-10, (name, rel)


@pytest.mark.gpu
def test_step_is_translation_invariant_and_deterministic(box):
    import torch

    from htr_gb300 import runtime
    base, gh = box
    a = base.copy()
    b = base.copy()
    for name, arr in b.arrays.items():
        arr.copy_(torch.roll(base.arrays[name], shifts=SHIFT, dims=(0, 1, 2)))
    dt = 2e-9
    runtime.rk3_step(a, gh, dt=dt, chemistry=True)
    runtime.rk3_step(b, gh, dt=dt, chemistry=True)
    torch.cuda.synchronize()
    for name in ("Conserved", "temperature", "pressure", "velocity", "shockSensorX", "shockSensorY",
                 "shockSensorZ", "mu", "lam", "Di", "SoS"):
        rolled = torch.roll(a[name], shifts=SHIFT, dims=(0, 1, 2))
        if rolled.dtype == torch.float64:
            diff = ((rolled - b[name]).abs().max() / rolled.abs().max()).item()
            print(f"{name}: max |shifted - rolled| / max = {diff:.3e}")
        assert torch.equal(rolled, b[name]), name
    assert torch.isfinite(a["Conserved"]).all()
    # the same step again from the same state: the same bits
    c = base.copy()
    runtime.rk3_step(c, gh, dt=dt, chemistry=True)
    torch.cuda.synchronize()
    for name in ("Conserved", "temperature", "shockSensorX"):
        assert torch.equal(a[name], c[name]), name


@pytest.mark.gpu
def test_boundary_layer_step_is_z_translation_invariant():
    """The 512 x 192 x 128 TENO-LAD boundary layer (NSCBC inflow/outflow in
    x, isothermal wall and outflow in y, periodic z): one fused step of the
    state rolled along z equals the rolled step bit for bit, NSCBC planes,
    walls and the interior's maximum Mach number included."""
    import torch

    from htr_gb300 import runtime, wall, workloads
    lib = runtime.lib()
    host = wall.boundary_layer(num=(512, 192, 128), seed=77)
    g, bc = host.meta["grid"], host.meta["bc"]
    m = workloads.make_mixture_struct(lib, host.meta["eos"], host.meta["mix"])
    gh = runtime.load_mixture(host.meta["eos"], m)
    a = host.to_device("cuda:0")
    del host
    g.fill(a, lib)
    workloads.derive_state(lib, a, gh, runtime.stream_handle())
    mach = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    dt = wall.BoundaryRun(lib, a, gh, bc, stream=runtime.stream_handle(), max_mach_buffer=mach).spectral_dt(0.8)
    b = a.copy()
    for name, arr in b.arrays.items():
        arr.copy_(torch.roll(a.arrays[name], shifts=37, dims=0))
    wall.FusedBoundaryRun(a, gh, bc).step(dt)
    wall.FusedBoundaryRun(b, gh, bc).step(dt)
    torch.cuda.synchronize()
    assert torch.isfinite(a["Conserved"]).all()
    for name in ("Conserved", "temperature", "pressure", "velocity", "mu", "dudtBoundary", "dTdtBoundary"):
        rolled = torch.roll(a[name], shifts=37, dims=0)
        diff = ((rolled - b[name]).abs().max() / rolled.abs().max().clamp_min(1e-300)).item()
        print(f"{name}: max |shifted - rolled| / max = {diff:.3e}")
        assert torch.equal(rolled, b[name]), name


@pytest.mark.gpu
def test_batched_tubes_are_independent_at_full_size():
    """The 4096-tube batch of the bench (128-8192 cells per tube, both
    mixtures in two strips): for 12 tubes sampled from each strip, one fused
    step of the whole strip equals the same step of a strip holding that
    tube alone, bit for bit — a tube's result does not depend on its
    neighbours or on its place in the strip."""
    import numpy as np
    import torch

    from htr_gb300 import abi, fluid, runtime, tubes, workloads
    lib = runtime.lib()
    insts = tubes.instances(4096, seed=4242)
    rng = np.random.default_rng(0)
    for eos in (abi.HTR_EOS_CONSTPROPMIX, abi.HTR_EOS_AIRMIX):
        group = [i for i in insts if i["eos"] == eos]
        host, offs = tubes.build_strip(group)
        m = workloads.make_mixture_struct(lib, eos, host.meta["mix"])
        gh = runtime.load_mixture(eos, m)
        dev = host.to_device("cuda:0")
        del host
        workloads.derive_state(lib, dev, gh, runtime.stream_handle())
        out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
        v = dev.view()
        abi.check(lib, lib.htr_CalculateMaxSpectralRadius(
            C.byref(v), dev.interior(), gh, C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)),
            runtime.stream_handle()), "cfl")
        air = eos == abi.HTR_EOS_AIRMIX
        dt = (0.01 if air else 0.5) * 0.8 / out.item()
        start = dev.copy()
        runtime.rk3_step(dev, gh, dt=dt, chemistry=air)
        for k in rng.choice(len(group), size=12, replace=False):
            o, L = int(offs[k]), int(group[k]["L"])
            alone = fluid.Fluid((L + 2, 1, 1), dev.nspec, device="cuda:0", fields=list(start.arrays))
            for name, arr in alone.arrays.items():
                arr.copy_(start.arrays[name][:, :, o:o + L + 2])
            alone.meta = dict(start.meta)
            runtime.rk3_step(alone, gh, dt=dt, chemistry=air)
            torch.cuda.synchronize()
            for name in ("Conserved", "temperature", "pressure", "velocity", "shockSensorX", "MassFracs"):
                assert torch.equal(alone[name], dev[name][:, :, o:o + L + 2]), (eos, int(k), L, name)
        assert torch.isfinite(dev["Conserved"]).all()
