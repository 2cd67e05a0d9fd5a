"""Batched 1-D shock tubes on the GPU against per-tube oracle steps.

Tubes of both mixtures (staggered Dirichlet ghosts, one-cell periodic y/z)
are packed end to end into one strip per mixture; one fused RK3 step of the
strip (htr_rk3_step_ws) must reproduce, tube by tube, one oracle step of
each tube on its own (RHS, update and primitive recovery on the interior,
ghosts imposed).  The per-tube task path (htr_rk3_step on each tube, the
plain drop-in) is checked against the same oracle steps.  Bar: every state
field within the pointwise bar of util.check; x shock sensors bit-exact.
"""
import ctypes as C

import numpy as np
import pytest

from htr_gb300 import abi, runtime, tubes, workloads

import oracle
from tests import util

FIELDS = ("Conserved", "temperature", "pressure", "Conserved_t", "MolarFracs", "MassFracs", "velocity",
          "rho", "mu", "lam", "Di", "SoS")


def _groups(seed=31, n=8):
    insts = tubes.instances(n, seed=seed, length=(12, 40))
    groups = {}
    for inst in insts:
        groups.setdefault(inst["eos"], []).append(inst)
    return groups


def _oracle_tubes(port, insts, chem):
    """Host tubes derived by the oracle, the common dt, and their oracle step."""
    eos = insts[0]["eos"]
    fls = [tubes.tube_fluid(i) for i in insts]
    m = workloads.make_mixture_struct(port, eos, fls[0].meta["mix"])
    h = oracle.load_mixture(port, eos, m)
    for f in fls:
        workloads.derive_state(port, f, h)
    dt = 0.1 * min(oracle.spectral_dt(port, f, h, 0.8) for f in fls)
    start = [f.copy() for f in fls]
    for f in fls:
        oracle.step(port, f, h, dt=dt, chemistry=chem, bnum=(1, 0, 0))
    return start, fls, m, dt


def _check(out, ref, name_prefix, sensors=("X",)):
    for name in FIELDS:
        ratio, info = util.pointwise(out[name], ref[name], name)
        assert ratio <= 1.0, (name_prefix, info)
    for d in sensors:
        assert np.array_equal(out[f"shockSensor{d}"], ref[f"shockSensor{d}"]), (name_prefix, d)


@pytest.mark.gpu
@pytest.mark.parametrize("eos", [abi.HTR_EOS_CONSTPROPMIX, abi.HTR_EOS_AIRMIX])
def test_batched_strip_equals_per_tube_oracle(eos):
    import torch
    port = oracle.port_lib()
    insts = _groups()[eos]
    chem = eos == abi.HTR_EOS_AIRMIX
    start, ref, m, dt = _oracle_tubes(port, insts, chem)
    strip, offs = tubes.pack(start)
    gh = runtime.load_mixture(eos, m)
    dev = strip.to_device("cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    runtime.rk3_step(dev, gh, dt=dt, chemistry=chem, fused=True, status_dev=C.c_void_p(status.data_ptr()))
    torch.cuda.synchronize()
    assert status.item() == 0
    out = dev.to_host()
    for k, (o, f) in enumerate(zip(offs, ref)):
        tube = {name: a[:, :, o:o + f.nx] for name, a in out.arrays.items()}
        _check(tube, f.arrays, f"tube {k}")


@pytest.mark.gpu
@pytest.mark.parametrize("implicit", [False, True], ids=["explicit", "implicit"])
@pytest.mark.parametrize("eos", [abi.HTR_EOS_CONSTPROPMIX, abi.HTR_EOS_AIRMIX])
def test_batched_strip_per_tube_dt(eos, implicit):
    """Each tube with its own step size (CFL 0.4 over its own spectral radius,
    for air also at most half its fastest chemical time scale, as one run of
    the reference computes dt per simulation): one fused step of the strip
    with per-cell step sizes (htr_rk3_step_cells_ws) equals, tube by tube,
    the oracle's step of that tube alone with its own dt.  With implicit
    chemistry (air), the tube's whole CFL step, far above its chemical time."""
    import torch
    if implicit and eos != abi.HTR_EOS_AIRMIX:
        pytest.skip("implicit chemistry needs a reacting mixture")
    port = oracle.port_lib()
    insts = _groups()[eos]
    chem = eos == abi.HTR_EOS_AIRMIX
    fls = [tubes.tube_fluid(i) for i in insts]
    m = workloads.make_mixture_struct(port, eos, fls[0].meta["mix"])
    h = oracle.load_mixture(port, eos, m)
    for f in fls:
        workloads.derive_state(port, f, h)
    strip, offs = tubes.pack([f.copy() for f in fls])
    gh = runtime.load_mixture(eos, m)
    dev = strip.to_device("cuda")
    widths = [f.nx for f in fls]
    dts = tubes.strip_dts(dev, offs, widths, gh, chemistry=chem and not implicit)
    assert len(set(dts)) == len(dts)  # every tube its own step
    ref, spreads = [], []
    for f, dt in zip(fls, dts):
        run = lambda g, dt=dt: oracle.step(port, g, h, dt=dt, chemistry=chem, bnum=(1, 0, 0), implicit=implicit)
        if implicit:
            r, sp = util.ulp_spread(run, f, FIELDS)
        else:
            r, sp = f.copy(), None
            run(r)
        ref.append(r)
        spreads.append(sp)
    dt_cell = torch.tensor(tubes.cell_dt(offs, widths, dts), dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    runtime.rk3_step_cells(dev, gh, dt_cell, chemistry=chem, implicit=implicit,
                           status_dev=C.c_void_p(status.data_ptr()))
    torch.cuda.synchronize()
    assert status.item() == 0
    out = dev.to_host()
    for k, (o, f, sp) in enumerate(zip(offs, ref, spreads)):
        tube = {name: a[:, :, o:o + f.nx] for name, a in out.arrays.items()}
        if sp is None:
            _check(tube, f.arrays, f"tube {k}")
        else:
            for name in FIELDS:
                util.check_within_spread(tube[name], f[name], name, sp[name])


@pytest.mark.gpu
@pytest.mark.parametrize("eos", [abi.HTR_EOS_CONSTPROPMIX, abi.HTR_EOS_AIRMIX])
def test_plain_per_tube_task_path(eos):
    import torch
    port = oracle.port_lib()
    insts = _groups()[eos]
    chem = eos == abi.HTR_EOS_AIRMIX
    start, ref, m, dt = _oracle_tubes(port, insts, chem)
    gh = runtime.load_mixture(eos, m)
    for k, (s, f) in enumerate(zip(start, ref)):
        dev = s.to_device("cuda")
        runtime.rk3_step(dev, gh, dt=dt, chemistry=chem, fused=False, interior=dev.interior((1, 0, 0)))
        torch.cuda.synchronize()
        _check(dev.to_host().arrays, f.arrays, f"tube {k}", sensors=("X", "Y", "Z"))


@pytest.mark.parametrize("eos", [abi.HTR_EOS_CONSTPROPMIX, abi.HTR_EOS_AIRMIX])
def test_oracle_tube_step_keeps_ghosts(eos):
    """CPU: one oracle step of a tube leaves its Dirichlet ghosts untouched and
    changes the interior."""
    port = oracle.port_lib()
    insts = _groups()[eos]
    start, ref, m, dt = _oracle_tubes(port, insts, eos == abi.HTR_EOS_AIRMIX)
    for s, f in zip(start, ref):
        for name in ("Conserved", "temperature", "pressure", "rho"):
            a, b = s[name], f[name]
            assert np.array_equal(a[:, :, [0, -1]], b[:, :, [0, -1]]), name
        assert not np.array_equal(s["Conserved"], f["Conserved"])
        assert np.isfinite(f["Conserved"]).all()


def test_strip_layout():
    insts = tubes.instances(5, seed=2, length=(10, 20))
    fls = [tubes.tube_fluid(i) for i in insts if i["eos"] == insts[0]["eos"]]
    strip, offs = tubes.pack(fls)
    assert strip.nx == sum(f.nx for f in fls) and strip.ny == strip.nz == 1
    for o, f in zip(offs, fls):
        t = strip["nType_x"][0, 0, o:o + f.nx]
        assert t[0] == tubes.L_S and t[-1] == tubes.R_S
        assert np.array_equal(t, tubes.node_types(f.nx - 2))


@pytest.mark.gpu
def test_mixed_batch_equals_each_instance_alone():
    """A batch of uneven instances of both mixtures -- shock tubes of gas and
    of air (packed into one strip per mixture), 2-D vortex boxes, 3-D
    Taylor-Green and reacting-air boxes of different sizes -- advanced by
    one CUDA graph launch per step (batch.Batch, launch shapes tuned per
    size class), each with its own step size: after two steps every instance
    equals, bit for bit, the same two steps of that instance alone."""
    import torch

    from htr_gb300 import batch
    insts = [batch.tube_instance(i, "cuda") for i in tubes.instances(7, seed=5, length=(12, 40))]
    assert {i["chemistry"] for i in insts} == {False, True}
    boxes = [workloads.vortex2d(12, seed=1), workloads.vortex2d(shape=(16, 10), seed=2),
             workloads.taylor_green(shape=(8, 6, 4), seed=3), workloads.air_box(shape=(6, 5, 4), seed=4),
             workloads.air_box(shape=(8, 8, 8), seed=5)]
    insts += [batch.box_instance(b, "cuda") for b in boxes]
    alone = []
    for inst in insts:
        f = inst["fluid"].copy()
        f.meta = dict(inst["fluid"].meta)
        alone.append(f)
    bt = batch.Batch(insts, "cuda", tune=True)
    assert len(bt.tunings) >= 3  # strips and boxes are tuned per size class
    for _ in range(2):
        bt.step()
    torch.cuda.synchronize()
    for inst, f in zip(insts, alone):
        for _ in range(2):
            runtime.rk3_step(f, inst["gh"], dt=inst["dt"], chemistry=inst["chemistry"])
        torch.cuda.synchronize()
        for name in ("Conserved", "temperature", "pressure", "velocity", "MassFracs", "mu", "Di",
                     "shockSensorX"):
            assert torch.equal(inst["fluid"][name], f[name]), (inst["fluid"].shape, name)
        assert torch.isfinite(f["Conserved"]).all()
    # every instance advanced by its own step size
    assert len({round(i["dt"], 15) for i in insts}) == len(insts)
