"""Launch-shape tuning of the fused stage: validation (no GPU needed), and on
the GPU that a tuned step gives bit-identical results."""
import os

import numpy as np
import pytest

from htr_gb300 import abi, runtime

import oracle
from tests import util


def _lib_or_skip():
    if not os.path.exists(runtime.LIB_PATH):
        pytest.skip("CUDA library not built")
    from htr_gb300 import autotune
    return autotune


def test_tuning_validation_and_roundtrip():
    at = _lib_or_skip()
    default = at.get_tuning()
    assert default.as_dict() == dict(prepass_block=256, diffusion_block=128, update_block=128,
                                     teno_blocks_per_sm=0, kg_x_tile=128)
    t = at.htr_stage_tuning(128, 64, 64, 16, 256)
    at.set_tuning(t)
    assert at.get_tuning().as_dict() == t.as_dict()
    for bad in (at.htr_stage_tuning(100, 64, 64, 16, 256), at.htr_stage_tuning(128, 256, 64, 16, 256),
                at.htr_stage_tuning(128, 64, 64, -1, 256), at.htr_stage_tuning(128, 64, 64, 33, 256), at.htr_stage_tuning(128, 64, 64, 8, 96)):
        with pytest.raises(abi.HtrError):
            at.set_tuning(bad)
    at.set_tuning(default)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tg", "air"])
def test_tuned_step_is_bit_identical(kind):
    import torch
    at = _lib_or_skip()
    shape = (20, 12, 10) if kind == "tg" else (14, 10, 8)
    fl, h, m = util.make_state(oracle.port_lib(), kind, shape, seed=13)
    gh = runtime.load_mixture(fl.meta["eos"], m)
    dt = 0.05 if kind == "tg" else 1e-9
    default = at.get_tuning()
    outs = []
    for t in (default, at.htr_stage_tuning(128, 64, 64, 3, 64), at.htr_stage_tuning(64, 32, 32, 16, 256)):
        at.set_tuning(t)
        dev = fl.to_device("cuda")
        runtime.rk3_step(dev, gh, dt=dt, chemistry=(kind == "air"))
        torch.cuda.synchronize()
        outs.append(dev.to_host())
    at.set_tuning(default)
    for o in outs[1:]:
        for name in o.arrays:
            assert np.array_equal(o[name], outs[0][name], equal_nan=True), name


def test_autotune_descent_keeps_only_real_gains(monkeypatch):
    """Coordinate descent of autotune() with the stage timer replaced by a
    cost model (no GPU): each parameter is tried from the best setting so
    far, a candidate is kept only when it beats the best by more than
    `gain`, and the winner is installed at the end."""
    from htr_gb300 import autotune as at
    state = {"t": at.htr_stage_tuning(256, 128, 128, 0, 128)}
    installed = []

    def get_tuning():
        return at.htr_stage_tuning(**state["t"].as_dict())

    def set_tuning(t):
        state["t"] = at.htr_stage_tuning(**t.as_dict())
        installed.append(t.as_dict())

    teno = {0: 10.0, 4: 12.0, 8: 11.0, 16: 9.5}
    tile = {64: 1.0, 128: 0.0, 256: -0.5}
    upd = {64: -0.05, 128: 0.0}  # 0.5 % faster: below the 1 % gain

    def stage_ms(grids, reps=3, workspace=None, originals=None):
        t = state["t"]
        return teno[t.teno_blocks_per_sm] + tile[t.kg_x_tile] + upd[t.update_block]

    class Fluid:
        def copy(self):
            return Fluid()

    monkeypatch.setattr(at, "get_tuning", get_tuning)
    monkeypatch.setattr(at, "set_tuning", set_tuning)
    monkeypatch.setattr(at, "stage_ms", stage_ms)
    best, t_best, t0, trials = at.autotune([(Fluid(), None, 1e-9, True)], reps=1)
    assert t0 == 10.0
    assert best == dict(prepass_block=256, diffusion_block=128, update_block=128, teno_blocks_per_sm=16,
                        kg_x_tile=256)
    assert t_best == 9.0
    assert installed[-1] == best and state["t"].as_dict() == best
    # every candidate of every parameter tried once, except the current value
    n_trials = sum(len(v) - 1 for v in at.CANDIDATES.values())
    assert len(trials) == 1 + n_trials
    assert 0 in at.CANDIDATES["teno_blocks_per_sm"]
