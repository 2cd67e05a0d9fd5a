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
