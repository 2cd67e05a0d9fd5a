"""Autotuner of the fused stage's launch shapes.

The batched and served forms run many grids of one shape family (long 1-D
strips, small 3-D boxes) whose best launch shapes differ from the 256^3
defaults.  `autotune` times candidate shapes of the fused stage
(htr_rk3_stage_profile: per-kernel CUDA-event times of one stage) on working
copies of the grids it is given, every repetition restored from the same
states, and keeps the fastest, one parameter at a time (coordinate descent
from the current setting), then installs it with htr_rk3_set_tuning.
The shapes change only how work is distributed, never the arithmetic, so a
tuned run gives the same results bit for bit.
"""
import ctypes as C

import numpy as np

from . import abi, runtime

CANDIDATES = {
    "kg_x_tile": (64, 128, 256),
    "teno_blocks_per_sm": (0, 4, 8, 16),
    "update_block": (64, 128),
    "diffusion_block": (64, 128),
    "prepass_block": (128, 256),
}


class htr_stage_tuning(C.Structure):
    _fields_ = [("prepass_block", C.c_int), ("diffusion_block", C.c_int), ("update_block", C.c_int),
                ("teno_blocks_per_sm", C.c_int), ("kg_x_tile", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _bind(l):
    l.htr_rk3_set_tuning.argtypes = [C.POINTER(htr_stage_tuning)]
    l.htr_rk3_set_tuning.restype = C.c_int
    l.htr_rk3_get_tuning.argtypes = [C.POINTER(htr_stage_tuning)]
    l.htr_rk3_get_tuning.restype = C.c_int
    l.htr_rk3_stage_profile.argtypes = [C.POINTER(abi.htr_fluid_view), abi.htr_rect3, abi.htr_rect3,
                                        C.POINTER(runtime.htr_step_params), C.c_void_p, C.c_void_p, C.c_size_t,
                                        C.POINTER(C.c_float), C.c_void_p]
    l.htr_rk3_stage_profile.restype = C.c_int
    return l


def get_tuning():
    l = _bind(runtime.lib())
    t = htr_stage_tuning()
    abi.check(l, l.htr_rk3_get_tuning(C.byref(t)), "htr_rk3_get_tuning")
    return t


def set_tuning(t):
    l = _bind(runtime.lib())
    abi.check(l, l.htr_rk3_set_tuning(C.byref(t)), "htr_rk3_set_tuning")


def stage_ms(grids, reps=3, workspace=None, originals=None):
    """Sum over `grids` (fluid, mixture handle, dt, chemistry) of the median
    stage time (sum of the stage's kernel times), in ms.  Each timed stage
    advances its grid; with `originals` (fluids of the same shapes) every
    repetition starts from a fresh copy of them."""
    l = _bind(runtime.lib())
    ws = workspace or runtime.Workspace()
    total = 0.0
    for k, (fl, gh, dt, chem) in enumerate(grids):
        v = fl.view()
        nb = runtime.workspace_bytes(fl, gh)
        ptr = ws.get(nb, fl.device)
        p = runtime.htr_step_params(runtime.SCHEMES["Hybrid"], 1.0, 0.0, dt, 1 if chem else 0)
        runs = []
        for _ in range(reps):
            if originals is not None:
                for name, a in fl.arrays.items():
                    a.copy_(originals[k].arrays[name])
            out = (C.c_float * 10)()  # htr_rk3_stage_profile writes 10 kernel times
            abi.check(l, l.htr_rk3_stage_profile(C.byref(v), fl.interior(), fl.bounds(), C.byref(p), gh,
                                                 C.c_void_p(ptr), nb, out, runtime.stream_handle()), "profile")
            runs.append(sum(out))
        total += float(np.median(runs))
    return total


def autotune(grids, reps=3, workspace=None, gain=0.01):
    """Coordinate descent over CANDIDATES; installs and returns (best tuning
    as a dict, its stage ms, the default's stage ms, trials).  Trials run on
    working copies of the grids, each repetition restored from the given
    states, which are left untouched."""
    work = [(fl.copy(), gh, dt, chem) for fl, gh, dt, chem in grids]
    orig = [g[0] for g in grids]
    best = get_tuning()
    stage_ms(work, 1, workspace, orig)  # warm-up
    t_best = t0 = stage_ms(work, reps, workspace, orig)
    trials = [(best.as_dict(), t_best)]
    for name, values in CANDIDATES.items():
        for val in values:
            if val == getattr(best, name):
                continue
            trial = htr_stage_tuning(**best.as_dict())
            setattr(trial, name, val)
            set_tuning(trial)
            t = stage_ms(work, reps, workspace, orig)
            trials.append((trial.as_dict(), t))
            if t < t_best * (1.0 - gain):
                best, t_best = trial, t
        set_tuning(best)
    del work
    return best.as_dict(), t_best, t0, trials
