"""Benchmark of the GB300 explicit RHS: FP64 RHS cell-updates/s.

Workload: 3-D periodic 256^3 box of 5-species reacting air (AirMix, 2 + 3
Park-type reactions), seeded synthetic fields (T 300-8000 K, p 0.1-10 bar,
Dirichlet mass fractions, Mach 0.5-3 solenoidal + compressive velocity),
hybrid TENO / Kennedy-Gruber Euler flux with the Ducros/TENO-A shock sensor,
diffusion with mixture-averaged transport, explicit chemistry sources, SSP
RK3.  One "step" is one RK3 time step (3 full RHS evaluations + state
refresh); a cell-update is one full RHS evaluation of one cell.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--n 256]

The step size is fixed for the run: min(CFL 0.8 acoustic step, half the
fastest chemical time scale of the initial state), so that explicit
chemistry stays stable; the RHS work per step does not depend on it.

Prints one JSON line (rank 0).  N > 1 runs N independent replicas (one grid
per GPU, no data exchange); value is the total over ranks.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from htr_gb300 import abi, serve, tubes, workloads  # noqa: E402

METRIC = "FP64 RHS cell-updates/s"
UNIT = "cell-updates/s"
# Compulsory bytes of one full-RHS cell-update at the reference field layout
# (5-species air): every input field read once, Conserved_t written once.
BYTES_PER_CELL_UPDATE_AIR = 495
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


_T0 = time.perf_counter()


def log(msg):
    """Progress of the run on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f}s] {msg}", file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_throughput(ms_local, updates_local, device):
    """Whole-job throughput of N independent replicas: the cell-updates of all
    ranks over the slowest rank's time.  Returns (updates/s, max ms)."""
    import torch
    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    u = torch.tensor([updates_local], dtype=torch.float64, device=device)
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(u, op=torch.distributed.ReduceOp.SUM)
    return u.item() / (t.item() * 1e-3), t.item()


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_state(n, seed, device, lib, runtime):
    fl = workloads.air_box(n, seed=seed)
    eos = fl.meta["eos"]
    m = workloads.make_mixture_struct(lib, eos, fl.meta["mix"])
    gh = runtime.load_mixture(eos, m)
    dev = fl.to_device(device)
    del fl
    workloads.derive_state(lib, dev, gh, runtime.stream_handle())
    return dev, gh, m


def choose_dt(dev, gh, lib, runtime):
    """min(CFL 0.8 acoustic step, 0.5 x fastest chemical time scale)."""
    import torch
    v = dev.view()
    out = torch.zeros(1, dtype=torch.float64, device=dev.device)
    s = runtime.stream_handle()
    abi.check(lib, lib.htr_CalculateMaxSpectralRadius(C.byref(v), dev.interior(), gh,
                                                      C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)), s), "cfl")
    abi.check(lib, lib.htr_InitializeTimeDerivatives(C.byref(v), dev.bounds(), 0, gh, s), "init")
    abi.check(lib, lib.htr_AddChemistrySources(C.byref(v), dev.interior(), gh, s), "chem")
    torch.cuda.synchronize()
    w = dev["Conserved_t"][..., :5].abs()
    rhoi = dev["Conserved"][..., :5]
    rho = dev["rho"][..., None]
    sig = rhoi > 1e-3 * rho
    tau = torch.where(sig, rhoi / w.clamp_min(1e-300), torch.full_like(rhoi, float("inf"))).min().item()
    return min(0.8 / out.item(), 0.5 * tau)


STAGE_KERNELS = ["prepass", "kg_faces_z", "kg_faces_y", "kg_faces_x", "teno_faces",
                 "diffusion_faces_z", "diffusion_faces_y", "diffusion_faces_x", "stage_update", "stage_transport"]


def kernel_profile(dev, gh, lib, runtime, dt, reps=3):
    """CUDA-event time of each kernel of one fused RHS stage (median of reps
    untimed stages, after the timed region), via htr_rk3_stage_profile."""
    from htr_gb300 import runtime as rt
    lib.htr_rk3_stage_profile.argtypes = [C.POINTER(abi.htr_fluid_view), abi.htr_rect3, abi.htr_rect3,
                                          C.POINTER(rt.htr_step_params), C.c_void_p, C.c_void_p, C.c_size_t,
                                          C.POINTER(C.c_float), C.c_void_p]
    lib.htr_rk3_stage_profile.restype = C.c_int
    v = dev.view()
    inner, fb = dev.interior(), dev.bounds()
    p = rt.htr_step_params(rt.SCHEMES["Hybrid"], 1.0, 0.0, dt, 1)
    nb = lib.htr_rk3_workspace_bytes(inner, gh)
    ws = rt._workspace.get(nb, dev.device)
    runs = []
    for _ in range(reps):
        out = (C.c_float * len(STAGE_KERNELS))()
        abi.check(lib, lib.htr_rk3_stage_profile(C.byref(v), inner, fb, C.byref(p), gh, C.c_void_p(ws), nb, out,
                                                 runtime.stream_handle()), "stage profile")
        runs.append(list(out))
    med = np.median(np.array(runs), axis=0)
    return {k: float(m) for k, m in zip(STAGE_KERNELS, med)}


# Algorithmic bytes per cell of each fused-stage kernel (5-species air; each
# value the kernel needs read once, each value it produces written once;
# face buffers hold 9 doubles per face, about one face per cell and direction)
NE, NS = 9, 5
KERNEL_BYTES = {
    # u, X, rhoE, p, rho, 3 metrics, 3 node types -> 9 gradients, MixW, H
    "prepass": 8 * (3 + NS + 1 + 1 + 1 + 3) + 3 * 4 + 8 * 11,
    # rho, p, H, Y, u, sensor, node type -> one face flux
    "kg_faces": 8 * (3 + NS + 3) + 1 + 4 + 8 * NE,
    # rhoYi, T, X, rho, mu, lam, Di, u, m_s, node type, 6 gradients, MixW -> face flux
    "diffusion_faces": 8 * (NS + 1 + NS + 1 + 1 + 1 + NS + 3 + 1 + 6 + 1) + 4 + 8 * NE,
    # 6 face fluxes/2 x 2 families, 6 metrics, Y, rho, p, T, Conserved_old, Conserved
    # -> Conserved_t, Conserved, T, p, rho, mu, lam, SoS, X, u, Di, Y
    "stage_update": 8 * (6 * NE + 6 + NS + 3 + 2 * NE) + 8 * (2 * NE + 6 + NS + 3 + NS + NS),
}
# Executed FP64 floating-point operations per cell (per face for the face
# kernels) of the same kernels: DADD + DMUL + 2 x DFMA thread instructions
# counted by ncu on the 96^3 case of this workload (profiles/
# stage_kernels_air96_hybrid.md, profiles/stage_update_transport_air96.md).  The kernels are bound by the FP64 pipe;
# this gives their achieved FP64 rate next to the memory roofline.
KERNEL_FP64_FLOPS = {"prepass": 80.0, "kg_faces": 168.0, "diffusion_faces": 320.0, "stage_update": 1289.0,
                     "stage_transport": 18.0}
# DRAM bytes per cell (dram__bytes_read.sum + dram__bytes_write.sum of one
# launch) measured by ncu on the 96^3 case (state larger than L2); the
# per-launch traffic scales with the cells (profiles/stage_kernels_air96_hybrid.md).
KERNEL_DRAM_BYTES = {"prepass": 248.0, "kg_faces": 124.0, "diffusion_faces": 316.0, "stage_update": 1202.0,
                     "stage_transport": 139.0}


STATE_FIELDS = ["Conserved", "pressure", "temperature", "MassFracs", "MolarFracs", "velocity",
                "rho", "mu", "lam", "Di", "SoS"]


def fp64_roofline(prof, dominant, fdom, ncell, fp64):
    """The dominant kernel against the FP64 pipe, the resource that bounds
    it: FP64 FLOP executed per cell (ncu DADD + DMUL + 2 DFMA counts,
    profiles/stage_kernels_air96_hybrid.md) x cells / its CUDA-event time,
    over the FP64 peak measured in this run by the DFMA-chain probe
    (MEASURED_PEAKS.json has no FP64 figure)."""
    flops = KERNEL_FP64_FLOPS.get(fdom)
    t = prof[dominant] * 1e-3
    achieved = flops * ncell / t / 1e12 if flops else None
    return {"bound": "fp64", "kernel": dominant, "achieved": achieved, "peak": fp64, "unit": "TFLOP/s",
            "frac": achieved / fp64 if (achieved and fp64) else None,
            "peak_source": "DFMA-chain probe run in this benchmark (libhtr_probe.so)",
            "flops_per_cell": flops, "cells": ncell, "launch_ms": prof[dominant],
            "flops_source": "ncu smsp__sass_thread_inst_executed_op_d{add,mul,fma} at 96^3, DFMA counted twice",
            "traffic": KERNEL_DRAM_BYTES[fdom] * ncell if fdom in KERNEL_DRAM_BYTES else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per cell at 96^3 x cells"}


def teno_face_fraction(dev, gh, lib, runtime):
    """Faces that the last fused hybrid stage (the kernel profile's)
    reconstructed with TENO, from the TENO queue counters, over all faces."""
    from htr_gb300 import runtime as rt
    inner = dev.interior()
    nb = lib.htr_rk3_workspace_bytes(inner, gh)
    ws = rt._workspace.get(nb, dev.device)
    c = (C.c_ulonglong * 3)()
    abi.check(lib, lib.htr_rk3_teno_face_counts(inner, gh, C.c_void_p(ws), nb, c, runtime.stream_handle()),
              "teno counts")
    n = [inner.hi[i] - inner.lo[i] + 1 for i in range(3)]
    faces = [(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2)) for d in range(3)]
    return {"value": sum(c) / sum(faces), "per_direction": [c[d] / faces[d] for d in range(3)],
            "teno_faces": [int(x) for x in c], "faces": faces,
            "note": "sensor-rejected faces of one fused hybrid stage of the timed state"}


def cpu_full_step(dev, gh, dt, runtime):
    """The CPU oracle (the port, all host threads) on one whole SSP-RK3 step
    of the benchmark's own grid and state (copied from the device), timed;
    the same step on the GPU from the same state is compared with it
    element by element (pointwise error over the bar max(1e-11 |cpu|,
    1e-12 max|cpu|))."""
    import torch

    import oracle
    port = oracle.port_lib()
    threads = os.cpu_count() or 1
    port.htr_oracle_set_threads(threads)
    host = dev.to_host()
    eos = abi.HTR_EOS_AIRMIX
    hp = oracle.load_mixture(port, eos, workloads.make_mixture_struct(port, eos, workloads.AIR_REF))
    t0 = time.perf_counter()
    oracle.step(port, host, hp, scheme="Hybrid", dt=dt, chemistry=True)
    el = time.perf_counter() - t0
    gpu = dev.copy()
    runtime.rk3_step(gpu, gh, dt=dt, chemistry=True)
    torch.cuda.synchronize()
    ratio = pointwise_ratio(gpu["Conserved"], host["Conserved"])
    flags = all(torch.equal(gpu[f"shockSensor{d}"].cpu(), torch.from_numpy(host[f"shockSensor{d}"])) for d in "XYZ")
    del gpu
    return {"value": 3.0 * dev.ncells / el, "unit": UNIT, "cores": threads, "kind": "port",
            "seconds": el, "same_config": True,
            "sample": f"one SSP-RK3 step (3 cell-updates per cell) of the benchmark's full "
                      f"{dev.nx}x{dev.ny}x{dev.nz} grid and state, OpenMP over all host threads",
            "parity": {"conserved_pointwise_ratio": ratio, "sensors_bit_exact": flags,
                       "note": "GPU step from the same state; ratio = max |gpu - cpu| / "
                               "max(1e-11 |cpu|, 1e-12 max|cpu| per component), <= 1 passes"}}


def pointwise_ratio(got, want):
    """max over elements of |got - want| / max(1e-11 |want|, 1e-12 max|want| of the component)."""
    import torch
    a = got.detach().cpu().double() if hasattr(got, "detach") else torch.from_numpy(np.asarray(got))
    b = want.detach().cpu().double() if hasattr(want, "detach") else torch.from_numpy(np.asarray(want))
    a = a.reshape(-1, a.shape[-1]) if a.dim() > 3 else a.reshape(-1, 1)
    b = b.reshape(-1, b.shape[-1]) if b.dim() > 3 else b.reshape(-1, 1)
    floor = 1e-12 * b.abs().max(dim=0).values
    bound = torch.maximum(1e-11 * b.abs(), floor[None, :])
    return float(((a - b).abs() / bound).max())


def e2e_pipelined(dev, gh, dt, steps, runtime, barrier, device):
    """End-to-end cell-updates/s through runtime.rk3_step with host state.

    Per step i (device state b = i % 2): the state fields are copied from
    pinned host memory on an H2D stream, the step runs on the compute stream
    once they have landed, and Conserved is read back on a D2H stream once the
    step is done.  The H2D copy of state b waits until the D2H copy of its
    previous step has finished.  The timed region spans the first H2D copy to
    the last D2H copy."""
    import torch
    devs = [dev, dev.copy()]
    host = {k: torch.empty_like(dev[k], device="cpu").pin_memory() for k in STATE_FIELDS}
    for k in STATE_FIELDS:
        host[k].copy_(dev[k])
    outs = [torch.empty_like(dev["Conserved"], device="cpu").pin_memory() for _ in range(2)]
    torch.cuda.synchronize()
    h2d = sum(host[k].numel() * host[k].element_size() for k in STATE_FIELDS)
    d2h = outs[0].numel() * outs[0].element_size()
    comp = torch.cuda.current_stream()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_done = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]
    n = max(6, steps)  # enough steps that the unhidden first copy and last read-back amortise
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(comp)
    s_in.wait_stream(comp)
    for i in range(n):
        b = i % 2
        with torch.cuda.stream(s_in):
            if i >= 2:
                s_in.wait_event(ev_out[b])
            for k in STATE_FIELDS:
                devs[b][k].copy_(host[k], non_blocking=True)
            ev_in[b].record(s_in)
        comp.wait_event(ev_in[b])
        runtime.rk3_step(devs[b], gh, dt=dt, chemistry=True, stream=comp)
        ev_done[b].record(comp)
        with torch.cuda.stream(s_out):
            s_out.wait_event(ev_done[b])
            outs[b].copy_(devs[b]["Conserved"], non_blocking=True)
            ev_out[b].record(s_out)
    comp.wait_stream(s_out)
    f1.record(comp)
    barrier()
    value, _ = replica_throughput(f0.elapsed_time(f1), 3.0 * dev.ncells * n, device)
    del devs[1]
    return value, h2d, d2h, n


def run_batched(args, device, runtime, lib, steps=3):
    """Batched 1-D shock tubes: every tube of one mixture packed into one strip,
    both strips advanced by one CUDA graph per SSP-RK3 step (fused stages);
    against the plain drop-in looped over the tubes (htr_rk3_step, one task
    kernel per reference task, on each tube in place).  A solve is one RK3
    step of one tube; both forms use the same per-mixture dt."""
    import torch
    insts = tubes.instances(args.tubes, seed=4242)
    stream = torch.cuda.current_stream()
    strips = []
    for eos in (abi.HTR_EOS_CONSTPROPMIX, abi.HTR_EOS_AIRMIX):
        group = [i for i in insts if i["eos"] == eos]
        if not group:
            continue
        host, offs = tubes.build_strip(group)
        m = workloads.make_mixture_struct(lib, eos, host.meta["mix"])
        gh = runtime.load_mixture(eos, m)
        dev = host.to_device(device)
        del host
        workloads.derive_state(lib, dev, gh, runtime.stream_handle())
        air = eos == abi.HTR_EOS_AIRMIX
        L = [i["L"] for i in group]
        # every tube its own step size: CFL 0.4 over its own spectral radius,
        # for air also at most half its fastest chemical time scale
        dts = tubes.strip_dts(dev, offs, [x + 2 for x in L], gh, cfl=tubes.TUBE_CFL, chemistry=air, lib=lib)
        dt_cell = torch.tensor(tubes.cell_dt(offs, [x + 2 for x in L], dts), dtype=torch.float64, device=device)
        strips.append(dict(dev=dev, gh=gh, dt=min(dts), dts=dts, dt_cell=dt_cell, offs=offs, L=L, chem=air))
    cells = sum(s["dev"].ncells for s in strips)
    ws = runtime.Workspace()
    ws.get(max(runtime.workspace_bytes(s["dev"], s["gh"]) for s in strips), device)
    # launch shapes for these strips (the arithmetic does not depend on them)
    from htr_gb300 import autotune
    default = autotune.get_tuning()
    log("batched: autotune")
    tuned, t_tuned, t_default, _ = autotune.autotune([(s["dev"], s["gh"], s["dt"], s["chem"]) for s in strips],
                                                     workspace=ws)

    def step_all(st):
        for s in strips:
            runtime.rk3_step_cells(s["dev"], s["gh"], s["dt_cell"], chemistry=s["chem"], stream=st, workspace=ws)

    log("batched: graph capture")
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        step_all(side)
    stream.wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side, capture_error_mode="relaxed"):
        step_all(side)
    graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        graph.replay()
    e1.record(stream)
    e1.synchronize()
    t_batched = e0.elapsed_time(e1) / steps
    # plain drop-in: htr_rk3_step on each tube, in place inside the strips
    p = runtime.htr_step_params
    used = C.c_double(0.0)
    sh = runtime.stream_handle()

    def loop_all():
        for s in strips:
            sv = s["dev"].view()
            for off, L, dt in zip(s["offs"], s["L"], s["dts"]):
                prm = p(runtime.SCHEMES["Hybrid"], 1.0, 0.0, dt, 1 if s["chem"] else 0)
                v, fb, inner = tubes.tube_view(sv, int(off), L)
                st = lib.htr_rk3_step(C.byref(v), inner, fb, C.byref(prm), s["gh"], C.byref(used), None, sh)
                if st:
                    abi.check(lib, st, "htr_rk3_step")

    log("batched: plain loop")
    loop_all()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    loop_all()
    f1.record(stream)
    f1.synchronize()
    t_plain = f0.elapsed_time(f1)
    n = len(insts)
    out = {"metric": "batched solves/s", "unit": "tube RK3 steps/s", "tubes": n, "cells": int(cells),
            "value": n / (t_batched * 1e-3), "ms_per_step": t_batched,
            "cell_updates_per_s": 3.0 * cells / (t_batched * 1e-3),
            "plain": {"value": n / (t_plain * 1e-3), "ms_per_step": t_plain,
                      "cell_updates_per_s": 3.0 * cells / (t_plain * 1e-3),
                      "form": "htr_rk3_step looped over the tubes (task kernels, one tube per call)"},
            "speedup_vs_plain": t_plain / t_batched,
            "autotune": {"tuning": tuned, "stage_ms_tuned": t_tuned, "stage_ms_default": t_default},
            "config": {"workload": f"{n} 1-D shock tubes, 128-8192 cells, gamma-1.4 gas or 5-species air "
                                   f"(1/2 each), staggered Dirichlet ends, hybrid scheme, SSP-RK3",
                       "form": "two strips (one per mixture), one CUDA graph per RK3 step, every tube "
                               "its own step size (htr_rk3_step_cells_ws)",
                       "dt": {("air" if s["chem"] else "gas"): [min(s["dts"]), max(s["dts"])] for s in strips}}}
    autotune.set_tuning(default)
    return out


def run_batched_mixed(device, runtime, lib, steps=5, seed=99):
    """Batched form with uneven shapes of both mixtures (batch.Batch): 512
    shock tubes (128-2048 cells, gas or air), 8 2-D vortex boxes (64^2 -
    256^2), 4 3-D Taylor-Green boxes (24^3 - 48^3) and 4 3-D reacting-air
    boxes (24^3 - 48^3), every instance its own step size, one CUDA graph
    launch per step; against the plain drop-in (htr_rk3_step, task kernels)
    looped over the instances.  A solve is one SSP-RK3 step of one
    instance."""
    import torch

    from htr_gb300 import batch
    rng = np.random.default_rng(seed)
    insts = [batch.tube_instance(i, device, lib) for i in tubes.instances(512, seed=seed, length=(128, 2048))]
    boxes = [workloads.vortex2d(int(rng.integers(64, 257)), seed=int(rng.integers(1 << 30))) for _ in range(8)]
    boxes += [workloads.taylor_green(int(rng.integers(24, 49)), seed=int(rng.integers(1 << 30))) for _ in range(4)]
    boxes += [workloads.air_box(int(rng.integers(24, 49)), seed=int(rng.integers(1 << 30))) for _ in range(4)]
    insts += [batch.box_instance(b, device, lib) for b in boxes]
    cells = sum(i["fluid"].ncells for i in insts)
    bt = batch.Batch(insts, device, tune=True)
    stream = torch.cuda.current_stream()
    bt.step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        bt.step()
    e1.record(stream)
    e1.synchronize()
    t_batch = e0.elapsed_time(e1) / steps
    p = runtime.htr_step_params
    used = C.c_double(0.0)
    sh = runtime.stream_handle()

    def loop_all():
        for i in insts:
            f = i["fluid"]
            prm = p(runtime.SCHEMES["Hybrid"], 1.0, 0.0, i["dt"], 1 if i["chemistry"] else 0)
            v = f.view()
            inner = f.interior((1, 0, 0)) if i["tube"] else f.interior()
            abi.check(lib, lib.htr_rk3_step(C.byref(v), inner, f.bounds(), C.byref(prm), i["gh"], C.byref(used),
                                            None, sh), "htr_rk3_step")

    loop_all()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    loop_all()
    f1.record(stream)
    f1.synchronize()
    t_plain = f0.elapsed_time(f1)
    n = len(insts)
    return {"metric": "batched solves/s", "unit": "instance RK3 steps/s", "instances": n, "cells": int(cells),
            "value": n / (t_batch * 1e-3), "ms_per_step": t_batch,
            "cell_updates_per_s": 3.0 * cells / (t_batch * 1e-3),
            "plain": {"value": n / (t_plain * 1e-3), "ms_per_step": t_plain,
                      "cell_updates_per_s": 3.0 * cells / (t_plain * 1e-3)},
            "speedup_vs_plain": t_plain / t_batch, "gpu_launches_per_step": bt.launches_per_step(),
            "autotune": bt.tunings,
            "config": {"workload": "512 shock tubes (128-2048 cells, gas or air) + 8 vortex boxes (64^2-256^2) + "
                                   "4 Taylor-Green boxes (24^3-48^3) + 4 reacting-air boxes (24^3-48^3)",
                       "form": "tubes in one strip per mixture, boxes as their own fused steps, one CUDA graph "
                               "with one branch per strip and box, one launch per step, per-instance dt"}}


def run_served(args, device, rate=200.0):
    """Served mix: Poisson arrivals (`rate` per s) of 1-D tubes (256-8192
    cells), 2-D vortex boxes (64^2-512^2) and 3-D reacting-air boxes
    (32^3-96^3), each submitted with its initial state (generated before the
    session) and asking for 20-100 RK3 steps (the served configuration's
    100-2000 scaled by 1/20 so the run stays bounded).  The server
    (continuous batching: the tubes of one mixture stepped together in one
    strip, the boxes as per-request CUDA graphs, on 8 streams; each round
    steps the boxes with the least remaining work up to --serve-round-cells
    cells; 150 GB budget)
    against the plain per-request path (one request at a time, task
    kernels)."""
    mix = serve.prepare(serve.request_mix(args.serve, rate=rate, seed=777, steps=(20, 100), tube=(256, 8192),
                                          vortex=(64, 512), box=(32, 96)))
    # warm the library, the allocator and the host-state generators
    warm = serve.request_mix(3, rate=1e6, seed=1, steps=(1, 1), tube=(64, 64), vortex=(16, 16), box=(8, 8))
    serve.Server(device=device, streams=2).run(warm)
    serve.run_plain([serve.Request(r.rid, r.kind, r.size, r.seed, r.steps, 0.0) for r in warm], device=device)
    log("served: server")
    rc = args.serve_round_cells if args.serve_round_cells > 0 else None
    server = serve.Server(device=device, hbm_budget=150e9, streams=8, round_cells=rc)
    t0 = time.perf_counter()
    server.run(mix)
    t_srv = time.perf_counter() - t0
    log("served: plain path")
    plain = [serve.Request(r.rid, r.kind, r.size, r.seed, r.steps, r.arrival, state=r.state) for r in mix]
    t0 = time.perf_counter()
    serve.run_plain(plain, device=device)
    t_plain = time.perf_counter() - t0
    a, b = serve.summary(mix, t_srv), serve.summary(plain, t_plain)
    cells = sum(int(np.prod(serve._grid(r)[:3])) * r.steps * 3 for r in mix)
    return {"metric": "served solves/s", "unit": "requests/s", "value": a["solves_per_s"],
            "tts_p50_s": a["tts_p50_s"], "tts_p99_s": a["tts_p99_s"],
            "cell_updates_per_s": cells / t_srv, "peak_reserved_bytes": server.peak,
            "plain": {"value": b["solves_per_s"], "tts_p50_s": b["tts_p50_s"], "tts_p99_s": b["tts_p99_s"],
                      "cell_updates_per_s": cells / t_plain},
            "speedup_vs_plain": t_plain / t_srv,
            "config": {"requests": len(mix), "arrival_rate_per_s": rate, "steps": [20, 100], "round_cells": rc,
                       "kinds": {k: sum(r.kind == k for r in mix) for k in ("tube", "vortex", "box")},
                       "sizes": {"tube": [256, 8192], "vortex": [64, 512], "box": [32, 96]},
                       "note": "steps scaled by 1/20 from the served configuration to bound the run; "
                               "each request carries its host initial state; both timings include "
                               "H2D, state derivation, dt, the steps and the D2H of the result"}}


def run_wall(args, device, runtime, lib):
    """Wall-bounded boundary layer: Mach-6 5-species air on a tanh-stretched
    grid (interior cells --wall), NSCBC inflow / outflow in x, isothermal
    wall and outflow in y, periodic z; TENO-LAD Euler flux, diffusion and
    explicit chemistry.  Each SSP-RK3 step runs the task entry points in the
    reference driver's order over the reference's zones (wall.BoundaryRun):
    per stage 3 Euler + 3 diffusion + chemistry kernels, the NSCBC terms of
    both outflows (with the interior's maximum Mach number, read back) and of
    the inflow, the RK update and the boundary-state refresh."""
    import torch
    from htr_gb300 import wall
    num = tuple(int(x) for x in args.wall.split(","))
    host = wall.boundary_layer(num=num, seed=77)
    g, bc = host.meta["grid"], host.meta["bc"]
    m = workloads.make_mixture_struct(lib, host.meta["eos"], host.meta["mix"])
    gh = runtime.load_mixture(host.meta["eos"], m)
    dev = host.to_device(device)
    del host
    g.fill(dev, lib)
    workloads.derive_state(lib, dev, gh, runtime.stream_handle())
    mach = torch.zeros(1, dtype=torch.float64, device=device)
    tasks = wall.BoundaryRun(lib, dev, gh, bc, stream=runtime.stream_handle(), max_mach_buffer=mach)
    fused = wall.FusedBoundaryRun(dev, gh, bc)
    dt = tasks.spectral_dt(0.8)
    stream = torch.cuda.current_stream()
    cells = num[0] * num[1] * num[2]
    start = {k: a.clone() for k, a in dev.arrays.items()}

    def timed(step):
        for k, a in dev.arrays.items():
            a.copy_(start[k])
        step(dt)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.wall_steps):
            step(dt)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), bool(torch.isfinite(dev["Conserved"]).all().item())

    ms_t, fin_t = timed(tasks.step)
    ms_f, fin_f = timed(lambda d: fused.step(d))
    # the same grid with the hybrid scheme (HTR's own boundary-layer cases),
    # fused boundary step, for comparison
    hyb = wall.FusedBoundaryRun(dev, gh, bc, scheme="Hybrid", workspace=fused.ws)
    ms_h, fin_h = timed(lambda d: hyb.step(d))
    cpu = None
    if args.cpu_baseline:
        # one step of the full grid on the CPU oracle (the port, all host
        # threads), from the same start state, against the fused GPU step
        import oracle
        log("wall: CPU baseline, one step of the full grid on the port")
        for k, a_ in dev.arrays.items():
            a_.copy_(start[k])
        torch.cuda.synchronize()
        ref = dev.to_host()
        port = oracle.port_lib()
        threads = os.cpu_count() or 1
        port.htr_oracle_set_threads(threads)
        eos = abi.HTR_EOS_AIRMIX
        hp = oracle.load_mixture(port, eos, workloads.make_mixture_struct(port, eos, workloads.AIR_REF))
        t0 = time.perf_counter()
        oracle.boundary_layer_step(port, ref, hp, dt, bc["xNeg"][1]["P"], bc["xPos"][1]["P"],
                                   (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"]))
        el = time.perf_counter() - t0
        fused.step(dt)
        torch.cuda.synchronize()
        cpu = {"value": 3.0 * cells / el, "unit": UNIT, "cores": threads, "kind": "port", "seconds": el,
               "same_config": True,
               "sample": f"one boundary-layer SSP-RK3 step of the full {num[0]}x{num[1]}x{num[2]} interior "
                         f"(TENO-LAD), the reference driver's task order over its zones",
               "parity": {"conserved_pointwise_ratio": pointwise_ratio(dev["Conserved"], ref["Conserved"]),
                          "note": "fused GPU step from the same state"}}
        del ref
    del start
    # task path kernels per stage: time derivatives, chemistry, 3 Euler, 3
    # diffusion, 2 x (max Mach), 2 outflow, 1 inflow, RK update, primitives,
    # 3 boundary states, wall, properties, 4 slabs of conserved variables
    per_stage_t = 2 + 3 + 3 + 2 + 2 + 1 + 1 + 1 + 3 + 1 + 1 + len(tasks.all_bcs)
    # fused: 3 plane zeroings, 2 max Mach, 2 outflow, 1 inflow, prepass,
    # 3 TENO face kernels (one per direction), 3 diffusion faces, update,
    # 3 wall kernels
    per_stage_f = 3 + 2 + 2 + 1 + 1 + 3 + 3 + 1 + 3
    best = "fused" if ms_f <= ms_t else "tasks"
    ms = min(ms_f, ms_t)
    return {"value": 3.0 * cells * args.wall_steps / (ms * 1e-3), "unit": UNIT,
            "ms_per_step": ms / args.wall_steps, "steps": args.wall_steps, "dt": dt, "finite": fin_t and fin_f,
            "path": best,
            "tasks": {"value": 3.0 * cells * args.wall_steps / (ms_t * 1e-3), "ms_per_step": ms_t / args.wall_steps,
                      "gpu_launches": args.wall_steps * (3 * per_stage_t + 2)},
            "fused": {"value": 3.0 * cells * args.wall_steps / (ms_f * 1e-3), "ms_per_step": ms_f / args.wall_steps,
                      "gpu_launches": args.wall_steps * (3 * per_stage_f + 2)},
            "hybrid_fused": {"value": 3.0 * cells * args.wall_steps / (ms_h * 1e-3),
                             "ms_per_step": ms_h / args.wall_steps, "finite": fin_h,
                             "note": "same grid and state, hybrid TENO/KG scheme instead of TENO-LAD"},
            "config": {"workload": "Mach-6 boundary layer, 5-species air (AirMix), tanh-stretched wall-normal "
                                   "grid, NSCBC inflow/outflow x, isothermal wall + outflow y, periodic z, "
                                   "TENO-LAD + diffusion + explicit chemistry, SSP-RK3",
                       "interior_cells": list(num), "grid_with_ghosts": list(g.shape), "cells": cells,
                       "tasks": "task entry points in the reference driver's order over its zones",
                       "fused": "htr_rk3_step_bc_ws: fused stage pipeline with the boundary rules"},
            "gpu_launches": args.wall_steps * (3 * (per_stage_f if best == "fused" else per_stage_t) + 2),
            **({"cpu": cpu} if cpu else {})}


def run_config1(args, device, runtime, lib, steps=200):
    """The plain small configuration: 32^3 periodic Taylor-Green box of a
    calorically perfect gas (gamma 1.4, Pr 0.71, power-law viscosity), +-1 %
    seeded perturbations, hybrid scheme with the Ducros / TENO-A sensor,
    viscous diffusion, SSP-RK3 at CFL 0.8 (dt fixed from the initial state).
    GPU: the fused step (a 32^3 grid is launch-latency bound, so the steps
    are replayed from one CUDA graph) timed over `steps` steps; against HBM
    at the reference layout's 263 B per single-species cell-update.  CPU:
    the port on all host threads, one step of the same grid and state, and
    the pointwise comparison of that step with the GPU's."""
    import torch

    import oracle
    fl = workloads.taylor_green(32, seed=0)
    eos = fl.meta["eos"]
    m = workloads.make_mixture_struct(lib, eos, fl.meta["mix"])
    gh = runtime.load_mixture(eos, m)
    dev = fl.to_device(device)
    workloads.derive_state(lib, dev, gh, runtime.stream_handle())
    dt = runtime.stable_dt(dev, gh, cfl=0.8, chemistry=False)
    start = dev.copy()
    ws = runtime.Workspace()
    stream = torch.cuda.current_stream()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        runtime.rk3_step(dev, gh, dt=dt, chemistry=False, stream=side, workspace=ws)
    stream.wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side, capture_error_mode="relaxed"):
        runtime.rk3_step(dev, gh, dt=dt, chemistry=False, stream=side, workspace=ws)
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        graph.replay()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    value = 3.0 * dev.ncells / (ms * 1e-3)
    peak, src = hbm_peak()
    gbs = 263.0 * value / 1e9
    # one step from the same start state on the GPU and on the port
    port = oracle.port_lib()
    threads = os.cpu_count() or 1
    port.htr_oracle_set_threads(threads)
    host = start.to_host()
    hp = oracle.load_mixture(port, eos, workloads.make_mixture_struct(port, eos, fl.meta["mix"]))
    t0 = time.perf_counter()
    oracle.step(port, host, hp, scheme="Hybrid", dt=dt, chemistry=False)
    el = time.perf_counter() - t0
    runtime.rk3_step(start, gh, dt=dt, chemistry=False)
    torch.cuda.synchronize()
    ratio = pointwise_ratio(start["Conserved"], host["Conserved"])
    flags = all(torch.equal(start[f"shockSensor{d}"].cpu(), torch.from_numpy(host[f"shockSensor{d}"])) for d in "XYZ")
    return {"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms, "steps": steps, "dt": dt,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "bytes_per_cell_update": 263, "peak_source": src + " (MEASURED_PEAKS.json)",
                         "note": "whole step at the reference layout's compulsory bytes; a 32^3 grid "
                                 "(33k cells) cannot fill 152 SMs, the steps are latency bound"},
            "cpu_baseline": {"value": 3.0 * host.ncells / el, "unit": UNIT, "cores": threads, "kind": "port",
                             "seconds": el, "sample": "one SSP-RK3 step of the same 32^3 grid and state"},
            "parity": {"conserved_pointwise_ratio": ratio, "sensors_bit_exact": flags},
            "config": {"workload": "32^3 periodic Taylor-Green, calorically perfect gas (ConstPropMix), "
                                   "hybrid TENO-A/KG + viscous diffusion, SSP-RK3 at CFL 0.8",
                       "form": "fused step, one CUDA graph replayed per step"}}


def run_restart(dev, device, reps=3):
    """Restart dump and load of the benchmark state through
    include/htr_restart.h (2 tiles plus master.hdf in a temporary
    directory): seconds and GB/s of restart fields, median of `reps`."""
    import shutil
    import tempfile

    import torch
    from htr_gb300 import fluid, restart
    back = fluid.Fluid(dev.shape, dev.nspec, device=device, fields=list(restart.IO_FIELDS))
    nbytes = sum(dev.arrays[k].numel() * 8 for k in restart.IO_FIELDS)
    base = tempfile.mkdtemp(prefix="htr_restart_")
    dump_s, load_s, equal, fbytes = [], [], True, 0
    try:
        for rep in range(reps):
            d = os.path.join(base, f"fluid_iter{rep:010d}")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            restart.dump(d, dev, tiles=(1, 1, 2), time_step=rep)
            t1 = time.perf_counter()
            for k in restart.IO_FIELDS:
                back.arrays[k].zero_()
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            restart.load(d, back)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            equal = equal and all(torch.equal(dev.arrays[k], back.arrays[k]) for k in restart.IO_FIELDS)
            fbytes = sum(os.path.getsize(os.path.join(d, x)) for x in os.listdir(d))
            dump_s.append(t1 - t0)
            load_s.append(t3 - t2)
            shutil.rmtree(d)
    finally:
        shutil.rmtree(base, ignore_errors=True)
    md, ml = sorted(dump_s)[len(dump_s) // 2], sorted(load_s)[len(load_s) // 2]
    return {"field_bytes": nbytes, "file_bytes": fbytes, "tiles": [1, 1, 2], "dump_s": md, "load_s": ml,
            "dump_gbps": nbytes / md / 1e9, "load_gbps": nbytes / ml / 1e9, "bit_identical": equal,
            "note": "host wall clock, device synchronised on both sides; files in the page cache (no fsync)"}


def fp64_peak(_lib=None):
    """FP64 TFLOP/s of the device, measured by the DFMA-chain probe of
    libhtr_probe.so (a benchmark library, not the product)."""
    from htr_gb300 import build as pkg_build
    if not os.path.exists(pkg_build.PROBE_LIB):
        return None
    lib = C.CDLL(pkg_build.PROBE_LIB)
    lib.htr_probe_fp64_tflops.argtypes = [C.c_int, C.POINTER(C.c_double)]
    lib.htr_probe_fp64_tflops.restype = C.c_int
    t = C.c_double(0)
    if lib.htr_probe_fp64_tflops(200000, C.byref(t)) != 0:
        return None
    return t.value


def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    from htr_gb300 import runtime
    lib = runtime.lib()
    log("building the state")
    dev, gh, mstruct = build_state(args.n, 1234 + rank, device, lib, runtime)
    ncell = dev.ncells
    dt = choose_dt(dev, gh, lib, runtime)
    stream = torch.cuda.current_stream()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    log("warm-up")
    for _ in range(args.warmup):
        runtime.rk3_step(dev, gh, dt=dt, chemistry=True)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        runtime.rk3_step(dev, gh, dt=dt, chemistry=True)
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    value, ms_max = replica_throughput(ms, 3.0 * ncell * args.steps, device)

    # end-to-end through the public API with pinned host buffers: every step
    # copies the time-dependent state host -> device, runs the step and reads
    # Conserved back.  Two device states alternate so that the copies of one
    # step overlap the compute of the previous one (copy streams + events).
    log("end-to-end")
    clocks_e2e = ClockSampler(local)
    clocks_e2e.start()
    e2e_value, h2d, d2h, e2e_steps = e2e_pipelined(dev, gh, dt, args.steps, runtime, barrier, device)
    clk_e2e = clocks_e2e.stop()

    result = None
    if rank == 0:
        log("kernel profile")
        prof = kernel_profile(dev, gh, lib, runtime, dt)
        teno = teno_face_fraction(dev, gh, lib, runtime)
        dominant = max(prof, key=prof.get)
        fdom = dominant.rsplit("_", 1)[0] if dominant[-2:] in ("_x", "_y", "_z") else dominant
        peak, peak_src = hbm_peak()
        fp64 = fp64_peak(lib)
        roof = fp64_roofline(prof, dominant, fdom, ncell, fp64)
        # the step as a whole against HBM, at the reference layout's
        # compulsory 495 B per cell-update
        step_gbs = BYTES_PER_CELL_UPDATE_AIR * 3.0 * ncell / (ms_max / args.steps * 1e-3) / 1e9
        roof["hbm"] = {"bytes_per_cell_update": BYTES_PER_CELL_UPDATE_AIR, "achieved": step_gbs, "peak": peak,
                       "unit": "GB/s", "frac": step_gbs / peak, "peak_source": peak_src + " (MEASURED_PEAKS.json)",
                       "of": "whole SSP-RK3 step: 3 cell-updates per cell per step x 495 B / step time",
                       "kernel_traffic_bytes_per_cell": KERNEL_DRAM_BYTES.get(fdom),
                       "kernel_hbm_frac": (KERNEL_DRAM_BYTES[fdom] * ncell / (prof[dominant] * 1e-3) / 1e9 / peak
                                           if fdom in KERNEL_DRAM_BYTES else None)}
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"periodic {args.n}^3 box, 5-species air (AirMix), hybrid TENO/KG + "
                                   f"diffusion + explicit chemistry, SSP-RK3",
                       "grid": [args.n] * 3, "cells": ncell, "species": 5, "scheme": "Hybrid",
                       "chemistry": "explicit", "rk_stages_per_step": 3, "dt": dt,
                       "l2": "inputs larger than L2 (state ~%.1f GB)" % (ncell * 480 / 1e9),
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                    "copies": "11 state fields H2D and Conserved D2H every step, pinned host memory, "
                              "double-buffered on copy streams overlapping the previous step",
                    "clocks": clk_e2e},
            "roofline": roof,
            "teno_face_fraction": teno,
            "kernel_ms_per_stage": prof,
            # per step: Ducros + shock sensors + Conserved_old copy, then per stage
            # prepass, 3 KG, 3 TENO (one per direction's queue), 3 diffusion, 1 update
            "gpu_launches": args.steps * (3 + 3 * 11),
            "clocks": clk,
        }
        if args.config1:
            try:
                log("config 1: 32^3 Taylor-Green")
                result["config1"] = run_config1(args, device, runtime, lib)
            except Exception as exc:
                result["config1"] = {"error": f"{type(exc).__name__}: {exc}"}
        if args.tubes > 0:
            try:
                log("batched tubes")
                result["batched"] = run_batched(args, device, runtime, lib)
            except Exception as exc:  # the headline line must still print
                result["batched"] = {"error": f"{type(exc).__name__}: {exc}"}
            try:
                log("batched mixed shapes")
                result["batched"]["mixed"] = run_batched_mixed(device, runtime, lib)
            except Exception as exc:
                result["batched"]["mixed"] = {"error": f"{type(exc).__name__}: {exc}"}
        if args.serve > 0:
            rates = [float(r) for r in args.serve_rates.split(",")]
            try:
                log(f"served mix at {rates[0]}/s")
                result["served"] = run_served(args, device, rates[0])
                if len(rates) > 1:
                    result["served"]["rates"] = {}
                    for r in rates[1:]:
                        log(f"served mix at {r}/s")
                        res = run_served(args, device, r)
                        result["served"]["rates"][str(r)] = {k: res[k] for k in ("value", "tts_p50_s", "tts_p99_s",
                                                                                 "speedup_vs_plain", "plain")}
            except Exception as exc:
                result["served"] = {"error": f"{type(exc).__name__}: {exc}"}
        if args.wall:
            try:
                log("wall-bounded boundary layer")
                result["wall"] = run_wall(args, device, runtime, lib)
            except Exception as exc:
                result["wall"] = {"error": f"{type(exc).__name__}: {exc}"}
        if args.restart:
            try:
                log("restart dump/load")
                result["restart"] = run_restart(dev, device)
            except Exception as exc:
                result["restart"] = {"error": f"{type(exc).__name__}: {exc}"}
        if args.cpu_baseline:
            log("CPU baseline: one SSP-RK3 step of the full grid on the port")
            result["cpu_baseline"] = cpu_full_step(dev, gh, dt, runtime)
            if isinstance(result.get("wall"), dict) and "cpu" in result["wall"]:
                result["cpu_baseline"]["wall"] = result["wall"].pop("cpu")
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return result


def cpu_choose_dt(lib, fl, h):
    """choose_dt on a host grid with a CPU library."""
    import oracle
    dt = oracle.spectral_dt(lib, fl, h, 0.8)
    v = fl.view()
    abi.check(lib, lib.htr_InitializeTimeDerivatives(C.byref(v), fl.bounds(), 0, h, None), "init")
    abi.check(lib, lib.htr_AddChemistrySources(C.byref(v), fl.interior(), h, None), "chem")
    w = np.abs(fl["Conserved_t"][..., :5])
    rhoi = fl["Conserved"][..., :5]
    sig = rhoi > 1e-3 * fl["rho"][..., None]
    with np.errstate(divide="ignore"):
        tau = np.where(sig, rhoi / np.maximum(w, 1e-300), np.inf).min()
    return min(dt, 0.5 * float(tau))


def run_reference(args):
    """Reference arm: the reference's CPU implementation of the path on the
    host cores, on this benchmark's own grid and seeded state (args.n^3
    5-species air, the GPU arm's rank-0 seed): the reference's compiled CPU
    tasks where they were built from the reference sources (oracle/_ref),
    else their bit-exact restatement, the port (the GPU machine, where the
    reference sources are not present).  One step of this arm is one SSP-RK3
    stage over the whole grid, in the reference driver's order: the shock
    sensors and Conserved_old at the first stage of every three, zeroed time
    derivatives, chemistry sources, Euler Z, Y, X, diffusion Z, Y, X, the RK
    update and the primitive / property refresh -- one cell-update of every
    cell -- so that W + K steps of the full grid fit in a few minutes.
    value = cells / median stage time."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    import oracle
    eos = abi.HTR_EOS_AIRMIX
    lib, kind = oracle.ref_lib(eos), "reference"
    threads = os.cpu_count() or 1
    if lib is None:
        lib, kind = oracle.port_lib(), "port"
        lib.htr_oracle_set_threads(threads)
    else:
        os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    log(f"reference arm ({kind}): building the {args.n}^3 state")
    fl = workloads.air_box(args.n, seed=1234)
    h = oracle.load_mixture(lib, eos, workloads.make_mixture_struct(lib, eos, fl.meta["mix"]))
    workloads.derive_state(lib, fl, h)
    dt = cpu_choose_dt(lib, fl, h)
    v = fl.view()
    times = []
    for i in range(args.warmup + args.steps):
        stage = i % 3 + 1
        t0 = time.perf_counter()
        if stage == 1:
            oracle.update_sensors(lib, fl, h, 1.0)
            abi.check(lib, lib.htr_InitializeTemporaries(C.byref(v), fl.bounds(), h, None), "tmp")
        oracle.update_derivatives(lib, fl, h, stage, dt, "Hybrid", True)
        abi.check(lib, lib.htr_UpdateVars(C.byref(v), fl.interior(), stage, dt, 0, h, None), "rk")
        oracle.refresh(lib, fl, h)
        el = time.perf_counter() - t0
        log(f"reference arm: step {i} (stage {stage}) {el:.2f} s")
        if i >= args.warmup:
            times.append(el)
    t = float(np.median(times))
    value = fl.ncells / t
    sample = (f"{args.steps} timed SSP-RK3 stages (after {args.warmup} untimed) of the full {args.n}^3 grid, "
              f"one cell-update of every cell each, median {t:.2f} s; OpenMP over {threads} host threads")
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"periodic {args.n}^3 box, 5-species air (AirMix), hybrid TENO/KG + "
                                   f"diffusion + explicit chemistry, SSP-RK3", "grid": [args.n] * 3,
                       "cells": fl.ncells, "dt": dt, "step": "one SSP-RK3 stage (1 cell-update per cell)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=256)
    p.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    p.add_argument("--tubes", type=int, default=4096, help="batched shock tubes (0: skip)")
    p.add_argument("--serve", type=int, default=32, help="served requests (0: skip)")
    p.add_argument("--serve-rates", default="200,50,2000",
                   help="Poisson arrival rates per s of the served mix, first reported")
    p.add_argument("--serve-round-cells", type=float, default=2e6,
                   help="cells of the boxes stepped per server round, least remaining work first (0: all)")
    p.add_argument("--wall", default="512,192,128", help="boundary-layer interior cells nx,ny,nz ('' skips)")
    p.add_argument("--wall-steps", type=int, default=10)
    p.add_argument("--no-restart", dest="restart", action="store_false", help="skip the restart dump/load timing")
    p.add_argument("--no-config1", dest="config1", action="store_false", help="skip the 32^3 Taylor-Green case")
    args = p.parse_args()
    res = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
