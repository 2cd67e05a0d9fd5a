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
                 "diffusion_faces_z", "diffusion_faces_y", "diffusion_faces_x", "stage_update"]


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
# stage_kernels_air96_hybrid.md).  The kernels are bound by the FP64 pipe;
# this gives their achieved FP64 rate next to the memory roofline.
KERNEL_FP64_FLOPS = {"prepass": 80.0, "kg_faces": 259.0, "diffusion_faces": 320.0, "stage_update": 2559.0}
# DRAM bytes per cell (dram__bytes_read.sum + dram__bytes_write.sum of one
# launch) measured by ncu on the 96^3 case (state larger than L2); the
# per-launch traffic scales with the cells (profiles/stage_kernels_air96_hybrid.md).
KERNEL_DRAM_BYTES = {"prepass": 248.0, "kg_faces": 124.0, "diffusion_faces": 316.0, "stage_update": 1029.0}


STATE_FIELDS = ["Conserved", "pressure", "temperature", "MassFracs", "MolarFracs", "velocity",
                "rho", "mu", "lam", "Di", "SoS"]


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
        if air:
            dt = choose_dt(dev, gh, lib, runtime)
        else:
            out = torch.zeros(1, dtype=torch.float64, device=device)
            v = dev.view()
            abi.check(lib, lib.htr_CalculateMaxSpectralRadius(
                C.byref(v), dev.interior(), gh, C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)),
                runtime.stream_handle()), "cfl")
            dt = 0.8 / out.item()
        strips.append(dict(dev=dev, gh=gh, dt=dt, offs=offs, L=[i["L"] for i in group], chem=air))
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
            runtime.rk3_step(s["dev"], s["gh"], dt=s["dt"], chemistry=s["chem"], stream=st, workspace=ws)

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
            prm = p(runtime.SCHEMES["Hybrid"], 1.0, 0.0, s["dt"], 1 if s["chem"] else 0)
            sv = s["dev"].view()
            for off, L in zip(s["offs"], s["L"]):
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
                       "form": "two strips (one per mixture), one CUDA graph per RK3 step",
                       "dt": {("air" if s["chem"] else "gas"): s["dt"] for s in strips}}}
    autotune.set_tuning(default)
    return out


def run_served(args, device):
    """Served mix: Poisson arrivals (200/s) of 1-D tubes (256-8192 cells), 2-D
    vortex boxes (64^2-512^2) and 3-D reacting-air boxes (32^3-96^3), each
    submitted with its initial state (generated before the session) and
    asking for 20-100 RK3 steps (the served configuration's 100-2000 scaled by
    1/20 so the run stays bounded).  The server (continuous batching,
    per-request CUDA graphs on 8 streams, 150 GB budget) against the plain
    per-request path (one request at a time, task kernels)."""
    mix = serve.prepare(serve.request_mix(args.serve, rate=200.0, seed=777, steps=(20, 100), tube=(256, 8192),
                                          vortex=(64, 512), box=(32, 96)))
    # warm the library, the allocator and the host-state generators
    warm = serve.request_mix(3, rate=1e6, seed=1, steps=(1, 1), tube=(64, 64), vortex=(16, 16), box=(8, 8))
    serve.Server(device=device, streams=2).run(warm)
    serve.run_plain([serve.Request(r.rid, r.kind, r.size, r.seed, r.steps, 0.0) for r in warm], device=device)
    log("served: server")
    server = serve.Server(device=device, hbm_budget=150e9, streams=8)
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
            "config": {"requests": len(mix), "arrival_rate_per_s": 200.0, "steps": [20, 100],
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
            "gpu_launches": args.wall_steps * (3 * (per_stage_f if best == "fused" else per_stage_t) + 2)}


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


def fp64_peak(lib):
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
    e2e_value, h2d, d2h, e2e_steps = e2e_pipelined(dev, gh, dt, args.steps, runtime, barrier, device)

    result = None
    if rank == 0:
        log("kernel profile")
        prof = kernel_profile(dev, gh, lib, runtime, dt)
        dominant = max(prof, key=prof.get)
        fdom = dominant.rsplit("_", 1)[0] if dominant[-2:] in ("_x", "_y", "_z") else dominant
        peak, peak_src = hbm_peak()
        per_cell = KERNEL_BYTES.get(fdom)
        bytes_launch = per_cell * ncell if per_cell is not None else None
        achieved = bytes_launch / (prof[dominant] * 1e-3) / 1e9 if bytes_launch else None
        fp64 = fp64_peak(lib)
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
                              "double-buffered on copy streams overlapping the previous step"},
            "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                         "peak_source": peak_src,
                         "traffic": KERNEL_DRAM_BYTES[fdom] * ncell if fdom in KERNEL_DRAM_BYTES else None,
                         "traffic_source": "ncu DRAM bytes per cell at 96^3 x cells", "bytes_per_launch": bytes_launch,
                         "bytes_per_cell": per_cell, "launch_ms": prof[dominant]},
            "fp64": {"peak_tflops_probe": fp64, "note": "measured in this run by a DFMA-chain probe",
                     "kernel": dominant,
                     "flops_per_cell": KERNEL_FP64_FLOPS.get(fdom),
                     "achieved_tflops": (KERNEL_FP64_FLOPS[fdom] * ncell / (prof[dominant] * 1e-3) / 1e12
                                         if fdom in KERNEL_FP64_FLOPS else None),
                     "frac": (KERNEL_FP64_FLOPS[fdom] * ncell / (prof[dominant] * 1e-3) / 1e12 / fp64
                              if fdom in KERNEL_FP64_FLOPS and fp64 else None),
                     "bound": "fp64 pipe (DADD/DMUL/DFMA plus compares, conversions and the "
                              "division/sqrt sequences)"},
            "kernel_ms_per_stage": prof,
            # per step: Ducros + shock sensors + Conserved_old copy, then per stage
            # prepass, 3 KG, 3 TENO (one per direction's queue), 3 diffusion, 1 update
            "gpu_launches": args.steps * (3 + 3 * 11),
            "clocks": clk,
        }
        if args.tubes > 0:
            try:
                log("batched tubes")
                result["batched"] = run_batched(args, device, runtime, lib)
            except Exception as exc:  # the headline line must still print
                result["batched"] = {"error": f"{type(exc).__name__}: {exc}"}
        if args.serve > 0:
            try:
                log("served mix")
                result["served"] = run_served(args, device)
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
            log("CPU baseline")
            result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return result


def cpu_baseline(budget_s=20.0, n=48, wall_num=(64, 48, 32)):
    """The CPU oracle (all host threads) on a bounded sample of the same workload:
    whole SSP-RK3 steps (sensors, 3 x (chemistry, Euler Z/Y/X, diffusion Z/Y/X,
    RK update, primitive and property refresh)) of an n^3 box, the same work
    per cell-update as the GPU step."""
    import oracle
    lib = oracle.ref_lib(abi.HTR_EOS_AIRMIX)
    kind = "reference"
    if lib is None:
        lib = oracle.port_lib()
        kind = "port"
    threads = os.cpu_count() or 1
    if kind == "port":
        lib.htr_oracle_set_threads(threads)
    fl = workloads.air_box(n, seed=1234)
    m = workloads.make_mixture_struct(lib, abi.HTR_EOS_AIRMIX, fl.meta["mix"])
    h = oracle.load_mixture(lib, abi.HTR_EOS_AIRMIX, m)
    workloads.derive_state(lib, fl, h)
    steps = 0
    t0 = time.perf_counter()
    while True:
        oracle.step(lib, fl, h, dt=1e-9, chemistry=True)
        steps += 1
        if time.perf_counter() - t0 > budget_s or steps >= 200:
            break
    el = time.perf_counter() - t0
    out = {"value": 3.0 * steps * fl.ncells / el, "unit": UNIT, "cores": threads, "kind": kind,
           "sample": f"{steps} SSP-RK3 steps (3 cell-updates per cell each) of a {n}^3 box of the same "
                     f"workload, {el:.1f} s, OpenMP over all host threads"}
    if wall_num:
        out["wall"] = cpu_wall_baseline(lib, kind, wall_num, budget_s=budget_s / 2)
    return out


def cpu_wall_baseline(lib, kind, num, budget_s=10.0):
    """The boundary-layer step (task composition of wall.BoundaryRun) on the
    CPU oracle over a bounded sample grid of the same workload; the
    Regent-defined pieces come from the port when the compiled reference
    lacks them."""
    import oracle
    from htr_gb300 import wall
    port = oracle.port_lib()
    fl = wall.boundary_layer(num=num, seed=77)
    fl.meta["grid"].fill(fl, port)
    m = workloads.make_mixture_struct(lib, abi.HTR_EOS_AIRMIX, fl.meta["mix"])
    h = oracle.load_mixture(lib, abi.HTR_EOS_AIRMIX, m)
    workloads.derive_state(lib, fl, h)
    bc = fl.meta["bc"]
    P = bc["xNeg"][1]["P"]
    Ls = (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"])
    if kind == "port":
        run = wall.BoundaryRun(port, fl, h, bc)
        dt = run.spectral_dt(0.8)
        step = lambda: run.step(dt)
    else:
        hp = oracle.load_mixture(port, abi.HTR_EOS_AIRMIX, workloads.make_mixture_struct(port, abi.HTR_EOS_AIRMIX,
                                                                                         fl.meta["mix"]))
        dt = wall.BoundaryRun(port, fl, hp, bc).spectral_dt(0.8)
        step = lambda: oracle.boundary_layer_step(lib, fl, h, dt, P, P, Ls, regent=port, regent_mix=hp)
    steps = 0
    t0 = time.perf_counter()
    while True:
        step()
        steps += 1
        if time.perf_counter() - t0 > budget_s or steps >= 50:
            break
    el = time.perf_counter() - t0
    cells = num[0] * num[1] * num[2]
    return {"value": 3.0 * steps * cells / el, "unit": UNIT, "kind": kind,
            "sample": f"{steps} boundary-layer SSP-RK3 steps of {num[0]}x{num[1]}x{num[2]} interior cells of the "
                      f"same workload, {el:.1f} s"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    base = cpu_baseline(budget_s=max(5.0, args.cpu_seconds / max(1, args.steps + args.warmup)))
    # K timed samples after W warm-up samples, each a bounded RHS sample
    vals = []
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(budget_s=max(2.0, args.cpu_seconds / max(1, args.steps + args.warmup)), wall_num=None)
        if i >= args.warmup:
            vals.append(b["value"])
    value = float(np.median(vals)) if vals else base["value"]
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"periodic {args.n}^3 box, 5-species air (AirMix), hybrid TENO/KG + "
                                   f"diffusion + explicit chemistry, SSP-RK3", "grid": [args.n] * 3,
                       "sample_grid": [48] * 3},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": base["cores"], "kind": base["kind"],
                             "sample": base["sample"], "wall": base.get("wall")},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=256)
    p.add_argument("--cpu-seconds", type=float, default=20.0)
    p.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    p.add_argument("--tubes", type=int, default=4096, help="batched shock tubes (0: skip)")
    p.add_argument("--serve", type=int, default=32, help="served requests (0: skip)")
    p.add_argument("--wall", default="512,192,128", help="boundary-layer interior cells nx,ny,nz ('' skips)")
    p.add_argument("--wall-steps", type=int, default=10)
    p.add_argument("--no-restart", dest="restart", action="store_false", help="skip the restart dump/load timing")
    args = p.parse_args()
    res = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
