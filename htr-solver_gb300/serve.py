"""Serving: simulation requests admitted as they arrive, stepped together.

A request asks for a number of SSP-RK3 steps of one seeded grid: a 1-D shock
tube, a 2-D vortex-advection box or a 3-D reacting-air box.  The server
keeps every admitted request's state resident on the device and advances
all of them round by round: each round issues one step of every active
request.  Shock tubes of one mixture are stepped together: packed into one
strip (TubeGroup), all of them advance in one fused step of the strip, each
by its own step size.  Each 2-D and 3-D box steps as the replay of its own
CUDA graph of one fused step (htr_rk3_step_ws on the request's own
workspace); the groups and the boxes run on the streams of a small pool, so
the steps of different requests overlap on the GPU.  Requests are
admitted in arrival order while their device memory (state + workspace) fits
the HBM budget; a finished request's result (Conserved) is copied to the host
and its memory released, which lets the next request in.  At most two rounds
are in flight, so the host never runs far ahead of the device.

`run_plain` is the reference point: the plain drop-in per request, one
request at a time in arrival order (htr_rk3_step, one task kernel per
reference task).

Times are seconds from the start of a session; time-to-solution is the
completion time minus the arrival time.
"""
import time
from dataclasses import dataclass

import numpy as np

from . import abi, runtime, tubes, workloads


@dataclass
class Request:
    rid: int
    kind: str          # "tube" | "vortex" | "box"
    size: int          # cells per side (tube: interior length)
    seed: int
    steps: int
    arrival: float     # s after the start of the session
    admitted: float = None
    done: float = None
    result: object = None   # host copy of Conserved after the last step
    state: object = None    # host Fluid submitted with the request (prepare())

    @property
    def tts(self):
        return None if self.done is None else self.done - self.arrival


def request_mix(n, rate, seed=0, steps=(100, 2000), tube=(256, 8192), vortex=(64, 512), box=(32, 96)):
    """n requests with Poisson arrivals of `rate` per second: tubes, 2-D
    vortex boxes and 3-D reacting boxes in equal proportion."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        kind = ("tube", "vortex", "box")[int(rng.integers(0, 3))]
        lo, hi = {"tube": tube, "vortex": vortex, "box": box}[kind]
        out.append(Request(i, kind, int(rng.integers(lo, hi + 1)), int(rng.integers(0, 2 ** 31)),
                           int(rng.integers(steps[0], steps[1] + 1)), t))
    return out


def host_fluid(req):
    """Host state of a request (primitives, node types, metrics): the one it
    was submitted with, else generated from its seed."""
    if req.state is not None:
        return req.state
    if req.kind == "tube":
        inst = tubes.instances(1, seed=req.seed, length=(req.size, req.size))[0]
        return tubes.tube_fluid(inst)
    if req.kind == "vortex":
        return workloads.vortex2d(req.size, seed=req.seed)
    return workloads.air_box(shape=(req.size,) * 3, seed=req.seed)


class Instance:
    """Device state of one admitted request."""

    def __init__(self, req, device, stream, graphs=True):
        import torch
        self.req = req
        self.stream = stream
        host = host_fluid(req)
        eos = host.meta["eos"]
        self.bnum = host.meta.get("bnum", (0, 0, 0))
        self.chem = eos == abi.HTR_EOS_AIRMIX
        l = runtime.lib()
        m = workloads.make_mixture_struct(l, eos, host.meta["mix"])
        self.gh = runtime.load_mixture(eos, m)
        with torch.cuda.stream(stream):
            self.dev = host.to_device(device)
            workloads.derive_state(l, self.dev, self.gh, runtime.stream_handle(stream))
            cfl = tubes.TUBE_CFL if req.kind == "tube" else 0.8
            self.dt = runtime.stable_dt(self.dev, self.gh, cfl=cfl, chemistry=self.chem, stream=stream)
            self.ws = runtime.Workspace()
            self.ws.get(runtime.workspace_bytes(self.dev, self.gh), device)
        self.bytes = sum(a.numel() * a.element_size() for a in self.dev.arrays.values()) + self.ws.nbytes
        self.cells = self.dev.ncells
        self.remaining = req.steps
        self.graph = None
        if graphs:
            g = torch.cuda.CUDAGraph()
            stream.synchronize()
            with torch.cuda.stream(stream):
                g.capture_begin(capture_error_mode="relaxed")
                self._step(stream)
                g.capture_end()
            self.graph = g
        self.done_event = None

    def _step(self, stream):
        runtime.rk3_step(self.dev, self.gh, dt=self.dt, chemistry=self.chem, stream=stream, workspace=self.ws)

    def step(self):
        import torch
        with torch.cuda.stream(self.stream):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._step(self.stream)
        self.remaining -= 1

    def finish(self):
        """Host copy of the result; releases the device state."""
        self.req.result = self.dev["Conserved"].cpu().numpy()
        self.dev = None
        self.ws = None
        self.graph = None


class TubeGroup:
    """Every admitted shock-tube request of one mixture, stepped together:
    the tubes are packed end to end into one device strip (their boundary
    ghost nodes keep each tube's stencils to itself) and advanced by one
    fused step of the strip per round, every tube by its own step size
    (htr_rk3_step_cells_ws), replayed from one CUDA graph.  The strip is
    rebuilt, and the graph captured again, when tubes join or leave; a tube's
    cells go through the same arithmetic in any strip, so its result does
    not depend on the other members."""

    def __init__(self, eos, device, stream, graphs=True):
        self.eos = eos
        self.device = device
        self.stream = stream
        self.graphs = graphs
        self.chem = eos == abi.HTR_EOS_AIRMIX
        l = runtime.lib()
        mix = tubes.AIR_REF if self.chem else tubes.GAS_PARAMS
        self.gh = runtime.load_mixture(eos, workloads.make_mixture_struct(l, eos, mix))
        self.members = []   # dicts: req, dev (the tube's Fluid, a view into the strip once packed), dt, remaining
        self.done = []      # members whose last step ran: (member, pinned host result, event)
        self.strip = None
        self.dt_cell = None
        self.ws = runtime.Workspace()
        self.graph = None
        self.dirty = False

    def admit(self, req):
        """Derive the tube's state and its own step size on the group's stream."""
        import torch
        host = host_fluid(req)
        l = runtime.lib()
        with torch.cuda.stream(self.stream):
            dev = host.to_device(self.device)
            workloads.derive_state(l, dev, self.gh, runtime.stream_handle(self.stream))
            dt = runtime.stable_dt(dev, self.gh, cfl=tubes.TUBE_CFL, chemistry=self.chem, stream=self.stream)
        self.members.append(dict(req=req, dev=dev, dt=dt, remaining=req.steps))
        self.dirty = True
        return sum(a.numel() * a.element_size() for a in dev.arrays.values())

    def rebuild(self):
        """Pack the current members into a new strip and capture its step."""
        import torch

        from .fluid import Fluid
        self.stream.synchronize()
        self.graph = None
        if not self.members:
            self.strip = self.dt_cell = None
            self.dirty = False
            return
        nsp = self.members[0]["dev"].nspec
        widths = [m["dev"].nx for m in self.members]
        names = list(self.members[0]["dev"].arrays)
        with torch.cuda.stream(self.stream):
            strip = Fluid((sum(widths), 1, 1), nsp, device=self.device, fields=names)
            for name in names:
                torch.cat([m["dev"].arrays[name] for m in self.members], dim=2, out=strip.arrays[name])
            self.dt_cell = torch.cat([torch.full((w,), m["dt"], dtype=torch.float64, device=self.device)
                                      for w, m in zip(widths, self.members)])
            off = 0
            for w, m in zip(widths, self.members):
                view = Fluid((w, 1, 1), nsp, device=self.device, fields=[])
                view.arrays = {n: strip.arrays[n][:, :, off:off + w] for n in names}
                m["dev"] = view
                off += w
            self.ws.get(runtime.workspace_bytes(strip, self.gh), self.device)
        self.strip = strip
        if self.graphs:
            g = torch.cuda.CUDAGraph()
            self.stream.synchronize()
            with torch.cuda.stream(self.stream):
                g.capture_begin(capture_error_mode="relaxed")
                self._step()
                g.capture_end()
            self.graph = g
        self.dirty = False

    def _step(self):
        runtime.rk3_step_cells(self.strip, self.gh, self.dt_cell, chemistry=self.chem, stream=self.stream,
                               workspace=self.ws)

    def step(self):
        """One step of every member; members that took their last step have
        their result copied to pinned host memory on the group's stream and
        leave the strip at the next rebuild."""
        import torch
        with torch.cuda.stream(self.stream):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._step()
            keep = []
            for m in self.members:
                m["remaining"] -= 1
                if m["remaining"] == 0:
                    c = m["dev"]["Conserved"]
                    out = torch.empty(c.shape, dtype=c.dtype, device="cpu").pin_memory()
                    out.copy_(c, non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(self.stream)
                    self.done.append((m, out, ev))
                    self.dirty = True
                else:
                    keep.append(m)
            self.members = keep


def _grid(req):
    """(nx, ny, nz, nspec) of a request's grid."""
    if req.kind == "tube":
        return req.size + 2, 1, 1, (5 if tubes.instances(1, seed=req.seed, length=(req.size, req.size))[0]["eos"]
                                    == abi.HTR_EOS_AIRMIX else 1)
    if req.kind == "vortex":
        return req.size, req.size, 1, 1
    return req.size, req.size, req.size, 5


def prepare(requests):
    """Generate every request's seeded initial state on the host, as a client
    would submit it (outside any timed session)."""
    for r in requests:
        r.state = None
        r.state = host_fluid(r)
    return requests


def estimate_bytes(req):
    """Device bytes a request holds while admitted: every field of its grid
    plus the fused-step workspace (the layout of stage_workspace_bytes) and
    the workspace's alignment slack."""
    nx, ny, nz, nsp = _grid(req)
    cells = nx * ny * nz
    neq = nsp + 4
    size = {"int32": 4, "float64": 8, "bool": 1}
    state = 0
    for _name, dt, comp in abi.FIELD_SPECS:
        c = {"nSpec": nsp, "nEq": neq}.get(comp, comp)
        state += cells * int(c) * size[dt]
    a256 = lambda b: (b + 255) // 256 * 256
    n = (nx, ny, nz)
    nf = [(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2)) for d in range(3)]
    work = (sum(2 * a256(8 * neq * f) for f in nf) + a256(16 * sum(nf)) + a256(4) + a256(8 * 11 * cells) +
            a256(8 * (3 + 2 * nsp) * cells))
    return int(state + work + 256)


def admissible(queue, now, used, budget, size=estimate_bytes):
    """How many requests at the head of the arrival-ordered queue can be
    admitted at time `now` with `used` bytes in use (first come, first served:
    a request that does not fit blocks the ones behind it)."""
    k = 0
    for req in queue:
        if req.arrival > now or used + size(req) > budget:
            break
        used += size(req)
        k += 1
    return k


class Server:
    """Continuous batching under an HBM budget (bytes)."""

    def __init__(self, device="cuda", hbm_budget=150e9, streams=8, graphs=True, admit_per_round=2,
                 batch_tubes=True, round_cells=None):
        import torch
        self.device = device
        # cells of the boxes stepped per round (None: every active box): the
        # boxes with the least remaining work (steps left x cells) go first
        # until their cells reach round_cells, so short requests finish early
        # (shortest remaining work first) while the round still fills the GPU
        self.round_cells = round_cells
        self.admit_per_round = admit_per_round  # admissions between rounds (keeps the device busy)
        self.budget = hbm_budget
        self.pool = [torch.cuda.Stream() for _ in range(streams)]
        self.graphs = graphs
        # shock tubes of one mixture are stepped together in one strip
        self.batch_tubes = batch_tubes
        self.groups = {}
        self.used = 0          # bytes reserved by admitted requests
        self.peak = 0
        self.rounds = 0
        self.over_estimate = 0.0  # max actual / reserved bytes of a request

    def run(self, requests, clock=time.perf_counter):
        import torch
        queue = sorted(requests, key=lambda r: r.arrival)
        active, finishing = [], []
        t0 = clock()
        prev_round, next_stream = [], 0
        while queue or active or finishing or any(g.members or g.done for g in self.groups.values()):
            now = clock() - t0
            # admission in arrival order while the budget allows
            admitted_now = 0
            grouped = sum(len(g.members) for g in self.groups.values())
            while queue and admissible(queue[:1], now, self.used, self.budget) and \
                    (admitted_now < self.admit_per_round or not (active or grouped)):
                admitted_now += 1
                req = queue.pop(0)
                reserved = estimate_bytes(req)
                if self.batch_tubes and req.kind == "tube":
                    eos = abi.HTR_EOS_AIRMIX if _grid(req)[3] == 5 else abi.HTR_EOS_CONSTPROPMIX
                    if eos not in self.groups:
                        self.groups[eos] = TubeGroup(eos, self.device, self.pool[next_stream % len(self.pool)],
                                                     self.graphs)
                        next_stream += 1
                    nbytes = self.groups[eos].admit(req)
                    self.over_estimate = max(self.over_estimate, nbytes / reserved)
                    grouped += 1
                else:
                    inst = Instance(req, self.device, self.pool[next_stream % len(self.pool)], self.graphs)
                    next_stream += 1
                    inst.reserved = reserved
                    self.over_estimate = max(self.over_estimate, inst.bytes / inst.reserved)
                    active.append(inst)
                req.admitted = clock() - t0
                req.reserved = reserved
                self.used += reserved
                self.peak = max(self.peak, self.used)
            # tubes that took their last step: results, then the strip without them
            for g in self.groups.values():
                for m, out, ev in list(g.done):
                    if ev.query():
                        m["req"].result = out.numpy()
                        m["req"].done = clock() - t0
                        self.used -= m["req"].reserved
                        g.done.remove((m, out, ev))
                if g.dirty:
                    g.rebuild()
            # retire requests whose last step completed
            for inst in list(finishing):
                if inst.done_event.query():
                    inst.finish()
                    inst.req.done = clock() - t0
                    self.used -= inst.reserved
                    finishing.remove(inst)
            stepping = [g for g in self.groups.values() if g.members]
            pending = any(g.done for g in self.groups.values())
            if not active and not stepping:
                if finishing or pending:
                    time.sleep(1e-4)
                elif queue:
                    time.sleep(max(0.0, min(queue[0].arrival - (clock() - t0), 0.01)))
                continue
            # one round: a step of every active request
            for ev in prev_round:
                ev.synchronize()
            cur = []
            for g in stepping:
                g.step()
                ev = torch.cuda.Event()
                ev.record(g.stream)
                cur.append(ev)
            for inst in self.select(active):
                inst.step()
                ev = torch.cuda.Event()
                ev.record(inst.stream)
                cur.append(ev)
                if inst.remaining == 0:
                    inst.done_event = ev
                    finishing.append(inst)
            active = [i for i in active if i.remaining > 0]
            prev_round = cur
            self.rounds += 1
        torch.cuda.synchronize()
        return requests


    def select(self, active):
        return round_selection(active, self.round_cells)


def round_selection(active, round_cells):
    """The boxes stepped in one round, in the order they were admitted: all
    of them without a cell budget, else those with the least remaining work
    (steps left x cells; ties by admission) until their cells reach
    round_cells.  Items need `remaining` and `cells`."""
    if round_cells is None or len(active) <= 1:
        return list(active)
    order = sorted(range(len(active)), key=lambda k: (active[k].remaining * active[k].cells, k))
    chosen, cells = set(), 0
    for k in order:
        chosen.add(k)
        cells += active[k].cells
        if cells >= round_cells:
            break
    return [inst for k, inst in enumerate(active) if k in chosen]


def run_plain(requests, device="cuda", clock=time.perf_counter):
    """The plain drop-in per request, in arrival order, one at a time."""
    import torch
    t0 = clock()
    for req in sorted(requests, key=lambda r: r.arrival):
        now = clock() - t0
        if req.arrival > now:
            time.sleep(req.arrival - now)
        host = host_fluid(req)
        eos = host.meta["eos"]
        chem = eos == abi.HTR_EOS_AIRMIX
        l = runtime.lib()
        m = workloads.make_mixture_struct(l, eos, host.meta["mix"])
        gh = runtime.load_mixture(eos, m)
        dev = host.to_device(device)
        workloads.derive_state(l, dev, gh, runtime.stream_handle())
        dt = runtime.stable_dt(dev, gh, cfl=tubes.TUBE_CFL if req.kind == "tube" else 0.8, chemistry=chem)
        req.admitted = clock() - t0
        inner = dev.interior(host.meta.get("bnum", (0, 0, 0)))
        for _ in range(req.steps):
            runtime.rk3_step(dev, gh, dt=dt, chemistry=chem, fused=False, interior=inner)
        req.result = dev["Conserved"].cpu().numpy()
        req.done = clock() - t0
        del dev
    torch.cuda.synchronize()
    return requests


def summary(requests, elapsed):
    tts = np.array([r.tts for r in requests])
    return {"solves_per_s": len(requests) / elapsed, "tts_p50_s": float(np.percentile(tts, 50)),
            "tts_p99_s": float(np.percentile(tts, 99)), "elapsed_s": elapsed, "requests": len(requests)}
