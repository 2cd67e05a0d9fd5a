"""Batched form: many independent grids of uneven size, of both mixtures,
advanced together, one CUDA graph launch per SSP-RK3 step of the whole batch.

A batch holds 1-D shock tubes and periodic 2-D / 3-D boxes (any sizes, gas or
five-species air).  The tubes of one mixture are packed end to end into one
strip (their boundary ghost nodes keep each tube's stencils to itself) and
stepped by one fused step of the strip with one step size per tube
(htr_rk3_step_cells_ws); every box is stepped by its own fused step
(htr_rk3_step_ws).  One step of the whole batch is captured once as a CUDA
graph whose branches -- one per strip and per box, captured on separate
streams forked from and joined back to the capture stream -- are
independent, so the GPU runs them concurrently and the host issues one
launch per step.  Every instance keeps its own step size (the CFL step of
its own grid, as each run of the reference computes it), and its result
does not depend on the other members: the same cells go through the same
arithmetic in any batch.  With tune=True the launch shapes (KG x tile, TENO
blocks per SM, block sizes) are chosen per size class of branch by the
autotuner and captured into each branch.
"""
from . import abi, runtime, tubes


class Batch:
    """Instances: dicts with keys fluid (device Fluid, state derived), gh
    (mixture handle), dt (its step size), chemistry (bool) and tube (True for
    a 1-D shock tube with boundary ghosts, to be packed into its mixture's
    strip).  After construction the instances' fluids are views into the
    batch's storage (tubes: into their strip)."""

    def __init__(self, instances, device="cuda", graph=True, tune=False):
        import torch

        from .fluid import Fluid
        self.device = device
        self.instances = instances
        self.branches = []  # (kind, payload) in capture order
        groups = {}
        for inst in instances:
            if inst.get("tube"):
                groups.setdefault(inst["fluid"].nspec, []).append(inst)
            else:
                self.branches.append(("box", inst))
        for nsp, members in groups.items():
            names = list(members[0]["fluid"].arrays)
            widths = [m["fluid"].nx for m in members]
            strip = Fluid((sum(widths), 1, 1), nsp, device=device, fields=names)
            for name in names:
                torch.cat([m["fluid"].arrays[name] for m in members], dim=2, out=strip.arrays[name])
            dt_cell = torch.cat([torch.full((w,), float(m["dt"]), dtype=torch.float64, device=device)
                                 for w, m in zip(widths, members)])
            off = 0
            for w, m in zip(widths, members):
                view = Fluid((w, 1, 1), nsp, device=device, fields=[])
                view.arrays = {n: strip.arrays[n][:, :, off:off + w] for n in names}
                view.meta = dict(m["fluid"].meta)
                m["fluid"] = view
                off += w
            self.branches.append(("strip", dict(fluid=strip, gh=members[0]["gh"], dt_cell=dt_cell,
                                                chemistry=members[0]["chemistry"], members=members)))
        self.streams = [torch.cuda.Stream(device=device) for _ in self.branches]
        self.workspaces = [runtime.Workspace() for _ in self.branches]
        for (kind, b), ws in zip(self.branches, self.workspaces):
            ws.get(runtime.workspace_bytes(b["fluid"], b["gh"]), device)
        self.tunings = {}  # size class -> launch shapes chosen for it
        if tune:
            self.autotune()
        self.graph = None
        if graph:
            self.capture()

    @staticmethod
    def size_class(kind, fluid):
        """Size class of a branch for launch-shape tuning: the strips of each
        mixture, and small (below 64 k cells) or large boxes of each mixture."""
        if kind == "strip":
            return f"strip, {fluid.nspec} species"
        return f"{'small' if fluid.ncells < 65536 else 'large'} box, {fluid.nspec} species"

    def autotune(self, reps=3):
        """Launch shapes per size class (autotune.autotune on that class's
        grids: KG x tile, TENO blocks per SM, block sizes).  The shapes are
        captured into the graph branch by branch; they never change the
        arithmetic."""
        from . import autotune as at
        default = at.get_tuning()
        classes = {}
        for (kind, b), ws in zip(self.branches, self.workspaces):
            classes.setdefault(self.size_class(kind, b["fluid"]), []).append((b, ws))
        for cls, items in classes.items():
            at.set_tuning(default)
            grids = [(b["fluid"], b["gh"], b["dt"] if "dt" in b else float(b["dt_cell"].min()), b["chemistry"])
                     for b, _ in items]
            best, t_best, t0, _ = at.autotune(grids, reps=reps, workspace=items[0][1])
            self.tunings[cls] = dict(tuning=best, stage_ms=t_best, stage_ms_default=t0)
        at.set_tuning(default)

    def _issue(self, stream):
        """One step of every branch, each on its own stream forked from and
        joined back to `stream`."""
        import torch
        from . import autotune as at
        default = at.get_tuning() if self.tunings else None
        fork = torch.cuda.Event()
        fork.record(stream)
        joins = []
        for (kind, b), s, ws in zip(self.branches, self.streams, self.workspaces):
            s.wait_event(fork)
            if self.tunings:
                at.set_tuning(at.htr_stage_tuning(**self.tunings[self.size_class(kind, b["fluid"])]["tuning"]))
            if kind == "strip":
                runtime.rk3_step_cells(b["fluid"], b["gh"], b["dt_cell"], chemistry=b["chemistry"], stream=s,
                                       workspace=ws)
            else:
                runtime.rk3_step(b["fluid"], b["gh"], dt=b["dt"], chemistry=b["chemistry"], stream=s,
                                 workspace=ws)
            ev = torch.cuda.Event()
            ev.record(s)
            joins.append(ev)
        if default is not None:
            at.set_tuning(default)
        for ev in joins:
            stream.wait_event(ev)

    def capture(self):
        """Capture one step of the whole batch as a CUDA graph (the step it
        runs while capturing is not executed)."""
        import torch
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
            self._issue(side)
        torch.cuda.current_stream(self.device).wait_stream(side)
        self.graph = g

    def step(self, stream=None):
        """One SSP-RK3 step of every instance (one graph launch)."""
        import torch
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        if self.graph is not None:
            with torch.cuda.stream(st):
                self.graph.replay()
        else:
            self._issue(st)

    def launches_per_step(self):
        """Kernel launches one step issues (for the benchmark's count): per
        branch the fused step's sensors, Conserved_old copy and cache reset,
        then per stage the prepass, three KG and three TENO face kernels,
        three diffusion face kernels and the update (fewer for directions of
        one cell)."""
        n = 0
        for kind, b in self.branches:
            fl = b["fluid"]
            active = sum(1 for x in (fl.nx, fl.ny, fl.nz) if x > 1)
            n += 3 + 3 * (1 + 3 * active + 1)
        return n


def tube_instance(inst, device, lib=None):
    """A batch instance of one shock tube (tubes.instances entry): its device
    state derived, its own step size (CFL tubes.TUBE_CFL, with chemistry also
    at most half its fastest chemical time)."""
    from . import workloads
    l = lib or runtime.lib()
    host = tubes.tube_fluid(inst)
    eos = host.meta["eos"]
    gh = runtime.load_mixture(eos, workloads.make_mixture_struct(l, eos, host.meta["mix"]))
    dev = host.to_device(device)
    dev.meta = dict(host.meta)
    workloads.derive_state(l, dev, gh, runtime.stream_handle())
    chem = eos == abi.HTR_EOS_AIRMIX
    dt = runtime.stable_dt(dev, gh, cfl=tubes.TUBE_CFL, chemistry=chem)
    return dict(fluid=dev, gh=gh, dt=dt, chemistry=chem, tube=True)


def box_instance(host, device, lib=None, cfl=0.8):
    """A batch instance of a periodic box (a host Fluid from workloads)."""
    from . import workloads
    l = lib or runtime.lib()
    eos = host.meta["eos"]
    gh = runtime.load_mixture(eos, workloads.make_mixture_struct(l, eos, host.meta["mix"]))
    dev = host.to_device(device)
    dev.meta = dict(host.meta)
    workloads.derive_state(l, dev, gh, runtime.stream_handle())
    chem = eos == abi.HTR_EOS_AIRMIX
    dt = runtime.stable_dt(dev, gh, cfl=cfl, chemistry=chem)
    return dict(fluid=dev, gh=gh, dt=dt, chemistry=chem, tube=False)
