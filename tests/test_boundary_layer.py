"""Grids with boundary conditions: zones, grid set-up, metrics and the
time step of the wall-bounded boundary-layer workload.

CPU:
  - zones.partition against zones written out by hand from the reference's
    partitioner for the boundary-layer BC set, and tie-break cases;
  - node types and cell centres of stretched axes;
  - the port's metrics against the reference's compiled InitializeMetric /
    CorrectGhostMetric (bit for bit, where the reference sources exist);
  - one SSP-RK3 step of the boundary layer: the library driver
    (wall.BoundaryRun) on the port against the oracle's own step
    (oracle.boundary_layer_step) on the reference's compiled tasks, and on
    the port, bit for bit.
GPU (-m gpu):
  - metrics on the device against the port, bit for bit;
  - one and two boundary-layer steps through the CUDA library against the
    oracle step on the port, within the pointwise bar of util.check.
"""
import ctypes as C

import numpy as np
import pytest

from htr_gb300 import abi, grid, runtime, wall, workloads, zones

import oracle
from tests import util

BL_BC = (("NSCBC_Inflow", "NSCBC_Outflow"), ("IsothermalWall", "NSCBC_Outflow"), ("Periodic", "Periodic"))
METRICS = ("dcsi_e", "deta_e", "dzet_e", "dcsi_d", "deta_d", "dzet_d", "dcsi_s", "deta_s", "dzet_s")


def _points(boxes):
    pts = set()
    for lo, hi in boxes:
        for k in range(lo[2], hi[2] + 1):
            for j in range(lo[1], hi[1] + 1):
                for i in range(lo[0], hi[0] + 1):
                    pts.add((i, j, k))
    return pts


@pytest.mark.parametrize("shape", [(8, 6, 3), (21, 14, 5)])
def test_zones_match_hand_derived(shape):
    z = zones.partition(shape, (1, 1, 0), BL_BC)
    h = oracle.boundary_layer_zones(*shape)
    assert z.all == h["all"] and z.interior == h["interior"]
    assert _points(z.solved) == _points([h["solved"]])
    for d in range(3):
        assert _points(z.divg[d]) == _points([h["divg"][d]])
    for s, name in enumerate(("xNeg", "xPos", "yNeg", "yPos")):
        assert _points(z.planes[s]) == _points([h[name]]), name
    assert not z.planes[4] and not z.planes[5]
    assert _points(z.all_bcs) == _points([h["all"]]) - _points([h["interior"]])
    assert _points(z.all_bcs) == _points(h["all_bcs"])


def test_zones_periodic_and_walls():
    per = zones.partition((6, 5, 4), (0, 0, 0), (("Periodic", "Periodic"),) * 3)
    assert all(not p for p in per.planes) and not per.all_bcs
    assert per.solved == [per.interior] and all(d == [per.interior] for d in per.divg)
    walls = zones.partition((6, 5, 4), (1, 1, 1), (("IsothermalWall", "AdiabaticWall"),) * 3)
    # walls everywhere: edges and corners go to x first, then y
    x_neg = _points(walls.planes[0])
    assert (0, 0, 0) in x_neg and (0, 4, 3) in x_neg
    assert (1, 0, 0) in _points(walls.planes[2]) and (1, 0, 0) not in _points(walls.planes[4])
    assert walls.solved == [walls.interior] and all(d == [walls.interior] for d in walls.divg)
    out = zones.partition((6, 5, 4), (1, 1, 0), (("NSCBC_Outflow", "NSCBC_Outflow"),
                                                 ("NSCBC_Outflow", "NSCBC_Outflow"), ("Periodic", "Periodic")))
    # an outflow-outflow edge belongs to both sides and is solved
    assert (5, 4, 0) in _points(out.planes[1]) and (5, 4, 0) in _points(out.planes[3])
    assert (5, 4, 0) in _points(out.solved)
    with pytest.raises(ValueError):
        zones.partition((6, 5, 4), (1, 1, 0), (("Mystery", "Mystery"), ("Mystery", "Mystery"),
                                               ("Periodic", "Periodic")))


def test_node_types_and_centres():
    g = grid.Grid((10, 8, 4), (1.0, 0.5, 0.25), BL_BC, kind=(("Uniform", 1.0), ("TanhMinus", 1.0), ("Uniform", 1.0)))
    assert g.shape == (12, 10, 4) and g.bnum == (1, 1, 0)
    assert list(g.ntype[0][:2]) == [grid.L_C, grid.LP1_C] and list(g.ntype[0][-3:]) == [grid.RM2_C, grid.RM1_C,
                                                                                          grid.R_C]
    assert list(g.ntype[1][:3]) == [grid.L_S, grid.LP1_S, grid.LP2_S]
    assert list(g.ntype[1][-3:]) == [grid.RM2_C, grid.RM1_C, grid.R_C]
    assert np.all(g.ntype[2] == grid.STD)
    assert g.center[0][0] == pytest.approx(-0.05) and g.center[0][-1] == pytest.approx(1.05)
    assert g.center[1][0] == 0.0  # staggered wall point on the wall
    dy = np.diff(g.center[1][1:-1])
    assert np.all(dy > 0) and dy[0] < dy[-1]  # clustered at the wall
    assert np.all(np.diff(g.center[2]) == pytest.approx(0.0625))


def _grid_fluid(bc, num, kind, width=(1.0, 0.6, 0.3)):
    g = grid.Grid(num, width, bc, kind=kind)
    return g, workloads.Fluid(g.shape, 1)


GRIDS = [
    (BL_BC, (12, 9, 4), (("Uniform", 1.0), ("TanhMinus", 1.0), ("Uniform", 1.0))),
    ((("Periodic", "Periodic"),) * 3, (9, 7, 5), (("Tanh", 1.3), ("Cosine", 1.0), ("SinhPlus", 0.8))),
    ((("IsothermalWall", "AdiabaticWall"), ("Dirichlet", "NSCBC_Outflow"), ("NSCBC_Inflow", "IsothermalWall")),
     (7, 6, 5), (("TanhPlus", 2.0), ("Sinh", 1.5), ("SinhMinus", 1.1))),
]


@pytest.mark.parametrize("case", range(len(GRIDS)))
def test_metric_port_matches_reference(case):
    ref = oracle.ref_lib(1)
    if ref is None:
        pytest.skip("reference CPU build not present on this machine")
    port = oracle.port_lib()
    bc, num, kind = GRIDS[case]
    outs = []
    for lib in (ref, port):
        g, fl = _grid_fluid(bc, num, kind)
        g.fill(fl, lib)
        outs.append(fl)
    for name in METRICS:
        assert np.array_equal(outs[0][name], outs[1][name]), name
        assert np.all(np.isfinite(outs[1][name])), name


def _bl(lib, num=(14, 10, 4), seed=3):
    fl = wall.boundary_layer(num=num, seed=seed)
    fl.meta["grid"].fill(fl, lib)
    m = workloads.make_mixture_struct(lib, fl.meta["eos"], fl.meta["mix"])
    h = oracle.load_mixture(lib, fl.meta["eos"], m)
    workloads.derive_state(lib, fl, h)
    return fl, h, m


def _oracle_step(lib, fl, h, dt, regent=None, regent_mix=None):
    bc = fl.meta["bc"]
    oracle.boundary_layer_step(lib, fl, h, dt, bc["xNeg"][1]["P"], bc["xPos"][1]["P"],
                               (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"]),
                               regent=regent, regent_mix=regent_mix)


def test_boundary_layer_driver_matches_oracle_step():
    port = oracle.port_lib()
    a, ha, _ = _bl(port)
    b, hb, _ = _bl(port)
    run = wall.BoundaryRun(port, a, ha, a.meta["bc"])
    dt = run.spectral_dt(0.8)
    for n in range(2):
        run.step(dt)
        _oracle_step(port, b, hb, dt)
        if n == 0:
            # the inflow derivatives see the imposed profile replace the noisy start
            assert np.any(a["dudtBoundary"][:, 1:, 0] != 0.0)
    for name in a.arrays:
        assert np.array_equal(a[name], b[name]), name
    assert np.all(np.isfinite(a["Conserved"]))
    assert np.array_equal(a["velocity_old_NSCBC"][:, 1:, 0], a["velocity"][:, 1:, 0])


@pytest.mark.parametrize("scheme", ["TENOLAD", "Hybrid"])
def test_boundary_layer_step_port_matches_reference(scheme):
    ref = oracle.ref_lib(2)
    if ref is None:
        pytest.skip("reference CPU build not present on this machine")
    port = oracle.port_lib()
    a, ha, _ = _bl(port)
    b, hb, _ = _bl(ref)
    for name in a.arrays:
        assert np.array_equal(a[name], b[name]), name
    run = wall.BoundaryRun(port, a, ha, a.meta["bc"], scheme=scheme)
    dt = run.spectral_dt(0.8)
    run.step(dt)
    bc = b.meta["bc"]
    oracle.boundary_layer_step(ref, b, hb, dt, bc["xNeg"][1]["P"], bc["xPos"][1]["P"],
                               (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"]), scheme=scheme,
                               regent=port, regent_mix=ha)
    for name in a.arrays:
        assert np.array_equal(a[name], b[name]), name


def test_boundary_run_rejects_unsupported():
    port = oracle.port_lib()
    fl, h, _ = _bl(port, num=(6, 5, 3))
    with pytest.raises(abi.HtrError):
        wall.BoundaryRun(port, fl, h, fl.meta["bc"], scheme="WENO")
    bc = dict(fl.meta["bc"])
    bc["yPos"] = ("IncomingShock", {})
    with pytest.raises(abi.HtrError):
        wall.BoundaryRun(port, fl, h, bc)


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(GRIDS)))
def test_gpu_metric_matches_port(case):
    import torch
    port = oracle.port_lib()
    bc, num, kind = GRIDS[case]
    g, host = _grid_fluid(bc, num, kind)
    g.fill(host, port)
    g2, dev = _grid_fluid(bc, num, kind)
    dev = dev.to_device("cuda")
    g2.fill(dev, runtime.lib())
    torch.cuda.synchronize()
    out = dev.to_host()
    for name in METRICS:
        assert np.array_equal(out[name], host[name]), name


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [1, 2])
def test_gpu_boundary_layer_steps(steps):
    import torch
    port = oracle.port_lib()
    host, hp, m = _bl(port, num=(24, 16, 6))
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    mach = torch.zeros(1, dtype=torch.float64, device="cuda")
    run = wall.BoundaryRun(runtime.lib(), dev, gh, host.meta["bc"], stream=runtime.stream_handle(),
                           max_mach_buffer=mach)
    dt = wall.BoundaryRun(port, host, hp, host.meta["bc"]).spectral_dt(0.8)
    for _ in range(steps):
        _oracle_step(port, host, hp, dt)
        run.step(dt)
    torch.cuda.synchronize()
    out = dev.to_host()
    util.check_fields(out, host, ("Conserved", "temperature", "pressure", "velocity", "MolarFracs"))


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [1, 2])
def test_gpu_fused_boundary_layer_steps(steps):
    """The fused boundary step (htr_rk3_step_bc_ws) against the oracle step."""
    import torch
    port = oracle.port_lib()
    host, hp, m = _bl(port, num=(24, 16, 6))
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    run = wall.FusedBoundaryRun(dev, gh, host.meta["bc"])
    dt = wall.BoundaryRun(port, host, hp, host.meta["bc"]).spectral_dt(0.8)
    for _ in range(steps):
        _oracle_step(port, host, hp, dt)
        run.step(dt)
    torch.cuda.synchronize()
    out = dev.to_host()
    util.check_fields(out, host, ("Conserved", "temperature", "pressure", "velocity", "MolarFracs", "rho", "SoS",
                                  "mu", "dudtBoundary"))


@pytest.mark.gpu
def test_gpu_fused_boundary_cfl_and_errors():
    import torch
    port = oracle.port_lib()
    host, hp, m = _bl(port, num=(12, 10, 4))
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    run = wall.FusedBoundaryRun(dev, gh, host.meta["bc"])
    dt_ref = wall.BoundaryRun(port, host, hp, host.meta["bc"]).spectral_dt(0.8)
    dt = run.step(cfl=0.8)
    torch.cuda.synchronize()
    assert dt == pytest.approx(dt_ref, rel=1e-12)
    bad = wall.FusedBoundaryRun(dev, gh, host.meta["bc"])
    bad.params.plane[0] = abi.rect((1, 0, 0), (1, 11, 3))  # not the ghost layer
    with pytest.raises(abi.HtrError):
        bad.step(dt)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["TENO", "TENOA"])
def test_gpu_fused_boundary_other_schemes(scheme):
    import torch
    port = oracle.port_lib()
    host, hp, m = _bl(port, num=(16, 12, 4))
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    dt = wall.BoundaryRun(port, host, hp, host.meta["bc"], scheme=scheme).spectral_dt(0.8)
    bc = host.meta["bc"]
    oracle.boundary_layer_step(port, host, hp, dt, bc["xNeg"][1]["P"], bc["xPos"][1]["P"],
                               (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"]), scheme=scheme)
    wall.FusedBoundaryRun(dev, gh, bc, scheme=scheme).step(dt)
    torch.cuda.synchronize()
    util.check(dev.to_host()["Conserved"], host["Conserved"], "Conserved")


@pytest.mark.gpu
def test_gpu_fused_boundary_step_graph_capture():
    """With a fixed dt the fused boundary step issues no host synchronisation:
    a captured step replays to the same bits as the direct call."""
    import torch
    port = oracle.port_lib()
    host, hp, m = _bl(port, num=(16, 12, 4))
    gh = runtime.load_mixture(host.meta["eos"], m)
    dt = wall.BoundaryRun(port, host, hp, host.meta["bc"]).spectral_dt(0.8)
    a = host.to_device("cuda")
    b = host.to_device("cuda")
    wall.FusedBoundaryRun(a, gh, host.meta["bc"]).step(dt)
    run_b = wall.FusedBoundaryRun(b, gh, host.meta["bc"])
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        run_b.stream = s
        g.capture_begin(capture_error_mode="relaxed")
        run_b.step(dt)
        g.capture_end()
    g.replay()
    torch.cuda.synchronize()
    oa, ob = a.to_host(), b.to_host()
    for name in ("Conserved", "temperature", "pressure", "dudtBoundary"):
        assert np.array_equal(oa[name], ob[name]), name


def _channel(lib, num=(12, 10, 6), seed=4):
    fl = wall.channel(num=num, seed=seed)
    fl.meta["grid"].fill(fl, lib)
    m = workloads.make_mixture_struct(lib, fl.meta["eos"], fl.meta["mix"])
    h = oracle.load_mixture(lib, fl.meta["eos"], m)
    workloads.derive_state(lib, fl, h)
    return fl, h, m


def test_channel_zones_and_step():
    """Walls on both sides of y, periodic x and z: no NSCBC point, every wall
    ghost unsolved; one step on the port keeps the walls at rest and the
    isothermal wall at its temperature."""
    port = oracle.port_lib()
    fl, h, _ = _channel(port)
    z = zones.partition(fl.shape, (0, 1, 0), (("Periodic", "Periodic"), ("IsothermalWall", "AdiabaticWall"),
                                              ("Periodic", "Periodic")))
    assert z.solved == [z.interior] and all(d == [z.interior] for d in z.divg)
    assert _points(z.planes[2]) == _points([((0, 0, 0), (11, 0, 5))])
    run = wall.BoundaryRun(port, fl, h, fl.meta["bc"])
    dt = run.spectral_dt(0.8)
    before = fl.copy()
    run.step(dt)
    assert np.all(fl["velocity"][:, 0] == 0.0) and np.all(fl["velocity"][:, -1] == 0.0)
    assert np.all(fl["temperature"][:, 0] == fl["temperature_profile"][:, 0])
    assert np.array_equal(fl["temperature"][:, -1], fl["temperature"][:, -2])  # adiabatic: copied
    assert np.all(np.isfinite(fl["Conserved"])) and not np.array_equal(fl["Conserved"], before["Conserved"])


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [False, True])
def test_gpu_channel_step(fused):
    import torch
    port = oracle.port_lib()
    host, hp, m = _channel(port)
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    ref_run = wall.BoundaryRun(port, host, hp, host.meta["bc"])
    dt = ref_run.spectral_dt(0.8)
    ref_run.step(dt)
    if fused:
        wall.FusedBoundaryRun(dev, gh, host.meta["bc"]).step(dt)
    else:
        mach = torch.zeros(1, dtype=torch.float64, device="cuda")
        wall.BoundaryRun(runtime.lib(), dev, gh, host.meta["bc"], stream=runtime.stream_handle(),
                         max_mach_buffer=mach).step(dt)
    torch.cuda.synchronize()
    out = dev.to_host()
    util.check(out["Conserved"], host["Conserved"], "Conserved")
    assert np.all(out["velocity"][:, 0] == 0.0) and np.all(out["velocity"][:, -1] == 0.0)


def test_zones_sensor_faces_match_hand_derived():
    for shape in ((8, 6, 3), (21, 14, 5)):
        z = zones.partition(shape, (1, 1, 0), BL_BC)
        h = oracle.boundary_layer_zones(*shape)
        for d in range(3):
            assert _points(z.faces[d]) == _points([h["faces"][d]]), d


def test_hybrid_boundary_layer_driver_matches_oracle():
    port = oracle.port_lib()
    a, ha, _ = _bl(port)
    b, hb, _ = _bl(port)
    run = wall.BoundaryRun(port, a, ha, a.meta["bc"], scheme="Hybrid")
    dt = run.spectral_dt(0.8)
    bc = a.meta["bc"]
    for _ in range(2):
        run.step(dt)
        oracle.boundary_layer_step(port, b, hb, dt, bc["xNeg"][1]["P"], bc["xPos"][1]["P"],
                                   (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"]), scheme="Hybrid")
    for name in a.arrays:
        assert np.array_equal(a[name], b[name]), name
    # sensors outside the faces zones keep their initial value
    assert np.all(a["shockSensorX"][:, :, -1]) and np.all(a["shockSensorY"][:, -1, :])
    assert not np.all(a["shockSensorX"])  # the noisy Mach-6 layer trips the sensor somewhere


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [False, True])
def test_gpu_hybrid_boundary_layer_step(fused):
    import torch
    port = oracle.port_lib()
    host, hp, m = _bl(port, num=(24, 16, 6))
    dev = host.to_device("cuda")
    gh = runtime.load_mixture(host.meta["eos"], m)
    bc = host.meta["bc"]
    dt = wall.BoundaryRun(port, host, hp, bc).spectral_dt(0.8)
    oracle.boundary_layer_step(port, host, hp, dt, bc["xNeg"][1]["P"], bc["xPos"][1]["P"],
                               (bc["xPos"][1]["LengthScale"], bc["yPos"][1]["LengthScale"]), scheme="Hybrid")
    if fused:
        wall.FusedBoundaryRun(dev, gh, bc, scheme="Hybrid").step(dt)
    else:
        mach = torch.zeros(1, dtype=torch.float64, device="cuda")
        wall.BoundaryRun(runtime.lib(), dev, gh, bc, scheme="Hybrid", stream=runtime.stream_handle(),
                         max_mach_buffer=mach).step(dt)
    torch.cuda.synchronize()
    out = dev.to_host()
    for d in "XYZ":
        assert np.array_equal(out[f"shockSensor{d}"], host[f"shockSensor{d}"]), d
    util.check(out["Conserved"], host["Conserved"], "Conserved")


def _pointwise_zones(shape, bnum, types):
    """The partitioner's rules applied point by point (an independent
    restatement used to check zones.partition's rectangle bookkeeping)."""
    nscbc_t = {"NSCBC_Inflow", "NSCBC_Outflow", "NSCBC_FarField", "RecycleRescaling", "IncomingShock"}
    wall_t = {"AdiabaticWall", "IsothermalWall", "SuctionAndBlowingWall"}
    nscbc = [t in nscbc_t for t in types]
    nscbc[4], nscbc[5] = types[2] in nscbc_t, types[3] in nscbc_t  # the z flags read the y sides

    def rank(t):
        if t in wall_t:
            return 0
        if t == "Dirichlet":
            return 1
        if t in ("NSCBC_Inflow", "RecycleRescaling"):
            return 2
        if t in ("NSCBC_Outflow", "IncomingShock", "NSCBC_FarField"):
            return 3
        return 9

    planes = [set() for _ in range(6)]
    divg = [set() for _ in range(3)]
    solved, faces = set(), [set() for _ in range(3)]
    for k in range(shape[2]):
        for j in range(shape[1]):
            for i in range(shape[0]):
                p = (i, j, k)
                sides = []
                for d in range(3):
                    if p[d] < bnum[d]:
                        sides.append(2 * d)
                    elif p[d] >= shape[d] - bnum[d]:
                        sides.append(2 * d + 1)
                if not sides:
                    solved.add(p)
                    for d in range(3):
                        divg[d].add(p)
                        faces[d].add(p)
                    continue
                # planes: best rank wins (lowest axis first); outflow-like sides all win
                best = min(rank(types[s]) for s in sides)
                if best == 3:
                    for s in sides:
                        planes[s].add(p)
                elif best < 3:
                    planes[next(s for s in sides if rank(types[s]) == best)].add(p)
                axes = [s // 2 for s in sides]
                if all(nscbc[s] for s in sides) and len(sides) <= 2:
                    solved.add(p)
                    for d in range(3):
                        if d not in axes:
                            divg[d].add(p)
                # sensor zones: the Neg ghost face of d; NSCBC sides towards d's Neg side
                for d in range(3):
                    other = [s for s in sides if s // 2 != d]
                    own = [s for s in sides if s // 2 == d]
                    if own and own != [2 * d]:
                        continue
                    if not other and own == [2 * d]:
                        faces[d].add(p)
                    elif other and all(nscbc[s] for s in other) and len(other) <= 2:
                        faces[d].add(p)
    return planes, divg, solved, faces


@pytest.mark.parametrize("seed", range(40))
def test_zones_match_pointwise_rules(seed):
    rng = np.random.default_rng(seed)
    kinds = ["NSCBC_Inflow", "NSCBC_Outflow", "IsothermalWall", "AdiabaticWall", "Dirichlet"]
    axes = []
    for d in range(3):
        if rng.random() < 0.3:
            axes.append(("Periodic", "Periodic"))
        else:
            axes.append((kinds[rng.integers(len(kinds))], kinds[rng.integers(len(kinds))]))
    bnum = tuple(0 if a[0] == "Periodic" else 1 for a in axes)
    shape = tuple(int(n) + 2 * b for n, b in zip(rng.integers(3, 6, size=3), bnum))
    types = [axes[0][0], axes[0][1], axes[1][0], axes[1][1], axes[2][0], axes[2][1]]
    z = zones.partition(shape, bnum, axes)
    planes, divg, solved, faces = _pointwise_zones(shape, bnum, types)
    for s in range(6):
        assert _points(z.planes[s]) == planes[s], (axes, s)
    for d in range(3):
        assert _points(z.divg[d]) == divg[d], (axes, d)
        assert _points(z.faces[d]) == faces[d], (axes, "faces", d)
    assert _points(z.solved) == solved, axes
