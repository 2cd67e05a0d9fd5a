"""Wall-bounded grids: a Mach-6 boundary layer over an isothermal wall, and
time steps of grids with boundary conditions.

Workloads.  `channel`: a periodic channel between an isothermal and an
adiabatic wall.  `boundary_layer`: 5-species air (AirMix) on a stretched grid, inflow
and outflow in x, an isothermal wall at yNeg and an outflow at yPos, periodic
z (the boundary types of HTR's flat-plate boundary-layer cases,
testcases/MultispeciesTBL).  The wall-normal axis is tanh-stretched towards
the wall, so every metric term is active.  Seeded state: a tanh velocity
profile of free-stream Mach 6 with the Crocco-Busemann temperature between
the 300 K wall and the free stream, uniform pressure, air with traces of NO,
N and O, plus 0.5 % seeded noise on velocity, temperature and pressure.

`BoundaryRun` advances such a grid by SSP-RK3 steps composed from the task
entry points in the order of the reference's driver (src/prometeo.rg:
1342-1486, 429-606): per stage the time derivatives over p_All, chemistry
over p_solved, Euler fluxes Z, Y, X and diffusion fluxes Z, Y, X over the
divergence zones, the NSCBC outflow terms (with the maximum Mach number of
the interior), the NSCBC inflow terms, the RK update over p_All, then the
primitive recovery of the interior, the boundary states (inflow, outflow,
then walls in the order z, y, x; src/prometeo_bc.rg:1445-1660), properties
everywhere and conserved variables of every boundary point; after the step
the inflow time derivatives (src/prometeo_bc.rg:1814-1879).  Zones come from
zones.partition.  It runs on any library exporting the C ABI: the CUDA
library on device fields, or a CPU build on host fields.
"""
import ctypes as C
import math

import numpy as np

from . import abi, zones
from .fluid import Fluid
from .grid import Grid, PERIODIC
from .workloads import AIR_REF

RK_C = ((1.0, 0.0, 1.0), (3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0), (1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0))
SUPPORTED = {PERIODIC, "NSCBC_Inflow", "NSCBC_Outflow", "IsothermalWall", "AdiabaticWall"}
SIDE_NAMES = ("XNeg", "XPos", "YNeg", "YPos", "ZNeg", "ZPos")

# species molar weights of AirMix (N2, O2, NO, N, O), kg/mol
W_AIR = np.array([2 * 14.0067e-3, 2 * 15.9994e-3, 14.0067e-3 + 15.9994e-3, 14.0067e-3, 15.9994e-3])
RGAS = 8.3144598


def boundary_layer(num=(512, 192, 128), seed=0, mach=6.0, T_inf=220.0, p_inf=1.0e4, T_wall=300.0,
                   width=(0.2, 0.02, 0.01), delta=0.004, stretching=1.0, noise=0.005):
    """Host Fluid of the boundary-layer workload (interior cells `num`;
    SI inputs, nondimensionalised with PRef 1 atm, TRef 300 K, LRef 1 m).
    Node types are set; metrics are filled by `Grid.fill` with a library."""
    bc = (("NSCBC_Inflow", "NSCBC_Outflow"), ("IsothermalWall", "NSCBC_Outflow"), (PERIODIC, PERIODIC))
    g = Grid(num, width, bc, kind=(("Uniform", 1.0), ("TanhMinus", stretching), ("Uniform", 1.0)))
    nx, ny, nz = g.shape
    rng = np.random.Generator(np.random.PCG64(seed))
    ref = AIR_REF
    Y = np.array([0.767, 0.233, 1.0e-4, 1.0e-6, 1.0e-5])
    Y = Y / Y.sum()
    X = (Y / W_AIR) / (Y / W_AIR).sum()
    MixW = float((X * W_AIR).sum())
    gamma = 1.4
    a_inf = math.sqrt(gamma * RGAS / MixW * T_inf)
    U = mach * a_inf
    Tr = T_inf * (1.0 + 0.89 * 0.5 * (gamma - 1.0) * mach * mach)
    yc = np.maximum(g.center[1], 0.0)
    f = np.tanh(3.0 * yc / delta)                      # u / U
    T_prof = T_wall + (Tr - T_wall) * f - (Tr - T_inf) * f * f
    shape3 = (nz, ny, nx)
    u_prof = np.zeros(shape3 + (3,))
    u_prof[..., 0] = (U * f)[None, :, None]
    T3 = np.broadcast_to(T_prof[None, :, None], shape3)
    # nondimensionalisation of AirMix (src/Mixtures/MultiComponent.inl:438-487)
    XiRef = np.where(np.array(ref["XiRef"]) > 0, np.array(ref["XiRef"]), 1e-60)
    MixWRef = float((XiRef * W_AIR).sum())
    rhoRef = ref["PRef"] * MixWRef / (RGAS * ref["TRef"])
    uRef = math.sqrt(ref["PRef"] / rhoRef)
    fl = Fluid(g.shape, 5)
    pert = lambda: 1.0 + noise * rng.uniform(-1.0, 1.0, size=shape3)
    vel = u_prof.copy()
    for k in range(3):
        vel[..., k] += noise * U * rng.uniform(-1.0, 1.0, size=shape3)
    vel[:, 0, :, :] = 0.0  # the wall ghost is at rest
    T = T3 * pert()
    T[:, 0, :] = T_wall
    fl["pressure"] = p_inf * pert() / ref["PRef"]
    fl["temperature"] = T / ref["TRef"]
    fl["MolarFracs"] = X
    fl["velocity"] = vel / uRef
    fl["MolarFracs_profile"] = X
    fl["temperature_profile"] = T3 / ref["TRef"]
    fl["velocity_profile"] = u_prof / uRef
    fl["velocity_old_NSCBC"] = fl["velocity"]
    fl["temperature_old_NSCBC"] = fl["temperature"]
    for name, d in (("nType_x", 0), ("nType_y", 1), ("nType_z", 2)):
        idx = [None, None, None]
        idx[2 - d] = slice(None)
        fl[name] = np.broadcast_to(g.ntype[d][tuple(idx)], shape3)
    for name in ("shockSensorX", "shockSensorY", "shockSensorZ"):
        fl[name] = True  # the reference's initial value (src/prometeo.rg:335-338)
    P = p_inf / ref["PRef"]
    fl.meta = dict(workload="boundary_layer", eos=abi.HTR_EOS_AIRMIX, seed=seed, mix=dict(ref), grid=g,
                   bnum=g.bnum, bc=dict(xNeg=("NSCBC_Inflow", {"P": P}),
                                        xPos=("NSCBC_Outflow", {"P": P, "LengthScale": width[0]}),
                                        yNeg=("IsothermalWall", {}),
                                        yPos=("NSCBC_Outflow", {"P": P, "LengthScale": width[1]}),
                                        zNeg=(PERIODIC, {}), zPos=(PERIODIC, {})),
                   scheme="TENOLAD", cfl=0.8, mach=mach)
    return fl


def channel(num=(64, 48, 32), seed=0, mach=0.5, T_wall=300.0, p0=1.0e5, width=(0.06, 0.02, 0.03),
            stretching=1.5, noise=0.01):
    """Host Fluid of a wall-bounded channel: periodic x and z, an isothermal
    wall (300 K) at yNeg and an adiabatic wall at yPos, both tanh-clustered
    (Tanh stretching), 5-species air, a parabolic streamwise velocity of
    centre-line Mach `mach` with 1 % seeded noise, uniform temperature and
    pressure.  Node types are set; metrics are filled by `Grid.fill`."""
    bc = ((PERIODIC, PERIODIC), ("IsothermalWall", "AdiabaticWall"), (PERIODIC, PERIODIC))
    g = Grid(num, width, bc, kind=(("Uniform", 1.0), ("Tanh", stretching), ("Uniform", 1.0)))
    nx, ny, nz = g.shape
    rng = np.random.Generator(np.random.PCG64(seed))
    ref = AIR_REF
    Y = np.array([0.767, 0.233, 1.0e-4, 1.0e-6, 1.0e-5])
    Y = Y / Y.sum()
    X = (Y / W_AIR) / (Y / W_AIR).sum()
    MixW = float((X * W_AIR).sum())
    U = mach * math.sqrt(1.4 * RGAS / MixW * T_wall)
    eta = np.clip(g.center[1] / width[1], 0.0, 1.0)
    shape3 = (nz, ny, nx)
    u = np.zeros(shape3 + (3,))
    u[..., 0] = (4.0 * U * eta * (1.0 - eta))[None, :, None]
    for k in range(3):
        u[..., k] += noise * U * rng.uniform(-1.0, 1.0, size=shape3)
    u[:, 0] = 0.0
    u[:, -1] = 0.0
    XiRef = np.where(np.array(ref["XiRef"]) > 0, np.array(ref["XiRef"]), 1e-60)
    MixWRef = float((XiRef * W_AIR).sum())
    rhoRef = ref["PRef"] * MixWRef / (RGAS * ref["TRef"])
    uRef = math.sqrt(ref["PRef"] / rhoRef)
    fl = Fluid(g.shape, 5)
    fl["pressure"] = p0 * (1.0 + noise * rng.uniform(-1.0, 1.0, size=shape3)) / ref["PRef"]
    fl["temperature"] = T_wall * (1.0 + noise * rng.uniform(-1.0, 1.0, size=shape3)) / ref["TRef"]
    fl["MolarFracs"] = X
    fl["velocity"] = u / uRef
    fl["MolarFracs_profile"] = X
    fl["temperature_profile"] = T_wall / ref["TRef"]
    fl["velocity_profile"] = 0.0
    for name, d in (("nType_x", 0), ("nType_y", 1), ("nType_z", 2)):
        idx = [None, None, None]
        idx[2 - d] = slice(None)
        fl[name] = np.broadcast_to(g.ntype[d][tuple(idx)], shape3)
    for name in ("shockSensorX", "shockSensorY", "shockSensorZ"):
        fl[name] = True
    fl.meta = dict(workload="channel", eos=abi.HTR_EOS_AIRMIX, seed=seed, mix=dict(ref), grid=g, bnum=g.bnum,
                   bc=dict(xNeg=(PERIODIC, {}), xPos=(PERIODIC, {}), yNeg=("IsothermalWall", {}),
                           yPos=("AdiabaticWall", {}), zNeg=(PERIODIC, {}), zPos=(PERIODIC, {})),
                   scheme="TENOLAD", cfl=0.8, mach=mach)
    return fl


def _rects(boxes):
    return [abi.rect(*b) for b in boxes]


class BoundaryRun:
    """SSP-RK3 steps of one grid with boundary conditions through `lib`.

    bc      {side: (FlowBC type, params)} for the six sides (xNeg ... zPos);
            NSCBC_Inflow takes P (the pressure of a supersonic inflow),
            NSCBC_Outflow takes P and LengthScale
    scheme  one of Hybrid, TENO, TENOA, TENOLAD, SkewSymmetric; the hybrid
            scheme updates the Ducros sensor everywhere and the shock sensor
            of direction d over its faces zone once per step
            (UpdateShockSensors, src/prometeo_sensor.rg:96-125)
    max_mach_buffer  where htr_CalculateMaxMachNumber writes: a device
            pointer for the CUDA library, None (a host double) for a CPU build
    """

    def __init__(self, lib, fl, mixh, bc, scheme="TENOLAD", chemistry=True, stream=None, max_mach_buffer=None,
                 vorticity_scale=1.0):
        self.lib, self.fl, self.mixh = lib, fl, mixh
        self.types = [bc[s][0] for s in zones.SIDES]
        self.params = [bc[s][1] for s in zones.SIDES]
        for t in self.types:
            if t not in SUPPORTED:
                raise abi.HtrError(f"boundary condition {t} is not supported by this driver")
        axes = tuple((self.types[2 * d], self.types[2 * d + 1]) for d in range(3))
        self.bnum = tuple(0 if a[0] == PERIODIC else 1 for a in axes)
        self.z = zones.partition(fl.shape, self.bnum, axes)
        if scheme not in ("Hybrid", "TENO", "TENOA", "TENOLAD", "SkewSymmetric"):
            raise abi.HtrError(f"scheme {scheme} is not supported by this driver")
        self.scheme, self.chemistry, self.vs = scheme, chemistry, vorticity_scale
        self.stream = stream
        self.mach_buf = max_mach_buffer
        self.all = abi.rect(*self.z.all)
        self.interior = abi.rect(*self.z.interior)
        self.solved = _rects(self.z.solved)
        self.divg = [_rects(r) for r in self.z.divg]
        self.planes = [_rects(p) for p in self.z.planes]
        self.all_bcs = _rects(self.z.all_bcs)
        self.faces = [_rects(f) for f in self.z.faces]

    def _ck(self, st, what):
        abi.check(self.lib, st, what)

    def max_mach(self, d):
        """max |u_d| / c over the interior (the reference's future)."""
        v = self.fl.view()
        if self.mach_buf is None:
            out = C.c_double(0.0)
            self._ck(self.lib.htr_CalculateMaxMachNumber(C.byref(v), self.interior, d, C.byref(out), self.stream),
                     "max mach")
            return out.value
        ptr = C.cast(C.c_void_p(self.mach_buf.data_ptr()), C.POINTER(C.c_double))
        self._ck(self.lib.htr_CalculateMaxMachNumber(C.byref(v), self.interior, d, ptr, self.stream), "max mach")
        return float(self.mach_buf.item())

    def spectral_dt(self, cfl):
        v = self.fl.view()
        if self.mach_buf is None:
            r = C.c_double(0.0)
            self._ck(self.lib.htr_CalculateMaxSpectralRadius(C.byref(v), self.interior, self.mixh, C.byref(r),
                                                             self.stream), "cfl")
            return cfl / r.value
        ptr = C.cast(C.c_void_p(self.mach_buf.data_ptr()), C.POINTER(C.c_double))
        self._ck(self.lib.htr_CalculateMaxSpectralRadius(C.byref(v), self.interior, self.mixh, ptr, self.stream),
                 "cfl")
        return cfl / float(self.mach_buf.item())

    def sensors(self):
        """UpdateShockSensors (src/prometeo_sensor.rg:96-125)."""
        v = self.fl.view()
        fb = self.fl.bounds()
        self._ck(self.lib.htr_UpdateDucrosSensor(C.byref(v), self.all, fb, self.vs, self.stream), "ducros")
        for d in range(3):
            fn = getattr(self.lib, f"htr_UpdateShockSensor{'XYZ'[d]}")
            for r in self.faces[d]:
                self._ck(fn(C.byref(v), r, fb, self.mixh, self.stream), "shock sensor")

    def derivatives(self, stage, dt):
        """UpdateDerivatives (src/prometeo.rg:480-606)."""
        lib, s, m = self.lib, self.stream, self.mixh
        v = self.fl.view()
        fb = self.fl.bounds()
        self._ck(lib.htr_InitializeTimeDerivatives(C.byref(v), self.all, 0, m, s), "init_t")
        if self.chemistry:
            for r in self.solved:
                self._ck(lib.htr_AddChemistrySources(C.byref(v), r, m, s), "chemistry")
        rk = (C.c_double * 2)(RK_C[stage - 1][0], RK_C[stage - 1][1])
        ddt = dt * RK_C[stage - 1][2]
        for d in (2, 1, 0):
            for r in self.divg[d]:
                if self.scheme == "SkewSymmetric":
                    st = getattr(lib, f"htr_UpdateUsingSkewSymmetricEulerFlux{'XYZ'[d]}")(C.byref(v), r, fb, m, s)
                else:
                    st = getattr(lib, f"htr_UpdateUsing{self.scheme}EulerFlux{'XYZ'[d]}")(C.byref(v), r, fb, rk, ddt,
                                                                                          m, s)
                self._ck(st, "euler")
        for d in (2, 1, 0):
            for r in self.divg[d]:
                self._ck(getattr(lib, f"htr_UpdateUsingDiffusionFlux{'XYZ'[d]}")(C.byref(v), r, fb, m, s), "diffusion")
        for d in range(3):
            sides = [2 * d, 2 * d + 1]
            if not any(self.types[k] == "NSCBC_Outflow" for k in sides):
                continue
            mach = self.max_mach(d)
            for k in sides:
                if self.types[k] != "NSCBC_Outflow":
                    continue
                prm = self.params[k]
                fn = getattr(lib, f"htr_UpdateUsingFluxNSCBCOutflow{SIDE_NAMES[k]}")
                for r in self.planes[k]:
                    self._ck(fn(C.byref(v), r, fb, m, mach, prm["LengthScale"], prm["P"], s), "nscbc outflow")
        for k in range(6):
            if self.types[k] == "NSCBC_Inflow":
                fn = getattr(lib, f"htr_UpdateUsingFluxNSCBCInflow{SIDE_NAMES[k]}")
                for r in self.planes[k]:
                    self._ck(fn(C.byref(v), r, m, s), "nscbc inflow")

    def refresh(self):
        """UpdatePrimitivesAndBCsFromConserved (src/prometeo.rg:429-478)."""
        lib, s, m = self.lib, self.stream, self.mixh
        v = self.fl.view()
        self._ck(lib.htr_UpdatePrimitiveFromConserved(C.byref(v), self.interior, m, s), "primitives")
        for k in range(6):
            t = self.types[k]
            for r in self.planes[k]:
                if t == "NSCBC_Inflow":
                    st = getattr(lib, f"htr_SetNSCBC_InflowBC{'XYZ'[k // 2]}")(C.byref(v), r, m, self.params[k]["P"], s)
                elif t == "NSCBC_Outflow":
                    st = lib.htr_SetNSCBC_OutflowBC(C.byref(v), r, m, None, s)
                else:
                    continue
                self._ck(st, "boundary state")
        for k in (4, 5, 2, 3, 0, 1):
            t = self.types[k]
            if t not in ("IsothermalWall", "AdiabaticWall"):
                continue
            fn = lib.htr_SetIsothermalWallBC if t == "IsothermalWall" else lib.htr_SetAdiabaticWallBC
            for r in self.planes[k]:
                self._ck(fn(C.byref(v), r, k, m, s), "wall")
        self._ck(lib.htr_UpdatePropertiesFromPrimitive(C.byref(v), self.all, m, s), "properties")
        for r in self.all_bcs:
            self._ck(lib.htr_UpdateConservedFromPrimitive(C.byref(v), r, m, s), "conserved")

    def step(self, dt=None, cfl=0.8):
        """One SSP-RK3 step; returns the step size."""
        if dt is None:
            dt = self.spectral_dt(cfl)
        if self.scheme == "Hybrid":
            self.sensors()
        v = self.fl.view()
        self._ck(self.lib.htr_InitializeTemporaries(C.byref(v), self.all, self.mixh, self.stream), "temporaries")
        for stage in (1, 2, 3):
            self.derivatives(stage, dt)
            self._ck(self.lib.htr_UpdateVars(C.byref(v), self.all, stage, dt, 0, self.mixh, self.stream), "rk")
            self.refresh()
        for k in range(6):
            if self.types[k] == "NSCBC_Inflow":
                for r in self.planes[k]:
                    self._ck(self.lib.htr_UpdateNSCBCGhostCellTimeDerivatives(C.byref(v), r, dt, self.stream),
                             "inflow time derivatives")
        return dt


class FusedBoundaryRun:
    """The same steps as BoundaryRun through htr_rk3_step_bc_ws: the fused
    stage pipeline over the whole grid with the NSCBC and wall rules folded
    into its per-cell kernel (CUDA library, device fields).  With a fixed dt
    the step issues no host synchronisation and can be graph-captured."""

    def __init__(self, fl, mixh, bc, scheme="TENOLAD", chemistry=True, stream=None, workspace=None,
                 vorticity_scale=1.0):
        from . import runtime
        self.rt = runtime
        self.lib = runtime.lib()
        self.fl, self.mixh = fl, mixh
        types = [bc[s][0] for s in zones.SIDES]
        params = [bc[s][1] for s in zones.SIDES]
        for t in types:
            if t not in runtime.BC_TYPES:
                raise abi.HtrError(f"boundary condition {t} is not supported by the fused boundary step")
        axes = tuple((types[2 * d], types[2 * d + 1]) for d in range(3))
        bnum = tuple(0 if a[0] == PERIODIC else 1 for a in axes)
        z = zones.partition(fl.shape, bnum, axes)
        nscbc = lambda t: t in ("NSCBC_Inflow", "NSCBC_Outflow")
        if types[4] != PERIODIC and (nscbc(types[4]) != nscbc(types[2]) or nscbc(types[5]) != nscbc(types[3])):
            # the reference's zones take the z sides' characteristic flags from
            # the y sides; the fused step reads the z sides' node types
            raise abi.HtrError("the fused boundary step needs z periodic, or z sides of the y sides' kinds")
        self.params = runtime.htr_bc_params()
        for k in range(6):
            self.params.type[k] = runtime.BC_TYPES[types[k]]
            self.params.P[k] = params[k].get("P", 0.0)
            self.params.LengthScale[k] = params[k].get("LengthScale", 0.0)
            if types[k] != PERIODIC:
                if len(z.planes[k]) != 1:
                    raise abi.HtrError(f"boundary plane {zones.SIDES[k]} is not one rectangle")
                self.params.plane[k] = abi.rect(*z.planes[k][0])
        for d in range(3):
            if len(z.faces[d]) != 1:
                raise abi.HtrError(f"sensor zone of direction {'xyz'[d]} is not one rectangle")
            self.params.sensor[d] = abi.rect(*z.faces[d][0])
        self.interior = abi.rect(*z.interior)
        self.scheme = runtime.SCHEMES[scheme]
        self.vs = vorticity_scale
        self.chemistry = chemistry
        self.stream = stream
        self.ws = workspace or runtime.Workspace()
        self.nbytes = self.lib.htr_rk3_workspace_bytes(fl.bounds(), mixh)
        self.ws.get(self.nbytes, fl.device)

    def step(self, dt=0.0, cfl=0.0, status_dev=None):
        """One SSP-RK3 step with step size dt (or cfl > 0); returns the dt used."""
        p = self.rt.htr_step_params(self.scheme, self.vs, cfl, dt, 1 if self.chemistry else 0)
        v = self.fl.view()
        used = C.c_double(0.0)
        ws = self.ws.get(self.nbytes, self.fl.device)
        st = self.lib.htr_rk3_step_bc_ws(C.byref(v), self.interior, self.fl.bounds(), C.byref(p),
                                         C.byref(self.params), self.mixh, C.c_void_p(ws), self.nbytes,
                                         C.byref(used), status_dev, self.rt.stream_handle(self.stream))
        abi.check(self.lib, st, "htr_rk3_step_bc_ws")
        return used.value
