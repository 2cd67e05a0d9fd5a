"""CPU oracles for the HTR explicit-RHS path.  TEST INFRASTRUCTURE ONLY.

Only the test suite, the smoke check and the CPU-baseline leg of bench.py
may load anything from this directory; the GPU product never does.

Two oracles implement the same C ABI as the CUDA library (include/htr_rhs.h):

* `ref`  — the reference solver's own CPU task code (HTR src/prometeo_*.cc),
  compiled unmodified against a Legion stand-in by oracle/ref/Makefile into
  oracle/_ref/libhtrref_<EOS>.so.  It can only be built where the reference
  sources are present; it is the pin for everything else.
* `port` — a from-scratch C++ restatement of the same algorithms
  (oracle/port/), built into oracle/_build/libhtroracle.so on every machine.
  It is checked against `ref` here and against golden vectors from `ref`
  (tests/golden/) everywhere.

`step` restates the driver order of one SSP-RK3 time step of the reference
(MainLoopHeader + MainLoopBody, src/prometeo.rg:1153-1172 and 1342-1486,
UpdateDerivatives :480-606, UpdatePrimitivesAndBCsFromConserved :428-478)
on top of any library exporting the ABI.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BUILD_DIR = os.path.join(HERE, "_build")

RK_C = ((1.0, 0.0, 1.0), (3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0), (1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0))

_cache = {}


def _abi():
    import sys
    if "htr_gb300" not in sys.modules:
        sys.path.insert(0, os.path.dirname(HERE))
        import __graft_entry__  # noqa: F401  (registers the package)
        __graft_entry__.load_package()
    return sys.modules["htr_gb300.abi"]


def ref_path(eos):
    name = {1: "ConstPropMix", 2: "AirMix"}[eos]
    return os.path.join(REF_DIR, f"libhtrref_{name}.so")


def ref_lib(eos):
    """The compiled reference for `eos`, or None where it was not built."""
    p = ref_path(eos)
    if not os.path.exists(p):
        return None
    key = ("ref", eos)
    if key not in _cache:
        lib = C.CDLL(p)
        _abi().bind(lib, {"htr_ref_mix_offsets": [C.POINTER(C.c_longlong), C.c_int]})
        lib.htr_ref_mix_sizeof.restype = C.c_size_t
        _cache[key] = lib
    return _cache[key]


def port_path():
    return os.path.join(BUILD_DIR, "libhtroracle.so")


def port_lib():
    """The from-scratch CPU restatement (built by build())."""
    key = ("port",)
    if key not in _cache:
        p = port_path()
        if not os.path.exists(p):
            raise FileNotFoundError(f"{p} missing: run __graft_entry__.build()")
        lib = C.CDLL(p)
        _abi().bind(lib)
        lib.htr_oracle_set_threads.argtypes = [C.c_int]
        lib.htr_oracle_set_threads.restype = C.c_int
        _cache[key] = lib
    return _cache[key]


def load_mixture(lib, eos, struct):
    h = C.c_void_p()
    st = lib.htr_load_mixture(eos, C.byref(struct), C.sizeof(struct), C.byref(h))
    _abi().check(lib, st, "htr_load_mixture")
    return h


def spectral_dt(lib, fl, mixh, cfl):
    v = fl.view()
    r = C.c_double(0.0)
    _abi().check(lib, lib.htr_CalculateMaxSpectralRadius(C.byref(v), fl.interior(), mixh,
                                                        C.byref(r), None), "cfl")
    return cfl / r.value


def update_derivatives(lib, fl, mixh, stage, dt, scheme="Hybrid", chemistry=True, bnum=(0, 0, 0),
                       old_derivatives=False, limiter=None):
    """One RHS evaluation in the reference's order (UpdateDerivatives,
    prometeo.rg:480-606).  old_derivatives: Conserved_t starts from
    -Conserved_t_old and the limiter's deltaTime is halved (the RK stages of
    implicit chemistry).  limiter = (RK_coeffs, deltaTime) overrides the
    stage's limiter arguments (the implicit pre-step passes ({0, 1}, dt/2))."""
    A = _abi()
    v = fl.view()
    allr = fl.bounds()
    inner = fl.interior(bnum)
    fb = fl.bounds()
    A.check(lib, lib.htr_InitializeTimeDerivatives(C.byref(v), allr, 1 if old_derivatives else 0, mixh, None),
            "init_t")
    if chemistry:
        A.check(lib, lib.htr_AddChemistrySources(C.byref(v), inner, mixh, None), "chem")
    if limiter is not None:
        rk = (C.c_double * 2)(*limiter[0])
        ddt = limiter[1]
    else:
        rk = (C.c_double * 2)(RK_C[stage - 1][0], RK_C[stage - 1][1])
        ddt = dt * RK_C[stage - 1][2]
        if old_derivatives:
            ddt *= 0.5
    for d in "ZYX":
        if scheme == "SkewSymmetric":
            fn = getattr(lib, f"htr_UpdateUsingSkewSymmetricEulerFlux{d}")
            st = fn(C.byref(v), inner, fb, mixh, None)
        else:
            fn = getattr(lib, f"htr_UpdateUsing{scheme}EulerFlux{d}")
            st = fn(C.byref(v), inner, fb, rk, ddt, mixh, None)
        A.check(lib, st, f"euler {scheme} {d}")
    for d in "ZYX":
        fn = getattr(lib, f"htr_UpdateUsingDiffusionFlux{d}")
        A.check(lib, fn(C.byref(v), inner, fb, mixh, None), f"diffusion {d}")


def update_sensors(lib, fl, mixh, vorticity_scale):
    A = _abi()
    v = fl.view()
    r = fl.bounds()
    A.check(lib, lib.htr_UpdateDucrosSensor(C.byref(v), r, r, vorticity_scale, None), "ducros")
    for d in "XYZ":
        fn = getattr(lib, f"htr_UpdateShockSensor{d}")
        A.check(lib, fn(C.byref(v), r, r, mixh, None), f"shock {d}")


def refresh(lib, fl, mixh, bnum=(0, 0, 0)):
    """UpdatePrimitivesAndBCsFromConserved (prometeo.rg:429-478) for periodic
    grids and constant (Dirichlet) ghost nodes, whose state stays imposed."""
    A = _abi()
    v = fl.view()
    A.check(lib, lib.htr_UpdatePrimitiveFromConserved(C.byref(v), fl.interior(bnum), mixh, None),
            "prim")
    A.check(lib, lib.htr_UpdatePropertiesFromPrimitive(C.byref(v), fl.bounds(), mixh, None),
            "props")


def step(lib, fl, mixh, scheme="Hybrid", vorticity_scale=1.0, cfl=0.8, dt=None, chemistry=True,
         stages=3, hook=None, bnum=(0, 0, 0), implicit=False):
    """One SSP-RK3 time step; returns the dt used.  `bnum` ghost layers per
    side hold Dirichlet states: the RHS, the RK update and the primitive
    recovery run on the interior only (the reference restores ghost
    conserved variables from their imposed primitives after each update).
    implicit: Integrator.implicitChemistry (prometeo.rg:1360-1398): the
    transport RHS of the start state (RK_coeffs {0, 1}, deltaTime dt/2),
    UpdateChemistry over dt, the refresh, then the RK stages without
    chemistry sources, from -Conserved_t_old and with dt halved
    (prometeo_rk.rg:59-112)."""
    A = _abi()
    if dt is None:
        dt = spectral_dt(lib, fl, mixh, cfl)
    if scheme == "Hybrid":
        update_sensors(lib, fl, mixh, vorticity_scale)
    v = fl.view()
    if implicit:
        update_derivatives(lib, fl, mixh, 1, dt, scheme, False, bnum, limiter=((0.0, 1.0), dt * 0.5))
        status = C.c_int(0)
        A.check(lib, lib.htr_UpdateChemistry(C.byref(v), fl.interior(bnum), dt, mixh, C.byref(status), None),
                "UpdateChemistry")
        if status.value != 0:
            raise A.HtrError(f"UpdateChemistry status {status.value}")
        refresh(lib, fl, mixh, bnum)
    A.check(lib, lib.htr_InitializeTemporaries(C.byref(v), fl.bounds(), mixh, None), "tmp")
    for s in range(1, stages + 1):
        update_derivatives(lib, fl, mixh, s, dt, scheme, chemistry and not implicit, bnum, old_derivatives=implicit)
        if hook is not None:
            hook(s, fl)
        A.check(lib, lib.htr_UpdateVars(C.byref(v), fl.interior(bnum), s, dt, 1 if implicit else 0, mixh, None),
                "rk")
        refresh(lib, fl, mixh, bnum)
    return dt


def boundary_layer_zones(nx, ny, nz):
    """Zones of a one-tile grid (one ghost layer in x and y, periodic z) with
    an NSCBC inflow at xNeg, NSCBC outflows at xPos and yPos and a wall at
    yNeg, written out by hand from PartitionZones
    (src/prometeo_partitioner.rg:431-1015): the xNeg-yNeg and xPos-yNeg edges
    go to the wall, xNeg-yPos to the inflow, xPos-yPos to both outflows; the
    flux divergence of x skips the x planes, that of y skips the y planes;
    the wall plane is not solved.  Sensor zones (p_{x,y,z}_faces): the
    interior and the Neg ghost face of the direction, plus the NSCBC x faces
    and the yPos outflow face with their edges towards the Neg sides."""
    X0, X1, Y0, Y1, Z1 = 0, nx - 1, 0, ny - 1, nz - 1
    box = lambda x0, x1, y0, y1: ((x0, y0, 0), (x1, y1, Z1))
    return dict(
        all=box(X0, X1, Y0, Y1), interior=box(1, X1 - 1, 1, Y1 - 1), solved=box(X0, X1, 1, Y1),
        divg=(box(1, X1 - 1, 1, Y1), box(X0, X1, 1, Y1 - 1), box(X0, X1, 1, Y1)),
        xNeg=box(X0, X0, 1, Y1), xPos=box(X1, X1, 1, Y1), yNeg=box(X0, X1, Y0, Y0), yPos=box(1, X1, Y1, Y1),
        faces=(box(X0, X1 - 1, 1, Y1), box(X0, X1, Y0, Y1 - 1), box(X0, X1, 1, Y1)),
        all_bcs=(box(X0, X0, Y0, Y1), box(X1, X1, Y0, Y1), box(1, X1 - 1, Y0, Y0), box(1, X1 - 1, Y1, Y1)))


def boundary_layer_step(lib, fl, mixh, dt, P_in, P_out, L_out, scheme="TENOLAD", regent=None, regent_mix=None,
                        vorticity_scale=1.0):
    """One SSP-RK3 step of a boundary-layer grid (zones above) in the
    reference's order: MainLoopBody (src/prometeo.rg:1342-1486) with
    UpdateDerivatives (:480-606), the NSCBC outflow terms of x then y with
    the interior's maximum Mach number (src/prometeo_rhs.rg:672-765), the
    inflow terms (:540-596), UpdatePrimitivesAndBCsFromConserved
    (:428-478) with UpdateGhostPrimitives (src/prometeo_bc.rg:1445-1660) and
    the inflow time derivatives (src/prometeo_bc.rg:1814-1879).  `regent`
    provides the Regent-defined pieces (wall state, maximum Mach number,
    NSCBC time derivatives) when `lib` lacks them, with its mixture handle
    `regent_mix`; L_out = (LengthScale of the x outflow, of the y outflow)."""
    A = _abi()
    R = regent if regent is not None else lib
    RM = regent_mix if regent is not None else mixh
    z = boundary_layer_zones(fl.nx, fl.ny, fl.nz)
    rc = lambda b: A.rect(*b)
    v = fl.view()
    fb = fl.bounds()
    if scheme == "Hybrid":
        # UpdateShockSensors (src/prometeo_sensor.rg:96-125)
        A.check(lib, lib.htr_UpdateDucrosSensor(C.byref(v), rc(z["all"]), fb, vorticity_scale, None), "ducros")
        for d in range(3):
            fn = getattr(lib, f"htr_UpdateShockSensor{'XYZ'[d]}")
            A.check(lib, fn(C.byref(v), rc(z["faces"][d]), fb, mixh, None), "shock")
    A.check(lib, lib.htr_InitializeTemporaries(C.byref(v), rc(z["all"]), mixh, None), "tmp")
    for s in range(1, 4):
        A.check(lib, lib.htr_InitializeTimeDerivatives(C.byref(v), rc(z["all"]), 0, mixh, None), "init_t")
        A.check(lib, lib.htr_AddChemistrySources(C.byref(v), rc(z["solved"]), mixh, None), "chem")
        rk = (C.c_double * 2)(RK_C[s - 1][0], RK_C[s - 1][1])
        ddt = dt * RK_C[s - 1][2]
        for d in (2, 1, 0):
            fn = getattr(lib, f"htr_UpdateUsing{scheme}EulerFlux{'XYZ'[d]}")
            A.check(lib, fn(C.byref(v), rc(z["divg"][d]), fb, rk, ddt, mixh, None), "euler")
        for d in (2, 1, 0):
            fn = getattr(lib, f"htr_UpdateUsingDiffusionFlux{'XYZ'[d]}")
            A.check(lib, fn(C.byref(v), rc(z["divg"][d]), fb, mixh, None), "diffusion")
        for d, side, L in ((0, "XPos", L_out[0]), (1, "YPos", L_out[1])):
            mach = C.c_double(0.0)
            A.check(R, R.htr_CalculateMaxMachNumber(C.byref(v), rc(z["interior"]), d, C.byref(mach), None), "mach")
            fn = getattr(lib, f"htr_UpdateUsingFluxNSCBCOutflow{side}")
            A.check(lib, fn(C.byref(v), rc(z[side[0].lower() + "Pos"]), fb, mixh, mach.value, L, P_out, None),
                    "outflow")
        A.check(lib, lib.htr_UpdateUsingFluxNSCBCInflowXNeg(C.byref(v), rc(z["xNeg"]), mixh, None), "inflow")
        A.check(lib, lib.htr_UpdateVars(C.byref(v), rc(z["all"]), s, dt, 0, mixh, None), "rk")
        A.check(lib, lib.htr_UpdatePrimitiveFromConserved(C.byref(v), rc(z["interior"]), mixh, None), "prim")
        A.check(lib, lib.htr_SetNSCBC_InflowBCX(C.byref(v), rc(z["xNeg"]), mixh, P_in, None), "in bc")
        A.check(lib, lib.htr_SetNSCBC_OutflowBC(C.byref(v), rc(z["xPos"]), mixh, None, None), "out bc x")
        A.check(lib, lib.htr_SetNSCBC_OutflowBC(C.byref(v), rc(z["yPos"]), mixh, None, None), "out bc y")
        A.check(R, R.htr_SetIsothermalWallBC(C.byref(v), rc(z["yNeg"]), 2, RM, None), "wall")
        A.check(lib, lib.htr_UpdatePropertiesFromPrimitive(C.byref(v), rc(z["all"]), mixh, None), "props")
        for b in z["all_bcs"]:
            A.check(lib, lib.htr_UpdateConservedFromPrimitive(C.byref(v), rc(b), mixh, None), "cons")
    A.check(R, R.htr_UpdateNSCBCGhostCellTimeDerivatives(C.byref(v), rc(z["xNeg"]), dt, None), "dudt")
    return dt
