"""ctypes mirror of include/htr_rhs.h and include/htr_mix.h.

The same C ABI is exported by the CUDA library of this package and by the
CPU oracles used in the tests, so one set of declarations drives both.
Field layout follows HTR's Fluid_columns (src/prometeo_types.h:49-114): one
array per field, element = the reference element type (components
contiguous), addressed with byte strides in x, y and z.
"""
import ctypes as C

HTR_EOS_CONSTPROPMIX = 1
HTR_EOS_AIRMIX = 2

HTR_VISC_CONSTANT = 0
HTR_VISC_POWERLAW = 1
HTR_VISC_SUTHERLAND = 2

STATUS_NAMES = {
    0: "HTR_OK",
    1: "HTR_ERR_ARGUMENT",
    2: "HTR_ERR_LAYOUT",
    3: "HTR_ERR_CUDA",
    4: "HTR_ERR_ITERATION_CAP",
    5: "HTR_ERR_UNSUPPORTED",
    6: "HTR_ERR_NO_DEVICE",
    7: "HTR_ERR_IO",
    8: "HTR_ERR_FORMAT",
}


HTR_OK = 0
HTR_ERR_ARGUMENT = 1
HTR_ERR_LAYOUT = 2
HTR_ERR_CUDA = 3
HTR_ERR_ITERATION_CAP = 4
HTR_ERR_UNSUPPORTED = 5
HTR_ERR_NO_DEVICE = 6
HTR_ERR_IO = 7
HTR_ERR_FORMAT = 8


class HtrError(RuntimeError):
    pass


class htr_field(C.Structure):
    _fields_ = [("base", C.c_void_p), ("stride", C.c_int64 * 3)]


class htr_rect3(C.Structure):
    _fields_ = [("lo", C.c_int64 * 3), ("hi", C.c_int64 * 3)]


# (name, dtype, components) in htr_fluid_view order; components may be
# "nSpec", "nEq" or an int.
FIELD_SPECS = [
    ("nType_x", "int32", 1), ("nType_y", "int32", 1), ("nType_z", "int32", 1),
    ("dcsi_e", "float64", 1), ("deta_e", "float64", 1), ("dzet_e", "float64", 1),
    ("dcsi_d", "float64", 1), ("deta_d", "float64", 1), ("dzet_d", "float64", 1),
    ("dcsi_s", "float64", 1), ("deta_s", "float64", 1), ("dzet_s", "float64", 1),
    ("rho", "float64", 1), ("mu", "float64", 1), ("lam", "float64", 1),
    ("Di", "float64", "nSpec"), ("SoS", "float64", 1),
    ("pressure", "float64", 1), ("temperature", "float64", 1),
    ("MassFracs", "float64", "nSpec"), ("MolarFracs", "float64", "nSpec"),
    ("velocity", "float64", 3),
    ("Conserved", "float64", "nEq"), ("Conserved_old", "float64", "nEq"),
    ("Conserved_t", "float64", "nEq"), ("Conserved_t_old", "float64", "nEq"),
    ("shockSensorX", "bool", 1), ("shockSensorY", "bool", 1), ("shockSensorZ", "bool", 1),
    ("DucrosSensor", "float64", 1),
    ("dudtBoundary", "float64", 3), ("dTdtBoundary", "float64", 1),
    ("velocity_old_NSCBC", "float64", 3), ("temperature_old_NSCBC", "float64", 1),
    ("MolarFracs_profile", "float64", "nSpec"), ("velocity_profile", "float64", 3),
    ("temperature_profile", "float64", 1),
]
FIELD_NAMES = [f[0] for f in FIELD_SPECS]


class htr_fluid_view(C.Structure):
    _fields_ = [(n, htr_field) for n in FIELD_NAMES]


# --- mixtures (include/htr_mix.h) -------------------------------------------

class htr_constpropmix_t(C.Structure):
    _fields_ = [
        ("R", C.c_double), ("gamma", C.c_double), ("viscosityModel", C.c_int),
        ("constantVisc", C.c_double), ("powerlawTempRef", C.c_double),
        ("powerlawViscRef", C.c_double), ("sutherlandSRef", C.c_double),
        ("sutherlandTempRef", C.c_double), ("sutherlandViscRef", C.c_double),
        ("Prandtl", C.c_double),
    ]


class htr_nasa9_t(C.Structure):
    _fields_ = [("TSwitch1", C.c_float), ("TSwitch2", C.c_float), ("TMin", C.c_float),
                ("TMax", C.c_float), ("cpH", C.c_double * 9), ("cpM", C.c_double * 9),
                ("cpL", C.c_double * 9)]


class htr_ljdata_t(C.Structure):
    _fields_ = [("Geom", C.c_uint8), ("sigma", C.c_double), ("kbOveps", C.c_double),
                ("mu", C.c_double), ("alpha", C.c_double), ("Z298", C.c_double)]


class htr_species_t(C.Structure):
    _fields_ = [("Name", C.c_char * 10), ("W", C.c_double), ("inx", C.c_uint8),
                ("cpCoeff", htr_nasa9_t), ("DiffCoeff", htr_ljdata_t)]


class htr_arrhenius_t(C.Structure):
    _fields_ = [("A", C.c_double), ("n", C.c_float), ("EovR", C.c_float)]


class htr_stoich_t(C.Structure):
    _fields_ = [("ind", C.c_uint8), ("nu", C.c_float)]


class htr_collider_t(C.Structure):
    _fields_ = [("ind", C.c_uint8), ("eff", C.c_float)]


class htr_reaction_t(C.Structure):
    _fields_ = [("ArrCoeff", htr_arrhenius_t), ("has_backward", C.c_bool),
                ("Neducts", C.c_uint8), ("Npducts", C.c_uint8),
                ("educts", htr_stoich_t * 2), ("pducts", htr_stoich_t * 2)]


class htr_tbreaction_t(C.Structure):
    _fields_ = [("ArrCoeff", htr_arrhenius_t), ("has_backward", C.c_bool),
                ("Neducts", C.c_uint8), ("Npducts", C.c_uint8), ("Nthirdb", C.c_uint8),
                ("educts", htr_stoich_t * 2), ("pducts", htr_stoich_t * 2),
                ("thirdb", htr_collider_t * 5)]


class htr_airmix_t(C.Structure):
    _fields_ = [("species", htr_species_t * 5), ("reactions", htr_reaction_t * 2),
                ("ThirdbodyReactions", htr_tbreaction_t * 3),
                ("PRef", C.c_double), ("TRef", C.c_double), ("XiRef", C.c_double * 5),
                ("MixWRef", C.c_double), ("iMixWRef", C.c_double), ("rhoRef", C.c_double),
                ("ieRef", C.c_double), ("iuRef", C.c_double), ("iCpRef", C.c_double),
                ("imuRef", C.c_double), ("ilamRef", C.c_double), ("iDiRef", C.c_double),
                ("iwiRef", C.c_double), ("iKiRef", C.c_double), ("Eps0", C.c_double),
                ("TMax", C.c_double), ("TMin", C.c_double)]


MIX_STRUCT = {HTR_EOS_CONSTPROPMIX: htr_constpropmix_t, HTR_EOS_AIRMIX: htr_airmix_t}
NSPEC = {HTR_EOS_CONSTPROPMIX: 1, HTR_EOS_AIRMIX: 5}

_P = C.POINTER
_V = _P(htr_fluid_view)
_R = htr_rect3
_M = C.c_void_p
_S = C.c_void_p
_D2 = _P(C.c_double)

# name -> argtypes (all return int)
PROTOTYPES = {
    "htr_load_mixture": [C.c_int, C.c_void_p, C.c_size_t, _P(C.c_void_p)],
    "htr_free_mixture": [_M],
    "htr_mixture_eos": [_M],
    "htr_constpropmix_init": [C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                              C.c_double, C.c_double, _P(htr_constpropmix_t)],
    "htr_airmix_init": [C.c_double, C.c_double, C.c_double, _D2, _P(htr_airmix_t)],
    "htr_UpdateDucrosSensor": [_V, _R, _R, C.c_double, _S],
    "htr_AddChemistrySources": [_V, _R, _M, _S],
    "htr_UpdateChemistry": [_V, _R, C.c_double, _M, _P(C.c_int), _S],
    "htr_UpdatePropertiesFromPrimitive": [_V, _R, _M, _S],
    "htr_UpdateConservedFromPrimitive": [_V, _R, _M, _S],
    "htr_UpdatePrimitiveFromConserved": [_V, _R, _M, _S],
    "htr_CalculateMaxSpectralRadius": [_V, _R, _M, _D2, _S],
    "htr_InitializeTemporaries": [_V, _R, _M, _S],
    "htr_InitializeTimeDerivatives": [_V, _R, C.c_int, _M, _S],
    "htr_UpdateVars": [_V, _R, C.c_int, C.c_double, C.c_int, _M, _S],
    "htr_decision_counters": [C.c_int, _P(C.c_ulonglong)],
    "htr_rk3_teno_face_counts": [_R, _M, C.c_void_p, C.c_size_t, _P(C.c_ulonglong), _S],
}
HTR_DECISION_COUNTERS = 7
# order of the counts of htr_decision_counters
DECISION_COUNTERS = ("teno_filtered", "teno_exact", "sensor_filtered", "sensor_exact", "cut_filtered",
                     "cut_exact", "limiter_blend")
for _d in "XYZ":
    for _s in ("Hybrid", "TENO", "TENOA", "TENOLAD"):
        PROTOTYPES[f"htr_UpdateUsing{_s}EulerFlux{_d}"] = [_V, _R, _R, _D2, C.c_double, _M, _S]
    PROTOTYPES[f"htr_UpdateUsingSkewSymmetricEulerFlux{_d}"] = [_V, _R, _R, _M, _S]
    PROTOTYPES[f"htr_UpdateUsingDiffusionFlux{_d}"] = [_V, _R, _R, _M, _S]
    PROTOTYPES[f"htr_UpdateShockSensor{_d}"] = [_V, _R, _R, _M, _S]


for _side in ("XNeg", "XPos", "YNeg", "YPos", "ZNeg", "ZPos"):
    PROTOTYPES[f"htr_UpdateUsingFluxNSCBCInflow{_side}"] = [_V, _R, _M, _S]
    PROTOTYPES[f"htr_UpdateUsingFluxNSCBCOutflow{_side}"] = [_V, _R, _R, _M, C.c_double, C.c_double, C.c_double, _S]
PROTOTYPES["htr_CalculateMaxMachNumber"] = [_V, _R, C.c_int, _P(C.c_double), _S]
for _d in "XYZ":
    PROTOTYPES[f"htr_SetNSCBC_InflowBC{_d}"] = [_V, _R, _M, C.c_double, _S]
PROTOTYPES["htr_SetNSCBC_OutflowBC"] = [_V, _R, _M, _P(C.c_int), _S]
PROTOTYPES["htr_SetIsothermalWallBC"] = [_V, _R, C.c_int, _M, _S]
PROTOTYPES["htr_SetAdiabaticWallBC"] = [_V, _R, C.c_int, _M, _S]
PROTOTYPES["htr_UpdateNSCBCGhostCellTimeDerivatives"] = [_V, _R, C.c_double, _S]
PROTOTYPES["htr_InitializeMetric"] = [_V, htr_field, _R, _R, _P(C.c_double), _S]
for _d in "XYZ":
    PROTOTYPES[f"htr_CorrectGhostMetric{_d}"] = [_V, htr_field, _R, _S]


# include/htr_restart.h
HTR_RESTART_HOST_VIEW = 1
HTR_RESTART_PROFILES = 2


class htr_restart_info(C.Structure):
    _fields_ = [("timeStep", C.c_int64), ("simTime", C.c_double), ("channelForcing", C.c_double)]


_CP = C.c_char_p
PROTOTYPES["htr_restart_tile_filename"] = [_CP, htr_rect3, C.c_char_p, C.c_size_t]
PROTOTYPES["htr_restart_write_tile"] = [_CP, _V, htr_rect3, C.c_int, C.c_int, _S]
PROTOTYPES["htr_restart_read_tile"] = [_CP, _V, htr_rect3, C.c_int, C.c_int, _S]
PROTOTYPES["htr_restart_write_master"] = [_CP, _P(htr_restart_info), htr_rect3, _P(C.c_int64), _P(htr_rect3),
                                          C.c_int, _P(C.c_char_p), _P(C.c_char_p)]
PROTOTYPES["htr_restart_read_master"] = [_CP, _P(htr_restart_info), _P(htr_rect3), _P(C.c_int64),
                                         _P(htr_rect3), C.c_int64]
PROTOTYPES["htr_h5_dataset_shape"] = [_CP, _CP, _P(C.c_int), _P(C.c_int64), _P(C.c_int64)]
PROTOTYPES["htr_h5_read_doubles"] = [_CP, _CP, _P(C.c_double), C.c_int64]
PROTOTYPES["htr_h5_string_attribute"] = [_CP, _CP, _CP, C.c_int64, C.c_char_p, C.c_size_t]


def bind(lib, extra=None):
    """Attach prototypes to every entry point `lib` exports."""
    protos = dict(PROTOTYPES)
    if extra:
        protos.update(extra)
    for name, args in protos.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = C.c_int
    if hasattr(lib, "htr_last_error"):
        lib.htr_last_error.argtypes = []
        lib.htr_last_error.restype = C.c_char_p
    return lib


def check(lib, status, what=""):
    if status != 0:
        msg = ""
        if hasattr(lib, "htr_last_error"):
            raw = lib.htr_last_error()
            msg = raw.decode() if raw else ""
        raise HtrError(f"{what}: {STATUS_NAMES.get(status, status)} {msg}".strip())


def rect(lo, hi):
    r = htr_rect3()
    for i in range(3):
        r.lo[i] = int(lo[i])
        r.hi[i] = int(hi[i])
    return r
