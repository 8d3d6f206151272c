"""ctypes mirror of include/mtg.h (the engine's C ABI).

Only structure layouts and status codes live here; the loader is in
``mt_gb300.engine``.
"""
import ctypes as C

MTG_OK = 0
MTG_E_CUDA = -1
MTG_E_CONFIG = -2
MTG_E_OVERFLOW = -3
MTG_E_NONFINITE = -4
MTG_E_TEA_EPS = -5
MTG_E_TIMEOUT = -6
MTG_E_STATE = -7

STATUS_NAMES = {
    MTG_OK: "MTG_OK",
    MTG_E_CUDA: "MTG_E_CUDA",
    MTG_E_CONFIG: "MTG_E_CONFIG",
    MTG_E_OVERFLOW: "MTG_E_OVERFLOW",
    MTG_E_NONFINITE: "MTG_E_NONFINITE",
    MTG_E_TEA_EPS: "MTG_E_TEA_EPS",
    MTG_E_TIMEOUT: "MTG_E_TIMEOUT",
    MTG_E_STATE: "MTG_E_STATE",
}

COORD_FLOATS = 7
ENERGY_TERMS = 7
ENERGY_NAMES = ("U_harm", "U_long", "U_lat", "U_psi", "U_fi", "U_teta", "U_lj")

_f = C.c_float
_i = C.c_int
_pi = C.POINTER(C.c_int)
_pu8 = C.POINTER(C.c_uint8)
_pf = C.POINTER(C.c_float)


class MtgParams(C.Structure):
    """mtg_params: scalar parameters of the hot path (Parameters, src/parameters.h:246-318)."""

    _fields_ = [
        ("dt", _f), ("Temp", _f), ("viscosity", _f),
        ("gammaR", _f), ("gammaTheta", _f), ("varR", _f), ("varTheta", _f),
        ("alpha", _f), ("freeze_temp", _f),
        ("C", _f), ("B_psi", _f), ("B_fi", _f), ("B_theta", _f), ("psi_0", _f), ("fi_0", _f),
        ("theta0_gtp", _f), ("theta0_gdp", _f),
        ("A_lat", _f), ("A_long", _f), ("D_lat", _f), ("D_long", _f), ("seam_coeff", _f),
        ("barrier", _i),
        ("a_barr_long", _f), ("r_barr_long", _f), ("w_barr_long", _f),
        ("a_barr_lat", _f), ("r_barr_lat", _f), ("w_barr_lat", _f),
        ("lj_on", _i), ("ljscale", _f), ("ljsigma6", _f), ("ljpairscutoff", _f),
        ("ljpairsupdatefreq", _i),
        ("is_wall", _i), ("rep_r", _f), ("rep_eps", _f), ("rep_leftborder", _f),
        ("is_assembly", _i),
        ("hdi_on", _i), ("tea_a", _f), ("tea_epsilon_freq", _i), ("tea_capricious", _i),
        ("tea_epsmax", _f),
        ("rseed", _i),
        ("device", _i),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class MtgTopology(C.Structure):
    """mtg_topology: uniform batch in the reference's Topology layout (src/mt.h:73-92)."""

    _fields_ = [
        ("Ntot", _i), ("Ntr", _i),
        ("maxHarmonicPerMonomer", _i), ("harmonicCount", _pi), ("harmonic", _pi),
        ("maxLongitudinalPerMonomer", _i), ("longitudinalCount", _pi), ("longitudinal", _pi),
        ("maxLateralPerMonomer", _i), ("lateralCount", _pi), ("lateral", _pi),
        ("maxLJPerMonomer", _i),
        ("fixed", _pu8), ("mon_type", _pi),
        ("extra", _pu8), ("gtp", _pi), ("on_tubule_cur", _pi),
        ("zs", _pf),
    ]


class MtgBatchTopology(C.Structure):
    """mtg_batch_topology: ragged batch (CSR offsets per trajectory)."""

    _fields_ = [
        ("ntraj", _i), ("offsets", _pi),
        ("maxHarmonicPerMonomer", _i), ("harmonicCount", _pi), ("harmonic", _pi),
        ("maxLongitudinalPerMonomer", _i), ("maxLateralPerMonomer", _i), ("maxLJPerMonomer", _i),
        ("longitudinalCount", _pi), ("longitudinal", _pi),
        ("lateralCount", _pi), ("lateral", _pi),
        ("fixed", _pu8), ("extra", _pu8),
        ("mon_type", _pi), ("gtp", _pi), ("on_tubule_cur", _pi),
        ("zs", _pf),
    ]


def ptr(a, ctype):
    """Pointer to a contiguous numpy array (or NULL for None)."""
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


class MtgTuning(C.Structure):
    """mtg_tuning: launch shapes chosen by the autotuner."""

    _fields_ = [("list_method", _i), ("step_block", _i), ("tea_slices", _i), ("tea_jparts", _i),
                ("plain_persistent", _i)]
