"""ctypes bindings of libpcfd.so (the C ABI in include/pcfd.h).

The library is loaded from the package directory; if it is absent the import
fails loudly - there is no CPU fallback for the device path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libpcfd.so"

PCFD_OK = 0
ERRORS = {1: "ARG", 2: "STATE", 3: "CUDA", 4: "MESH", 5: "NOMEM", 6: "UNSUPPORTED", 7: "NUMERIC"}
(PCFD_ERR_ARG, PCFD_ERR_STATE, PCFD_ERR_CUDA, PCFD_ERR_MESH, PCFD_ERR_NOMEM, PCFD_ERR_UNSUPPORTED,
 PCFD_ERR_NUMERIC) = range(1, 8)

# boundary condition types: the reference's BCTypes values (ucs/bc_defines.h:4)
BC_PARALLEL = 0
BC_DIRICHLET = 1
BC_NEUMANN = 2
BC_IMPERMEABLE_WALL = 3
BC_NOSLIP = 4
BC_FARFIELD_VISCOUS = 5
BC_FARFIELD = 6
BC_SONIC_INFLOW = 7
BC_SONIC_OUTFLOW = 8
BC_SYMMETRY = 9

# learned preconditioner network sizes (PCFD_LP_* in include/pcfd.h)
LP_NIN = 11
LP_HIDDEN = 64
LP_NEDGE = 4
LP_NOUT = 5
LP_LAYERS = 3
LP_NPARAM = 26821


class BoxParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("jitter", C.c_double), ("seed", C.c_uint64),
        ("ramp_deg", C.c_double), ("ramp_x0", C.c_double), ("y_ratio", C.c_double),
        ("tags", C.c_int * 6), ("jitter_mode", C.c_int),
        ("wall_start_i", C.c_int), ("upstream_tag", C.c_int), ("wall_ar_max", C.c_double),
    ]


class MeshView(C.Structure):
    _fields_ = [
        ("nnode", C.c_int), ("nbnode", C.c_int), ("nedge", C.c_int), ("nbedge", C.c_int),
        ("edges", C.POINTER(C.c_int)), ("edge_area", C.POINTER(C.c_double)),
        ("bedges", C.POINTER(C.c_int)), ("bedge_area", C.POINTER(C.c_double)),
        ("bfactag", C.POINTER(C.c_int)),
        ("xyz", C.POINTER(C.c_double)), ("vol", C.POINTER(C.c_double)), ("sw", C.POINTER(C.c_double)),
        ("ipsp", C.POINTER(C.c_int)), ("psp", C.POINTER(C.c_int)),
    ]


class Params(C.Structure):
    _fields_ = [
        ("gamma", C.c_double), ("mach", C.c_double), ("flowdir", C.c_double * 3),
        ("Re", C.c_double), ("Pr", C.c_double), ("PrT", C.c_double), ("ref_temperature", C.c_double),
        ("sorder", C.c_int), ("chi", C.c_double), ("viscous", C.c_int), ("limiter", C.c_int),
        ("venkat_K", C.c_double), ("no_cvbc", C.c_int), ("jac_boundary_eval", C.c_int), ("ntags", C.c_int),
        ("bc_type", C.POINTER(C.c_int)), ("bc_twall", C.POINTER(C.c_double)),
        ("torder", C.c_int), ("time_step", C.c_double), ("tinf", C.c_double), ("pinf", C.c_double),
    ]


class NewtonOpts(C.Structure):
    _fields_ = [
        ("iter", C.c_int), ("cfl", C.c_double), ("cfl_start", C.c_double), ("cfl_ramp_steps", C.c_int),
        ("nsgs", C.c_int), ("jac_update_freq", C.c_int), ("jac_precision", C.c_int), ("linear_solver", C.c_int),
        ("fgmres_m", C.c_int), ("fgmres_restarts", C.c_int), ("fgmres_rtol", C.c_double),
        ("limiter_refresh", C.c_int), ("limiter_freeze", C.c_int), ("first_order_steps", C.c_int),
        ("lp_directions", C.c_int),
    ]


class NewtonReport(C.Structure):
    _fields_ = [
        ("res", C.c_double * 6), ("dqnorm", C.c_double), ("dtmin", C.c_double), ("lin_res", C.c_double),
        ("lin_iters", C.c_int), ("cfl", C.c_double), ("lp_fallbacks", C.c_int),
    ]


CHEM_MAX_SPECIES = 16
CHEM_MAX_REACTIONS = 32
CHEM_MAX_LOCAL = 16
CHEM_MAX_TRANSPORT_FITS = 4


class ChemReaction(C.Structure):
    _fields_ = [
        ("type", C.c_int), ("A", C.c_double), ("EA", C.c_double), ("n", C.c_double), ("third_bodies", C.c_int),
        ("nlocal", C.c_int), ("global_", C.c_int * CHEM_MAX_LOCAL), ("nup", C.c_double * CHEM_MAX_LOCAL),
        ("nupp", C.c_double * CHEM_MAX_LOCAL), ("tbeff", C.c_double * CHEM_MAX_LOCAL),
    ]


class ChemModelC(C.Structure):
    _fields_ = [
        ("nspecies", C.c_int), ("mw", C.c_double * CHEM_MAX_SPECIES),
        ("nasa_lo", (C.c_double * 7) * CHEM_MAX_SPECIES), ("nasa_hi", (C.c_double * 7) * CHEM_MAX_SPECIES),
        ("nreactions", C.c_int), ("rx", ChemReaction * CHEM_MAX_REACTIONS),
        ("nmu", C.c_int * CHEM_MAX_SPECIES),
        ("mu_fit", ((C.c_double * 6) * CHEM_MAX_TRANSPORT_FITS) * CHEM_MAX_SPECIES),
        ("nk", C.c_int * CHEM_MAX_SPECIES),
        ("k_fit", ((C.c_double * 6) * CHEM_MAX_TRANSPORT_FITS) * CHEM_MAX_SPECIES),
    ]


_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_LLP = C.POINTER(C.c_longlong)
class ChemRef(C.Structure):
    """pcfd_chem_ref: the reacting equation set's reference scales."""
    _fields_ = [("density", C.c_double), ("pressure", C.c_double), ("temperature", C.c_double),
                ("specific_enthalpy", C.c_double), ("velocity", C.c_double), ("viscosity", C.c_double),
                ("conductivity", C.c_double)]


class ChemFluxOpts(C.Structure):
    """pcfd_chem_flux_opts: beta, the gauge reference pressure, symmetry2D."""
    _fields_ = [("beta", C.c_double), ("pref", C.c_double), ("symmetry2D", C.c_int)]


_FP = C.POINTER(C.c_float)

# name -> (restype, argtypes); every symbol include/pcfd.h declares
PROTOTYPES = {
    "pcfd_mesh_box_create": (_P, [C.POINTER(BoxParams)]),
    "pcfd_mesh_from_elements": (_P, [C.c_int, _DP, C.c_int, _IP, _IP, C.c_int, _IP]),
    "pcfd_mesh_build": (C.c_int, [_P]),
    "pcfd_mesh_view_get": (C.c_int, [_P, C.POINTER(MeshView)]),
    "pcfd_mesh_stats": (C.c_int, [_P, _IP, _IP, _IP, _IP, _DP, _DP]),
    "pcfd_mesh_rcm_order": (C.c_int, [_P, _IP]),
    "pcfd_mesh_reorder_rcm": (C.c_int, [_P, _IP]),
    "pcfd_mesh_renumber": (C.c_int, [_P, _IP]),
    "pcfd_mesh_destroy": (None, [_P]),
    "pcfd_mesh_last_error": (C.c_char_p, []),
    "pcfd_create": (C.c_int, [C.POINTER(MeshView), C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "pcfd_destroy": (C.c_int, [_P]),
    "pcfd_set_state": (C.c_int, [_P, _DP, C.c_int, C.c_int]),
    "pcfd_set_qold": (C.c_int, [_P, _DP, C.c_int, C.c_int]),
    "pcfd_forces": (C.c_int, [_P, _IP, C.c_int, _DP]),
    "pcfd_get_state": (C.c_int, [_P, _DP, C.c_int, C.c_int]),
    "pcfd_get_qinf": (C.c_int, [_P, _DP]),
    "pcfd_update_bcs": (C.c_int, [_P]),
    "pcfd_gradient": (C.c_int, [_P, _DP]),
    "pcfd_limiter": (C.c_int, [_P, _DP]),
    "pcfd_residual": (C.c_int, [_P, _DP, _DP]),
    "pcfd_residual_full": (C.c_int, [_P, _DP]),
    "pcfd_get_residual": (C.c_int, [_P, _DP]),
    "pcfd_bench_residual_full": (C.c_int, [_P, C.c_int, _DP, _DP]),
    "pcfd_bench_spmv": (C.c_int, [_P, C.c_int, C.c_int, _DP]),
    "pcfd_bench_sgs": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _DP]),
    "pcfd_timestep": (C.c_int, [_P, C.c_double, _DP, _DP]),
    "pcfd_set_jacobian_precision": (C.c_int, [_P, C.c_int]),
    "pcfd_jacobian": (C.c_int, [_P]),
    "pcfd_get_jacobian": (C.c_int, [_P, _DP, C.c_longlong]),
    "pcfd_nblocks": (C.c_longlong, [_P]),
    "pcfd_crs_structure": (C.c_int, [_P, _IP, _IP, _IP]),
    "pcfd_sgs": (C.c_int, [_P, C.c_int, _DP, _DP]),
    "pcfd_fgmres": (C.c_int, [_P, C.c_int, C.c_int, C.c_double, C.c_int, _DP, _DP, C.POINTER(C.c_int)]),
    "pcfd_matvec": (C.c_int, [_P, _DP, _DP, C.c_int]),
    "pcfd_sgs_rhs": (C.c_int, [_P, C.c_int, _DP, _DP, C.c_int]),
    "pcfd_coloring": (C.c_int, [_P, _IP, _IP]),
    "pcfd_apply_dq": (C.c_int, [_P, _DP, _DP]),
    "pcfd_newton_step": (C.c_int, [_P, C.POINTER(NewtonOpts), C.POINTER(NewtonReport)]),
    "pcfd_set_device": (C.c_int, [C.c_int]),
    "pcfd_set_residual_arithmetic": (C.c_int, [_P, C.c_int]),
    "pcfd_get_limiter": (C.c_int, [_P, _DP]),
    "pcfd_chem_create": (C.c_int, [C.POINTER(ChemModelC), C.POINTER(_P)]),
    # array arguments as void*: host arrays (dev = 0) or device addresses (dev = 1)
    "pcfd_chem_find_T_given_P": (C.c_int, [_P, C.POINTER(ChemRef), C.c_longlong, _P, _P, _P, _P,
                                           C.POINTER(C.c_longlong), C.c_int]),
    "pcfd_chem_conservative_to_native": (C.c_int, [_P, C.POINTER(ChemRef), C.c_longlong, _P, _P, _P, C.c_int]),
    "pcfd_chem_native_to_conservative": (C.c_int, [_P, C.POINTER(ChemRef), C.c_longlong, _P, _P, _P, _P, C.c_int]),
    "pcfd_chem_aux": (C.c_int, [_P, C.POINTER(ChemRef), C.c_longlong, _P, _P, _P, _P, _P, C.c_int]),
    "pcfd_chem_temporal_terms": (C.c_int, [_P, C.POINTER(ChemRef), C.c_longlong, _P, _P, _P, _P, C.c_double,
                                           C.c_double, C.c_int, _P, C.c_int]),
    "pcfd_chem_transport": (C.c_int, [_P, C.POINTER(ChemRef), C.c_longlong, _DP, _DP, _DP, _DP, C.c_int]),
    "pcfd_chem_residual_ho": (C.c_int, [_P, C.POINTER(ChemRef), C.POINTER(ChemFluxOpts), C.c_double, C.c_double,
                                        C.c_int, _P, _P, _P, _P, _DP, C.c_int]),
    "pcfd_chem_limiter": (C.c_int, [_P, C.c_double, _P, _P, _P, C.c_int]),
    "pcfd_chem_update_bcs": (C.c_int, [_P, C.POINTER(ChemRef), C.c_int, _IP, _DP, _DP, C.c_int, _P, C.c_int]),
    "pcfd_chem_gradient": (C.c_int, [_P, _P, _IP, C.c_int, _P, C.c_int]),
    "pcfd_chem_viscous_residual": (C.c_int, [_P, C.POINTER(ChemRef), C.POINTER(ChemFluxOpts), C.c_double, C.c_int,
                                             _P, _P, _P, C.c_int]),
    "pcfd_chem_source_jacobian": (C.c_int, [_P, C.POINTER(ChemRef), C.c_double, C.c_longlong, _P, _P, _P,
                                            C.c_int]),
    "pcfd_chem_hllc_flux": (C.c_int, [_P, C.POINTER(ChemRef), C.POINTER(ChemFluxOpts), C.c_longlong, _P,
                                      C.c_longlong, _P, _P, _P, C.POINTER(C.c_longlong), C.c_int]),
    "pcfd_chem_attach_mesh": (C.c_int, [_P, C.POINTER(MeshView)]),
    "pcfd_chem_residual": (C.c_int, [_P, C.POINTER(ChemRef), C.POINTER(ChemFluxOpts), C.c_double, C.c_int, _P, _P,
                                     _P, C.c_int]),
    "pcfd_chem_destroy": (C.c_int, [_P]),
    "pcfd_chem_production_rates": (C.c_int, [_P, C.c_longlong, _DP, _DP, _DP]),
    "pcfd_chem_production_rates_dev": (C.c_int, [_P, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, _DP]),
    "pcfd_set_limiter": (C.c_int, [_P, _DP]),
    "pcfd_lp_init": (C.c_int, [_P, C.c_ulonglong]),
    "pcfd_lp_get_params": (C.c_int, [_P, _FP]),
    "pcfd_lp_set_params": (C.c_int, [_P, _FP]),
    "pcfd_lp_forward": (C.c_int, [_P, _FP, _FP]),
    "pcfd_lp_loss_grad": (C.c_int, [_P, _FP, _FP, _FP, _DP]),
    "pcfd_lp_features": (C.c_int, [_P, _DP, _FP, _DP]),
    "pcfd_lp_collect": (C.c_int, [_P, C.c_int, C.c_double, C.c_int, _IP]),
    "pcfd_lp_clear_samples": (C.c_int, [_P]),
    "pcfd_lp_train": (C.c_int, [_P, C.c_int, C.c_double, _DP, _DP]),
    "pcfd_lp_apply": (C.c_int, [_P, C.c_int, _DP, _DP]),
    "pcfd_device_sync": (C.c_int, []),
    "pcfd_profile_enable": (C.c_int, [_P, C.c_int]),
    "pcfd_profile_reset": (C.c_int, [_P]),
    "pcfd_profile_get": (C.c_int, [_P, C.c_int, C.c_char_p, C.c_int, _DP, _LLP]),
    "pcfd_launch_count": (C.c_longlong, [_P]),
    "pcfd_get_health": (C.c_int, [_P, _LLP]),
    "pcfd_residual_norms_noalloc": (C.c_int, [C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]),
    "pcfd_last_error": (C.c_char_p, []),
    "pcfd_build_info": (C.c_char_p, []),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libpcfd.so and attach prototypes; raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            "libpcfd.so not found at %s; build it with `python -m proteuscfd_gb300.build` "
            "(there is no CPU fallback)" % p)
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class PcfdError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__("%s failed: PCFD_ERR_%s (%d): %s" % (where, ERRORS.get(code, "?"), code, msg))
        self.code = code


def check(rc: int, where: str) -> None:
    if rc != PCFD_OK:
        msg = load().pcfd_last_error()
        raise PcfdError(rc, where, msg.decode() if msg else "")


def fptr(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_FP)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_DP)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_IP)
