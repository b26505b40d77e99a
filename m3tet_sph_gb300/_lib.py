"""ctypes binding of the C ABI in include/m3sph.h (libm3sph.so, built in-tree).

There is no CPU fallback: if the library cannot be loaded, or no CUDA device is visible when a
mesh is created, the calls raise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB = None
LIB_PATH = Path(__file__).resolve().parent / "libm3sph.so"

OK, ERR_BAD_INPUT, ERR_CUDA, ERR_NAN, ERR_NOT_CONVERGED, ERR_NEG_JAC, ERR_NOT_FOUND, ERR_NO_DEVICE = range(8)


class M3SphError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"m3sph error {code}: {msg}")
        self.code = code


class Level(C.Structure):
    _fields_ = [("nel", C.c_int32), ("nnod", C.c_int32), ("nvnod", C.c_int32),
                ("EL2NOD", C.POINTER(C.c_uint32)), ("isplit", C.POINTER(C.c_uint8)),
                ("GCOORD", C.POINTER(C.c_double)), ("GCOORD_SPH", C.POINTER(C.c_double)),
                ("elclass", C.POINTER(C.c_uint8)), ("niso", C.c_int32),
                ("els_iso", C.POINTER(C.c_uint32)), ("cubic_sph_rot", C.POINTER(C.c_double))]


class SlmOpts(C.Structure):
    _fields_ = [("method_BT", C.c_int32), ("method_interp", C.c_int32), ("monotonic", C.c_int32),
                ("method_wght", C.c_int32), ("r_cmb", C.c_double), ("r_surf", C.c_double)]


class LocateInfo(C.Structure):
    _fields_ = [("npt", C.c_int32), ("nwalk", C.c_int32), ("nties", C.c_int32), ("ngap", C.c_int32),
                ("nbrute", C.c_int32), ("nlost", C.c_int32), ("nambig", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Physics(C.Structure):
    _fields_ = [("g", C.c_double), ("Bscale", C.c_double), ("Dens0", C.c_double),
                ("minVisc", C.c_double), ("maxVisc", C.c_double)]


class Opts(C.Structure):
    _fields_ = [("rtol_Pat", C.c_double), ("rtol_U", C.c_double), ("itmax_Pat", C.c_int32),
                ("itmin_Pat", C.c_int32), ("itmax_U", C.c_int32), ("precision", C.c_int32),
                ("smoother", C.c_int32), ("target_rel_residual", C.c_double)]


class Info(C.Structure):
    _fields_ = [("itPat", C.c_int32), ("nitU", C.c_int32), ("nitZ", C.c_int32), ("nvcycle", C.c_int32),
                ("norm_rP", C.c_double), ("rel_residual", C.c_double), ("t_setup_ms", C.c_double),
                ("t_iter_ms", C.c_double), ("smoother_fallbacks", C.c_int32), ("status", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RockParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("Visc0", "Dens0", "T_ref", "alpha", "Ea", "Va", "g", "L0", "a_UM2LM",
                                          "minDens", "maxDens", "minVisc", "maxVisc")]


class DiffusionOpts(C.Structure):
    _fields_ = [("kappa", C.c_double), ("theta", C.c_double), ("tol", C.c_double), ("itmax", C.c_int32),
                ("theta_cone", C.c_double)]


class StepOpts(C.Structure):
    _fields_ = [("stokes", Opts), ("slm", SlmOpts), ("rock_prop", C.c_int32), ("rock", RockParams),
                ("dt_adv_limit", C.c_double), ("dtmax", C.c_double), ("diffusion", C.c_int32)]


class StepInfo(C.Structure):
    _fields_ = [("stokes", Info), ("locate", LocateInfo), ("dt", C.c_double), ("dt_adv", C.c_double),
                ("time", C.c_double), ("t_rock_ms", C.c_double), ("t_stokes_ms", C.c_double),
                ("t_dt_ms", C.c_double), ("t_advect_ms", C.c_double), ("t_total_ms", C.c_double),
                ("status", C.c_int32), ("t_diffusion_ms", C.c_double), ("diffusion_its", C.c_int32)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["stokes"] = self.stokes.as_dict()
        d["locate"] = self.locate.as_dict()
        return d


# exported symbols and their argtypes (None = opaque handle pointer)
P = C.c_void_p
DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int32)
SIGNATURES = {
    "m3sph_last_error": ([], C.c_char_p),
    "m3sph_device_count": ([IP], C.c_int),
    "m3sph_mesh_create": ([C.c_int32, C.POINTER(Level), C.c_int32, C.POINTER(P)], C.c_int),
    "m3sph_mesh_destroy": ([P], C.c_int),
    "m3sph_mesh_ncolors": ([P, C.c_int32, IP], C.c_int),
    "m3sph_stokes_setup": ([P, DP, DP, IP, DP, C.c_int32, C.POINTER(Physics), C.c_int32], C.c_int),
    "m3sph_stokes_solve": ([P, DP, DP, C.POINTER(Opts), C.POINTER(Info)], C.c_int),
    "m3sph_stokes_set_vel_bc": ([P, IP, DP, C.c_int32], C.c_int),
    "m3sph_mgpcg": ([P, DP, DP, C.c_double, C.c_int32, C.c_int32, IP, DP], C.c_int),
    "m3sph_stokes_apply": ([P, DP, DP], C.c_int),
    "m3sph_grad_apply": ([P, DP, DP], C.c_int),
    "m3sph_div_apply": ([P, DP, DP], C.c_int),
    "m3sph_force_vector": ([P, DP], C.c_int),
    "m3sph_element_matrices": ([P, DP, DP, DP], C.c_int),
    "m3sph_level_apply32": ([P, C.c_int32, P, P], C.c_int),
    "m3sph_level_apply": ([P, C.c_int32, DP, DP], C.c_int),
    "m3sph_transfer_matrix": ([P, C.c_int32, C.POINTER(C.c_int64), IP, IP, DP], C.c_int),
    "m3sph_prolong": ([P, C.c_int32, DP, DP], C.c_int),
    "m3sph_restrict": ([P, C.c_int32, DP, DP], C.c_int),
    "m3sph_vcycle": ([P, DP, DP], C.c_int),
    "m3sph_stokes_step_device": ([P, C.POINTER(Opts), C.POINTER(Info)], C.c_int),
    "m3sph_solution": ([P, DP, DP], C.c_int),
    "m3sph_calculate_dt": ([P, C.c_double, C.c_double, DP, DP], C.c_int),
    "m3sph_rock_prop": ([P, C.POINTER(RockParams), DP, DP, DP], C.c_int),
    "m3sph_diffusion_setup": ([P, C.POINTER(DiffusionOpts), IP, DP, C.c_int32], C.c_int),
    "m3sph_diffusion3d": ([P, DP, C.c_double, IP], C.c_int),
    "m3sph_set_temperature": ([P, DP, C.c_double], C.c_int),
    "m3sph_get_temperature": ([P, DP], C.c_int),
    "m3sph_time_step": ([P, C.POINTER(StepOpts), C.POINTER(StepInfo)], C.c_int),
    "m3sph_get_properties": ([P, DP, DP], C.c_int),
    "m3sph_set_pressure": ([P, DP], C.c_int),
    "m3sph_stream": ([P, C.POINTER(P)], C.c_int),
    "m3sph_tsearch_sph": ([P, DP, C.c_int32, IP, IP, DP, C.POINTER(LocateInfo)], C.c_int),
    "m3sph_locate_timing": ([P, DP, C.c_int32, C.c_int32, DP, C.POINTER(LocateInfo)], C.c_int),
    "m3sph_interp3d_tet": ([P, IP, DP, C.c_int32, DP, C.c_int32, C.c_int32, DP], C.c_int),
    "m3sph_interp3d_cubic": ([P, IP, DP, C.c_int32, DP, C.c_int32, C.c_int32, DP], C.c_int),
    "m3sph_interp3d_cubic_noalloc": ([P, P, P, C.c_int32, P, C.c_int32, C.c_int32, P], C.c_int),
    "m3sph_advect_slm": ([P, DP, DP, DP, DP, C.c_double, C.POINTER(SlmOpts), IP, IP, C.POINTER(LocateInfo)], C.c_int),
    "m3sph_ml_nparam": ([IP], C.c_int),
    "m3sph_ml_set_params": ([P, C.POINTER(C.c_float), C.c_int32], C.c_int),
    "m3sph_ml_get_params": ([P, C.POINTER(C.c_float)], C.c_int),
    "m3sph_ml_reserve": ([P, C.c_int64], C.c_int),
    "m3sph_ml_collect": ([P, C.c_uint64, C.c_int32, C.c_int32, C.POINTER(C.c_int64)], C.c_int),
    "m3sph_ml_train_epoch": ([P, C.c_int32, C.c_float, C.c_uint64, DP], C.c_int),
    "m3sph_ml_add_pairs": ([P, DP, DP, C.c_int32, C.c_int32, C.POINTER(C.c_int64)], C.c_int),
    "m3sph_ml_gradients": ([P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float), DP], C.c_int),
    "m3sph_ml_forward": ([P, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float)], C.c_int),
    "m3sph_ml_sweep32": ([P, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
    "m3sph_level_inverse_diag32": ([P, C.c_int32, C.POINTER(C.c_float)], C.c_int),
    "m3sph_ml_features": ([P, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
    "m3sph_set_option": ([P, C.c_char_p, C.c_int32], C.c_int),
    "m3sph_launch_count": ([C.POINTER(C.c_ulonglong)], C.c_int),
    "m3sph_apply_timing": ([P, C.c_int32, C.c_int32, C.c_int32, DP], C.c_int),
}


def lib():
    """Load libm3sph.so (raises if it is missing: there is no CPU implementation)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise M3SphError(ERR_NO_DEVICE, f"{LIB_PATH} not built; run __graft_entry__.build()")
    L = C.CDLL(str(LIB_PATH))
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _LIB = L
    return L


def check(code):
    if code != OK:
        raise M3SphError(code, lib().m3sph_last_error().decode())


def dptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(DP)


def iptr(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(IP)


def u32ptr(a):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def u8ptr(a):
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def device_count():
    n = C.c_int32(0)
    code = lib().m3sph_device_count(C.byref(n))
    return n.value if code == OK else 0


def launch_count():
    n = C.c_ulonglong(0)
    check(lib().m3sph_launch_count(C.byref(n)))
    return n.value


def fptr(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))
