"""ctypes binding of the C ABI declared in include/hc.h (libhcgb300.so).

The library is the only compute path: if it is missing, loading raises; there
is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libhcgb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "hc.h")

HC_OK, HC_ERR_ARG, HC_ERR_CUDA, HC_ERR_NONPHYSICAL, HC_ERR_TIMEOUT, HC_ERR_UNSUPPORTED = range(6)
STATUS_NAMES = {0: "HC_OK", 1: "HC_ERR_ARG", 2: "HC_ERR_CUDA", 3: "HC_ERR_NONPHYSICAL",
                4: "HC_ERR_TIMEOUT", 5: "HC_ERR_UNSUPPORTED"}

FLUX = {"roe": 0, "slau": 1, "slau_ref": 2, "ausmpup": 3, "rusanov": 4, "central": 5, "roe_ws": 6,
        "roe_face": 7}
SCALING = {"convective": 0, "acoustic": 1, "adaptive": 2}
BASIS = {"primitive": 0, "conserved": 1}
LIMITER = {"nolimit1": 0, "nolimit2": 1, "nolimit3": 2, "vanalbada": 3, "minmod": 4,
           "superbee": 5, "mc": 6, "vanleer": 7, "vanleer_ref": 8, "cada3": 9}
RK = {"ssp11": 0, "ssp22": 1, "ssp33": 2, "ssp34": 3}
PRECISION = {"fp64": 0, "fp32": 1, "fp64_df": 2}
DTMODE = {"global": 0, "local": 1}
BC = {"periodic": 0, "fixed": 1, "riemann": 2, "entropy": 3, "wall": 4}
LAW = {"euler": 0, "scalar": 1}


class HCError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("flux", C.c_int), ("limiter", C.c_int), ("rk", C.c_int), ("precision", C.c_int),
                ("dt_mode", C.c_int), ("cfl", C.c_double), ("law", C.c_int), ("basis", C.c_int)]


class StepStats(C.Structure):
    _fields_ = [("dt", C.c_double), ("t", C.c_double), ("resnorm", C.c_double), ("status", C.c_int),
                ("bad_cell", C.c_int), ("kernel_launches", C.c_longlong)]


# hc_fix: corrections of the reference's defects (off by default)
FIX = {"mach_split_p1": 1, "farfield_transverse": 2}


def fix_mask(corrections) -> int:
    """A correction mask from None, an int, "all", or names of FIX."""
    if corrections is None:
        return 0
    if isinstance(corrections, int):
        return corrections
    if isinstance(corrections, str):
        return sum(FIX.values()) if corrections == "all" else FIX[corrections]
    return sum(FIX[c] for c in set(corrections))


_lib = None


def _declare(lib):
    p, i, d, v = C.c_void_p, C.c_int, C.c_double, C.c_void_p
    dp = C.POINTER(C.c_double)
    sig = {
        "hc_context_create": [C.POINTER(Config), C.POINTER(p)],
        "hc_context_destroy": [p],
        "hc_set_stream": [p, v],
        "hc_get_stream": [p, C.POINTER(C.c_void_p)],
        "hc_mesh_upload": [p, i, i, dp],
        "hc_mesh_upload_1d": [p, i, dp],
        "hc_set_species": [p, d, d, d],
        "hc_set_low_mach": [p, i, i, d, d],
        "hc_set_tile": [p, i],
        "hc_set_corrections": [p, C.c_uint],
        "hc_set_adjoint_tapes": [p, C.c_int],
        "hc_inject_stalled_copy": [p, C.c_int],
        "hc_set_staged_loads": [p, C.c_int],
        "hc_set_time": [p, d],
        "hc_wall_force": [p, dp, dp],
        "hc_set_bcs": [p, C.POINTER(C.c_int), C.POINTER(dp)],
        "hc_state_upload": [p, dp],
        "hc_state_download": [p, dp],
        "hc_state_upload_device": [p, v],
        "hc_state_download_device": [p, v],
        "hc_residual": [p, dp],
        "hc_face_signatures": [p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), p, p],
        "hc_step": [p, i, C.POINTER(StepStats)],
        "hc_step_async": [p, i],
        "hc_step_host": [p, i, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(StepStats)],
        "hc_sync": [p, C.POINTER(StepStats)],
        "hc_steady_run": [p, C.POINTER(SteadyControls), dp, C.c_longlong, C.POINTER(SteadyStats)],
        "hc_smooth_1d": [p, i, v, v, C.c_longlong, i, d, i],
        "hc_spectral_radius": [v, v, C.c_longlong, v, v],
        "hc_spectral_radius_noalloc": [v, v, C.c_longlong, v, v],
        "hc_mesh_cylinder_nodes": [i, i, d, d, d, dp],
        "hc_mesh_linspace_nodes": [i, i, d, d, d, d, dp],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int
    lib.hc_last_error_string.restype = C.c_char_p
    lib.hc_last_error_string.argtypes = []
    lib.hc_version.restype = C.c_char_p
    lib.hc_version.argtypes = []


def load(build_if_missing: bool = True):
    """Load libhcgb300.so (building it with nvcc when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError(f"{LIB_PATH} not built")
        from . import build as _build
        _build.build()
    lib = C.CDLL(LIB_PATH)
    _declare(lib)
    _declare_batch(lib)
    _declare_adjoint(lib)
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != HC_OK:
        raise HCError(code, load().hc_last_error_string().decode())


def header_symbols() -> list[str]:
    """Function names declared in include/hc.h."""
    import re
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(hc_[a-z0-9_]+)\s*\(", txt)))


class Schedule(C.Structure):
    _fields_ = [("tile", C.c_int), ("ctas_per_sm", C.c_int), ("order", C.c_int), ("ms_per_step", C.c_float)]


TILE = {"8x32": 0, "4x32": 1, "16x16": 2, "16x16/128": 3}
ORDER = {"natural": 0, "largest_first": 1}
BATCH_MODE = {"persistent": 0, "per_instance": 1}


def _declare_batch(lib):
    p, i, d = C.c_void_p, C.c_int, C.c_double
    dp = C.POINTER(C.c_double)
    sig = {
        "hc_batch_create": [C.POINTER(Config), i, C.POINTER(i), C.POINTER(i), C.POINTER(dp), C.POINTER(i),
                            C.POINTER(dp), d, d, d, C.POINTER(p)],
        "hc_batch_destroy": [p],
        "hc_batch_set_stream": [p, p],
        "hc_batch_state_upload": [p, i, dp],
        "hc_batch_state_upload_device": [p, i, C.c_void_p],
        "hc_batch_state_download": [p, i, dp],
        "hc_batch_set_schedule": [p, C.POINTER(Schedule)],
        "hc_batch_set_corrections": [p, C.c_uint],
        "hc_batch_set_adjoint_tapes": [p, C.c_int],
        "hc_batch_get_schedule": [p, C.POINTER(Schedule)],
        "hc_batch_step_async": [p, i, i],
        "hc_batch_graph_capture": [p, i],
        "hc_batch_graph_launch": [p],
        "hc_batch_sync": [p, C.POINTER(StepStats)],
        "hc_batch_autotune": [p, i, C.POINTER(Schedule)],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int
    lib.hc_batch_kernel_launches.argtypes = [p]
    lib.hc_batch_kernel_launches.restype = C.c_longlong


class Objective(C.Structure):
    _fields_ = [("kind", C.c_int), ("scale", C.c_double), ("dir", C.c_double * 2),
                ("target", C.POINTER(C.c_double)), ("weight", C.c_double * 4), ("target_on_device", C.c_int)]


class DualTimeControls(C.Structure):
    _fields_ = [("outer_steps", C.c_int), ("dt", C.c_double), ("cfl_outer", C.c_double), ("scheme", C.c_int),
                ("inner_max", C.c_int), ("inner_drop", C.c_double), ("check_every", C.c_int)]


class DualTimeStats(C.Structure):
    _fields_ = [("outer_steps", C.c_longlong), ("inner_steps", C.c_longlong), ("last_inner", C.c_int),
                ("dt", C.c_double), ("t", C.c_double), ("res0_last", C.c_double), ("res_last", C.c_double)]


MULTISTEP = {"bdf1": 0, "bdf2": 1, "trapezium": 2}


class SteadyControls(C.Structure):
    _fields_ = [("max_steps", C.c_longlong), ("residual_drop", C.c_double), ("check_every", C.c_int),
                ("use_residual_smoothing", C.c_int), ("smoothing_factor", C.c_double)]


class SteadyStats(C.Structure):
    _fields_ = [("res0", C.c_double), ("res", C.c_double), ("steps", C.c_longlong),
                ("history_len", C.c_longlong), ("converged", C.c_int)]


class AdjointStats(C.Structure):
    _fields_ = [("J", C.c_double), ("forward_steps", C.c_longlong), ("adjoint_steps", C.c_longlong),
                ("kernel_launches", C.c_longlong), ("ms_forward", C.c_double), ("ms_total", C.c_double),
                ("ms_recompute", C.c_double), ("replays", C.c_longlong), ("stage_tapes", C.c_longlong),
                ("ms_reverse", C.c_double)]


OBJECTIVE = {"drag": 0, "l2": 1}


def _declare_adjoint(lib):
    p, i = C.c_void_p, C.c_int
    dp = C.POINTER(C.c_double)
    lib.hc_objective_forward.argtypes = [p, i, C.POINTER(Objective), dp, dp, dp]
    lib.hc_objective_forward.restype = C.c_int
    lib.hc_adjoint_gradient.argtypes = [p, i, i, C.POINTER(Objective), dp, dp, dp, dp, C.POINTER(AdjointStats)]
    lib.hc_adjoint_gradient.restype = C.c_int
    lib.hc_batch_adjoint_gradient.argtypes = [p, i, i, C.POINTER(Objective), C.POINTER(dp), dp, C.POINTER(dp),
                                              C.POINTER(AdjointStats)]
    lib.hc_batch_adjoint_gradient.restype = C.c_int
    lib.hc_batch_adjoint_record.argtypes = [p, i, i, C.POINTER(Objective), C.POINTER(dp), dp]
    lib.hc_batch_adjoint_reverse.argtypes = [p, C.POINTER(dp), i, C.POINTER(AdjointStats)]
    lib.hc_adjoint_record.argtypes = [p, i, i, C.POINTER(Objective), dp, dp, dp]
    lib.hc_adjoint_reverse.argtypes = [p, dp, dp, i, C.POINTER(AdjointStats)]
    lib.hc_dual_time_run.argtypes = [p, C.POINTER(DualTimeControls), C.POINTER(DualTimeStats)]
    lib.hc_dual_time_run.restype = C.c_int
