"""ctypes binding of libcmaqchem.so (include/cmaqchem.h).

The library is built in-tree by ``python -m cmaq_gb300.build``; loading fails loudly
when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from functools import lru_cache
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libcmaqchem.so"

SOLVER_ROS3, SOLVER_EBI, SOLVER_GEAR = 0, 1, 2
SCHED_STATIC, SCHED_QUEUE = 0, 1
CELL_DT_UNDERFLOW, CELL_MAXITER, CELL_NONFINITE = 1, 2, 4


class ChemError(RuntimeError):
    pass


class Cfg(C.Structure):
    _fields_ = [("mechanism", C.c_char_p), ("solver", C.c_int), ("schedule", C.c_int), ("rtol", C.c_double),
                ("atol", C.c_double), ("ncols", C.c_int), ("nrows", C.c_int), ("nlays", C.c_int),
                ("nspcsd", C.c_int), ("cgrid_index", C.POINTER(C.c_int)), ("device", C.c_int),
                ("max_iter", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("accepted_steps", C.c_longlong), ("rejected_steps", C.c_longlong),
                ("failed_cells", C.c_longlong), ("sunlit_cells", C.c_longlong), ("sunlit_attempts", C.c_longlong),
                ("device_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class MechInfo(C.Structure):
    _fields_ = [("nspec", C.c_int), ("nrxns", C.c_int), ("ischan", C.c_int), ("nphotab", C.c_int),
                ("nhetero", C.c_int), ("iarray_day", C.c_int), ("iarray_night", C.c_int),
                ("flops_step_day", C.c_double), ("flops_step_night", C.c_double)]


@lru_cache(maxsize=None)
def lib(variant: str = "default") -> C.CDLL:
    """The library build of one register-cap variant (see cmaq_gb300/build.py)."""
    path = LIB_PATH if variant == "default" else LIB_PATH.parent / variant / "libcmaqchem.so"
    if not path.exists():
        raise ChemError(f"{path} is not built; run `python -m cmaq_gb300.build {variant}` (needs nvcc)")
    L = C.CDLL(str(path))
    vp, fp, dp, ip, u8p = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
    L.cmaqchem_init.argtypes = [C.POINTER(Cfg), C.POINTER(vp)]
    L.cmaqchem_step.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, ip, C.POINTER(Stats)]
    L.cmaqchem_step_device.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, ip, vp,
                                       C.POINTER(Stats)]
    L.cmaqchem_steps_device.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, ip, C.c_int, vp,
                                        C.POINTER(Stats)]
    L.cmaqchem_step_ddm_device.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, ip, vp, C.c_int,
                                           vp, vp, vp, C.POINTER(Stats)]
    L.cmaqchem_cell_stats.argtypes = [vp, vp, vp]
    L.cmaqchem_ros3_solve_device.argtypes = [vp, C.c_longlong, vp, vp, vp, C.c_double, vp, vp, vp, vp]
    L.cmaqchem_ebi_solve_device.argtypes = [vp, C.c_longlong, vp, vp, C.c_int, vp, vp, vp]
    L.cmaqchem_gear_solve_device.argtypes = [vp, C.c_longlong, vp, vp, vp, C.c_double, vp, vp]
    L.cmaqchem_gear_tolerances.argtypes = [vp, C.c_float, C.c_float, C.c_float]
    L.cmaqchem_adj_forward.argtypes = [vp, C.c_longlong, vp, vp, C.c_longlong, vp, vp, vp, C.c_int, C.c_double,
                                       vp, vp, vp, C.c_size_t, vp]
    L.cmaqchem_adj_backward.argtypes = [vp, C.c_longlong, vp, vp, C.c_longlong, vp, vp, vp, C.c_int, C.c_double,
                                        vp, vp, vp, C.c_size_t, vp, vp, vp]
    L.cmaqchem_rconst_device.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.cmaqchem_mech_info_get.argtypes = [C.c_char_p, C.POINTER(MechInfo), ip]
    L.cmaqchem_destroy.argtypes = [vp]
    L.cmaqchem_destroy.restype = None
    L.cmaqchem_last_error.argtypes = [C.c_char_p, C.c_size_t]
    L.cmaqchem_diag_fp64_peak.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.cmaqchem_diag_fp64_issue.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.cmaqchem_diag_fp64_peak_long.argtypes = [C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.cmaqchem_diag_set_tuning.argtypes = [vp, C.c_char_p, C.c_int]
    L.cmaqchem_diag_fp64_rate.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.cmaqchem_diag_phase_cycles.argtypes = [C.c_int, C.POINTER(C.c_ulonglong), C.c_int]
    L.cmaqchem_kmt2_workspace_doubles.argtypes = [C.c_longlong]
    L.cmaqchem_kmt2_workspace_doubles.restype = C.c_longlong
    L.cmaqchem_kmt2_default_lanes.argtypes = [C.c_int]
    L.cmaqchem_kmt2_default_lanes.restype = C.c_longlong
    L.cmaqchem_kmt2_solve_device.argtypes = [C.c_longlong, vp, vp, vp, vp, vp, vp, C.c_longlong, vp]
    L.cmaqchem_kmt2_solve.argtypes = [C.c_longlong, vp, vp, vp, vp, vp, C.c_int]
    L.cmaqchem_aqchem_device.argtypes = [C.c_longlong, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_longlong, vp]
    L.cmaqchem_hetchem_layout.argtypes = [C.c_char_p, ip, ip, ip]
    L.cmaqchem_hetchem_rates_device.argtypes = [C.c_char_p, C.c_longlong, vp, vp, vp, vp, vp, vp, vp]
    L.cmaqchem_hetchem_rates.argtypes = [C.c_char_p, C.c_longlong, vp, vp, vp, vp, vp, vp, C.c_int]
    return L


def fp64_peak(device: int = 0) -> tuple[float, float]:
    """Measured FP64 FMA throughput (TFLOP/s) and kernel time (ms) of `device`."""
    tf, ms = C.c_double(), C.c_double()
    if lib().cmaqchem_diag_fp64_peak(device, C.byref(tf), C.byref(ms)) != 0:
        raise ChemError("FP64 peak measurement failed")
    return tf.value, ms.value


def fp64_peak_long(device: int = 0, target_ms: float = 1000.0) -> tuple[float, float]:
    """Measured FP64 FMA throughput (TFLOP/s) of a kernel of about target_ms, and its time (ms)."""
    tf, ms = C.c_double(), C.c_double()
    if lib().cmaqchem_diag_fp64_peak_long(device, C.c_double(target_ms), C.byref(tf), C.byref(ms)) != 0:
        raise ChemError("FP64 peak measurement failed")
    return tf.value, ms.value


def fp64_rate(device: int = 0, op: int = 0, chains: int = 8, threads: int = 256, blocks_per_sm: int = 8) -> float:
    """FP64 lane operations per clock per SM (at the maximum SM clock) of one kernel shape
    (op 0 fma, 1 mul, 2 add; independent chains per thread; threads; blocks per SM)."""
    r, ms = C.c_double(), C.c_double()
    if lib().cmaqchem_diag_fp64_rate(device, op, chains, threads, blocks_per_sm, C.byref(r), C.byref(ms)) != 0:
        raise ChemError("FP64 rate measurement failed")
    return r.value


def fp64_issue(device: int = 0, active_lanes: int = 1) -> float:
    """Clock cycles per link of a dependent FP64 FMA chain of one warp with active_lanes lanes."""
    c = C.c_double()
    if lib().cmaqchem_diag_fp64_issue(device, int(active_lanes), C.byref(c)) != 0:
        raise ChemError("FP64 issue measurement failed")
    return c.value


def last_error(L: C.CDLL | None = None) -> str:
    buf = C.create_string_buffer(4096)
    (L or lib()).cmaqchem_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, L: C.CDLL | None = None) -> int:
    if rc < 0:
        raise ChemError(last_error(L))
    return rc


def mech_info(mechanism: str):
    info = MechInfo()
    check(lib().cmaqchem_mech_info_get(mechanism.encode(), C.byref(info), None))
    order = (C.c_int * info.nspec)()
    check(lib().cmaqchem_mech_info_get(mechanism.encode(), None, order))
    return info, list(order)
