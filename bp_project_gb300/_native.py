"""ctypes binding of libsarbp.so (C ABI declared in include/sarbp.h).

The library is the only compute path of this package: if it is missing or
cannot be loaded, every entry point raises instead of falling back to a CPU
implementation.  Build it with ``python -m bp_project_gb300.build`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIBRARY = Path(__file__).resolve().parent / "libsarbp.so"

MODE_IDS = {"fp64": 0, "fp32": 1, "mixed": 2, "split": 3}

SARBP_OK = 0
SARBP_ERR_VALUE = 1
SARBP_ERR_TYPE = 2
SARBP_ERR_WORKSPACE = 3
SARBP_ERR_CUDA = 4
SARBP_ERR_PLAN = 5
SARBP_ERR_ENVELOPE = 6

_EXCEPTIONS = {
    SARBP_ERR_VALUE: ValueError,
    SARBP_ERR_TYPE: TypeError,
    SARBP_ERR_WORKSPACE: ValueError,
    SARBP_ERR_CUDA: RuntimeError,
    SARBP_ERR_PLAN: RuntimeError,
    SARBP_ERR_ENVELOPE: ValueError,
}


class PolarGrid(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("r0", ctypes.c_double), ("dr", ctypes.c_double),
                ("u0", ctypes.c_double), ("du", ctypes.c_double), ("nr", ctypes.c_int32), ("nu", ctypes.c_int32),
                ("side", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Lattice(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("step_row", ctypes.c_double * 3),
                ("step_col", ctypes.c_double * 3), ("rows", ctypes.c_int32), ("cols", ctypes.c_int32)]


class FFBPNode(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("r0", ctypes.c_double), ("dr", ctypes.c_double),
                ("u0", ctypes.c_double), ("du", ctypes.c_double), ("nr", ctypes.c_int32), ("nu", ctypes.c_int32),
                ("a", ctypes.c_int32), ("b", ctypes.c_int32), ("left", ctypes.c_int32), ("right", ctypes.c_int32),
                ("side", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class BatchScene(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("pulses", ctypes.c_int32), ("samples", ctypes.c_int32),
                ("pos", ctypes.c_void_p), ("weight", ctypes.c_void_p), ("phase", ctypes.c_void_p),
                ("range_start", ctypes.c_double), ("data_dr", ctypes.c_double), ("k", ctypes.c_double),
                ("kind", ctypes.c_int32), ("lattice", Lattice), ("nodes", ctypes.POINTER(FFBPNode)),
                ("n_nodes", ctypes.c_int32), ("crop_r0", ctypes.c_int32), ("crop_u0", ctypes.c_int32),
                ("crop_nr", ctypes.c_int32), ("crop_nu", ctypes.c_int32), ("tile_lc", ctypes.c_int32),
                ("chunk_pulses", ctypes.c_int32), ("out", ctypes.c_void_p)]


BATCH_DIRECT = 0
BATCH_FFBP = 1

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_Z = ctypes.c_size_t
_I64 = ctypes.c_int64

# name -> (argtypes, restype); mirrors include/sarbp.h.
SIGNATURES = {
    "sarbp_version": ([], ctypes.c_char_p),
    "sarbp_abi_version": ([], _I),
    "sarbp_status_string": ([_I], ctypes.c_char_p),
    "sarbp_last_error": ([], ctypes.c_char_p),
    "sarbp_launch_count": ([], ctypes.c_uint64),
    "sarbp_direct_polar_workspace": ([_I, ctypes.POINTER(PolarGrid), _I, _I], _Z),
    "sarbp_direct_polar": ([_P, _I, _I, _P, _P, _P, ctypes.POINTER(PolarGrid), _D, _D, _D, _I, _I, _I, _P, _P, _Z,
                            _P], _I),
    "sarbp_static_scratch_elements": ([], _Z),
    "sarbp_direct_polar_static": ([_P, _I, _I, _P, _P, _P, ctypes.POINTER(PolarGrid), _D, _D, _D, _I, _I, _P, _P],
                                  _I),
    "sarbp_backproject_points_workspace": ([_I, _I, _I], _Z),
    "sarbp_backproject_points": ([_P, _I, _I, _P, _P, _P, _P, _I, _D, _D, _D, _I, _I, _P, _P, _Z, _P], _I),
    "sarbp_backproject_lattice_workspace": ([_I, ctypes.POINTER(Lattice), _I], _Z),
    "sarbp_backproject_lattice": ([_P, _I, _I, _P, _P, _P, ctypes.POINTER(Lattice), _D, _D, _D, _I, _I, _P, _P, _Z,
                                   _P], _I),
    "sarbp_backproject_lattice_adjoint_workspace": ([ctypes.POINTER(Lattice), _I], _Z),
    "sarbp_backproject_lattice_adjoint": ([_P, _I, _I, _P, _P, _P, ctypes.POINTER(Lattice), _D, _D, _D, _P, _P, _P, _P,
                                           _P, _Z, _P], _I),
    "sarbp_batch_create": ([ctypes.POINTER(BatchScene), _I, _I, ctypes.POINTER(_P)], _I),
    "sarbp_batch_destroy": ([_P], None),
    "sarbp_batch_workspace_bytes": ([_P], _Z),
    "sarbp_batch_launch_count": ([_P], _I),
    "sarbp_batch_info": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                          ctypes.POINTER(_D)], _I),
    "sarbp_batch_bind": ([_P, _P, _Z, _P], _I),
    "sarbp_batch_execute": ([_P, _P], _I),
    "sarbp_batch_set_trace": ([_P, _P], _I),
    "sarbp_batch_set_concurrent": ([_P, _I], _I),
    "sarbp_rc_prepare": ([_P, _I, _I, _I, _P, _P], _I),
    "sarbp_decode_iq": ([_P, _I, _I64, _I, _I, _P, _P], _I),
    "sarbp_rc_filter": ([_P, _P, _I, _I, _I, _P, _P], _I),
    "sarbp_rc_crop": ([_P, _I, _I, _I, _I, ctypes.c_float, _P, _P], _I),
    "sarbp_tile_argmax": ([_P, _I, _I, _I, _I, _P, _P, _P], _I),
    "sarbp_sosfiltfilt_workspace": ([_I, _I, _I], _Z),
    "sarbp_sosfiltfilt": ([_P, _I, _I, _P, _P, _I, _P, _I, _P, _P, _Z, _P], _I),
    "sarbp_regrid": ([_P, ctypes.POINTER(PolarGrid), ctypes.POINTER(PolarGrid), _D, _I, _P, _P], _I),
    "sarbp_merge_regrid": ([_P, ctypes.POINTER(PolarGrid), _P, ctypes.POINTER(PolarGrid), ctypes.POINTER(PolarGrid),
                            _D, _I, _P, _P], _I),
    "sarbp_add_inplace": ([_P, _P, _I64, _P], _I),
    "sarbp_cast_c128_to_c64": ([_P, _P, _I64, _P], _I),
    "sarbp_crop": ([_P, _I, _I, _I, _I, _I, _P, _P], _I),
    "sarbp_ffbp_plan_create": ([ctypes.POINTER(FFBPNode), _I, _I, _I, _I, _I, _I, ctypes.POINTER(_P)], _I),
    "sarbp_ffbp_plan_destroy": ([_P], None),
    "sarbp_ffbp_workspace_bytes": ([_P], _Z),
    "sarbp_ffbp_launch_count": ([_P], _I),
    "sarbp_ffbp_bind": ([_P, _P, _Z, _P], _I),
    "sarbp_ffbp_execute": ([_P, _P, _I, _I, _P, _P, _P, _D, _D, _D, _P, _P], _I),
    "sarbp_evaluate_image": ([_P, ctypes.POINTER(PolarGrid), _P, _I, _D, _P, _P], _I),
    "sarbp_evaluate_lattice": ([_P, ctypes.POINTER(PolarGrid), ctypes.POINTER(Lattice), _D, _P, _P], _I),
    "sarbp_target_contributions": ([_P, _I, _I, _P, _P, _I, _D, _D, _D, _P, _P], _I),
    "sarbp_fill_range_phase_lut": ([_I, _D, _D, _D, _P, _P], _I),
    "sarbp_direct_polar_lut": ([_P, _I, _I, _P, _P, _P, ctypes.POINTER(PolarGrid), _D, _D, _D, _P, _P, _P], _I),
    "sarbp_direct_polar_phase32": ([_P, _I, _I, _P, _P, _P, ctypes.POINTER(PolarGrid), _D, _D, _D, _I, _P, _P], _I),
    "sarbp_fp32_peak": ([_I, _I, ctypes.POINTER(_D)], _I),
    "sarbp_wait_timeouts": ([ctypes.POINTER(_I)], _I),
    "sarbp_ffbp_set_node_image": ([_P, _I, _P, _P], _I),
    "sarbp_ffbp_set_merge_queue": ([_P, _I], _I),
    "sarbp_ffbp_set_staging": ([_P, _I], _I),
    "sarbp_ffbp_staging": ([_P, _P], _I),
    "sarbp_ffbp_set_wait_limit": ([_P, _D, _I], _I),
    "sarbp_ffbp_status": ([_P, ctypes.POINTER(_I)], _I),
}

_lock = threading.Lock()
_lib = None


def load() -> ctypes.CDLL:
    """Load libsarbp.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIBRARY.exists():
                raise RuntimeError(
                    f"{LIBRARY} is missing: build the CUDA library first "
                    "(python -m bp_project_gb300.build); there is no CPU fallback")
            lib = ctypes.CDLL(str(LIBRARY))
            for name, (args, res) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = res
            _lib = lib
    return _lib


def check(status: int, what: str = "") -> None:
    """Map a sarbp status code to the exception type the reference raises."""
    if status == SARBP_OK:
        return
    lib = load()
    msg = lib.sarbp_last_error().decode(errors="replace") or lib.sarbp_status_string(status).decode()
    raise _EXCEPTIONS.get(status, RuntimeError)(f"{what}: {msg}" if what else msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def mode_id(mode: str) -> int:
    try:
        return MODE_IDS[mode]
    except KeyError:
        raise ValueError(f"mode must be one of {tuple(MODE_IDS)}") from None


def launch_count() -> int:
    return int(load().sarbp_launch_count())


def polar_grid(origin, r0, dr, nr, u0, du, nu, side) -> PolarGrid:
    g = PolarGrid()
    g.origin[:] = [float(v) for v in origin]
    g.r0, g.dr, g.u0, g.du = float(r0), float(dr), float(u0), float(du)
    g.nr, g.nu, g.side = int(nr), int(nu), int(side)
    return g


def lattice(origin, step_row, step_col, rows, cols) -> Lattice:
    lat = Lattice()
    lat.origin[:] = [float(v) for v in origin]
    lat.step_row[:] = [float(v) for v in step_row]
    lat.step_col[:] = [float(v) for v in step_col]
    lat.rows, lat.cols = int(rows), int(cols)
    return lat
