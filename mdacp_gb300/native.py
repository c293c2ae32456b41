"""ctypes binding of libmdg.so (include/mdg.h).

The library must exist in-tree (built by mdacp_gb300.build or
__graft_entry__.build()); there is no fallback implementation: loading fails
loudly when it is missing.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmdg.so")
CHECK_LIB_PATH = os.path.join(HERE, "libmdg_check.so")

MDG_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "capacity", 4: "bad particle state", 5: "no state"}
FP64, MIXED, MIXED_PLAIN = 0, 1, 2
PRECISIONS = {"fp64": FP64, "mixed": MIXED, "mixed_plain": MIXED_PLAIN}
NVE, LANGEVIN, NOSEHOOVER = 0, 1, 2
REBUILD_HALFMARGIN, REBUILD_REFERENCE = 0, 1
REBUILD_POLICIES = {"halfmargin": REBUILD_HALFMARGIN, "reference": REBUILD_REFERENCE}


class Params(ctypes.Structure):
    _fields_ = [("capacity", ctypes.c_int32), ("precision", ctypes.c_int32), ("box", ctypes.c_double * 3),
                ("cutoff", ctypes.c_double), ("margin", ctypes.c_double), ("dt", ctypes.c_double),
                ("thermostat", ctypes.c_int32), ("langevin_half_drift_compat", ctypes.c_int32),
                ("temperature", ctypes.c_double), ("gamma", ctypes.c_double), ("tau", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("list_capacity", ctypes.c_int32), ("device", ctypes.c_int32),
                ("use_graphs", ctypes.c_int32), ("rebuild_policy", ctypes.c_int32), ("prune_buffer", ctypes.c_double),
                ("check_list_length", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("rebuilds", ctypes.c_int64), ("list_capacity", ctypes.c_int32),
                ("max_neighbours", ctypes.c_int32), ("listed_pairs", ctypes.c_int64),
                ("cells", ctypes.c_int32 * 3), ("particles", ctypes.c_int32), ("zeta", ctypes.c_double),
                ("elapsed_ms", ctypes.c_double), ("kernel_launches", ctypes.c_int64),
                ("inner_pairs", ctypes.c_int64), ("prunes", ctypes.c_int64)]


# Every exported symbol of include/mdg.h, with (restype, argtypes).
_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "mdg_version": (ctypes.c_char_p, []),
    "mdg_params_default": (None, [ctypes.POINTER(Params)]),
    "mdg_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(_P)]),
    "mdg_destroy": (ctypes.c_int, [_P]),
    "mdg_last_error": (ctypes.c_char_p, [_P]),
    "mdg_set_state": (ctypes.c_int, [_P, _D, _D, ctypes.c_int32]),
    "mdg_get_state": (ctypes.c_int, [_P, _D, _D]),
    "mdg_make_pairlist": (ctypes.c_int, [_P]),
    "mdg_calculate": (ctypes.c_int, [_P, ctypes.c_int32]),
    "mdg_synchronize": (ctypes.c_int, [_P]),
    "mdg_calculate_profiled": (ctypes.c_int, [_P, ctypes.c_int32, _D]),
    "mdg_calculate_phases": (ctypes.c_int, [_P, ctypes.c_int32, _D]),
    "mdg_observe": (ctypes.c_int, [_P, _D]),
    "mdg_forces": (ctypes.c_int, [_P, _D]),
    "mdg_pairs": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32), ctypes.c_int64,
                                 ctypes.POINTER(ctypes.c_int64)]),
    "mdg_set_seed": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "mdg_set_thermostat": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_double]),
    "mdg_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
    "mdg_set_state_device": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32]),
    "mdg_get_state_device": (ctypes.c_int, [_P, _P, _P]),
    "mdg_observe_noalloc": (ctypes.c_int, [_P, _P, ctypes.c_int32, _D, ctypes.c_double, _P, _P]),
    "mdg_write_dump": (ctypes.c_int, [ctypes.c_char_p, _D, _D, ctypes.c_int32, ctypes.c_int32]),
    "mdg_write_cdview": (ctypes.c_int, [ctypes.c_char_p, _D, _D, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                        ctypes.c_int32]),
    "mdg_write_configuration": (ctypes.c_int, [ctypes.c_char_p, _D, _D, ctypes.c_int32]),
    "mdg_write_stream": (ctypes.c_int, [ctypes.c_char_p, _D, _D, ctypes.c_int32, ctypes.c_int32]),
    "mdg_read_stream": (ctypes.c_int, [ctypes.c_char_p, _D, _D, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                       _D, _D]),
    "mdg_save_dump": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "mdg_save_cdview": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "mdg_make_configuration": (ctypes.c_int, [_D, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                              ctypes.c_double, _P, _P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                              _P]),
    "mdg_make_velocity": (ctypes.c_int, [ctypes.c_double, ctypes.c_int32, _P, ctypes.c_int32, _P]),
    "mdg_make_state": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
}
MAKERS = {"fcc": 0, "extract": 1, "droplet": 2, "collision": 3}

_lib = None


def load(path=None):
    """Loads libmdg.so and declares every entry point; raises if it is missing.

    MDG_LIBRARY=check selects the bounds-checked build (libmdg_check.so, made
    by build.build(check=True)) for the whole process."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or (CHECK_LIB_PATH if os.environ.get("MDG_LIBRARY") == "check" else LIB_PATH)
    if not os.path.exists(p):
        raise RuntimeError("libmdg.so not built (%s); run __graft_entry__.build()" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class MDGError(RuntimeError):
    pass


def check(rc, handle=None, create=False):
    """Raises MDGError for a failed call, with the handle's message (or, for
    create=True, the calling thread's last mdg_create failure)."""
    if rc != MDG_OK:
        msg = ERRORS.get(rc, "error %d" % rc)
        if handle or create:
            detail = load().mdg_last_error(handle if handle else None)
            if detail:
                msg += ": " + detail.decode()
        raise MDGError(msg)
