"""ctypes binding of libmulskips_gpu.so (include/mulskips_gpu.h).

The library is the product path; there is no CPU implementation behind these
calls.  Loading fails loudly when the library was not built.
"""
import ctypes as C
import os

import numpy as np

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmulskips_gpu.so")

MKS_NCLASS = 64
ERRORS = {0: "ok", 1: "bad argument", 2: "CUDA error", 3: "invariant violated", 4: "tile capacity",
          5: "unsupported", 6: "bounded wait timed out"}


class MksConfig(C.Structure):
    _fields_ = [("lenx", C.c_int32), ("leny", C.c_int32), ("lenz", C.c_int32),
                ("ncrystal", C.c_int32), ("ncov", C.c_int32), ("list_crystal", C.c_int32 * 3),
                ("ptrans_zig", C.c_double), ("sf", C.c_double), ("seed", C.c_uint64),
                ("list_cov", C.c_int32 * 3), ("explicit_nn", C.c_int32)]


class MksEvent(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32), ("itrans", C.c_int8),
                ("arm", C.c_int8), ("pad", C.c_int16)]


EVENT_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("itrans", "i1"), ("arm", "i1"),
                        ("pad", "<i2")])


class MksObservables(C.Structure):
    _fields_ = [("events", C.c_int64), ("time", C.c_double), ("atoms", C.c_int64),
                ("undercoord", C.c_int64), ("mc_sites", C.c_int64), ("voids", C.c_int64),
                ("species", C.c_int64 * 3), ("mean_height", C.c_double), ("rms_roughness", C.c_double),
                ("total_rate", C.c_double), ("nonepitaxial", C.c_int64), ("covered", C.c_int64)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["species"] = list(self.species)
        return d


class MksLaParams(C.Structure):
    _fields_ = [("P0", C.c_float * 3), ("Tm", C.c_float * 3), ("Tflex", C.c_float * 3), ("sigma", C.c_float * 3),
                ("Tb", C.c_float), ("Ta", C.c_float), ("t0", C.c_float), ("w", C.c_float), ("L_nm", C.c_float),
                ("zsurf", C.c_float), ("score", C.c_int32), ("liquid_weighting", C.c_int32)]


class MksStatus(C.Structure):
    _fields_ = [("error", C.c_int32), ("pending_tiles", C.c_int32), ("fallback_tiles", C.c_int64),
                ("windows", C.c_int64), ("active", C.c_int32), ("stop_reason", C.c_int32)]


# every entry point declared in include/mulskips_gpu.h, with its ctypes signature
SIGNATURES = {
    "mks_create": (C.c_int, [C.POINTER(MksConfig), C.POINTER(C.c_void_p)]),
    "mks_destroy": (None, [C.c_void_p]),
    "mks_version": (C.c_char_p, []),
    "mks_last_error": (C.c_int, [C.c_char_p, C.c_int32]),
    "mks_set_rates": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mks_set_coverage_rates": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mks_init_flat": (C.c_int, [C.c_void_p, C.c_char, C.c_int32]),
    "mks_load_lattice": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mks_get_lattice": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mks_batch_set_tiling": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mks_batch_get_tiling": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mks_load_lists": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p]),
    "mks_get_lists": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p]),
    "mks_state_size": (C.c_int64, [C.c_void_p]),
    "mks_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "mks_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "mks_replay": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "mks_replay_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "mks_run": (C.c_int, [C.c_void_p, C.c_double, C.c_int64, C.c_int64, C.c_double,
                          C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "mks_frame_sites": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "mks_write_frame": (C.c_int, [C.c_void_p, C.c_char_p, C.c_double, C.c_int64, C.c_void_p]),
    "mks_class_histogram": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "mks_site_rates": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "mks_set_colours": (C.c_int, [C.c_void_p, C.c_int32]),
    "mks_batch_lr_accumulate": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mks_batch_lr_result": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "mks_get_colours": (C.c_int32, [C.c_void_p]),
    "mks_get_observables": (C.c_int, [C.c_void_p, C.POINTER(MksObservables)]),
    "mks_get_status": (C.c_int, [C.c_void_p, C.POINTER(MksStatus)]),
    "mks_batch_create": (C.c_int, [C.POINTER(MksConfig), C.c_int32, C.POINTER(C.c_void_p)]),
    "mks_batch_set_rates": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mks_batch_set_coverage_rates": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mks_batch_init_flat": (C.c_int, [C.c_void_p, C.c_char, C.c_void_p]),
    "mks_batch_run": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_double,
                                C.POINTER(C.c_int64)]),
    "mks_batch_observables": (C.c_int, [C.c_void_p, C.POINTER(MksObservables)]),
    "mks_batch_size": (C.c_int32, [C.c_void_p]),
    "mks_set_tiling": (C.c_int, [C.c_void_p, C.c_int32]),
    "mks_get_tiling": (C.c_int32, [C.c_void_p]),
    "mks_set_schedule": (C.c_int, [C.c_void_p, C.c_int32]),
    "mks_suggest_tau": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p]),
    "mks_batch_set_la": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mks_batch_get_score": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "mks_batch_la_counts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mks_batch_class_histogram": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "mks_prefetch_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "mks_swap_state": (C.c_int, [C.c_void_p]),
    "mks_get_clock": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                C.POINTER(C.c_int64)]),
    "mks_set_clock": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_int64, C.c_int64]),
    "mks_debug_hold_tile": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64]),
    "mks_batch_load_temperature": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "mks_batch_set_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "mks_batch_init_shape": (C.c_int, [C.c_void_p, C.c_int32, C.c_char_p, C.c_void_p, C.c_void_p]),
    "mks_batch_get_state": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    "mks_init_shape": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_void_p]),
    "mks_batch_init_cad": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "mks_batch_init_cad_alloy": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_double, C.c_uint64]),
    "mks_batch_init_points": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64]),
    "mks_init_points": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]),
    "mks_batch_init_cad_la": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_double, C.c_double]),
    "mks_batch_set_tabulated": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mks_batch_get_phases": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "mks_batch_load_lattice": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "mks_batch_lr_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "mks_batch_init_alloy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]),
    "mks_last_run_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                     C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
}

_lib = None


def lib():
    """Load libmulskips_gpu.so; raises if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise RuntimeError(f"{_LIB_PATH} is missing: build it with mulskips_gb300.build.build_all() "
                               "(the GB300 engine has no CPU implementation)")
        L = C.CDLL(_LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class MksError(RuntimeError):
    pass


def check(rc):
    if rc != 0:
        buf = C.create_string_buffer(512)
        lib().mks_last_error(buf, 512)
        raise MksError(f"{ERRORS.get(rc, rc)}: {buf.value.decode(errors='replace')}")


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)
