"""ctypes binding of ``include/dax_gb300.h`` (the C ABI of libdax_gb300.so).

Loading fails loudly when the library has not been built: there is no CPU
fallback anywhere in this package.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libdax_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "dax_gb300.h")

SUCCESS = 0
ERROR_BAD_VALUE = 1
ERROR_OUT_OF_MEMORY = 2
ERROR_EXECUTION = 3
ERROR_CUDA = 4
ERROR_CAPACITY = 5
ERROR_TIMEOUT = 6
ERROR_UNSUPPORTED = 7


class UniformGridDesc(ctypes.Structure):
    """dax_gb300_uniform_grid."""

    _fields_ = [("origin", ctypes.c_float * 3), ("spacing", ctypes.c_float * 3),
                ("extent_min", ctypes.c_int32 * 3), ("extent_max", ctypes.c_int32 * 3)]


class DaxError(RuntimeError):
    """Raised for a non-zero dax_gb300_status; ``code`` holds the status."""

    def __init__(self, code, msg):
        super().__init__("dax_gb300 status %d: %s" % (code, msg))
        self.code = code


class ErrorControlBadValue(DaxError):
    pass


class ErrorControlOutOfMemory(DaxError):
    pass


class ErrorExecution(DaxError):
    pass


_ERR_TYPES = {ERROR_BAD_VALUE: ErrorControlBadValue, ERROR_OUT_OF_MEMORY: ErrorControlOutOfMemory,
              ERROR_EXECUTION: ErrorExecution, ERROR_TIMEOUT: ErrorExecution}

_lib = None

vp = ctypes.c_void_p
f32 = ctypes.c_float
i32 = ctypes.c_int
i64 = ctypes.c_int64
sz = ctypes.c_size_t
gp = ctypes.POINTER(UniformGridDesc)

SIGNATURES = {
    "dax_gb300_abi_version": ([], i32),
    "dax_gb300_last_error": ([], ctypes.c_char_p),
    "dax_gb300_synchronize": ([vp], i32),
    "dax_gb300_classify_words": ([i64], i64),
    "dax_gb300_classify_points": ([vp, i64, i32, f32, f32, vp, vp], i32),
    "dax_gb300_mc_classify_count": ([gp, vp, f32, vp, vp, vp], i32),
    "dax_gb300_mc_scratch_bytes": ([gp], sz),
    "dax_gb300_mc_count": ([gp, vp, f32, vp, sz, vp], i32),
    "dax_gb300_mc_totals": ([vp, ctypes.POINTER(i64), ctypes.POINTER(i64), vp], i32),
    "dax_gb300_mc_generate": ([gp, vp, f32, i32, vp, sz, vp, i64, vp, i64, vp, vp, vp, vp], i32),
    "dax_gb300_mc_pipeline": ([gp, vp, f32, i32, vp, sz, vp, i64, vp, i64, vp, vp, vp, vp], i32),
    "dax_gb300_interpolate_point_field": ([vp, vp, vp, i64, vp, vp, vp], i32),
    "dax_gb300_threshold_classify_count": ([gp, vp, f32, f32, vp, vp], i32),
    "dax_gb300_threshold_scratch_bytes": ([gp], sz),
    "dax_gb300_threshold_count": ([gp, vp, f32, f32, vp, sz, vp], i32),
    "dax_gb300_threshold_compact_point_field": ([gp, vp, sz, vp, ctypes.c_int, vp, i64, vp], i32),
    "dax_gb300_threshold_totals": ([vp, ctypes.POINTER(i64), ctypes.POINTER(i64), vp], i32),
    "dax_gb300_threshold_generate": ([gp, vp, f32, f32, vp, sz, vp, i64, vp, vp, i64, vp], i32),
    "dax_gb300_cell_gradient": ([gp, vp, vp, vp], i32),
    "dax_gb300_field_adjoint": ([gp, vp, f32, vp, sz, vp, vp, vp, vp], i32),
    "dax_gb300_mc_batch_create": ([i32, gp, vp, vp, ctypes.POINTER(vp)], i32),
    "dax_gb300_mc_batch_destroy": ([vp], i32),
    "dax_gb300_mc_batch_scratch_bytes": ([vp], sz),
    "dax_gb300_mc_batch_count": ([vp, vp, sz, vp], i32),
    "dax_gb300_mc_batch_totals": ([vp, vp, vp, vp, vp], i32),
    "dax_gb300_mc_batch_generate": ([vp, i32, vp, sz, vp, i64, vp, i64, vp], i32),
    "dax_gb300_mc_batch_capture": ([vp, i32, vp, sz, vp, i64, vp, i64, ctypes.POINTER(vp)], i32),
    "dax_gb300_mc_batch_autotune": ([vp, i32, vp, sz, vp, i64, vp, i64, vp,
                                     ctypes.POINTER(ctypes.c_float)], i32),
    "dax_gb300_mc_batch_set_config": ([vp, i32, i32], i32),
    "dax_gb300_mc_batch_sizes": ([vp, ctypes.POINTER(i64), ctypes.POINTER(i64)], i32),
    "dax_gb300_mc_batch_cell_gradient": ([vp, vp, vp], i32),
    "dax_gb300_mc_batch_field_adjoint": ([vp, vp, sz, vp, vp, vp, vp], i32),
    "dax_gb300_mc_batch_get_config": ([vp, ctypes.POINTER(i32), ctypes.POINTER(i32)], i32),
    "dax_gb300_graph_launch": ([vp, vp], i32),
    "dax_gb300_graph_destroy": ([vp], i32),
    "dax_gb300_mc_noalloc": ([gp, vp, f32, i32, vp, i64, vp, i64, vp, vp], i32),
    "dax_gb300_slice_field": ([gp, vp, vp, vp, ctypes.POINTER(f32), vp], i32),
    "dax_gb300_slice_count": ([gp, vp, vp, vp, sz, vp], i32),
    "dax_gb300_slice_generate": ([gp, vp, vp, ctypes.c_int, vp, sz, vp, i64, vp, i64, vp, vp, vp,
                                  vp], i32),
    "dax_gb300_tetrahedralize": ([gp, vp, vp], i32),
    "dax_gb300_point_coordinates": ([gp, vp, vp], i32),
    "dax_gb300_mt_classify_count": ([vp, i64, vp, i64, f32, vp, vp], i32),
    "dax_gb300_mt_scratch_bytes": ([i64], sz),
    "dax_gb300_mt_count": ([vp, i64, vp, i64, f32, vp, sz, vp], i32),
    "dax_gb300_mt_merge_scratch_bytes": ([i64, i64], sz),
    "dax_gb300_mt_merge": ([vp, i64, vp, i64, f32, vp, sz, vp, sz, ctypes.POINTER(i64), vp], i32),
    "dax_gb300_mt_generate": ([vp, vp, i64, vp, i64, f32, ctypes.c_int, vp, sz, vp, sz, vp, i64,
                               vp, i64, vp, vp, vp, vp], i32),
    "dax_gb300_mc_counted_scratch_bytes": ([gp], sz),
    "dax_gb300_mc_counted_scan": ([gp, vp, vp, sz, ctypes.POINTER(i64), vp], i32),
    "dax_gb300_mc_counted_merge": ([gp, vp, f32, vp, vp, sz, vp, sz, ctypes.POINTER(i64), vp], i32),
    "dax_gb300_mc_counted_generate": ([gp, vp, f32, vp, ctypes.c_int, vp, sz, vp, sz, vp, i64, vp,
                                       i64, vp, vp, vp, vp], i32),
    "dax_gb300_interpolate_point_field_n": ([vp, vp, vp, i64, vp, i64, ctypes.c_int, vp, vp], i32),
    "dax_gb300_point_magnitude": ([gp, vp, vp], i32),
    "dax_gb300_write_vtk_polydata": ([ctypes.c_char_p, vp, i64, vp, i64, ctypes.c_int], i32),
    "dax_gb300_mandelbulb_field": ([gp, vp, vp], i32),
    "dax_gb300_mandelbulb_clip_count": ([gp, vp, f32, vp, vp, vp, vp, vp], i32),
    "dax_gb300_colors_and_norms": ([vp, i64, vp, vp, vp], i32),
    "dax_gb300_report_error": ([ctypes.c_int, ctypes.c_char_p], i32),
    "dax_gb300_set_blocks_per_sm": ([ctypes.c_int, ctypes.c_int], i32),
    "dax_gb300_set_fused_count": ([ctypes.c_int, ctypes.c_int], i32),
    "dax_gb300_get_fused_count": ([ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], i32),
    "dax_gb300_set_pipeline_slabs": ([ctypes.c_int], i32),
    "dax_gb300_device_alloc": ([ctypes.POINTER(vp), ctypes.c_uint64], i32),
    "dax_gb300_device_free": ([vp], i32),
    "dax_gb300_set_alloc_limit": ([ctypes.c_uint64], i32),
    "dax_gb300_memcpy": ([vp, vp, ctypes.c_uint64, ctypes.c_int], i32),
    "dax_gb300_timer_create": ([ctypes.POINTER(vp)], i32),
    "dax_gb300_timer_start": ([vp, vp], i32),
    "dax_gb300_timer_elapsed": ([vp, vp, ctypes.POINTER(ctypes.c_double)], i32),
    "dax_gb300_timer_destroy": ([vp], i32),
    "dax_gb300_set_pipeline_options": ([ctypes.c_int, ctypes.c_int, ctypes.c_int], i32),
    "dax_gb300_pipeline_timeline": ([ctypes.c_int, vp, ctypes.c_int, vp], i32),
    "dax_gb300_mc_pipeline_plan": ([gp, ctypes.c_int, vp], i32),
    "dax_gb300_selfcheck_division": ([vp, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64,
                                      ctypes.c_uint32, vp, vp], i32),
    "dax_gb300_scan_scratch_bytes": ([i64], sz),
    "dax_gb300_scan": ([vp, vp, i64, i32, i32, vp, sz, vp, vp], i32),
    "dax_gb300_sort_scratch_bytes": ([i64, i32, i32], sz),
    "dax_gb300_sort_by_key": ([vp, vp, i64, i32, i32, i32, vp, sz, vp], i32),
    "dax_gb300_compact_scratch_bytes": ([i64, i32], sz),
    "dax_gb300_unique": ([vp, i64, i32, vp, sz, ctypes.POINTER(i64), vp], i32),
    "dax_gb300_stream_compact": ([vp, i32, vp, i32, i64, vp, vp, sz, ctypes.POINTER(i64), vp], i32),
    "dax_gb300_bounds": ([vp, i64, vp, i64, i32, i32, vp, vp], i32),
}

TYPE_I32, TYPE_U32, TYPE_F32, TYPE_I64, TYPE_U64 = 0, 1, 2, 3, 4


def header_symbols():
    """Function names declared in include/dax_gb300.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|size_t|const char\*)\s+(dax_gb300_\w+)\s*\(", text,
                                 re.M)))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libdax_gb300.so is not built; run daxtoolkit_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(status):
    if status != SUCCESS:
        msg = lib().dax_gb300_last_error().decode(errors="replace")
        raise _ERR_TYPES.get(status, DaxError)(status, msg)
    return status


def call(name, *args):
    return check(getattr(lib(), name)(*args))
