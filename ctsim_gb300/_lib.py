"""ctypes binding of libctgpu.so (include/ctgpu.h).

The library must have been built (``python -m ctsim_gb300.build`` or
``__graft_entry__.build()``); loading fails loudly otherwise -- there is no CPU
fallback in this package.
"""
import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libctgpu.so")

CTGPU_OK = 0
ERRORS = {1: "invalid argument", 2: "unsupported", 3: "CUDA error", 4: "out of memory",
          5: "kernel wait timeout", 6: "I/O error"}
RUN_POSTPROCESS = 1
RUN_ACCUMULATE = 2


class CtgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ctgpu error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


class Geometry(C.Structure):
    """ctgpu_geometry: the .pj header fields."""
    _fields_ = [("geometry", C.c_int32), ("n_det", C.c_int32), ("n_view", C.c_int32),
                ("reserved", C.c_int32), ("rot_start", C.c_double), ("rot_inc", C.c_double),
                ("det_start", C.c_double), ("det_inc", C.c_double),
                ("view_diameter", C.c_double), ("focal_length", C.c_double),
                ("source_detector_length", C.c_double), ("fan_beam_angle", C.c_double)]


class Roi(C.Structure):
    _fields_ = [("x_min", C.c_double), ("y_min", C.c_double), ("x_max", C.c_double),
                ("y_max", C.c_double)]


class BatchProblem(C.Structure):
    """ctgpu_batch_problem"""
    _fields_ = [("geometry", Geometry), ("nx", C.c_int), ("ny", C.c_int),
                ("filter_name", C.c_char_p), ("filter_param", C.c_double),
                ("filter_method", C.c_char_p), ("zeropad", C.c_int),
                ("filter_generation", C.c_char_p), ("interp_name", C.c_char_p),
                ("backproj_name", C.c_char_p), ("d_sino", C.c_void_p), ("sino_pitch", C.c_int),
                ("h_view_angles", C.c_void_p), ("d_image", C.c_void_p)]


BATCH_AUTOTUNE = 1
BATCH_GRAPH = 2

_lib = None

# (name, argtypes) for every exported entry point; used for loading and for
# the symbol-export test.
_d, _i, _p, _s, _f = C.c_double, C.c_int, C.c_void_p, C.c_char_p, C.c_float
_pp = C.POINTER(C.c_void_p)
SIGNATURES = {
    "ctgpu_last_error": ([], C.c_char_p),
    "ctgpu_abi_version": ([], _i),
    "ctgpu_sync": ([_p], _i),
    "ctgpu_phantom_create": ([_pp], _i),
    "ctgpu_phantom_create_builtin": ([_s, _pp], _i),
    "ctgpu_phantom_add_element": ([_p, _s, _d, _d, _d, _d, _d, _d], _i),
    "ctgpu_phantom_read_file": ([_p, _s], _i),
    "ctgpu_phantom_bounds": ([_p, C.POINTER(_d), C.POINTER(_i)], _i),
    "ctgpu_phantom_destroy": ([_p], None),
    "ctgpu_phantom_rasterize": ([_p, _i, _i, _d, _i, _p, C.POINTER(_d), C.POINTER(_d), _p], _i),
    "ctgpu_scanner_create": ([_p, _s, _i, _i, _i, _i, _d, _d, _d, _d, _d, _pp], _i),
    "ctgpu_scanner_geometry": ([_p, C.POINTER(Geometry)], _i),
    "ctgpu_collect_projections": ([_p, _p, _i, _i, _i, _i, _p, _i, _p, _p], _i),
    "ctgpu_collect_projections_batch": ([_p, _pp, _i, _p, _i, C.c_longlong, _p, _p], _i),
    "ctgpu_collect_projections_host": ([_p, _p, _i, _i, _i, _i, _p, _p], _i),
    "ctgpu_scanner_destroy": ([_p], None),
    "ctgpu_recon_create": ([C.POINTER(Geometry), _i, _i, _s, _d, _s, _i, _s, _s, _i, _s,
                            C.POINTER(Roi), _pp], _i),
    "ctgpu_recon_image_axes": ([_p, C.POINTER(_d), C.POINTER(_d)], _i),
    "ctgpu_recon_filter": ([_p, _p, _i, _i, _p, _i, _p], _i),
    "ctgpu_recon_backproject": ([_p, _p, _i, _p, _i, _p, _i, _p], _i),
    "ctgpu_recon_postprocess": ([_p, _p, _p], _i),
    "ctgpu_recon_run": ([_p, _p, _i, _p, _i, _i, _p, _i, _p], _i),
    "ctgpu_recon_run_host": ([_p, _p, _p, _p], _i),
    "ctgpu_recon_run_batch": ([_p, _i, _p, _i, C.c_longlong, _p, _p, C.c_longlong, _i, _p], _i),
    "ctgpu_recon_run_batch_host": ([_p, _i, _p, _p, _p, _i], _i),
    "ctgpu_recon_backproject_batch": ([_p, _i, _p, _i, C.c_longlong, _p, _i, _p, C.c_longlong,
                                       _i, _p], _i),
    "ctgpu_recon_project": ([_p, _p, _p, _i, _p, _i, _f, _p], _i),
    "ctgpu_recon_destroy": ([_p], None),
    "ctgpu_helical180li_size": ([C.POINTER(Geometry), _i, _i, C.POINTER(_i)], _i),
    "ctgpu_helical180li": ([C.POINTER(Geometry), _p, _i, _i, _p, _i, _p, C.POINTER(_i), _p], _i),
    "ctgpu_halfscan_feather": ([C.POINTER(Geometry), _p, _i, _i, _p], _i),
    "ctgpu_helical180li_equilinear_size": ([C.POINTER(Geometry), _i, _i, C.POINTER(_i)], _i),
    "ctgpu_helical180li_equilinear": ([C.POINTER(Geometry), _p, _i, _i, _p, _i, _p, C.POINTER(_i),
                                       _p], _i),
    "ctgpu_halfscan_feather_equilinear": ([C.POINTER(Geometry), _p, _i, _i, _p], _i),
    "ctgpu_interpolate_to_parallel": ([C.POINTER(Geometry), _p, _i, _p, _p, _i,
                                       C.POINTER(Geometry), _p, _p], _i),
    "ctgpu_helical_plan_create": ([C.POINTER(Geometry), _i, _i, _pp], _i),
    "ctgpu_helical_plan_views": ([_p, C.POINTER(_i)], _i),
    "ctgpu_helical_plan_run": ([_p, _p, _i, _p, _i, _p, _i, C.c_longlong, _p, _p], _i),
    "ctgpu_helical_plan_destroy": ([_p], None),
    "ctgpu_raysum_ellipse_gradient": ([_p, _p, _p, _i, _p, _p], _i),
    "ctgpu_collect_projections_ellipsoids": ([_p, _p, _i, _d, _d, _p, _i, _p, _p], _i),
    "ctgpu_batch_create": ([C.POINTER(BatchProblem), _i, _i, _pp], _i),
    "ctgpu_batch_run": ([_p, _p], _i),
    "ctgpu_batch_shape": ([_p, C.POINTER(_i), C.POINTER(_i)], _i),
    "ctgpu_batch_destroy": ([_p], None),
    "ctgpu_backproject_diff_noalloc": ([C.POINTER(Geometry), _i, _i, _s, C.POINTER(Roi), _p, _i,
                                        _p, _i, _p, _i, _p], _i),
}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libctgpu.so is not built (python -m ctsim_gb300.build); "
                               "this package has no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(rc):
    if rc != CTGPU_OK:
        raise CtgpuError(rc, lib().ctgpu_last_error().decode(errors="replace"))
    return rc


def enc(s):
    return s.encode() if isinstance(s, str) else s
