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


class PjInfo(C.Structure):
    """ctgpu_pj_info: a .pj header"""
    _fields_ = [("geometry", Geometry), ("calc_time", C.c_double), ("date", C.c_int32 * 6),
                ("header_size", C.c_int32), ("remark_length", C.c_int32)]


class IfInfo(C.Structure):
    """ctgpu_if_info: an .if header"""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("pixel_format", C.c_int32),
                ("pixel_size", C.c_int32), ("data_type", C.c_int32), ("n_labels", C.c_int32),
                ("increment_known", C.c_int32), ("extent_known", C.c_int32),
                ("increment", C.c_double * 2), ("extent", C.c_double * 4),
                ("offset_pv", C.c_double), ("scale_pv", C.c_double),
                ("header_size", C.c_int32), ("reserved", C.c_int32)]


class IfLabel(C.Structure):
    """ctgpu_if_label"""
    _fields_ = [("type", C.c_int32), ("date", C.c_int32 * 6), ("calc_time", C.c_double),
                ("text", C.c_char_p), ("text_length", C.c_int32), ("reserved", C.c_int32)]


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
    "ctgpu_collect_projections_multi": ([_pp, _pp, _i, _pp, _p, _pp, _p], _i),
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
    "ctgpu_recon_host_chunks": ([_p, _i, _p, _i], _i),
    "ctgpu_recon_set_host_chunks": ([_p, _p, _i], _i),
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
    "ctgpu_convert_polar": ([C.POINTER(Geometry), _p, _i, _p, _i, _i, _s, _p, _p], _i),
    "ctgpu_convert_fft_polar": ([C.POINTER(Geometry), _p, _i, _p, _i, _i, _s, _i, _p, _p,
                                 C.POINTER(_i), _p], _i),
    "ctgpu_image_ifft_magnitude": ([_p, _p, _i, _i, _p, _p], _i),
    "ctgpu_reconstruct_fourier": ([C.POINTER(Geometry), _p, _i, _p, _i, _i, _s, _i, _p, _p], _i),
    "ctgpu_pj_read_header": ([_s, C.POINTER(PjInfo), _s, _i], _i),
    "ctgpu_pj_read_device": ([_s, _p, _i, _p, C.POINTER(_i), _p], _i),
    "ctgpu_pj_write_device": ([_s, C.POINTER(PjInfo), _s, _p, _i, _p, _p], _i),
    "ctgpu_pj_pack": ([_p, _i, _p, _i, _i, _p, _p], _i),
    "ctgpu_pj_unpack": ([_p, _i, _i, _p, _i, _p, _p, _p], _i),
    "ctgpu_if_read_header": ([_s, C.POINTER(IfInfo)], _i),
    "ctgpu_if_read_labels": ([_s, C.POINTER(IfLabel), _i, _s, C.c_size_t, C.POINTER(_i)], _i),
    "ctgpu_if_read_device": ([_s, _p, _p], _i),
    "ctgpu_if_write_device": ([_s, C.POINTER(IfInfo), C.POINTER(IfLabel), _i, _p, _p], _i),
    "ctgpu_sino_to_image": ([_p, _i, _i, _i, _p, _p], _i),
    "ctgpu_image_compare": ([_p, _p, _i, _i, _i, C.c_size_t, _p, _p], _i),
    "ctgpu_image_compare_device": ([_p, _p, _i, _i, _i, C.c_size_t, _p, _p], _i),
    "ctgpu_image_arith": ([_s, _p, _p, _p, C.c_size_t, _p], _i),
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
