"""TEST INFRASTRUCTURE ONLY: ctypes binding of the FP64 CPU restatement
(oracle/ctoracle.c) of CTSim's simulate-and-reconstruct path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker / CPU baseline.  The GPU library never imports
it.  Build the shared object with ``make -C oracle oracle``.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

GEOMETRIES = {"parallel": 0, "equiangular": 1, "equilinear": 2}
BACKPROJ = {"trig": 0, "table": 1, "diff": 2, "idiff": 3}
INTERP = {"nearest": 0, "linear": 1, "cubic": 2}


class _PElem(C.Structure):
    _fields_ = [("type", C.c_int), ("cx", C.c_double), ("cy", C.c_double), ("u", C.c_double),
                ("v", C.c_double), ("rot", C.c_double), ("atten", C.c_double),
                ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
                ("ymax", C.c_double), ("phm2obj", C.c_double * 9), ("obj2phm", C.c_double * 9)]


class _Phantom(C.Structure):
    _fields_ = [("n", C.c_int), ("unit_pulse", C.c_int), ("cap", C.c_int),
                ("e", C.POINTER(_PElem)),
                ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
                ("ymax", C.c_double)]


class _Scanner(C.Structure):
    _fields_ = [("fail", C.c_int), ("geometry", C.c_int), ("nDet", C.c_int), ("nView", C.c_int),
                ("offsetView", C.c_int), ("nSample", C.c_int)] + [
        (n, C.c_double) for n in (
            "rotLen rotInc detInc detLen detStart viewDiameter scanDiameter focalLength "
            "centerDetectorLength sourceDetectorLength fanBeamAngle xCenter yCenter "
            "angularDetLen angularDetInc xs1 ys1 xs2 ys2 xd1 yd1 xd2 yd2").split()] + [
        ("incmtx", C.c_double * 9)]


class _ProcSig(C.Structure):
    _fields_ = [("fail", C.c_int), ("filterId", C.c_int), ("method", C.c_int),
                ("generation", C.c_int), ("geometry", C.c_int), ("nSignal", C.c_int),
                ("nFilterPoints", C.c_int), ("nOutput", C.c_int), ("zeropad", C.c_int),
                ("interpFactor", C.c_int), ("signalInc", C.c_double), ("bandwidth", C.c_double),
                ("param", C.c_double), ("focalLength", C.c_double), ("sdl", C.c_double),
                ("filter", C.POINTER(C.c_double)), ("cosTable", C.POINTER(C.c_double)),
                ("sinTable", C.POINTER(C.c_double)), ("nTable", C.c_int)]


class Geom(C.Structure):
    """Scan geometry as stored in a .pj header."""
    _fields_ = [("geometry", C.c_int), ("nDet", C.c_int), ("nView", C.c_int),
                ("rotInc", C.c_double), ("detInc", C.c_double), ("focalLength", C.c_double),
                ("sourceDetectorLength", C.c_double), ("viewDiameter", C.c_double),
                ("fanBeamAngle", C.c_double)]


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libctoracle.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle not built: run `make -C oracle oracle`")
        _LIB = C.CDLL(path)
        d, i, p = C.c_double, C.c_int, C.c_void_p
        _LIB.ora_scanner_init.argtypes = [C.POINTER(_Scanner), C.POINTER(_Phantom), i, i, i, i,
                                          i, d, d, d, d, d]
        _LIB.ora_collect_projections.argtypes = [C.POINTER(_Scanner), C.POINTER(_Phantom), i, i,
                                                 i, i, p, p, i]
        _LIB.ora_phantom_add.argtypes = [C.POINTER(_Phantom), i, d, d, d, d, d, d]
        _LIB.ora_phantom_builtin.argtypes = [C.POINTER(_Phantom), C.c_char_p]
        _LIB.ora_phantom_init.argtypes = [C.POINTER(_Phantom), i]
        _LIB.ora_phantom_free.argtypes = [C.POINTER(_Phantom)]
        _LIB.ora_name_to_pelem_type.argtypes = [C.c_char_p]
        _LIB.ora_raysum.argtypes = [C.POINTER(_Phantom), d, d, d, d]
        _LIB.ora_raysum.restype = d
        _LIB.ora_procsig_init.argtypes = [C.POINTER(_ProcSig), i, i, d, d, i, d, i, i, i, i, d, d]
        _LIB.ora_procsig_free.argtypes = [C.POINTER(_ProcSig)]
        _LIB.ora_filter_views.argtypes = [C.POINTER(_ProcSig), p, i, p, i]
        for n in ("ora_filter_id", "ora_filter_method_id", "ora_filter_generation_id"):
            getattr(_LIB, n).argtypes = [C.c_char_p]
        _LIB.ora_backproject.argtypes = [C.POINTER(Geom), p, i, p, i, i, i, i, p, i, i, p, i, i]
        _LIB.ora_reconstruct.argtypes = [C.POINTER(Geom), p, p, i, i, i, d, i, i, i, i, i, p, i]
        _LIB.ora_helical180li.argtypes = [C.POINTER(Geom), p, i, i, p, p, C.POINTER(C.c_int)]
        _LIB.ora_halfscan_feather.argtypes = [C.POINTER(Geom), p, i]
        _LIB.ora_helical180li_ex.argtypes = [C.POINTER(Geom), p, i, i, p, p, C.POINTER(C.c_int), i]
        _LIB.ora_halfscan_feather_ex.argtypes = [C.POINTER(Geom), p, i, i]
        _LIB.ora_collect_ellipsoids.argtypes = [C.POINTER(_Scanner), p, i, d, d, p, p, i]
        _LIB.ora_ellipse_gradient.argtypes = [C.POINTER(_Scanner), C.POINTER(_Phantom), p, p]
        _LIB.ora_interpolate_to_parallel.argtypes = [C.POINTER(Geom), d, d, p, p, p, p, p]
        _LIB.ora_image_compare.argtypes = [p, p, i, i, p]
        _LIB.ora_convert_polar.argtypes = [C.POINTER(Geom), d, d, p, p, i, i, i, p]
        _LIB.ora_convert_fft_polar.argtypes = [C.POINTER(Geom), d, d, p, p, i, i, i, i, p, p]
        _LIB.ora_add_zeropad_factor.argtypes = [i, i]
        _LIB.ora_ifft_magnitude.argtypes = [p, p, i, i, p]
        _LIB.ora_ifft_magnitude.restype = None
        _LIB.ora_phantom_to_image.argtypes = [C.POINTER(_Phantom), i, i, d, i, p, p, i]
        _LIB.ora_project_image.argtypes = [C.POINTER(Geom), p, i, i, p, i, p, i]
        _LIB.ora_frequency_response.argtypes = [i, d, d, d]
        _LIB.ora_frequency_response.restype = d
        _LIB.ora_spatial_response.argtypes = [i, d, d, d]
        _LIB.ora_spatial_response.restype = d
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def nthreads_default():
    return os.cpu_count() or 1


class Phantom:
    """Phantom in the reference's element-list order (elements prepended)."""

    def __init__(self, name=None, elements=None, filename=None, max_elems=256):
        self._p = _Phantom()
        lib().ora_phantom_init(C.byref(self._p), max_elems)
        self.elements = []   # in insertion order: (type, cx, cy, u, v, rot_deg, atten)
        if name is not None:
            if not lib().ora_phantom_builtin(C.byref(self._p), name.encode()):
                raise ValueError("unknown phantom %s" % name)
        for e in elements or []:
            self.add(*e)
        if filename is not None:
            for e in read_phm(filename):
                self.add(*e)

    def add(self, typ, cx, cy, u, v, rot_deg, atten):
        t = lib().ora_name_to_pelem_type(typ.encode()) if isinstance(typ, str) else typ
        if not lib().ora_phantom_add(C.byref(self._p), t, cx, cy, u, v, rot_deg, atten):
            raise ValueError("bad element %r" % (typ,))
        self.elements.append((typ, cx, cy, u, v, rot_deg, atten))

    @property
    def bounds(self):
        return (self._p.xmin, self._p.xmax, self._p.ymin, self._p.ymax)

    def bboxes(self):
        return [(self._p.e[k].xmin, self._p.e[k].ymin, self._p.e[k].xmax, self._p.e[k].ymax)
                for k in range(self._p.n)]

    def raysum(self, x1, y1, x2, y2):
        return lib().ora_raysum(C.byref(self._p), x1, y1, x2, y2)

    def __del__(self):
        try:
            lib().ora_phantom_free(C.byref(self._p))
        except Exception:
            pass


def read_phm(filename):
    """Phantom file: `type cx cy u v rot atten` per line (libctsim/phantom.cpp:184-213)."""
    out = []
    with open(filename) as f:
        toks = f.read().split()
    for k in range(0, len(toks) - 6, 7):
        t = toks[k:k + 7]
        out.append((t[0],) + tuple(float(x) for x in t[1:]))
    return out


class Scanner:
    def __init__(self, phantom, geometry, ndet, nview, offset_view=0, nsample=1, rotangle=None,
                 fl_ratio=2.0, cd_ratio=2.0, view_ratio=1.0, scan_ratio=1.0):
        if rotangle is None:   # fraction of a circle, phm2pj defaults (tools/phm2pj.cpp:272-277)
            rotangle = 0.5 if geometry == "parallel" else 1.0
        self.phantom = phantom
        self._s = _Scanner()
        ok = lib().ora_scanner_init(C.byref(self._s), C.byref(phantom._p), GEOMETRIES[geometry],
                                    ndet, nview, offset_view, nsample,
                                    rotangle * 6.28318530717958647692, fl_ratio, cd_ratio,
                                    view_ratio, scan_ratio)
        if not ok:
            raise ValueError("scanner creation failed")
        self.offset_view = offset_view

    def __getattr__(self, k):
        return getattr(self._s, k)

    def geom(self):
        s = self._s
        return Geom(s.geometry, s.nDet, s.nView, s.rotInc, s.detInc, s.focalLength,
                    s.sourceDetectorLength, s.viewDiameter, s.fanBeamAngle)

    def collect(self, start=0, count=None, nthreads=None):
        s = self._s
        count = s.nView if count is None else count
        sino = np.zeros((s.nView, s.nDet), np.float64)
        ang = np.zeros(s.nView, np.float64)
        lib().ora_collect_projections(C.byref(s), C.byref(self.phantom._p), start, count,
                                      self.offset_view, start, _ptr(sino), _ptr(ang),
                                      nthreads or nthreads_default())
        return sino, ang


def interpolate_to_parallel(geom, rot_start, det_start, sino, angles):
    """Projections::interpolateToParallel: returns (data [nView, nDet] float32,
    angles, (rotInc, detStart, detInc))."""
    sino = np.ascontiguousarray(sino, np.float32)
    angles = np.ascontiguousarray(angles, np.float64)
    out = np.zeros_like(sino)
    oa = np.zeros(sino.shape[0], np.float64)
    hdr = np.zeros(3, np.float64)
    rc = lib().ora_interpolate_to_parallel(C.byref(geom), rot_start, det_start, _ptr(sino),
                                           _ptr(angles), _ptr(out), _ptr(oa), _ptr(hdr))
    if rc != 0:
        raise ValueError("interpolateToParallel: parallel input")
    return out, oa, tuple(hdr)


def ellipse_gradient(scanner, gsino):
    """FP64 d(sum gsino * sino)/d(cx, cy, u, v, rot_deg, atten) of the scanner's
    phantom's ellipses, in the order they were added ([n, 6])."""
    s = scanner._s
    p = scanner.phantom._p
    g = np.ascontiguousarray(gsino, np.float64)
    out = np.zeros(6 * p.n, np.float64)
    lib().ora_ellipse_gradient(C.byref(s), C.byref(p), _ptr(g), _ptr(out))
    out = out.reshape(p.n, 6)[::-1].copy()   # list order is last added first
    out[:, 4] *= np.pi / 180.0
    return out


def collect_ellipsoids(scanner, ellipsoids, z0, dz, nthreads=None):
    """Helical scan of a 3-D ellipsoid phantom (restatement only): view v sees
    the cross-section at z0 + v dz.  ellipsoids: rows (cx, cy, cz, a, b, c,
    rot_deg, atten)."""
    s = scanner._s
    ell = np.ascontiguousarray(ellipsoids, np.float64).reshape(-1, 8)
    sino = np.zeros((s.nView, s.nDet), np.float64)
    ang = np.zeros(s.nView, np.float64)
    lib().ora_collect_ellipsoids(C.byref(s), _ptr(ell), ell.shape[0], z0, dz, _ptr(sino), _ptr(ang),
                                 nthreads or nthreads_default())
    return sino, ang


class ProcessSignal:
    def __init__(self, filter_name, method, ndet, det_inc, param=-1.0, generation="direct",
                 zeropad=1, interp_factor=1, geometry="parallel", focal_length=0.0, sdl=0.0):
        L = lib()
        fid = L.ora_filter_id(filter_name.encode())
        mid = L.ora_filter_method_id(method.encode())
        gid = L.ora_filter_generation_id(generation.encode())
        self._ps = _ProcSig()
        gi = GEOMETRIES[geometry] if isinstance(geometry, str) else geometry
        if not L.ora_procsig_init(C.byref(self._ps), fid, mid, 1.0 / det_inc, det_inc, ndet, param,
                                  gid, zeropad, interp_factor, gi, focal_length, sdl):
            raise ValueError("ProcessSignal init failed")
        self.ndet = ndet

    @property
    def n_filter_points(self):
        return self._ps.nFilterPoints

    def filter_array(self):
        return np.ctypeslib.as_array(self._ps.filter, (self._ps.nFilterPoints,)).copy()

    def filter(self, sino, nthreads=None):
        sino = np.ascontiguousarray(sino, np.float32)
        out = np.zeros(sino.shape, np.float64)
        lib().ora_filter_views(C.byref(self._ps), _ptr(sino), sino.shape[0], _ptr(out),
                               nthreads or nthreads_default())
        return out

    def __del__(self):
        try:
            lib().ora_procsig_free(C.byref(self._ps))
        except Exception:
            pass


def backproject(geom, filtered, angles, nx, ny, backproj="table", interp="linear", roi=None,
                post_process=True, nthreads=None, start_view=0):
    filtered = np.ascontiguousarray(filtered, np.float64)
    angles = np.ascontiguousarray(angles, np.float64)
    img = np.zeros((nx, ny), np.float64)
    roi_a = None if roi is None else np.ascontiguousarray(roi, np.float64)
    lib().ora_backproject(C.byref(geom), _ptr(filtered), filtered.shape[1], _ptr(angles),
                          start_view, filtered.shape[0], nx, ny,
                          None if roi_a is None else _ptr(roi_a), BACKPROJ[backproj],
                          INTERP[interp], _ptr(img), int(post_process),
                          nthreads or nthreads_default())
    return img


def reconstruct(geom, sino, angles, nx, ny, filter_name="abs_bandlimit", param=-1.0,
                method="convolution", zeropad=1, generation="direct", backproj="idiff",
                interp="linear", nthreads=None):
    L = lib()
    sino = np.ascontiguousarray(sino, np.float32)
    angles = np.ascontiguousarray(angles, np.float64)
    img = np.zeros((nx, ny), np.float64)
    ok = L.ora_reconstruct(C.byref(geom), _ptr(sino), _ptr(angles), nx, ny,
                           L.ora_filter_id(filter_name.encode()), param,
                           L.ora_filter_method_id(method.encode()), zeropad,
                           L.ora_filter_generation_id(generation.encode()), BACKPROJ[backproj],
                           INTERP[interp], _ptr(img), nthreads or nthreads_default())
    if not ok:
        raise ValueError("reconstruct failed")
    return img


def helical180li(geom, sino, interp_view=-1, allow_equilinear=False):
    """Helical180LI; allow_equilinear: the equilinear restatement (no reference
    counterpart) instead of the reference's refusal."""
    sino = np.ascontiguousarray(sino, np.float32)
    out = np.zeros_like(sino)
    ang = np.zeros(sino.shape[0], np.float64)
    n = C.c_int(0)
    rc = lib().ora_helical180li_ex(C.byref(geom), _ptr(sino), sino.shape[0], interp_view,
                                   _ptr(out), _ptr(ang), C.byref(n), int(allow_equilinear))
    if rc != 0:
        raise ValueError("Helical180LI failed: %d" % rc)
    return out[:n.value].copy(), ang[:n.value].copy()


def halfscan_feather(geom, sino, true_gamma=False):
    """HalfScanFeather; true_gamma: the equilinear detector's fan angle (the
    restatement that goes with helical180li(allow_equilinear=True))."""
    data = np.ascontiguousarray(sino, np.float32).copy()
    rc = lib().ora_halfscan_feather_ex(C.byref(geom), _ptr(data), data.shape[0], int(true_gamma))
    if rc != 0:
        raise ValueError("HalfScanFeather failed: %d" % rc)
    return data


def phantom_to_image(phantom, nx, ny, view_ratio=1.0, nsample=1, nthreads=None):
    img = np.zeros((nx, ny), np.float64)
    ext = np.zeros(4, np.float64)
    lib().ora_phantom_to_image(C.byref(phantom._p), nx, ny, view_ratio, nsample, _ptr(img),
                               _ptr(ext), nthreads or nthreads_default())
    return img, ext


def project_image(geom, image, angles, nthreads=None):
    image = np.ascontiguousarray(image, np.float64)
    angles = np.ascontiguousarray(angles, np.float64)
    sino = np.zeros((len(angles), geom.nDet), np.float64)
    lib().ora_project_image(C.byref(geom), _ptr(image), image.shape[0], image.shape[1],
                            _ptr(angles), len(angles), _ptr(sino), nthreads or nthreads_default())
    return sino


def image_compare(a, b):
    """ImageFile::comparativeStatistics of two FP32 images [nx, ny] (column-major
    storage, v[ix][iy]): (d, r, e)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    assert a.shape == b.shape and a.ndim == 2
    out = np.zeros(3, np.float64)
    rc = lib().ora_image_compare(_ptr(a), _ptr(b), a.shape[0], a.shape[1], _ptr(out))
    if rc == 0:
        raise ValueError("comparativeStatistics: empty image")
    return tuple(out)


POLAR_INTERP = {"nearest": 0, "bilinear": 1}


def convert_polar(geom, rot_start, det_start, sino, angles, nx, ny, interp):
    """Projections::convertPolar: FP32 image [nx, ny] (columns >= ny stay zero)."""
    sino = np.ascontiguousarray(sino, np.float32)
    angles = np.ascontiguousarray(angles, np.float64)
    out = np.zeros((nx, ny), np.float32)
    lib().ora_convert_polar(C.byref(geom), rot_start, det_start, _ptr(sino), _ptr(angles), nx, ny,
                            POLAR_INTERP[interp], _ptr(out))
    return out


def convert_fft_polar(geom, rot_start, det_start, sino, angles, nx, ny, interp, zeropad):
    """Projections::convertFFTPolar: (real [nx, ny], imag [nx, ny], transform length)."""
    sino = np.ascontiguousarray(sino, np.float32)
    angles = np.ascontiguousarray(angles, np.float64)
    re = np.zeros((nx, ny), np.float32)
    im = np.zeros((nx, ny), np.float32)
    n = lib().ora_convert_fft_polar(C.byref(geom), rot_start, det_start, _ptr(sino), _ptr(angles),
                                    nx, ny, POLAR_INTERP[interp], zeropad, _ptr(re), _ptr(im))
    return re, im, n


def ifft_magnitude(re, im):
    """ImageFile::ifft, magnitude, shuffleFourierToNaturalOrder of a complex image."""
    re = np.ascontiguousarray(re, np.float32)
    im = np.ascontiguousarray(im, np.float32)
    out = np.zeros_like(re)
    lib().ora_ifft_magnitude(_ptr(re), _ptr(im), re.shape[0], re.shape[1], _ptr(out))
    return out


def reconstruct_fourier(geom, rot_start, det_start, sino, angles, nx, ny, interp, zeropad):
    """The GUI's Fourier reconstruction: convertFFTPolar, ifft, magnitude, shuffle."""
    re, im, _ = convert_fft_polar(geom, rot_start, det_start, sino, angles, nx, ny, interp, zeropad)
    return ifft_magnitude(re, im)
