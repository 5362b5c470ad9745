"""GB300 (sm_103a) implementation of CTSim's simulate-and-reconstruct path.

Python mirror of the reference's C++ interface for this path (the native
library behind it is libctgpu.so, C ABI in include/ctgpu.h):

    Phantom             libctsim/phantom.cpp     (createFromPhantom / addPElem / createFromFile)
    Scanner             libctsim/scanner.cpp     (Scanner ctor, collectProjections)
    Projections         libctsim/projections.cpp (initFromScanner, read, write,
                                                  Helical180LI, HalfScanFeather)
    ImageFile           libctsim/imagefile.cpp   (nx x ny FP32, column-major v[ix][iy])
    Reconstructor       libctsim/reconstruct.cpp (ctor, reconstructAllViews,
                                                  reconstructView, postProcessing)

Host arrays are numpy; the device-resident entry points in ``ctsim_gb300.device``
take torch CUDA tensors (torch provides memory and streams only; the compute is
the library's own kernels).  Constructors raise CtgpuError where the reference
sets fail()/failMessage().
"""
import ctypes as C

import numpy as np

from . import fileio
from ._lib import (CtgpuError, Geometry, Roi, RUN_ACCUMULATE, RUN_POSTPROCESS, check, enc,
                   lib)

GEOMETRY_PARALLEL, GEOMETRY_EQUIANGULAR, GEOMETRY_EQUILINEAR = 0, 1, 2
GEOMETRY_NAMES = ("parallel", "equiangular", "equilinear")
TWOPI = 6.28318530717958647692

__all__ = ["Phantom", "Scanner", "Projections", "ImageFile", "Reconstructor", "CtgpuError",
           "Geometry", "fileio", "sync"]


def sync(stream=None):
    """Wait for `stream` (cudaStream_t as int, or None) and report kernel-side failures."""
    check(lib().ctgpu_sync(C.c_void_p(stream or 0)))


class Phantom:
    """Phantom(name) for a built-in phantom ("herman", "shepp-logan",
    "unit-pulse"), Phantom() for an empty one, Phantom.from_file(path)."""

    def __init__(self, name=None):
        self._h = C.c_void_p()
        if name is None:
            check(lib().ctgpu_phantom_create(C.byref(self._h)))
        else:
            check(lib().ctgpu_phantom_create_builtin(enc(name), C.byref(self._h)))
        self.name = name or ""

    @classmethod
    def from_file(cls, path):
        p = cls()
        check(lib().ctgpu_phantom_read_file(p._h, enc(path)))
        p.name = path
        return p

    def add_element(self, typ, cx, cy, u, v, rot_deg, atten):
        """Phantom::addPElem: rot in degrees."""
        check(lib().ctgpu_phantom_add_element(self._h, enc(typ), cx, cy, u, v, rot_deg, atten))

    addPElem = add_element

    @property
    def bounds(self):
        b = (C.c_double * 4)()
        n = C.c_int()
        check(lib().ctgpu_phantom_bounds(self._h, b, C.byref(n)))
        return tuple(b)

    @property
    def n_elements(self):
        n = C.c_int()
        check(lib().ctgpu_phantom_bounds(self._h, None, C.byref(n)))
        return n.value

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ctgpu_phantom_destroy(self._h)
            self._h = None

    def rasterize(self, nx, ny, view_ratio=1.0, nsample=1):
        """Phantom::convertToImagefile (phm2if) on the device: returns (image
        [nx, ny] float32 CUDA tensor, extent (xmin, xmax, ymin, ymax),
        increment (xinc, yinc))."""
        import torch
        img = torch.zeros((nx, ny), dtype=torch.float32, device="cuda")
        ext = (C.c_double * 4)()
        inc = (C.c_double * 2)()
        check(lib().ctgpu_phantom_rasterize(self._h, nx, ny, float(view_ratio), int(nsample),
                                            C.c_void_p(img.data_ptr()), ext, inc, None))
        sync()
        return img, tuple(ext), tuple(inc)



class Scanner:
    """Scanner(phm, geometry, nDet, nView, offsetView, nSample, rotAngle, focalLengthRatio,
    centerDetectorRatio, viewRatio, scanRatio) -- rotAngle in radians, as the
    reference's constructor takes it (phm2pj passes a fraction of a circle x 2 pi)."""

    def __init__(self, phm, geometry, nDet, nView, offsetView=0, nSample=1, rotAngle=None,
                 focalLengthRatio=2.0, centerDetectorRatio=2.0, viewRatio=1.0, scanRatio=1.0):
        if rotAngle is None:
            rotAngle = (0.5 if geometry == "parallel" else 1.0) * TWOPI
        self._h = C.c_void_p()
        check(lib().ctgpu_scanner_create(phm._h, enc(geometry), nDet, nView, offsetView, nSample,
                                         rotAngle, focalLengthRatio, centerDetectorRatio,
                                         viewRatio, scanRatio, C.byref(self._h)))
        self.phantom = phm
        self.offsetView = offsetView
        self.nSample = nSample

    def geometry(self):
        g = Geometry()
        check(lib().ctgpu_scanner_geometry(self._h, C.byref(g)))
        return g

    @property
    def nDet(self):
        return self.geometry().n_det

    @property
    def nView(self):
        return self.geometry().n_view

    @property
    def detInc(self):
        return self.geometry().det_inc

    def collectProjections(self, proj, phm=None, iStartView=0, iNumViews=None, iOffsetView=None,
                           iStorageOffset=None):
        """Scanner::collectProjections into a host Projections object."""
        phm = phm or self.phantom
        nv = proj.nView - iStartView if iNumViews is None else iNumViews
        off = self.offsetView if iOffsetView is None else iOffsetView
        store = iStartView if iStorageOffset is None else iStorageOffset
        data = np.ascontiguousarray(proj.data, np.float32)
        ang = np.ascontiguousarray(proj.angles, np.float64)
        check(lib().ctgpu_collect_projections_host(
            self._h, phm._h, iStartView, nv, off, store, data.ctypes.data_as(C.c_void_p),
            ang.ctypes.data_as(C.c_void_p)))
        proj.data, proj.angles = data, ang
        return proj

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ctgpu_scanner_destroy(self._h)
            self._h = None


class Projections(fileio.ProjectionFile):
    """Sinogram container = the .pj file contents (host numpy arrays)."""

    @classmethod
    def from_scanner(cls, sc):
        g = sc.geometry()
        return cls(g.n_view, g.n_det, g.geometry, 0.0, g.rot_start, g.rot_inc, g.det_start,
                   g.det_inc, g.view_diameter, g.focal_length, g.source_detector_length,
                   g.fan_beam_angle, angles=np.zeros(g.n_view),
                   data=np.zeros((g.n_view, g.n_det), np.float32))

    @classmethod
    def read(cls, path):
        pj = fileio.read_pj(path)
        pj.__class__ = cls
        return pj

    def write(self, path):
        fileio.write_pj(path, self)

    def ctgpu_geometry(self):
        """The header fields as the C ABI's ctgpu_geometry."""
        return Geometry(int(self.geometry), self.nDet, self.nView, 0, self.rotStart, self.rotInc,
                        self.detStart, self.detInc, self.viewDiameter, self.focalLength,
                        self.sourceDetectorLength, self.fanBeamAngle)

    def helical180li(self, interp_view=-1):
        """Projections::Helical180LI (+ nothing else); returns self, updated in place."""
        from . import device
        out, ang = device.helical180li_host(self.ctgpu_geometry(), self.data, interp_view)
        self.data, self.angles, self.nView = out, ang, out.shape[0]
        return self

    Helical180LI = helical180li

    def halfscan_feather(self):
        from . import device
        self.data = device.halfscan_feather_host(self.ctgpu_geometry(), self.data)
        return self

    HalfScanFeather = halfscan_feather

    def interpolate_to_parallel(self):
        """Projections::interpolateToParallel: a new parallel-beam Projections
        (self for parallel data)."""
        from . import device
        import copy
        if int(self.geometry) == 0:
            return self
        out, g, ang = device.interpolate_to_parallel(self.ctgpu_geometry(),
                                                     device._to_device(self.data), self.angles)
        sync()
        q = copy.copy(self)
        q.geometry, q.rotStart, q.rotInc = 0, g.rot_start, g.rot_inc
        q.detStart, q.detInc = g.det_start, g.det_inc
        q.angles = ang
        q.data = out[:, :self.nDet].cpu().numpy()
        q.calcTime = 0.0
        q.remark = (self.remark or "") + "; Interpolate to Parallel"
        return q

    interpolateToParallel = interpolate_to_parallel


class ImageFile(fileio.ImageFileData):
    """nx x ny FP32 image, column-major v[ix][iy] (F32Image)."""

    def __init__(self, nx, ny):
        super().__init__(nx, ny, 7, 4, 1, data=np.zeros((nx, ny), np.float32))

    def getArray(self):
        return self.data

    def write(self, path, labels=()):
        fileio.write_if(path, self, labels)


class Reconstructor:
    """Reconstructor(proj, im, filterName, filterParam, filterMethodName, zeropad,
    filterGenerationName, interpName, interpFactor, backprojName, trace=0, roi=None)"""

    def __init__(self, proj, im, filterName="abs_bandlimit", filterParam=-1.0,
                 filterMethodName="convolution", zeropad=1, filterGenerationName="direct",
                 interpName="linear", interpFactor=1, backprojName="idiff", trace=0, roi=None):
        self.proj, self.im = proj, im
        g = proj.ctgpu_geometry() if hasattr(proj, "ctgpu_geometry") else proj
        self._g = g
        r = None if roi is None else Roi(*roi)
        self._h = C.c_void_p()
        check(lib().ctgpu_recon_create(C.byref(g), im.nx, im.ny, enc(filterName), filterParam,
                                       enc(filterMethodName), zeropad, enc(filterGenerationName),
                                       enc(interpName), interpFactor, enc(backprojName),
                                       C.byref(r) if r else None, C.byref(self._h)))
        ext = (C.c_double * 4)()
        inc = (C.c_double * 2)()
        check(lib().ctgpu_recon_image_axes(self._h, ext, inc))
        im.extent, im.extent_known = tuple(ext), 1
        im.increment, im.increment_known = tuple(inc), 1

    def reconstructAllViews(self):
        data = np.ascontiguousarray(self.proj.data, np.float32)
        ang = np.ascontiguousarray(self.proj.angles, np.float64)
        out = np.zeros((self.im.nx, self.im.ny), np.float32)
        check(lib().ctgpu_recon_run_host(self._h, data.ctypes.data_as(C.c_void_p),
                                         ang.ctypes.data_as(C.c_void_p),
                                         out.ctypes.data_as(C.c_void_p)))
        self.im.data = out
        return self.im

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ctgpu_recon_destroy(self._h)
            self._h = None
