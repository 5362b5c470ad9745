"""Readers and writers for CTSim's two binary file formats, little-endian.

``.pj`` projection files: header then one record per view
(libctsim/projections.cpp:485-546 header, :860-889 per-view record):

    u16 headerSize, u16 signature 'PJ', u32 nView, u32 nDet, u32 geometry,
    f64 calcTime, rotStart, rotInc, detStart, detInc, viewDiameter,
        focalLength, sourceDetectorLength, fanBeamAngle,
    u16 year, month, day, hour, minute, second, u16 remarkLength, remark bytes
    per view: f64 viewAngle, u32 nDet, nDet x f32

``.if`` image files (libctsim/array2dfile.cpp:443-478 header, :481-520 data,
labels after the data): column-major pixels, ``v[ix][iy]``.
"""
import struct
from dataclasses import dataclass, field

import numpy as np

PJ_SIGNATURE = ord("P") * 256 + ord("J")
IF_SIGNATURE = ord("I") * 256 + ord("F")
GEOMETRY_NAMES = ["parallel", "equiangular", "equilinear", "linogram"]

_PJ_HEAD = struct.Struct("<HHIII9d7H")


@dataclass
class ProjectionFile:
    nView: int
    nDet: int
    geometry: int
    calcTime: float = 0.0
    rotStart: float = 0.0
    rotInc: float = 0.0
    detStart: float = 0.0
    detInc: float = 0.0
    viewDiameter: float = 0.0
    focalLength: float = 0.0
    sourceDetectorLength: float = 0.0
    fanBeamAngle: float = 0.0
    date: tuple = (0, 0, 0, 0, 0, 0)
    remark: str = ""
    angles: np.ndarray = None     # (nView,) float64
    data: np.ndarray = None       # (nView, nDet) float32

    @property
    def phmLen(self):
        """include/projections.h:165"""
        return self.viewDiameter / 1.414213562373095049


def read_pj(path):
    with open(path, "rb") as f:
        buf = f.read()
    h = _PJ_HEAD.unpack_from(buf, 0)
    hsize, sig, nview, ndet, geom = h[:5]
    if sig != PJ_SIGNATURE:
        raise ValueError("%s: not a projection file" % path)
    dbl = h[5:14]
    date = h[14:20]
    rlen = h[20]
    remark = buf[_PJ_HEAD.size:_PJ_HEAD.size + rlen].decode("latin-1")
    if _PJ_HEAD.size + rlen != hsize:
        raise ValueError("%s: header size mismatch" % path)
    rec = np.dtype([("angle", "<f8"), ("ndet", "<u4"), ("det", "<f4", (ndet,))])
    views = np.frombuffer(buf, dtype=rec, count=nview, offset=hsize)
    return ProjectionFile(nview, ndet, geom, *dbl, date=tuple(date), remark=remark,
                          angles=views["angle"].astype(np.float64),
                          data=np.ascontiguousarray(views["det"], dtype=np.float32))


def write_pj(path, pj):
    remark = pj.remark.encode("latin-1")
    hsize = _PJ_HEAD.size + len(remark)
    head = _PJ_HEAD.pack(hsize, PJ_SIGNATURE, pj.nView, pj.nDet, pj.geometry, pj.calcTime,
                         pj.rotStart, pj.rotInc, pj.detStart, pj.detInc, pj.viewDiameter,
                         pj.focalLength, pj.sourceDetectorLength, pj.fanBeamAngle,
                         *pj.date, len(remark))
    rec = np.dtype([("angle", "<f8"), ("ndet", "<u4"), ("det", "<f4", (pj.nDet,))])
    views = np.zeros(pj.nView, rec)
    views["angle"] = pj.angles
    views["ndet"] = pj.nDet
    views["det"] = pj.data
    with open(path, "wb") as f:
        f.write(head + remark)
        f.write(views.tobytes())


_IF_HEAD = struct.Struct("<HHHHHIIHH2dH6d")


@dataclass
class ImageFileData:
    nx: int
    ny: int
    pixel_format: int
    pixel_size: int
    data_type: int
    increment: tuple = (0.0, 0.0)
    increment_known: int = 0
    extent: tuple = (0.0, 0.0, 0.0, 0.0)
    extent_known: int = 0
    offsetPV: float = 0.0
    scalePV: float = 1.0
    labels: list = field(default_factory=list)
    data: np.ndarray = None    # (nx, ny) real part, column-major storage order
    imag: np.ndarray = None


def read_if(path):
    with open(path, "rb") as f:
        buf = f.read()
    h = _IF_HEAD.unpack_from(buf, 0)
    (hsize, sig, pfmt, psize, nlabels, nx, ny, dtype_, inc_known, incx, incy, ext_known,
     xmin, xmax, ymin, ymax, offpv, scalepv) = h
    if sig != IF_SIGNATURE:
        raise ValueError("%s: not an image file" % path)
    dt = {4: "<f4", 8: "<f8"}[psize]
    n = nx * ny
    data = np.frombuffer(buf, dt, count=n, offset=hsize).reshape(nx, ny).copy()
    off = hsize + n * psize
    imag = None
    if dtype_ == 2:   # DATA_TYPE_COMPLEX (include/array2dfile.h:130-132)
        imag = np.frombuffer(buf, dt, count=n, offset=off).reshape(nx, ny).copy()
        off += n * psize
    labels = []
    for _ in range(nlabels):
        ltype, y, mo, d, hh, mi, s = struct.unpack_from("<7H", buf, off)
        ct, = struct.unpack_from("<d", buf, off + 14)
        slen, = struct.unpack_from("<H", buf, off + 22)
        txt = buf[off + 24:off + 24 + slen].decode("latin-1")
        labels.append((ltype, txt, ct, (y, mo, d, hh, mi, s)))
        off += 24 + slen
    return ImageFileData(nx, ny, pfmt, psize, dtype_, (incx, incy), inc_known,
                         (xmin, xmax, ymin, ymax), ext_known, offpv, scalepv, labels, data, imag)


def write_if(path, img, labels=()):
    """Write a real FP32 (PIXEL_FLOAT32 = 7) or FP64 (PIXEL_FLOAT64 = 8) image
    (include/array2dfile.h:118-132)."""
    data = np.asarray(img.data)
    psize = data.dtype.itemsize
    pfmt = 7 if psize == 4 else 8
    head = _IF_HEAD.pack(_IF_HEAD.size, IF_SIGNATURE, pfmt, psize, len(labels), img.nx, img.ny,
                         1, img.increment_known, img.increment[0], img.increment[1],
                         img.extent_known, *img.extent, img.offsetPV, img.scalePV)
    out = [head, np.ascontiguousarray(data).astype(data.dtype.newbyteorder("<")).tobytes()]
    for (ltype, txt, ct, date) in labels:
        b = txt.encode("latin-1")
        out.append(struct.pack("<7HdH", ltype, *date, ct, len(b)) + b)
    with open(path, "wb") as f:
        f.write(b"".join(out))
