"""Device-resident entry points on torch CUDA tensors.

torch supplies device memory and the current stream; every operation is a
call through the C ABI into libctgpu.so's kernels.  Sinograms are
[views, pitch] float32 with pitch a multiple of 4 (``alloc_sinogram``);
images are [nx, ny] float32 (column-major v[ix][iy], as CTSim's ImageFile).
"""
import ctypes as C

import numpy as np

from ._lib import (Geometry, IfInfo, IfLabel, PjInfo, Roi, RUN_ACCUMULATE, RUN_POSTPROCESS,
                   check, enc, lib)


def _torch():
    import torch
    return torch


def stream_handle(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _ptr(t):
    if not t.is_cuda or not t.is_contiguous() or t.dtype != _torch().float32:
        raise ValueError("expected a contiguous float32 CUDA tensor")
    return C.c_void_p(t.data_ptr())


def _ptrd(t):
    if not t.is_cuda or not t.is_contiguous() or t.dtype != _torch().float64:
        raise ValueError("expected a contiguous float64 CUDA tensor")
    return C.c_void_p(t.data_ptr())


def pitch_for(n_det):
    return (n_det + 3) & ~3


def alloc_sinogram(n_view, n_det, device="cuda"):
    torch = _torch()
    return torch.zeros((n_view, pitch_for(n_det)), dtype=torch.float32, device=device)


def raysums(scanner, phantom, sino, start_view=0, n_views=None, offset_view=None,
            storage_offset=None, stream=None):
    """Scanner::collectProjections into a device sinogram; returns the view angles."""
    g = scanner.geometry()
    nv = g.n_view - start_view if n_views is None else n_views
    off = scanner.offsetView if offset_view is None else offset_view
    store = start_view if storage_offset is None else storage_offset
    ang = np.zeros(max(g.n_view, store + nv), np.float64)
    check(lib().ctgpu_collect_projections(scanner._h, phantom._h, start_view, nv, off, store,
                                          _ptr(sino), sino.shape[1],
                                          ang.ctypes.data_as(C.c_void_p), stream_handle(stream)))
    return ang


def raysums_batch(scanner, phantoms, sinos, stream=None):
    """collectProjections of every phantom with one scanner, one launch:
    sinos [B, n_view, pitch] device tensor; returns the view angles."""
    g = scanner.geometry()
    if sinos.shape[0] != len(phantoms) or sinos.shape[1] < g.n_view or not sinos.is_contiguous():
        raise ValueError("sinos must be a contiguous [B, n_view, pitch] tensor")
    hs = (C.c_void_p * len(phantoms))(*[p._h.value if hasattr(p._h, "value") else p._h
                                        for p in phantoms])
    ang = np.zeros(g.n_view, np.float64)
    check(lib().ctgpu_collect_projections_batch(scanner._h, hs, len(phantoms), _ptr(sinos),
                                                sinos.shape[2], sinos.stride(0),
                                                ang.ctypes.data_as(C.c_void_p),
                                                stream_handle(stream)))
    return ang


def raysums_multi(scanners, phantoms, sinos, stream=None):
    """collectProjections of many (scanner, phantom) problems of different
    geometry, detectors and views in one ray launch
    (ctgpu_collect_projections_multi): sinos[k] a device [n_view_k, pitch_k]
    tensor; returns the view angles of every problem."""
    n = len(scanners)
    if len(phantoms) != n or len(sinos) != n:
        raise ValueError("one phantom and one sinogram per scanner")
    geos = [sc.geometry() for sc in scanners]
    for g, t in zip(geos, sinos):
        if t.shape[0] < g.n_view or t.shape[1] < g.n_det:
            raise ValueError("sinogram smaller than its scan")
    angs = [np.zeros(g.n_view, np.float64) for g in geos]

    def hv(x):
        return x.value if hasattr(x, "value") else x
    sh = (C.c_void_p * n)(*[hv(sc._h) for sc in scanners])
    ph = (C.c_void_p * n)(*[hv(p._h) for p in phantoms])
    sp = (C.c_void_p * n)(*[_ptr(t).value for t in sinos])
    pitches = (C.c_int * n)(*[t.shape[1] for t in sinos])
    ap = (C.c_void_p * n)(*[a.ctypes.data for a in angs])
    check(lib().ctgpu_collect_projections_multi(sh, ph, n, sp, pitches, ap,
                                                stream_handle(stream)))
    return angs


class ReconPlan:
    """A Reconstructor for device tensors (ctgpu_recon)."""

    def __init__(self, geometry, nx, ny, filter_name="abs_bandlimit", filter_param=-1.0,
                 filter_method="convolution", zeropad=1, filter_generation="direct",
                 interp="linear", interp_factor=1, backproj="idiff", roi=None):
        self.geometry = geometry
        self.nx, self.ny = nx, ny
        r = None if roi is None else Roi(*roi)
        self._h = C.c_void_p()
        check(lib().ctgpu_recon_create(C.byref(geometry), nx, ny, enc(filter_name), filter_param,
                                       enc(filter_method), zeropad, enc(filter_generation),
                                       enc(interp), interp_factor, enc(backproj),
                                       C.byref(r) if r else None, C.byref(self._h)))

    def axes(self):
        ext = (C.c_double * 4)()
        inc = (C.c_double * 2)()
        check(lib().ctgpu_recon_image_axes(self._h, ext, inc))
        return tuple(ext), tuple(inc)

    def filter(self, sino, out, n_views=None, stream=None):
        nv = sino.shape[0] if n_views is None else n_views
        check(lib().ctgpu_recon_filter(self._h, _ptr(sino), sino.shape[1], nv, _ptr(out),
                                       out.shape[1], stream_handle(stream)))
        return out

    def backproject(self, filtered, angles, image, accumulate=False, stream=None):
        ang = np.ascontiguousarray(angles, np.float64)
        check(lib().ctgpu_recon_backproject(self._h, _ptr(filtered), filtered.shape[1],
                                            ang.ctypes.data_as(C.c_void_p), len(ang),
                                            _ptr(image), int(accumulate), stream_handle(stream)))
        return image

    def postprocess(self, image, stream=None):
        check(lib().ctgpu_recon_postprocess(self._h, _ptr(image), stream_handle(stream)))
        return image

    def run(self, sino, angles, image, start_view=0, n_views=-1, postprocess=True,
            accumulate=False, stream=None):
        ang = np.ascontiguousarray(angles, np.float64)
        flags = (RUN_POSTPROCESS if postprocess else 0) | (RUN_ACCUMULATE if accumulate else 0)
        check(lib().ctgpu_recon_run(self._h, _ptr(sino), sino.shape[1],
                                    ang.ctypes.data_as(C.c_void_p), start_view, n_views,
                                    _ptr(image), flags, stream_handle(stream)))
        return image

    def run_batch(self, sinos, angles, images, postprocess=True, stream=None):
        """sinos [B, n_view, pitch], images [B, nx, ny]: one filter launch per slice,
        one backprojection launch for the batch."""
        if not (sinos.is_contiguous() and images.is_contiguous()):
            raise ValueError("batched tensors must be contiguous")
        ang = np.ascontiguousarray(angles, np.float64)
        check(lib().ctgpu_recon_run_batch(
            self._h, sinos.shape[0], C.c_void_p(sinos.data_ptr()), sinos.shape[2],
            sinos.stride(0), ang.ctypes.data_as(C.c_void_p), C.c_void_p(images.data_ptr()),
            images.stride(0), RUN_POSTPROCESS if postprocess else 0, stream_handle(stream)))
        return images

    def backproject_batch(self, filtered, angles, images, postprocess=True, stream=None):
        """filtered [B, n_view, pitch] -> images [B, nx, ny] in one launch."""
        ang = np.ascontiguousarray(angles, np.float64)
        check(lib().ctgpu_recon_backproject_batch(
            self._h, filtered.shape[0], C.c_void_p(filtered.data_ptr()), filtered.shape[2],
            filtered.stride(0), ang.ctypes.data_as(C.c_void_p), len(ang),
            C.c_void_p(images.data_ptr()), images.stride(0),
            RUN_POSTPROCESS if postprocess else 0, stream_handle(stream)))
        return images

    def run_host(self, sino, angles):
        """reconstructAllViews with host numpy buffers (copies inside the call)."""
        s = np.ascontiguousarray(sino, np.float32)
        a = np.ascontiguousarray(angles, np.float64)
        out = np.zeros((self.nx, self.ny), np.float32)
        check(lib().ctgpu_recon_run_host(self._h, s.ctypes.data_as(C.c_void_p),
                                         a.ctypes.data_as(C.c_void_p),
                                         out.ctypes.data_as(C.c_void_p)))
        return out

    def run_batch_host(self, sinos, angles, out=None, postprocess=True):
        """run_batch with host buffers: sinos [B, n_view, n_det] (numpy array or
        CPU tensor, ideally page-locked), images returned in `out` [B, nx, ny]
        (allocated as numpy if None).  Copies overlap the reconstruction."""
        def host_ptr(x, dtype):
            if hasattr(x, "data_ptr"):
                if x.is_cuda or not x.is_contiguous():
                    raise ValueError("host buffers must be contiguous CPU tensors")
                return C.c_void_p(x.data_ptr())
            if x.dtype != dtype or not x.flags.c_contiguous:
                raise ValueError("host buffers must be contiguous %s arrays" % np.dtype(dtype))
            return x.ctypes.data_as(C.c_void_p)
        B = sinos.shape[0]
        if tuple(sinos.shape[1:]) != (self.geometry.n_view, self.geometry.n_det):
            raise ValueError("sinos must be [B, n_view, n_det]")
        if out is None:
            out = np.zeros((B, self.nx, self.ny), np.float32)
        if tuple(out.shape) != (B, self.nx, self.ny):
            raise ValueError("out must be [B, nx, ny]")
        ang = np.ascontiguousarray(angles, np.float64)
        check(lib().ctgpu_recon_run_batch_host(self._h, B, host_ptr(sinos, np.float32),
                                               ang.ctypes.data_as(C.c_void_p),
                                               host_ptr(out, np.float32),
                                               RUN_POSTPROCESS if postprocess else 0))
        return out

    def host_chunks(self, n_batch):
        """the chunk sizes run_batch_host uses for n_batch slices on this GPU"""
        sizes = (C.c_int * 64)()
        n = lib().ctgpu_recon_host_chunks(self._h, int(n_batch), C.cast(sizes, C.c_void_p), 64)
        if n < 0:
            check(n)
        if n > 64:
            sizes = (C.c_int * n)()
            n = lib().ctgpu_recon_host_chunks(self._h, int(n_batch), C.cast(sizes, C.c_void_p), n)
        return list(sizes[:n])

    def set_host_chunks(self, sizes=()):
        """fix run_batch_host's chunk sizes (used in turn); () restores the planned ones"""
        arr = (C.c_int * max(len(sizes), 1))(*[int(x) for x in sizes])
        check(lib().ctgpu_recon_set_host_chunks(self._h, C.cast(arr, C.c_void_p), len(sizes)))

    def project(self, image, angles, out, scale=1.0, stream=None):
        ang = np.ascontiguousarray(angles, np.float64)
        check(lib().ctgpu_recon_project(self._h, _ptr(image), ang.ctypes.data_as(C.c_void_p),
                                        len(ang), _ptr(out), out.shape[1], float(scale),
                                        stream_handle(stream)))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ctgpu_recon_destroy(self._h)
            self._h = None


class BatchPlan:
    """Many reconstructions of uneven sizes, one persistent backprojection
    launch (ctgpu_batch).  `problems`: sequence of dicts with keys geometry,
    nx, ny, sino (device [n_view, pitch] tensor), angles, image (device
    [nx, ny] tensor) and optionally filter_name, filter_param, filter_method,
    zeropad, filter_generation, interp, backproj.  The tensors must outlive
    the plan; run() reads the sinograms and writes the images."""

    def __init__(self, problems, autotune=True, graph=True):
        from ._lib import BatchProblem, BATCH_AUTOTUNE, BATCH_GRAPH
        arr = (BatchProblem * len(problems))()
        self._keep = []
        for i, q in enumerate(problems):
            ang = np.ascontiguousarray(q["angles"], np.float64)
            names = [enc(q.get(k, d)) for k, d in (("filter_name", "abs_bandlimit"),
                                                   ("filter_method", "convolution"),
                                                   ("filter_generation", "direct"),
                                                   ("interp", "linear"), ("backproj", "table"))]
            self._keep += [ang] + names + [q["sino"], q["image"]]
            g = q["geometry"]
            arr[i] = BatchProblem(g, q["nx"], q["ny"], names[0], float(q.get("filter_param", -1.0)),
                                  names[1], int(q.get("zeropad", 1)), names[2], names[3], names[4],
                                  q["sino"].data_ptr(), q["sino"].shape[1],
                                  ang.ctypes.data, q["image"].data_ptr())
        self._h = C.c_void_p()
        flags = (BATCH_AUTOTUNE if autotune else 0) | (BATCH_GRAPH if graph else 0)
        check(lib().ctgpu_batch_create(arr, len(problems), flags, C.byref(self._h)))

    def run(self, stream=None):
        check(lib().ctgpu_batch_run(self._h, stream_handle(stream)))

    def shape(self):
        a, b = C.c_int(), C.c_int()
        check(lib().ctgpu_batch_shape(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ctgpu_batch_destroy(self._h)
            self._h = None


def helical180li(geometry, sino, interp_view=-1, stream=None, equilinear=False):
    """Projections::Helical180LI on a device sinogram; returns (out, angles).
    equilinear=True: the equilinear restatement (true detector fan angles),
    which the reference does not have."""
    torch = _torch()
    n = C.c_int()
    size = lib().ctgpu_helical180li_equilinear_size if equilinear else lib().ctgpu_helical180li_size
    run = lib().ctgpu_helical180li_equilinear if equilinear else lib().ctgpu_helical180li
    check(size(C.byref(geometry), sino.shape[0], interp_view, C.byref(n)))
    out = torch.empty((n.value, sino.shape[1]), dtype=torch.float32, device=sino.device)
    ang = np.zeros(n.value, np.float64)
    check(run(C.byref(geometry), _ptr(sino), sino.shape[0], interp_view, _ptr(out),
              sino.shape[1], ang.ctypes.data_as(C.c_void_p), C.byref(n), stream_handle(stream)))
    return out, ang


def halfscan_feather(geometry, sino, stream=None, equilinear=False):
    """Projections::HalfScanFeather, in place on a device sinogram (equilinear:
    the restatement with true detector fan angles)."""
    fn = lib().ctgpu_halfscan_feather_equilinear if equilinear else lib().ctgpu_halfscan_feather
    check(fn(C.byref(geometry), _ptr(sino), sino.shape[0], sino.shape[1], stream_handle(stream)))
    return sino


def interpolate_to_parallel(geometry, sino, angles, stream=None):
    """Projections::interpolateToParallel of a device fan-beam sinogram:
    returns (parallel sinogram, its Geometry, its view angles)."""
    torch = _torch()
    ang = np.ascontiguousarray(angles, np.float64)
    out = torch.zeros((geometry.n_view, pitch_for(geometry.n_det)), dtype=torch.float32,
                      device=sino.device)
    g2 = Geometry()
    oa = np.zeros(geometry.n_view, np.float64)
    check(lib().ctgpu_interpolate_to_parallel(C.byref(geometry), _ptr(sino), sino.shape[1],
                                              ang.ctypes.data_as(C.c_void_p), _ptr(out),
                                              out.shape[1], C.byref(g2),
                                              oa.ctypes.data_as(C.c_void_p), stream_handle(stream)))
    return out, g2, oa


class HelicalPlan:
    """Helical180LI (+ HalfScanFeather) at many interpolation views of one data
    set (ctgpu_helical_plan): tables once, all slices in one launch."""

    def __init__(self, geometry, n_view_in, equilinear=False, feather=True):
        flags = (1 if equilinear else 0) | (2 if feather else 0)
        self._h = C.c_void_p()
        check(lib().ctgpu_helical_plan_create(C.byref(geometry), n_view_in, flags,
                                              C.byref(self._h)))
        n = C.c_int()
        check(lib().ctgpu_helical_plan_views(self._h, C.byref(n)))
        self.n_view_out = n.value

    def run(self, sino, interp_views, out=None, stream=None):
        """sino [n_view_in, pitch] device tensor -> out [n_slices, n_view_out,
        pitch]; returns (out, angles [n_slices, n_view_out])."""
        torch = _torch()
        iv = np.ascontiguousarray(interp_views, np.int32)
        if out is None:
            out = torch.empty((len(iv), self.n_view_out, sino.shape[1]), dtype=torch.float32,
                              device=sino.device)
        ang = np.zeros((len(iv), self.n_view_out), np.float64)
        check(lib().ctgpu_helical_plan_run(self._h, _ptr(sino), sino.shape[1],
                                           iv.ctypes.data_as(C.c_void_p), len(iv), _ptr(out),
                                           out.shape[2], out.stride(0),
                                           ang.ctypes.data_as(C.c_void_p), stream_handle(stream)))
        return out, ang

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ctgpu_helical_plan_destroy(self._h)
            self._h = None


def raysums_ellipsoids(scanner, ellipsoids, z0, dz, sino, stream=None):
    """Helical scan of a 3-D ellipsoid phantom (rows cx, cy, cz, a, b, c,
    rot_deg, atten): view v sees the cross-section at z0 + v dz.  Returns the
    view angles."""
    g = scanner.geometry()
    ell = np.ascontiguousarray(ellipsoids, np.float64).reshape(-1, 8)
    ang = np.zeros(g.n_view, np.float64)
    check(lib().ctgpu_collect_projections_ellipsoids(
        scanner._h, ell.ctypes.data_as(C.c_void_p), ell.shape[0], float(z0), float(dz),
        _ptr(sino), sino.shape[1], ang.ctypes.data_as(C.c_void_p), stream_handle(stream)))
    return ang


def _to_device(a):
    torch = _torch()
    a = np.ascontiguousarray(a, np.float32)
    t = torch.zeros((a.shape[0], pitch_for(a.shape[1])), dtype=torch.float32, device="cuda")
    t[:, :a.shape[1]] = torch.from_numpy(a).cuda()
    return t


def helical180li_host(geometry, data, interp_view=-1):
    g = Geometry.from_buffer_copy(geometry)
    g.n_view = data.shape[0]
    out, ang = helical180li(g, _to_device(data), interp_view)
    from . import sync
    sync()
    return out[:, :data.shape[1]].cpu().numpy(), ang


def halfscan_feather_host(geometry, data):
    g = Geometry.from_buffer_copy(geometry)
    g.n_view = data.shape[0]
    t = _to_device(data)
    halfscan_feather(g, t)
    from . import sync
    sync()
    return t[:, :data.shape[1]].cpu().numpy()


# ---------------------------------------------------------------- file I/O --
def read_pj_header(path):
    """ctgpu_pj_read_header: (PjInfo, remark)."""
    info = PjInfo()
    buf = C.create_string_buffer(65536)
    check(lib().ctgpu_pj_read_header(enc(str(path)), C.byref(info), buf, len(buf)))
    return info, buf.value.decode("latin-1")


def read_pj(path, device="cuda", stream=None):
    """A .pj file straight into device memory (ctgpu_pj_read_device): returns
    (PjInfo, remark, sino [n_view, pitch] FP32 tensor, angles [n_view] FP64
    tensor, views read)."""
    torch = _torch()
    info, remark = read_pj_header(path)
    g = info.geometry
    sino = torch.empty((g.n_view, pitch_for(g.n_det)), dtype=torch.float32, device=device)
    ang = torch.empty((g.n_view,), dtype=torch.float64, device=device)
    n = C.c_int()
    check(lib().ctgpu_pj_read_device(enc(str(path)), _ptr(sino), sino.shape[1], _ptrd(ang),
                                     C.byref(n), stream_handle(stream)))
    return info, remark, sino, ang, n.value


def write_pj(path, info, remark, sino, angles, stream=None):
    """ctgpu_pj_write_device: sino [n_view, pitch] and angles (FP64) on the device."""
    check(lib().ctgpu_pj_write_device(enc(str(path)), C.byref(info), enc(remark or ""),
                                      _ptr(sino), sino.shape[1], _ptrd(angles),
                                      stream_handle(stream)))


def pj_pack(sino, n_det, angles, out=None, stream=None):
    """.pj view records of a device sinogram, device to device (ctgpu_pj_pack):
    an int32 tensor of n_view * (3 + n_det) words (the bytes of the file after
    its header)."""
    torch = _torch()
    nv = sino.shape[0]
    if out is None:
        out = torch.empty(nv * (3 + n_det), dtype=torch.int32, device=sino.device)
    check(lib().ctgpu_pj_pack(_ptr(sino), sino.shape[1], _ptrd(angles), nv, n_det,
                              C.c_void_p(out.data_ptr()), stream_handle(stream)))
    return out


def pj_unpack(records, n_view, n_det, sino=None, angles=None, stream=None):
    """Inverse of pj_pack (ctgpu_pj_unpack): returns (sino [n_view, pitch],
    angles, records whose detector count differs from n_det, first such view)."""
    torch = _torch()
    dev = records.device
    if sino is None:
        sino = torch.empty((n_view, pitch_for(n_det)), dtype=torch.float32, device=dev)
    if angles is None:
        angles = torch.empty((n_view,), dtype=torch.float64, device=dev)
    status = torch.tensor([0, -1], dtype=torch.int32, device=dev)
    check(lib().ctgpu_pj_unpack(C.c_void_p(records.data_ptr()), n_view, n_det, _ptr(sino),
                                sino.shape[1], _ptrd(angles), C.c_void_p(status.data_ptr()),
                                stream_handle(stream)))
    st = status.cpu().numpy().view(np.uint32)
    return sino, angles, int(st[0]), int(st[1])


def read_if_header(path):
    info = IfInfo()
    check(lib().ctgpu_if_read_header(enc(str(path)), C.byref(info)))
    return info


def read_if_labels(path):
    """[(type, text, calc_time, date)] of an .if file."""
    info = read_if_header(path)
    n = info.n_labels
    labels = (IfLabel * max(n, 1))()
    text = C.create_string_buffer(n * 65536 + 1)
    got = C.c_int()
    check(lib().ctgpu_if_read_labels(enc(str(path)), labels, n, text, len(text), C.byref(got)))
    return [(l.type, (l.text or b"").decode("latin-1"), l.calc_time, tuple(l.date))
            for l in labels[:got.value]]


def read_if(path, device="cuda", stream=None):
    """An .if file's real pixels into a device FP32 tensor [nx, ny]
    (ctgpu_if_read_device): returns (IfInfo, image)."""
    torch = _torch()
    info = read_if_header(path)
    im = torch.empty((info.nx, info.ny), dtype=torch.float32, device=device)
    check(lib().ctgpu_if_read_device(enc(str(path)), _ptr(im), stream_handle(stream)))
    return info, im


def write_if(path, image, info=None, labels=(), stream=None):
    """ctgpu_if_write_device: image [nx, ny] FP32 on the device; labels as
    (type, text, calc_time[, date])."""
    if info is None:
        info = IfInfo()
        info.scale_pv = 1.0
    info.nx, info.ny = image.shape
    arr = (IfLabel * max(len(labels), 1))()
    keep = []
    for k, l in enumerate(labels):
        b = l[1].encode("latin-1")
        keep.append(b)
        arr[k].type = l[0]
        arr[k].text = b
        arr[k].text_length = len(b)
        arr[k].calc_time = l[2]
        if len(l) > 3:
            arr[k].date[:] = list(l[3])
    check(lib().ctgpu_if_write_device(enc(str(path)), C.byref(info), arr, len(labels),
                                      _ptr(image), stream_handle(stream)))


def sino_to_image(sino, n_det, out=None, stream=None):
    """pj2if: image [n_det, n_view] with v[ix][iy] = sino[n_view - 1 - iy][ix]."""
    torch = _torch()
    nv = sino.shape[0]
    if out is None:
        out = torch.empty((n_det, nv), dtype=torch.float32, device=sino.device)
    check(lib().ctgpu_sino_to_image(_ptr(sino), sino.shape[1], nv, n_det, _ptr(out),
                                    stream_handle(stream)))
    return out


def image_compare(a, b, stream=None):
    """ImageFile::comparativeStatistics of device images a, b: [nx, ny] ->
    (d, r, e), or [n, nx, ny] -> array [n, 3]."""
    batched = a.dim() == 3
    if not batched:
        a, b = a.unsqueeze(0), b.unsqueeze(0)
    assert a.shape == b.shape and a.is_contiguous() and b.is_contiguous()
    n, nx, ny = a.shape
    out = np.zeros((n, 3), np.float64)
    check(lib().ctgpu_image_compare(_ptr(a), _ptr(b), n, nx, ny, nx * ny,
                                    out.ctypes.data_as(C.c_void_p), stream_handle(stream)))
    return out if batched else tuple(out[0])


def image_compare_device(a, b, out=None, stream=None):
    """image_compare of [n, nx, ny] device images with the results left on the
    device (out: float64 [n, 3]); no synchronisation."""
    torch = _torch()
    assert a.shape == b.shape and a.dim() == 3 and a.is_contiguous() and b.is_contiguous()
    n, nx, ny = a.shape
    if out is None:
        out = torch.empty((n, 3), dtype=torch.float64, device=a.device)
    check(lib().ctgpu_image_compare_device(_ptr(a), _ptr(b), n, nx, ny, nx * ny, _ptrd(out),
                                           stream_handle(stream)))
    return out


def image_arith(op, a, b, out=None, stream=None):
    """ImageFile add / subtract / multiply / divide of device FP32 images."""
    torch = _torch()
    assert a.shape == b.shape and a.is_contiguous() and b.is_contiguous()
    if out is None:
        out = torch.empty_like(a)
    check(lib().ctgpu_image_arith(enc(op), _ptr(a), _ptr(b), _ptr(out), a.numel(),
                                  stream_handle(stream)))
    return out


# ------------------------------------------------- polar / direct Fourier --
def _angles_ptr(angles):
    if angles is None:
        return None, None
    a = np.ascontiguousarray(angles, np.float64)
    return a, a.ctypes.data_as(C.c_void_p)


def convert_polar(geometry, sino, angles, nx, ny, interp="bilinear", stream=None):
    """Projections::convertPolar of device rows sino [n_view, pitch]: FP32 [nx, ny]."""
    torch = _torch()
    out = torch.empty((nx, ny), dtype=torch.float32, device=sino.device)
    keep, ap = _angles_ptr(angles)
    check(lib().ctgpu_convert_polar(C.byref(geometry), _ptr(sino), sino.shape[1], ap, nx, ny,
                                    enc(interp), _ptr(out), stream_handle(stream)))
    return out


def convert_fft_polar(geometry, sino, angles, nx, ny, interp="bilinear", zeropad=1,
                      stream=None):
    """Projections::convertFFTPolar: (real [nx, ny], imag [nx, ny], transform length)."""
    torch = _torch()
    re = torch.empty((nx, ny), dtype=torch.float32, device=sino.device)
    im = torch.empty_like(re)
    n = C.c_int()
    keep, ap = _angles_ptr(angles)
    check(lib().ctgpu_convert_fft_polar(C.byref(geometry), _ptr(sino), sino.shape[1], ap, nx, ny,
                                        enc(interp), zeropad, _ptr(re), _ptr(im), C.byref(n),
                                        stream_handle(stream)))
    return re, im, n.value


def image_ifft_magnitude(re, im, stream=None):
    """ImageFile::ifft + magnitude + shuffleFourierToNaturalOrder."""
    torch = _torch()
    out = torch.empty_like(re)
    check(lib().ctgpu_image_ifft_magnitude(_ptr(re), _ptr(im), re.shape[0], re.shape[1],
                                           _ptr(out), stream_handle(stream)))
    return out


def reconstruct_fourier(geometry, sino, angles, nx, ny, interp="bilinear", zeropad=1,
                        stream=None):
    """The GUI's Fourier reconstruction: convertFFTPolar, ifft, magnitude, shuffle."""
    torch = _torch()
    out = torch.empty((nx, ny), dtype=torch.float32, device=sino.device)
    keep, ap = _angles_ptr(angles)
    check(lib().ctgpu_reconstruct_fourier(C.byref(geometry), _ptr(sino), sino.shape[1], ap, nx,
                                          ny, enc(interp), zeropad, _ptr(out),
                                          stream_handle(stream)))
    return out
