"""The allocation-free diff backprojection, for callers that cannot allocate
device memory (host applications that own every device allocation, real-time
loops that must not block on the allocator), against the library's
allocating entry point: ctgpu_backproject_diff_noalloc vs
ctgpu_recon_backproject with a "diff" plan, through the C ABI, two different
calls in a row (the fixed scratch keeps the first call's contents); then 720
views (several blocks of view records), a region of interest, nearest
interpolation and a view range accumulated onto an earlier one."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

CASES = [  # golden scan, nx, ny, interpolation
    ("herman_par", 40, 40, "linear"),
    ("shepp_par_even", 33, 31, "cubic"),
]


def _geom(cg, hdr):
    g, nd, nv, rs, ri, ds, di, vd, fl, sdl, fan = hdr
    return cg.Geometry(int(g), int(nd), int(nv), 0, rs, ri, ds, di, vd, fl, sdl, fan)


def test_noalloc_diff_matches_allocating_path(golden):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device
    from ctsim_gb300._lib import RUN_POSTPROCESS, check, lib
    scans = golden("scans")
    for name, nx, ny, interp in CASES:   # two calls in a row
        g = _geom(cg, scans[name + "/hdr"])
        ang = np.ascontiguousarray(scans[name + "/angles"], np.float64)
        sino = device.alloc_sinogram(g.n_view, g.n_det)
        sino[:, :g.n_det] = torch.from_numpy(scans[name + "/data"]).cuda()
        plan = device.ReconPlan(g, nx, ny, "abs_bandlimit", -1.0, "convolution", 1, "direct",
                                interp, 1, "diff")
        filtered = device.alloc_sinogram(g.n_view, g.n_det)
        plan.filter(sino, filtered)
        ref = torch.zeros((nx, ny), device="cuda")
        plan.backproject(filtered, ang, ref)
        plan.postprocess(ref)
        out = torch.full((nx, ny), 123.0, device="cuda")
        check(lib().ctgpu_backproject_diff_noalloc(
            C.byref(g), nx, ny, interp.encode(), None, C.c_void_p(filtered.data_ptr()),
            filtered.shape[1], ang.ctypes.data_as(C.c_void_p), g.n_view,
            C.c_void_p(out.data_ptr()), RUN_POSTPROCESS, device.stream_handle()))
        cg.sync()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 1e-6, name


def _noalloc(lib, g, nx, ny, interp, roi, filtered, ang, out, flags, stream):
    from ctsim_gb300._lib import Roi, check
    r = None if roi is None else C.byref(Roi(*roi))
    check(lib().ctgpu_backproject_diff_noalloc(
        C.byref(g), nx, ny, interp.encode(), r, C.c_void_p(filtered.data_ptr()),
        filtered.shape[1], ang.ctypes.data_as(C.c_void_p), len(ang),
        C.c_void_p(out.data_ptr()), flags, stream))


def test_noalloc_many_views_roi_nearest_and_accumulate():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device
    from ctsim_gb300._lib import RUN_ACCUMULATE, RUN_POSTPROCESS, lib
    ph = cg.Phantom("shepp-logan")
    sc = cg.Scanner(ph, "parallel", 129, 720, nSample=1)
    g = sc.geometry()
    sino = device.alloc_sinogram(720, 129)
    ang = np.ascontiguousarray(device.raysums(sc, ph, sino), np.float64)
    nx, ny = 64, 48
    roi = (-0.45, -0.3, 0.55, 0.62)
    sh = device.stream_handle()
    for interp, r in (("nearest", roi), ("cubic", roi), ("linear", None)):
        plan = device.ReconPlan(g, nx, ny, "abs_bandlimit", -1.0, "convolution", 1, "direct",
                                interp, 1, "diff", roi=r)
        filtered = device.alloc_sinogram(720, 129)
        plan.filter(sino, filtered)
        ref = torch.zeros((nx, ny), device="cuda")
        plan.backproject(filtered, ang, ref)
        raw = ref.clone()
        plan.postprocess(ref)
        out = torch.full((nx, ny), 7.0, device="cuda")
        _noalloc(lib, g, nx, ny, interp, r, filtered, ang, out, RUN_POSTPROCESS, sh)
        cg.sync()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 1e-6, (interp, r)
        # views [0, 300) and then [300, 720) added onto them, without PostProcessing
        acc = torch.full((nx, ny), 7.0, device="cuda")
        _noalloc(lib, g, nx, ny, interp, r, filtered[:300], ang[:300], acc, 0, sh)
        _noalloc(lib, g, nx, ny, interp, r, filtered[300:], ang[300:], acc, RUN_ACCUMULATE, sh)
        cg.sync()
        assert rel_l2(acc.cpu().numpy(), raw.cpu().numpy()) < 1e-6, (interp, r)


def test_noalloc_rejects_oversized_requests():
    import ctsim_gb300 as cg
    from ctsim_gb300._lib import lib
    g = cg.Geometry(0, 1024, 4096, 0, 0.0, 0.001, 0.0, 0.01, 2.6, 2.6, 5.2, 0.0)
    ang = np.zeros(4096)
    rc = lib().ctgpu_backproject_diff_noalloc(C.byref(g), 2048, 2048, b"linear", None,
                                              C.c_void_p(16), 1024,
                                              ang.ctypes.data_as(C.c_void_p), 4096,
                                              C.c_void_p(16), 0, None)
    assert rc == 1
    assert b"too large for the fixed 16 MiB scratch" in lib().ctgpu_last_error()
