"""The allocation-free diff backprojection, for callers that cannot allocate
device memory (graph capture that must not grow the pool, host applications
that own every device allocation, real-time loops), against the library's
allocating entry point: ctgpu_backproject_diff_noalloc vs
ctgpu_recon_backproject with a "diff" plan, through the C ABI, two different
calls in a row (the fixed scratch keeps the first call's contents)."""
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
