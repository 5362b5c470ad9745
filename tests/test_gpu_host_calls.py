"""The host-buffer entry points against their device counterparts (GPU), bit
for bit: ctgpu_recon_run_host (the sinogram goes up as dense rows, read at
pitch nDet) against ctgpu_recon_run on the padded device rows, and
ctgpu_collect_projections_host (rows written densely and copied down in one
piece) against the device ray-sums, with a view sub-range, an offset view
and a storage offset (Scanner::collectProjections, libctsim/scanner.cpp:
295-419; Reconstructor::reconstructAllViews, libctsim/reconstruct.cpp:
142-147)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


@pytest.mark.parametrize("geo,nd,interp", [("equiangular", 733, "cubic"),
                                           ("parallel", 256, "linear"),
                                           ("equilinear", 97, "nearest")])
def test_run_host_equals_device_run(gpu, geo, nd, interp):
    torch, cg, device, phantoms = gpu
    nv, n = 180, 160
    ph = phantoms.make_phantom(phantoms.random_ellipses(seed=nd, n=9))
    sc = cg.Scanner(ph, geo, nd, nv)
    sino = device.alloc_sinogram(nv, nd)
    ang = device.raysums(sc, ph, sino)
    cg.sync()
    plan = device.ReconPlan(sc.geometry(), n, n, "abs_hamming", 0.54, "fft", 2, "direct", interp,
                            1, "table")
    img = torch.zeros((n, n), device="cuda")
    plan.run(sino, ang, img)
    cg.sync()
    host = plan.run_host(np.ascontiguousarray(sino[:, :nd].cpu().numpy()), ang)
    assert np.array_equal(host, img.cpu().numpy())


@pytest.mark.parametrize("geo,nd,ns", [("equiangular", 733, 1), ("parallel", 128, 2),
                                       ("equilinear", 65, 3)])
def test_collect_host_equals_device(gpu, geo, nd, ns):
    torch, cg, device, phantoms = gpu
    nv = 96
    ph = phantoms.make_phantom(phantoms.random_ellipses(seed=nd + ns, n=7))
    sc = cg.Scanner(ph, geo, nd, nv, nSample=ns)
    dev = device.alloc_sinogram(nv, nd)
    ang = device.raysums(sc, ph, dev)
    cg.sync()
    ref = dev[:, :nd].cpu().numpy()
    proj = cg.Projections.from_scanner(sc)
    sc.collectProjections(proj)
    assert np.array_equal(proj.data, ref)
    assert np.array_equal(proj.angles, ang)
    # views [20, 60) of the scan, stored from row 20: the rest keeps its values
    proj2 = cg.Projections.from_scanner(sc)
    proj2.data[:] = -1.0
    sc.collectProjections(proj2, iStartView=20, iNumViews=40)
    assert np.array_equal(proj2.data[20:60], ref[20:60])
    assert (proj2.data[:20] == -1.0).all() and (proj2.data[60:] == -1.0).all()
    # the same views stored from row 0, the device call's offset view against
    # the host call's
    dev2 = device.alloc_sinogram(nv, nd)
    device.raysums(sc, ph, dev2, start_view=20, n_views=40, offset_view=5)
    cg.sync()
    proj3 = cg.Projections.from_scanner(sc)
    sc.collectProjections(proj3, iStartView=20, iNumViews=40, iOffsetView=5, iStorageOffset=0)
    assert np.array_equal(proj3.data[:40], dev2[20:60, :nd].cpu().numpy())
