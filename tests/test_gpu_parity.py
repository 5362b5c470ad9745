"""GPU parity: libctgpu.so (called through its C ABI) against the reference's own
outputs (golden fixtures) and the FP64 oracle.  Tolerance: rel-L2 <= 1e-5 for
FP32 results against FP64 (the path's precision target); bit-exact where the
reference itself computes in FP32 with FP64 weights (helical)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5
SCANS = {  # name: (phantom, geometry, nray, Scanner kwargs) -- tests/golden/make_golden.py
    "c1": ("shepp-logan", "parallel", 2, {}),
    "herman_par": ("herman", "parallel", 2, {}),
    "shepp_eqa": ("shepp-logan", "equiangular", 1, {}),
    "shepp_eqa_even": ("shepp-logan", "equiangular", 3, {}),
    "herman_eql": ("herman", "equilinear", 2, {}),
    "herman_eqa": ("herman", "equiangular", 1, {}),
    "shepp_par_even": ("shepp-logan", "parallel", 1, {"offsetView": 3}),
    "pulse_par": ("unit-pulse", "parallel", 1, {}),
    "shepp_eql_ratio": ("shepp-logan", "equilinear", 1,
                        {"focalLengthRatio": 3.0, "centerDetectorRatio": 1.5, "viewRatio": 1.2,
                         "scanRatio": 0.9}),
}


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device
    return torch, cg, device


def geom_from_hdr(cg, hdr):
    g, nd, nv, rs, ri, ds, di, vd, fl, sdl, fan = hdr
    return cg.Geometry(int(g), int(nd), int(nv), 0, rs, ri, ds, di, vd, fl, sdl, fan)


def to_dev(torch, device, a):
    t = device.alloc_sinogram(a.shape[0], a.shape[1])
    t[:, :a.shape[1]] = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    return t


@pytest.mark.parametrize("name", list(SCANS))
def test_raysums_match_reference(gpu, golden, name):
    torch, cg, device = gpu
    d = golden("scans")
    phm, geo, nray, kw = SCANS[name]
    hdr = d[name + "/hdr"]
    ph = cg.Phantom(phm)
    sc = cg.Scanner(ph, geo, int(hdr[1]), int(hdr[2]), nSample=nray, **kw)
    g = sc.geometry()
    assert g.det_inc == hdr[6] and g.view_diameter == hdr[7] and g.fan_beam_angle == hdr[10]
    sino = device.alloc_sinogram(g.n_view, g.n_det)
    ang = device.raysums(sc, ph, sino)
    cg.sync()
    np.testing.assert_array_equal(ang, d[name + "/angles"])
    out = sino[:, :g.n_det].cpu().numpy()
    ref = d[name + "/data"]
    print("raysums %s: rel-L2 %.3g, max |err| / max %.3g" % (
        name, rel_l2(out, ref), np.abs(out - ref).max() / max(np.abs(ref).max(), 1e-30)))
    assert rel_l2(out, ref) < TOL, rel_l2(out, ref)
    assert np.abs(out - ref).max() <= 1e-4 * max(np.abs(ref).max(), 1e-30)


def test_raysums_subrange_and_storage_offset(gpu, golden):
    torch, cg, device = gpu
    d = golden("scans")
    ph = cg.Phantom("herman")
    sc = cg.Scanner(ph, "parallel", 101, 60, nSample=2)
    sino = device.alloc_sinogram(60, 101)
    a1 = device.raysums(sc, ph, sino, start_view=0, n_views=25)
    a2 = device.raysums(sc, ph, sino, start_view=25, n_views=35)
    cg.sync()
    out = sino[:, :101].cpu().numpy()
    assert rel_l2(out, d["herman_par/data"]) < TOL
    # a sub-range restarts the reference's angle accumulation at iStartView * rotInc
    np.testing.assert_allclose(np.concatenate([a1[:25], a2[25:]]), d["herman_par/angles"],
                               rtol=0, atol=1e-14)


def test_raysums_host_entry_point(gpu, golden):
    torch, cg, device = gpu
    d = golden("scans")
    ph = cg.Phantom("shepp-logan")
    sc = cg.Scanner(ph, "equiangular", 133, 96)
    pj = cg.Projections.from_scanner(sc)
    sc.collectProjections(pj, ph)
    assert rel_l2(pj.data, d["shepp_eqa/data"]) < TOL
    np.testing.assert_array_equal(pj.angles, d["shepp_eqa/angles"])


def test_reconstructions_match_reference(gpu, golden):
    torch, cg, device = gpu
    scans = golden("scans")
    rec = golden("recons")
    n = len([k for k in rec.files if k.endswith("/cfg")])
    worst = 0
    for k in range(n):
        sc, nx, ny, bp, ip, flt, meth, zp, gen, prm = rec["%d/cfg" % k]
        g = geom_from_hdr(cg, scans[sc + "/hdr"])
        sino = to_dev(torch, device, scans[sc + "/data"])
        plan = device.ReconPlan(g, int(nx), int(ny), flt, float(prm), meth, int(zp), gen, ip, 1, bp)
        img = torch.zeros((int(nx), int(ny)), dtype=torch.float32, device="cuda")
        plan.run(sino, scans[sc + "/angles"], img)
        cg.sync()
        ref = rec["%d/image64" % k]
        e = rel_l2(img.cpu().numpy(), ref)
        worst = max(worst, e)
        assert e < TOL, "case %d %s: rel-L2 %.3g" % (k, rec["%d/cfg" % k], e)
    print("worst reconstruction rel-L2 %.3g" % worst)


def test_reconstructor_host_api(gpu, golden):
    torch, cg, device = gpu
    scans = golden("scans")
    rec = golden("recons")
    pj = cg.Projections(320, 367, 0, 0, 0, *scans["c1/hdr"][4:],
                        angles=scans["c1/angles"], data=scans["c1/data"])
    im = cg.ImageFile(256, 256)
    r = cg.Reconstructor(pj, im, "abs_bandlimit", -1, "convolution", 1, "direct", "linear", 1,
                         "table")
    r.reconstructAllViews()
    assert rel_l2(im.data, rec["0/image64"]) < TOL


def test_filter_matches_oracle(gpu, oracle):
    torch, cg, device = gpu
    rng = np.random.default_rng(3)
    nd, nv = 733, 5
    x = rng.random((nv, nd)).astype(np.float32)
    xd = to_dev(torch, device, x)
    cases = [("abs_bandlimit", "convolution", 1, "direct", 0),
             ("abs_hamming", "fft", 2, "direct", 1),
             ("abs_hamming", "fourier", 1, "direct", 2),
             ("shepp", "fft", 2, "direct", 0),
             ("abs_cosine", "convolution", 1, "inverse-fourier", 0),
             ("abs_hanning", "fft", 1, "inverse-fourier", 1),
             ("abs_sinc", "convolution", 1, "direct", 2),
             ("triangle", "fourier", 0, "direct", 0)]
    names = ("parallel", "equiangular", "equilinear")
    for flt, meth, zp, gen, geo in cases:
        g = cg.Geometry(geo, nd, nv, 0, 0, 0.01, 0, 0.0021, 2.6, 2.6, 5.2, 1.0)
        plan = device.ReconPlan(g, 16, 16, flt, 0.54, meth, zp, gen, "linear", 1, "table")
        out = device.alloc_sinogram(nv, nd)
        plan.filter(xd, out)
        cg.sync()
        ref = oracle.ProcessSignal(flt, meth, nd, 0.0021, param=0.54,
                                   generation=gen, zeropad=zp, geometry=names[geo],
                                   focal_length=2.6, sdl=5.2).filter(x)
        e = rel_l2(out[:, :nd].cpu().numpy(), ref)
        assert e < TOL, (flt, meth, zp, gen, geo, e)


@pytest.mark.parametrize("nd", [3, 64, 129, 367, 1500, 2049, 4500, 8192])
def test_filter_sizes_against_oracle(gpu, oracle, nd):
    """Every FFT filter kernel variant (transform lengths 8 to 16384: 128 to
    1024 threads, radix-8 and radix-16 passes), with three views (the last
    CTA's pair holds one), against the FP64 oracle; detectors past 8192 are
    rejected."""
    torch, cg, device = gpu
    rng = np.random.default_rng(nd)
    nv = 3
    x = rng.random((nv, nd)).astype(np.float32)
    xd = to_dev(torch, device, x)
    g = cg.Geometry(1, nd, nv, 0, 0, 0.01, 0, 0.0021, 2.6, 2.6, 5.2, 1.0)
    plan = device.ReconPlan(g, 16, 16, "abs_hamming", 0.54, "fft", 1, "direct", "linear", 1,
                            "table")
    out = device.alloc_sinogram(nv, nd)
    plan.filter(xd, out)
    cg.sync()
    ref = oracle.ProcessSignal("abs_hamming", "fft", nd, 0.0021, param=0.54, generation="direct",
                               zeropad=1, geometry="equiangular", focal_length=2.6,
                               sdl=5.2).filter(x)
    e = rel_l2(out[:, :nd].cpu().numpy(), ref)
    assert e < TOL, (nd, e)
    if nd == 8192:
        big = 8193
        gb = cg.Geometry(1, big, 1, 0, 0, 0.01, 0, 0.0021, 2.6, 2.6, 5.2, 1.0)
        pb = device.ReconPlan(gb, 16, 16, "abs_hamming", 0.54, "fft", 1, "direct", "linear", 1,
                              "table")
        with pytest.raises(cg.CtgpuError) as ei:
            pb.filter(device.alloc_sinogram(1, big), device.alloc_sinogram(1, big))
        assert ei.value.code == 2


def test_helical_bit_exact(gpu, golden):
    torch, cg, device = gpu
    d = golden("helical")
    for k in range(2):
        g = geom_from_hdr(cg, d["%d/in_hdr" % k])
        sino = to_dev(torch, device, d["%d/in_data" % k])
        out, ang = device.helical180li(g, sino, int(d["%d/interpview" % k]))
        g.n_view = out.shape[0]
        device.halfscan_feather(g, out)
        cg.sync()
        np.testing.assert_array_equal(ang, d["%d/out_angles" % k])
        np.testing.assert_array_equal(out[:, :g.n_det].cpu().numpy(), d["%d/out_data" % k])


def test_projector_is_adjoint_of_backprojector(gpu):
    torch, cg, device = gpu
    g = cg.Geometry(0, 129, 90, 0, 0, np.pi / 90, 0, 0.021, 2.6, 2.6, 5.2, 0.0)
    ang = np.arange(90) * (np.pi / 90)
    plan = device.ReconPlan(g, 96, 80, "abs_bandlimit", -1, "convolution", 1, "direct", "linear",
                            1, "table")
    torch.manual_seed(0)
    x = torch.randn((96, 80), device="cuda")
    y = device.alloc_sinogram(90, 129)
    y[:, :129] = torch.randn((90, 129), device="cuda")
    ax = device.alloc_sinogram(90, 129)
    plan.project(x, ang, ax)
    bty = torch.zeros((96, 80), device="cuda")
    plan.backproject(y, ang, bty)
    cg.sync()
    lhs = float((ax[:, :129].double() * y[:, :129].double()).sum())
    rhs = float((x.double() * bty.double()).sum())
    scale = float(ax.double().norm() * y.double().norm())
    assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs, scale)


def test_projector_matches_oracle(gpu, oracle):
    torch, cg, device = gpu
    g = cg.Geometry(0, 129, 45, 0, 0, np.pi / 45, 0, 0.021, 2.6, 2.6, 5.2, 0.0)
    og = oracle.Geom(0, 129, 45, np.pi / 45, 0.021, 2.6, 5.2, 2.6, 0.0)
    ang = np.arange(45) * (np.pi / 45)
    plan = device.ReconPlan(g, 64, 64, "abs_bandlimit", -1, "convolution", 1, "direct", "linear",
                            1, "table")
    rng = np.random.default_rng(2)
    x = rng.random((64, 64))
    ax = device.alloc_sinogram(45, 129)
    plan.project(torch.from_numpy(x.astype(np.float32)).cuda(), ang, ax)
    cg.sync()
    ref = oracle.project_image(og, x, ang)
    assert rel_l2(ax[:, :129].cpu().numpy(), ref) < TOL


def test_zero_views_and_accumulate(gpu, golden):
    torch, cg, device = gpu
    scans = golden("scans")
    g = geom_from_hdr(cg, scans["herman_par/hdr"])
    sino = to_dev(torch, device, scans["herman_par/data"])
    ang = scans["herman_par/angles"]
    plan = device.ReconPlan(g, 40, 40, "abs_bandlimit", -1, "convolution", 1, "direct", "cubic", 1,
                            "idiff")
    full = torch.zeros((40, 40), device="cuda")
    plan.run(sino, ang, full)
    # view sub-ranges accumulated, then PostProcessing: reconstructView(start, count) x 2
    part = torch.full((40, 40), 7.0, device="cuda")
    plan.run(sino, ang, part, start_view=0, n_views=23, postprocess=False)   # overwrites
    plan.run(sino, ang, part, start_view=23, n_views=37, postprocess=False, accumulate=True)
    plan.postprocess(part)
    cg.sync()
    assert rel_l2(part.cpu().numpy(), full.cpu().numpy()) < 1e-6
    plan.run(sino, ang, part, start_view=0, n_views=23, postprocess=False)
    plan.run(sino, ang, part, start_view=23, n_views=37, postprocess=True, accumulate=True)
    cg.sync()
    assert rel_l2(part.cpu().numpy(), full.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("geo,interp,bp", [("equiangular", "cubic", "table"),
                                           ("parallel", "linear", "idiff"),
                                           ("equilinear", "nearest", "table"),
                                           ("parallel", "cubic", "diff")])
def test_batched_launch_equals_single(gpu, geo, interp, bp):
    torch, cg, device = gpu
    from ctsim_gb300 import phantoms
    B, nd, nv, n = 5, 181, 120, 96
    sinos, angs = [], None
    for b in range(B):
        ph = phantoms.make_phantom(phantoms.random_ellipses(seed=50 + b, n=7))
        sc = cg.Scanner(ph, geo, nd, nv)
        s = device.alloc_sinogram(nv, nd)
        angs = device.raysums(sc, ph, s)
        sinos.append(s)
    g = sc.geometry()
    plan = device.ReconPlan(g, n, n, "abs_hamming", 0.54, "fft", 2, "direct", interp, 1, bp)
    batch = torch.stack(sinos)
    out = torch.zeros((B, n, n), device="cuda")
    plan.run_batch(batch, angs, out)
    single = torch.zeros((n, n), device="cuda")
    for b in range(B):
        plan.run(sinos[b], angs, single)
        cg.sync()
        assert rel_l2(out[b].cpu().numpy(), single.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("pinned", [False, True])
def test_batch_host_equals_device_batch(gpu, pinned):
    """ctgpu_recon_run_batch_host (copies overlapped with the reconstruction)
    gives the device batch's images; 37 slices of 64 x 64."""
    torch, cg, device = gpu
    from ctsim_gb300 import phantoms
    B, nd, nv, n = 37, 129, 90, 64
    sinos, angs = [], None
    for b in range(B):
        ph = phantoms.make_phantom(phantoms.random_ellipses(seed=300 + b, n=5))
        sc = cg.Scanner(ph, "equiangular", nd, nv)
        s = device.alloc_sinogram(nv, nd)
        angs = device.raysums(sc, ph, s)
        sinos.append(s)
    g = sc.geometry()
    plan = device.ReconPlan(g, n, n, "abs_hamming", 0.54, "fft", 2, "direct", "cubic", 1, "table")
    batch = torch.stack(sinos)
    ref = torch.zeros((B, n, n), device="cuda")
    plan.run_batch(batch, angs, ref)
    cg.sync()
    host = batch[:, :, :nd].contiguous().cpu()
    if pinned:
        host = host.pin_memory()
        out = torch.zeros((B, n, n), dtype=torch.float32).pin_memory()
    else:
        host = host.numpy()
        out = None
    res = plan.run_batch_host(host, angs, out)
    res = res.numpy() if hasattr(res, "numpy") else res
    r = ref.cpu().numpy()
    for b in range(B):
        assert rel_l2(res[b], r[b]) < 1e-7, b


@pytest.mark.parametrize("geo,interp,backproj", [("equiangular", "cubic", "table"),
                                                  ("parallel", "linear", "trig"),
                                                  ("parallel", "linear", "diff"),
                                                  ("parallel", "nearest", "idiff")])
def test_batch_host_chunks_share_records(gpu, geo, interp, backproj):
    """A host batch split into chunks of different sizes, a later one larger
    than the first, consecutive chunks on two compute streams with their own
    buffers (sized for the largest chunk up front; each set's first chunk
    builds the (tile, view) records its later chunks use): the device batch's
    images, bit for bit.  The chunk plan covers every slice once for any
    batch size."""
    torch, cg, device = gpu
    from ctsim_gb300 import phantoms
    nd, nv, n = 367, 360, 256
    ph0 = phantoms.make_phantom(phantoms.random_ellipses(seed=900, n=5))
    sc = cg.Scanner(ph0, geo, nd, nv)
    g = sc.geometry()
    plan = device.ReconPlan(g, n, n, "abs_hamming", 0.54, "fft", 2, "direct", interp, 1, backproj)
    for b in (1, 2, 7, 33, 100, 500):
        sizes = plan.host_chunks(b)
        assert sum(sizes) == b and min(sizes) >= 1, (b, sizes)
    B = next((b for b in (24, 16, 40, 64)
              if len(plan.host_chunks(b)) >= 2 and max(plan.host_chunks(b)[1:]) > plan.host_chunks(b)[0]),
             None)
    assert B is not None, [plan.host_chunks(b) for b in (24, 16, 40, 64)]
    phs = [phantoms.make_phantom(phantoms.random_ellipses(seed=900 + b, n=5)) for b in range(B)]
    batch = torch.zeros((B, nv, device.pitch_for(nd)), device="cuda")
    angs = device.raysums_batch(sc, phs, batch)
    ref = torch.zeros((B, n, n), device="cuda")
    plan.run_batch(batch, angs, ref)
    cg.sync()
    host = batch[:, :, :nd].contiguous().cpu().pin_memory()
    out = torch.zeros((B, n, n), dtype=torch.float32).pin_memory()
    for _ in range(2):   # the second call finds every buffer in place
        out.zero_()
        plan.run_batch_host(host, angs, out)
        assert torch.equal(out, ref.cpu()), plan.host_chunks(B)
    # chunk sizes fixed by the caller: used in turn, the last one cut short
    planned = plan.host_chunks(B)
    plan.set_host_chunks([3, 5])
    fixed = plan.host_chunks(B)
    assert sum(fixed) == B and fixed[:4] == [3, 5, 3, 5], fixed
    out.zero_()
    plan.run_batch_host(host, angs, out)
    assert torch.equal(out, ref.cpu()), fixed
    plan.set_host_chunks()
    assert plan.host_chunks(B) == planned


@pytest.mark.parametrize("geo,n,interp,bp", [("equiangular", 512, "cubic", "table"),
                                             ("parallel", 256, "linear", "table"),
                                             ("equilinear", 128, "nearest", "table"),
                                             ("parallel", 96, "cubic", "table"),
                                             ("parallel", 512, "linear", "idiff"),
                                             ("parallel", 256, "nearest", "idiff"),
                                             ("parallel", 128, "cubic", "idiff")])
def test_single_slice_view_groups(gpu, geo, n, interp, bp):
    """A single slice of few tiles splits its views into groups whose partial
    images are summed in order: the same image as the batched (unsplit)
    launch to FP32 rounding, also when the views come in two accumulated
    halves (reconstructView + postProcessing)."""
    torch, cg, device = gpu
    from ctsim_gb300 import phantoms
    nd, nv = int(1.4 * n) | 1, 360
    ph = phantoms.make_phantom(phantoms.random_ellipses(seed=77, n=8))
    sc = cg.Scanner(ph, geo, nd, nv)
    sino = device.alloc_sinogram(nv, nd)
    ang = device.raysums(sc, ph, sino)
    plan = device.ReconPlan(sc.geometry(), n, n, "abs_hamming", 0.54, "fft", 2, "direct", interp,
                            1, bp)
    one = torch.zeros((n, n), device="cuda")
    plan.run(sino, ang, one)
    batch = torch.zeros((2, n, n), device="cuda")
    plan.run_batch(torch.stack([sino, sino]), ang, batch)
    halves = torch.zeros((n, n), device="cuda")
    plan.run(sino, ang, halves, start_view=0, n_views=nv // 2, accumulate=True, postprocess=False)
    plan.run(sino, ang, halves, start_view=nv // 2, n_views=nv - nv // 2, accumulate=True,
             postprocess=True)
    cg.sync()
    ref = batch[0].cpu().numpy()
    assert torch.equal(batch[0], batch[1])
    assert rel_l2(one.cpu().numpy(), ref) < 1e-6, rel_l2(one.cpu().numpy(), ref)
    assert rel_l2(halves.cpu().numpy(), ref) < 1e-6, rel_l2(halves.cpu().numpy(), ref)


@pytest.mark.parametrize("geo,nray", [("parallel", 2), ("equiangular", 1), ("equilinear", 3)])
def test_raysums_batch_equals_single(gpu, geo, nray):
    """ctgpu_collect_projections_batch (all phantoms in one launch) writes the
    same sinogram bits as one collectProjections per phantom."""
    torch, cg, device = gpu
    from ctsim_gb300 import phantoms as P
    phs = [cg.Phantom("herman"), cg.Phantom("shepp-logan")] + \
          [P.make_phantom(P.random_ellipses(seed=70 + i, n=3 + 4 * i)) for i in range(4)]
    sc = cg.Scanner(phs[0], geo, 157, 96, nSample=nray)
    g = sc.geometry()
    pitch = device.pitch_for(157)
    batch = torch.zeros((len(phs), 96, pitch), device="cuda")
    ang_b = device.raysums_batch(sc, phs, batch)
    for i, ph in enumerate(phs):
        one = device.alloc_sinogram(96, 157)
        ang = device.raysums(sc, ph, one)
        cg.sync()
        assert np.array_equal(ang, ang_b)
        assert torch.equal(one[:, :157], batch[i, :, :157]), i


@pytest.mark.parametrize("name", ["shepp_eqa", "shepp_eqa_even", "herman_eql", "herman_eqa",
                                  "shepp_eql_ratio"])
def test_interpolate_to_parallel_matches_reference(gpu, golden, name):
    """Projections::interpolateToParallel on the device against the reference's
    own output (ref_harness rebin on the reference's scan)."""
    torch, cg, device = gpu
    d, r = golden("scans"), golden("rebin")
    g = geom_from_hdr(cg, d[name + "/hdr"])
    data = d[name + "/data"]
    sino = torch.zeros((g.n_view, device.pitch_for(g.n_det)), device="cuda")
    sino[:, :g.n_det] = torch.from_numpy(data).cuda()
    out, g2, ang = device.interpolate_to_parallel(g, sino, d[name + "/angles"])
    cg.sync()
    ref, rh = r[name + "/data"], r[name + "/hdr"]
    np.testing.assert_array_equal(ang, r[name + "/angles"])
    assert (g2.geometry, g2.rot_inc, g2.det_start, g2.det_inc) == (0, rh[4], rh[5], rh[6])
    o = out[:, :g.n_det].cpu().numpy()
    err = np.abs(o - ref).max() / np.abs(ref).max()
    print("interpolateToParallel %s: max |err| / max %.3g" % (name, err))
    assert err <= 1e-6, err


def test_rasterize_matches_reference(gpu, golden):
    """Phantom::convertToImagefile (phm2if) on the device: bit for bit against
    the reference's FP32-image build, and within FP32 rounding of its FP64
    build."""
    torch, cg, device = gpu
    r = golden("raster")
    k = 0
    while "%d/cfg" % k in r:
        phm, n, ns = r["%d/cfg" % k]
        img, ext, inc = cg.Phantom(str(phm)).rasterize(int(n), int(n), 1.0, int(ns))
        a = img.cpu().numpy()
        np.testing.assert_array_equal(a, r["%d/image32" % k])
        ref64 = r["%d/image" % k]
        assert np.abs(a - ref64).max() <= 1e-6 * max(np.abs(ref64).max(), 1e-30)
        k += 1
    assert k == 3


def test_roi_reconstructions_match_reference(gpu, golden):
    """A plan with a region of interest (ctgpu_recon_create's roi,
    ReconstructionROI of libctsim/backprojectors.cpp:284-315; a swapped and a
    clamped ROI among them) against the reference's FP64 image of the same
    ROI, rel-L2 <= 1e-5."""
    torch, cg, device = gpu
    scans = golden("scans")
    d = golden("roi")
    k = 0
    while "%d/cfg" % k in d:
        name, nx, ny, bp, ip = d["%d/cfg" % k]
        nx, ny = int(nx), int(ny)
        g = geom_from_hdr(cg, scans[name + "/hdr"])
        plan = device.ReconPlan(g, nx, ny, "abs_bandlimit", -1.0, "convolution", 1, "direct", ip,
                                1, bp, roi=tuple(d["%d/roi" % k]))
        img = torch.zeros((nx, ny), device="cuda")
        plan.run(to_dev(torch, device, scans[name + "/data"]), scans[name + "/angles"], img)
        cg.sync()
        ref = d["%d/image64" % k]
        e = rel_l2(img.cpu().numpy(), ref)
        print("ROI %s %s/%s: rel-L2 %.3g" % (name, bp, ip, e))
        assert e < TOL, (d["%d/cfg" % k], e)
        k += 1
    assert k == 6
