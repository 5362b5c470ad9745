"""Parity at the sizes the benchmark times, against the FP64 oracle (GPU).

- The uneven batch's extreme shapes, in one ctgpu_batch launch: a 1024 x 1024
  image from 1440 views x 1434 detectors for each geometry (parallel,
  equiangular, equilinear), next to a 128 x 128 image from 180 views x 179
  detectors; 20 random ellipses each, abs_hamming 0.54 by FFT with zero-pad 2,
  cubic interpolation.
- The helical workload: 16 ellipsoids, equilinear 1024 detectors, 1152 views
  per rotation x 8 rotations; 180LI z-interpolation with feathering at 64
  slice positions through one helical plan; the FBP of all 64 slices at
  1024 x 1024 (Shepp by FFT, zero-pad 2, linear) as one ctgpu_batch.  The
  first, a middle and the last slice are checked.
- The main workload's timed step, ctgpu_recon_run_batch: one filter launch
  over B x 720 rows (which also writes the interval rows), then one batched
  backprojection of the B slices (equiangular 733 x 720, 12 ellipses,
  512 x 512, cubic), B = 3.

Tolerances: rel-L2 <= 1e-5 against FP64 for sinograms and images (the path's
precision bar).  The z-interpolated rows, fed the same FP32 scan as the
oracle, agree to 1e-6 of the largest sample (FP64 weights on both sides; the
device's atan may differ from the host's in the last bit).  Each image is
compared with the oracle's reconstruction of the same FP32 sinogram the GPU
read, so the sinogram and image errors are measured separately.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

GEOS = ("parallel", "equiangular", "equilinear")


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


def _ogeom(po, g, n_view=None):
    return po.Geom(g.geometry, g.n_det, g.n_view if n_view is None else n_view, g.rot_inc,
                   g.det_inc, g.focal_length, g.source_detector_length, g.view_diameter,
                   g.fan_beam_angle)


def test_uneven_batch_extreme_shapes(gpu, oracle):
    torch, cg, device, phantoms = gpu
    po = oracle
    shapes = [(1024, 1440, 1434, geo) for geo in GEOS] + [(128, 180, 179, "parallel")]
    probs, scans = [], []
    for i, (side, nv, nd, geo) in enumerate(shapes):
        elems = phantoms.random_ellipses(seed=300 + i, n=20)
        ph = phantoms.make_phantom(elems)
        sc = cg.Scanner(ph, geo, nd, nv)
        sino = device.alloc_sinogram(nv, nd)
        ang = device.raysums(sc, ph, sino)
        probs.append(dict(geometry=sc.geometry(), nx=side, ny=side, sino=sino, angles=ang,
                          image=torch.full((side, side), float("nan"), device="cuda"),
                          filter_name="abs_hamming", filter_param=0.54, filter_method="fft",
                          zeropad=2, interp="cubic", backproj="table"))
        scans.append((elems, geo, nd, nv))
    batch = device.BatchPlan(probs, autotune=False, graph=False)
    batch.run()
    cg.sync()
    for q, (elems, geo, nd, nv) in zip(probs, scans):
        g = q["geometry"]
        s_gpu = q["sino"][:, :nd].cpu().numpy()
        osc = po.Scanner(po.Phantom(elements=elems), geo, nd, nv)
        s_ref, a_ref = osc.collect()
        np.testing.assert_array_equal(q["angles"], a_ref)
        e_s = rel_l2(s_gpu, s_ref)
        ref = po.reconstruct(_ogeom(po, g), s_gpu, q["angles"], q["nx"], q["ny"],
                             filter_name="abs_hamming", param=0.54, method="fft", zeropad=2,
                             backproj="table", interp="cubic")
        img = q["image"].cpu().numpy()
        assert np.isfinite(img).all()
        e_i = rel_l2(img, ref)
        print("batch %s %d^2 x %d views x %d det: sinogram rel-L2 %.3g, image rel-L2 %.3g"
              % (geo, q["nx"], nv, nd, e_s, e_i))
        assert e_s < 1e-5, (geo, q["nx"], e_s)
        assert e_i < 1e-5, (geo, q["nx"], e_i)


def test_helical_workload_full_size(gpu, oracle):
    torch, cg, device, phantoms = gpu
    po = oracle
    ell = phantoms.random_ellipsoids(seed=77, n=16, z_half=1.0)
    nrot, nvr, ndet, nslice, side = 8, 1152, 1024, 64, 1024
    nview = nrot * nvr
    z0, dz = -1.0, 2.0 / nview
    foot = phantoms.ellipsoid_footprint(ell)
    sc = cg.Scanner(phantoms.make_phantom(foot), "equilinear", ndet, nview,
                    rotAngle=nrot * 2 * np.pi)
    g = sc.geometry()
    sino = device.alloc_sinogram(nview, ndet)
    ang = device.raysums_ellipsoids(sc, ell, z0, dz, sino)
    hplan = device.HelicalPlan(g, nview, equilinear=True, feather=True)
    last = hplan.n_view_out - 1
    ivs = np.linspace(last + 1, nview - last - 2, nslice).astype(int)
    zsino, angs = hplan.run(sino, ivs)
    gh = cg.Geometry.from_buffer_copy(g)
    gh.n_view = hplan.n_view_out
    probs = [dict(geometry=gh, nx=side, ny=side, sino=zsino[k], angles=angs[k],
                  image=torch.full((side, side), float("nan"), device="cuda"),
                  filter_name="shepp", filter_param=-1.0, filter_method="fft", zeropad=2,
                  interp="linear", backproj="table") for k in range(nslice)]
    batch = device.BatchPlan(probs, autotune=False, graph=False)
    batch.run()
    cg.sync()

    # the scan
    osc = po.Scanner(po.Phantom(elements=foot), "equilinear", ndet, nview, rotangle=nrot)
    s_ref, a_ref = po.collect_ellipsoids(osc, ell, z0, dz)
    np.testing.assert_allclose(ang, a_ref, rtol=0, atol=1e-12)
    data = sino[:, :ndet].cpu().numpy()
    e_s = rel_l2(data, s_ref)
    print("helical scan 1024 det x %d views: rel-L2 %.3g" % (nview, e_s))
    assert e_s < 1e-5, e_s

    og = osc.geom()
    for k in (0, nslice // 2, nslice - 1):
        r, rang = po.helical180li(og, data, int(ivs[k]), allow_equilinear=True)
        og2 = _ogeom(po, gh)
        r = po.halfscan_feather(og2, r, true_gamma=True)
        np.testing.assert_allclose(angs[k], rang, rtol=0, atol=1e-12)
        z = zsino[k, :, :ndet].cpu().numpy()
        assert np.abs(z - r).max() <= 1e-6 * np.abs(r).max(), k
        ref = po.reconstruct(og2, z, angs[k], side, side, filter_name="shepp", param=-1.0,
                             method="fft", zeropad=2, backproj="table", interp="linear")
        img = probs[k]["image"].cpu().numpy()
        assert np.isfinite(img).all()
        e_i = rel_l2(img, ref)
        print("helical slice %d (view %d, %d views) 1024^2: image rel-L2 %.3g"
              % (k, ivs[k], gh.n_view, e_i))
        assert e_i < 1e-5, (k, e_i)


def test_bench_timed_sequence(gpu, oracle):
    """plan.run_batch over the batch's B slices (one filter launch over the
    B x 720 rows that also writes the interval rows, then one backprojection
    launch), as the benchmark's timed step does."""
    torch, cg, device, phantoms = gpu
    po = oracle
    B, nd, nv, nx = 3, 733, 720, 512
    elems = [phantoms.random_ellipses(seed=b, n=12) for b in range(B)]
    phs = [phantoms.make_phantom(e) for e in elems]
    sc = cg.Scanner(phs[0], "equiangular", nd, nv, nSample=1)
    g = sc.geometry()
    pitch = device.pitch_for(nd)
    sinos = torch.zeros((B, nv, pitch), device="cuda")
    images = torch.full((B, nx, nx), float("nan"), device="cuda")
    plan = device.ReconPlan(g, nx, nx, "abs_hamming", 0.54, "fft", 2, "direct", "cubic", 1,
                            "table")
    ang = device.raysums_batch(sc, phs, sinos)
    plan.run_batch(sinos, ang, images)
    cg.sync()
    osc = po.Scanner(po.Phantom(elements=elems[0]), "equiangular", nd, nv, nsample=1)
    for b in range(B):
        osc.phantom = po.Phantom(elements=elems[b])
        s_ref, a_ref = osc.collect()
        np.testing.assert_array_equal(ang, a_ref)
        s_gpu = sinos[b, :, :nd].cpu().numpy()
        e_s = rel_l2(s_gpu, s_ref)
        ref = po.reconstruct(osc.geom(), s_gpu, ang, nx, nx, filter_name="abs_hamming",
                             param=0.54, method="fft", zeropad=2, backproj="table",
                             interp="cubic")
        e_i = rel_l2(images[b].cpu().numpy(), ref)
        print("timed sequence slice %d: sinogram rel-L2 %.3g, image rel-L2 %.3g" % (b, e_s, e_i))
        assert e_s < 1e-5, (b, e_s)
        assert e_i < 1e-5, (b, e_i)
