"""Helical scan of a 3-D ellipsoid phantom with an equilinear detector, the
equilinear 180LI z-interpolation and half-scan feathering, and the FBP of
several slices through the batched path -- each stage against the FP64
oracle's restatement (the reference has no 3-D phantoms and no equilinear
180LI, so parity is with the restatement only).  Tolerances: ray-sums and
images rel-L2 <= 1e-5; the interpolation, fed the same FP32 sinogram, to
1e-6 of the largest sample (FP64 weights on both sides; the device's atan may
differ from the host's in the last bit)."""
import os
import sys

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

ROT = 3.0          # rotations
NV_ROT = 120       # views per rotation
NDET = 129


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
    import pyoracle as po
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    ell = phantoms.random_ellipsoids(seed=5, n=8, z_half=1.0)
    foot = phantoms.ellipsoid_footprint(ell)
    nview = int(ROT * NV_ROT)
    z0, dz = -1.0, 2.0 / nview
    sc = cg.Scanner(phantoms.make_phantom(foot), "equilinear", NDET, nview,
                    rotAngle=ROT * 2 * np.pi)
    osc = po.Scanner(po.Phantom(elements=foot), "equilinear", NDET, nview, rotangle=ROT)
    sino = device.alloc_sinogram(nview, NDET)
    ang = device.raysums_ellipsoids(sc, ell, z0, dz, sino)
    cg.sync()
    ref, ref_ang = po.collect_ellipsoids(osc, ell, z0, dz)
    return dict(torch=torch, po=po, cg=cg, device=device, sc=sc, osc=osc, sino=sino, ang=ang,
                ref=ref, ref_ang=ref_ang, ell=ell)


def test_ellipsoid_scan_matches_oracle(setup):
    S = setup
    g = S["sc"].geometry()
    out = S["sino"][:, :g.n_det].cpu().numpy()
    np.testing.assert_allclose(S["ang"], S["ref_ang"], rtol=0, atol=1e-12)
    assert np.abs(S["ref"]).max() > 0.1
    e = rel_l2(out, S["ref"])
    print("3-D ellipsoid helical scan: rel-L2 %.3g" % e)
    assert e < 1e-5, e


@pytest.mark.parametrize("interp_view", [-1, 200])
def test_equilinear_180li_and_feather_match_oracle(setup, interp_view):
    S = setup
    po, device = S["po"], S["device"]
    g = S["sc"].geometry()
    data = S["sino"][:, :g.n_det].cpu().numpy()
    out, ang = device.helical180li(g, S["sino"], interp_view, equilinear=True)
    S["cg"].sync()
    og = S["osc"].geom()
    ref, ref_ang = po.helical180li(og, data, interp_view, allow_equilinear=True)
    np.testing.assert_allclose(ang, ref_ang, rtol=0, atol=1e-12)
    o = out[:, :g.n_det].cpu().numpy()
    assert np.abs(o - ref).max() <= 1e-6 * np.abs(ref).max()
    # the reference refuses equilinear data in its own entry point
    with pytest.raises(S["cg"].CtgpuError):
        device.helical180li(g, S["sino"], interp_view)
    gh = S["cg"].Geometry.from_buffer_copy(g)
    gh.n_view = out.shape[0]
    device.halfscan_feather(gh, out, equilinear=True)
    S["cg"].sync()
    og.nView = out.shape[0]
    fref = po.halfscan_feather(og, ref, true_gamma=True)
    f = out[:, :g.n_det].cpu().numpy()
    assert np.abs(f - fref).max() <= 2e-6 * np.abs(fref).max()


def test_slices_fbp_through_batch_matches_oracle(setup):
    """z-interpolate at several slice positions, feather, and reconstruct all
    slices in one ctgpu_batch (each slice has its own view angles)."""
    S = setup
    torch, po, cg, device = S["torch"], S["po"], S["cg"], S["device"]
    g = S["sc"].geometry()
    og = S["osc"].geom()
    data = S["sino"][:, :g.n_det].cpu().numpy()
    views = [130, 180, 230]
    n = 48
    probs, refs = [], []
    for iv in views:
        out, ang = device.helical180li(g, S["sino"], iv, equilinear=True)
        gh = cg.Geometry.from_buffer_copy(g)
        gh.n_view = out.shape[0]
        device.halfscan_feather(gh, out, equilinear=True)
        probs.append(dict(geometry=gh, nx=n, ny=n, sino=out, angles=ang,
                          image=torch.zeros((n, n), device="cuda"), filter_name="shepp",
                          filter_param=-1.0, filter_method="fft", zeropad=2, interp="linear",
                          backproj="table"))
        r, rang = po.helical180li(og, data, iv, allow_equilinear=True)
        og2 = po.Geom(og.geometry, og.nDet, r.shape[0], og.rotInc, og.detInc, og.focalLength,
                      og.sourceDetectorLength, og.viewDiameter, og.fanBeamAngle)
        r = po.halfscan_feather(og2, r, true_gamma=True)
        refs.append(po.reconstruct(og2, r, rang, n, n, filter_name="shepp", param=-1.0,
                                   method="fft", zeropad=2, backproj="table", interp="linear"))
    batch = device.BatchPlan(probs, autotune=False, graph=False)
    batch.run()
    cg.sync()
    for q, r in zip(probs, refs):
        e = rel_l2(q["image"].cpu().numpy(), r)
        print("helical slice FBP: rel-L2 %.3g" % e)
        assert e < 1e-5, e


@pytest.mark.parametrize("equilinear", [False, True])
def test_helical_plan_equals_slice_by_slice(setup, equilinear):
    """ctgpu_helical_plan (tables once, all slices in one launch) gives the
    per-slice 180LI + feathering: bit for bit for the reference's equiangular
    case, to 1e-6 for the equilinear restatement (host vs device atan)."""
    S = setup
    torch, cg, device, phantoms = S["torch"], S["cg"], S["device"], None
    g = cg.Geometry.from_buffer_copy(S["sc"].geometry())
    if not equilinear:
        g.geometry = 1   # the same data read as equiangular, to exercise that path
    views = [100, 150, 151, 260]
    plan = device.HelicalPlan(g, g.n_view, equilinear=equilinear, feather=True)
    out, ang = plan.run(S["sino"], views)
    cg.sync()
    for z, iv in enumerate(views):
        o, a = device.helical180li(g, S["sino"], iv, equilinear=equilinear)
        gh = cg.Geometry.from_buffer_copy(g)
        gh.n_view = o.shape[0]
        device.halfscan_feather(gh, o, equilinear=equilinear)
        cg.sync()
        np.testing.assert_array_equal(ang[z], a)
        x, y = out[z, :, :g.n_det], o[:, :g.n_det]
        if equilinear:
            assert (x - y).abs().max().item() <= 1e-6 * y.abs().max().item()
        else:
            assert torch.equal(x, y), z
