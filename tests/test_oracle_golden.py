"""The FP64 oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from CTSim compiled from source)."""
import numpy as np
import pytest

from conftest import rel_l2

SCANS = ["c1", "herman_par", "shepp_eqa", "shepp_eqa_even", "herman_eql", "herman_eqa",
         "shepp_par_even", "pulse_par", "shepp_eql_ratio"]
SCAN_ARGS = {  # phantom, geometry, nray, extra Scanner kwargs (tests/golden/make_golden.py)
    "c1": ("shepp-logan", "parallel", 2, {}),
    "herman_par": ("herman", "parallel", 2, {}),
    "shepp_eqa": ("shepp-logan", "equiangular", 1, {}),
    "shepp_eqa_even": ("shepp-logan", "equiangular", 3, {}),
    "herman_eql": ("herman", "equilinear", 2, {}),
    "herman_eqa": ("herman", "equiangular", 1, {}),
    "shepp_par_even": ("shepp-logan", "parallel", 1, {"offset_view": 3}),
    "pulse_par": ("unit-pulse", "parallel", 1, {}),
    "shepp_eql_ratio": ("shepp-logan", "equilinear", 1,
                        {"fl_ratio": 3.0, "cd_ratio": 1.5, "view_ratio": 1.2, "scan_ratio": 0.9}),
}


def geom_from_hdr(po, hdr):
    g, nd, nv, _rs, ri, _ds, di, vd, fl, sdl, fan = hdr
    return po.Geom(int(g), int(nd), int(nv), ri, di, fl, sdl, vd, fan)


@pytest.mark.parametrize("name", SCANS)
def test_oracle_raysums_match_reference(oracle, golden, name):
    d = golden("scans")
    phm, geo, nray, kw = SCAN_ARGS[name]
    hdr = d[name + "/hdr"]
    sc = oracle.Scanner(oracle.Phantom(phm), geo, int(hdr[1]), int(hdr[2]), nsample=nray, **kw)
    assert sc.detInc == hdr[6] and sc.viewDiameter == hdr[7] and sc.fanBeamAngle == hdr[10]
    sino, ang = sc.collect()
    np.testing.assert_array_equal(ang, d[name + "/angles"])
    ref = d[name + "/data"]
    # the reference stores FP32; the oracle's FP64 sums round to the same floats
    mism = np.count_nonzero(sino.astype(np.float32) != ref)
    assert mism <= max(1, ref.size // 100000), mism
    assert rel_l2(sino, ref) < 1e-7


def test_oracle_reconstructions_match_reference(oracle, golden):
    scans = golden("scans")
    rec = golden("recons")
    n = len([k for k in rec.files if k.endswith("/cfg")])
    for k in range(n):
        sc, nx, ny, bp, ip, flt, meth, zp, gen, prm = rec["%d/cfg" % k]
        g = geom_from_hdr(oracle, scans[sc + "/hdr"])
        img = oracle.reconstruct(g, scans[sc + "/data"], scans[sc + "/angles"], int(nx), int(ny),
                                 filter_name=flt, param=float(prm), method=meth, zeropad=int(zp),
                                 generation=gen, backproj=bp, interp=ip)
        ref = rec["%d/image64" % k]
        scale = np.abs(ref).max()
        np.testing.assert_allclose(img, ref, rtol=0, atol=1e-12 * scale,
                                   err_msg="case %d %s" % (k, rec["%d/cfg" % k]))
        # and the reference's shipped FP32-image build differs from FP64 only by rounding
        assert rel_l2(rec["%d/image32" % k], ref) < 2e-6


def test_oracle_filters_match_reference(oracle, golden):
    d = golden("filters")
    x = d["input"]
    names = {0: "parallel", 1: "equiangular", 2: "equilinear"}
    for k, (gid, fl, sdl, f, m, gen, zp) in enumerate(d["cases"]):
        ps = oracle.ProcessSignal(f, m, x.shape[1], 0.0123, param=0.54, generation=gen,
                                  zeropad=int(zp), geometry=names[int(gid)], focal_length=fl,
                                  sdl=sdl)
        out = ps.filter(x)
        ref = d["%d" % k]
        scale = max(np.abs(ref).max(), 1e-300)
        np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * scale,
                                   err_msg="case %s" % (d["cases"][k],))


def test_oracle_fft_method_equals_fourier(oracle):
    rng = np.random.default_rng(5)
    x = rng.random((3, 45)).astype(np.float32)
    for geo in ("parallel", "equiangular", "equilinear"):
        a = oracle.ProcessSignal("abs_hamming", "fourier", 45, 0.01, param=0.54, zeropad=2,
                                 geometry=geo, focal_length=2.0, sdl=4.0).filter(x)
        b = oracle.ProcessSignal("abs_hamming", "fft", 45, 0.01, param=0.54, zeropad=2,
                                 geometry=geo, focal_length=2.0, sdl=4.0).filter(x)
        np.testing.assert_allclose(b, a, rtol=0, atol=1e-11 * np.abs(a).max())


def test_oracle_helical_matches_reference(oracle, golden):
    d = golden("helical")
    for k in range(2):
        g = geom_from_hdr(oracle, d["%d/in_hdr" % k])
        h, ang = oracle.helical180li(g, d["%d/in_data" % k], int(d["%d/interpview" % k]))
        np.testing.assert_array_equal(ang, d["%d/out_angles" % k])
        g.nView = h.shape[0]
        f = oracle.halfscan_feather(g, h)
        np.testing.assert_array_equal(f, d["%d/out_data" % k])


def test_oracle_raster_matches_reference(oracle, golden):
    d = golden("raster")
    for k in range(3):
        phm, n, ns = d["%d/cfg" % k]
        img, _ = oracle.phantom_to_image(oracle.Phantom(phm), int(n), int(n), 1.0, int(ns))
        np.testing.assert_allclose(img, d["%d/image" % k], rtol=0, atol=1e-12)


def test_oracle_projector_is_adjoint_of_backprojector(oracle, golden):
    scans = golden("scans")
    g = geom_from_hdr(oracle, scans["herman_par/hdr"])
    ang = scans["herman_par/angles"]
    rng = np.random.default_rng(1)
    x = rng.standard_normal((24, 20))
    y = rng.standard_normal((len(ang), g.nDet))
    ax = oracle.project_image(g, x, ang)
    bty = oracle.backproject(g, y, ang, 24, 20, "table", "linear", post_process=False)
    assert abs(np.vdot(ax, y) - np.vdot(x, bty)) < 1e-12 * abs(np.vdot(ax, y))


@pytest.mark.parametrize("name", ["shepp_eqa", "shepp_eqa_even", "herman_eql", "herman_eqa",
                                  "shepp_eql_ratio"])
def test_oracle_interpolate_to_parallel(oracle, golden, name):
    """ora_interpolate_to_parallel bit for bit against the reference's
    Projections::interpolateToParallel on the same scan."""
    d, r = golden("scans"), golden("rebin")
    h = d[name + "/hdr"]
    g = oracle.Geom(int(h[0]), int(h[1]), int(h[2]), h[4], h[6], h[8], h[9], h[7], h[10])
    out, ang, hdr = oracle.interpolate_to_parallel(g, h[3], h[5], d[name + "/data"],
                                                   d[name + "/angles"])
    rh = r[name + "/hdr"]
    assert hdr == (rh[4], rh[5], rh[6])
    np.testing.assert_array_equal(ang, r[name + "/angles"])
    np.testing.assert_array_equal(out, r[name + "/data"])


@pytest.mark.parametrize("k", range(5))
def test_oracle_image_compare_matches_reference(oracle, golden, k):
    """ImageFile::comparativeStatistics restated: the same numbers, bit for bit."""
    g = golden("io")
    assert oracle.image_compare(g["comp/%d/a" % k], g["comp/%d/b" % k]) == \
        tuple(g["comp/%d/dre" % k])


@pytest.mark.parametrize("name", ["herman_eql", "shepp_eqa_even", "pulse_par"])
def test_file_formats_restated(golden, tmp_path, name):
    """The host restatement of the .pj layout rewrites the reference's file byte
    for byte, and pj2if is the view-reversed transpose of its data."""
    from ctsim_gb300.fileio import read_pj, write_pj
    g = golden("io")
    src = tmp_path / "in.pj"
    src.write_bytes(g[name + "/pj"].tobytes())
    pj = read_pj(src)
    out = tmp_path / "out.pj"
    write_pj(out, pj)
    assert out.read_bytes() == src.read_bytes()
    np.testing.assert_array_equal(pj.data[::-1].T, g[name + "/pj2if"])


@pytest.mark.parametrize("k", range(7))
def test_oracle_convert_polar_matches_reference(oracle, golden, k):
    """Projections::convertPolar restated: the reference's image bit for bit
    (columns the reference's loop writes)."""
    d = golden("polar")
    name, nx, ny, interp = d["%d/cfg" % k]
    hdr = d["%d/hdr" % k]
    out = oracle.convert_polar(geom_from_hdr(oracle, hdr), hdr[3], hdr[5], d["%d/data" % k],
                               d["%d/angles" % k], int(nx), int(ny), interp)
    c = min(int(nx), int(ny))
    np.testing.assert_array_equal(out[:c], d["%d/image" % k][:c])


PHM_FILES = {"elements": ("tests", "golden", "elements.phm")}


def test_oracle_phantom_file_raysums_match_reference(oracle, golden, tmp_path):
    """Phantom files (Phantom::createFromFile) with every element type at
    non-zero attenuation -- rectangles, sectors, a segment, a triangle, an
    ellipse -- and a seeded random-ellipse phantom written by
    phantoms.write_phm, scanned by the reference's phm2pj --phmfile."""
    import os
    from conftest import ROOT
    from ctsim_gb300.phantoms import random_ellipses, write_phm
    d = golden("phmfile")
    rnd = tmp_path / "random12.phm"
    write_phm(str(rnd), random_ellipses(seed=2, n=12))
    assert rnd.read_text() == str(d["random12/text"])   # the seeded draw is reproducible
    files = {"elements": os.path.join(ROOT, *PHM_FILES["elements"]), "random12": str(rnd)}
    types = {e[0] for e in oracle.read_phm(files["elements"])}
    assert types == {"rectangle", "sector", "segment", "triangle", "ellipse"}
    for name in ("el_par", "el_eqa", "el_eql", "rnd_eqa"):
        phm, geo, nd, nv, nr = d[name + "/cfg"]
        sc = oracle.Scanner(oracle.Phantom(filename=files[phm]), geo, int(nd), int(nv),
                            nsample=int(nr))
        hdr = d[name + "/hdr"]
        assert sc.detInc == hdr[6] and sc.viewDiameter == hdr[7] and sc.fanBeamAngle == hdr[10]
        sino, ang = sc.collect()
        np.testing.assert_array_equal(ang, d[name + "/angles"])
        ref = d[name + "/data"]
        assert np.abs(ref).max() > 0.1
        mism = np.count_nonzero(sino.astype(np.float32) != ref)
        assert mism <= max(1, ref.size // 100000), (name, mism)
        assert rel_l2(sino, ref) < 1e-7, name


def test_oracle_phantom_file_raster_matches_reference(oracle, golden):
    import os
    from conftest import ROOT
    d = golden("phmfile")
    ph = oracle.Phantom(filename=os.path.join(ROOT, *PHM_FILES["elements"]))
    for k in range(2):
        n, ns = d["raster%d/cfg" % k]
        img, _ = oracle.phantom_to_image(ph, int(n), int(n), 1.0, int(ns))
        np.testing.assert_allclose(img, d["raster%d/image" % k], rtol=0, atol=1e-12)


def test_oracle_roi_reconstructions_match_reference(oracle, golden):
    """Backprojection restricted to a region of interest (ReconstructionROI,
    libctsim/backprojectors.cpp:284-315), including a swapped and a clamped
    ROI, against the reference's FP64-image build fed the same filtered rows."""
    scans = golden("scans")
    d = golden("roi")
    k = 0
    while "%d/cfg" % k in d:
        name, nx, ny, bp, ip = d["%d/cfg" % k]
        g = geom_from_hdr(oracle, scans[name + "/hdr"])
        ps = oracle.ProcessSignal("abs_bandlimit", "convolution", g.nDet, g.detInc,
                                  geometry=int(g.geometry), focal_length=g.focalLength,
                                  sdl=g.sourceDetectorLength)
        filt = ps.filter(scans[name + "/data"])
        img = oracle.backproject(g, filt, scans[name + "/angles"], int(nx), int(ny), bp, ip,
                                 roi=d["%d/roi" % k])
        ref = d["%d/image64" % k]
        np.testing.assert_allclose(img, ref, rtol=0, atol=1e-12 * np.abs(ref).max(),
                                   err_msg=str(d["%d/cfg" % k]))
        k += 1
    assert k == 6


def test_oracle_phantom_grows_past_its_initial_room(oracle):
    """A phantom of more elements than its initial room (256): the element list
    grows, keeps the reference's order (last added first), and a ray's sum is
    the sum of the elements' own sums."""
    rng = np.random.default_rng(3)
    elems = [("ellipse", float(x), float(y), 0.02, 0.03, 0.0, 1.0)
             for x, y in rng.uniform(-0.9, 0.9, size=(600, 2))]
    big = oracle.Phantom(elements=elems)
    assert len(big.bboxes()) == 600
    # the list's first element is the last one added
    x0, y0 = elems[-1][1], elems[-1][2]
    b = big.bboxes()[0]
    assert b[0] <= x0 <= b[2] and b[1] <= y0 <= b[3]
    total = big.raysum(-2.0, 0.1, 2.0, 0.1)
    parts = sum(oracle.Phantom(elements=[e]).raysum(-2.0, 0.1, 2.0, 0.1) for e in elems)
    assert abs(total - parts) <= 1e-12 * max(1.0, abs(parts))
