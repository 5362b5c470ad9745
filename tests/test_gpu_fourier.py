"""Polar and direct-Fourier images on the device against the reference and the
FP64 oracle.

- convertPolar: against the reference's own images (tests/golden/polar.npz,
  from ref_harness polar).  The reference's arithmetic is FP64 and is
  repeated in FP64; only atan2 may differ in its last bit, so bilinear pixels
  agree to 1e-6 of the image's range and nearest pixels to the sample either
  side of a rounding boundary (>= 99 % identical).
- convertFFTPolar, ifft + magnitude, the Fourier reconstruction: the
  reference needs FFTW (absent), so these are checked against the oracle's
  FP64 restatement; the device's transforms are FP32, bar rel-L2 <= 2e-5
  (the FFT's rounding grows with log N, the direct DFT's with sqrt N)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device
    return torch, cg, device


def geometry(cg, hdr):
    g, nd, nv, rs, ri, ds, di, vd, fl, sdl, fan = hdr
    return cg.Geometry(int(g), int(nd), int(nv), 0, rs, ri, ds, di, vd, fl, sdl, fan)


def oracle_geom(po, hdr):
    g, nd, nv, _rs, ri, _ds, di, vd, fl, sdl, fan = hdr
    return po.Geom(int(g), int(nd), int(nv), ri, di, fl, sdl, vd, fan)


def upload(torch, device, data):
    nv, nd = data.shape
    s = torch.zeros((nv, device.pitch_for(nd)), dtype=torch.float32, device="cuda")
    s[:, :nd] = torch.from_numpy(np.ascontiguousarray(data)).cuda()
    return s


@pytest.mark.parametrize("k", range(7))
def test_convert_polar_matches_reference(gpu, golden, k):
    torch, cg, device = gpu
    d = golden("polar")
    name, nx, ny, interp = d["%d/cfg" % k]
    nx, ny = int(nx), int(ny)
    g = geometry(cg, d["%d/hdr" % k])
    img = device.convert_polar(g, upload(torch, device, d["%d/data" % k]), d["%d/angles" % k],
                               nx, ny, interp).cpu().numpy()
    ref = d["%d/image" % k]
    c = min(nx, ny)
    assert not img[c:].any()   # columns the reference's loop never reaches
    a, b = img[:c], ref[:c]
    span = float(np.abs(ref).max())
    if interp == "bilinear":
        assert np.abs(a - b).max() <= 1e-6 * span, (name, np.abs(a - b).max())
    else:
        assert (a == b).mean() >= 0.99, (name, (a == b).mean())


def test_convert_polar_large_against_oracle(gpu, golden, oracle):
    """a 733 x 720 equiangular scan rebinned, 256 x 256 and 300 x 200 polar images"""
    torch, cg, device = gpu
    from ctsim_gb300 import phantoms
    ph = phantoms.make_phantom(phantoms.random_ellipses(seed=5, n=12))
    sc = cg.Scanner(ph, "equiangular", 733, 720)
    sino = device.alloc_sinogram(720, 733)
    ang = device.raysums(sc, ph, sino)
    g = sc.geometry()
    data = sino[:, :733].cpu().numpy()
    og = oracle.Geom(g.geometry, g.n_det, g.n_view, g.rot_inc, g.det_inc, g.focal_length,
                     g.source_detector_length, g.view_diameter, g.fan_beam_angle)
    for nx, ny, interp in ((256, 256, "bilinear"), (300, 200, "nearest")):
        img = device.convert_polar(g, sino, ang, nx, ny, interp).cpu().numpy()
        ref = oracle.convert_polar(og, g.rot_start, g.det_start, data, ang, nx, ny, interp)
        if interp == "bilinear":
            assert np.abs(img - ref).max() <= 1e-6 * np.abs(ref).max()
        else:
            assert (img == ref).mean() >= 0.99


@pytest.mark.parametrize("name,nx,ny,interp,zeropad", [
    ("herman_par", 48, 48, "bilinear", 1), ("herman_par", 40, 40, "nearest", 2),
    ("shepp_eqa", 36, 36, "bilinear", 0), ("shepp_par_even", 33, 31, "bilinear", 1),
    ("herman_eql", 32, 32, "nearest", 0)])
def test_convert_fft_polar_against_oracle(gpu, golden, oracle, name, nx, ny, interp, zeropad):
    torch, cg, device = gpu
    d = golden("scans")
    hdr = d[name + "/hdr"]
    g = geometry(cg, hdr)
    re, im, n = device.convert_fft_polar(g, upload(torch, device, d[name + "/data"]),
                                         d[name + "/angles"], nx, ny, interp, zeropad)
    rr, ri, n_ref = oracle.convert_fft_polar(oracle_geom(oracle, hdr), hdr[3], hdr[5],
                                             d[name + "/data"], d[name + "/angles"], nx, ny,
                                             interp, zeropad)
    assert n == n_ref
    got = re.cpu().numpy() + 1j * im.cpu().numpy()
    want = rr + 1j * ri
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err <= 2e-5, err


@pytest.mark.parametrize("nx,ny", [(64, 64), (48, 40), (37, 64), (256, 128)])
def test_ifft_magnitude_against_oracle(gpu, oracle, nx, ny):
    torch, cg, device = gpu
    rng = np.random.default_rng(nx * 1000 + ny)
    re = rng.standard_normal((nx, ny)).astype(np.float32)
    im = rng.standard_normal((nx, ny)).astype(np.float32)
    got = device.image_ifft_magnitude(torch.from_numpy(re).cuda(),
                                      torch.from_numpy(im).cuda()).cpu().numpy()
    want = oracle.ifft_magnitude(re, im)
    assert rel_l2(got, want) <= 2e-5, rel_l2(got, want)


@pytest.mark.parametrize("name,zeropad", [("herman_par", 1), ("shepp_eqa", 2)])
def test_reconstruct_fourier_against_oracle(gpu, golden, oracle, name, zeropad):
    torch, cg, device = gpu
    d = golden("scans")
    hdr = d[name + "/hdr"]
    g = geometry(cg, hdr)
    got = device.reconstruct_fourier(g, upload(torch, device, d[name + "/data"]),
                                     d[name + "/angles"], 64, 64, "bilinear",
                                     zeropad).cpu().numpy()
    want = oracle.reconstruct_fourier(oracle_geom(oracle, hdr), hdr[3], hdr[5],
                                      d[name + "/data"], d[name + "/angles"], 64, 64, "bilinear",
                                      zeropad)
    assert rel_l2(got, want) <= 2e-5, rel_l2(got, want)


def test_polar_rejects_unknown_interpolation(gpu, golden):
    torch, cg, device = gpu
    d = golden("scans")
    g = geometry(cg, d["herman_par/hdr"])
    with pytest.raises(cg.CtgpuError) as ei:
        device.convert_polar(g, upload(torch, device, d["herman_par/data"]), None, 16, 16,
                             "bicubic")
    assert ei.value.code == 1
