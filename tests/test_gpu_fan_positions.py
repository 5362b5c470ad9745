"""Fan-beam positions of the table backprojector at the edges of their
formulation (GPU), against the FP64 oracle.

The (tile, view) records measure an equiangular pixel's angle from a
reference ray that meets the detector at an integer position: the tile
centre's ray turned back by up to one detector interval (a short series for
the turn's sine and cosine, `sincos` past 0.1 rad), which also widens the
range of the arctangent's argument.  Equilinear positions carry the anchor's
fraction and the detector scale in the numerator.  Tiles past the image's
edge are bounded by their own distance from the source, and a tile that
reaches the source takes the FP64 path for all its pixels.  These cases take
few detectors (turns of several tenths of a radian), short focal lengths
with coarse images (tiles past the image's corners around the source; the
z^15 series and atanf), image sides that are no multiple of the 32-pixel
tile, fine images (the z^5 / z^7 series), and every interpolation (nearest:
FP64 re-evaluation next to the rounding jumps), each image within 1e-5
rel-L2 of the FP64 reconstruction (libctsim/backprojectors.cpp:656-743, the
equiangular and equilinear BackprojectView).
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

CASES = [  # geometry, detectors, image side, focal length ratio, views
    ("equiangular", 5, 24, 2.0, 90),
    ("equiangular", 9, 40, 1.3, 90),
    ("equiangular", 65, 256, 2.0, 90),
    ("equiangular", 301, 1024, 3.0, 60),
    ("equiangular", 733, 300, 1.5, 90),
    ("equilinear", 5, 24, 2.0, 90),
    ("equilinear", 33, 96, 1.3, 90),
    ("equilinear", 257, 512, 2.0, 60),
    ("equilinear", 601, 300, 1.5, 90),
]


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


@pytest.mark.parametrize("interp", ["nearest", "linear", "cubic"])
@pytest.mark.parametrize("geo,nd,n,fl,nv", CASES)
def test_fan_positions_against_oracle(gpu, oracle, geo, nd, n, fl, nv, interp):
    torch, cg, device, phantoms = gpu
    elems = phantoms.random_ellipses(seed=nd + n, n=9)
    sc = cg.Scanner(phantoms.make_phantom(elems), geo, nd, nv, focalLengthRatio=fl)
    sino = device.alloc_sinogram(nv, nd)
    ang = device.raysums(sc, phantoms.make_phantom(elems), sino)
    plan = device.ReconPlan(sc.geometry(), n, n, "abs_hamming", 0.54, "fft", 2, "direct", interp,
                            1, "table")
    img = torch.full((n, n), float("nan"), device="cuda")
    plan.run(sino, ang, img)
    cg.sync()
    osc = oracle.Scanner(oracle.Phantom(elements=elems), geo, nd, nv, nsample=1, fl_ratio=fl)
    ref = oracle.reconstruct(osc.geom(), sino[:, :nd].cpu().numpy(), ang, n, n,
                             filter_name="abs_hamming", param=0.54, method="fft", zeropad=2,
                             backproj="table", interp=interp)
    got = img.cpu().numpy()
    assert np.isfinite(got).all()
    err = rel_l2(got, ref)
    assert err < 1e-5, err


@pytest.mark.parametrize("interp", ["nearest", "cubic"])
def test_fan_positions_in_one_batch(gpu, oracle, interp):
    """The same geometries as one uneven batch (one persistent launch over
    every problem's tiles): each image within 1e-5 rel-L2 of the FP64
    reconstruction."""
    torch, cg, device, phantoms = gpu
    probs, refs = [], []
    for geo, nd, n, fl, nv in CASES:
        elems = phantoms.random_ellipses(seed=nd + n + 7, n=9)
        sc = cg.Scanner(phantoms.make_phantom(elems), geo, nd, nv, focalLengthRatio=fl)
        sino = device.alloc_sinogram(nv, nd)
        ang = device.raysums(sc, phantoms.make_phantom(elems), sino)
        cg.sync()
        probs.append(dict(geometry=sc.geometry(), nx=n, ny=n, sino=sino, angles=ang,
                          image=torch.full((n, n), float("nan"), device="cuda"),
                          filter_name="abs_hamming", filter_param=0.54, filter_method="fft",
                          zeropad=2, interp=interp, backproj="table"))
        osc = oracle.Scanner(oracle.Phantom(elements=elems), geo, nd, nv, nsample=1, fl_ratio=fl)
        refs.append(oracle.reconstruct(osc.geom(), sino[:, :nd].cpu().numpy(), ang, n, n,
                                       filter_name="abs_hamming", param=0.54, method="fft",
                                       zeropad=2, backproj="table", interp=interp))
    batch = device.BatchPlan(probs, autotune=False, graph=False)
    batch.run()
    cg.sync()
    for case, q, ref in zip(CASES, probs, refs):
        got = q["image"].cpu().numpy()
        assert np.isfinite(got).all(), case
        err = rel_l2(got, ref)
        assert err < 1e-5, (case, err)


@pytest.mark.parametrize("geo", ["parallel", "equiangular", "equilinear"])
@pytest.mark.parametrize("nd", [2, 3, 4])
def test_few_detectors(gpu, oracle, geo, nd):
    """Two to four detectors: the cubic rows are all linear end intervals
    (libctsupport/interpolator.cpp:37-75), windows span the whole padded
    row; every interpolation against the FP64 reconstruction."""
    torch, cg, device, phantoms = gpu
    elems = phantoms.random_ellipses(seed=3, n=5)
    nv, n = 30, 20
    sc = cg.Scanner(phantoms.make_phantom(elems), geo, nd, nv)
    sino = device.alloc_sinogram(nv, nd)
    ang = device.raysums(sc, phantoms.make_phantom(elems), sino)
    cg.sync()
    osc = oracle.Scanner(oracle.Phantom(elements=elems), geo, nd, nv, nsample=1)
    for interp in ("nearest", "linear", "cubic"):
        plan = device.ReconPlan(sc.geometry(), n, n, "abs_hamming", 0.54, "fft", 2, "direct",
                                interp, 1, "table")
        img = torch.full((n, n), float("nan"), device="cuda")
        plan.run(sino, ang, img)
        cg.sync()
        ref = oracle.reconstruct(osc.geom(), sino[:, :nd].cpu().numpy(), ang, n, n,
                                 filter_name="abs_hamming", param=0.54, method="fft", zeropad=2,
                                 backproj="table", interp=interp)
        got = img.cpu().numpy()
        assert np.isfinite(got).all(), interp
        tol = 1e-5 * float(np.abs(ref).max()) + 1e-7
        assert float(np.abs(got - ref).max()) <= tol, interp
