"""Scanner geometry ratios (GPU) against the FP64 oracle: focal length,
centre-detector length, view and scan ratios across their useful range,
with several rays per detector (libctsim/scanner.cpp:86-224 sets the
geometry up from them, :295-419 collects the ray-sums).  For each geometry
the device's ray-sums and view angles against the oracle's, and the table
backprojection (cubic) of the device sinogram against the oracle's FP64
reconstruction of the same sinogram, each within 1e-5 rel-L2.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

RATIOS = [  # focal length, centre-detector length, view, scan; rays per detector
    (1.2, 2.0, 1.0, 1.0, 1),
    (1.5, 1.5, 1.0, 1.0, 2),
    (4.0, 3.0, 1.0, 1.0, 1),
    (10.0, 2.0, 1.0, 1.0, 1),
    (2.0, 2.0, 0.8, 1.0, 1),
    (2.0, 2.0, 1.5, 1.0, 3),
    (2.0, 2.0, 1.0, 0.7, 1),
    (2.0, 2.0, 1.0, 1.2, 2),
    (3.0, 1.2, 1.3, 0.9, 4),
]


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


@pytest.mark.parametrize("ratios", RATIOS)
@pytest.mark.parametrize("geo", ["parallel", "equiangular", "equilinear"])
def test_ratios_against_oracle(gpu, oracle, geo, ratios):
    torch, cg, device, phantoms = gpu
    fl, cd, vr, sr, ns = ratios
    nd, nv, n = 127, 120, 96
    elems = phantoms.random_ellipses(seed=11, n=8)
    sc = cg.Scanner(phantoms.make_phantom(elems), geo, nd, nv, nSample=ns, focalLengthRatio=fl,
                    centerDetectorRatio=cd, viewRatio=vr, scanRatio=sr)
    sino = device.alloc_sinogram(nv, nd)
    ang = device.raysums(sc, phantoms.make_phantom(elems), sino)
    cg.sync()
    osc = oracle.Scanner(oracle.Phantom(elements=elems), geo, nd, nv, nsample=ns, fl_ratio=fl,
                         cd_ratio=cd, view_ratio=vr, scan_ratio=sr)
    ref_sino, ref_ang = osc.collect()
    got = sino[:, :nd].cpu().numpy()
    assert np.array_equal(ang, ref_ang)
    assert rel_l2(got, ref_sino) < 1e-5, rel_l2(got, ref_sino)
    plan = device.ReconPlan(sc.geometry(), n, n, "abs_hamming", 0.54, "fft", 2, "direct", "cubic",
                            1, "table")
    img = torch.full((n, n), float("nan"), device="cuda")
    plan.run(sino, ang, img)
    cg.sync()
    ref = oracle.reconstruct(osc.geom(), got, ang, n, n, filter_name="abs_hamming", param=0.54,
                             method="fft", zeropad=2, backproj="table", interp="cubic")
    out = img.cpu().numpy()
    assert np.isfinite(out).all()
    assert rel_l2(out, ref) < 1e-5, rel_l2(out, ref)
