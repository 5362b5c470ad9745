"""Projections::interpolateToParallel on the device (GPU) against the FP64
oracle over the scanner's geometry ratios (libctsim/projections.cpp:
1250-1328): fan-beam scans of both detector shapes at several focal lengths,
centre-detector, view and scan ratios, rebinned from the device sinogram;
the parallel angles and header equal, the rows within 1e-6 of the largest
value, as for the reference's own scans."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RATIOS = [(2.0, 2.0, 1.0, 1.0), (1.3, 1.5, 1.0, 1.0), (4.0, 3.0, 1.3, 0.9), (2.0, 2.0, 1.0, 0.7),
          (10.0, 1.2, 0.8, 1.2)]


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


@pytest.mark.parametrize("ratios", RATIOS)
@pytest.mark.parametrize("geo,nd", [("equiangular", 127), ("equilinear", 128)])
def test_rebin_ratios_against_oracle(gpu, oracle, geo, nd, ratios):
    torch, cg, device, phantoms = gpu
    fl, cd, vr, sr = ratios
    nv = 120
    elems = phantoms.random_ellipses(seed=23, n=8)
    sc = cg.Scanner(phantoms.make_phantom(elems), geo, nd, nv, focalLengthRatio=fl,
                    centerDetectorRatio=cd, viewRatio=vr, scanRatio=sr)
    sino = device.alloc_sinogram(nv, nd)
    ang = device.raysums(sc, phantoms.make_phantom(elems), sino)
    cg.sync()
    g = sc.geometry()
    out, g2, ang2 = device.interpolate_to_parallel(g, sino, ang)
    cg.sync()
    osc = oracle.Scanner(oracle.Phantom(elements=elems), geo, nd, nv, nsample=1, fl_ratio=fl,
                         cd_ratio=cd, view_ratio=vr, scan_ratio=sr)
    host = sino[:, :nd].cpu().numpy()
    ref, ref_ang, hdr = oracle.interpolate_to_parallel(osc.geom(), g.rot_start, g.det_start, host,
                                                       ang)
    np.testing.assert_array_equal(ang2, ref_ang)
    assert (g2.geometry, g2.rot_inc, g2.det_start, g2.det_inc) == (0,) + tuple(hdr)
    o = out[:, :nd].cpu().numpy()
    err = np.abs(o - ref).max() / np.abs(ref).max()
    assert err <= 1e-6, err
