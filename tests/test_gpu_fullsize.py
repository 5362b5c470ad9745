"""Full-size configurations against the FP64 oracle (GPU).

Fan-beam: 12 seeded random ellipses, equiangular, 733 detectors x 720 views
over 360 degrees, focal length 2 view radii, abs_hamming 0.54 by FFT with
zeropad 2, cubic interpolation, 512 x 512 image.  Tolerance rel-L2 <= 1e-5
against FP64 for both the sinogram and the image."""
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
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


def test_fan_beam_c2_full_size(gpu, oracle):
    torch, cg, device, phantoms = gpu
    elems = phantoms.random_ellipses(seed=2, n=12)
    ph = phantoms.make_phantom(elems)
    sc = cg.Scanner(ph, "equiangular", 733, 720, nSample=1)
    g = sc.geometry()
    sino = device.alloc_sinogram(720, 733)
    ang = device.raysums(sc, ph, sino)
    plan = device.ReconPlan(g, 512, 512, "abs_hamming", 0.54, "fft", 2, "direct", "cubic", 1,
                            "table")
    img = torch.zeros((512, 512), device="cuda")
    plan.run(sino, ang, img)
    cg.sync()
    s_gpu = sino[:, :733].cpu().numpy()

    oph = oracle.Phantom(elements=elems)
    osc = oracle.Scanner(oph, "equiangular", 733, 720, nsample=1)
    s_ref, a_ref = osc.collect()
    np.testing.assert_array_equal(ang, a_ref)
    e_s = rel_l2(s_gpu, s_ref)
    assert e_s < 1e-5, e_s
    # reconstruct the reference's FP32-stored sinogram with the oracle in FP64
    i_ref = oracle.reconstruct(osc.geom(), s_ref.astype(np.float32), a_ref, 512, 512,
                               filter_name="abs_hamming", param=0.54, method="fft", zeropad=2,
                               backproj="table", interp="cubic")
    # and the GPU's from the same FP32 sinogram
    plan.run(device.alloc_sinogram(720, 733).copy_(
        torch.nn.functional.pad(torch.from_numpy(s_ref.astype(np.float32)), (0, 3)).cuda()),
        a_ref, img)
    cg.sync()
    e_i = rel_l2(img.cpu().numpy(), i_ref)
    print("equiangular 733 x 720 -> 512^2: sinogram rel-L2 %.3g, image rel-L2 %.3g" % (e_s, e_i))
    assert e_i < 1e-5, e_i


@pytest.mark.parametrize("bp,interp", [("idiff", "linear"), ("table", "nearest"),
                                       ("diff", "cubic"), ("trig", "linear")])
def test_parallel_512_full_size(gpu, oracle, bp, interp):
    torch, cg, device, phantoms = gpu
    ph = cg.Phantom("shepp-logan")
    sc = cg.Scanner(ph, "parallel", 733, 720, nSample=2)
    g = sc.geometry()
    sino = device.alloc_sinogram(720, 733)
    ang = device.raysums(sc, ph, sino)
    plan = device.ReconPlan(g, 512, 512, "abs_bandlimit", -1, "convolution", 1, "direct", interp,
                            1, bp)
    img = torch.zeros((512, 512), device="cuda")
    plan.run(sino, ang, img)
    cg.sync()
    s = sino[:, :733].cpu().numpy()
    i_ref = oracle.reconstruct(
        oracle.Geom(g.geometry, g.n_det, g.n_view, g.rot_inc, g.det_inc, g.focal_length,
                    g.source_detector_length, g.view_diameter, g.fan_beam_angle),
        s, ang, 512, 512, backproj=bp, interp=interp)
    e = rel_l2(img.cpu().numpy(), i_ref)
    print("parallel 733x720 -> 512^2 %s/%s image rel-L2 %.3g" % (bp, interp, e))
    assert e < 1e-5, e
