"""Many scans of uneven shapes in one ray launch
(ctgpu_collect_projections_multi): every geometry, 1-3 rays per detector,
detector counts from 101 to 1434, view counts from 60 to 1440, built-in,
file and random phantoms (all element types).  Each problem's sinogram and
view angles must equal, bit for bit, what ctgpu_collect_projections writes for
the problem alone (the same records and arithmetic per ray), which the
reference-pinned tests cover."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


def test_multi_scan_equals_single_scans(gpu):
    torch, cg, device, phantoms = gpu
    import os
    specs = [  # phantom, geometry, nDet, nView, nSample, Scanner kwargs
        (cg.Phantom("herman"), "parallel", 101, 60, 2, {}),
        (cg.Phantom("shepp-logan"), "equiangular", 133, 96, 1, {}),
        (cg.Phantom.from_file(os.path.join(GOLDEN, "elements.phm")), "equilinear", 131, 100, 2,
         {}),
        (phantoms.make_phantom(phantoms.random_ellipses(seed=2, n=12)), "equiangular", 733, 720,
         1, {}),
        (phantoms.make_phantom(phantoms.random_ellipses(seed=5, n=20)), "parallel", 1434, 1440,
         1, {}),
        (cg.Phantom("shepp-logan"), "equiangular", 134, 90, 3, {}),
        (cg.Phantom("shepp-logan"), "equilinear", 97, 64, 1,
         {"focalLengthRatio": 3.0, "centerDetectorRatio": 1.5, "viewRatio": 1.2,
          "scanRatio": 0.9}),
        (cg.Phantom.from_file(os.path.join(GOLDEN, "elements.phm")), "parallel", 121, 90, 2, {}),
    ]
    scs = [cg.Scanner(ph, geo, nd, nv, nSample=ns, **kw) for ph, geo, nd, nv, ns, kw in specs]
    phs = [sp[0] for sp in specs]
    multi = [torch.full((sc.geometry().n_view, device.pitch_for(sc.geometry().n_det)),
                        float("nan"), device="cuda") for sc in scs]
    angs = device.raysums_multi(scs, phs, multi)
    cg.sync()
    for k, (sc, ph) in enumerate(zip(scs, phs)):
        g = sc.geometry()
        one = device.alloc_sinogram(g.n_view, g.n_det)
        a1 = device.raysums(sc, ph, one)
        cg.sync()
        np.testing.assert_array_equal(angs[k], a1)
        assert torch.equal(multi[k][:, :g.n_det], one[:, :g.n_det]), k
        assert float(one[:, :g.n_det].abs().max()) > 0
    # a second call in a row (staging buffers reused) gives the same
    again = [torch.zeros_like(t) for t in multi]
    device.raysums_multi(scs, phs, again)
    cg.sync()
    for k, sc in enumerate(scs):
        n = sc.geometry().n_det
        assert torch.equal(again[k][:, :n], multi[k][:, :n]), k


def test_multi_scan_rejects_unit_pulse(gpu):
    torch, cg, device, phantoms = gpu
    ph = cg.Phantom("unit-pulse")
    sc = cg.Scanner(ph, "parallel", 65, 8)
    with pytest.raises(cg.CtgpuError) as ei:
        device.raysums_multi([sc], [ph], [device.alloc_sinogram(8, 65)])
    assert ei.value.code == 2
