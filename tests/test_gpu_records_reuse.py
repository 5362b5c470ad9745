"""ctgpu_recon_run keeps the (tile, view) records of its last call and builds
them again only for other view angles (GPU).

Every image must equal, bit for bit, the one a fresh plan makes for the same
sinogram and angles: the same angles again, other angles, a view sub-range,
and calls of the other entry points (the batched run, the host-buffer batch,
the plain backprojection) that rewrite the plan's scratch in between.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


@pytest.mark.parametrize("geo,interp", [("equiangular", "cubic"), ("parallel", "linear"),
                                        ("equilinear", "nearest")])
def test_records_follow_the_angles(gpu, geo, interp):
    torch, cg, device, phantoms = gpu
    nd, nv, side = 367, 360, 96
    ph = phantoms.make_phantom(phantoms.random_ellipses(seed=31, n=10))
    sc = cg.Scanner(ph, geo, nd, nv)
    sino = device.alloc_sinogram(nv, nd)
    ang = np.asarray(device.raysums(sc, ph, sino), np.float64)
    other = ang + 0.0123

    def make():
        return device.ReconPlan(sc.geometry(), side, side, "abs_hamming", 0.54, "fft", 2,
                                "direct", interp, 1, "table")

    def fresh(a, start=0, n=-1):
        out = torch.full((side, side), float("nan"), device="cuda")
        make().run(sino, a, out, start_view=start, n_views=n)
        cg.sync()
        return out

    refs = {"a": fresh(ang), "b": fresh(other), "sub": fresh(ang, 40, 200)}
    plan = make()
    out = torch.full((side, side), float("nan"), device="cuda")

    def check(key, a, start=0, n=-1):
        out.fill_(float("nan"))
        plan.run(sino, a, out, start_view=start, n_views=n)
        cg.sync()
        assert torch.equal(out, refs[key]), key

    check("a", ang)
    check("a", ang)            # records kept
    check("b", other)          # other angles: rebuilt
    check("a", ang)
    check("sub", ang, 40, 200)  # fewer views
    check("a", ang)
    # the batched run rebuilds the records in the same scratch
    sinos = sino[None].contiguous()
    imgs = torch.zeros((1, side, side), device="cuda")
    plan.run_batch(sinos, other, imgs)
    cg.sync()
    check("a", ang)
    # so does the plain backprojection of filtered rows
    filt = torch.zeros_like(sino)
    plan.filter(sino, filt)
    plan.backproject(filt, other, torch.zeros((side, side), device="cuda"))
    cg.sync()
    check("a", ang)
    # and the host-buffer batch
    h = plan.run_batch_host(np.ascontiguousarray(sino[:, :nd].cpu().numpy())[None], other)
    assert np.isfinite(h).all()
    check("a", ang)
