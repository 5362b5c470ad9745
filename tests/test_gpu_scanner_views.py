"""A scanner keeps its views' ray records on the device and rebuilds them only
for another view range (GPU).

Every scan must equal, bit for bit, the same scan by a fresh scanner: one
scanner object is used for full scans, view sub-ranges with and without an
offset view, the batched and the multi-scan entry points, and 3-D ellipsoid
scans, in an order that changes the view range between calls and returns to
earlier ones.
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


@pytest.mark.parametrize("geo,ns", [("equiangular", 1), ("parallel", 2), ("equilinear", 1)])
def test_view_ranges_in_turn(gpu, geo, ns):
    torch, cg, device, phantoms = gpu
    nd, nv = 257, 240
    ph = phantoms.make_phantom(phantoms.random_ellipses(seed=41, n=9))
    ph2 = phantoms.make_phantom(phantoms.random_ellipses(seed=42, n=14))

    def scanner():
        return cg.Scanner(ph, geo, nd, nv, nSample=ns)

    def scan(sc, p, start=0, n=None, off=None):
        sino = torch.full((nv, device.pitch_for(nd)), float("nan"), device="cuda")
        ang = device.raysums(sc, p, sino, start_view=start, n_views=n, offset_view=off)
        cg.sync()
        rows = slice(start, start + (nv - start if n is None else n))
        return sino[rows, :nd].clone(), ang[rows].copy()

    cases = [(ph, 0, None, None), (ph, 30, 100, None), (ph2, 0, None, None), (ph, 30, 100, 7),
             (ph2, 30, 100, None), (ph, 0, None, None), (ph2, 5, 200, 3)]
    refs = [scan(scanner(), *c) for c in cases]
    sc = scanner()
    for c, (rs, ra) in zip(cases, refs):
        s, a = scan(sc, *c)
        assert torch.equal(s, rs), c
        assert np.array_equal(a, ra), c
    # the batched and multi-scan calls on the same scanner, then a sub-range again
    sinos = torch.zeros((2, nv, device.pitch_for(nd)), device="cuda")
    ang = device.raysums_batch(sc, [ph, ph2], sinos)
    cg.sync()
    full0, full2 = refs[0], refs[2]
    assert torch.equal(sinos[0, :, :nd], full0[0]) and torch.equal(sinos[1, :, :nd], full2[0])
    assert np.array_equal(ang, full0[1])
    msinos = [torch.zeros((nv, device.pitch_for(nd)), device="cuda") for _ in range(2)]
    device.raysums_multi([sc, sc], [ph2, ph], msinos)
    cg.sync()
    assert torch.equal(msinos[0][:, :nd], full2[0]) and torch.equal(msinos[1][:, :nd], full0[0])
    s, a = scan(sc, *cases[1])
    assert torch.equal(s, refs[1][0])


def test_ellipsoid_scans_share_the_views(gpu):
    torch, cg, device, phantoms = gpu
    ell = phantoms.random_ellipsoids(seed=5, n=6, z_half=1.0)
    nd, nv = 129, 360

    def scanner():
        return cg.Scanner(phantoms.make_phantom(phantoms.ellipsoid_footprint(ell)), "equilinear",
                          nd, nv, rotAngle=2 * 2 * np.pi)

    def scan(sc, z0, dz):
        sino = device.alloc_sinogram(nv, nd)
        device.raysums_ellipsoids(sc, ell, z0, dz, sino)
        cg.sync()
        return sino[:, :nd].clone()

    sc = scanner()
    for z0, dz in ((-1.0, 2.0 / nv), (-0.5, 1.0 / nv), (-1.0, 2.0 / nv)):
        assert torch.equal(scan(sc, z0, dz), scan(scanner(), z0, dz)), (z0, dz)


@pytest.mark.parametrize("geo,ns,n_el", [("equiangular", 1, 150), ("parallel", 3, 60),
                                         ("equilinear", 1, 500)])
def test_large_phantoms_against_oracle(gpu, oracle, geo, ns, n_el):
    """Phantoms with enough elements that a ray block holds fewer views (or
    opts in to more than 48 KB of shared memory for one view), against the
    FP64 oracle, with a view count no multiple of the views per block."""
    torch, cg, device, phantoms = gpu
    nd, nv = 97, 75
    elems = phantoms.random_ellipses(seed=n_el, n=n_el)
    sc = cg.Scanner(phantoms.make_phantom(elems), geo, nd, nv, nSample=ns)
    sino = device.alloc_sinogram(nv, nd)
    ang = device.raysums(sc, phantoms.make_phantom(elems), sino)
    cg.sync()
    osc = oracle.Scanner(oracle.Phantom(elements=elems), geo, nd, nv, nsample=ns)
    ref, a_ref = osc.collect()
    s = sino[:, :nd].cpu().numpy().astype(np.float64)
    err = float(np.linalg.norm(s - ref) / np.linalg.norm(ref))
    assert np.array_equal(ang, a_ref)
    assert err < 1e-5, err
