"""Differentiable projector / FBP (parallel, 512 x 512, 720 views, 733 detectors):
dot-product tests, central finite differences and the FP64 reference gradient."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import autograd
    from scipy.ndimage import gaussian_filter
    g = cg.Geometry(0, 733, 720, 0, 0.0, np.pi / 720, 0.0, 2.6021529547665097 / 733,
                    2.6021529547665097, 2.6021529547665097, 5.2043059095330194, 0.0)
    ang = np.arange(720) * (np.pi / 720)
    op = autograd.ParallelOperator(g, 512, 512, ang)
    return torch, cg, autograd, op, g, ang, gaussian_filter


def phantom_image(oracle, gaussian_filter, seed=4):
    from ctsim_gb300 import phantoms
    ph = oracle.Phantom(elements=phantoms.random_ellipses(seed, 12))
    img, _ = oracle.phantom_to_image(ph, 512, 512, 1.0, 2)
    return gaussian_filter(img, 1.0)


def _smooth_sino(torch, op, oracle, gf, g, ang, seed):
    """a structured sinogram: the FP64 projection of a smoothed phantom image"""
    og = oracle.Geom(0, 733, 720, g.rot_inc, g.det_inc, g.focal_length,
                     g.source_detector_length, g.view_diameter, 0.0)
    s64 = oracle.project_image(og, phantom_image(oracle, gf, seed=seed), ang) * op.scale
    s = torch.zeros_like(op.new_sino())
    s[:, :733] = torch.from_numpy(s64.astype(np.float32)).cuda()
    return s


def test_projector_dot_product(setup, oracle):
    """<P x, y> = <x, P^T y> to 1e-6 of <P x, y>, with x a smoothed phantom
    image and y the projection of another one (so that the inner product is
    not a small difference of large terms)."""
    torch, cg, ag, op, g, ang, gf = setup
    x = torch.from_numpy(phantom_image(oracle, gf, seed=6).astype(np.float32)).cuda()
    x.requires_grad_(True)
    y = _smooth_sino(torch, op, oracle, gf, g, ang, seed=7)
    px = ag.project(x, op)
    (gx,) = torch.autograd.grad((px * y).sum(), x)
    lhs = float((px.detach().double() * y.double()).sum())
    rhs = float((x.detach().double() * gx.double()).sum())
    print("projector dot product: <Px,y> %.9g, <x,P^T y> %.9g, rel %.3g"
          % (lhs, rhs, abs(lhs - rhs) / abs(lhs)))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs), (lhs, rhs)


def test_fbp_dot_product(setup, oracle):
    """<FBP s, w> = <s, FBP^T w> to 1e-6 of <FBP s, w>, with s the projection
    of a smoothed phantom and w another smoothed phantom image."""
    torch, cg, ag, op, g, ang, gf = setup
    s = _smooth_sino(torch, op, oracle, gf, g, ang, seed=8).requires_grad_(True)
    w = torch.from_numpy(phantom_image(oracle, gf, seed=10).astype(np.float32)).cuda()
    f = ag.fbp(s, op)
    (gs,) = torch.autograd.grad((f * w).sum(), s)
    lhs = float((f.detach().double() * w.double()).sum())
    rhs = float((s.detach().double() * gs.double()).sum())
    print("FBP dot product: <FBP s,w> %.9g, <s,FBP^T w> %.9g, rel %.3g"
          % (lhs, rhs, abs(lhs - rhs) / abs(lhs)))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs), (lhs, rhs)


def test_projection_loss_gradient(setup, oracle):
    torch, cg, ag, op, g, ang, gf = setup
    x_np = phantom_image(oracle, gf)
    b_np = phantom_image(oracle, gf, seed=9)
    og = oracle.Geom(0, 733, 720, g.rot_inc, g.det_inc, g.focal_length,
                     g.source_detector_length, g.view_diameter, 0.0)
    # b = P(x_b) in FP64 so the target is exact
    b64 = oracle.project_image(og, b_np, ang) * op.scale
    b = torch.zeros_like(op.new_sino())
    b[:, :733] = torch.from_numpy(b64.astype(np.float32)).cuda()
    x = torch.from_numpy(x_np.astype(np.float32)).cuda().requires_grad_(True)
    loss = ((ag.project(x, op) - b) ** 2).sum()
    (gx,) = torch.autograd.grad(loss, x)
    # FP64 reference gradient: 2 scale B(P x - b)
    r64 = oracle.project_image(og, x_np, ang) * op.scale - b64
    g64 = 2 * op.scale * oracle.backproject(og, r64, ang, 512, 512, "table", "linear",
                                            post_process=False)
    e = rel_l2(gx.cpu().numpy(), g64)
    assert e < 1e-5, e
    # central finite differences along a random direction, h = 1e-3
    # direction with entries +-1, step h = 1e-3 per pixel
    torch.manual_seed(3)
    d = torch.randint(0, 2, (512, 512), device="cuda").float() * 2 - 1
    h = 1e-3

    def L(z):
        r = ag.project(z, op) - b
        return float((r.double() ** 2).sum())
    fd = (L(x.detach() + h * d) - L(x.detach() - h * d)) / (2 * h)
    an = float((gx.double() * d.double()).sum())
    assert abs(fd - an) <= 1e-3 * abs(an) + 1e-6, (fd, an)


def test_fbp_loss_gradient(setup, oracle):
    """d||FBP(s) - x_ref||^2 / ds against the FP64 reference gradient
    2 F^T (rotScale B^T (FBP64(s) - x_ref)) -- the oracle's FP64
    backprojection and its transpose, the reference's convolution filter in
    FP64 (F^T from the reversed taps, so F's symmetry is not assumed) -- to
    1e-5 rel-L2, and against central finite differences (h = 1e-3)."""
    torch, cg, ag, op, g, ang, gf = setup
    x_np = phantom_image(oracle, gf)
    x_ref = torch.from_numpy(x_np.astype(np.float32)).cuda()
    torch.manual_seed(5)
    s = torch.zeros_like(op.new_sino())
    s[:, :733] = torch.rand((720, 733), device="cuda")
    s.requires_grad_(True)
    loss = ((ag.fbp(s, op) - x_ref) ** 2).sum()
    (gs,) = torch.autograd.grad(loss, s)

    # FP64 reference gradient
    og = oracle.Geom(0, 733, 720, g.rot_inc, g.det_inc, g.focal_length,
                     g.source_detector_length, g.view_diameter, 0.0)
    ps = oracle.ProcessSignal("abs_bandlimit", "convolution", 733, g.det_inc)
    h = ps.filter_array()
    n = 733

    def conv_rows(a, taps):   # out[i] = detInc sum_j a[j] taps[i - j + n - 1]
        return np.stack([g.det_inc * np.convolve(r, taps)[n - 1:2 * n - 1] for r in a])
    s64 = s.detach()[:, :n].cpu().double().numpy()
    rot = np.pi / 720
    fbp64 = oracle.backproject(og, conv_rows(s64, h), ang, 512, 512, "table", "linear",
                               post_process=True)
    r64 = fbp64 - x_np.astype(np.float32).astype(np.float64)
    g64 = 2 * rot * conv_rows(oracle.project_image(og, r64, ang), h[::-1])
    e = rel_l2(gs[:, :n].cpu().numpy(), g64)
    print("FBP loss gradient vs FP64 reference: rel-L2 %.3g" % e)
    assert e < 1e-5, e
    assert float(gs[:, n:].abs().max()) == 0.0

    d = torch.zeros_like(s)
    d[:, :733] = torch.randint(0, 2, (720, 733), device="cuda").float() * 2 - 1
    hh = 1e-3

    def L(z):
        r = ag.fbp(z, op) - x_ref
        return float((r.double() ** 2).sum())
    fd = (L(s.detach() + hh * d) - L(s.detach() - hh * d)) / (2 * hh)
    an = float((gs.double() * d.double()).sum())
    assert abs(fd - an) <= 1e-3 * abs(an) + 1e-6, (fd, an)


@pytest.mark.parametrize("geo", ["parallel", "equiangular", "equilinear"])
def test_ellipse_parameter_gradient(setup, oracle, geo):
    """d/d(cx, cy, u, v, rot, atten) of sum(G * R(theta)) for 12 ellipses through
    the autograd Function: the adjoint kernel against the oracle's FP64
    gradient of the same rays (itself pinned to FP64 central differences in
    tests/test_oracle_gradient.py), per entry to 1e-6 of the larger of the
    entry and 1% of its column's largest.  Central differences with h = 1e-3
    do not apply here: a ray-sum is not differentiable at the tangent rays
    (the chord has a square-root edge), so a step of that size measures the
    kinks, not the derivative."""
    torch, cg, autograd, op, g, ang, _ = setup
    from ctsim_gb300 import device, phantoms
    rows = phantoms.random_ellipses(seed=21, n=12)
    theta = np.array([r[1:] for r in rows], np.float64)
    nd, nv = 257, 180
    sc = cg.Scanner(phantoms.make_phantom(rows), geo, nd, nv)
    eop = autograd.EllipseProjector(sc)
    G = np.random.default_rng(2).standard_normal((nv, nd)).astype(np.float32)
    Gd = torch.zeros((nv, device.pitch_for(nd)), device="cuda")
    Gd[:, :nd] = torch.from_numpy(G).cuda()
    t = torch.tensor(theta, requires_grad=True)
    sino = autograd.ellipse_raysums(t, eop)
    loss = (sino * Gd).sum()
    loss.backward()
    grad = t.grad.numpy()
    osc = oracle.Scanner(oracle.Phantom(elements=rows), geo, nd, nv)
    ref = oracle.ellipse_gradient(osc, G.astype(np.float64))
    scale = np.abs(ref).max(axis=0)
    err = np.abs(grad - ref) / np.maximum(np.abs(ref), 1e-2 * scale)
    print("%s ellipse-parameter gradient vs FP64 reference: max rel %.3g" % (geo, err.max()))
    assert err.max() < 1e-6, err.max()
    # the loss ||R(theta) - b||^2 of a perturbed phantom: its gradient is the
    # same adjoint applied to 2 (R - b)
    b = autograd.ellipse_raysums(torch.tensor(theta * 1.01), eop).detach()
    t2 = torch.tensor(theta, requires_grad=True)
    r = autograd.ellipse_raysums(t2, eop)
    ((r - b) ** 2).sum().backward()
    resid = (2 * (r - b)).detach()[:, :nd].cpu().numpy().astype(np.float64)
    ref2 = oracle.ellipse_gradient(osc, resid)
    s2 = np.abs(ref2).max(axis=0)
    e2 = np.abs(t2.grad.numpy() - ref2) / np.maximum(np.abs(ref2), 1e-2 * s2)
    assert e2.max() < 1e-6, e2.max()
