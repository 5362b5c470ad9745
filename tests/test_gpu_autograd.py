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


def test_projector_dot_product(setup):
    torch, cg, ag, op, g, ang, gf = setup
    torch.manual_seed(1)
    x = torch.randn((512, 512), device="cuda", requires_grad=True)
    y = torch.zeros_like(op.new_sino())
    y[:, :733] = torch.randn((720, 733), device="cuda")
    px = ag.project(x, op)
    (gx,) = torch.autograd.grad((px * y).sum(), x)
    lhs = float((px.double() * y.double()).sum())
    rhs = float((x.detach().double() * gx.double()).sum())
    # <Ax, y> = <x, A^T y>, relative to the Cauchy-Schwarz scale |Ax| |y|
    scale = float(px.double().norm() * y.double().norm())
    assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs, scale)


def test_fbp_dot_product(setup):
    torch, cg, ag, op, g, ang, gf = setup
    torch.manual_seed(2)
    s = torch.zeros_like(op.new_sino())
    s[:, :733] = torch.randn((720, 733), device="cuda")
    s.requires_grad_(True)
    w = torch.randn((512, 512), device="cuda")
    f = ag.fbp(s, op)
    (gs,) = torch.autograd.grad((f * w).sum(), s)
    lhs = float((f.double() * w.double()).sum())
    rhs = float((s.detach().double() * gs.double()).sum())
    scale = float(f.double().norm() * w.double().norm())
    assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs, scale)


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
    torch, cg, ag, op, g, ang, gf = setup
    x_ref = torch.from_numpy(phantom_image(oracle, gf).astype(np.float32)).cuda()
    torch.manual_seed(5)
    s = torch.zeros_like(op.new_sino())
    s[:, :733] = torch.rand((720, 733), device="cuda")
    s.requires_grad_(True)
    loss = ((ag.fbp(s, op) - x_ref) ** 2).sum()
    (gs,) = torch.autograd.grad(loss, s)
    d = torch.zeros_like(s)
    d[:, :733] = torch.randint(0, 2, (720, 733), device="cuda").float() * 2 - 1
    h = 1e-3

    def L(z):
        r = ag.fbp(z, op) - x_ref
        return float((r.double() ** 2).sum())
    fd = (L(s.detach() + h * d) - L(s.detach() - h * d)) / (2 * h)
    an = float((gs.double() * d.double()).sum())
    assert abs(fd - an) <= 1e-3 * abs(an) + 1e-6, (fd, an)
