"""Differentiable forward projection and FBP (parallel geometry) as
torch.autograd.Functions on the library's kernels.

    P(x)   = scale * B^T x     pixel image -> sinogram (ctgpu_recon_project)
    FBP(b) = rotScale * B(F b) sinogram -> image (ctgpu_recon_filter + _backproject)

B is the parallel table backprojector with linear interpolation
(libctsim/backprojectors.cpp:444-481) without its rotScale, B^T its exact
transpose (same FP64 anchors and FP32 positions, weights (1-frac, frac)), and
F the plan's filter, a Toeplitz operator (applied as an FFT convolution)
that is symmetric for parallel beams (even filter kernels; no fan
pre-weighting), so F^T = F.  Hence
    dP^T  = scale * B,      dFBP^T = F (rotScale * B^T).
Views are recomputed in the backward pass, nothing per view is stored.
Images are [nx, ny] float32 CUDA tensors, sinograms [n_view, pitch].

    R(theta) = analytic ray-sums of a phantom of ellipses with parameters
               theta [n, 6] = (cx, cy, u, v, rot_deg, atten) per ellipse
               (ctgpu_collect_projections), any geometry;
    dR^T g   = ctgpu_raysum_ellipse_gradient (chord-length derivatives,
               outline-box pre-rejection held fixed).
"""
import numpy as np
import torch

from . import device


class ParallelOperator:
    """Bundles a parallel-beam plan (table backprojector, linear interpolation)."""

    def __init__(self, geometry, nx, ny, angles, filter_name="abs_bandlimit", filter_param=-1.0,
                 filter_method="convolution", zeropad=1, scale=None):
        if geometry.geometry != 0:
            raise ValueError("differentiable operators are defined for parallel geometry")
        self.geometry = geometry
        self.nx, self.ny = nx, ny
        self.angles = np.ascontiguousarray(angles, np.float64)
        self.plan = device.ReconPlan(geometry, nx, ny, filter_name, filter_param, filter_method,
                                     zeropad, "direct", "linear", 1, "table")
        (ext, inc) = self.plan.axes()
        # pixel area / detector spacing turns the pixel sum into a line integral
        self.scale = inc[0] * inc[1] / geometry.det_inc if scale is None else scale
        self.rot_scale = np.pi / geometry.n_view
        self.n_det = geometry.n_det

    def new_sino(self):
        return device.alloc_sinogram(len(self.angles), self.n_det)

    def project(self, x):
        out = self.new_sino()
        self.plan.project(x.contiguous(), self.angles, out, self.scale)
        return out

    def backproject(self, s, scale):
        img = torch.zeros((self.nx, self.ny), device=s.device, dtype=torch.float32)
        self.plan.backproject(s.contiguous(), self.angles, img)
        return img * scale

    def filter(self, s):
        out = self.new_sino()
        self.plan.filter(s.contiguous(), out)
        return out


class _Project(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op):
        ctx.op = op
        return op.project(x)

    @staticmethod
    def backward(ctx, g):
        op = ctx.op
        return op.backproject(g, op.scale), None


class _FBP(torch.autograd.Function):
    @staticmethod
    def forward(ctx, s, op):
        ctx.op = op
        return op.backproject(op.filter(s), op.rot_scale)

    @staticmethod
    def backward(ctx, g):
        op = ctx.op
        pg = op.new_sino()
        op.plan.project(g.contiguous(), op.angles, pg, op.rot_scale)
        return op.filter(pg), None


def project(x, op):
    """Differentiable P(x): [nx, ny] -> [n_view, pitch] (pitch columns past n_det are 0)."""
    return _Project.apply(x, op)


def fbp(sino, op):
    """Differentiable FBP(sino): [n_view, pitch] -> [nx, ny]."""
    return _FBP.apply(sino, op)


class EllipseProjector:
    """Analytic ray-sums of a phantom of ellipses as a function of their
    parameters, with a fixed scanner (its geometry is not re-derived from the
    parameters)."""

    def __init__(self, scanner):
        self.scanner = scanner
        self.geometry = scanner.geometry()

    def phantom(self, params):
        from . import Phantom
        p = Phantom()
        for row in np.asarray(params, np.float64).reshape(-1, 6):
            p.add_element("ellipse", *[float(x) for x in row])
        return p

    def project(self, params):
        out = device.alloc_sinogram(self.geometry.n_view, self.geometry.n_det)
        device.raysums(self.scanner, self.phantom(params), out)
        return out

    def gradient(self, params, g):
        import ctypes as C
        from ._lib import check, lib
        p = self.phantom(params)
        n = np.asarray(params).reshape(-1, 6).shape[0]
        out = np.zeros((n, 6), np.float64)
        gg = g.contiguous().float()
        check(lib().ctgpu_raysum_ellipse_gradient(self.scanner._h, p._h, C.c_void_p(gg.data_ptr()),
                                                  gg.shape[1], out.ctypes.data_as(C.c_void_p),
                                                  None))
        return out


class _EllipseRaysums(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, op):
        ctx.op = op
        ctx.params = params.detach().cpu().numpy().astype(np.float64)
        ctx.dtype, ctx.device = params.dtype, params.device
        return op.project(ctx.params)

    @staticmethod
    def backward(ctx, g):
        grad = ctx.op.gradient(ctx.params, g)
        return torch.from_numpy(grad).to(dtype=ctx.dtype, device=ctx.device), None


def ellipse_raysums(params, op):
    """Sinogram [n_view, pitch] of the ellipses `params` [n, 6] (cx, cy, u, v,
    rot_deg, atten); differentiable in params."""
    return _EllipseRaysums.apply(params, op)
