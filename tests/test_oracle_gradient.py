"""The oracle's FP64 ellipse-parameter gradient (the reference for the GPU
adjoint kernel) against FP64 central differences of the oracle's own
ray-sums.  h = 1e-7 (1e-5 degrees for the rotation): a ray-sum has kinks at
tangent rays, and a smaller step straddles fewer of them.  CPU only."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))


@pytest.mark.parametrize("geo", ["parallel", "equiangular", "equilinear"])
def test_ellipse_gradient_matches_central_differences(oracle, geo):
    from ctsim_gb300 import phantoms
    rows = phantoms.random_ellipses(seed=21, n=12)
    theta = np.array([r[1:] for r in rows], np.float64)
    nd, nv = 129, 90
    osc = oracle.Scanner(oracle.Phantom(elements=rows), geo, nd, nv)
    G = np.random.default_rng(2).standard_normal((nv, nd))
    grad = oracle.ellipse_gradient(osc, G)
    base = osc.phantom

    def L(th):
        osc.phantom = oracle.Phantom(elements=[("ellipse",) + tuple(r) for r in th])
        s, _ = osc.collect()
        osc.phantom = base
        return float((s * G).sum())

    fd = np.zeros_like(theta)
    for k in range(theta.shape[0]):
        for j in range(6):
            h = 1e-5 if j == 4 else 1e-7
            tp, tm = theta.copy(), theta.copy()
            tp[k, j] += h
            tm[k, j] -= h
            fd[k, j] = (L(tp) - L(tm)) / (2 * h)
    scale = np.abs(fd).max(axis=0)
    err = np.abs(grad - fd) / np.maximum(np.abs(fd), 1e-2 * scale)
    assert np.median(err) < 1e-5, np.median(err)
    assert err.max() < 2e-3, err.max()
