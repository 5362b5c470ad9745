"""Batched reconstruction of problems of uneven sizes (ctgpu_batch): one
persistent backprojection launch over every (problem, tile), set-up launches
as parallel branches, optional CUDA-graph replay and launch-shape autotuning.
Each problem's image must equal the single-problem plan's (same kernels'
arithmetic, so the tolerance is FP32 round-off of nothing: 1e-7), and one
problem is checked against the FP64 oracle at the path's 1e-5."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

GEOS = ("parallel", "equiangular", "equilinear")


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


def make_problems(torch, cg, device, phantoms, seed, n):
    """n seeded problems: side, views, geometry, interpolation and filter drawn
    per problem; sinograms simulated on the device."""
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(n):
        side = int(rng.choice([40, 64, 96, 128, 160]))
        nv = int(rng.integers(60, 240))
        nd = int(round(1.4 * side))
        geo = GEOS[i % 3]
        ph = phantoms.make_phantom(phantoms.random_ellipses(seed=seed * 1000 + i,
                                                            n=int(rng.integers(5, 21))))
        sc = cg.Scanner(ph, geo, nd, nv)
        sino = device.alloc_sinogram(nv, nd)
        ang = device.raysums(sc, ph, sino)
        interp = ("nearest", "linear", "cubic")[int(rng.integers(0, 3))]
        method, zp = (("convolution", 1), ("fft", 2))[int(rng.integers(0, 2))]
        bp = "trig" if geo == "parallel" and rng.random() < 0.3 else "table"
        probs.append(dict(geometry=sc.geometry(), nx=side, ny=side, sino=sino, angles=ang,
                          image=torch.full((side, side), float("nan"), device="cuda"),
                          filter_name="abs_hamming", filter_param=0.54, filter_method=method,
                          zeropad=zp, interp=interp, backproj=bp))
    return probs


def single(device, q):
    plan = device.ReconPlan(q["geometry"], q["nx"], q["ny"], q["filter_name"], q["filter_param"],
                            q["filter_method"], q["zeropad"], "direct", q["interp"], 1,
                            q["backproj"])
    import torch
    out = torch.zeros((q["nx"], q["ny"]), device="cuda")
    plan.run(q["sino"], q["angles"], out)
    return out


@pytest.mark.parametrize("autotune,graph", [(False, False), (True, True)])
def test_batch_equals_single_problems(gpu, autotune, graph):
    torch, cg, device, phantoms = gpu
    probs = make_problems(torch, cg, device, phantoms, seed=11, n=14)
    batch = device.BatchPlan(probs, autotune=autotune, graph=graph)
    refs = [single(device, q) for q in probs]
    for rep in range(2):   # with graph=True the second run replays the captured graph
        for q in probs:
            q["image"].fill_(float("nan"))
        batch.run()
        cg.sync()
        for i, (q, r) in enumerate(zip(probs, refs)):
            a, b = q["image"].cpu().numpy(), r.cpu().numpy()
            assert np.isfinite(a).all(), (rep, i)
            # the single-slice run may sum its views in groups (FP32 order)
            assert rel_l2(a, b) < 1e-6, (rep, i, q["geometry"].geometry, q["interp"], rel_l2(a, b))
    bps, cv = batch.shape()
    assert bps in (2, 3, 4) and cv in (8, 16)


def test_batch_graph_reads_current_inputs(gpu):
    """A replayed graph reads the sinograms' current contents."""
    torch, cg, device, phantoms = gpu
    probs = make_problems(torch, cg, device, phantoms, seed=12, n=5)
    batch = device.BatchPlan(probs, autotune=False, graph=True)
    batch.run()
    batch.run()
    cg.sync()
    first = [q["image"].clone() for q in probs]
    for q in probs:
        q["sino"].mul_(2.0)
    batch.run()
    cg.sync()
    for q, f in zip(probs, first):
        assert rel_l2(q["image"].cpu().numpy(), 2.0 * f.cpu().numpy()) < 1e-6


def test_batch_problem_against_oracle(gpu):
    torch, cg, device, phantoms = gpu
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
    import pyoracle as po
    probs = make_problems(torch, cg, device, phantoms, seed=13, n=6)
    batch = device.BatchPlan(probs, autotune=False, graph=False)
    batch.run()
    cg.sync()
    for q in probs[:3]:   # one per geometry
        g = q["geometry"]
        s = q["sino"][:, :g.n_det].cpu().numpy()
        meth = q["filter_method"]
        ref = po.reconstruct(po.Geom(g.geometry, g.n_det, g.n_view, g.rot_inc, g.det_inc,
                                     g.focal_length, g.source_detector_length, g.view_diameter,
                                     g.fan_beam_angle),
                             s, q["angles"], q["nx"], q["ny"], filter_name=q["filter_name"],
                             param=q["filter_param"], method=meth, zeropad=q["zeropad"],
                             backproj=q["backproj"], interp=q["interp"])
        e = rel_l2(q["image"].cpu().numpy(), ref)
        assert e < 1e-5, (g.geometry, q["interp"], q["filter_method"], e)


def test_batch_rejects_diff(gpu):
    torch, cg, device, phantoms = gpu
    probs = make_problems(torch, cg, device, phantoms, seed=14, n=3)
    probs[0]["backproj"] = "diff"   # problem 0 is parallel
    with pytest.raises(cg.CtgpuError) as ei:
        device.BatchPlan(probs)
    assert ei.value.code == 2
