"""Sharded reconstruction on the GPU: two gloo ranks (separate processes, both
on GPU 0) each filter and backproject their view block through libctgpu.so,
and the partial images are summed in host memory by the all-reduce (the
reference's MPI pjrec scheme, tools/pjrec.cpp:375-418).  No kernel of one rank
waits on the other: the ranks meet only in the host-side sum.

- One slice (sharding.reconstruct_sharded): the Shepp-Logan slice
  (parallel 367 x 320, abs_bandlimit by convolution, table / linear, 256 x 256)
  against the single-process plan.run to 1e-6 rel-L2 (FP32 summation order)
  and against the reference's FP64 image to 1e-5.
- A batch of three equiangular slices sharded by view block
  (sharding.reconstruct_views_batch: one filter launch over the rank's rows,
  one batched backprojection, the sum, PostProcessing) against the
  single-process batch to 1e-6.
"""
import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu


def _rank_main(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(0)
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    from ctsim_gb300.sharding import reconstruct_sharded, reconstruct_views_batch, view_block
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)

    # one slice
    d = np.load(os.path.join(ROOT, "tests", "golden", "scans.npz"))
    g, nd, nv, rs, ri, ds, di, vd, fl, sdl, fan = d["c1/hdr"]
    geom = cg.Geometry(int(g), int(nd), int(nv), 0, rs, ri, ds, di, vd, fl, sdl, fan)
    sino = device.alloc_sinogram(int(nv), int(nd))
    sino[:, :int(nd)] = torch.from_numpy(d["c1/data"]).cuda()
    ang = d["c1/angles"]
    plan = device.ReconPlan(geom, 256, 256, "abs_bandlimit", -1.0, "convolution", 1, "direct",
                            "linear", 1, "table")
    img = torch.zeros((256, 256), device="cuda")
    reconstruct_sharded(plan, sino, ang, img, rank, world)

    # a batch of slices sharded by view block
    B, n_det, n_view, side = 3, 129, 120, 64
    phs = [phantoms.make_phantom(phantoms.random_ellipses(seed=40 + b, n=12)) for b in range(B)]
    sc = cg.Scanner(phs[0], "equiangular", n_det, n_view)
    pitch = device.pitch_for(n_det)
    sinos = torch.zeros((B, n_view, pitch), device="cuda")
    angs = device.raysums_batch(sc, phs, sinos)
    bplan = device.ReconPlan(sc.geometry(), side, side, "abs_hamming", 0.54, "fft", 2, "direct",
                             "cubic", 1, "table")
    start, count = view_block(n_view, rank, world)
    block = sinos[:, start:start + count].contiguous()
    filtered = torch.empty_like(block)
    images = torch.zeros((B, side, side), device="cuda")
    reconstruct_views_batch(bplan, block, angs, start, filtered, images)
    torch.cuda.synchronize()
    if rank == 0:
        single = torch.zeros((256, 256), device="cuda")
        plan.run(sino, ang, single)
        whole = torch.zeros((B, side, side), device="cuda")
        bplan.run_batch(sinos, angs, whole)
        torch.cuda.synchronize()
        np.savez(os.path.join(out_dir, "out.npz"), sharded=img.cpu().numpy(),
                 single=single.cpu().numpy(), batch_sharded=images.cpu().numpy(),
                 batch_whole=whole.cpu().numpy())
    dist.destroy_process_group()


def test_two_ranks_on_one_gpu_match_single_process(golden, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import torch.multiprocessing as mp
    port = 31000 + (os.getpid() % 2000)
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    out = np.load(tmp_path / "out.npz")
    e1 = rel_l2(out["sharded"], out["single"])
    rec = golden("recons")
    e2 = rel_l2(out["sharded"], rec["0/image64"])
    e3 = rel_l2(out["batch_sharded"], out["batch_whole"])
    print("sharded Shepp-Logan slice vs single process %.3g, vs reference FP64 %.3g; batch %.3g" % (e1, e2, e3))
    assert e1 < 1e-6, e1
    assert e2 < 1e-5, e2
    assert e3 < 1e-6, e3
    assert np.abs(out["batch_whole"]).max() > 0
