"""Multi-process logic on CPU with gloo ranks (no GPU): the view-block split
of the reference's MPI scheme and the partial-image sum, checked with the FP64
oracle doing each rank's backprojection."""
import os

import numpy as np
import pytest

from conftest import ROOT


def test_view_blocks_cover_all_views():
    from ctsim_gb300.sharding import view_block
    for n in (1, 7, 320, 721):
        for world in (1, 2, 3, 8):
            blocks = [view_block(n, r, world) for r in range(world)]
            assert blocks[0][0] == 0
            for (s0, c0), (s1, _) in zip(blocks, blocks[1:]):
                assert s0 + c0 == s1
            assert sum(c for _, c in blocks) == n
            assert max(c for _, c in blocks) - min(c for _, c in blocks) <= 1


def _rank_main(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch
    import torch.distributed as dist
    import pyoracle as po
    from ctsim_gb300.sharding import reduce_partial_images, view_block
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    d = np.load(os.path.join(ROOT, "tests", "golden", "scans.npz"))
    g, nd, nv, rs, ri, ds, di, vd, fl, sdl, fan = d["herman_par/hdr"]
    geom = po.Geom(int(g), int(nd), int(nv), ri, di, fl, sdl, vd, fan)
    ps = po.ProcessSignal("abs_bandlimit", "convolution", int(nd), di)
    filt = ps.filter(d["herman_par/data"], nthreads=1)
    start, count = view_block(int(nv), rank, world)
    part = po.backproject(geom, filt[start:start + count], d["herman_par/angles"], 40, 40,
                          "idiff", "linear", post_process=False, nthreads=1, start_view=start)
    t = torch.from_numpy(part)
    reduce_partial_images(t)
    t *= np.pi / int(nv)
    if rank == 0:
        np.save(os.path.join(out_dir, "img.npy"), t.numpy())
    dist.destroy_process_group()


def test_two_gloo_ranks_match_single_process(golden, oracle, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = 29500 + (os.getpid() % 1000)
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(tmp_path / "img.npy")
    rec = golden("recons")
    k = [i for i in range(len([f for f in rec.files if f.endswith("/cfg")]))
         if list(rec["%d/cfg" % i][:5]) == ["herman_par", 40, 40, "idiff", "linear"]][0]
    ref = rec["%d/image64" % k]
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
