"""The persistent FFT filter of batched launches and the interval rows it
writes for the backprojection (GPU).

- Filtering many rows in one launch (the persistent kernel: transform lengths
  512 to 4096; 8192 stays on the per-pair kernel) against the FP64 oracle,
  with an odd view count (the last pair holds one view) and with an
  unaligned row pitch (the kernel's element-wise path): rel-L2 <= 1e-5.
- ctgpu_recon_run_batch, whose filter launch also writes the interval rows
  (no separate row pass), gives the same bits as filtering first and then
  backprojecting the filtered batch (which builds the rows from the stored
  filtered samples): both evaluate the same FP32 expressions on the same
  values.  Each batch has enough rows that the stand-alone filter call takes
  the same kernel as the batched run; with an odd view count the transforms
  pair the views differently, and the images then agree to 1e-6.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    return torch, cg, device, phantoms


@pytest.mark.parametrize("nd", [200, 367, 733, 1434, 2100])
def test_many_rows_against_oracle(gpu, oracle, nd):
    torch, cg, device, phantoms = gpu
    rng = np.random.default_rng(nd)
    nv = 1301   # 651 pairs: more blocks than one wave of the per-pair kernel
    x = rng.random((nv, nd)).astype(np.float32)
    g = cg.Geometry(1, nd, nv, 0, 0, 0.01, 0, 0.0021, 2.6, 2.6, 5.2, 1.0)
    plan = device.ReconPlan(g, 16, 16, "abs_hamming", 0.54, "fft", 2, "direct", "cubic", 1,
                            "table")
    ref = oracle.ProcessSignal("abs_hamming", "fft", nd, 0.0021, param=0.54, generation="direct",
                               zeropad=2, geometry="equiangular", focal_length=2.6,
                               sdl=5.2).filter(x)
    for pitch in (device.pitch_for(nd), nd):   # aligned rows, and rows at pitch nDet
        xd = torch.zeros((nv, pitch), device="cuda")
        xd[:, :nd] = torch.from_numpy(x).cuda()
        out = torch.full((nv, pitch), 7.0, device="cuda")
        plan.filter(xd, out)
        cg.sync()
        e = rel_l2(out[:, :nd].cpu().numpy(), ref)
        print("filter nd %d pitch %d: rel-L2 %.3g" % (nd, pitch, e))
        assert e < 1e-5, (nd, pitch, e)


@pytest.mark.parametrize("geo,interp,nd,nv,side", [
    ("equiangular", "cubic", 733, 720, 128),
    ("parallel", "linear", 367, 320, 96),
    ("equilinear", "nearest", 1434, 180, 64),
    ("parallel", "cubic", 200, 90, 40),
    ("equiangular", "linear", 2100, 60, 48),
    ("parallel", "cubic", 200, 91, 40),
])
def test_fused_rows_equal_separate_pass(gpu, geo, interp, nd, nv, side):
    torch, cg, device, phantoms = gpu
    # enough rows that the stand-alone filter call also takes the batched
    # (persistent) kernel: a single-slice call of few rows uses the narrow one
    B = max(2, -(-1300 // nv))
    phs = [phantoms.make_phantom(phantoms.random_ellipses(seed=70 + b, n=12)) for b in range(B)]
    sc = cg.Scanner(phs[0], geo, nd, nv)
    pitch = device.pitch_for(nd)
    sinos = torch.zeros((B, nv, pitch), device="cuda")
    ang = device.raysums_batch(sc, phs, sinos)
    plan = device.ReconPlan(sc.geometry(), side, side, "abs_hamming", 0.54, "fft", 2, "direct",
                            interp, 1, "table")
    fused = torch.full((B, side, side), float("nan"), device="cuda")
    plan.run_batch(sinos, ang, fused)
    filt = torch.zeros_like(sinos)
    plan.filter(sinos.view(B * nv, pitch), filt.view(B * nv, pitch))
    sep = torch.full((B, side, side), float("nan"), device="cuda")
    plan.backproject_batch(filt, ang, sep)
    cg.sync()
    assert torch.isfinite(fused).all()
    if nv % 2 == 0:
        assert torch.equal(fused, sep), float((fused - sep).abs().max())
    else:
        # an odd view count pairs the views of a slice's last transform
        # differently in the batched run (within the slice) and in the one long
        # row list (across slices); an FFT's rounding depends on the partner
        e = rel_l2(fused.cpu().numpy(), sep.cpu().numpy())
        assert e < 1e-6, e
