"""Phantom files on the GPU against the reference's own outputs (GPU).

tests/golden/elements.phm holds every element type at non-zero attenuation:
two rectangles (one rotated), two sectors, a segment, a triangle and an
ellipse.  It is read by Phantom.from_file (ctgpu_phantom_read_file,
Phantom::createFromFile) and by the drop-in `phm2pj --phmfile` / `phm2if
--phmfile`, and the results are compared with the reference's phm2pj / phm2if
on the same file (tests/golden/phmfile.npz).  A seeded random-ellipse
phantom written as a phantom file is scanned the same way.

Tolerances as for the built-in phantoms: ray-sums rel-L2 <= 1e-5 and every
sample within 1e-4 of the largest; the rasteriser bit for bit against the
reference's FP32-image build.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, rel_l2

pytestmark = pytest.mark.gpu

TOOL = os.path.join(ROOT, "ctsim_gb300", "ctgpu_ctsimtext")
ELEMENTS = os.path.join(GOLDEN, "elements.phm")
SCANS = ("el_par", "el_eqa", "el_eql", "rnd_eqa")


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctsim_gb300 as cg
    from ctsim_gb300 import device
    return torch, cg, device


@pytest.fixture(scope="module")
def files(tmp_path_factory, golden):
    d = golden("phmfile")
    rnd = tmp_path_factory.mktemp("phm") / "random12.phm"
    rnd.write_text(str(d["random12/text"]))
    return {"elements": ELEMENTS, "random12": str(rnd)}


@pytest.mark.parametrize("name", SCANS)
def test_phantom_file_raysums_match_reference(gpu, golden, files, name):
    torch, cg, device = gpu
    d = golden("phmfile")
    phm, geo, nd, nv, nr = d[name + "/cfg"]
    ph = cg.Phantom.from_file(files[str(phm)])
    assert ph.n_elements == (7 if phm == "elements" else 12)
    sc = cg.Scanner(ph, str(geo), int(nd), int(nv), nSample=int(nr))
    g = sc.geometry()
    hdr = d[name + "/hdr"]
    assert g.det_inc == hdr[6] and g.view_diameter == hdr[7] and g.fan_beam_angle == hdr[10]
    sino = device.alloc_sinogram(g.n_view, g.n_det)
    ang = device.raysums(sc, ph, sino)
    cg.sync()
    np.testing.assert_array_equal(ang, d[name + "/angles"])
    out = sino[:, :g.n_det].cpu().numpy()
    ref = d[name + "/data"]
    e = rel_l2(out, ref)
    print("phantom file %s: rel-L2 %.3g, max |err| / max %.3g"
          % (name, e, np.abs(out - ref).max() / np.abs(ref).max()))
    assert e < 1e-5, e
    assert np.abs(out - ref).max() <= 1e-4 * np.abs(ref).max()


def test_phm2pj_phmfile_cli_matches_reference(gpu, golden, files, tmp_path):
    from ctsim_gb300.fileio import read_pj
    d = golden("phmfile")
    if not os.path.exists(TOOL):
        pytest.skip("tools not built")
    for name in ("el_eqa", "rnd_eqa"):
        phm, geo, nd, nv, nr = d[name + "/cfg"]
        pj = tmp_path / (name + ".pj")
        r = subprocess.run([TOOL, "phm2pj", str(pj), str(nd), str(nv), "--phmfile",
                            files[str(phm)], "--geometry", str(geo), "--nray", str(nr)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        p = read_pj(str(pj))
        np.testing.assert_array_equal(p.angles, d[name + "/angles"])
        assert p.viewDiameter == d[name + "/hdr"][7]
        assert rel_l2(p.data, d[name + "/data"]) < 1e-5


def test_phantom_file_raster_matches_reference(gpu, golden, tmp_path):
    torch, cg, device = gpu
    d = golden("phmfile")
    ph = cg.Phantom.from_file(ELEMENTS)
    for k in range(2):
        n, ns = d["raster%d/cfg" % k]
        img, _, _ = ph.rasterize(int(n), int(n), 1.0, int(ns))
        a = img.cpu().numpy()
        np.testing.assert_array_equal(a, d["raster%d/image32" % k])
        ref64 = d["raster%d/image" % k]
        assert np.abs(a - ref64).max() <= 1e-6 * np.abs(ref64).max()
    if os.path.exists(TOOL):
        from ctsim_gb300.fileio import read_if
        f = tmp_path / "p.if"
        r = subprocess.run([TOOL, "phm2if", str(f), "48", "48", "--phmfile", ELEMENTS,
                            "--nsample", "2"], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        np.testing.assert_array_equal(read_if(str(f)).data, d["raster0/image32"])
