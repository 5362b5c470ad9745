"""The drop-in command-line tools (C++ classes on the C ABI) against the
reference's own files (golden fixtures)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu
TOOL = os.path.join(ROOT, "ctsim_gb300", "ctgpu_ctsimtext")


@pytest.fixture(scope="module")
def tool():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.path.exists(TOOL):
        pytest.skip("tools not built")
    return TOOL


def run(*a):
    r = subprocess.run([str(x) for x in a], capture_output=True, text=True)
    return r.returncode, r.stdout + r.stderr


def test_phm2pj_pjrec_match_reference(tool, golden, tmp_path):
    from ctsim_gb300.fileio import read_if, read_pj
    d = golden("scans")
    rec = golden("recons")
    pj = tmp_path / "c1.pj"
    rc, out = run(tool, "phm2pj", pj, 367, 320, "--nray", 2, "--phantom", "shepp-logan")
    assert rc == 0, out
    p = read_pj(pj)
    assert p.nView == 320 and p.nDet == 367 and p.geometry == 0
    assert p.detInc == d["c1/hdr"][6] and p.viewDiameter == d["c1/hdr"][7]
    np.testing.assert_array_equal(p.angles, d["c1/angles"])
    assert rel_l2(p.data, d["c1/data"]) < 1e-5
    assert p.remark.startswith("phm2pj: NDet=367, Nview=320, NRay=2, RotAngle=0.5")
    im = tmp_path / "c1.if"
    rc, out = run(tool, "pjrec", pj, im, 256, 256, "--backproj", "table")
    assert rc == 0, out
    i = read_if(im)
    assert i.nx == 256 and i.ny == 256 and i.pixel_size == 4
    assert rel_l2(i.data, rec["0/image64"]) < 1e-5
    assert len(i.labels) == 2 and i.labels[1][1].startswith("pjrec: 256x256, abs_bandlimit")


def test_pjhinterp_matches_reference(tool, golden, tmp_path):
    from ctsim_gb300.fileio import ProjectionFile, read_pj, write_pj
    d = golden("helical")
    hdr = d["0/in_hdr"]
    src = ProjectionFile(int(hdr[2]), int(hdr[1]), int(hdr[0]), 0.0, hdr[3], hdr[4], hdr[5],
                         hdr[6], hdr[7], hdr[8], hdr[9], hdr[10], angles=d["0/in_angles"],
                         data=d["0/in_data"])
    fin, fout = tmp_path / "h.pj", tmp_path / "hi.pj"
    write_pj(fin, src)
    rc, out = run(tool, "pjHinterp", fin, fout)
    assert rc == 0, out
    o = read_pj(fout)
    np.testing.assert_array_equal(o.angles, d["0/out_angles"])
    np.testing.assert_array_equal(o.data, d["0/out_data"])


def test_cli_errors_match_reference(tool, tmp_path):
    rc, out = run(tool, "phm2pj", tmp_path / "x.pj", 10, 10)
    assert rc == 1 and "No phantom defined" in out
    rc, out = run(tool, "phm2pj", tmp_path / "x.pj", 10, 10, "--phantom", "nope")
    assert rc == 1 and "Invalid phantom name nope" in out
    rc, out = run(tool, "pjrec", tmp_path / "missing.pj", tmp_path / "x.if", 8, 8)
    assert rc == 1 and "Unable to read projectfile" in out


def test_phm2if_matches_reference(tool, golden, tmp_path):
    """phm2if (Phantom::convertToImagefile) writes the reference's FP32 image
    bit for bit, with the image axes and history label."""
    from ctsim_gb300.fileio import read_if
    r = golden("raster")
    for k in range(3):
        phm, n, ns = r["%d/cfg" % k]
        f = tmp_path / ("p%d.if" % k)
        rc, out = run(tool, "phm2if", f, int(n), int(n), "--phantom", str(phm), "--nsample",
                      int(ns))
        assert rc == 0, out
        im = read_if(f)
        assert im.nx == int(n) and im.pixel_size == 4
        np.testing.assert_array_equal(im.data, r["%d/image32" % k])
        assert im.labels[-1][1].startswith("phm2if: nx=%d, ny=%d, viewRatio=1, nsample=%d, phantom=%s"
                                           % (int(n), int(n), int(ns), phm))
    rc, out = run(tool, "phm2if", tmp_path / "x.if", 8, 8)
    assert rc == 1 and "No phantom defined" in out


@pytest.mark.parametrize("name", ["herman_eql", "pulse_par"])
def test_pj2if_matches_reference(tool, golden, tmp_path, name):
    from ctsim_gb300.fileio import read_if
    g = golden("io")
    pj = tmp_path / "in.pj"
    pj.write_bytes(g[name + "/pj"].tobytes())
    out = tmp_path / "out.if"
    rc, log = run(tool, "pj2if", pj, out, "--polar")
    assert rc == 0, log
    raw = out.read_bytes()
    assert raw[:88] == g[name + "/pj2if_head"].tobytes()
    im = read_if(out)
    np.testing.assert_array_equal(im.data, g[name + "/pj2if"])
    assert [[l[0], l[1]] for l in im.labels] == g[name + "/pj2if_labels"].tolist()
    rc, log = run(tool, "pj2if", tmp_path / "missing.pj", out)
    assert rc == 1


def test_if2_comp_and_arithmetic(tool, golden, tmp_path):
    from ctsim_gb300.fileio import ImageFileData, read_if, write_if
    g = golden("io")
    fa, fb = tmp_path / "a.if", tmp_path / "b.if"
    a, b = g["comp/0/a"], g["comp/0/b"]
    write_if(fa, ImageFileData(64, 64, 7, 4, 1, data=a), [(1, "image a", 0.5, (2020, 1, 1, 0, 0, 0))])
    write_if(fb, ImageFileData(64, 64, 7, 4, 1, data=b), [(1, "image b", 0.25, (2020, 1, 1, 0, 0, 0))])
    rc, out = run(tool, "if2", fa, fb, "--comp")
    assert rc == 0, out
    assert out == str(g["comp/0/printed"])   # d=..., r=..., e=... as the reference prints it
    fo = tmp_path / "o.if"
    rc, out = run(tool, "if2", fa, fb, fo, "--sub")
    assert rc == 0, out
    o = read_if(fo)
    np.testing.assert_array_equal(o.data, a - b)
    assert [l[1] for l in o.labels] == ["if2 file 1: image a", "if2 file 2: image b",
                                        "Subtract Images"]
    fc = tmp_path / "c.if"
    write_if(fc, ImageFileData(3, 64, 7, 4, 1, data=a[:3]))
    rc, out = run(tool, "if2", fa, fc, "--comp")
    assert rc == 1 and "do not match" in out
