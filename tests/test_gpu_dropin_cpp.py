"""The drop-in C++ classes from a C++ caller: a small program against
include/ctsim_gpu.h and libctgpu.so (tests/cpp/dropin_check.cpp), built here
with the host compiler, checked against the reference's golden outputs."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu
LIBDIR = os.path.join(ROOT, "ctsim_gb300")


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.path.exists(os.path.join(LIBDIR, "libctgpu.so")):
        pytest.skip("library not built")
    exe = str(tmp_path_factory.mktemp("cpp") / "dropin_check")
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-std=c++17", "-O1", os.path.join(ROOT, "tests", "cpp", "dropin_check.cpp"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
           "-L" + LIBDIR, "-lctgpu", "-L" + os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("building the C++ caller failed:\n" + r.stderr[-2000:])
    return exe


@pytest.mark.parametrize("k", [0, 2, 4])
def test_projections_convert_polar(prog, golden, tmp_path, k):
    from ctsim_gb300.fileio import ProjectionFile, write_pj
    d = golden("polar")
    name, nx, ny, interp = d["%d/cfg" % k]
    hdr = d["%d/hdr" % k]
    g, nd, nv, rs, ri, ds, di, vd, fl, sdl, fan = hdr
    pj = ProjectionFile(int(nv), int(nd), int(g), 0.0, rs, ri, ds, di, vd, fl, sdl, fan,
                        angles=d["%d/angles" % k], data=d["%d/data" % k])
    f = tmp_path / "p.pj"
    write_pj(f, pj)
    out = tmp_path / "o.f32"
    r = subprocess.run([prog, "polar", str(f), str(nx), str(ny), interp, str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    img = np.fromfile(out, np.float32).reshape(int(nx), int(ny))
    ref = d["%d/image" % k]
    c = min(int(nx), int(ny))
    if interp == "bilinear":
        assert np.abs(img[:c] - ref[:c]).max() <= 1e-6 * np.abs(ref).max()
    else:
        assert (img[:c] == ref[:c]).mean() >= 0.99


def test_imagefile_compare_and_subtract(prog, golden, tmp_path):
    from ctsim_gb300.fileio import ImageFileData, read_if, write_if
    g = golden("io")
    a, b, dre = g["comp/0/a"], g["comp/0/b"], g["comp/0/dre"]
    fa, fb = tmp_path / "a.if", tmp_path / "b.if"
    write_if(fa, ImageFileData(64, 64, 7, 4, 1, data=a), [(1, "image a", 0.5, (2020, 1, 1, 0, 0, 0))])
    write_if(fb, ImageFileData(64, 64, 7, 4, 1, data=b), [(1, "image b", 0.5, (2020, 1, 1, 0, 0, 0))])
    r = subprocess.run([prog, "comp", str(fa), str(fb)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # imagefile.cpp:243-256, printed with the stream's default precision
    want = ("  Normalized root mean squared distance (d): %s\n"
            "      Normalized mean absolute distance (r): %s\n"
            "Worst case distance (2x2 pixel average) (e): %s\n") % tuple(
                "%g" % v for v in dre)
    assert r.stdout == want
    fo = tmp_path / "o.if"
    r = subprocess.run([prog, "sub", str(fa), str(fb), str(fo)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    o = read_if(fo)
    np.testing.assert_array_equal(o.data, a - b)
    assert [l[1] for l in o.labels] == ["if2 file 1: image a", "if2 file 2: image b"]
