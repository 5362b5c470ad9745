"""Host-only modes of the drop-in command-line tools, against the reference's
own output (tests/golden/io.npz): pjinfo's scan summary, --dump,
--binaryheader and --binaryviews are byte-identical.  No GPU is needed; the
tool must have been built."""
import os
import subprocess

import pytest

from conftest import ROOT

TOOL = os.path.join(ROOT, "ctsim_gb300", "ctgpu_ctsimtext")


@pytest.fixture(scope="module")
def tool():
    if not os.path.exists(TOOL):
        pytest.skip("tools not built")
    return TOOL


@pytest.mark.parametrize("key,extra", [
    ("info", []), ("dump", ["--dump", "--startview", "2", "--endview", "5"]),
    ("binhdr", ["--binaryheader"]), ("binviews", ["--binaryviews", "--startview", "3",
                                                  "--endview", "4"])])
def test_pjinfo_matches_reference(tool, golden, tmp_path, key, extra):
    g = golden("io")
    pj = tmp_path / "h.pj"
    pj.write_bytes(g["herman_eql/pj"].tobytes())
    r = subprocess.run([tool, "pjinfo", str(pj)] + extra, capture_output=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout == g["pjinfo/" + key].tobytes()


def test_pjinfo_usage_errors(tool, tmp_path):
    r = subprocess.run([tool, "pjinfo"], capture_output=True)
    assert r.returncode == 1
    r = subprocess.run([tool, "pjinfo", str(tmp_path / "missing.pj")], capture_output=True)
    assert r.returncode == 1
