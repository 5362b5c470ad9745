"""The C ABI library loads and exports every entry point include/ctgpu.h declares."""
import os
import re

import pytest

from conftest import ROOT


def _declared():
    with open(os.path.join(ROOT, "include", "ctgpu.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ctgpu_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = _declared()
    assert "ctgpu_recon_run" in names and "ctgpu_collect_projections" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol():
    from ctsim_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libctgpu.so not built")
    L = _lib.lib()
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing
    assert L.ctgpu_abi_version() == 1
    # every declared symbol has a ctypes signature in the Python binding
    assert set(_declared()) <= set(_lib.SIGNATURES), set(_declared()) - set(_lib.SIGNATURES)


def test_errors_without_gpu_work():
    """Argument validation happens on the host and reports the reference's messages."""
    import ctsim_gb300 as cg
    from ctsim_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libctgpu.so not built")
    with pytest.raises(cg.CtgpuError, match="Invalid phantom name"):
        cg.Phantom("nope")
    p = cg.Phantom("herman")
    with pytest.raises(cg.CtgpuError, match="Invalid geometry name"):
        cg.Scanner(p, "linogramx", 10, 10)
    with pytest.raises(cg.CtgpuError, match="nView & nDet must be greater than 0"):
        cg.Scanner(p, "parallel", 0, 10)
    with pytest.raises(cg.CtgpuError, match="Focal length must be larger"):
        cg.Scanner(p, "equiangular", 11, 10, focalLengthRatio=0.5)
    with pytest.raises(cg.CtgpuError, match="Unknown PhantomElement type"):
        p.add_element("hexagon", 0, 0, 1, 1, 0, 1)


def test_preinterpolation_factor_rejected_without_gpu_work():
    """A preinterpolation factor other than 1 is refused on the host (the
    reference gives it meaning only in its FFTW filter, which cannot be
    pinned, and in idiff's nearest index)."""
    import ctsim_gb300 as cg
    from ctsim_gb300 import _lib, device
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libctgpu.so not built")
    g = cg.Geometry(0, 65, 48, 0, 0.0, 0.06544984694978735, -0.5, 0.0176, 1.1, 0.0, 0.0, 0.0)
    for method in ("convolution", "fft", "fourier"):
        with pytest.raises(cg.CtgpuError, match="preinterpolation factor") as ei:
            device.ReconPlan(g, 32, 32, "abs_bandlimit", -1.0, method, 1, "direct", "linear", 2,
                             "idiff")
        assert ei.value.code == 2
