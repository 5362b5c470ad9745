"""Build libctgpu.so (and the command-line tools) for sm_103a with nvcc.

    python -m ctsim_gb300.build            # incremental
    python -m ctsim_gb300.build --force

Objects go to ctsim_gb300/_build/, the library to ctsim_gb300/libctgpu.so.
Translation units compile in parallel; nothing here needs cmake or torch.
"""
import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libctgpu.so")
TOOL = os.path.join(PKG, "ctgpu_ctsimtext")
# roofline denominators measured by the benchmark (FP32 FMA, shared-memory and
# L2 gather bandwidth); not part of libctgpu
PEAKS_LIB = os.path.join(PKG, "libctpeaks.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code keeps the reference's FP64 rounding: no contraction into FMAs
# (aarch64 compilers contract by default), so geometry, filters and view
# steps come out bit-identical on x86 and Arm.
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17",
                  "-Xcompiler", "-fPIC,-O2,-Wall,-ffp-contract=off",
                  "-I" + os.path.join(ROOT, "include")]
# per-file device flags: the helical weights are FP64 expressions the
# reference evaluates without fused multiply-adds
FILE_FLAGS = {"k_helical.cu": ["--fmad=false"], "k_fourier.cu": ["--fmad=false"]}
# extra nvcc flags for every translation unit, e.g. tuning macros
# (CTGPU_NVCC_FLAGS="-DCTGPU_BP_CTAS_PER_SM=5")
EXTRA_FLAGS = os.environ.get("CTGPU_NVCC_FLAGS", "").split()

LIB_SOURCES = ["k_common.cu", "k_raysum.cu", "k_filter.cu", "k_backproject.cu", "k_helical.cu",
               "ctgpu_api.cpp", "filter_design.cpp", "ctsim_api.cpp", "k_noalloc.cu", "k_rebin.cu",
               "k_fileio.cu", "ctgpu_io.cpp", "k_fourier.cu", "ctgpu_fourier.cpp"]
TOOL_SOURCES = ["tools/ctsimtext.cpp"]
PEAKS_SOURCES = ["peaks/k_peaks.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, force):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not force and not _stale(obj, [src] + _headers()):
        return obj, None
    cmd = [nvcc()] + NVFLAGS + EXTRA_FLAGS + FILE_FLAGS.get(os.path.basename(src), []) + \
        ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr)
    return obj, None


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in LIB_SOURCES]
    tool_srcs = [os.path.join(CSRC, s) for s in TOOL_SOURCES]
    peak_srcs = [os.path.join(CSRC, s) for s in PEAKS_SOURCES]
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs + tool_srcs + peak_srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("compilation failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results[:len(srcs)]]
    if force or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        subprocess.run(cmd, check=True)
    nt = len(srcs) + len(tool_srcs)
    tobjs = [o for o, _ in results[len(srcs):nt]]
    pobjs = [o for o, _ in results[nt:]]
    if pobjs and (force or _stale(PEAKS_LIB, pobjs)):
        subprocess.run([nvcc()] + ARCH + ["-shared", "-o", PEAKS_LIB] + pobjs + ["-lcudart"],
                       check=True)
    if tobjs and (force or _stale(TOOL, tobjs + [LIB])):
        cmd = [nvcc()] + ARCH + ["-o", TOOL] + tobjs + ["-L" + PKG, "-lctgpu", "-lcudart",
                                                       "-Xlinker", "-rpath=$ORIGIN"]
        subprocess.run(cmd, check=True)
    if verbose:
        print("built", LIB, TOOL)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    build(force=a.force, verbose=True)


if __name__ == "__main__":
    sys.exit(main())
