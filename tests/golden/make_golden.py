"""Regenerate the golden fixtures in this directory from the reference itself.

Runs the CTSim 5.2.0 binaries compiled from the unmodified sources by
``make -C oracle ref`` (oracle/_ref/ctsimtext with FP32 images as shipped,
oracle/_ref/fp64/ctsimtext with IMAGEFILE_64_BITS, oracle/_ref/ref_harness
for the filtered rows the CLIs do not write out) and stores their outputs as
small compressed .npz files.  Needs the reference sources, so it runs only in
the development container; the fixtures it writes are committed and travel.

    python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from ctsim_gb300.fileio import read_if, read_pj  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ctsimtext")
REF64 = os.path.join(ROOT, "oracle", "_ref", "fp64", "ctsimtext")
HARN = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

FILTERS = ["abs_bandlimit", "abs_hamming", "abs_hanning", "abs_cosine", "shepp", "abs_sinc",
           "bandlimit", "sinc", "hamming", "hanning", "cosine", "triangle"]


def run(*args):
    subprocess.run([str(a) for a in args], check=True, stdout=subprocess.DEVNULL)


def pj_arrays(prefix, pj):
    return {prefix + "data": pj.data, prefix + "angles": pj.angles,
            prefix + "hdr": np.array([pj.geometry, pj.nDet, pj.nView, pj.rotStart, pj.rotInc,
                                      pj.detStart, pj.detInc, pj.viewDiameter, pj.focalLength,
                                      pj.sourceDetectorLength, pj.fanBeamAngle], np.float64)}


# (name, phantom, geometry, ndet, nview, nray, extra phm2pj args)
SCANS = [
    ("c1", "shepp-logan", "parallel", 367, 320, 2, []),
    ("herman_par", "herman", "parallel", 101, 60, 2, []),
    ("shepp_eqa", "shepp-logan", "equiangular", 133, 96, 1, []),
    ("shepp_eqa_even", "shepp-logan", "equiangular", 134, 90, 3, []),
    ("herman_eql", "herman", "equilinear", 128, 80, 2, []),
    ("herman_eqa", "herman", "equiangular", 99, 72, 1, []),
    ("shepp_par_even", "shepp-logan", "parallel", 64, 50, 1, ["--offsetview", "3"]),
    ("pulse_par", "unit-pulse", "parallel", 65, 8, 1, []),
    ("shepp_eql_ratio", "shepp-logan", "equilinear", 97, 64, 1,
     ["--focal-length", "3", "--center-detector-length", "1.5", "--view-ratio", "1.2",
      "--scan-ratio", "0.9"]),
]


def make_scans(tmp):
    out = {}
    for name, phm, geo, nd, nv, nr, extra in SCANS:
        f = os.path.join(tmp, name + ".pj")
        run(REF, "phm2pj", f, nd, nv, "--phantom", phm, "--geometry", geo, "--nray", nr, *extra)
        out.update(pj_arrays(name + "/", read_pj(f)))
    np.savez_compressed(os.path.join(HERE, "scans.npz"), **out)
    return out


# (scan, nx, ny, backproj, interp, filter, method, zeropad, generation, filter-param)
RECONS = [("c1", 256, 256, "table", "linear", "abs_bandlimit", "convolution", 1, "direct", -1)]
for bp in ("trig", "table", "diff", "idiff"):
    for ip in ("nearest", "linear", "cubic"):
        RECONS.append(("herman_par", 40, 40, bp, ip, "abs_bandlimit", "convolution", 1, "direct", -1))
        RECONS.append(("shepp_par_even", 33, 31, bp, ip, "abs_hamming", "convolution", 1, "direct", 0.54))
for ip in ("nearest", "linear", "cubic"):
    for sc in ("shepp_eqa", "shepp_eqa_even", "herman_eql", "shepp_eql_ratio"):
        RECONS.append((sc, 36, 36, "table", ip, "abs_hamming", "convolution", 1, "direct", 0.54))
RECONS += [
    ("shepp_eqa", 32, 32, "table", "cubic", "abs_hamming", "fourier", 2, "direct", 0.54),
    ("shepp_eqa", 32, 32, "table", "cubic", "shepp", "fourier", 1, "direct", -1),
    ("herman_eql", 32, 32, "table", "linear", "abs_cosine", "fouier-table", 1, "direct", -1),
    ("herman_par", 32, 32, "idiff", "linear", "abs_bandlimit", "fourier", 0, "inverse-fourier", -1),
    ("herman_par", 32, 32, "idiff", "linear", "abs_hanning", "convolution", 1, "inverse-fourier", -1),
]


def make_recons(tmp, scans):
    out = {}
    for k, (sc, nx, ny, bp, ip, flt, meth, zp, gen, prm) in enumerate(RECONS):
        pjf = os.path.join(tmp, sc + ".pj")
        args = ["pjrec", pjf, os.path.join(tmp, "r.if"), nx, ny, "--backproj", bp, "--interp", ip,
                "--filter", flt, "--filter-method", meth, "--zeropad", zp,
                "--filter-generation", gen]
        if prm >= 0:
            args += ["--filter-param", prm]
        run(REF64, *args)
        out["%d/image64" % k] = read_if(os.path.join(tmp, "r.if")).data
        run(REF, *args)
        out["%d/image32" % k] = read_if(os.path.join(tmp, "r.if")).data
        out["%d/cfg" % k] = np.array([sc, nx, ny, bp, ip, flt, meth, zp, gen, prm], dtype=object)
    np.savez_compressed(os.path.join(HERE, "recons.npz"), **out)


def make_filters(tmp):
    rng = np.random.default_rng(2024)
    nd, nv = 29, 2
    x = rng.random((nv, nd)).astype(np.float32)
    fin = os.path.join(tmp, "fin.f32")
    fout = os.path.join(tmp, "fout.f64")
    x.tofile(fin)
    out = {"input": x}
    cases = []
    for gid, fl, sdl in ((0, 0.0, 0.0), (1, 2.6, 5.2), (2, 2.6, 5.2)):
        for f in FILTERS:
            for m in ("convolution", "fourier", "fouier-table"):
                for gen in ("direct", "inverse-fourier"):
                    for zp in ((1,) if m == "convolution" else (0, 1, 2)):
                        run(HARN, "filter", gid, nd, nv, repr(0.0123), repr(fl), repr(sdl), f, "0.54",
                            m, zp, gen, 1, fin, fout)
                        out["%d" % len(cases)] = np.fromfile(fout).reshape(nv, nd)
                        cases.append((gid, fl, sdl, f, m, gen, zp))
    out["cases"] = np.array(cases, dtype=object)
    np.savez_compressed(os.path.join(HERE, "filters.npz"), **out)


def make_helical(tmp):
    out = {}
    for k, (nd, nv, rot, iv) in enumerate([(101, 360, 3, -1), (64, 300, 2.5, 130)]):
        f = os.path.join(tmp, "h.pj")
        run(REF, "phm2pj", f, nd, nv, "--phantom", "herman", "--geometry", "equiangular",
            "--nray", 1, "--rotangle", rot)
        run(REF, "pjHinterp", f, os.path.join(tmp, "hi.pj"), "--interpview", iv)
        out.update(pj_arrays("%d/in_" % k, read_pj(f)))
        out.update(pj_arrays("%d/out_" % k, read_pj(os.path.join(tmp, "hi.pj"))))
        out["%d/interpview" % k] = np.array(iv)
    np.savez_compressed(os.path.join(HERE, "helical.npz"), **out)


# fan-beam scans rebinned to parallel rays (Projections::interpolateToParallel)
REBINS = ["shepp_eqa", "shepp_eqa_even", "herman_eql", "herman_eqa", "shepp_eql_ratio"]


def make_rebin(tmp):
    out = {}
    for name in REBINS:
        pjf = os.path.join(tmp, name + ".pj")
        if not os.path.exists(pjf):
            sc = [s for s in SCANS if s[0] == name][0]
            run(REF, "phm2pj", pjf, sc[3], sc[4], "--phantom", sc[1], "--geometry", sc[2],
                "--nray", sc[5], *sc[6])
        run(HARN, "rebin", pjf, os.path.join(tmp, "rb.pj"))
        out.update(pj_arrays(name + "/", read_pj(os.path.join(tmp, "rb.pj"))))
    np.savez_compressed(os.path.join(HERE, "rebin.npz"), **out)


def make_raster(tmp):
    out = {}
    for k, (phm, n, ns) in enumerate([("herman", 48, 2), ("shepp-logan", 40, 3),
                                      ("shepp-logan", 64, 1)]):
        f = os.path.join(tmp, "p.if")
        run(REF64, "phm2if", f, n, n, "--phantom", phm, "--nsample", ns)
        out["%d/image" % k] = read_if(f).data
        run(REF, "phm2if", f, n, n, "--phantom", phm, "--nsample", ns)
        out["%d/image32" % k] = read_if(f).data
        out["%d/cfg" % k] = np.array([phm, n, ns], dtype=object)
    np.savez_compressed(os.path.join(HERE, "raster.npz"), **out)


# device-resident file I/O: reference-written .pj files byte for byte, pj2if
# images, and comparativeStatistics (if2 --comp) of image pairs
IO_SCANS = ["herman_eql", "shepp_eqa_even", "pulse_par"]


def make_io(tmp):
    from ctsim_gb300.fileio import ImageFileData, write_if
    out = {}
    for name in IO_SCANS:
        pjf = os.path.join(tmp, name + ".pj")
        sc = [s for s in SCANS if s[0] == name][0]
        run(REF, "phm2pj", pjf, sc[3], sc[4], "--phantom", sc[1], "--geometry", sc[2],
            "--nray", sc[5], *sc[6])
        with open(pjf, "rb") as f:
            out[name + "/pj"] = np.frombuffer(f.read(), np.uint8)
        iff = os.path.join(tmp, name + ".if")
        run(REF, "pj2if", pjf, iff)
        im = read_if(iff)
        out[name + "/pj2if"] = im.data
        with open(iff, "rb") as f:
            out[name + "/pj2if_head"] = np.frombuffer(f.read(88), np.uint8)
        out[name + "/pj2if_labels"] = np.array([[l[0], l[1]] for l in im.labels], dtype=object)
        if name == IO_SCANS[0]:   # pjinfo's four outputs (tools/pjinfo.cpp)
            for key, extra in (("info", []), ("dump", ["--dump", "--startview", "2",
                                                         "--endview", "5"]),
                               ("binhdr", ["--binaryheader"]),
                               ("binviews", ["--binaryviews", "--startview", "3", "--endview",
                                             "4"])):
                r = subprocess.run([REF, "pjinfo", pjf] + extra, check=True,
                                   capture_output=True)
                out["pjinfo/" + key] = np.frombuffer(r.stdout, np.uint8)
    # image pairs: rasteriser vs reconstruction, odd sizes, identical, random
    fa, fb = os.path.join(tmp, "a.if"), os.path.join(tmp, "b.if")
    pjs = os.path.join(tmp, "s.pj")
    run(REF, "phm2pj", pjs, 64, 50, "--phantom", "shepp-logan", "--nray", 1)
    rng = np.random.default_rng(77)
    pairs = []
    for k in range(5):
        if k == 0:
            run(REF, "phm2if", fa, 64, 64, "--phantom", "shepp-logan", "--nsample", 2)
            run(REF, "pjrec", pjs, fb, 64, 64, "--filter", "abs_hamming", "--filter-param", 0.54)
        elif k == 1:
            run(REF, "phm2if", fa, 33, 47, "--phantom", "herman", "--nsample", 3)
            run(REF, "phm2if", fb, 33, 47, "--phantom", "herman", "--nsample", 1)
        elif k == 2:
            run(REF, "phm2if", fa, 40, 40, "--phantom", "herman", "--nsample", 2)
            run(REF, "phm2if", fb, 40, 40, "--phantom", "herman", "--nsample", 2)
        else:
            nx, ny = ((5, 6), (41, 30))[k - 3]
            for fn in (fa, fb):
                d = (rng.standard_normal((nx, ny)) * 3 + 1).astype(np.float32)
                write_if(fn, ImageFileData(nx, ny, 7, 4, 1, data=d))
        r = subprocess.run([HARN, "comp", fa, fb], check=True, capture_output=True, text=True)
        out["comp/%d/a" % k] = read_if(fa).data
        out["comp/%d/b" % k] = read_if(fb).data
        out["comp/%d/dre" % k] = np.array([float(x) for x in r.stdout.split()], np.float64)
        if k == 0:
            r = subprocess.run([REF, "if2", fa, fb, "--comp"], check=True, capture_output=True,
                               text=True)
            out["comp/0/printed"] = np.array(r.stdout)
    np.savez_compressed(os.path.join(HERE, "io.npz"), **out)


# Projections::convertPolar of reference scans (ref_harness polar)
POLARS = [("herman_par", 48, 48, "nearest"), ("herman_par", 48, 48, "bilinear"),
          ("shepp_par_even", 40, 32, "bilinear"), ("shepp_par_even", 33, 33, "nearest"),
          ("shepp_eqa", 36, 36, "bilinear"), ("shepp_eqa_even", 30, 30, "nearest"),
          ("herman_eql", 30, 30, "bilinear")]


def make_polar(tmp):
    out = {}
    for k, (name, nx, ny, interp) in enumerate(POLARS):
        pjf = os.path.join(tmp, name + ".pj")
        if not os.path.exists(pjf):
            sc = [s for s in SCANS if s[0] == name][0]
            run(REF, "phm2pj", pjf, sc[3], sc[4], "--phantom", sc[1], "--geometry", sc[2],
                "--nray", sc[5], *sc[6])
        f = os.path.join(tmp, "polar.f32")
        run(HARN, "polar", pjf, nx, ny, interp, f)
        out["%d/image" % k] = np.fromfile(f, np.float32).reshape(nx, ny)
        out.update(pj_arrays("%d/" % k, read_pj(pjf)))
        out["%d/cfg" % k] = np.array([name, nx, ny, interp], dtype=object)
    np.savez_compressed(os.path.join(HERE, "polar.npz"), **out)


# Phantom files read by the reference (Phantom::createFromFile): every element
# type with non-zero attenuation (elements.phm, committed beside this script),
# and one seeded random-ellipse phantom as the benchmarks draw them
PHM_SCANS = [  # (name, phm file, geometry, ndet, nview, nray)
    ("el_par", "elements", "parallel", 121, 90, 2),
    ("el_eqa", "elements", "equiangular", 120, 96, 2),
    ("el_eql", "elements", "equilinear", 131, 100, 2),
    ("rnd_eqa", "random12", "equiangular", 129, 120, 1),
]


def make_phmfile(tmp):
    from ctsim_gb300.phantoms import random_ellipses, write_phm
    files = {"elements": os.path.join(HERE, "elements.phm"),
             "random12": os.path.join(tmp, "random12.phm")}
    write_phm(files["random12"], random_ellipses(seed=2, n=12))
    out = {"random12/text": np.array(open(files["random12"]).read())}
    for name, phm, geo, nd, nv, nr in PHM_SCANS:
        f = os.path.join(tmp, name + ".pj")
        run(REF, "phm2pj", f, nd, nv, "--phmfile", files[phm], "--geometry", geo, "--nray", nr)
        out.update(pj_arrays(name + "/", read_pj(f)))
        out[name + "/cfg"] = np.array([phm, geo, nd, nv, nr], dtype=object)
    for k, (n, ns) in enumerate([(48, 2), (37, 3)]):
        f = os.path.join(tmp, "p.if")
        run(REF64, "phm2if", f, n, n, "--phmfile", files["elements"], "--nsample", ns)
        out["raster%d/image" % k] = read_if(f).data
        run(REF, "phm2if", f, n, n, "--phmfile", files["elements"], "--nsample", ns)
        out["raster%d/image32" % k] = read_if(f).data
        out["raster%d/cfg" % k] = np.array([n, ns])
    np.savez_compressed(os.path.join(HERE, "phmfile.npz"), **out)


# reconstructions restricted to a region of interest (Backproject's
# ReconstructionROI, libctsim/backprojectors.cpp:284-315; reachable through the
# API, not pjrec): the reference's filtered rows (abs_bandlimit, convolution)
# backprojected by the FP64-image build with the ROI
ROIS = [  # (scan, nx, ny, backproj, interp, (xmin, ymin, xmax, ymax))
    ("herman_par", 40, 36, "table", "linear", (-0.3, -0.45, 0.5, 0.35)),
    ("herman_par", 33, 40, "idiff", "cubic", (-0.3, -0.45, 0.5, 0.35)),
    ("herman_par", 40, 40, "diff", "nearest", (0.6, -0.2, -0.4, 0.5)),
    ("herman_par", 40, 40, "trig", "linear", (0.6, -0.2, -0.4, 0.5)),
    ("shepp_eqa", 36, 36, "table", "cubic", (-0.3, -0.45, 0.5, 0.35)),
    ("herman_eql", 36, 30, "table", "linear", (-5.0, -0.4, 0.3, 5.0)),
]


def make_roi(tmp):
    out = {}
    harn64 = os.path.join(ROOT, "oracle", "_ref", "ref_harness64")
    for k, (name, nx, ny, bp, ip, roi) in enumerate(ROIS):
        pjf = os.path.join(tmp, name + ".pj")
        sc = [x for x in SCANS if x[0] == name][0]
        run(REF, "phm2pj", pjf, sc[3], sc[4], "--phantom", sc[1], "--geometry", sc[2],
            "--nray", sc[5], *sc[6])
        pj = read_pj(pjf)
        fin, ff = os.path.join(tmp, "s.f32"), os.path.join(tmp, "f.f64")
        np.ascontiguousarray(pj.data, np.float32).tofile(fin)
        run(HARN, "filter", pj.geometry, pj.nDet, pj.nView, repr(pj.detInc), repr(pj.focalLength),
            repr(pj.sourceDetectorLength), "abs_bandlimit", "-1", "convolution", 1, "direct", 1,
            fin, ff)
        fo = os.path.join(tmp, "img.f64")
        run(harn64, "bp", pjf, ff, nx, ny, bp, ip, fo, *[repr(v) for v in roi])
        out["%d/image64" % k] = np.fromfile(fo).reshape(nx, ny)
        out["%d/cfg" % k] = np.array([name, nx, ny, bp, ip], dtype=object)
        out["%d/roi" % k] = np.array(roi, np.float64)
    np.savez_compressed(os.path.join(HERE, "roi.npz"), **out)


def main():
    for b in (REF, REF64, HARN):
        if not os.path.exists(b):
            sys.exit("reference not built: run `make -C oracle ref`")
    only = sys.argv[1:]
    with tempfile.TemporaryDirectory() as tmp:
        if not only:
            scans = make_scans(tmp)
            make_recons(tmp, scans)
            make_filters(tmp)
            make_helical(tmp)
            make_raster(tmp)
        if not only or "rebin" in only:
            make_rebin(tmp)
        if "raster" in only:
            make_raster(tmp)
        if not only or "io" in only:
            make_io(tmp)
        if not only or "polar" in only:
            make_polar(tmp)
        if not only or "phmfile" in only:
            make_phmfile(tmp)
        if not only or "roi" in only:
            make_roi(tmp)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print("%-14s %8d bytes" % (f, os.path.getsize(os.path.join(HERE, f))))


if __name__ == "__main__":
    main()
