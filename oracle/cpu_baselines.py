"""TEST INFRASTRUCTURE ONLY: time the reference's own CPU reconstruction beside
the oracle port on the equiangular workload's slice, so that the port's speed
(the CPU arm the benchmark can run on machines without the reference) is
stated relative to CTSim itself.

Needs the reference binaries (`make -C oracle ref`) and the oracle
(`make -C oracle oracle`).  The slice: 12 seeded random ellipses
(phantoms.random_ellipses(seed=7)) written as a phantom file and scanned by the
reference's phm2pj (equiangular, 733 detectors x 720 views over 360 degrees),
then reconstructed at 512 x 512 with table backprojection and cubic
interpolation over the first VIEWS views:

- reference: ref_harness timerec (Reconstructor::reconstructView per thread
  over a contiguous view block, one private image per thread, images summed:
  the GUI's worker-thread scheme, src/threadrecon.cpp:176-255), abs_hamming
  0.54 by direct convolution (the reference's FFT method needs FFTW, which is
  absent);
- port: pyoracle.reconstruct with the same filter by convolution, and by the
  radix-2 FFT the port adds (zero-pad 2), views and image columns over OpenMP
  threads.

    python oracle/cpu_baselines.py [--views 120] [--threads 1,8]

Prints one JSON line per (implementation, method, threads) and a summary of
port / reference ratios.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

REF = os.path.join(HERE, "_ref", "ctsimtext")
HARN = os.path.join(HERE, "_ref", "ref_harness")
N_DET, N_VIEW, NX = 733, 720, 512


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--views", type=int, default=120)
    ap.add_argument("--threads", default="1,%d" % (os.cpu_count() or 1))
    ap.add_argument("--repeat", type=int, default=2)
    args = ap.parse_args()
    for b in (REF, HARN):
        if not os.path.exists(b):
            sys.exit("reference not built: run `make -C oracle ref`")
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    import pyoracle as po
    from ctsim_gb300.fileio import read_pj
    from ctsim_gb300.phantoms import random_ellipses, write_phm
    threads = [int(t) for t in args.threads.split(",")]
    nv = min(args.views, N_VIEW)
    rows = []
    with tempfile.TemporaryDirectory() as tmp:
        phm = os.path.join(tmp, "c2.phm")
        pjf = os.path.join(tmp, "c2.pj")
        write_phm(phm, random_ellipses(seed=7, n=12))
        subprocess.run([REF, "phm2pj", pjf, str(N_DET), str(N_VIEW), "--phmfile", phm,
                        "--geometry", "equiangular", "--nray", "1"], check=True,
                       stdout=subprocess.DEVNULL)
        pj = read_pj(pjf)
        geom = po.Geom(pj.geometry, pj.nDet, nv, pj.rotInc, pj.detInc, pj.focalLength,
                       pj.sourceDetectorLength, pj.viewDiameter, pj.fanBeamAngle)
        sino = np.ascontiguousarray(pj.data[:nv], np.float32)
        ang = np.ascontiguousarray(pj.angles[:nv], np.float64)
        for t in threads:
            best = None
            for _ in range(args.repeat):
                r = subprocess.run([HARN, "timerec", pjf, str(NX), str(NX), "abs_hamming",
                                    "convolution", "table", "cubic", str(t), str(nv), "0.54",
                                    "1"], check=True, capture_output=True, text=True)
                d = json.loads(r.stdout)
                best = d if best is None or d["pv_per_s"] > best["pv_per_s"] else best
            rows.append({"impl": "reference", "method": "convolution", "threads": t,
                         "views": nv, "pv_per_s": best["pv_per_s"]})
            for method, zp in (("convolution", 1), ("fft", 2)):
                rate = 0.0
                for _ in range(args.repeat):
                    t0 = time.perf_counter()
                    po.reconstruct(geom, sino, ang, NX, NX, filter_name="abs_hamming", param=0.54,
                                   method=method, zeropad=zp, backproj="table", interp="cubic",
                                   nthreads=t)
                    rate = max(rate, NX * NX * nv / (time.perf_counter() - t0))
                rows.append({"impl": "port", "method": method, "threads": t, "views": nv,
                             "pv_per_s": rate})
    for r in rows:
        print(json.dumps(r))
    ref = {r["threads"]: r["pv_per_s"] for r in rows if r["impl"] == "reference"}
    for r in rows:
        if r["impl"] == "port":
            print("port %-11s %2d threads: %.3e pv/s = %.2f x reference convolution (%d threads)"
                  % (r["method"], r["threads"], r["pv_per_s"], r["pv_per_s"] / ref[r["threads"]],
                     r["threads"]))


if __name__ == "__main__":
    main()
