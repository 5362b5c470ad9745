"""Benchmark: FBP pixel-view updates/s (and ray-sums/s) on GB300 vs the CPU path.

Workload (one GPU): the equiangular fan-beam configuration -- seeded
12-ellipse phantoms, 733 detectors x 720 views over 360 degrees, focal length
2 view radii, abs_hamming(0.54) filter by FFT with zeropad 2, cubic
interpolation, 512 x 512 FP32 image.  A step reconstructs a batch of B such
slices (default 64) whose sinograms were simulated on the device beforehand;
the batch's sinograms (B x 2.1 MB) and images (B x 1 MB) exceed the 129 MB L2,
so no flush is needed between steps.  The ray-sum phase (simulating the same
batch) is timed separately over the same number of steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl reference]

--impl reference times the CPU implementation of the same path on the host's
cores: the FP64 restatement in oracle/ (the reference's own binaries are not
available on this machine), FFT filtering, table backprojection with cubic
interpolation, views split over all threads.  One JSON line on rank 0.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DET, N_VIEW, NX = 733, 720, 512
PV_PER_SLICE = NX * NX * N_VIEW
RAYS_PER_SLICE = N_DET * N_VIEW
METRIC = "FBP pixel-view updates/s"
UNIT = "pixel-view updates/s"
# algorithmic work per unit for the dominant kernel (equiangular, cubic):
# 4 samples x 4 B gathered per pixel-view update; 30 + 30 FLOP
BYTES_PER_PV = 16
FLOP_PER_PV = 60
# GB300 CUDA cores: 128 FP32 lanes per SM, an FMA counts 2 FLOP
FP32_LANES_PER_SM = 128
CONFIG_NAME = ("equiangular 733 det x 720 views (360 deg), 12 random ellipses, abs_hamming 0.54 "
               "FFT zeropad 2, cubic, 512x512 FP32")


def peaks():
    """(HBM GB/s, its source, max SM MHz) from MEASURED_PEAKS.json, else the fallback"""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured", d.get("sm_max_mhz", 2070.0)
    return 6800.0, "fallback", 2070.0


def measured_device_peaks(stream_handle):
    """FP32 FMA and gather-bandwidth peaks measured on this GPU by the
    microkernels of libctpeaks.so (ctsim_gb300/csrc/peaks/k_peaks.cu), CUDA
    events, best of 5 launches each."""
    import ctypes as C
    path = os.path.join(ROOT, "ctsim_gb300", "libctpeaks.so")
    lib = C.CDLL(path)
    lib.ctpeaks_measure.argtypes = [C.c_void_p, C.c_void_p]
    out = (C.c_double * 8)()
    if lib.ctpeaks_measure(out, stream_handle) != 0:
        raise RuntimeError("ctpeaks_measure failed")
    return {"ffma_tflops": out[0], "ffma2_tflops": out[1], "lds128_gbs": out[2],
            "l2_gather16_gbs": out[3], "l2_read_gbs": out[4], "sms": int(out[5]),
            "how": "CUDA events, best of 5: scalar FFMA and packed FFMA2 (8 chains/thread, "
                   "4 x 256 threads/SM); LDS.128 of consecutive 16-B words; 16-B "
                   "pseudo-random gathers and coalesced 16-B reads from a 16 MiB "
                   "L2-resident buffer (ld.global.cg)"}


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


def reduce_max(value, world):
    """max over ranks (the timing rule); identity on one rank"""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler is running
            t0 = time.time()
            while not self.rows and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.start = len(self.rows)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = self.rows[getattr(self, "start", 0):] or self.rows
        self.rows = rows
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


cpu_raysum_rate = [None]   # ray-sums/s of the oracle's collect in the last cpu_fbp_rate call


def cpu_fbp_rate(seed, seconds=10.0, nthreads=None, views=None):
    """The CPU path (FP64 oracle port) on a bounded sample: FBP of whole slices
    until `seconds` have passed (at least one).  Returns (pv/s, sample text, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    import pyoracle as po
    from ctsim_gb300 import phantoms
    nthreads = nthreads or (os.cpu_count() or 1)
    ph = po.Phantom(elements=phantoms.random_ellipses(seed, 12))
    sc = po.Scanner(ph, "equiangular", N_DET, N_VIEW, nsample=1)
    t0 = time.perf_counter()
    sino, ang = sc.collect(nthreads=nthreads)
    cpu_raysum_rate[0] = RAYS_PER_SLICE / (time.perf_counter() - t0)
    nv = N_VIEW if views is None else min(views, N_VIEW)
    geom = sc.geom()
    geom.nView = nv   # the oracle reads geom.nView rows
    done, t0 = 0, time.perf_counter()
    while True:
        po.reconstruct(geom, np.ascontiguousarray(sino[:nv], np.float32), ang[:nv], NX, NX,
                       filter_name="abs_hamming", param=0.54, method="fft", zeropad=2,
                       backproj="table", interp="cubic", nthreads=nthreads)
        done += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    pv = done * NX * NX * nv
    return pv / el, "%d slice(s) of %d views, FFT zeropad 2, table/cubic, %d threads, %.1f s" % (
        done, nv, nthreads, el), nthreads


def oracle_parity(elems0, elems, g, sino, image, angles):
    """One slice of the timed batch against the FP64 oracle: its ray-sums
    (scanner geometry from the batch's first phantom, as on the device) and
    the oracle's FBP of the same FP32 sinogram the device read.  The oracle
    is the checker here; nothing timed runs through it."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    import pyoracle as po
    osc = po.Scanner(po.Phantom(elements=elems0), "equiangular", N_DET, N_VIEW, nsample=1)
    osc.phantom = po.Phantom(elements=elems)
    s_ref, a_ref = osc.collect()
    s_gpu = sino[:, :N_DET].cpu().numpy().astype(np.float64)
    ref = po.reconstruct(osc.geom(), s_gpu.astype(np.float32), angles, NX, NX,
                         filter_name="abs_hamming", param=0.54, method="fft", zeropad=2,
                         backproj="table", interp="cubic")
    img = image.cpu().numpy().astype(np.float64)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return {"sinogram_rel_l2": rel(s_gpu, s_ref), "image_rel_l2": rel(img, ref),
            "angles_equal": bool(np.array_equal(np.asarray(angles), a_ref)),
            "tolerance": 1e-5}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    rates = []
    sample = None
    for i in range(args.warmup + args.steps):
        r, sample, threads = cpu_fbp_rate(seed=1000 + i, seconds=0.0, views=args.ref_views)
        if i >= args.warmup:
            rates.append(r)
    value = float(np.mean(rates))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": PV_PER_SLICE * (args.ref_views or N_VIEW) / N_VIEW / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-ellipse phantoms)",
            "config": {"workload": CONFIG_NAME, "step": "one slice per step",
                       "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


INSTR_PER_PV = [None]   # thread instructions per pixel-view update (ncu summary)


def traffic_per_launch(batch):
    """DRAM bytes (read + write) of one backprojection launch of `batch` slices,
    from the committed ncu summary of the same kernel (captured at its own
    batch size; the traffic grows in proportion to the slices)."""
    p = os.path.join(ROOT, "profiles", "backproject_equiangular_cubic_512_ncu.md")
    if not os.path.exists(p):
        return None, None
    vals = {}
    with open(p) as f:
        for line in f:
            for key in ("traffic_bytes_per_launch:", "traffic_batch_slices:", "captured_at_commit:",
                        "thread_instructions_per_update:"):
                if line.startswith(key):
                    vals[key] = line.split(":", 1)[1].strip()
    if "traffic_bytes_per_launch:" not in vals or "traffic_batch_slices:" not in vals:
        return None, None
    src = "profiles/backproject_equiangular_cubic_512_ncu.md, captured at commit %s" % \
        vals.get("captured_at_commit:", "unknown")
    INSTR_PER_PV[0] = float(vals["thread_instructions_per_update:"]) \
        if "thread_instructions_per_update:" in vals else None
    return (float(vals["traffic_bytes_per_launch:"]) * batch /
            float(vals["traffic_batch_slices:"]), src)


def batched_uneven(args, torch, cg, device, phantoms, rank):
    """The uneven batch: 64 seeded problems (5-20 random ellipses each), image
    side from {128, 256, 512, 1024}, views U[180, 1440], detectors 1.4 x side,
    geometry parallel / equiangular / equilinear; abs_hamming 0.54 by FFT with
    zero-pad 2, cubic.  Sinograms simulated on the device; all reconstructions
    run as one ctgpu_batch (autotuned launch shape, CUDA-graph replay), timed
    with CUDA events over `steps` runs, next to the same problems run one plan
    after another."""
    rng = np.random.default_rng(2024 + rank)
    geos = ("parallel", "equiangular", "equilinear")
    probs, total_pv = [], 0
    scans = []
    for i in range(args.batched_problems):
        side = int(rng.choice([128, 256, 512, 1024]))
        nv = int(rng.integers(180, 1441))
        nd = int(round(1.4 * side))
        geo = geos[int(rng.integers(0, 3))]
        n_el = int(rng.integers(5, 21))
        ph = phantoms.make_phantom(phantoms.random_ellipses(seed=i, n=n_el))
        sc = cg.Scanner(ph, geo, nd, nv)
        sino = device.alloc_sinogram(nv, nd)
        ang = device.raysums(sc, ph, sino)
        scans.append((sc, ph, sino, nd * nv, nd * nv * n_el))
        probs.append(dict(geometry=sc.geometry(), nx=side, ny=side, sino=sino, angles=ang,
                          image=torch.zeros((side, side), device="cuda"),
                          filter_name="abs_hamming", filter_param=0.54, filter_method="fft",
                          zeropad=2, interp="cubic", backproj="table"))
        total_pv += side * side * nv
    batch = device.BatchPlan(probs, autotune=True, graph=True)
    stream = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 2)):
        batch.run()
    cg.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        batch.run()
    e1.record(stream)
    torch.cuda.synchronize()
    cg.sync()
    ms = e0.elapsed_time(e1) / args.steps
    # the same problems one plan after another (one filter + one backprojection each)
    plans = [device.ReconPlan(q["geometry"], q["nx"], q["ny"], "abs_hamming", 0.54, "fft", 2,
                              "direct", "cubic", 1, "table") for q in probs]
    for q, pl in zip(probs, plans):
        pl.run(q["sino"], q["angles"], q["image"])
    cg.sync()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for q, pl in zip(probs, plans):
        pl.run(q["sino"], q["angles"], q["image"])
    s1.record(stream)
    torch.cuda.synchronize()
    cg.sync()
    seq_ms = s0.elapsed_time(s1)
    bps, cv = batch.shape()
    # the same 64 scans in one ray launch, against the
    # per-problem sinograms made above
    msinos = [torch.empty_like(q[2]) for q in scans]
    # warm-up calls: the host staging uses two page-locked buffers in turn,
    # the second made on the second call
    for _ in range(max(args.warmup, 3)):
        device.raysums_multi([q[0] for q in scans], [q[1] for q in scans], msinos)
    torch.cuda.synchronize()
    same = all(torch.equal(m[:, :q[0].geometry().n_det], q[2][:, :q[0].geometry().n_det])
               for m, q in zip(msinos, scans))
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    for _ in range(args.steps):
        device.raysums_multi([q[0] for q in scans], [q[1] for q in scans], msinos)
    r1.record(stream)
    torch.cuda.synchronize()
    cg.sync()
    ray_ms = r0.elapsed_time(r1) / args.steps
    rays = sum(q[3] for q in scans)
    pairs = sum(q[4] for q in scans)
    return {"metric": METRIC, "value": total_pv / (ms / 1e3), "unit": UNIT,
            "raysums": {"ms_per_run": ray_ms, "ray_sums": rays,
                        "ray_sums_per_s": rays / (ray_ms / 1e3),
                        "ray_element_pairs_per_s": pairs / (ray_ms / 1e3),
                        "launch": "ctgpu_collect_projections_multi: every problem's scan in one "
                                  "ray launch (host records staged in one copy)",
                        "equal_to_per_problem_scans": bool(same)},
            "ms_per_run": ms, "problems": len(probs), "pixel_view_updates_per_run": total_pv,
            "sides": sorted({q["nx"] for q in probs}),
            "launch": "one persistent backprojection launch + per-problem filter / set-up "
                      "branches, replayed as a CUDA graph",
            "autotuned_shape": {"blocks_per_sm": bps, "views_per_stage_cap": cv},
            "one_plan_after_another": {"value": total_pv / (seq_ms / 1e3), "ms_per_run": seq_ms}}


def helical_3d(args, torch, cg, device, phantoms, rank):
    """The helical workload: 16 seeded ellipsoids over z in [-1, 1], equilinear
    detector of 1024, 1152 views per rotation, 8 rotations (z advances 0.25
    per rotation, the ray plane of each view at its own z), 180-degree linear
    z-interpolation with the equilinear fan angles and half-scan feathering at
    64 slice positions, then the FBP of the 64 slices at 1024 x 1024 (Shepp
    filter by FFT, zero-pad 2, linear interpolation) as one ctgpu_batch.
    Each phase timed with CUDA events over `steps` repetitions."""
    ell = phantoms.random_ellipsoids(seed=77 + rank, n=16, z_half=1.0)
    nrot, nvr, ndet, nslice, side = 8, 1152, 1024, 64, 1024
    nview = nrot * nvr
    z0, dz = -1.0, 2.0 / nview
    sc = cg.Scanner(phantoms.make_phantom(phantoms.ellipsoid_footprint(ell)), "equilinear", ndet,
                    nview, rotAngle=nrot * 2 * np.pi)
    g = sc.geometry()
    sino = device.alloc_sinogram(nview, ndet)
    stream = torch.cuda.current_stream()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        for _ in range(max(args.warmup, 3)):   # host staging: two buffers, used in turn
            fn()
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        cg.sync()
        return a.elapsed_time(b) / reps

    scan_ms = timed(lambda: device.raysums_ellipsoids(sc, ell, z0, dz, sino), args.steps)
    hplan = device.HelicalPlan(g, nview, equilinear=True, feather=True)
    last = hplan.n_view_out - 1
    ivs = np.linspace(last + 1, nview - last - 2, nslice).astype(int)
    zsino = torch.empty((nslice, hplan.n_view_out, sino.shape[1]), device="cuda")
    angs = [None]

    def interp():
        angs[0] = hplan.run(sino, ivs, zsino)[1]

    interp_ms = timed(interp, args.steps)
    gh = cg.Geometry.from_buffer_copy(g)
    gh.n_view = hplan.n_view_out
    probs = [dict(geometry=gh, nx=side, ny=side, sino=zsino[k], angles=angs[0][k],
                  image=torch.zeros((side, side), device="cuda"), filter_name="shepp",
                  filter_param=-1.0, filter_method="fft", zeropad=2, interp="linear",
                  backproj="table") for k in range(nslice)]
    batch = device.BatchPlan(probs, autotune=True, graph=True)
    batch.run()
    fbp_ms = timed(batch.run, args.steps)
    pv = nslice * side * side * gh.n_view
    return {"workload": "16 ellipsoids, equilinear 1024 det, 1152 views/rotation x 8, "
                        "64 slices of 1024x1024, Shepp FFT zero-pad 2",
            "scan": {"ms": scan_ms, "ray_sums_per_s": nview * ndet / (scan_ms / 1e3),
                     "ray_element_pairs_per_s": nview * ndet * 16 / (scan_ms / 1e3)},
            "z_interpolation": {"ms": interp_ms, "slices": nslice,
                                "launch": "one ctgpu_helical_plan run (180LI + feathering)"},
            "fbp": {"ms": fbp_ms, "views_per_slice": gh.n_view,
                    "value": pv / (fbp_ms / 1e3), "unit": UNIT}}


def files_io(args, torch, cg, device, sinos, angles, images, B):
    """Files on device-resident data, on the main workload's B sinograms and
    images: the .pj record pack / unpack kernels and pj2if's transpose over all
    B x 720 views (135 MB each way, larger than L2), if2 --comp's statistics
    over the B image pairs in one call (kernels, and the host-result call),
    and .pj files written and read straight from and to device memory
    (page-cache files)."""
    import tempfile
    stream = torch.cuda.current_stream()
    nv = B * N_VIEW
    flat = sinos.view(nv, -1)
    ang = torch.from_numpy(np.tile(np.asarray(angles, np.float64), B)).cuda()
    rec = torch.empty(nv * (3 + N_DET), dtype=torch.int32, device="cuda")
    back = torch.empty_like(flat)
    back_ang = torch.empty_like(ang)
    status = torch.tensor([0, -1], dtype=torch.int32, device="cuda")
    L = cg._lib.lib()
    C = __import__("ctypes")
    sh = device.stream_handle()

    def pack():
        cg._lib.check(L.ctgpu_pj_pack(C.c_void_p(flat.data_ptr()), flat.shape[1],
                                      C.c_void_p(ang.data_ptr()), nv, N_DET,
                                      C.c_void_p(rec.data_ptr()), sh))

    def unpack():
        cg._lib.check(L.ctgpu_pj_unpack(C.c_void_p(rec.data_ptr()), nv, N_DET,
                                        C.c_void_p(back.data_ptr()), back.shape[1],
                                        C.c_void_p(back_ang.data_ptr()),
                                        C.c_void_p(status.data_ptr()), sh))

    def ev():
        return torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        for _ in range(max(args.warmup, 3)):   # host staging: two buffers, used in turn
            fn()
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    reps = max(args.steps, 3)
    pack_ms = timed(pack, reps)
    unpack_ms = timed(unpack, reps)
    ok_records = bool(torch.equal(back[:, :N_DET], flat[:, :N_DET]) and torch.equal(back_ang, ang))
    rec_bytes = nv * (12 + 4 * N_DET)
    pack_bytes = nv * (4 * N_DET + 8) + rec_bytes
    unpack_bytes = rec_bytes + nv * (4 * flat.shape[1] + 8)
    # pj2if's transpose over all B x 720 views at once (135 MB each way)
    imgs_t = torch.empty((N_DET, nv), dtype=torch.float32, device="cuda")
    tr_ms = timed(lambda: device.sino_to_image(flat, N_DET, out=imgs_t), reps)
    other = images + 1e-3 * torch.randn_like(images)
    dre = torch.empty((B, 3), dtype=torch.float64, device="cuda")
    cmp_ms = timed(lambda: device.image_compare_device(images, other, out=dre), reps)
    t0 = time.perf_counter()
    for _ in range(reps):
        host_dre = device.image_compare(images, other)
    cmp_host_ms = (time.perf_counter() - t0) / reps * 1e3
    ok_cmp = bool(np.array_equal(host_dre, dre.cpu().numpy()))
    # files: B .pj files written from and read back to device memory
    tmpd = "/dev/shm" if os.path.isdir("/dev/shm") else None
    info = cg._lib.PjInfo()
    info.geometry.n_view, info.geometry.n_det = N_VIEW, N_DET
    rd = torch.empty_like(sinos)
    rd_ang = torch.empty((B, N_VIEW), dtype=torch.float64, device="cuda")
    ang1 = ang[:N_VIEW].contiguous()
    with tempfile.TemporaryDirectory(dir=tmpd) as td:
        paths = [os.path.join(td, "s%02d.pj" % b) for b in range(B)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for b in range(B):
            device.write_pj(paths[b], info, "bench", sinos[b], ang1)
        w_s = time.perf_counter() - t0
        fbytes = sum(os.path.getsize(p) for p in paths)
        t0 = time.perf_counter()
        for b in range(B):
            n = C.c_int()
            cg._lib.check(L.ctgpu_pj_read_device(paths[b].encode(), C.c_void_p(rd[b].data_ptr()),
                                                 rd.shape[2], C.c_void_p(rd_ang[b].data_ptr()),
                                                 C.byref(n), sh))
        r_s = time.perf_counter() - t0
    ok_files = bool(torch.equal(rd[:, :, :N_DET], sinos[:, :, :N_DET]))
    hbm, src, _ = peaks()

    def gbs(nbytes, ms):
        return nbytes / (ms / 1e3) / 1e9

    return {
        "workload": "%d sinograms 720 x 733 (pitch %d), %d images 512 x 512" % (B, flat.shape[1], B),
        "pj_pack": {"ms": pack_ms, "views": nv, "algorithmic_bytes": pack_bytes,
                    "gbs": gbs(pack_bytes, pack_ms), "frac_hbm": gbs(pack_bytes, pack_ms) / hbm},
        "pj_unpack": {"ms": unpack_ms, "algorithmic_bytes": unpack_bytes,
                      "gbs": gbs(unpack_bytes, unpack_ms),
                      "frac_hbm": gbs(unpack_bytes, unpack_ms) / hbm,
                      "round_trip_exact": ok_records},
        "pj2if_transpose": {"ms": tr_ms, "views": nv,
                            "gbs": gbs(8 * nv * N_DET, tr_ms),
                            "frac_hbm": gbs(8 * nv * N_DET, tr_ms) / hbm},
        "if2_compare": {"ms": cmp_ms, "pairs": B, "launches": 2,
                        "algorithmic_bytes": 8 * B * NX * NX,
                        "gbs": gbs(8 * B * NX * NX, cmp_ms),
                        "frac_hbm": gbs(8 * B * NX * NX, cmp_ms) / hbm,
                        "host_call_ms": cmp_host_ms, "host_equals_device": ok_cmp},
        "pj_files": {"files": B, "bytes": fbytes, "write_gbs": fbytes / w_s / 1e9,
                     "read_gbs": fbytes / r_s / 1e9, "round_trip_exact": ok_files,
                     "storage": tmpd or "default temp directory"},
        "hbm_peak_gbs": hbm, "hbm_peak_source": src,
    }


def fourier_recon(args, torch, cg, device, sinos, g, angles, B):
    """The direct-Fourier path on the main workload's equiangular scans:
    rebinning to parallel rays, convertFFTPolar (N = 1024), the inverse 2-D
    transform with magnitude, per 512 x 512 image; convertPolar alone; the
    oracle's restatement of one image on the host as the CPU figure."""
    import sys as _sys
    n = min(B, 8)
    out = torch.empty((NX, NX), dtype=torch.float32, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timed(fn):
        fn(0)
        torch.cuda.synchronize()
        ev[0].record()
        for b in range(n):
            fn(b)
        ev[1].record()
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / n

    rec_ms = timed(lambda b: out.copy_(device.reconstruct_fourier(g, sinos[b], angles, NX, NX,
                                                                   "bilinear", 1)))
    pol_ms = timed(lambda b: device.convert_polar(g, sinos[b], angles, NX, NX, "bilinear"))
    _sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    og = po.Geom(g.geometry, g.n_det, g.n_view, g.rot_inc, g.det_inc, g.focal_length,
                 g.source_detector_length, g.view_diameter, g.fan_beam_angle)
    data = sinos[0, :, :N_DET].cpu().numpy()
    t0 = time.perf_counter()
    ref = po.reconstruct_fourier(og, g.rot_start, g.det_start, data, angles, NX, NX, "bilinear", 1)
    cpu_s = time.perf_counter() - t0
    got = device.reconstruct_fourier(g, sinos[0], angles, NX, NX, "bilinear", 1).cpu().numpy()
    err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    return {"workload": "733 x 720 equiangular -> parallel -> 512 x 512, bilinear, zeropad 1 "
                        "(transform length 1024)",
            "reconstruct_fourier_ms_per_image": rec_ms, "images_per_s": 1e3 / rec_ms,
            "convert_polar_ms_per_image": pol_ms,
            "rel_l2_vs_fp64_oracle": err,
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "images/s", "cores": 1,
                             "kind": "port", "sample": "one image, FP64 restatement "
                             "(radix-2 FFTs)"}}


def batch_vs_plan(args):
    """The cost of the uneven-batch path's generality: N identical problems of
    the main workload's shape (equiangular 733 x 720 -> 512 x 512, cubic,
    abs_hamming FFT zero-pad 2) as one ctgpu_batch and through one plan's
    ctgpu_recon_run_batch, each timed with CUDA events over `steps` runs.
    Prints one JSON line; nothing else runs."""
    import torch
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms
    torch.cuda.set_device(0)
    n = args.batch_vs_plan
    probs = []
    for i in range(n):
        ph = phantoms.make_phantom(phantoms.random_ellipses(seed=i, n=12))
        sc = cg.Scanner(ph, "equiangular", N_DET, N_VIEW)
        sino = device.alloc_sinogram(N_VIEW, N_DET)
        ang = device.raysums(sc, ph, sino)
        probs.append(dict(geometry=sc.geometry(), nx=NX, ny=NX, sino=sino, angles=ang,
                          image=torch.zeros((NX, NX), device="cuda"),
                          filter_name="abs_hamming", filter_param=0.54, filter_method="fft",
                          zeropad=2, interp="cubic", backproj="table"))
    batch = device.BatchPlan(probs, autotune=False, graph=False)
    plan = device.ReconPlan(probs[0]["geometry"], NX, NX, "abs_hamming", 0.54, "fft", 2,
                            "direct", "cubic", 1, "table")
    sinos = torch.stack([q["sino"] for q in probs])
    images = torch.zeros((n, NX, NX), device="cuda")
    stream = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        cg.sync()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        cg.sync()
        return a.elapsed_time(b) / args.steps

    batch_ms = timed(batch.run)
    plan_ms = timed(lambda: plan.run_batch(sinos, probs[0]["angles"], images))
    pv = n * PV_PER_SLICE
    print(json.dumps({"metric": METRIC, "unit": UNIT, "problems": n, "config": CONFIG_NAME,
                      "batch": {"value": pv / batch_ms * 1e3, "ms": batch_ms,
                                "shape": batch.shape()},
                      "plan_batch": {"value": pv / plan_ms * 1e3, "ms": plan_ms}}))
    return 0


def run_gpu(args):
    import torch
    import ctsim_gb300 as cg
    from ctsim_gb300 import device, phantoms

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    B = args.batch
    stream = torch.cuda.current_stream()
    from ctsim_gb300 import sharding
    # views: every rank holds its view block of the same B slices and the
    # partial images are summed (NCCL) inside the step; problems: each rank
    # reconstructs its own B slices of a global batch of B x world
    shard_views = world > 1 and args.shard == "views"
    v0, vc = sharding.view_block(N_VIEW, rank, world) if shard_views else (0, N_VIEW)
    # --- inputs: B seeded phantoms, simulated on the device --------------------
    first = 0 if shard_views else sharding.problem_block(B * world, rank, world)[0]
    elems = [phantoms.random_ellipses(seed=first + b, n=12) for b in range(B)]
    phs = [phantoms.make_phantom(e) for e in elems]
    # one scanner (its geometry from the first phantom) scans every phantom
    sc = cg.Scanner(phs[0], "equiangular", N_DET, N_VIEW, nSample=1)
    g = sc.geometry()
    pitch = device.pitch_for(N_DET)
    sinos = torch.zeros((B, N_VIEW, pitch), device="cuda")
    filtered = torch.zeros((B, N_VIEW, pitch), device="cuda")
    images = torch.zeros((B, NX, NX), device="cuda")
    plan = device.ReconPlan(g, NX, NX, "abs_hamming", 0.54, "fft", 2, "direct", "cubic", 1, "table")
    angles = [None]

    block = torch.zeros((B, vc, pitch), device="cuda") if shard_views else None
    fblock = torch.zeros_like(block) if shard_views else None

    def raysum_step():
        # every phantom's ray-sums in one launch
        angles[0] = device.raysums_batch(sc, phs, sinos)

    def fbp_step(bp_events=None):
        if shard_views:
            # this rank's view block of every slice: one filter launch, one
            # batched backprojection without PostProcessing, the image sum
            # over the ranks, PostProcessing
            plan.filter(block.view(B * vc, pitch), fblock.view(B * vc, pitch))
            if bp_events is not None:
                bp_events[0].record(stream)
            plan.backproject_batch(fblock, angles[0][v0:v0 + vc], images, postprocess=False)
            if bp_events is not None:
                bp_events[1].record(stream)
            sharding.reduce_partial_images(images)
            for b in range(B):
                plan.postprocess(images[b])
            return
        # ctgpu_recon_run_batch: one filter launch for the batch's B x n_view
        # rows, which also writes the interval rows; the tile records; one
        # backprojection launch for the B slices
        plan.run_batch(sinos, angles[0], images)

    for _ in range(max(args.warmup, 1)):
        raysum_step()
        if shard_views:
            block.copy_(sinos[:, v0:v0 + vc])
        fbp_step()
    cg.sync()
    dev_peaks = measured_device_peaks(device.stream_handle())
    torch.cuda.synchronize()

    # --- timed: FBP --------------------------------------------------------------
    bp_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
             for _ in range(args.steps)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for k in range(args.steps):
            fbp_step(bp_ev[k])
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    cg.sync()
    fbp_ms = reduce_max(e0.elapsed_time(e1), world)
    if shard_views:
        bp_avg_ms = float(np.mean([s.elapsed_time(e) for (s, e) in bp_ev]))
        filt_avg_ms = None
    else:
        # the step's kernels apart, CUDA events on the launching stream: the
        # filter launch over B x n_view rows, and the batched backprojection
        # (its tile records, and here its own interval-row pass, then the main
        # kernel; the ncu launch list gives the main kernel's share)
        fe = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        for k in range(args.steps):
            fe[k][0].record(stream)
            plan.filter(sinos.view(B * N_VIEW, pitch), filtered.view(B * N_VIEW, pitch))
            fe[k][1].record(stream)
            bp_ev[k][0].record(stream)
            plan.backproject_batch(filtered, angles[0], images)
            bp_ev[k][1].record(stream)
        torch.cuda.synchronize()
        cg.sync()
        filt_avg_ms = float(np.mean([s.elapsed_time(e) for (s, e) in fe]))
        bp_avg_ms = float(np.mean([s.elapsed_time(e) for (s, e) in bp_ev]))

    # --- timed: ray-sums -----------------------------------------------------------
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    r0.record(stream)
    for k in range(args.steps):
        raysum_step()
    r1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    cg.sync()
    ray_ms = reduce_max(r0.elapsed_time(r1), world)

    # --- e2e: the C-ABI host-buffer batch call, copies inside ---------------------
    # page-locked host sinograms [B, n_view, n_det] in, images [B, nx, ny] out;
    # ctgpu_recon_run_batch_host overlaps the copies of one chunk with the
    # reconstruction of the previous one and returns when the images are in
    # host memory
    host_images = torch.zeros((B, NX, NX), dtype=torch.float32).pin_memory()
    if shard_views:
        # this rank's view block from page-locked host memory, the sharded
        # step (image sum inside), the images back to the host
        host_block = sinos[:, v0:v0 + vc, :N_DET].contiguous().cpu().pin_memory()
        e2e_chunks = [B]

        def e2e_call():
            block[:, :, :N_DET].copy_(host_block, non_blocking=True)
            fbp_step()
            host_images.copy_(images, non_blocking=True)
            torch.cuda.current_stream().synchronize()
        h2d_bytes = B * vc * N_DET * 4 + vc * 8
    else:
        host_sinos = sinos[:, :, :N_DET].contiguous().cpu().pin_memory()
        e2e_chunks = plan.host_chunks(B)

        def e2e_call():
            plan.run_batch_host(host_sinos, angles[0], host_images)
        h2d_bytes = B * N_VIEW * N_DET * 4 + len(e2e_chunks) * N_VIEW * 8
    e2e_call()
    barrier(world)
    e2e_steps = max(1, args.steps)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        e2e_call()
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    # parity spot check against the device path, and of the per-slice host call
    dev_imgs = images.cpu().numpy()
    e2e_err = float(np.linalg.norm(host_images.numpy() - dev_imgs) / np.linalg.norm(dev_imgs))
    single_err = None
    if not shard_views:
        one = plan.run_host(host_sinos[B - 1].numpy(), angles[0])
        single_err = float(np.linalg.norm(one - dev_imgs[B - 1]) /
                           np.linalg.norm(dev_imgs[B - 1]))
    # one slice through the single-slice entry point (the C++ Reconstructor's
    # and pjrec's call; device-resident sinogram), CUDA events
    one_img = torch.zeros((NX, NX), device="cuda")
    for _ in range(max(args.warmup, 1)):
        plan.run(sinos[0], angles[0], one_img)
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(max(args.steps, 1)):
        plan.run(sinos[0], angles[0], one_img)
    s1.record(stream)
    torch.cuda.synchronize()
    cg.sync()
    single_ms = s0.elapsed_time(s1) / max(args.steps, 1)
    # the same slice end to end through ctgpu_recon_run_host (pjrec's and the
    # C++ Reconstructor's host-buffer call): sinogram up, image back, per call
    host_one = np.ascontiguousarray(sinos[0, :, :N_DET].cpu().numpy())
    plan.run_host(host_one, angles[0])
    reps = max(args.steps, 5)
    t0 = time.perf_counter()
    for _ in range(reps):
        plan.run_host(host_one, angles[0])
    single_host_ms = (time.perf_counter() - t0) / reps * 1e3

    batched = batched_uneven(args, torch, cg, device, phantoms, rank) \
        if args.batched_problems > 0 else None
    helical = helical_3d(args, torch, cg, device, phantoms, rank) if args.helical else None
    files = files_io(args, torch, cg, device, sinos, angles[0], images, B) if args.files else None
    fourier = fourier_recon(args, torch, cg, device, sinos, g, angles[0], B) \
        if args.fourier else None

    if rank != 0:
        return 0
    steps = args.steps
    # views: the ranks share the B slices (total work fixed); problems: each
    # rank adds its own B slices
    slices_total = B if shard_views else B * world
    ray_world = 1 if shard_views else world   # views: every rank scans the same phantoms
    total_pv = PV_PER_SLICE * slices_total * steps
    value = total_pv / (fbp_ms / 1e3)
    hbm, src, sm_mhz = peaks()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_nominal = sms * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    fp32_peak = max(dev_peaks["ffma_tflops"], dev_peaks["ffma2_tflops"])
    bp_s = bp_avg_ms / 1e3
    flops = FLOP_PER_PV * PV_PER_SLICE * B
    traffic, traffic_src = traffic_per_launch(B)
    gather_gbs = BYTES_PER_PV * PV_PER_SLICE * B / bp_s / 1e9
    cpu_v, cpu_sample, cpu_threads = cpu_fbp_rate(seed=7, seconds=args.cpu_seconds,
                                                  views=args.ref_views)
    parity = oracle_parity(elems[0], elems[B - 1], g, sinos[B - 1], images[B - 1], angles[0])
    parity["slice"] = B - 1
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": fbp_ms / steps, "higher_is_better": True,
        "scaling": "strong" if shard_views else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded random-ellipse phantoms, simulated on the device)",
        "config": {"workload": CONFIG_NAME, "batch_slices_per_step": B,
                   "l2": "inputs larger than L2 (%d sinograms x 2.1 MB + %d images x 1 MB)" % (B, B),
                   "parallelism": ("view blocks of %d slices over %d GPUs, NCCL image sum in "
                                   "the step" % (B, world)) if shard_views else
                                  ("%d slices per GPU, contiguous ranges of a batch of %d, "
                                   "no exchange" % (B, B * world)) if world > 1 else
                                  "single GPU"},
        "raysums": {"metric": "ray-sums/s", "value": RAYS_PER_SLICE * B * steps * ray_world / (ray_ms / 1e3),
                    "ms_per_step": ray_ms / steps,
                    "ray_element_pairs_per_s": RAYS_PER_SLICE * 12 * B * steps * ray_world / (ray_ms / 1e3),
                    "launch": "all %d phantoms in one launch" % B,
                    # nominal 60 FLOP per ray-element pair (box test, two affine
                    # maps, circle clip with its square root, back-map and length)
                    "roofline": {"bound": "fp32 issue", "flop_per_pair": 60,
                                 "achieved": RAYS_PER_SLICE * 12 * B * steps * ray_world * 60 /
                                             (ray_ms / 1e3) / 1e12,
                                 "peak": fp32_peak, "unit": "TFLOP/s",
                                 "frac": RAYS_PER_SLICE * 12 * B * steps * ray_world * 60 /
                                         (ray_ms / 1e3) / 1e12 / fp32_peak,
                                 "note": "one launch: each block builds the FP64 element records "
                                         "of its 4 views, then their rays; ncu: issue slots 77 % "
                                         "busy, FP64 pipe 24 % (profiles/raysum_equiangular_733x720_ncu.md)"},
                    "cpu_baseline": {"value": cpu_raysum_rate[0], "unit": "ray-sums/s",
                                     "cores": cpu_threads, "kind": "port",
                                     "sample": "one 733 x 720 equiangular scan of 12 ellipses"}},
        "roofline": {"kernel": "backproject_table_kernel<equiangular,cubic>", "bound": "fp32",
                     "achieved": flops / bp_s / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": flops / bp_s / 1e12 / fp32_peak,
                     "peak_source": "measured in-run (packed FFMA2 microkernel, the higher of "
                                    "FFMA2 %.1f and FFMA %.1f TFLOP/s); nominal %.1f TFLOP/s "
                                    "(%d SMs x %d lanes x 2 FLOP x %.0f MHz)"
                                    % (dev_peaks["ffma2_tflops"], dev_peaks["ffma_tflops"],
                                       fp32_nominal, sms, FP32_LANES_PER_SM, sm_mhz),
                     "frac_of_nominal": flops / bp_s / 1e12 / fp32_nominal,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "algorithmic_flops_per_launch": flops, "flop_per_pixel_view": FLOP_PER_PV,
                     "avg_launch_ms": bp_avg_ms, "slices_per_launch": B,
                     "hbm": {"achieved_gbs": traffic / bp_s / 1e9 if traffic else None,
                             "peak_gbs": hbm, "peak_source": src,
                             "frac": traffic / bp_s / 1e9 / hbm if traffic else None},
                     "gather": {"bytes_per_pixel_view": BYTES_PER_PV,
                                "achieved_gbs": gather_gbs,
                                "served_from": "shared memory (rows staged by bulk copies)",
                                "l2_gather16_peak_gbs": dev_peaks["l2_gather16_gbs"],
                                "frac_of_l2_gather": gather_gbs / dev_peaks["l2_gather16_gbs"],
                                "lds128_peak_gbs": dev_peaks["lds128_gbs"],
                                "frac_of_lds128": gather_gbs / dev_peaks["lds128_gbs"],
                                "l2_read_peak_gbs": dev_peaks["l2_read_gbs"],
                                "peak_source": "measured in-run"},
                     # what the kernel executes: thread instructions per
                     # update (the ncu summary) at the live launch time,
                     # against 4 schedulers x 32 lanes per SM per cycle
                     "issue": None if INSTR_PER_PV[0] is None else {
                         "thread_instructions_per_update": INSTR_PER_PV[0],
                         "achieved_tinst_per_s": INSTR_PER_PV[0] * PV_PER_SLICE * B / bp_s,
                         "peak_tinst_per_s": sms * 4 * 32 * sm_mhz * 1e6,
                         "frac": INSTR_PER_PV[0] * PV_PER_SLICE * B / bp_s /
                                 (sms * 4 * 32 * sm_mhz * 1e6),
                         "source": "instruction count from the profile's ncu capture"},
                     "device_peaks": dev_peaks},
        "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cpu_threads, "kind": "port",
                         "sample": cpu_sample},
        "parity_vs_fp64_oracle": parity,
        "e2e": {"value": PV_PER_SLICE * slices_total * e2e_steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": h2d_bytes * world,
                "d2h_bytes_per_step": B * NX * NX * 4 * world,
                "steps": e2e_steps, "ms_per_step": e2e_s / e2e_steps * 1e3,
                "path": ("view-sharded step with page-locked host blocks in and images out "
                         "(sharding.reconstruct_views_batch's calls)") if shard_views else
                        "ctgpu_recon_run_batch_host (page-locked host buffers, chunks of "
                        "%s slices, copies overlapped with compute)" % "+".join(map(str, e2e_chunks)),
                "parity_vs_device_rel_l2": e2e_err,
                "single_slice_run_host_rel_l2": single_err},
        # per step: one filter launch; interval rows, tile records and the
        # backprojection itself for the batch
        "single_slice": {"ms": single_ms, "value": PV_PER_SLICE / (single_ms / 1e3), "unit": UNIT,
                         "call": "ctgpu_recon_run (one slice, its views in groups of blocks; "
                                 "the same angles each call, so the plan keeps its tile records)",
                         "e2e": {"value": PV_PER_SLICE / (single_host_ms / 1e3), "unit": UNIT,
                                 "ms": single_host_ms,
                                 "h2d_bytes_per_call": N_VIEW * N_DET * 4 + N_VIEW * 8,
                                 "d2h_bytes_per_call": NX * NX * 4,
                                 "call": "ctgpu_recon_run_host (pageable numpy buffers, "
                                         "synchronous)"}},
        # per step: filter (rows fused), tile records, backprojection; sharded
        # by views: filter, interval rows, tile records, backprojection and B
        # PostProcessing launches
        "gpu_launches": steps * ((4 + B) if shard_views else 3),
        "filter": None if filt_avg_ms is None else {
            "kernel": "fft_filter_persistent_kernel<11>", "avg_launch_ms": filt_avg_ms,
            "rows_per_launch": B * N_VIEW,
            "algorithmic_bytes_per_launch": B * N_VIEW * N_DET * 8,
            "achieved_gbs": B * N_VIEW * N_DET * 8 / (filt_avg_ms / 1e3) / 1e9,
            "frac_hbm": B * N_VIEW * N_DET * 8 / (filt_avg_ms / 1e3) / 1e9 / hbm,
            # FFT-filter FLOP per view: two transforms of 2.5 N log2 N and a 6 N product
            "flop_per_launch": B * N_VIEW * (2 * 2.5 * 2048 * 11 + 6 * 2048),
            "note": "two views per complex transform of length 2048; the launch of "
                    "ctgpu_recon_run_batch also writes the 16-byte interval rows"},
        "batched_uneven": batched,
        "helical": helical,
        "files": files,
        "fourier": fourier,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--shard", default="problems", choices=["problems", "views"],
                    help="with several GPUs: each rank its own slices of a global batch "
                         "(problems, weak scaling) or every rank a view block of the same "
                         "slices with the images summed in the step (views, strong scaling)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--helical", type=int, default=1,
                    help="measure the helical 3-D workload after the main one (0: skip)")
    ap.add_argument("--fourier", type=int, default=1,
                    help="measure the direct-Fourier reconstruction after the main workload "
                         "(0: skip)")
    ap.add_argument("--files", type=int, default=1,
                    help="measure the device-resident file I/O after the main workload (0: skip)")
    ap.add_argument("--batched-problems", type=int, default=64,
                    help="problems of the uneven batch measured after the main workload (0: skip)")
    ap.add_argument("--ref-views", type=int, default=None,
                    help="views per CPU sample slice (default: all 720)")
    ap.add_argument("--batch-vs-plan", type=int, default=0,
                    help="only compare N identical problems as one ctgpu_batch and through "
                         "one plan, then exit (0: the normal run)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.batch_vs_plan > 0:
        return batch_vs_plan(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
