"""Benchmark of the per-pixel Mandelbrot path on GB300.

Workload (one step): the 1920x1080 view with 4x4 multisampling (33,177,600
samples) at -0.743643887037151+0.131825904205330i, width 1e-12, N 50,000,
series tolerance 1e-10 -- rendered by the FP32-floatexp perturbation kernel,
with the plain FP64 perturbation kernel measured beside it on the same
precomputed orbit.  The metric is pixel-iterations per second: the sum of
the samples' escape counts (series-skipped iterations included, interior
samples counted as N) over the render time.

`value`  : device time of the render kernel, inputs resident, L2 flushed
           between steps.
`e2e`    : the same through the C ABI with host buffers, as the reference
           renders a view: the host precompute (probe search, orbit, series),
           upload of its tables, render, multisample reduce, copy of the
           reduced grid to host.
The line also carries `c3_deep`: the 3840x2160 view at width 1e-300 rendered
on the FE32 path and, for comparison, on the plain FP64 path over the whole
frame; and `exact_vs_reference_mp`: both C2 grids against the reference's own
arbitrary-precision continuation on a seeded sample.
--impl reference : the reference algorithm (the oracle's restatement of
           mandelbrot.cpp, arbitrary-precision continuation) on the host cores.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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
PEAKS_SRC = os.path.join(ROOT, "bench_peaks.cu")
PEAKS_LIB = os.path.join(ROOT, "_bench_build", "libbench_peaks.so")


def build_peaks(force=False):
    """Compiles bench_peaks.cu (the FP32 / FP64 issue-ceiling probes, the
    roofline denominators) for sm_103a into _bench_build/; the library is the
    benchmark's, not the product's."""
    if not force and os.path.exists(PEAKS_LIB) and os.path.getmtime(PEAKS_LIB) >= os.path.getmtime(PEAKS_SRC):
        return PEAKS_LIB
    os.makedirs(os.path.dirname(PEAKS_LIB), exist_ok=True)
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    tmp = PEAKS_LIB + ".tmp%d" % os.getpid()
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-Xcompiler", "-fPIC",
                    "-shared", PEAKS_SRC, "-o", tmp], check=True)
    os.replace(tmp, PEAKS_LIB)
    return PEAKS_LIB


def peak_flops(kind):
    """Measured FP32 FMA (0), FP64 FMA (1) or FP64 unfused multiply + add (2)
    flop/s of the current GPU."""
    import ctypes
    lib = ctypes.CDLL(build_peaks())
    lib.bench_peak_flops.restype = ctypes.c_int
    lib.bench_peak_flops.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    v = ctypes.c_double(0.0)
    rc = lib.bench_peak_flops(int(kind), ctypes.byref(v))
    if rc:
        raise RuntimeError("bench_peak_flops(%d) failed: %d" % (kind, rc))
    return v.value
sys.path.insert(0, ROOT)

CENTER = ("-0.743643887037151", "0.131825904205330")
WIDTH = "1e-12"
NR, NC, SC, N_ITER, TOL = 1080, 1920, 4, 50000, 1e-10
METRIC = "pixel-iters/s on 1 GB300: FP32-floatexp vs plain FP64, >=99.99% px exact iter"
# Algorithmic flops of one perturbation step (t = 2Z + d: 2 add; t*d: 4 mul
# 2 add; + eps: 2 add; Y = Z + d: 2 add; |Y|^2: 2 mul 1 add; |d|^2: 2 mul 1 add).
FLOPS_PER_ITER = 18


def step_string_for(cols):
    from decimal import Decimal, getcontext
    getcontext().prec = 40
    return str(Decimal(WIDTH) / Decimal(cols))


def step_string():
    return step_string_for(NC)


def workload_config():
    return {"workload": "newman C2 view 1920x1080 x 4x4 samples, width 1e-12, N 50000",
            "center": "%s%+si" % (CENTER[0], CENTER[1].lstrip("+")), "rows": NR, "cols": NC,
            "multisample": SC, "samples": NR * NC * SC * SC, "max_iter": N_ITER,
            "sa_tolerance": TOL, "l2": "flushed (256 MB write) between timed steps"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(ms, device=None):
    """The largest of every rank's step time (the job is as slow as its
    slowest replica); the value itself with one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# FE32 step: 1.339e12 thread instructions for 1.209e10 steps, the iteration
# kernel alone (--fe32-overlap 0) on the central 540x960-pixel crop (ncu,
# smsp__thread_inst_executed.sum of fe_iter_kernel)
INSTR_PER_ITER = 110.7


def issue_roofline(executed, iter_ms, clocks):
    """Thread instructions per second of the FE32 iteration pass against the
    GPU's issue peak (4 x 32 lanes per SM per clock)."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if not mhz or not iter_ms:
        return None
    achieved = executed * INSTR_PER_ITER / (iter_ms * 1e-3)
    peak = 4 * 32 * sms * mhz * 1e6
    return {"achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "T thread-instr/s",
            "frac": achieved / peak, "instr_per_iter": INSTR_PER_ITER,
            "note": "FE32 steps of the iteration pass (the overlapped FP64 rework's "
                    "instructions are not counted); inactive lanes count as lost issue"}


def replica_value(units_per_replica, world, ms):
    """Whole-job throughput of `world` independent replicas, each processing
    units_per_replica in a step of ms (the slowest rank's) milliseconds."""
    return units_per_replica * world / (ms * 1e-3)


def c1_double_loop(nm):
    """The 640x480 view at -0.75+0i, width 3, N 1024, where the reference
    takes its double loop (getIterationsHW): the GPU's double loop (device
    time, 3 renders after a warm-up) against the oracle's restatement of the
    reference on the whole frame, one thread and all host threads; the escape
    counts must agree everywhere."""
    from oracle import oracle
    nr, nc, N, step = 480, 640, 1024, "0.0046875"
    m = nm.Mandelbrot(nr, nc)
    m.set_view("-0.75", "0", step, step, N, TOL)
    m.set_path(nm.PATH_REFERENCE)
    m.precompute()
    m.render()
    gpu = []
    for _ in range(3):
        m.render()
        gpu.append(m.stat(nm.STAT_KERNEL_NS) * 1e-6)
    g = m.grid()["iterations"]
    out = {"samples": nr * nc, "effective_iters": int(g.astype(np.int64).sum()),
           "gpu_ms": min(gpu)}
    for label, threads in (("cpu_ms_1_thread", 1), ("cpu_ms_all_threads", os.cpu_count() or 1)):
        o = oracle.OracleView(nr, nc)
        o.set_view("-0.75", "0", step, step, N, TOL)
        o.precompute(threads=threads)
        t0 = time.perf_counter()
        it, _ = o.render_rows(0, nr, threads=threads)
        out[label] = (time.perf_counter() - t0) * 1e3
        out["identical"] = bool(np.array_equal(it, g))
    out["cores"] = os.cpu_count() or 1
    return out


def cpu_reference(seconds, threads, seed=7):
    """The reference algorithm on the host: getIterations with its
    arbitrary-precision continuation, on a seeded random sample of the
    workload's samples until `seconds` of work is done.  Returns
    (pixel-iters/s, samples, threads)."""
    from oracle import oracle
    o = oracle.OracleView(NR, NC)
    o.set_view(CENTER[0], CENTER[1], step_string(), step_string(), N_ITER, TOL)
    o.scale_up(SC)
    o.precompute(threads=threads)
    rng = np.random.default_rng(seed)
    nr, nc = o.rows, o.cols
    total_it, total_px, elapsed = 0, 0, 0.0
    batch = max(16, 8 * threads)
    while elapsed < seconds:
        k = rng.choice(nr * nc, size=batch, replace=False)
        t0 = time.perf_counter()
        it, _ = o.render_pixels(k // nc, k % nc, oracle.MODE_REF, threads=threads)
        elapsed += time.perf_counter() - t0
        total_it += int(it.astype(np.int64).sum())
        total_px += batch
    return total_it / elapsed, total_px, threads


def reference_agreement(nm, grids, n_samples, seed=11):
    """Escape counts of the grids (name -> escape-count array of the
    workload) against the reference's own semantics -- getIterations with its
    arbitrary-precision continuation (the oracle's MODE_REF) -- on a seeded
    random sample of the workload's samples, on all host threads."""
    from oracle import oracle
    threads = os.cpu_count() or 1
    o = oracle.OracleView(NR, NC)
    o.set_view(CENTER[0], CENTER[1], step_string(), step_string(), N_ITER, TOL)
    o.scale_up(SC)
    o.precompute(threads=threads)
    nr, nc = o.rows, o.cols
    rng = np.random.default_rng(seed)
    k = rng.choice(nr * nc, size=n_samples, replace=False)
    rr, cc = (k // nc).astype(np.int32), (k % nc).astype(np.int32)
    t0 = time.perf_counter()
    it, _ = o.render_pixels(rr, cc, oracle.MODE_REF, threads=threads)
    cpu_s = time.perf_counter() - t0
    out = {"samples": int(n_samples), "seed": seed, "oracle": "MODE_REF (MP continuation)",
           "cpu_s": cpu_s, "threads": threads}
    for name, g in grids.items():
        out["exact_" + name] = float((g[rr, cc] == it).mean())
    return out


def mp_path(nm, stream, flush):
    """The reference-exact path on the same workload: the reference's series
    front and its arbitrary-precision continuation with GMP mpf's truncations
    reproduced on the GPU; one render timed (device time, L2 flushed)."""
    m = nm.Mandelbrot(NR, NC)
    m.set_view(CENTER[0], CENTER[1], step_string(), step_string(), N_ITER, TOL)
    m.scaleUp(SC)
    m.set_path(nm.PATH_MP)
    m.precompute()
    m.upload()
    times = []
    for i in range(2):
        with torch_stream(stream):
            flush.zero_()
        e0, e1 = cuda_events()
        e0.record(stream)
        m.render_rows(0, m.rows(), stream.cuda_stream)
        e1.record(stream)
        m.synchronize()
        stream.synchronize()
        if i:
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    g = m.grid()["iterations"]
    eff = int(g.astype(np.int64).sum())
    executed = m.stat(nm.STAT_EXECUTED_ITERS)
    return {"ms": ms, "value": eff / (ms * 1e-3), "unit": "pixel-iters/s",
            "executed_iters": executed, "executed_iters_per_s": executed / (ms * 1e-3),
            "precision_bits": m.stat(nm.STAT_PRECISION_BITS)}, g


def c3_deep(nm, steps, flush, stream, args=None):
    """The 3840x2160 view at width 1e-300 (N 1,000,000, 1100-bit orbit at the
    view center, floatexp series; seeded boundary-following center): the FE32
    frame timed over `steps` renders, and the plain FP64 path over the WHOLE
    frame on the same orbit, with the exact-count fraction between them."""
    from decimal import Decimal, getcontext
    nr, nc, N, bits = 2160, 3840, 1000000, 1100
    cre, cim, width = deep_view()
    getcontext().prec = 340
    step = str(Decimal(width) / nc)
    m = nm.Mandelbrot(nr, nc)
    m.set_view(cre, cim, step, step, N, TOL, bits)
    m.set_path(nm.PATH_FE32)
    m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    m.set_option(nm.OPT_KEEP_SMOOTH64, 1)
    apply_orbit_options(nm, m, args)
    t0 = time.perf_counter()
    m.precompute()
    precompute_s = time.perf_counter() - t0
    m.upload()

    def timed(mm, k, w):
        ts = []
        for i in range(w + k):
            with torch_stream(stream):
                flush.zero_()
            e0, e1 = cuda_events()
            e0.record(stream)
            mm.render_rows(0, mm.rows(), stream.cuda_stream)
            e1.record(stream)
            mm.synchronize()
            stream.synchronize()
            if i >= w:
                ts.append(e0.elapsed_time(e1))
        return ts

    fe_times = timed(m, steps, 1)
    fe_ms = float(np.mean(fe_times))
    g = m.grid()
    s64 = m.smoothing64()
    eff = int(g["iterations"].astype(np.int64).sum())
    executed = m.stat(nm.STAT_EXECUTED_ITERS)
    rework = m.stat(nm.STAT_FP64_REWORK)
    timeouts = m.stat(nm.STAT_WAIT_TIMEOUTS)
    fp = m.copy()
    fp.set_path(nm.PATH_FP64)
    fp.set_option(nm.OPT_KEEP_SMOOTH64, 1)
    fp.upload()
    fp_times = timed(fp, 1, 0)
    fp_ms = float(np.mean(fp_times))
    gf = fp.grid()
    same = gf["iterations"] == g["iterations"]
    d = np.abs(fp.smoothing64() - s64)[same]
    fe_rate = eff / (fe_ms * 1e-3)
    fp_rate = eff / (fp_ms * 1e-3)
    return {"workload": "3840x2160, 1 sample a pixel, width 1e-300, N 1000000, 1100-bit "
                        "orbit at the seeded deep center, floatexp series",
            "width": width, "orbit_length": m.stat(nm.STAT_ORBIT_LENGTH),
            "precompute_s": precompute_s, "fe32_ms": fe_ms,
            "fe32_step_ms": [round(t, 3) for t in fe_times], "fe32_value": fe_rate,
            "fp64_ms_whole_frame": fp_ms, "fp64_value": fp_rate, "unit": "pixel-iters/s",
            "speedup_vs_fp64": fp_ms / fe_ms,
            "exact_iter_fraction_vs_fp64": float(same.mean()),
            "max_dsmooth_exact_samples": float(d.max()) if d.size else None,
            "executed_iters": executed, "effective_iters": eff,
            "executed_iters_per_s": executed / (fe_ms * 1e-3),
            "fp64_rework_samples": rework, "wait_timeouts": timeouts,
            "cardioid_undecided": m.stat(nm.STAT_CARDIOID_UNDECIDED),
            "interior_fraction": float((g["iterations"] == N).mean())}


def apply_orbit_options(nm, m, args):
    """--orbit-stage / --l2-window: the FE32 iteration pass's staged orbit
    prefix and persisting L2 window (library defaults when not given)."""
    if getattr(args, "orbit_stage", None) is not None:
        m.set_option(nm.OPT_ORBIT_STAGE, args.orbit_stage)
    if getattr(args, "l2_window", None) is not None:
        m.set_option(nm.OPT_L2_WINDOW, args.l2_window)
    if getattr(args, "fe32_overlap", None) is not None:
        m.set_option(nm.OPT_FE32_OVERLAP, args.fe32_overlap)


def torch_stream(stream):
    import torch
    return torch.cuda.stream(stream)


def cuda_events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    value, px, cores = cpu_reference(min(20.0, 4.0 * max(1, args.steps)), threads)
    line = {"metric": METRIC, "value": value, "unit": "pixel-iters/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "mpf",
            "data": "synthetic view (no dataset)", "config": workload_config(),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "pixel-iters/s", "cores": cores,
                             "kind": "port",
                             "sample": "%d random samples of the 33,177,600, reference "
                                       "getIterations (MP continuation)" % px},
            "e2e": {"value": value, "unit": "pixel-iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    global NR, NC
    import torch
    import newman_gb300 as nm

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    step = step_string()
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def make(path):
        m = nm.Mandelbrot(NR, NC)
        m.set_view(CENTER[0], CENTER[1], step, step, N_ITER, TOL)
        m.scaleUp(SC)
        m.set_path(path)
        apply_orbit_options(nm, m, args)
        return m

    primary = nm.PATH_FE32 if args.path == "fe32" else nm.PATH_FP64
    if args.profile:
        # One render per path of the central 1/div x 1/div crop of the workload
        # (same center and sample step, fewer samples): the case the ncu
        # captures run on.
        NR, NC = NR // args.profile, NC // args.profile
        for path in (nm.PATH_FE32, nm.PATH_FP64, nm.PATH_MP):
            mm = make(path)
            mm.precompute()
            mm.render()
            print("profile case %dx%d samples, path %d: %.1f ms, rework %d, executed steps %d" % (
                mm.rows(), mm.cols(), path, mm.stat(nm.STAT_KERNEL_NS) * 1e-6,
                mm.stat(nm.STAT_FP64_REWORK), mm.stat(nm.STAT_EXECUTED_ITERS)))
        return
    m = make(primary)
    t0 = time.perf_counter()
    m.precompute()
    precompute_s = time.perf_counter() - t0
    m.upload()
    # the plain FP64 path on the same precomputed orbit (value copy)
    fp = m.copy()
    fp.set_path(nm.PATH_FP64)
    fp.upload()

    def render_timed(mm, k, w):
        times = []
        for i in range(w + k):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                mm.render_rows(0, mm.rows(), stream.cuda_stream)
                e1.record(stream)
            mm.synchronize()
            stream.synchronize()
            if i >= w:
                times.append(e0.elapsed_time(e1))
        return times

    render_timed(m, 0, args.warmup)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        launches0 = m.stat(nm.STAT_KERNEL_LAUNCHES)
        wall0 = time.perf_counter()
        times = render_timed(m, args.steps, 0)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        launches = m.stat(nm.STAT_KERNEL_LAUNCHES) - launches0
    barrier()
    ms = max_over_ranks(float(np.mean(times)), device="cuda")
    g = m.grid()
    eff_iters = int(g["iterations"].astype(np.int64).sum())
    executed = m.stat(nm.STAT_EXECUTED_ITERS)
    rework = m.stat(nm.STAT_FP64_REWORK)
    front_fp64 = m.stat(nm.STAT_FRONT_FP64)
    timeouts = m.stat(nm.STAT_WAIT_TIMEOUTS)
    undecided = m.stat(nm.STAT_CARDIOID_UNDECIDED)
    k_main_ms = m.stat(nm.STAT_KERNEL_NS) * 1e-6
    k_rework_ms = m.stat(nm.STAT_REWORK_KERNEL_NS) * 1e-6
    k_iter_ms = m.stat(nm.STAT_ITER_KERNEL_NS) * 1e-6
    value = replica_value(eff_iters, world, ms)

    # the plain FP64 path: timed on the same workload, and the comparison grid
    fp64_ms = None
    if primary != nm.PATH_FP64:
        render_timed(fp, 0, 1)
        fp64_ms = float(np.mean(render_timed(fp, max(1, min(args.steps, 2)), 0)))
    gf = fp.grid()
    same = gf["iterations"] == g["iterations"]
    exact = float(same.mean())
    dsm = np.abs(gf["smoothing"].astype(np.float64) - g["smoothing"])
    max_dsmooth_exact = float(dsm[same].max()) if same.any() else None
    red_fe = m.reduce(SC)
    red_fp = fp.reduce(SC)
    exact_px = float((red_fe["iterations"] == red_fp["iterations"]).mean())
    agreement, mp_line = None, None
    if rank == 0 and not args.no_mp:
        mp_line, g_mp = mp_path(nm, stream, flush)
    if rank == 0 and not args.no_cpu and args.ref_samples > 0:
        grids = {"fe32": g["iterations"], "fp64": gf["iterations"]}
        if mp_line is not None:
            grids["mp"] = g_mp
        agreement = reference_agreement(nm, grids, args.ref_samples)
    del gf, dsm, same

    # e2e through the C ABI with host buffers, as the reference renders a view
    # (precompute(), then the rows): the host precompute (probe search, orbit,
    # series), the upload of its tables, the render, the multisample reduce and
    # the copy of the reduced grid to host; L2 flushed before every step
    red = np.empty((NR, NC), nm.ESCAPE_DTYPE)
    e2e_times, pre_times = [], []
    for i in range(1 + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m.precompute()
        t1 = time.perf_counter()
        m.upload()
        m.render()
        m.reduce(SC, red)
        if i:
            e2e_times.append(time.perf_counter() - t0)
            pre_times.append(t1 - t0)
    e2e_s = float(np.mean(e2e_times))
    n_sample = NR * SC * NC * SC
    h2d = 16 * (NC * SC + NR * SC) + 8 * (NC * SC + NR * SC)
    xlen = m.stat(nm.STAT_ORBIT_LENGTH)
    h2d += xlen * 16 * 6 + xlen * 8 + (xlen + 2) * 16

    line = None
    if rank == 0:
        peak32 = peak_flops(0)
        peak64 = peak_flops(2)
        peak = peak32 if primary == nm.PATH_FE32 else peak64
        # dominant kernel: the FE32 (or FP64) render kernel, its own duration
        main_ms = k_iter_ms if k_iter_ms > 0 else (k_main_ms if k_main_ms > 0 else ms)
        achieved = executed * FLOPS_PER_ITER / (main_ms * 1e-3)
        line = {
            "metric": METRIC, "value": value, "unit": "pixel-iters/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 float-float + int exponent" if primary == nm.PATH_FE32 else "fp64",
            "data": "synthetic view (no dataset)", "config": workload_config(),
            "path": args.path,
            "exact_iter_fraction_vs_fp64": exact, "exact_iter_fraction_reduced_px": exact_px,
            "max_dsmooth_exact_samples": max_dsmooth_exact,
            "fp64_front_fraction": front_fp64 / float(NR * NC * SC * SC),
            "fp64_rework_fraction": rework / float(NR * NC * SC * SC),
            "fp64_path": None if fp64_ms is None else {
                "ms_per_step": fp64_ms, "value": eff_iters / (fp64_ms * 1e-3),
                "unit": "pixel-iters/s"},
            "speedup_vs_fp64": None if fp64_ms is None else fp64_ms / ms,
            "kernel_ms": {"render_passes": k_main_ms, "iteration_pass": k_iter_ms,
                          "fp64_rework": k_rework_ms},
            "executed_iters_per_step": executed, "effective_iters_per_step": eff_iters,
            "executed_iters_per_s": executed / (ms * 1e-3),
            "wait_timeouts": timeouts, "cardioid_undecided": undecided,
            "precompute_s": precompute_s, "wall_s": wall,
            # kernels the library launched during the timed steps (its own count)
            "gpu_launches": launches,
            "roofline": {"bound": "fp32" if primary == nm.PATH_FE32 else "fp64",
                         "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "flops_per_iter": FLOPS_PER_ITER,
                         "peak_source": "measured by bench_peaks.cu on this GPU "
                                        "(FP32 FMA / FP64 unfused mul+add issue rate)",
                         # the limit that binds: instruction issue.  A float-float
                         # step executes INSTR_PER_ITER thread instructions (ncu,
                         # FE32 warps alone on the C2 view); peak = 4 schedulers x
                         # 32 lanes x SMs x the SM clock sampled during the run
                         "issue": None if primary != nm.PATH_FE32 else issue_roofline(
                             executed, k_iter_ms, clocks.summary())},
            "clocks": clocks.summary(),
            "e2e": {"value": eff_iters / e2e_s, "unit": "pixel-iters/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": NR * NC * 8,
                    "ms_per_step": e2e_s * 1e3,
                    "precompute_ms": float(np.mean(pre_times)) * 1e3,
                    "includes": "nm_precompute (host probe search, orbit, series), table "
                                "upload, render, reduce, reduced grid to host; L2 flushed"},
            "exact_vs_reference_mp": agreement,
            "mp_path": mp_line,
        }
        if not args.no_cpu:
            v, px, cores = cpu_reference(args.cpu_seconds, 1)
            line["cpu_baseline"] = {"value": v, "unit": "pixel-iters/s", "cores": cores,
                                    "kind": "port",
                                    "sample": "%d random samples of the 33,177,600, reference "
                                              "getIterations (MP continuation), 1 thread" % px}
            line["c1_double_loop"] = c1_double_loop(nm)
        if not args.no_deep:
            line["c3_deep"] = c3_deep(nm, max(1, min(args.steps, 5)), flush, stream, args)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_rows(args):
    """The C2 view split by rows across the ranks (strong scaling): every rank
    precomputes the same view and renders its block of rows
    (newman_gb300.shard); the step time is the slowest rank's; the rows are
    gathered to rank 0 on the host after the timed steps and checked against
    rank 0's own render of the whole view."""
    import torch
    import torch.distributed as dist
    import newman_gb300 as nm
    from newman_gb300.shard import gather_rows, row_range
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("gloo")
    m = nm.Mandelbrot(NR, NC)
    m.set_view(CENTER[0], CENTER[1], step_string(), step_string(), N_ITER, TOL)
    m.scaleUp(SC)
    m.set_path(nm.PATH_FE32)
    m.precompute()
    m.upload()
    r0, r1 = row_range(m.rows(), rank, world)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    times = []
    for i in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = cuda_events()
        if world > 1:
            dist.barrier()
        e0.record(stream)
        m.render_rows(r0, r1, stream.cuda_stream)
        e1.record(stream)
        m.synchronize()
        stream.synchronize()
        if i >= args.warmup:
            times.append(e0.elapsed_time(e1))
    ms = max_over_ranks(float(np.mean(times))) if world > 1 else float(np.mean(times))
    part = m.grid()[r0:r1].copy()
    full = gather_rows(part, m.rows(), m.cols(), rank, world) if world > 1 else m.grid()
    if rank == 0:
        eff = int(full["iterations"].astype(np.int64).sum())
        m.render()
        identical = bool(np.array_equal(full, m.grid()))
        print(json.dumps({
            "metric": METRIC + " (one view split by rows)", "value": eff / (ms * 1e-3),
            "unit": "pixel-iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "fp32 float-float + int exponent",
            "data": "synthetic view (no dataset)", "config": workload_config(),
            "shard": "rows", "gathered_equals_whole_render": identical}), flush=True)
    if world > 1:
        dist.destroy_process_group()


def video_views(nframes, nr, nc, w0="4.0", w1="1e-200", n0=1000, n1=500000):
    """Frames of the batched zoom video: widths geometric from w0 to w1, N
    linear from n0 to n1, into the C2 center."""
    from decimal import Decimal, getcontext
    getcontext().prec = 60
    a, b = Decimal(w0), Decimal(w1)
    out = []
    for k in range(nframes):
        t = Decimal(k) / Decimal(max(1, nframes - 1))
        out.append((str((a * (b / a) ** t) / nc), int(round(n0 + (n1 - n0) * float(t)))))
    return out


def run_video(args):
    """240 frames of 1280x720 with 2x2 samples (widths 4 -> 1e-200, N 1e3 ->
    5e5): all frames on the FE32 path in one batched CUDA-graph launch against
    frame-at-a-time plain FP64 (the reference's double loop on the frames it
    renders with doubles, the FP64 perturbation path on the others)."""
    import concurrent.futures as cf
    import torch
    import newman_gb300 as nm
    torch.cuda.set_device(0)
    nf, nr, nc, sc = args.frames, 720, 1280, 2
    views = video_views(nf, nr, nc)

    def frame(step, N, path):
        # every frame on the FE32 path: the double-loop frames certified
        # against the double loop, the others against the FP64 path
        m = nm.Mandelbrot(nr, nc)
        m.set_view(CENTER[0], CENTER[1], step, step, N, TOL)
        m.scaleUp(sc)
        m.set_path(path)
        if not m.useHardware():
            m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
        m.precompute()
        return m

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 8) as ex:
        fe_frames = list(ex.map(lambda v: frame(v[0], v[1], nm.PATH_FE32), views))
    precompute_s = time.perf_counter() - t0
    batch = nm.Batch(sc=sc)
    for f in fe_frames:
        batch.add(f)
    tuned = None
    if args.autotune:
        tuned = batch.autotune(stride=max(1, nf // 10))
    for _ in range(args.warmup):
        batch.render()
    times = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            batch.render()
            times.append(batch.stat(nm.STAT_KERNEL_NS) * 1e-6)
    ms = float(np.mean(times))
    executed = batch.stat(nm.STAT_EXECUTED_ITERS)
    rework = batch.stat(nm.STAT_FP64_REWORK)
    out = batch.frames_out()
    eff = int(sum(int(f.grid()["iterations"].astype(np.int64).sum()) for f in fe_frames))

    # frame at a time, plain FP64 (the reference's double path where it applies)
    fp_frames = [f.copy() for f in fe_frames]
    fp_ms = 0.0
    for f in fp_frames:
        f.set_path(nm.PATH_REFERENCE if f.useHardware() else nm.PATH_FP64)
        f.upload()
        f.render()  # warm
        f.render()
        fp_ms += f.stat(nm.STAT_KERNEL_NS) * 1e-6
    same = total = 0
    for a, b in zip(fe_frames, fp_frames):
        ga, gb = a.grid()["iterations"], b.grid()["iterations"]
        same += int((ga == gb).sum())
        total += ga.size
    # e2e: one graph launch plus the reduced frames to host
    e2e = []
    for _ in range(2):
        t1 = time.perf_counter()
        batch.render()
        batch.frames_out()
        e2e.append(time.perf_counter() - t1)
    line = {
        "metric": "frames/s, %d-frame zoom video (1280x720, 2x2 samples, widths 4 -> 1e-200)" % nf,
        "value": nf / (ms * 1e-3), "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 float-float + int exponent (deep frames)",
        "data": "synthetic views (no dataset)",
        "config": {"workload": "newman C4 batched zoom video", "frames": nf, "rows": nr,
                   "cols": nc, "multisample": sc, "widths": ["4.0", "1e-200"],
                   "max_iter": [1000, 500000], "autotuned": tuned},
        "frame_at_a_time_fp64": {"ms": fp_ms, "value": nf / (fp_ms * 1e-3), "unit": "frames/s"},
        "speedup_vs_fp64_frame_at_a_time": fp_ms / ms,
        "exact_iter_fraction_vs_fp64": same / total, "fp64_rework_samples": rework,
        "executed_iters_per_step": executed, "effective_iters_per_step": eff,
        "pixel_iters_per_s": eff / (ms * 1e-3), "precompute_s": precompute_s,
        "clocks": clocks.summary(),
        "e2e": {"value": nf / float(np.mean(e2e)), "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": sum(o.nbytes for o in out)},
    }
    print(json.dumps(line), flush=True)


def deep_view(k=72):
    """The view of step k of the seeded boundary-following walk committed in
    tests/golden/deep_centers.json (start: the C2 center at width 1e-12; each
    step recenters on the 64x64 render's highest non-maximal escape count and
    divides the width by 1e4): the center chosen at step k-1 and the width of
    step k (k = 72: 1e-300)."""
    with open(os.path.join(ROOT, "tests", "golden", "deep_centers.json")) as f:
        walk = json.load(f)
    s = walk["steps"]
    return s[k - 1]["next_center_re"], s[k - 1]["next_center_im"], s[k]["width"]


def run_deep(args):
    """3840x2160, 1 sample a pixel, width 1e-300, N 1,000,000, reference orbit
    at 1100 bits at the seeded deep center: the FE32 path over the whole frame
    (timed), the plain FP64 path over a band of rows for the exactness and the
    speed comparison (a whole FP64 frame takes minutes)."""
    import torch
    from decimal import Decimal, getcontext
    import newman_gb300 as nm
    torch.cuda.set_device(0)
    nr, nc, N, bits = 2160, 3840, 1000000, 1100
    cre, cim, width = deep_view()
    getcontext().prec = 340
    if args.profile:
        # one FE32 render of a 1/DIV-size crop (same center and width): the ncu case
        nr, nc = nr // args.profile, nc // args.profile
    step = str(Decimal(width) / nc)

    def make(path, rows=nr):
        m = nm.Mandelbrot(rows, nc)
        m.set_view(cre, cim, step, step, N, TOL, bits)
        m.set_path(path)
        m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
        apply_orbit_options(nm, m, args)
        return m

    m = make(nm.PATH_FE32)
    t0 = time.perf_counter()
    m.precompute()
    precompute_s = time.perf_counter() - t0
    if args.profile:
        m.render()
        print("profile case %dx%d, FE32: %.1f ms (+ %.1f ms rework after the pass), rework %d, "
              "FP64 fronts %d, executed FE32 steps %d" % (
                  nr, nc, m.stat(nm.STAT_KERNEL_NS) * 1e-6, m.stat(nm.STAT_REWORK_KERNEL_NS) * 1e-6,
                  m.stat(nm.STAT_FP64_REWORK), m.stat(nm.STAT_FRONT_FP64),
                  m.stat(nm.STAT_EXECUTED_ITERS)))
        return
    for _ in range(args.warmup):
        m.render()
    times = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            m.render()
            times.append(m.stat(nm.STAT_KERNEL_NS) * 1e-6 + m.stat(nm.STAT_REWORK_KERNEL_NS) * 1e-6)
    ms = float(np.mean(times))
    g = m.grid()["iterations"]
    eff = int(g.astype(np.int64).sum())
    executed = m.stat(nm.STAT_EXECUTED_ITERS)
    rework = m.stat(nm.STAT_FP64_REWORK)
    front_fp64 = m.stat(nm.STAT_FRONT_FP64)
    # the plain FP64 path over rows [r0, r1) of the same view and orbit
    band = max(1, nr // args.deep_band)
    r0 = (nr - band) // 2
    fp = m.copy()
    fp.set_path(nm.PATH_FP64)
    fp.upload()
    fp.render_rows(r0, r0 + band)
    fp.synchronize()
    fp_ms = fp.stat(nm.STAT_KERNEL_NS) * 1e-6
    gf = fp.grid()["iterations"][r0:r0 + band]
    gb = g[r0:r0 + band]
    exact = float((gf == gb).mean())
    eff_band = int(gb.astype(np.int64).sum())
    fe_rate = eff / (ms * 1e-3)
    fp_rate = eff_band / (fp_ms * 1e-3)
    line = {
        "metric": "pixel-iters/s, deep view 3840x2160 at width 1e-300 (FE32 vs plain FP64)",
        "value": fe_rate, "unit": "pixel-iters/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 float-float + int exponent",
        "data": "synthetic view (seeded boundary-following walk, tests/golden/deep_centers.json)",
        "config": {"workload": "newman C3 deep view", "rows": nr, "cols": nc, "multisample": 1,
                   "width": width, "max_iter": N, "precision_bits": bits,
                   "center_re": cre[:40] + "...", "center_im": cim[:40] + "...",
                   "reference": "orbit at the view center, floatexp series"},
        "orbit_length": m.stat(nm.STAT_ORBIT_LENGTH), "precompute_s": precompute_s,
        "executed_iters_per_step": executed, "effective_iters_per_step": eff,
        "step_ms": [round(t, 3) for t in times],
        "fp64_rework_samples": rework, "fp64_front_samples": front_fp64, "max_escape": int(g[g < N].max()) if (g < N).any() else None,
        "interior_fraction": float((g == N).mean()),
        "fp64_band": {"rows": [r0, r0 + band], "ms": fp_ms, "value": fp_rate,
                      "unit": "pixel-iters/s", "exact_iter_fraction_vs_fe32": exact},
        "speedup_vs_fp64": fe_rate / fp_rate,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def learned_views(count=10, seed=5):
    """The deep views of the learned-scheduling workload: stopping widths
    log-uniform in [1e-500, 1e-50] (seeded); each view has its stopping width
    and is centered where the seeded boundary-following walk
    (tests/golden/deep_centers.json) stands when its width first reaches the
    stopping width."""
    with open(os.path.join(ROOT, "tests", "golden", "deep_centers.json")) as f:
        steps = json.load(f)["steps"]
    from decimal import Decimal
    rng = np.random.default_rng(seed)
    out = []
    for e in sorted(rng.uniform(50.0, 500.0, count)):
        log_w = [Decimal(s["width"]).log10() for s in steps]
        k = next((i for i in range(1, len(steps)) if log_w[i] <= Decimal(-e)), len(steps) - 1)
        ce = int(np.ceil(e))
        width = "%.12fe-%d" % (10.0 ** (ce - e), ce)
        out.append({"stop": "1e-%.2f" % e, "k": k, "width": width,
                    "cre": steps[k - 1]["next_center_re"], "cim": steps[k - 1]["next_center_im"]})
    return out


PREVIEW_EXTRA = 512  # previews stop samples this many steps past the orbit's length


def tile_log(nm, m, sc, tile_px=32, preview_px=8):
    """Per-tile features (from a preview with one sample per preview_px x
    preview_px pixels, capped at the orbit length + PREVIEW_EXTRA) and the
    logged per-tile work of one whole render of m, on tiles of tile_px x
    tile_px pixels."""
    tile = tile_px * sc
    m.set_option(nm.OPT_TILE_W, tile)
    m.set_option(nm.OPT_TILE_H, tile)
    m.set_option(nm.OPT_LOG_TILE_COSTS, 1)
    m.render()
    costs = m.tile_costs().astype(np.float64).ravel()
    m.set_option(nm.OPT_LOG_TILE_COSTS, 0)
    f = preview_px * sc
    p = m.preview(f)
    if not p.useHardware() and p.stat(nm.STAT_ORBIT_LENGTH) == 0:
        p.precompute()
    if not p.useHardware():
        p.set_option(nm.OPT_ITER_CAP, p.stat(nm.STAT_ORBIT_LENGTH) + PREVIEW_EXTRA)
    p.render()
    return p.tile_features(tile // f, tile // f), costs


def centred_log(costs):
    y = np.log2(1.0 + costs)
    return (y - y.mean()).astype(np.float32)


def spearman(a, b):
    ra = np.argsort(np.argsort(a)).astype(np.float64)
    rb = np.argsort(np.argsort(b)).astype(np.float64)
    return float(np.corrcoef(ra, rb)[0, 1]) if ra.std() > 0 and rb.std() > 0 else None


def run_learned(args):
    """Learned-scheduled deep renders: the cost model trained on the tile costs
    of the C1, C2 and C3 views, then 10 seeded deep views (3840x2160, 2x2
    samples, N 2,000,000) rendered with the static tile order and with the
    predicted longest-first order (preview and prediction included in its
    time); the images must be identical."""
    import torch
    from decimal import Decimal, getcontext
    import newman_gb300 as nm
    torch.cuda.set_device(0)
    getcontext().prec = 700
    t_all = time.perf_counter()

    # training data: tile costs logged on the C1, C2 and C3 views
    def view(nr, nc, sc, cre, cim, width, N, bits=0, path=nm.PATH_FE32):
        m = nm.Mandelbrot(nr, nc)
        step = str(Decimal(width) / nc)
        m.set_view(cre, cim, step, step, N, TOL, bits)
        if sc > 1:
            m.scaleUp(sc)
        if not m.useHardware():
            m.set_path(path)
            m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
            m.precompute()
        return m

    dcre, dcim, dwidth = deep_view()
    train_views = [("C1", view(480, 640, 1, "-0.75", "0", "3.0", 1024), 1),
                   ("C2", view(NR, NC, SC, CENTER[0], CENTER[1], WIDTH, N_ITER), SC),
                   ("C3", view(2160, 3840, 1, dcre, dcim, dwidth, 1000000, 1100), 1)]
    X, Y, train_info = [], [], {}
    for name, m, sc in train_views:
        feats, costs = tile_log(nm, m, sc)
        X.append(feats)
        Y.append(centred_log(costs))
        train_info[name] = {"tiles": int(len(costs)), "cost_spread_log2": float(np.ptp(Y[-1]))}
        if name == "C3":
            c3_view, c3_costs = m, costs
        del m
    train_views = None
    X, Y = np.concatenate(X), np.concatenate(Y)
    model = nm.CostModel(seed=2026)
    t0 = time.perf_counter()
    loss = model.train(X, Y, epochs=args.epochs, lr=2e-3)
    train_s = time.perf_counter() - t0
    var = float(np.var(Y))

    def evaluate(m, sc, costs):
        """Static, learned (capped preview + nm_order_tiles, timed) and
        true-cost orders of one view; their images must agree."""

        def timed_render(order):
            m.set_tile_order(order)
            m.render()  # warm
            ts = []
            for _ in range(args.steps):
                m.render()
                ts.append(m.stat(nm.STAT_KERNEL_NS) * 1e-6 + m.stat(nm.STAT_REWORK_KERNEL_NS) * 1e-6)
            return float(np.mean(ts)), m.grid()

        ms_static, g_static = timed_render(None)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p = m.preview(8 * sc)
        if not p.useHardware():
            p.set_option(nm.OPT_ITER_CAP, m.stat(nm.STAT_ORBIT_LENGTH) + PREVIEW_EXTRA)
        p.render()
        m.order_tiles(p, model)
        torch.cuda.synchronize()
        over_ms = (time.perf_counter() - t0) * 1e3
        order = m.tile_order()
        pred = model.predict(p.tile_features(32 // 8, 32 // 8))  # for the error report (untimed)
        ms_learned, g_learned = timed_render(order)
        ms_oracle, g_oracle = timed_render(np.argsort(-costs, kind="stable").astype(np.int32))
        same = bool(np.array_equal(g_static, g_learned) and np.array_equal(g_static, g_oracle))
        y = centred_log(costs)
        err = pred - pred.mean() - y
        return {"orbit_length": m.stat(nm.STAT_ORBIT_LENGTH), "ms_static": ms_static,
                "ms_learned": ms_learned, "ms_overhead": over_ms, "ms_cost_order": ms_oracle,
                "speedup_with_overhead": ms_static / (ms_learned + over_ms),
                "identical": same, "spearman": spearman(pred, costs),
                "mae_log2": float(np.abs(err).mean()), "cost_spread_log2": float(np.ptp(y))}

    # the 1e-300 view (C3), whose frame time its longest samples set
    c3_row = evaluate(c3_view, 1, c3_costs)
    del c3_view

    # the deep views
    nr, nc, sc, N = 2160, 3840, 2, 2000000
    rows, t_static, t_learned, t_oracle, t_over = [], 0.0, 0.0, 0.0, 0.0
    identical = c3_row["identical"]
    for vw in learned_views():
        m = view(nr, nc, sc, vw["cre"], vw["cim"], vw["width"], N)
        feats, costs = tile_log(nm, m, sc)  # tile size set, costs for the error report
        r = evaluate(m, sc, costs)
        r.update({"width": vw["width"], "stop": vw["stop"]})
        rows.append(r)
        identical &= r["identical"]
        t_static += r["ms_static"]
        t_learned += r["ms_learned"]
        t_over += r["ms_overhead"]
        t_oracle += r["ms_cost_order"]
        del m
    speedup = t_static / (t_learned + t_over)
    sp = [r["spearman"] for r in rows if r["spearman"] is not None]
    line = {
        "metric": "learned tile order: render speedup over the static order, 10 deep views",
        "value": speedup, "unit": "x", "n_gpus": 1, "steps": args.steps, "warmup": 1,
        "ms_per_step": t_learned + t_over, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 float-float + int exponent; model fp16 weights, fp32 accumulate",
        "data": "synthetic views (seeded boundary-following walk, tests/golden/deep_centers.json)",
        "config": {"workload": "newman C5 learned-scheduled deep renders", "rows": nr, "cols": nc,
                   "multisample": sc, "max_iter": N, "views": len(rows), "tile_px": 32,
                   "preview_px": 8, "model": "18-64-64-64-1 ReLU MLP",
                   "train_views": train_info, "epochs": args.epochs},
        "train": {"tiles": int(len(Y)), "loss": loss, "target_variance": var, "seconds": train_s},
        "ms_static_total": t_static, "ms_learned_total": t_learned, "ms_overhead_total": t_over,
        "ms_cost_order_total": t_oracle, "speedup_without_overhead": t_static / t_learned,
        "c3": c3_row,
        "speedup_cost_order": t_static / t_oracle, "bit_identical": identical,
        "prediction": {"spearman_mean": float(np.mean(sp)) if sp else None,
                       "mae_log2_mean": float(np.mean([r["mae_log2"] for r in rows]))},
        "views": rows, "wall_s": time.perf_counter() - t_all,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--path", default="fe32", choices=["fe32", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mp", action="store_true",
                    help="leave out the reference-exact path's render of the workload")
    ap.add_argument("--no-deep", action="store_true",
                    help="leave out the 3840x2160 width-1e-300 comparison of the default line")
    ap.add_argument("--ref-samples", type=int, default=100000,
                    help="samples of the reference-semantics (MP continuation) check")
    ap.add_argument("--profile", type=int, default=0,
                    help="render each path once on a 1/DIV-size crop and exit (ncu case)")
    ap.add_argument("--workload", default="c2", choices=["c2", "video", "deep", "learned"])
    ap.add_argument("--epochs", type=int, default=400, help="learned workload: training epochs")
    ap.add_argument("--deep-band", type=int, default=16,
                    help="deep workload: the FP64 comparison renders 1/DEEP_BAND of the rows")
    ap.add_argument("--frames", type=int, default=240)
    ap.add_argument("--shard", default="replicas", choices=["replicas", "rows"],
                    help="rows: one C2 view split by rows across the ranks (strong scaling)")
    ap.add_argument("--orbit-stage", type=int, default=None,
                    help="FE32: orbit entries staged in shared memory (NM_OPT_ORBIT_STAGE)")
    ap.add_argument("--fe32-overlap", type=int, default=None,
                    help="FE32: 0 = the FP64 rework after the iteration pass (NM_OPT_FE32_OVERLAP)")
    ap.add_argument("--l2-window", type=int, default=None,
                    help="FE32: 1 = persisting L2 window on the orbit (NM_OPT_L2_WINDOW)")
    ap.add_argument("--autotune", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "video":
        run_video(args)
    elif args.workload == "deep":
        run_deep(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.shard == "rows":
        run_rows(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
