"""Benchmark: GameOfLife 16384^2, 2000 generations (GLUP/s), plus per-workload lines.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one whole run of the workload: the 16384^2 u8 grid (already in HBM for `value`),
2000 generations of the reference rule, population count.  `value` uses the bit-packed form
(identical states to the u8 form); `e2e` is the same run through the C-ABI host-buffer entry
point appfis_gb_life_job from pinned host memory (upload, pack, 2000 generations, unpack,
download of the final grid and the population).  Under torchrun every rank runs its own
replica (weak scaling); rank 0 prints one JSON line.

--impl reference times the reference's own CPU path (the reference headers built with
APPFIS_CPU, OpenMP on every host core, single-rank MPI stand-in; oracle/_ref) on a bounded
sample of the same grid, falling back to the oracle restatement when that build is absent.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "GLUP/s + % of HBM roofline per app; batched/mixed vs plain FP32 at fixed error"
GOL_NX = GOL_NY = 16384
GOL_GENS = 2000
GOL_SEED = 42
GOL_P = 0.3
WORKLOAD = "GameOfLife 16384x16384 u8 cells, periodic, Bernoulli(0.3) seed 42, 2000 generations, reference rule"


TB_GENS = 16  # generations per time-blocked bit-packed launch (life.cu TB_STEPS)


def profiled_traffic(kernel):
    """DRAM bytes (read + write) per launch of `kernel` from its ncu summary under profiles/
    (a line `traffic_bytes_per_launch: <kernel> <bytes>`), or None."""
    import glob
    import re
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as f:
            for line in f:
                m = re.search(r"traffic_bytes_per_launch:\s*%s\s+([0-9.eE+]+)" % re.escape(kernel), line)
                if m:
                    return float(m.group(1))
    return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle sampling (every 50 ms) around a timed region; the summary keeps
    the samples whose timestamps fall inside the region (mark_start / mark_end), and all samples
    only if none does."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)  # nvidia-smi start-up
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        import datetime
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 10:
                        rows.append(parts)
            os.unlink(self.path)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        def stamp(x):
            try:
                return datetime.datetime.strptime(x, "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                return None

        inside = [r for r in rows if self.t0 is not None and stamp(r[0]) is not None
                  and self.t0 - 0.05 <= stamp(r[0]) <= self.t1 + 0.05]
        use = inside or rows
        sm = [num(r[2]) for r in use if num(r[2]) is not None]
        mx = [num(r[3]) for r in use if num(r[3]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in use for k in range(4) if r[6 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(use), "samples_in_timed_region": len(inside)}


# ----------------------------------------------------------------------------- distributed
def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_gol_record():
    """The reference CPU path's result for this exact workload (population and a hash of the
    final state), recorded by tests/golden/make_golden.py --full-gol; None when absent."""
    p = os.path.join(ROOT, "tests", "golden", "gol_%dx%d_g%d.json" % (GOL_NX, GOL_NY, GOL_GENS))
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


# ----------------------------------------------------------------------------- CPU baseline
def cpu_gol_sample(cells, gens):
    """Reference OpenMP path (oracle/_ref/ref_gol) on the full grid for `gens` generations;
    returns (GLUP/s, cores, kind).  Falls back to the oracle restatement."""
    from oracle import build_ref
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    ny, nx = cells.shape
    if build_ref.exe_path("gol") is None:
        try:
            build_ref.build()
        except Exception:
            pass
    if build_ref.exe_path("gol") is not None:
        res, _ = O.run_ref("gol", [nx, ny, gens, cores, "{in0}", "{out0}"], [cells], [(np.uint8, 0)])
        return nx * ny * gens / res["seconds"] / 1e9, cores, "reference"
    t = time.perf_counter()
    O.gol(cells, gens, threads=cores)
    return nx * ny * gens / (time.perf_counter() - t) / 1e9, cores, "port"


def cpu_app_samples():
    """The reference's own OpenMP path (oracle/_ref harnesses, every host core) on a bounded
    sample of each other workload: GLUP/s of the sweep loop only (the harness's timer)."""
    from oracle import build_ref
    from oracle import oracle as O
    from appfis_gb300 import workloads as W

    cores = os.cpu_count() or 1
    out = {}

    def one(name, fn):
        if build_ref.exe_path(name) is None:
            out[name] = {"unavailable": "reference harness not built"}
            return
        try:
            lups, secs, sample = fn()
            out[name] = {"glups": lups / secs / 1e9, "seconds": secs, "cores": cores, "kind": "reference",
                         "sample": sample}
        except Exception as e:  # report, do not hide
            out[name] = {"error": "%s: %s" % (type(e).__name__, e)}

    def heat():
        c = W.HEAT2D
        nx, ny, it = c["nx"], c["ny"], c["iters"]
        f = W.heat2d_padded(nx, ny, c["top"], c["seed"])
        res, _ = O.run_ref("heat2d", [nx, ny, it, cores, c["r"], c["top"], "{in0}", "{out0}"],
                           [np.ascontiguousarray(f[1:-1, 1:-1])], [(np.float32, 0)])
        return nx * ny * it, res["seconds"], "the whole workload: %dx%d FP32, %d iterations" % (nx, ny, it)

    def himeno():
        c = W.HIMENO
        nx, ny, nz, it = c["nx"], c["ny"], c["nz"], 10
        coef = W.himeno_coef(nx, ny, nz)
        p = W.himeno_p(nx, ny, nz)
        res, _ = O.run_ref("himeno", [nx, ny, nz, it, cores, c["omega"], "{in0}", "{in1}", "{out0}", "{out1}"],
                           [coef, np.ascontiguousarray(p[1:-1, 1:-1, 1:-1])], [(np.float32, 0), (np.float64, 0)])
        return nx * ny * nz * it, res["seconds"], "the full %dx%dx%d grid, %d of the %d sweeps" % (nx, ny, nz, it, c["iters"])

    def fdtd():
        n, it = 512, 2
        f = np.ascontiguousarray(W.fdtd_padded(n, n, n, 42)[4:-4, 4:-4, 4:-4])
        res, _ = O.run_ref("fdtd", [n, n, n, it, cores, 0.1, "{in0}", "{out0}"], [f], [(np.float32, 0)])
        return n ** 3 * it, res["seconds"], "512^3 FP32, %d steps of the reference form (same 25-point reads)" % it

    def triton():
        # every fourth domain of the 32-domain batch (the same generator and seeds), each for its
        # first 40 steps, through the reference's FP64 solver (its only precision)
        c = W.TRITON
        sizes = W.triton_sizes(c["n_domains"], c["side_lo"], c["side_hi"], c["seed"])
        steps, cells, secs, picked = 40, 0, 0.0, []
        for d in range(0, c["n_domains"], 4):
            ny, nx = sizes[d]
            dem, h = W.triton_domain(ny, nx, c["seed"] + 1000 * (d + 1))
            args = [nx, ny, cores, c["dx"], c["courant"], c["hextra"], c["manning"], c["t_end"], c["t_end"], c["time_step"], steps,
                    "{in0}", "{in1}", "{out0}", "{out1}"]
            res, _ = O.run_ref("triton", args, [dem, h], [(np.float64, 0), (np.float64, 0)])
            cells += nx * ny * int(res["steps"])
            secs += res["seconds"]
            picked.append("%dx%d" % (nx, ny))
        return cells, secs, "domains %s of the 32-domain batch (every fourth), FP64, first %d steps each" % (
            ", ".join(picked), steps)

    one("heat2d", heat)
    one("himeno", himeno)
    one("fdtd", fdtd)
    one("triton", triton)
    return out


def apps_unchanged():
    """The reference's sample applications, unchanged, on three builds on this machine: the
    reference's CPU path (OpenMP, every core), the reference's own GPU path (APPFIS_CUDA for
    sm_103a) and the drop-in headers (generic functor kernels of this engine; both GPU builds
    with nvcc's default FMA contraction); GameOfLife, Himeno and FDTD3d also with their one
    UseFastKernel line (the hand-written kernels; appfis_gb300/Appfis/Fast.hpp).  GLUP/s from each
    application's own COMPUTE timer (its printed `Compute:` seconds; the flood application: its `BLUPS:`
    line, since its step count follows the time step)."""
    import re
    from concurrent.futures import ThreadPoolExecutor

    from oracle import build_ref
    from tests.dropin import build_apps

    cases = [("HeatDiffusion", ["-dimx=256", "-dimy=256", "-dimz=256", "-iteration=100"], 256 ** 3 * 100),
             ("GameOfLife", ["-dimx=4096", "-dimy=4096", "-iteration=200"], 4096 ** 2 * 200),
             ("Himeno", ["-dimx=129", "-dimy=129", "-dimz=257", "-iteration=100"], 129 * 129 * 257 * 100),
             ("FDTD3d", ["-dimx=256", "-dimy=256", "-dimz=256", "-iteration=50"], 256 ** 3 * 50),
             # the flood application on a 1024^2 synthetic case to 600 s (FP64; its step count follows
             # the CFL time step, so GLUP/s is the application's own BLUPS line)
             ("Triton", ["case.cfg"], None)]
    apps = [c[0] for c in cases]
    with ThreadPoolExecutor(max_workers=8) as ex:
        ref = dict(zip(apps, ex.map(build_ref.app_ref_exe, apps)))
        refgpu = dict(zip(apps, ex.map(build_ref.app_refgpu_exe, apps)))
    gbx = build_apps.build(apps, exact=False)  # nvcc's default contraction, like the reference's GPU build
    fast = build_apps.build(build_apps.FAST_APPS, fast=True)  # the same sources plus their UseFastKernel line
    cores = os.cpu_count() or 1
    out = {}
    from appfis_gb300 import workloads as W
    with tempfile.TemporaryDirectory() as td:
        W.write_triton_case(td, 1024, 1024, 11, 600)
        for app, args, lups in cases:
            row = {"args": " ".join(args) if lups else "1024x1024 synthetic case (fractal DEM, point source), 600 s"}
            builds = [("reference_cpu", ref[app], ["-thread=%d" % cores]), ("reference_gpu", refgpu[app], []),
                      ("dropin_gpu", gbx[app], [])]
            if app in fast:
                builds.append(("dropin_fast_kernel_gpu", fast[app], []))
            for name, exe, extra in builds:
                r = subprocess.run([exe] + args + extra, capture_output=True, text=True, timeout=900, cwd=td)
                m = re.search(r"^Compute:\s*(\S+)", r.stdout, re.M)
                b = re.search(r"^BLUPS:\s*(\S+)", r.stdout, re.M)
                if r.returncode != 0 or not m or (lups is None and not b):
                    row[name] = {"error": (r.stderr or r.stdout)[-300:]}
                    continue
                secs = float(m.group(1))
                row[name] = {"compute_s": secs, "glups": lups / secs / 1e9 if lups else float(b.group(1))}
            out[app] = row
    return {"apps_unchanged": out, "cores": cores}


def run_reference(args, rank, world):
    if rank != 0:
        return
    from appfis_gb300 import workloads as W

    cells = W.gol_cells(GOL_NX, GOL_NY, GOL_P, GOL_SEED)
    gens = args.ref_gens
    vals = []
    kind = cores = None
    for s in range(args.warmup + args.steps):
        v, cores, kind = cpu_gol_sample(cells, gens)
        if s >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    sample = "16384x16384 grid, %d generations per step (of the 2000-generation workload)" % gens
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GLUP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": GOL_NX * GOL_NY * gens / value / 1e6,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "i32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_generations": gens},
            "cpu_baseline": {"value": value, "unit": "GLUP/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "GLUP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- our arm
def run_ours(args, rank, world, local):
    import torch

    import appfis_gb300 as gb
    from appfis_gb300 import build as gb_build
    from appfis_gb300 import workloads as W

    gb_build.build()
    L = gb.lib()
    hbm_peak, peak_kind = peaks()
    N = GOL_NX * GOL_NY
    gens = GOL_GENS
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    cells = W.gol_cells(GOL_NX, GOL_NY, GOL_P, GOL_SEED)
    host_in = torch.from_numpy(cells).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    d_cells = host_in.to(dev).view(-1)
    nw = N // 32
    wa = torch.empty(nw, dtype=torch.int32, device=dev)
    wb = torch.empty(nw, dtype=torch.int32, device=dev)
    ua = torch.empty(N, dtype=torch.uint8, device=dev)
    ub = torch.empty(N, dtype=torch.uint8, device=dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    ci = ctypes.c_int(0)

    def step_bits():
        gb.call("appfis_gb_life_pack", d_cells.data_ptr(), wa.data_ptr(), GOL_NX, GOL_NY, sp)
        wb.zero_()
        gb.call("appfis_gb_life_bits", wa.data_ptr(), wb.data_ptr(), GOL_NX, GOL_NY, gens, 0, ctypes.byref(ci), sp)
        latest = wa if ci.value == 0 else wb
        gb.call("appfis_gb_life_population_bits", latest.data_ptr(), nw, cnt.data_ptr(), sp)

    def step_u8():
        ua.copy_(d_cells)
        ub.zero_()
        gb.call("appfis_gb_life_u8", ua.data_ptr(), ub.data_ptr(), GOL_NX, GOL_NY, gens, 0, ctypes.byref(ci), sp)
        latest = ua if ci.value == 0 else ub
        gb.call("appfis_gb_life_population_u8", latest.data_ptr(), N, cnt.data_ptr(), sp)

    def timed(step, k, w, sample_clocks=False):
        for _ in range(w):
            step()
        torch.cuda.synchronize(dev)
        barrier(world)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        sampler = ClockSampler(local) if sample_clocks else None
        if sampler:
            sampler.__enter__()
            sampler.mark_start()
        e0.record(stream)
        for _ in range(k):
            step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        if sampler:
            sampler.mark_end()
            sampler.__exit__()
        barrier(world)
        ms = max_over_ranks(e0.elapsed_time(e1), world) / k
        return ms, (sampler.summary() if sampler else None)

    # headline: bit-packed form, inputs resident in HBM; the step (pack, 125 time-blocked launches,
    # population) is replayed from a CUDA graph captured once
    def step_bits_cur():
        s_ = torch.cuda.current_stream(dev).cuda_stream
        gb.call("appfis_gb_life_pack", d_cells.data_ptr(), wa.data_ptr(), GOL_NX, GOL_NY, s_)
        wb.zero_()
        gb.call("appfis_gb_life_bits", wa.data_ptr(), wb.data_ptr(), GOL_NX, GOL_NY, gens, 0, ctypes.byref(ci), s_)
        latest = wa if ci.value == 0 else wb
        gb.call("appfis_gb_life_population_bits", latest.data_ptr(), nw, cnt.data_ptr(), s_)

    replay_bits = graph_of(torch, step_bits_cur)
    ms_stream_bits, _ = timed(step_bits, args.steps, args.warmup)
    ms_bits, clocks = timed(replay_bits, args.steps, args.warmup, sample_clocks=True)
    population = int(cnt.item())
    value = N * gens / (ms_bits * 1e-3) / 1e9 * world

    # dominant kernel alone: average launch duration over G launches issued from the stream
    def kernel_avg(fn_name, a, b, g):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gb.call(fn_name, a.data_ptr(), b.data_ptr(), GOL_NX, GOL_NY, g, 0, ctypes.byref(ci), sp)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / g

    # the dominant kernel is life_bits_tb: one launch advances the whole grid by TB_GENS
    # generations.  Its launch time comes from a CUDA graph of TB_LAUNCHES back-to-back launches
    # (no launch gaps, no copies: an odd launch count ends in (a, b) by itself), replayed 4 times.
    TB_LAUNCHES = 25
    gb.call("appfis_gb_life_pack", d_cells.data_ptr(), wa.data_ptr(), GOL_NX, GOL_NY, sp)
    wb.zero_()

    def tb_launches():
        gb.call("appfis_gb_life_bits", wa.data_ptr(), wb.data_ptr(), GOL_NX, GOL_NY, TB_LAUNCHES * TB_GENS, 0,
                ctypes.byref(ci), torch.cuda.current_stream(dev).cuda_stream)

    replay_tb = graph_of(torch, tb_launches)
    bits_ms = _time(torch, stream, replay_tb, reps=4, warmup=2) / TB_LAUNCHES  # per launch
    # its bound is the integer/logic pipe, not HBM: per word (32 cells) and generation the source
    # issues 11 lop3 on that pipe (2 for the row summary, 6 for the bit-sliced count, 3 for the
    # reference rule); its 2 funnel shifts run on the FMA pipe (ncu pipe counters: replacing them
    # by integer multiply-adds left the logic pipe's instruction count unchanged).  The logic pipe
    # retires 64 lanes per SM and clock
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    word_gens = (N // 32) * TB_GENS
    logic_ops = 11 * word_gens
    ops_achieved = logic_ops / (bits_ms * 1e-3) / 1e12  # Tops/s
    bits_bytes = N * 3 / 8 * TB_GENS
    bits_achieved = bits_bytes / (bits_ms * 1e-3) / 1e9

    # u8 form (the byte-per-cell reference layout)
    ms_u8, _ = timed(step_u8, max(1, min(args.steps, 3)), 1)
    pop_u8 = int(cnt.item())
    ua.copy_(d_cells)
    ub.zero_()
    kernel_avg("appfis_gb_life_u8", ua, ub, 10)
    u8_ms = kernel_avg("appfis_gb_life_u8", ua, ub, 100)
    u8_bytes = N * 3
    u8_achieved = u8_bytes / (u8_ms * 1e-3) / 1e9

    # end to end through the C ABI from pinned host buffers
    pop = ctypes.c_int64(0)

    def step_e2e():
        gb.call("appfis_gb_life_job", host_in.data_ptr(), host_out.data_ptr(), GOL_NX, GOL_NY, gens, 0, 1,
                ctypes.byref(pop))

    for _ in range(args.warmup):
        step_e2e()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    e2e_value = N * gens / e2e_s / 1e9 * world
    assert pop.value == population == pop_u8, "forms disagree on the population"
    import hashlib
    final_sha = hashlib.sha256(host_out.numpy().tobytes()).hexdigest()  # the e2e run's final grid

    alu_mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    alu_peak = sms * 64 * alu_mhz * 1e6 / 1e12  # Tops/s
    ref_gol = reference_gol_record()
    line = {
        "metric": METRIC, "value": value, "unit": "GLUP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_bits, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "bit-packed (32 cells/word), states identical to u8; step replayed "
                   "from a CUDA graph (stream launches: %.3f ms)" % ms_stream_bits,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "each step starts from the 268 MB u8 grid (larger than L2); the packed state (67 MB for "
                         "both buffers) stays L2-resident across generations within a step",
                   "population": population,
                   "population_equals_reference_cpu_path": (population == ref_gol["live"]) if ref_gol else None,
                   "final_state_equals_reference_cpu_path": (final_sha == ref_gol["sha256"]) if ref_gol else None},
        "e2e": {"value": e2e_value, "unit": "GLUP/s", "h2d_bytes_per_step": N, "d2h_bytes_per_step": N + 8,
                "ms_per_step": e2e_s * 1e3},
        "gpu_launches": args.steps * (gens // 16 + gens % 16 + 2),  # pack, time-blocked sweeps, remainder, population
        "roofline": {"bound": "alu", "achieved": ops_achieved, "peak": alu_peak, "unit": "Tops/s",
                     "frac": ops_achieved / alu_peak, "traffic": profiled_traffic("life_bits_tb"),
                     "kernel": "life_bits_tb", "generations_per_launch": TB_GENS,
                     "ops": "32-bit lop3 instructions per lane (the logic pipe; the row summary's funnel shifts "
                            "run on the FMA pipe)",
                     "ops_per_word_generation": 11, "algorithmic_ops_per_launch": logic_ops,
                     "avg_launch_ms": bits_ms, "launches_per_step": GOL_GENS // TB_GENS,
                     "launch_timing": "CUDA graph of %d back-to-back launches" % TB_LAUNCHES,
                     "peak_source": "%d SMs x 64 logic lanes per clock x %.0f MHz (median SM clock of the timed region)"
                                    % (sms, alu_mhz),
                     "hbm_effective": {"achieved_gbs": bits_achieved, "peak_gbs": hbm_peak,
                                       "frac": bits_achieved / hbm_peak, "peak_source": peak_kind,
                                       "algorithmic_bytes_per_launch": bits_bytes,
                                       "note": "compulsory bytes of 16 one-generation sweeps (0.375 B per cell each); "
                                               "the tile stays on chip for the 16 generations, so DRAM moves only "
                                               "`traffic` per launch"}},
        "forms": {
            "bits": {"glups": value, "ms_per_step": ms_bits, "kernel_ms": bits_ms, "achieved_gbs": bits_achieved},
            "u8": {"glups": N * gens / (ms_u8 * 1e-3) / 1e9 * world, "ms_per_step": ms_u8, "kernel_ms": u8_ms,
                   "kernel": "life_u8_bulk", "achieved_gbs": u8_achieved, "frac": u8_achieved / hbm_peak,
                   "bytes_per_lup": 3, "traffic": profiled_traffic("life_u8_bulk")},
        },
        "clocks": clocks,
    }
    if not args.no_apps:
        from appfis_gb300 import workloads as W2
        per = {}
        for nm, fn in (("heat2d", lambda: bench_heat(torch, gb, W2, dev, stream, hbm_peak)),
                       ("himeno", lambda: bench_himeno(torch, gb, W2, dev, stream, hbm_peak)),
                       ("fdtd3d", lambda: bench_fdtd(torch, gb, W2, dev, stream, hbm_peak)),
                       ("flood", lambda: bench_flood(torch, gb, W2, dev, stream))):
            if nm not in args.apps.split(","):
                continue
            try:
                per[nm] = fn()
            except Exception as e:  # report, do not hide: the line still carries the headline
                per[nm] = {"error": "%s: %s" % (type(e).__name__, e)}
        line["per_app"] = per
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, kind = cpu_gol_sample(cells, args.ref_gens)
        line["cpu_baseline"] = {"value": v, "unit": "GLUP/s", "cores": cores, "kind": kind,
                                "sample": "16384x16384 grid, %d generations" % args.ref_gens}
        if not args.no_apps:
            line["cpu_baseline"]["per_app"] = cpu_app_samples()
    if rank == 0:
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- other workloads
def _events(torch, stream):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time(torch, stream, fn, reps=2, warmup=1):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = _events(torch, stream)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps  # ms


def graph_of(torch, fn):
    """Captures fn() (library calls on the current stream) into a CUDA graph; returns replay()."""
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        fn()  # warm: workspace allocated outside the capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        fn()
    return g.replay


def bench_heat(torch, gb, W, dev, sp, hbm):
    c = W.HEAT2D
    nx, ny, it = c["nx"], c["ny"], c["iters"]
    f = torch.from_numpy(W.heat2d_padded(nx, ny, c["top"], c["seed"])).to(dev)
    a, b = f.clone(), f.clone()
    ci = ctypes.c_int(0)

    def run():
        gb.call("appfis_gb_heat2d", a.data_ptr(), b.data_ptr(), nx, ny, nx + 2, it, c["r"], c["r"], ctypes.byref(ci),
                torch.cuda.current_stream().cuda_stream)

    ms = _time(torch, sp, run)
    ms_g = _time(torch, sp, graph_of(torch, run))
    a.copy_(f)
    b.copy_(f)
    run()
    out32 = (a if ci.value == 0 else b).double()
    f64 = f.double()
    a64, b64 = f64.clone(), f64.clone()
    gb.call("appfis_gb_heat2d_f64", a64.data_ptr(), b64.data_ptr(), nx, ny, nx + 2, it, float(c["r"]), float(c["r"]),
            ctypes.byref(ci), sp.cuda_stream)
    ref64 = a64 if ci.value == 0 else b64
    lups = nx * ny * it
    best = min(ms, ms_g)
    gbs = lups * 8 / (best * 1e-3) / 1e9
    return {"workload": "heat2d 1024^2 FP32, 1000 iterations, Dirichlet", "glups": lups / (best * 1e-3) / 1e9, "ms": best,
            "ms_stream_launches": ms, "ms_cuda_graph": ms_g, "bytes_per_lup": 8, "effective_gbs": gbs, "frac_of_hbm": gbs / hbm,
            "note": "8.4 MB working set is L2-resident; 8 sweeps per launch on chip (4x4 point blocks in registers, "
                    "block edges through shared memory; 125 launches, replayed from a CUDA graph); HBM fraction is nominal",
            "form": "plain FP32 (bit-identical to the reference CPU path)",
            "error_vs_fp64": _err(out32, ref64), "l2_norm": float(out32[1:-1, 1:-1].norm().item()),
            "l2_norm_fp64": float(ref64[1:-1, 1:-1].norm().item())}


def _err(x, ref):
    """Error of a result against the FP64 result of the same workload: max |x - ref|, the
    relative L2 error ||x - ref|| / ||ref|| and max |ref| (computed in double on the device)."""
    d = x.double() - ref
    return {"max_abs": float(d.abs().max().item()), "rel_l2": float((d.norm() / ref.norm().clamp_min(1e-300)).item()),
            "ref_max_abs": float(ref.abs().max().item())}


def _pad_x(t, pitch):
    """Copy of t with its last (x) axis padded with zeros to `pitch` elements."""
    out = t.new_zeros(tuple(t.shape[:-1]) + (pitch,))
    out[..., : t.shape[-1]] = t
    return out


def bench_himeno(torch, gb, W, dev, sp, hbm):
    """Both forms on rows padded to 264 elements (16-byte aligned FP16 and FP32 rows: the
    TMA-staged kernels), plus one-sweep times of the register-prefetch kernels on the dense
    259-element rows for comparison."""
    c = W.HIMENO
    nx, ny, nz, it, om = c["nx"], c["ny"], c["nz"], c["iters"], c["omega"]
    pitch = (nx + 2 + 7) // 8 * 8
    coef_d = torch.from_numpy(W.himeno_coef(nx, ny, nz)).to(dev)
    p0_d = torch.from_numpy(W.himeno_p(nx, ny, nz)).to(dev)
    coef = _pad_x(coef_d, pitch)
    p0 = _pad_x(p0_d, pitch)
    ptrs = (ctypes.c_void_p * 12)(*[coef[k].data_ptr() for k in range(12)])
    field = pitch * (ny + 2) * (nz + 2)
    pa, pb = p0.clone(), p0.clone()
    half = torch.empty(13 * field, dtype=torch.float16, device=dev)
    gosa = torch.zeros(it, dtype=torch.float64, device=dev)
    ci = ctypes.c_int(0)
    res = {}

    def plain():
        pa.copy_(p0)
        gb.call("appfis_gb_himeno", ptrs, pa.data_ptr(), pb.data_ptr(), nx, ny, nz, pitch, it, om, gosa.data_ptr(),
                ctypes.byref(ci), sp.cuda_stream)

    def mixed():
        pa.copy_(p0)
        gb.call("appfis_gb_himeno_mixed", ptrs, pa.data_ptr(), pb.data_ptr(), half.data_ptr(), nx, ny, nz, pitch, it, 20, om,
                gosa.data_ptr(), ctypes.byref(ci), sp.cuda_stream)

    lups = nx * ny * nz * it
    ms_p = _time(torch, sp, plain)
    out_p = (pa if ci.value == 0 else pb).clone()
    g_p = gosa.clone()
    ms_m = _time(torch, sp, mixed)
    out_m = (pa if ci.value == 0 else pb).clone()
    g_m = gosa.clone()

    def sweep_ms(ptr_list, a, b, pt, n=20):
        one = lambda: gb.call("appfis_gb_himeno", ptr_list, a.data_ptr(), b.data_ptr(), nx, ny, nz, pt, n, om,
                              gosa.data_ptr(), ctypes.byref(ci), sp.cuda_stream)
        return _time(torch, sp, one, reps=1) / n

    # FP64 reference of the same 400 sweeps (appfis_gb_himeno_f64; dense 259-element rows)
    coef64 = coef_d.double()
    ptr64 = (ctypes.c_void_p * 12)(*[coef64[k].data_ptr() for k in range(12)])
    q64a, q64b = p0_d.double(), torch.zeros_like(p0_d, dtype=torch.float64)
    g64 = torch.zeros(it, dtype=torch.float64, device=dev)
    gb.call("appfis_gb_himeno_f64", ptr64, q64a.data_ptr(), q64b.data_ptr(), nx, ny, nz, nx + 2, it, float(om), g64.data_ptr(),
            ctypes.byref(ci), sp.cuda_stream)
    p64 = q64a if ci.value == 0 else q64b
    del coef64

    def himeno_err(out, g):
        e = _err(out[..., : nx + 2], p64)
        e["gosa_rel_err_last"] = float(abs(g[-1].item() - g64[-1].item()) / abs(g64[-1].item()))
        e["gosa_rel_err_max"] = float(((g - g64).abs() / g64.abs().clamp_min(1e-300)).max().item())
        return e

    err_p, err_m = himeno_err(out_p, g_p), himeno_err(out_m, g_m)
    gosa64_last = float(g64[-1].item())
    del q64a, q64b, p64
    tma_ms = sweep_ms(ptrs, pa, pb, pitch)
    dptrs = (ctypes.c_void_p * 12)(*[coef_d[k].data_ptr() for k in range(12)])
    da, db = p0_d.clone(), p0_d.clone()
    ring_ms = sweep_ms(dptrs, da, db, nx + 2)
    del da, db
    gbs = nx * ny * nz * 56 / (tma_ms * 1e-3) / 1e9
    res["plain"] = {"glups": lups / (ms_p * 1e-3) / 1e9, "ms": ms_p, "bytes_per_lup": 56, "sweep_ms": tma_ms,
                    "kernel": "himeno_tma<plain>", "achieved_gbs": gbs, "frac_of_hbm": gbs / hbm,
                    "traffic": profiled_traffic("himeno_tma<plain>"),
                    "ring_kernel_sweep_ms_dense_rows": ring_ms, "gosa_last": float(g_p[-1].item()),
                    "gosa_last_fp64": gosa64_last, "error_vs_fp64": err_p}
    b_m = (19 * 30 + 62) / 20.0
    res["mixed_fp16_defect_correction"] = {
        "glups": lups / (ms_m * 1e-3) / 1e9, "ms": ms_m, "bytes_per_lup_avg": b_m, "period": 20,
        "speedup_vs_plain": ms_p / ms_m, "max_abs_diff_vs_plain_fp32": float((out_m - out_p).abs().max().item()),
        "gosa_last": float(g_m[-1].item()),
        "gosa_rel_diff_vs_plain": float(((g_m - g_p).abs() / g_p.abs().clamp_min(1e-300)).max().item()),
        "error_vs_fp64": err_m}
    res["workload"] = "himeno 257x257x513 FP32, 400 iterations, per-sweep FP64 gosa; rows padded to %d" % pitch
    return res


def bench_fdtd(torch, gb, W, dev, sp, hbm):
    """plain: the single-step FP32 TMA tile (the reference functor's data flow, one step per
    launch).  Chosen forms: what the autotuner (appfis_gb_star_r4_tune) picks for FP32 and for
    FP16 storage among the single-step tiles and the two-step time-blocked tiles, times z chunks;
    each with its 200-step time, speed-up over plain and error against the FP64 form."""
    c = W.FDTD
    nx, ny, nz, it = c["nx"], c["ny"], c["nz"], c["iters"]
    w = (ctypes.c_float * 5)(*W.fdtd_weights())
    f32 = torch.from_numpy(W.fdtd_padded(nx, ny, nz, c["seed"])).to(dev)
    a, b = f32.clone(), f32.clone()
    h0 = f32.half()
    ha, hb = h0.clone(), h0.clone()
    ci = ctypes.c_int(0)
    res = {}
    TMA_X4, AUTO = 8, 0
    names = {8: "star_r4_tma (4 x points / thread)", 9: "star_r4_tma (2 x points / thread)", 10: "star_r4_vec",
             13: "star_r4_tma (4 x points x 4 rows / thread)",
             11: "star_r4_tb2 (two steps per launch, 64 x 16)", 12: "star_r4_tb2 (two steps per launch, 64 x 8)"}

    def run(x, y, x0, dt, iters, tile):
        def f():
            x.copy_(x0)
            gb.call("appfis_gb_star_r4", x.data_ptr(), y.data_ptr(), dt, nx, ny, nz, nx + 8, iters, 1, 0.0, w, tile, 0,
                    ctypes.byref(ci), sp.cuda_stream)
        return f

    def steps_only(x, y, dt, tile, n=10):  # n steps on the current state, no reset: kernel time per step
        one = lambda: gb.call("appfis_gb_star_r4", x.data_ptr(), y.data_ptr(), dt, nx, ny, nz, nx + 8, n, 1, 0.0, w, tile, 0,
                              ctypes.byref(ci), sp.cuda_stream)
        return _time(torch, sp, one, reps=1) / n

    lups = nx * ny * nz * it
    # FP64 reference of the same 200 steps (appfis_gb_star_r4_f64, the weights in double)
    w64 = (ctypes.c_double * 5)(*W.fdtd_weights())
    x64 = f32.double()
    y64 = x64.clone()
    gb.call("appfis_gb_star_r4_f64", x64.data_ptr(), y64.data_ptr(), nx, ny, nz, nx + 8, it, 1, 0.0, w64, ctypes.byref(ci),
            sp.cuda_stream)
    r64 = x64 if ci.value == 0 else y64

    ms32 = _time(torch, sp, run(a, b, f32, 0, it, TMA_X4))
    err32 = _err((a if ci.value == 0 else b), r64)
    s32 = steps_only(a, b, 0, TMA_X4)
    g32 = nx * ny * nz * 8 / (s32 * 1e-3) / 1e9
    res["workload"] = "fdtd3d radius-4 star 512^3, 200 steps of u <- u + 0.1*L8(u), zero halo of 4"
    res["plain_fp32"] = {"glups": lups / (ms32 * 1e-3) / 1e9, "ms": ms32, "bytes_per_lup": 8, "sweep_ms": s32,
                         "kernel": "star_r4_tma<float>", "achieved_gbs": g32, "frac_of_hbm": g32 / hbm,
                         "traffic": profiled_traffic("star_r4_tma<float>"), "error_vs_fp64": err32}
    # one step of every tile (10 steps each, per-step time)
    tiles = {}
    for tname, tid in (("tma_x4", 8), ("tma_x4_4rows", 13), ("tma_x2", 9), ("tb2_64x16", 11), ("tb2_64x8", 12), ("vec", 10)):
        for dname, x, y, dt in (("fp32", a, b, 0), ("fp16", ha, hb, 3)):
            tiles["%s_%s_ms" % (tname, dname)] = steps_only(x, y, dt, tid)
    res["step_ms_by_tile"] = tiles
    for label, x, y, x0, dt, bpl in (("chosen_fp32", a, b, f32, 0, 8), ("chosen_fp16_storage", ha, hb, h0, 3, 4)):
        tile, kz, tms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_float(0)
        x.copy_(x0)
        gb.call("appfis_gb_star_r4_tune", x.data_ptr(), y.data_ptr(), dt, nx, ny, nz, nx + 8, 1, 0.0, w, ctypes.byref(tile),
                ctypes.byref(kz), ctypes.byref(tms), sp.cuda_stream)
        ms = _time(torch, sp, run(x, y, x0, dt, it, AUTO))  # AUTO runs the tuned choice
        err = _err((x if ci.value == 0 else y).float(), r64)
        sm = steps_only(x, y, dt, AUTO)
        gbs = nx * ny * nz * bpl / (sm * 1e-3) / 1e9
        res[label] = {"glups": lups / (ms * 1e-3) / 1e9, "ms": ms, "speedup_vs_plain": ms32 / ms, "sweep_ms": sm,
                      "tuned": {"tile": tile.value, "kernel": names.get(tile.value, str(tile.value)),
                                "steps_per_launch": 2 if tile.value in (11, 12) else 1,
                                "zchunk": kz.value, "tuner_ms_per_step": tms.value},
                      "bytes_per_lup": bpl, "achieved_gbs": gbs, "frac_of_hbm": gbs / hbm, "error_vs_fp64": err}
    del x64, y64, r64
    return res


def bench_flood(torch, gb, W, dev, sp):
    from appfis_gb300 import _lib
    c = W.TRITON
    doms = W.triton_batch(c["n_domains"], c["side_lo"], c["side_hi"], c["seed"])
    nd = len(doms)
    bufs, descs, inter = [], (_lib.FloodDomain * nd)(), []
    for k, (dem, h) in enumerate(doms):
        ny, nx = dem.shape
        pitch = ((nx + 2 + 31) // 32) * 32
        f = torch.empty((8, ny + 2, pitch), dtype=torch.float32, device=dev)
        bufs.append(f)
        d = descs[k]
        d.nx, d.ny, d.pitch = nx, ny, pitch
        d.h[0], d.h[1], d.qx[0], d.qx[1], d.qy[0], d.qy[1] = [f[m].data_ptr() for m in range(6)]
        d.dem, d.n2 = f[6].data_ptr(), f[7].data_ptr()
        inter.append((torch.from_numpy(dem).to(dev), torch.from_numpy(h).to(dev)))
    prm = _lib.FloodParams(c["dx"], c["courant"], c["hextra"], c["t_end"], c["t_end"], c["time_step"], 0.0, 0)
    steps = torch.zeros(nd, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)

    def setup():
        for k in range(nd):
            gb.call("appfis_gb_flood_setup", ctypes.byref(descs[k]), _lib.F32, inter[k][0].data_ptr(), inter[k][1].data_ptr(),
                    None, None, c["manning"], sp.cuda_stream)

    def batched():
        setup()
        gb.call("appfis_gb_flood_run", descs, nd, _lib.F32, ctypes.byref(prm), None, steps.data_ptr(), None,
                status.data_ptr(), sp.cuda_stream)

    def one_by_one():
        setup()
        for k in range(nd):
            gb.call("appfis_gb_flood_run", ctypes.byref(descs[k]), 1, _lib.F32, ctypes.byref(prm), None,
                    steps[k:k + 1].data_ptr(), None, status.data_ptr(), sp.cuda_stream)

    ms_b = _time(torch, sp, batched, reps=1)
    st = steps.cpu().numpy().astype(np.int64)
    assert int(status.item()) == 0
    cells = np.array([d[0].size for d in doms], dtype=np.int64)
    cell_steps = float((cells * st).sum())
    # mass: FP64 sum of h before / after the batched run
    m0 = [float(h.sum().item()) for _, h in inter]
    m1 = []
    for k in range(nd):
        b = int(st[k]) & 1
        ny, nx = doms[k][0].shape
        m1.append(float(bufs[k][b][1:ny + 1, 1:nx + 1].double().sum().item()))
    drift = max(abs(a - b) / a for a, b in zip(m0, m1))
    def final_state(k, n):  # interiors of h, qx, qy of domain k after n steps (buffers h0 h1 qx0 qx1 qy0 qy1 dem n2)
        b = int(n) & 1
        ny, nx = doms[k][0].shape
        return torch.stack([bufs[k][b], bufs[k][2 + b], bufs[k][4 + b]])[:, 1:ny + 1, 1:nx + 1]

    dense = [final_state(k, st[k]).clone() for k in range(nd)]
    # the same fused pass loading its rows directly instead of staging them by TMA
    prm.flags = _lib.FLOOD_UNSTAGED
    ms_u = _time(torch, sp, batched, reps=1)
    same_u = bool((steps.cpu().numpy().astype(np.int64) == st).all()) and all(
        torch.equal(final_state(k, st[k]), dense[k]) for k in range(nd))
    # the two-pass form of the same full sweep (fix + dt, then update; bit-identical fields)
    prm.flags = _lib.FLOOD_TWO_PHASE
    ms_2 = _time(torch, sp, batched, reps=1)
    same2 = bool((steps.cpu().numpy().astype(np.int64) == st).all()) and all(
        torch.equal(final_state(k, st[k]), dense[k]) for k in range(nd))
    # the same batch leaving out strips that are dry with dry neighbours (bit-identical fields)
    prm.flags = _lib.FLOOD_SKIP_DRY
    ms_k = _time(torch, sp, batched, reps=1)
    st_k = steps.cpu().numpy().astype(np.int64)
    assert int(status.item()) == 0
    same = bool((st_k == st).all()) and all(torch.equal(final_state(k, st_k[k]), dense[k]) for k in range(nd))
    prm.flags = 0
    # FP64 reference of the same batch (the FP64 form matches the reference CPU path to 1e-9);
    # run with the dry strips left out, which leaves every field bit-identical
    bufs64, descs64 = [], (_lib.FloodDomain * nd)()
    for k, (dem, h) in enumerate(doms):
        ny, nx = dem.shape
        pitch = ((nx + 2 + 15) // 16) * 16
        f = torch.empty((8, ny + 2, pitch), dtype=torch.float64, device=dev)
        bufs64.append(f)
        d = descs64[k]
        d.nx, d.ny, d.pitch = nx, ny, pitch
        d.h[0], d.h[1], d.qx[0], d.qx[1], d.qy[0], d.qy[1] = [f[m].data_ptr() for m in range(6)]
        d.dem, d.n2 = f[6].data_ptr(), f[7].data_ptr()
        gb.call("appfis_gb_flood_setup", ctypes.byref(d), _lib.F64, inter[k][0].data_ptr(), inter[k][1].data_ptr(), None, None,
                c["manning"], sp.cuda_stream)
    prm64 = _lib.FloodParams(c["dx"], c["courant"], c["hextra"], c["t_end"], c["t_end"], c["time_step"], 0.0, 0)
    prm64.flags = _lib.FLOOD_SKIP_DRY
    steps64 = torch.zeros(nd, dtype=torch.int32, device=dev)
    ms64 = _time(torch, sp, lambda: gb.call("appfis_gb_flood_run", descs64, nd, _lib.F64, ctypes.byref(prm64), None,
                                            steps64.data_ptr(), None, status.data_ptr(), sp.cuda_stream), reps=1, warmup=0)
    assert int(status.item()) == 0
    st64 = steps64.cpu().numpy().astype(np.int64)
    l1_rel, hmax, m64 = [], 0.0, []
    for k in range(nd):
        ny, nx = doms[k][0].shape
        h32 = dense[k][0].double()
        h64 = bufs64[k][int(st64[k]) & 1][1:ny + 1, 1:nx + 1]
        vol = float(h64.sum().item())
        m64.append(vol)
        l1_rel.append(float((h32 - h64).abs().sum().item()) / vol)
        hmax = max(hmax, float((h32 - h64).abs().max().item()))
    err_flood = {"l1_depth_err_over_volume_max": max(l1_rel), "l1_depth_err_over_volume_mean": float(np.mean(l1_rel)),
                 "max_abs_depth_err_m": hmax,
                 "mass_rel_change_fp64_max": max(abs(a - b) / a for a, b in zip(m0, m64)),
                 "fp64_steps_min": int(st64.min()), "fp64_steps_max": int(st64.max()), "fp64_ms": ms64,
                 "note": "FP32 batch vs the FP64 batch at t = 600 s (same domains; both land on t_end exactly)"}
    del bufs64
    ms_s = _time(torch, sp, one_by_one, reps=1)
    setup_ms = _time(torch, sp, setup, reps=1)
    hbm, _ = peaks()
    g_b = cell_steps * 32 / ((ms_b - setup_ms) * 1e-3) / 1e9  # fused pass: 32 B per cell-step
    g_2 = cell_steps * 48 / ((ms_2 - setup_ms) * 1e-3) / 1e9  # two passes: 16 B + 32 B
    return {"workload": "flood model, 32 domains (sides 512-3072, %.1f M cells), fractal DEM, to t = 600 s" % (cells.sum() / 1e6),
            "batched_fp32": {"glups": cell_steps / ((ms_b - setup_ms) * 1e-3) / 1e9, "ms": ms_b - setup_ms,
                             "kernel": "flood_fused (one pass per step; rows staged by TMA, 4-row stages)",
                             "bytes_per_cell_step": 32, "achieved_gbs": g_b,
                             "frac_of_hbm": g_b / hbm,
                             "steps_min": int(st.min()), "steps_max": int(st.max()), "cell_steps": cell_steps,
                             "mass_rel_change_max": drift, "error_vs_fp64": err_flood},
            "batched_fp32_row_loads": {"glups": cell_steps / ((ms_u - setup_ms) * 1e-3) / 1e9, "ms": ms_u - setup_ms,
                                       "kernel": "flood_fused, rows loaded directly (APPFIS_GB_FLOOD_UNSTAGED)",
                                       "fields_identical_to_staged": same_u},
            "batched_fp32_two_phase": {"glups": cell_steps / ((ms_2 - setup_ms) * 1e-3) / 1e9, "ms": ms_2 - setup_ms,
                                       "kernel": "flood_persistent (fix + dt, then update)", "bytes_per_cell_step": 48,
                                       "achieved_gbs": g_2, "frac_of_hbm": g_2 / hbm, "fields_identical_to_fused": same2},
            "batched_fp32_skip_dry": {"glups": cell_steps / ((ms_k - setup_ms) * 1e-3) / 1e9, "ms": ms_k - setup_ms,
                                      "fields_identical_to_full_sweep": same,
                                      "note": "strips whose cells and neighbour strips are exactly dry are left out "
                                              "(APPFIS_GB_FLOOD_SKIP_DRY); GLUP/s counts every cell-step"},
            "one_domain_per_launch_fp32": {"glups": cell_steps / ((ms_s - setup_ms) * 1e-3) / 1e9, "ms": ms_s - setup_ms},
            "batched_speedup": (ms_s - setup_ms) / (ms_b - setup_ms)}


def profile_small(name, torch, gb, W, dev, sp):
    """A few launches of one workload's kernels at the benchmark size (no timing)."""
    ci = ctypes.c_int(0)
    if name == "heat":
        c = W.HEAT2D
        f = torch.from_numpy(W.heat2d_padded(c["nx"], c["ny"], c["top"], c["seed"])).to(dev)
        a, b = f.clone(), f.clone()
        gb.call("appfis_gb_heat2d", a.data_ptr(), b.data_ptr(), c["nx"], c["ny"], c["nx"] + 2, 16, c["r"], c["r"],
                ctypes.byref(ci), sp.cuda_stream)
    elif name == "himeno":
        c = W.HIMENO
        nx, ny, nz = c["nx"], c["ny"], c["nz"]
        pitch = (nx + 2 + 7) // 8 * 8  # 16-byte rows: the TMA-staged kernels
        coef = _pad_x(torch.from_numpy(W.himeno_coef(nx, ny, nz)).to(dev), pitch)
        p0 = _pad_x(torch.from_numpy(W.himeno_p(nx, ny, nz)).to(dev), pitch)
        ptrs = (ctypes.c_void_p * 12)(*[coef[k].data_ptr() for k in range(12)])
        pa, pb = p0.clone(), p0.clone()
        half = torch.empty(13 * p0.numel(), dtype=torch.float16, device=dev)
        gosa = torch.zeros(8, dtype=torch.float64, device=dev)
        gb.call("appfis_gb_himeno", ptrs, pa.data_ptr(), pb.data_ptr(), nx, ny, nz, pitch, 5, c["omega"], gosa.data_ptr(),
                ctypes.byref(ci), sp.cuda_stream)
        gb.call("appfis_gb_himeno_mixed", ptrs, pa.data_ptr(), pb.data_ptr(), half.data_ptr(), nx, ny, nz, pitch, 5, 20,
                c["omega"], gosa.data_ptr(), ctypes.byref(ci), sp.cuda_stream)
    elif name == "himeno-small":
        nx, ny, nz = 129, 129, 257
        pitch = (nx + 2 + 7) // 8 * 8
        coef = _pad_x(torch.from_numpy(W.himeno_coef(nx, ny, nz)).to(dev), pitch)
        p0 = _pad_x(torch.from_numpy(W.himeno_p(nx, ny, nz)).to(dev), pitch)
        ptrs = (ctypes.c_void_p * 12)(*[coef[k].data_ptr() for k in range(12)])
        pa, pb = p0.clone(), p0.clone()
        half = torch.empty(13 * p0.numel(), dtype=torch.float16, device=dev)
        gosa = torch.zeros(8, dtype=torch.float64, device=dev)
        for spp in (1, 2):  # 1 + 2 inner sweeps: himeno_mixed2, then himeno_mixed_tb2
            gb.call("appfis_gb_himeno_mixed_ex", ptrs, pa.data_ptr(), pb.data_ptr(), half.data_ptr(), nx, ny, nz, pitch, 4, 1000,
                    0.8, spp, gosa.data_ptr(), ctypes.byref(ci), sp.cuda_stream)
    elif name == "fdtd":
        c = W.FDTD
        nx, ny, nz = c["nx"], c["ny"], c["nz"]
        w = (ctypes.c_float * 5)(*W.fdtd_weights())
        f = torch.from_numpy(W.fdtd_padded(nx, ny, nz, c["seed"])).to(dev)
        a, b = f.clone(), f.clone()
        gb.call("appfis_gb_star_r4", a.data_ptr(), b.data_ptr(), 0, nx, ny, nz, nx + 8, 5, 1, 0.0, w, 8, 0, ctypes.byref(ci),
                sp.cuda_stream)
        h = f.half()
        ha, hb = h.clone(), h.clone()
        gb.call("appfis_gb_star_r4", ha.data_ptr(), hb.data_ptr(), 3, nx, ny, nz, nx + 8, 5, 1, 0.0, w, 8, 0, ctypes.byref(ci),
                sp.cuda_stream)
        # the two-step time-blocked tile: 2 launches (4 steps) in FP32, then in FP16 storage
        for x, y, dt in ((a, b, 0), (ha, hb, 3)):
            gb.call("appfis_gb_star_r4", x.data_ptr(), y.data_ptr(), dt, nx, ny, nz, nx + 8, 4, 1, 0.0, w, 11, 0,
                    ctypes.byref(ci), sp.cuda_stream)


def profile_case(name, local):
    """Short fixed launch sequences for ncu captures.
    life:   16384^2 GameOfLife, 20 bit-packed generations (one life_bits_tb launch of 16 + 4
            life_bits_sweep) then 20 u8 sweeps (life_u8_bulk)
    himeno: 257x257x513 (rows padded to 264), 5 plain sweeps (himeno_tma<0>), 5 mixed sweeps
            (himeno_tma<1>, himeno_correct)
    fdtd:   512^3, 5 FP32 steps then 5 FP16 steps (star_r4_tma), then 2 two-step launches in FP32
            and 2 in FP16 (star_r4_tb2)
    heat:   1024^2, 16 iterations (2 heat2d_regs launches)
    himeno-small: 129x129x257, the mixed form with one inner sweep per launch (himeno_mixed2),
            then with two (himeno_mixed_tb2), 4 sweeps each (~0.3 GB)
    flood:  the 32-domain batch (80 M cells, ~2.6 GB), 20 steps (one flood_fused launch)
    flood-small: the first 6 domains of the batch (15.8 M cells), 20 steps (one flood_fused launch,
    rows staged by TMA); flood-small-rows: the same with the rows loaded directly"""
    import torch

    import appfis_gb300 as gb
    from appfis_gb300 import workloads as W

    dev = torch.device("cuda", local)
    sp = torch.cuda.current_stream(dev)
    if name != "life":
        fn = {"himeno": bench_himeno, "fdtd": bench_fdtd, "heat": bench_heat}.get(name)
        if name in ("flood", "flood-small", "flood-small-rows"):
            from appfis_gb300 import _lib
            c = W.TRITON
            doms = W.triton_batch(c["n_domains"], c["side_lo"], c["side_hi"], c["seed"])
            if name != "flood":
                doms = doms[:6]
            _lib.flood_job(doms, c["dx"], c["courant"], c["hextra"], c["manning"], c["t_end"], c["t_end"], c["time_step"],
                           max_steps=20, dtype=_lib.F32, flags=_lib.FLOOD_UNSTAGED if name == "flood-small-rows" else 0)
        else:
            profile_small(name, torch, gb, W, dev, sp)
        torch.cuda.synchronize(dev)
        print("profile case %s done" % name)
        return
    cells = torch.from_numpy(W.gol_cells(GOL_NX, GOL_NY, GOL_P, GOL_SEED)).to(dev).view(-1)
    N = GOL_NX * GOL_NY
    wa = torch.empty(N // 32, dtype=torch.int32, device=dev)
    wb = torch.zeros_like(wa)
    ub = torch.zeros_like(cells)
    ci = ctypes.c_int(0)
    sp = torch.cuda.current_stream(dev).cuda_stream
    gb.call("appfis_gb_life_pack", cells.data_ptr(), wa.data_ptr(), GOL_NX, GOL_NY, sp)
    gb.call("appfis_gb_life_bits", wa.data_ptr(), wb.data_ptr(), GOL_NX, GOL_NY, 20, 0, ctypes.byref(ci), sp)
    gb.call("appfis_gb_life_u8", cells.data_ptr(), ub.data_ptr(), GOL_NX, GOL_NY, 20, 0, ctypes.byref(ci), sp)
    torch.cuda.synchronize(dev)
    print("profile case %s done" % name)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--ref-gens", type=int, default=8, help="generations per CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-apps", action="store_true", help="skip the per-workload measurements")
    ap.add_argument("--apps", default="heat2d,himeno,fdtd3d,flood", help="comma-separated per-workload measurements")
    ap.add_argument("--apps-unchanged", action="store_true",
                    help="time the reference's sample applications on its CPU path, its GPU path and the drop-in")
    ap.add_argument("--profile-case", choices=["life", "himeno", "himeno-small", "fdtd", "heat", "flood", "flood-small",
                                                  "flood-small-rows"], default=None,
                    help="launch a short fixed sequence of the named workload's kernels (for ncu), no timing")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_setup(args.gpus)
    if args.profile_case:
        profile_case(args.profile_case, local)
    elif args.apps_unchanged:
        if rank == 0:
            from appfis_gb300 import build as gb_build
            gb_build.build()
            print(json.dumps(apps_unchanged()), flush=True)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
