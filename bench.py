"""Benchmark of the tube-segmentation hot path on GB300.

Workload (default): the 256^3 synthetic vessel tree, 500 GVF iterations with
16-bit (FP16) field storage and FP32 arithmetic.  One step is one pass of the
hot path over the volume, with inputs resident in HBM:
    blur (sigma 0.5) -> vector field -> small-radius TDF (r 1..3) ->
    GVF (500 Jacobi iterations) -> GVF finish -> large-radius TDF (r 2.5..7)
    -> combine -> candidate centerpoints (threshold, pyramid-order compaction,
    cross-section filter, per-cube arg-max, vertex list).
value = voxel-iterations of GVF per step (N * 500) / step time, in
Gvoxel-iter/s: the metric of the workload, measured over the whole step.

e2e: the same step driven through the C ABI from pinned HOST memory: every
step's volume is copied host->device and its TDF, radius and vertex list
device->host inside the timed region, on a copy stream overlapped with the
neighbouring steps' compute.

Multi-GPU: the path does not shard here; --gpus N runs N independent
replicas (one volume per GPU), value = sum over ranks.

--impl reference: the CPU restatement of the reference's kernels (the oracle;
the OpenCL reference cannot run on these machines) on all host cores, --steps
timed steps after --warmup untimed ones, each step the whole hot path with all
GVF iterations on a bounded sample of the volume (a z-slab of it), so that
the run ends within minutes.  Nothing is extrapolated.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tube-segmentation-framework_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np

METRIC = "GVF Gvoxel-iters/s (FP16 vs FP32 store, TDF err<=1e-3), fwd+adjoint ms @256^3"
UNIT = "Gvoxel-iter/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="tsf", choices=["tsf", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--iters", type=int, default=500)
    ap.add_argument("--storage", default="f16", choices=["f32", "f16", "bf16", "snorm16"])
    ap.add_argument("--mu", type=float, default=0.05)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-slab-planes-1core", type=int, default=8,
                    help="z-planes of the one-core CPU baseline sample (0: skip)")
    ap.add_argument("--reference-slab-planes", type=int, default=16,
                    help="z-planes of the volume one reference-arm step processes")
    ap.add_argument("--accuracy", action="store_true",
                    help="instead of timing: errors of every storage format against the FP64 oracle")
    ap.add_argument("--polish", action="store_true",
                    help="16-bit GVF with its last --polish-iters iterations in FP32: vertex list against the FP64 "
                         "oracle and step time against the FP16 and FP32 paths")
    ap.add_argument("--polish-iters", type=int, default=4)
    ap.add_argument("--fmg", action="store_true",
                    help="instead of the default workload: the 512x512x400 lung CT with multigrid GVF")
    ap.add_argument("--fmg-cycles", type=int, default=10)
    ap.add_argument("--calibrate", action="store_true",
                    help="instead of the default workload: the differentiation configuration (192^3 vessel tree, "
                         "300 GVF iterations, checkpoint every 17, FP32) -- timing, dL/dmu against an FP64 central "
                         "difference, and 20 Adam steps on mu and the blur sigma")
    ap.add_argument("--mra", action="store_true",
                    help="instead of the default workload: the 512^3 MRA-like volume, 1000 GVF iterations in FP16 "
                         "storage -- the full pipeline step, and forward + adjoint with memory-budgeted checkpointing")
    ap.add_argument("--adjoint", action="store_true",
                    help="time the forward + adjoint (gradient) pass alone and print its JSON line")
    ap.add_argument("--stage", choices=["spline", "circle", "segment", "crop", "gvf"],
                    help="time one stage alone and print its JSON line (a small, self-contained command for "
                         "kernel profiles): a TDF on the vessel-tree field after --iters GVF iterations, the "
                         "segmentation of that step's centerlines, or the lung cropping of the 512x512x400 CT")
    ap.add_argument("--summarize-ncu-csv", metavar="CSV",
                    help="print a per-kernel table (launches, total time, share) of an ncu "
                         "--metrics gpu__time_duration.sum --csv launch list and exit")
    return ap.parse_args()


# workload parameters (config 1 of the benchmark: 256^3 vessel tree)
PARAMS = dict(large_blur=0.5, fmax=0.2, vsign=1, rmin=1.0, rmax=7.0, rstep=0.5,
              tdf_high=0.5, cube_size=4)


def mem_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def reduce_max(value: float, world: int, device="cuda") -> float:
    """The largest value over the ranks (the timed region of the slowest rank)."""
    if world <= 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput of `world` independent replicas: all ranks' units
    over the slowest rank's time."""
    return world * units_per_rank / seconds_max


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.first = 0

    def start(self, ready_s=3.0):
        """Starts sampling every 100 ms and returns once the first sample has
        arrived (at most ready_s), so that the sampler is live when the timed
        region begins; only samples after mark() count."""
        try:
            import shutil
            # into a pipe nvidia-smi's output is block-buffered: ask for lines
            pre = ["stdbuf", "-oL"] if shutil.which("stdbuf") else []
            self.proc = subprocess.Popen(pre + ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                                "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            t0 = time.time()
            while not self.lines and self.proc.poll() is None and time.time() - t0 < ready_s:
                time.sleep(0.01)
            self.first = len(self.lines)
        except Exception:
            self.proc = None

    def mark(self):
        """Samples from here on belong to the timed region."""
        self.first = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.th.join(timeout=5)            # the lines still in the pipe
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[self.first:]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


class Pipeline:
    """Device buffers and workspaces for one volume; step() runs the hot path."""

    def __init__(self, T, torch, shape, storage, iters, mu):
        self.T, self.torch = T, torch
        Z, Y, X = shape
        self.shape, self.storage, self.iters, self.mu = shape, storage, iters, mu
        dt = T.storage_dtype(storage)
        dev = "cuda"
        L = T.load()
        st = T.STORAGE[storage]
        self.vol = torch.empty(shape, dtype=torch.float32, device=dev)
        self.blurred = torch.empty_like(self.vol)
        self.f0 = torch.empty((3, Z, Y, X), dtype=dt, device=dev)
        self.v = torch.empty_like(self.f0)
        self.f4_small = torch.empty((Z, Y, X, 4), dtype=dt, device=dev)
        self.field = torch.empty((Z, Y, X, 4), dtype=dt, device=dev)
        self.Ts = torch.empty(shape, dtype=torch.float32, device=dev)
        self.Rs = torch.empty_like(self.Ts)
        self.Tl = torch.empty_like(self.Ts)
        self.Rl = torch.empty_like(self.Ts)
        self.gvf_ws = T.workspace(L.tsf_gvf_workspace_size(X, Y, Z, st))
        self.cand_ws = T.workspace(L.tsf_candidates_workspace_size(X, Y, Z))
        self.tdf_ws = T.workspace(L.tsf_tdf_workspace_size(X, Y, Z, st))   # x-paired texels (16-bit storage)
        self.max_vertices = 1 << 16
        self.verts = torch.zeros((self.max_vertices, 3), dtype=torch.int32, device=dev)
        self.last = None
        self.gvf_mode = 0                   # 0: default kernel choice; 1: register-vector kernel

    def gvf_only(self):
        T = self.T
        self.v.copy_(self.f0)
        T.gvf(self.f0, self.mu, self.iters, self.storage, v=self.v, ws=self.gvf_ws, mode=self.gvf_mode)

    def step(self, events=None):
        T, P, s = self.T, PARAMS, self.storage
        rec = (lambda name: events.append((name, self._ev()))) if events is not None else (lambda name: None)
        rec("start")
        T.blur(self.vol, P["large_blur"], out=self.blurred)
        # small-radius pass on the un-diffused field of the unblurred volume (small-blur 0)
        self._vf(self.vol, None, self.f4_small)
        T._check(T.load().tsf_tdf_circle_ws(T._ptr(self.f4_small), *self._xyz(), T.STORAGE[s], P["rmin"], 3.0, 0.5,
                                            T._ptr(self.Ts), 0, T._ptr(self.Rs), T._ptr(self.tdf_ws),
                                            self.tdf_ws.numel(), T._stream()))
        rec("tdf_small")
        self._vf(self.blurred, self.f0, None)
        rec("vector_field")
        self.gvf_only()
        rec("gvf")
        T.gvf_finish(self.v, s, out=self.field)
        T._check(T.load().tsf_tdf_circle_ws(T._ptr(self.field), *self._xyz(), T.STORAGE[s], max(2.5, P["rmin"]),
                                            P["rmax"], P["rstep"], T._ptr(self.Tl), 0, T._ptr(self.Rl),
                                            T._ptr(self.tdf_ws), self.tdf_ws.numel(), T._stream()))
        T.tdf_combine(self.Ts, self.Rs, self.Tl, self.Rl)
        rec("tdf_large")
        self.last = self._candidates()
        rec("candidates")

    def _ev(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    def _xyz(self):
        Z, Y, X = self.shape
        return X, Y, Z

    def _vf(self, src, planar, f4):
        T = self.T
        X, Y, Z = self._xyz()
        T._check(T.load().tsf_vector_field(T._ptr(src), X, Y, Z, PARAMS["fmax"], PARAMS["vsign"],
                                           T.STORAGE[self.storage], T._ptr(planar), T._ptr(f4), T._stream()))

    def _candidates(self):
        import ctypes as C
        T = self.T
        X, Y, Z = self._xyz()
        nc, nv = C.c_int64(0), C.c_int64(0)
        code = T.load().tsf_candidates(T._ptr(self.Tl), 0, T._ptr(self.Rl), T._ptr(self.field),
                                       T.STORAGE[self.storage], X, Y, Z, PARAMS["tdf_high"], PARAMS["cube_size"],
                                       T._ptr(self.verts), self.max_vertices, None, None, 0, C.byref(nc),
                                       C.byref(nv), T._ptr(self.cand_ws), self.cand_ws.numel(), T._stream())
        if code not in (0, 4):
            T._check(code)
        return {"status": code, "n_candidates": nc.value, "n_vertices": nv.value}


def run_tsf(args, rank, world):
    import torch
    import synthetic
    import tsf_gb300 as T

    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    dev_index = torch.cuda.current_device()
    n = args.size
    shape = (n, n, n)
    vol = synthetic.vascular_tree(shape, seed=args.seed + rank)
    host = torch.from_numpy(vol).pin_memory()
    pipe = Pipeline(T, torch, shape, args.storage, args.iters, args.mu)
    pipe.vol.copy_(host, non_blocking=True)
    torch.cuda.synchronize()
    N = n ** 3

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident timed region --------------------------------------------
    clocks = ClockSampler(dev_index)
    clocks.start()                        # live before the warm-up; samples counted from mark()
    for _ in range(args.warmup):
        pipe.step()
    torch.cuda.synchronize()
    barrier()
    clocks.mark()
    l0 = T.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.profiler.start()           # a profiler started with collection off records only this region
    e0.record()
    for _ in range(args.steps):
        pipe.step()
    e1.record()
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    launches = T.kernel_launches() - l0
    barrier()
    clk = clocks.stop()
    ms = reduce_max(e0.elapsed_time(e1) / args.steps, world)
    value = replica_throughput(N * args.iters, ms * 1e-3, world) / 1e9

    # ---- per-stage times (one instrumented step) ------------------------------------
    evs = []
    pipe.step(events=evs)
    torch.cuda.synchronize()
    stages = {}
    for (a, ea), (b, eb) in zip(evs[:-1], evs[1:]):
        stages[b] = round(ea.elapsed_time(eb), 4)

    # ---- GVF kernel: average launch duration, both storage formats ------------------
    def gvf_kernel_stats(storage, mu, mode=0):
        p = pipe if storage == args.storage else Pipeline(T, torch, shape, storage, args.iters, mu)
        p.gvf_mode = mode
        if p is not pipe:
            p.vol.copy_(pipe.vol)
            T.blur(p.vol, PARAMS["large_blur"], out=p.blurred)
            p._vf(p.blurred, p.f0, None)
        p.mu = mu
        p.gvf_only()
        torch.cuda.synchronize()
        la = T.kernel_launches()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        reps = 2
        a.record()
        for _ in range(reps):
            p.gvf_only()
        b.record()
        torch.cuda.synchronize()
        nl = (T.kernel_launches() - la) / reps
        gvf_ms = a.elapsed_time(b) / reps
        p.mu = args.mu
        p.gvf_mode = 0
        return gvf_ms, nl

    gvf_ms, gvf_launches = gvf_kernel_stats(args.storage, args.mu)
    gvf_ms_mu01, _ = gvf_kernel_stats(args.storage, 0.1)
    f32_ms, _ = gvf_kernel_stats("f32", args.mu)
    vec_ms, _ = gvf_kernel_stats(args.storage, args.mu, mode=1)

    # ---- the whole path with FP32 storage (same volume, same steps) -------------------
    path32_ms = None
    if args.storage != "f32":
        p32 = Pipeline(T, torch, shape, "f32", args.iters, args.mu)
        p32.vol.copy_(pipe.vol)
        p32.step()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(2):
            p32.step()
        b.record()
        torch.cuda.synchronize()
        path32_ms = a.elapsed_time(b) / 2
        del p32
    s_bytes = 4 if args.storage == "f32" else 2
    iters_per_launch = args.iters / gvf_launches
    launch_s = gvf_ms * 1e-3 / gvf_launches
    algo_bytes = 9 * s_bytes * N * iters_per_launch
    peaks = mem_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = algo_bytes / launch_s / 1e9

    # ---- e2e through the C ABI with host buffers --------------------------------------
    # Every step copies its volume in from pinned host memory and its TDF, radius
    # and vertex list out; the copies run on a second stream, overlapped with the
    # neighbouring steps' compute: the volume of step j + 1 is uploaded into the
    # other of two input buffers while step j computes (once step j - 1, which
    # read that buffer, is done), and step j's results are copied device to
    # device into staging buffers and downloaded while step j + 1 computes.
    out_T = torch.empty(shape, dtype=torch.float32).pin_memory()
    out_R = torch.empty(shape, dtype=torch.float32).pin_memory()
    out_V = torch.empty((pipe.max_vertices, 3), dtype=torch.int32).pin_memory()
    main, copy = torch.cuda.current_stream(), torch.cuda.Stream()
    vols = [pipe.vol, torch.empty_like(pipe.vol)]
    stage_T, stage_R, stage_V = torch.empty_like(pipe.Tl), torch.empty_like(pipe.Rl), torch.empty_like(pipe.verts)

    def e2e_run(nsteps):
        ev_in = torch.cuda.Event()
        with torch.cuda.stream(copy):
            vols[0].copy_(host, non_blocking=True)
        ev_in.record(copy)
        ev_out = None
        nvs = []
        for j in range(nsteps):
            main.wait_event(ev_in)                       # this step's volume has landed
            pipe.vol = vols[j % 2]
            if j + 1 < nsteps:                           # next volume, into the buffer step j - 1 read
                ev_free = torch.cuda.Event()
                ev_free.record(main)
                copy.wait_event(ev_free)
                with torch.cuda.stream(copy):
                    vols[(j + 1) % 2].copy_(host, non_blocking=True)
                ev_in = torch.cuda.Event()
                ev_in.record(copy)
            pipe.step()
            nv = min(pipe.last["n_vertices"], pipe.max_vertices)
            if ev_out is not None:
                main.wait_event(ev_out)                  # the previous download has left the staging buffers
            stage_T.copy_(pipe.Tl)
            stage_R.copy_(pipe.Rl)
            if nv:
                stage_V[:nv].copy_(pipe.verts[:nv])
            ev_done = torch.cuda.Event()
            ev_done.record(main)
            copy.wait_event(ev_done)
            with torch.cuda.stream(copy):
                out_T.copy_(stage_T, non_blocking=True)
                out_R.copy_(stage_R, non_blocking=True)
                if nv:
                    out_V[:nv].copy_(stage_V[:nv], non_blocking=True)
            ev_out = torch.cuda.Event()
            ev_out.record(copy)
            nvs.append(nv)
        torch.cuda.synchronize()
        return nvs

    e2e_run(max(1, args.warmup))
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    nvs = e2e_run(args.steps)
    torch.cuda.synchronize()
    e2e_s = reduce_max((time.perf_counter() - t0) / args.steps, world)
    e2e_value = replica_throughput(N * args.iters, e2e_s, world) / 1e9
    h2d = N * 4
    d2h = N * 4 * 2 + int(np.mean(nvs)) * 12

    res = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 arithmetic, %s field storage" % args.storage, "data": "synthetic",
        "config": {"workload": "vessel tree %d^3, GVF %d iterations, mu %.2f, %s storage, full hot path"
                               % (n, args.iters, args.mu, args.storage),
                   "volume": [n, n, n], "gvf_iterations": args.iters, "mu": args.mu,
                   "storage": args.storage, "params": PARAMS,
                   "l2": "inputs larger than L2 (GVF streams 3 x %.0f MB per iteration)" % (3 * N * s_bytes / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "stages_ms": stages,
        "gvf": {"ms": round(gvf_ms, 3), "gvox_iter_s": round(N * args.iters / (gvf_ms * 1e-3) / 1e9, 2),
                "launches": gvf_launches, "iterations_per_launch": iters_per_launch,
                "gvox_iter_s_mu_0_1": round(N * args.iters / (gvf_ms_mu01 * 1e-3) / 1e9, 2),
                "f32_store_gvox_iter_s": round(N * args.iters / (f32_ms * 1e-3) / 1e9, 2),
                "speedup_vs_f32_store": round(f32_ms / gvf_ms, 3),
                "register_vector_kernel_gvox_iter_s": round(N * args.iters / (vec_ms * 1e-3) / 1e9, 2),
                "device_error": T.gvf_device_error()},
        "candidates": pipe.last,
        "f32_path": None if path32_ms is None else {
            "ms_per_step": round(path32_ms, 3),
            "speedup_of_%s_path" % args.storage: round(path32_ms / ms, 3)},
        "roofline": {"bound": "hbm", "kernel": "GVF iteration", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": "measured" if peaks else "fallback",
                     "bytes_per_launch": algo_bytes, "traffic": None},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_s * 1e3, 3)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    res["fwd_adjoint"] = fwd_adjoint_timing(torch, pipe, args)
    res["linking"] = linking_timing(torch, T, pipe, rank == 0 and world == 1 and not args.no_cpu_baseline)
    res["segmentation"] = segmentation_timing(torch, T, pipe,
                                              rank == 0 and world == 1 and not args.no_cpu_baseline)
    res["spline_tdf"] = spline_timing(torch, T, pipe, rank == 0 and world == 1 and not args.no_cpu_baseline)
    res["run_api"] = run_api_timing(args, vol)
    res["seed_sweep"] = seed_sweep(torch, pipe, args, rank)
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.storage in ("f16", "bf16"):
        res["exact_centerline_16bit"] = exact_centerline_timing(args)
    traffic = _traffic_from_profile(args.storage)
    if traffic:
        res["roofline"]["traffic"] = traffic
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(args, vol)
    return res


def exact_centerline_timing(args):
    """The 16-bit step that reproduces the FP64 run's vertex list (GVF in the
    16-bit format for K - 4 iterations and 4 in snorm16, the field in snorm16
    for the finish and the large-radius pass, the small-radius pass on the FP32
    field) beside the FP32 step; the vertex list is compared with the FP64
    oracle run of the same method on the host (bench.py --polish for more
    variants)."""
    import types
    a = types.SimpleNamespace(**vars(args))
    a.polish_iters = 4
    st, k = args.storage, a.polish_iters
    name = "%s+%d_snorm16_polish_f32_small" % (st, k)
    r = run_polish(a, only=("f32", name))
    v = r[name]
    return {"variant": "%d iterations in %s, the last %d in snorm16; snorm16 field for the finish and the "
                       "large-radius pass; FP32 small-radius field" % (args.iters - k, st, k),
            "ms": v["ms"], "f32_path_ms": r["f32"]["ms"], "speedup_vs_f32_path": round(r["f32"]["ms"] / v["ms"], 3),
            "same_vertex_list_as_fp64": v["same_vertex_list"], "vertices": v["vertices"],
            "fp64_vertices": r["fp64_vertices"], "oracle_s": r["oracle_s"]}


def seed_sweep(torch, pipe, args, rank, steps=5):
    """The step on the vessel-tree volumes of three seeds (this run's seed and
    the next two; the measurement plan asks for the median over seeds): ms per
    step and vertices for each, CUDA events over `steps` steps after one
    warm-up.  Leaves the last volume in the pipeline."""
    import synthetic
    n = args.size
    seeds = [args.seed + rank + i for i in range(3)]
    ms, verts = [], []
    for sd in seeds:
        pipe.vol.copy_(torch.from_numpy(synthetic.vascular_tree((n, n, n), seed=sd)))
        pipe.step()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            pipe.step()
        b.record()
        torch.cuda.synchronize()
        ms.append(round(a.elapsed_time(b) / steps, 3))
        verts.append(int(pipe.last["n_vertices"]))
    return {"seeds": seeds, "ms_per_step": ms, "median_ms": float(np.median(ms)), "vertices": verts}


def fwd_adjoint_timing(torch, pipe, args, storage=None, checkpoint_every=None):
    """Forward (both TDF passes, GVF K iterations) and forward + hand-written
    adjoint of the loss mean((T - G)^2) with respect to the volume, mu and
    sigma, on the benchmark volume, in the benchmark's storage format with a
    GVF checkpoint every ceil(sqrt(K)) iterations (the adjoint recomputes the
    states between checkpoints)."""
    import math
    import calibration as CAL
    storage = storage or args.storage
    C = checkpoint_every or int(math.ceil(math.sqrt(args.iters)))
    p = CAL.Params(mu=args.mu, sigma=PARAMS["large_blur"], iterations=args.iters, fmax=PARAMS["fmax"],
                   rmin=PARAMS["rmin"], rmax=PARAMS["rmax"], rstep=PARAMS["rstep"], checkpoint_every=C,
                   storage=storage)
    vol = pipe.vol
    G = torch.zeros_like(vol)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    Tc, state = CAL.forward(vol, p)               # allocates the adjoint workspace once
    gT = ((2.0 / vol.numel()) * (Tc - G)).contiguous()
    CAL.backward(state, gT, p)                    # warm-up: first launches, tensor maps, buffers
    torch.cuda.synchronize()
    ev[0].record()
    Tc, state = CAL.forward(vol, p, reuse=state)
    ev[1].record()
    torch.cuda.synchronize()
    # the timed forward + adjoint, with a mark after each stage (CUDA events
    # on the launching stream and host wall time)
    marks = []

    def mark(name):
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        marks.append((name, e, time.perf_counter()))

    retries0 = torch.cuda.memory_stats().get("num_alloc_retries", 0)
    t_host0 = time.perf_counter()
    ev[2].record()
    Tc, state = CAL.forward(vol, p, reuse=state)
    mark("forward")
    gT = ((2.0 / Tc.numel()) * (Tc - G)).contiguous()
    mark("loss")
    gI, dmu, dsig = CAL.backward(state, gT, p, mark=mark)
    ev[3].record()
    torch.cuda.synchronize()
    t_host = time.perf_counter() - t_host0
    retries = torch.cuda.memory_stats().get("num_alloc_retries", 0) - retries0
    fwd = ev[0].elapsed_time(ev[1])
    both = ev[2].elapsed_time(ev[3])
    stages, prev, prev_h = {}, ev[2], t_host0
    for name, e, th in marks:
        stages[name] = {"gpu_ms": round(prev.elapsed_time(e), 3), "host_ms": round((th - prev_h) * 1e3, 3)}
        prev, prev_h = e, th
    bw = {k: v["gpu_ms"] for k, v in stages.items() if k not in ("forward", "loss")}
    return {"storage": storage, "iterations": args.iters, "volume": list(vol.shape), "backward_ms": bw,
            "timed_stages": stages, "host_ms": round(t_host * 1e3, 3), "alloc_retries": int(retries),
            "checkpoint_every": int(state["checkpoint_every"]),
            "adjoint_workspace_gb": round(state["gvf_ws"].numel() / 1e9, 2),
            "fwd_ms": round(fwd, 3), "fwd_adjoint_ms": round(both, 3), "ratio": round(both / fwd, 3),
            "note": "loss mean((TDF - G)^2); gradients w.r.t. the volume, mu and blur sigma"}


def run_api_timing(args, vol, repeats=3):
    """The drop-in C++ API end to end: run(filename, paramList, kernel_dir)
    on the benchmark volume written as an .mhd/.raw file (MET_FLOAT,
    toFloat window [0, 1]) with the workload's parameters (FP16 GVF storage,
    the reference's 16-bit TDF, linking with the Synthetic-Vascusynth
    constants, inverse-gradient segmentation), timed on the host clock by the
    C++ driver (tests/cpp/test_api.cpp bench): file read, uploads, the whole
    pipeline and the getters' copies of the TDF, centerline and segmentation."""
    import tempfile
    import build as tsf_build
    exe = tsf_build.API_TESTS
    if not os.path.exists(exe):
        return {"error": "C++ driver not built"}
    P = PARAMS
    n = args.size
    with tempfile.TemporaryDirectory() as d:
        base = os.path.join(d, "vol")
        with open(base + ".mhd", "w") as f:
            f.write("ObjectType = Image\nNDims = 3\nDimSize = %d %d %d\nElementType = MET_FLOAT\n"
                    "ElementDataFile = vol.raw\n" % (n, n, n))
        np.ascontiguousarray(vol, np.float32).tofile(base + ".raw")
        cmd = [exe, "bench", base + ".mhd", str(repeats), "--minimum", "0", "--maximum", "1", "--mode", "white",
               "--large-blur", str(P["large_blur"]), "--small-blur", "0", "--fmax", str(P["fmax"]),
               "--gvf-mu", str(args.mu), "--gvf-iterations", str(args.iters), "--radius-min", str(P["rmin"]),
               "--radius-max", str(P["rmax"]), "--radius-step", str(P["rstep"]), "--tdf-high", str(P["tdf_high"]),
               "--cube-size", str(P["cube_size"]), "--gvf-storage", args.storage, "--16bit-vectors", "true",
               "--min-mean-tdf", "0.3", "--max-distance", "10", "--min-tree-length", "3"]
        p = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    if p.returncode != 0:
        return {"error": (p.stdout + p.stderr)[-400:]}
    r = json.loads(p.stdout.strip().splitlines()[-1])
    med = float(np.median(r["run_ms"]))
    return {"ms_per_volume": round(med, 2), "volumes_per_s": round(1e3 / med, 3),
            "gvox_iter_s": round(n ** 3 * args.iters / (med * 1e-3) / 1e9, 2), "runs_ms": r["run_ms"],
            "run_call_ms": round(float(np.median(r["run_call_ms"])), 2),
            "getters_ms": round(float(np.median(r["getters_ms"])), 2),
            "vertices": r["vertices"], "segmented_voxels": r["segmented_voxels"],
            "note": "run() through the C++ API, host clock, median of %d after one warm-up; includes reading the "
                    "%d MB .raw file" % (repeats, n ** 3 * 4 // 1000000)}


def linking_timing(torch, T, pipe, with_cpu):
    """Centerline linking of the step's vertices (tsf_link_centerpoints +
    tsf_rasterize_trees; the Synthetic-Vascusynth linking parameters), CUDA
    events over 5 repetitions after one warm-up, and the oracle on the host."""
    nv = min(pipe.last["n_vertices"], pipe.max_vertices)
    if nv < 2:
        return None
    v = pipe.verts[:nv].contiguous()
    shape = pipe.Tl.shape
    T.link_centerpoints(v, pipe.Tl, 0.3, 10.0)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    a.record()
    for _ in range(reps):
        edges, labels, sizes = T.link_centerpoints(v, pipe.Tl, 0.3, 10.0)
        T.rasterize_trees(v, edges, labels, sizes, 3, shape)
    b.record()
    torch.cuda.synchronize()
    out = {"vertices": nv, "edges": int(edges.shape[0]), "ms": round(a.elapsed_time(b) / reps, 3),
           "note": "includes the host synchronisation that returns the edge count"}
    if with_cpu:
        import oracle as O
        vh, Th = v.cpu().numpy(), pipe.Tl.cpu().numpy()
        t0 = time.perf_counter()
        e, l, s_ = O.link_centerpoints(vh, Th, 0.3, 10.0)
        O.rasterize_trees(vh, e, l, s_, 3, Th.shape)
        out["cpu_oracle_ms"] = round((time.perf_counter() - t0) * 1e3, 3)
        out["cpu_cores"] = O.get_threads()
    return out


def segmentation_timing(torch, T, pipe, with_cpu):
    """Segmentation of the step's linked centerlines (trees of at least 3
    vertices, the Synthetic-Vascusynth parameters) on the step's GVF field and
    radius: inverse-gradient growing (tsf_segment_inverse_gradient, which
    synchronises once per batch of grow iterations) and spheres
    (tsf_segment_spheres), CUDA events over 5 repetitions after one warm-up,
    and the oracle's inverse-gradient growing on the host."""
    nv = min(pipe.last["n_vertices"], pipe.max_vertices)
    if nv < 2:
        return None
    v = pipe.verts[:nv].contiguous()
    shape = pipe.Tl.shape
    edges, labels, sizes = T.link_centerpoints(v, pipe.Tl, 0.3, 10.0)
    cl = T.rasterize_trees(v, edges, labels, sizes, 3, shape)
    R = pipe.Rl
    seg, iters = T.segment_inverse_gradient(cl, pipe.field, R, storage=pipe.storage)
    T.segment_spheres(cl, R)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    a.record()
    for _ in range(reps):
        T.segment_inverse_gradient(cl, pipe.field, R, storage=pipe.storage)
    b.record()
    torch.cuda.synchronize()
    ig_ms = a.elapsed_time(b) / reps
    a.record()
    for _ in range(reps):
        sph = T.segment_spheres(cl, R)
    b.record()
    torch.cuda.synchronize()
    out = {"centerline_voxels": int(cl.sum()), "grow_iterations": iters,
           "segmented_voxels": int(seg.to(torch.int32).sum()), "inverse_gradient_ms": round(ig_ms, 3),
           "sphere_voxels": int(sph.to(torch.int32).sum()),
           "sphere_ms": round(a.elapsed_time(b) / reps, 3)}
    if with_cpu:
        import oracle as O
        F = pipe.field
        if pipe.storage == "snorm16":       # max(-1, s / 32767), divided on the host
            Fh = np.maximum(np.float32(-1.0), F.cpu().numpy().astype(np.float32) / np.float32(32767.0))
        else:
            Fh = F.float().cpu().numpy()
        t0 = time.perf_counter()
        ref, rit = O.segment_inverse_gradient(cl.cpu().numpy(), Fh, R.cpu().numpy())
        out["cpu_oracle_inverse_gradient_ms"] = round((time.perf_counter() - t0) * 1e3, 3)
        out["cpu_cores"] = O.get_threads()
        out["matches_oracle"] = bool(rit == iters and (ref == seg.cpu().numpy()).all())
    return out


def spline_timing(torch, T, pipe, with_cpu):
    """The spline TDF (tsf_tdf_spline, the large-radius TDF of the
    use-spline-tdf presets) on the step's GVF field, from max(1.5, rmin) to
    rmax in the workload's steps, beside the circle-fitting TDF on the same
    field and radii; CUDA events over 3 repetitions after one warm-up, and the
    oracle on a 64-slice slab of the field on the host."""
    P = PARAMS
    rmin = max(1.5, P["rmin"])
    Tsp, Rsp = T.tdf_spline(pipe.field, rmin, P["rmax"], P["rstep"], storage=pipe.storage)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    a.record()
    for _ in range(reps):
        Tsp, Rsp = T.tdf_spline(pipe.field, rmin, P["rmax"], P["rstep"], storage=pipe.storage)
    b.record()
    torch.cuda.synchronize()
    sp_ms = a.elapsed_time(b) / reps
    a.record()
    for _ in range(reps):
        T.tdf_circle(pipe.field, rmin, P["rmax"], P["rstep"], storage=pipe.storage)
    b.record()
    torch.cuda.synchronize()
    out = {"radii": [rmin, P["rmax"], P["rstep"]], "ms": round(sp_ms, 3),
           "circle_fit_same_radii_ms": round(a.elapsed_time(b) / reps, 3),
           "valid_voxels": int((Tsp > 0).sum())}
    if with_cpu:
        import oracle as O
        F = pipe.field
        if pipe.storage == "snorm16":       # max(-1, s / 32767), divided on the host
            Fh = np.maximum(np.float32(-1.0), F.cpu().numpy().astype(np.float32) / np.float32(32767.0))
        else:
            Fh = F.float().cpu().numpy()
        z0 = Fh.shape[0] // 2 - 32
        slab = np.ascontiguousarray(Fh[z0:z0 + 64])
        t0 = time.perf_counter()
        O.tdf_spline(slab, rmin, P["rmax"], P["rstep"])
        cpu_s = time.perf_counter() - t0
        out["cpu_oracle_ms_per_volume"] = round(cpu_s * 1e3 * Fh.shape[0] / 64, 1)
        out["cpu_cores"] = O.get_threads()
        out["cpu_sample"] = "64-slice slab of the field, scaled to the volume"
    return out


def run_stage(args):
    """One stage alone.  spline / circle: the vessel tree (--size^3), blur,
    vector field and --iters GVF iterations in --storage, then the TDF 3 times
    after one warm-up (CUDA events; spline from max(1.5, rmin), circle from
    max(2.5, rmin), both to the workload's rmax; circle is timed without and
    with the paired-texel workspace).  segment: one pipeline step
    with --iters GVF iterations, then segmentation_timing.  crop:
    crop_timing on the 512x512x400 lung CT.  gvf: the streaming and the
    register-vector GVF kernels (tsf_gvf_mode 0, 1) timed over --iters
    iterations."""
    import torch
    import synthetic
    import tsf_gb300 as T
    n, st, P = args.size, args.storage, PARAMS
    if args.stage == "crop":
        hu = synthetic.lung_ct((400, 512, 512), seed=args.seed)
        return {"stage": "crop", "workload": "lung-airway CT 512x512x400 int16",
                "lung_cropping": crop_timing(torch, T, hu, False)}
    if args.stage == "segment":
        pipe = Pipeline(T, torch, (n, n, n), st, args.iters, args.mu)
        pipe.vol.copy_(torch.from_numpy(synthetic.vascular_tree((n, n, n), seed=args.seed)))
        pipe.step()
        torch.cuda.synchronize()
        return {"stage": "segment", "workload": "vessel tree %d^3, GVF %d iterations, %s storage" % (n, args.iters, st),
                "segmentation": segmentation_timing(torch, T, pipe, False)}
    vol = torch.from_numpy(synthetic.vascular_tree((n, n, n), seed=args.seed)).cuda()
    b = T.blur(vol, P["large_blur"])
    f0, _ = T.vector_field(b, P["fmax"], P["vsign"], storage=st)
    if args.stage == "gvf":
        # each GVF kernel choice: one warm-up call of --iters iterations, then one timed call
        out = {"stage": "gvf", "workload": "vessel tree %d^3, %s storage, %d iterations per call" % (n, st, args.iters)}
        ws = T.workspace(T.load().tsf_gvf_workspace_size(n, n, n, T.STORAGE[st]))
        for mode, name in ((0, "streaming"), (1, "register_vector"), (3, "two_per_launch")):
            v = f0.clone()
            T.gvf(f0, args.mu, args.iters, st, v=v, ws=ws, mode=mode)
            torch.cuda.synchronize()
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            T.gvf(f0, args.mu, args.iters, st, v=v, ws=ws, mode=mode)
            e.record()
            torch.cuda.synchronize()
            out[name + "_us_per_iteration"] = round(a.elapsed_time(e) * 1e3 / args.iters, 2)
        # the low-memory variant (three one-component passes; 4 stored values moved
        # per component-voxel-iteration: v, f0_c and |f0|^2 read, v written)
        _, f4 = T.vector_field(b, P["fmax"], P["vsign"], storage=st, planar=False, field4=True)
        ows = T.workspace(T.load().tsf_gvf_one_component_workspace_size(n, n, n, T.STORAGE[st]))
        T.gvf_one_component(f4, args.mu, args.iters, st, ws=ows)
        torch.cuda.synchronize()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        T.gvf_one_component(f4, args.mu, args.iters, st, ws=ows)
        e.record()
        torch.cuda.synchronize()
        us = a.elapsed_time(e) * 1e3 / args.iters
        out["one_component_us_per_iteration"] = round(us, 2)
        out["one_component_gb_s"] = round(12 * (4 if st == "f32" else 2) * n ** 3 / (us * 1e-6) / 1e9, 1)
        return out
    v = T.gvf(f0, args.mu, args.iters, storage=st)
    field = T.gvf_finish(v, storage=st)
    runs = {}
    if args.stage == "spline":
        runs["spline"] = lambda: T.tdf_spline(field, max(1.5, P["rmin"]), P["rmax"], P["rstep"], storage=st)
    else:
        ws = T.workspace(T.load().tsf_tdf_workspace_size(n, n, n, T.STORAGE[st]))
        runs["circle"] = lambda: T.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"], storage=st)
        runs["circle_paired"] = lambda: T.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"], storage=st,
                                                     ws=ws)
        runs["circle_paired_sample_per_lane"] = lambda: T.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"],
                                                                     storage=st, ws=ws, samples=32, mode=2)
        runs["circle_paired_closed_eigen"] = lambda: T.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"],
                                                                  storage=st, ws=ws, eigen=1)
        runs["circle_paired_12_samples"] = lambda: T.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"],
                                                                storage=st, ws=ws, samples=12)
        _, fsm = T.vector_field(vol, P["fmax"], P["vsign"], storage=st, planar=False, field4=True)
        runs["small_paired"] = lambda: T.tdf_circle(fsm, P["rmin"], 3.0, 0.5, storage=st, ws=ws)
        runs["small_paired_queue"] = lambda: T.tdf_circle(fsm, P["rmin"], 3.0, 0.5, storage=st, ws=ws,
                                                          samples=32, mode=3)
        runs["small_paired_sample_per_lane"] = lambda: T.tdf_circle(fsm, P["rmin"], 3.0, 0.5, storage=st, ws=ws,
                                                                    samples=32, mode=2)
        runs["small_paired_closed_eigen"] = lambda: T.tdf_circle(fsm, P["rmin"], 3.0, 0.5, storage=st, ws=ws,
                                                                 eigen=1)
    for run in runs.values():
        run()
    torch.cuda.synchronize()
    out = {"stage": args.stage, "workload": "vessel tree %d^3, GVF %d iterations, %s storage" % (n, args.iters, st)}
    for name, run in runs.items():
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(3):
            Tt, _ = run()
        e.record()
        torch.cuda.synchronize()
        out[name + "_ms"] = round(a.elapsed_time(e) / 3, 3)
        out[name + "_nonzero"] = int((Tt != 0).sum())
    return out


def run_calibrate(args):
    """The differentiation configuration: 192^3 vessel tree (the 128^3
    generator), loss mean((TDF - G)^2) against the generator's Gaussian
    centerline map (sigma 1), adjoint of 300 GVF iterations with a checkpoint
    every 17, FP32.  Reports forward and forward + adjoint times, dL/dmu
    against a central difference of the FP64 oracle of the same method (with
    the step halved until the difference is smooth: slopes and curvatures at h
    and 2h agree), and 20 Adam steps on (mu, sigma)."""
    import torch
    import synthetic
    import calibration as CAL
    import oracle as O
    n = 192 if args.size == 256 else args.size
    K = 300 if args.iters == 500 else args.iters
    shape = (n, n, n)
    vol, truth = synthetic.vascular_tree(shape, seed=args.seed, with_truth=True)
    G = synthetic.centerline_gaussian(shape, truth["points"], 1.0)
    mk = lambda: CAL.Params(mu=args.mu, sigma=PARAMS["large_blur"], iterations=K, fmax=PARAMS["fmax"],
                            rmin=PARAMS["rmin"], rmax=PARAMS["rmax"], rstep=PARAMS["rstep"], checkpoint_every=17)
    p = mk()
    vd, Gd = torch.from_numpy(vol).cuda(), torch.from_numpy(G).cuda()
    L, gI, dmu, dsig, state = CAL.loss_and_grad(vd, Gd, p)          # warm-up, allocates the workspace
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    e[0].record()
    CAL.forward(vd, p, reuse=state)
    e[1].record()
    torch.cuda.synchronize()
    e[2].record()
    L, gI, dmu, dsig, state = CAL.loss_and_grad(vd, Gd, p, state)
    e[3].record()
    torch.cuda.synchronize()
    fwd, both = e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3])
    out = {"workload": "vessel tree %d^3, GVF %d iterations (checkpoint every 17), FP32, loss mean((TDF - G)^2)"
                       % (n, K),
           "fwd_ms": round(fwd, 3), "fwd_adjoint_ms": round(both, 3), "ratio": round(both / fwd, 3),
           "loss": L, "dmu": dmu, "dsigma": dsig, "grad_volume_finite": bool(torch.isfinite(gI).all())}
    del state
    torch.cuda.empty_cache()

    vol64 = vol.astype(np.float64)
    fs = O.vector_field(vol64, PARAMS["fmax"], PARAMS["vsign"], "f32", f64=True)
    Ts64, _ = O.tdf_circle(fs, PARAMS["rmin"], 3.0, 0.5, f64=True)
    f4 = O.vector_field(O.blur(vol, PARAMS["large_blur"], f64=True), PARAMS["fmax"], PARAMS["vsign"], "f32", f64=True)

    def Lo(dm):
        mu = float(np.float32(args.mu + dm))
        F = O.gvf_finish(O.gvf(f4, mu, K, f64=True), f64=True)
        Tl, _ = O.tdf_circle(F, max(2.5, PARAMS["rmin"]), PARAMS["rmax"], PARAMS["rstep"], f64=True)
        T64 = np.where(Tl < Ts64, Ts64, Tl)
        return float(((T64 - G) ** 2).mean())

    t0 = time.perf_counter()
    f0 = Lo(0.0)
    fd, used = None, None
    for h in (1e-4, 2.5e-5):
        fp, fm, fp2, fm2 = Lo(h), Lo(-h), Lo(2 * h), Lo(-2 * h)
        d1, d2 = (fp - fm) / (2 * h), (fp2 - fm2) / (4 * h)
        c1, c2 = (fp + fm - 2 * f0) / (h * h), (fp2 + fm2 - 2 * f0) / (4 * h * h)
        smooth = abs(d1 - d2) <= 1e-3 * max(abs(d1), 1e-9) and abs(c1 - c2) <= 0.05 * max(abs(c1), abs(c2)) + \
            1e-13 * max(1.0, abs(f0)) / (h * h)
        fd, used = d1, {"h": h, "smooth": bool(smooth), "d_h": d1, "d_2h": d2}
        if smooth:
            break
    out["dmu_fp64_central_difference"] = fd
    out["dmu_fd_detail"] = used
    out["dmu_rel_err"] = abs(dmu - fd) / max(abs(fd), 1e-30)
    out["fd_oracle_s"] = round(time.perf_counter() - t0, 1)

    p = mk()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p, hist = CAL.calibrate(vd, Gd, p, steps=20)
    torch.cuda.synchronize()
    out["adam"] = {"steps": 20, "s_per_step": round((time.perf_counter() - t0) / 21, 4),
                   "loss_first": hist[0]["loss"], "loss_last": hist[-1]["loss"],
                   "mu": [hist[0]["mu"], p.mu], "sigma": [hist[0]["sigma"], p.sigma]}
    return out


def run_mra(args):
    """The MRA-like workload (bright tubes of radii 5 -> 0.8 on 0.1, Rician
    noise sigma 0.08; 512^3, FP16 field storage, 1000 GVF iterations): the
    full hot-path step (CUDA events over one step after one warm-up), then the
    forward + hand-written adjoint of mean((TDF - G)^2) in the same storage
    (straight-through rounding) with the checkpoint interval chosen against
    60 % of the free device memory -- the full tape (1000 states) would not
    fit, the checkpointed one must."""
    import torch
    import synthetic
    import tsf_gb300 as T
    import calibration as CAL
    n = 512 if args.size == 256 else args.size
    K = 1000 if args.iters == 500 else args.iters
    st = "f16" if args.storage == "f16" else args.storage
    shape = (n, n, n)
    vol = synthetic.mra_tree(shape, seed=args.seed)
    out = {"workload": "MRA-like %d^3, Rician noise, %s storage, GVF %d iterations" % (n, st, K)}
    pipe = Pipeline(T, torch, shape, st, K, args.mu)
    pipe.vol.copy_(torch.from_numpy(vol))
    pipe.step()
    torch.cuda.synchronize()
    evs = []
    pipe.step(evs)
    torch.cuda.synchronize()
    stages = {name: round(evs[i - 1][1].elapsed_time(evs[i][1]), 3) for i, (name, _) in enumerate(evs) if i > 0}
    total = evs[0][1].elapsed_time(evs[-1][1])
    out["step"] = {"ms": round(total, 3), "volumes_per_s": round(1000.0 / total, 4), "stages_ms": stages,
                   "gvox_iter_s": round(n ** 3 * K / (stages.get("gvf", total) * 1e-3) / 1e9, 1),
                   "n_vertices": int(pipe.last["n_vertices"])}
    if args.accuracy:
        import oracle as O
        O.build()
        t0 = time.perf_counter()
        field64, T64, R64, refv = fp64_vessel_method(O, vol, K, args.mu)
        nv = min(pipe.last["n_vertices"], pipe.max_vertices)
        out["fp64_agreement"] = dict(
            fp64_agreement(T.to_float(pipe.field, st).cpu().numpy(), pipe.Tl.cpu().numpy(), pipe.Rl.cpu().numpy(),
                           pipe.verts[:nv].cpu().numpy(), field64, T64, R64, refv),
            oracle_s=round(time.perf_counter() - t0, 1))
        del field64, T64, R64
    vol_d = pipe.vol.clone()
    del pipe
    torch.cuda.empty_cache()
    state_bytes = 3 * n ** 3 * T.load().tsf_storage_bytes(T.STORAGE[st])
    p = CAL.Params(mu=args.mu, sigma=PARAMS["large_blur"], iterations=K, fmax=PARAMS["fmax"], rmin=PARAMS["rmin"],
                   rmax=PARAMS["rmax"], rstep=PARAMS["rstep"], storage=st)
    G = torch.zeros_like(vol_d)
    Tc, state = CAL.forward(vol_d, p)                     # allocates the adjoint workspace once
    CAL.backward(state, ((2.0 / vol_d.numel()) * (Tc - G)).contiguous(), p)
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    e[0].record()
    Tc, state = CAL.forward(vol_d, p, reuse=state)
    e[1].record()
    torch.cuda.synchronize()
    e[2].record()
    Tc, state = CAL.forward(vol_d, p, reuse=state)
    gI, dmu, dsig = CAL.backward(state, ((2.0 / Tc.numel()) * (Tc - G)).contiguous(), p)
    e[3].record()
    torch.cuda.synchronize()
    fwd, both = e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3])
    C = state["checkpoint_every"]
    out["fwd_adjoint"] = {"storage": st, "iterations": K, "checkpoint_every": C,
                          "adjoint_workspace_gb": round(state["gvf_ws"].numel() / 1e9, 2),
                          "full_tape_gb": round(K * state_bytes / 1e9, 1),
                          "fwd_ms": round(fwd, 3), "fwd_adjoint_ms": round(both, 3), "ratio": round(both / fwd, 3),
                          "dmu": float(dmu), "dsigma": float(dsig), "grad_finite": bool(torch.isfinite(gI).all())}
    return out


def run_adjoint(args):
    """Forward + adjoint timing alone on the vessel-tree volume (the same
    measurement the default run reports under fwd_adjoint)."""
    import types
    import torch
    import synthetic
    n = args.size
    vol = torch.from_numpy(synthetic.vascular_tree((n, n, n), seed=args.seed)).cuda()
    return {"workload": "vessel tree %d^3, GVF %d iterations, forward + adjoint" % (n, args.iters),
            "fwd_adjoint": fwd_adjoint_timing(torch, types.SimpleNamespace(vol=vol), args)}


def summarize_ncu_csv(path):
    """Per-kernel launches, total device time and share of an ncu launch list."""
    import csv
    import collections
    import re
    rows = list(csv.reader(open(path)))
    hi = next(i for i, r in enumerate(rows) if "Kernel Name" in r and "Metric Value" in r)
    K, V, U = (rows[hi].index(c) for c in ("Kernel Name", "Metric Value", "Metric Unit"))
    scale = {"ns": 1e-6, "nsecond": 1e-6, "us": 1e-3, "usecond": 1e-3, "ms": 1.0, "msecond": 1.0,
             "s": 1e3, "second": 1e3}
    tot, cnt = collections.defaultdict(float), collections.Counter()
    for r in rows[hi + 1:]:
        if len(r) <= V:
            continue
        name = re.sub(r"^void ", "", re.sub(r"\(.*", "", r[K]).strip())
        name = re.sub(r"<.*", "", name).replace("tsf::", "")
        tot[name] += float(r[V].replace(",", "")) * scale.get(r[U], 1.0)
        cnt[name] += 1
    total = sum(tot.values())
    lines = ["| kernel | launches | total ms | share |", "|---|---|---|---|"]
    for k, v in sorted(tot.items(), key=lambda kv: -kv[1]):
        lines.append("| `%s` | %d | %.3f | %.1f %% |" % (k, cnt[k], v, 100 * v / total))
    lines.append("| total | %d | %.3f | 100 %% |" % (sum(cnt.values()), total))
    return "\n".join(lines)


def _traffic_from_profile(storage):
    """DRAM bytes per GVF launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "gvf_traffic.json")
    try:
        d = json.load(open(p))
        return d.get(storage)
    except Exception:
        return None


def cpu_path(O, vol, storage, iters, mu):
    """One pass of the hot path through the oracle (the CPU restatement of the
    reference's kernels) on whatever threads the oracle is set to use: blur,
    vector fields, small-radius TDF, all `iters` GVF iterations, finish,
    large-radius TDF, combine, candidate stage.  Returns per-stage seconds."""
    P = PARAMS
    t = {}
    t0 = time.perf_counter()
    b = O.blur(vol, P["large_blur"])
    f_small = O.vector_field(vol, P["fmax"], P["vsign"], storage)
    t["blur_vf_small"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    Ts, Rs = O.tdf_circle(f_small, P["rmin"], 3.0, 0.5)
    t["tdf_small"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    f4 = O.vector_field(b, P["fmax"], P["vsign"], storage)
    t["vector_field"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    v = O.gvf(f4, mu, iters, storage)
    t["gvf"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    field = O.gvf_finish(v, storage)
    Tl, Rl = O.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"])
    Tl, Rl = O.combine(Ts, Rs, Tl, Rl)
    t["tdf_large"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.centerpoints(Tl, Rl, field, P["tdf_high"], P["cube_size"])
    t["candidates"] = time.perf_counter() - t0
    return t


def slab(vol, planes):
    """The middle `planes` z-planes of a volume (a bounded sample of the
    workload: same rows, same per-voxel work)."""
    z0 = (vol.shape[0] - planes) // 2
    return np.ascontiguousarray(vol[z0:z0 + planes])


def cpu_baseline(args, vol=None):
    """The oracle (CPU restatement of the reference kernels) timed on the
    host: the whole workload -- full volume, every stage, all GVF iterations
    -- on all host cores, and a z-slab of it (all iterations) on one core.
    Nothing is extrapolated."""
    import oracle as O
    import synthetic
    O.build()
    if vol is None:
        vol = synthetic.vascular_tree((args.size,) * 3, seed=args.seed)
    n = args.size
    N = n ** 3
    cores = O.get_threads()
    t = cpu_path(O, vol, args.storage, args.iters, args.mu)
    total = sum(t.values())
    one = {}
    planes = args.cpu_slab_planes_1core
    if planes > 0:
        sv = slab(vol, planes)
        O.set_threads(1)
        try:
            t1 = cpu_path(O, sv, args.storage, args.iters, args.mu)
        finally:
            O.set_threads(cores)
        tot1 = sum(t1.values())
        one = {"value": round(sv.size * args.iters / tot1 / 1e9, 5), "unit": UNIT, "cores": 1,
               "sample": "%dx%dx%d z-slab of the volume, every stage, all %d GVF iterations; %.1f s"
                         % (n, n, planes, args.iters, tot1),
               "stage_s": {a: round(b_, 3) for a, b_ in t1.items()}}
    return {"value": round(N * args.iters / total / 1e9, 5), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "the whole workload: %d^3 volume, every stage, all %d GVF iterations; %.1f s of CPU work"
                      % (n, args.iters, total),
            "stage_s": {a: round(b_, 3) for a, b_ in t.items()}, "one_core": one}


def run_reference(args):
    """The reference arm: the oracle on all host cores, K timed steps after W
    warm-up steps, each step one pass of the hot path (all GVF iterations) over
    a z-slab of the benchmark volume, so that the run stays within minutes."""
    import oracle as O
    import synthetic
    O.build()
    cores = O.get_threads()
    n = args.size
    vol = slab(synthetic.vascular_tree((n, n, n), seed=args.seed), args.reference_slab_planes)
    for _ in range(args.warmup):
        cpu_path(O, vol, args.storage, args.iters, args.mu)
    times, stages = [], {}
    for _ in range(args.steps):
        t0 = time.perf_counter()
        st = cpu_path(O, vol, args.storage, args.iters, args.mu)
        times.append(time.perf_counter() - t0)
        for k_, v_ in st.items():
            stages[k_] = stages.get(k_, 0.0) + v_ / args.steps
    step_s = sum(times) / len(times)
    value = vol.size * args.iters / step_s / 1e9
    sample = ("%dx%dx%d z-slab of the %d^3 vessel tree per step, every stage, all %d GVF iterations"
              % (n, n, vol.shape[0], n, args.iters))
    line = {"metric": METRIC, "impl": "reference", "value": round(value, 5), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 arithmetic, %s field storage" % args.storage, "data": "synthetic",
            "config": {"workload": "vessel tree %d^3, GVF %d iterations, mu %.2f, %s storage, full hot path"
                                   % (n, args.iters, args.mu, args.storage),
                       "implementation": "CPU restatement of the reference kernels (the oracle); the OpenCL "
                                         "reference cannot run: no OpenCL platform on these machines",
                       "sample": sample},
            "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "stage_s": {a: round(b_, 4) for a, b_ in stages.items()},
            "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


def fp64_agreement(field4, Tg, Rg, verts, field64, T64, R64, ref_vertices):
    """Errors of a GPU run (field4 as float [Z,Y,X,4], combined T and R, vertex
    list) against the FP64 oracle run of the same method: GVF field (xyz) max
    abs error, TDF abs errors (T in [0, 1]), radius agreement where both T are
    positive, and the centerpoint (vertex) agreement."""
    dF = np.abs(field4[..., :3].astype(np.float64) - field64[..., :3])
    dT = np.abs(Tg.astype(np.float64) - T64)
    both = (Tg > 0) & (T64 > 0)
    vset, gset = set(map(tuple, ref_vertices.tolist())), set(map(tuple, verts.tolist()))
    inter = len(vset & gset)
    return {"gvf_max_abs_err": float(dF.max()), "gvf_mean_abs_err": float(dF.mean()),
            "tdf_max_abs_err": float(dT.max()), "tdf_p999_abs_err": float(np.quantile(dT, 0.999)),
            "tdf_mean_abs_err": float(dT.mean()), "tdf_frac_within_1e-3": float((dT <= 1e-3).mean()),
            "radius_equal_frac": float((Rg[both] == R64[both]).mean()) if both.any() else 1.0,
            "vertices": int(len(gset)), "fp64_vertices": int(len(vset)), "vertices_equal_fp64": inter,
            "vertex_jaccard": round(inter / max(1, len(vset | gset)), 5),
            "same_vertex_list": bool(np.array_equal(verts, ref_vertices))}


def fp64_vessel_method(O, vol, iters, mu):
    """The FP64 oracle run of the vessel-tree step (blur, vector field, small
    and large TDF, combine, candidates) with the bench's parameters."""
    P = PARAMS
    b64 = O.blur(vol, P["large_blur"], f64=True)
    f64 = O.vector_field(b64, P["fmax"], P["vsign"], "f32", f64=True)
    field64 = O.gvf_finish(O.gvf(f64, mu, iters, f64=True), f64=True)
    fs64 = O.vector_field(vol.astype(np.float64), P["fmax"], P["vsign"], "f32", f64=True)
    Ts64, Rs64 = O.tdf_circle(fs64, P["rmin"], 3.0, 0.5, f64=True)
    Tl64, Rl64 = O.tdf_circle(field64, max(2.5, P["rmin"]), P["rmax"], P["rstep"], f64=True)
    T64, R64 = O.combine(Ts64, Rs64, Tl64, Rl64, f64=True)
    ref = O.centerpoints(T64, R64, field64, P["tdf_high"], P["cube_size"], f64=True)
    return field64, T64, R64, ref["vertices"]


def run_accuracy(args):
    """GVF field, TDF, centerpoint, centerline and segmentation agreement of the
    GPU path for each storage format against the FP64 oracle run of the same
    method (same volume, same parameters).  TDF errors are absolute (T is in
    [0, 1])."""
    import torch
    import oracle as O
    import synthetic
    import tsf_gb300 as T

    O.build()
    n = args.size
    shape = (n, n, n)
    vol = synthetic.vascular_tree(shape, seed=args.seed)
    P = PARAMS
    t0 = time.perf_counter()
    b64 = O.blur(vol, P["large_blur"], f64=True)
    f64 = O.vector_field(b64, P["fmax"], P["vsign"], "f32", f64=True)
    v64 = O.gvf(f64, args.mu, args.iters, f64=True)
    field64 = O.gvf_finish(v64, f64=True)
    fs64 = O.vector_field(vol.astype(np.float64), P["fmax"], P["vsign"], "f32", f64=True)
    Ts64, Rs64 = O.tdf_circle(fs64, P["rmin"], 3.0, 0.5, f64=True)
    Tl64, Rl64 = O.tdf_circle(field64, max(2.5, P["rmin"]), P["rmax"], P["rstep"], f64=True)
    T64, R64 = O.combine(Ts64, Rs64, Tl64, Rl64, f64=True)
    ref = O.centerpoints(T64, R64, field64, P["tdf_high"], P["cube_size"], f64=True)
    # linking (Synthetic-Vascusynth: min-mean-tdf 0.3, max-distance 10, min-tree-length 3)
    # and inverse-gradient segmentation of the FP64 method's results
    e64, l64, s64 = O.link_centerpoints(ref["vertices"], T64.astype(np.float32), 0.3, 10.0)
    cl64 = O.rasterize_trees(ref["vertices"], e64, l64, s64, 3, shape)
    seg64, _ = O.segment_inverse_gradient(cl64, field64.astype(np.float32), R64.astype(np.float32))
    t_oracle = time.perf_counter() - t0
    out = {"size": n, "iterations": args.iters, "mu": args.mu, "oracle_s": round(t_oracle, 1),
           "fp64_vertices": int(len(ref["vertices"])), "fp64_centerline_voxels": int(cl64.sum()),
           "fp64_segmented_voxels": int(seg64.sum()),
           "note": "linking, rasterisation and segmentation of the FP64 method's TDF, radius and field run in the "
                   "oracle's float restatement; Dice = 2|A and B| / (|A| + |B|)"}
    dice = lambda a, b: round(2.0 * float(np.logical_and(a, b).sum()) / max(1.0, float(a.sum() + b.sum())), 6)
    vset = set(map(tuple, ref["vertices"].tolist()))
    for st in ("f32", "f16", "bf16", "snorm16"):
        pipe = Pipeline(T, torch, shape, st, args.iters, args.mu)
        pipe.vol.copy_(torch.from_numpy(vol))
        pipe.step()
        torch.cuda.synchronize()
        v = T.to_float(pipe.v, st).cpu().numpy()
        Tg = pipe.Tl.cpu().numpy()
        dT = np.abs(Tg.astype(np.float64) - T64)
        got = pipe.verts[: min(pipe.last["n_vertices"], pipe.max_vertices)].cpu().numpy()
        gset = set(map(tuple, got.tolist()))
        inter = len(vset & gset)
        out[st] = {"gvf_max_abs_err": float(np.abs(v - v64).max()),
                   "tdf_max_abs_err": float(dT.max()),
                   "tdf_p999_abs_err": float(np.quantile(dT, 0.999)),
                   "tdf_mean_abs_err": float(dT.mean()),
                   "tdf_frac_within_1e-3": float((dT <= 1e-3).mean()),
                   "vertices": int(len(gset)), "vertices_equal_fp64": inter,
                   "vertex_jaccard": round(inter / max(1, len(vset | gset)), 5),
                   "same_vertex_list": bool(np.array_equal(got, ref["vertices"]))}
        dv = pipe.verts[: min(pipe.last["n_vertices"], pipe.max_vertices)].contiguous()
        edges, labels, sizes = T.link_centerpoints(dv, pipe.Tl, 0.3, 10.0)
        cl = T.rasterize_trees(dv, edges, labels, sizes, 3, shape)
        seg, _ = T.segment_inverse_gradient(cl, pipe.field, pipe.Rl, storage=st)
        cl, seg = cl.cpu().numpy() != 0, seg.cpu().numpy() != 0
        out[st]["centerline_dice"] = dice(cl, cl64 != 0)
        out[st]["segmentation_dice"] = dice(seg, seg64 != 0)
        del pipe
        torch.cuda.empty_cache()
    return out


def run_polish(args, only=None):
    """The 16-bit path that reproduces the FP64 centerline: GVF in --storage
    for K - k iterations, then k in FP32 (the iterate converted, f0 in FP32),
    the finished field in FP32 and the small-radius pass on the FP32 field of
    the raw volume; both TDF passes, combine and the candidate stage as in the
    benchmark step.  Variants store the polished field in snorm16 or in the
    16-bit format again for the finish and the large-radius pass, and the
    small-radius field in snorm16, FP32 or the 16-bit format; one runs the last
    k iterations in snorm16 instead of FP32.  Reports, per
    variant, the vertex list against the FP64 oracle run of the same method and
    the step time (CUDA events, median of 3 after a warm-up) next to the plain
    16-bit and FP32 paths."""
    import torch
    import oracle as O
    import synthetic
    import tsf_gb300 as T
    O.build()
    n, K, k = args.size, args.iters, args.polish_iters
    shape = (n, n, n)
    P = PARAMS
    vol = synthetic.vascular_tree(shape, seed=args.seed)
    t0 = time.perf_counter()
    _, _, _, V64 = fp64_vessel_method(O, vol, K, args.mu)
    t_oracle = time.perf_counter() - t0
    g = torch.from_numpy(vol).cuda()
    L = T.load()
    ws16 = T.workspace(L.tsf_tdf_workspace_size(n, n, n, T.STORAGE[args.storage]))

    def path(st, kp, fin_st, small_st, pol_st="f32"):
        b = T.blur(g, P["large_blur"])
        f0, _ = T.vector_field(b, P["fmax"], P["vsign"], st)
        v = T.gvf(f0, args.mu, K - kp, st)
        if kp:
            fp, _ = T.vector_field(b, P["fmax"], P["vsign"], pol_st)
            v = T.gvf(fp, args.mu, kp, pol_st, v=T.convert_field(v, st, pol_st))
            vst = pol_st
        else:
            vst = st
        if fin_st != vst:
            v = T.convert_field(v, vst, fin_st)
        field = T.gvf_finish(v, fin_st)
        _, fs = T.vector_field(g, P["fmax"], P["vsign"], small_st, planar=False, field4=True)
        wss = ws16 if small_st != "f32" else None
        wsl = ws16 if fin_st != "f32" else None
        Ts, Rs = T.tdf_circle(fs, P["rmin"], 3.0, 0.5, storage=small_st, ws=wss)
        Tl, Rl = T.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"], storage=fin_st, ws=wsl)
        T.tdf_combine(Ts, Rs, Tl, Rl)
        return T.candidates(Tl, Rl, field, fin_st, P["tdf_high"], P["cube_size"], raise_on_range=False)

    st = args.storage
    variants = {"%s" % st: (st, 0, st, st), "f32": ("f32", 0, "f32", "f32"),
                "%s+%d_f32_polish" % (st, k): (st, k, "f32", "f32"),
                "%s+%d_f32_polish_%s_small" % (st, k, st): (st, k, "f32", st),
                # the polished field stored in snorm16 (finer than f16 near unit magnitude) for the finish and
                # the large-radius pass, the small-radius field in snorm16 or FP32; or back in the 16-bit format
                "%s+%d_f32_polish_snorm16_tdf" % (st, k): (st, k, "snorm16", "snorm16"),
                "%s+%d_f32_polish_snorm16_large_f32_small" % (st, k): (st, k, "snorm16", "f32"),
                "%s+%d_f32_polish_%s_large_f32_small" % (st, k, st): (st, k, st, "f32"),
                # the last k iterations in snorm16 instead of FP32, the field left in snorm16
                "%s+%d_snorm16_polish_f32_small" % (st, k): (st, k, "snorm16", "f32", "snorm16")}
    if only is not None:
        variants = {name: a for name, a in variants.items() if name in only}
    s64 = set(map(tuple, V64.tolist()))
    out = {"size": n, "iterations": K, "mu": args.mu, "fp64_vertices": int(len(V64)), "oracle_s": round(t_oracle, 1),
           "note": "step = blur, vector fields, GVF, finish, both TDF passes, combine, candidates; CUDA events, "
                   "median of 3 after one warm-up"}
    for name, a in variants.items():
        r = path(*a)
        torch.cuda.synchronize()
        times = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = path(*a)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        got = r["vertices"].cpu().numpy()
        sg = set(map(tuple, got.tolist()))
        out[name] = {"ms": round(float(np.median(times)), 2), "vertices": int(len(got)),
                     "missing_fp64": len(s64 - sg), "extra": len(sg - s64),
                     "same_vertex_list": bool(np.array_equal(got, V64))}
    return out


def run_fmg_workload(args):
    """The 512x512x400 lung-airway CT (int16 HU, window [-1100, -600], dark
    tubes: vsign -1) through the hot path with full-multigrid GVF (3 levels,
    V-cycles) and FP16 storage; reported as ms per volume and per stage."""
    import torch
    import synthetic
    import tsf_gb300 as T

    shape = (400, 512, 512)
    hu = synthetic.lung_ct(shape, seed=args.seed)
    st = "f16"
    L = T.load()
    Z, Y, X = shape
    dt = T.storage_dtype(st)
    vol = torch.from_numpy(synthetic.window_to_unit(hu)).cuda()
    P = dict(fmax=0.3, vsign=-1, blur=1.0, rmin=1.0, rmax=9.0, rstep=0.5, tdf_high=0.45, cube_size=4)
    b = torch.empty_like(vol)
    f4 = torch.empty((Z, Y, X, 4), dtype=dt, device="cuda")
    f4s = torch.empty_like(f4)
    out = torch.empty_like(f4)
    ws = T.workspace(L.tsf_gvf_fmg_workspace_size(X, Y, Z, T.STORAGE[st]))
    Ts = torch.empty_like(vol); Rs = torch.empty_like(vol); Tl = torch.empty_like(vol); Rl = torch.empty_like(vol)
    cws = T.workspace(L.tsf_candidates_workspace_size(X, Y, Z))
    tws = T.workspace(L.tsf_tdf_workspace_size(X, Y, Z, T.STORAGE[st]))
    verts = torch.zeros((1 << 16, 3), dtype=torch.int32, device="cuda")
    import ctypes as C

    def step(evs=None):
        rec = (lambda: evs.append(torch.cuda.Event(enable_timing=True)) or evs[-1].record()) if evs is not None \
            else (lambda: None)
        rec()
        T._check(L.tsf_vector_field(T._ptr(vol), X, Y, Z, P["fmax"], P["vsign"], T.STORAGE[st], None, T._ptr(f4s), T._stream()))
        T._check(L.tsf_tdf_circle_ws(T._ptr(f4s), X, Y, Z, T.STORAGE[st], P["rmin"], 3.0, 0.5, T._ptr(Ts), 0, T._ptr(Rs),
                                     T._ptr(tws), tws.numel(), T._stream()))
        T.blur(vol, P["blur"], out=b)
        T._check(L.tsf_vector_field(T._ptr(b), X, Y, Z, P["fmax"], P["vsign"], T.STORAGE[st], None, T._ptr(f4), T._stream()))
        rec()
        T._check(L.tsf_gvf_fmg(T._ptr(f4), T._ptr(out), X, Y, Z, 0.2, args.fmg_cycles, T.STORAGE[st], T._ptr(ws), ws.numel(), T._stream()))
        rec()
        T._check(L.tsf_tdf_circle_ws(T._ptr(out), X, Y, Z, T.STORAGE[st], 2.5, P["rmax"], P["rstep"], T._ptr(Tl), 0,
                                     T._ptr(Rl), T._ptr(tws), tws.numel(), T._stream()))
        T.tdf_combine(Ts, Rs, Tl, Rl)
        rec()
        nc, nv = C.c_int64(0), C.c_int64(0)
        L.tsf_candidates(T._ptr(Tl), 0, T._ptr(Rl), T._ptr(out), T.STORAGE[st], X, Y, Z, P["tdf_high"], P["cube_size"],
                         T._ptr(verts), 1 << 16, None, None, 0, C.byref(nc), C.byref(nv), T._ptr(cws), cws.numel(),
                         T._stream())
        rec()
        return nc.value, nv.value

    for _ in range(2):
        step()
    torch.cuda.synchronize()
    l0 = T.kernel_launches()
    evs = []
    nc, nv = step(evs)
    torch.cuda.synchronize()
    launches = T.kernel_launches() - l0
    names = ["tdf_small_and_fields", "fmg_gvf", "tdf_large", "candidates"]
    stages = {k: round(evs[i].elapsed_time(evs[i + 1]), 3) for i, k in enumerate(names)}
    total = evs[0].elapsed_time(evs[-1])
    res = {"workload": "lung-airway CT 512x512x400, FMG GVF %d cycles x 3 components, FP16 storage" % args.fmg_cycles,
           "ms_per_volume": round(total, 3), "volumes_per_s": round(1000.0 / total, 3), "stages_ms": stages,
           "kernel_launches": int(launches), "n_candidates": nc, "n_vertices": nv,
           "lung_cropping": crop_timing(torch, T, hu, not args.no_cpu_baseline)}
    if args.accuracy:
        # the FP64 oracle run of the same method: small TDF on the unblurred
        # field, blur, FMG GVF, large TDF, combine, candidates
        import oracle as O
        O.build()
        t0 = time.perf_counter()
        v32 = synthetic.window_to_unit(hu)
        fs64 = O.vector_field(v32.astype(np.float64), P["fmax"], P["vsign"], "f32", f64=True)
        Ts64, Rs64 = O.tdf_circle(fs64, P["rmin"], 3.0, 0.5, f64=True)
        del fs64
        f64 = O.vector_field(O.blur(v32, P["blur"], f64=True), P["fmax"], P["vsign"], "f32", f64=True)
        field64 = O.fmg_gvf(f64, 0.2, args.fmg_cycles, "f32", f64=True)
        del f64
        Tl64, Rl64 = O.tdf_circle(field64, 2.5, P["rmax"], P["rstep"], f64=True)
        T64, R64 = O.combine(Ts64, Rs64, Tl64, Rl64, f64=True)
        refv = O.centerpoints(T64, R64, field64, P["tdf_high"], P["cube_size"], f64=True)["vertices"]
        res["fp64_agreement"] = dict(
            fp64_agreement(T.to_float(out, st).cpu().numpy(), Tl.cpu().numpy(), Rl.cpu().numpy(),
                           verts[: min(nv, 1 << 16)].cpu().numpy(), field64, T64, R64, refv),
            oracle_s=round(time.perf_counter() - t0, 1))
    return res


def crop_timing(torch, T, hu, with_cpu):
    """The lung cropping scan lines (cropDatasetLung over the three slice
    directions) on the raw int16 HU volume: CUDA events over 5 repetitions
    after one warm-up; the kernels read the volume twice (the z-columns serve
    the x and the y slices, the x-rows the z slices)."""
    d = torch.from_numpy(hu).cuda()
    T.crop_scan_lines(d, 1)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    a.record()
    for _ in range(reps):
        cx, cy, cz = T.crop_scan_lines(d, 1)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    out = {"ms": round(ms, 3), "bytes_read": 2 * hu.nbytes, "GBs": round(2 * hu.nbytes / ms / 1e6, 1),
           "max_counts": [int(c.max()) for c in (cx, cy, cz)]}
    if with_cpu:
        import oracle as O
        t0 = time.perf_counter()
        ref = O.crop_scan_lines(hu, 1)
        out["cpu_oracle_ms"] = round((time.perf_counter() - t0) * 1e3, 3)
        out["cpu_cores"] = 1
        out["matches_oracle"] = all(np.array_equal(g.cpu().numpy(), r) for g, r in zip((cx, cy, cz), ref))
    return out


def main():
    args = parse()
    if args.summarize_ncu_csv:
        print(summarize_ncu_csv(args.summarize_ncu_csv))
        return
    if args.adjoint:
        print(json.dumps(run_adjoint(args)))
        return
    if args.mra:
        print(json.dumps(run_mra(args)))
        return
    if args.calibrate:
        print(json.dumps(run_calibrate(args)))
        return
    if args.stage:
        print(json.dumps(run_stage(args)))
        return
    if args.fmg:
        print(json.dumps(run_fmg_workload(args)))
        return
    if args.accuracy:
        print(json.dumps(run_accuracy(args)))
        return
    if args.polish:
        print(json.dumps(run_polish(args)))
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    res = run_tsf(args, rank, world)
    if rank == 0:
        print(json.dumps(res))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
