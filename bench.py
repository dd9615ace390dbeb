"""Benchmark: map-pair alignments per second on GB300.

One alignment = the work of ``main.py orig`` on one map pair (threshold and
grid sizing, fastVEC of both maps, target spectra, the rotational search,
top-N, the +-5 degree refinement, the rotated top-N models and their float64
scores), on seeded synthetic maps.

Default workload ``prop128_s3_a10``: 128^3 / 64^3 blob-map pairs (the
128^3/64^3 generator) at s = 3, A = 10 (24624 rotations), each aligned with the
learned rotation proposal (the committed network ranks the grid, the exact
search correlates the best 5%, the exhaustive search is the fallback).  A
step aligns a batch of held-out pairs (seeds outside the training range).
The same pairs are also aligned with the exhaustive search: the line reports
both rates and the fraction of pairs whose top-1 rotation the two forms
agree on.  A step runs ``Aligner.align_many`` over its pairs: every stage is
launched for all pairs before the host waits.  The line also reports the
rate with the global stage (fastVEC, spectra, proposal, global search of
every pair) replayed as one CUDA graph (``graph_replay``; ``--graph`` makes
that the headline).  ``--workload pair200_s2_a10``:
one 200^3 / 100^3 pair per step, exhaustive search (no network).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``value``: device-resident maps, K steps timed with CUDA events between a
barrier + synchronize on both sides, whole-job alignments/s (max over ranks).
``e2e``: the same steps through ``Aligner.align_host_many`` with the maps copied
from pinned host memory every step and the results read back.
``--impl reference``: the reference algorithm's CPU path on this host's cores
(the oracle restatement: C fastVEC with OpenMP, numpy/scipy FFT search with
every core), exhaustive like the reference, timed on a bounded sample of the
same workload and scaled to a full alignment.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "prop128_s3_a10"
METRIC = "map-pair alignments/s: learned-proposal vs exhaustive on GPU at ≥99% top-1 match"
UNIT = "alignments/s"
HELD_OUT_SEED0 = 30_000_000     # training used seeds [0, 20000)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=WORKLOAD,
                    choices=["prop128_s3_a10", "pair200_s2_a10", "uneven64_s4_a15", "prob128_s3_a15"])
    ap.add_argument("--pairs", type=int, default=16, help="pairs per step (prop128_s3_a10)")
    ap.add_argument("--mode", default="V", choices=list("VOCPL"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--no-exhaustive", action="store_true",
                    help="skip the exhaustive form on the same pairs (profiling runs)")
    ap.add_argument("--graph", action="store_true",
                    help="headline value with the global stage replayed as one CUDA graph")
    ap.add_argument("--no-graph-replay", action="store_true",
                    help="skip the CUDA-graph measurement (profiler launch lists)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        """Start sampling every 50 ms; returns once nvidia-smi is answering
        (its first line, at most 5 s), with that line discarded, so the
        samples kept are those taken after this call."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
            return
        t0 = time.time()
        while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)
        self.lines.clear()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def pass_model(dim, mode):
    """Algorithmic work of each search pass for one rotation (V: 3 channels).
    FLOPs: a 3-D real FFT of N points is 2.5 N log2 N, split evenly over the
    three axes; the spectrum product is 8 flops per channel and half-spectrum
    element.  Bytes: what each pass must read and write in global memory."""
    N = dim ** 3
    H = dim // 2 + 1
    Nh = dim * dim * H
    C = {"V": 3, "prob": 7}.get(mode, 1)
    G = 2 if mode == "prob" else 1
    axis = 2.5 * N * np.log2(dim)          # one axis of one real 3-D FFT
    return {
        "pass_a": {"flop": C * 2 * axis, "bytes": N * 20 + C * Nh * 8},
        "pass_b": {"flop": C * axis + 8 * C * Nh + G * axis, "bytes": C * Nh * 8 * 2 + G * Nh * 8},
        "pass_c": {"flop": G * 2 * axis + N, "bytes": G * Nh * 8},
    }


def workload_pairs(args, rank, dev):
    """Device maps, pinned host copies and origins of the step's pairs."""
    import torch
    from vesper_python_gb300 import proposal, synth
    pairs = []
    if args.workload == "prop128_s3_a10":
        for i in range(args.pairs):
            m1, m2, o1, o2 = proposal.blob_pair_torch(HELD_OUT_SEED0 + rank * args.pairs + i, device=dev.device)
            pairs.append((m1, m2, m1.cpu().pin_memory(), m2.cpu().pin_memory(), o1, o2, 1.0))
    else:
        pr = synth.workload_pair(args.workload, seed=rank)   # weak scaling: one pair per rank
        h1 = torch.from_numpy(pr.map1).pin_memory()
        h2 = torch.from_numpy(pr.map2).pin_memory()
        pairs.append((dev.to_dev(pr.map1), dev.to_dev(pr.map2), h1, h2, pr.orig1, pr.orig2, pr.width))
    return pairs


def run_gb300(args):
    import torch
    import torch.distributed as dist

    from vesper_python_gb300 import align, proposal, synth
    from vesper_python_gb300 import vesper as vg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = synth.WORKLOADS[args.workload]
    mode = {"V": "VecProduct", "O": "Overlap", "C": "CC", "P": "PCC", "L": "Laplacian"}[args.mode]
    dev = vg.Device(f"cuda:{local}")
    use_prop = args.workload == "prop128_s3_a10"
    if use_prop and mode != "VecProduct":
        raise SystemExit("the learned proposal workload runs in mode V")
    net = proposal.load_weights(dev)[0] if use_prop else None
    p = align.AlignParams(t=w["t"], T=w["T"], g=w["g"], s=w["s"], A=w["A"], N=w["N"], mode=mode, batch=args.batch,
                          proposal=net)
    p_exh = align.AlignParams(t=w["t"], T=w["T"], g=w["g"], s=w["s"], A=w["A"], N=w["N"], mode=mode,
                              batch=args.batch)
    pairs = workload_pairs(args, rank, dev)
    al = align.Aligner(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev.device)   # > 129 MB L2

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def maxr(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    dev_items = [(m1, m2, wd, wd, o1, o2) for (m1, m2, _, _, o1, o2, wd) in pairs]
    host_items = [(h1, h2, wd, wd, o1, o2) for (_, _, h1, h2, o1, o2, wd) in pairs]

    graph = False

    def step(params):
        flush.zero_()
        out = al.align_many(dev_items, params, graph=graph)
        return out, al.launches

    def timed(params):
        for _ in range(args.warmup):
            step(params)
        barrier()
        clk = ClockSampler(local)
        clk.start()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        launches = 0
        e0.record()
        for _ in range(args.steps):
            res, nl = step(params)
            launches += nl
        e1.record()
        barrier()
        return maxr(e0.elapsed_time(e1)), res, launches, clk.stop()

    # the same steps with the global stage replayed as one CUDA graph (captured
    # in the warm-up for this batch's shapes and geometry; a batch of new maps
    # with another grid geometry captures again)
    ms_g = None
    if not args.no_graph_replay or args.graph:
        graph = True
        ms_g, _, _, _ = timed(p)
    graph = bool(args.graph)
    ms, res, launches, clocks = timed(p)
    npairs = len(pairs)
    value = world * npairs * args.steps / (ms / 1e3)
    value_graph = world * npairs * args.steps / (ms_g / 1e3) if ms_g else None
    fallbacks = 0
    if use_prop:
        # fallbacks in one step of the proposal form
        al.align_many(dev_items, p)
        fallbacks = sum(al.proposal_info["fallback"])
    # ---- per-stage and per-pass device time: one more step with events ------
    stages = {}
    al.stages = stages       # stage boundaries only: events between stages (eager launches)
    al.align_many(dev_items, p)
    barrier()
    al.stages = None
    prof = {}
    al.profile = prof        # events around every search launch (slower; its own step)
    al.align_many(dev_items, p)
    barrier()
    al.profile = None
    # ---- end to end: host maps copied in every step -------------------------
    def host_step(params):
        flush.zero_()
        al.align_host_many(host_items, params)
        return al.d2h_bytes
    host_step(p)
    barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    d2h = 0
    for _ in range(args.steps):
        d2h += host_step(p)
    t1.record()
    barrier()
    e2e_ms = maxr(t0.elapsed_time(t1))
    e2e_value = world * npairs * args.steps / (e2e_ms / 1e3)
    h2d = sum(int(h1.numel() * 4 + h2.numel() * 4) for (_, _, h1, h2, _, _, _) in pairs)
    # ---- the exhaustive form on the same pairs --------------------------------
    exh = None
    if use_prop and not args.no_exhaustive:
        ms_x, res_x, _, _ = timed(p_exh)
        agree = sum(int(a.top[0][0] == b.top[0][0]) for a, b in zip(res, res_x))
        agree_model = sum(int(a.models[0].angle == b.models[0].angle and
                              abs(a.models[0].dot_score - b.models[0].dot_score) <= 1e-4 * abs(b.models[0].dot_score))
                          for a, b in zip(res, res_x))
        exh = {"value": round(world * npairs * args.steps / (ms_x / 1e3), 4), "unit": UNIT,
               "ms_per_step": round(ms_x / args.steps, 3),
               "top1_agreement": agree / npairs, "refined_model1_agreement": agree_model / npairs,
               "proposal_speedup": round(ms_x / ms, 3), "proposal_fallbacks_per_step": fallbacks}
    dim = res[0].dim
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    # ---- roofline of the dominant search pass ---------------------------------
    pm = pass_model(dim, args.mode)
    names = ["pass_a", "pass_b", "pass_c"]
    pass_ms = prof["pass_ms"][:3]
    pass_n = prof["pass_launches"][:3]
    top = int(np.argmax(pass_ms))
    plan_path = vg.search_plan(dim, mode, 0, 1, None, dev)[0]
    nrot_step = None
    if use_prop:
        k = int(np.ceil(0.05 * len(vg.calc_angle_comb(p.A))))
        nrot_step = npairs * (k + 10 * 27)
    else:
        nrot_step = npairs * (len(vg.calc_angle_comb(p.A)) + 10 * 27)
    per_launch_rot = nrot_step / max(1, pass_n[top])
    avg_s = pass_ms[top] / max(1, pass_n[top]) / 1e3
    peak, peak_kind = peaks()
    ach_bytes = pm[names[top]]["bytes"] * per_launch_rot / avg_s / 1e9
    ach_flop = pm[names[top]]["flop"] * per_launch_rot / avg_s / 1e12
    sm_mhz = clocks.get("sm_mhz") or 1900.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    # DRAM bytes of the kernel per launch: the ncu capture's bytes per rotation
    # (profiles/traffic_<workload>.txt) times the rotations of an average launch
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", f"traffic_{args.workload}.txt")
    if os.path.exists(tr_path) and args.mode == "V":
        for ln in open(tr_path):
            f = ln.split()
            if len(f) == 2 and not ln.startswith("#") and f[0] == names[top]:
                traffic = int(round(float(f[1]) * per_launch_rot))
    kname = {0: "k_pass_", 1: "k_rpass_", 2: "k_fused"}[plan_path]
    kname = kname + names[top][-1] if plan_path != 2 else kname
    if use_prop:
        wl = (f"{args.workload}: {npairs} pairs per step, map1 128^3 / map2 64^3 (seeded blob maps, held-out seeds), "
              f"s=3, A=10 (24624 rotations, 5% correlated after the learned proposal, exhaustive fallback) "
              f"+ refinement, g=16, N=10, mode V")
        data = "synthetic (seeded 128^3 / 64^3 blob-map pairs at 1 A, generated on the GPU)"
    else:
        wl = (f"{args.workload}: map1 200^3, map2 100^3, s=2, A=10 (24624 rotations + refinement), g=16, N=10, "
              f"mode {args.mode}, exhaustive search")
        data = "synthetic (seeded blob maps, 200^3 and 100^3 at 1 A)"
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 fastVEC, target spectra, rescoring; bf16 weights)",
        "data": data,
        "config": {"workload": wl, "grid_side": dim, "pairs_per_step": npairs,
                   "rotations": len(vg.calc_angle_comb(p.A)),
                   "l2": "flushed before every step (256 MB write)", "parallelism": f"replicas x{world}",
                   "global_stage": "one CUDA graph replay per step" if args.graph else "eager launches"},
        "graph_replay": {"value": round(value_graph, 4), "unit": UNIT, "ms_per_step": round(ms_g / args.steps, 3),
                         "note": "global stage as one CUDA graph, captured once for this batch's shapes"}
        if value_graph else None,
        "e2e": {"value": round(e2e_value, 4), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(d2h / args.steps)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": f"search {names[top]} ({kname})", "achieved": round(ach_bytes, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(ach_bytes / peak, 4), "traffic": traffic,
                     "peak_source": peak_kind,
                     "fp32": {"achieved_tflops": round(ach_flop, 3), "peak_tflops": round(fp32_peak, 1),
                              "frac": round(ach_flop / fp32_peak, 4)}},
        "stage_ms_profiled_step": {k: round(v, 3) for k, v in stages.items()},
        "pass_ms_profiled_step": [round(x, 3) for x in prof["pass_ms"]],
        "clocks": clocks,
    }
    if exh is not None:
        line["exhaustive"] = exh
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, threads=1, budget_s=12.0)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_uneven(args):
    """64 pairs of uneven sizes (map1 side in {64..256}, map2 = map1 / 2, blob
    count proportional to volume) at s = 4, A = 15, exhaustive search: one
    align_many call per step with the global stage replayed as one CUDA graph.
    Reports alignments/s and the per-pair latency (batch start to the pair's
    last kernel, device events) p50/p99; also the same batch without the
    graph and each pair aligned alone."""
    import torch
    from vesper_python_gb300 import align, proposal, synth
    from vesper_python_gb300 import vesper as vg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = vg.Device(f"cuda:{local}")
    w = synth.UNEVEN_WORKLOAD
    p = align.AlignParams(t=w["t"], T=w["T"], g=w["g"], s=w["s"], A=w["A"], N=w["N"])
    items, host_items, sides = [], [], []
    for i in range(w["pairs"]):
        seed, side, nblob, radius = synth.uneven_spec(i + rank * w["pairs"])
        m1, m2, o1, o2 = proposal.blob_pair_torch(seed, side=side, nblob=nblob, radius=radius, device=dev.device)
        items.append((m1, m2, 1.0, 1.0, o1, o2))
        host_items.append((m1.cpu().pin_memory(), m2.cpu().pin_memory(), 1.0, 1.0, o1, o2))
        sides.append(side)
    al = align.Aligner(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev.device)

    def timed(graph, steps, warmup):
        for _ in range(warmup):
            al.align_many(items, p, graph)
        torch.cuda.synchronize()
        lat = []
        launches = 0
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        total = 0.0
        for _ in range(steps):
            flush.zero_()
            al.pair_events = []
            e0.record()
            res = al.align_many(items, p, graph)
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
            lat += [e0.elapsed_time(e) for e in al.pair_events]
            launches += al.launches
            al.pair_events = None
        return total / steps, np.array(lat), launches, res

    clk = ClockSampler(local)
    clk.start()
    ms, lat, launches, res = timed(True, args.steps, args.warmup)
    clocks = clk.stop()
    ms_ng, lat_ng, _, res_ng = timed(False, max(1, args.steps), 1)
    same = all(a.top == b.top and [m.dot_score for m in a.models] == [m.dot_score for m in b.models]
               for a, b in zip(res, res_ng))
    # e2e: maps copied from pinned host memory every step
    al.align_host_many(host_items, p, True)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    d2h = 0
    for _ in range(args.steps):
        flush.zero_()
        al.align_host_many(host_items, p, True)
        d2h += al.d2h_bytes
    t1.record()
    torch.cuda.synchronize()
    e2e_ms = t0.elapsed_time(t1) / args.steps
    # each pair alone (one align_device per pair); the first pass over the
    # pairs warms the single-pair path (its scratch buffers), the second is timed
    for it in items:
        al.align_device(*it, p)
    torch.cuda.synchronize()
    solo = []
    for it in items:
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record()
        al.align_device(*it, p)
        a1.record()
        torch.cuda.synchronize()
        solo.append(a0.elapsed_time(a1))
    solo = np.array(solo)
    n = len(items)
    dims = sorted({r.dim for r in res})
    pct = lambda a, q: round(float(np.percentile(a, q)), 3)
    line = {
        "metric": METRIC, "value": round(n / (ms / 1e3), 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 fastVEC, target spectra, rescoring)",
        "data": "synthetic (seeded blob-map pairs of uneven sizes at 1 A, generated on the GPU)",
        "config": {"workload": f"uneven64_s4_a15: {n} pairs per step, map1 side in {sorted(set(sides))} "
                               f"(map2 = side/2, blobs proportional to volume), s=4, A=15 "
                               f"({len(vg.calc_angle_comb(p.A))} rotations + refinement), g=16, N=10, mode V, "
                               f"exhaustive search, global stage as one CUDA graph",
                   "grid_sides": dims, "pairs_per_step": n,
                   "l2": "flushed before every step (256 MB write)", "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99), "note": "batch start to the pair's last kernel"},
        "without_graph": {"value": round(n / (ms_ng / 1e3), 4), "latency_p50_ms": pct(lat_ng, 50),
                          "latency_p99_ms": pct(lat_ng, 99), "same_results": bool(same)},
        "one_pair_at_a_time": {"value": round(n / (solo.sum() / 1e3), 4), "latency_p50_ms": pct(solo, 50),
                               "latency_p99_ms": pct(solo, 99)},
        "graph": {"captures": al.graph_captures, "replays": al.graph_replays},
        "e2e": {"value": round(n / (e2e_ms / 1e3), 4), "unit": UNIT,
                "h2d_bytes_per_step": int(sum(h1.numel() * 4 + h2.numel() * 4 for (h1, h2, *_r) in host_items)),
                "d2h_bytes_per_step": int(d2h / args.steps)},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_prob(args):
    """prob128_s3_a15: one 128^3 / 64^3 pair with four probability channels
    per step (Dirichlet(0.5) inside the thresholded density, rotated with map2),
    s = 3, grids padded to 64^3, A = 15 (7,488 rotations), alpha = 0.5.  A step
    is the prob-mode alignment on the device: fastVEC of the two densities and
    the eight probability maps, target spectra, the statistics pass and the
    mixed pass over the grid, top-N, and the mixed pass over the refinement
    set.  Timed with the float32 pass B (headline) and with the split-BF16
    tensor-core pass B (search path 3); the line reports both and how far the
    split-BF16 scores are from the float32 ones."""
    import contextlib
    import io

    import torch

    from vesper_python_gb300 import synth
    from vesper_python_gb300 import vesper as vg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = vg.Device(f"cuda:{local}")
    w = synth.WORKLOADS["prob128_s3_a15"]
    pr = synth.workload_pair("prob128_s3_a15", seed=rank)
    d, s_, g = int(w["pad"]), float(w["s"]), float(w["g"])
    geo = []
    for src, orig, th in ((pr.map1, pr.orig1, w["t"]), (pr.map2, pr.orig2, w["T"])):
        m = vg.mrc_obj.from_array(src, 1.0, orig)
        with contextlib.redirect_stdout(io.StringIO()):
            _, mn = vg.mrc_set_vox_size(m, th, s_)
        geo.append((dev.to_dev(m.data), np.float64(m.xwidth), m.orig.astype(np.float64),
                    np.asarray(mn.cent, np.float64) - 0.5 * s_ * d))
    pmaps = [[dev.to_dev(np.ascontiguousarray(pm[..., k], np.float32)) for k in range(4)]
             for pm in (pr.prob1, pr.prob2)]
    angles = vg.calc_angle_comb(w["A"])
    mats = vg.rot_matrices_device(angles, dev, key=("grid", float(w["A"])))
    n = len(angles)
    rd3 = 1.0 / d ** 3
    alpha = float(w["alpha"])

    def fields(i):
        # prob mode keeps fastVEC's density in float32 (main.py:345)
        src, sw, so, no = geo[i]
        _, d32, vec = vg.fastvec_device(src, sw, so, d, s_, no, g, dev=dev)
        probs = torch.stack([vg.fastvec_device(pm, sw, so, d, s_, no, g, dev=dev)[1] for pm in pmaps[i]])
        return d32.double(), vec, probs

    def step(path):
        opts = (path, 0, 0)
        tdata, tvec, tprobs = fields(0)
        qdata, qvec, qprobs = fields(1)
        spec = vg.target_spectra_device(tdata, tvec, "prob", 0.0, probs=tprobs, dev=dev)
        s1, _ = vg.search_device(spec, qdata, qvec, "prob", 0.0, mats, probs=qprobs, dev=dev, opts=opts)
        h = s1.cpu().numpy().astype(np.float64) * rd3
        mix = (alpha, float(np.std(h[:, 0])), float(np.mean(h[:, 0])), float(np.std(h[:, 1])),
               float(np.mean(h[:, 1])))
        s2, l2 = vg.search_device(spec, qdata, qvec, "prob", 0.0, mats, probs=qprobs, mix=mix, dev=dev, opts=opts)
        top = [int(t) for t in vg.topn_device(s2, w["N"], column=2, dev=dev).cpu().numpy() if t >= 0]
        ref = vg.refine_angle_list([angles[t] for t in top])
        rs, rl = vg.search_device(spec, qdata, qvec, "prob", 0.0, dev.to_dev(vg.rot_matrices(ref)), probs=qprobs,
                                  mix=mix, dev=dev, opts=opts)
        rtop = [int(t) for t in vg.topn_device(rs, w["N"], column=2, dev=dev).cpu().numpy() if t >= 0]
        return s1, s2, top, rtop

    out = {}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev.device)
    for path in (-1, 3):
        for _ in range(args.warmup):
            res = step(path)
        torch.cuda.synchronize()
        clk = ClockSampler(local)
        clk.start()
        total = 0.0
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            res = step(path)
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        out[path] = (total / args.steps, res, clk.stop())
    ms, (s1, s2, top, rtop), clocks = out[-1]
    ms3, (t1, t2, ttop, trtop), _ = out[3]
    a1, b1 = s1.cpu().numpy().astype(np.float64), t1.cpu().numpy().astype(np.float64)
    a2, b2 = s2.cpu().numpy().astype(np.float64), t2.cpu().numpy().astype(np.float64)
    rel = lambda x, y: float(np.max(np.abs(x - y)) / max(np.max(np.abs(x)), 1e-300))
    line = {
        "metric": "prob-mode map-pair alignments/s", "value": round(1e3 / ms, 4), "unit": "alignments/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 FFT (f64 target spectra); split-BF16 pass B in the comparison",
        "data": "synthetic (seeded 128^3 / 64^3 blob-map pair at 1 A, 4 Dirichlet(0.5) probability channels)",
        "config": {"workload": f"prob128_s3_a15: one pair per step, s={s_}, grids padded to {d}^3, A={w['A']} "
                               f"({n} rotations, statistics pass + mixed pass) + refinement, alpha={alpha}, "
                               f"g={g}, N={w['N']}; fastVEC of the densities and the 8 probability maps in the step",
                   "grid_side": d, "l2": "flushed before every step (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "split_bf16_pass_b": {"value": round(1e3 / ms3, 4), "ms_per_step": round(ms3, 3),
                              "max_rel_diff_vs_f32": {"vec_score": rel(a1[:, 0], b1[:, 0]),
                                                      "prob_score": rel(a1[:, 1], b1[:, 1]),
                                                      "mixed_score": rel(a2[:, 2], b2[:, 2])},
                              "top_n_same": top == ttop, "refined_top_n_same": rtop == trtop},
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)




def cpu_baseline(args, threads, budget_s):
    """The reference algorithm on this host's CPU (the oracle restatement,
    exhaustive search like the reference), timed on a bounded sample and
    scaled to one full alignment."""
    from oracle import vesper_oracle as orc
    from vesper_python_gb300 import synth
    w = synth.WORKLOADS[args.workload]
    if args.workload == "prop128_s3_a10":
        pair = synth.make_pair(HELD_OUT_SEED0, w["side1"], w["nblob"], w["radius"])
    else:
        pair = synth.workload_pair(args.workload, seed=0)
    m1 = orc.OMap(pair.map1, 1.0, pair.orig1)
    m2 = orc.OMap(pair.map2, 1.0, pair.orig2)
    d1, o1, c1, _ = orc.set_vox_size(m1, w["t"], w["s"])
    d2, o2, c2, _ = orc.set_vox_size(m2, w["T"], w["s"])
    dim, o1, o2 = orc.unify(d1, o1, c1, d2, o2, c2, w["s"])
    rng = np.random.default_rng(0)
    nvox = dim ** 3
    nsamp = 600 if threads == 1 else 600 * threads
    # fastVEC sample: random destination voxels of both maps
    t_fv = 0.0
    for m, o in ((m1, o1), (m2, o2)):
        idx = rng.choice(nvox, size=min(nsamp, nvox), replace=False)
        t0 = time.perf_counter()
        orc.fastvec(m.data, np.float64(m.xwidth), m.orig.astype(np.float64), dim, w["s"], o, w["g"], idx=idx,
                    nthreads=threads)
        t_fv += (time.perf_counter() - t0) * nvox / len(idx)
    # search sample: the rotation loop on real fields
    data1, vec1 = orc.fastvec(m1.data, np.float64(m1.xwidth), m1.orig.astype(np.float64), dim, w["s"], o1, w["g"],
                              idx=np.arange(0), nthreads=threads)
    rngv = np.random.default_rng(1)
    vec1 = rngv.normal(size=vec1.shape).astype(np.float32)
    data2 = np.where(rngv.random((dim,) * 3) < 0.3, rngv.uniform(0.5, 2, (dim,) * 3), 0.0)
    vec2 = rngv.normal(size=vec1.shape).astype(np.float32)
    ts = orc.target_spectra(orc.mode_field("V", data1, vec1))
    angles = orc.calc_angle_comb(w["A"])
    R = len(angles) + 10 * 27
    t0 = time.perf_counter()
    n = 0
    while True:
        orc.rot_and_search(ts, "V", data2, vec2, angles[n * 997 % len(angles)], 0.0, workers=threads)
        n += 1
        if time.perf_counter() - t0 > budget_s * 0.5 or n >= 200:
            break
    t_rot = (time.perf_counter() - t0) / n
    total = t_fv + R * t_rot
    return {"value": round(1.0 / total, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{args.workload}: fastVEC on {nsamp} random voxels per map (scaled to {nvox}), exhaustive "
                      f"search on {n} rotations (scaled to {R}); {t_fv:.1f} s fastVEC + {R * t_rot:.1f} s search "
                      f"per alignment",
            "seconds_per_alignment": round(total, 2)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(args, threads=threads, budget_s=4.0)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 / v, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (CPU)",
            "data": "synthetic (seeded blob-map pairs at 1 A)",
            "config": {"workload": f"{args.workload}: CPU restatement of the reference path (exhaustive search), "
                                   f"mode {args.mode}"},
            "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": cb["sample"]},
            "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "uneven64_s4_a15":
        run_uneven(a)
    elif a.workload == "prob128_s3_a15":
        run_prob(a)
    else:
        run_gb300(a)
