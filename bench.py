"""Benchmark: map-pair alignments per second on GB300.

One alignment = the work of ``main.py orig`` on one map pair (threshold and
grid sizing, fastVEC of both maps, target spectra, the rotational search,
top-N, the +-5 degree refinement, the rotated top-N models and their float64
scores), on seeded synthetic maps.

Headline workload ``prop128_s3_a10``: 128^3 / 64^3 blob-map pairs (the
128^3/64^3 generator) at s = 3, A = 10 (24624 rotations), each aligned with the
learned rotation proposal (the committed network ranks the grid, the exact
search correlates the best 5%, the exhaustive search is the fallback).  A
step aligns a batch of held-out pairs (seeds outside the training range).
The same pairs are also aligned with the exhaustive search: the line reports
both rates and the fraction of pairs whose top-1 rotation the two forms
agree on.  A step runs ``Aligner.align_many`` over its pairs with
graph=True: the global stage (fastVEC, spectra, proposal, global search of
every pair) and the refinement + rescoring stage each replay as one CUDA
graph, captured in the warm-up for the batch's shapes (every kernel of the
step still runs each step).  The line also reports the same steps with
eager launches (``eager``; ``--eager`` makes that the headline).

At one GPU the same line carries, under ``configs``, the other benchmarked
configurations, each with its own device-timed value, end-to-end value, FP32
roofline and CPU baseline (at most 5 timed steps after 3 warm-up steps):

  pair200_s2_a10   one 200^3 / 100^3 pair per step, s = 2, A = 10 (side 75),
                   exhaustive, modes V, O, C, P and L
  uneven64_s4_a15  64 pairs of uneven sizes per step, s = 4, A = 15, global
                   stage as one CUDA graph, per-pair latency p50 / p99
  prob128_s3_a15   prob-mode alignment of one 128^3 / 64^3 pair with four
                   probability channels, grids padded to 64^3, A = 15, with
                   the float32 and the split-BF16 pass B, errors of both
                   against a float64 restatement

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
  python bench.py --workload pair200_s2_a10 [--mode V|O|C|P|L]   (one config alone)
  python bench.py --case <name> [arg]                              (profiling case)

``value``: device-resident maps, K steps timed with CUDA events between a
barrier + synchronize on both sides, whole-job alignments/s (max over ranks).
``e2e``: the same steps through the host entry points with the maps copied
from pinned host memory every step and the results read back.
Roofline: FP32 CUDA-core throughput of the dominant search pass, algorithmic
FLOPs (a real 3-D FFT of N points is 2.5 N log2 N, split evenly over its
three axes; 8 flops per channel and half-spectrum element for the product)
over the pass's device time, against the FP32 FMA rate measured here.
``--impl reference``: the reference algorithm's CPU path on this host's cores
(the oracle restatement: C fastVEC single-threaded as the reference's serial
numba loop, numpy whole-array gather and scipy FFTs with every core as the
reference's threaded FFTW plans), exhaustive like the reference, timed on a
bounded sample of the headline workload's first pair and scaled to a full
alignment.
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
EVAL_SEED0, EVAL_PAIRS = 10_000_000, 200   # held-out recall set
SUB_STEPS, SUB_WARMUP = 5, 3    # timed / warm-up steps of each sub-configuration
MODE_NAMES = {"V": "VecProduct", "O": "Overlap", "C": "CC", "P": "PCC", "L": "Laplacian"}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per rotation of the
# dominant search kernel (search pass A), mode V, by grid side, from ncu
# captures of ``bench.py --case search<d> <nrot> <batch>`` at the batches the
# workloads run (256 rotations per launch at sides 28-32, 128 at 75), caches
# left as the previous launches leave them (profiles/search_pass_a_dram.md).
PASS_A_DRAM_PER_ROT = {28: 264845, 30: 266378, 32: 290951, 75: 4726406}


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
    ap.add_argument("--no-configs", action="store_true",
                    help="headline only (no pair200 / uneven64 / prob128 sub-objects)")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--no-exhaustive", action="store_true",
                    help="skip the exhaustive form on the same pairs (profiling runs)")
    ap.add_argument("--eager", action="store_true",
                    help="headline value with eager launches instead of the CUDA graphs")
    ap.add_argument("--no-graph-replay", action="store_true",
                    help="skip the second form's measurement (eager, or graphs with --eager; profiler lists)")
    ap.add_argument("--sub-config", action="store_true",
                    help="run --workload as a sub-configuration of the default line (its steps capped at "
                         f"{SUB_STEPS} after {SUB_WARMUP} warm-up) and print its object")
    ap.add_argument("--profile-step", action="store_true",
                    help="run one more step of the headline form between cudaProfilerStart and cudaProfilerStop "
                         "(for ncu --profile-from-start off: a launch list of exactly one step)")
    ap.add_argument("--case", nargs="+", default=None, metavar="NAME",
                    help="run one small profiling case of bench_cases.py instead of a workload")
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


# ---------------------------------------------------------------------------
# roofline: algorithmic FLOPs of the search passes and the measured FP32 rate
# ---------------------------------------------------------------------------

def channels(code):
    """(forward channels, inverse volumes) of a search: V 3/1, O/C/P/L 1/1,
    prob 7/2 (vector and probability volumes, both needed in either pass)."""
    if code == 0:
        return 3, 1
    if code == 5:
        return 7, 2
    return 1, 1


def pass_flops(dim, code):
    """Algorithmic FLOPs per rotation of each search pass: FLOP_rot =
    (C_fwd + C_inv) 2.5 N log2 N + 8 C_fwd Nh + N split over pass A (forward z
    and y axes), pass B (forward x axis, product, inverse x axis) and pass C
    (inverse y and z axes, argmax compare)."""
    N = dim ** 3
    Nh = dim * dim * (dim // 2 + 1)
    cf, ci = channels(code)
    axis = 2.5 * N * np.log2(dim)      # one axis of one real 3-D transform
    a = cf * 2 * axis
    b = cf * axis + 8 * cf * Nh + ci * axis
    c = ci * 2 * axis + N
    return {"pass_a": a, "pass_b": b, "pass_c": c, "search": a + b + c}


_FP32_PEAK = {}


def fp32_peak(dev):
    """Measured FP32 FMA rate of this GPU (TFLOP/s) and its SM count:
    vesper_fp32_peak_probe over 8 blocks of 256 threads per SM, best of 5
    timed launches."""
    import ctypes

    import torch
    from vesper_python_gb300 import _native
    if dev.device in _FP32_PEAK:
        return _FP32_PEAK[dev.device]
    sms = torch.cuda.get_device_properties(dev.device).multi_processor_count
    out = torch.zeros(sms * 8, dtype=torch.float32, device=dev.device)
    flops = ctypes.c_double(0)
    best = 0.0
    for i in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _native.check(dev.lib.vesper_fp32_peak_probe(sms * 8, 256, 4096, ctypes.c_void_p(out.data_ptr()),
                                                     ctypes.byref(flops), dev.stream))
        e1.record()
        torch.cuda.synchronize()
        if i:
            best = max(best, flops.value / (e0.elapsed_time(e1) / 1e3) / 1e12)
    _FP32_PEAK[dev.device] = (best, sms)
    return best, sms


def search_roofline(prof, dev, clocks, kernels):
    """FP32 roofline of the dominant search pass from a profiled step.
    ``prof`` holds the summed device time and launch count of each pass and
    every profiled call's (side, mode code, rotations, mixed); ``kernels``
    names the kernel of each pass.  A fused search (one kernel per call) is
    reported as a whole."""
    names = ["pass_a", "pass_b", "pass_c"]
    flop = {k: 0.0 for k in names + ["search"]}
    rot_by_side = {}
    for (d, code, n, _mixed, path) in prof["calls"]:
        pf = pass_flops(d, code)
        if path == 2:       # fused: the whole search runs in the pass-A slot
            pf = {"pass_a": pf["search"], "pass_b": 0.0, "pass_c": 0.0, "search": pf["search"]}
        for k in flop:
            flop[k] += pf[k] * n
        rot_by_side[d] = rot_by_side.get(d, 0) + n
    ms = prof["pass_ms"][:3]
    nl = prof["pass_launches"][:3]
    fused = nl[1] == 0 and nl[2] == 0
    top = 0 if fused else int(np.argmax(ms))
    k = "search" if fused else names[top]
    peak, sms = fp32_peak(dev)
    sm_mhz = clocks.get("sm_mhz") or 0.0
    nominal = sms * 128 * 2 * sm_mhz * 1e6 / 1e12 if sm_mhz else None
    t_top = ms[top] / 1e3
    ach = flop[k] / t_top / 1e12 if t_top > 0 else 0.0
    t_all = sum(ms) / 1e3
    # DRAM bytes per launch of pass A: the measured bytes per rotation at the
    # searched sides times the rotations of an average launch (mode V; null
    # when a searched side or mode has no capture)
    traffic = None
    codes = {c for (_d, c, _n, _m, _p) in prof["calls"]}
    if not fused and top == 0 and codes == {0} and all(d in PASS_A_DRAM_PER_ROT for d in rot_by_side):
        traffic = int(round(sum(PASS_A_DRAM_PER_ROT[d] * n for d, n in rot_by_side.items()) / max(1, nl[0])))
    return {
        "bound": "fp32", "kernel": f"search {k} ({kernels.get(k, k)})",
        "achieved": round(ach, 3), "peak": round(peak, 2), "unit": "TFLOP/s", "frac": round(ach / peak, 4),
        "traffic": traffic, "traffic_unit": "DRAM bytes per launch",
        "peak_source": f"measured FP32 FMA rate ({sms} SMs, vesper_fp32_peak_probe)",
        "nominal_tflops_at_sampled_clock": round(nominal, 1) if nominal else None,
        "flop_per_launch": round(flop[k] / max(1, nl[top])),
        "launches": int(nl[top]), "ms": round(ms[top], 3),
        "whole_search": {"achieved": round(flop["search"] / t_all / 1e12, 3) if t_all > 0 else 0.0,
                         "frac": round(flop["search"] / t_all / 1e12 / peak, 4) if t_all > 0 else 0.0,
                         "ms": round(sum(ms), 3)},
        "rotations_by_side": {str(d): n for d, n in sorted(rot_by_side.items())},
    }


def kernel_names(dev, dim, mode):
    from vesper_python_gb300 import vesper as vg
    path = vg.search_plan(dim, mode, 0, 1, None, dev)[0]
    if path == 2:
        return {"search": "k_fused"}
    pre = "k_rpass_" if path == 1 else "k_pass_"
    return {"pass_a": pre + "a", "pass_b": pre + "b", "pass_c": pre + "c"}


# ---------------------------------------------------------------------------
# the headline: learned proposal vs exhaustive on the 128^3 / 64^3 pairs
# ---------------------------------------------------------------------------

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


def _host_pair(item):
    """A synth.MapPair of host copies of one (map1, map2, w1, w2, orig1,
    orig2) item."""
    from vesper_python_gb300 import synth
    return synth.MapPair(item[0].cpu().numpy(), item[1].cpu().numpy(), np.asarray(item[4], np.float64),
                         np.asarray(item[5], np.float64), float(item[2]), None, None)


def _gpu_fields(al, item, p):
    """Host copies of one pair's coarse fields (target data/vec, query
    data/vec, the target's fastVEC average) as the device path computes
    them: the inputs of a CPU baseline's search sample."""
    res = al.align_many([item], p)
    fl = al.last_fields[0]
    out = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in fl.items()}
    out["dim"] = res[0].dim
    return out


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
    mode = MODE_NAMES[args.mode]
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

    headline_graph = not args.eager
    graph = headline_graph

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

    # the same steps in the other form (eager launches, or the CUDA graphs
    # with --eager); graphs are captured in the warm-up for this batch's shapes
    # and geometry (a batch of new maps with other geometry captures again)
    ms_alt = None
    if not args.no_graph_replay:
        graph = not headline_graph
        ms_alt, _, _, _ = timed(p)
    graph = headline_graph
    ms, res, launches, clocks = timed(p)
    if args.profile_step:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        step(p)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    npairs = len(pairs)
    value = world * npairs * args.steps / (ms / 1e3)
    value_alt = world * npairs * args.steps / (ms_alt / 1e3) if ms_alt else None
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
    stages_graph = {}
    if not args.no_graph_replay or headline_graph:
        al.stages = stages_graph     # the same in the graph form: the two replays and the host work around them
        al.align_many(dev_items, p, graph=True)
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
        al.align_host_many(host_items, params, graph=headline_graph)
        return al.d2h_bytes

    def timed_host(params):
        host_step(params)
        barrier()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        d2h = 0
        for _ in range(args.steps):
            d2h += host_step(params)
        t1.record()
        barrier()
        return maxr(t0.elapsed_time(t1)), d2h

    e2e_ms, d2h = timed_host(p)
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
        e2e_x, d2h_x = timed_host(p_exh)
        exh = {"value": round(world * npairs * args.steps / (ms_x / 1e3), 4), "unit": UNIT,
               "ms_per_step": round(ms_x / args.steps, 3),
               "e2e": {"value": round(world * npairs * args.steps / (e2e_x / 1e3), 4), "unit": UNIT,
                       "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(d2h_x / args.steps)},
               "top1_agreement": agree / npairs, "refined_model1_agreement": agree_model / npairs,
               "proposal_speedup": round(ms_x / ms, 3), "proposal_fallbacks_per_step": fallbacks}
    dims = sorted({r.dim for r in res})
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    roof = search_roofline(prof, dev, clocks, kernel_names(dev, res[0].dim, mode))
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
        "config": {"workload": wl, "grid_sides": dims, "pairs_per_step": npairs,
                   "rotations": len(vg.calc_angle_comb(p.A)),
                   "l2": "flushed before every step (256 MB write)", "parallelism": f"replicas x{world}",
                   "form": ("CUDA graphs: global stage, then refinement + rescoring, replayed every step "
                            "(captured in the warm-up for this batch's shapes)") if headline_graph else
                           "eager launches"},
        ("eager" if headline_graph else "graphs"): {"value": round(value_alt, 4), "unit": UNIT,
                                                    "ms_per_step": round(ms_alt / args.steps, 3)}
        if value_alt else None,
        "e2e": {"value": round(e2e_value, 4), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(d2h / args.steps)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "stage_ms_profiled_step": {k: round(v, 3) for k, v in stages.items()},
        "stage_ms_graph_step": {k: round(v, 3) for k, v in stages_graph.items()},
        "profiled_step_note": "one eager step with events at stage boundaries; one graph-form step with events "
                              "between its two replays; one with events around every search launch (global "
                              "searches)",
        "pass_ms_profiled_step": [round(x, 3) for x in prof["pass_ms"]],
        "clocks": clocks,
    }
    if exh is not None:
        line["exhaustive"] = exh
    if world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline_exhaustive(args.workload, args.mode, 10.0, _host_pair(dev_items[0]),
                                     fields=_gpu_fields(al, dev_items[0], p_exh))
        line["cpu_baseline"] = cb
        if exh is not None:
            exh["vs_cpu_baseline"] = round(exh["value"] / cb["value"], 1)
            exh["e2e_vs_cpu_baseline"] = round(exh["e2e"]["value"] / cb["value"], 1)
    if world == 1 and use_prop and not args.no_exhaustive:
        # held-out recall of the committed network on a fixed seeded set (the
        # evaluation seeds, disjoint from training and from the bench pairs)
        ev, _ = proposal.evaluate(dev, net, list(range(EVAL_SEED0, EVAL_SEED0 + EVAL_PAIRS)),
                                  vg.rot_matrices_device(vg.calc_angle_comb(p.A), dev, key=("grid", float(p.A))),
                                  frac=p.proposal_frac, N=p.N, fallback_z=p.proposal_fallback_z)
        line["recall"] = {"pairs": ev["pairs"], "top1_agreement": ev["top1_agreement"],
                          "top10_recall": round(ev["topN_recall"], 5), "fallback_rate": ev["fallback_rate"],
                          "winner_in_subset": ev["winner_in_subset_net"],
                          "max_score_rel_err_when_agreeing": ev["max_score_rel_err_when_agreeing"],
                          "seeds": f"{EVAL_SEED0}..{EVAL_SEED0 + EVAL_PAIRS - 1} (held out)"}
    if world == 1 and use_prop and not args.no_configs:
        del flush, al
        torch.cuda.empty_cache()
        line["configs"] = {
            "pair200_s2_a10": config_pair200(args, dev),
            "uneven64_s4_a15": run_sub_process(args, "uneven64_s4_a15"),
            "prob128_s3_a15": run_sub_process(args, "prob128_s3_a15"),
        }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_sub_process(args, workload):
    """One sub-configuration in a fresh process (``--sub-config``): its
    timings do not inherit this process's allocations, graphs and threads.
    Returns its JSON object (or the error)."""
    import subprocess
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", workload, "--steps", str(args.steps),
           "--warmup", str(args.warmup), "--sub-config"]
    if args.no_cpu_baseline:
        cmd.append("--no-cpu-baseline")
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE")}
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"error": f"exit {r.returncode}: " + (r.stderr.strip().splitlines() or ["no output"])[-1][:300]}
    return json.loads(lines[-1])


# ---------------------------------------------------------------------------
# configuration 1: the 200^3 / 100^3 pair, all five modes
# ---------------------------------------------------------------------------

def config_pair200(args, dev):
    import torch

    from vesper_python_gb300 import align, synth
    w = synth.WORKLOADS["pair200_s2_a10"]
    pr = synth.workload_pair("pair200_s2_a10", seed=0)
    items = [(dev.to_dev(pr.map1), dev.to_dev(pr.map2), pr.width, pr.width, pr.orig1, pr.orig2)]
    h1, h2 = torch.from_numpy(pr.map1).pin_memory(), torch.from_numpy(pr.map2).pin_memory()
    host_items = [(h1, h2, pr.width, pr.width, pr.orig1, pr.orig2)]
    h2d = int(h1.numel() * 4 + h2.numel() * 4)
    al = align.Aligner(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev.device)
    steps, warmup = min(args.steps, SUB_STEPS), SUB_WARMUP
    out = {"config": {"workload": "pair200_s2_a10: one pair per step, map1 200^3 / map2 100^3 (1500 blobs, 70 A "
                                  "sphere), s=2, A=10 (24624 rotations + refinement), g=16, N=10, exhaustive; "
                                  "headline fields from mode V; CUDA graphs per step (modes CC and PCC: eager, "
                                  "their spectra need a host value)",
                      "l2": "flushed before every step (256 MB write)"},
           "steps": steps, "warmup": warmup, "unit": UNIT, "modes": {}}
    fields_v = None
    for m in "VOCPL":
        p = align.AlignParams(t=w["t"], T=w["T"], g=w["g"], s=w["s"], A=w["A"], N=w["N"], mode=MODE_NAMES[m])
        for _ in range(warmup):
            flush.zero_()
            al.align_many(items, p, graph=True)
        torch.cuda.synchronize()
        clk = ClockSampler(torch.cuda.current_device())
        clk.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        total, launches = 0.0, 0
        for _ in range(steps):
            flush.zero_()
            e0.record()
            res = al.align_many(items, p, graph=True)
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
            launches += al.launches
        clocks = clk.stop()
        prof = {}
        al.profile = prof
        al.align_many(items, p)
        torch.cuda.synchronize()
        al.profile = None
        ms = total / steps
        ent = {"value": round(1e3 / ms, 4), "ms_per_step": round(ms, 3), "gpu_launches_per_step": launches // steps,
               "grid_side": res[0].dim,
               "roofline": search_roofline(prof, dev, clocks, kernel_names(dev, res[0].dim, MODE_NAMES[m])),
               "pass_ms_profiled_step": [round(x, 3) for x in prof["pass_ms"]], "clocks": clocks}
        if m == "V":
            al.align_host_many(host_items, p, graph=True)
            torch.cuda.synchronize()
            e0.record()
            d2h = 0
            for _ in range(steps):
                flush.zero_()
                al.align_host_many(host_items, p, graph=True)
                d2h += al.d2h_bytes
            e1.record()
            torch.cuda.synchronize()
            ent["e2e"] = {"value": round(1e3 / (e0.elapsed_time(e1) / steps), 4), "unit": UNIT,
                          "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(d2h / steps)}
            fields_v = _gpu_fields(al, items[0], p)
        out["modes"][m] = ent
    v = out["modes"]["V"]
    out.update({"value": v["value"], "ms_per_step": v["ms_per_step"], "e2e": v["e2e"], "roofline": v["roofline"],
                "gpu_launches": v["gpu_launches_per_step"] * steps, "clocks": v["clocks"]})
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_exhaustive("pair200_s2_a10", "V", 8.0, pr, fields=fields_v)
        out["vs_cpu_baseline"] = round(out["value"] / out["cpu_baseline"]["value"], 1)
        out["e2e_vs_cpu_baseline"] = round(out["e2e"]["value"] / out["cpu_baseline"]["value"], 1)
    return out


# ---------------------------------------------------------------------------
# configuration 2: 64 pairs of uneven sizes
# ---------------------------------------------------------------------------

def run_uneven(args, sub=False):
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
    steps = min(args.steps, SUB_STEPS) if sub else args.steps
    warmup = SUB_WARMUP if sub else args.warmup
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
    ms, lat, launches, res = timed(True, steps, warmup)
    clocks = clk.stop()
    ms_ng, lat_ng, _, res_ng = timed(False, max(1, steps), 1)
    same = all(a.top == b.top and [m.dot_score for m in a.models] == [m.dot_score for m in b.models]
               for a, b in zip(res, res_ng))
    prof = {}
    al.profile = prof
    al.align_many(items, p)
    torch.cuda.synchronize()
    al.profile = None
    # e2e: maps copied from pinned host memory every step
    al.align_host_many(host_items, p, True)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    d2h = 0
    for _ in range(steps):
        flush.zero_()
        al.align_host_many(host_items, p, True)
        d2h += al.d2h_bytes
    t1.record()
    torch.cuda.synchronize()
    e2e_ms = t0.elapsed_time(t1) / steps
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
    # pass roofline over the whole batch (every side's register / radix-pass
    # searches; the fused sides' time counts in whole_search only)
    roof = search_roofline(prof, dev, clocks, {"pass_a": "k_rpass_a / k_pass_a", "pass_b": "k_rpass_b / k_pass_b",
                                               "pass_c": "k_rpass_c / k_pass_c", "search": "k_fused"})
    line = {
        "metric": METRIC, "value": round(n / (ms / 1e3), 4), "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
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
                "d2h_bytes_per_step": int(d2h / steps)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_uneven(items, sides, budget_s=8.0)
        line["vs_cpu_baseline"] = round(line["value"] / line["cpu_baseline"]["value"], 1)
        line["e2e_vs_cpu_baseline"] = round(line["e2e"]["value"] / line["cpu_baseline"]["value"], 1)
    if sub:
        for k in ("metric", "n_gpus", "higher_is_better", "scaling", "vs_baseline"):
            line.pop(k)
        return line
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# configuration 3: prob mode at side 64, float32 vs split-BF16 vs float64
# ---------------------------------------------------------------------------

def run_prob(args, sub=False):
    """prob128_s3_a15: one 128^3 / 64^3 pair with four probability channels
    per step (Dirichlet(0.5) inside the thresholded density, rotated with map2),
    s = 3, grids padded to 64^3, A = 15 (7,488 rotations), alpha = 0.5.  A step
    is the prob-mode alignment on the device: fastVEC of the two densities and
    the eight probability maps, target spectra, the statistics pass and the
    mixed pass over the grid, top-N, and the mixed pass over the refinement
    set.  Timed with the float32 pass B (headline) and with the split-BF16
    tensor-core pass B (search path 3); the line reports both, how far each
    form's scores are from a float64 restatement (the oracle with float64
    FFTs, same gather) on a sample of rotations, and the end-to-end rate with
    the maps and probability channels copied from pinned host memory and the
    refined scores read back every step."""
    import contextlib
    import io

    import torch

    from vesper_python_gb300 import synth
    from vesper_python_gb300 import vesper as vg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = vg.Device(f"cuda:{local}")
    steps = min(args.steps, SUB_STEPS) if sub else args.steps
    warmup = SUB_WARMUP if sub else args.warmup
    w = synth.WORKLOADS["prob128_s3_a15"]
    pr = synth.workload_pair("prob128_s3_a15", seed=rank)
    d, s_, g = int(w["pad"]), float(w["s"]), float(w["g"])
    geo = []
    host_maps = []
    for src, orig, th in ((pr.map1, pr.orig1, w["t"]), (pr.map2, pr.orig2, w["T"])):
        m = vg.mrc_obj.from_array(src, 1.0, orig)
        with contextlib.redirect_stdout(io.StringIO()):
            _, mn = vg.mrc_set_vox_size(m, th, s_)
        host_maps.append(torch.from_numpy(np.ascontiguousarray(m.data, np.float32)).pin_memory())
        geo.append((dev.to_dev(m.data), np.float64(m.xwidth), m.orig.astype(np.float64),
                    np.asarray(mn.cent, np.float64) - 0.5 * s_ * d))
    host_probs = [torch.from_numpy(np.ascontiguousarray(np.moveaxis(pm, 3, 0), np.float32)).pin_memory()
                  for pm in (pr.prob1, pr.prob2)]
    pmaps = [[dev.to_dev(np.ascontiguousarray(pm[..., k], np.float32)) for k in range(4)]
             for pm in (pr.prob1, pr.prob2)]
    angles = vg.calc_angle_comb(w["A"])
    mats = vg.rot_matrices_device(angles, dev, key=("grid", float(w["A"])))
    n = len(angles)
    rd3 = 1.0 / d ** 3
    alpha = float(w["alpha"])
    dsrc = [torch.empty_like(geo[i][0]) for i in range(2)]
    dprob = [torch.empty(tuple(host_probs[i].shape), dtype=torch.float32, device=dev.device) for i in range(2)]

    def fields(i, from_host):
        # prob mode keeps fastVEC's density in float32 (main.py:345)
        src, sw, so, no = geo[i]
        pm = pmaps[i]
        if from_host:
            dsrc[i].copy_(host_maps[i], non_blocking=True)
            dprob[i].copy_(host_probs[i], non_blocking=True)
            src, pm = dsrc[i], [dprob[i][k] for k in range(4)]
        _, d32, vec = vg.fastvec_device(src, sw, so, d, s_, no, g, dev=dev)
        probs = torch.stack([vg.fastvec_device(p_, sw, so, d, s_, no, g, dev=dev)[1] for p_ in pm])
        return d32.double(), vec, probs

    def step(path, from_host=False, prof=None):
        opts = (path, 0, 0)
        tdata, tvec, tprobs = fields(0, from_host)
        qdata, qvec, qprobs = fields(1, from_host)
        spec = vg.target_spectra_device(tdata, tvec, "prob", 0.0, probs=tprobs, dev=dev)
        s1, _ = vg.search_device(spec, qdata, qvec, "prob", 0.0, mats, probs=qprobs, dev=dev, opts=opts,
                                 profile=prof)
        h = s1.cpu().numpy().astype(np.float64) * rd3
        mix = (alpha, float(np.std(h[:, 0])), float(np.mean(h[:, 0])), float(np.std(h[:, 1])),
               float(np.mean(h[:, 1])))
        s2, l2 = vg.search_device(spec, qdata, qvec, "prob", 0.0, mats, probs=qprobs, mix=mix, dev=dev, opts=opts,
                                  profile=prof)
        top = [int(t) for t in vg.topn_device(s2, w["N"], column=2, dev=dev).cpu().numpy() if t >= 0]
        ref = vg.refine_angle_list([angles[t] for t in top])
        rs, rl = vg.search_device(spec, qdata, qvec, "prob", 0.0, dev.to_dev(vg.rot_matrices(ref)), probs=qprobs,
                                  mix=mix, dev=dev, opts=opts, profile=prof)
        rtop = [int(t) for t in vg.topn_device(rs, w["N"], column=2, dev=dev).cpu().numpy() if t >= 0]
        rsc = rs[rtop].cpu().numpy()          # the refined models' scores (read back)
        return s1, s2, top, rtop, mix, rsc, (tdata, tvec, tprobs, qdata, qvec, qprobs)

    out = {}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev.device)
    for path in (-1, 3):
        for _ in range(warmup):
            res = step(path)
        torch.cuda.synchronize()
        clk = ClockSampler(local)
        clk.start()
        total = 0.0
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            res = step(path)
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        out[path] = (total / steps, res, clk.stop())
    ms, (s1, s2, top, rtop, mix, _, flds), clocks = out[-1]
    ms3, (t1, t2, ttop, trtop, _, _, _), _ = out[3]
    # end to end: maps and probability channels from pinned host memory
    step(-1, from_host=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        flush.zero_()
        step(-1, from_host=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / steps
    h2d = int(sum(t.numel() * 4 for t in host_maps + host_probs))
    # statistics-pass scores, both top-N lists, the refined models' scores
    d2h = int(n * 2 * 4 + 2 * w["N"] * 4 + w["N"] * 3 * 4)
    prof = {}
    step(-1, prof=prof)
    torch.cuda.synchronize()
    roof = search_roofline(prof, dev, clocks, kernel_names(dev, d, "prob"))
    a1, b1 = s1.cpu().numpy().astype(np.float64), t1.cpu().numpy().astype(np.float64)
    a2, b2 = s2.cpu().numpy().astype(np.float64), t2.cpu().numpy().astype(np.float64)
    rel = lambda x, y: float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))
    line = {
        "metric": "prob-mode map-pair alignments/s", "value": round(1e3 / ms, 4), "unit": "alignments/s",
        "n_gpus": world, "steps": steps, "warmup": warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 FFT (f64 target spectra); split-BF16 pass B in the comparison",
        "data": "synthetic (seeded 128^3 / 64^3 blob-map pair at 1 A, 4 Dirichlet(0.5) probability channels)",
        "config": {"workload": f"prob128_s3_a15: one pair per step, s={s_}, grids padded to {d}^3, A={w['A']} "
                               f"({n} rotations, statistics pass + mixed pass) + refinement, alpha={alpha}, "
                               f"g={g}, N={w['N']}; fastVEC of the densities and the 8 probability maps in the step",
                   "grid_side": d, "l2": "flushed before every step (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(1e3 / e2e_ms, 4), "unit": "alignments/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": roof,
        "split_bf16_pass_b": {"value": round(1e3 / ms3, 4), "ms_per_step": round(ms3, 3),
                              "max_rel_diff_vs_f32": {"vec_score": rel(b1[:, 0], a1[:, 0]),
                                                      "prob_score": rel(b1[:, 1], a1[:, 1]),
                                                      "mixed_score": rel(b2[:, 2], a2[:, 2])},
                              "top_n_same": top == ttop, "refined_top_n_same": rtop == trtop},
        "vs_fp64": prob_fp64_errors(flds, angles, mix, a1, b1, a2, b2),
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_prob(flds, geo, pmaps, d, s_, g, n, budget_s=8.0)
        line["vs_cpu_baseline"] = round(line["value"] / line["cpu_baseline"]["value"], 1)
        line["e2e_vs_cpu_baseline"] = round(line["e2e"]["value"] / line["cpu_baseline"]["value"], 1)
    if sub:
        for k in ("metric", "n_gpus", "higher_is_better", "scaling", "vs_baseline"):
            line.pop(k)
        return line
    if rank == 0:
        print(json.dumps(line), flush=True)


def prob_fp64_errors(flds, angles, mix, a1, b1, a2, b2, nsample=12):
    """Errors of the float32 and split-BF16 scores against the oracle with
    float64 FFTs (same gather, same statistics) on ``nsample`` rotations
    spread over the grid, relative to the largest float64 score of each kind."""
    from oracle import vesper_oracle as orc
    td, tv, tp, qd, qv, qp = [t.cpu().numpy() for t in flds]
    tspec = orc.target_spectra([tv[..., 0], tv[..., 1], tv[..., 2]] + list(tp))
    sel = np.linspace(0, len(angles) - 1, nsample).astype(int)
    st = (mix[1], mix[2], mix[3], mix[4])
    r = [orc.rot_and_search_prob(tspec, qd.astype(np.float32), qv, list(qp), angles[i], mix[0], st, fp64=True)
         for i in sel]
    ref = np.array([[x[0], x[2], x[4]] for x in r], np.float64)
    out = {}
    for name, s_1, s_2 in (("f32", a1, a2), ("split_bf16", b1, b2)):
        got = np.stack([s_1[sel, 0], s_1[sel, 1], s_2[sel, 2]], axis=1)
        err = np.max(np.abs(got - ref), axis=0) / np.max(np.abs(ref), axis=0)
        out[name] = {"vec_score": float(err[0]), "prob_score": float(err[1]), "mixed_score": float(err[2])}
    out["rotations"] = int(nsample)
    out["note"] = "max |score - float64 score| / max |float64 score| over the sampled rotations"
    return out


# ---------------------------------------------------------------------------
# CPU baselines: the reference algorithm on the host cores (oracle port)
# ---------------------------------------------------------------------------

def _cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _fastvec_sample_seconds(src, width, orig, dim, s, dest_orig, g, nsamp, rng):
    """Single-threaded C fastVEC (the reference's serial numba loop) on
    ``nsamp`` random destination voxels, scaled to the whole grid."""
    from oracle import vesper_oracle as orc
    nvox = dim ** 3
    idx = rng.choice(nvox, size=min(nsamp, nvox), replace=False)
    t0 = time.perf_counter()
    orc.fastvec(src, np.float64(width), np.asarray(orig, np.float64), dim, s, dest_orig, g, idx=idx, nthreads=1)
    return (time.perf_counter() - t0) * nvox / len(idx)


def _search_rotation_seconds(mode, tdata, tvec, qdata, qvec, ave, angles, budget_s, threads, max_rot=200):
    """Average seconds per rotation of the reference's per-rotation work:
    numpy whole-array gather, scipy FFTs with ``threads`` workers (the
    reference's threaded FFTW plans), product, inverse, argmax."""
    from oracle import vesper_oracle as orc
    ts = orc.target_spectra(orc.mode_field(mode, tdata, tvec, ave))
    t0 = time.perf_counter()
    n = 0
    while True:
        F = orc.rot_matrix_f32(angles[n * 997 % len(angles)])
        nv, nd = orc.rot_mrc_numpy(qdata, qvec, F)
        orc.best_trans(orc.correlate(ts, orc.mode_field(mode, nd, nv, ave), workers=threads))
        n += 1
        if time.perf_counter() - t0 > budget_s or n >= max_rot:
            break
    return (time.perf_counter() - t0) / n, n


def _oracle_grid(w, pair):
    """Thresholded maps, the unified grid side and both grid origins."""
    from oracle import vesper_oracle as orc
    m1 = orc.OMap(pair.map1, pair.width, pair.orig1)
    m2 = orc.OMap(pair.map2, pair.width, pair.orig2)
    d1, o1, c1, _ = orc.set_vox_size(m1, w["t"], w["s"])
    d2, o2, c2, _ = orc.set_vox_size(m2, w["T"], w["s"])
    dim, o1, o2 = orc.unify(d1, o1, c1, d2, o2, c2, w["s"])
    return m1, o1, m2, o2, dim


def _oracle_fields(w, pair):
    """Coarse fields of a pair by the oracle (C fastVEC on every core)."""
    from oracle import vesper_oracle as orc
    m1, o1, m2, o2, dim = _oracle_grid(w, pair)
    data1, vec1 = orc.fastvec(m1.data, np.float64(m1.xwidth), m1.orig.astype(np.float64), dim, w["s"], o1, w["g"])
    data2, vec2 = orc.fastvec(m2.data, np.float64(m2.xwidth), m2.orig.astype(np.float64), dim, w["s"], o2, w["g"])
    return {"tdata": data1, "tvec": vec1, "qdata": data2, "qvec": vec2,
            "ave": float(np.mean(data1[data1 > 0])), "dim": dim}


def cpu_baseline_exhaustive(workload, mode_letter, budget_s, pair, fields=None):
    """One exhaustive alignment of ``pair`` on the CPU (oracle port):
    single-threaded fastVEC of both maps on random voxels, plus the rotation
    loop on the pair's real fastVEC fields with scipy FFT workers on every
    core, timed on a sample of rotations and scaled to the grid and the
    refinement set."""
    from oracle import vesper_oracle as orc
    from vesper_python_gb300 import synth
    w = synth.WORKLOADS[workload]
    threads = _cores()
    if fields is None:
        fields = _oracle_fields(w, pair)
    m1, o1, m2, o2, dim = _oracle_grid(w, pair)
    rng = np.random.default_rng(0)
    nsamp = 400
    t_fv = sum(_fastvec_sample_seconds(m.data, m.xwidth, m.orig, dim, w["s"], o, w["g"], nsamp, rng)
               for m, o in ((m1, o1), (m2, o2)))
    angles = orc.calc_angle_comb(w["A"])
    R = len(angles) + w["N"] * 27
    t_rot, n = _search_rotation_seconds(mode_letter, fields["tdata"], fields["tvec"], fields["qdata"],
                                        fields["qvec"], fields.get("ave", 0.0), angles, budget_s * 0.6, threads)
    total = t_fv + R * t_rot
    return {"value": round(1.0 / total, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{workload} first pair (grid side {dim}), mode {mode_letter}: fastVEC of both maps on "
                      f"{nsamp} random voxels each, 1 thread (the reference's serial numba loop), scaled to "
                      f"{dim ** 3} voxels; exhaustive search on the pair's real fastVEC fields, {n} rotations "
                      f"(numpy whole-array gather, scipy FFTs with {threads} workers), scaled to {R} rotations "
                      f"(grid + refinement); {t_fv:.1f} s fastVEC + {R * t_rot:.1f} s search per alignment",
            "seconds_per_alignment": round(total, 2)}


def cpu_baseline_uneven(items, sides, budget_s):
    """The uneven batch on the CPU (oracle port): every 8th pair's fastVEC
    (random voxels, 1 thread) and rotation loop (sampled, every core) timed
    and scaled to its own grid; the batch's time = 64 x their mean."""
    from oracle import vesper_oracle as orc
    from vesper_python_gb300 import synth
    w = synth.UNEVEN_WORKLOAD
    threads = _cores()
    rng = np.random.default_rng(0)
    angles = orc.calc_angle_comb(w["A"])
    R = len(angles) + w["N"] * 27
    per_pair = []
    sel = list(range(0, len(items), 8))
    for i in sel:
        pair = _host_pair(items[i])
        f = _oracle_fields(w, pair)
        m1, o1, m2, o2, dim = _oracle_grid(w, pair)
        t_fv = sum(_fastvec_sample_seconds(m.data, m.xwidth, m.orig, dim, w["s"], o, w["g"], 60, rng)
                   for m, o in ((m1, o1), (m2, o2)))
        t_rot, _ = _search_rotation_seconds("V", f["tdata"], f["tvec"], f["qdata"], f["qvec"], 0.0, angles,
                                            budget_s * 0.6 / len(sel), threads, max_rot=40)
        per_pair.append(t_fv + R * t_rot)
    total = len(items) * float(np.mean(per_pair))
    return {"value": round(len(items) / total, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"uneven64_s4_a15: {len(sel)} of the {len(items)} pairs (every 8th, map1 sides "
                      f"{[sides[i] for i in sel]}): fastVEC on 60 random voxels per map (1 thread) and the "
                      f"rotation loop on the pair's real fastVEC fields (numpy gather, scipy FFTs with {threads} "
                      f"workers), each scaled to its grid and {R} rotations; batch = {len(items)} x their mean "
                      f"({total:.0f} s)",
            "seconds_per_alignment": round(total / len(items), 2)}


def cpu_baseline_prob(flds, geo, pmaps, d, s_, g, nrot, budget_s):
    """The prob-mode alignment on the CPU (oracle port): fastVEC of the two
    densities and eight probability maps on random voxels (1 thread), and the
    per-rotation prob search (numpy gather with per-channel masks, 7 forward
    and 2 inverse scipy FFTs with every core) on the pair's real fields,
    sampled and scaled to both passes and the refinement set."""
    from oracle import vesper_oracle as orc
    threads = _cores()
    rng = np.random.default_rng(0)
    nsamp = 60
    t_fv = 0.0
    for i in range(2):
        src, sw, so, no = geo[i]
        t_fv += _fastvec_sample_seconds(src.cpu().numpy(), sw, so, d, s_, no, g, nsamp, rng)
        for pm in pmaps[i]:
            t_fv += _fastvec_sample_seconds(pm.cpu().numpy(), sw, so, d, s_, no, g, nsamp, rng)
    td, tv, tp, qd, qv, qp = [t.cpu().numpy() for t in flds]
    qd = qd.astype(np.float32)
    tspec = orc.target_spectra([tv[..., 0], tv[..., 1], tv[..., 2]] + list(tp))
    angles = orc.calc_angle_comb(15.0)
    t0 = time.perf_counter()
    n = 0
    while True:
        F = orc.rot_matrix_f32(angles[n * 997 % len(angles)])
        nv, nd, ps = orc.rot_mrc_numpy(qd, qv, F, list(qp))
        cv = orc.correlate(tspec[:3], [nv[..., 0], nv[..., 1], nv[..., 2]], workers=threads)
        cp = orc.correlate(tspec[3:], ps, workers=threads)
        orc.best_trans(cv)
        orc.best_trans(cp)
        n += 1
        if time.perf_counter() - t0 > budget_s * 0.6 or n >= 100:
            break
    t_rot = (time.perf_counter() - t0) / n
    R = 2 * nrot + 270
    total = t_fv + R * t_rot
    return {"value": round(1.0 / total, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"prob128_s3_a15: fastVEC of 2 densities + 8 probability maps on {nsamp} random voxels each "
                      f"(1 thread), scaled to {d}^3; prob rotation search on the pair's real fields, {n} rotations "
                      f"(numpy gather, 7 forward + 2 inverse scipy FFTs with {threads} workers), scaled to {R} "
                      f"(both passes + refinement); {t_fv:.1f} s fastVEC + {R * t_rot:.1f} s search per alignment",
            "seconds_per_alignment": round(total, 2)}


def run_reference(args):
    """The reference algorithm on this host's CPU cores (oracle port),
    exhaustive like the reference, on the headline workload's first pair:
    each step times a bounded sample and scales it to one alignment."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from vesper_python_gb300 import synth
    w = synth.WORKLOADS[args.workload]
    pair = synth.make_pair(HELD_OUT_SEED0, w["side1"], w["nblob"], w["radius"]) \
        if args.workload == "prop128_s3_a10" else synth.workload_pair(args.workload, seed=0)
    fields = _oracle_fields(w, pair)
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline_exhaustive(args.workload, args.mode, 3.0, pair, fields=fields)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 / v, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (CPU)",
            "data": "synthetic (seeded blob-map pairs at 1 A)",
            "config": {"workload": f"{args.workload}: CPU restatement of the reference path (exhaustive search), "
                                   f"mode {args.mode}"},
            "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": cb["cores"], "kind": "port",
                             "sample": cb["sample"]},
            "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.case:
        import bench_cases
        bench_cases.main(a.case)
    elif a.impl == "reference":
        run_reference(a)
    elif a.workload == "uneven64_s4_a15":
        sub_line = run_uneven(a, sub=a.sub_config)
        if a.sub_config:
            print(json.dumps(sub_line), flush=True)
    elif a.workload == "prob128_s3_a15":
        sub_line = run_prob(a, sub=a.sub_config)
        if a.sub_config:
            print(json.dumps(sub_line), flush=True)
    else:
        run_gb300(a)
