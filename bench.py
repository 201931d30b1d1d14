"""Benchmark: marginal ancestral reconstruction throughput on the
2,000-tip x 30,000-site workload (coalescent tree, branch lengths Exp(5e-4),
GTR with transition/transversion ratio 3, 90% invariant sites -> ~3k
compressed patterns), seeded synthetic data.

One step = one full marginal reconstruction of the tree (branch matrices,
post-order, root, pre-order, per-tree log-likelihood) with its inputs resident
in HBM.  Metric: node-pattern updates per second (nodes x patterns per step /
step time).  The FP32-scaled kernels are the measured path; the FP64 plain
kernel, the end-to-end call through host buffers, the roofline of the
dominant kernel and the CPU reference are reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: independent replicas (one process per GPU, torchrun), no
collective on the data path; rank 0 prints the max-over-ranks timing.
"""

import argparse
import collections
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

REFERENCE_BUDGET_S = 90.0
METRIC = "node-pattern updates/s (marginal reconstruction, FP32-scaled; FP64 plain beside it)"
UNIT = "node-pattern updates/s"
WORKLOAD = "c1: 2000-tip coalescent tree x 30000 nucleotide sites (90% invariant), GTR kappa=3, marginal"


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _reduce_max(x, device, world):
    """Max of a per-rank float over all ranks (the job time is the slowest
    rank's); identity on one process."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    v = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(v, op=dist.ReduceOp.MAX)
    return float(v.item())


def _peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic(kernel_key):
    try:
        with open(os.path.join(HERE, "profiles", "traffic.json")) as fh:
            d = json.load(fh)
        return d.get(kernel_key)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region; the raw
    samples go to ``clocks_<gpu>.csv`` in $TT_BENCH_OUT (default: the system's
    temporary directory).  Entering waits (at most 5 s) for the first sample, so
    that sampling covers the region and not only nvidia-smi's start-up."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        out = os.environ.get("TT_BENCH_OUT") or tempfile.gettempdir()
        self.path = os.path.join(out, "clocks_%d.csv" % index)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line)
            self.first.set()
        self.first.set()

    def __enter__(self):
        import threading
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")
        self.first = threading.Event()
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return self
        self.reader = threading.Thread(target=self._read, daemon=True)
        self.reader.start()
        self.first.wait(5.0)
        return self

    def __exit__(self, *exc):
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.reader.join(timeout=5)
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            with open(self.path, "w") as fh:
                fh.writelines(self.lines)
        except OSError:
            pass

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, util, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in list(self.lines):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
            if len(parts) > 9:
                try:
                    util.append(float(parts[9]))
                except ValueError:
                    pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
               "samples": len(sm)}
        if util:  # share of each sample period with a kernel running (nvidia-smi utilization.gpu)
            out["gpu_busy_pct_mean"] = round(statistics.fmean(util), 1)
        return out


def build_workload(seed=1, **over):
    from treetime_gb300 import TreeAnc, synth
    wl = synth.make_workload("c1", seed=seed, **over)
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision="f32")
    return t, wl


def c1_config(t):
    """The workload's `config` entry, the same in both arms."""
    n_tip = t.tree.count_terminals()
    P = t.data.compressed_length
    return {"workload": WORKLOAD, "tips": n_tip, "nodes": 2 * n_tip - 1, "patterns": P, "sites": t.data.full_length,
            "node_patterns_per_step": (2 * n_tip - 1) * P, "seed": 1,
            "l2": "flushed (512 MiB write) before every timed step (GPU arm)", "parallelism": "single GPU"}


def joint_bytes(layout, P, w=4):
    """Algorithmic bytes of one joint reconstruction: per internal node and
    pattern its sum of messages written and read (2 x w x 8 bytes, FP32
    pairs), its argmax table (w bytes) and its state (1 byte); one code byte
    per tip and pattern."""
    return P * (layout.n_int * (2 * w * 8 + w + 1) + layout.n_tip)


def algorithmic_bytes(layout, P, w=4, e=4, s=4):
    """Bytes per marginal reconstruction of one tree: P * [N_int * (5*w*e +
    3*s + 1) + n_tips * 1] + P * (8 + 4): five profile touches per internal
    node (write own partial, read it as a child, read the parent posterior,
    read own partial, write own posterior), three scale words, one state byte;
    one code byte per tip; the FP64 site log-likelihood and the multiplicity."""
    return P * (layout.n_int * (5 * w * e + 3 * s + 1) + layout.n_tip * 1) + P * (8 + 4)


def run_gpu(args):
    import torch
    from treetime_gb300 import engine

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    t, wl = build_workload()
    t.device = dev
    sess = t._get_session()
    layout, model = sess["layout"], sess["model"]
    # launch shape of the FP32 kernel picked by the autotuner (outside the timed region)
    from treetime_gb300 import autotune
    if args.shape:  # fixed launch shape (profiling runs: timings under a profiler would mislead the tuner)
        best, table = tuple(int(x) for x in args.shape.split("/")), {}
    else:
        best, table = autotune.tune(sess["forest"].inputs, 4, model, device=dev, use_cache=False)
    forest = engine.Forest(sess["forest"].inputs, 4, device=dev, threads=best[0], ctas_per_sm=best[1],
                           ranges_per_sm=best[2])
    bufs = engine.Buffers(forest)
    P = t.data.compressed_length
    N = layout.n_nodes
    units = N * P
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    # one step = one marginal reconstruction, replayed from a captured CUDA graph (the buffer
    # clears and the three launches, no host work between kernels)
    graphs = {prec: engine.CapturedMarginal(forest, model, bufs, precision=prec) for prec in ("f32", "f64")}

    def step(prec):
        return graphs[prec].replay()

    def timed(prec, k, w):
        for _ in range(w):
            step(prec)
        torch.cuda.synchronize()
        times = []
        for _ in range(k):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            step(prec)
            b.record()
            b.synchronize()
            times.append(a.elapsed_time(b))
        return times

    # parity of the measured path against the FP64 kernel on this workload
    lh64 = float(graphs["f64"].replay(sync=True)["tree_lh"][0].item())
    lh32 = float(graphs["f32"].replay(sync=True)["tree_lh"][0].item())
    rel_err = abs(lh32 - lh64) / abs(lh64)

    # FP64 plain kernel (reported beside the measured path)
    t64 = timed("f64", max(3, min(50, args.steps // 10)), 1)

    # the measured path
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t32 = timed("f32", args.steps, args.warmup)
        # dominant kernel alone, same stream, for the roofline
        kt = []
        pm, status = engine.branch_pmats(forest, model, bufs, need32=True)
        for _ in range(min(args.steps, 50)):
            flush.zero_()
            graphs["f32"].replay()  # fresh inputs for the kernel timed alone
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.zero_()
            a.record()
            _marginal_only(engine, forest, model, bufs, pm, "f32")
            b.record()
            b.synchronize()
            kt.append(a.elapsed_time(b))
        torch.cuda.synchronize()
        ms32 = _reduce_max(sum(t32) / len(t32), dev, world)

        # end to end through the drop-in call (host alignment in, node attributes out)
        e2e_ms, h2d, d2h = _public_e2e(t, args.steps, args.warmup, flush)
        # end to end through the captured graph (pinned host buffers, copies inside the timed region)
        e2eg_ms, gh2d, gd2h = _e2e(engine, t, forest, graphs["f32"], args.steps, args.warmup, flush)
        # joint reconstruction of the same configuration
        joint = _joint_block(engine, t, forest, model, bufs, layout, P, args, flush)

    # batched: k independent instances of this configuration (seeds 1..k: their own trees,
    # alignments and models) as one forest and one captured launch sequence -- the batched form of
    # the configuration
    batched = None
    if args.c1_batch > 1:
        k = args.c1_batch
        binputs, bgtrs = _c1_instances(k, sess["forest"].inputs[0], t.gtr)
        bmodel = engine.DeviceModel(bgtrs, dev)
        bforest = engine.Forest(binputs, 4, device=dev)
        bcap = engine.CapturedMarginal(bforest, bmodel, engine.Buffers(bforest), precision="f32")
        for _ in range(3):
            bcap.replay()
        torch.cuda.synchronize()
        bt, bk = [], []
        kbufs = engine.Buffers(bforest)  # the marginal kernel timed alone writes into these
        bpm, _ = engine.branch_pmats(bforest, bmodel, kbufs, need32=True)
        for _ in range(min(args.steps, 50)):
            flush.zero_()
            a0, b0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record()
            bcap.replay()
            b0.record()
            b0.synchronize()
            bt.append(a0.elapsed_time(b0))
            flush.zero_()
            a1, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a1.record()
            _marginal_only(engine, bforest, bmodel, kbufs, bpm, "f32")
            b1.record()
            b1.synchronize()
            bk.append(a1.elapsed_time(b1))
        bms, bkm = sum(bt) / len(bt), sum(bk) / len(bk)
        bab = sum(algorithmic_bytes(ti.layout, ti.n_patterns) for ti in binputs)
        bunits = sum(ti.layout.n_nodes * ti.n_patterns for ti in binputs)
        batched = {"reconstructions": k, "value": bunits / (bms * 1e-3), "unit": UNIT, "ms_per_step": bms,
                   "node_patterns_per_step": bunits,
                   "roofline": {"achieved": bab / (bkm * 1e-3) / 1e9, "frac": bab / (bkm * 1e-3) / 1e9 / _peaks()[0],
                                "kernel_ms": bkm, "ranges": int(len(bforest.work_f32_host)),
                                "algorithmic_bytes_per_launch": bab,
                                "traffic": _traffic("marginal_f32_q4/c1x%d" % k)},
                   "note": "%d independent instances of the configuration (seeds 1..%d: own coalescent tree, "
                           "alignment and GTR each), one forest, one captured launch sequence per step; L2 "
                           "flushed before every step" % (k, k)}

    # serving: a short run of the request loop (p50 / p99 latency)
    serving_block = _serving_block(dev, args) if args.serving_seconds > 0 and world == 1 else None

    pipeline = _config_pipeline(t)
    if rank != 0:
        return None
    peak, peak_kind = _peaks()
    ab = algorithmic_bytes(layout, P)
    k_ms = sum(kt) / len(kt)
    achieved = ab / (k_ms * 1e-3) / 1e9
    traffic = _traffic("marginal_f32_q4/c1")
    clocks = clk.summary()
    cfg = c1_config(t)
    if world > 1:
        cfg["parallelism"] = "replicas"
    res = {
        "metric": METRIC,
        "value": world * units / (ms32 * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms32,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded coalescent tree, GTR-evolved alignment)",
        "config": cfg,
        "fp64_plain": {"value": units / (statistics.mean(t64) * 1e-3), "ms_per_step": statistics.mean(t64)},
        "fp32_over_fp64": statistics.mean(t64) / ms32,
        "rel_logLH_err_vs_fp64": rel_err,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "marginal_f32_kernel<Q=4,W=4,LPP=1,NT=%d,MINB=%d,HM=0>" % (forest.threads, forest.ctas_per_sm),
                     "ranges": int(len(forest.work_f32_host)),
                     "range_patterns": int(forest.work_f32_host[:, 2].max()),
                     "algorithmic_bytes_per_launch": ab, "kernel_ms": k_ms},
        "e2e": {"value": units / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms,
                "path": "TreeAnc.infer_ancestral_sequences(marginal=True) per step: the tip codes copied from pinned "
                        "host memory into the session's device inputs first, the node states, site and tree "
                        "log-likelihoods back on the host after it; host clock"},
        "e2e_graph": {"value": units / (e2eg_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": gh2d,
                      "d2h_bytes_per_step": gd2h, "ms_per_step": e2eg_ms,
                      "path": "the captured graph with pinned host inputs and outputs copied every step; CUDA events"},
        "gpu_launches": 3 * args.steps,
        "joint": joint,
        "serving": serving_block,
        "batched": batched,
        "config_pipeline": pipeline,
        "autotune": {"best": {"threads": best[0], "ctas_per_sm": best[1], "ranges_per_sm": best[2]},
                     "ms": table},
        "clocks": clocks,
    }
    if not args.no_cpu_baseline and world == 1:
        res["cpu_baseline"] = cpu_baseline(t)
    return res


def _config_pipeline(t, repeats=3):
    """The configuration's whole step through the public TreeAnc calls:
    marginal reconstruction (FP32-scaled), joint reconstruction (FP64) and
    optimal_t_compressed on every branch (optimize_branch_lengths_joint), host
    clock, median of `repeats`.  The steps follow one another as in TreeTime's
    optimisation loop (each reconstruction sees the lengths of the step
    before); the tree's branch lengths are restored afterwards."""
    import torch
    nodes = list(t.tree.find_clades())
    saved = [(n.branch_length, getattr(n, "mutation_length", n.branch_length)) for n in nodes]
    parts = {"marginal": [], "joint": [], "branch_lengths": []}
    for _ in range(repeats + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t.infer_ancestral_sequences(marginal=True)
        t1 = time.perf_counter()
        t.infer_ancestral_sequences(marginal=False)
        t2 = time.perf_counter()
        t.optimize_branch_lengths_joint()
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        parts["marginal"].append(t1 - t0)
        parts["joint"].append(t2 - t1)
        parts["branch_lengths"].append(t3 - t2)
    for n, (bl, ml) in zip(nodes, saved):
        n.branch_length, n.mutation_length = bl, ml
    out = {k: statistics.median(v[1:]) * 1e3 for k, v in parts.items()}
    out["total_ms"] = sum(out.values())
    out["note"] = ("one TreeTime step of this configuration through TreeAnc: infer_ancestral_sequences(marginal=True), "
                   "(marginal=False), optimize_branch_lengths_joint; host clock, per-call set-up and copies included")
    return out


C2_WORKLOAD = ("c2: 500-tip Yule tree x 1500 amino-acid sites (21 states incl. gap, no compression), "
               "site-specific GTR (per-site pi ~ Dirichlet(0.5), shared W ~ U(0.1, 5)), TreeTime's interpolated P(t)")


def run_c2(args):
    """--workload c2: marginal reconstruction under GTR_site_specific (each
    site its own eigenbasis), FP32 beside FP64, L2 flushed before every step."""
    import torch
    from treetime_gb300 import TreeAnc, engine, synth
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl = synth.make_workload("c2", seed=2 + rank)
    t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], compress=False, verbose=0, precision="f32",
                device=dev)
    sess = t._get_session()
    forest, bufs, layout, gtr = sess["forest"], sess["bufs"], sess["layout"], t.gtr
    P, N = t.data.compressed_length, layout.n_nodes
    units = N * P
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def timed(prec, k, w):
        for _ in range(w):
            engine.marginal_site_specific(forest, gtr, bufs, precision=prec, sync=False)
        torch.cuda.synchronize()
        ts = []
        for _ in range(k):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            engine.marginal_site_specific(forest, gtr, bufs, precision=prec, sync=False)
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return ts

    lh64 = float(engine.marginal_site_specific(forest, gtr, bufs, precision="f64")["tree_lh"][0].item())
    lh32 = float(engine.marginal_site_specific(forest, gtr, bufs, precision="f32")["tree_lh"][0].item())
    t64 = timed("f64", max(3, min(20, args.steps // 10)), 1)
    with ClockSampler(local) as clk:
        t32 = timed("f32", args.steps, args.warmup)
    ms32, ms64 = sum(t32) / len(t32), sum(t64) / len(t64)
    if rank != 0:
        return None
    q, w = gtr.n_states, forest.w
    # profile traffic as for c1 (w = 24 floats per row), plus each site's eigensystem read once
    ab = P * (layout.n_int * (5 * w * 4 + 3 * 4 + 1) + layout.n_tip) + P * 12 + P * (2 * q * q + 2 * q + 1) * 8
    peak, peak_kind = _peaks()
    res = {
        "metric": METRIC, "value": world * units / (ms32 * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Yule tree, site-specific-model alignment)",
        "config": {"workload": C2_WORKLOAD, "tips": layout.n_tip, "nodes": N, "patterns": P,
                   "node_patterns_per_step": units, "approximate": bool(gtr.approximate),
                   "l2": "flushed (512 MiB write) before every timed step", "parallelism": "single GPU"},
        "fp64_plain": {"value": units / (ms64 * 1e-3), "ms_per_step": ms64},
        "fp32_over_fp64": ms64 / ms32, "rel_logLH_err_vs_fp64": abs(lh32 - lh64) / abs(lh64),
        "roofline": {"bound": "hbm", "achieved": ab / (ms32 * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": ab / (ms32 * 1e-3) / 1e9 / peak, "traffic": _traffic("marginal_ss_f32/c2"),
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": ab,
                     "note": "step time (eigen-basis transport per node and site, two launches)"},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        # TreeTime's site-specific path interpolates every site's matrix on every branch (about
        # 2 s per branch here), so the whole tree would take tens of minutes: time a 6-tip tree
        # drawn the same way (1,500 sites, same model family) instead
        from oracle import anc
        from treetime_gb300.tree import parse_newick, to_newick
        ws = synth.make_workload("c2", seed=20, n=6)
        ts = TreeAnc(tree=ws["tree"], aln=ws["aln"], gtr=ws["gtr"], compress=False, verbose=0, device=dev)
        tree = anc.prepare_tree(parse_newick(to_newick(ts.tree)))
        aln = dict(zip(ts.data.sequence_names, ts.data.compressed_codes.view("S1").astype("U1")))
        t0 = time.perf_counter()
        anc.marginal(tree, aln, ts.data.multiplicity(), ts.gtr, ts.data.full_length)
        secs = time.perf_counter() - t0
        su = (2 * 6 - 1) * ts.data.compressed_length
        res["cpu_baseline"] = {"value": su / secs, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": "one marginal reconstruction of a 6-tip tree x 1500 sites drawn like "
                                         "the workload (numpy restatement of TreeTime, 1 process)", "seconds": secs}
    return res


BLGRID_WORKLOAD = ("blgrid: BranchLenInterpolator likelihood grids ('marginal' mode, TreeTime's 125-point grids) "
                   "of every branch of the 2000-tip x 30000-site tree, from its FP32 reconstruction's profiles")
BLGRID_METRIC = "branch-length grid evaluations/s (log P of one pattern at one grid point of one branch)"
BLGRID_UNIT = "evaluations/s"


def _fma_rate(engine, dev, prec="f64"):
    """Measured FMA issue rate of this GPU (FMAs/s, FP64 or FP32), from the
    library's probe kernel: best of 3 launches of SMs x 8 CTAs x 256 threads x
    8 independent chains x `iters` FMAs, CUDA events on the launching stream."""
    import torch
    lib = engine._lib.load()
    blocks = int(lib.tt_device_sm_count()) * 8
    f32 = prec == "f32"
    sink = torch.empty(blocks * 256, dtype=torch.float32 if f32 else torch.float64, device=dev)
    iters = 4096 * (32 if f32 else 1)
    pr = engine._lib.TT_PREC_F32 if f32 else engine._lib.TT_PREC_F64
    engine.check(lib.tt_fma_probe(64, blocks, pr, engine._p(sink), engine._stream()), "tt_fma_probe")
    best = float("inf")
    for _ in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        engine.check(lib.tt_fma_probe(iters, blocks, pr, engine._p(sink), engine._stream()), "tt_fma_probe")
        b.record()
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return blocks * 256 * 8 * iters / (best * 1e-3)


def run_blgrid(args):
    """--workload blgrid: the likelihood grids of every branch (TreeTime's
    BranchLenInterpolator values in 'marginal' mode) from the profiles of a
    marginal reconstruction, one launch per branch group (internal nodes,
    tips); FP64 arithmetic (per-pattern eigen sums and a table-driven log)."""
    import torch
    from treetime_gb300 import engine
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    t, wl = build_workload()
    t.device = dev
    t.infer_ancestral_sequences(marginal=True)
    nodes = [n for n in t.tree.find_clades() if n.up is not None]
    sess = t._get_session()
    forest = sess["forest"]
    model = engine.model_for(t.gtr, dev)
    padded, lengths = engine.branch_len_grids([n.mutation_length for n in nodes], t.one_mutation)
    P, q = t.data.compressed_length, t.gtr.n_states
    evals = int(lengths.sum()) * P
    prec = t._gpu_precision()
    groups = []
    for idx, kk, pp, pp_row, pc_row, pc in t._profile_branch_groups(nodes):
        groups.append((engine._to_dev(np.asarray(kk, np.int32), dev), pp,
                       engine._to_dev(np.asarray(pp_row, np.int64), dev), pc,
                       engine._to_dev(np.asarray(pc_row, np.int64), dev), engine._to_dev(padded[idx], dev), idx))
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def step():
        return [engine.prob_t_profiles_grid_dev(forest, model, dn, pp, dpr, pc, dcr, prec, t.gtr.gap_index, True, dg)
                for dn, pp, dpr, pc, dcr, dg, _ in groups]

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ts = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            step()
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
    ms = _reduce_max(sum(ts) / len(ts), dev, world)
    # end to end through the public call: host grids, uploads, the launches, the results back
    e2e = []
    for i in range(max(3, min(args.steps, 10))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = t.branch_length_grids(nodes)
        e2e.append(time.perf_counter() - t0)
    e2e_ms = statistics.median(e2e) * 1e3
    f32_kernel = prec == "f32" and q <= 5
    # the FP64 kernel on the profiles of an FP64 reconstruction of the same tree, beside it
    fp64 = None
    if f32_kernel:
        from treetime_gb300 import TreeAnc
        from treetime_gb300.tree import parse_newick, to_newick
        # its own copy of the tree: the nodes of `t` keep their FP32 results
        t64 = TreeAnc(tree=parse_newick(to_newick(t.tree)), aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision="f64",
                      device=dev)
        t64.infer_ancestral_sequences(marginal=True)
        n64 = [n for n in t64.tree.find_clades() if n.up is not None]
        t64.branch_length_grids(n64)
        torch.cuda.synchronize()
        k64 = []
        for _ in range(3):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            t64.branch_length_grids(n64)
            b.record()
            b.synchronize()
            k64.append(a.elapsed_time(b))
        ms64 = min(k64)
        r64 = _fma_rate(engine, dev, "f64")
        # accuracy of the FP32 path (FP32 reconstruction, FP32 grid kernel) against the FP64 path
        g64 = {n.name: v for n, v in t64.branch_length_grids(n64).items()}
        dabs = max(float(np.max(np.abs(res[n][1] - g64[n.name][1]))) for n in nodes)
        drel = max(float(np.max(np.abs(res[n][1] - g64[n.name][1]) / np.maximum(np.abs(g64[n.name][1]), 1.0)))
                   for n in nodes)
        # FP64 instructions per evaluation: q FMAs of the eigen sum, 1 add of the 1e-24 floor, the
        # table log (1 subtract for the reduced argument, 1 multiply by 1/F, 6 polynomial FMAs, 2 FMAs
        # to assemble) and 1 FMA to accumulate weight * log: q + 12
        fp64 = {"ms_per_step": ms64, "value": evals / (ms64 * 1e-3),
                "note": "FP64 kernel (eigenbasis sums, table-driven FP64 log) on an FP64 reconstruction's "
                        "profiles, timed through TreeAnc.branch_length_grids (host grids and copies included)",
                "roofline": {"bound": "fp64", "achieved": evals * (q + 12) / (ms64 * 1e-3) / 1e12,
                             "peak": r64 / 1e12, "unit": "T FP64 instructions/s",
                             "frac": evals * (q + 12) / (ms64 * 1e-3) / r64},
                "f32_path_vs_f64_path": {"max_abs_diff": dabs, "max_rel_diff": drel,
                                         "note": "-log P on every grid point of every branch; relative to "
                                                 "max(|value|, 1)"}}
    if rank != 0:
        return None
    if f32_kernel:
        # FP32 arithmetic per evaluation: q*q + q FMAs of pc.P(t).pp, the 1e-24 offset, the weight
        # multiply, 4 of the compensated sum and one logf (counted as one operation)
        opq = q * q + q + 7
        rate = _fma_rate(engine, dev, "f32")
        roof = {"bound": "fp32", "achieved": evals * opq / (ms * 1e-3) / 1e12, "peak": rate / 1e12,
                "unit": "T FP32 operations/s", "frac": evals * opq / (ms * 1e-3) / rate, "traffic": None,
                "peak_source": "measured live (FP32 FMA probe kernel)", "ops_per_evaluation": opq,
                "kernel": "prob_t_profiles_grid_f32_kernel<%d>" % q}
    else:
        rate = _fma_rate(engine, dev, "f64")
        roof = {"bound": "fp64", "achieved": evals * (q + 12) / (ms * 1e-3) / 1e12, "peak": rate / 1e12,
                "unit": "T FP64 instructions/s", "frac": evals * (q + 12) / (ms * 1e-3) / rate, "traffic": None,
                "peak_source": "measured live (FP64 FMA probe kernel)", "ops_per_evaluation": q + 12,
                "kernel": "prob_t_profiles_grid_kernel<%d>" % q}
    out = {
        "metric": BLGRID_METRIC, "value": world * evals / (ms * 1e-3), "unit": BLGRID_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if f32_kernel else "f64",
        "data": "synthetic (seeded coalescent tree, GTR-evolved alignment)",
        "config": {"workload": BLGRID_WORKLOAD, "branches": len(nodes), "patterns": P,
                   "grid_points": int(lengths.sum()), "evaluations_per_step": evals, "profiles": prec,
                   "l2": "flushed (512 MiB write) before every timed step", "parallelism": "single GPU"},
        "roofline": roof,
        "fp64_kernel": fp64,
        "e2e": {"value": evals / (e2e_ms * 1e-3), "unit": BLGRID_UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(padded.nbytes + sum(len(g[6]) * 20 for g in groups)),
                "d2h_bytes_per_step": int(padded.nbytes)},
        "gpu_launches": len(groups) * args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        # TreeTime's own evaluation (numpy, per grid point) for a sample of branches
        from oracle import anc
        mult = t.data.multiplicity()
        chosen = nodes[::max(1, len(nodes) // 400)]
        errs, aerrs, done, secs = [], [], 0, 0.0
        for n in chosen:
            grid, y = res[n]
            pp, pc = np.asarray(n.marginal_outgroup_LH, np.float64), np.asarray(n.marginal_subtree_LH, np.float64)
            t0 = time.perf_counter()
            want = anc.branch_len_log_prob(t.gtr, grid, "marginal", profile_pair=(pp, pc), multiplicity=mult)
            secs += time.perf_counter() - t0
            done += len(grid) * P
            errs.append(float(np.max(np.abs(y - want) / np.maximum(np.abs(want), 1.0))))
            aerrs.append(float(np.max(np.abs(y - want))))
            if secs > 20.0:
                break
        out["cpu_baseline"] = {"value": done / secs, "unit": BLGRID_UNIT, "cores": 1, "kind": "port",
                               "sample": "%d branches' grids (every %d-th branch) by the numpy restatement of "
                                         "TreeTime's BranchLenInterpolator evaluation, 1 process"
                                         % (len(errs), max(1, len(nodes) // 400)), "seconds": secs}
        out["max_rel_err_vs_oracle"] = max(errs)
        out["max_abs_err_vs_oracle"] = max(aerrs)
    return out


GTRINF_WORKLOAD = ("gtrinf: substitution counts of 'marginal' GTR inference (TreeAnc.infer_gtr) over every branch of "
                   "the 2000-tip x 30000-site tree, from its FP32 reconstruction's profiles")
GTRINF_METRIC = "branch-pattern mutation matrices/s (q x q joint state distribution of one pattern on one branch)"
GTRINF_UNIT = "branch-patterns/s"


def run_gtrinf(args):
    """--workload gtrinf: the counting step of TreeAnc.infer_gtr(marginal=True)
    -- per branch and pattern the normalised q x q joint distribution of the
    states at both ends, summed into n_ija and T_ia -- for all branches: one
    counting launch and one chunk-reduction launch per branch group (internal
    nodes, tips); L2 flushed before every step."""
    import torch
    from treetime_gb300 import engine
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    t, wl = build_workload()
    t.device = dev
    t.infer_ancestral_sequences(marginal=True)
    sess = t._get_session()
    forest = sess["forest"]
    model = engine.model_for(t.gtr, dev)
    nodes = t._counting_branches()
    P, q, w = t.data.compressed_length, t.gtr.n_states, forest.w
    units = len(nodes) * P
    prec = t._gpu_precision()
    engine.branch_pmats(forest, model, sess["bufs"])
    p64 = sess["bufs"].cache[("p64", torch.float64)]
    groups = []
    for idx, kk, pp, pp_row, pc_row, pc in t._profile_branch_groups(nodes):
        groups.append((engine._to_dev(np.asarray(kk, np.int32), dev), pp,
                       engine._to_dev(np.asarray(pp_row, np.int64), dev), pc,
                       engine._to_dev(np.asarray(pc_row, np.int64), dev), len(kk), pc_row[0] < 0))
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def step():
        return [engine.mutation_counts(forest, model, p64, 0, dn, pp, dpr, pc, dcr, prec)
                for dn, pp, dpr, pc, dcr, _, _ in groups]

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ts = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            step()
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
    ms = _reduce_max(sum(ts) / len(ts), dev, world)
    e2e = []
    for _ in range(max(3, min(args.steps, 20))):
        t0 = time.perf_counter()
        t._substitution_counts(True)[0].sum().item()
        e2e.append(time.perf_counter() - t0)
    e2e_ms = statistics.median(e2e) * 1e3
    if rank != 0:
        return None
    # algorithmic bytes: each branch reads the two profile rows of every pattern (a tip's child
    # row is its 1-byte code), the offset branch matrices are written once, the chunk slices are
    # written and read back once, the counts written
    sms = engine._lib.load().tt_device_sm_count()
    ab = 0
    es = 4 if prec == "f32" else 8
    for _, _, _, _, _, nb, tips in groups:
        ab += nb * P * (w * es + (1 if tips else w * es))
        chunks = max(1, min(64, nb, -(-(sms * 2048) // P)))
        ab += forest.n_nodes * q * (w * 8 + q * es) + 2 * chunks * (q * q + q) * P * 8 + (q * q + q) * P * 8
    peak, peak_kind = _peaks()
    achieved = ab / (ms * 1e-3) / 1e9
    out = {
        "metric": GTRINF_METRIC, "value": world * units / (ms * 1e-3), "unit": GTRINF_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == "f32" else "f64",
        "data": "synthetic (seeded coalescent tree, GTR-evolved alignment)",
        "config": {"workload": GTRINF_WORKLOAD, "branches": len(nodes), "patterns": P, "profiles": prec,
                   "l2": "flushed (512 MiB write) before every timed step", "parallelism": "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": peak_kind, "algorithmic_bytes_per_step": ab,
                     "note": "both groups' offset, counting and reduction launches per step"},
        "e2e": {"value": units / (e2e_ms * 1e-3), "unit": GTRINF_UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(sum(g[5] * 20 for g in groups)),
                "d2h_bytes_per_step": int((q * q + q) * P * 8)},
        "gpu_launches": 3 * len(groups) * args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        from oracle import anc
        mult = t.data.multiplicity()
        L = t.data.full_length
        done, secs = 0, 0.0
        chosen = nodes[::max(1, len(nodes) // 2000)]
        for n in chosen:
            pp, pc = np.asarray(n.marginal_outgroup_LH, np.float64), np.asarray(n.marginal_subtree_LH, np.float64)
            t0 = time.perf_counter()
            mut = np.transpose(anc.branch_mutation_matrix(t.gtr, pp, pc, anc.branch_length_to_gtr(n, L)), (1, 2, 0))
            _ = 0.5 * mut.sum(axis=0) * mult + 0.5 * mut.sum(axis=1) * mult, mut * mult
            secs += time.perf_counter() - t0
            done += P
            if secs > 20.0:
                break
        out["cpu_baseline"] = {"value": done / secs, "unit": GTRINF_UNIT, "cores": 1, "kind": "port",
                               "sample": "%d branches (every %d-th) through the numpy restatement of TreeTime's "
                                         "counting step, 1 process" % (done // P, max(1, len(nodes) // 2000)),
                               "seconds": secs}
    return out


FITCH_WORKLOAD = ("fitch: Fitch parsimony reconstruction (TreeAnc.infer_ancestral_sequences(method='fitch')) of the "
                  "2000-tip x 30000-site tree")


def run_fitch(args):
    """--workload fitch: one Fitch reconstruction per step through the public
    call (pass up, root lists to the host and TreeTime's random choices, pass
    down, N_diff against the previous reconstruction); the device passes are
    also timed alone.  L2 flushed before every step."""
    import torch
    from treetime_gb300 import engine
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    t, wl = build_workload()
    t.device = dev
    P = t.data.compressed_length
    layout = t._get_session()["layout"]
    units = layout.n_nodes * P
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        t.infer_ancestral_sequences(method="fitch")
    torch.cuda.synchronize()
    ts = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            t.infer_ancestral_sequences(method="fitch")
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
    ms = _reduce_max(statistics.median(ts) * 1e3, dev, world)
    # the two device passes alone (CUDA events), as the library's C entries run them
    sess = t._get_session()
    forest, bufs = sess["forest"], sess["bufs"]
    lib = engine._lib.load()
    lists = bufs.get("fitch_lists", (forest.prof_rows, 16), torch.uint8)
    status = bufs.get("status", (1,), torch.int32)
    chars = bufs.get("fitch_chars", (forest.state_rows,), torch.uint8)
    root_chars = engine._to_dev(np.full(P, ord("A"), np.uint8), dev)
    kt = []
    for _ in range(min(args.steps, 20)):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        engine.check(lib.tt_fitch_up(engine.C.byref(forest.struct), engine._p(lists), None, engine._p(status),
                                     engine._stream()), "tt_fitch_up")
        engine.check(lib.tt_fitch_down(engine.C.byref(forest.struct), engine._p(lists), engine._p(root_chars),
                                       engine._p(chars), None, None, None, None, engine._stream()), "tt_fitch_down")
        b.record()
        b.synchronize()
        kt.append(a.elapsed_time(b))
    k_ms = statistics.median(kt)
    if rank != 0:
        return None
    # algorithmic bytes of the two passes: per internal node and pattern a 16-byte list written
    # and read back by the parent, read again going down, one character written; per tip a code
    ab = P * (layout.n_int * (16 * 3 + 1) + layout.n_tip)
    peak, peak_kind = _peaks()
    out = {
        "metric": "node-patterns/s (Fitch parsimony reconstruction)", "value": world * units / (ms * 1e-3),
        "unit": "node-patterns/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded coalescent tree, GTR-evolved alignment)",
        "config": {"workload": FITCH_WORKLOAD, "nodes": layout.n_nodes, "patterns": P,
                   "l2": "flushed (512 MiB write) before every timed step", "parallelism": "single GPU",
                   "timing": "host clock around the public call (it reads the root lists back and makes "
                             "TreeTime's random choices on the host)"},
        "device_passes": {"ms": k_ms, "value": units / (k_ms * 1e-3)},
        "roofline": {"bound": "hbm", "achieved": ab / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": ab / (k_ms * 1e-3) / 1e9 / peak, "traffic": None, "peak_source": peak_kind,
                     "note": "both passes; one thread per pattern walks the tree (latency bound)"},
        "e2e": {"value": units / (ms * 1e-3), "unit": "node-patterns/s", "ms_per_step": ms,
                "h2d_bytes_per_step": P, "d2h_bytes_per_step": 16 * P + 8},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        from oracle import anc
        from treetime_gb300.tree import parse_newick, to_newick
        tree = anc.prepare_tree(parse_newick(to_newick(t.tree)))
        chars = np.asarray(t.data.compressed_codes).view("S1").astype("U1")
        caln = {k: chars[i] for i, k in enumerate(t.data.sequence_names)}
        Ps = max(1, min(P, 200))
        t0 = time.perf_counter()
        anc.fitch(tree, {k: v[:Ps] for k, v in caln.items()}, Ps, np.random.default_rng(0))
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": layout.n_nodes * Ps / secs, "unit": "node-patterns/s", "cores": 1,
                               "kind": "port", "sample": "the first %d patterns of the workload through the "
                               "Python restatement of TreeTime's Fitch (lists per node and position), 1 process"
                               % Ps, "seconds": secs}
    return out


BRENT_WORKLOAD = ("brent: profile-mode Brent (optimal_marginal_branch_length, scipy's Brent parameters, tol 1e-10) "
                  "on every branch of the 2000-tip x 30000-site tree from its FP32 reconstruction's profiles")


def run_brent(args):
    """--workload brent: the branch-length optimiser of optimize_tree_marginal
    -- profile-mode Brent on all 3,998 branches in one launch per branch group
    (internal nodes, tips) -- from the FP32 reconstruction (FP32 objective);
    the FP64 kernel on an FP64 reconstruction beside it.  L2 flushed before
    every step."""
    import torch
    from treetime_gb300 import TreeAnc, engine
    from treetime_gb300.tree import parse_newick, to_newick
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    over = {} if args.brent_invariant is None else {"invariant_frac": args.brent_invariant}
    t, wl = build_workload(**over)
    t.device = dev
    t.infer_ancestral_sequences(marginal=True)
    nodes = [n for n in t.tree.find_clades() if n.up is not None]
    P = t.data.compressed_length
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    dev_ms = []

    def timed(tt, nn, k, w):
        for _ in range(w):
            tt._marginal_branch_lengths(nn, 1e-10)
        ts = []
        dev_ms.clear()
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            e0.record()
            res = tt._marginal_branch_lengths(nn, 1e-10)
            e1.record()
            ts.append(time.perf_counter() - t0)
            e1.synchronize()
            dev_ms.append(e0.elapsed_time(e1))
        return statistics.median(ts) * 1e3, res

    with ClockSampler(local) as clk:
        ms, r32 = timed(t, nodes, args.steps, args.warmup)
    device_ms = statistics.median(dev_ms)
    ms = _reduce_max(ms, dev, world)
    t64 = TreeAnc(tree=parse_newick(to_newick(t.tree)), aln=wl["aln"], gtr=wl["gtr"], verbose=0, precision="f64",
                  device=dev)
    t64.infer_ancestral_sequences(marginal=True)
    n64 = [n for n in t64.tree.find_clades() if n.up is not None]
    ms64, r64 = timed(t64, n64, 3, 1)
    if rank != 0:
        return None
    rel = np.abs(r32 - r64) / np.maximum(np.abs(r64), 1e-12)
    out = {
        "metric": "branches optimised/s (profile-mode Brent, all branches of one tree)",
        "value": world * len(nodes) / (ms * 1e-3), "unit": "branches/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded coalescent tree, GTR-evolved alignment)",
        "config": {"workload": BRENT_WORKLOAD, "branches": len(nodes), "patterns": P,
                   "invariant_frac": 0.9 if args.brent_invariant is None else args.brent_invariant,
                   "l2": "flushed (512 MiB write) before every timed step", "parallelism": "single GPU",
                   "timing": "host clock around TreeAnc._marginal_branch_lengths (uploads of the branch lists, "
                             "two launches, the lengths back)"},
        "device_ms_per_step": device_ms,
        "fp64_path": {"ms_per_step": ms64, "value": len(n64) / (ms64 * 1e-3),
                      "note": "FP64 reconstruction, FP64 objective (optimal_t_profiles_kernel)"},
        "f32_vs_f64_lengths": {"median_rel": float(np.median(rel)), "p99_rel": float(np.percentile(rel, 99)),
                               "max_rel": float(rel.max())},
        "roofline": {"bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None,
                     "traffic": None, "note": "~30 dependent objective evaluations per branch, each a CTA-wide sum"},
        "e2e": {"value": len(nodes) / (ms * 1e-3), "unit": "branches/s", "ms_per_step": ms,
                "h2d_bytes_per_step": len(nodes) * 20, "d2h_bytes_per_step": len(nodes) * 12},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        from oracle import anc
        mult = t.data.multiplicity()
        done, secs = 0, 0.0
        for n in n64[::50]:
            pp, pc = np.asarray(n.marginal_outgroup_LH), np.asarray(n.marginal_subtree_LH)
            t0 = time.perf_counter()
            anc.optimal_t_compressed(t64.gtr, (pp, pc), mult, profiles=True, tol=1e-10)
            secs += time.perf_counter() - t0
            done += 1
            if secs > 20.0:
                break
        out["cpu_baseline"] = {"value": done / secs, "unit": "branches/s", "cores": 1, "kind": "port",
                               "sample": "%d branches (every 50th) through the numpy restatement of TreeTime's "
                                         "optimal_t_compressed(profiles=True) with scipy's Brent, 1 process" % done,
                               "seconds": secs}
    return out


COMPRESS_WORKLOAD = ("compress: pattern compression (SequenceData.make_compressed_alignment) of the 2000-tip x "
                     "30000-site alignment (2000 x 30000 bytes)")


def run_compress(args):
    """--workload compress: column classification on the device
    (tt_compress_columns over the alignment resident in HBM, timed alone), and
    the public call engine.compress_columns (alignment copied in, keys back,
    patterns assembled on the host) beside the vectorised host compression and
    TreeTime's per-column loop (the oracle) on a sample of columns."""
    import torch
    from treetime_gb300 import engine, synth
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl = synth.make_workload("c1", seed=1)
    from treetime_gb300.seqdata import SequenceData, compress_codes
    sd = SequenceData(wl["aln"], compress=False, ambiguous="N")
    codes = np.ascontiguousarray(sd.codes)
    n, L = codes.shape
    amb = ord("N")
    lib = engine._lib.load()
    d = engine._to_dev(codes, dev)
    key = torch.empty(L, dtype=torch.int64, device=dev)
    fixed = torch.empty(L, dtype=torch.int32, device=dev)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def kernel():
        engine.check(lib.tt_compress_columns(engine._p(d), n, L, amb, engine._p(key), engine._p(fixed),
                                             engine._stream()), "tt_compress_columns")

    for _ in range(args.warmup):
        kernel()
    torch.cuda.synchronize()
    kt = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            kernel()
            b.record()
            b.synchronize()
            kt.append(a.elapsed_time(b))
    k_ms = _reduce_max(sum(kt) / len(kt), dev, world)
    e2e = []
    for _ in range(max(3, min(args.steps, 10))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pc, mult, f2c, c2f = engine.compress_columns(codes, amb, dev)
        e2e.append(time.perf_counter() - t0)
    e2e_ms = statistics.median(e2e) * 1e3
    t0 = time.perf_counter()
    hpc, hmult, hf2c, _ = compress_codes(codes, amb)
    host_ms = (time.perf_counter() - t0) * 1e3
    same = bool(np.array_equal(pc, hpc) and np.array_equal(mult, hmult) and np.array_equal(f2c, hf2c))
    if rank != 0:
        return None
    ab = n * L + L * 12
    peak, peak_kind = _peaks()
    out = {
        "metric": "alignment sites compressed/s", "value": world * L / (k_ms * 1e-3), "unit": "sites/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": k_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded c1 alignment)",
        "config": {"workload": COMPRESS_WORKLOAD, "sequences": n, "sites": L, "patterns": int(len(mult)),
                   "l2": "flushed (512 MiB write) before every timed step", "parallelism": "single GPU"},
        "roofline": {"bound": "hbm", "achieved": ab / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": ab / (k_ms * 1e-3) / 1e9 / peak, "traffic": None, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": ab},
        "e2e": {"value": L / (e2e_ms * 1e-3), "unit": "sites/s", "ms_per_step": e2e_ms, "h2d_bytes_per_step": n * L,
                "d2h_bytes_per_step": L * 12,
                "note": "engine.compress_columns: alignment up, keys down, patterns assembled on the host"},
        "host_vectorised_ms": host_ms, "identical_to_host": same,
        "gpu_launches": args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        from oracle import anc
        names = sd.sequence_names
        m = 2000
        arrays = {k: codes[i, :m].view("S1").astype("U1") for i, k in enumerate(names)}
        t0 = time.perf_counter()
        anc.compress_alignment(names, arrays, "N")
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": m / secs, "unit": "sites/s", "cores": 1, "kind": "port",
                               "sample": "the first %d columns through the restatement of TreeTime's per-column "
                                         "loop, 1 process" % m, "seconds": secs}
    return out


C3_WORKLOAD = ("c3: 256 independent coalescent trees, tips log-uniform in [50, 5000], sites log-uniform in "
               "[1k, 30k], branch means log-uniform in [1e-4, 0.05], a random GTR per tree; the whole batch is "
               "one forest, one captured launch sequence per step")


def run_c3(args):
    """--workload c3: the batched workload.  Every rank builds its own batch
    (replicas; seeds differ by rank) and runs the marginal pass over the whole
    forest as one captured CUDA graph per step.  Inputs (tens of GB) are far
    larger than L2, so no flush is needed between steps."""
    import torch
    from treetime_gb300 import engine, synth
    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    inputs, gtrs = synth.forest_c3(n_trees=args.c3_trees, seed=3 + rank)
    build_s = time.perf_counter() - t0
    model = engine.DeviceModel(gtrs, device=dev)
    forest = engine.Forest(inputs, 4, device=dev)
    bufs = engine.Buffers(forest)
    units = sum(ti.layout.n_nodes * ti.n_patterns for ti in inputs)
    cap = engine.CapturedMarginal(forest, model, bufs, precision="f32")
    lh32 = cap.replay(sync=True)["tree_lh"].cpu().numpy().copy()

    def timed(fn, k, w):
        for _ in range(w):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return ts

    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t32 = timed(cap.replay, args.steps, args.warmup)
        pm, _ = engine.branch_pmats(forest, model, bufs, need32=True)
        kt = timed(lambda: _marginal_only(engine, forest, model, bufs, pm, "f32"), min(args.steps, 10), 1)
    ms32 = _reduce_max(sum(t32) / len(t32), dev, world)

    # end to end: every tree's tip codes, branch lengths and multiplicities from pinned host
    # memory, states and site log-likelihoods back, every step
    codes_h = torch.from_numpy(np.concatenate([ti.tip_codes.reshape(-1) for ti in inputs])).pin_memory()
    bl_h = torch.from_numpy(forest.bl_host.copy()).pin_memory()
    mult_h = torch.from_numpy(np.concatenate([ti.mult for ti in inputs])).pin_memory()
    states_h = torch.empty(forest.state_rows, dtype=torch.uint8).pin_memory()
    lh_h = torch.empty(forest.n_patterns, dtype=torch.float64).pin_memory()

    def one_e2e():
        forest.d_codes[: codes_h.numel()].copy_(codes_h, non_blocking=True)
        forest.d_bl.copy_(bl_h, non_blocking=True)
        forest.d_mult.copy_(mult_h, non_blocking=True)
        out = cap.replay()
        states_h.copy_(out["states"], non_blocking=True)
        lh_h.copy_(out["site_lh"], non_blocking=True)
        return float(out["tree_lh"].sum().item())

    te = timed(one_e2e, min(args.steps, 10), 1)
    e2e_ms = sum(te) / len(te)
    h2d = codes_h.numel() + bl_h.numel() * 8 + mult_h.numel() * 8
    d2h = states_h.numel() + lh_h.numel() * 8 + 8

    # FP64 plain kernel on the same forest when its buffers fit beside the FP32 ones
    fp64 = None
    free, _ = torch.cuda.mem_get_info(dev)
    need64 = forest.prof_rows * forest.w * 8 * 2 + forest.n_nodes * forest.q * forest.w * 8 * 2
    if getattr(args, "no_fp64", False):
        fp64 = {"skipped": "--no-fp64"}
    elif free > 1.15 * need64:
        cap64 = engine.CapturedMarginal(forest, model, bufs, precision="f64")
        lh64 = cap64.replay(sync=True)["tree_lh"].cpu().numpy().copy()
        t64 = timed(cap64.replay, 3, 1)
        rel = np.abs(lh32 - lh64) / np.abs(lh64)
        w = int(np.argmax(rel))
        tw = inputs[w]
        fp64 = {"value": units / (sum(t64) / len(t64) * 1e-3), "ms_per_step": sum(t64) / len(t64),
                "max_rel_logLH_err_fp32_vs_fp64": float(rel.max()),
                "median_rel_logLH_err_fp32_vs_fp64": float(np.median(rel)),
                "trees_over_1e-6": int((rel > 1e-6).sum()), "trees": len(inputs),
                "worst_tree": {"tips": tw.layout.n_tip, "patterns": tw.n_patterns, "sites": int(round(tw.mult.sum())),
                               "mean_branch_length": float(np.mean(tw.bl)), "logLH_fp64": float(lh64[w]),
                               "abs_err": float(abs(lh32[w] - lh64[w]))}}
    else:
        fp64 = {"skipped": "FP64 buffers (%.0f GB) do not fit beside the FP32 ones (%.0f GB free)"
                % (need64 / 1e9, free / 1e9)}

    if rank != 0:
        return None
    peak, peak_kind = _peaks()
    ab = sum(algorithmic_bytes(ti.layout, ti.n_patterns) for ti in inputs)
    k_ms = sum(kt) / len(kt)
    res = {
        "metric": METRIC, "value": world * units / (ms32 * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded coalescent trees, GTR-evolved alignments)",
        "config": {"workload": C3_WORKLOAD if args.c3_trees == 256 else C3_WORKLOAD + " (first %d trees)" % args.c3_trees,
                   "trees": len(inputs), "nodes": forest.n_nodes,
                   "patterns": forest.n_patterns, "node_patterns_per_step": units,
                   "l2": "inputs (%.0f GB of profile rows) far larger than L2; no flush" % (forest.prof_rows * 32 / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU", "build_seconds": build_s,
                   "ranges": int(len(forest.work_f32_host))},
        "fp64_plain": fp64,
        "roofline": {"bound": "hbm", "achieved": ab / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": ab / (k_ms * 1e-3) / 1e9 / peak, "traffic": _traffic("marginal_f32_q4/c3"),
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": ab, "kernel_ms": k_ms,
                     "kernel": "marginal_f32_kernel<Q=4,W=4,LPP=1,NT=%d,MINB=%d,HM=0>" % (forest.threads, forest.ctas_per_sm)},
        "e2e": {"value": units / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms},
        "gpu_launches": 3 * args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        res["cpu_baseline"] = cpu_baseline_forest(inputs, gtrs)
        res["cpu_baseline_all_cores"] = cpu_baseline_forest_pool(inputs, gtrs)
    return res


def cpu_baseline_forest(inputs, gtrs, budget_node_patterns=4e7, seed=0):
    """The oracle marginal on a seeded random sample of the batch's trees (one
    process), bounded to about ``budget_node_patterns`` node-pattern updates."""
    from oracle import anc
    from treetime_gb300.tree import Tree
    rng = np.random.default_rng(seed)
    order = rng.permutation(len(inputs))
    done_units, secs, used = 0, 0.0, 0
    for k in order:
        ti = inputs[k]
        u = ti.layout.n_nodes * ti.n_patterns
        if done_units + u > budget_node_patterns and used > 0:
            continue
        root = ti.layout.nodes[ti.layout.n_int - 1]
        tree = anc.prepare_tree(Tree(root=root))
        tips = ti.layout.nodes[ti.layout.n_int:]
        chars = ti.tip_codes.view("S1").astype("U1")
        aln = {t.name: chars[r] for t, r in zip(tips, ti.tip_row)}
        L = int(round(ti.mult.sum()))
        t0 = time.perf_counter()
        anc.marginal(tree, aln, ti.mult, _model_state(gtrs[k]), L)
        secs += time.perf_counter() - t0
        done_units += u
        used += 1
        if done_units >= budget_node_patterns:
            break
    return {"value": done_units / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d trees of the batch (seeded random), %.2e node-pattern updates, numpy restatement of "
                      "TreeTime, 1 process" % (used, done_units), "seconds": secs}


def _forest_tree_job(job):
    """One tree of the batch through the oracle marginal (pool worker):
    (newick, {tip: characters}, multiplicities, model state, L) -> seconds."""
    from oracle import anc
    from treetime_gb300.tree import Tree, parse_newick
    nwk, aln, mult, model, L = job
    tree = anc.prepare_tree(Tree(root=parse_newick(nwk).root))
    t0 = time.perf_counter()
    anc.marginal(tree, aln, mult, model, L)
    return time.perf_counter() - t0


def cpu_baseline_forest_pool(inputs, gtrs, budget_node_patterns_per_core=3e7, seed=0):
    """The oracle marginal on a seeded random sample of the batch's trees, the
    trees spread over a spawn-started pool of os.cpu_count() processes (the
    trees are independent), bounded to about ``budget_node_patterns_per_core``
    node-pattern updates per process; wall clock around the pool's map."""
    import multiprocessing as mp
    from treetime_gb300.tree import Tree, to_newick
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    jobs, units = [], 0
    for k in rng.permutation(len(inputs)):
        ti = inputs[k]
        u = ti.layout.n_nodes * ti.n_patterns
        if units + u > budget_node_patterns_per_core * cores and jobs:
            continue
        root = ti.layout.nodes[ti.layout.n_int - 1]
        tips = ti.layout.nodes[ti.layout.n_int:]
        chars = ti.tip_codes.view("S1").astype("U1")
        aln = {t.name: chars[r] for t, r in zip(tips, ti.tip_row)}
        jobs.append((to_newick(Tree(root=root)), aln, ti.mult, _model_state(gtrs[k]), int(round(ti.mult.sum()))))
        units += u
        if units >= budget_node_patterns_per_core * cores:
            break
    jobs.sort(key=lambda j: -len(j[2]) * len(j[1]))  # largest first: better balance over the pool
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_forest_tree_job, jobs[-1:] * cores)  # workers started and modules imported
        t0 = time.perf_counter()
        pool.map(_forest_tree_job, jobs, chunksize=1)
        wall = time.perf_counter() - t0
    return {"value": units / wall, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d trees of the batch (seeded random), %.2e node-pattern updates, numpy restatement of "
                      "TreeTime, trees over a pool of %d processes" % (len(jobs), units, cores),
            "seconds": wall}


C4_WORKLOAD = ("c4: serving loop, Poisson arrivals (200 req/s unless --c4-rate); 90% nucleotide jobs drawn from the c3 size "
               "distribution (half reconstruction, half branch-length optimisation), 10% protein jobs of c2 shape "
               "(site-specific model); 3 ancestral/branch-length iterations per job, device-resident state, "
               "admission by free HBM, one stream per admitted job")


def run_c4(args):
    """--workload c4: the serving loop under Poisson arrivals.  The request
    pool (64 distinct nucleotide jobs from the batch's size distribution, 2
    protein jobs) is generated before the timed window; requests sample it."""
    import torch
    from treetime_gb300 import TreeAnc, serving, synth
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(40 + rank)
    nuc, nuc_gtrs = synth.forest_c3(n_trees=64, seed=41 + rank)
    prot = []
    for s in range(2):
        wl = synth.make_workload("c2", seed=50 + s + 10 * rank)
        t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], compress=False, verbose=0, device=dev)
        prot.append((t._get_session()["forest"].inputs[0], t.gtr))
    rate, window = args.c4_rate, args.c4_seconds
    n = int(rng.poisson(rate * window))
    arrivals = np.sort(rng.uniform(0.0, window, size=n))
    jobs = []
    for i in range(n):
        if rng.random() < 0.1:
            ti, g = prot[int(rng.integers(len(prot)))]
            jobs.append(serving.Job(ti, g, kind="marginal", iterations=3))
        else:
            k = int(rng.integers(len(nuc)))
            jobs.append(serving.Job(nuc[k], nuc_gtrs[k], kind="marginal" if rng.random() < 0.5 else "optimize",
                                    iterations=3))
    # warm: one job of each kind (kernels configured, allocator and pinned pools primed)
    warm = [serving.Job(nuc[0], nuc_gtrs[0], "marginal"), serving.Job(nuc[1], nuc_gtrs[1], "optimize"),
            serving.Job(prot[0][0], prot[0][1], "marginal")]
    serving.Server(device=dev, max_slots=args.c4_slots).serve(warm, [0.0, 0.0, 0.0])
    srv = serving.Server(device=dev, max_slots=args.c4_slots)
    with ClockSampler(local) as clk:
        done, wall = srv.serve(jobs, arrivals)
    st = serving.latency_stats(done)
    # device time of each kind of job run alone (one slot, events between phases), on a sample of
    # the pool, and what the served mix would take at those times back to back
    solo = {}
    sample = {"nucleotide_marginal": [serving.Job(nuc[k], nuc_gtrs[k], "marginal") for k in range(16)],
              "nucleotide_optimize": [serving.Job(nuc[k], nuc_gtrs[k], "optimize") for k in range(16)],
              "protein_marginal": [serving.Job(prot[k % len(prot)][0], prot[k % len(prot)][1], "marginal")
                                   for k in range(4)]}
    for kind, js in sample.items():
        serving.Server(device=dev, max_slots=1, phase_events=True).serve(js, [0.0] * len(js))
        ph = collections.Counter()
        for j in js:
            ph.update(j.phase_ms)
        solo[kind] = {k: round(v / len(js), 3) for k, v in ph.items()}
        solo[kind]["node_patterns_per_iteration"] = float(np.mean([j.node_patterns for j in js]))
    served_kind = lambda j: ("protein_marginal" if j.site_specific else
                             "nucleotide_optimize" if j.kind == "optimize" else "nucleotide_marginal")
    solo_s = sum(sum(v for k, v in solo[served_kind(j)].items() if k != "node_patterns_per_iteration")
                 for j in done) / 1e3
    if rank != 0:
        return None
    return {
        "metric": METRIC, "value": world * st["node_pattern_updates"] / wall, "unit": UNIT, "n_gpus": world,
        "steps": len(done), "warmup": len(warm), "ms_per_step": wall * 1e3 / max(1, len(done)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded request pool: c3-distribution nucleotide trees, c2-shape protein trees)",
        "config": {"workload": C4_WORKLOAD, "arrival_rate_per_s": rate, "window_s": window, "requests": n,
                   "slots": args.c4_slots, "pool": {"nucleotide": len(nuc), "protein": len(prot)},
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "latency_s": {"p50": st["p50"], "p99": st["p99"], "max": st["max"]},
        "served": {"jobs": len(done), "wall_s": wall, "jobs_per_s": len(done) / wall,
                   "node_pattern_updates": st["node_pattern_updates"], "peak_concurrent_jobs": srv.peak_active,
                   "scheduler_host_s": {k: round(v, 3) for k, v in srv.host_s.items()},
                   "kinds": {"nucleotide_marginal": sum(1 for j in done if j.kind == "marginal" and not j.site_specific),
                             "nucleotide_optimize": sum(1 for j in done if j.kind == "optimize"),
                             "protein_marginal": sum(1 for j in done if j.site_specific)}},
        # library kernels per iteration: protein 2 (pass, tree sums); nucleotide 3 (branch matrices,
        # pass, tree sums) plus 2 Brent launches for branch-length jobs
        "gpu_launches": int(sum(j.iterations * (2 if j.site_specific else 3 + (2 if j.kind == "optimize" else 0))
                                for j in done)),
        "clocks": clk.summary(),
        "solo_device_ms_per_job": solo,
        "solo_device_s_for_the_served_mix": round(solo_s, 3),
    }


def _marginal_only(engine, forest, model, bufs, pm, prec):
    """Launch only the marginal pruning kernel (branch matrices already made)."""
    import ctypes as C
    import torch
    from treetime_gb300 import _lib
    lib = _lib.load()
    dt = torch.float32 if prec == "f32" else torch.float64
    w = forest.w
    g = bufs.get
    o = _lib.TTMarginalOut(engine._p(g("partial", (forest.prof_rows, w), dt)),
                           engine._p(g("posterior", (forest.prof_rows, w), dt)), None, None, None,
                           engine._p(g("states", (forest.state_rows,), torch.uint8)),
                           engine._p(g("site_lh", (forest.n_patterns,), torch.float64)),
                           engine._p(g("tree_lh", (len(forest.inputs),), torch.float64)), None, None, 0, 0)
    _lib.check(lib.tt_marginal(C.byref(forest.struct), C.byref(model.struct), C.byref(pm),
                               _lib.TT_PREC_F32 if prec == "f32" else _lib.TT_PREC_F64, C.byref(o), None,
                               engine._stream()), "tt_marginal")


def _public_e2e(t, steps, warmup, flush):
    """The drop-in call end to end, every step: the step's tip codes are copied
    from pinned host memory into the session's device inputs (as a new
    alignment of the same tree would be), TreeAnc.infer_ancestral_sequences
    (marginal=True) runs (branch lengths up, the reconstruction, the internal
    nodes' states, the site and tree log-likelihoods and the changed-site count
    down) and the root's sequence is read.  Host clock, device synchronised on
    both sides.  Returns (ms per step, bytes up, bytes down)."""
    import torch
    sess = t._get_session()
    forest, lay = sess["forest"], sess["layout"]
    P = t.data.compressed_length
    codes_h = torch.from_numpy(np.ascontiguousarray(t.data.compressed_codes).reshape(-1)).pin_memory()
    h2d = codes_h.numel() + lay.n_nodes * 8
    d2h = lay.n_int * P + P * 8 + 8 + 8
    root = t.tree.root

    def one():
        forest.d_codes[: codes_h.numel()].copy_(codes_h, non_blocking=True)
        t.infer_ancestral_sequences(marginal=True)
        return root._cseq[0], t.tree.total_sequence_LH

    for _ in range(max(3, warmup)):
        one()
    times = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        one()
        torch.cuda.synchronize()
        times.append((time.perf_counter() - t0) * 1e3)
    return sum(times) / len(times), int(h2d), int(d2h)


def _joint_only(engine, forest, model, bufs, pm):
    """Launch only the joint kernel (branch matrices already made)."""
    import ctypes as C
    import torch
    from treetime_gb300 import _lib
    lib = _lib.load()
    w = forest.w
    g = bufs.get
    o = _lib.TTJointOut(engine._p(g("joint_msg", (forest.prof_rows, 2, w), torch.float32)),
                        engine._p(g("cx", (forest.prof_rows, w), torch.uint8)),
                        engine._p(g("states", (forest.state_rows,), torch.uint8)),
                        engine._p(g("joint_site_lh", (forest.n_patterns,), torch.float64)),
                        engine._p(g("joint_tree_lh", (len(forest.inputs),), torch.float64)), None, None, 0, 0,
                        int(forest.prof_rows))
    _lib.check(lib.tt_joint(C.byref(forest.struct), C.byref(model.struct), C.byref(pm), C.byref(o), None,
                            engine._stream()), "tt_joint")


def _joint_block(engine, t, forest, model, bufs, layout, P, args, flush):
    """Joint reconstruction of the configuration: device time of one
    reconstruction (branch matrices, the kernel, the tree sums; CUDA events),
    the kernel alone against its algorithmic bytes, and the public call
    TreeAnc.infer_ancestral_sequences(marginal=False) (host clock)."""
    import torch
    units = layout.n_nodes * P
    steps = max(5, min(args.steps, 50))
    for _ in range(3):
        engine.joint(forest, model, bufs, sync=False)
    torch.cuda.synchronize()
    full, kern = [], []
    pm, _ = engine.branch_pmats(forest, model, bufs, needlog=True)
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        engine.joint(forest, model, bufs, sync=False)
        b.record()
        b.synchronize()
        full.append(a.elapsed_time(b))
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        _joint_only(engine, forest, model, bufs, pm)
        b.record()
        b.synchronize()
        kern.append(a.elapsed_time(b))
    pub = []
    for _ in range(6):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t.infer_ancestral_sequences(marginal=False)
        pub.append((time.perf_counter() - t0) * 1e3)
    ms, kms = sum(full) / len(full), sum(kern) / len(kern)
    ab = joint_bytes(layout, P)
    peak, kind = _peaks()
    return {"value": units / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
            "public_call_ms": statistics.median(pub[1:]),
            "roofline": {"bound": "hbm", "achieved": ab / (kms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": ab / (kms * 1e-3) / 1e9 / peak, "peak_source": kind,
                         "kernel": "joint_kernel<Q=4,W=4,LPP=1,NT=%d,HM=0>" % forest.threads, "kernel_ms": kms,
                         "algorithmic_bytes_per_launch": ab, "traffic": _traffic("joint_q4/c1")},
            "arithmetic": "double-float (FP32 pairs) max-plus; states checked against the oracle in tests"}


def _c1_instances(k, first, first_gtr):
    """k independent instances of the configuration: the bench's own (seed 1)
    and seeds 2..k, each with its own tree, alignment and GTR (model index =
    position)."""
    import copy
    inputs, gtrs = [], []
    for s in range(1, k + 1):
        if s == 1:
            ti, g = first, first_gtr
        else:
            t, _ = build_workload(seed=s)
            ti, g = t._get_session()["forest"].inputs[0], t.gtr
        ti = copy.copy(ti)
        ti.model = len(gtrs)
        inputs.append(ti)
        gtrs.append(g)
    return inputs, gtrs


def _serving_block(dev, args):
    """A short run of the serving loop (Poisson arrivals at --c4-rate for
    --serving-seconds): 90% nucleotide jobs on trees of the batch's size
    distribution (a pool of 24 trees and alignments; every request brings its
    own freshly drawn GTR, so no device model is reused), half reconstruction
    and half branch-length jobs, 10% protein jobs (site-specific model, two
    trees and four models).  Reports p50 / p99 latency, throughput and the
    device-model cache builds and hits."""
    from treetime_gb300 import TreeAnc, engine, serving, synth
    from treetime_gb300.gtr import GTR
    rng = np.random.default_rng(77)
    nuc, _ = synth.forest_c3(n_trees=24, seed=71)
    prot = []
    for s in range(2):
        wl = synth.make_workload("c2", seed=80 + s)
        t = TreeAnc(tree=wl["tree"], aln=wl["aln"], gtr=wl["gtr"], compress=False, verbose=0, device=dev)
        prot.append(t._get_session()["forest"].inputs[0])
    prot_models = [synth.gtr_c2(np.random.default_rng(90 + s), prot[0].n_patterns) for s in range(4)]
    rate, window = args.c4_rate, args.serving_seconds
    n = int(rng.poisson(rate * window))
    arrivals = np.sort(rng.uniform(0.0, window, size=n))
    jobs = []
    for i in range(n):
        if rng.random() < 0.1:
            jobs.append(serving.Job(prot[int(rng.integers(2))], prot_models[int(rng.integers(4))], kind="marginal",
                                    iterations=3))
        else:
            g = GTR.random(mu=1.0, alphabet="nuc_nogap", rng=rng)
            jobs.append(serving.Job(nuc[int(rng.integers(len(nuc)))], g,
                                    kind="marginal" if rng.random() < 0.5 else "optimize", iterations=3))
    warm = [serving.Job(nuc[0], GTR.random(mu=1.0, alphabet="nuc_nogap", rng=rng), "marginal"),
            serving.Job(nuc[1], GTR.random(mu=1.0, alphabet="nuc_nogap", rng=rng), "optimize"),
            serving.Job(prot[0], prot_models[0], "marginal")]
    serving.Server(device=dev, max_slots=args.c4_slots).serve(warm, [0.0, 0.0, 0.0])
    before = dict(engine.CACHE_STATS)
    srv = serving.Server(device=dev, max_slots=args.c4_slots)
    done, wall = srv.serve(jobs, arrivals)
    st = serving.latency_stats(done)
    cache = {k: engine.CACHE_STATS[k] - before.get(k, 0) for k in engine.CACHE_STATS}
    return {"window_s": window, "arrival_rate_per_s": rate, "requests": n, "jobs_done": len(done),
            "jobs_per_s": len(done) / wall, "p50_s": st["p50"], "p99_s": st["p99"], "max_s": st["max"],
            "node_pattern_updates_per_s": st["node_pattern_updates"] / wall,
            "device_model_cache": cache,
            "requests_from": "24 nucleotide trees of the batch's size distribution, each request with a fresh "
                             "random GTR; 2 protein trees x 4 site-specific models"}


def _e2e(engine, t, forest, graph, steps, warmup, flush):
    """Host buffers in, host buffers out: tip codes, branch lengths and
    multiplicities are copied from pinned host memory, the reconstruction runs
    (the captured graph, which reads the forest's input buffers in place), and
    the states and per-pattern log-likelihoods come back to pinned host memory,
    every step."""
    import torch
    codes_h = torch.from_numpy(np.ascontiguousarray(t.data.compressed_codes).reshape(-1)).pin_memory()
    bl_h = torch.from_numpy(forest.bl_host.copy()).pin_memory()
    mult_h = torch.from_numpy(t.data.multiplicity().copy()).pin_memory()
    states_h = torch.empty(forest.state_rows, dtype=torch.uint8).pin_memory()
    lh_h = torch.empty(forest.n_patterns, dtype=torch.float64).pin_memory()
    h2d = codes_h.numel() + bl_h.numel() * 8 + mult_h.numel() * 8
    d2h = states_h.numel() + lh_h.numel() * 8 + 8

    def one():
        forest.d_codes[: codes_h.numel()].copy_(codes_h, non_blocking=True)
        forest.d_bl.copy_(bl_h, non_blocking=True)
        forest.d_mult.copy_(mult_h, non_blocking=True)
        out = graph.replay()
        states_h.copy_(out["states"], non_blocking=True)
        lh_h.copy_(out["site_lh"], non_blocking=True)
        return float(out["tree_lh"][0].item())

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        one()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    return sum(times) / len(times), int(h2d), int(d2h)


# ----------------------------------------------------------------------------
# CPU reference: TreeTime's marginal algorithm restated in numpy (the oracle)
# ----------------------------------------------------------------------------
def _oracle_chunk(args):
    newick, names, codes, mult, gtr_state, full_length = args
    from oracle import anc
    from treetime_gb300.tree import parse_newick
    tree = anc.prepare_tree(parse_newick(newick))
    chars = codes.view("S1").astype("U1")
    aln = {k: chars[i] for i, k in enumerate(names)}
    t0 = time.perf_counter()
    anc.marginal(tree, aln, mult, gtr_state, full_length)
    return time.perf_counter() - t0


def _model_state(gtr):
    """Picklable copy of the model attributes the oracle reads."""
    import types
    return types.SimpleNamespace(v=gtr.v, v_inv=gtr.v_inv, eigenvals=gtr.eigenvals, mu=gtr.mu, Pi=gtr.Pi,
                                 alphabet=gtr.alphabet, profile_map=dict(gtr.profile_map), gap_index=gtr.gap_index,
                                 is_site_specific=False)


def _oracle_inputs(t, p_slices):
    from treetime_gb300.tree import to_newick
    nwk = to_newick(t.tree)
    names = t.data.sequence_names
    codes = t.data.compressed_codes
    mult = t.data.multiplicity()
    m = _model_state(t.gtr)
    return [(nwk, names, np.ascontiguousarray(codes[:, s]), mult[s], m, t.data.full_length) for s in p_slices]


def cpu_baseline(t):
    """The oracle marginal on the full workload, one process (bounded: one
    reconstruction, ~5-20 s)."""
    P = t.data.compressed_length
    N = t.tree.count_terminals() * 2 - 1
    secs = _oracle_chunk(_oracle_inputs(t, [slice(0, P)])[0])
    return {"value": N * P / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "one full marginal reconstruction of the workload (numpy restatement of TreeTime, 1 process)",
            "seconds": secs}


def run_reference(args):
    """--impl reference: the CPU implementation of the path (numpy
    restatement of TreeTime's marginal algorithm) on all host cores: patterns
    split across a spawn-started process pool (patterns are independent)."""
    world, rank, local = _dist()
    if rank != 0:
        return None
    import multiprocessing as mp
    t, wl = build_workload()
    P = t.data.compressed_length
    N = t.tree.count_terminals() * 2 - 1
    cores = os.cpu_count() or 1
    chunks = [slice(i * P // cores, (i + 1) * P // cores) for i in range(cores)]
    inputs = _oracle_inputs(t, chunks)
    ctx = mp.get_context("spawn")
    # one step is the whole workload on all cores (smaller samples would be dominated by the
    # per-node Python overhead); the timed steps stop after REFERENCE_BUDGET_S seconds
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_oracle_chunk, inputs)
        times = []
        t_start = time.perf_counter()
        for _ in range(args.steps):
            t0 = time.perf_counter()
            pool.map(_oracle_chunk, inputs)
            times.append(time.perf_counter() - t0)
            if time.perf_counter() - t_start > REFERENCE_BUDGET_S and len(times) >= 3:
                break
    sec = sum(times) / len(times)
    v = N * P / sec
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": len(times),
            "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded coalescent tree, GTR-evolved alignment)",
            "config": c1_config(t),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "full marginal reconstruction per step, patterns split over %d processes"
                                       % cores},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="c1",
                    choices=["c1", "c2", "c3", "c4", "blgrid", "gtrinf", "fitch", "brent", "compress"],
                    help="c1: the 2,000-tip x 30k-site tree (the headline line); c3: the batch of 256 trees")
    ap.add_argument("--no-fp64", action="store_true", help="c3: skip the FP64 arm (profiling runs)")
    ap.add_argument("--c4-seconds", type=float, default=10.0, help="c4: arrival window (s)")
    ap.add_argument("--c4-rate", type=float, default=200.0, help="c4: mean arrival rate (requests/s)")
    ap.add_argument("--brent-invariant", type=float, default=None,
                    help="brent: invariant-site fraction of the 2,000-tip alignment (default 0.9; lower values "
                         "give more patterns than the kernel's shared memory holds)")
    ap.add_argument("--c1-batch", type=int, default=8, help="c1: reconstructions in the batched measurement (1: none)")
    ap.add_argument("--c4-slots", type=int, default=16, help="c4: jobs admitted at the same time")
    ap.add_argument("--serving-seconds", type=float, default=2.0,
                    help="c1: arrival window of the short serving run in the default line (0: none)")
    ap.add_argument("--shape", default="", help="c1: fixed FP32 launch shape threads/ctas_per_sm/ranges_per_sm "
                                                 "instead of the autotuner (profiling runs)")
    ap.add_argument("--c3-trees", type=int, default=256,
                    help="trees in the c3 batch (fewer: the first trees of the same seeded draw, for profiling)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        res = run_reference(args)
    else:
        from treetime_gb300 import build
        build.build()
        res = {"c1": run_gpu, "c2": run_c2, "c3": run_c3, "c4": run_c4, "blgrid": run_blgrid,
               "gtrinf": run_gtrinf, "fitch": run_fitch, "brent": run_brent,
               "compress": run_compress}[args.workload](args)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
