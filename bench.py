"""Benchmark: one sigmify round (ParaFROST's GPU inprocessing round) per step.

Workload (default, community-20m): a seeded community-attachment CNF with 20M
variables and 80M clauses (200 communities, modularity 0.8, clause length
geometric with mean 3.5 clipped to [2, 64], power-law variable frequency with
exponent 2.5; 280M literals), synthetic, generated in-process. aig-2.2m is the
Tseitin encoding of a seeded random AIG with 2M AND and 200k XOR gates over 50k
inputs (6.8M clauses). A step = device-side awaken (copy of the resident input +
literal sort + signatures) + one full round with the reference's default phase
settings and -all (VE, SUB, BCE, ERE). Metric unit: input clauses simplified per
second (whole job; N GPUs run N independent replicas: the round does not shard,
so there is no collective). The line also carries every phase's live size,
elected variables, algorithmic bytes and device time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload W]

The reference arm times the reference's CPU simplifier on the host cores: the
compiled reference (oracle/_ref) when present, else the oracle port of it
(oracle/_build), in the same unit: on the full AIG workload, and on a 1/10-size
formula of the same generator for the community workload (a full 80M-clause
round takes about 1.5 minutes on one core, too long for every step).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

WORKLOADS = {
    "aig-2.2m": dict(gen="aig_tseitin", kw=dict(num_inputs=50_000, num_and=2_000_000, num_xor=200_000, seed=1),
                     sample_kw=dict(num_inputs=50_000, num_and=2_000_000, num_xor=200_000, seed=1)),
    "community-20m": dict(gen="community", kw=dict(seed=1),
                          sample_kw=dict(num_vars=2_000_000, num_clauses=8_000_000, seed=1)),
    # the same generator at a tenth of the size (profiling captures)
    "community-2m": dict(gen="community", kw=dict(num_vars=2_000_000, num_clauses=8_000_000, seed=1),
                         sample_kw=dict(num_vars=2_000_000, num_clauses=8_000_000, seed=1)),
    "ksat3-10k": dict(gen="random_ksat", kw=dict(num_vars=10_000, num_clauses=42_600, k=3, seed=1),
                      sample_kw=dict(num_vars=10_000, num_clauses=42_600, k=3, seed=1)),
    # batched workload: 4096 random k-SAT formulas (k in 2..5 per clause), clause counts
    # log-uniform in [1k, 200k], clause/variable ratio U[3.0, 4.5]; one batched round
    # per step; unit formulas/s
    "batch-4096": dict(gen="batch_ksat", kw=dict(num_formulas=4096, cmin=1_000, cmax=200_000, seed=1),
                       sample_kw=dict(num_formulas=4096, cmin=1_000, cmax=200_000, seed=1), batch=True),
    # serving: Poisson arrivals of unrolled-AIG requests (10k-5M clauses), rates swept
    "serve-aig": dict(gen="serving_requests", kw=dict(num=32, seed=1), sample_kw=dict(num=32, seed=1), serve=True),
}
BATCH_UNIT = "CNFs/s"
SERVE_UNIT = "req/s"
SERVE_RATES = (100, 300, 1000, 3000, 5000)
METRIC = "sigmify round ms & HBM GB/s; batched CNFs/s, p50/p99 latency vs plain GPU"
UNIT = "clauses/s"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def make_workload(name: str, sample: bool = False):
    from parafrost_gb300 import cnfgen
    spec = WORKLOADS[name]
    kw = spec["sample_kw"] if sample else spec["kw"]
    return getattr(cnfgen, spec["gen"])(**kw)


def cpu_round_seconds(nv, lits, off) -> tuple:
    """Reference CPU simplifier on one formula: (seconds, kind)."""
    import oracle_runner as orr
    from parafrost_gb300.options import Options
    if orr.reference_available():
        recs = orr.run_reference(nv, lits, off, Options(all=1), level=0)
        t = [d for (k, ph, st, d) in recs if k == "timing"][0]
        return (int(t[0]) | (int(t[1]) << 32)) / 1e6, "reference"
    from parafrost_gb300 import build
    build.build_oracle()
    st, _, secs = orr.run_oracle(nv, lits, off, Options(all=1), level=0)
    return secs, "port"


FORMULAS = None  # --formulas: a smaller batch of the same generator (quick runs)
EXTRA_OPTS: dict = {}  # --opt NAME=VALUE for the single-formula workloads


def batch_forms(name: str):
    from parafrost_gb300 import cnfgen
    kw = dict(WORKLOADS[name]["kw"])
    if FORMULAS:
        kw["num_formulas"] = FORMULAS
    return list(cnfgen.batch_ksat(**kw))


def _oracle_round_seconds(job):
    """One formula through the reference CPU simplifier (a process-pool job)."""
    nv, lits, off = job
    return cpu_round_seconds(nv, lits, off)[0]


def cpu_batch_rate(forms, sample: int, workers: int) -> tuple:
    """Formulas/s of the CPU simplifier on `sample` formulas spread evenly over the
    batch (every len/sample-th), `workers` processes, one formula per process at a
    time: (rate, kind, description)."""
    import multiprocessing as mp
    from parafrost_gb300 import build
    build.build_oracle()
    import oracle_runner as orr
    kind = "reference" if orr.reference_available() else "port"
    step = max(1, len(forms) // sample)
    jobs = forms[::step][:sample]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(workers) as pool:
        pool.map(_oracle_round_seconds, jobs, chunksize=1)
    secs = time.perf_counter() - t0
    desc = (f"{len(jobs)} of the {len(forms)} formulas (every {step}th, "
            f"{sum(j[2].size - 1 for j in jobs)} clauses), one round each, {workers} processes")
    return len(jobs) / secs, kind, desc


def run_reference(args) -> dict:
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    if WORKLOADS[args.workload].get("batch") or WORKLOADS[args.workload].get("serve"):
        if WORKLOADS[args.workload].get("serve"):
            from parafrost_gb300 import cnfgen
            forms = cnfgen.serving_requests(**WORKLOADS[args.workload]["kw"])
        else:
            forms = batch_forms(args.workload)
        unit = SERVE_UNIT if WORKLOADS[args.workload].get("serve") else BATCH_UNIT
        workers = max(1, os.cpu_count() or 1)
        rates = []
        for _ in range(args.warmup + args.steps):
            rate, kind, desc = cpu_batch_rate(forms, max(workers, 16), workers)
            rates.append(rate)
        value = float(np.mean(rates[args.warmup:]))
        return {"metric": METRIC, "value": value, "unit": unit, "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * len(forms) / value,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic", "config": {"workload": args.workload, "sample": True},
                "cpu_baseline": {"value": value, "unit": unit, "cores": workers, "kind": kind, "sample": desc},
                "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    nv, lits, off = make_workload(args.workload, sample=True)
    ncls = off.size - 1
    for _ in range(args.warmup):
        cpu_round_seconds(nv, lits, off)
    times = []
    kind = "port"
    for _ in range(args.steps):
        s, kind = cpu_round_seconds(nv, lits, off)
        times.append(s)
    tot = float(np.sum(times))
    value = ncls * args.steps / tot
    spec = WORKLOADS[args.workload]
    full = spec["sample_kw"] == spec["kw"]
    sample = (f"{spec['sample_kw']} ({ncls} clauses, {'the full workload' if full else 'a smaller formula of the same generator'}),"
              " one full round per step, 1 thread (the reference simplifier has no threads)")
    return {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic",
            "config": {"workload": args.workload, "sample": not full, "clauses": int(ncls), "literals": int(lits.size),
                       "vars": int(nv), "options": "-all, phases=5"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# Kernel names in the ncu captures summarised under profiles/.
NCU_NAMES = {"mis_rounds": "mis_rounds_k", "bve_decide": "bve_warp_k", "sub": "sub_warp_k", "bve_write": "bve_write_warp_k"}


def profiled_line(kernel: str, workload: str):
    """The 'traffic:' line of `kernel` on `workload` in the committed ncu summary
    profiles/dram_traffic.txt, as a dict, or None."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                if not line.startswith("traffic:"):
                    continue
                kv = dict(x.split("=", 1) for x in line.split()[1:])
                if kv.get("kernel") == NCU_NAMES.get(kernel) and kv.get("workload") == workload:
                    return kv
    except (OSError, ValueError):
        pass
    return None


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per launch (read + write) of `kernel` on `workload`, or None."""
    kv = profiled_line(kernel, workload)
    try:
        return float(kv["bytes_per_launch"]) if kv else None
    except (KeyError, ValueError):
        return None


def profiled_utilisation(kernel: str, workload: str):
    """SM and DRAM throughput (% of peak) of the profiled launch, or None: what bounds
    a kernel whose algorithmic bytes are far below the copy peak."""
    kv = profiled_line(kernel, workload)
    if not kv or "sm_pct" not in kv:
        return None
    return {"sm_throughput_pct": float(kv["sm_pct"]), "dram_throughput_pct": float(kv["dram_pct"]),
            "launch": kv.get("measured_launch"), "source": "profiles/dram_traffic.txt (ncu captures named there)"}


def phase_rows(stats, peak: float) -> list:
    """Every phase of a round: live clauses and literals entering it, variables
    elected, algorithmic bytes, device time, and their ratio against the peak."""
    rows = []
    for r in stats.as_dict()["phases"]:
        gbs = r["bytes"] / (r["ms"] / 1e3) / 1e9 if r["ms"] > 0 else None
        rows.append({**r, "gbs": gbs, "frac": gbs / peak if gbs else None})
    return rows


def flush_l2(buf):
    buf.add_(1)


def run_ours(args) -> dict:
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from parafrost_gb300.options import Options
    from parafrost_gb300.sigma import ResultBuffers, Simplifier

    nv, lits, off = make_workload(args.workload)
    ncls = off.size - 1
    dev = torch.device("cuda", local)
    d_lits = torch.from_numpy(lits.view(np.int32)).to(dev)
    d_off = torch.from_numpy(off.view(np.int64)).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    opts = Options(all=1, **EXTRA_OPTS)
    s = Simplifier(opts)

    def step():
        s.awaken_device(nv, d_lits.data_ptr(), d_off.data_ptr(), ncls)
        return s.sigmify()

    for _ in range(max(args.warmup, 3)):
        st = step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    allocs0 = s.lib.pf_device_alloc_count()
    for i in range(args.steps):
        flush_l2(flush)
        ev[i][0].record()
        st = step()
        ev[i][1].record()
        stats.append(st)
    torch.cuda.synchronize()
    allocs = s.lib.pf_device_alloc_count() - allocs0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    tot_ms = float(np.sum(step_ms))
    if world > 1:
        t = torch.tensor([tot_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot_ms = float(t.item())
    ms = tot_ms / args.steps
    value = world * ncls * args.steps / (tot_ms / 1e3)
    last = stats[-1]
    round_ms = float(np.mean([x.ms_total for x in stats]))
    alg = float(np.mean([x.algorithmic_bytes for x in stats]))
    launches = int(np.sum([x.kernel_launches for x in stats]))
    stage_ms = {k: float(np.mean([x.as_dict()["ms_stage"][k] for x in stats])) for k in stats[0].as_dict()["ms_stage"]}

    # e2e through the C ABI with host buffers: upload (H2D), round, download (D2H)
    pin_l = torch.from_numpy(lits.view(np.int32)).pin_memory()
    pin_o = torch.from_numpy(off.view(np.int64)).pin_memory()
    hl, ho = pin_l.numpy().view(np.uint32), pin_o.numpy().view(np.uint64)
    e2e_steps = 0 if args.no_e2e else max(1, min(args.steps, 5))
    d2h = 0
    # results land in reused page-locked buffers (as a serving loop keeps them)
    pinned = []

    def pinned_alloc(nbytes):
        t = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
        pinned.append(t)
        return t.numpy()

    outbuf = ResultBuffers(pinned_alloc)
    if e2e_steps:
        s.result(out=outbuf)  # sizes the buffers from the last round's result, untimed
    parts = np.zeros(3)  # upload, round, download (each call returns after its copies)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ta = time.perf_counter()
        s.awaken(nv, hl, ho)
        tb = time.perf_counter()
        s.sigmify()
        tc = time.perf_counter()
        res = s.result(out=outbuf)
        parts += [tb - ta, tc - tb, time.perf_counter() - tc]
        d2h = res.lits.nbytes + res.offsets.nbytes + res.units.nbytes + res.resolved.nbytes + res.eliminated.nbytes
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / max(e2e_steps, 1)
    parts_ms = (parts * 1e3 / max(e2e_steps, 1)).round(3).tolist()
    e2e_value = world * ncls / e2e_s if e2e_steps else None

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    round_gbs = alg / (round_ms / 1e3) / 1e9
    # per-kernel figures over the timed steps (CUDA events around each launch on the
    # library's stream); the roofline is the dominant kernel's
    kern = {}
    for k in stats[0].as_dict()["kernels"]:
        ms_k = float(np.sum([x.as_dict()["kernels"][k]["ms"] for x in stats]))
        by_k = float(np.sum([x.as_dict()["kernels"][k]["bytes"] for x in stats]))
        n_k = int(np.sum([x.as_dict()["kernels"][k]["launches"] for x in stats]))
        kern[k] = {"ms_per_step": ms_k / args.steps, "launches_per_step": n_k / args.steps,
                   "bytes_per_launch": by_k / max(n_k, 1), "ms_per_launch": ms_k / max(n_k, 1),
                   "gbs": by_k / (ms_k / 1e3) / 1e9 if ms_k > 0 else None}
    dom = max(kern, key=lambda k: kern[k]["ms_per_step"])
    achieved = kern[dom]["gbs"] or 0.0
    traffic = profiled_traffic(dom, args.workload)
    util = profiled_utilisation(dom, args.workload)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "u32", "data": "synthetic",
           "config": {"workload": args.workload, "clauses": int(ncls), "literals": int(lits.size), "vars": int(nv),
                      "options": "-all, phases=5" + "".join(f", {k}={v}" for k, v in EXTRA_OPTS.items()),
                      "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}"},
           "round_ms": round_ms, "stage_ms": stage_ms,
           "step_ms": [round(x, 3) for x in step_ms], "round_ms_each": [round(x.ms_total, 3) for x in stats],
           "device_allocs_per_step": allocs / args.steps,
           "host_syncs_per_round": int(last.host_syncs), "prop_waves": int(last.prop_waves),
           "result": {"clauses_after": int(last.clauses_after), "phases": int(last.phases_run),
                      "status": int(last.status), "mis_rounds": int(last.mis_rounds),
                      "launches_per_round": int(last.kernel_launches)},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                        "algorithmic_bytes_per_launch": kern[dom]["bytes_per_launch"],
                        "ms_per_launch": kern[dom]["ms_per_launch"],
                        "peak_source": "MEASURED_PEAKS.json (hbm_gbs, of measured)" if peaks else "fallback",
                        "ncu_utilisation": util},
           "kernels": kern,
           "round_roofline": {"achieved": round_gbs, "frac": round_gbs / peak,
                              "scope": "whole round: algorithmic bytes / round device time"},
           "phases": phase_rows(last, peak),
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(lits.nbytes + off.nbytes),
                   "d2h_bytes_per_step": int(d2h),
                   "ms": {"upload": parts_ms[0], "round": parts_ms[1], "download": parts_ms[2]}},
           "gpu_launches": launches, "clocks": clk}
    s.close()
    if rank == 0 and not args.no_cpu_baseline:
        spec = WORKLOADS[args.workload]
        snv, sl, so = (nv, lits, off) if spec["sample_kw"] == spec["kw"] else make_workload(args.workload, sample=True)
        secs, kind = cpu_round_seconds(snv, sl, so)
        out["cpu_baseline"] = {"value": (so.size - 1) / secs, "unit": UNIT, "cores": 1, "kind": kind,
                               "sample": f"{WORKLOADS[args.workload]['sample_kw']} ({so.size - 1} clauses), one round"}
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


def run_ours_batch(args) -> dict:
    """Batched workload: one batched round over all formulas per step (inputs
    resident in device memory); e2e through the batch C ABI with host buffers."""
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from parafrost_gb300.options import Options
    from parafrost_gb300.sigma import ResultBuffers, Simplifier, pack_batch, lits_offsets_begin

    forms = batch_forms(args.workload)
    # formulas are independent: each rank takes a footprint-balanced share
    from parafrost_gb300.shard import shard_formulas
    forms = [forms[i] for i in shard_formulas(forms, world)[rank]]
    nv, lits, off = pack_batch(forms)
    cb, lits, off = lits_offsets_begin(forms, lits, off)
    nf, ncls = len(forms), int(off.size - 1)
    dev = torch.device("cuda", local)
    d_lits = torch.from_numpy(lits.view(np.int32)).to(dev)
    d_off = torch.from_numpy(off.view(np.int64)).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    opts = Options(all=1, **EXTRA_OPTS)
    tuned = None
    if args.tune:
        # launch-shape knobs tuned on every 32nd formula of the batch (untimed)
        from parafrost_gb300.tune import tune
        opts, seen = tune(forms[::32], opts, repeats=3)
        tuned = {"chosen": {k: getattr(opts, k) for k in seen}, "round_ms": seen, "sample": f"every 32nd of {nf} formulas"}
    s = Simplifier(opts)

    def step():
        s.upload_batch_device(nv, cb, d_lits.data_ptr(), d_off.data_ptr())
        return s.sigmify()

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    for i in range(args.steps):
        flush_l2(flush)
        ev[i][0].record()
        stats.append(step())
        ev[i][1].record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    tot_ms = float(np.sum([a.elapsed_time(b) for a, b in ev]))
    total_forms = nf
    if world > 1:
        t = torch.tensor([tot_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot_ms = float(t.item())
        n = torch.tensor([nf], device=dev)
        torch.distributed.all_reduce(n)
        total_forms = int(n.item())
    value = total_forms * args.steps / (tot_ms / 1e3)
    last = stats[-1]
    kern = {}
    for k in last.as_dict()["kernels"]:
        ms_k = float(np.sum([x.as_dict()["kernels"][k]["ms"] for x in stats]))
        by_k = float(np.sum([x.as_dict()["kernels"][k]["bytes"] for x in stats]))
        n_k = int(np.sum([x.as_dict()["kernels"][k]["launches"] for x in stats]))
        kern[k] = {"ms_per_step": ms_k / args.steps, "launches_per_step": n_k / args.steps,
                   "bytes_per_launch": by_k / max(n_k, 1), "ms_per_launch": ms_k / max(n_k, 1),
                   "gbs": by_k / (ms_k / 1e3) / 1e9 if ms_k > 0 else None}
    dom = max(kern, key=lambda k: kern[k]["ms_per_step"])
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = kern[dom]["gbs"] or 0.0

    # e2e: host buffers through the batch C ABI (upload, round, per-formula download)
    pin_l = torch.from_numpy(lits.view(np.int32)).pin_memory()
    pin_o = torch.from_numpy(off.view(np.int64)).pin_memory()
    hl, ho = pin_l.numpy().view(np.uint32), pin_o.numpy().view(np.uint64)
    e2e_steps = 0 if args.no_e2e else 1
    d2h = 0
    pinned = []

    def pinned_alloc(nbytes):
        t = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
        pinned.append(t)
        return t.numpy()

    outbuf = ResultBuffers(pinned_alloc)
    if e2e_steps:
        s.batch_results(out=outbuf)  # sizes the reused buffers from the last round, untimed
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.upload_batch(nv, cb, hl, ho)
        s.sigmify()
        res = s.batch_results(out=outbuf)
        d2h = sum(r.lits.nbytes + r.offsets.nbytes + r.units.nbytes + r.resolved.nbytes + r.eliminated.nbytes
                  for _, _, r in res)
    e2e_s = (time.perf_counter() - t0) / max(e2e_steps, 1)
    e2e_value = world * nf / e2e_s if e2e_steps else None
    s.close()

    # the same formulas one by one through the single-formula API (plain launches,
    # one round per formula), on an evenly spread sample
    seq = None
    if not args.no_sequential:
        step_k = max(1, nf // 128)
        sample = forms[::step_k][:128]
        one = Simplifier(opts)
        dl = [(torch.from_numpy(np.asarray(l, dtype=np.uint32).view(np.int32)).to(dev),
               torch.from_numpy(np.asarray(o, dtype=np.uint64).view(np.int64)).to(dev), v) for v, l, o in sample]
        for dlits, doff, v in dl[:3]:  # warm-up
            one.awaken_device(v, dlits.data_ptr(), doff.data_ptr(), doff.numel() - 1)
            one.sigmify()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for dlits, doff, v in dl:
            one.awaken_device(v, dlits.data_ptr(), doff.data_ptr(), doff.numel() - 1)
            one.sigmify()
        torch.cuda.synchronize()
        seq = len(dl) / (time.perf_counter() - t0)
        one.close()

    out = {"metric": METRIC, "value": value, "unit": BATCH_UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
           "scaling": "weak" if world > 1 else "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
           "config": {"workload": args.workload, "formulas": total_forms, "clauses_rank0": ncls,
                      "literals_rank0": int(lits.size), "options": "-all, phases=5",
                      "l2": "inputs larger than L2; 256 MB flush between steps",
                      "parallelism": f"formulas split over {world} ranks" if world > 1 else "one batched round"},
           "round_ms": float(np.mean([x.ms_total for x in stats])),
           "stage_ms": {k: float(np.mean([x.as_dict()["ms_stage"][k] for x in stats])) for k in last.as_dict()["ms_stage"]},
           "result": {"clauses_after": int(last.clauses_after), "phases": int(last.phases_run),
                      "launches_per_round": int(last.kernel_launches)},
           "sequential_cnfs_per_s": seq,
           "tuned": tuned,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "traffic": profiled_traffic(dom, args.workload), "kernel": dom,
                        "algorithmic_bytes_per_launch": kern[dom]["bytes_per_launch"],
                        "ms_per_launch": kern[dom]["ms_per_launch"],
                        "peak_source": "MEASURED_PEAKS.json (hbm_gbs, of measured)" if peaks else "fallback"},
           "kernels": kern,
           "e2e": {"value": e2e_value, "unit": BATCH_UNIT, "h2d_bytes_per_step": int(lits.nbytes + off.nbytes),
                   "d2h_bytes_per_step": int(d2h)},
           "gpu_launches": int(np.sum([x.kernel_launches for x in stats])), "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        workers = max(1, os.cpu_count() or 1)
        rate, kind, desc = cpu_batch_rate(batch_forms(args.workload), max(workers, 16), workers)
        out["cpu_baseline"] = {"value": rate, "unit": BATCH_UNIT, "cores": workers, "kind": kind, "sample": desc}
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


def run_ours_serve(args) -> dict:
    """Serving sweep: open-loop Poisson arrivals at each rate, batched server and
    plain (one request per round) server; latency from arrival to result on host."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from parafrost_gb300 import cnfgen
    from parafrost_gb300.options import Options
    from parafrost_gb300.serve import Server, poisson_load, summarize

    pool = cnfgen.serving_requests(**WORKLOADS[args.workload]["kw"])
    per_rate = args.requests
    free, _ = torch.cuda.mem_get_info()
    budget = int(free * 0.6)
    sweep = []
    clocks = Clocks(local)
    clocks.start()
    for mode in ("batched", "plain"):
        with Server(Options(all=1), hbm_budget=budget, mode=mode) as srv:
            poisson_load(srv, pool, rate=1000.0, num=max(args.warmup, 3), seed=99)  # warm-up
        for rate in SERVE_RATES:
            with Server(Options(all=1), hbm_budget=budget, mode=mode) as srv:
                reqs = poisson_load(srv, pool, rate=float(rate), num=per_rate, seed=rate)
            row = summarize(reqs, srv)
            row.update(rate=rate, mode=mode)
            sweep.append(row)
            if mode == "plain" and row["p99_ms"] and row["p99_ms"] > 60_000:
                break  # saturated far beyond the rate: higher rates only queue longer
    clk = clocks.stop()
    top = [r for r in sweep if r["mode"] == "batched"][-1]
    value = top["formulas_per_s"]
    return {"metric": METRIC, "value": value, "unit": SERVE_UNIT, "n_gpus": 1, "steps": per_rate,
            "warmup": args.warmup, "ms_per_step": 1e3 / value if value else None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": args.workload, "pool": len(pool),
                       "pool_clauses": int(sum(f[2].size - 1 for f in pool)), "requests_per_rate": per_rate,
                       "rates": list(SERVE_RATES), "hbm_budget_bytes": budget,
                       "workers": {"batched": 2, "plain": 1},
                       "timing": "wall clock from scheduled arrival to result on host"},
            "sweep": sweep, "admitted_hbm_bytes": max(r["max_footprint_bytes"] for r in sweep),
            "e2e": {"value": value, "unit": SERVE_UNIT,
                    "h2d_bytes_per_step": int(np.mean([f[1].nbytes + f[2].nbytes for f in pool])),
                    "d2h_bytes_per_step": None},
            "gpu_launches": int(sum(r["gpu_launches"] for r in sweep)), "clocks": clk}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="community-20m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-sequential", action="store_true", help="batched workload: skip the one-by-one comparison")
    ap.add_argument("--formulas", type=int, default=None, help="batched workload: number of formulas")
    ap.add_argument("--requests", type=int, default=160, help="serving workload: requests per arrival rate")
    ap.add_argument("--tune", action="store_true", help="batched workload: autotune the launch knobs first")
    ap.add_argument("--opt", action="append", default=[], metavar="NAME=VALUE",
                    help="a simplifier option for the single-formula workloads (e.g. ot_buckets=1)")
    args = ap.parse_args()
    global EXTRA_OPTS
    EXTRA_OPTS = {k: int(v) for k, v in (o.split("=", 1) for o in args.opt)}
    global FORMULAS
    FORMULAS = args.formulas
    if args.impl == "reference":
        out = run_reference(args)
    else:
        from parafrost_gb300 import build
        build.build_cuda()
        if WORKLOADS[args.workload].get("serve"):
            out = run_ours_serve(args)
        elif WORKLOADS[args.workload].get("batch"):
            out = run_ours_batch(args)
        else:
            out = run_ours(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
