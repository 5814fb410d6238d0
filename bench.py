"""Benchmark: pattern-node updates/s of the Felsenstein-pruning likelihood engine.

Workload (one step = one full log-likelihood evaluation from scratch: every
internal partial recomputed, then the root-branch lnL): protein LG+G4,
100 taxa x 50,000 sites simulated on a seeded Yule tree (mean branch 0.05,
alpha 0.8, empirical frequencies), FP64 drop-in path.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times IQ-TREE 2's own likelihood kernels
(tree/phylokernelnew.h compiled by oracle/ref from the reference's sources:
the SIMD kernels the reference installs on the host, OpenMP over all host
cores) on full evaluations of the same workload; where those sources are not
at hand it falls back to the C restatement (the oracle) on a pattern sample.
Prints one JSON line on rank 0.
"""
from __future__ import annotations

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

from iqtree2_gb300 import simulate  # noqa: E402

WORKLOADS = {
    # the headline: protein LG+G4, 100 taxa x 50,000 sites
    "protein": dict(workload="protein LG+G4 100 taxa x 50000 sites, full lnL (98 partial updates + root lnL)",
                    model="LG+G4", taxa=100, sites=50000, seed=2, mean_bl=0.05, alpha=0.8),
    # the same model on 10,000 sites (~1 GB of partials): the small case for ncu captures
    "protein-small": dict(workload="protein LG+G4 100 taxa x 10000 sites, full lnL", model="LG+G4", taxa=100,
                          sites=10000, seed=2, mean_bl=0.05, alpha=0.8),
    "dna": dict(workload="DNA GTR+G4 16 taxa x 1000 sites, full lnL", model="GTR+G4", taxa=16, sites=1000,
                seed=1, mean_bl=0.1, alpha=0.5),
    # 200 taxa on 30,000 sites (~1.1 GB of partials): the DNA case for ncu captures
    "dna-mid": dict(workload="DNA GTR+G4 200 taxa x 30000 sites, full lnL", model="GTR+G4", taxa=200,
                    sites=30000, seed=4, mean_bl=0.1, alpha=0.5),
    "dna-large": dict(workload="DNA GTR+G4 200 taxa x 100000 sites, full lnL", model="GTR+G4", taxa=200,
                      sites=100000, seed=4, mean_bl=0.1, alpha=0.5),
    "codon": dict(workload="codon GY94+G4 40 taxa x 10000 codons, full lnL", model="GY94+G4", taxa=40,
                  sites=10000, seed=3, mean_bl=0.1, alpha=0.5),
}
WORKLOAD = WORKLOADS["protein"]
METRIC = "pattern-node updates/s"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum, one pass, caches
# kept warm between launches) of the traversal kernels of one full evaluation at
# the workload's own size, from the captures summarised in profiles/ (the bench
# does not run ncu itself); None where no capture was made.
TRAFFIC_BYTES = {
    "protein": (2581.7e6, "profiles/k_traverse_tc_ring_protein100x50k.md"),  # the tuned deep-ring schedule
    "dna-large": (2219.6e6, "profiles/k_level_dna_dna200x100k.md"),
    "codon": (438.3e6, "profiles/k_traverse_tc_ws_flow_codon40x10k.md"),  # the dataflow schedule
}
# schedules the autotuner may pick instead, with their own captures
TRAFFIC_BY_SCHEDULE = {
    ("codon", "0/level-ws/s2/k2"): (418.7e6, "profiles/k_traverse_tc_ws_codon40x10k.md"),
}


def traffic_of(key, tile):
    """DRAM bytes per evaluation of the schedule that ran, from its ncu summary."""
    return TRAFFIC_BY_SCHEDULE.get((key, str(tile)), TRAFFIC_BYTES.get(key, (None, None)))


def dataset(w=None):
    w = w or WORKLOAD
    if w["model"] == "LG+G4":
        return simulate.protein_lg_dataset(w["taxa"], w["sites"], w["seed"], mean_bl=w["mean_bl"], alpha=w["alpha"])
    if w["model"] == "GTR+G4":
        return simulate.dna_gtr_dataset(w["taxa"], w["sites"], w["seed"], mean_bl=w["mean_bl"], alpha=w["alpha"])
    return simulate.codon_gy94_dataset(w["taxa"], w["sites"], w["seed"], mean_bl=w["mean_bl"], alpha=w["alpha"])


def topology_ops(ds):
    """Full traversal toward the root branch used by computeLikelihood."""
    from iqtree2_gb300.topology import Topology
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    # computeLikelihood evaluates at the farthest leaf's branch; any leaf branch has the same work
    leaf = 0
    nb = topo.adj[leaf][0][0]
    ops = topo.branch_ops(nb, leaf)
    return topo, ops, topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)


def kernel_name(use_tc, n, tile, bf16=False):
    """Dominant kernel of a path, from the autotuned label (tile/schedule[/sD][/kP])."""
    if use_tc:
        depth = next((int(t[1:]) for t in tile.split("/") if t.startswith("s")), 2)
        if "/level-tm" in tile and not bf16:
            return "k_traverse_tc_tm"
        if "/level-ring" in tile and not bf16:
            return "k_traverse_tc_ring"
        np_ = 64 if n > 32 else 32
        bf = 'true' if bf16 else 'false'
        if "/flow-tcw" in tile:  # dataflow, whole (op, tile) items
            return f"k_traverse_tc_ws<{np_},{depth},{bf},false,true>"
        if "/flow-tc" in tile:  # dataflow, category-split items
            return f"k_traverse_tc_ws<{np_},{depth},{bf},true,true>"
        name = "k_traverse_tc_ws" if "/level-ws" in tile else "k_traverse_tc"
        return f"{name}<{np_},{depth},{bf}>"
    if tile.startswith("1/"):
        return "k_level_dna" if "/level" in tile else "k_traverse_dna<LNL>"
    nq = {4: 1, 20: 5}.get((n + 3) // 4 * 4, 0)
    return f"k_level_mixed<{nq}>" if "/level" in tile else f"k_traverse_mixed<{nq},LNL>"


def tc_mma_flops(ops, n, C, nptn, bf16=False):
    """MMA flops the tensor-core kernel executes: per internal child, category
    and 128-pattern tile, M=128 x N x K (N, K padded); split TF32 runs 3 passes,
    BF16 one (K per stage padded to 16)."""
    npad = (n + 3) // 4 * 4
    N = 32 if npad <= 32 else 64
    ksplit = 2 if (npad > 32 and npad % 16 == 0) else 1
    K = ((npad // ksplit + 15) // 16 * 16) * ksplit if bf16 else (npad + 7) // 8 * 8
    tiles = (nptn + 127) // 128
    children = sum((c0 >= 0) + (c1 >= 0) for (_, c0, c1, _, _) in ops)
    return (1 if bf16 else 3) * 2 * 128 * N * K * C * children * tiles


def algorithmic_cost(ops, ntaxa, n, C, nptn, mixed=False):
    """Bytes and flops one traversal + root-lnL launch must move/execute.

    FP64 path: 8-byte eigen-space partials, uint8 scale counts, eigen-space
    flops (6n^2+n)C per internal-internal update. Mixed path: 4-byte
    standard-basis partials padded to npad states, int32 exponents, standard
    flops (4n^2+n)C per internal-internal update.
    """
    npad = (n + 3) // 4 * 4
    if mixed:
        blk, sc = C * npad * 4, 4
        f_ii, f_ti, f_tt = (4 * n * n + n) * C, (2 * n * n + n) * C, n * C
    else:
        blk, sc = C * n * 8, 1
        f_ii, f_ti, f_tt = (6 * n * n + n) * C, (4 * n * n + n) * C, (2 * n * n + n) * C
    bytes_per_ptn = 0.0
    flops_per_ptn = 0.0
    for (_, c0, c1, _, _) in ops:
        tips = (c0 < 0) + (c1 < 0)
        if tips == 2:
            bytes_per_ptn += 2 + blk + sc
            flops_per_ptn += f_tt
        elif tips == 1:
            bytes_per_ptn += 1 + blk + sc + blk + sc
            flops_per_ptn += f_ti
        else:
            bytes_per_ptn += 2 * (blk + sc) + blk + sc
            flops_per_ptn += f_ii
    # root lnL: read one partial + one tip state + freq, write pattern lnL
    bytes_per_ptn += blk + sc + 1 + 8 + 8
    flops_per_ptn += 3 * n * C
    return bytes_per_ptn * nptn, flops_per_ptn * nptn


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock and throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        """Start sampling every 20 ms; returns once the first sample has arrived
        (at most 5 s), so that samples cover the timed region that follows."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.005)
        self.skip = len(self.lines)  # samples taken before the timed region

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[getattr(self, "skip", 0):] or self.lines[-1:]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _number(v):
    """A peak given as a number, or as {"value": number, ...}."""
    if isinstance(v, dict):
        v = v.get("value", v.get("gbs", v.get("tflops")))
    return float(v) if isinstance(v, (int, float)) and v > 0 else None


def measured_peaks():
    """The measured copy bandwidth (hbm_gbs) and bf16 GEMM rate of this machine's
    GPUs from MEASURED_PEAKS.json, else the fallback figures."""
    try:
        with open(PEAKS_PATH) as f:
            d = json.load(f)
    except (OSError, ValueError):
        d = None
    if isinstance(d, dict) and _number(d.get("hbm_gbs")):
        out = dict(d)
        out["hbm_gbs"] = _number(d["hbm_gbs"])
        out["bf16_tflops"] = _number(d.get("bf16_tflops")) or 1900.0
        return out, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp64_peak_tflops(device=0):
    """FP64 denominator measured in this run: cuBLAS DGEMM (torch.matmul on
    float64 operands, 6144^3, on the device), the dense FP64 rate a library
    reaches on this GPU."""
    import torch
    n = 6144
    g = torch.Generator(device=f"cuda:{device}").manual_seed(1)
    a = torch.rand(n, n, dtype=torch.float64, device=f"cuda:{device}", generator=g)
    b = torch.rand(n, n, dtype=torch.float64, device=f"cuda:{device}", generator=g)
    for _ in range(2):
        c = a @ b
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 4
    ev0.record()
    for _ in range(reps):
        c = a @ b
    ev1.record()
    torch.cuda.synchronize()
    del a, b, c
    return 2.0 * n ** 3 * reps / (ev0.elapsed_time(ev1) / 1e3) / 1e12


def reference_kernel_baseline(ds, ops, leaf, nb, min_seconds=3.0, max_reps=50):
    """IQ-TREE 2's own kernels timed on full evaluations of the whole workload:
    tree/phylokernelnew.h built by oracle/ref (the fast build: the reference's
    optimisation with FMA contraction) with the SIMD kernels the reference
    installs on this host, OpenMP over all host cores (2 packets per thread,
    as PhyloTree::setNumThreads). SAFE for state counts other than 4 and 20, as
    setLikelihoodKernel chooses. None where the reference's sources are absent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import refkernels
        if not refkernels.available():
            return None
        cores = os.cpu_count() or 1
        m = ds.model
        r = refkernels.RefTree(m, ds.patterns, ds.freq, ds.edges, ds.lengths, safe=m.nstates not in (4, 20),
                               kind=refkernels.KIND_SIMD, nthreads=cores, fast=True)
        vsize, fma = refkernels.simd_info(fast=True)
    except (ImportError, RuntimeError, OSError) as ex:  # no compiler or sources on this host
        return {"unavailable": f"reference kernels not built: {ex}"}
    lnl = r.branch_lnl(nb, leaf)  # warm-up: first touch of the partial buffers
    t0, reps = time.perf_counter(), 0
    while True:
        lnl = r.branch_lnl(nb, leaf)  # every partial recomputed (the harness clears them)
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or reps >= max_reps:
            break
    upd = reps * len(ops) * ds.nptn
    return {"value": upd / el, "unit": METRIC, "cores": cores, "kind": "reference", "lnl": lnl,
            "sample": f"{reps} full evaluations of the whole workload ({ds.nptn} patterns x {len(ops)} partial "
                      f"updates + branch lnL) in {el:.1f}s: IQ-TREE's tree/phylokernelnew.h kernels "
                      f"({vsize}-lane SIMD{' with FMA' if fma else ''}, OpenMP {cores} threads), built from "
                      f"the reference's sources by oracle/ref"}


def cpu_baseline(ds, ops, a, b, length, sample_ptn=8000, min_seconds=10.0):
    """The C restatement of the reference kernels (the oracle: strict IEEE,
    scalar, OpenMP over all host cores) on a pattern sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    cores = os.cpu_count() or 1
    pats = np.ascontiguousarray(ds.patterns[:, :sample_ptn])
    freq = ds.freq[:sample_ptn]
    t = oracle.OracleTree(ds.model, pats, freq, ds.edges, ds.lengths, nthreads=cores)
    lengths = ds.lengths.copy()
    t.compute_likelihood()  # warm-up
    upd0, t0, reps = t.num_updates(), time.perf_counter(), 0
    while True:
        t.set_lengths(lengths)  # invalidate every partial: full recomputation
        t.compute_likelihood()
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or reps >= 5000:
            break
    upd = t.num_updates() - upd0
    return {"value": upd / el, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{pats.shape[1]} of {ds.nptn} patterns x {len(ops)} partial updates, {reps} full "
                      f"evaluations in {el:.1f}s (oracle C restatement, OpenMP)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    ds = dataset()
    _, ops, a, b, length = topology_ops(ds)
    leaf, nb = 0, None
    from iqtree2_gb300.topology import Topology
    nb = Topology(ds.edges, ds.lengths, ds.ntaxa).adj[0][0][0]
    per_step = max(1.0, 60.0 / max(args.steps, 1))
    first = reference_kernel_baseline(ds, ops, leaf, nb, min_seconds=0.5, max_reps=max(args.warmup, 1))
    if first and "value" in first:
        vals = [reference_kernel_baseline(ds, ops, leaf, nb, min_seconds=per_step, max_reps=1000)
                for _ in range(args.steps)]
        note = ("IQ-TREE 2's own likelihood kernels (tree/phylokernelnew.h) built from its sources by oracle/ref, "
                "the SIMD kernels it installs on this host, all host cores, full evaluations of the workload")
    else:
        for _ in range(args.warmup):
            cpu_baseline(ds, ops, a, b, length, min_seconds=0.5)
        vals = [cpu_baseline(ds, ops, a, b, length, min_seconds=max(3.0, 30.0 / max(args.steps, 1)))
                for _ in range(args.steps)]
        note = ("reference kernels restated in C (the reference's kernel sources are not on this host); "
                "a bounded pattern sample, all host cores")
    v = statistics.median([x["value"] for x in vals])
    cb = dict(vals[0])
    cb["value"] = v
    cb.pop("lnl", None)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": WORKLOAD, "cpu_baseline": cb,
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": note}
    print(json.dumps(line))


def measure_path(eng, ops_arr, a, b, length, steps, warmup, stream, local, dist):
    """Time `steps` full evaluations on device-resident inputs (CUDA events on the
    engine's stream) and the dominant kernel per launch."""
    import torch
    for _ in range(warmup):
        lnl = eng.compute_likelihood(ops_arr, a, b, length)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    eng.set_timing(True)
    clocks = ClockSampler(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    launches0 = eng.launches()
    ev0.record(stream)
    for _ in range(steps):
        lnl = eng.compute_likelihood(ops_arr, a, b, length)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = eng.launches() - launches0
    clk = clocks.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    kern_ms, kern_n = eng.timing()
    eng.set_timing(False)
    if dist:
        t = torch.tensor([elapsed_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    return dict(lnl=lnl, elapsed_ms=elapsed_ms, kern_avg_s=kern_ms / max(kern_n, 1) / 1e3, clocks=clk,
                launches=launches)


def make_engine(ds, topo, precision, local, stream):
    from iqtree2_gb300 import engine
    m = ds.model
    eng = engine.Engine(ds.nptn, m.nstates, m.ncat, ds.ntaxa, m.state_unknown, topo.nslots,
                        precision=precision, device=local, max_ops=topo.nslots)
    eng.set_stream(stream.cuda_stream)
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    return eng


def e2e_path(eng, ds, ops_arr, a, b, length, steps):
    """End to end through the C ABI from pinned host buffers: model, pattern
    weights and tip states copied every step, the lnL read back."""
    import torch
    m = ds.model
    pinned = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in (ds.patterns, ds.freq)]
    h_patterns, h_freq = (t.numpy() for t in pinned)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        eng.set_model(m)
        eng.set_patterns(h_freq)
        eng.set_tip_states(h_patterns)
        lnl = eng.compute_likelihood(ops_arr, a, b, length)
    sec = (time.perf_counter() - t0) / steps
    h2d = ds.patterns.nbytes + ds.freq.nbytes + sum(x.nbytes for x in (m.eval, m.evec, m.inv_evec, m.rates,
                                                                        m.props, m.tip_lh, m.pi)) + ops_arr.nbytes
    return sec, lnl, int(h2d)


def extra_workload(key, args, stream, local, peaks, peak_src, fp64_peak):
    """Another configuration in the default run: the mixed headline path
    (autotuned), the FP64 drop-in beside it, the roofline of the dominant
    kernel and IQ-TREE's own CPU kernels on the same workload."""
    import torch
    from iqtree2_gb300 import autotune, engine
    w = WORKLOADS[key]
    ds = dataset(w)
    topo, ops, a, b, length = topology_ops(ds)
    m = ds.model
    ops_arr = engine.Engine.ops_array(ops)
    upd = len(ops) * ds.nptn
    use_tc = 16 <= m.nstates <= 64
    eng = make_engine(ds, topo, engine.TF32X3 if use_tc else engine.F32, local, stream)
    tile, _ = autotune.tune(eng, ops_arr, a, b, length)
    steps = max(5, args.steps // 4)
    r = measure_path(eng, ops_arr, a, b, length, steps, args.warmup, stream, local, None)
    e2e_s, _, h2d = e2e_path(eng, ds, ops_arr, a, b, length, 3)
    eng.close()
    torch.cuda.synchronize()
    eng64 = make_engine(ds, topo, engine.F64, local, stream)
    r64 = measure_path(eng64, ops_arr, a, b, length, 3, 1, stream, local, None)
    eng64.close()
    bmx, fmx = algorithmic_cost(ops, ds.ntaxa, m.nstates, m.ncat, ds.nptn, mixed=True)
    b64, f64 = algorithmic_cost(ops, ds.ntaxa, m.nstates, m.ncat, ds.nptn, mixed=False)
    achieved = bmx / r["kern_avg_s"] / 1e9
    value = upd * steps / (r["elapsed_ms"] / 1e3)
    v64 = upd * 3 / (r64["elapsed_ms"] / 1e3)
    nb = topo.adj[0][0][0]
    out = {
        "workload": w["workload"], "nptn": ds.nptn, "value": value, "unit": METRIC,
        "ms_per_step": r["elapsed_ms"] / steps, "dtype": "tf32x3" if use_tc else "f32", "tile": tile,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "peak_source": peak_src,
                     "traffic": traffic_of(key, tile)[0],
                     "traffic_source": traffic_of(key, tile)[1],
                     "kernel": kernel_name(use_tc, m.nstates, tile), "algorithmic_bytes_per_launch": bmx,
                     "kernel_ms": r["kern_avg_s"] * 1e3, "fp32_tflops": fmx / r["kern_avg_s"] / 1e12},
        "e2e": {"value": upd / e2e_s, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 32},
        "lnl": {"mixed": r["lnl"], "fp64": r64["lnl"], "rel_err": abs(r["lnl"] - r64["lnl"]) / abs(r64["lnl"])},
        "fp64_path": {"value": v64, "ms_per_step": r64["elapsed_ms"] / 3,
                      "fp64_frac": f64 / r64["kern_avg_s"] / 1e12 / fp64_peak if fp64_peak else None},
        "speedup_vs_fp64_path": value / v64,
        "gpu_launches": r["launches"], "clocks": r["clocks"],
    }
    if use_tc:
        mma = tc_mma_flops(ops, m.nstates, m.ncat, ds.nptn)
        out["roofline"]["tensor"] = {"mma_tflops": mma / r["kern_avg_s"] / 1e12, "mma_flops_per_launch": mma}
    if not args.no_cpu_baseline:
        cb = reference_kernel_baseline(ds, ops, 0, nb, min_seconds=2.0)
        if not cb or "value" not in cb:
            cb = cpu_baseline(ds, ops, a, b, length, min_seconds=3.0)
        cb.pop("lnl", None)
        out["cpu_baseline"] = cb
    return out


def branch_optimisation_dna16(args):
    """The CPU-runnable configuration: DNA GTR+G4, 16 taxa x 1,000 sites --
    full lnL plus Newton-Raphson on every branch (optimizeAllBranches) on the
    GPU's FP64 drop-in (host drivers + C ABI) and on the CPU restatement of
    the reference's drivers and kernels (the oracle), same tree and model."""
    from iqtree2_gb300 import engine
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    ds = dataset(WORKLOADS["dna"])
    t = engine.GpuTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths)
    o = oracle.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths, nthreads=1)
    reps = max(3, args.steps // 20)

    def timed(tree):
        tree.set_lengths(ds.lengths)
        tree.optimize_all_branches()  # warm-up
        t0 = time.perf_counter()
        for _ in range(reps):
            tree.set_lengths(ds.lengths)
            lnl = tree.optimize_all_branches()
        return (time.perf_counter() - t0) / reps, lnl

    g_s, g_lnl = timed(t)
    t.set_device_newton(2)
    b_s, _ = timed(t)
    t.set_device_newton(False)
    h_s, _ = timed(t)
    t.set_device_newton(True)
    c_s, c_lnl = timed(o)
    upd0 = t.num_updates()
    t.set_lengths(ds.lengths)
    t.optimize_all_branches()
    gpu_updates = t.num_updates() - upd0
    t.close()
    return {"workload": "DNA GTR+G4 16 taxa x 1000 sites: lnL + optimizeAllBranches (all-branch Newton-Raphson)",
            "gpu_fp64_ms": g_s * 1e3, "gpu_fp64_branch_newton_ms": b_s * 1e3, "gpu_fp64_host_newton_ms": h_s * 1e3,
            "cpu_oracle_1core_ms": c_s * 1e3,
            "speedup": c_s / g_s,
            "optimisations_per_s": 1.0 / g_s, "pattern_node_updates_per_run": gpu_updates,
            "lnl": {"gpu_fp64": g_lnl, "cpu": c_lnl, "rel_err": abs(g_lnl - c_lnl) / abs(c_lnl)},
            "note": "GPU: host drivers (csrc/tree.cpp) over the FP64 kernels (the lane kernel for this short "
                    "4-state alignment), minimizeNewton as one thread-block-cluster kernel per branch, each "
                    "optimizeAllBranches pass enqueued whole with the lengths in device memory and one host wait "
                    "per pass (gpu_fp64_branch_newton_ms: one host wait per branch, iqgpu_newton_branch; "
                    "gpu_fp64_host_newton_ms: the host loop, one launch and read-back per derivative); CPU: the C "
                    "restatement of the same drivers and kernels, one thread (the alignment has ~600 patterns)"}


def run_ours(args):
    import torch
    from iqtree2_gb300 import engine

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)

    ds = dataset()
    topo, ops, a, b, length = topology_ops(ds)
    m = ds.model
    stream = torch.cuda.Stream()
    ops_arr = engine.Engine.ops_array(ops)
    updates_per_step = len(ops) * ds.nptn
    peaks, peak_src = measured_peaks()

    # FP64 drop-in path, reported beside the headline, with its own end-to-end
    # figure (the precision-matched comparison with the reference's FP64 kernels)
    b64, f64 = algorithmic_cost(ops, ds.ntaxa, m.nstates, m.ncat, ds.nptn, mixed=False)
    r64 = None
    fp64_peak = None
    if not args.headline_only:
        fp64_peak = fp64_peak_tflops(local)
        eng64 = make_engine(ds, topo, engine.F64, local, stream)
        r64 = measure_path(eng64, ops_arr, a, b, length, max(3, args.steps // 4), args.warmup, stream, local, dist)
        e2e64_s, _, h2d64 = e2e_path(eng64, ds, ops_arr, a, b, length, 3)
        eng64.close()

    # headline: mixed-precision path (split-TF32 tensor cores for 16..64 states,
    # FP32 CUDA cores otherwise); schedule / pattern tile picked by the autotuner
    from iqtree2_gb300 import autotune
    use_tc = args.precision == "tf32x3" or (args.precision == "auto" and 16 <= m.nstates <= 64)
    prec = engine.TF32X3 if use_tc else engine.F32
    beside = None
    if use_tc and not args.headline_only:  # the FP32 CUDA-core kernel, reported beside the tensor-core headline
        engc = make_engine(ds, topo, engine.F32, local, stream)
        ctile, ctile_ms = autotune.tune(engc, ops_arr, a, b, length)
        rc_ = measure_path(engc, ops_arr, a, b, length, max(3, args.steps // 4), args.warmup, stream, local, dist)
        beside = dict(kernel_ms=rc_["kern_avg_s"] * 1e3, lnl=rc_["lnl"], tile=ctile,
                      value=updates_per_step * max(3, args.steps // 4) / (rc_["elapsed_ms"] / 1e3))
        engc.close()
    eng = make_engine(ds, topo, prec, local, stream)
    if args.config:  # fixed configuration (profiling runs): no tuning
        fixed = next((c for c in autotune.candidates(eng) if autotune.label(c) == args.config), None)
        if fixed is None:
            raise SystemExit(f"--config {args.config}: not a candidate here "
                             f"({', '.join(autotune.label(c) for c in autotune.candidates(eng))})")
        autotune.apply(eng, fixed)
        tile, tile_ms = args.config, {}
    else:
        tile, tile_ms = autotune.tune(eng, ops_arr, a, b, length)
    r = measure_path(eng, ops_arr, a, b, length, args.steps, args.warmup, stream, local, dist)
    value = updates_per_step * args.steps * world / (r["elapsed_ms"] / 1e3)
    bmx, fmx = algorithmic_cost(ops, ds.ntaxa, m.nstates, m.ncat, ds.nptn, mixed=True)

    # end to end through the C ABI from pinned host buffers: inputs copied each
    # step, lnL read back
    e2e_steps = max(2, min(args.steps, 10))
    e2e_s, lnl_e2e, h2d = e2e_path(eng, ds, ops_arr, a, b, length, e2e_steps)
    assert lnl_e2e == r["lnl"]
    if use_tc and not args.headline_only:  # BF16 operands (one MMA pass), reported beside: speed and lnL error
        engb = make_engine(ds, topo, engine.BF16, local, stream)
        btile, _ = autotune.tune(engb, ops_arr, a, b, length)
        rb = measure_path(engb, ops_arr, a, b, length, max(3, args.steps // 4), args.warmup, stream, local, dist)
        engb.close()
    if rank != 0:
        return
    achieved = bmx / r["kern_avg_s"] / 1e9
    npad = (m.nstates + 3) // 4 * 4
    slot_mb = (ds.nptn + 127) // 128 * 128 * m.ncat * npad * 4 / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["elapsed_ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "tf32x3" if use_tc else "f32", "data": "synthetic",
        "config": dict(WORKLOAD, path=("mixed: split-TF32 (3-pass) tcgen05 contraction, " if use_tc else
                                       "mixed: FP32 CUDA-core contraction, ") +
                       "FP32 standard-basis partials, per-pattern 2^k exponents, FP64 exp/log/sums",
                       nptn=ds.nptn, parallelism=f"replicas x{world}",
                       tile=tile, tile_ms={str(k): v for k, v in tile_ms.items()},
                       l2=f"inputs larger than L2 ({len(ops)} partials x {slot_mb:.1f} MB written and read "
                          f"per step, L2 129 MB)"),
        "full_lnl_evals_per_s": 1e3 * args.steps / r["elapsed_ms"],
        "lnl": {"mixed": r["lnl"], "fp64": r64["lnl"] if r64 else None,
                "rel_err": abs(r["lnl"] - r64["lnl"]) / abs(r64["lnl"]) if r64 else None},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"],
                     "traffic": traffic_of(args.workload, tile)[0],
                     "traffic_source": traffic_of(args.workload, tile)[1], "peak_source": peak_src,
                     "kernel": kernel_name(use_tc, m.nstates, tile), "algorithmic_bytes_per_launch": bmx,
                     "fp32_tflops": fmx / r["kern_avg_s"] / 1e12, "flops_per_launch": fmx,
                     "kernel_ms": r["kern_avg_s"] * 1e3},
        "fp64_path": None if r64 is None else {
            "value": updates_per_step * max(3, args.steps // 4) / (r64["elapsed_ms"] / 1e3),
            "ms_per_step": r64["elapsed_ms"] / max(3, args.steps // 4),
            "kernel": ("k_traverse_f64_wide<NORM,LNL>" if m.nstates == 20 and m.ncat <= 4
                       else "k_traverse_f64_cat (SAFE walk) + k_traverse_f64 epilogue" if m.nstates > 20
                       else f"k_traverse_f64<{m.nstates},NORM,LNL>"),
            "hbm_frac": b64 / r64["kern_avg_s"] / 1e9 / peaks["hbm_gbs"],
            "fp64_tflops": f64 / r64["kern_avg_s"] / 1e12, "fp64_peak_tflops": fp64_peak,
            "fp64_peak_source": "cuBLAS DGEMM 6144^3 measured in this run",
            "fp64_frac": f64 / r64["kern_avg_s"] / 1e12 / fp64_peak,
            "e2e": {"value": updates_per_step / e2e64_s, "unit": METRIC, "h2d_bytes_per_step": h2d64,
                    "d2h_bytes_per_step": 32}},
        "e2e": {"value": updates_per_step / e2e_s, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": 8 * 4},
        "clocks": r["clocks"],
        "gpu_launches": r["launches"],
    }
    if use_tc and not args.headline_only:
        line["bf16"] = dict(kernel_ms=rb["kern_avg_s"] * 1e3, tile=btile, kernel=kernel_name(True, m.nstates, btile, True),
                            value=updates_per_step * max(3, args.steps // 4) / (rb["elapsed_ms"] / 1e3),
                            lnl=rb["lnl"], rel_err_vs_fp64=abs(rb["lnl"] - r64["lnl"]) / abs(r64["lnl"]),
                            mma_tflops=tc_mma_flops(ops, m.nstates, m.ncat, ds.nptn, bf16=True) / rb["kern_avg_s"] / 1e12)
        line["cuda_core_f32"] = beside
    if use_tc:
        mma = tc_mma_flops(ops, m.nstates, m.ncat, ds.nptn)
        line["roofline"]["tensor"] = {"mma_flops_per_launch": mma, "mma_tflops": mma / r["kern_avg_s"] / 1e12,
                                      "note": "executed split-TF32 MMA flops (3 passes, padded N/K), upper "
                                              "bound (tail ops may run on CUDA cores)"}
    if r64:
        line["speedup_vs_fp64_path"] = value / line["fp64_path"]["value"]
    if not args.no_cpu_baseline:
        ref = reference_kernel_baseline(ds, ops, 0, topo.adj[0][0][0], min_seconds=5.0)
        port = cpu_baseline(ds, ops, a, b, length, min_seconds=5.0)
        if ref and "value" in ref:
            ref.pop("lnl", None)
            line["cpu_baseline"] = ref
            line["cpu_baseline_port"] = port
        else:
            line["cpu_baseline"] = port
    if world == 1 and args.workload == "protein" and not args.headline_only:
        # the other configurations, each with its own roofline and CPU baseline
        line["workloads"] = {k: extra_workload(k, args, stream, local, peaks, peak_src, fp64_peak)
                             for k in ("dna-large", "codon")}
        line["branch_opt_dna16x1k"] = branch_optimisation_dna16(args)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def run_batched(args):
    """Batched evaluation on DNA GTR+G4, 200 taxa x 100,000 sites: NNI candidates
    (one graph-captured launch sequence for all candidates vs one candidate at a
    time through the kernel-level calls), UFBoot RELL scores of 1,000 replicates
    and 12 uneven partitions with separate GTR+G4 (one graph launch vs one
    evaluation per partition). Synthetic data simulated under the model."""
    import torch
    from iqtree2_gb300 import autotune, engine
    from iqtree2_gb300.topology import Topology
    torch.cuda.set_device(0)
    reps = max(args.steps, 3)
    ds = simulate.dna_gtr_dataset(200, 100000, 4)
    topo = Topology(ds.edges, ds.lengths, ds.ntaxa)
    m = ds.model
    ncand = 64
    cands = topo.nni_candidates(ncand)
    ncand = len(cands)
    nslots = topo.nslots + 2 * ncand
    eng = engine.Engine(ds.nptn, 4, m.ncat, ds.ntaxa, m.state_unknown, nslots, precision=engine.F32,
                        max_ops=max(nslots, 2 * ncand))
    eng.set_model(m)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    leaf, nb = 0, topo.adj[0][0][0]
    bops = engine.Engine.ops_array(topo.branch_ops(nb, leaf))
    autotune.tune(eng, bops, topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb))
    eng.compute_partials(topo.all_partials_ops())
    entries = topo.nni_batch_entries(cands, topo.nslots)

    # NNI: all candidates in one batch (graph replay after the first call)
    for _ in range(args.warmup):
        lnl_b, bl_b = eng.nni_batch(entries)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        lnl_b, bl_b = eng.nni_batch(entries)
    nni_batch_s = (time.perf_counter() - t0) / reps

    # the same candidates one at a time: two partials, safeguarded Newton on the
    # central branch (one derivative launch and read-back per step), final lnL
    def one_by_one():
        out = []
        for (subs, scr, lens, central) in entries:
            eng.compute_partials([(scr[0], subs[0], subs[1], lens[0], lens[1]),
                                  (scr[1], subs[2], subs[3], lens[2], lens[3])])
            x, first = central, True
            for _ in range(10):
                df, ddf = eng.likelihood_derv([], scr[0], scr[1], x, theta_computed=not first)
                first = False
                step = -df / ddf if ddf < 0 else (0.1 if df > 0 else -0.1) * x
                nx = min(max(x + step, 1e-6), 10.0)
                if abs(nx - x) < 1e-6:
                    x = nx
                    break
                x = nx
            out.append(eng.lnl_from_buffer(x))
        return np.array(out)

    lnl_seq = one_by_one()
    t0 = time.perf_counter()
    for _ in range(max(1, reps // 3)):
        lnl_seq = one_by_one()
    nni_seq_s = (time.perf_counter() - t0) / max(1, reps // 3)

    # UFBoot RELL: 1,000 replicate weight vectors resident, scores for 64 trees
    rng = np.random.default_rng(5)
    weights = simulate.bootstrap_weights(ds.freq, 1000, rng)
    eng.set_boot_weights(weights)
    plh0 = eng.pattern_lh()
    trees = plh0[None, :] + rng.normal(0.0, 1e-3, size=(64, ds.nptn))
    for _ in range(args.warmup):
        scores = eng.rell(trees)
    t0 = time.perf_counter()
    for _ in range(reps):
        scores = eng.rell(trees)
    rell_s = (time.perf_counter() - t0) / reps
    want = trees @ weights.T.astype(np.float64)
    rell_err = float(np.max(np.abs(scores - want) / np.abs(want)))
    # the per-tree UFBoot step: scores of the tree just evaluated, inputs on the device
    for _ in range(args.warmup):
        cur = eng.rell_current()
    t0 = time.perf_counter()
    for _ in range(reps):
        cur = eng.rell_current()
    rell_cur_s = (time.perf_counter() - t0) / reps
    eng.close()

    # 12 uneven partitions, separate GTR+G4, one tree
    sizes = [2000, 4000, 6000, 8000, 10000, 12000, 14000, 16000, 20000, 24000, 28000, 30000]
    parts = simulate.partitioned_dna_datasets(200, sizes, 7)
    ptopo = Topology(parts[0].edges, parts[0].lengths, parts[0].ntaxa)
    pnb = ptopo.adj[leaf][0][0]
    pops = engine.Engine.ops_array(ptopo.branch_ops(pnb, leaf))
    pa, pb, plen = ptopo.ref(leaf, pnb), ptopo.ref(pnb, leaf), ptopo.edge_len(leaf, pnb)
    pengs = []
    for d in parts:
        e = engine.Engine(d.nptn, 4, d.model.ncat, d.ntaxa, d.model.state_unknown, ptopo.nslots,
                          precision=engine.F32, max_ops=ptopo.nslots)
        e.set_model(d.model)
        e.set_patterns(d.freq)
        e.set_tip_states(d.patterns)
        autotune.tune(e, pops, pa, pb, plen)
        pengs.append(e)
    for _ in range(args.warmup):
        seq = [e.compute_likelihood(pops, pa, pb, plen) for e in pengs]
    t0 = time.perf_counter()
    for _ in range(reps):
        seq = [e.compute_likelihood(pops, pa, pb, plen) for e in pengs]
    part_seq_s = (time.perf_counter() - t0) / reps
    grp = engine.Group(pengs)
    grp.prepare([pops] * len(pengs), [pa] * len(pengs), [pb] * len(pengs), [plen] * len(pengs))
    for _ in range(args.warmup):
        tot, per = grp.lnl()
    t0 = time.perf_counter()
    for _ in range(reps):
        tot, per = grp.lnl()
    part_graph_s = (time.perf_counter() - t0) / reps
    assert list(per) == seq
    part_updates = len(pops) * sum(d.nptn for d in parts)
    grp.close()
    for e in pengs:
        e.close()

    line = {
        "metric": "NNI candidate evaluations/s", "value": ncand / nni_batch_s,
        "unit": "candidate evaluations/s", "n_gpus": 1, "steps": reps, "warmup": args.warmup,
        "higher_is_better": True, "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "DNA GTR+G4 200 taxa x 100000 sites: 64 NNI candidates, 1000 UFBoot replicates, "
                               "12 partitions of 2k-30k sites with separate GTR+G4", "nptn": ds.nptn},
        "nni": {"candidates": ncand, "batch_ms": nni_batch_s * 1e3, "one_by_one_ms": nni_seq_s * 1e3,
                "speedup": nni_seq_s / nni_batch_s,
                "max_abs_dlnl_batch_vs_one_by_one": float(np.max(np.abs(lnl_b - lnl_seq))),
                "note": "one evaluation = two partials + Newton-Raphson on the central branch + lnL"},
        "rell": {"replicates": 1000, "trees": 64, "ms": rell_s * 1e3,
                 "replicate_tree_scores_per_s": 64 * 1000 / rell_s, "max_rel_err_vs_fp64_numpy": rell_err,
                 "current_tree_ms": rell_cur_s * 1e3,
                 "note": "trees: host FP64 pattern lnL in; current tree: device-resident pattern lnL"},
        "partitions": {"count": len(sizes), "sites": sizes, "graph_ms": part_graph_s * 1e3,
                       "one_by_one_ms": part_seq_s * 1e3, "speedup": part_seq_s / part_graph_s,
                       "graph_updates_per_s": part_updates / part_graph_s, "lnl": tot},
    }
    print(json.dumps(line))


def run_serve(args):
    """Serving: seeded stream of lnL + one round of branch optimisation jobs;
    70% DNA GTR+G4 / 30% protein LG+G4, taxa log-U[8, max], sites log-U[500,
    max]; inputs simulated on the device, generation untimed. Two regimes per
    precision: the specified Poisson rate (--rate, 200/s: far above what one
    GPU completes, so latency is mostly queueing of a burst) on the first
    --requests jobs, and a steady state below capacity (--steady-requests jobs
    at --steady-rate for the mixed path, --steady-requests-fp64 at
    --steady-rate-fp64 for FP64), where p99 is a tail of a stationary queue.
    Reports p50/p99 latency (completion - arrival) and throughput."""
    from iqtree2_gb300 import engine, serving
    rng = np.random.default_rng(args.seed)
    njobs = max(args.requests, args.steady_requests, args.steady_requests_fp64)
    jobs = []
    t_gen = time.perf_counter()
    for k in range(njobs):
        kind = "dna" if rng.random() < 0.7 else "protein"
        taxa = int(round(np.exp(rng.uniform(np.log(8), np.log(args.max_taxa)))))
        sites = int(round(np.exp(rng.uniform(np.log(500), np.log(args.max_sites)))))
        jobs.append(simulate.serving_dataset(kind, max(taxa, 4), sites, int(rng.integers(1 << 30))))
    t_gen = time.perf_counter() - t_gen
    out = {"metric": "serve latency (completion - arrival)", "unit": "s", "data": "synthetic (device-simulated, seeded)",
           "config": {"workload": f"70% DNA GTR+G4 / 30% LG+G4, taxa log-U[8,{args.max_taxa}], "
                                  f"sites log-U[500,{args.max_sites}], lnL + 1 round of branch NR",
                      "max_active": args.max_active, "jobs_generated": njobs, "generation_s": t_gen}}
    lnl = {}

    def run(name, prec, rate, n):
        srv = serving.Server(max_active=args.max_active)
        res, wall = serving.poisson_stream(srv, jobs[:n], rate, args.seed, precision=prec)
        st = srv.stats()
        srv.close()
        ok = [r for r in res if r["status"] == 0]
        lat = np.array([r["latency"] for r in ok])
        qw = np.array([r["queue_wait"] for r in ok])
        lnl.setdefault(name, {}).update({r["id"] - res[0]["id"]: r["lnl_initial"] for r in ok})
        return {"rate_per_s": rate, "requests": n, "completed": len(ok), "refused": st["refused"],
                "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
                "p50_queue_wait_s": float(np.percentile(qw, 50)) if len(qw) else None,
                "throughput_jobs_per_s": len(ok) / wall, "wall_s": wall, "peak_active": st["peak_active"],
                "peak_hbm_gb": st["peak_bytes"] / 1e9, "arena_gb": st["arena_bytes"] / 1e9,
                "recycled_slot_jobs": sum(1 for r in ok if r["slots"] < 3 * (r["ntaxa"] - 2)),
                "full_traversal_updates": sum((r["ntaxa"] - 2) * r["nptn"] for r in ok)}

    for name, prec in (("mixed_f32", engine.F32), ("fp64", engine.F64)):
        if name == "fp64" and args.no_fp64_serve:
            continue
        out[name] = {"burst": run(name, prec, args.rate, args.requests)}
        steady = (args.steady_rate, args.steady_requests) if prec == engine.F32 else \
            (args.steady_rate_fp64, args.steady_requests_fp64)
        if steady[1] > 0:
            out[name]["steady"] = run(name, prec, *steady)
    if "fp64" in lnl:
        common = set(lnl["fp64"]) & set(lnl["mixed_f32"])
        out["lnl_max_rel_err_mixed_vs_fp64"] = max(
            (abs(lnl["mixed_f32"][k] - lnl["fp64"][k]) / abs(lnl["fp64"][k]) for k in common), default=None)
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="protein", choices=sorted(WORKLOADS))
    ap.add_argument("--mode", default="headline", choices=["headline", "serve", "batched", "branchopt"])
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--max-taxa", type=int, default=2000)
    ap.add_argument("--max-sites", type=int, default=500000)
    ap.add_argument("--max-active", type=int, default=16)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--no-fp64-serve", action="store_true")
    ap.add_argument("--steady-rate", type=float, default=12.0)
    ap.add_argument("--steady-requests", type=int, default=500)
    ap.add_argument("--steady-rate-fp64", type=float, default=0.8)  # FP64 completes ~1.2 of these jobs/s
    ap.add_argument("--steady-requests-fp64", type=int, default=120)
    ap.add_argument("--config", default=None,
                    help="fixed traversal configuration instead of the autotuner, as the autotuner labels it "
                         "(tile/schedule[/sD][/kP], e.g. 0/level/s2/k1)")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the paths reported beside the headline (FP64, CUDA-core FP32, BF16)")
    ap.add_argument("--precision", default="auto", choices=["auto", "f32", "tf32x3"],
                    help="headline contraction: auto = split-TF32 tensor cores for 16..64 states")
    args = ap.parse_args()
    global WORKLOAD
    WORKLOAD = WORKLOADS[args.workload]
    if args.mode == "serve":
        run_serve(args)
    elif args.mode == "batched":
        run_batched(args)
    elif args.mode == "branchopt":  # the DNA 16 x 1,000 all-branch optimisation alone
        print(json.dumps({"mode": "branchopt", **branch_optimisation_dna16(args)}))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
