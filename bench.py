"""Benchmark: AVOS transitive closure on GB300.

Default workload (the batched dense closure): 4096 independent pedigree components with sizes
log-uniform in [16, 4096], generation depth 1.5*log2(n), int32, closed in one batched run per
step.  The metric is AVOS relaxations/s with the algorithmic count sum(n^3) per step (the
reference's C warshall performs all n^3 relaxations of every component).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank closes its own seeded set of 4096 components (weak scaling,
no data-path collective); rank 0 prints one JSON line with the whole-job throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

COUNT, LO, HI, SEED = 4096, 16, 4096, 3
CPU_SAMPLE_RELAX = 6.0e10        # bounded CPU sample: ~10-30 s of C warshall on the host cores
METRIC = "avos_relaxations_per_s"
UNIT = "relax/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    return ap.parse_args()


def workload(rank: int):
    from redblackgraph_gb300 import synth
    sizes, seeds = synth.batch_components(COUNT, LO, HI, seed=SEED + 1000 * rank)
    return sizes, seeds


def config(l2_note: str):
    return {"workload": "batched dense AVOS closure", "components": COUNT,
            "n_range": [LO, HI], "sizes": "log-uniform", "generations": "max(2, round(1.5*log2 n))",
            "parents": "father 2 / mother 3, p=0.9 each, uniform over earlier generations",
            "storage": "int32 dense", "l2": l2_note}


# ------------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling during the timed region (read only; never changes settings)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        self.tmp.flush()
        rows = [r.split(",") for r in Path(self.tmp.name).read_text().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if len(r) > 5 + k and r[5 + k].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


# ------------------------------------------------------------------------------- CPU side
def octave(n):
    return int(np.floor(np.log2(max(int(n), 1))))


def cpu_sample(sizes, budget_per_octave=CPU_SAMPLE_RELAX / 8):
    """Stratified sample: in every size octave [2^k, 2^(k+1)) the smallest components are taken
    until their sum(n^3) reaches the octave budget (at least one per octave)."""
    picked = []
    for k in sorted({octave(n) for n in sizes}):
        members = sorted((int(i) for i in np.flatnonzero([octave(n) == k for n in sizes])),
                         key=lambda i: int(sizes[i]))
        acc = 0.0
        for i in members:
            if picked and acc > 0 and acc + float(sizes[i]) ** 3 > budget_per_octave:
                break
            picked.append(i)
            acc += float(sizes[i]) ** 3
    return picked


def cpu_closure_rate(sizes, seeds, idx, threads=None):
    """Time the oracle's C restatement of the reference's warshall (the CPU baseline) on the
    sampled components, one component per host thread (ctypes releases the GIL), and
    extrapolate each size octave's sum(n^3) by that octave's measured per-core rate.

    Returns (relax/s of the whole workload on `threads` cores, wall seconds of the sample,
    threads, oracle outputs by sample position, matrices)."""
    from oracle import oracle as orc
    from redblackgraph_gb300 import synth
    mats = [synth.pedigree(int(sizes[i]), synth.generations_for(int(sizes[i])), int(seeds[i]),
                           dtype=np.int32) for i in idx]
    threads = threads or os.cpu_count() or 1
    orc.lib()

    def one(k):
        t0 = time.perf_counter()
        res = orc.warshall(mats[k])
        return k, res, time.perf_counter() - t0

    big_first = sorted(range(len(mats)), key=lambda k: -mats[k].shape[0])
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        done = list(ex.map(one, big_first))
    wall = time.perf_counter() - t0
    outs = {k: res for k, res, _ in done}
    per_oct_w, per_oct_t = {}, {}
    for k, _, dt in done:
        o = octave(mats[k].shape[0])
        per_oct_w[o] = per_oct_w.get(o, 0.0) + float(mats[k].shape[0]) ** 3
        per_oct_t[o] = per_oct_t.get(o, 0.0) + dt
    overall = sum(per_oct_t.values()) / sum(per_oct_w.values())
    t_single = 0.0
    for n in sizes:
        o = octave(n)
        t_single += float(n) ** 3 * (per_oct_t[o] / per_oct_w[o] if o in per_oct_w else overall)
    total = float((np.asarray(sizes, dtype=np.float64) ** 3).sum())
    return total / (t_single / threads), wall, threads, outs, mats


# ------------------------------------------------------------------------------- GPU side
def build_device_batch(sizes, seeds, device):
    import torch
    from redblackgraph_gb300 import synth
    idx, val, offsets = synth.batch_edges(sizes, seeds)
    total = int((sizes * sizes).sum())
    buf = torch.zeros(total, dtype=torch.int32, device=device)
    buf[torch.from_numpy(idx).to(device)] = torch.from_numpy(val.astype(np.int32)).to(device)
    return buf, offsets


def int32_peak_ops(device_index: int, sm_max_mhz):
    """Nominal int32 lane throughput: SMs x 128 lanes x maximum SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(device_index).multi_processor_count
    mhz = sm_max_mhz or 2070.0
    return sms * 128 * mhz * 1e6, sms


def tile_traffic_per_launch():
    p = ROOT / "profiles" / "fw_tile_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("bytes_per_launch")
        except (ValueError, OSError):
            return None
    return None


def profile_kernels(fn):
    """Run fn() with the library's per-kernel CUDA-event timers on; returns {kernel: (ms, n)}."""
    import ctypes
    from redblackgraph_gb300 import _lib
    L = _lib.load()
    L.rbg_profile_begin()
    fn()
    ms = (ctypes.c_double * 4)()
    n = (ctypes.c_int64 * 4)()
    _lib.check(L.rbg_profile_end(ms, n), "profile")
    names = ["fw_tile_kernel", "fw_panel_kernel", "fw_diag_kernel", "convert/finalize"]
    return {names[k]: (ms[k], int(n[k])) for k in range(4)}


def run_ours(args, rank, world):
    import torch
    import torch.distributed as dist
    from redblackgraph_gb300 import _lib
    from redblackgraph_gb300.dense import fw_batch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    dev = torch.device("cuda", torch.cuda.current_device())
    L = _lib.load()
    sizes, seeds = workload(rank)
    work_per_step = float((sizes.astype(np.float64) ** 3).sum())
    buf, offsets = build_device_batch(sizes, seeds, dev)
    out = torch.empty_like(buf)

    results = None
    for _ in range(max(args.warmup, 3) if args.warmup >= 3 else 3):
        out, results = fw_batch(buf, sizes, offsets, out=out)
    assert all(r.status == 0 for r in results), "closure reported an error"
    executed = float(sum(r.executed for r in results))

    stream = torch.cuda.current_stream()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = L.rbg_launch_count()
    with ClockSampler(dev.index) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        kprof = profile_kernels(lambda: [fw_batch(buf, sizes, offsets, out=out)
                                         for _ in range(args.steps)])
        e1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    launches = L.rbg_launch_count() - launches0
    t = e0.elapsed_time(e1) / 1e3
    if world > 1:
        tt = torch.tensor([t], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    clocks = clk.summary()
    return dict(t=t, work=work_per_step, executed=executed, kprof=kprof, launches=launches,
                clocks=clocks, sizes=sizes, seeds=seeds, out=out, offsets=offsets,
                bytes=buf.numel() * 4)


def sample_parity(sizes, offsets, out, cpu_outs, idx, mats):
    """The GPU closures of the CPU-sample components against the oracle's (bit-exact)."""
    from redblackgraph_gb300.device import to_host
    ok = True
    for k, i in enumerate(idx):
        n, o = int(sizes[i]), int(offsets[i])
        W = to_host(out[o:o + n * n]).reshape(n, n)
        Wo = cpu_outs[k][0]
        ok &= bool((W == Wo).all())
    return ok


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        return main_reference(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    r = run_ours(args, rank, world)
    total_work = r["work"] * args.steps * world
    value = total_work / r["t"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["t"] / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded pedigree components generated in-process",
            "config": config(f"inputs larger than L2: {r['bytes'] / 1e9:.1f} GB resident per step"),
            "gpu_launches": int(r["launches"]), "clocks": r["clocks"]}
    # roofline of the dominant kernel (phase-3 tile kernel): int32 lane operations
    tms, tn = r["kprof"]["fw_tile_kernel"]
    peak, sms = int32_peak_ops(0, r["clocks"].get("sm_max_mhz"))
    tile_relax_per_step = r["executed"]
    line["roofline"] = {
        "bound": "int32_alu", "unit": "Tops/s",
        "achieved": None, "peak": peak / 1e12, "frac": None,
        "traffic": tile_traffic_per_launch(),
        "peak_source": f"nominal: {sms} SMs x 128 int32 lanes x max SM clock",
        "ops_per_relaxation": 2,
        "kernel_ms_per_step": {k: v[0] / args.steps for k, v in r["kprof"].items()},
        "kernel_launches_per_step": {k: v[1] / args.steps for k, v in r["kprof"].items()},
        "executed_relaxations_per_step": tile_relax_per_step,
        "algorithmic_relaxations_per_step": r["work"],
    }
    if tms > 0:
        ach = tile_relax_per_step * 2 / (tms / args.steps / 1e3) / 1e12
        line["roofline"]["achieved"] = ach
        line["roofline"]["frac"] = ach / (peak / 1e12)
    if rank == 0:
        idx = cpu_sample(r["sizes"])
        rate, tcpu, threads, outs, mats = cpu_closure_rate(r["sizes"], r["seeds"], idx)
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(idx)} of {COUNT} components (smallest of every size octave up to "
                      f"{CPU_SAMPLE_RELAX / 8:.1e} relaxations per octave, sum n^3 = "
                      f"{sum(int(r['sizes'][i]) ** 3 for i in idx):.3e}) closed in {tcpu:.1f} s "
                      "by the C restatement of the reference warshall, one component per host "
                      "thread; each octave's sum(n^3) extrapolated by its measured rate",
            "sample_bit_exact_vs_gpu": sample_parity(r["sizes"], r["offsets"], r["out"], outs, idx, mats)}
        line["e2e"] = None
        print(json.dumps(line))


def main_reference(args, rank, world):
    if rank != 0:
        return
    sizes, seeds = workload(0)
    idx = cpu_sample(sizes)
    work = float(sum(int(sizes[i]) ** 3 for i in idx))
    rates, total_t = [], 0.0
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_closure_rate(sizes, seeds, idx[: max(1, len(idx) // 8)], threads)
    for _ in range(args.steps):
        rate, t, threads, _, _ = cpu_closure_rate(sizes, seeds, idx, threads)
        rates.append(rate)
        total_t += t
    value = statistics.median(rates)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded pedigree components generated in-process",
            "config": config("CPU run"), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{len(idx)} of {COUNT} components per step (smallest of "
                                       f"every size octave, sum n^3 = {work:.3e}); C restatement "
                                       "of the reference's warshall (core C gufunc), one "
                                       "component per host thread, each octave extrapolated by "
                                       "its measured rate"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
