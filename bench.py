"""Benchmark: AVOS transitive closure on GB300.

Default workload (the batched dense closure): 4096 seeded pedigrees with sizes log-uniform in
[16, 4096] and generation depth 1.5*log2(n), laid out as one block-diagonal forest (int32).
Its connected components (a pedigree may hold isolated founders, so there are more components
than pedigrees) are closed in one batched run per step.  The metric is AVOS relaxations/s with
the algorithmic count sum(n^3) over the components (the reference's C warshall performs all n^3
relaxations of every component).

  value  batched closure with the dense blocks resident in HBM (CUDA events on the stream);
         every component is numbered oldest first, so the batch takes the DAG path
  e2e    component_wise_closure on the forest in pinned host memory: CSR upload, component
         split, the closure straight from the CSR graph and download of the merged CSR per step

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank closes its own seeded forest (weak scaling, no data-path
collective); rank 0 prints one JSON line with the whole-job throughput.
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
# int32 operations per dense AVOS relaxation in the ALU roofline (shift, and, or for the product,
# min for the sum); the blocked kernels execute 2 (IMAD + IMNMX) after their lane encoding
OPS_PER_RELAXATION = 4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--count", type=int, default=COUNT,
                    help="pedigrees in the forest (smaller values: profiling cases)")
    ap.add_argument("--hi", type=int, default=HI, help="largest pedigree size")
    ap.add_argument("--serve", type=int, default=1, help="also run the serving workload (0: skip)")
    ap.add_argument("--serve-count", type=int, default=0, help="requests in the serving stream")
    ap.add_argument("--only", choices=["spgemm", "dag", "compose", "single", "serve", "anynum", "dense", "matmul"],
                    default=None,
                    help="run one secondary workload alone and print its JSON (profiling cases)")
    ap.add_argument("--secondary", type=int, default=1,
                    help="also measure the per-component plain path, one n=8192 int64 closure and "
                         "the 2M-vertex squaring SpGEMM (0: skip)")
    args = ap.parse_args()
    globals()["COUNT"], globals()["HI"] = args.count, args.hi
    return args


def workload(rank: int):
    """The 4096 seeded pedigrees as one block-diagonal forest, and its connected components
    (numbered by least vertex, vertices ascending) found on the host by scipy."""
    from scipy.sparse.csgraph import connected_components
    from redblackgraph_gb300 import synth
    sizes, seeds = synth.batch_components(COUNT, LO, HI, seed=SEED + 1000 * rank)
    forest, base = synth.batch_forest(sizes, seeds)
    k, lab = connected_components(forest, directed=True, connection="weak")
    order = np.argsort(lab, kind="stable")
    csizes = np.bincount(lab, minlength=k).astype(np.int64)
    cstart = np.concatenate([[0], np.cumsum(csizes)])
    return dict(sizes=sizes, seeds=seeds, forest=forest, csizes=csizes, cstart=cstart, order=order)


def config(w=None):
    c = {"workload": "batched dense AVOS closure", "pedigrees": COUNT,
         "n_range": [LO, HI], "sizes": "log-uniform", "generations": "max(2, round(1.5*log2 n))",
         "parents": "father 2 / mother 3, p=0.9 each, uniform over earlier generations",
         "storage": "int32 dense"}
    if w is not None:
        c["components"] = int(w["csizes"].size)
        c["vertices"] = int(w["forest"].shape[0])
        c["components_note"] = ("connected components of the forest of the pedigrees (a pedigree "
                                "can hold isolated founders); the work is their sum n^3")
    return c


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
    until their sum(n^3) reaches the octave budget or 64 are taken (at least one per octave)."""
    picked = []
    for k in sorted({octave(n) for n in sizes}):
        members = sorted((int(i) for i in np.flatnonzero([octave(n) == k for n in sizes])),
                         key=lambda i: int(sizes[i]))
        acc, m = 0.0, 0
        for i in members:
            if picked and acc > 0 and (acc + float(sizes[i]) ** 3 > budget_per_octave or m >= 64):
                break
            picked.append(i)
            acc += float(sizes[i]) ** 3
            m += 1
    return picked


def component_matrix(w, c):
    """Dense int32 matrix of connected component c of the forest (vertices ascending)."""
    v = w["order"][w["cstart"][c]:w["cstart"][c + 1]]
    return w["forest"][v][:, v].toarray().astype(np.int32)


def cpu_closure_rate(w, idx, threads=None):
    """Time the oracle's C restatement of the reference's warshall (the CPU baseline) on the
    sampled components, one component per host thread (ctypes releases the GIL), and
    extrapolate each size octave's sum(n^3) by that octave's measured per-core rate.

    Returns (relax/s of the whole workload on `threads` cores, wall seconds of the sample,
    threads, oracle outputs by sample position)."""
    from oracle import oracle as orc
    sizes = w["csizes"]
    mats = [component_matrix(w, int(i)) for i in idx]
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
    return total / (t_single / threads), wall, threads, outs


# ------------------------------------------------------------------------------- GPU side
def build_device_batch(w, device):
    """Split the forest into components and densify them with the library's own component
    path (the same calls component_wise_closure makes); checks the split against the host's."""
    import torch
    from redblackgraph_gb300.components import label_components, densify
    from redblackgraph_gb300.device import to_device
    f = w["forest"]
    ip = to_device(f.indptr.astype(np.int64), device)
    ij = to_device(f.indices.astype(np.int32), device)
    iv = to_device(f.data.astype(np.int32), device)
    comps = label_components(ip, ij, f.shape[0])
    assert comps.count == w["csizes"].size and (comps.sizes == w["csizes"]).all(), \
        "device component split differs from the host's"
    blocks = densify(ip, ij, iv, comps)
    torch.cuda.synchronize()
    return blocks


def run_matmul(n=4096, seed=9, steps=5):
    """The dense AVOS product (rb.array @, rbg_avos_matmul) on its natural operands: the closure
    W of one n=4096 pedigree (int32, 18 generations) times the pedigree's own matrix A, the step
    that extends every ancestor path by one generation.  n^3 products per call; ALU roofline at
    OPS_PER_RELAXATION int32 operations per product (the product's shift, and, or, and the sum's
    min).  The same product for a 512-vertex pedigree is checked against the oracle's C-core
    product."""
    import torch
    from oracle import oracle as orc
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.core.avos import matmul_device
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    stream = torch.cuda.current_stream()
    A = synth.pedigree(n, synth.generations_for(n), seed, dtype=np.int32)
    da = to_device(A)
    W, res = fw_dense(da)
    torch.cuda.synchronize()
    out = torch.empty_like(W)
    for _ in range(2):
        _, rc, _ = matmul_device(W, da, out=out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        _, rc, flags = matmul_device(W, da, out=out)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / steps
    As = synth.pedigree(512, synth.generations_for(512), seed + 1, dtype=np.int32)
    das = to_device(As)
    Ws, _ = fw_dense(das)
    Cs, rcs, _ = matmul_device(Ws, das)
    torch.cuda.synchronize()
    C, st, _ = orc.matmul(to_host(Ws), As)
    exact = bool(rc == 0 and rcs == 0 and st == 0 and (to_host(Cs) == C).all())
    peak, sms = int32_peak_ops(0, None)
    ach = float(n) ** 3 * OPS_PER_RELAXATION / t / 1e12
    return {"workload": f"W (x) A: W the closure of one pedigree, n={n}, {synth.generations_for(n)} generations, "
                        "A its matrix, int32",
            "value": float(n) ** 3 / t, "unit": "products/s", "ms": t * 1e3, "status": int(rc),
            "roofline": {"bound": "int32_alu", "unit": "Tops/s", "achieved": ach, "peak": peak / 1e12,
                         "frac": ach / (peak / 1e12), "kernel": "rbg_avos_matmul",
                         "ops_per_product": OPS_PER_RELAXATION,
                         "peak_source": f"nominal: {sms} SMs x 128 int32 lanes x max SM clock"},
            "bit_exact_vs_oracle_n512": exact}


def int32_peak_ops(device_index: int, sm_max_mhz):
    """Nominal int32 lane throughput: SMs x 128 lanes x maximum SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(device_index).multi_processor_count
    mhz = sm_max_mhz or 2070.0
    return sms * 128 * mhz * 1e6, sms


def scan_traffic(algorithmic_bytes):
    """DRAM bytes of the full-size scan and write launches: the committed ncu capture of a
    smaller batch, scaled by dense cells (their traffic grows with the cells they read and
    write)."""
    p = ROOT / "profiles" / "tri_scan_kernel_traffic.txt"
    try:
        d = json.loads(p.read_text())
        return d["dram_bytes_per_launch"] * algorithmic_bytes / d["algorithmic_bytes_per_launch"]
    except (ValueError, OSError, KeyError, ZeroDivisionError):
        return None


def phase_traffic():
    """DRAM bytes per launch of the phase kernels, from the committed ncu capture summary."""
    p = ROOT / "profiles" / "fw_phase_traffic.txt"
    try:
        return json.loads(p.read_text())
    except (ValueError, OSError):
        return None


def profile_kernels(fn):
    """Run fn() with the library's per-kernel CUDA-event timers on; returns {kernel: (ms, n)}."""
    import ctypes
    from redblackgraph_gb300 import _lib
    L = _lib.load()
    L.rbg_profile_begin()
    fn()
    ms = (ctypes.c_double * 9)()
    n = (ctypes.c_int64 * 9)()
    _lib.check(L.rbg_profile_end_slots(ms, n, 9), "profile")
    names = ["fw_tile_kernel", "fw_panel_kernel", "fw_diag_kernel", "convert/finalize",
             "tri_scan_kernel", "dag_closure", "tri_stats_kernel", "tri_write_kernel", "any_numbering_replay"]
    return {names[k]: (ms[k], int(n[k])) for k in range(9)}


def run_ours(args, rank, world, w):
    import torch
    import torch.distributed as dist
    from redblackgraph_gb300.sharding import max_over_ranks
    from redblackgraph_gb300 import _lib
    from redblackgraph_gb300.dense import fw_batch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    dev = torch.device("cuda", torch.cuda.current_device())
    L = _lib.load()
    blocks = build_device_batch(w, dev)
    sizes, offsets, buf = blocks.sizes, blocks.offsets, blocks.flat
    work_per_step = float((sizes.astype(np.float64) ** 3).sum())
    out = torch.empty_like(buf)

    results = None
    # the first warm-up call tunes the tile shape of every round (closing the batch with both
    # shapes); later calls replay the tuned launch sequence as a CUDA graph
    mode = _lib.MODE_GRAPH | _lib.MODE_AUTOTUNE
    for _ in range(max(args.warmup, 3)):
        out, results = fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True)
    assert (results["status"] == 0).all(), "closure reported an error"
    executed = float(results["executed"].sum())

    stream = torch.cuda.current_stream()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = L.rbg_launch_count()
    with ClockSampler(dev.index) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True)
        e1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    launches = L.rbg_launch_count() - launches0
    # per-kernel split from one more step with event timers between the launches (untimed)
    kprof = profile_kernels(lambda: fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True))
    kprof = {k: (v[0] * args.steps, v[1] * args.steps) for k, v in kprof.items()}
    t = e0.elapsed_time(e1) / 1e3
    t = max_over_ranks(t, dev)          # the slowest rank's time (weak scaling)
    clocks = clk.summary()
    paths = {int(p): int((results["path"] == p).sum()) for p in np.unique(results["path"])}
    res = dict(t=t, work=work_per_step, executed=executed, kprof=kprof, launches=launches,
               clocks=clocks, out=out, offsets=offsets, bytes=buf.numel() * 4,
               cells=float((sizes.astype(np.float64) ** 2).sum()), paths=paths)
    if args.secondary and rank == 0:
        res["blocked"] = run_blocked(args, buf, sizes, offsets, out, mode | _lib.MODE_NO_DAG)
    del buf, blocks
    res["e2e"] = run_e2e(args, rank, world, w, dev, work_per_step)
    return res


def run_blocked(args, buf, sizes, offsets, out, mode):
    """The same resident batch on the blocked kernels only (RBG_MODE_NO_DAG): the path every
    matrix takes when its vertices are not numbered in a topological order."""
    import torch
    from redblackgraph_gb300.dense import fw_batch
    for _ in range(3):
        _, res = fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True)
    assert (res["status"] == 0).all()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / args.steps
    kp = profile_kernels(lambda: fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True))
    return dict(t=t, executed=float(res["executed"].sum()), kprof=kp)


def run_e2e(args, rank, world, w, dev, work_per_step):
    """The same closure through the public API with host buffers: component_wise_closure on the
    forest held in pinned host memory (H2D of the CSR, component split, the closure straight
    from the CSR graph -- or, for components not numbered in a topological order, densify,
    batched closure and compaction -- and D2H of the merged CSR inside every timed step)."""
    from redblackgraph_gb300.sharding import max_over_ranks
    import torch
    import torch.distributed as dist
    import scipy.sparse as sp
    from redblackgraph_gb300.sparse import component_wise_closure
    f = w["forest"]

    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory()
        v = t.numpy().view(a.dtype)
        v[:] = a
        return t, v

    keep = [pinned(np.ascontiguousarray(x)) for x in (f.data, f.indices, f.indptr)]
    M = sp.csr_matrix(f.shape, dtype=np.int32)
    M.data, M.indices, M.indptr = keep[0][1], keep[1][1], keep[2][1]   # the pinned arrays themselves
    assert all(np.shares_memory(a, k[1]) for a, k in zip((M.data, M.indices, M.indptr), keep))
    h2d = int(M.data.nbytes + M.indices.nbytes + M.indptr.nbytes)
    steps = max(1, args.steps)
    r = None
    for _ in range(max(args.warmup, 3) if args.warmup > 0 else 3):
        r = component_wise_closure(M)
    stream = torch.cuda.current_stream()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        r = component_wise_closure(M)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    t = max_over_ranks(t, dev)          # the slowest rank's time (weak scaling)
    W = r.W
    d2h = int(W.indptr.nbytes + W.indices.nbytes + W.data.nbytes)   # the merged CSR as copied back
    return dict(t=t, steps=steps, value=work_per_step * steps * world / t, h2d=h2d, d2h=d2h, W=W,
                diameter=int(r.diameter))


def sample_parity(w, offsets, out, cpu_outs, idx, W_e2e=None):
    """The GPU closures of the CPU-sample components against the oracle's (bit-exact), both from
    the batched run and from the public-API run."""
    from redblackgraph_gb300.device import to_host
    ok = True
    for k, i in enumerate(idx):
        n, o = int(w["csizes"][i]), int(offsets[i])
        Wo = cpu_outs[k][0]
        ok &= bool((to_host(out[o:o + n * n]).reshape(n, n) == Wo).all())
        if W_e2e is not None:
            v = w["order"][w["cstart"][i]:w["cstart"][i + 1]]
            ok &= bool((W_e2e[v][:, v].toarray() == Wo).all())
    return ok


def run_plain(w):
    """The same components closed one launch sequence per component (the plain per-graph GPU
    path, ``rbg_fw_dense`` on each block): one timed pass over the batch."""
    import torch
    from redblackgraph_gb300.components import densify, label_components
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device
    f = w["forest"]
    dev = torch.device("cuda", torch.cuda.current_device())
    ip, ij, iv = (to_device(f.indptr.astype(np.int64), dev), to_device(f.indices.astype(np.int32), dev),
                  to_device(f.data.astype(np.int32), dev))
    blocks = densify(ip, ij, iv, label_components(ip, ij, f.shape[0]))
    out = torch.empty_like(blocks.flat)
    views = [(blocks.flat[o:o + n * n].view(n, n), out[o:o + n * n].view(n, n))
             for n, o in zip(blocks.sizes.tolist(), blocks.offsets.tolist())]
    for a, b in views[:64] + views[-64:]:
        fw_dense(a, out=b)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for a, b in views:
        fw_dense(a, out=b)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    work = float((blocks.sizes.astype(np.float64) ** 3).sum())
    del views, out, blocks
    torch.cuda.empty_cache()
    return {"value": work / t, "unit": UNIT, "ms_per_step": t * 1e3,
            "how": "rbg_fw_dense once per component over the same 16,761 blocks, one timed pass"}


def renumbered(w, seed=23):
    """The same forest with every component's vertices renumbered at random (a permutation of
    the component's own vertex ids), so that each dense block has entries on both sides of the
    diagonal: matrices not numbered in a topological order."""
    rng = np.random.default_rng(seed)
    N = w["forest"].shape[0]
    perm = np.arange(N, dtype=np.int64)              # perm[old] = new
    for c in range(w["csizes"].size):
        v = w["order"][w["cstart"][c]:w["cstart"][c + 1]]
        perm[v] = rng.permutation(v)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(N, dtype=np.int64)         # inv[new] = old
    f = w["forest"][inv][:, inv].tocsr()
    f.sort_indices()
    # each component keeps its vertex set, so the components and their ascending vertex lists
    # (w["order"]) are unchanged
    return dict(w, forest=f)


def run_any_numbering(w, steps=5):
    """The headline's components renumbered at random (entries on both sides of the diagonal):
    the DAG path with the sequential loop replayed on each closure's pattern, against the blocked
    kernels on the same batch (the path such matrices took before); a sample of components is
    checked bit-exact against the oracle's sequential loop."""
    import torch
    from oracle import oracle as orc
    from redblackgraph_gb300 import _lib
    from redblackgraph_gb300.dense import fw_batch
    from redblackgraph_gb300.device import to_host
    wr = renumbered(w)
    dev = torch.device("cuda", torch.cuda.current_device())
    blocks = build_device_batch(wr, dev)
    sizes, offsets, buf = blocks.sizes, blocks.offsets, blocks.flat
    work = float((sizes.astype(np.float64) ** 3).sum())
    out = torch.empty_like(buf)
    line = {"how": "rbg_fw_batch on the resident blocks of the same forest with every component's "
                   "vertices renumbered at random (seeded)", "unit": UNIT}
    stream = torch.cuda.current_stream()
    for name, mode in (("dag_path", _lib.MODE_GRAPH), ("blocked_kernels", _lib.MODE_GRAPH | _lib.MODE_NO_DAG)):
        for _ in range(3):
            _, res = fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True)
        assert (res["status"] == 0).all()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / steps
        kp = profile_kernels(lambda: fw_batch(buf, sizes, offsets, out=out, mode=mode, as_array=True))
        paths = {{1: "blocked32", 2: "blocked64", 3: "exact", 4: "dag"}.get(int(p), str(p)):
                 int((res["path"] == p).sum()) for p in np.unique(res["path"])}
        line[name] = {"value": work / t, "ms_per_step": t * 1e3, "paths": paths,
                      "kernel_ms_per_step": {k: v[0] for k, v in kp.items() if v[1]}}
        if name == "dag_path":
            # oracle sample: the largest component of every size octave up to 1024 vertices
            # (seconds of the C restatement of the reference's warshall)
            by_oct = {}
            for i, n in enumerate(sizes.tolist()):
                o = octave(n)
                if n <= 1024 and (o not in by_oct or n > sizes[by_oct[o]]):
                    by_oct[o] = i
            idx = sorted(by_oct.values())
            ok, both = True, 0
            for i in idx:
                n, o = int(sizes[i]), int(offsets[i])
                A = to_host(buf[o:o + n * n]).reshape(n, n)
                both += int(np.tril(A, -1).any() and np.triu(A, 1).any())
                Wo, do, so, _ = orc.warshall(A)
                ok &= so == 0 and int(res["diameter"][i]) == do
                ok &= bool((to_host(out[o:o + n * n]).reshape(n, n) == Wo).all())
            line[name]["sample_bit_exact_vs_oracle"] = bool(ok)
            line[name]["sample"] = (f"{len(idx)} components, the largest of every size octave up to 1024 "
                                    f"vertices; {both} of them with entries on both sides of the diagonal")
    line["dag_vs_blocked"] = line["blocked_kernels"]["ms_per_step"] / line["dag_path"]["ms_per_step"]
    del buf, blocks, out
    torch.cuda.empty_cache()
    return line


def dense_layered_dag(n, layers, p, seed, dtype=np.int32):
    """A dense DAG the DAG path does not take (rows of hundreds of entries): vertices in `layers`
    layers numbered in layer order, every vertex linked to each vertex of an earlier layer with
    probability p (values 2 / 3), diagonal +-1.  Its closure is dense and its values stay below
    bit `layers` (one bit per edge of a path)."""
    rng = np.random.default_rng(seed)
    layer = np.sort(rng.integers(0, layers, size=n))
    link = (layer[:, None] > layer[None, :]) & (rng.random((n, n)) < p)
    A = np.where(link, rng.integers(2, 4, size=(n, n)), 0).astype(dtype)
    np.fill_diagonal(A, rng.choice(np.array([-1, 1], dtype=dtype), size=n))
    return A


def run_dense_blocked(n=4096, layers=24, p=0.5, seed=5, steps=5):
    """The blocked Floyd-Warshall kernels on the workload they exist for: one dense layered DAG
    (n=4096, int32; every row has hundreds of entries, so the DAG path declines it), whose
    closure is dense, so nearly every tile item runs all 64 steps of its round.  ALU roofline on
    the executed relaxations; a 1024-vertex instance of the same generator is checked bit-exact
    against the oracle's sequential loop."""
    import torch
    from oracle import oracle as orc
    from redblackgraph_gb300 import _lib
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    stream = torch.cuda.current_stream()
    small = dense_layered_dag(1024, layers, p, seed + 1)
    Wo, do, so, _ = orc.warshall(small)
    ds = to_device(small)
    Ws, rs = fw_dense(ds)
    torch.cuda.synchronize()
    exact = bool(so == 0 and rs.status == 0 and rs.diameter == do and (to_host(Ws) == Wo).all())
    A = dense_layered_dag(n, layers, p, seed)
    d = to_device(A)
    out = torch.empty_like(d)
    for _ in range(3):
        _, res = fw_dense(d, out=out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fw_dense(d, out=out)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / steps
    kp = {k: v for k, v in profile_kernels(lambda: fw_dense(d, out=out)).items() if v[1]}
    phase_ms = sum(kp[k][0] for k in ("fw_tile_kernel", "fw_panel_kernel", "fw_diag_kernel") if k in kp)
    peak, sms = int32_peak_ops(0, None)
    alu = res.executed * OPS_PER_RELAXATION / (phase_ms / 1e3) / 1e12 if phase_ms else None
    nnz_out = int(np.count_nonzero(to_host(out)))
    return {"workload": f"one dense layered DAG, n={n}, {layers} layers, link probability {p}, int32 "
                        f"({int(np.count_nonzero(A)) / n:.0f} entries per row, {nnz_out / n / n:.0%} of the "
                        "closure non-zero)",
            "value": n ** 3 / t, "unit": UNIT, "ms": t * 1e3, "path": int(res.path), "status": int(res.status),
            "diameter": int(res.diameter), "executed_relaxations": int(res.executed),
            "roofline": {"bound": "int32_alu", "unit": "Tops/s", "achieved": alu, "peak": peak / 1e12,
                         "frac": alu / (peak / 1e12) if alu else None,
                         "kernel": "fw_diag_kernel + fw_panel_kernel + fw_tile_kernel",
                         "ops_per_relaxation": OPS_PER_RELAXATION,
                         "peak_source": f"nominal: {sms} SMs x 128 int32 lanes x max SM clock"},
            "kernel_ms": {k: v[0] for k, v in kp.items()},
            "bit_exact_vs_oracle_n1024": exact}


def fullsize_fixture(name):
    """The digest helpers and the reference's digests of one bench input (tests/golden/
    fullsize.json, made by running the reference's own CPU code on that input)."""
    import importlib.util
    gold = ROOT / "tests" / "golden"
    spec = importlib.util.spec_from_file_location("make_fullsize", gold / "make_fullsize.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    try:
        fx = json.loads((gold / "fullsize.json").read_text()).get(name)
    except (OSError, ValueError):
        fx = None
    return mk, fx


def run_single_dense(n=8192, generations=30, seed=1, steps=5):
    """One dense closure of a single n=8192, 30-generation pedigree with int64 entries (what
    rb.array(A).transitive_closure() runs), on the DAG path (the pedigree is numbered oldest
    first; RBG_MODE_GRAPH: one graph launch per call) and on the blocked kernels
    (RBG_MODE_NO_DAG), each checked against the digest and diameter of the reference's own
    warshall on the same input."""
    import torch
    from oracle import oracle as orc
    from redblackgraph_gb300 import _lib, synth
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    A = synth.pedigree(n, generations, seed, dtype=np.int64)
    mk, fx = fullsize_fixture("dense8192")
    input_ok = bool(fx) and mk.dense_digest(A) == fx["input_sha256"]
    d = to_device(A)
    out = torch.empty_like(d)
    stream = torch.cuda.current_stream()

    def timed(mode):
        for _ in range(3):
            _, res = fw_dense(d, out=out, mode=mode)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            _, res = fw_dense(d, out=out, mode=mode)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / steps
        kp = profile_kernels(lambda: fw_dense(d, out=out, mode=mode))
        W = to_host(out)
        exact = bool(input_ok and mk.dense_digest(W) == fx["closure_sha256"] and res.diameter == fx["diameter"])
        return t, res, {k: v for k, v in kp.items() if v[1]}, exact

    t_dag, r_dag, kp_dag, ok_dag = timed(_lib.MODE_GRAPH)
    t_blk, r_blk, kp_blk, ok_blk = timed(_lib.MODE_NO_DAG)
    hbm = hbm_peak_gbs()
    io_bytes = 16.0 * n * n                     # every int64 cell read once and written once
    hbm_ms = sum(kp_dag[k][0] for k in ("tri_scan_kernel", "tri_write_kernel") if k in kp_dag)
    ach = io_bytes / (hbm_ms / 1e3) / 1e9 if hbm_ms else None
    phase_ms = sum(kp_blk[k][0] for k in ("fw_tile_kernel", "fw_panel_kernel", "fw_diag_kernel") if k in kp_blk)
    peak, sms = int32_peak_ops(0, None)
    alu = r_blk.executed * OPS_PER_RELAXATION / (phase_ms / 1e3) / 1e12 if phase_ms else None
    # CPU: the C restatement of the reference warshall at n=1024 (int64), extrapolated by n^3
    m = 1024
    B = synth.pedigree(m, generations_for_small(m), seed, dtype=np.int64)
    orc.lib()
    t0 = time.perf_counter()
    orc.warshall(B)
    tc = time.perf_counter() - t0
    cpu_rate = m ** 3 / tc
    return {"workload": f"one pedigree, n={n}, {generations} generations, int64 entries",
            "value": n ** 3 / t_dag, "unit": UNIT, "ms": t_dag * 1e3, "path": int(r_dag.path),
            "diameter": int(r_dag.diameter), "status": int(r_dag.status),
            "bit_exact_vs_reference_fixture": ok_dag,
            "roofline": {"bound": "hbm", "unit": "GB/s", "kernel": "tri_scan_kernel + tri_write_kernel",
                         "achieved": ach, "peak": hbm, "frac": ach / hbm if ach else None,
                         "algorithmic_bytes_per_launch": io_bytes,
                         "step_gb_s": io_bytes / t_dag / 1e9, "step_frac": io_bytes / t_dag / 1e9 / hbm,
                         "kernel_ms": {k: v[0] for k, v in kp_dag.items()},
                         "note": "the closure by levels and the statistics (latency-bound) take the "
                                 "rest of the step"},
            "blocked_kernels": {"value": n ** 3 / t_blk, "unit": UNIT, "ms": t_blk * 1e3,
                                "path": int(r_blk.path), "bit_exact_vs_reference_fixture": ok_blk,
                                "roofline": {"bound": "int32_alu", "unit": "Tops/s", "achieved": alu,
                                             "peak": peak / 1e12, "frac": alu / (peak / 1e12) if alu else None,
                                             "kernel": "fw_diag_kernel + fw_panel_kernel + fw_tile_kernel",
                                             "ops_per_relaxation": OPS_PER_RELAXATION,
                                             "executed_relaxations": int(r_blk.executed),
                                             "peak_source": f"nominal: {sms} SMs x 128 int32 lanes x max SM clock"},
                                "kernel_ms": {k: v[0] for k, v in kp_blk.items()}},
            "reference_full_run_s": fx.get("reference_seconds") if fx else None,
            "reference_full_run_note": "the reference's compiled C warshall on the whole input, one x86 "
                                       "core of the build container (tests/golden/make_fullsize.py)",
            "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"C restatement of the reference warshall, one n={m} int64 "
                                       f"pedigree in {tc:.1f} s; n^3 extrapolation"}}


def run_compose(n=8192, family=128, ops=16, seed=11):
    """Incremental closure updates (relational composition) on one resident closed forest of
    n=8192 vertices in families of 128 (int32), against closing the graph again: `ops` edge
    compositions in place, each joining the founder of an untouched family to a deep vertex of
    another (every descendant of the founder gains that vertex's ancestors), then `ops` vertex
    compositions growing the buffer in place (a new vertex with two parents in one family and an
    untouched family's founder as its child).  Per-operation host wall time (the call synchronises)
    and entries rewritten; the first edge and the first vertex composition are checked against
    the oracle's restatement of the C core gufuncs on the full matrix."""
    import torch
    from oracle import oracle as orc
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.composition import edge_compose_device, vertex_compose_device
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device
    A = synth.forest(n, 12, seed, family=family, reach=3, dtype=np.int32).toarray()
    d = to_device(A)
    W = torch.empty_like(d)
    for _ in range(3):
        fw_dense(d, out=W)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    _, res = fw_dense(d, out=W)
    e1.record(stream)
    torch.cuda.synchronize()
    t_close = e0.elapsed_time(e1)
    Wh = W.cpu().numpy()
    fams = n // family
    rng = np.random.default_rng(seed)
    order = rng.permutation(fams)
    diag = np.diag(Wh)
    buf = torch.zeros((n + ops, n + ops), dtype=torch.int32, device="cuda")
    buf[:n, :n] = W
    R = buf[:n, :n]
    first_ok = []
    edge_ms, edge_upd, vert_ms, vert_upd = [], [], [], []
    # edges: founder of family X (position 0) gains a deep vertex of family Y as a parent
    for t in range(ops):
        X, Y = int(order[2 * t]), int(order[2 * t + 1])
        a = X * family
        b = Y * family + family - 1 - int(rng.integers(0, 8))
        rel = 2 if diag[b] == -1 else 3
        if t == 0:
            exp, info = orc.edge_compose(Wh, a, b, rel)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, res = edge_compose_device(R, a, b, rel, out=R)
        edge_ms.append((time.perf_counter() - t0) * 1e3)
        edge_upd.append(int(res.updated))
        if t == 0:
            first_ok.append(bool(info[0] == 0 and res.status == 0 and (R.cpu().numpy() == exp).all()))
    # vertices: parents in family X (two deep vertices), child = founder of untouched family Z
    base = 2 * ops
    for t in range(ops):
        m = n + t
        X, Z = int(order[base + 2 * t]), int(order[base + 2 * t + 1])
        f = X * family + family - 1
        while diag[f] != -1:
            f -= 1
        mo = X * family + family - 1
        while diag[mo] != 1:
            mo -= 1
        c = Z * family
        color = -1 if t % 2 == 0 else 1
        u = torch.zeros(m, dtype=torch.int32, device="cuda")
        v = torch.zeros(m, dtype=torch.int32, device="cuda")
        u[f], u[mo] = 2, 3
        v[c] = 2 if color == -1 else 3
        if t == 0:
            Rh = buf[:m, :m].cpu().numpy()
            exp, info = orc.vertex_compose(Rh, u.cpu().numpy(), v.cpu().numpy(), color)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, res = vertex_compose_device(buf, u, v, color, out=buf, n=m)
        vert_ms.append((time.perf_counter() - t0) * 1e3)
        vert_upd.append(int(res.updated))
        if t == 0:
            first_ok.append(bool(info[0] == 0 and res.status == 0 and (buf[:m + 1, :m + 1].cpu().numpy() == exp).all()))
    return {"workload": f"closed forest, n={n}, families of {family}, int32; {ops} edge and {ops} vertex "
                        "compositions in place",
            "recompute_closure_ms": t_close,
            "edge_ms_median": statistics.median(edge_ms), "edge_updated_median": statistics.median(edge_upd),
            "vertex_ms_median": statistics.median(vert_ms), "vertex_updated_median": statistics.median(vert_upd),
            "edge_vs_recompute": t_close / statistics.median(edge_ms),
            "first_ops_bit_exact_vs_oracle": all(first_ok)}


def generations_for_small(m):
    from redblackgraph_gb300 import synth
    return synth.generations_for(m)


def run_spgemm_forest(seed=7):
    """Closure by repeated squaring (R <- R (+) R^2 until R is stable) of a 2,000,000-vertex
    pedigree forest (25 generations, int64 values, int32 indices), resident on the device: per
    squaring the time, the algorithmic bytes (12 nnz(A) + 8(n+1) + 12 products + 12 nnz(C) +
    8(n+1)) and the achieved GB/s against the measured HBM copy bandwidth."""
    import torch
    from oracle import oracle as orc
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.spgemm import DeviceCSR, SEM_C64, spgemm
    A = synth.forest(2_000_000, 25, seed, family=64, reach=3, p_parent=0.97, dtype=np.int64)
    n = A.shape[0]
    R0 = DeviceCSR.from_scipy(A)
    stream = torch.cuda.current_stream()

    def closure(rec):
        R = R0
        for it in range(64):
            st = {}
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            Rn, rc, _ = spgemm(R, R, R=R, sem=SEM_C64, stats=st)
            e1.record(stream)
            rec.append((e0, e1, R.nnz, Rn.nnz, st["products"]))
            if rc != 0:
                raise OverflowError("squaring overflowed")
            if Rn.equal(R):
                return Rn, it + 1
            R = Rn
        return R, 64

    closure([])                                 # warm-up
    torch.cuda.synchronize()
    rec = []
    R, iters = closure(rec)
    torch.cuda.synchronize()
    mk, fx = fullsize_fixture("forest2m")
    fixed_point_ok = bool(fx) and mk.csr_digest(A) == fx["input_sha256"] and \
        mk.csr_digest(R.to_scipy()) == fx["closure_sha256"]
    # the same loop in its semi-naive form (squaring_closure: R (+) D R (+) R D once the last step
    # changed at most half of R), timed end to end on the stream, host decisions included
    from redblackgraph_gb300.spgemm import squaring_closure
    squaring_closure(R0, sem=SEM_C64, seminaive=True)           # warm-up
    torch.cuda.synchronize()
    steps = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    Rs, changed = squaring_closure(R0, sem=SEM_C64, steps=steps, seminaive=True)
    e1.record(stream)
    torch.cuda.synchronize()
    semi_ms = e0.elapsed_time(e1)
    semi_ok = bool(fx) and mk.csr_digest(Rs.to_scipy()) == fx["closure_sha256"]
    peak = hbm_peak_gbs()
    rows, tb, tms = [], 0.0, 0.0
    for e0, e1, nnz_a, nnz_c, prods in rec:
        ms = e0.elapsed_time(e1)
        b = 12.0 * nnz_a + 8.0 * (n + 1) + 12.0 * prods + 12.0 * nnz_c + 8.0 * (n + 1)
        rows.append({"ms": round(ms, 3), "nnz_in": nnz_a, "products": prods, "nnz_out": nnz_c,
                     "algorithmic_gb": round(b / 1e9, 3), "gb_s": round(b / (ms / 1e3) / 1e9, 1)})
        tb += b
        tms += ms
    # the first squaring against the oracle's C restatement of rb_matrix @ and the merge
    from redblackgraph_gb300.spgemm import DeviceCSR as _D
    first = _D.from_scipy(A)
    C1, _, _ = spgemm(first, first, R=first, sem=SEM_C64)
    t1 = time.perf_counter()
    P, _ = orc.rb_matmul_csr(A, A)
    tcpu = time.perf_counter() - t1
    Pm = P.tocsr()
    Pm.sort_indices()
    got = C1.to_scipy()
    merged = _merge_minabs_host(A, Pm)
    same = bool((got != merged).nnz == 0)
    return {"workload": f"pedigree forest, n={n}, 25 generations, nnz(A)={A.nnz} "
                        f"({(A.nnz - n) / n:.2f} parent edges per vertex), int64 values, int32 indices",
            "squarings": rows, "iterations": iters, "total_ms": tms,
            "value": tb / (tms / 1e3) / 1e9, "unit": "GB/s",
            "roofline": {"bound": "hbm", "achieved": tb / (tms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": tb / (tms / 1e3) / 1e9 / peak, "peak_source": "measured copy bandwidth"},
            "first_squaring_bit_exact_vs_oracle": same,
            "bit_exact_vs_reference_fixture": fixed_point_ok,
            "semi_naive": {"total_ms": semi_ms, "changing_steps": changed,
                           "steps": [{"form": f, "products": pr, "nnz_in": a, "nnz_out": b} for f, pr, a, b in steps],
                           "products": int(sum(x[1] for x in steps)),
                           "full_squaring_products": int(sum(r["products"] for r in rows)),
                           "vs_full_squaring_loop": (tms / semi_ms) if semi_ms > 0 else None,
                           "how": "redblackgraph_gb300.spgemm.squaring_closure(seminaive=True), an option "
                                  "(the drop-ins run the plain loop): the same R after every step, CUDA events "
                                  "around the whole loop (diff kernels and host decisions included); slower "
                                  "than the plain loop here because every step still merges all of R and "
                                  "computes its difference",
                           "bit_exact_vs_reference_fixture": semi_ok},
            "fixture_note": "the squaring's fixed point against the digest of the reference's Cython DAG "
                            "closure of the same forest (tests/golden/fullsize.json)",
            "cpu_baseline": {"first_product_s": tcpu, "gpu_first_squaring_ms": rows[0]["ms"],
                             "cores": 1, "kind": "port",
                             "sample": "C restatement of rb_matrix @ (pass 1/2) on A @ A"}}


def run_dag_forest(seed=7):
    """Closure of the same 2,000,000-vertex pedigree forest by topological levels (rbg_dag_closure
    then rbg_dag_gather: the reference's parents-first DAG closure with int32 values), timed with
    CUDA events from the resident CSR to the resident closure CSR.  Algorithmic bytes: A once
    (12 nnz(A) + 8 (n + 1)), every candidate once (8 per parent-row entry, 12 per parent edge for
    that row's position), the closure rows written to the pool (8 nnz(C)), then read and written
    as the CSR (16 nnz(C) + 8 (n + 1)).  Checked against the digest and diameter of the
    reference's Cython DAG closure of the same forest."""
    import torch
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.dag import dag_closure_device
    from redblackgraph_gb300.spgemm import DeviceCSR
    A = synth.forest(2_000_000, 25, seed, family=64, reach=3, p_parent=0.97, dtype=np.int32)
    n = A.shape[0]
    D = DeviceCSR.from_scipy(A)
    stream = torch.cuda.current_stream()
    dag_closure_device(D)                        # warm-up
    torch.cuda.synchronize()
    times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        C, mx, levels = dag_closure_device(D)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    clen = np.diff(C.indptr.cpu().numpy())
    aj = A.indices
    rows = np.repeat(np.arange(n), np.diff(A.indptr))
    off = aj != rows
    cand = int(clen[aj[off]].sum())
    edges = int(off.sum())
    b = 12.0 * A.nnz + 8.0 * (n + 1) + 8.0 * cand + 12.0 * edges + 24.0 * C.nnz + 8.0 * (n + 1)
    diameter = (mx.bit_length() - 1) if mx > 1 else 0
    mk, fx = fullsize_fixture("forest2m")
    same = bool(fx) and mk.csr_digest(A) == fx["input_sha256"] and \
        mk.csr_digest(C.to_scipy()) == fx["closure_sha256"] and diameter == fx["diameter"]
    peak = hbm_peak_gbs()
    return {"workload": f"pedigree forest, n={n}, 25 generations, nnz(A)={A.nnz}, int32 values",
            "ms": ms, "runs_ms": [round(t, 3) for t in times], "levels": levels, "nnz_closure": int(C.nnz),
            "candidates": cand, "diameter": diameter,
            "algorithmic_gb": b / 1e9, "gb_s": b / (ms / 1e3) / 1e9,
            "roofline": {"bound": "hbm", "achieved": b / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": b / (ms / 1e3) / 1e9 / peak, "peak_source": "measured copy bandwidth"},
            "bit_exact_vs_reference_fixture": same,
            "fixture_note": "closure and diameter against the digest of the reference's Cython DAG closure "
                            "of the same forest (tests/golden/fullsize.json)"}


def _merge_minabs_host(X, Y):
    """X (+) Y with the squaring merge's rule, for the check only (the smaller |value|, X's on a
    tie, zeros dropped)."""
    import scipy.sparse as sp
    X = sp.csr_matrix(X, dtype=np.int64)
    Y = sp.csr_matrix(Y, dtype=np.int64)
    xc, yc = X.tocoo(), Y.tocoo()
    keys_x = xc.row.astype(np.int64) * X.shape[1] + xc.col
    keys_y = yc.row.astype(np.int64) * X.shape[1] + yc.col
    allk = np.union1d(keys_x, keys_y)
    vx = np.zeros(allk.size, np.int64)
    vy = np.zeros(allk.size, np.int64)
    vx[np.searchsorted(allk, keys_x)] = xc.data
    vy[np.searchsorted(allk, keys_y)] = yc.data
    v = np.where(vx == 0, vy, np.where(vy == 0, vx, np.where(np.abs(vy) < np.abs(vx), vy, vx)))
    keep = v != 0
    return sp.csr_matrix((v[keep].astype(np.int32), (allk[keep] // X.shape[1], allk[keep] % X.shape[1])),
                         shape=X.shape)


def hbm_peak_gbs():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


SERVE = dict(count=2000, rate=2000.0, lookup_fraction=0.5, lo=64, hi=16384, seed=11, warm=64,
             budget=150 << 30)


def serve_stats(st, reqs):
    lat = st.latency_ms
    return {"p50_ms": lat["all"]["p50"], "p99_ms": lat["all"]["p99"],
            "closure_p50_ms": lat["closure"]["p50"], "closure_p99_ms": lat["closure"]["p99"],
            "lookup_p50_ms": lat["lookup"]["p50"], "lookup_p99_ms": lat["lookup"]["p99"],
            "throughput_req_s": len(reqs) / st.makespan_s,
            "closure_relax_per_s": st.relaxations / st.makespan_s,
            "makespan_s": st.makespan_s, "batches": st.batches, "max_batch": st.max_batch,
            "lookup_launches": st.lookup_launches, "evictions": st.evictions, "reloads": st.reloads,
            "peak_arena_gb": st.peak_arena_bytes / 1e9,
            "errors": sum(1 for r in reqs if r.kind == "closure" and r.result[0] != 0),
            **({"mutations": st.mutations, "mutation_p50_ms": lat["mutation"]["p50"],
                "mutation_p99_ms": lat["mutation"]["p99"]} if st.mutations else {})}


def run_serving(count=None):
    """The serving workload: Poisson arrivals of closure and lookup requests on resident graphs,
    served with continuous batching and, for comparison, one request at a time."""
    import torch
    from redblackgraph_gb300.serving import GpuExecutor, Policy, Server, make_stream
    cfg = dict(SERVE)
    if count:
        cfg["count"] = count
    allreq = make_stream(cfg["count"], cfg["rate"], cfg["lookup_fraction"], cfg["lo"], cfg["hi"],
                         cfg["seed"], warm=cfg["warm"])
    warm, reqs = allreq[:cfg["warm"]], allreq[cfg["warm"]:]
    ex = GpuExecutor(arena_bytes=cfg["budget"], slots=2)
    ex.prepare(allreq)
    out = {"workload": f"Poisson arrivals at {cfg['rate']:.0f} req/s, {cfg['count']} requests, "
                       f"{int(cfg['lookup_fraction'] * 100)}% relationship lookups / "
                       f"{100 - int(cfg['lookup_fraction'] * 100)}% closures, pedigrees log-uniform in "
                       f"[{cfg['lo']}, {cfg['hi']}] (int32 up to 4096 vertices, int64 above), "
                       f"{cfg['warm']} graphs closed and resident before the stream, "
                       f"{cfg['budget'] >> 30} GiB resident-graph budget",
           "latency": "arrival to completion on the host clock"}
    for name, pol in (("batched", Policy(inflight=2)), ("unbatched", Policy.unbatched_baseline())):
        for r in allreq:
            r.done, r.result = float("nan"), None
        srv = Server(ex, cfg["budget"], pol)
        srv.run(warm)
        torch.cuda.synchronize()
        st = srv.run(reqs)
        out[name] = serve_stats(st, reqs)
    # the same stream with a fifth of the lookups turned into mutations (links and new vertices
    # applied to the resident closures by relational composition)
    mreq = make_stream(cfg["count"], cfg["rate"], cfg["lookup_fraction"], cfg["lo"], cfg["hi"],
                       cfg["seed"], warm=cfg["warm"], mutation_fraction=0.2)
    mwarm, mreqs = mreq[:cfg["warm"]], mreq[cfg["warm"]:]
    srv = Server(ex, cfg["budget"], Policy(inflight=2))
    srv.run(mwarm)
    torch.cuda.synchronize()
    st = srv.run(mreqs)
    out["batched_with_mutations"] = serve_stats(st, mreqs)
    ex.close()
    del ex
    torch.cuda.empty_cache()
    return out


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        return main_reference(args, rank, world)
    if args.only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        fn = {"spgemm": run_spgemm_forest, "dag": run_dag_forest, "compose": run_compose,
              "single": run_single_dense, "anynum": lambda: run_any_numbering(workload(0)),
              "dense": run_dense_blocked, "matmul": run_matmul,
              "serve": lambda: run_serving(args.serve_count)}[args.only]
        print(json.dumps(fn()))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    w = workload(rank)
    r = run_ours(args, rank, world, w)
    total_work = r["work"] * args.steps * world
    value = total_work / r["t"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["t"] / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded pedigree components generated in-process",
            "config": config(w), "l2": f"inputs larger than L2: {r['bytes'] / 1e9:.1f} GB resident per step",
            "gpu_launches": int(r["launches"]), "clocks": r["clocks"]}
    # roofline of the dominant kernels: on the DAG path (every component here is numbered oldest
    # first) the scan reads every input cell once and the write stores every output cell once;
    # the two take equal time and together move 8 bytes per dense cell
    kp = r["kprof"]
    per = {k: v[0] / args.steps for k, v in kp.items()}
    hbm_ms = per["tri_scan_kernel"] + per["tri_write_kernel"]
    hbm = hbm_peak_gbs()
    hbm_bytes = r["cells"] * 4 * 2
    line["paths"] = {{1: "blocked32", 2: "blocked64", 3: "exact", 4: "dag"}.get(k, str(k)): v
                     for k, v in r["paths"].items()}
    ach = hbm_bytes / (hbm_ms / 1e3) / 1e9 if hbm_ms > 0 else None
    line["roofline"] = {
        "bound": "hbm", "unit": "GB/s", "kernel": "tri_scan_kernel + tri_write_kernel",
        "achieved": ach, "peak": hbm, "frac": ach / hbm if ach else None,
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)",
        "algorithmic_bytes_per_launch": hbm_bytes,
        "algorithmic_bytes_note": "the scan reads every input cell once (4 bytes per cell of the sum n^2 dense "
                                  "cells), the write stores every output cell once (4 bytes per cell); one "
                                  "launch of each per step",
        "per_kernel_gb_s": {k: r["cells"] * 4 / (per[k] / 1e3) / 1e9 for k in ("tri_scan_kernel", "tri_write_kernel")
                            if per.get(k)},
        "traffic": scan_traffic(hbm_bytes),
        "traffic_unit": "DRAM bytes per step of the two kernels (ncu capture of a smaller batch scaled by "
                        "dense cells, profiles/tri_scan_kernel_traffic.txt)",
        "kernel_ms_per_step": per,
        "kernel_launches_per_step": {k: v[1] / args.steps for k, v in kp.items()},
        "step_hbm_gb_s": hbm_bytes / (r["t"] / args.steps) / 1e9,
        "executed_products_per_step": r["executed"],
        "algorithmic_relaxations_per_step": r["work"],
    }
    if "blocked" in r:
        b = r["blocked"]
        bk = b["kprof"]
        phase_ms = sum(bk[k][0] for k in ("fw_tile_kernel", "fw_panel_kernel", "fw_diag_kernel"))
        peak, sms = int32_peak_ops(0, r["clocks"].get("sm_max_mhz"))
        ach = b["executed"] * OPS_PER_RELAXATION / (phase_ms / 1e3) / 1e12 if phase_ms > 0 else None
        tr = phase_traffic()
        traffic = sum(tr["bytes_per_launch"][k] * bk[k][1] for k in tr["bytes_per_launch"] if k in bk) if tr else None
        line["blocked_kernels_same_batch"] = {
            "value": r["work"] / b["t"], "unit": UNIT, "ms_per_step": b["t"] * 1e3,
            "how": "rbg_fw_batch with RBG_MODE_NO_DAG on the same resident blocks: snapshot-exact blocked "
                   "Floyd-Warshall for every component (the path of matrices not numbered in a "
                   "topological order)",
            "roofline": {"bound": "int32_alu", "unit": "Tops/s", "achieved": ach, "peak": peak / 1e12,
                         "frac": ach / (peak / 1e12) if ach else None,
                         "kernel": "fw_diag_kernel + fw_panel_kernel + fw_tile_kernel",
                         "peak_source": f"nominal: {sms} SMs x 128 int32 lanes x max SM clock",
                         "ops_per_relaxation": OPS_PER_RELAXATION, "executed_relaxations_per_step": b["executed"],
                         "traffic": traffic,
                         "traffic_unit": "DRAM bytes per step of the three phase kernels (per-launch bytes "
                                         "from profiles/fw_phase_traffic.txt x launches)"},
            "kernel_ms_per_step": {k: v[0] for k, v in bk.items() if v[1]}}
    e = r["e2e"]
    line["e2e"] = {"value": e["value"], "unit": UNIT, "h2d_bytes_per_step": e["h2d"],
                   "d2h_bytes_per_step": e["d2h"], "ms_per_step": e["t"] / e["steps"] * 1e3,
                   "api": "redblackgraph_gb300.sparse.component_wise_closure(forest CSR in pinned "
                          "host memory) -> merged CSR on the host",
                   "diameter": e["diameter"]}
    if rank == 0:
        idx = cpu_sample(w["csizes"])
        rate, tcpu, threads, outs = cpu_closure_rate(w, idx)
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(idx)} of {w['csizes'].size} components (smallest of every size octave up "
                      f"to {CPU_SAMPLE_RELAX / 8:.1e} relaxations or 64 components per octave, sum "
                      f"n^3 = {sum(int(w['csizes'][i]) ** 3 for i in idx):.3e}) closed in {tcpu:.1f} s "
                      "by the C restatement of the reference warshall, one component per host "
                      "thread; each octave's sum(n^3) extrapolated by its measured rate",
            "sample_bit_exact_vs_gpu": sample_parity(w, r["offsets"], r["out"], outs, idx, e["W"])}
    r.pop("out", None)
    import torch
    torch.cuda.empty_cache()
    if args.secondary and rank == 0:
        plain = run_plain(w)
        line["plain_one_launch_per_component"] = plain
        line["batched_vs_plain"] = value / plain["value"]
        line["single_graph"] = run_single_dense()
        line["spgemm_squaring"] = run_spgemm_forest()
        line["dag_levels"] = run_dag_forest()
        line["relational_composition"] = run_compose()
        line["any_numbering"] = run_any_numbering(w)
        line["dense_blocked"] = run_dense_blocked()
        try:
            line["avos_matmul"] = run_matmul()
        except Exception as exc:                 # a secondary line never costs the headline
            line["avos_matmul"] = {"error": f"{type(exc).__name__}: {exc}"}
    if args.serve:
        line["serving"] = run_serving(args.serve_count)
    if rank == 0:
        print(json.dumps(line))


def main_reference(args, rank, world):
    if rank != 0:
        return
    w = workload(0)
    idx = cpu_sample(w["csizes"])
    work = float(sum(int(w["csizes"][i]) ** 3 for i in idx))
    rates, total_t = [], 0.0
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_closure_rate(w, idx[: max(1, len(idx) // 8)], threads)
    for _ in range(args.steps):
        rate, t, threads, _ = cpu_closure_rate(w, idx, threads)
        rates.append(rate)
        total_t += t
    value = statistics.median(rates)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded pedigree components generated in-process",
            "config": config(w), "l2": "CPU run", "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{len(idx)} of {w['csizes'].size} components per step "
                                       f"(smallest of every size octave, sum n^3 = {work:.3e}); C "
                                       "restatement of the reference's warshall (core C gufunc), "
                                       "one component per host thread, each octave extrapolated "
                                       "by its measured rate"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
