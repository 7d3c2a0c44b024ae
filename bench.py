#!/usr/bin/env python
"""Benchmark: batched SeqCS.DOS.median on one GB300 (and N replicas).

Default workload: 65,536 affine pairs (lognormal lengths, median 800,
clipped 50-4,000; second sequence 10% substitutions + 2% indels; gap opening
3, extension 1, substitution 1). A "step" is one full batch: every pair's
band-doubling fill, traceback, median and worst cost.

  value  GCUPS over matrix cells (sum of len(a)*len(b)), inputs resident in
         HBM, timed with CUDA events on the launch stream
  e2e    the same through poyalgn_median_batch with pinned host buffers
         (host->device inputs and device->host outputs inside the timing)

`--impl reference` times the reference path's CPU implementation (the
reference algn.c build when it loads on this host, else the oracle's C
restatement) on all host cores over bounded samples.
Multi-GPU (torchrun): each rank aligns its own batch (weak scaling), no
collective on the data path; value = all ranks' cells / max rank time.
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

METRIC = ("GCUPS & alignments/s batched+served vs plain per-pair kernel, 1 GB300, "
          "bit-exact; p50/p99")
OPS_PER_CELL = {"affine": 51, "linear": 8}   # int32 ops per DP cell
DM_BYTES = {"affine": 1, "linear": 1}        # direction bytes written per cell (lean affine: 1)
# DRAM bytes (read + write) the class kernels and the deferred traceback moved
# per computed cell in one ncu capture of the 8,192-pair affine batch (4.03 GB
# for 2.62 G cells with the doubling's unstoppable passes skipped; 4.80 GB for
# 3.12 G cells before); the traffic grows with the computed cells, so it
# scales to the full batch.
DRAM_BYTES_PER_CELL = {"affine": 1.54}


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=["affine_pairs", "plain_pairs"],
                    default="affine_pairs")
    ap.add_argument("--pairs", type=int, default=0, help="override the pair count")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the untimed check of every pair against the oracle")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU work of the host baseline sample")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default pipeline ladder")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the downpass and serving measurements")
    ap.add_argument("--serve-seconds", type=float, default=1.0,
                    help="arrival window of each serving rate")
    ap.add_argument("--serve-slots", type=int, default=2, help="server execution slots")
    ap.add_argument("--serve-batch", type=int, default=8192, help="server pairs per batch")
    ap.add_argument("--percall-seconds", type=float, default=3.0,
                    help="timed seconds of each per-call workload (--leg percall)")
    ap.add_argument("--newkk-arena-mb", type=int, default=0,
                    help="bound the Newkk direction arena (MB; 0: library default)")
    ap.add_argument("--mem-gb", type=float, default=0.0,
                    help="cap each context's direction slabs and traceback arena (GB; 0: "
                         "library defaults), e.g. to keep a profiled case small")
    ap.add_argument("--leg", choices=["main", "peak", "plain", "percall", "downpass", "long",
                                      "serving", "distance", "newkk", "powell3d"],
                    default="main", help="run one measurement alone and print its object")
    return ap.parse_args(argv)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def make_workload(name: str, n_pairs: int, rank: int):
    from poy5_gb300 import workloads as wl
    if name == "affine_pairs":
        return wl.affine_pairs(n_pairs or 65536, seed=wl.SEED_BASE + 2 + 1000 * rank)
    return wl.plain_pairs(n_pairs or 4096, seed=wl.SEED_BASE + 1 + 1000 * rank)


def cells_full(w) -> int:
    return int(sum(len(a) * len(b) for a, b in w.pairs))


def host_oracle():
    """The CPU implementation of the path on this host: the reference algn.c
    build when it loads here (x86 with the POY sources), else the port."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    if oracle_lib.available("ref"):
        try:
            return oracle_lib.Oracle("ref"), "reference"
        except OSError:
            pass
    return oracle_lib.Oracle("port"), "port"


def host_cpu() -> str:
    """Model name of this host's CPU (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def cpu_rate(w, target_s: float, threads: int, single_thread_ref: bool = True):
    """Cells/s and pairs/s of the host CPU implementation on a bounded
    sample of `w` (pairs taken in order until ~target_s of work)."""
    orc, kind = host_oracle()
    cm = orc.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    pairs = w.pairs
    if kind == "reference":
        # the reference harness is single-threaded per process workspace
        threads = 1
        t0 = time.perf_counter()
        n = 0
        cells = 0
        while n < len(pairs) and time.perf_counter() - t0 < target_s:
            a, b = pairs[n]
            orc.median(cm, a, b, w.affine)
            cells += len(a) * len(b)
            n += 1
        dt = time.perf_counter() - t0
    else:
        probe = pairs[:64]
        t0 = time.perf_counter()
        orc.median_batch(cm, [a for a, _ in probe], [b for _, b in probe], w.affine, threads)
        per_pair = (time.perf_counter() - t0) / len(probe)
        n = int(min(len(pairs), max(64, target_s / max(per_pair, 1e-7))))
        sample = pairs[:n]
        t0 = time.perf_counter()
        orc.median_batch(cm, [a for a, _ in sample], [b for _, b in sample], w.affine, threads)
        dt = time.perf_counter() - t0
        cells = sum(len(a) * len(b) for a, b in sample)
    return {"cells_per_s": cells / dt, "pairs_per_s": n / dt, "pairs": n,
            "seconds": dt, "threads": threads, "kind": kind}


def measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def run_gpu(args):
    import ctypes as C

    import torch

    import poy5_gb300 as pg
    from poy5_gb300 import _lib, schedule

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = make_workload(args.workload, args.pairs, rank)
    model = "affine" if w.affine else "linear"
    ctx = pg.Context(local)
    if args.mem_gb:
        ctx.set_memory_budget(int(args.mem_gb * 2**30), int(args.mem_gb * 2**30))
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    lib = _lib.load()
    pk = pg.pack_pairs(w.pairs)
    n = pk.npairs
    dev = torch.device("cuda", local)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb), t(pk.out_off)]
    d_int = [torch.zeros(n, dtype=torch.int32, device=dev) for _ in range(7)]
    d_out = [torch.zeros(pk.out_bytes, dtype=torch.uint8, device=dev) for _ in range(4)]
    P = lambda x: C.c_void_p(x.data_ptr())
    stream = torch.cuda.current_stream(dev)

    def plain_step():
        rc = lib.poyalgn_median_batch_device(
            ctx.handle, cm.handle, n, pk.max_pair_len, pk.out_bytes,
            *(P(x) for x in d_in), *(P(x) for x in d_int[:6]), *(P(x) for x in d_out),
            P(d_int[6]), C.c_void_p(stream.cuda_stream))
        _lib.check(rc)

    # pipeline shapes tuned on the workload itself (untimed setup): a sample
    # smaller than the batch favours the ladders whose narrow classes finish
    # their longest pairs soonest, not the ones with the highest throughput
    tuned = None
    if not args.no_autotune:
        from poy5_gb300 import tune
        tuned = tune.autotune(ctx, cm, pk, reps=3)
    # the whole batch captured once as a CUDA graph and replayed per step
    graph = C.c_void_p()
    _lib.check(lib.poyalgn_batch_graph_create(
        ctx.handle, cm.handle, n, pk.max_pair_len, pk.out_bytes, *(P(x) for x in d_in),
        *(P(x) for x in d_int[:6]), *(P(x) for x in d_out), P(d_int[6]), C.byref(graph)))

    def step():
        _lib.check(lib.poyalgn_batch_graph_launch(graph, C.c_void_p(stream.cuda_stream)))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    status = d_int[5].cpu().numpy()
    if not np.all(status == 0):
        raise RuntimeError(f"{int((status != 0).sum())} pairs failed: {np.unique(status)}")
    passes = d_int[6].cpu().numpy()
    launches_per_step = ctx.last_launches()
    # the integer issue rates of this GPU (the roofline's measured peak),
    # measured before the timed region with its own clock sample
    pclk = ClockSampler(local)
    pclk.start()
    peak = pg.int32_rates(local)
    peak["clocks"] = pclk.stop()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    # per-launch timing over a second set of steps (same work, events per launch)
    ctx.profile_begin(args.steps)
    for _ in range(args.steps):
        plain_step()
    torch.cuda.synchronize(dev)
    prof = ctx.profile_end()
    clk = clocks.stop()

    # end to end through the host-pointer entry point, pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        h_in = [pin(pk.seqs), pin(pk.offa), pin(pk.lena), pin(pk.offb), pin(pk.lenb),
                pin(pk.out_off)]
        h_int = [torch.zeros(n, dtype=torch.int32).pin_memory() for _ in range(7)]
        h_out = [torch.zeros(pk.out_bytes, dtype=torch.uint8).pin_memory() for _ in range(4)]

        def e2e_step():
            rc = lib.poyalgn_median_batch(ctx.handle, cm.handle, n, *(P(x) for x in h_in),
                                          *(P(x) for x in h_int[:6]), *(P(x) for x in h_out),
                                          P(h_int[6]))
            _lib.check(rc)

        e2e_step()
        barrier()
        t0 = time.perf_counter()
        e2e_each = []
        for _ in range(args.steps):
            t1 = time.perf_counter()
            e2e_step()
            e2e_each.append(round((time.perf_counter() - t1) * 1e3, 2))
        e2e_s = (time.perf_counter() - t0) / args.steps
        barrier()
        h2d = int(pk.seqs.nbytes + pk.offa.nbytes * 3 + pk.lena.nbytes * 2)
        d2h = int(7 * 4 * n + 4 * pk.out_bytes)
        e2e = {"seconds": e2e_s, "h2d": h2d, "d2h": d2h, "step_ms": e2e_each}

    # every pair of the timed batch against the oracle (untimed; rank 0)
    parity = None
    if rank == 0 and not args.no_parity:
        parity = batch_parity(w, pk, [x.cpu().numpy() for x in d_int[:6]],
                              [x.cpu().numpy() for x in d_out])

    # the plain per-call path: one drop-in stub call per pair (sample)
    plain = plain_per_call(ctx, cm, w, seconds=3.0)

    cells = cells_full(w)
    full = None
    if not w.affine:
        gaps = lambda s: int(np.count_nonzero((s >= 16) & ((s & 16) != 0)))
        full = schedule.linear_full_plane(pk.lena, pk.lenb, [gaps(a) for a, _ in w.pairs],
                                          [gaps(b) for _, b in w.pairs])
    mnz = cm.tables()["min_non0_cost"]
    computed = int(schedule.cells_computed(pk.lena, pk.lenb, passes, mnz, w.affine, full,
                                           skipped_passes(w, pk, mnz, full)).sum())
    lib.poyalgn_batch_graph_free(graph)
    return dict(w=w, model=model, n=n, ms=ms, cells=cells, computed=computed, prof=prof,
                clocks=clk, e2e=e2e, launches=launches_per_step, passes=passes,
                world=world, rank=rank, pk=pk, plain=plain, tuned=tuned, peak=peak,
                parity=parity)


def skipped_passes(w, pk, mnz: int, full) -> np.ndarray:
    """Per pair, the leading doubling passes the library counts as run
    without filling them: linear pairs off the full plane, and affine pairs
    on the lean cell (no gap state in either sequence, every state far below
    HIGH: n (largest gap-free cost + gap opening + 1) + gap opening < HIGH / 4
    for the subs / indel matrix)."""
    from poy5_gb300 import schedule
    s = schedule.unstoppable_passes(pk.lena, pk.lenb, mnz, w.affine)
    if not w.affine:
        return np.where(np.asarray(full, bool), 0, s)
    mc = max(w.subs, w.indel)
    n = np.maximum(pk.lena, pk.lenb).astype(np.int64)
    gapfree = np.array([not (np.any(a[1:] & 16) or np.any(b[1:] & 16)) for a, b in w.pairs])
    lean = gapfree & (n * (mc + w.gap_open + 1) + w.gap_open < 1000000 // 4)
    return np.where(lean, s, 0)


def batch_parity(w, pk, ints, bufs) -> dict:
    """Every pair of a GPU batch against the oracle's C restatement run over
    the same pairs on all host cores: cost, worst cost, aligned pair, median
    and median with gaps, byte for byte."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    orc = oracle_lib.Oracle("port")
    ocm = orc.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    t0 = time.perf_counter()
    ref = orc.median_batch(ocm, [a for a, _ in w.pairs], [b for _, b in w.pairs], w.affine,
                           os.cpu_count() or 1)
    out = oracle_lib.compare_batch(ref, ints, bufs, pk.out_off, pk.cap)
    out["against"] = "oracle port, every pair of the timed batch"
    out["seconds"] = round(time.perf_counter() - t0, 1)
    return out


def plain_per_call(ctx, cm, w, seconds: float = 3.0) -> dict:
    """One per-call drop-in invocation per pair (what POY's OCaml would do
    through the stub library): algn_CAML_align_affine_3, or simple_2 +
    backtrace_2d for the linear model; host buffers in and out."""
    import poy5_gb300 as pg
    al = pg.Align(ctx)
    t0 = time.perf_counter()
    n = cells = 0
    while n < len(w.pairs) and time.perf_counter() - t0 < seconds:
        a, b = w.pairs[n]
        al.align_2(a, b, cm)
        cells += len(a) * len(b)
        n += 1
    dt = time.perf_counter() - t0
    return {"gcups": cells / dt / 1e9, "alignments_per_s": n / dt, "pairs": n}


def run_percall(local: int, seconds: float = 3.0) -> dict:
    """The drop-in per-call stubs alone, one call sequence per pair as POY's
    OCaml makes them: algn_CAML_align_affine_3 on the affine pair workload,
    simple_2 + backtrace_2d on the plain pairwise workload (host buffers)."""
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    ctx = pg.Context(local)
    out = {}
    for w in (wl.affine_pairs(n_pairs=4096), wl.plain_pairs()):
        cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
        plain_per_call(ctx, cm, w, seconds=min(0.3, seconds))  # warm-up
        r = plain_per_call(ctx, cm, w, seconds=seconds)
        out[w.name] = {"alignments_per_s": round(r["alignments_per_s"], 1),
                       "gcups": round(r["gcups"], 3), "pairs": r["pairs"]}
    ctx.close()
    return out


def run_downpass(local: int, reps: int = 5) -> dict:
    """Downpass of the 256-taxon Yule tree over device-resident leaves, one
    batch per tree level; its CPU counterpart is the host implementation run
    level by level on all host cores."""
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    t = wl.yule_tree()
    ctx = pg.Context(local)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, t.subs, t.indel, t.gap_open)
    store = pg.Store(ctx, 64 << 20)
    leaves = [store.add(s) for s in t.leaves]
    n0 = len(store)
    for _ in range(2):
        pg.downpass(store, cm, leaves, t.left, t.right)
        store.truncate(n0)
    t0 = time.perf_counter()
    for k in range(reps):
        res = pg.downpass(store, cm, leaves, t.left, t.right)
        if k < reps - 1:
            store.truncate(n0)
    dt = (time.perf_counter() - t0) / reps
    nl = len(t.leaves)
    length = lambda ch: (len(t.leaves[ch]) if ch < nl else
                         len(store.read(int(res.internal_node[ch - nl]))))
    cells = sum(length(a) * length(b) for a, b in zip(t.left, t.right))
    # host implementation, level by level (nodes of a level run in parallel)
    host_oracle()  # puts the oracle's loader on the path
    import oracle_lib
    orc, kind = oracle_lib.Oracle("port"), "port"
    ocm = orc.cm(subs=t.subs, indel=t.indel)
    levels = pg.tree_levels(nl, t.left, t.right)
    seqs = list(t.leaves) + [None] * len(t.left)
    tot = 0
    c0 = time.perf_counter()
    for lv in range(1, int(levels.max()) + 1):
        ks = np.flatnonzero(levels == lv)
        out = orc.median_batch(ocm, [seqs[t.left[k]] for k in ks], [seqs[t.right[k]] for k in ks],
                               False)
        for j, k in enumerate(ks):
            o = int(out["out_off"][j])
            seqs[nl + k] = out["med"][o:o + out["mlen"][j]]
        tot += int(out["cost"].sum())
    cpu_s = time.perf_counter() - c0
    up = run_uppass(store, cm, t, leaves, res, seqs, orc, ocm, reps)
    store.close()
    return {"workload": t.name, "internal_nodes": len(t.left), "levels": res.levels,
            "ms": round(dt * 1e3, 3), "total_cost": res.total_cost,
            "gcups": round(cells / dt / 1e9, 3), "medians_per_s": round(len(t.left) / dt, 1),
            "cpu_baseline": {"ms": round(cpu_s * 1e3, 1), "kind": kind,
                             "cores": os.cpu_count() or 1, "total_cost": tot},
            "total_cost_matches_cpu": tot == res.total_cost, "uppass": up}


def run_uppass(store, cm, t, leaves, down, seqs, orc, ocm, reps: int) -> dict:
    """Uppass of the same tree after its downpass (SeqCS.DOS.median_3_no_union
    top down, one batch of 2 alignments per node per depth), and the host
    implementation depth by depth on all cores beside it (the same
    alignments, the cheaper one kept, its no-gap median)."""
    import poy5_gb300 as pg
    n1 = len(store)
    for _ in range(2):
        pg.uppass(store, cm, leaves, t.left, t.right, down.internal_node)
        store.truncate(n1)
    t0 = time.perf_counter()
    for k in range(reps):
        up = pg.uppass(store, cm, leaves, t.left, t.right, down.internal_node)
        if k < reps - 1:
            store.truncate(n1)
    dt = (time.perf_counter() - t0) / reps
    nl, ni = len(t.leaves), len(t.left)
    parent = np.full(ni, -1)
    for k in range(ni):
        for ch in (t.left[k], t.right[k]):
            if ch >= nl:
                parent[ch - nl] = k
    depth = np.zeros(ni, int)
    for k in range(ni - 2, -1, -1):
        depth[k] = depth[parent[k]] + 1
    tab = orc.tables(ocm)
    med_t, lcm, gap = tab["median"], tab["lcm"], tab["gap"]
    final = [None] * ni
    final[ni - 1] = seqs[nl + ni - 1]
    fcost = np.zeros(ni, np.int64)
    c0 = time.perf_counter()
    for d in range(1, int(depth.max()) + 1):
        ks = np.flatnonzero(depth == d)
        pa = [final[parent[k]] for k in ks for _ in (0, 1)]
        ch = [seqs[c] for k in ks for c in (t.left[k], t.right[k])]
        out = orc.median_batch(ocm, pa, ch, t.affine)
        for j, k in enumerate(ks):
            a, b = 2 * j, 2 * j + 1
            q = a if out["cost"][a] < out["cost"][b] else b
            o, n = int(out["out_off"][q]), int(out["alen"][q])
            m = med_t[(out["ea"][o:o + n].astype(np.int64) << lcm) + out["eb"][o:o + n]]
            final[k] = np.concatenate([[gap], m[m != gap]]).astype(np.uint8)
            fcost[k] = out["cost"][q]
    cpu_s = time.perf_counter() - c0
    same = np.array_equal(fcost, up.final_cost) and all(
        np.array_equal(store.read(int(up.final_node[k])), final[k]) for k in range(ni))
    return {"ms": round(dt * 1e3, 3), "levels": up.levels,
            "final_cost_sum": int(up.final_cost.sum()),
            "cpu_baseline": {"ms": round(cpu_s * 1e3, 1), "kind": "port",
                             "cores": os.cpu_count() or 1},
            "final_states_match_cpu": bool(same)}


def run_long(local: int, cpu_pairs: int = 1, parity_pairs: int = 4, n_pairs: int = 512,
             mem_gb: float = 0.0) -> dict:
    """The long-pair stress workload (512 pairs of 20-50 kb, 15% substitutions,
    2% indels, linear 1/2): one timed batch with inputs resident on the
    device, direction bytes written per filled cell as the HBM figure, and
    the host implementation on the first pair(s) beside it."""
    import ctypes as C
    import torch
    import poy5_gb300 as pg
    from poy5_gb300 import _lib, schedule
    from poy5_gb300 import workloads as wl
    w = wl.long_pairs(n_pairs=n_pairs)
    ctx = pg.Context(local)
    if mem_gb:
        ctx.set_memory_budget(int(mem_gb * 2**30), int(mem_gb * 2**30))
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    lib = _lib.load()
    pk = pg.pack_pairs(w.pairs)
    n = pk.npairs
    dev = torch.device("cuda", local)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb), t(pk.out_off)]
    d_int = [torch.zeros(n, dtype=torch.int32, device=dev) for _ in range(7)]
    d_out = [torch.zeros(pk.out_bytes, dtype=torch.uint8, device=dev) for _ in range(4)]
    P = lambda x: C.c_void_p(x.data_ptr())
    st = torch.cuda.current_stream(dev)

    def step():
        _lib.check(lib.poyalgn_median_batch_device(
            ctx.handle, cm.handle, n, pk.max_pair_len, pk.out_bytes, *(P(x) for x in d_in),
            *(P(x) for x in d_int[:6]), *(P(x) for x in d_out), P(d_int[6]),
            C.c_void_p(st.cuda_stream)))

    step()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    step()
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    ctx.profile_begin(1)
    step()
    torch.cuda.synchronize(dev)
    prof = ctx.profile_end()
    status = d_int[5].cpu().numpy()
    passes = d_int[6].cpu().numpy()
    cells = cells_full(w)
    gaps = lambda s: int(np.count_nonzero((s >= 16) & ((s & 16) != 0)))
    full = schedule.linear_full_plane(pk.lena, pk.lenb, [gaps(a) for a, _ in w.pairs],
                                      [gaps(b) for _, b in w.pairs])
    mnz = cm.tables()["min_non0_cost"]
    computed = int(schedule.cells_computed(pk.lena, pk.lenb, passes, mnz, False, full,
                                           skipped_passes(w, pk, mnz, full)).sum())
    # full-length parity: the longest pairs (both sequences past 40 kb)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    longest = [int(k) for k in np.argsort(-(pk.lena.astype(np.int64) + pk.lenb))[:parity_pairs]]
    sub = [w.pairs[k] for k in longest]
    spk = pg.pack_pairs(sub)
    ints = [x.cpu().numpy()[longest] for x in d_int[:6]]
    host = [x.cpu().numpy() for x in d_out]
    bufs = []
    for h, ln in zip(host, (ints[2], ints[2], ints[3], ints[4])):
        g = np.zeros(spk.out_bytes, np.uint8)
        for j, k in enumerate(longest):
            e = int(pk.out_off[k] + pk.cap[k])
            f = int(spk.out_off[j] + spk.cap[j])
            g[f - ln[j]:f] = h[e - ln[j]:e]
        bufs.append(g)
    porc = oracle_lib.Oracle("port")
    pcm = porc.cm(subs=w.subs, indel=w.indel)
    t0 = time.perf_counter()
    ref = porc.median_batch(pcm, [a for a, _ in sub], [b for _, b in sub], False, len(sub))
    par = oracle_lib.compare_batch(ref, ints, bufs, spk.out_off, spk.cap)
    par.update({"against": "oracle port (64-bit indices)", "seconds": round(time.perf_counter() - t0, 1),
                "min_len": int(min(min(len(a), len(b)) for a, b in sub))})
    # host implementation on the first pair(s), single pair at a time
    orc, kind = host_oracle()
    ocm = orc.cm(subs=w.subs, indel=w.indel)
    c0 = time.perf_counter()
    ccells = 0
    for a, b in w.pairs[:cpu_pairs]:
        orc.median(ocm, a, b, False)
        ccells += len(a) * len(b)
    cpu_s = time.perf_counter() - c0
    return {"workload": w.name, "pairs": n, "ms": round(ms, 2),
            "status_ok": int((status == 0).sum()), "gcups": round(cells / ms / 1e6, 2),
            "gcups_computed_cells": round(computed / ms / 1e6, 2),
            "dm_write_gbs": round(computed / ms / 1e6, 2), "passes_mean": round(float(passes.mean()), 2),
            "launch_ms": {k: round(v, 3) for k, v in prof.items() if k != "batches"},
            "parity": par,
            "cpu_baseline": {"gcups": round(ccells / cpu_s / 1e9, 4), "kind": kind, "cores": 1,
                             "sample": f"first {cpu_pairs} pair(s), one thread"}}


def e2e_pinned(lib, ctx, cm, pk, steps: int) -> float:
    """Seconds per poyalgn_median_batch call on pinned host buffers (one
    untimed call first)."""
    import ctypes as C
    import torch
    from poy5_gb300 import _lib
    P = lambda x: C.c_void_p(x.data_ptr())
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    n = pk.npairs
    h_in = [pin(pk.seqs), pin(pk.offa), pin(pk.lena), pin(pk.offb), pin(pk.lenb),
            pin(pk.out_off)]
    h_int = [torch.zeros(n, dtype=torch.int32).pin_memory() for _ in range(7)]
    h_out = [torch.zeros(pk.out_bytes, dtype=torch.uint8).pin_memory() for _ in range(4)]

    def step():
        _lib.check(lib.poyalgn_median_batch(ctx.handle, cm.handle, n, *(P(x) for x in h_in),
                                            *(P(x) for x in h_int[:6]),
                                            *(P(x) for x in h_out), P(h_int[6])))

    step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    return (time.perf_counter() - t0) / steps


def run_plain(local: int, steps: int = 10, warmup: int = 3) -> dict:
    """The plain pairwise workload (4,096 linear pairs, lengths 200-600, 1 %
    ambiguity codes; subs 1, indel 2): the batch on device-resident inputs
    (CUDA graph replay, CUDA events), end to end through
    poyalgn_median_batch with pinned host buffers, every pair against the
    oracle, and the oracle on all host cores over the whole batch."""
    import ctypes as C
    import torch
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    from poy5_gb300 import workloads as wl
    w = wl.plain_pairs()
    ctx = pg.Context(local)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    lib = _lib.load()
    pk = pg.pack_pairs(w.pairs)
    n = pk.npairs
    dev = torch.device("cuda", local)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb), t(pk.out_off)]
    d_int = [torch.zeros(n, dtype=torch.int32, device=dev) for _ in range(7)]
    d_out = [torch.zeros(pk.out_bytes, dtype=torch.uint8, device=dev) for _ in range(4)]
    P = lambda x: C.c_void_p(x.data_ptr())
    st = torch.cuda.current_stream(dev)
    graph = C.c_void_p()
    _lib.check(lib.poyalgn_batch_graph_create(
        ctx.handle, cm.handle, n, pk.max_pair_len, pk.out_bytes, *(P(x) for x in d_in),
        *(P(x) for x in d_int[:6]), *(P(x) for x in d_out), P(d_int[6]), C.byref(graph)))
    step = lambda: _lib.check(lib.poyalgn_batch_graph_launch(graph, C.c_void_p(st.cuda_stream)))
    for _ in range(warmup):
        step()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        step()
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    launches = ctx.last_launches()
    lib.poyalgn_batch_graph_free(graph)
    ints = [x.cpu().numpy() for x in d_int[:6]]
    bufs = [x.cpu().numpy() for x in d_out]
    # end to end: pinned host buffers, copies inside the call
    e2e_s = e2e_pinned(lib, ctx, cm, pk, steps)
    cells = cells_full(w)
    par = batch_parity(w, pk, ints, bufs)
    cpu = cpu_rate(w, 1e9, os.cpu_count() or 1)  # the whole batch
    return {"workload": w.name, "pairs": n, "ms": round(ms, 3),
            "gcups": round(cells / ms / 1e6, 2), "alignments_per_s": round(n / ms * 1e3, 1),
            "gpu_launches_per_step": launches,
            "e2e": {"ms": round(e2e_s * 1e3, 3), "gcups": round(cells / e2e_s / 1e9, 2),
                    "h2d_bytes_per_step": int(pk.seqs.nbytes + 5 * 8 * n),
                    "d2h_bytes_per_step": int(4 * pk.out_bytes + 28 * n)},
            "parity": par,
            "cpu_baseline": {"gcups": round(cpu["cells_per_s"] / 1e9, 4), "kind": cpu["kind"],
                             "cores": cpu["threads"], "ms": round(cpu["seconds"] * 1e3, 1),
                             "sample": f"all {cpu['pairs']} pairs",
                             "alignments_per_s": round(cpu["pairs_per_s"], 1)}}


def run_distance(local: int, n_pairs: int = 8192, reps: int = 3) -> dict:
    """DOS.distance (cost only) of serving-distribution pairs, affine: the
    full unbanded fill of algn_CAML_cost_affine_3, inputs resident."""
    import ctypes as C
    import torch
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    from poy5_gb300 import workloads as wl
    w = wl.serving_pairs(n_pairs=n_pairs)
    ctx = pg.Context(local)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    lib = _lib.load()
    pk = pg.pack_pairs(w.pairs)
    dev = torch.device("cuda", local)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb)]
    cost = torch.zeros(pk.npairs, dtype=torch.int32, device=dev)
    status = torch.zeros(pk.npairs, dtype=torch.int32, device=dev)
    P = lambda x: C.c_void_p(x.data_ptr())
    st = torch.cuda.current_stream(dev)

    def step():
        _lib.check(lib.poyalgn_distance_batch_device(
            ctx.handle, cm.handle, pk.npairs, pk.max_pair_len, *(P(x) for x in d_in), 0,
            P(cost), P(status), C.c_void_p(st.cuda_stream)))

    step()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        step()
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    cells = cells_full(w)
    ok = int((status.cpu().numpy() == 0).sum())
    return {"workload": f"serving_pairs_{n_pairs}_distance", "pairs": pk.npairs,
            "status_ok": ok, "ms": round(ms, 2), "gcups": round(cells / ms / 1e6, 2),
            "alignments_per_s": round(pk.npairs / ms * 1e3, 1)}


def run_powell3d(local: int, n_triples: int = 8192, reps: int = 2, cpu_triples: int = 1024) -> dict:
    """Three-sequence alignment (Sequence.Align.align_3_powell ->
    powell_3D_align) on readjust-shaped triples: the host-pointer batch API
    end to end (inputs and outputs through host memory) and its summed kernel
    time; the oracle port on all host cores on the first `cpu_triples`
    triples beside it, with every output of those triples compared."""
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    from poy5_gb300.three_d import pack_triples
    w = wl.readjust_triples(n_triples=n_triples)
    ctx = pg.Context(local)
    pg.powell_3d_batch(ctx, w.triples, w.mm, w.go, w.ge)  # warm-up
    walls, kms = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        res = pg.powell_3d_batch(ctx, w.triples, w.mm, w.go, w.ge)
        walls.append(time.perf_counter() - t0)
        kms.append(res.kernel_ms)
    wall = float(np.median(walls))
    kms_ = float(np.median(kms))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    orc = oracle_lib.Oracle("port")
    sub = w.triples[:cpu_triples]
    seqs, off, lens, out_off, cap = pack_triples(sub)
    threads = os.cpu_count() or 1
    c0 = time.perf_counter()
    ref = orc.powell_3d_batch(seqs, off, lens, out_off, w.mm, w.go, w.ge, nthreads=threads)
    cpu_s = time.perf_counter() - c0
    # parity on the sample: costs, lengths and the three aligned sequences
    bad = int((ref["status"] != 0).sum()) + int((res.status[:len(sub)] != 0).sum())
    bad += int((ref["cost"] != res.cost[:len(sub)]).sum())
    for k in range(len(sub)):
        n = int(ref["rlen"][k])
        e_ref = int(out_off[k] + cap[k])
        got = res.aligned(k)
        if n != int(res.rlen[k]) or any(not np.array_equal(ref[x][e_ref - n:e_ref], g)
                                        for x, g in zip(("ra", "rb", "rc"), got)):
            bad += 1
    # the per-call drop-in (one powell_3d call per triple, what unmodified POY
    # issues) on the first 16 triples, and one host thread on the same ones
    few = w.triples[:16]
    t0 = time.perf_counter()
    for tr in few:
        pg.align_3_powell(ctx, *tr, w.mm, w.go, w.ge)
    call_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for tr in few:
        orc.powell_3d(*tr, w.mm, w.go, w.ge)
    one_s = time.perf_counter() - t0
    nt = len(w.triples)
    return {"workload": w.name, "triples": nt, "status_ok": int((res.status == 0).sum()),
            "per_call": {"calls": len(few), "ms_per_call": round(call_s / len(few) * 1e3, 2),
                         "host_one_thread_ms_per_call": round(one_s / len(few) * 1e3, 2)},
            "e2e_ms": round(wall * 1e3, 1), "kernel_ms": round(kms_, 1),
            "launch_rounds": res.rounds,
            "triples_per_s": round(nt / wall, 1),
            "triples_per_s_kernel": round(nt / (kms_ / 1e3), 1),
            "cost_sum": int(res.cost.sum()),
            "parity": {"against": "oracle port", "triples": len(sub), "mismatches": bad},
            "cpu_baseline": {"triples_per_s": round(len(sub) / cpu_s, 1), "kind": "port",
                             "cores": threads, "cpu_model": host_cpu(),
                             "sample": f"first {len(sub)} triples of {w.name} ({cpu_s:.1f} s)"}}


def run_newkk(local: int, n_pairs: int = 65536, reps: int = 2, cpu_s: float = 8.0,
              arena_mb: int = 0) -> dict:
    """DOS.median with use_ukk (Algn_Newkk, src/newkkonen.c) on the affine
    pair workload: device-resident inputs (value) and the host-pointer API
    with the copies inside the timed region (e2e); the oracle's restatement
    on the host cores on a bounded sample beside it, and a parity sample."""
    import ctypes as C
    import concurrent.futures as cf
    import torch
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    from poy5_gb300 import workloads as wl
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    w = wl.affine_pairs(n_pairs=n_pairs)
    ctx = pg.Context(local)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    if arena_mb:
        pg.NewkkAlign(ctx).set_arena_words(arena_mb << 19)
    lib = _lib.load()
    pk = pg.pack_pairs(w.pairs)
    dev = torch.device("cuda", local)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb), t(pk.out_off)]
    ints = [torch.zeros(pk.npairs, dtype=torch.int32, device=dev) for _ in range(7)]
    outs = [torch.zeros(max(pk.out_bytes, 1), dtype=torch.uint8, device=dev) for _ in range(4)]
    P = lambda x: C.c_void_p(x.data_ptr())
    st = torch.cuda.current_stream(dev)
    max_len = int(max(pk.lena.max(), pk.lenb.max()))

    def step():
        _lib.check(lib.poyalgn_newkk_median_batch_device(
            ctx.handle, cm.handle, pk.npairs, *(P(x) for x in d_in), max_len,
            *(P(x) for x in ints[:6]), *(P(x) for x in outs), P(ints[6]),
            C.c_void_p(st.cuda_stream)))

    step()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        step()
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    launches = ctx.last_launches()
    status = ints[5].cpu().numpy()
    passes = ints[6].cpu().numpy()
    # e2e: the host-pointer entry point (copies in and out inside the call)
    t0 = time.perf_counter()
    res = pg.newkk_median_batch(ctx, cm, pk)
    e2e_ms = (time.perf_counter() - t0) * 1e3
    cells = cells_full(w)
    # parity sample and CPU baseline: the oracle's restatement
    orc = oracle_lib.Oracle("port")
    ocm = orc.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    par_bad = 0
    for k in range(64):
        a, b = w.pairs[k]
        r = orc.newkk_median(ocm, a, b)
        d = res.pair(k)
        if not (d.cost == r.cost and np.array_equal(d.aligned_a, r.ea)
                and np.array_equal(d.aligned_b, r.eb) and np.array_equal(d.median, r.median)):
            par_bad += 1
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    n_cpu, ccells = 0, 0

    def one(k):
        a, b = w.pairs[k]
        orc.newkk_median(ocm, a, b)
        return len(a) * len(b)

    with cf.ThreadPoolExecutor(threads) as ex:
        while time.perf_counter() - t0 < cpu_s and n_cpu < len(w.pairs):
            chunk = range(n_cpu, min(n_cpu + 4 * threads, len(w.pairs)))
            ccells += sum(ex.map(one, chunk))
            n_cpu += len(chunk)
    cpu_dt = time.perf_counter() - t0
    return {"workload": f"affine_pairs_{n_pairs}_newkk", "pairs": pk.npairs,
            "status_ok": int((status == 0).sum()), "ms": round(ms, 2),
            "gcups": round(cells / ms / 1e6, 2),
            "alignments_per_s": round(pk.npairs / ms * 1e3, 1),
            "e2e": {"ms": round(e2e_ms, 2), "gcups": round(cells / e2e_ms / 1e6, 2),
                    "h2d_bytes": int(pk.seqs.nbytes + 5 * 8 * pk.npairs),
                    "d2h_bytes": int(4 * pk.out_bytes + 28 * pk.npairs)},
            "passes_mean": round(float(passes.mean()), 2), "gpu_launches": launches,
            "parity_sample": {"pairs": 64, "mismatches": par_bad, "against": "oracle port"},
            "cpu_baseline": {"gcups": round(ccells / cpu_dt / 1e9, 4), "kind": "port",
                             "cores": threads,
                             "sample": f"first {n_cpu} pairs ({cpu_dt:.1f} s)",
                             "alignments_per_s": round(n_cpu / cpu_dt, 2)}}


def run_serving(local: int, seconds: float = 1.0, nslots: int = 2,
                max_batch_pairs: int = 8192) -> dict:
    """Open-loop Poisson replay against the continuous-batching server: each
    request has U{1..64} pairs of a resident pool (lognormal lengths, median
    1,000, clipped 100-5,000, ~30% divergence), affine 3/1/1."""
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    w = wl.serving_pairs(n_pairs=4096)
    ctx = pg.Context(local)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    store = pg.Store(ctx, 64 << 20)
    na = np.array([store.add(a) for a, _ in w.pairs], np.int32)
    nb = np.array([store.add(b) for _, b in w.pairs], np.int32)
    pair_cells = np.array([len(a) * len(b) for a, b in w.pairs], np.int64)
    cfg = dict(nslots=nslots, max_batch_pairs=max_batch_pairs,
               max_waiting_pairs=max(16384, 2 * nslots * max_batch_pairs))
    rng = np.random.default_rng(wl.SEED_BASE + 4)

    def sweep(kind, rates):
        srv = pg.Server(store, cm, hbm_budget=24 << 30, kind=kind, **cfg)
        srv.replay(pg.poisson_trace(rng, 2000.0, 200, na, nb))  # warm-up
        points = []
        for rate in rates:
            nreq = int(min(rate * seconds, 40000))
            tr = pg.poisson_trace(rng, float(rate), nreq, na, nb)
            res = srv.replay(tr)
            ok = res.served()
            lat = res.latency_s[ok] * 1e3
            pair_ok = np.repeat(ok, tr.npairs)
            cells = int(pair_cells[tr.node_a[pair_ok]].sum())
            points.append({"rate_req_s": rate, "requests": nreq, "refused": int((~ok).sum()),
                           "p50_ms": round(float(np.percentile(lat, 50)), 3) if len(lat) else None,
                           "p99_ms": round(float(np.percentile(lat, 99)), 3) if len(lat) else None,
                           "alignments_per_s": round(int(pair_ok.sum()) / res.wall_s, 1),
                           "gcups": round(cells / res.wall_s / 1e9, 3)})
        st = srv.stats()
        srv.close()
        return {"batches": st["batches"], "points": points}

    from poy5_gb300.serve import DISTANCE, MEDIAN
    rates = (250, 1000, 5000, 20000, 50000, 100000, 200000)
    dist = sweep(DISTANCE, rates)
    med = sweep(MEDIAN, rates)
    store.close()
    return {"workload": "serving_requests_poisson_1-64pairs_lognormal1000", **cfg,
            "distance": dist, "median": med, "cpu_baseline": serving_cpu(w)}


def serving_cpu(w, target_s: float = 5.0) -> dict:
    """DOS.median of the serving pool's pairs on all host cores (the host
    implementation; a pilot of 64 pairs sizes a sample of about target_s)."""
    host_oracle()
    import oracle_lib
    orc = oracle_lib.Oracle("port")
    ocm = orc.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    pairs = w.pairs
    t0 = time.perf_counter()
    orc.median_batch(ocm, [a for a, _ in pairs[:64]], [b for _, b in pairs[:64]], True)
    pilot = time.perf_counter() - t0
    n = int(min(len(pairs), max(64, 64 * target_s / max(pilot, 1e-6))))
    sub = pairs[:n]
    t0 = time.perf_counter()
    orc.median_batch(ocm, [a for a, _ in sub], [b for _, b in sub], True)
    dt = time.perf_counter() - t0
    cells = sum(len(a) * len(b) for a, b in sub)
    return {"alignments_per_s": round(n / dt, 1), "gcups": round(cells / dt / 1e9, 4),
            "kind": "port", "cores": os.cpu_count(), "cpu_model": host_cpu(),
            "sample": f"first {n} pairs of the serving pool, DOS.median ({dt:.1f} s)"}


def _reduce(x: float, world: int, op: str) -> float:
    """All-reduce one scalar across ranks (NCCL on GPUs, gloo on CPU)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def reduce_max(x: float, world: int) -> float:
    return _reduce(x, world, "max")


def reduce_sum(x: float, world: int) -> float:
    return _reduce(x, world, "sum")


def gpu_line(args, r) -> dict:
    world = r["world"]
    ms = reduce_max(r["ms"], world)
    cells = reduce_sum(r["cells"], world)
    pairs = reduce_sum(r["n"], world)
    computed = reduce_sum(r["computed"], world)
    gcups = cells / (ms * 1e-3) / 1e9
    model = r["model"]
    prof = r["prof"]
    nb = max(prof["batches"], 1)
    cls_ms = {k: v / nb for k, v in prof.items() if k.startswith("class")}
    fill_ms = sum(cls_ms.values())
    dom = max(cls_ms, key=cls_ms.get)
    peaks = measured_peaks()
    # HBM view of the class kernels: direction codes written per filled cell,
    # sequences read, outputs written (algorithmic bytes)
    pk = r["pk"]
    alg_bytes = (r["computed"] * DM_BYTES[model] + int(pk.seqs.nbytes) + 4 * int(pk.out_bytes))
    gbs = alg_bytes / (fill_ms * 1e-3) / 1e9
    hbm_peak = peaks.get("hbm_gbs")
    clk = r["clocks"]
    sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz") or 2070.0
    nsm = 152
    try:
        import torch
        nsm = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    # measured integer issue rate, scaled from the microbenchmark's clock to
    # the clock sampled during the timed steps
    pk_ = r["peak"]
    pmhz = pk_["clocks"].get("sm_mhz") or sm_mhz
    int_peak = pk_["peak_tops"] * (sm_mhz / pmhz)
    int_ach = r["computed"] * OPS_PER_CELL[model] / (fill_ms * 1e-3) / 1e12
    nominal = nsm * 128 * sm_mhz * 1e6 / 1e12
    line = {
        "metric": METRIC, "value": round(gcups, 3), "unit": "GCUPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
        "config": {"workload": r["w"].name, "pairs_per_gpu": r["n"],
                   "cost_model": (f"affine open {r['w'].gap_open} ext {r['w'].indel} "
                                  f"subs {r['w'].subs}" if r["w"].affine else
                                  f"linear subs {r['w'].subs} indel {r['w'].indel}"),
                   "cells_per_gpu": r["cells"], "cells_computed_per_gpu": r["computed"],
                   "parallelism": f"replicas{world}",
                   "launch": "one CUDA graph per step (captured batch launch sequence)",
                   "ladder": (r["tuned"]["ladder"] if r["tuned"] else "default"),
                   "l2": "inputs+outputs+direction slabs > 129 MB L2 (no flush needed)"},
        "alignments_per_s": round(pairs / (ms * 1e-3), 1),
        "gcups_computed_cells": round(computed / (ms * 1e-3) / 1e9, 3),
        "gpu_launches": r["launches"] * args.steps,
        "roofline": {"bound": "int32", "kernel": "class kernels (band fill), dominant " + dom,
                     "ops_per_cell": OPS_PER_CELL[model],
                     "achieved": round(int_ach, 2), "peak": round(int_peak, 2),
                     "unit": "Tops", "frac": round(int_ach / int_peak, 4),
                     "traffic": (round(r["computed"] * DRAM_BYTES_PER_CELL[model])
                                 if model in DRAM_BYTES_PER_CELL else None),
                     "traffic_source": "ncu dram bytes per computed cell (class kernels), "
                                       "scaled by computed cells; per step",
                     "peak_source": (f"measured: poyalgn_int32_peak, fastest single-op kind "
                                     f"({pk_['peak_kind']}) {pk_['peak_tops']:.2f} "
                                     f"T thread-inst/s at {pmhz:.0f} MHz, scaled to "
                                     f"{sm_mhz:.0f} MHz"),
                     "achieved_source": "computed cells x ops per cell / summed class-kernel "
                                        "event time per step (launch_ms)",
                     "frac_of_nominal_128_lanes": round(int_ach / nominal, 4)},
        "int32_rates_tinst_s": {k: round(v["tinst_per_s"], 2)
                                for k, v in pk_["kinds"].items()},
        "roofline_hbm": {"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm_peak,
                         "unit": "GB/s", "frac": round(gbs / hbm_peak, 4) if hbm_peak else None,
                         "bytes": "direction bytes per computed cell + sequences + outputs",
                         "peak_source": "measured" if hbm_peak else None},
        "launch_ms": {k: round(v / nb, 3) for k, v in prof.items() if k != "batches"},
        "clocks": {"sm_mhz": clk.get("sm_mhz"), "sm_max_mhz": clk.get("sm_max_mhz"),
                   "reasons": clk.get("reasons")},
        "passes_mean": round(float(np.mean(r["passes"])), 3),
        "plain_per_call": {"value": round(r["plain"]["gcups"], 3), "unit": "GCUPS",
                           "alignments_per_s": round(r["plain"]["alignments_per_s"], 1),
                           "sample": f"first {r['plain']['pairs']} pairs, one stub call each"},
        "batched_over_plain": round(gcups / max(r["plain"]["gcups"], 1e-9), 1),
    }
    if r["parity"]:
        line["parity"] = r["parity"]
    if r["e2e"]:
        e = r["e2e"]
        e_s = reduce_max(e["seconds"], world)
        line["e2e"] = {"value": round(cells / e_s / 1e9, 3), "unit": "GCUPS",
                       "h2d_bytes_per_step": e["h2d"], "d2h_bytes_per_step": e["d2h"],
                       "alignments_per_s": round(pairs / e_s, 1), "step_ms": e["step_ms"]}
    return line


def main(argv=None):
    args = parse_args(argv)
    rank, world, local = dist_info()
    if args.leg != "main" and args.impl == "gpu":
        import torch
        torch.cuda.set_device(local)
        if args.leg == "peak":
            import poy5_gb300 as pg
            clk = ClockSampler(local)
            clk.start()
            out = pg.int32_rates(local)
            out["clocks"] = clk.stop()
        elif args.leg == "plain":
            out = run_plain(local)
        elif args.leg == "percall":
            out = run_percall(local, args.percall_seconds)
        elif args.leg == "downpass":
            out = run_downpass(local)
        elif args.leg == "long":
            out = run_long(local, n_pairs=args.pairs or 512, mem_gb=args.mem_gb)
        elif args.leg == "serving":
            out = run_serving(local, args.serve_seconds, args.serve_slots, args.serve_batch)
        elif args.leg == "newkk":
            out = run_newkk(local, args.pairs or 65536, arena_mb=args.newkk_arena_mb)
        elif args.leg == "powell3d":
            out = run_powell3d(local, args.pairs or 8192)
        else:
            out = run_distance(local, args.pairs or 8192)
        print(json.dumps({"leg": args.leg, **out}))
        return 0
    if args.impl == "reference":
        if rank != 0:
            return 0
        w = make_workload(args.workload, args.pairs, 0)
        threads = os.cpu_count() or 1
        per = max(args.cpu_seconds / max(args.steps, 1), 1.0)
        for _ in range(args.warmup):
            cpu_rate(w, min(per, 1.0), threads)
        rates = [cpu_rate(w, per, threads) for _ in range(args.steps)]
        cps = float(np.median([x["cells_per_s"] for x in rates]))
        aps = float(np.median([x["pairs_per_s"] for x in rates]))
        kind = rates[0]["kind"]
        v = round(cps / 1e9, 4)
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "GCUPS",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(1e3 * float(np.median([x["seconds"] for x in rates])), 1),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "int32", "data": "synthetic (seeded)",
                "config": {"workload": w.name, "pairs_per_step": rates[0]["pairs"]},
                "alignments_per_s": round(aps, 2),
                "cpu_baseline": {"value": v, "unit": "GCUPS", "cores": rates[0]["threads"],
                                 "kind": kind, "cpu_model": host_cpu(),
                                 "sample": f"first {rates[0]['pairs']} pairs of {w.name} per step"},
                "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    r = run_gpu(args)
    line = gpu_line(args, r)
    if rank == 0:
        cpu = cpu_rate(r["w"], args.cpu_seconds, os.cpu_count() or 1)
        line["cpu_baseline"] = {
            "value": round(cpu["cells_per_s"] / 1e9, 4), "unit": "GCUPS",
            "cores": cpu["threads"], "kind": cpu["kind"], "cpu_model": host_cpu(),
            "sample": f"first {cpu['pairs']} pairs of {r['w'].name} ({cpu['seconds']:.1f} s)",
            "alignments_per_s": round(cpu["pairs_per_s"], 2)}
        if world == 1 and not args.no_extras:
            line["plain_pairs"] = run_plain(local)
            line["downpass"] = run_downpass(local)
            line["long_pairs"] = run_long(local)
            line["distance"] = run_distance(local)
            try:
                line["newkk"] = run_newkk(local)
            except Exception as e:  # keep the headline line if this leg fails
                line["newkk"] = {"error": f"{type(e).__name__}: {e}"[:300]}
            line["serving"] = run_serving(local, args.serve_seconds, args.serve_slots,
                                          args.serve_batch)
            try:
                line["powell3d"] = run_powell3d(local)
            except Exception as e:  # keep the headline line if this leg fails
                line["powell3d"] = {"error": f"{type(e).__name__}: {e}"[:300]}
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
