"""Benchmark: all-pairs Needleman-Wunsch distance matrix on one GB300.

Workload (default): benchmark configuration 2 -- 10,000 synthetic protein
sequences in 50 families of 200, lognormal root lengths (median 350, sigma
0.6, clipped 30-4000), ~5e7 pairs, scored by the batched persistent
length-bucketed kernels (int16x2 DPX lanes with int32 for pairs the overflow
guard routes there).  One step = the full 10,000 x 10,000 distance matrix.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  value = GCUPS (sum over i<j of L_i*L_j per
second) with codes and matrix resident in HBM; e2e = the same metric through
the host-buffer C ABI call (nwg_score_all: codes host->device, matrix
device->host inside the timed region).  The line also carries the serving
run (Poisson job arrivals, continuous batching): p50/p99 job latency and
sustained GCUPS beside the same jobs run one by one, then a sweep of the
arrival rate (500-4000 jobs/s) to where the server stops keeping up, and the configuration-3
pipeline (matrix -> neighbor joining -> cherry traceback of 8,000 sequences,
checked against the reference's own tree) with the NJ and traceback
rooflines.  --impl reference times the
reference's recurrence restated on the CPU (its CUDA does not build on CUDA
13) on every host core, on a bounded sample of the same pairs.

Multi-GPU (torchrun, N>1): every rank scores its own replica of the workload
(families drawn with a rank-dependent seed); no data-path collective; the
result is weak scaling, value = all ranks' cells / max rank time.
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

CONFIG = 2
METRIC = "nw_gcups_batched"
UNIT = "GCUPS"
# DRAM bytes per launch of the dominant kernel of this workload, from one ncu capture of
# the full-size launch (profiles/wave_kernel_24_v4_w16_config2_small.md); reported only
# when that kernel is the dominant one of the run
NCU_TRAFFIC = {"wave_kernel<R=24,int16x2,V=4,W=16>": 69883392 + 127747584}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def replica_seed(rank: int) -> int:
    """Seed of the workload replica a rank scores (rank 0: the configuration's own seed)."""
    from mestrado_gb300 import synth
    return synth.config_seed(CONFIG) + 1000003 * rank


def aggregate_gcups(world, cells: float, seconds: float) -> float:
    """Whole-job GCUPS: the cells of every rank over the slowest rank's time."""
    return _sum_over_ranks(world, float(cells)) / _max_over_ranks(world, seconds) / 1e9


class ClockSampler:
    """nvidia-smi clock/throttle sampling while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

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
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": float(max(power)) if power else None}


def cpu_baseline(S, target_s: float, threads: int, seed: int = 7):
    """Oracle (the reference's recurrence restated in C, OpenMP over pairs) on a
    seeded random sample of the workload's pairs sized to ~target_s seconds."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_py as O
    O.build()
    codes, off = O.encode(S)
    n = len(S)
    rng = np.random.default_rng(seed)
    L = S.lengths.astype(np.float64)

    def sample(k):
        i = rng.integers(0, n, k)
        j = rng.integers(0, n, k)
        m = i != j
        return i[m].astype(np.int32), j[m].astype(np.int32)

    pi, pj = sample(64 * threads)
    t0 = time.perf_counter()
    O.score_list(codes, off, pi, pj, threads=threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    rate = float((L[pi] * L[pj]).sum()) / dt
    want_cells = rate * target_s
    mean_cells = float((L[pi] * L[pj]).mean())
    k = int(max(64, want_cells / mean_cells))
    pi, pj = sample(k)
    cells = float((L[pi] * L[pj]).sum())
    t0 = time.perf_counter()
    O.score_list(codes, off, pi, pj, threads=threads)
    dt = time.perf_counter() - t0
    value = cells / dt / 1e9
    # one core, on a sample of about a quarter of target_s
    k1 = int(max(16, value * 1e9 / threads * target_s / 4 / mean_cells))
    qi, qj = sample(k1)
    c1 = float((L[qi] * L[qj]).sum())
    t0 = time.perf_counter()
    O.score_list(codes, off, qi, qj, threads=1)
    d1 = time.perf_counter() - t0
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(pi)} seeded random pairs of configuration {CONFIG} ({cells:.3g} cells, "
                      f"{dt:.1f} s), GCUPS = cells / time",
            "one_core": {"value": c1 / d1 / 1e9, "pairs": len(qi), "seconds": d1}}


def _serve_arrivals(srv, jobs, keep=()):
    """Submit `jobs` ((arrival_s, seqs) pairs) to `srv` at their arrival times
    and wait for each from a second thread; returns (infos, kept results,
    wall seconds from the first arrival, largest submit lag)."""
    import queue
    count = len(jobs)
    q: "queue.Queue" = queue.Queue()
    infos = [None] * count
    kept = {}

    def waiter():
        for _ in range(count):
            k, jid = q.get()
            D, J, info = srv.wait(jid, len(jobs[k][1]))
            infos[k] = info
            if k in keep:
                kept[k] = (D, J)

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    lag = 0.0
    for k, (ta, S) in enumerate(jobs):
        dt = t0 + ta - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        else:
            lag = max(lag, -dt)
        q.put((k, srv.submit(S)))
    th.join()
    return infos, kept, time.perf_counter() - t0, lag


def serving_sweep(rates=(500.0, 1000.0, 2000.0, 3000.0, 4000.0), seconds: float = 5.0):
    """The serving workload at higher Poisson rates, `seconds` of arrivals
    each (one Server, warmed): per rate the latency percentiles, the mean
    batch size and the sustained against the offered cell rate.  A rate is
    kept up with when the last job returns within a second of the last
    arrival and sustained >= 0.95 x offered."""
    from mestrado_gb300 import Server, synth
    out = []
    srv = Server(10, 2, hbm_budget=16 << 30, max_batch_jobs=256)
    for _, S in synth.serving_jobs(16, 200.0, seed=99):
        srv.wait(srv.submit(S), len(S))
    for rate in rates:
        jobs = synth.serving_jobs(max(1, int(seconds * rate)), rate, seed=1000 + int(rate))
        cells = float(sum(S.cells() for _, S in jobs))
        infos, _, wall, lag = _serve_arrivals(srv, jobs)
        lat = np.array([i["latency_ms"] for i in infos])
        batch = np.array([i["batch_jobs"] for i in infos])
        span = jobs[-1][0]
        offered = cells / span / 1e9
        sustained = cells / wall / 1e9
        out.append({"rate_jobs_per_s": rate, "jobs": len(jobs),
                    "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                                   "max": float(lat.max())},
                    "batch_jobs_mean": float(batch.mean()), "batch_jobs_max": int(batch.max()),
                    "offered_gcups": offered, "sustained_gcups": sustained,
                    "kept_up": bool(wall - span < 1.0 and sustained >= 0.95 * offered),
                    "submit_lag_max_s": lag, "ok": all(i["status"] == 0 for i in infos)})
    srv.close()
    return out


def serving_leg(seconds: float, rate: float = 200.0, sample_jobs: int = 200, sweep: bool = True):
    """The serving workload: Poisson arrivals at `rate` jobs/s for `seconds`
    (each job a family of log-uniform 8-512 sequences, lognormal root length
    median 250, sigma 0.5, clipped 30-2000), submitted at their arrival times
    to one Server; latency = submit -> matrix and tree on the host.  Beside it,
    the first `sample_jobs` jobs run job by job through a context (plain
    per-pair form, and the batched form), scoring + NJ, host buffers."""
    from mestrado_gb300 import MODE_BATCHED, MODE_PLAIN, Context, Server, synth
    count = max(1, int(seconds * rate))
    jobs = synth.serving_jobs(count, rate)
    warm = synth.serving_jobs(16, rate, seed=99)
    cells = np.array([S.cells() for _, S in jobs], dtype=np.float64)
    check = set(np.random.default_rng(5).choice(count, size=min(count, 24), replace=False).tolist())
    srv = Server(10, 2, hbm_budget=16 << 30, max_batch_jobs=256)
    for _, S in warm:
        srv.wait(srv.submit(S), len(S))
    infos, kept, wall, lag = _serve_arrivals(srv, jobs, check)
    srv.close()
    lat = np.array([i["latency_ms"] for i in infos])
    qms = np.array([i["queue_ms"] for i in infos])
    batch = np.array([i["batch_jobs"] for i in infos])
    ok = all(i["status"] == 0 for i in infos)
    # job by job through a context, and the exactness check of the kept jobs
    ctx = Context(10, 2)
    ctx.autotune()
    keys = ("i", "j", "node", "len_i", "len_j")
    parity = ok
    for k, (D, J) in kept.items():
        S = jobs[k][1]
        Dr = ctx.score_all(S)
        parity = parity and bool(np.array_equal(D, Dr))
        if len(S) > 1:
            Jr = ctx.nj(Dr)
            parity = parity and all(tuple(a[x] for x in keys) == tuple(b[x] for x in keys) for a, b in zip(J, Jr))
    m = min(sample_jobs, count)
    jbj = {}
    for name, mode in (("plain", MODE_PLAIN), ("batched", MODE_BATCHED)):
        for _, S in warm[:4]:
            ctx.score_all(S, mode=mode)
        ts, tn = [], []
        for _, S in jobs[:m]:
            t1 = time.perf_counter()
            D = ctx.score_all(S, mode=mode)
            t2 = time.perf_counter()
            if len(S) > 1:
                ctx.nj(D)
            ts.append(t2 - t1)
            tn.append(time.perf_counter() - t1)
        c = float(cells[:m].sum())
        jbj[name] = {"gcups_scoring": c / sum(ts) / 1e9, "gcups_with_nj": c / sum(tn) / 1e9,
                     "job_p50_ms": float(np.percentile(tn, 50) * 1e3),
                     "job_p99_ms": float(np.percentile(tn, 99) * 1e3),
                     "jobs_per_s": m / sum(tn)}
    ctx.close()
    served = cells.sum() / wall / 1e9
    return {
        "workload": f"Poisson arrivals at {rate:g} jobs/s for {seconds:g} s ({count} jobs), seeded; per job "
                    "log-uniform 8-512 seqs, root lognormal (median 250, sigma 0.5, clipped 30-2000)",
        "jobs": count, "rate_jobs_per_s": rate, "wall_s": wall, "submit_lag_max_s": lag,
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p90": float(np.percentile(lat, 90)),
                       "p99": float(np.percentile(lat, 99)), "max": float(lat.max()), "mean": float(lat.mean())},
        "queue_ms": {"p50": float(np.percentile(qms, 50)), "p99": float(np.percentile(qms, 99))},
        "batch_jobs": {"mean": float(batch.mean()), "max": int(batch.max())},
        "sustained_gcups": served,
        "offered_gcups": float(cells.sum() / jobs[-1][0] / 1e9),
        "job_by_job": {"jobs": m, **jbj},
        "serving_over_plain_job_by_job": served / jbj["plain"]["gcups_with_nj"],
        "exact": parity, "checked_jobs": len(kept),
        "reference_identical_jobs": int(sum(i["nj_reference_identical"] for i in infos)),
        "rate_sweep": serving_sweep() if sweep else None,
    }


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0}, "fallback"


def config1_leg():
    """Configuration 1: 2,000 sequences in 10 families of 200 (lengths about
    300-600), all pairs, in the plain form (one thread per pair, int32, one
    launch per pair-length group) and in the batched form, device-resident,
    each timed once after a warm-up with CUDA events on the library's stream;
    the two matrices must be equal."""
    import torch

    from mestrado_gb300 import MODE_BATCHED, MODE_PLAIN, Context, encode, synth
    S = synth.config(1)
    n = len(S)
    cells = S.cells()
    codes, off = encode(S)
    ctx = Context(10, 2)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.autotune()
    d_codes = torch.from_numpy(codes).to("cuda")
    out = {}
    mats = {}
    for name, mode in (("plain", MODE_PLAIN), ("batched", MODE_BATCHED)):
        d_D = torch.empty((n, n), dtype=torch.float32, device="cuda")
        with torch.cuda.stream(stream):
            ctx.score_all_dev(d_codes.data_ptr(), off, d_D.data_ptr(), n, mode)   # warm-up (plan, graph)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.score_all_dev(d_codes.data_ptr(), off, d_D.data_ptr(), n, mode)
            b.record(stream)
            torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        out[name] = {"gcups": cells / (ms / 1e3) / 1e9, "ms": ms}
        mats[name] = d_D.cpu().numpy()
    ctx.close()
    return {"workload": "configuration 1: 2000 seqs, 10 families x 200, root 450, p_s 0.08 (lengths about "
                        "300-600), all pairs incl. diagonal; device-resident",
            "pairs": n * (n + 1) // 2, "cells": cells, **out,
            "batched_over_plain": out["batched"]["gcups"] / out["plain"]["gcups"],
            "matrices_equal": bool(np.array_equal(mats["plain"], mats["batched"]))}


def pipeline_leg(cpu_nj_n: int = 2000):
    """Configuration 3 end to end through the public API (host buffers): 8,000
    sequences -> distance matrix -> neighbor joining -> cherry traceback,
    checked against the tree the reference's own buildTree made on the same
    matrix (tests/golden/cfg3).  NJ roofline: the live upper triangle read
    once per join (4 B per live pair; the candidate pass revisits only rows
    whose float minimum is near the global one).  Traceback roofline: 0.5 B
    of direction flags written per DP cell.  CPU: the oracle's neighbor
    joining (the reference's buildTree restated, one core) on the leading
    cpu_nj_n x cpu_nj_n block of the same matrix, beside the device on the
    same block."""
    import hashlib

    from mestrado_gb300 import Context, cherries, encode, newick, synth
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_py as O
    from test_nj_cpu import golden_joins
    gold = os.path.join(ROOT, "tests", "golden", "cfg3")
    meta = json.load(open(os.path.join(gold, "meta.json")))
    S = synth.config(3)
    n = len(S)
    ctx = Context(10, 2)
    ctx.autotune()
    ctx.score_all(S)                                   # plan, graph and tuning warm
    # one untimed pass of the later stages: their kernels' first launches (module
    # loading) and their buffers stay out of the timed pass
    Dw = ctx.score_all(S)
    jw = ctx.nj(Dw)
    _, lw, rw = cherries(jw["i"], jw["j"], len(S))
    cw, ow = encode(S)
    ctx.align_pairs(cw, ow, lw, rw)
    ctx.msa(codes=cw, offsets=ow, left=jw["i"], right=jw["j"])
    del Dw
    t0 = time.perf_counter()
    D = ctx.score_all(S)
    t1 = time.perf_counter()
    joins, st = ctx.nj(D, stats=True)
    t2 = time.perf_counter()
    node, left, right = cherries(joins["i"], joins["j"], n)
    codes, off = encode(S)
    t3 = time.perf_counter()
    aln, ast = ctx.align_pairs(codes, off, left, right, stats=True)
    t4 = time.perf_counter()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    # progressive alignment of all 8,000 along the tree (this library's definition: the reference's
    # computeMSA is an empty loop), and the oracle's restatement of it on configuration 0 (64 sequences)
    rows, mst = ctx.msa(codes=codes, offsets=off, left=joins["i"], right=joins["j"], stats=True)
    t5m = time.perf_counter()
    from fasta import read_fasta
    _, seqs0 = read_fasta(os.path.join(ROOT, "tests", "golden", "cfg0", "input.fasta"))
    j0 = golden_joins("cfg0")
    tc0 = time.perf_counter()
    O.msa(seqs0, j0["i"], j0["j"])
    tc1 = time.perf_counter()
    ctx.msa(seqs0, j0["i"], j0["j"])
    tc2 = time.perf_counter()
    rows_ok = all(rows[k].replace(b"-", b"") == S[k] for k in range(0, n, max(1, n // 200)))
    ref = golden_joins("cfg3")
    exact = (hashlib.sha256(D.tobytes()).hexdigest() == meta["D_sha256"] and len(joins) == len(ref) and
             all((a["node"], a["i"], a["j"], a["len_i"], a["len_j"]) == (b["node"], b["i"], b["j"], b["len_i"], b["len_j"])
                 for a, b in zip(joins, ref)) and
             newick(joins, [f">s{i}" for i in range(n)]) == open(os.path.join(gold, "tree.nwk")).read())
    peaks, src = _peaks()
    hbm = float(peaks["hbm_gbs"])
    nj_bytes = sum(4.0 * m * (m - 1) / 2 for m in range(2, n + 1))
    nj_gbs = nj_bytes / (st["device_ms"] * 1e-3) / 1e9
    L = S.lengths.astype(np.float64)
    tb_cells = float((L[left] * L[right]).sum())
    tb_s = ast["kernel_ms"] * 1e-3 if ast.get("kernel_ms") else (t4 - t3)   # the match kernels (DP + walk)
    tb_gbs = 0.5 * tb_cells / tb_s / 1e9
    # CPU neighbor joining (oracle, one core) and the device on the same leading block
    m = min(cpu_nj_n, n)
    Dm = np.ascontiguousarray(D[:m, :m])
    t5 = time.perf_counter()
    O.nj(Dm.copy())
    t6 = time.perf_counter()
    ctx.nj(Dm)
    t7 = time.perf_counter()
    ctx.nj(Dm)
    t8 = time.perf_counter()
    ctx.close()
    return {
        "workload": "configuration 3: 8,000 seqs (40 families x 200, root length U[100,300]), all pairs -> NJ -> "
                    "pairwise alignment of every guide-tree cherry -> progressive alignment along the tree; host "
                    "buffers through the public API",
        "exact_vs_reference_tree": bool(exact),
        "score_s": t1 - t0, "nj_s": t2 - t1, "nj_device_s": st["device_ms"] * 1e-3, "nj_launches": st["launches"],
        "nj_rebuilds": st["rebuilds"], "nj_ambiguous_steps": st["ambiguous_steps"],
        "traceback_s": t4 - t3, "cherries": int(len(left)), "total_s": t5m - t0,
        "msa": {"s": t5m - t4, "device_s": mst["kernel_ms"] * 1e-3, "columns": len(rows[0]) if rows else 0,
                "cells": mst["cells"], "gcups": mst["cells"] / max(mst["kernel_ms"] * 1e-3, 1e-9) / 1e9,
                "launches": mst["launches"], "rows_are_sequences": bool(rows_ok),
                "cpu_config0": {"oracle_one_core_s": tc1 - tc0, "device_s": tc2 - tc1, "n": len(seqs0),
                                "kind": "port"}},
        "nj_roofline": {"bound": "hbm", "achieved": nj_gbs, "peak": hbm, "unit": "GB/s", "frac": nj_gbs / hbm,
                        "bytes": nj_bytes, "peak_source": src},
        "traceback_roofline": {"bound": "hbm", "achieved": tb_gbs, "peak": hbm, "unit": "GB/s", "frac": tb_gbs / hbm,
                               "cells": tb_cells, "kernel_s": tb_s, "gcups": tb_cells / tb_s / 1e9,
                               "d2h_s": ast.get("d2h_ms", 0.0) * 1e-3, "peak_source": src},
        "cpu_nj": {"n": m, "oracle_one_core_s": t6 - t5, "device_s": t8 - t7, "kind": "port",
                   "note": "the reference's buildTree restated (exact argmin), one core"},
    }


def run_reference(args, world, rank):
    if rank != 0:
        return
    from mestrado_gb300 import synth
    S = synth.config(CONFIG)
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_py as O
    O.build()
    codes, off = O.encode(S)
    n = len(S)
    rng = np.random.default_rng(3)
    L = S.lengths.astype(np.float64)
    # size one step to ~4 s on this host
    pi = rng.integers(0, n, 32 * threads).astype(np.int32)
    pj = rng.integers(0, n, 32 * threads).astype(np.int32)
    t0 = time.perf_counter()
    O.score_list(codes, off, pi, pj, threads=threads)
    rate = float((L[pi] * L[pj]).sum()) / max(time.perf_counter() - t0, 1e-3)
    k = int(max(64, rate * 4.0 / float((L[pi] * L[pj]).mean())))
    pi = rng.integers(0, n, k).astype(np.int32)
    pj = rng.integers(0, n, k).astype(np.int32)
    cells = float((L[pi] * L[pj]).sum())
    for _ in range(args.warmup):
        O.score_list(codes, off, pi[: max(1, k // 8)], pj[: max(1, k // 8)], threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.score_list(codes, off, pi, pj, threads=threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    v = cells * args.steps / tot / 1e9
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": f"configuration {CONFIG}: 10000 seqs, 50 families x 200, lognormal "
                               "lengths (median 350, sigma 0.6, 30-4000)",
                   "sample_pairs": int(k), "l2": "host run"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{k} seeded random pairs per step ({cells:.3g} cells); the reference's "
                                   "recurrence (NeedlemanWunsch.cu:22-161) restated in C, OpenMP over pairs; "
                                   "its own CUDA kernel does not build on CUDA 13"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_shard(args, world, rank, local):
    """--shard: ONE configuration-2 matrix split over the ranks (strong
    scaling): rank k scores its cell-balanced row block against the columns
    from its first row on (nwg_score_block), the blocks are all-gathered
    over the process group (host buffers) and mirrored into the full matrix
    on every rank (mestrado_gb300/shard.py).  value = the matrix's cells per
    step / the slowest rank's step time; the timed region includes the
    host-side gather, so value and e2e are the same measurement."""
    import torch
    torch.cuda.set_device(local)
    from mestrado_gb300 import Context, shard, synth
    S = synth.generate(synth.config_spec(CONFIG), replica_seed(0))
    if args.subset:
        S = S.subset(range(min(args.subset, len(S))))
    seqs = [S[i] for i in range(len(S))]
    n, cells = len(seqs), S.cells()
    ctx = Context(10, 2)
    ctx.autotune()
    for _ in range(args.warmup):
        D = shard.sharded_score_all(ctx, seqs, rank, world, device="cpu")
    clocks = ClockSampler(local)
    clocks.start()
    _barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        D = shard.sharded_score_all(ctx, seqs, rank, world, device="cpu")
    _barrier(world)
    t = _max_over_ranks(world, time.perf_counter() - t0)
    clk = clocks.stop()
    b = shard.tile_plan([len(s) for s in seqs], world)
    value = cells * args.steps / t / 1e9
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "int16x2+int32", "data": "synthetic",
            "config": {"workload": f"configuration {CONFIG}: one {n} x {n} matrix split over {world} rank(s) by "
                                   "cell-balanced row blocks, all-gathered on the host",
                       "cells_per_step": cells, "parallelism": f"row-block split over {world} GPU(s)",
                       "row_bounds": [int(x) for x in b],
                       "block_cells": [float(c) for c in shard.block_cells([len(s) for s in seqs], b)]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(sum(len(s) for s in seqs)),
                    "d2h_bytes_per_step": int(4 * (b[rank + 1] - b[rank]) * (n - b[rank]))},
            "matrix_symmetric": bool(np.array_equal(D, D.T)),
            "gpu_launches": None, "clocks": clk}), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--subset", type=int, default=0,
                    help="score only the first N sequences (whole families first); for profiling runs")
    ap.add_argument("--no-pipeline", action="store_true", help="skip the configuration-3 pipeline leg")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="length of the serving run (Poisson arrivals at 200 jobs/s, configuration 4: "
                         "60 s); 0 skips it")
    ap.add_argument("--shard", action="store_true",
                    help="N>1: split ONE configuration-2 matrix over the ranks (strong scaling) instead of replicas")
    ap.add_argument("--no-serve-sweep", action="store_true",
                    help="skip the sweep of the serving arrival rate (500-4000 jobs/s, 5 s each)")
    ap.add_argument("--quick", action="store_true",
                    help="device-resident timing only (no e2e, plain, CPU or parity legs); for profiling runs")
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.shard:
        run_shard(args, world, rank, local)
        return

    import torch
    torch.cuda.set_device(local)
    from mestrado_gb300 import MODE_BATCHED, MODE_PLAIN, Context, encode, synth

    spec = synth.config_spec(CONFIG)
    seed = replica_seed(rank)
    S = synth.generate(spec, seed)
    if args.subset:
        S = S.subset(range(min(args.subset, len(S))))
    n = len(S)
    cells = S.cells()
    codes, off = encode(S)
    ctx = Context(10, 2)
    # a dedicated stream: the library launches on it and the CUDA events below
    # are recorded on it (torch's default stream has handle 0, which the C ABI
    # reads as "use the context's own stream")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    d_codes = torch.from_numpy(codes).to("cuda")
    d_D = torch.empty((n, n), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > L2

    # kernel choice per length class (cached per device after the first run)
    tuning = ctx.autotune()

    # roofline denominator: the ALU pipe, which executes the DPX max
    # operations, at its full rate.  The int32 cell-update form 2 (4 DPX + 1
    # add per cell, registers only, every SM) keeps that pipe 99.98 % busy
    # (ncu), so its cells/s x 4 is the pipe's lane-op rate in this run; the
    # leanest cell update needs 1.5 ALU lane-ops per int16x2 cell (2 viaddmax +
    # 1 vimax3 per two-cell word) and 3 per int32 cell.
    alu_lane_ops = ctx.dpx_peak(False, form=2) * 4.0
    peak16 = alu_lane_ops / 1.5
    peak32 = alu_lane_ops / 3.0
    micro16 = ctx.dpx_peak(True)    # the fastest complete cell update, for reference

    for _ in range(args.warmup):
        ctx.score_all_dev(d_codes.data_ptr(), off, d_D.data_ptr(), n, MODE_BATCHED)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    _barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches = 0
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()                      # L2 flushed between timed steps
        ev[k][0].record(stream)
        st = ctx.score_all_dev(d_codes.data_ptr(), off, d_D.data_ptr(), n, MODE_BATCHED, stats=False)
        ev[k][1].record(stream)
        launches += 0 if st is None else st["launches"]
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    _barrier(world)
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    tot_s = sum(step_ms) / 1e3
    tot_s_max = _max_over_ranks(world, tot_s)
    value = aggregate_gcups(world, float(cells) * args.steps, tot_s)

    # launches of one step and the dominant launch, timed alone (events around each launch)
    ctx.set_launch_timing(True)
    flush.zero_()
    st = ctx.score_all_dev(d_codes.data_ptr(), off, d_D.data_ptr(), n, MODE_BATCHED, stats=True)
    recs = ctx.launch_records()
    ctx.set_launch_timing(False)
    timed_sum_ms = sum(r["ms"] for r in recs)
    per_step_launches = st["launches"]
    launches = per_step_launches * args.steps
    dom = max(recs, key=lambda r: r["ms"]) if recs else None

    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                              "quick": True, "n": n, "cells_per_step": cells,
                              "launch_records": recs, "peak16_gcups": peak16 / 1e9, "tuning": tuning}),
                  flush=True)
        return

    # parity spot check of this run's matrix against the oracle (small sample)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_py as O
    O.build()
    rng = np.random.default_rng(17)
    pi = rng.integers(0, n, 64)
    pj = rng.integers(0, n, 64)
    Dh = d_D.cpu().numpy()
    ref = O.score_list(codes, off, pi, pj, threads=os.cpu_count() or 1)
    parity = bool(np.array_equal(Dh[pi, pj], ref.astype(np.float32))) and bool(np.array_equal(Dh, Dh.T))

    # end to end through the host-buffer C ABI call: pinned codes in, matrix out
    h_codes = torch.from_numpy(codes).pin_memory()
    h_D = torch.empty((n, n), dtype=torch.float32).pin_memory()
    ctx.set_stream(None)
    torch.cuda.synchronize()
    e2e_times = []
    for k in range(max(1, args.steps)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.score_all(codes=h_codes.numpy(), offsets=off, out=h_D.numpy(), mode=MODE_BATCHED)
        e2e_times.append(time.perf_counter() - t0)
    e2e = {"value": aggregate_gcups(world, float(cells) * len(e2e_times), sum(e2e_times)), "unit": UNIT,
           "h2d_bytes_per_step": int(codes.nbytes + off.nbytes), "d2h_bytes_per_step": int(n * n * 4)}
    parity = parity and bool(np.array_equal(h_D.numpy(), Dh))
    ctx.set_stream(stream.cuda_stream)

    # plain form (one thread per pair, int32, launch per length group) once, for the batched/plain ratio
    plain = None
    if not args.no_plain:
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.score_all_dev(d_codes.data_ptr(), off, d_D.data_ptr(), n, MODE_PLAIN)
        b.record(stream)
        torch.cuda.synchronize()
        pms = a.elapsed_time(b)
        plain = {"gcups": cells / (pms / 1e3) / 1e9, "ms": pms,
                 "matrix_equal": bool(np.array_equal(d_D.cpu().numpy(), Dh))}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(S, args.cpu_seconds, os.cpu_count() or 1)

    if rank != 0:
        return
    config1 = None if args.no_plain else config1_leg()
    serving = serving_leg(args.serve_seconds, sweep=not args.no_serve_sweep) if args.serve_seconds > 0 else None
    pipeline = None if args.no_pipeline else pipeline_leg()
    roof = None
    if dom is not None:
        peak = peak16 if dom["lanes16"] else peak32
        ach = dom["cells"] / (dom["ms"] / 1e3)
        kname = (f"wave_kernel<R={dom['rows_per_lane']},{'int16x2' if dom['lanes16'] else 'int32'},"
                 f"V={dom['variant']},W={dom['lanes']}>")
        roof = {"bound": "int", "achieved": ach / 1e9, "peak": peak / 1e9, "unit": "GCUPS",
                "frac": ach / peak, "traffic": NCU_TRAFFIC.get(kname),
                "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                "kernel": kname,
                "launch_ms": dom["ms"], "launch_cells": dom["cells"],
                "peak_source": "ALU-pipe ceiling measured in this run: nwg_dpx_peak_form(int32, form 2) "
                               "saturates the ALU pipe (ncu 99.98 %), x 4 ALU lane-ops per cell = the pipe's "
                               "lane-op rate, / 1.5 ALU lane-ops per int16x2 cell of the leanest update",
                "peak_int32_gcups": peak32 / 1e9,
                "alu_lane_ops_per_s": alu_lane_ops,
                "cell_update_microbenchmark_gcups": micro16 / 1e9}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot_s_max / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16x2+int32", "data": "synthetic",
        "config": {"workload": f"configuration {CONFIG}: {n} seqs, 50 families x 200, lognormal lengths "
                               "(median 350, sigma 0.6, clipped 30-4000), all pairs incl. diagonal",
                   "pairs": n * (n + 1) // 2, "cells_per_step": cells, "l2": "flushed (256 MB write) between steps",
                   "parallelism": f"{world} replica(s)"},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "launches_per_step": per_step_launches,
        "launch_records": [{k: r[k] for k in ("rows_per_lane", "variant", "lanes", "lanes16", "grid", "cells", "ms")}
                           for r in recs],
        "tuning": tuning,
        "sequential_launch_sum_ms": timed_sum_ms,
        "reruns": st["reruns"],
        "plain": plain,
        "batched_over_plain": (value / world) / plain["gcups"] if plain else None,
        "parity_sample_ok": parity,
        "pairs_int16": st["pairs_int16"], "pairs_int32": st["pairs_int32"],
        "wall_s": wall,
        "clocks": clk,
        "config1": config1,
        "serving": serving,
        "pipeline": pipeline,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
