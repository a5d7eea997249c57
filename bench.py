#!/usr/bin/env python
"""Benchmark of the read-to-contig Smith-Waterman hot path on GB300.

One step = one pass of the path (forward + begin pass, all pairs) over the batch of
synthetic pairs of the uneven-length workload (4,000,000 pairs: 60% 150 bp, 30% 250 bp,
10% 50-150 bp reads against lognormal(ln 400, 0.6) references in [64, 2048]; seed 2).

  value  GCUPS of the batched form with the pairs already resident in HBM
         (forward cells = sum len(read) * len(ref); begin-pass cells are overhead).
  e2e    the same through the C ABI with pinned HOST buffers: copies in, both passes,
         results out, every step.
  plain  the plain drop-in kernel on the same pairs, for the batched-vs-plain ratio.

Prints one JSON line on rank 0.  `--impl reference` times the reference's own CPU
implementation of the path instead -- its SSW (src/ssw), compiled on this host (through an
SSE2-to-NEON shim on aarch64) and called as klign calls it, one Aligner per host thread, on
bounded samples of the workload -- with the oracle port beside it, and the reference's
own CUDA kernels (ADEPT) on the same GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SCORING = (1, 3, 5, 2, 2)  # match, mismatch, gap open, gap extend, ambiguity (magnitudes)
# packed int16x2 ops per two cell updates in the minimal recurrence: H - gO; the E and F
# add-max updates; diagonal + profile; the 3-way max with relu; the max tracking
K_OPS_PER_CELL_PAIR = 6
WORKLOAD_NAME = "uneven read/ref lengths, 4M pairs (60% 150bp, 30% 250bp, 10% U[50,150]bp; ref lognormal(ln400,0.6) in [64,2048])"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


CPU_PORT = ("the oracle's result contract vectorised across pairs (oracle/sw_lanes.cpp: 8 pairs per 128-bit "
            "vector, 4 vectors interleaved on aarch64, portable GCC vectors; bit-exact with the scalar restatement)")


def _ref_implementation() -> str:
    from oracle import oracle

    how = ("with SSE2" if oracle.reference_build_kind() == "sse2" else
           "through the SSE2-to-NEON shim oracle/sse2_shim (bit-exact with the x86_64 SSE2 build on the 150/300 bp "
           "workload, tests/test_oracle.py)")
    return ("the reference's own SSW (src/ssw/ssw.cpp + ssw_core.cpp, unmodified) compiled on this host " + how +
            ", called as klign calls it (Aligner(1,3,5,2,2).Align(contig, read, len, Filter(true,false,0,32767), "
            "&aln, max(len/2,15)), src/klign.cpp:257), one Aligner per thread, pairs handed out 64 at a time")


def _cpu_engine():
    """(kind, run(pairs, threads), description) of the CPU baseline: the reference SSW where
    it is built on this host, else the oracle port."""
    from oracle import oracle

    if oracle.reference_available():
        return "reference", (lambda p, t: oracle.ref_align_batch(p, SCORING, t)), _ref_implementation()
    return "port", (lambda p, t: oracle.align_batch_lanes(p, SCORING, t)), CPU_PORT


def _timed_sample(run, pairs, threads: int, budget_s: float):
    """Times run() on the leading sample of pairs that takes about budget_s."""
    n_probe = min(pairs.n, 20000)
    t0 = time.perf_counter()
    run(pairs.slice(0, n_probe), threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    n = int(min(pairs.n, max(n_probe, n_probe * budget_s / dt)))
    sample = pairs.slice(0, n)
    t0 = time.perf_counter()
    run(sample, threads)
    return n, sample.cells(), time.perf_counter() - t0


def cpu_baseline(pairs, budget_s: float = 12.0) -> dict:
    """The reference SSW (or, where it is not built, the oracle port) timed on all host
    cores on a bounded leading sample of the batch; the port beside it."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    kind, run, impl = _cpu_engine()
    n, cells, dt = _timed_sample(run, pairs, threads, budget_s)
    out = {"value": cells / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": kind,
           "sample": f"first {n} pairs of the same workload ({cells:.3g} forward cells, {dt:.1f} s)",
           "implementation": impl, "alignments_per_s": n / dt}
    if kind == "reference":
        pn, pcells, pdt = _timed_sample(lambda p, t: oracle.align_batch_lanes(p, SCORING, t), pairs, threads,
                                        budget_s / 2)
        out["port"] = {"value": pcells / pdt / 1e9, "unit": "GCUPS", "cores": threads,
                       "sample": f"first {pn} pairs ({pdt:.1f} s)", "implementation": CPU_PORT}
    return out


def _adept_gpu(args) -> dict | None:
    """ADEPT, the reference's own CUDA kernels for this path (compiled for sm_103a from the
    reference sources into oracle/_ref), on the main arm's workload with inputs resident:
    the same-GPU comparator.  None when the cubin or a GPU is missing."""
    import torch
    from oracle import adept

    if not (adept.available() and torch.cuda.is_available()):
        return None
    from mhm2_staging_gb300 import workloads
    from oracle import oracle

    n = args.pairs or workloads.CONFIG_PAIRS[args.config]
    pairs = workloads.generate(args.config, n=n, gen_lib=oracle.GEN_SO)
    ad = adept.Adept(0)
    batch = ad.upload(pairs)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    fwd, rev, tot = [], [], []
    for s in range(args.warmup + args.steps):
        ad.run(batch, SCORING, 0, ev)
        if s >= args.warmup:
            fwd.append(ev[0].elapsed_time(ev[1]))
            rev.append(ev[2].elapsed_time(ev[3]))
            tot.append(ev[0].elapsed_time(ev[3]))
    k = min(n, 20000)
    want = oracle.align_batch(pairs.slice(0, k), SCORING, None)[:, 0]
    agree = float((ad.scores(batch)[:k] == want).mean())
    ms = statistics.mean(tot)
    return {"value": pairs.cells() / (ms * 1e-3) / 1e9, "unit": "GCUPS", "ms_per_step": ms,
            "fwd_ms": statistics.mean(fwd), "rev_ms": statistics.mean(rev), "pairs": n,
            "kernels": "ADEPT sequence_dna_kernel + sequence_dna_reverse (src/adept-sw/kernel.cpp) compiled "
                       "for sm_103a, launched with the reference driver's shapes, inputs resident",
            "score_agreement_with_oracle": agree, "agreement_sample": k}


def run_reference(args) -> None:
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from mhm2_staging_gb300 import workloads
    from oracle import oracle

    oracle.build()  # liboracle.so, the generator; libssw_ref.so where its sources are here
    threads = os.cpu_count() or 1
    per_step = args.ref_pairs
    # inputs from the oracle's own build of the seeded generator (nothing of the product loaded)
    pairs = workloads.generate(args.config, n=per_step * (args.steps + args.warmup), seed=args.config,
                               gen_lib=oracle.GEN_SO)
    kind, run, impl = _cpu_engine()

    def timed(fn) -> tuple[list, list]:
        times, cells = [], []
        for s in range(args.warmup + args.steps):
            sub = pairs.slice(s * per_step, (s + 1) * per_step)
            t0 = time.perf_counter()
            fn(sub, threads)
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                times.append(dt)
                cells.append(sub.cells())
        return times, cells

    times, cells = timed(run)
    tot = sum(times)
    gcups = sum(cells) / tot / 1e9
    sample = f"{per_step} pairs per step of the same workload, steps {args.warmup}.. of the seeded stream"
    line = {
        "impl": "reference", "metric": "GCUPS", "value": gcups, "unit": "GCUPS", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16 (SSW's u8 then i16 saturating passes)"
        if kind == "reference" else "int32", "data": "synthetic (seeded generator)",
        "config": {"workload": WORKLOAD_NAME, "pairs_per_step": per_step, "scoring": list(SCORING),
                   "cache": "inputs larger than L2 (CPU run)"},
        "alignments_per_s": per_step * args.steps / tot,
        "cpu_baseline": {"value": gcups, "unit": "GCUPS", "cores": threads, "kind": kind, "sample": sample,
                         "implementation": impl},
        "e2e": {"value": gcups, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if kind == "reference":
        pt, pc = timed(lambda p, t: oracle.align_batch_lanes(p, SCORING, t))
        line["port"] = {"value": sum(pc) / sum(pt) / 1e9, "unit": "GCUPS", "cores": threads, "sample": sample,
                        "implementation": CPU_PORT}
    ad = _adept_gpu(args)
    if ad is not None:
        line["adept_gpu"] = ad
    print(json.dumps(line), flush=True)


SERVING_WORKLOAD = ("serving: 200 MB resident contigs (lognormal(ln 2000, 1.0) in [200, 200000]), request batches "
                    "log-uniform in [1k, 64k], reads U[100,250] bp, window read +-200 bp")


def serving_measure(batches_per_level: int, slots: int, pool_n: int) -> dict:
    """Serving workload: 200 MB of resident contigs; request batches (sizes log-uniform in
    [1k, 64k] requests, reads U[100,250] bp from the contigs, 2% divergence) aligned against
    their seed-hit windows (read +-200 bp).  First the saturated throughput (every batch
    submitted at once), then open-loop Poisson arrivals at 25/50/90% of it, with the
    latency percentiles of the batches (submission to completion)."""
    from mhm2_staging_gb300 import serving as S

    rng = np.random.default_rng(3)
    contigs = S.generate_contigs(200 << 20, seed=3)
    pool = S.generate_requests(contigs, pool_n, seed=3)

    def batches(count: int):
        out, at = [], 0
        for _ in range(count):
            k = int(np.exp(rng.uniform(np.log(1024), np.log(65536))))
            if at + k > pool.n:
                at = 0
            out.append(pool.slice(at, at + k))
            at += k
        return out

    srv = S.Server(slots=slots, max_pairs_per_batch=65536)
    srv.load_contigs(contigs)
    clk = ClockSampler(0)
    # warm-up (slot set-up and tuning on real batches)
    for t in [srv.submit(b) for b in batches(3 * slots)]:
        srv.wait(t)
    # saturated throughput
    sat = batches(batches_per_level)
    clk.start()
    t0 = time.perf_counter()
    ts = [srv.submit(b) for b in sat]
    for t in ts:
        srv.wait(t)
    wall = time.perf_counter() - t0
    sat_pairs = sum(b.n for b in sat)
    sat_cells = float(sum(S.windows(contigs, b)[0].cells() for b in sat))
    peak = sat_pairs / wall
    mean_batch = sat_pairs / len(sat)
    loads = []
    for frac in (0.25, 0.5, 0.9):
        bl = batches(batches_per_level)
        r = S.run_open_loop(srv, bl, rate_hz=frac * peak / mean_batch, seed=int(frac * 100))
        r["load"] = frac
        r["offered_pairs_per_s"] = frac * peak
        loads.append(r)
    clocks = clk.stop()
    st = srv.stats()
    srv.close()
    return {"workload": SERVING_WORKLOAD, "slots": slots, "max_pairs_per_batch": 65536,
            "batches_per_level": batches_per_level,
            "saturated": {"pairs_per_s": peak, "gcups": sat_cells / wall / 1e9, "batches": len(sat), "wall_s": wall},
            "loads": loads, "server": st, "clocks": clocks}


def run_serving(args) -> None:
    """The serving workload alone (serving_measure), as its own JSON line: the headline is
    the p99 batch latency at 90% of the saturated load."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from mhm2_staging_gb300 import build as mbuild

    mbuild.build()
    m = serving_measure(args.serving_batches, args.slots, args.serving_pool)
    line = {
        "metric": "p99 batch latency at 90% of saturated load", "value": m["loads"][-1]["p99_ms"], "unit": "ms",
        "n_gpus": 1, "steps": args.serving_batches, "warmup": 3 * args.slots, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16x2 (int32 re-run on overflow)",
        "data": "synthetic (seeded contigs and seed-hit requests)",
        "config": {"workload": SERVING_WORKLOAD, "slots": args.slots, "max_pairs_per_batch": 65536,
                   "scoring": list(SCORING), "form": "batched persistent per micro-batch"},
        "saturated": m["saturated"], "loads": m["loads"], "server": m["server"], "clocks": m["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_paths(drv, dev, torch, stream) -> dict:
    """GCUPS of the other measured workloads on the same driver, inputs resident on the
    device (each: 2 warm-up calls, then 3 timed with CUDA events on the driver's stream):
    the 150/300 bp batch (plain and batched form), the 1M-pair read/ref mix with 30%
    unrelated reads, the 200k long-reference batch, and the 200k-pair slice of the uneven
    batch with every pair re-run by the int32 engine (int16 ceiling 0), and the same slice in
    score2 mode (SSW's second-best score as well) and in CIGAR mode (SSW's report_cigar
    output as well; beside it the oracle's CIGAR port timed on the host cores on a sample)."""
    from mhm2_staging_gb300 import FORM_BATCHED, FORM_PLAIN, workloads
    from mhm2_staging_gb300.driver import DevicePairs, limits

    out = {}
    specs = [("150bp_vs_300bp_10k_pairs_plain", 0, 10_000, FORM_PLAIN, None),
             ("150bp_vs_300bp_10k_pairs_batched", 0, 10_000, FORM_BATCHED, None),
             ("reads_100_250bp_1M_pairs_30pct_unrelated", 1, 1_000_000, FORM_BATCHED, None),
             ("reads_100_250bp_1M_pairs_30pct_unrelated_plain", 1, 1_000_000, FORM_PLAIN, None),
             ("250bp_vs_2_8kb_refs_200k_pairs", 4, 200_000, FORM_BATCHED, None),
             ("uneven_200k_pairs_all_int32", 2, 200_000, FORM_BATCHED, 0),
             ("uneven_200k_pairs_score2_mode", 2, 200_000, FORM_BATCHED, "score2"),
             ("uneven_200k_pairs_cigar_mode", 2, 200_000, FORM_BATCHED, "cigar")]
    default_ceiling = limits().int16_ceiling
    for name, cfg, n, form, ceiling in specs:
        pp = workloads.generate(cfg, n=n)
        tens = [torch.from_numpy(x).to(dev) for x in (pp.a_seq, pp.a_off, pp.a_len, pp.b_seq, pp.b_off, pp.b_len)]
        o = torch.empty((pp.n, 5), dtype=torch.int32, device=dev)
        cells = float(pp.cells())
        dp = DevicePairs(*(t.data_ptr() for t in tens), n=pp.n, max_a_len=int(pp.a_len.max()),
                         max_b_len=int(pp.b_len.max()), cells=cells, a_bytes=int((pp.a_off + pp.a_len).max()),
                         b_bytes=int((pp.b_off + pp.b_len).max()))
        score2 = ceiling == "score2"
        cigar = ceiling == "cigar"
        drv.set_score2(score2)
        drv.set_cigar(cigar)
        drv.set_int16_ceiling(default_ceiling if ceiling is None or score2 or cigar else ceiling)
        for _ in range(2):
            drv.align_pairs_device(dp, o.data_ptr(), form=form)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fwd = []
        for _ in range(3):
            drv.align_pairs_device(dp, o.data_ptr(), form=form)
            fwd.append(drv.last_timing()["fwd_ms"])
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / 3
        t = drv.last_timing()
        out[name] = {"gcups": cells / (ms * 1e-3) / 1e9, "ms_per_step": ms, "pairs": pp.n, "cells": cells,
                     "fwd_gcups": cells / (statistics.mean(fwd) * 1e-3) / 1e9,
                     "int32_reruns": int(t["n_overflow16"]), "form": "plain" if form == FORM_PLAIN else "batched"}
        if cigar:
            cg = drv.last_cigar(pp.n)
            out[name].update({"alignments_per_s": pp.n / (ms * 1e-3), "cigar_ms": t["cigar_ms"],
                              "cigar_generic_pairs": int(t["n_cigar_generic"]),
                              "cigar_ops": int(cg.op_off[-1]), "cigar_pairs": int((cg.nops > 0).sum())})
            out[name]["cpu_port"] = _cigar_cpu_port(pp)
        del tens, o
        torch.cuda.empty_cache()
    drv.set_int16_ceiling(default_ceiling)
    drv.set_score2(False)
    drv.set_cigar(False)
    out["klign_caller_200k_candidates"] = _klign_caller_path(drv)
    out["protein_100k_pairs_100_500aa"] = _protein_path()
    out["uneven_1M_pairs_in_20k_pair_calls_host"] = _block_calls_path(drv)
    out["uneven_1M_pairs_cpp_dropin_20k_blocks"] = _cpp_dropin_path()
    return out


def _cpp_dropin_path(n: int = 1_000_000, per_block: int = 20_000, passes: int = 3) -> dict:
    """klign's GPU call sequence through the C++ drop-in header (klign_block_bench): the
    uneven workload's first 1M pairs as 20,000-pair std::vector<std::string> blocks,
    run_kernel_forwards -> kernel_block -> run_kernel_backwards -> kernel_block ->
    get_aln_results per block (src/klign.cpp:356-388), in its own process on its own
    handle; the plain drop-in form (as klign calls it) and the batched form."""
    import tempfile

    from mhm2_staging_gb300 import build as mbuild
    from mhm2_staging_gb300 import workloads

    pp = workloads.generate(2, n=n)
    out = {"interface": "include/adept-sw/driver.hpp (C++ header over the C ABI), klign's call sequence"}
    with tempfile.TemporaryDirectory() as td:
        f = Path(td) / "pairs.bin"
        pp.write_file(f)
        for form in ("plain", "batched"):
            r = subprocess.run([str(mbuild.block_bench_path()), str(f), str(per_block), str(passes), form],
                               capture_output=True, text=True, timeout=600)
            out[form] = (json.loads(r.stdout.strip().splitlines()[-1]) if r.returncode == 0 else
                         {"error": (r.stdout + r.stderr)[-400:]})
    return out


def _block_calls_path(drv, n: int = 1_000_000, per_call: int = 20_000) -> dict:
    """klign's call size (KLIGN_GPU_BLOCK_SIZE, 20,000 pairs): the uneven workload's first
    1M pairs in 20,000-pair synchronous calls through the C ABI from host (pageable) arrays,
    as klign's strings are; copies in, both passes and results out inside each call.  Plain
    and batched form."""
    from mhm2_staging_gb300 import FORM_BATCHED, FORM_PLAIN, workloads

    pp = workloads.generate(2, n=n)
    blocks = [pp.slice(i, i + per_call) for i in range(0, pp.n, per_call)]
    res = {"pairs": pp.n, "pairs_per_call": per_call, "calls": len(blocks), "cells": float(pp.cells())}
    for name, form in (("plain", FORM_PLAIN), ("batched", FORM_BATCHED)):
        for b in blocks[:2]:
            drv.align_pairs(b, form=form, hints=True)
        t0 = time.perf_counter()
        for b in blocks:
            drv.align_pairs(b, form=form, hints=True)
        dt = time.perf_counter() - t0
        res[name] = {"alignments_per_s": pp.n / dt, "gcups": pp.cells() / dt / 1e9, "ms_per_call": 1e3 * dt / len(blocks)}
    return res


def _protein_pairs(n: int, seed: int = 8):
    """Seeded protein pairs: A of U[100, 500] residues; B = A with 10% substitutions and 2%
    deletions between random flanks (one pair in three unrelated)."""
    from mhm2_staging_gb300 import Pairs
    from mhm2_staging_gb300.protein import PROTEIN_LETTERS

    letters = np.frombuffer(PROTEIN_LETTERS.encode(), dtype=np.uint8)
    rng = np.random.default_rng(seed)
    a, b = [], []
    for k in range(n):
        x = letters[rng.integers(0, 20, int(rng.integers(100, 501)))]
        if k % 3 == 0:
            y = letters[rng.integers(0, 20, int(rng.integers(100, 501)))]
        else:
            y = x.copy()
            sub = rng.random(y.shape[0]) < 0.1
            y[sub] = letters[rng.integers(0, 24, int(sub.sum()))]
            y = y[rng.random(y.shape[0]) > 0.02]
            y = np.concatenate([letters[rng.integers(0, 20, int(rng.integers(0, 40)))], y,
                                letters[rng.integers(0, 20, int(rng.integers(0, 40)))]])
        a.append(x.tobytes())
        b.append(y.tobytes())
    return Pairs.from_lists(a, b)


def _protein_path(n: int = 100_000) -> dict:
    """Protein alignment (mhsw_align_protein, host arrays in and out) with a seeded 24 x 24
    matrix (diagonal 4..11, elsewhere -4..3), gaps 11/1; 1 warm-up call, 3 timed (wall
    clock, synchronous call).  GCUPS count the forward cells.  Beside it the oracle port
    on the first 20,000 pairs."""
    from mhm2_staging_gb300 import GPUDriver
    from mhm2_staging_gb300.protein import protein_encoding

    pairs = _protein_pairs(n)
    rng = np.random.default_rng(2024)
    m = rng.integers(-4, 4, (24, 24))
    m = (np.triu(m) + np.triu(m, 1).T).astype(np.int16)
    np.fill_diagonal(m, rng.integers(4, 12, 24))
    enc = protein_encoding()
    d = GPUDriver()
    d.init(0, 1, 1, -1, -11, -1, 0)
    d.align_protein(pairs, m, enc)
    t0 = time.perf_counter()
    for _ in range(3):
        d.align_protein(pairs, m, enc)
    dt = (time.perf_counter() - t0) / 3
    cells = float(pairs.cells())
    from oracle import oracle  # the CPU baseline beside the path line

    sub = pairs.slice(0, 20_000)
    t0 = time.perf_counter()
    oracle.protein_batch(sub, m, enc, 11, 1, os.cpu_count() or 1)
    cdt = time.perf_counter() - t0
    return {"gcups": cells / dt / 1e9, "ms_per_call": dt * 1e3, "pairs": n, "cells": cells,
            "cpu_port": {"gcups": float(sub.cells()) / cdt / 1e9, "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"first {sub.n} pairs ({cdt:.1f} s)"}}


def _klign_caller_path(drv, n: int = 200_000) -> dict:
    """klign's caller side on the device (mhsw_klign_align): seed-hit candidates from host
    arrays to klign's Aln fields in host arrays, against 64 MB of resident contigs; 1 warm-up
    call, then 3 timed (wall clock: the call is synchronous).  Beside it the CPU
    restatement (oracle/klign_caller.py with the C SW oracle) on the first 20,000."""
    from mhm2_staging_gb300 import serving as S
    from mhm2_staging_gb300.klign import ResidentContigs, generate_candidates, klign_align
    from oracle import klign_caller

    ct = S.generate_contigs(64 << 20, seed=3)
    cand = generate_candidates(ct, n, seed=21)
    rc = ResidentContigs(ct)
    r = klign_align(drv, rc, cand)
    t0 = time.perf_counter()
    for _ in range(3):
        r = klign_align(drv, rc, cand)
    dt = (time.perf_counter() - t0) / 3
    # klign's SAM run: CIGAR mode at its post-assembly scoring (src/klign.cpp:1061-1064),
    # the SAM CIGAR strings and mismatches built on the host from the returned ops
    from mhm2_staging_gb300 import FORM_BATCHED, GPUDriver

    dc = GPUDriver()
    dc.init(0, 1, 2, -4, -4, -2, 0)
    dc.set_ambiguity(-1)
    dc.set_form(FORM_BATCHED)
    dc.set_cigar(True)
    rcg = klign_align(dc, rc, cand, cigar_ops=True)
    t0 = time.perf_counter()
    for _ in range(3):
        rcg = klign_align(dc, rc, cand, cigar_ops=True)
    dtc = (time.perf_counter() - t0) / 3
    rc.close()
    sub = cand.slice(0, 20_000)
    t0 = time.perf_counter()
    klign_caller.klign_align(ct.seq, ct.off, ct.len, sub.read_seq, sub.read_off, sub.read_len, sub.cid,
                             sub.pos_in_ctg, sub.pos_in_read, sub.strand, sub.kmer_len, SCORING, False,
                             os.cpu_count() or 1)
    cdt = time.perf_counter() - t0
    return {"candidates_per_s": n / dt, "ms_per_call": dt * 1e3, "candidates": n, "aligned": r["n_aligned"],
            "perfect_fraction": float(r["perfect"].mean()),
            "cigar_mode": {"candidates_per_s": n / dtc, "ms_per_call": dtc * 1e3, "scoring": [2, 4, 4, 2, 1],
                           "aligned": rcg["n_aligned"],
                           "cigar_ops": int(rcg["cigar_batch"].op_off[-1]),
                           "note": "each aligned candidate's BAM-encoded CIGAR ops and mismatches in host "
                                   "arrays (perfect matches: <overlap>=)"},
            "cpu_port": {"candidates_per_s": sub.n / cdt, "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"first {sub.n} candidates ({cdt:.1f} s)"}}


def _cigar_cpu_port(pairs, n: int = 20_000) -> dict:
    """The oracle's CIGAR port (score, begins and SSW's report_cigar output) on the host
    cores, on the first n pairs of the same slice."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    sub = pairs.slice(0, min(n, pairs.n))
    t0 = time.perf_counter()
    oracle.cigar_batch(sub, SCORING, threads, ops_cap=1024)
    dt = time.perf_counter() - t0
    return {"alignments_per_s": sub.n / dt, "cores": threads, "kind": "port",
            "sample": f"first {sub.n} pairs of the slice ({dt:.1f} s)"}


def _call_breakdown(recs: list[dict]) -> dict:
    """Per-call device phases of pipelined host-batch calls (mhsw_call_history), ms: each
    call's copies in, the GPU's idle time before its kernels (after the previous call's
    kernels ended), its kernels, and its result copy out.  A call's kernels start when both
    its copies in have ended and the stream is free."""
    out = {"copy_in_ms": [], "kernels_ms": [], "idle_before_kernels_ms": [], "copy_out_ms": [],
           "kernels_waited_for_copies": 0}
    prev_end = None
    for r in recs:
        start = max(r["stream_ready"], r["copy_in_end"]) if r["copy_in_end"] >= 0 else r["stream_ready"]
        out["copy_in_ms"].append(round(r["copy_in_end"] - r["copy_in_start"], 3) if r["copy_in_end"] >= 0 else None)
        out["kernels_ms"].append(round(r["begin_done"] - start, 3))
        out["copy_out_ms"].append(round(r["done"] - r["begin_done"], 3))
        if prev_end is not None:
            out["idle_before_kernels_ms"].append(round(max(0.0, start - prev_end), 3))
            if r["copy_in_end"] > r["stream_ready"]:
                out["kernels_waited_for_copies"] += 1
        prev_end = r["done"]
    if recs:
        out["span_ms"] = round(recs[-1]["done"] - (recs[0]["copy_in_start"] if recs[0]["copy_in_start"] >= 0
                                                    else recs[0]["stream_ready"]), 3)
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--pairs", type=int, default=None, help="override pairs per GPU (smaller runs)")
    ap.add_argument("--ref-pairs", type=int, default=200000, help="pairs per step of the reference arm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-paths", action="store_true", help="skip the per-workload path measurements")
    ap.add_argument("--cigar", action="store_true",
                    help="CIGAR mode in the timed regions (SSW's report_cigar output as well; e2e copies it back)")
    ap.add_argument("--workload", choices=["batch", "serving", "protein", "klign"], default="batch",
                    help="batch: the uneven-length batch (default); serving: latency under offered load; "
                         "protein: the protein path alone (--pairs pairs, default 100000)")
    ap.add_argument("--slots", type=int, default=3, help="serving: micro-batches in flight")
    ap.add_argument("--serving-batches", type=int, default=400, help="serving: request batches per load level")
    ap.add_argument("--serving-pool", type=int, default=2_000_000, help="serving: distinct requests generated")
    ap.add_argument("--serving-batches-default", type=int, default=200,
                    help="serving leg of the default run: request batches per load level")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving leg of the default run")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "protein":
        print(json.dumps({"workload": "protein", **_protein_path(args.pairs or 100_000)}), flush=True)
        return None
    if args.workload == "klign":
        from mhm2_staging_gb300 import GPUDriver

        kd = GPUDriver()
        kd.init(0, 1, SCORING[0], -SCORING[1], -SCORING[2], -SCORING[3], 0)
        kd.set_ambiguity(-SCORING[4])
        print(json.dumps({"workload": "klign caller side, 200k candidates vs 64 MB contigs",
                          **_klign_caller_path(kd, args.pairs or 200_000)}), flush=True)
        return None

    ws, rank, local = _dist()
    import torch

    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from mhm2_staging_gb300 import FORM_BATCHED, FORM_PLAIN, GPUDriver, workloads
    from mhm2_staging_gb300 import build as mbuild
    from mhm2_staging_gb300.driver import DevicePairs, probe_dpx_rate

    mbuild.build()
    dev = torch.device("cuda", local)
    n_per = args.pairs or workloads.CONFIG_PAIRS[args.config]
    # weak scaling: each rank aligns its own n_per pairs (a disjoint slice of the seeded stream)
    pairs = workloads.generate(args.config, n=n_per, first=rank * n_per)
    cells_local = float(pairs.cells())

    drv = GPUDriver()
    drv.init(local, ws, SCORING[0], -SCORING[1], -SCORING[2], -SCORING[3], 0)
    drv.set_ambiguity(-SCORING[4])
    drv.set_cigar(args.cigar)
    stream = torch.cuda.ExternalStream(drv.stream(), device=dev)

    # resident inputs
    tens = [torch.from_numpy(x).to(dev) for x in (pairs.a_seq, pairs.a_off, pairs.a_len, pairs.b_seq, pairs.b_off,
                                                 pairs.b_len)]
    out_dev = torch.empty((pairs.n, 5), dtype=torch.int32, device=dev)
    torch.cuda.synchronize(dev)
    dp = DevicePairs(*(t.data_ptr() for t in tens), n=pairs.n, max_a_len=int(pairs.a_len.max()),
                     max_b_len=int(pairs.b_len.max()), cells=cells_local,
                     a_bytes=int((pairs.a_off + pairs.a_len).max()), b_bytes=int((pairs.b_off + pairs.b_len).max()))

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    def allmax(x: float) -> float:
        if ws == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    def allsum(x: float) -> float:
        if ws == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
        return float(t.item())

    # ---- warm-up (the first call tunes the batched form on a sample of the batch) -----
    tuning = None
    for i in range(max(args.warmup, 3)):
        w0 = time.perf_counter()
        drv.align_pairs_device(dp, out_dev.data_ptr(), form=FORM_BATCHED)
        torch.cuda.synchronize(dev)
        if i == 0:
            tuning = drv.last_tuning()
            tuning["first_call_wall_ms"] = (time.perf_counter() - w0) * 1e3
    tuning["rows_per_lane"] = ("8-lane groups: 2K rows per lane with K = 4/6/8/10 for A up to 64/96/128/160 rows; "
                               "16-lane groups: K = 6/8 for A up to 192/256 rows, 256-row strips beyond; A above "
                               "lane_rows goes to 16-lane groups")

    # ---- timed region: device-resident batched form ----------------------------------
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    fwd_ms, rev_ms, launches = [], [], 0
    e0.record(stream)
    for _ in range(args.steps):
        drv.align_pairs_device(dp, out_dev.data_ptr(), form=FORM_BATCHED)
        t = drv.last_timing()
        fwd_ms.append(t["fwd_ms"])
        rev_ms.append(t["rev_ms"])
        launches += int(t["launches"])
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    clk = clocks.stop()
    ms_local = e0.elapsed_time(e1) / args.steps
    ms = allmax(ms_local)
    cells_all = allsum(cells_local)
    pairs_all = allsum(float(pairs.n))
    gcups = cells_all / (ms * 1e-3) / 1e9
    last = drv.last_timing()

    # ---- plain drop-in kernel on the same resident pairs ------------------------------
    plain = None
    if not args.no_plain:
        drv.align_pairs_device(dp, out_dev.data_ptr(), form=FORM_PLAIN)
        torch.cuda.synchronize(dev)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        psteps = max(1, min(args.steps, 3))
        pf = []
        for _ in range(psteps):
            drv.align_pairs_device(dp, out_dev.data_ptr(), form=FORM_PLAIN)
            pf.append(drv.last_timing()["fwd_ms"])
        p1.record(stream)
        torch.cuda.synchronize(dev)
        pms = allmax(p0.elapsed_time(p1) / psteps)
        plain = {"gcups": cells_all / (pms * 1e-3) / 1e9, "ms_per_step": pms,
                 "fwd_kernel_gcups": cells_local / (statistics.mean(pf) * 1e-3) / 1e9}

    # ---- e2e: pinned host buffers through the C ABI ------------------------------------
    from mhm2_staging_gb300.driver import Pairs

    keep_pinned = []  # the pinned tensors behind the host arrays (freed when main returns)

    def pinned(x: np.ndarray) -> np.ndarray:
        t = torch.empty(x.shape, dtype={np.uint8: torch.uint8, np.int64: torch.int64,
                                        np.int32: torch.int32}[x.dtype.type], pin_memory=True)
        a = t.numpy()
        a[...] = x
        keep_pinned.append(t)
        return a

    hp = Pairs(*(pinned(x) for x in (pairs.a_seq, pairs.a_off, pairs.a_len, pairs.b_seq, pairs.b_off, pairs.b_len)))
    hout = pinned(np.zeros((pairs.n, 5), dtype=np.int32))
    h2d = int(hp.a_seq.nbytes + hp.b_seq.nbytes + hp.a_off.nbytes + hp.b_off.nbytes + hp.a_len.nbytes +
              hp.b_len.nbytes)
    d2h = int(hout.nbytes)
    hp.extents()  # the batch's extents, known to the caller (as klign knows its longest read/contig)
    # Steps go through the async halves of the batch call (mhsw_align_pairs_async, then
    # mhsw_align_wait once at the end): the handle keeps four calls in flight on four
    # input sets, so later steps' copies in run while step k's kernels do.  Every step still
    # copies its inputs from pinned host memory and its results back inside the timed
    # region.  The one-call-at-a-time figure is reported beside it as e2e_sequential.
    houts = [hout] + [pinned(np.zeros((pairs.n, 5), dtype=np.int32)) for _ in range(3)]
    for o in houts:  # warm: sizes the input sets, whose calls take turns
        drv.align_pairs_async(hp, form=FORM_BATCHED, out=o, hints=True)
    drv.wait()
    # this host's copy rate: one plain pinned host -> device copy of the step's read bytes,
    # on torch's own stream with its own buffers, all freed here (it varies between hosts;
    # the pipelined e2e hides it while it stays below the kernels' time)
    hbuf = torch.empty(hp.a_seq.shape[0], dtype=torch.uint8, pin_memory=True)
    hbuf.numpy()[...] = hp.a_seq
    dbuf = torch.empty_like(hbuf, device=dev)
    dbuf.copy_(hbuf, non_blocking=True)
    torch.cuda.synchronize(dev)
    c0 = torch.cuda.Event(enable_timing=True)
    c1 = torch.cuda.Event(enable_timing=True)
    c0.record()
    dbuf.copy_(hbuf, non_blocking=True)
    c1.record()
    torch.cuda.synchronize(dev)
    h2d_gbs = hbuf.numel() / (c0.elapsed_time(c1) * 1e-3) / 1e9
    del dbuf, hbuf
    barrier()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    cg = None
    for k in range(args.e2e_steps):
        drv.align_pairs_async(hp, form=FORM_BATCHED, out=houts[k % 4], hints=True)
        if args.cigar:
            cg = drv.last_cigar(pairs.n)  # CIGAR mode completes each call before the next
    drv.wait()
    e2e_s = allmax((time.perf_counter() - t0) / args.e2e_steps)
    e2e_calls = _call_breakdown(drv.call_history(args.e2e_steps))
    if args.cigar:
        d2h += int(cg.nops.nbytes + cg.mismatches.nbytes + cg.op_off.nbytes + cg.ops.nbytes)
    e2e_gcups = cells_all / e2e_s / 1e9
    # the e2e results must equal the resident-input results
    ref_out = out_dev.cpu().numpy()
    assert all(np.array_equal(o, ref_out) for o in houts), "e2e results differ from device-resident results"
    barrier()
    seq_wall, seq_dev = [], []  # per call: wall time and device span (copies in, kernels, copy out)
    t0 = time.perf_counter()
    for _ in range(2):
        t1 = time.perf_counter()
        drv.align_pairs(hp, form=FORM_BATCHED, out=hout, hints=True)
        if args.cigar:
            drv.last_cigar(pairs.n)
        seq_wall.append((time.perf_counter() - t1) * 1e3)
        seq_dev.append(drv.last_timing()["total_ms"])
    e2e_seq_s = allmax((time.perf_counter() - t0) / 2)
    seq_t = drv.last_timing()

    # ---- other paths of the scope: per-workload GCUPS, device-resident ----------------
    paths = None
    if rank == 0 and not args.no_paths:
        drv.set_cigar(False)
        paths = run_paths(drv, dev, torch, stream)

    # ---- roofline of the dominant kernel (the persistent forward kernel) -------------
    dpx_ops, sm_hz = probe_dpx_rate(local)
    hbm_peak, hbm_basis = 6800.0, "fallback 6.8 TB/s"
    mp = ROOT / "MEASURED_PEAKS.json"
    if mp.exists():
        try:
            hbm_peak, hbm_basis = float(json.loads(mp.read_text())["hbm_gbs"]), "measured copy bandwidth"
        except (KeyError, ValueError):
            pass
    peak_gcups = dpx_ops * 2 / K_OPS_PER_CELL_PAIR / 1e9
    fwd_avg = statistics.mean(fwd_ms)
    achieved = cells_local / (fwd_avg * 1e-3) / 1e9
    alg_bytes = float(pairs.a_seq.nbytes + pairs.b_seq.nbytes + pairs.a_off.nbytes + pairs.b_off.nbytes +
                      pairs.a_len.nbytes + pairs.b_len.nbytes + 4 * 4 * pairs.n)
    traffic = None
    prof = ROOT / "profiles" / "fwd_persist_traffic.json"
    if prof.exists():
        try:
            pj = json.loads(prof.read_text())
            traffic = pj["dram_bytes_per_cell"] * cells_local
        except (KeyError, ValueError):
            traffic = None
    roofline = {
        "bound": "int", "achieved": achieved, "peak": peak_gcups, "unit": "GCUPS", "frac": achieved / peak_gcups,
        "traffic": traffic, "kernel": "k_fwd_persist (batched forward pass)",
        "peak_basis": f"measured packed-int16 DPX add-max rate {dpx_ops / 1e12:.2f} T/s x 2 cells / "
                      f"{K_OPS_PER_CELL_PAIR} ops per packed cell pair",
        "hbm": {"achieved": alg_bytes / (fwd_avg * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": alg_bytes / (fwd_avg * 1e-3) / 1e9 / hbm_peak, "peak_basis": hbm_basis},
    }

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(pairs)

    # ---- serving (200 MB resident contigs), bounded: saturated, then 25/50/90% load ----
    serving = None
    if rank == 0 and ws == 1 and not args.no_serving:
        del tens, out_dev
        torch.cuda.empty_cache()
        serving = serving_measure(args.serving_batches_default, args.slots, 1_000_000)

    if rank == 0:
        line = {
            "metric": "GCUPS", "value": gcups, "unit": "GCUPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int16x2 (int32 re-run on overflow)",
            "data": "synthetic (seeded generator, workload shapes of the reference's measured configs)",
            "config": {"workload": (WORKLOAD_NAME if args.config == 2 and args.pairs is None else
                                    f"config {args.config}, {n_per} pairs per GPU") +
                       (" in CIGAR mode" if args.cigar else ""), "pairs_per_gpu": n_per,
                       "scoring": list(SCORING), "form": "batched persistent",
                       "cache": "inputs larger than L2 (2.6 GB resident per GPU)", "parallelism": f"replicas x{ws}"},
            "alignments_per_s": pairs_all / (ms * 1e-3),
            "fwd_ms": statistics.mean(fwd_ms), "rev_ms": statistics.mean(rev_ms),
            "plain": plain, "batched_vs_plain": (gcups / plain["gcups"]) if plain else None,
            "e2e": {"value": e2e_gcups, "unit": "GCUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "host_to_device_gbs": h2d_gbs,
                    "ms_per_step": e2e_s * 1e3, "steps": args.e2e_steps,
                    "mode": "async calls, four in flight: later steps' copies overlap step k's kernels",
                    "calls": e2e_calls},
            "e2e_sequential": {"value": cells_all / e2e_seq_s / 1e9, "unit": "GCUPS", "ms_per_step": e2e_seq_s * 1e3,
                               "device_ms": seq_t["total_ms"], "fwd_ms": seq_t["fwd_ms"], "rev_ms": seq_t["rev_ms"],
                               "call_wall_ms": seq_wall, "call_device_ms": seq_dev,
                               "mode": "1 handle, one synchronous call at a time; device_ms = the last call's "
                                       "device span from its first copy in to its result copy out (the rest "
                                       "of ms_per_step is host time); call_* = each call's wall time and "
                                       "device span"},
            "gpu_launches": launches,
            "tuning": tuning,
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
            "paths": paths, "serving": serving,
            "overflow16_pairs": int(last["n_overflow16"]), "rev_wavefront_pairs": int(last["n_rev_wide"]),
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
