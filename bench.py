#!/usr/bin/env python3
"""Benchmark: wavelet matrix + wavelet tree + rank/select construction of a
1 GiB uint8 text (n = 2^30, Zipf(1.0) over 256 symbols, 8 levels) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step builds both structures and their rank/select support from a text
resident in HBM.  `value` is whole-job text GB/s (n bytes per step per rank
over the max-over-ranks device time); `e2e` is the same metric through the
public host API (pinned host text in, both structures' bit vectors out).
Ranks run independent replicas (weak scaling, no collective on the data path).
`--impl reference` times pwm's parallel CPU construction paths (the oracle's
restatements of wx_ppc and wx_dd_ps, + rank/select) on the host cores
instead, on the same full-size text, without loading the GPU library.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "WM/WT build text GB/s"
N_DEFAULT = 1 << 30
LEVELS = 8


def workload_config(n):
    return {"workload": f"one uint8 text of n={n} symbols, Zipf(s=1.0) ranks over 256 symbols mapped by a seeded "
                        "permutation, levels=8; wavelet matrix + levelwise wavelet tree + rank/select support",
            "n": n, "word_width": 1, "levels": LEVELS, "structures": ["matrix", "tree"], "rank_select": True,
            "l2": "inputs larger than L2 (1 GiB text, 2 GiB of bit vectors)",
            "generator": "counter-based splitmix64 (pwm_gb300/csrc/gen.hpp), ZIPF256, seed 1 + rank"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.lines = []
        self.proc = None

    def start(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"]
        if self.gpu_id:
            cmd += ["-i", self.gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)
        if not self.lines:  # very short region: one snapshot
            cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"]
            if self.gpu_id:
                cmd += ["-i", self.gpu_id]
            try:
                self.lines = subprocess.run(cmd, capture_output=True, text=True, timeout=20).stdout.splitlines()
            except Exception:
                pass
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """dram bytes per launch of the split pass from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "split_pass_traffic.json")) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch_full_size")
    except Exception:
        return None


def parse_profile(text):
    out = {}
    for line in text.strip().splitlines():
        name, groups, launches, ms, nbytes = line.split()
        out[name] = {"groups": int(groups), "launches": int(launches), "ms": float(ms), "bytes": int(nbytes)}
    return out


CPU_LEGS = ("ppc", "dd_ps")
CPU_LEG_NAMES = {"ppc": "pwm wx_ppc (parallel prefix counting)", "dd_ps": "pwm wx_dd_ps (domain decomposition)"}


def cpu_step_times(orc, text, threads, runs, warmup):
    """Seconds per step of each CPU leg (matrix + tree + rank/select of all
    levels): `warmup` untimed and `runs` timed steps per leg."""
    bufs = orc.cpu_step_buffers(text.size, LEVELS)
    times = {leg: [] for leg in CPU_LEGS}
    for _ in range(warmup):
        for leg in CPU_LEGS:
            orc.cpu_step(text, LEVELS, threads, bufs, leg)
    for _ in range(runs):
        for leg in CPU_LEGS:
            t0 = time.perf_counter()
            orc.cpu_step(text, LEVELS, threads, bufs, leg)
            times[leg].append(time.perf_counter() - t0)
    return times


def cpu_legs_summary(n, times, threads):
    legs = {leg: {"name": CPU_LEG_NAMES[leg], "seconds_per_step": statistics.median(ts),
                  "value": n / statistics.median(ts) / 1e9, "runs": len(ts)} for leg, ts in times.items()}
    best = max(legs, key=lambda k: legs[k]["value"])
    return legs, best


def cpu_baseline(n):
    """pwm's two parallel CPU paths, restated by the oracle (OpenMP, all host
    cores), on the same full-size workload: the 2^30 Zipf text (the oracle's
    copy of the generator, without the GPU library), matrix + tree +
    rank/select of all levels; one warm-up and one timed step per leg."""
    from oracle.oracle import Oracle
    orc = Oracle()
    threads = os.cpu_count() or 1
    text = orc.generate(2, replica_seed(0), n, 1)
    times = cpu_step_times(orc, text, threads, runs=1, warmup=1)
    legs, best = cpu_legs_summary(n, times, threads)
    return {"value": legs[best]["value"], "unit": "GB/s", "cores": threads, "kind": "port", "leg": best,
            "legs": legs,
            "sample": f"the full workload (n={n} uint8 Zipf text, levels=8): matrix + tree + rank/select of every "
                      "level, with the oracle's OpenMP restatements of pwm's wx_ppc and wx_dd_ps (value: the faster "
                      "leg); one warm-up and one timed step per leg"}


def batched_vs_per_text(torch, pg, ctx, count=4096, seed=1, reps=5, per_text=True):
    """The batched workload: 4096 uint8 texts (log-normal lengths, 85%
    DNA-like with 3 levels, 15% Zipf bytes with 8 levels), matrix + tree of
    every text.  Batched: one CUDA graph per build whose persistent kernel
    takes (text, pass, tile) items from a device work queue, tile sizes tuned
    per text class by the library (first build, cached in the context).
    Per text: each text its own single-text batch (the same kernels, one
    graph launch per text), launched back to back on the stream with no host
    synchronisation in between.  CUDA events; texts resident on the device."""
    import numpy as np
    texts, offs, levels = pg.generate_batch(seed, count)
    total = int(offs[-1])
    d = torch.from_numpy(texts).cuda()
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    b = pg.Batch(offs, levels, word_width=1, tree=True, context=ctx)
    b.build(d.data_ptr())  # tunes new classes, plans, records the graph
    b.check()
    first_build_s = time.perf_counter() - t0
    for _ in range(3):
        b.build(d.data_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.build(d.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    b.check()
    batched_ms = e0.elapsed_time(e1) / reps
    vpt = [b.tile_vectors(i) for i in range(count)]
    if not per_text:  # (profiling runs: the batched builds only)
        b.free()
        return {"texts": count, "symbols": total, "batched_ms": batched_ms,
                "batched_gbs": total / (batched_ms / 1e3) / 1e9}
    # per-text: a batch of one text each (graphs recorded up front, untimed)
    base = d.data_ptr()
    per = []
    for i in range(count):
        one = np.array([0, int(offs[i + 1] - offs[i])], dtype=np.uint64)
        x = pg.Batch(one, levels[i:i + 1], word_width=1, tree=True, context=ctx)
        x.build(base + int(offs[i]))
        per.append(x)
    torch.cuda.synchronize()
    for i in range(count):
        per[i].build(base + int(offs[i]))
    e0.record(stream)
    for _ in range(2):
        for i in range(count):
            per[i].build(base + int(offs[i]))
    e1.record(stream)
    torch.cuda.synchronize()
    per_ms = e0.elapsed_time(e1) / 2
    # spot check: batch == per-text for a few texts
    same = True
    for i in range(0, count, max(1, count // 16)):
        a_, c = b.download(i, 0), per[i].download(0, 0)
        same &= all(np.array_equal(np.asarray(a_.bvs()[l]), np.asarray(c.bvs()[l])) for l in range(int(levels[i])))
        same &= a_.zeros() == c.zeros()
        a_, c = b.download(i, 1), per[i].download(0, 1)
        same &= all(np.array_equal(np.asarray(a_.bvs()[l]), np.asarray(c.bvs()[l])) for l in range(int(levels[i])))
    for x in per:
        x.free()
    b.free()
    lens = (offs[1:] - offs[:-1]).astype(np.float64)
    alg = float(2 * (lens * levels.astype(np.float64)).sum() + 2 * 8 * (np.ceil(lens / 64) * levels).sum())
    peak, peak_kind = measured_peak()
    return {"texts": count, "symbols": total, "levels_mix": {"3": int((levels == 3).sum()), "8": int((levels == 8).sum())},
            "batched_gbs": total / (batched_ms / 1e3) / 1e9, "batched_ms": batched_ms,
            "per_text_gbs": total / (per_ms / 1e3) / 1e9, "per_text_ms": per_ms,
            "speedup": per_ms / batched_ms, "engine": "tile (persistent work queue)",
            "tile_vectors_per_thread": {str(v): vpt.count(v) for v in sorted(set(vpt))},
            "first_build_s": first_build_s,
            "roofline": {"algorithmic_bytes": alg, "achieved_gbs": alg / (batched_ms / 1e3) / 1e9,
                         "frac": alg / (batched_ms / 1e3) / 1e9 / peak, "peak": peak, "peak_source": peak_kind},
            "per_text": "each text a batch of one (one graph launch per text), launched back to back, no host sync",
            "identical_to_per_text": bool(same), "structures": ["matrix", "tree"]}


def other_workloads(torch, pg, ctx, reps=3, only=None, cap_n=0):
    """Build times of the other configured workloads (resident text, CUDA
    events on the library's stream; the drop-in Huffman builds host to host):
    2^26 DNA-like bytes with 2 levels (matrix + tree), 2^30 bytes uniform
    over 64 values with 6 levels (matrix + tree in one tile pass), the 1 GiB
    Zipf text built as 16 shards and merged (pwm's wx_dd_*), 2^28
    16-bit symbols with 16 levels (plain matrix + tree, and Huffman-shaped
    matrix and tree with pwm's codes from the host builder), 2^26 32-bit
    symbols over 2^20 values with 20 levels (matrix + rank/select)."""
    import numpy as np
    out = {}
    stream = torch.cuda.current_stream()

    def timed(name, n, width, levels, dist, param, tree, rs, shards=0):
        if only is not None and name not in only:
            return None
        if cap_n:  # a smaller case of the same workload (profiling)
            n = min(n, cap_n)
        dtype = {1: torch.uint8, 2: torch.int16, 4: torch.int32}[width]
        t = torch.empty(n, dtype=dtype, device="cuda")
        pg.generate(dist, 3, n, width, param=param, device_ptr=t.data_ptr(), context=ctx)
        ds = pg.DeviceStructure(n, width, levels, matrix=True, tree=tree, rank_select=rs, context=ctx)
        build = (lambda: ds.build_sharded(t.data_ptr(), shards)) if shards else (lambda: ds.build(t.data_ptr()))
        build()
        ctx.lib.pwmgpu_ctx_profile(ctx.h, 1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            build()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        buf = ctypes.create_string_buffer(1 << 16)
        ctx.check(ctx.lib.pwmgpu_ctx_profile_read(ctx.h, buf, len(buf)))
        ctx.lib.pwmgpu_ctx_profile(ctx.h, 0)
        prof = parse_profile(buf.value.decode())
        ds.check()
        ds.free()
        out[name] = {"n": n, "word_width": width, "levels": levels, "structures": ["matrix"] + (["tree"] if tree else []),
                     "rank_select": rs, "ms": ms, "text_gbs": n * width / ms / 1e6}
        if shards:
            m = prof.get("merge", {})
            out[name]["shards"] = shards
            if m.get("ms"):
                # the merge reads and writes every level of both structures once
                out[name]["merge_ms"] = m["ms"] / reps
                out[name]["merge_gbs"] = m["bytes"] / (m["ms"] / 1e3) / 1e9
        return t

    timed("dna_2p26_levels2", 1 << 26, 1, 2, pg.GEN_DNA4, 0, True, False)
    timed("uniform64_2p30_levels6", 1 << 30, 1, 6, pg.GEN_UNIFORM, 64, True, False)
    timed("zipf_2p30_levels8_16_shards", 1 << 30, 1, 8, pg.GEN_ZIPF256, 0, True, False, shards=16)
    t16 = timed("mix16_2p28_levels16", 1 << 28, 2, 16, pg.GEN_MIX16, 0, True, False)
    timed("uniform20_2p26_levels20", 1 << 26, 4, 20, pg.GEN_UNIFORM, 1 << 20, False, True)
    if only is not None:  # (profiling runs: the named builds only)
        return out
    # pwm's reduce_alphabet on the device (the 2^28 16-bit text; histogram,
    # first occurrences, host ranking of the symbols, remap): wall time
    out16 = torch.empty_like(t16)
    pg.reduce_alphabet(t16.data_ptr(), t16.numel(), 2, out16.data_ptr(), context=ctx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        max_char = pg.reduce_alphabet(t16.data_ptr(), t16.numel(), 2, out16.data_ptr(), context=ctx)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    out["alphabet_reduction_mix16_2p28"] = {"n": int(t16.numel()), "word_width": 2, "distinct_symbols": max_char + 1,
                                            "ms": ms, "text_gbs": t16.numel() * 2 / ms / 1e6}
    del out16
    host16 = t16.cpu().numpy().view(np.uint16)
    del t16
    for tree in (False, True):
        pg.huffman_codes(host16, tree, ctx)  # warm-up (staging ring, scratch)
        t0 = time.perf_counter()
        codes = pg.huffman_codes(host16, tree, ctx)
        codes_ms = (time.perf_counter() - t0) * 1e3
        cons = pg.wx_huff_ps(np.uint16, tree, context=ctx)
        cons.compute(host16, host16.size, 0, codes=codes)
        t1 = time.perf_counter()
        ws = cons.compute(host16, host16.size, 0, codes=codes)
        t2 = time.perf_counter()
        # the same call with pageable buffers handed to the driver unstaged
        ctx.set_host_copy_threads(0)
        u0 = time.perf_counter()
        cons.compute(host16, host16.size, 0, codes=codes)
        u1 = time.perf_counter()
        ctx.set_host_copy_threads(-1)
        # device-resident: the same codes, a device text, the structure kept in
        # HBM; the kernels' time from the library's CUDA events, and the call
        d_text = torch.from_numpy(host16.view(np.int16)).cuda()
        torch.cuda.synchronize()
        ds = pg.DeviceStructure.huffman(d_text.data_ptr(), host16.size, 2, tree=tree, rank_select=False,
                                        codes=codes[:2], context=ctx)
        ds.free()
        ctx.lib.pwmgpu_ctx_profile(ctx.h, 1)
        t3 = time.perf_counter()
        ds = pg.DeviceStructure.huffman(d_text.data_ptr(), host16.size, 2, tree=tree, rank_select=False,
                                        codes=codes[:2], context=ctx)
        ds.check()
        t4 = time.perf_counter()
        buf = ctypes.create_string_buffer(1 << 16)
        ctx.check(ctx.lib.pwmgpu_ctx_profile_read(ctx.h, buf, len(buf)))
        ctx.lib.pwmgpu_ctx_profile(ctx.h, 0)
        prof = parse_profile(buf.value.decode())
        kern_ms = sum(v["ms"] for v in prof.values())
        hbytes = sum(v["bytes"] for k, v in prof.items() if k == "split_pass")
        ds.free()
        del d_text
        out["mix16_2p28_huffman_" + ("tree" if tree else "matrix")] = {
            "n": int(host16.size), "word_width": 2, "levels": ws.levels(), "codes_ms": codes_ms,
            "build_host_to_host_ms": (t2 - t1) * 1e3, "text_gbs_host_to_host": host16.nbytes / (t2 - t1) / 1e9,
            "build_host_to_host_unstaged_ms": (u1 - u0) * 1e3,
            "device_call_ms": (t4 - t3) * 1e3, "device_kernels_ms": kern_ms,
            "device_kernel_groups": {k: round(v["ms"], 3) for k, v in prof.items()},
            "split_pass_roofline_frac": (hbytes / (prof["split_pass"]["ms"] / 1e3) / 1e9 / measured_peak()[0])
            if prof.get("split_pass", {}).get("ms") else None}
    out["queries_mix16_2p28"] = query_rates(torch, pg, ctx, host16)
    del host16
    out["semi_external_zipf_2p31_levels8"] = semi_external_rate(torch, pg, ctx)
    return out


def semi_external_rate(torch, pg, ctx, n=1 << 31, budget=4 << 30, reps=3):
    """Semi-external build (pwmgpu_compute_semi_external) of a 2 GiB Zipf
    text, 8 levels, matrix + tree, through a 4 GiB device budget: pinned host
    text in, pinned host arrays out; wall time of the call (best of reps)."""
    t = torch.empty(n, dtype=torch.uint8, device="cuda")
    pg.generate(pg.GEN_ZIPF256, 4, n, 1, device_ptr=t.data_ptr(), context=ctx)
    host = t.cpu().pin_memory()
    del t
    lw = (((n + 63) // 64) + 15) // 16 * 16
    om = torch.empty(8 * lw, dtype=torch.int64).pin_memory()
    ot = torch.empty(8 * lw, dtype=torch.int64).pin_memory()
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        pg.compute_semi_external(host.numpy(), 8, device_budget=budget, out=(om, ot), context=ctx)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return {"n": n, "levels": 8, "structures": ["matrix", "tree"], "device_budget": budget,
            "ms": best * 1e3, "text_gbs_host_to_host": n / best / 1e9,
            "host_bytes_moved": 2 * n + 2 * 8 * lw * 8}


def query_rates(torch, pg, ctx, host16, nq=1 << 22, reps=3):
    """Access/rank/select rates (millions of queries per second) on the 2^28
    16-bit text: the plain matrix (16 levels) against the Huffman-shaped
    matrix with pwm's codes, whose queries walk only their symbol's code.
    Uniform positions, symbols drawn from the text, occurrences uniform
    within each symbol's count; device arrays, CUDA events."""
    import numpy as np
    rng = np.random.default_rng(11)
    n = host16.size
    d_text = torch.from_numpy(host16.view(np.int16)).cuda()
    sym_np = host16[rng.integers(0, n, nq)].astype(np.int64)
    counts = np.bincount(host16, minlength=1 << 16)
    occ_np = 1 + np.floor(rng.random(nq) * counts[sym_np]).astype(np.int64)
    pos = torch.from_numpy(rng.integers(0, n, nq).astype(np.int64)).cuda()
    sym = torch.from_numpy(sym_np).cuda()
    occ = torch.from_numpy(occ_np).cuda()
    res = torch.empty(nq, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    codes = pg.huffman_codes(host16, False, ctx)
    plain = pg.DeviceStructure(n, 2, 16, matrix=True, rank_select=True, context=ctx)
    plain.build(d_text.data_ptr())
    huff = pg.DeviceStructure.huffman(d_text.data_ptr(), n, 2, tree=False, rank_select=True, codes=codes[:2],
                                      context=ctx)
    out = {"queries": nq, "mean_code_length": float((codes[0] * counts[:codes[0].size]).sum()) / n}
    for name, ds in (("plain_matrix", plain), ("huffman_matrix", huff)):
        rates = {}
        for op, opname, a, b in ((pg.Q_ACCESS, "access", pos, None), (pg.Q_RANK, "rank", sym, pos),
                                 (pg.Q_SELECT, "select", sym, occ)):
            def run():
                ds.query(0, op, a.data_ptr(), b.data_ptr() if b is not None else None, nq, res.data_ptr())
            run()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                run()
            e1.record(stream)
            torch.cuda.synchronize()
            rates[opname + "_mqps"] = nq * reps / (e0.elapsed_time(e1) / 1e3) / 1e6
        ds.check()
        out[name] = rates
    plain.free()
    huff.free()
    return out


def serving_requests(pg, count, seed=7, nq=10_000):
    """The serving mix: the batched workload's uint8 texts (log-normal
    lengths; 85% DNA-like with 3 levels, 15% Zipf bytes with 8 levels) plus 5%
    uint32 texts uniform over 2^20 values with 20 levels (same length law,
    clamped to 2^26); every request carries nq access/rank/select queries at
    uniform positions, symbols taken from the text."""
    import numpy as np
    rng = np.random.default_rng(seed)
    texts, offs, levels = pg.generate_batch(seed, count)
    reqs = []
    for i in range(count):
        if rng.random() < 0.05:
            n = int(min(max(round(np.exp(rng.normal(np.log(2 ** 16), 1.5))), 2 ** 10), 2 ** 26))
            t, L = rng.integers(0, 1 << 20, n).astype(np.uint32), 20
        else:
            t, L = texts[int(offs[i]):int(offs[i + 1])], int(levels[i])
        n = t.size
        ops = rng.integers(0, 3, nq).astype(np.uint8)
        sym = t[rng.integers(0, n, nq)].astype(np.uint64)
        counts = np.bincount(t.astype(np.int64), minlength=1 << L)
        occ = 1 + np.floor(rng.random(nq) * counts[sym.astype(np.int64)]).astype(np.uint64)
        a = np.where(ops == 0, rng.integers(0, n, nq).astype(np.uint64), sym)
        b = np.where(ops == 1, rng.integers(0, n + 1, nq).astype(np.uint64), occ)
        reqs.append((t, L, ops, a, b, i % 2))  # queries alternate between the matrix and the tree
    return reqs


def serve_run(pg, reqs, rate, slots, budget):
    """Poisson arrivals at `rate` requests/s (rate None: one at a time, each
    submitted when the previous finished; "saturate": all submitted at once,
    the server's maximum throughput).  Every request builds a matrix and a
    tree with rank/select, then answers its queries on one of them.  A
    collector waits for and releases every request.  Returns latency and
    throughput figures."""
    import numpy as np
    srv = pg.Server(budget, slots=slots)
    infos = [None] * len(reqs)
    ids = [None] * len(reqs)
    ready = threading.Semaphore(0)

    def collector():
        for k in range(len(reqs)):
            ready.acquire()
            infos[k] = srv.wait(ids[k])
            srv.release(ids[k])

    col = threading.Thread(target=collector)
    col.start()
    rng = np.random.default_rng(11)
    t0 = time.perf_counter()
    t_next = t0
    for k, (t, L, ops, a, b, which) in enumerate(reqs):
        if rate is not None and rate != "saturate":
            t_next += rng.exponential(1.0 / rate)
            delay = t_next - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
        ids[k], _ = srv.submit(t, L, matrix=True, tree=True, which=which, ops=ops, a=a, b=b)
        ready.release()
        if rate is None:
            srv.wait(ids[k])
    col.join()
    stats = srv.stats()
    srv.close()
    lat = np.array([i.done_s - i.submit_s for i in infos]) * 1e3
    svc = np.array([i.done_s - i.start_s for i in infos]) * 1e3
    span = max(i.done_s for i in infos) - min(i.submit_s for i in infos)
    sym = sum(int(r[0].size) for r in reqs)
    byt = sum(int(r[0].nbytes) for r in reqs)
    return {"offered_req_s": rate, "requests": len(reqs), "throughput_req_s": len(reqs) / span,
            "text_gbs": byt / span / 1e9, "symbols": sym, "queries_per_request": int(reqs[0][2].size),
            "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
            "service_ms_p50": float(np.percentile(svc, 50)), "service_ms_p99": float(np.percentile(svc, 99)),
            "peak_device_bytes": stats["peak_bytes"], "slots": slots}


def serving_bench(pg, count=2000, slots=8, budget=150 * 10 ** 9):
    """p50/p99 request latency and throughput of the continuous-batching
    server over `count` requests per offered rate: Poisson rates 100, 1000
    and 10000 requests/s and saturation (all requests at once), next to
    one-at-a-time construction (one slot, closed loop).  `at_saturation`
    repeats the figures of the saturated run (the highest throughput)."""
    reqs = serving_requests(pg, count)
    serve_run(pg, reqs[:64], None, 1, budget)  # warm-up
    out = {"workload": "batched-workload uint8 texts + 5% uint32 (2^20 values, 20 levels); build (matrix + tree + "
                       "rank/select) then 10^4 access/rank/select queries per request on the matrix or the tree "
                       "(alternating); budget 150 GB",
           "requests_per_rate": count, "one_at_a_time": serve_run(pg, reqs, None, 1, budget), "rates": []}
    for rate in (100, 1000, 10000, "saturate"):
        out["rates"].append(serve_run(pg, reqs, rate, slots, budget))
    out["at_saturation"] = out["rates"][-1]
    return out


def run_reference(args, rank):
    """pwm's own CPU path for this workload on the host cores: the oracle's
    OpenMP restatements of wx_ppc and wx_dd_ps (pwm's two parallel
    constructions; the reference source tree is not present where this
    runs, so its headers cannot be compiled here) over the full 2^30 text,
    matrix + tree + rank/select of every level.  Each step runs both legs;
    `value` is the faster leg's.  Rank 0 alone runs under torchrun."""
    if rank != 0:
        return 0
    from oracle.oracle import Oracle
    orc = Oracle()
    n = args.n
    threads = os.cpu_count() or 1
    text = orc.generate(2, replica_seed(0), n, 1)
    times = cpu_step_times(orc, text, threads, runs=max(args.steps, 1), warmup=args.warmup)
    legs, best = cpu_legs_summary(n, times, threads)
    value = legs[best]["value"]
    dt = legs[best]["seconds_per_step"]
    line = {"metric": METRIC, "value": value, "unit": "GB/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": workload_config(n),
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port", "leg": best,
                             "legs": legs,
                             "sample": f"the full workload per step (n={n}); pwm's wx_ppc and wx_dd_ps through the "
                                       "oracle's OpenMP restatements (pwm's own headers are not on this host); "
                                       "value: the faster leg, median over the steps"},
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---- replicas across ranks (one text per rank, no collective on the data
# ---- path): the helpers the launch under torchrun uses, also run by the
# ---- gloo tests on CPU
def replica_seed(rank):
    """Each rank builds its own text (weak scaling)."""
    return 1 + rank


def max_over_ranks(x, dist, device):
    """The slowest rank's time (the job's time)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, n, seconds):
    """Whole-job text GB/s: all ranks' symbols over the slowest rank's time."""
    return world * n / seconds / 1e9


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--pass-levels", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--engine", default="tile", choices=["tile", "warp"])
    ap.add_argument("--no-other", action="store_true")
    # profiling runs: the batched builds without the per-text baseline, and
    # only the named other workloads (comma-separated)
    ap.add_argument("--no-per-text", action="store_true")
    ap.add_argument("--other-only", default=None)
    ap.add_argument("--other-n", type=int, default=0, help="cap the other workloads' sizes (profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import numpy as np
    import torch
    import pwm_gb300 as pg

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()

    # a dedicated stream, current for torch and given to the library, so that
    # CUDA events recorded on it bracket the library's launches
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = pg.Context(device=local, stream=ctypes_stream(stream))
    if args.pass_levels:
        ctx.set_pass_levels(args.pass_levels)
    if args.engine == "warp":
        ctx.set_engine(pg.ENGINE_WARP)
    n = args.n
    text = torch.empty(n, dtype=torch.uint8, device="cuda")
    pg.generate(pg.GEN_ZIPF256, replica_seed(rank), n, 1, device_ptr=text.data_ptr(), context=ctx)
    ds = pg.DeviceStructure(n, 1, LEVELS, matrix=True, tree=True, rank_select=True, context=ctx)
    for _ in range(args.warmup):
        ds.build(text.data_ptr())
    ds.check()

    gpu_uuid = None
    try:
        gpu_uuid = str(torch.cuda.get_device_properties(local).uuid)
        if not gpu_uuid.startswith("GPU-"):
            gpu_uuid = "GPU-" + gpu_uuid
    except Exception:
        gpu_uuid = None
    sampler = ClockSampler(gpu_uuid)

    # ---- device-resident timed region ------------------------------------
    ctx.lib.pwmgpu_ctx_profile(ctx.h, 1)
    launches0 = ctx.launches
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)  # let the sampler start before the region
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ds.build(text.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    ds.check()
    launches = ctx.launches - launches0
    buf = ctypes.create_string_buffer(1 << 16)
    ctx.check(ctx.lib.pwmgpu_ctx_profile_read(ctx.h, buf, len(buf)))
    ctx.lib.pwmgpu_ctx_profile(ctx.h, 0)
    prof = parse_profile(buf.value.decode())
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dist, "cuda")
    value = job_throughput(world, n, ms / 1e3)

    # ---- end to end through the public host API --------------------------
    host_text = text.cpu().pin_memory()
    vm, vt = ds.view(0), ds.view(1)
    out_wm = torch.empty(vm.total_words, dtype=torch.int64).pin_memory()
    out_wt = torch.empty(vt.total_words, dtype=torch.int64).pin_memory()
    zeros = np.zeros(LEVELS, dtype=np.uint64)
    zp = zeros.ctypes.data_as(pg._lib.u64p)

    wm_ptr = ctypes.cast(out_wm.data_ptr(), pg._lib.u64p)
    wt_ptr = ctypes.cast(out_wt.data_ptr(), pg._lib.u64p)

    def e2e_step():
        # host text in, both structures out: the levels stream back while the build runs
        ctx.check(ctx.lib.pwmgpu_wx_compute_host(ctx.h, ds.h, host_text.data_ptr(), wm_ptr, zp, wt_ptr))

    for _ in range(max(3, args.warmup)):  # the first host-to-host calls allocate and pin their buffers
        e2e_step()
    barrier()
    torch.cuda.synchronize()
    # each call returns once its outputs are on the host: timed one by one,
    # the median reported (an occasional slow call, e.g. a page of the pinned
    # arrays first touched by the host, does not set the number)
    e2e_steps_s = []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        e2e_step()
        e2e_steps_s.append(time.perf_counter() - t0)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(statistics.median(e2e_steps_s), dist, "cuda")
    e2e_value = job_throughput(world, n, e2e_s)

    if rank == 0:
        peak, peak_kind = measured_peak()
        sp = prof.get("split_pass", {})
        achieved = (sp["bytes"] / (sp["ms"] / 1e3) / 1e9) if sp.get("ms") else None
        roof = {"bound": "hbm", "kernel": "split_pass", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "peak_source": peak_kind,
                "traffic": ncu_traffic(),
                "algorithmic_bytes_per_launch": (sp["bytes"] / sp["groups"]) if sp.get("groups") else None,
                "avg_launch_ms": (sp["ms"] / sp["groups"]) if sp.get("groups") else None}
        # whole step against the roofline of its algorithmic bytes (2 structures + rank/select)
        words = (n + 63) // 64
        step_bytes = 2 * LEVELS * (n + 8 * words) + 2 * LEVELS * (8 * words + 8 * (words // 32 + 1))
        line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": workload_config(n),
                "roofline": roof,
                "step_roofline": {"algorithmic_bytes": step_bytes, "achieved_gbs": step_bytes / (ms / 1e3) / 1e9,
                                  "frac": step_bytes / (ms / 1e3) / 1e9 / peak},
                "kernels": prof, "gpu_launches": launches,
                "e2e": {"value": e2e_value, "unit": "GB/s", "statistic": "median of %d calls" % args.e2e_steps,
                        "calls_ms": [round(x * 1e3, 3) for x in e2e_steps_s], "h2d_bytes_per_step": n,
                        "d2h_bytes_per_step": 8 * (vm.total_words + vt.total_words) + 8 * LEVELS,
                        "seconds_per_step": e2e_s},
                "clocks": clocks}
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(n)
        if world == 1 and not args.no_batch:
            line["batched"] = batched_vs_per_text(torch, pg, ctx, per_text=not args.no_per_text)
        if world == 1 and not args.no_serve:
            line["serving"] = serving_bench(pg)
        if world == 1 and not args.no_other:
            line["other_workloads"] = other_workloads(
                torch, pg, ctx, only=args.other_only.split(",") if args.other_only else None, cap_n=args.other_n)
        print(json.dumps(line))
    ds.free()
    if dist:
        dist.destroy_process_group()
    return 0


def ctypes_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


if __name__ == "__main__":
    sys.exit(main())
