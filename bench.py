#!/usr/bin/env python
"""Throughput of the strobealign seed → lookup → NAM path on GB300.

Workload (one "step"): the repeat-rich mid-size configuration — a synthetic 100 Mbp
reference in 20 contigs (5% of bases in duplicated 1-10 kb segments copied 2-20x at
0.5-2% divergence, plus short tandem repeats), indexed on the GPU with the
150 bp parameters, and 1M paired-end 2x150 bp read pairs (2M reads, insert
~Normal(300, 30), 1% substitutions, 0.1% 1-3 bp indels).  A step maps all 2M reads:
randstrobes, index lookup, hit collection, NAM merge, rescue and NAM sort.

value  reads/s with inputs resident in HBM (device C-ABI entry point, CUDA events on
       the launching stream).
e2e    reads/s through the host C-ABI entry point (gbsa_map_reads): pinned host
       reads in, NAMs / offsets / fractions back to host, copies inside the timing.
The CPU baseline is the CPU restatement of the reference path on a bounded sample
of the same reads with all host cores.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbsa|reference]
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbsa", choices=["gbsa", "reference"])
    ap.add_argument("--config", default="C2", choices=["C1", "C2", "C3", "C4"],
                    help="workload (C2 is the headline configuration)")
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the workload (tests only)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU baseline sample time")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-rates", default="1000,2000,2500,3000,3500,4000,6000",
                    help="request rates (req/s) of the served-form measurement; empty to skip")
    ap.add_argument("--serve-seconds", type=float, default=4.0,
                    help="arrival window per rate (4 s: ~8-16k requests, enough for a stable p99)")
    ap.add_argument("--no-fastq", dest="fastq", action="store_false", help="skip the FASTQ staging measurement")
    ap.add_argument("--no-l2-window", dest="l2_window", action="store_false",
                    help="map without the L2 access-policy window on the bucket table (for comparison)")
    ap.add_argument("--other-configs", default="C1,C3,C4",
                    help="configurations checked for parity (and timed) after the headline one; empty to skip")
    return ap.parse_args()


# read units per config at scale 1 (pairs count as one unit): C1 100k single-end
# reads; C2 1M pairs; C3 ~2M reads half single-end, half in pairs; C4 5M pairs
UNITS = {"C1": 100_000, "C2": 1_000_000, "C3": 1_333_333, "C4": 5_000_000}


def workload(scale, rank, config="C2"):
    from gpu_index_test_gb300 import synth

    gp = synth.genome_params("C1" if config == "C3" else config, scale=scale, seed=1)
    rp = synth.read_params(config, n_units=max(1000, int(UNITS[config] * scale)), seed=11 + rank)
    t0 = time.perf_counter()
    g = synth.make_genome(gp)
    reads = synth.make_reads(g, rp)
    return g, reads, time.perf_counter() - t0, gp, rp


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, world, device=None):
    """The largest of the ranks' values of x (one all-reduce MAX; the ranks map their own
    shards of reads with no other exchange); x itself for one rank.  NCCL wants device
    tensors, gloo host ones."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, seconds):
    """Whole-job units per second: every rank processed units_per_rank in at most seconds."""
    return world * units_per_rank / seconds


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(config):
    """Per-launch DRAM bytes of each stage's kernel on a configuration's full workload, from
    the committed ncu summaries ({} when none was captured)."""
    try:
        with open(os.path.join(HERE, "profiles", "traffic.json")) as f:
            return json.load(f).get(config, {})
    except (OSError, ValueError):
        return {}


# batch slots of the served form and reads per slot (a batch packs queued requests up to this)
SERVE_SLOTS = 8
SERVE_BATCH_READS = 100_000


def lookup_roofline(alg_lookup, sectors, packed, nams, stage_ms, fused, ms, gather_gbs):
    """The seeding + lookup stage against the measured HBM copy bandwidth and against the
    random-gather ceiling of the index's own tables (32-byte sectors the reference's probes
    touch), and the whole batch's algorithmic bytes over its time: the definitions of the
    headline line's roofline, for another form or configuration."""
    peak, peak_kind = peaks()
    lk = "seed_lookup" if fused else "lookup"
    t = stage_ms.get(lk, 0.0) / 1e3
    alg = alg_lookup + (packed if fused else 0)
    out = {"kernel": lk, "stage_ms": round(stage_ms.get(lk, 0.0), 3), "alg_bytes_per_launch": int(alg),
           "achieved": round(alg / t / 1e9, 1) if t > 0 else None, "peak": peak, "unit": "GB/s",
           "frac": round(alg / t / 1e9 / peak, 4) if t > 0 else None, "peak_source": peak_kind}
    g = sectors * 32 / t / 1e9 if t > 0 else 0.0
    out["gather"] = {"sectors_per_launch": int(sectors), "achieved": round(g, 1), "peak": round(gather_gbs, 1),
                     "frac": round(g / gather_gbs, 4) if gather_gbs > 0 and t > 0 else None,
                     "peak_source": "gbsa_bench_gather_index on this index"}
    whole = packed + alg_lookup + 44 * nams
    out["whole_batch"] = {"alg_bytes": int(whole), "ms": round(ms, 3), "achieved": round(whole / (ms / 1e3) / 1e9, 1),
                          "frac": round(whole / (ms / 1e3) / 1e9 / peak, 4)}
    return out


def serve_measure(idx, g, rates, seconds, scale, index_name, slots=SERVE_SLOTS, max_reads=100_000,
                  batch_reads=SERVE_BATCH_READS):
    """Served form: Poisson arrivals of requests of 1k-100k reads (log-uniform) of
    100-250 bp pairs against the resident index, continuous batching onto `slots` batch
    slots; p50/p99 latency from each request's scheduled arrival to its completion;
    every request checked byte for byte against one plain-form map_reads of the whole
    request pool (a read's NAMs depend only on the read, so this is the request mapped
    alone).  The schedule runs through gbsa_server_replay (native submit, completion and
    checker threads), so no interpreter delays sit between the schedule and the server.
    The rates sweep up to saturation; the highest rate with p99 < 20 ms is reported."""
    import torch
    from gpu_index_test_gb300 import abi, native, synth

    pool = synth.make_reads(g, synth.ReadParams(seed=123, n_units=max(2000, int(1_000_000 * scale)), len_min=100,
                                                len_max=250, paired_frac=1.0, insert_mean=400, insert_sd=50))
    pm = native.Mapper(idx, max_reads=pool.n, max_bases=int(pool.lengths.sum()))
    plain = pm.map_reads(pool)
    # algorithmic bytes and gather sectors per read of the request pool: the counting
    # instance on the pool's first reads, mapped as one batch
    sample = pool.subset(np.arange(min(pool.n, 200_000)))
    pm.set_count_bytes(True)
    pm.map_reads(sample)
    s_alg, s_sec = pm.last_alg_bytes(), pm.last_alg_sectors()
    pm.set_count_bytes(False)
    pm.free()
    s_packed = int(((sample.lengths.astype(np.int64) + 3) // 4).sum())
    s_nams = int(plain[1][sample.n])
    npr = max(24, int(np.ceil(len(plain[0]) / pool.n * 2.5)))
    srv = native.Server(idx, workers=slots, max_reads=batch_reads, max_bases=batch_reads * 250)
    g0 = srv.stats()
    n_slots, slot_nams = 48, max_reads * npr
    plain_bytes = np.ascontiguousarray(plain[0])
    plain_off_u = np.ascontiguousarray(plain[1], np.uint64)
    plain_frac = np.ascontiguousarray(plain[2], np.float32)
    plain_resc = np.ascontiguousarray(plain[3], np.uint8)
    pool_offs = np.ascontiguousarray(pool.offsets, np.uint64)
    pool_lens = np.ascontiguousarray(pool.lengths, np.uint32)
    bufs = [(torch.empty(slot_nams * 44, dtype=torch.uint8).pin_memory(),
             torch.empty(max_reads + 1, dtype=torch.int64).pin_memory(),
             torch.empty(max_reads, dtype=torch.float32).pin_memory(),
             torch.empty(max_reads, dtype=torch.uint8).pin_memory()) for _ in range(n_slots)]
    buf_ptrs = [tuple(t.data_ptr() for t in b) for b in bufs]
    seq_ptr = pool.seq.ctypes.data
    results = []
    for rate in rates:
        rng = np.random.default_rng(1000 + int(rate))
        arrivals, t = [], 0.0
        while True:
            t += rng.exponential(1.0 / rate)
            if t > seconds:
                break
            n = int(np.exp(rng.uniform(np.log(1000), np.log(max_reads)))) // 2 * 2
            n = min(n, pool.n // 2 * 2)
            start = int(rng.integers(0, (pool.n - n) // 2 + 1)) * 2
            arrivals.append((t, start, n))
        # the schedule is replayed by the library's native load replay: submit calls at their
        # times from a native thread, completions collected and every request's results
        # compared byte for byte with the pool's plain-form results on native checker threads
        # before its buffers are reused (no interpreter between the schedule and the server)
        reqs = np.zeros(len(arrivals), abi.REPLAY_REQUEST)
        reqs["at_us"] = [a[0] * 1e6 for a in arrivals]
        reqs["start"] = [a[1] for a in arrivals]
        reqs["n_reads"] = [a[2] for a in arrivals]
        info0 = srv.info()
        sub_us, done_us, status, mismatch = srv.replay(
            seq_ptr, pool_offs, pool_lens, reqs, buf_ptrs, slot_nams, max_reads,
            expected=(plain_bytes.ctypes.data, plain_off_u.ctypes.data, plain_frac.ctypes.data, plain_resc.ctypes.data))
        info1 = srv.info()
        ok_req = status == 0
        failed = int((~ok_req).sum())
        lat = (done_us - reqs["at_us"])[ok_req] / 1e3
        lat_srv = (done_us - sub_us)[ok_req] / 1e3
        lat_n = reqs["n_reads"][ok_req]
        reads_done = int(lat_n.sum())
        t_last = float(done_us[ok_req].max()) / 1e6 if ok_req.any() else 0.0
        exact = bool(mismatch.sum() == 0)
        lat_ms = np.sort(lat)
        small = np.sort(lat[lat_n <= 10_000])
        n_req = len(arrivals)
        delay = np.sort(sub_us - reqs["at_us"]) / 1e3
        results.append({
            "rate_req_s": rate, "requests": n_req, "failed": failed,
            "offered_reads_per_s": round(sum(a[2] for a in arrivals) / seconds, 1),
            "reads_per_s": round(reads_done / max(1e-9, t_last), 1),
            "p50_ms": round(float(lat_ms[len(lat_ms) // 2]), 2) if len(lat_ms) else None,
            "p99_ms": round(float(lat_ms[min(len(lat_ms) - 1, int(len(lat_ms) * 0.99))]), 2) if len(lat_ms) else None,
            "max_ms": round(float(lat_ms[-1]), 2) if len(lat_ms) else None,
            # from the submit call, and how late the replay's submit calls were against the schedule
            "p99_ms_from_submit": round(float(np.percentile(lat_srv, 99)), 2) if len(lat_srv) else None,
            "p99_submit_delay_ms": round(float(delay[min(len(delay) - 1, int(len(delay) * 0.99))]), 2)
            if len(delay) else None,
            "requests_le_10k_reads": int(len(small)),
            "p50_ms_le_10k_reads": round(float(small[len(small) // 2]), 2) if len(small) else None,
            "p99_ms_le_10k_reads": round(float(small[min(len(small) - 1, int(len(small) * 0.99))]), 2)
            if len(small) else None,
            "batches": info1["batches"] - info0["batches"],
            "requests_per_batch": round((info1["requests"] - info0["requests"])
                                        / max(1, info1["batches"] - info0["batches"]), 2),
            "bit_exact_vs_plain": bool(exact and failed == 0),
        })
    info = srv.info()
    growth = srv.stats()
    srv.free()
    # the plain form one request at a time (gbsa_map_reads per request, host buffers, the
    # same request sizes): what the served form replaces
    one = None
    if results:
        rng = np.random.default_rng(999)
        L = native.lib()
        pm = native.Mapper(idx, max_reads=max_reads, max_bases=max_reads * 250)
        b0 = buf_ptrs[0]
        sizes = [int(np.exp(rng.uniform(np.log(1000), np.log(max_reads)))) // 2 * 2 for _ in range(300)]
        starts = [int(rng.integers(0, (pool.n - n) // 2 + 1)) * 2 for n in sizes]

        def one_req(start, n):
            rc = L.gbsa_map_reads(pm.h, seq_ptr, pool_offs.ctypes.data + 8 * start, pool_lens.ctypes.data + 4 * start,
                                  n, b0[0], slot_nams, b0[1], b0[2], b0[3])
            if rc != 0:
                raise RuntimeError(f"gbsa_map_reads failed: {rc}")
        for st_, n_ in zip(starts[:10], sizes[:10]):
            one_req(st_, n_)
        t1 = time.perf_counter()
        for st_, n_ in zip(starts, sizes):
            one_req(st_, n_)
        dt = time.perf_counter() - t1
        pm.free()
        one = {"requests": len(sizes), "reads_per_s": round(sum(sizes) / dt, 1),
               "ms_per_request": round(dt / len(sizes) * 1e3, 3)}
    ok = [r for r in results if r["p99_ms"] is not None and r["p99_ms"] < 20.0 and r["bit_exact_vs_plain"]]
    sat = max(ok, key=lambda r: r["reads_per_s"]) if ok else None
    # the latency target is stated for requests of up to 10k reads
    ok10 = [r for r in results if r["p99_ms_le_10k_reads"] is not None and r["p99_ms_le_10k_reads"] < 20.0
            and r["bit_exact_vs_plain"]]
    sat10 = max(ok10, key=lambda r: r["reads_per_s"]) if ok10 else None
    # the served throughput against the random-gather ceiling of the index's own tables
    # and the HBM copy bandwidth: the pool's sectors and algorithmic bytes per read times
    # the reads served per second
    roof = None
    if results:
        try:
            _, _, g_gbs = native.bench_gather_index(idx)
            peak, peak_kind = peaks()
            sec_read = s_sec / sample.n
            alg_read = (s_packed + s_alg + 44 * s_nams) / sample.n

            def at(r):
                rs = r["reads_per_s"]
                return {"rate_req_s": r["rate_req_s"], "reads_per_s": rs,
                        "gather_gbs": round(rs * sec_read * 32 / 1e9, 1),
                        "gather_frac": round(rs * sec_read * 32 / 1e9 / g_gbs, 4) if g_gbs > 0 else None,
                        "alg_gbs": round(rs * alg_read / 1e9, 1), "hbm_frac": round(rs * alg_read / 1e9 / peak, 4)}
            roof = {"sectors_per_read": round(sec_read, 2), "alg_bytes_per_read": round(alg_read, 1),
                    "sample": f"counting instance on the first {sample.n} reads of the request pool",
                    "gather_peak_gbs": round(g_gbs, 1), "gather_peak_source": "gbsa_bench_gather_index on this index",
                    "hbm_peak_gbs": peak, "hbm_peak_source": peak_kind,
                    "at_saturation": at(sat) if sat else None,
                    "at_peak": at(max(results, key=lambda r: r["reads_per_s"]))}
        except Exception as e:   # recorded, not fatal
            roof = {"error": f"{type(e).__name__}: {e}"}
    return {"index": index_name, "slots": info["slots"], "slot_bytes": info["slot_bytes"],
            "graph_during_requests": {k: growth[k] - g0[k] for k in growth},
            "memory_budget_bytes": info["budget"], "batch_reads": batch_reads,
            "request_reads": "1k-100k log-uniform, 100-250 bp pairs", "rates": results,
            "saturation": ({"rate_req_s": sat["rate_req_s"], "reads_per_s": sat["reads_per_s"], "p99_ms": sat["p99_ms"]}
                           if sat else None),
            "saturation_le_10k_reads": ({"rate_req_s": sat10["rate_req_s"], "reads_per_s": sat10["reads_per_s"],
                                         "p99_ms_le_10k_reads": sat10["p99_ms_le_10k_reads"]} if sat10 else None),
            "peak_reads_per_s": round(max(r["reads_per_s"] for r in results), 1) if results else None,
            "plain_one_request_at_a_time": one, "roofline": roof,
            "vs_plain_one_at_a_time": (round(max(r["reads_per_s"] for r in results) / one["reads_per_s"], 2)
                                       if one else None)}


def fastq_pipeline(m, reads, plain_nams, plain_offs, chunk_mb=48):
    """Input staging: the reads written as two mate FASTQ files (in memory), parsed in
    chunks by the library's parser into pinned buffers while the GPU maps the previous
    chunk (gbsa_map_reads); reports the parse rate and the FASTQ-to-NAMs rate, and
    checks every chunk's NAMs byte for byte against the plain run of the same reads."""
    import threading

    import torch
    from gpu_index_test_gb300 import native

    n = reads.n // 2 * 2
    mates = []
    for mate in (0, 1):
        recs = []
        for i in range(mate, n, 2):
            o, l = int(reads.offsets[i]), int(reads.lengths[i])
            s = reads.seq[o:o + l].tobytes()
            recs.append(b"@r%d/%d\n%s\n+\n%s\n" % (i // 2, mate + 1, s, b"I" * l))
        mates.append(b"".join(recs))
    total_bytes = len(mates[0]) + len(mates[1])
    t0 = time.perf_counter()
    native.fastq_parse_pairs(mates[0], mates[1])
    parse_s = time.perf_counter() - t0
    chunk = chunk_mb << 20
    slots = []
    for _ in range(2):
        seq_t = torch.empty(2 * chunk, dtype=torch.uint8).pin_memory()
        off_t = torch.empty(chunk // 4 + 2, dtype=torch.int64).pin_memory()
        len_t = torch.empty(chunk // 4 + 1, dtype=torch.int32).pin_memory()
        slots.append((seq_t.numpy(), off_t.numpy().view(np.uint64), len_t.numpy().view(np.uint32)))
    # every chunk's NAMs land in their own region of one pinned buffer (checked after timing)
    cap = int(len(plain_nams) * 1.05) + (1 << 20)
    h_all = torch.empty(cap * 44, dtype=torch.uint8).pin_memory()
    h_off = torch.empty(n + 2, dtype=torch.int64).pin_memory()
    L = native.lib()
    plain_bytes = np.ascontiguousarray(plain_nams).view(np.uint8)
    pos = [0, 0]
    state = {}
    views = [memoryview(mates[0]), memoryview(mates[1])]

    def parse(slot):
        end = [min(len(mates[j]), pos[j] + chunk) for j in (0, 1)]
        final = end[0] == len(mates[0]) and end[1] == len(mates[1])
        r, u1, u2 = native.fastq_parse_pairs(views[0][pos[0]:end[0]], views[1][pos[1]:end[1]], final=final,
                                             out=slots[slot])
        pos[0] += u1
        pos[1] += u2
        state[slot] = r

    t0 = time.perf_counter()
    parse(0)
    done_reads, done_nams, slot, parts = 0, 0, 0, []
    while state.get(slot) is not None and state[slot].n > 0:
        r = state.pop(slot)
        nxt = 1 - slot
        th = None
        if pos[0] < len(mates[0]) or pos[1] < len(mates[1]):
            th = threading.Thread(target=parse, args=(nxt,))
            th.start()
        k = r.n
        rc = L.gbsa_map_reads(m.h, r.seq.ctypes.data, r.offsets.ctypes.data, r.lengths.ctypes.data, k,
                              h_all.data_ptr() + 44 * done_nams, cap - done_nams, h_off.data_ptr() + 8 * done_reads,
                              None, None)
        if rc != 0:
            raise RuntimeError(f"gbsa_map_reads failed: {rc}")
        tot = int(h_off[done_reads + k])
        parts.append((done_reads, k, done_nams, tot))
        done_reads += k
        done_nams += tot
        if th is not None:
            th.join()
        slot = nxt
    pipe_s = time.perf_counter() - t0
    got = h_all[: done_nams * 44].numpy()
    exact = done_reads == n
    for r0, k, a_got, tot in parts:
        a0, a1 = int(plain_offs[r0]), int(plain_offs[r0 + k])
        exact = exact and tot == a1 - a0 and np.array_equal(got[a_got * 44:(a_got + tot) * 44],
                                                            plain_bytes[a0 * 44:a1 * 44])
    return {"fastq_bytes": total_bytes, "reads": done_reads, "parse_gb_s": round(total_bytes / parse_s / 1e9, 2),
            "parse_reads_per_s": round(n / parse_s, 1), "chunk_mb_per_file": chunk_mb,
            "fastq_to_nams_reads_per_s": round(done_reads / pipe_s, 1),
            "bit_exact_vs_plain": bool(exact)}


def mem_available_gb():
    try:
        with open("/proc/meminfo") as f:
            for ln in f:
                if ln.startswith("MemAvailable:"):
                    return int(ln.split()[1]) / 1e6
    except OSError:
        pass
    return 0.0


# Genomes above this are not indexed on the host: the GPU's index is exported, checked
# against the oracle without a host build (oracle_py.verify_index) and loaded into it.
HOST_BUILD_MAX_BP = 500_000_000


def oracle_index_for(g, gpu_index=None):
    """The oracle's index of genome g: built on the host, or for a genome above
    HOST_BUILD_MAX_BP the GPU's index after it passed the sort-free check.  Returns
    (index or None, record of how it was obtained)."""
    from oracle import oracle_py

    p = oracle_py.params_from_read_length(150)
    t0 = time.perf_counter()
    if gpu_index is None or int(g.lengths.sum()) <= HOST_BUILD_MAX_BP:
        idx = oracle_py.Index.build(p, g)
        return idx, {"how": "built on the host by the oracle", "index_build_s": round(time.perf_counter() - t0, 2)}
    info = gpu_index.info()
    need = 2.2 * (16 * info.size + 8 * ((1 << info.bits) + 1)) / 1e9 + 8
    if mem_available_gb() < need:
        return None, {"how": f"skipped: host memory below {need:.0f} GB"}
    rs, st = gpu_index.export()
    t_exp = time.perf_counter() - t0
    t0 = time.perf_counter()
    verdict, rep = oracle_py.verify_index(p, g, rs, st, info.bits, info.filter_cutoff)
    rec = {"how": "GPU index exported and checked by the oracle without a host build (generated entries as a "
                  "multiset, sorted order, bucket table, filter cutoff), then loaded into the oracle",
           "export_s": round(t_exp, 2), "verify_s": round(time.perf_counter() - t0, 2), "verify": verdict,
           "entries": int(info.size), "bits": int(info.bits)}
    if verdict != "equal":
        rec["report"] = rep
        return None, rec
    idx = oracle_py.Index.load(p, rs, st, info.bits, info.filter_cutoff)
    del rs, st
    return idx, rec


def cpu_baseline(g, reads, target_s, gpu_result=None, gpu_index=None):
    """The oracle (CPU restatement of the reference path) on a bounded sample."""
    from gpu_index_test_gb300 import abi

    idx, how = oracle_index_for(g, gpu_index)
    if idx is None:
        return {"index": how}, False
    build_s = how.get("index_build_s")
    cores = os.cpu_count() or 1
    opt = abi.map_options()
    cal = reads.subset(np.arange(min(reads.n, 20000)))
    t0 = time.perf_counter()
    idx.map_reads(cal, opt, n_threads=cores)
    per_read = (time.perf_counter() - t0) / cal.n
    n = int(min(reads.n, max(cal.n, target_s / max(per_read, 1e-9))))
    sample = reads.subset(np.arange(n))
    t0 = time.perf_counter()
    nams, offs, frac, resc = idx.map_reads(sample, opt, n_threads=cores)
    dt = time.perf_counter() - t0
    exact = None
    if gpu_result is not None:
        gn, go, gf, gr = gpu_result(n) if callable(gpu_result) else gpu_result
        exact = bool((go[: n + 1] == offs).all() and (gf[:n] == frac).all() and (gr[:n] == resc).all())
        if exact:
            k = int(offs[-1])
            exact = all((gn[f][:k] == nams[f]).all() for f in abi.NAM_COMPARED)
    return {"value": n / dt, "unit": "reads/s", "cores": cores, "kind": "port",
            "sample": f"first {n} of the {reads.n} reads, all {cores} host threads, {dt:.1f} s",
            "index_build_s": build_s, "index": how}, exact


# Child process of the reference arm: the workload's reads as a case file of the
# reference driver and the index as a .sti file (written by the oracle: the reference's
# populate is commented out, so the reference only reads indexes).  Run apart so that
# the arm's own process loads neither the data generator nor the oracle.
_REF_PREP = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import bench
from oracle import oracle_py
out, config, scale = sys.argv[2], sys.argv[3], float(sys.argv[4])
g, reads, _, gp, rp = bench.workload(scale, 0, config)
p = oracle_py.params_from_read_length(150)
oracle_py.Index.build(p, g).write_sti(out + "/index.sti")
with open(out + "/case.bin", "wb") as f:
    np.array([150, 2], np.int32).tofile(f)
    np.array([reads.n], np.uint32).tofile(f)
    reads.lengths.astype(np.uint32).tofile(f)
    reads.seq.tofile(f)
json.dump({"genome_bp": int(gp.total_len), "contigs": int(gp.n_contigs), "reads": int(reads.n),
           "len_min": int(rp.len_min), "len_max": int(rp.len_max), "paired": float(rp.paired_frac)},
          open(out + "/meta.json", "w"))
"""


def _ref_config(meta, args):
    class _P:
        pass

    gp, rp = _P(), _P()
    gp.total_len, gp.n_contigs = meta["genome_bp"], meta["contigs"]
    rp.len_min, rp.len_max, rp.paired_frac = meta["len_min"], meta["len_max"], meta["paired"]

    class _R:
        n = meta["reads"]

    return config_of(gp, rp, _R, args)


def run_reference(args):
    """--impl reference: the reference's own CPU path (query randstrobes with its
    SyncmerIterator / RandstrobeIterator, find_nams, find_nams_rescue; oracle/_ref/
    ref_driver built from its sources, oracle/build_ref.sh) on all host cores, timed over
    a bounded sample of the workload's reads; the CPU restatement when the reference's
    sources are not at hand."""
    import shutil
    import tempfile

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import __graft_entry__

    __graft_entry__.build()
    ref = os.path.join(HERE, "oracle", "_ref", "ref_driver")
    if not os.path.exists(ref):
        return run_reference_port(args, "reference sources not staged on this host (oracle/stage_ref.sh)")
    tmp = tempfile.mkdtemp(prefix="gbsa_ref_")
    try:
        subprocess.run([sys.executable, "-c", _REF_PREP, HERE, tmp, args.config, str(args.scale)], check=True)
        meta = json.load(open(os.path.join(tmp, "meta.json")))
        cores = os.cpu_count() or 1
        case, sti = os.path.join(tmp, "case.bin"), os.path.join(tmp, "index.sti")

        def drive(reps, max_reads):
            r = subprocess.run([ref, "time", case, sti, str(cores), str(reps), str(max_reads)], check=True,
                               stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            return json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])

        cal = drive(1, 20000)
        per_read = cal["seconds"] / max(1, cal["reads"])
        step_budget = max(1.0, 60.0 / max(1, args.steps + args.warmup))
        n = int(min(meta["reads"], max(1000, step_budget / max(per_read, 1e-9))))
        res = drive(args.warmup + args.steps, n)
        times = res["rep_seconds"][args.warmup:] or res["rep_seconds"]
        dt = sum(times) / len(times)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    v = n / dt
    sample = (f"first {n} of {meta['reads']} reads per step, {cores} host threads (reads 256 at a time), "
              f"mean of {len(times)} steps after {args.warmup} warm-up")
    line = {
        "impl": "reference", "metric": "reads/s seed+lookup+NAM", "value": v, "unit": "reads/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": _ref_config(meta, args),
        "cpu_baseline": {"value": v, "unit": "reads/s", "cores": cores, "kind": "reference", "sample": sample,
                         "code": "the reference's SyncmerIterator, RandstrobeIterator, StrobemerIndex::read/find, "
                                 "find_nams, find_nams_rescue (step2/), built from its own sources by "
                                 "oracle/build_ref.sh; index written by the oracle (.sti v2)"},
        "e2e": {"value": v, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_reference_port(args, why):
    """The CPU restatement of the reference path on the host cores (the reference's own
    sources are not at hand on this host)."""
    from gpu_index_test_gb300 import abi
    from oracle import oracle_py

    g, reads, _, gp, rp = workload(args.scale, 0, args.config)
    p = oracle_py.params_from_read_length(150)
    idx = oracle_py.Index.build(p, g)
    cores = os.cpu_count() or 1
    opt = abi.map_options()
    cal = reads.subset(np.arange(min(reads.n, 20000)))
    t0 = time.perf_counter()
    idx.map_reads(cal, opt, n_threads=cores)
    per_read = (time.perf_counter() - t0) / cal.n
    step_budget = max(1.0, 60.0 / max(1, args.steps + args.warmup))
    n = int(min(reads.n, max(1000, step_budget / max(per_read, 1e-9))))
    sample = reads.subset(np.arange(n))
    for _ in range(args.warmup):
        idx.map_reads(sample, opt, n_threads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        idx.map_reads(sample, opt, n_threads=cores)
    dt = (time.perf_counter() - t0) / args.steps
    v = n / dt
    line = {
        "impl": "reference", "metric": "reads/s seed+lookup+NAM", "value": v, "unit": "reads/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": config_of(gp, rp, reads, args),
        "cpu_baseline": {"value": v, "unit": "reads/s", "cores": cores, "kind": "port",
                         "sample": f"first {n} of {reads.n} reads per step, {cores} host threads",
                         "why_port": why},
        "e2e": {"value": v, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def batched_measure(idx, reads, items, d_seq, d_off, d_len, plain_out, plain_ms, plain_e2e_s, steps, small=10_000):
    """The batched form beside the plain one on the same reads: device reads/s (the
    graph per batch, inputs in HBM), e2e reads/s (host entry point, pinned buffers,
    copies inside the timing), per-batch latency for small batches of `small` reads
    (plain device entry point against the batched one), and a byte compare of the
    batched form's NAMs, offsets, fractions and rescue flags with the plain form's."""
    import torch
    from gpu_index_test_gb300 import abi, native

    dev = d_seq.device
    stream = torch.cuda.current_stream(dev)
    n = reads.n
    cap = 30 * n
    b = native.Batcher(idx, max_reads=n, max_bases=int(reads.lengths.sum()))
    cfg = b.config().as_dict()
    tuned = native.batch_config_default()[1]
    d_items = torch.from_numpy(items.view(np.int32)).to(dev)
    n_items = len(items) - 1
    d_nams = torch.empty(cap * 44, dtype=torch.uint8, device=dev)
    d_noff = torch.empty(n + 1, dtype=torch.int64, device=dev)
    d_frac = torch.empty(n, dtype=torch.float32, device=dev)
    d_resc = torch.empty(n, dtype=torch.uint8, device=dev)

    def step(k=n, k_items=n_items):
        return b.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), k, d_nams.data_ptr(), cap,
                                  d_noff.data_ptr(), d_frac.data_ptr(), d_resc.data_ptr(), d_items.data_ptr(), k_items,
                                  stream.cuda_stream)

    for _ in range(3):
        tot = step()
    torch.cuda.synchronize()
    p_nams, p_noff, p_frac, p_resc, p_tot = plain_out
    exact = bool(tot == p_tot and torch.equal(d_nams[: tot * 44], p_nams[: tot * 44]) and torch.equal(d_noff, p_noff)
                 and torch.equal(d_frac, p_frac) and torch.equal(d_resc, p_resc))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # stage times inside the batch graph (events as graph nodes; one batch after the timing)
    b.set_profile(True)
    step()
    step()
    torch.cuda.synchronize()
    stage = {k: round(v, 3) for k, v in b.stage_ms().items()}
    b.set_profile(False)
    # small batches: before the e2e calls, whose chunks take more sets of the batcher's work
    # areas (for 10M reads most of the device)
    # the first `small` reads (whole items) through both device entry points
    k_items = int(np.searchsorted(items, small, side="right")) - 1
    k = int(items[k_items])
    pm = native.Mapper(idx, max_reads=k, max_bases=int(reads.lengths[:k].sum()))

    def small_plain():
        return pm.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), k, d_nams.data_ptr(), cap,
                                   d_noff.data_ptr(), d_frac.data_ptr(), d_resc.data_ptr(), stream.cuda_stream)

    lat = {}
    for name, fn in (("plain", small_plain), ("batched", lambda: step(k, k_items))):
        for _ in range(5):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(50):
            fn()
        torch.cuda.synchronize()
        lat[name] = (time.perf_counter() - t0) / 50
    pm.free()
    # e2e: host entry point, pinned reads in, NAMs / offsets / fractions / flags out
    h_seq = torch.from_numpy(reads.seq).pin_memory()
    h_nams = torch.empty(cap * 44, dtype=torch.uint8).pin_memory()
    h_noff = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    h_frac = torch.empty(n, dtype=torch.float32).pin_memory()
    h_resc = torch.empty(n, dtype=torch.uint8).pin_memory()
    L = native.lib()

    def e2e():
        rc = L.gbsa_batcher_map(b.h, h_seq.data_ptr(), reads.offsets.ctypes.data, reads.lengths.ctypes.data, n,
                                items.ctypes.data, n_items, h_nams.data_ptr(), cap, h_noff.data_ptr(),
                                h_frac.data_ptr(), h_resc.data_ptr())
        if rc != 0:
            raise RuntimeError(f"gbsa_batcher_map failed: {rc}")

    e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        e2e()
    e2e_s = (time.perf_counter() - t0) / steps
    e2e_exact = bool(int(h_noff[n]) == p_tot and torch.equal(h_noff, p_noff.cpu())
                     and torch.equal(h_nams[: p_tot * 44], p_nams[: p_tot * 44].cpu()))
    stats = b.stats()
    b.free()
    return {
        "form": "one CUDA graph per batch; seeding + lookup one persistent kernel pulling work items (read pairs) "
                "from a device queue; NAM phase kernels in the same graph",
        "config": cfg, "config_source": "tuned.json (autotuner)" if tuned else "built-in",
        "device_reads_per_s": round(n / (ms / 1e3), 1), "ms_per_batch": round(ms, 3),
        "vs_plain_device": round(plain_ms / ms, 3), "stage_ms": stage,
        "e2e_reads_per_s": round(n / e2e_s, 1), "vs_plain_e2e": round(plain_e2e_s / e2e_s, 3),
        "small_batches": {"reads": k, "plain_ms": round(lat["plain"] * 1e3, 3),
                          "batched_ms": round(lat["batched"] * 1e3, 3),
                          "plain_reads_per_s": round(k / lat["plain"], 1),
                          "batched_reads_per_s": round(k / lat["batched"], 1),
                          "vs_plain": round(lat["plain"] / lat["batched"], 3),
                          "timing": "host wall clock per call (each call returns after its batch ends), 50 calls"},
        "bit_exact_vs_plain": exact, "e2e_bit_exact_vs_plain": e2e_exact, "graph": stats,
    }


def other_config(name, scale, cpu_seconds, steps=3, serve=None):
    """Device throughput and parity of another configuration: its genome and reads, the
    GPU index, one warm-up and `steps` timed device batches (CUDA events), then the
    oracle on a bounded sample of the same reads compared with the GPU's NAMs, offsets,
    fractions and rescue flags (for a genome above HOST_BUILD_MAX_BP the oracle uses the
    GPU's index after checking it without a host build)."""
    import torch
    from gpu_index_test_gb300 import abi, native, synth

    g, reads, gen_s, gp, rp = workload(scale, 0, name)
    p = native.params_from_read_length(150)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    idx = native.Index.build(p, g)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    info = idx.info()
    n = reads.n
    m = native.Mapper(idx, abi.map_options(), max_reads=n, max_bases=int(reads.lengths.sum()))
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    d_seq = torch.from_numpy(reads.seq).to(dev)
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).to(dev)
    d_len = torch.from_numpy(reads.lengths.view(np.int32)).to(dev)
    cap = 30 * n
    d_nams = torch.empty(cap * 44, dtype=torch.uint8, device=dev)
    d_noff = torch.empty(n + 1, dtype=torch.int64, device=dev)
    d_frac = torch.empty(n, dtype=torch.float32, device=dev)
    d_resc = torch.empty(n, dtype=torch.uint8, device=dev)

    def step():
        return m.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n, d_nams.data_ptr(), cap,
                                  d_noff.data_ptr(), d_frac.data_ptr(), d_resc.data_ptr(), stream.cuda_stream)

    step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        total = step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    fused = bool(m.fused_lookup())
    # the lookup against the HBM and gather ceilings, as for the headline line: the
    # counting instance's bytes and sectors, the stage times of one profiled batch and
    # the gather ceiling of this index's own tables
    try:
        m.set_count_bytes(True)
        step()
        c_alg, c_sec = m.last_alg_bytes(), m.last_alg_sectors()
        m.set_count_bytes(False)
        m.set_profile(True)
        step()
        c_stages = m.stage_ms()
        m.set_profile(False)
        _, _, c_gbs = native.bench_gather_index(idx)
        c_packed = int(((reads.lengths.astype(np.int64) + 3) // 4).sum())
        roof = lookup_roofline(c_alg, c_sec, c_packed, int(total), c_stages, fused, ms, c_gbs)
        roof["traffic"] = ncu_traffic(name).get(roof["kernel"]) if scale == 1.0 else None
        roof["stage_ms_all"] = {k: round(v, 3) for k, v in c_stages.items()}
    except Exception as e:   # recorded, not fatal
        roof = {"error": f"{type(e).__name__}: {e}"}
    noff = d_noff.cpu().numpy().view(np.uint64)
    # the batched form on the same reads (work items: single-end reads and pairs)
    items = synth.read_items(rp)
    d_items = torch.from_numpy(items.view(np.int32)).to(dev)
    b = native.Batcher(idx, max_reads=n, max_bases=int(reads.lengths.sum()))
    b_nams = torch.empty(cap * 44, dtype=torch.uint8, device=dev)
    b_noff = torch.empty(n + 1, dtype=torch.int64, device=dev)
    b_frac = torch.empty(n, dtype=torch.float32, device=dev)
    b_resc = torch.empty(n, dtype=torch.uint8, device=dev)

    def bstep():
        return b.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n, b_nams.data_ptr(), cap,
                                  b_noff.data_ptr(), b_frac.data_ptr(), b_resc.data_ptr(), d_items.data_ptr(),
                                  len(items) - 1, stream.cuda_stream)

    bstep()
    bstep()
    e0.record(stream)
    for _ in range(steps):
        btot = bstep()
    e1.record(stream)
    torch.cuda.synchronize()
    bms = e0.elapsed_time(e1) / steps
    b_exact = bool(btot == total and torch.equal(b_nams[: total * 44], d_nams[: total * 44])
                   and torch.equal(b_noff, d_noff) and torch.equal(b_frac, d_frac) and torch.equal(b_resc, d_resc))
    b.free()
    del b_nams, b_noff, b_frac, b_resc, d_items

    def first(k):
        t = int(noff[k])
        return (d_nams[: t * 44].cpu().numpy().view(abi.NAM), noff[: k + 1], d_frac[:k].cpu().numpy(),
                d_resc[:k].cpu().numpy())

    m.free()
    served = None
    if serve:
        # the served form on this index (resident), before the oracle's check
        served = serve_measure(idx, g, serve[0], serve[1], scale, WORKLOADS[name].split(":")[0] + " index, resident")
    cpu, exact = cpu_baseline(g, reads, cpu_seconds, first, gpu_index=idx)
    idx.free()
    del d_nams, d_seq, d_off, d_len, d_noff, d_frac, d_resc
    torch.cuda.empty_cache()
    return {"workload": WORKLOADS[name], "genome_bp": int(gp.total_len), "reads_per_batch": int(n),
            "index_entries": int(info.size), "index_bits": int(info.bits), "index_build_gpu_s": round(build_s, 3),
            "form": "seeding and lookup fused" if fused else "seeding and lookup as two kernels (index over 2 GiB)",
            "device_reads_per_s": round(n / (ms / 1e3), 1), "ms_per_batch": round(ms, 3), "nams": int(total),
            "roofline": roof,
            "batched": {"device_reads_per_s": round(n / (bms / 1e3), 1), "ms_per_batch": round(bms, 3),
                        "vs_plain_device": round(ms / bms, 3), "work_items": int(len(items) - 1),
                        "bit_exact_vs_plain": b_exact},
            "cpu_baseline": cpu, "bit_exact_vs_cpu_sample": exact}, served


# the served form runs on the human-scale index (resident in HBM) when it is built
SERVE_CONFIG = "C4"

WORKLOADS = {
    "C1": "C1 plain small: synthetic 5 Mbp single contig, 100k single-end 150 bp reads",
    "C2": "C2 repeat-rich mid-size: synthetic 100 Mbp / 20 contigs (5% segmental duplications, STRs), "
          "1M paired-end 2x150 bp pairs = 2M reads per step",
    "C3": "C3 uneven lengths: the C1 genome, ~2M reads of 50-500 bp (log-uniform), half single-end, half paired",
    "C4": "C4 human-scale: synthetic 3.1 Gbp / 24 contigs (~45% repeat families, duplications, STRs), "
          "5M paired-end 2x150 bp pairs = 10M reads per step",
}


def config_of(gp, rp, reads, args):
    return {
        "workload": WORKLOADS[args.config],
        "genome_bp": gp.total_len, "contigs": gp.n_contigs, "reads_per_step": reads.n,
        "read_len": rp.len_min if rp.len_min == rp.len_max else f"{rp.len_min}-{rp.len_max}",
        "paired": rp.paired_frac, "params": "from_read_length(150): k=20 s=16 l=1 u=7 q=255 max_dist=80",
        "rescue": "R=2, rescue_cutoff=2*filter_cutoff, count cap 1000", "nam_order": "score",
        "l2": "reads and index sizes as listed; no L2 flush between steps (C2, C4: inputs larger than L2)",
        "scale": args.scale,
    }


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import __graft_entry__

    __graft_entry__.build()
    from gpu_index_test_gb300 import abi, native, synth

    g, reads, gen_s, gp, rp = workload(args.scale, rank, args.config)
    p = native.params_from_read_length(150)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    idx = native.Index.build(p, g)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    info = idx.info()
    n = reads.n
    m = native.Mapper(idx, abi.map_options(), max_reads=n, max_bases=int(reads.lengths.sum()))
    l2_window_bytes = m.set_l2_window(args.l2_window)

    dev = torch.device("cuda", local)
    d_seq = torch.from_numpy(reads.seq).to(dev)
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).to(dev)
    d_len = torch.from_numpy(reads.lengths.view(np.int32)).to(dev)
    cap = 30 * n
    d_nams = torch.empty(cap * 44, dtype=torch.uint8, device=dev)
    d_noff = torch.empty(n + 1, dtype=torch.int64, device=dev)
    d_frac = torch.empty(n, dtype=torch.float32, device=dev)
    d_resc = torch.empty(n, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        tot = m.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n, d_nams.data_ptr(), cap,
                                 d_noff.data_ptr(), d_frac.data_ptr(), d_resc.data_ptr(), stream.cuda_stream)
        if tot > cap:
            raise RuntimeError("NAM capacity too small")
        return tot

    # random-gather peaks: a buffer the size of the index (larger than L2, within the
    # GPU's TLB reach like the index) and one that fits L2
    gather_peaks = (native.bench_gather(512 << 20)[1], native.bench_gather(16 << 20)[1]) if rank == 0 else (0.0, 0.0)
    gather_index = native.bench_gather_index(idx) if rank == 0 else (0.0, 0.0, 0.0)

    # warm-up (first one also counts algorithmic bytes of the lookup stage)
    m.set_count_bytes(True)
    total_nams = step()
    alg_lookup = m.last_alg_bytes()
    sectors_lookup = m.last_alg_sectors()
    counts = m.last_counts()
    m.set_count_bytes(False)
    for _ in range(max(0, args.warmup - 1)):
        step()
    torch.cuda.synchronize()

    # timed region
    m.set_profile(True)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = native.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    stage_acc = {}
    ev0.record(stream)
    for _ in range(args.steps):
        step()
        for k, v in m.stage_ms().items():
            stage_acc[k] = stage_acc.get(k, 0.0) + v
    ev1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches = native.launch_count() - l0
    clocks = sampler.stop()
    resc, n_block_sorted = m.rescue_cycles()
    nam_cyc = m.nam_cycles()
    m.set_profile(False)
    mhz = clocks.get("sm_mhz") or 2000.0

    def dist(a, div=1.0):
        """p50 / p99 / max / sum of a per-read quantity (cycles / div = microseconds)."""
        if not len(a):
            return None
        v = np.sort(a.astype(np.float64)) / div
        return {"n": int(len(v)), "p50": round(float(v[len(v) // 2]), 1),
                "p99": round(float(v[int(len(v) * 0.99)]), 1), "max": round(float(v[-1]), 1),
                "sum": round(float(v.sum()), 1)}

    rescue_profile = None
    if len(resc):
        worst = resc[np.argsort(resc[:, 0] + resc[:, 3])[-3:]]
        rescue_profile = {
            "total_us": dist(resc[:, 0], mhz), "plan_us": dist(resc[:, 1], mhz),
            "merge_us": dist(resc[:, 2], mhz), "sort_us": dist(resc[:, 3], mhz),
            "hit_bound": dist(resc[:, 4]), "nams": dist(resc[:, 5]), "walk_us": dist(resc[:, 6], mhz),
            "max_run": dist(resc[:, 7]), "block_sorted_reads": n_block_sorted,
            "block_sort_small_us": dist(resc[(resc[:, 5] > 256) & (resc[:, 5] <= 2048), 3], mhz),
            "block_sort_large_us": dist(resc[resc[:, 5] > 2048, 3], mhz),
            "worst": worst.tolist(),
        }
    # the next stage after the NAM sort: read-pair types (gpu_pre_cal_type) of the
    # last batch's pairs (mates are interleaved), timed alone on the same stream
    pair_types = None
    if rank == 0 and n >= 2:
        d_types = torch.empty(n // 2, dtype=torch.uint8, device=dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        classify = lambda: native.classify_pairs_device(d_nams.data_ptr(), d_noff.data_ptr(), n // 2,
                                                          d_types.data_ptr(), 0, 0.5, 300.0, 100.0,
                                                          stream.cuda_stream)
        classify()
        e0.record(stream)
        for _ in range(5):
            classify()
        e1.record(stream)
        torch.cuda.synchronize()
        pair_types = {"ms": round(e0.elapsed_time(e1) / 5, 4),
                      "counts": np.bincount(d_types.cpu().numpy(), minlength=5).tolist()}
    # the first alignment step: seed extension (reverse_nam_if_needed + extend_seed_part)
    # of each read's best NAM of the last batch, timed alone on the same stream
    seed_ext, ext_in = None, None
    if rank == 0 and total_nams > 0:
        noff = d_noff.cpu().numpy()
        cnt = np.diff(noff)
        owners = np.nonzero(cnt > 0)[0].astype(np.uint32)
        d_sel = torch.from_numpy(noff[:-1][cnt > 0].astype(np.int64)).to(dev)
        d_best = d_nams[: int(noff[-1]) * 44].view(-1, 44).index_select(0, d_sel).contiguous()
        d_own = torch.from_numpy(owners.view(np.int32)).to(dev)
        d_ref = torch.from_numpy(g.seq).to(dev)
        d_roff = torch.from_numpy(g.offsets.astype(np.uint64).view(np.int64)).to(dev)
        d_rlen = torch.from_numpy(g.lengths.astype(np.uint64).view(np.int64)).to(dev)
        n_ext = len(owners)
        d_ext = torch.empty(n_ext * abi.SEED_ALIGNMENT.itemsize, dtype=torch.uint8, device=dev)
        extend = lambda: native.extend_seeds_device(d_ref.data_ptr(), d_roff.data_ptr(), d_rlen.data_ptr(),
                                                    len(g.lengths), d_seq.data_ptr(), d_off.data_ptr(),
                                                    d_len.data_ptr(), n, d_best.data_ptr(), d_own.data_ptr(), n_ext,
                                                    p.k, d_ext.data_ptr(), stream=stream.cuda_stream)
        extend()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            extend()
        e1.record(stream)
        torch.cuda.synchronize()
        ms_ext = e0.elapsed_time(e1) / 5
        ext = d_ext.cpu().numpy().view(abi.SEED_ALIGNMENT)
        # algorithmic bytes per NAM: the read and its projected reference window (L bytes
        # each), the NAM (44 B), its read index (4 B) and the record out (36 B)
        alg = int((2 * reads.lengths[owners].astype(np.int64) + 84).sum())
        ext_peak, ext_peak_src = peaks()
        achieved = alg / (ms_ext * 1e-3) / 1e9
        seed_ext = {"nams": int(n_ext), "ms": round(ms_ext, 4), "nams_per_s": round(n_ext / (ms_ext * 1e-3), 1),
                    "aligned_ungapped_frac": round(float(ext["done"].mean()), 4),
                    "consistent_frac": round(float(ext["consistent"].mean()), 4),
                    "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": round(ext_peak, 1),
                                 "unit": "GB/s", "frac": round(achieved / ext_peak, 4), "peak_source": ext_peak_src,
                                 "alg_bytes_per_launch": alg},
                    "timing": "each call: the kernel and its 4-byte status read, 5 calls after one warm-up"}
        # mate rescue: each read's mate (mates are interleaved) from the read's best NAM
        mates = (owners ^ 1).astype(np.uint32)
        d_mates = torch.from_numpy(mates.view(np.int32)).to(dev)
        d_resc_out = torch.empty(n_ext * abi.MATE_RESCUE.itemsize, dtype=torch.uint8, device=dev)
        rescue = lambda: native.rescue_mates_device(d_ref.data_ptr(), d_roff.data_ptr(), d_rlen.data_ptr(),
                                                    len(g.lengths), d_seq.data_ptr(), d_off.data_ptr(),
                                                    d_len.data_ptr(), n, d_best.data_ptr(), d_mates.data_ptr(),
                                                    n_ext, p.k, d_resc_out.data_ptr(), stream=stream.cuda_stream)
        rescue()
        e0.record(stream)
        for _ in range(5):
            rescue()
        e1.record(stream)
        torch.cuda.synchronize()
        ms_resc = e0.elapsed_time(e1) / 5
        mres = d_resc_out.cpu().numpy().view(abi.MATE_RESCUE)
        seed_ext["mate_rescue"] = {"nams": int(n_ext), "ms": round(ms_resc, 4),
                                   "nams_per_s": round(n_ext / (ms_resc * 1e-3), 1),
                                   "mate_unaligned_frac": round(float(mres["is_unaligned"].mean()), 4)}
        ext_in = (d_best.cpu().numpy().view(abi.NAM).reshape(-1), owners, ext, mates, mres)
    nam_profile = None
    if len(nam_cyc):
        worst = nam_cyc[np.argsort(nam_cyc[:, 0])[-3:]]
        nam_profile = {"total_us": dist(nam_cyc[:, 0], mhz), "merge_us": dist(nam_cyc[:, 3], mhz),
                       "hits": dist(nam_cyc[:, 1]), "nams": dist(nam_cyc[:, 2]),
                       "worst_cycles_hits_nams": worst[:, :3].tolist()}
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, world, dev)
    value = job_throughput(n, world, ms / 1e3)

    # device results of the last step, for the parity check in the CPU-baseline leg
    gpu_res = None
    if rank == 0 and not args.no_cpu_baseline:
        k = total_nams
        raw = d_nams[: k * 44].cpu().numpy()
        gpu_res = (raw.view(abi.NAM), d_noff.cpu().numpy().view(np.uint64), d_frac.cpu().numpy(),
                   d_resc.cpu().numpy())

    # end-to-end through the host entry point: pinned host reads in, results out
    h_seq = torch.from_numpy(reads.seq).pin_memory()
    h_nams = torch.empty(cap * 44, dtype=torch.uint8).pin_memory()
    h_noff = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    h_frac = torch.empty(n, dtype=torch.float32).pin_memory()
    h_resc = torch.empty(n, dtype=torch.uint8).pin_memory()
    offs_np = reads.offsets
    lens_np = reads.lengths
    L = native.lib()

    def e2e_step():
        rc = L.gbsa_map_reads(m.h, h_seq.data_ptr(), offs_np.ctypes.data, lens_np.ctypes.data, n, h_nams.data_ptr(),
                              cap, h_noff.data_ptr(), h_frac.data_ptr(), h_resc.data_ptr())
        if rc != 0:
            raise RuntimeError(f"gbsa_map_reads failed: {rc}")

    e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world, dev)
    tot_nams_e2e = int(h_noff[n].item())
    h2d = int(reads.seq.nbytes) + 12 * n
    d2h = 44 * tot_nams_e2e + 8 * (n + 1) + 4 * n + n

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # roofline of the dominant kernel on the critical path (the rescue chain runs on a
    # second stream beside the NAM kernels; its stage times include that overlap)
    stage_ms = {k: v / args.steps for k, v in stage_acc.items()}
    fused = m.fused_lookup()
    main_stages = ("seed_lookup", "lookup_long", "nams", "nams_warp") if fused else ("seed", "lookup", "nams", "nams_warp")
    dom = max(main_stages, key=lambda k: stage_ms.get(k, 0.0))
    # NAMs the step outputs (the NAM-state arena's slots, counts["nam_slots"], include the
    # room the lane merge reserves: two per hit)
    q, hits, nams_n = counts["queries"], counts["hits"], int(total_nams)
    packed = int(((reads.lengths.astype(np.int64) + 3) // 4).sum())
    # Algorithmic bytes as the measurement plan defines them per read: the 2-bit packed
    # read (ceil(L/4) B), the lookup's probes (bucket bound pair, entries examined,
    # filter probe, run walk; counted live by the kernel's counting instance) and 44 B
    # per output NAM.  Seeding + lookup carry the first two, the NAM stages the third.
    alg = {
        "seed_lookup": packed + alg_lookup, "lookup_long": 0,   # one kernel (indexes up to 2 GiB)
        "seed": packed, "lookup": alg_lookup,                   # two kernels (larger indexes)
        "seed_long": 0,
        "nams": 44 * nams_n, "nams_warp": 0, "rescue": 0, "rescue_sort": 0,
    }
    # Bytes the kernels pass between their own phases through HBM / L2 (not algorithmic):
    # query records written and read back, index positions, per-query hit counts and
    # offsets, hit records written (seeding + lookup) and read (NAM stages), NAM states
    # written unsorted and sorted.
    inter = {
        "seed_lookup": 16 * q + 16 * q + 8 * q + 8 * q + 16 * hits,
        "seed": 16 * q, "lookup": 16 * q + 8 * q + 8 * q + 16 * hits,
        "nams": 16 * hits + 64 * nams_n,
    }
    peak, peak_kind = peaks()
    achieved = alg[dom] / (stage_ms[dom] / 1e3) / 1e9 if stage_ms[dom] > 0 else 0.0
    # the ncu figures are per launch of the full-size workload
    tr = ncu_traffic(args.config).get(dom) if args.scale == 1.0 else None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "traffic": tr, "alg_bytes_per_launch": alg[dom],
                "alg_bytes_terms": ({"packed_reads": packed, "lookup_probes": int(alg_lookup)}
                                    if dom in ("seed_lookup", "seed", "lookup") else {"nams_44B": 44 * nams_n}),
                "intermediate_bytes_per_launch": inter.get(dom),
                "stage_ms": {k: round(v, 3) for k, v in stage_ms.items()}}
    step_alg = packed + alg_lookup + 44 * nams_n
    roofline["whole_step"] = {"alg_bytes": int(step_alg), "ms": round(ms, 3),
                              "achieved": round(step_alg / (ms / 1e3) / 1e9, 1),
                              "frac": round(step_alg / (ms / 1e3) / 1e9 / peak, 4)}
    # the lookup against the achievable random-gather bandwidth of its own footprint:
    # the dependent bucket-pair -> first-entry gather on this index's buffers, measured
    # before the timed region (sector form: 32 B per distinct sector the reference's
    # probes touch); inside the fused kernel the rate is taken over the whole kernel
    # (seeding included), a lower bound for the gathers
    lk_stage = "seed_lookup" if fused else "lookup"
    lk_s = stage_ms.get(lk_stage, 0.0) / 1e3
    g_probes, g_sectors, g_gbs = gather_index
    gather_hbm, gather_l2 = gather_peaks
    lk_gbs = sectors_lookup * 32 / lk_s / 1e9 if lk_s > 0 else 0.0
    roofline["gather"] = {
        "kernel": lk_stage, "sectors_per_launch": int(sectors_lookup), "achieved": round(lk_gbs, 1), "unit": "GB/s",
        "peak": round(g_gbs, 1), "frac": round(lk_gbs / g_gbs, 4) if g_gbs > 0 else None,
        "peak_source": "gbsa_bench_gather_index: uniform random keys, bucket bound pair then the bucket's first "
                       "entry (dependent) on this index's own tables, 8 probes in flight per thread",
        "peak_probes_per_s": round(g_probes, 1),
        "flat_buffer_gather_gbs": {"512MB": round(gather_hbm, 1), "16MB": round(gather_l2, 1)},
    }

    batched = None
    staging_wanted = world == 1 and args.fastq and args.config == "C2"
    if not staging_wanted:
        # nothing below maps through the plain mapper: its work areas (two sets after the
        # chunked e2e calls; about 240 GB for the 10M reads of C4) make room for the batched form's
        m.free()
    if rank == 0:
        items = synth.read_items(rp)
        tot_plain = int(d_noff[n].item())
        batched = batched_measure(idx, reads, items, d_seq, d_off, d_len, (d_nams, d_noff, d_frac, d_resc, tot_plain),
                                  ms, e2e_s, max(3, args.steps))
        if batched is not None and fused and batched.get("stage_ms"):
            # the same reads and index as the plain line: the same algorithmic bytes and
            # sectors, over the persistent queue kernel's stage time
            batched["roofline"] = lookup_roofline(alg_lookup, sectors_lookup, packed, nams_n, batched["stage_ms"],
                                                  True, batched["ms_per_batch"], g_gbs)
            batched["roofline"]["kernel"] = "seed_lookup (persistent work-queue kernel)"

    staging = None
    if staging_wanted:
        staging = fastq_pipeline(m, reads, h_nams[: tot_nams_e2e * 44].numpy().view(abi.NAM),
                                 h_noff.numpy().view(np.uint64))

    served = None
    rates = [float(x) for x in args.serve_rates.split(",") if x.strip()]
    other_names = [x.strip() for x in args.other_configs.split(",") if x.strip()]
    if rates and world == 1 and (SERVE_CONFIG not in other_names or args.no_cpu_baseline):
        # the served form on this configuration's index when the human-scale one is not built
        served = serve_measure(idx, g, rates, args.serve_seconds, args.scale,
                               WORKLOADS[args.config].split(":")[0] + " index, resident")

    cpu = None
    exact = None
    if not args.no_cpu_baseline:
        cpu, exact = cpu_baseline(g, reads, args.cpu_seconds, gpu_res)
        if seed_ext is not None:
            # the oracle on the first NAMs (one host thread), checked against the GPU records
            from oracle import oracle_py
            nb, ob, eb, mb, rb = ext_in
            n_cpu = min(len(nb), 400000)
            t0 = time.perf_counter()
            ref_ext = oracle_py.extend_seeds(g.seq, g.offsets, g.lengths, reads.seq, reads.offsets, reads.lengths,
                                             nb[:n_cpu], ob[:n_cpu], p.k)
            cpu_s = time.perf_counter() - t0
            seed_ext["cpu_baseline"] = {"value": round(n_cpu / cpu_s, 1), "unit": "NAMs/s", "cores": 1,
                                        "kind": "port", "sample": f"the first {n_cpu} NAMs"}
            seed_ext["bit_exact_vs_cpu_sample"] = bool((ref_ext == eb[:n_cpu]).all())
            n_cpu = min(len(nb), 100000)
            t0 = time.perf_counter()
            ref_resc = oracle_py.rescue_mates(g.seq, g.offsets, g.lengths, reads.seq, reads.offsets, reads.lengths,
                                              nb[:n_cpu], mb[:n_cpu], p.k)
            cpu_s = time.perf_counter() - t0
            seed_ext["mate_rescue"]["cpu_baseline"] = {"value": round(n_cpu / cpu_s, 1), "unit": "NAMs/s",
                                                       "cores": 1, "kind": "port",
                                                       "sample": f"the first {n_cpu} NAMs"}
            seed_ext["mate_rescue"]["bit_exact_vs_cpu_sample"] = bool((ref_resc == rb[:n_cpu]).all())

    others = None
    names = [x.strip() for x in args.other_configs.split(",") if x.strip() and x.strip() != args.config]
    if names and world == 1 and not args.no_cpu_baseline:
        others = {}
        for nm in names:
            try:
                sv = (rates, args.serve_seconds) if rates and nm == SERVE_CONFIG else None
                others[nm], got = other_config(nm, args.scale, min(args.cpu_seconds, 8.0), serve=sv)
                if got is not None:
                    served = got
            except Exception as e:   # recorded, not fatal: the headline line still prints
                others[nm] = {"error": f"{type(e).__name__}: {e}"}

    line = {
        "metric": "reads/s seed+lookup+NAM", "value": round(value, 1), "unit": "reads/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": dict(config_of(gp, rp, reads, args), index_entries=int(info.size), index_bits=int(info.bits),
                       filter_cutoff=int(info.filter_cutoff), index_build_gpu_s=round(build_s, 3),
                       l2_window_bytes=int(l2_window_bytes),
                       form=("seeding and lookup fused (a warp per read)" if fused else
                             "seeding and lookup as two kernels (index over 2 GiB)")
                       + ", then NAM kernels on two streams"),
        "e2e": {"value": round(job_throughput(n, world, e2e_s), 1), "unit": "reads/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": roofline,
        "batched": batched,
        "served": served,
        "fastq_staging": staging,
        "cpu_baseline": cpu,
        "bit_exact_vs_cpu_sample": exact,
        "other_configs": others,
        "clocks": clocks,
        "gpu_launches": int(launches),
        "work": dict(counts, nams_per_step=int(total_nams), rescue_profile=rescue_profile, nam_profile=nam_profile,
                     pair_types=pair_types, seed_extension=seed_ext),
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
