"""Autotuner of the batched form's kernel shapes.

Sweeps, over the C-ABI (gbsa_batcher_*):
  seed_variant   the persistent seeding + lookup kernel's shape: warps per block (reads
                 in flight per CTA), resident blocks per SM, and the shared-memory read
                 window (longest read seeded in shared memory: 512 or 256 bases)
  lane_max_hits  the NAM merge's split between one lane per read and one warp per read
  sort_variant   the block size of the sort of rescued reads with many NAMs
  lane_variant   the lane-per-read NAM merge: open NAMs in shared memory with a
                 register budget of 96, 80 or 64, or open NAMs in registers
  warp_variant   the register budget of the warp-per-read NAM merge (96, 80 or 64) and its
                 blocks per SM (5, or 4 beside the sorts)
(the first three as a grid, then the two register budgets as a grid at the best of
the first) on the repeat-rich mid-size configuration (150 bp pairs), the uneven length configuration
(50-500 bp, single-end and pairs mixed) and a tenth of the human-scale one (repeat
families, 150 bp pairs), timing each shape's graph
launches with CUDA events and checking its output byte for byte against the plain
form's; then the host entry point's chunk size on end-to-end reads/s over the whole
mid-size configuration (100 Mbp, 1M pairs).  The fastest
shape (sum of the workloads' times relative to the best on each) is written to
tuned.json next to the library, which gbsa_batcher_create reads; the whole sweep is
written as a table to the path given by --table.

  python -m gpu_index_test_gb300.autotune [--out PATH] [--table PATH] [--scale S]

The reference fixes its launch shapes by hand (step2/main.cu:4458-4487: 32 threads per
block for seeding, 8 for the lookup).
"""
import argparse
import json
import os
import time

import numpy as np

from . import abi, native, synth
from ._build_paths import GBSA_SO

LANE_MAX_HITS = (64, 96, 128, 160)
SORT_VARIANTS = (0, 1)
REG_VARIANTS = (0, 1, 2, 3, 4)   # warp merge: 3, 4 launched four blocks per SM
LANE_VARIANTS = (0, 1, 2, 3, 4, 5, 6)   # 3-6: the open NAMs in registers
CHUNKS = (1 << 16, 1 << 17, 1 << 18, 1 << 19, 1 << 20)


def _workloads(scale):
    """(name, genome, reads, items) workloads the sweep times: the benchmark's mid-size
    and uneven-length configurations whole, and a tenth of the human-scale one (kernel
    shapes that differ by a few percent on small slices order differently at full size)."""
    out = []
    gp = synth.genome_params("C2", scale=scale, seed=201)
    g = synth.make_genome(gp)
    rp = synth.read_params("C2", n_units=max(2000, int(1_000_000 * scale)), seed=202)
    out.append(("C2: 100 Mbp repeat-rich genome, 1M pairs of 150 bp", g, synth.make_reads(g, rp), synth.read_items(rp)))
    gp = synth.genome_params("C1", scale=scale, seed=203)
    g = synth.make_genome(gp)
    rp = synth.read_params("C3", n_units=max(2000, int(1_333_333 * scale)), seed=204)
    out.append(("C3: 5 Mbp genome, 2M reads of 50-500 bp, half pairs", g, synth.make_reads(g, rp),
                synth.read_items(rp)))
    gp = synth.genome_params("C4", scale=0.1 * scale, seed=207)
    g = synth.make_genome(gp)
    rp = synth.read_params("C4", n_units=max(2000, int(1_000_000 * scale)), seed=208)
    out.append(("C4 tenth: 310 Mbp genome with 45% repeat families, 1M pairs of 150 bp", g, synth.make_reads(g, rp),
                synth.read_items(rp)))
    return out


def _device_run(torch, idx, reads, items, make, reps):
    """Times reps batches of one runner (plain or batched) on reads already in HBM;
    returns (ms per batch, outputs of the last batch as host arrays)."""
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    n = reads.n
    cap = 40 * n + 4096
    d = {
        "seq": torch.from_numpy(reads.seq).to(dev),
        "off": torch.from_numpy(reads.offsets.view(np.int64)).to(dev),
        "len": torch.from_numpy(reads.lengths.view(np.int32)).to(dev),
        "items": torch.from_numpy(items.view(np.int32)).to(dev),
        "nams": torch.zeros(cap * 44, dtype=torch.uint8, device=dev),
        "noff": torch.zeros(n + 1, dtype=torch.int64, device=dev),
        "frac": torch.zeros(n, dtype=torch.float32, device=dev),
        "resc": torch.zeros(n, dtype=torch.uint8, device=dev),
    }
    run = make(d, n, cap, stream.cuda_stream)
    for _ in range(2):
        tot = run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(reps):
        e0.record(stream)
        tot = run()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    outs = (d["nams"][: tot * 44].cpu().numpy(), d["noff"].cpu().numpy(), d["frac"].cpu().numpy(),
            d["resc"].cpu().numpy())
    return float(np.median(times)), outs


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def sweep(scale=1.0, reps=7, log=print):
    """Shapes are (seed_variant, lane_max_hits, sort_variant, lane_variant, warp_variant)."""
    grid = [(v, l, s, 0, 0) for v in range(abi.SEED_VARIANTS) for l in LANE_MAX_HITS for s in SORT_VARIANTS]
    pick, rows, exact, score, plain_ms = _sweep(grid, scale, reps, log)
    regs = [pick[:3] + (lv, wv) for lv in LANE_VARIANTS for wv in REG_VARIANTS]
    pick2, rows2, exact2, _, _ = _sweep(regs, scale, reps, log)
    rows.update(rows2)
    exact.update(exact2)
    names = list(plain_ms)
    best = {nm: min(rows[sh][nm] for sh in rows if exact[sh]) for nm in names}
    score = {sh: sum(rows[sh][nm] / best[nm] for nm in names) for sh in rows if exact[sh]}
    return min(score, key=score.get), rows, exact, score, plain_ms


def _sweep(shapes, scale, reps, log):
    import torch

    p = native.params_from_read_length(150)
    rows = {sh: {} for sh in shapes}
    exact = {sh: True for sh in shapes}
    plain_ms = {}
    for name, g, reads, items in _workloads(scale):
        idx = native.Index.build(p, g)
        m = native.Mapper(idx, max_reads=reads.n, max_bases=int(reads.lengths.sum()))

        def plain(d, n, cap, st, m=m):
            return lambda: m.map_reads_device(d["seq"].data_ptr(), d["off"].data_ptr(), d["len"].data_ptr(), n,
                                              d["nams"].data_ptr(), cap, d["noff"].data_ptr(), d["frac"].data_ptr(),
                                              d["resc"].data_ptr(), st)

        plain_ms[name], ref = _device_run(torch, idx, reads, items, plain, reps)
        m.free()
        for sh in shapes:
            cfg = abi.batch_config(sh[0], sh[1], sh[2], 1 << 19, sh[3], sh[4])
            b = native.Batcher(idx, config=cfg, max_reads=reads.n, max_bases=int(reads.lengths.sum()))

            def batched(d, n, cap, st, b=b):
                return lambda: b.map_reads_device(d["seq"].data_ptr(), d["off"].data_ptr(), d["len"].data_ptr(), n,
                                                  d["nams"].data_ptr(), cap, d["noff"].data_ptr(),
                                                  d["frac"].data_ptr(), d["resc"].data_ptr(), d["items"].data_ptr(),
                                                  len(items) - 1, st)

            ms, out = _device_run(torch, idx, reads, items, batched, reps)
            b.free()
            rows[sh][name] = ms
            exact[sh] &= _same(out, ref)
            log(f"{name[:8]} variant={sh[0]} lane_max_hits={sh[1]} sort={sh[2]} regs={sh[3]},{sh[4]}: {ms:.3f} ms "
                f"(plain {plain_ms[name]:.3f}) exact={exact[sh]}")
        idx.free()
    names = list(plain_ms)
    best = {nm: min(rows[sh][nm] for sh in shapes if exact[sh]) for nm in names}
    score = {sh: sum(rows[sh][nm] / best[nm] for nm in names) for sh in shapes if exact[sh]}
    pick = min(score, key=score.get)
    return pick, rows, exact, score, plain_ms


def tune_chunks(pick, scale=1.0, log=print):
    """End-to-end reads/s of the host entry point per chunk size, with the picked shape."""
    import torch

    p = native.params_from_read_length(150)
    # the whole mid-size configuration (100 Mbp, 1M pairs): the copies and the index's
    # cache behaviour both depend on the sizes
    g = synth.make_genome(synth.genome_params("C2", scale=scale, seed=205))
    rp = synth.read_params("C2", n_units=max(4000, int(1_000_000 * scale)), seed=206)
    reads, items = synth.make_reads(g, rp), synth.read_items(rp)
    idx = native.Index.build(p, g)
    n = reads.n
    cap = 40 * n
    h_seq = torch.from_numpy(reads.seq).pin_memory()
    h_nams = torch.empty(cap * 44, dtype=torch.uint8).pin_memory()
    h_noff = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    h_frac = torch.empty(n, dtype=torch.float32).pin_memory()
    h_resc = torch.empty(n, dtype=torch.uint8).pin_memory()
    L = native.lib()
    res = {}
    for ch in CHUNKS:
        b = native.Batcher(idx, config=abi.batch_config(pick[0], pick[1], pick[2], ch, pick[3], pick[4]),
                           max_reads=min(n, 2 * ch),
                           max_bases=int(reads.lengths.sum()))

        def run():
            rc = L.gbsa_batcher_map(b.h, h_seq.data_ptr(), reads.offsets.ctypes.data, reads.lengths.ctypes.data, n,
                                    items.ctypes.data, len(items) - 1, h_nams.data_ptr(), cap, h_noff.data_ptr(),
                                    h_frac.data_ptr(), h_resc.data_ptr())
            assert rc == 0, rc

        run()
        run()
        t0 = time.perf_counter()
        for _ in range(3):
            run()
        res[ch] = n / ((time.perf_counter() - t0) / 3)
        b.free()
        log(f"chunk_reads={ch}: {res[ch] / 1e6:.1f} M reads/s e2e")
    idx.free()
    return max(res, key=res.get), res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(os.path.dirname(GBSA_SO), "tuned.json"))
    ap.add_argument("--table", default=None, help="write the sweep as a markdown table here")
    ap.add_argument("--scale", type=float, default=1.0)
    args = ap.parse_args()
    import torch

    t0 = time.time()
    pick, rows, exact, score, plain_ms = sweep(args.scale)
    chunk, chunk_rates = tune_chunks(pick, args.scale)
    cfg = {"seed_variant": pick[0], "lane_max_hits": pick[1], "sort_variant": pick[2], "chunk_reads": chunk,
           "lane_variant": pick[3], "warp_variant": pick[4], "device": torch.cuda.get_device_name(0),
           "tuned_s": round(time.time() - t0, 1)}
    with open(args.out, "w") as f:
        json.dump(cfg, f, indent=1)
        f.write("\n")
    print(json.dumps(cfg))
    if args.table:
        names = list(plain_ms)
        with open(args.table, "w") as f:
            f.write("| seed_variant | lane_max_hits | sort_variant | lane_variant | warp_variant | "
                    + " | ".join(f"{n} ms" for n in names) + " | score | bit-exact |\n")
            f.write("|---" * (7 + len(names)) + "|\n")
            f.write("| plain form | | | | | " + " | ".join(f"{plain_ms[n]:.3f}" for n in names) + " | | |\n")
            for sh in sorted(rows, key=lambda s: score.get(s, 1e9)):
                f.write(f"| {sh[0]} | {sh[1]} | {sh[2]} | {sh[3]} | {sh[4]} | "
                        + " | ".join(f"{rows[sh][n]:.3f}" for n in names)
                        + f" | {score.get(sh, float('nan')):.3f} | {exact[sh]} |\n")
            f.write("\n| chunk_reads | e2e reads/s |\n|---|---|\n")
            for ch, r in chunk_rates.items():
                f.write(f"| {ch} | {r / 1e6:.1f} M |\n")


if __name__ == "__main__":
    main()
