"""The batched form (gbsa_batcher_*) against the plain form and the oracle (GB300 only).

A batch runs as one launch of a CUDA graph captured over the batcher's work areas;
seeding and lookup are one persistent kernel pulling work items (a read, or both
mates of a pair) from a device queue.  Every comparison is bit-exact: NAM records,
offsets, nonrepetitive fractions and rescue flags.
"""
import numpy as np
import pytest

from golden_cases import nams_equal
from gpu_index_test_gb300 import abi, native, synth
from oracle import oracle_py

pytestmark = pytest.mark.gpu


def same(a, b):
    return (a[1] == b[1]).all() and (a[2] == b[2]).all() and (a[3] == b[3]).all() and nams_equal(a[0], b[0])


@pytest.fixture(scope="module")
def c3():
    """Uneven lengths (50-500 bp, log-uniform), half single-end, half pairs, on a 1 Mbp
    genome with duplications and tandem repeats (rescued reads with many NAMs)."""
    g = synth.make_genome(synth.GenomeParams(seed=101, total_len=1_000_000, n_contigs=3, dup_frac=0.05,
                                             str_frac=0.01))
    rp = synth.read_params("C3", n_units=12_000, seed=102)
    reads = synth.make_reads(g, rp)
    items = synth.read_items(rp)
    idx = native.Index.build(native.params_from_read_length(150), g)
    o = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    return g, reads, items, idx, o


def test_batched_form_matches_oracle_on_uneven_reads_and_pairs(c3):
    g, reads, items, idx, o = c3
    y = o.map_reads(reads, n_threads=8)
    b = native.Batcher(idx, max_reads=reads.n)
    x = b.map_reads(reads, items)
    assert same(x, y)
    # again (now a graph replay), and without items (every read its own work item)
    assert same(b.map_reads(reads, items), y)
    assert same(b.map_reads(reads), y)
    st = b.stats()
    assert st["graph_launches"] >= 2 and st["captures"] >= 1


@pytest.mark.parametrize("variant", range(abi.SEED_VARIANTS))
def test_every_tuned_variant_is_bit_exact(c3, variant):
    """Each shape the autotuner may pick (seeding + lookup variant, lane / warp split of
    the NAM merge, sort block size, register budgets of the two merges) gives the plain
    form's output."""
    g, reads, items, idx, o = c3
    ref = native.Mapper(idx).map_reads(reads)
    regs = ((0, 0), (1, 1), (2, 2), (3, 3), (4, 4), (5, 3), (6, 0))
    for j, (lane_max, sort_variant) in enumerate(((160, 0), (64, 1), (96, 0), (128, 1))):
        lv, wv = regs[(j + variant) % 7]
        cfg = abi.batch_config(variant, lane_max, sort_variant, 4096, lv, wv)
        b = native.Batcher(idx, config=cfg, max_reads=reads.n)
        assert same(b.map_reads(reads, items), ref)   # several chunks of ~4096 reads, three sets of work areas
        b.free()


def test_batched_device_entry_point_and_graph_reuse(c3):
    """The device entry point with work items in device memory: one graph serves
    batches of different sizes (each its own slice of the reads), bit-exact with the
    plain form's device entry point."""
    torch = pytest.importorskip("torch")
    g, reads, items, idx, o = c3
    dev = torch.device("cuda:0")
    b = native.Batcher(idx, max_reads=reads.n)
    m = native.Mapper(idx, max_reads=reads.n)
    st = torch.cuda.current_stream(dev).cuda_stream
    for lo_item, hi_item in ((0, len(items) - 1), (100, 2100), (5000, 5400), (0, len(items) - 1)):
        r0, r1 = int(items[lo_item]), int(items[hi_item])
        sub = reads.subset(np.arange(r0, r1))
        it = (items[lo_item:hi_item + 1] - r0).astype(np.uint32)
        n = sub.n
        d_seq = torch.from_numpy(sub.seq).to(dev)
        d_off = torch.from_numpy(sub.offsets.view(np.int64)).to(dev)
        d_len = torch.from_numpy(sub.lengths.view(np.int32)).to(dev)
        d_it = torch.from_numpy(it.view(np.int32)).to(dev)
        cap = 60 * n + 1024
        outs = []
        for form in ("batched", "plain"):
            d_nams = torch.zeros(cap * 44, dtype=torch.uint8, device=dev)
            d_noff = torch.zeros(n + 1, dtype=torch.int64, device=dev)
            d_frac = torch.zeros(n, dtype=torch.float32, device=dev)
            d_resc = torch.zeros(n, dtype=torch.uint8, device=dev)
            if form == "batched":
                tot = b.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n, d_nams.data_ptr(),
                                         cap, d_noff.data_ptr(), d_frac.data_ptr(), d_resc.data_ptr(),
                                         d_it.data_ptr(), len(it) - 1, st)
            else:
                tot = m.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n, d_nams.data_ptr(),
                                         cap, d_noff.data_ptr(), d_frac.data_ptr(), d_resc.data_ptr(), st)
            torch.cuda.synchronize()
            assert tot <= cap
            outs.append((d_nams[: tot * 44].cpu().numpy().view(abi.NAM), d_noff.cpu().numpy().view(np.uint64),
                         d_frac.cpu().numpy(), d_resc.cpu().numpy()))
        assert same(outs[0], outs[1])
    assert b.stats()["graph_launches"] >= 3


def test_batched_stage_times_inside_the_graph(c3):
    """Stage events recorded inside the batch graph (external event nodes) time the graph's
    launches; profiling on or off, the output is the same."""
    g, reads, items, idx, o = c3
    b = native.Batcher(idx, max_reads=reads.n)
    ref = b.map_reads(reads, items)
    b.set_profile(True)
    got = b.map_reads(reads, items)
    st = b.stage_ms()
    b.set_profile(False)
    again = b.map_reads(reads, items)
    b.free()
    assert same(got, ref) and same(again, ref)
    assert st["seed_lookup"] > 0 and st["nams"] > 0 and st["rescue"] >= 0


def test_batched_form_grows_its_work_areas():
    """Reads inside a tandem-repeat-rich genome outgrow small work areas: the batch runs
    again with larger ones and is captured anew; the results equal the plain form's."""
    g = synth.make_genome(synth.GenomeParams(seed=111, total_len=400_000, n_contigs=2, str_frac=0.05))
    rp = synth.ReadParams(seed=112, n_units=6000, len_min=150, len_max=150, paired_frac=1.0)
    reads = synth.make_reads(g, rp)
    idx = native.Index.build(native.params_from_read_length(150), g)
    ref = native.Mapper(idx).map_reads(reads)
    b = native.Batcher(idx, max_reads=1024, max_bases=1024 * 20)
    for _ in range(2):
        assert same(b.map_reads(reads, synth.read_items(rp)), ref)


def _rows(req):
    """A request's reads in the pool: (start, n) for a run, or an index array."""
    start, n = req
    return np.arange(start, start + n) if n is not None else np.asarray(start)


def _serve(srv, pool, reqs):
    bufs = {}
    for tag, req in enumerate(reqs):
        rows = _rows(req)
        n = len(rows)
        offs = np.ascontiguousarray(pool.offsets[rows])
        lens = np.ascontiguousarray(pool.lengths[rows])
        cap = 64 * n + 64
        out = (np.zeros(cap, abi.NAM), np.zeros(n + 1, np.uint64), np.zeros(max(1, n), np.float32),
               np.zeros(max(1, n), np.uint8))
        bufs[tag] = (offs, lens, out)
        srv.submit(pool.seq.ctypes.data, offs.ctypes.data, lens.ctypes.data, n, out[0].ctypes.data, cap,
                   out[1].ctypes.data, out[2].ctypes.data, out[3].ctypes.data, tag)
    done = {}
    while len(done) < len(reqs):
        for tag, st, tot in srv.poll(wait_ms=-1):
            done[tag] = (st, tot)
    return bufs, done


def test_server_batches_requests_and_each_equals_alone():
    """Small requests submitted together are mapped in shared batches (continuous
    batching: fewer batches than requests) on two slots, and each request's NAMs,
    offsets, fractions and flags equal those of the request mapped alone."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=121))
    pool = synth.make_reads(g, synth.ReadParams(seed=122, n_units=20_000, len_min=100, len_max=250, paired_frac=1.0,
                                                insert_mean=400, insert_sd=50))
    idx = native.Index.build(native.params_from_read_length(150), g)
    rng = np.random.default_rng(123)
    reqs = []
    for _ in range(80):
        n = int(rng.integers(1, 400)) * 2
        reqs.append((int(rng.integers(0, (pool.n - n) // 2)) * 2, n))
    reqs.append((0, 0))   # an empty request
    # requests whose reads lie far apart in the caller's buffer (gathered into staging)
    for k in range(6):
        reqs.insert(10 * k + 3, (np.sort(rng.choice(pool.n, 300, replace=False)), None))
    srv = native.Server(idx, workers=2, max_reads=16384)
    bufs, done = _serve(srv, pool, reqs)
    info = srv.info()
    stats = srv.stats()
    srv.free()
    assert info["slots"] == 2 and info["requests"] == len(reqs) and info["batches"] < len(reqs)
    assert stats["graph_launches"] >= info["batches"] - stats["eager_runs"]
    m = native.Mapper(idx)
    for tag, req in enumerate(reqs):
        st, tot = done[tag]
        assert st == 0
        rows = _rows(req)
        n = len(rows)
        alone = m.map_reads(pool.subset(rows))
        offs, lens, (nams, noff, frac, resc) = bufs[tag]
        assert tot == len(alone[0]) and (noff == alone[1]).all()
        assert nams_equal(nams[:tot], alone[0])
        assert (frac[:n] == alone[2]).all() and (resc[:n] == alone[3]).all()


def test_server_replay_checks_every_request():
    """gbsa_server_replay: requests submitted at their times from native threads, each
    compared byte for byte with the pool's plain-form results; a request whose expected
    results were altered (one NAM's score) is flagged, the others are not."""
    import torch
    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=131))
    pool = synth.make_reads(g, synth.ReadParams(seed=132, n_units=8000, len_min=100, len_max=250, paired_frac=1.0,
                                                insert_mean=400, insert_sd=50))
    idx = native.Index.build(native.params_from_read_length(150), g)
    m = native.Mapper(idx)
    exp = m.map_reads(pool)
    rng = np.random.default_rng(133)
    k = 60
    reqs = np.zeros(k, abi.REPLAY_REQUEST)
    reqs["at_us"] = np.sort(rng.uniform(0, 20_000, k))
    reqs["n_reads"] = rng.integers(1, 300, k) * 2
    reqs["start"] = [int(rng.integers(0, (pool.n - n) // 2)) * 2 for n in reqs["n_reads"]]
    max_reads, cap = 1024, 64 * 1024
    bufs = [(torch.empty(cap * 44, dtype=torch.uint8).pin_memory(), torch.empty(max_reads + 1, dtype=torch.int64).pin_memory(),
             torch.empty(max_reads, dtype=torch.float32).pin_memory(), torch.empty(max_reads, dtype=torch.uint8).pin_memory())
            for _ in range(4)]
    ptrs = [tuple(t.data_ptr() for t in b) for b in bufs]
    nams = np.ascontiguousarray(exp[0])
    off = np.ascontiguousarray(exp[1], np.uint64)
    frac, resc = np.ascontiguousarray(exp[2]), np.ascontiguousarray(exp[3])
    # plant a mistake in the expected results of request 7 (its first read with NAMs)
    s7, n7 = int(reqs["start"][7]), int(reqs["n_reads"][7])
    j = int(off[s7])
    assert off[s7 + n7] > off[s7]
    nams["score"][j] += 1.0
    srv = native.Server(idx, workers=2, max_reads=max_reads)
    offs = np.ascontiguousarray(pool.offsets, np.uint64)
    lens = np.ascontiguousarray(pool.lengths, np.uint32)
    sub, done, st, mis = srv.replay(pool.seq.ctypes.data, offs, lens, reqs, ptrs, cap, max_reads,
                                    expected=(nams.ctypes.data, off.ctypes.data, frac.ctypes.data, resc.ctypes.data))
    srv.free()
    assert (st == 0).all()
    r_j = int(np.searchsorted(off, j, side="right")) - 1   # the read that holds NAM j
    hit = (reqs["start"] <= r_j) & (r_j < reqs["start"] + reqs["n_reads"])
    assert hit[7] and (mis == hit.astype(np.uint8)).all()
    assert (done >= sub).all() and (sub >= reqs["at_us"] - 1.0).all()


def test_server_memory_budget_limits_slots():
    """Slots are created against the device-memory budget: a budget below one slot's
    work areas leaves a single slot, which still serves every request."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.005, seed=124))
    pool = synth.make_reads(g, synth.read_params("C2", n_units=2000, seed=125))
    idx = native.Index.build(native.params_from_read_length(150), g)
    srv = native.Server(idx, workers=6, max_reads=8192, memory_budget=1)
    info = srv.info()
    assert info["slots"] == 1 and info["slot_bytes"] > 0 and info["budget"] == 1
    bufs, done = _serve(srv, pool, [(0, 1000), (1000, 2000), (3000, 1000)])
    srv.free()
    assert all(st == 0 for st, _ in done.values())
