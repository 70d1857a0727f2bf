"""CUDA path against the oracle and the reference's golden outputs (GB300 only).

Every comparison is bit-exact: randstrobe hashes and coordinates, index contents
and order, bucket table, find / get_count results, nonrepetitive_fraction, the
rescue decision, and the NAM records (ref_id, query/ref start/end, n_hits, score,
is_rc) in the defined order.
"""
import hashlib
import os
import tempfile

import numpy as np
import pytest

from golden_cases import CASE_NAMES, Case, nams_equal
from gpu_index_test_gb300 import abi, native, synth
from oracle import oracle_py

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=CASE_NAMES)
def gcase(request):
    c = Case(request.param)
    p = native.params_from_read_length(c.read_length_param)
    idx = native.Index.build(p, c.genome)
    return c, p, idx


def test_index_build_matches_golden(gcase):
    c, p, idx = gcase
    info = idx.info()
    assert (info.bits, info.filter_cutoff, info.size) == (c.bits, c.filter_cutoff, c.index_size)
    rs, st = idx.export()
    h = hashlib.sha256()
    h.update(rs.tobytes())
    h.update(st.tobytes())
    assert h.hexdigest() == c.index_sha256


def test_index_stats_match_oracle(gcase):
    c, p, idx = gcase
    o = oracle_py.Index.build(oracle_py.params_from_read_length(c.read_length_param), c.genome)
    a, b = idx.info(), o.info()
    for f in ("size", "bits", "filter_cutoff", "tot_strobemer_count", "tot_occur_once", "tot_high_ab", "tot_mid_ab",
              "index_cutoff", "distinct_strobemers"):
        assert getattr(a, f) == getattr(b, f), f


def test_randstrobes_match_reference(gcase):
    c, p, _ = gcase
    q, offs = native.randstrobes_query(p, c.reads)
    assert (offs == c.ref_query_offsets).all()
    for f in ("hash", "start", "end", "is_reverse"):
        assert (q[f] == c.ref_queries[f]).all(), f


def test_find_and_count_match_oracle(gcase):
    c, p, idx = gcase
    o = oracle_py.Index.build(oracle_py.params_from_read_length(c.read_length_param), c.genome)
    rs, _ = idx.export()
    rng = np.random.default_rng(3)
    keys = np.concatenate([rs["hash"][:: max(1, len(rs) // 5000)], rng.integers(0, 2**63, 3000, dtype=np.uint64),
                           c.ref_queries["hash"][:5000], rs["hash"][:3]])
    got = idx.find(keys)
    exp = np.array([o.find(int(k)) for k in keys], np.uint64)
    assert (got == exp).all()
    found = got[got != np.uint64(2**64 - 1)]
    cnt = idx.get_count(found)
    assert (cnt == np.array([o.get_count(int(x)) for x in found], np.uint32)).all()


def test_nams_match_reference(gcase):
    c, p, idx = gcase
    m = native.Mapper(idx, abi.map_options(rescue_level=c.rescue_level))
    nams, offs, frac, resc = m.map_reads(c.reads)
    assert (frac == c.ref_frac).all()
    assert (resc == c.ref_rescued).all()
    assert (offs == c.ref_nam_offsets).all()
    bad = [i for i in range(c.reads.n)
           if not nams_equal(nams[int(offs[i]):int(offs[i + 1])],
                             c.ref_nams[int(c.ref_nam_offsets[i]):int(c.ref_nam_offsets[i + 1])])]
    assert not bad, bad[:10]


def test_find_nams_entry_points_match_oracle(gcase):
    c, p, idx = gcase
    o = oracle_py.Index.build(oracle_py.params_from_read_length(c.read_length_param), c.genome)
    m = native.Mapper(idx)
    q, qoff = c.ref_queries, c.ref_query_offsets
    full = np.zeros(len(q), abi.QUERY_RANDSTROBE)
    for f in ("hash", "start", "end", "is_reverse"):
        full[f] = q[f]
    nams, offs, frac = m.find_nams(full, qoff)
    cutoff = 2 * idx.info().filter_cutoff
    rn, roffs, _ = m.find_nams(full, qoff, rescue=True, rescue_cutoff=cutoff)
    for i in range(0, c.reads.n, 3):
        qi = full[int(qoff[i]):int(qoff[i + 1])]
        on, ofr = o.find_nams(qi)
        assert ofr == frac[i]
        assert nams_equal(nams[int(offs[i]):int(offs[i + 1])], oracle_py.sort_nams(on)), i
        orr = o.find_nams_rescue(qi, cutoff)
        assert nams_equal(rn[int(roffs[i]):int(roffs[i + 1])], oracle_py.sort_nams(orr)), i


def test_sti_round_trip(gcase):
    c, p, idx = gcase
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "x.sti")
        idx.write_sti(path)
        assert hashlib.sha256(open(path, "rb").read()).hexdigest() == c.sti_sha256
        back = native.Index.read_sti(path, p)
        a, b = idx.export(), back.export()
        assert (a[0] == b[0]).all() and (a[1] == b[1]).all()
        assert back.info().filter_cutoff == idx.info().filter_cutoff
        bad = native.params_from_read_length(250)
        with pytest.raises(native.GbsaError) as e:
            native.Index.read_sti(path, bad)
        assert e.value.code == abi.GBSA_ERR_INDEX_FILE


@pytest.mark.parametrize("mode", [abi.GBSA_SORT_REF_MATE2, abi.GBSA_SORT_REF_MATE1])
def test_reference_sort_modes(gcase, mode):
    c, p, idx = gcase
    o = oracle_py.Index.build(oracle_py.params_from_read_length(c.read_length_param), c.genome)
    opt = abi.map_options(rescue_level=2, sort_mode=mode)
    sub = c.reads.subset(np.arange(0, c.reads.n, 4))
    a = native.Mapper(idx, opt).map_reads(sub)
    b = o.map_reads(sub, opt, n_threads=4)
    assert (a[1] == b[1]).all()
    assert nams_equal(a[0], b[0])


def test_rescue_cap_100(gcase):
    c, p, idx = gcase
    o = oracle_py.Index.build(oracle_py.params_from_read_length(c.read_length_param), c.genome)
    opt = abi.map_options(rescue_level=2, rescue_count_cap=100)
    rescued = np.nonzero(c.ref_rescued)[0]
    sub = c.reads.subset(rescued if len(rescued) else np.arange(10))
    a = native.Mapper(idx, opt).map_reads(sub)
    b = o.map_reads(sub, opt, n_threads=4)
    assert (a[1] == b[1]).all() and nams_equal(a[0], b[0])


def test_larger_repeat_rich_genome_against_oracle():
    gp = synth.genome_params("C2", scale=0.05, seed=77)   # 5 Mbp, 20 contigs, duplications + STRs
    g = synth.make_genome(gp)
    reads = synth.make_reads(g, synth.read_params("C2", n_units=4000, seed=78))
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    o = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    a, b = idx.export(), (o.randstrobes(), o.starts())
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()
    assert idx.info().filter_cutoff == o.info().filter_cutoff
    x = native.Mapper(idx).map_reads(reads)
    y = o.map_reads(reads, n_threads=8)
    assert (x[1] == y[1]).all() and (x[2] == y[2]).all() and (x[3] == y[3]).all()
    assert nams_equal(x[0], y[0])


def test_variable_length_reads_against_oracle():
    g = synth.make_genome(synth.genome_params("C1", scale=0.1, seed=5))
    reads = synth.make_reads(g, synth.read_params("C3", n_units=3000, seed=6))
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    o = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    x = native.Mapper(idx).map_reads(reads)
    y = o.map_reads(reads, n_threads=8)
    assert (x[1] == y[1]).all() and nams_equal(x[0], y[0])


def _compare_profile(p, g, reads):
    """Index, query randstrobes and NAMs of the CUDA path against the oracle for params p."""
    idx = native.Index.build(p, g)
    o = oracle_py.Index.build(p, g)
    a, b = idx.export(), (o.randstrobes(), o.starts())
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()
    q, offs = native.randstrobes_query(p, reads)
    for r in range(0, reads.n, 7):
        o0, o1 = int(reads.offsets[r]), int(reads.offsets[r]) + int(reads.lengths[r])
        ref = oracle_py.randstrobes_query(p, bytes(reads.seq[o0:o1]))
        got = q[int(offs[r]):int(offs[r + 1])]
        assert len(got) == len(ref)
        for f in ("hash", "start", "end", "is_reverse"):
            assert (got[f] == ref[f]).all(), (r, f)
    x = native.Mapper(idx).map_reads(reads)
    y = o.map_reads(reads, n_threads=8)
    assert (x[1] == y[1]).all() and (x[2] == y[2]).all() and (x[3] == y[3]).all()
    assert nams_equal(x[0], y[0])


@pytest.mark.parametrize("read_len,len_min,len_max", [(300, 300, 300), (500, 500, 500), (500, 1200, 3000)])
def test_long_read_profiles_against_oracle(read_len, len_min, len_max):
    """Profiles for 300 / 500 bp reads (k=22 s=18, k=23 s=17): s-mers wider than 16
    bases take the 64-bit hashing path; reads above 1024 bases take the long-read
    seeding kernel."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.003, seed=31))
    reads = synth.make_reads(g, synth.ReadParams(seed=32, n_units=800 if len_max <= 500 else 150, len_min=len_min,
                                                 len_max=len_max, paired_frac=1.0, insert_mean=2 * len_max + 100,
                                                 insert_sd=30))
    p = native.params_from_read_length(read_len)
    assert p.s > 16
    _compare_profile(p, g, reads)


def test_wide_strobe_mask_against_oracle():
    """A strobe mask wider than 32 bits (q = all ones) takes the 64-bit selection path."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.003, seed=33))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=800, seed=34))
    p = native.params_make(150, 20, 16, 1, 7, -1, 80)
    assert p.q == (1 << 64) - 1
    _compare_profile(p, g, reads)


@pytest.mark.parametrize("mode", [abi.GBSA_SORT_SCORE, abi.GBSA_SORT_REF_MATE2])
def test_tandem_repeat_rescue_against_oracle(mode):
    """A genome with 5% short tandem repeats: hundreds of rescued reads end with more
    than 256 NAMs (block sorts) and some with more than 2048 (cluster sorts)."""
    import dataclasses
    gp = dataclasses.replace(synth.genome_params("C2", scale=0.01, seed=41), str_frac=0.05)
    g = synth.make_genome(gp)
    reads = synth.make_reads(g, synth.read_params("C2", n_units=3000, seed=42))
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    o = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    opt = abi.map_options(rescue_level=2, sort_mode=mode)
    x = native.Mapper(idx, opt).map_reads(reads)
    y = o.map_reads(reads, opt, n_threads=8)
    counts = np.diff(y[1].astype(np.int64))
    assert (counts > 2048).sum() >= 5 and (counts > 256).sum() >= 100
    assert (x[1] == y[1]).all() and (x[2] == y[2]).all() and (x[3] == y[3]).all()
    assert nams_equal(x[0], y[0])


@pytest.mark.parametrize("hits", [1, 3000])
def test_block_rescue_merge_against_oracle(hits):
    """Rescued reads merged by a whole block each (every rescued read with hits=1; the
    heavy ones with 3000), against the oracle: reads of 5% short tandem repeats with
    thousands of open NAMs, and the plain form's warp merge on the same reads."""
    import dataclasses
    gp = dataclasses.replace(synth.genome_params("C2", scale=0.01, seed=43), str_frac=0.05)
    g = synth.make_genome(gp)
    reads = synth.make_reads(g, synth.read_params("C2", n_units=3000, seed=44))
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    o = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    opt = abi.map_options(rescue_level=2)
    m = native.Mapper(idx, opt)
    m.set_rescue_block(0)
    warp = m.map_reads(reads)
    m.set_rescue_block(hits)
    x = m.map_reads(reads)
    y = o.map_reads(reads, opt, n_threads=8)
    assert x[3].sum() >= 100
    assert (x[1] == y[1]).all() and (x[2] == y[2]).all() and (x[3] == y[3]).all()
    assert nams_equal(x[0], y[0])
    assert (warp[1] == x[1]).all() and nams_equal(warp[0], x[0])
    # block merges take a batch with fewer rescued reads than the rescue kernel's warps
    few = reads.subset(np.nonzero(x[3])[0][:500])
    m.set_rescue_block(0)
    a = m.map_reads(few)
    m.set_rescue_block(hits)
    b = m.map_reads(few)
    assert (a[1] == b[1]).all() and nams_equal(a[0], b[0]) and (a[3] == b[3]).all()
    # the find_nams_rescue entry point (every read rescued) through the block merge
    m.set_rescue_block(1)
    q, qoff = native.randstrobes_query(p, reads.subset(np.arange(0, reads.n, 7)))
    cutoff = 2 * idx.info().filter_cutoff
    rn, roffs, _ = m.find_nams(q, qoff, rescue=True, rescue_cutoff=cutoff)
    for i in range(len(qoff) - 1):
        orr = o.find_nams_rescue(q[int(qoff[i]):int(qoff[i + 1])], cutoff)
        assert nams_equal(rn[int(roffs[i]):int(roffs[i + 1])], oracle_py.sort_nams(orr)), i


def test_read_bytes_and_alignments_against_oracle():
    """Reads of every start alignment (mod 4) and of lengths around the 4-base packing
    units, with lowercase bases, U/u, N/n, raw codes 0-3 and other bytes mixed in:
    query randstrobes read by read and NAMs equal the oracle's."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.003, seed=71))
    base = synth.make_reads(g, synth.read_params("C2", n_units=1500, seed=72))
    rng = np.random.default_rng(73)
    p = native.params_from_read_length(150)
    lens_choice = [p.k - 1, p.k, 31, 32, 33, 63, 64, 65, 127, 129, 150]
    parts, offs, lens = [], [], []
    pos = 0
    for r in range(base.n):
        o = int(base.offsets[r])
        L = min(int(base.lengths[r]), lens_choice[r % len(lens_choice)])
        x = base.seq[o:o + L].copy()
        kind = r % 6
        if kind == 1:    # lowercase runs
            m = rng.random(L) < 0.4
            x[m] = x[m] | 0x20
        elif kind == 2:  # U / u for T
            m = (x == ord("T")) & (rng.random(L) < 0.5)
            x[m] = np.where(rng.random(m.sum()) < 0.5, ord("U"), ord("u"))
        elif kind == 3:  # N / n
            m = rng.random(L) < 0.03
            x[m] = np.where(rng.random(m.sum()) < 0.5, ord("N"), ord("n"))
        elif kind == 4:  # raw codes and other bytes
            m = rng.random(L) < 0.02
            x[m] = rng.choice(np.array([0, 1, 2, 3, ord("R"), ord("."), 0xFF, 0x20, 0x61 ^ 0x80], np.uint8), m.sum())
        gap = int(rng.integers(0, 4))
        parts.append(np.full(gap, ord("N"), np.uint8))
        pos += gap
        parts.append(x)
        offs.append(pos)
        lens.append(L)
        pos += L
    reads = synth.Reads(np.concatenate(parts), np.array(offs, np.uint64), np.array(lens, np.uint32))
    assert len(set(np.array(offs) % 4)) == 4
    q, qo = native.randstrobes_query(p, reads)
    for r in range(reads.n):
        o0 = int(reads.offsets[r])
        ref = oracle_py.randstrobes_query(p, bytes(reads.seq[o0:o0 + int(reads.lengths[r])]))
        got = q[int(qo[r]):int(qo[r + 1])]
        assert len(got) == len(ref), r
        for f in ("hash", "start", "end", "is_reverse"):
            assert (got[f] == ref[f]).all(), (r, f)
    idx = native.Index.build(p, g)
    o = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    x = native.Mapper(idx).map_reads(reads)
    y = o.map_reads(reads, n_threads=8)
    assert (x[1] == y[1]).all() and (x[2] == y[2]).all() and nams_equal(x[0], y[0])


def test_index_with_2_28_buckets_against_oracle():
    """The human-scale bucket table (bits = 28, the value pick_bits gives a 3.1 Gbp
    genome; 2^28 + 1 starts, a 1 GB 32-bit copy) forced on a 20 Mbp genome: the GPU
    index equals the oracle's entry for entry and bucket for bucket, passes the
    oracle's sort-free check, and both lookup forms (fused, and the two kernels that
    indexes over 2 GiB use) give the oracle's NAMs."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.2, seed=91))
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g, bits=28)
    info = idx.info()
    assert info.bits == 28
    op = oracle_py.params_from_read_length(150)
    o = oracle_py.Index.build(op, g, bits=28)
    rs, st = idx.export()
    assert len(st) == (1 << 28) + 1
    assert (rs == o.randstrobes()).all() and (st == o.starts()).all()
    assert info.filter_cutoff == o.info().filter_cutoff
    assert oracle_py.verify_index(op, g, rs, st, 28, info.filter_cutoff)[0] == "equal"
    del rs, st
    reads = synth.make_reads(g, synth.read_params("C2", n_units=15_000, seed=92))
    y = o.map_reads(reads, n_threads=8)
    m = native.Mapper(idx)
    for fuse_limit in (None, 0):
        if fuse_limit is not None:
            m.set_fuse_limit(fuse_limit)
        x = m.map_reads(reads)
        assert bool(m.fused_lookup()) == (fuse_limit is None)
        assert (x[1] == y[1]).all() and (x[2] == y[2]).all() and (x[3] == y[3]).all()
        assert nams_equal(x[0], y[0])


def test_l2_window_gives_the_same_nams():
    """With the bucket table held in L2 through an access-policy window (the default
    when the table fits one) and without it, the NAMs are the same."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.05, seed=93))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=20_000, seed=94))
    idx = native.Index.build(native.params_from_read_length(150), g)
    m = native.Mapper(idx)
    on = m.set_l2_window(True)
    a = m.map_reads(reads)
    assert m.set_l2_window(False) == 0
    b = m.map_reads(reads)
    assert on >= 0
    assert (a[1] == b[1]).all() and (a[2] == b[2]).all() and (a[3] == b[3]).all()
    assert nams_equal(a[0], b[0])


def test_two_kernel_seeding_and_lookup_matches_fused():
    """Indexes over 2 GiB of entries run seeding and lookup as two kernels; forced
    here on a small index, the NAMs equal those of the fused kernel (which ran), for
    150 bp reads and for reads over the fused kernel's 512-base buffers."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=81))
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    for rp in (synth.read_params("C2", n_units=20_000, seed=82),
               synth.ReadParams(seed=83, n_units=3000, len_min=300, len_max=900, paired_frac=0.0)):
        reads = synth.make_reads(g, rp)
        m = native.Mapper(idx)
        a = m.map_reads(reads)
        assert m.fused_lookup()
        m.set_fuse_limit(0)
        b = m.map_reads(reads)
        assert not m.fused_lookup()
        assert (a[1] == b[1]).all() and (a[2] == b[2]).all() and (a[3] == b[3]).all()
        assert nams_equal(a[0], b[0])


def test_read_layouts_give_the_same_nams():
    """map_reads copies the span of the read buffer when the reads lie inside it (in
    any order) and gathers them otherwise; both layouts give the NAMs of the
    back-to-back layout, read by read."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.003, seed=51))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=1500, seed=52))
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    m = native.Mapper(idx)
    base = m.map_reads(reads)
    perm = np.random.default_rng(53).permutation(reads.n)
    shuffled = synth.Reads(reads.seq, reads.offsets[perm].copy(), reads.lengths[perm].copy())
    # the last read moved far behind the others (a copy of the same bases): gathered
    gap = 4 * len(reads.seq) + 12345
    o_last, l_last = int(reads.offsets[-1]), int(reads.lengths[-1])
    far_seq = np.concatenate([reads.seq, np.full(gap, ord("N"), np.uint8), reads.seq[o_last:o_last + l_last]])
    far_offs = reads.offsets.copy()
    far_offs[-1] = len(reads.seq) + gap
    far = synth.Reads(far_seq, far_offs, reads.lengths.copy())
    for layout, order in ((shuffled, perm), (far, np.arange(reads.n))):
        x = m.map_reads(layout)
        for j, r in enumerate(order):
            a = x[0][int(x[1][j]):int(x[1][j + 1])]
            b = base[0][int(base[1][r]):int(base[1][r + 1])]
            assert len(a) == len(b) and nams_equal(a, b)
        assert (x[2] == base[2][order]).all() and (x[3] == base[3][order]).all()


def test_pipelined_map_reads_matches_single_batch():
    """A call of 300k reads is cut into chunks whose transfers overlap the mapping of
    the next; the results equal those of one unpipelined batch, also when the first
    NAM capacity is too small (the call reports the total and is retried)."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.02, seed=61))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=150_000, seed=62))
    assert reads.n >= 2 * (1 << 17)   # at least two chunks
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    m = native.Mapper(idx)
    m.set_pipeline(1)
    a = m.map_reads(reads)
    m.set_pipeline(3)
    b = m.map_reads(reads, capacity=1024)
    assert (a[1] == b[1]).all() and (a[2] == b[2]).all() and (a[3] == b[3]).all()
    assert nams_equal(a[0], b[0])
    o = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    sub = reads.subset(np.arange(0, reads.n, 97))
    y = o.map_reads(sub, n_threads=8)
    x = m.map_reads(sub)
    assert (x[1] == y[1]).all() and nams_equal(x[0], y[0])


def _str_reads(g, n, seed, read_len=150):
    """n reads of read_len bases that start inside short tandem repeats of the genome:
    positions where the sequence repeats itself at a shift of 2-6 bases for at least
    100 bases."""
    seq = g.seq
    inside = np.zeros(len(seq), bool)
    for u in range(2, 7):
        c = np.concatenate([[0], np.cumsum(seq[u:] == seq[:-u])])
        ok = (c[100:] - c[:-100]) == 100
        inside[: len(ok)] |= ok
    starts = np.flatnonzero(inside[: len(seq) - read_len])
    pick = np.random.default_rng(seed).choice(starts, n)
    rs = np.ascontiguousarray(seq[pick[:, None] + np.arange(read_len)].ravel())
    return synth.Reads(rs, np.arange(n, dtype=np.uint64) * read_len, np.full(n, read_len, np.uint32))


def test_pipelined_map_reads_with_growing_work_areas():
    """A call of 600k reads whose last 150k start inside short tandem repeats: the
    pipelined call cuts it into a half chunk, a full one and two quarter chunks that
    alternate between two sets of work areas; the tail chunks outgrow the work areas
    sized for their bases, which grow while the next chunk is in flight, and the chunks
    run again.  Results equal one batch's and the oracle's."""
    import dataclasses
    gp = dataclasses.replace(synth.genome_params("C2", scale=0.01, seed=63), str_frac=0.05)
    g = synth.make_genome(gp)
    normal = synth.make_reads(g, synth.read_params("C2", n_units=225_000, seed=64))
    rep = _str_reads(g, 600_000 - normal.n, seed=65)
    reads = synth.Reads(np.concatenate([normal.seq, rep.seq]),
                        np.concatenate([normal.offsets, rep.offsets + np.uint64(len(normal.seq))]),
                        np.concatenate([normal.lengths, rep.lengths]))
    assert reads.n == 600_000 and rep.n >= 140_000
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    opt = abi.map_options(rescue_level=2)
    m = native.Mapper(idx, opt)
    m.set_pipeline(2)
    x = m.map_reads(reads)
    assert m.retries() > 0
    one = native.Mapper(idx, opt)
    one.set_pipeline(1)
    y = one.map_reads(reads)
    assert (x[1] == y[1]).all() and (x[2] == y[2]).all() and (x[3] == y[3]).all()
    assert nams_equal(x[0], y[0])
    # a second call reuses the grown work areas
    r0 = m.retries()
    z = m.map_reads(reads)
    assert m.retries() == r0 and (z[1] == y[1]).all() and nams_equal(z[0], y[0])
    o = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    sub = reads.subset(np.arange(0, reads.n, 211))
    w = o.map_reads(sub, opt, n_threads=8)
    v = m.map_reads(sub)
    assert (v[1] == w[1]).all() and (v[2] == w[2]).all() and nams_equal(v[0], w[0])


def test_errors_leave_the_mapper_usable():
    """A read over GBSA_MAX_READ_LEN in a late chunk of a pipelined call, or in a
    device-resident batch, fails the call with GBSA_ERR_READ_TOO_LONG; a device call with
    too small a NAM capacity reports GBSA_ERR_CAPACITY and the total.  The same mapper
    then maps the valid reads exactly as a fresh one."""
    import torch
    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=95))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=150_000, seed=96))
    idx = native.Index.build(native.params_from_read_length(150), g)
    want = native.Mapper(idx).map_reads(reads)
    bad_len = abi.GBSA_MAX_READ_LEN + 1
    seq = np.concatenate([reads.seq, np.full(bad_len, ord("A"), np.uint8)])
    offs = reads.offsets.copy()
    lens = reads.lengths.copy()
    r = reads.n - 10   # in the last chunk
    offs[r], lens[r] = len(reads.seq), bad_len
    bad = synth.Reads(seq, offs, lens)
    m = native.Mapper(idx)
    m.set_pipeline(2)
    with pytest.raises(native.GbsaError) as e:
        m.map_reads(bad)
    assert e.value.code == abi.GBSA_ERR_READ_TOO_LONG
    got = m.map_reads(reads)
    assert (got[1] == want[1]).all() and nams_equal(got[0], want[0])
    # device-resident batch
    dev = torch.device("cuda:0")
    n = reads.n
    d_seq = torch.from_numpy(bad.seq).to(dev)
    d_off = torch.from_numpy(bad.offsets.view(np.int64)).to(dev)
    d_len = torch.from_numpy(bad.lengths.view(np.int32)).to(dev)
    cap = int(want[1][-1])
    d_n = torch.empty(cap * 44, dtype=torch.uint8, device=dev)
    d_o = torch.empty(n + 1, dtype=torch.int64, device=dev)
    with pytest.raises(native.GbsaError) as e:
        m.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n, d_n.data_ptr(), cap, d_o.data_ptr())
    assert e.value.code == abi.GBSA_ERR_READ_TOO_LONG
    d_seq = torch.from_numpy(reads.seq).to(dev)
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).to(dev)
    d_len = torch.from_numpy(reads.lengths.view(np.int32)).to(dev)
    tot = m.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n, d_n.data_ptr(), cap // 2,
                             d_o.data_ptr())
    assert tot == cap
    tot = m.map_reads_device(d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n, d_n.data_ptr(), cap,
                             d_o.data_ptr())
    torch.cuda.synchronize()
    assert tot == cap
    assert (d_o.cpu().numpy().view(np.uint64) == want[1]).all()
    assert nams_equal(d_n.cpu().numpy().view(abi.NAM), want[0])


def test_sector_count_and_gather_bench():
    """The lookup's sector form lies between one sector per query (the bucket bounds)
    and one per 16 B counted plus two per query; the gather benchmark reports a
    positive rate, higher for a buffer that fits L2."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.003, seed=71))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=2000, seed=72))
    idx = native.Index.build(native.params_from_read_length(150), g)
    m = native.Mapper(idx)
    m.set_count_bytes(True)
    m.map_reads(reads)
    q = m.last_counts()["queries"]
    b, sec = m.last_alg_bytes(), m.last_alg_sectors()
    assert q > 0 and q <= sec <= b // 16 + 2 * q
    hbm = native.bench_gather(1 << 30)[1]
    l2 = native.bench_gather(16 << 20)[1]
    assert hbm > 100 and l2 > hbm
    probes, sectors, gbs = native.bench_gather_index(idx)
    assert probes > 0 and probes <= sectors <= 2 * probes and gbs > 0


@pytest.mark.parametrize("params", [(0.5, 300.0, 100.0), (0.3, 250.3, 37.7)])
def test_pair_classification_against_oracle(params):
    """Pair types of mapped read pairs on the GPU equal the oracle's, with mates
    interleaved and with mate 1 lists first (the reference's layout)."""
    import torch
    thr, mu, sigma = params
    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=81))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=3000, seed=82))
    idx = native.Index.build(native.params_from_read_length(150), g)
    nams, offs, _, _ = native.Mapper(idx).map_reads(reads)
    n_pairs = reads.n // 2
    counts = np.diff(offs.astype(np.int64))
    per_end = [nams[int(offs[r]):int(offs[r + 1])] for r in range(reads.n)]
    order_h = list(range(0, reads.n, 2)) + list(range(1, reads.n, 2))
    offs_h = np.zeros(reads.n + 1, np.uint64)
    offs_h[1:] = np.cumsum(counts[order_h])
    nams_h = np.concatenate([per_end[r] for r in order_h])
    dev = torch.device("cuda:0")
    seen = set()
    for layout, (nn, oo) in ((abi.GBSA_PAIRS_INTERLEAVED, (nams, offs)), (abi.GBSA_PAIRS_HALVES, (nams_h, offs_h))):
        d_n = torch.from_numpy(np.ascontiguousarray(nn).view(np.uint8).copy()).to(dev)
        d_o = torch.from_numpy(oo.astype(np.int64)).to(dev)
        d_t = torch.zeros(n_pairs, dtype=torch.uint8, device=dev)
        native.classify_pairs_device(d_n.data_ptr(), d_o.data_ptr(), n_pairs, d_t.data_ptr(), layout, thr, mu, sigma)
        got = d_t.cpu().numpy()
        ref = oracle_py.classify_pairs(nn, oo, n_pairs, layout, thr, mu, sigma)
        assert (got == ref).all()
        seen |= set(got.tolist())
    assert {3, 4} <= seen


@pytest.mark.parametrize("str_frac", [0.0, 0.05])
def test_nam_pair_scoring_against_oracle(str_frac):
    """NAM-pair scoring on the GPU equals the oracle's for mapped read pairs, mate 1
    sorted as sort_nams_single2 and mate 2 as Nam::operator<, in both mate layouts; on a
    genome with tandem repeats some pairs have hundreds of NAMs and fill the heap."""
    import dataclasses
    import torch
    gp = dataclasses.replace(synth.genome_params("C2", scale=0.01, seed=91), str_frac=str_frac)
    g = synth.make_genome(gp)
    reads = synth.make_reads(g, synth.read_params("C2", n_units=4000, seed=92))
    idx = native.Index.build(native.params_from_read_length(150), g)
    n_pairs = reads.n // 2
    mate1 = reads.subset(np.arange(0, reads.n, 2))
    mate2 = reads.subset(np.arange(1, reads.n, 2))
    a = native.Mapper(idx, abi.map_options(rescue_level=2, sort_mode=abi.GBSA_SORT_REF_MATE1)).map_reads(mate1)
    b = native.Mapper(idx, abi.map_options(rescue_level=2, sort_mode=abi.GBSA_SORT_REF_MATE2)).map_reads(mate2)
    c1, c2 = np.diff(a[1].astype(np.int64)), np.diff(b[1].astype(np.int64))
    # halves: mate 1 lists, then mate 2 lists; interleaved: mate 1, mate 2 per pair
    nams_h = np.concatenate([a[0], b[0]])
    offs_h = np.concatenate([a[1], b[1][1:] + a[1][-1]]).astype(np.uint64)
    ends = [a[0][int(a[1][i]):int(a[1][i + 1])] for i in range(n_pairs)]
    ends2 = [b[0][int(b[1][i]):int(b[1][i + 1])] for i in range(n_pairs)]
    inter = [x for i in range(n_pairs) for x in (ends[i], ends2[i])]
    offs_i = np.zeros(reads.n + 1, np.uint64)
    offs_i[1:] = np.cumsum([len(e) for e in inter])
    nams_i = np.concatenate(inter)
    dev = torch.device("cuda:0")
    tries = 20
    for layout, (nn, oo) in ((abi.GBSA_PAIRS_HALVES, (nams_h, offs_h)), (abi.GBSA_PAIRS_INTERLEAVED, (nams_i, offs_i))):
        d_n = torch.from_numpy(np.ascontiguousarray(nn).view(np.uint8).copy()).to(dev)
        d_o = torch.from_numpy(oo.astype(np.int64)).to(dev)
        d_p = torch.zeros(n_pairs * tries * 3, dtype=torch.int32, device=dev)
        d_c = torch.zeros(n_pairs, dtype=torch.int32, device=dev)
        native.nam_pairs_device(d_n.data_ptr(), d_o.data_ptr(), n_pairs, d_p.data_ptr(), d_c.data_ptr(), layout,
                                300.0, 100.0, tries)
        got = d_p.cpu().numpy().view(abi.NAM_PAIR).reshape(n_pairs, tries)
        got_c = d_c.cpu().numpy().astype(np.uint32)
        ref, ref_c = oracle_py.nam_pairs(nn, oo, n_pairs, layout, 300.0, 100.0, tries)
        assert (got_c == ref_c).all()
        for p in range(n_pairs):
            k = int(ref_c[p])
            assert (got[p][:k] == ref[p][:k]).all(), p
    both = (c1 > 0) & (c2 > 0)
    assert both.sum() > n_pairs // 2 and (ref_c[both] > 0).all()
    assert ((ref["i1"] >= 0) & (ref["i2"] >= 0)).any()
    if str_frac > 0:
        assert (np.maximum(c1, c2) > 200).any()


def test_server_requests_match_plain_form():
    """Requests of uneven sizes served by three workers give, request by request, the
    NAMs of one plain map_reads call over all reads; a request above the maximum is
    refused."""
    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=91))
    pool = synth.make_reads(g, synth.ReadParams(seed=92, n_units=20_000, len_min=100, len_max=250, paired_frac=1.0,
                                                insert_mean=400, insert_sd=50))
    idx = native.Index.build(native.params_from_read_length(150), g)
    plain = native.Mapper(idx).map_reads(pool)
    srv = native.Server(idx, workers=3, max_reads=8192)
    rng = np.random.default_rng(93)
    reqs, bufs = [], {}
    for tag in range(40):
        n = int(rng.integers(1, 4096)) * 2
        start = int(rng.integers(0, (pool.n - n) // 2)) * 2
        offs = np.ascontiguousarray(pool.offsets[start:start + n])
        lens = np.ascontiguousarray(pool.lengths[start:start + n])
        cap = 64 * n
        out = (np.zeros(cap, abi.NAM), np.zeros(n + 1, np.uint64), np.zeros(n, np.float32), np.zeros(n, np.uint8))
        bufs[tag] = (offs, lens, out, start, n)
        srv.submit(pool.seq.ctypes.data, offs.ctypes.data, lens.ctypes.data, n, out[0].ctypes.data, cap,
                   out[1].ctypes.data, out[2].ctypes.data, out[3].ctypes.data, tag)
    with pytest.raises(RuntimeError):
        big = np.zeros(8193, np.uint64)
        srv.submit(pool.seq.ctypes.data, big.ctypes.data, big.ctypes.data, 8193, 0, 0, 0, 0, 0, 999)
    done = {}
    while len(done) < 40:
        for tag, st, tot in srv.poll(wait_ms=-1):
            done[tag] = (st, tot)
    srv.free()
    for tag, (st, tot) in done.items():
        assert st == 0
        offs, lens, (nams, noff, frac, resc), start, n = bufs[tag]
        a, b = int(plain[1][start]), int(plain[1][start + n])
        assert tot == b - a and (noff == plain[1][start:start + n + 1] - a).all()
        assert nams_equal(nams[:tot], plain[0][a:b])
        assert (frac == plain[2][start:start + n]).all() and (resc == plain[3][start:start + n]).all()


def test_launch_count_grows():
    before = native.launch_count()
    g = synth.make_genome(synth.GenomeParams(seed=9, total_len=100_000))
    native.Index.build(native.params_from_read_length(150), g)
    assert native.launch_count() > before
