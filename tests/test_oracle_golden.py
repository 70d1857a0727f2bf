"""The oracle (CPU restatement) against the reference's own outputs in tests/golden/.

The fixtures were produced by running the reference's compiled CPU code
(oracle/ref_driver.cu: StrobemerIndex::read, SyncmerIterator, RandstrobeIterator,
find_nams, find_nams_rescue) — see tests/golden/make_golden.py.
"""
import hashlib

import numpy as np
import pytest

from golden_cases import CASE_NAMES, Case, kat, nams_equal
from gpu_index_test_gb300 import abi
from oracle import oracle_py


def test_xxh64_known_answers():
    ins, outs = kat()
    for a, b in zip(ins, outs):
        assert oracle_py.xxh64(int(a)) == int(b)


def test_params_profiles():
    p = oracle_py.params_from_read_length(150)
    assert (p.k, p.s, p.t_syncmer, p.l, p.u, p.q, p.max_dist, p.w_min, p.w_max) == (20, 16, 3, 1, 7, 255, 80, 5, 11)
    p = oracle_py.params_from_read_length(500)
    assert (p.k, p.s, p.w_min, p.w_max, p.max_dist) == (23, 17, 5, 15, 255)
    p = oracle_py.params_from_read_length(50)
    assert (p.k, p.s, p.l, p.u, p.w_min, p.w_max, p.max_dist) == (20, 16, -3, 2, 1, 6, 20)
    with pytest.raises(ValueError):
        oracle_py.params_from_read_length(150, k=21, s=18)  # (k - s) odd


@pytest.fixture(scope="module", params=CASE_NAMES)
def case(request):
    c = Case(request.param)
    p = oracle_py.params_from_read_length(c.read_length_param)
    idx = oracle_py.Index.build(p, c.genome)
    return c, p, idx


def test_index_matches_fixture(case):
    c, p, idx = case
    info = idx.info()
    assert (info.bits, info.filter_cutoff, info.size) == (c.bits, c.filter_cutoff, c.index_size)
    h = hashlib.sha256()
    h.update(idx.randstrobes().tobytes())
    h.update(idx.starts().tobytes())
    assert h.hexdigest() == c.index_sha256


def test_randstrobes_match_reference(case):
    c, p, _ = case
    for i in range(c.reads.n):
        got = oracle_py.randstrobes_query(p, c.read(i))
        ref = c.ref_queries[int(c.ref_query_offsets[i]) : int(c.ref_query_offsets[i + 1])]
        assert len(got) == len(ref), i
        for f in ("hash", "start", "end", "is_reverse"):
            assert (got[f] == ref[f]).all(), (i, f)


def test_nams_match_reference(case):
    c, p, idx = case
    nams, offs, frac, resc = idx.map_reads(c.reads, abi.map_options(rescue_level=c.rescue_level), n_threads=4)
    assert (frac == c.ref_frac).all()
    assert (resc == c.ref_rescued).all()
    assert (offs == c.ref_nam_offsets).all()
    for i in range(c.reads.n):
        a = nams[int(offs[i]) : int(offs[i + 1])]
        b = c.ref_nams[int(c.ref_nam_offsets[i]) : int(c.ref_nam_offsets[i + 1])]
        assert nams_equal(a, b), i


def _nam(ref_id, is_rc, qs, rs, n_hits):
    n = np.zeros(1, abi.NAM)
    n["ref_id"], n["is_rc"], n["query_start"], n["ref_start"], n["n_hits"] = ref_id, is_rc, qs, rs, n_hits
    n["query_end"], n["ref_end"] = qs + 50, rs + 50
    return n


def test_pair_classification_cases():
    """gpu_pre_cal_type restated: each type and the boundaries of its comparisons
    (dropoff ratio exactly 0.5, diagonal distance exactly mu + 10 sigma = 1300)."""
    fwd = lambda rs, h=5, ref=3: _nam(ref, 0, 0, rs, h)
    rev = lambda rs, h=5, ref=3: _nam(ref, 1, 10, rs + 10, h)   # diagonal rs
    cases = [
        ([], [], 0),
        ([fwd(1000)], [], 1),
        ([], [rev(1100)], 2),
        ([fwd(1000)], [rev(1190)], 3),                 # r1 ---> <--- r2, distance 190
        ([fwd(1000)], [rev(2299)], 3),                 # distance 1299
        ([fwd(1000)], [rev(2300)], 4),                 # distance 1300 is not below the bound
        ([rev(1190)], [fwd(1000)], 3),                 # r2 ---> <--- r1
        ([fwd(1000)], [fwd(1190)], 4),                 # same orientation
        ([fwd(1000)], [rev(1190, ref=4)], 4),          # other reference
        ([fwd(1000, h=2)], [rev(1190)], 4),            # top NAM with <= 2 hits: dropoff 1
        ([fwd(1000, h=10), fwd(5000, h=5)], [rev(1190)], 4),   # dropoff exactly 0.5
        ([fwd(1000, h=10), fwd(5000, h=4)], [rev(1190)], 3),   # dropoff 0.4
        ([rev(1000)], [fwd(1190)], 4),                 # reverse mate upstream
    ]
    ends = []
    for m1, m2, _ in cases:
        ends += [m1, m2]
    offs = np.zeros(len(ends) + 1, np.uint64)
    offs[1:] = np.cumsum([len(e) for e in ends])
    nams = np.concatenate([x for e in ends for x in e]) if offs[-1] else np.zeros(0, abi.NAM)
    got = oracle_py.classify_pairs(nams, offs, len(cases), abi.GBSA_PAIRS_INTERLEAVED)
    assert list(got) == [c[2] for c in cases]
    # the same pairs with mate 1 lists first, then mate 2 lists
    halves = [c[0] for c in cases] + [c[1] for c in cases]
    offs_h = np.zeros(len(halves) + 1, np.uint64)
    offs_h[1:] = np.cumsum([len(e) for e in halves])
    nams_h = np.concatenate([x for e in halves for x in e])
    got_h = oracle_py.classify_pairs(nams_h, offs_h, len(cases), abi.GBSA_PAIRS_HALVES)
    assert list(got_h) == [c[2] for c in cases]



def test_nam_pair_scoring_cases():
    """get_best_scoring_nam_pairs_sort3 restated, on hand-worked cases (mu 300, sigma
    100: mate 2's diagonal within [d1, d1 + 1300) of a forward mate 1, within
    (d1 - 1300, d1] of a reverse one): pairing and its window edges on both strands,
    pruning at half the best joint count, single-end entries (max_tries per reference
    and strand) and the cut to max_tries, an absent end ordered as an all-zero NAM, and
    reference ids from 3000 on never paired."""
    fwd = lambda rs, h=5, ref=3: _nam(ref, 0, 0, rs, h)
    rev = lambda rs, h=5, ref=3: _nam(ref, 1, 10, rs + 10, h)   # diagonal rs
    cases = [
        ([fwd(1000)], [rev(1190, h=4)], 20, [(9, 0, 0)]),
        ([fwd(1000)], [rev(2300, h=4)], 20, [(5, 0, -1), (4, -1, 0)]),    # window end: no pair
        ([fwd(1000)], [rev(999, h=4)], 20, [(5, 0, -1), (4, -1, 0)]),     # below the window
        ([rev(1190, h=6)], [fwd(1000, h=3)], 20, [(9, 0, 0)]),             # mate 1 reverse
        ([fwd(1000, h=10), fwd(5000, h=2)], [rev(1100, h=10), rev(5100, h=2)], 20, [(20, 0, 0)]),
        ([fwd(1000 * k) for k in range(1, 6)], [rev(90000, ref=4)], 3,
         [(5, -1, 0), (5, 0, -1), (5, 1, -1)]),
        ([fwd(1000, ref=3000)], [rev(1190, ref=3000)], 20, [(5, -1, 0), (5, 0, -1)]),
        ([fwd(1000)], [], 20, []),
    ]
    for layout in (abi.GBSA_PAIRS_INTERLEAVED, abi.GBSA_PAIRS_HALVES):
        for m1, m2, tries, want in cases:
            ends = [m1, m2]
            offs = np.zeros(3, np.uint64)
            offs[1:] = np.cumsum([len(e) for e in ends])
            nams = np.concatenate([x for e in ends for x in e])
            out, cnt = oracle_py.nam_pairs(nams, offs, 1, layout, 300.0, 100.0, tries)
            got = [tuple(int(v) for v in out[0][i]) for i in range(int(cnt[0]))]
            assert got == want, (m1, m2, got)


def test_nam_pair_heap_keeps_the_best_forty():
    """More than 40 candidate pairs: the list holds the 40 best joint counts (the
    heap), sorted by score."""
    m1 = [_nam(3, 0, 0, 1000 + 10 * i, 40 - i // 2) for i in range(30)]
    m2 = [_nam(3, 1, 10, 1100 + 10 * i + 10, 40 - i // 3) for i in range(30)]
    import itertools
    m2 = sorted(m2, key=lambda n: int(n["ref_start"][0] - n["query_start"][0]))
    nams = np.concatenate(m1 + m2)
    offs = np.array([0, len(m1), len(m1) + len(m2)], np.uint64)
    out, cnt = oracle_py.nam_pairs(nams, offs, 1, abi.GBSA_PAIRS_INTERLEAVED, 300.0, 100.0, 64)
    got = out[0][: int(cnt[0])]
    paired = got[(got["i1"] >= 0) & (got["i2"] >= 0)]
    assert len(paired) == abi.GBSA_NAM_PAIRS_TOP_K
    assert (np.diff(got["score"]) <= 0).all()
    # the heap's 40 are the 40 largest joint counts among all pairs in the window
    joint = sorted((int(a["n_hits"][0]) + int(b["n_hits"][0]) for a, b in itertools.product(m1, m2)
                    if 0 <= int(b["ref_start"][0] - b["query_start"][0]) - int(a["ref_start"][0]) < 1300),
                   reverse=True)
    assert sorted(paired["score"].tolist(), reverse=True) == joint[:40]


def test_index_verifier_accepts_the_oracle_index_and_finds_planted_faults(case):
    """The sort-free index check (used on indexes too large to build on the host) accepts
    the oracle's own index and names a planted fault: a changed entry, two swapped
    entries, a moved bucket bound and another filter cutoff."""
    c, p, idx = case
    rs, st = idx.randstrobes(), idx.starts()
    info = idx.info()
    check = lambda r, s, fc=info.filter_cutoff: oracle_py.verify_index(p, c.genome, r, s, info.bits, fc)[0]
    assert check(rs, st) == "equal"
    if len(rs) < 3:
        return
    bad = rs.copy()
    bad[len(bad) // 2]["position"] += 1
    assert check(bad, st) in ("entry multiset", "entry order")
    i = int(np.nonzero(rs["hash"][1:] != rs["hash"][:-1])[0][0])   # rs[i] < rs[i + 1]
    bad = rs.copy()
    bad[[i, i + 1]] = bad[[i + 1, i]]
    assert check(bad, st) == "entry order"
    bst = st.copy()
    j = int(np.nonzero(bst[1:] > bst[:-1])[0][0]) + 1
    bst[j] -= 1
    assert check(rs, bst) == "bucket table"
    assert check(rs, st, info.filter_cutoff + 1) == "filter cutoff"
