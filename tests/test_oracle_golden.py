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
