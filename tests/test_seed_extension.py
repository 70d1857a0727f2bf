"""Seed extension of NAMs: reverse_nam_if_needed + extend_seed_part (step2/main.cu:759-793,
582-643) with my_hamming_align (main.cu:506-580).

The CPU tests check the oracle (C++) against a second, line-by-line Python restatement
of the reference on small cases, including the edge cases the reference's code has:
a NAM whose orientation is wrong (a false reverse hit), k-mers that match in neither
orientation, a read overhanging its contig, the 5% Hamming limit on both sides, N and
lower-case bases, and NAMs outside their read or contig.  The GPU tests compare
gbsa_extend_seeds_device with the oracle on NAMs from the mapper and on altered ones.
The oracle's extension and mate rescue are also checked against the reference's own
functions, compiled from its main.cu, on the read pairs of tests/golden/align_ref.npz
(tests/test_align_plan.py)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))

from gpu_index_test_gb300 import abi  # noqa: E402
import oracle_py  # noqa: E402

K = 20
_RC = {ord(a): ord(b) for a, b in zip("ACGTUacgtu", "TGCAATGCAA")}


def _revcomp(b: bytes) -> bytes:
    """The reads' rc copy (main.cu:1893-1900) through revcomp_table (main.cu:1832-1849)."""
    return bytes(_RC.get(c, ord("N")) for c in reversed(b))


def _py_extend(ref: bytes, read: bytes, nam, k=K, match=2, mismatch=8, end_bonus=10):
    """The reference's two functions restated in plain Python (small cases only)."""
    L = len(read)
    rc = _revcomp(read)
    is_rc, qs, qe = int(nam["is_rc"]), int(nam["query_start"]), int(nam["query_end"])
    rs, re_ = int(nam["ref_start"]), int(nam["ref_end"])
    # reverse_nam_if_needed
    seq, seq_rc = (rc, read) if is_rc else (read, rc)
    ok = ref[rs:rs + k] == seq[qs:qs + k] and ref[re_ - k:re_] == seq[qe - k:qe]
    if not ok:
        qs2, qe2 = L - qe, L - qs
        if ref[rs:rs + k] == seq_rc[qs2:qs2 + k] and ref[re_ - k:re_] == seq_rc[qe2 - k:qe2]:
            is_rc, qs, qe, ok = 1 - is_rc, qs2, qe2, True
    out = dict(ref_id=int(nam["ref_id"]), ref_start=0, edit_distance=0, global_ed=0, score=0, length=0,
               query_start=qs, query_end=qe, is_rc=is_rc, done=0, consistent=int(ok))
    # extend_seed_part
    query = rc if is_rc else read
    pstart = max(0, rs - qs)
    pend = min(re_ + L - qe, len(ref))
    if pend - pstart == L and ok:
        segm = ref[pstart:pstart + L]
        hd, limit, i = 0, int(L * 0.05), 0
        while i < L and hd <= limit:
            hd += query[i] != segm[i]
            i += 1
        if float(np.float32(hd) / np.float32(L)) < 0.05:   # (float) hd / size, compared in double
            # my_hamming_align
            start, score, best_start, best_end, best_score = 0, end_bonus, 0, 0, 0
            for i in range(L):
                score += match if query[i] == segm[i] else -mismatch
                if score < 0:
                    start, score = i + 1, 0
                if score > best_score:
                    best_start, best_score, best_end = start, score, i + 1
            if score + end_bonus > best_score:
                best_score, best_end, best_start = score + end_bonus, L, start
            mm = sum(query[i] != segm[i] for i in range(best_start, best_end))
            out.update(done=1, edit_distance=mm, global_ed=mm + best_start + (L - best_end), score=best_score,
                       ref_start=pstart + best_start, length=best_end - best_start)
    return out


def _nam(qs, qe, rs, re_, is_rc=0, ref_id=0):
    n = np.zeros(1, abi.NAM)
    n["query_start"], n["query_end"], n["ref_start"], n["ref_end"] = qs, qe, rs, re_
    n["is_rc"], n["ref_id"] = is_rc, ref_id
    return n[0]


def _oracle_one(ref: bytes, read: bytes, nam, **kw):
    params = abi.align_params(**kw) if kw else None
    return oracle_py.extend_seeds(np.frombuffer(ref, np.uint8), [0], [len(ref)], np.frombuffer(read, np.uint8), [0],
                                  [len(read)], np.array([nam]), [0], K, params)[0]


def _same(rec, py):
    for f, v in py.items():
        assert int(rec[f]) == v, (f, int(rec[f]), v)


def _genome(n, seed):
    return np.random.default_rng(seed).choice(np.frombuffer(b"ACGT", np.uint8), n).tobytes()


def test_exact_and_single_mismatch_cases():
    ref = _genome(400, 1)
    read = ref[100:250]
    got = _oracle_one(ref, read, _nam(10, 140, 110, 240))
    assert got["done"] == 1 and got["consistent"] == 1
    assert (got["score"], got["ref_start"], got["length"], got["edit_distance"]) == (150 * 2 + 20, 100, 150, 0)
    # one mismatch in the middle costs match + mismatch; one at the last base is soft-clipped
    mid = bytearray(read)
    mid[75] = ord("A") if mid[75] != ord("A") else ord("C")
    got = _oracle_one(ref, bytes(mid), _nam(10, 60, 110, 160))
    assert (got["score"], got["edit_distance"], got["global_ed"]) == (149 * 2 - 8 + 20, 1, 1)
    end = bytearray(read)
    end[149] = ord("A") if end[149] != ord("A") else ord("C")
    got = _oracle_one(ref, bytes(end), _nam(10, 60, 110, 160))
    _same(got, _py_extend(ref, bytes(end), _nam(10, 60, 110, 160)))
    assert got["done"] == 1


def test_false_reverse_nam_is_flipped():
    """A NAM given in the wrong orientation is turned around when its k-mers match
    the other strand (main.cu:779-790)."""
    ref = _genome(500, 2)
    read = _revcomp(ref[200:350])             # the read comes from the reverse strand
    nam = _nam(150 - 140, 150 - 10, 210, 340, is_rc=0)   # coordinates of the forward view, orientation wrong
    got = _oracle_one(ref, read, nam)
    _same(got, _py_extend(ref, read, nam))
    assert got["is_rc"] == 1 and got["consistent"] == 1 and got["done"] == 1
    assert (got["query_start"], got["query_end"]) == (10, 140) and got["ref_start"] == 200


def test_inconsistent_and_overhanging_nams_are_left_to_a_gapped_aligner():
    ref = _genome(500, 3)
    read = ref[100:250]
    other = _genome(150, 4)
    got = _oracle_one(ref, other, _nam(10, 140, 110, 240))
    assert (got["consistent"], got["done"]) == (0, 0)
    # the read projected over the contig start: [pstart, pend) is shorter than the read
    read0 = _genome(30, 5) + ref[0:120]
    nam = _nam(30, 150, 0, 120)
    got = _oracle_one(ref, read0, nam)
    _same(got, _py_extend(ref, read0, nam))
    assert got["consistent"] == 1 and got["done"] == 0


@pytest.mark.parametrize("n_mm,done", [(4, 1), (5, 0), (9, 0)])
def test_hamming_limit_of_five_percent(n_mm, done):
    """L = 100: the limit is 5 mismatches, and 5/100 in float (0.0500000007) is not
    below 0.05 in double, so 4 mismatches pass and 5 do not."""
    ref = _genome(300, 6)
    read = bytearray(ref[100:200])
    for j in range(n_mm):
        p = 30 + 7 * j
        read[p] = ord("A") if read[p] != ord("A") else ord("G")
    nam = _nam(0, 25, 100, 125)
    got = _oracle_one(ref, bytes(read), nam)
    _same(got, _py_extend(ref, bytes(read), nam))
    assert got["done"] == done


def test_n_and_lower_case_bases_compare_as_bytes():
    ref = bytearray(_genome(300, 7))
    ref[150] = ord("N")
    read = bytearray(ref[100:250])
    read[60] = ord("n")        # n against N: a mismatch (bytes differ)
    read[10] = ord(read[10:11].decode().lower())
    for nam in (_nam(70, 140, 170, 240), _nam(10, 80, 110, 180, is_rc=1)):
        got = _oracle_one(bytes(ref), bytes(read), nam)
        _same(got, _py_extend(bytes(ref), bytes(read), nam))


def test_random_cases_against_the_python_restatement():
    rng = np.random.default_rng(8)
    ref = bytearray(_genome(3000, 9))
    for p in rng.choice(3000, 15, replace=False):
        ref[p] = ord("N")
    ref = bytes(ref)
    n_done = n_flip = 0
    for t in range(300):
        L = int(rng.integers(60, 260))
        a = int(rng.integers(0, 3000 - L))
        read = bytearray(ref[a:a + L])
        for _ in range(int(rng.integers(0, 8))):
            read[int(rng.integers(0, L))] = int(rng.choice(np.frombuffer(b"ACGTNacgt", np.uint8)))
        strand = int(rng.integers(0, 2))
        read = bytes(read) if strand == 0 else _revcomp(bytes(read))
        # (qs, qe) in the view of the read that matches the reference (forward for
        # strand 0, reverse complement for strand 1) against [a + qs, a + qe)
        qs = int(rng.integers(0, L - K - 1))
        qe = int(rng.integers(qs + K, L + 1))
        shift = int(rng.integers(-2, 3)) if t % 5 == 0 else 0
        rs = max(0, a + qs + shift)
        re_ = min(len(ref), rs + (qe - qs))
        if re_ - rs < K:
            continue
        if t % 4:
            nam = _nam(qs, qe, rs, re_, is_rc=strand)
        else:   # the other strand claimed, in its mirrored coordinates (a false reverse hit)
            nam = _nam(L - qe, L - qs, rs, re_, is_rc=1 - strand)
        got = _oracle_one(ref, read, nam)
        py = _py_extend(ref, read, nam)
        _same(got, py)
        n_done += py["done"]
        n_flip += py["is_rc"] != int(nam["is_rc"])
    assert n_done > 50 and n_flip > 10


def test_align_parameters_are_used():
    ref = _genome(300, 10)
    read = bytearray(ref[50:200])
    read[20] = ord("A") if read[20] != ord("A") else ord("T")
    nam = _nam(40, 100, 90, 150)
    got = _oracle_one(ref, bytes(read), nam, match=1, mismatch=4, gap_open=6, gap_extend=1, end_bonus=5)
    _same(got, _py_extend(ref, bytes(read), nam, match=1, mismatch=4, end_bonus=5))


def test_nams_outside_their_read_or_contig_are_refused():
    ref = _genome(300, 11)
    read = ref[50:200]
    for nam in (_nam(140, 160, 190, 210), _nam(10, 25, 60, 75), _nam(10, 60, 280, 330), _nam(10, 60, 60, 110, ref_id=1)):
        with pytest.raises(ValueError):
            _oracle_one(ref, read, nam)


@pytest.mark.gpu
def test_seed_extension_against_oracle():
    """gbsa_extend_seeds_device equals the oracle on the best NAMs of mapped reads of
    both orientations, on the same NAMs claiming the wrong orientation, and on reads
    with N and lower-case bases; a NAM outside its contig fails the call, which stays
    usable."""
    import torch
    from gpu_index_test_gb300 import native, synth
    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=95))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=3000, seed=96))
    seq = reads.seq.copy()
    rng = np.random.default_rng(97)
    seq[rng.choice(len(seq), len(seq) // 500, replace=False)] = ord("N")
    low = rng.choice(len(seq), len(seq) // 200, replace=False)
    seq[low] = np.frombuffer(bytes(seq[low]).lower(), np.uint8)
    reads.seq = seq
    idx = native.Index.build(native.params_from_read_length(150), g)
    nams, offs, _, _ = native.Mapper(idx, abi.map_options(rescue_level=2)).map_reads(reads)
    sel, owner = [], []
    for r in range(reads.n):
        a, b = int(offs[r]), int(offs[r + 1])
        for j in range(a, min(b, a + 3)):
            sel.append(j)
            owner.append(r)
    nn = nams[np.array(sel)].copy()
    owner = np.array(owner, np.uint32)
    wrong = nn.copy()                          # the wrong orientation in the other strand's coordinates
    L = reads.lengths[owner].astype(np.int32)
    wrong["is_rc"] = 1 - wrong["is_rc"]
    wrong["query_start"], wrong["query_end"] = L - nn["query_end"], L - nn["query_start"]
    all_nams = np.concatenate([nn, wrong])
    all_owner = np.concatenate([owner, owner])
    k = native.params_from_read_length(150).k
    ref = oracle_py.extend_seeds(g.seq, g.offsets, g.lengths, reads.seq, reads.offsets, reads.lengths, all_nams,
                                 all_owner, k)
    dev = torch.device("cuda:0")

    def up(a, dt=None):
        a = np.ascontiguousarray(a if dt is None else a.astype(dt))
        return torch.from_numpy(a.view(np.uint8).copy()).to(dev)

    d = [up(g.seq), up(g.offsets, np.uint64), up(g.lengths, np.uint64), up(reads.seq), up(reads.offsets, np.uint64),
         up(reads.lengths, np.uint32), up(all_nams), up(all_owner, np.uint32)]
    out = torch.zeros(len(all_nams) * abi.SEED_ALIGNMENT.itemsize, dtype=torch.uint8, device=dev)
    native.extend_seeds_device(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), len(g.lengths), d[3].data_ptr(),
                               d[4].data_ptr(), d[5].data_ptr(), reads.n, d[6].data_ptr(), d[7].data_ptr(),
                               len(all_nams), k, out.data_ptr())
    got = out.cpu().numpy().view(abi.SEED_ALIGNMENT)
    assert (got == ref).all(), np.nonzero(got != ref)[0][:10]
    half = len(nn)
    assert ref["done"][:half].mean() > 0.5 and (ref["is_rc"][half:] == ref["is_rc"][:half]).mean() > 0.9
    assert ((ref["done"] == 1) & (ref["edit_distance"] > 0)).any() and (ref["done"] == 0).any()
    # a NAM past its contig's end fails the call; the next call works
    bad = all_nams[:4].copy()
    bad["ref_end"][2] = int(g.lengths[bad["ref_id"][2]]) + 5
    d_bad = up(bad)
    with pytest.raises(native.GbsaError):
        native.extend_seeds_device(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), len(g.lengths),
                                   d[3].data_ptr(), d[4].data_ptr(), d[5].data_ptr(), reads.n, d_bad.data_ptr(),
                                   d[7].data_ptr(), 4, k, out.data_ptr())
    native.extend_seeds_device(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), len(g.lengths), d[3].data_ptr(),
                               d[4].data_ptr(), d[5].data_ptr(), reads.n, d[6].data_ptr(), d[7].data_ptr(),
                               len(all_nams), k, out.data_ptr())
    assert (out.cpu().numpy().view(abi.SEED_ALIGNMENT) == ref).all()


# ---- mate rescue: rescue_mate_part with has_shared_substring (main.cu:695-757, 657-693) ----

_MOD8 = [0, 0, 0, 1, 3, 0, 0, 2]   # nt2int_mod8 (main.cu:645-654)


def _py_shared(read: bytes, ref: bytes, k):
    sub, step = 2 * k // 3, k // 3

    def h(s, i):
        v = 0
        for j in range(sub):
            v = ((v << 2) | _MOD8[s[i + j] % 8]) & 0xFFFFFFFF
        return v
    h0 = {h(read, i) for i in range(0, max(0, len(read) - sub), step)}
    return any(h(ref, i) in h0 for i in range(0, max(0, len(ref) - sub)))


def _py_rescue(ref: bytes, mate: bytes, nam, k=K, mu=300.0, sigma=100.0):
    L = len(mate)
    spread = np.float32(5.0 * float(np.float32(sigma)) + float(np.float32(mu)))   # one fused multiply-add
    qs, qe, rs, re_ = (int(nam[f]) for f in ("query_start", "query_end", "ref_start", "ref_end"))
    if int(nam["is_rc"]):
        seq = mate
        a = int(np.float32(np.float32(rs - qs) - spread))
        b = rs - qs + L // 2
    else:
        seq = _revcomp(mate)
        a = re_ + (L - qe) - L // 2
        b = int(np.float32(np.float32(re_ + (L - qe)) + spread))
    ws, we = max(0, min(a, len(ref))), min(len(ref), max(0, b))
    unaligned = we < ws + k or not _py_shared(seq, ref[ws:we], k)
    return dict(ref_id=int(nam["ref_id"]), window_start=ws, window_end=we, edit_distance=L if unaligned else 0,
                is_rc=int(nam["is_rc"]), done=int(unaligned), is_unaligned=int(unaligned))


def _oracle_rescue(ref: bytes, mate: bytes, nam, **kw):
    return oracle_py.rescue_mates(np.frombuffer(ref, np.uint8), [0], [len(ref)], np.frombuffer(mate, np.uint8), [0],
                                  [len(mate)], np.array([nam]), [0], K, **kw)[0]


def test_mate_rescue_random_cases():
    rng = np.random.default_rng(20)
    ref = bytearray(_genome(6000, 21))
    for p in rng.choice(6000, 20, replace=False):
        ref[p] = ord("N") if p % 2 else ord(chr(ref[p]).lower())
    ref = bytes(ref)
    seen = set()
    for t in range(200):
        L = int(rng.integers(60, 200))
        a = int(rng.integers(0, 5000))
        ins = int(rng.integers(L, 600))
        mate = _revcomp(ref[a + ins - L:a + ins]) if a + ins <= len(ref) else _genome(L, t)
        if t % 3 == 0:
            mate = _genome(L, 1000 + t)           # a mate from elsewhere: usually nothing shared
        qs = int(rng.integers(0, 40))
        nam = _nam(qs, qs + 40, a + qs, a + qs + 40, is_rc=int(rng.integers(0, 2)))
        got = _oracle_rescue(ref, mate, nam)
        _same(got, _py_rescue(ref, mate, nam))
        seen.add(int(got["done"]))
    assert seen == {0, 1}


def test_mate_rescue_window_clamps_and_float_positions():
    """Windows clamp to the contig (shorter than k: unaligned), and positions past 2^24
    go through float as in the reference (the window bound rounds to a float)."""
    ref = _genome(3000, 22)
    mate = ref[2800:2950]
    for nam in (_nam(0, 40, 2950, 2990, is_rc=0), _nam(10, 50, 5, 45, is_rc=1), _nam(0, 40, 1000, 1040, is_rc=0)):
        _same(_oracle_rescue(ref, mate, nam), _py_rescue(ref, mate, nam))
    big = np.random.default_rng(23).choice(np.frombuffer(b"ACGT", np.uint8), 20_000_001).tobytes()
    mate = _revcomp(big[19_000_300:19_000_450])
    for nam in (_nam(3, 43, 19_000_003, 19_000_043, is_rc=0), _nam(7, 47, 17_777_778, 17_777_818, is_rc=1)):
        got = _oracle_rescue(big, mate, nam)
        _same(got, _py_rescue(big, mate, nam))
    got = _oracle_rescue(big, mate, _nam(7, 47, 17_777_778, 17_777_818, is_rc=1))
    # ref_start - query_start = 17_777_771 is odd, and floats between 2^24 and 2^25 are even
    assert got["window_start"] == int(np.float32(np.float32(17_777_771) - np.float32(800)))
    assert got["window_start"] != 17_777_771 - 800


def test_mate_rescue_parameters_and_limits():
    ref = _genome(3000, 24)
    mate = _revcomp(ref[900:1050])
    nam = _nam(0, 40, 600, 640, is_rc=0)
    for mu, sigma in ((300.0, 100.0), (250.0, 33.3), (500.0, 80.0)):
        _same(_oracle_rescue(ref, mate, nam, mu=mu, sigma=sigma), _py_rescue(ref, mate, nam, mu=mu, sigma=sigma))
    with pytest.raises(ValueError):   # 82 sampled substrings in a 500-base mate
        _oracle_rescue(ref, _genome(500, 25), nam)
    with pytest.raises(ValueError):
        _oracle_rescue(ref, mate, _nam(0, 40, 600, 640, ref_id=3))


@pytest.mark.gpu
def test_mate_rescue_against_oracle():
    """gbsa_rescue_mates_device equals the oracle for each pair's mates rescued from the
    other end's best NAM, and for mates paired with a read from elsewhere."""
    import torch
    from gpu_index_test_gb300 import native, synth
    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=98))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=3000, seed=99))
    idx = native.Index.build(native.params_from_read_length(150), g)
    nams, offs, _, _ = native.Mapper(idx, abi.map_options(rescue_level=2)).map_reads(reads)
    cnt = np.diff(offs.astype(np.int64))
    ends = np.nonzero(cnt > 0)[0]
    best = nams[offs[:-1][ends].astype(np.int64)]
    mates = (ends ^ 1).astype(np.uint32)                 # mates are interleaved
    other = np.random.default_rng(100).integers(0, reads.n, len(ends)).astype(np.uint32)
    all_nams = np.concatenate([best, best])
    all_mates = np.concatenate([mates, other])
    k = native.params_from_read_length(150).k
    ref = oracle_py.rescue_mates(g.seq, g.offsets, g.lengths, reads.seq, reads.offsets, reads.lengths, all_nams,
                                 all_mates, k)
    dev = torch.device("cuda:0")

    def up(a, dt=None):
        a = np.ascontiguousarray(a if dt is None else a.astype(dt))
        return torch.from_numpy(a.view(np.uint8).copy()).to(dev)

    d = [up(g.seq), up(g.offsets, np.uint64), up(g.lengths, np.uint64), up(reads.seq), up(reads.offsets, np.uint64),
         up(reads.lengths, np.uint32), up(all_nams), up(all_mates, np.uint32)]
    out = torch.zeros(len(all_nams) * abi.MATE_RESCUE.itemsize, dtype=torch.uint8, device=dev)
    native.rescue_mates_device(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), len(g.lengths), d[3].data_ptr(),
                               d[4].data_ptr(), d[5].data_ptr(), reads.n, d[6].data_ptr(), d[7].data_ptr(),
                               len(all_nams), k, out.data_ptr())
    got = out.cpu().numpy().view(abi.MATE_RESCUE)
    assert (got == ref).all(), np.nonzero(got != ref)[0][:10]
    half = len(best)
    assert ref["done"][:half].mean() < 0.2 and ref["done"][half:].mean() > 0.5


@pytest.mark.parametrize("k", [9, 32])
def test_other_k_values(k):
    """k = 32 makes the rescue's substrings 21 bases (their 32-bit hashes keep the last
    16), k = 9 makes them 6 bases; the extension's k-mer checks use k bases."""
    rng = np.random.default_rng(30 + k)
    ref = _genome(4000, 31 + k)
    for t in range(40):
        L = int(rng.integers(80, 180))
        a = int(rng.integers(0, 3000))
        read = bytearray(ref[a:a + L])
        for _ in range(int(rng.integers(0, 4))):
            read[int(rng.integers(0, L))] = ord("ACGT"[int(rng.integers(0, 4))])
        read = bytes(read)
        qs = int(rng.integers(0, L - k - 1))
        nam = _nam(qs, qs + k + int(rng.integers(0, L - k - qs)), a + qs, 0, is_rc=int(rng.integers(0, 2)))
        nam["ref_end"] = nam["ref_start"] + (nam["query_end"] - nam["query_start"])
        got = oracle_py.extend_seeds(np.frombuffer(ref, np.uint8), [0], [len(ref)], np.frombuffer(read, np.uint8),
                                     [0], [L], np.array([nam]), [0], k)[0]
        _same(got, _py_extend(ref, read, nam, k=k))
        mate = _revcomp(ref[a + 200:a + 200 + L]) if t % 2 else _genome(L, 500 + t)
        got = oracle_py.rescue_mates(np.frombuffer(ref, np.uint8), [0], [len(ref)], np.frombuffer(mate, np.uint8),
                                     [0], [L], np.array([nam]), [0], k)[0]
        _same(got, _py_rescue(ref, mate, nam, k=k))


@pytest.mark.gpu
@pytest.mark.parametrize("k", [9, 32])
def test_other_k_values_on_the_gpu(k):
    """The two device entry points at k = 9 and k = 32 equal the oracle."""
    import torch
    from gpu_index_test_gb300 import native
    rng = np.random.default_rng(60 + k)
    ref = _genome(20000, 61 + k)
    reads, nams, mates = [], [], []
    for t in range(300):
        L = int(rng.integers(80, 180))
        a = int(rng.integers(0, 19000 - L))
        read = bytearray(ref[a:a + L])
        for _ in range(int(rng.integers(0, 4))):
            read[int(rng.integers(0, L))] = ord("ACGT"[int(rng.integers(0, 4))])
        reads.append(bytes(read) if t % 3 else _revcomp(bytes(read)))
        qs = int(rng.integers(0, L - k - 1))
        qe = qs + k + int(rng.integers(0, L - k - qs))
        nams.append(_nam(qs, qe, a + qs, a + qe, is_rc=int(rng.integers(0, 2))))
        mates.append((t + 1) % 300)
    seq = np.frombuffer(b"".join(reads), np.uint8)
    lens = np.array([len(r) for r in reads], np.uint32)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.uint64)
    nn = np.array(nams)
    own = np.arange(300, dtype=np.uint32)
    mt = np.array(mates, np.uint32)
    refa = np.frombuffer(ref, np.uint8)
    want_e = oracle_py.extend_seeds(refa, [0], [len(ref)], seq, offs, lens, nn, own, k)
    want_r = oracle_py.rescue_mates(refa, [0], [len(ref)], seq, offs, lens, nn, mt, k)
    dev = torch.device("cuda:0")
    up = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(dev)
    d = [up(refa), up(np.array([0], np.uint64)), up(np.array([len(ref)], np.uint64)), up(seq), up(offs), up(lens),
         up(nn), up(own), up(mt)]
    e = torch.zeros(300 * abi.SEED_ALIGNMENT.itemsize, dtype=torch.uint8, device=dev)
    r = torch.zeros(300 * abi.MATE_RESCUE.itemsize, dtype=torch.uint8, device=dev)
    args = [d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), 1, d[3].data_ptr(), d[4].data_ptr(), d[5].data_ptr(),
            300, d[6].data_ptr()]
    native.extend_seeds_device(*args, d[7].data_ptr(), 300, k, e.data_ptr())
    native.rescue_mates_device(*args, d[8].data_ptr(), 300, k, r.data_ptr())
    assert (e.cpu().numpy().view(abi.SEED_ALIGNMENT) == want_e).all()
    assert (r.cpu().numpy().view(abi.MATE_RESCUE) == want_r).all()
    assert want_e["done"].any()
