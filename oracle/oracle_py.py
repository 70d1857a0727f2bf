"""ctypes wrapper of oracle/liboracle.so — TEST INFRASTRUCTURE ONLY.

The CPU restatement of the reference path that the CUDA path is checked against.
Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg only.
"""
import ctypes as C
import os

import numpy as np

from gpu_index_test_gb300 import abi
from gpu_index_test_gb300._build_paths import ORACLE_SO

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            raise RuntimeError(f"oracle library missing: {ORACLE_SO} (run __graft_entry__.build())")
        L = C.CDLL(ORACLE_SO)
        P = C.POINTER(abi.Params)
        L.oracle_xxh64.restype = C.c_uint64
        L.oracle_xxh64.argtypes = [C.c_uint64]
        L.oracle_params_from_read_length.restype = C.c_int
        L.oracle_params_from_read_length.argtypes = [C.c_int] * 7 + [P]
        L.oracle_pick_bits.restype = C.c_int
        L.oracle_pick_bits.argtypes = [P, C.c_uint64]
        L.oracle_syncmers.restype = C.c_int64
        L.oracle_syncmers.argtypes = [P, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint64]
        L.oracle_randstrobes_query.restype = C.c_int64
        L.oracle_randstrobes_query.argtypes = [P, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64]
        L.oracle_index_build.restype = C.c_void_p
        L.oracle_index_build.argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_float]
        L.oracle_index_load.restype = C.c_void_p
        L.oracle_index_load.argtypes = [P, C.c_void_p, C.c_uint64, C.c_void_p, C.c_int, C.c_uint32]
        L.oracle_index_free.restype = None
        L.oracle_index_free.argtypes = [C.c_void_p]
        L.oracle_index_info.restype = None
        L.oracle_index_info.argtypes = [C.c_void_p, C.POINTER(abi.IndexInfo)]
        L.oracle_index_randstrobes.restype = C.c_void_p
        L.oracle_index_randstrobes.argtypes = [C.c_void_p]
        L.oracle_index_starts.restype = C.c_void_p
        L.oracle_index_starts.argtypes = [C.c_void_p]
        L.oracle_index_write_sti.restype = C.c_int
        L.oracle_index_write_sti.argtypes = [C.c_void_p, C.c_char_p]
        L.oracle_find.restype = C.c_uint64
        L.oracle_find.argtypes = [C.c_void_p, C.c_uint64]
        L.oracle_get_count.restype = C.c_uint32
        L.oracle_get_count.argtypes = [C.c_void_p, C.c_uint64]
        L.oracle_is_filtered.restype = C.c_int
        L.oracle_is_filtered.argtypes = [C.c_void_p, C.c_uint64]
        L.oracle_find_nams.restype = C.c_int64
        L.oracle_find_nams.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.POINTER(C.c_float)]
        L.oracle_find_nams_rescue.restype = C.c_int64
        L.oracle_find_nams_rescue.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint64]
        L.oracle_sort_nams.restype = None
        L.oracle_sort_nams.argtypes = [C.c_void_p, C.c_uint64, C.c_int]
        L.oracle_classify_pairs.restype = C.c_int
        L.oracle_classify_pairs.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_float, C.c_float,
                                            C.c_float, C.c_void_p]
        L.oracle_nam_pairs.restype = C.c_int
        L.oracle_nam_pairs.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_float, C.c_float,
                                       C.c_uint32, C.c_void_p, C.c_void_p]
        vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
        L.oracle_extend_seeds.restype = C.c_int
        L.oracle_extend_seeds.argtypes = [vp, vp, vp, u32, vp, vp, vp, u32, vp, vp, u64, C.c_int, vp, vp]
        L.oracle_rescue_mates.restype = C.c_int
        L.oracle_rescue_mates.argtypes = [vp, vp, vp, u32, vp, vp, vp, u32, vp, vp, u64, C.c_int, C.c_float,
                                          C.c_float, vp]
        L.oracle_map_reads.restype = C.c_int
        L.oracle_map_reads.argtypes = [C.c_void_p, C.POINTER(abi.MapOptions), C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_plan_pairs.restype = C.c_int64
        L.oracle_plan_pairs.argtypes = [vp, vp, u32, C.c_int, vp, vp, vp, u32, C.c_float, vp, vp, u64]
        L.oracle_index_verify.restype = C.c_int
        L.oracle_index_verify.argtypes = [P, vp, vp, vp, u32, C.c_float, vp, u64, vp, C.c_int, u32, C.c_int, vp]
        L.oracle_algorithmic_bytes.restype = C.c_int
        L.oracle_algorithmic_bytes.argtypes = [C.c_void_p, C.POINTER(abi.MapOptions), C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64), C.c_int]
        _lib = L
    return _lib


def xxh64(x):
    return lib().oracle_xxh64(int(x))


def params_from_read_length(r, k=abi.GBSA_DEFAULT, s=abi.GBSA_DEFAULT, l=abi.GBSA_DEFAULT, u=abi.GBSA_DEFAULT,
                            c=abi.GBSA_DEFAULT, max_seed_len=abi.GBSA_DEFAULT):
    p = abi.Params()
    rc = lib().oracle_params_from_read_length(r, k, s, l, u, c, max_seed_len, C.byref(p))
    if rc != abi.GBSA_OK:
        raise ValueError("bad parameters")
    return p


def syncmers(p, seq: bytes):
    buf = np.frombuffer(seq, np.uint8) if len(seq) else np.zeros(1, np.uint8)
    cap = max(1, len(seq))
    h = np.zeros(cap, np.uint64)
    pos = np.zeros(cap, np.uint64)
    n = lib().oracle_syncmers(C.byref(p), buf.ctypes.data, len(seq), h.ctypes.data, pos.ctypes.data, cap)
    return h[:n].copy(), pos[:n].copy()


def randstrobes_query(p, seq: bytes):
    buf = np.frombuffer(seq, np.uint8) if len(seq) else np.zeros(1, np.uint8)
    cap = 2 * max(1, len(seq)) + 2
    out = np.zeros(cap, abi.QUERY_RANDSTROBE)
    n = lib().oracle_randstrobes_query(C.byref(p), buf.ctypes.data, len(seq), out.ctypes.data, cap)
    assert n >= 0
    return out[:n].copy()


VERIFY_CHECKS = {0: "equal", 1: "entry count", 2: "entry order", 3: "entry multiset", 4: "bucket table",
                 5: "filter cutoff"}


def verify_index(p, genome, randstrobes, starts, bits, filter_cutoff, f=0.0002, n_threads=0):
    """Checks an index built elsewhere (exported to host arrays) against the restatement
    without building one: (first failed check or "equal", report dict)."""
    rs = np.ascontiguousarray(randstrobes)
    st = np.ascontiguousarray(starts, np.uint64)
    rep = np.zeros(5, np.uint64)
    rc = lib().oracle_index_verify(C.byref(p), genome.seq.ctypes.data,
                                   np.ascontiguousarray(genome.offsets, np.uint64).ctypes.data,
                                   np.ascontiguousarray(genome.lengths, np.uint64).ctypes.data, len(genome.lengths),
                                   f, rs.ctypes.data if len(rs) else None, len(rs), st.ctypes.data, bits,
                                   filter_cutoff, n_threads, rep.ctypes.data)
    return VERIFY_CHECKS.get(rc, str(rc)), {"expected_entries": int(rep[0]), "entries": int(rep[1]),
                                            "first_unordered": int(rep[2]), "expected_filter_cutoff": int(rep[3]),
                                            "first_bucket_diff": int(rep[4])}


class Index:
    def __init__(self, handle, p):
        self.h = handle
        self.params = p

    @classmethod
    def build(cls, p, genome, bits=-1, f=0.0002):
        h = lib().oracle_index_build(C.byref(p), genome.seq.ctypes.data, genome.offsets.ctypes.data,
                                     genome.lengths.ctypes.data, len(genome.lengths), bits, f)
        if not h:
            raise ValueError("bad bits")
        return cls(h, p)

    @classmethod
    def load(cls, p, randstrobes, starts, bits, filter_cutoff):
        randstrobes = np.ascontiguousarray(randstrobes)
        starts = np.ascontiguousarray(starts, np.uint64)
        h = lib().oracle_index_load(C.byref(p), randstrobes.ctypes.data, len(randstrobes), starts.ctypes.data,
                                    bits, filter_cutoff)
        return cls(h, p)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_index_free(self.h)
            self.h = None

    def info(self):
        i = abi.IndexInfo()
        lib().oracle_index_info(self.h, C.byref(i))
        return i

    def randstrobes(self):
        i = self.info()
        if i.size == 0:
            return np.zeros(0, abi.REF_RANDSTROBE)
        a = (C.c_char * (16 * i.size)).from_address(lib().oracle_index_randstrobes(self.h))
        return np.frombuffer(a, abi.REF_RANDSTROBE).copy()

    def starts(self):
        i = self.info()
        n = (1 << i.bits) + 1
        a = (C.c_char * (8 * n)).from_address(lib().oracle_index_starts(self.h))
        return np.frombuffer(a, np.uint64).copy()

    def write_sti(self, path):
        assert lib().oracle_index_write_sti(self.h, path.encode()) == 0

    def find(self, h):
        return lib().oracle_find(self.h, int(h))

    def get_count(self, pos):
        return lib().oracle_get_count(self.h, int(pos))

    def is_filtered(self, pos):
        return bool(lib().oracle_is_filtered(self.h, int(pos)))

    def find_nams(self, queries):
        q = np.ascontiguousarray(queries)
        cap = 64 + 200 * len(q)
        out = np.zeros(cap, abi.NAM)
        fr = C.c_float()
        n = lib().oracle_find_nams(self.h, q.ctypes.data if len(q) else None, len(q), out.ctypes.data, cap, C.byref(fr))
        assert n >= 0
        return out[:n].copy(), fr.value

    def find_nams_rescue(self, queries, rescue_cutoff, count_cap=1000):
        q = np.ascontiguousarray(queries)
        cap = 64 + 2000 * len(q)
        out = np.zeros(cap, abi.NAM)
        n = lib().oracle_find_nams_rescue(self.h, q.ctypes.data if len(q) else None, len(q), rescue_cutoff,
                                          count_cap, out.ctypes.data, cap)
        assert n >= 0
        return out[:n].copy()

    def map_reads(self, reads, opt=None, n_threads=0, capacity=None):
        opt = opt or abi.map_options()
        n = reads.n
        cap = capacity or max(1024, 64 * n)
        while True:
            nams = np.zeros(cap, abi.NAM)
            offs = np.zeros(n + 1, np.uint64)
            frac = np.zeros(n, np.float32)
            resc = np.zeros(n, np.uint8)
            rc = lib().oracle_map_reads(self.h, C.byref(opt), reads.seq.ctypes.data, reads.offsets.ctypes.data,
                                        reads.lengths.ctypes.data, n, nams.ctypes.data, cap, offs.ctypes.data,
                                        frac.ctypes.data, resc.ctypes.data, n_threads)
            if rc == abi.GBSA_ERR_CAPACITY:
                cap = int(offs[-1]) + 16
                continue
            assert rc == 0
            return nams[: int(offs[-1])], offs, frac, resc

    def algorithmic_bytes(self, reads, opt=None, n_threads=0):
        opt = opt or abi.map_options()
        out = C.c_uint64()
        lib().oracle_algorithmic_bytes(self.h, C.byref(opt), reads.seq.ctypes.data, reads.offsets.ctypes.data,
                                       reads.lengths.ctypes.data, reads.n, C.byref(out), n_threads)
        return out.value


def sort_nams(nams, mode=abi.GBSA_SORT_SCORE):
    a = np.ascontiguousarray(nams).copy()
    if len(a):
        lib().oracle_sort_nams(a.ctypes.data, len(a), mode)
    return a


def classify_pairs(nams, offsets, n_pairs, layout=abi.GBSA_PAIRS_INTERLEAVED, dropoff=0.5, mu=300.0, sigma=100.0):
    """gpu_pre_cal_type restated: pair types 0..4 for the sorted NAM lists of 2 * n_pairs ends."""
    a = np.ascontiguousarray(nams)
    o = np.ascontiguousarray(offsets, np.uint64)
    out = np.zeros(max(1, n_pairs), np.uint8)
    assert lib().oracle_classify_pairs(a.ctypes.data if len(a) else None, o.ctypes.data, n_pairs, layout, dropoff,
                                       mu, sigma, out.ctypes.data) == 0
    return out[:n_pairs]


def nam_pairs(nams, offsets, n_pairs, layout=abi.GBSA_PAIRS_INTERLEAVED, mu=300.0, sigma=100.0, max_tries=20):
    """get_best_scoring_nam_pairs_sort3 restated, cut to max_tries: (records of shape
    (n_pairs, max_tries), counts)."""
    a = np.ascontiguousarray(nams)
    o = np.ascontiguousarray(offsets, np.uint64)
    out = np.zeros((max(1, n_pairs), max_tries), abi.NAM_PAIR)
    cnt = np.zeros(max(1, n_pairs), np.uint32)
    assert lib().oracle_nam_pairs(a.ctypes.data if len(a) else None, o.ctypes.data, n_pairs, layout, mu, sigma,
                                  max_tries, out.ctypes.data, cnt.ctypes.data) == 0
    return out[:n_pairs], cnt[:n_pairs]


def plan_pairs(nams, offsets, n_pairs, types, pairs, pair_counts, layout=abi.GBSA_PAIRS_INTERLEAVED, max_tries=20,
               dropoff=0.5):
    """align_PE_part0..4's orchestration restated as step lists: (plans, steps)."""
    a = np.ascontiguousarray(nams)
    o = np.ascontiguousarray(offsets, np.uint64)
    t = np.ascontiguousarray(types, np.uint8)
    jp = np.ascontiguousarray(pairs, abi.NAM_PAIR)
    jc = np.ascontiguousarray(pair_counts, np.uint32)
    plans = np.zeros(max(1, n_pairs), abi.PAIR_PLAN)
    cap = max(1, n_pairs * (2 + 2 * max_tries))
    steps = np.zeros(cap, abi.ALIGN_STEP)
    n = lib().oracle_plan_pairs(a.ctypes.data if len(a) else None, o.ctypes.data, n_pairs, layout, t.ctypes.data,
                                jp.ctypes.data, jc.ctypes.data, max_tries, dropoff, plans.ctypes.data,
                                steps.ctypes.data, cap)
    assert 0 <= n <= cap
    return plans[:n_pairs], steps[:n]


def run_align_steps(ref_seqs, ref_offsets, ref_lengths, read_seqs, read_offsets, read_lengths, nams, offsets, steps,
                    k, mu=300.0, sigma=100.0):
    """A plan's steps through the restated seed extension and mate rescue, as
    gbsa_run_align_steps_device returns them: (extension records, rescue records)."""
    offsets = np.asarray(offsets, np.uint64)
    idx = (offsets[steps["nam_read"].astype(np.int64)] + steps["nam"].astype(np.uint64)).astype(np.int64)
    step_nams = np.ascontiguousarray(np.asarray(nams)[idx]) if len(steps) else np.zeros(0, abi.NAM)
    ext = extend_seeds(ref_seqs, ref_offsets, ref_lengths, read_seqs, read_offsets, read_lengths, step_nams,
                       steps["nam_read"], k)
    resc = np.zeros(len(steps), abi.MATE_RESCUE)
    r = np.nonzero(steps["kind"] == abi.GBSA_STEP_RESCUE)[0]
    if len(r):
        rn = step_nams[r].copy()
        rn["is_rc"] = ext["is_rc"][r]
        rn["query_start"] = ext["query_start"][r]
        rn["query_end"] = ext["query_end"][r]
        resc[r] = rescue_mates(ref_seqs, ref_offsets, ref_lengths, read_seqs, read_offsets, read_lengths, rn,
                               steps["read"][r], k, mu, sigma)
        for f in ("ref_start", "edit_distance", "global_ed", "score", "length", "done"):
            ext[f][r] = 0
    return ext, resc


def extend_seeds(ref_seqs, ref_offsets, ref_lengths, read_seqs, read_offsets, read_lengths, nams, nam_reads, k,
                 params=None):
    """reverse_nam_if_needed + extend_seed_part restated: one abi.SEED_ALIGNMENT record
    per NAM.  Raises ValueError for a NAM outside its read or contig."""
    rs = np.ascontiguousarray(ref_seqs, np.uint8)
    ro = np.ascontiguousarray(ref_offsets, np.uint64)
    rl = np.ascontiguousarray(ref_lengths, np.uint64)
    qs = np.ascontiguousarray(read_seqs, np.uint8)
    qo = np.ascontiguousarray(read_offsets, np.uint64)
    ql = np.ascontiguousarray(read_lengths, np.uint32)
    a = np.ascontiguousarray(nams)
    nr = np.ascontiguousarray(nam_reads, np.uint32)
    p = abi.align_params() if params is None else np.ascontiguousarray(params, abi.ALIGN_PARAMS)
    out = np.zeros(max(1, len(a)), abi.SEED_ALIGNMENT)
    rc = lib().oracle_extend_seeds(rs.ctypes.data, ro.ctypes.data, rl.ctypes.data, len(rl), qs.ctypes.data,
                                   qo.ctypes.data, ql.ctypes.data, len(ql), a.ctypes.data if len(a) else None,
                                   nr.ctypes.data if len(nr) else None, len(a), k, p.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise ValueError("a NAM names a read or contig out of range or leaves its read or contig")
    return out[:len(a)]


def rescue_mates(ref_seqs, ref_offsets, ref_lengths, read_seqs, read_offsets, read_lengths, nams, mate_reads, k,
                 mu=300.0, sigma=100.0):
    """rescue_mate_part with has_shared_substring restated: one abi.MATE_RESCUE record per
    NAM.  Raises ValueError for an out-of-range NAM or a mate with too many substrings."""
    rs = np.ascontiguousarray(ref_seqs, np.uint8)
    ro = np.ascontiguousarray(ref_offsets, np.uint64)
    rl = np.ascontiguousarray(ref_lengths, np.uint64)
    qs = np.ascontiguousarray(read_seqs, np.uint8)
    qo = np.ascontiguousarray(read_offsets, np.uint64)
    ql = np.ascontiguousarray(read_lengths, np.uint32)
    a = np.ascontiguousarray(nams)
    mr = np.ascontiguousarray(mate_reads, np.uint32)
    out = np.zeros(max(1, len(a)), abi.MATE_RESCUE)
    rc = lib().oracle_rescue_mates(rs.ctypes.data, ro.ctypes.data, rl.ctypes.data, len(rl), qs.ctypes.data,
                                   qo.ctypes.data, ql.ctypes.data, len(ql), a.ctypes.data if len(a) else None,
                                   mr.ctypes.data if len(mr) else None, len(a), k, mu, sigma, out.ctypes.data)
    if rc != 0:
        raise ValueError("a NAM names a contig or mate out of range, or its mate has too many substrings")
    return out[:len(a)]
