"""ctypes binding of libgbsa.so (the C-ABI declared in include/gbsa.h).

Mirrors the reference interfaces of the path:
  IndexParameters.from_read_length   step2/indexparameters.cpp:150-182
  StrobemerIndex (populate, find, get_count, is_filtered, read, write)
                                     step2/index.hpp:37-183, step2/index.cu:73-134
  randstrobes_query                  step2/randstrobes.cu:195-241
  find_nams / find_nams_rescue       step2/nam.hpp:11-20
Errors raise GbsaError carrying the C status code (BadParameter → GBSA_ERR_PARAM,
InvalidIndexFile → GBSA_ERR_INDEX_FILE, …).  There is no CPU fallback: when the
library is missing or no GPU is visible, calls fail loudly.
"""
import ctypes as C
import os
import re

import numpy as np

from . import abi
from ._build_paths import GBSA_SO, INCLUDE_DIR

_lib = None


class GbsaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbsa error {code}: {msg}")
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(GBSA_SO):
            raise RuntimeError(f"CUDA library missing: {GBSA_SO} (run __graft_entry__.build())")
        L = C.CDLL(GBSA_SO)
        P = C.POINTER(abi.Params)
        vp, u64, u32, i32 = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int
        proto = {
            "gbsa_last_error": (C.c_char_p, []),
            "gbsa_version": (i32, []),
            "gbsa_launch_count": (u64, []),
            "gbsa_params_from_read_length": (i32, [i32] * 7 + [P]),
            "gbsa_params_make": (i32, [u64, i32, i32, i32, i32, i32, i32, P]),
            "gbsa_pick_bits": (i32, [P, u64]),
            "gbsa_index_build": (i32, [P, vp, vp, vp, u32, i32, C.c_float, C.POINTER(vp)]),
            "gbsa_index_load": (i32, [P, vp, u64, vp, i32, u32, C.POINTER(vp)]),
            "gbsa_index_read_sti": (i32, [C.c_char_p, P, C.POINTER(vp)]),
            "gbsa_index_write_sti": (i32, [vp, C.c_char_p]),
            "gbsa_index_get_info": (i32, [vp, C.POINTER(abi.IndexInfo)]),
            "gbsa_index_get_params": (i32, [vp, P]),
            "gbsa_index_export": (i32, [vp, vp, vp]),
            "gbsa_index_free": (None, [vp]),
            "gbsa_find": (i32, [vp, vp, u64, vp]),
            "gbsa_get_count": (i32, [vp, vp, u64, vp]),
            "gbsa_randstrobes_query": (i32, [P, vp, vp, vp, u32, vp, u64, vp, C.POINTER(u64)]),
            "gbsa_mapper_create": (i32, [vp, C.POINTER(abi.MapOptions), u32, u64, C.POINTER(vp)]),
            "gbsa_mapper_free": (None, [vp]),
            "gbsa_map_reads": (i32, [vp, vp, vp, vp, u32, vp, u64, vp, vp, vp]),
            "gbsa_map_reads_device": (i32, [vp, vp, vp, vp, u32, vp, u64, vp, vp, vp, C.POINTER(u64), vp]),
            "gbsa_find_nams": (i32, [vp, vp, vp, u32, i32, u32, vp, u64, vp, vp]),
            "gbsa_mapper_set_count_bytes": (None, [vp, i32]),
            "gbsa_mapper_last_alg_bytes": (u64, [vp]),
            "gbsa_mapper_last_alg_sectors": (u64, [vp]),
            "gbsa_bench_gather": (i32, [u64, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "gbsa_bench_gather_index": (i32, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.POINTER(C.c_double)]),
            "gbsa_classify_pairs_device": (i32, [vp, vp, u32, i32, C.c_float, C.c_float, C.c_float, vp, vp]),
            "gbsa_nam_pairs_device": (i32, [vp, vp, u32, i32, C.c_float, C.c_float, u32, vp, vp, vp]),
            "gbsa_extend_seeds_device": (i32, [vp, vp, vp, u32, vp, vp, vp, u32, vp, vp, u64, i32, vp, vp, vp]),
            "gbsa_rescue_mates_device": (i32, [vp, vp, vp, u32, vp, vp, vp, u32, vp, vp, u64, i32, C.c_float,
                                               C.c_float, vp, vp]),
            "gbsa_server_create": (i32, [vp, vp, u32, u32, u64, vp]),
            "gbsa_server_create_ex": (i32, [vp, vp, C.POINTER(abi.ServerConfig), vp]),
            "gbsa_server_info": (i32, [vp, C.POINTER(u32), C.POINTER(u64), C.POINTER(u64), C.POINTER(u64),
                                       C.POINTER(u64)]),
            "gbsa_server_stats": (i32, [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
            "gbsa_server_replay": (i32, [vp, vp, vp, vp, vp, u32, u32, vp, u64, vp, vp, vp, u32, vp, vp, vp, vp, vp,
                                         vp, vp, vp]),
            "gbsa_server_submit": (i32, [vp, vp, vp, vp, u32, vp, u64, vp, vp, vp, u64]),
            "gbsa_server_poll": (u32, [vp, vp, vp, vp, u32, i32]),
            "gbsa_server_free": (None, [vp]),
            "gbsa_fastq_parse": (i32, [vp, u64, i32, vp, u64, vp, vp, u32, C.POINTER(u32), C.POINTER(u64),
                                       C.POINTER(u64)]),
            "gbsa_fastq_parse_pairs": (i32, [vp, u64, vp, u64, i32, vp, u64, vp, vp, u32, C.POINTER(u32),
                                             C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
            "gbsa_mapper_set_profile": (i32, [vp, i32]),
            "gbsa_mapper_stage_ms": (i32, [vp, vp, i32]),
            "gbsa_mapper_last_counts": (i32, [vp, vp]),
            "gbsa_randstrobes_query_noalloc": (i32, [P, vp, vp, vp, u32, vp, u64, vp, C.POINTER(u64), vp]),
            "gbsa_mapper_rescue_cycles": (i32, [vp, vp, u32, vp]),
            "gbsa_mapper_nam_cycles": (i32, [vp, vp, u32, vp]),
            "gbsa_mapper_set_pipeline": (i32, [vp, u32]),
            "gbsa_mapper_retries": (u64, [vp]),
            "gbsa_mapper_fused_lookup": (i32, [vp]),
            "gbsa_mapper_set_fuse_limit": (i32, [vp, u64]),
            "gbsa_mapper_set_l2_window": (i32, [vp, i32, C.POINTER(u64)]),
            "gbsa_mapper_set_rescue_block": (i32, [vp, u32]),
            "gbsa_batch_config_default": (i32, [C.POINTER(abi.BatchConfig), C.POINTER(i32)]),
            "gbsa_plan_pairs_device": (i32, [vp, vp, u32, i32, vp, vp, vp, u32, C.c_float, vp, vp, u64,
                                             C.POINTER(u64), vp]),
            "gbsa_run_align_steps_device": (i32, [vp, vp, vp, u32, vp, vp, vp, u32, vp, vp, vp, u64, i32, vp,
                                                  C.c_float, C.c_float, vp, vp, vp]),
            "gbsa_batcher_create": (i32, [vp, C.POINTER(abi.MapOptions), C.POINTER(abi.BatchConfig), u32, u64,
                                          C.POINTER(vp)]),
            "gbsa_batcher_free": (None, [vp]),
            "gbsa_batcher_get_config": (i32, [vp, C.POINTER(abi.BatchConfig)]),
            "gbsa_batcher_stats": (i32, [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
            "gbsa_batcher_set_profile": (i32, [vp, i32]),
            "gbsa_batcher_stage_ms": (i32, [vp, vp, i32]),
            "gbsa_batcher_map_device": (i32, [vp, vp, vp, vp, u32, vp, u32, vp, u64, vp, vp, vp, C.POINTER(u64),
                                              vp]),
            "gbsa_batcher_map": (i32, [vp, vp, vp, vp, u32, vp, u32, vp, u64, vp, vp, vp]),
        }
        for name, (res, args) in proto.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def header_symbols():
    """Function names declared in include/gbsa.h."""
    txt = open(os.path.join(INCLUDE_DIR, "gbsa.h")).read()
    return sorted(set(re.findall(r"\b(gbsa_[a-z0-9_]+)\s*\(", txt)))


def _check(rc):
    if rc != abi.GBSA_OK:
        raise GbsaError(rc, lib().gbsa_last_error().decode())


def launch_count():
    return lib().gbsa_launch_count()


def params_from_read_length(r, k=abi.GBSA_DEFAULT, s=abi.GBSA_DEFAULT, l=abi.GBSA_DEFAULT, u=abi.GBSA_DEFAULT,
                            c=abi.GBSA_DEFAULT, max_seed_len=abi.GBSA_DEFAULT):
    p = abi.Params()
    _check(lib().gbsa_params_from_read_length(r, k, s, l, u, c, max_seed_len, C.byref(p)))
    return p


def params_make(canonical_read_length, k, s, l, u, q, max_dist):
    """Explicit parameters (IndexParameters(r, k, s, l, u, q, max_dist)); q = -1 sets all 64 mask bits."""
    p = abi.Params()
    _check(lib().gbsa_params_make(canonical_read_length, k, s, l, u, q, max_dist, C.byref(p)))
    return p


def bench_gather(buffer_bytes):
    """Random 32 B gather bandwidth over a device buffer: (sectors/s, GB/s)."""
    a, b = C.c_double(), C.c_double()
    _check(lib().gbsa_bench_gather(buffer_bytes, C.byref(a), C.byref(b)))
    return a.value, b.value


def bench_gather_index(index):
    """The lookup's dependent gather pattern (bucket pair, then the bucket's first entry)
    on the index's own buffers: (probes/s, sectors/s, GB/s)."""
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    _check(lib().gbsa_bench_gather_index(index.h, C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


def classify_pairs_device(d_nams, d_nam_offsets, n_pairs, d_types, layout=0, dropoff=0.5, mu=300.0, sigma=100.0,
                          stream=None):
    """Pair types (gpu_pre_cal_type) from device NAM lists; all pointers are device addresses."""
    _check(lib().gbsa_classify_pairs_device(d_nams, d_nam_offsets, n_pairs, layout, dropoff, mu, sigma, d_types,
                                            stream))


def nam_pairs_device(d_nams, d_nam_offsets, n_pairs, d_pairs, d_counts, layout=0, mu=300.0, sigma=100.0,
                     max_tries=20, stream=None):
    """NAM-pair scoring (get_best_scoring_nam_pairs_sort3) from device NAM lists: mate 1
    in GBSA_SORT_REF_MATE1 order, mate 2 in GBSA_SORT_REF_MATE2 order; max_tries records
    per pair into d_pairs and their count into d_counts.  Device addresses."""
    _check(lib().gbsa_nam_pairs_device(d_nams, d_nam_offsets, n_pairs, layout, mu, sigma, max_tries, d_pairs,
                                       d_counts, stream))


def extend_seeds_device(d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs, d_read_offsets,
                        d_read_lengths, n_reads, d_nams, d_nam_reads, n_nams, k, d_out, params=None, stream=None):
    """Seed extension of NAMs (reverse_nam_if_needed + extend_seed_part): one
    gbsa_seed_alignment per NAM into d_out.  Device addresses; params is an
    abi.ALIGN_PARAMS record (host), the reference's defaults when None."""
    p = abi.align_params() if params is None else np.ascontiguousarray(params, abi.ALIGN_PARAMS)
    _check(lib().gbsa_extend_seeds_device(d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs,
                                          d_read_offsets, d_read_lengths, n_reads, d_nams, d_nam_reads, n_nams, k,
                                          p.ctypes.data, d_out, stream))


def rescue_mates_device(d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs, d_read_offsets,
                        d_read_lengths, n_reads, d_nams, d_mate_reads, n_nams, k, d_out, mu=300.0, sigma=100.0,
                        stream=None):
    """Mate rescue (rescue_mate_part with has_shared_substring): one gbsa_mate_rescue per
    NAM into d_out.  Device addresses; mu and sigma are the insert-size estimate (the
    reference's defaults when not given)."""
    _check(lib().gbsa_rescue_mates_device(d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs,
                                          d_read_offsets, d_read_lengths, n_reads, d_nams, d_mate_reads, n_nams, k,
                                          mu, sigma, d_out, stream))


def plan_pairs_device(d_nams, d_nam_offsets, n_pairs, d_types, d_pairs, d_pair_counts, d_plans, d_steps, step_cap,
                      layout=0, max_tries=20, dropoff=0.5, stream=None):
    """The alignment orchestration (align_PE_part0..4) as step lists: plans into d_plans,
    steps into d_steps; returns the step count (raises GbsaError GBSA_ERR_CAPACITY when
    above step_cap).  Device addresses."""
    n = C.c_uint64()
    _check(lib().gbsa_plan_pairs_device(d_nams, d_nam_offsets, n_pairs, layout, d_types, d_pairs, d_pair_counts,
                                        max_tries, dropoff, d_plans, d_steps, step_cap, C.byref(n), stream))
    return n.value


def run_align_steps_device(d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs, d_read_offsets,
                           d_read_lengths, n_reads, d_nams, d_nam_offsets, d_steps, n_steps, k, d_ext, d_resc,
                           params=None, mu=300.0, sigma=100.0, stream=None):
    """Runs a plan's steps: seed extensions into d_ext, mate rescues into d_resc (one
    record of each per step).  Device addresses."""
    p = abi.align_params() if params is None else np.ascontiguousarray(params, abi.ALIGN_PARAMS)
    _check(lib().gbsa_run_align_steps_device(d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs,
                                             d_read_offsets, d_read_lengths, n_reads, d_nams, d_nam_offsets, d_steps,
                                             n_steps, k, p.ctypes.data, mu, sigma, d_ext, d_resc, stream))


def _u8(a):
    a = np.ascontiguousarray(a, np.uint8)
    return a if len(a) else np.zeros(1, np.uint8)


class Index:
    """Device-resident StrobemerIndex."""

    def __init__(self, handle, params):
        self.h = C.c_void_p(handle)
        self.params = params

    @classmethod
    def build(cls, params, genome, bits=-1, f=0.0002):
        h = C.c_void_p()
        _check(lib().gbsa_index_build(C.byref(params), _u8(genome.seq).ctypes.data,
                                      np.ascontiguousarray(genome.offsets, np.uint64).ctypes.data,
                                      np.ascontiguousarray(genome.lengths, np.uint64).ctypes.data,
                                      len(genome.lengths), bits, f, C.byref(h)))
        return cls(h.value, params)

    @classmethod
    def load(cls, params, randstrobes, starts, bits, filter_cutoff):
        rs = np.ascontiguousarray(randstrobes)
        st = np.ascontiguousarray(starts, np.uint64)
        h = C.c_void_p()
        _check(lib().gbsa_index_load(C.byref(params), rs.ctypes.data if len(rs) else None, len(rs), st.ctypes.data,
                                     bits, filter_cutoff, C.byref(h)))
        return cls(h.value, params)

    @classmethod
    def read_sti(cls, path, params):
        h = C.c_void_p()
        _check(lib().gbsa_index_read_sti(path.encode(), C.byref(params), C.byref(h)))
        return cls(h.value, params)

    def write_sti(self, path):
        _check(lib().gbsa_index_write_sti(self.h, path.encode()))

    def free(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().gbsa_index_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def info(self):
        i = abi.IndexInfo()
        _check(lib().gbsa_index_get_info(self.h, C.byref(i)))
        return i

    def export(self):
        i = self.info()
        rs = np.zeros(max(1, i.size), abi.REF_RANDSTROBE)
        st = np.zeros((1 << i.bits) + 1, np.uint64)
        _check(lib().gbsa_index_export(self.h, rs.ctypes.data, st.ctypes.data))
        return rs[: i.size], st

    def find(self, hashes):
        h = np.ascontiguousarray(hashes, np.uint64)
        out = np.zeros(max(1, len(h)), np.uint64)
        _check(lib().gbsa_find(self.h, h.ctypes.data, len(h), out.ctypes.data))
        return out[: len(h)]

    def get_count(self, positions):
        p = np.ascontiguousarray(positions, np.uint64)
        out = np.zeros(max(1, len(p)), np.uint32)
        _check(lib().gbsa_get_count(self.h, p.ctypes.data, len(p), out.ctypes.data))
        return out[: len(p)]


def randstrobes_query(params, reads):
    """Query randstrobes of every read: (records, offsets[n+1])."""
    n = reads.n
    offs = np.zeros(n + 1, np.uint64)
    tot = C.c_uint64()
    cap = int(reads.lengths.sum()) * 2 // 3 + 64
    while True:
        out = np.zeros(max(1, cap), abi.QUERY_RANDSTROBE)
        rc = lib().gbsa_randstrobes_query(C.byref(params), _u8(reads.seq).ctypes.data,
                                          np.ascontiguousarray(reads.offsets, np.uint64).ctypes.data,
                                          np.ascontiguousarray(reads.lengths, np.uint32).ctypes.data, n,
                                          out.ctypes.data, cap, offs.ctypes.data, C.byref(tot))
        if rc == abi.GBSA_ERR_CAPACITY:
            cap = tot.value
            continue
        _check(rc)
        return out[: tot.value], offs


class Mapper:
    """Device work areas for batches of reads through seed → lookup → NAM (+ rescue)."""

    def __init__(self, index, opt=None, max_reads=1 << 20, max_bases=None):
        self.index = index
        self.opt = opt or abi.map_options()
        h = C.c_void_p()
        _check(lib().gbsa_mapper_create(index.h, C.byref(self.opt), max_reads,
                                        max_bases or max_reads * 160, C.byref(h)))
        self.h = h

    def free(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().gbsa_mapper_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def set_count_bytes(self, on=True):
        lib().gbsa_mapper_set_count_bytes(self.h, 1 if on else 0)

    def last_alg_bytes(self):
        return lib().gbsa_mapper_last_alg_bytes(self.h)

    def last_alg_sectors(self):
        """32 B sectors of the lookup's gathers in the last batch (with set_count_bytes)."""
        return lib().gbsa_mapper_last_alg_sectors(self.h)

    STAGES = ("seed_lookup", "seed_long", "lookup_long", "nams", "nams_warp", "rescue", "rescue_sort")

    def set_profile(self, on=True):
        _check(lib().gbsa_mapper_set_profile(self.h, 1 if on else 0))

    def last_counts(self):
        a = np.zeros(7, np.uint64)
        lib().gbsa_mapper_last_counts(self.h, a.ctypes.data)
        return dict(zip(("queries", "hits", "nam_slots", "rescued", "long_reads", "ovf_bytes", "warp_nam_reads"),
                        (int(x) for x in a)))

    def retries(self):
        """Batches run again after a work area grew, since the mapper was created."""
        return int(lib().gbsa_mapper_retries(self.h))

    def rescue_cycles(self, cap=1 << 24):
        """Per rescued read: cycles (total, plan, merge, sort), hit bound, NAMs,
        cycles of the run walks, longest run; and the count of block-sorted reads."""
        a = np.zeros(cap, np.uint64)
        n = (C.c_uint32 * 2)()
        _check(lib().gbsa_mapper_rescue_cycles(self.h, a.ctypes.data, cap, n))
        k = min(cap // 8, n[0])
        return a[: 8 * k].reshape(-1, 8), int(n[1])

    def set_pipeline(self, chunks):
        """Chunks a large map_reads call is cut into for overlapped transfers (1 = off)."""
        _check(lib().gbsa_mapper_set_pipeline(self.h, chunks))

    def nam_cycles(self, cap=1 << 22):
        """Per read of the warp find_nams kernel: (cycles, hits, NAMs, merge cycles)."""
        a = np.zeros(cap, np.uint64)
        n = (C.c_uint32 * 1)()
        _check(lib().gbsa_mapper_nam_cycles(self.h, a.ctypes.data, cap, n))
        k = min(cap // 4, n[0])
        return a[: 4 * k].reshape(-1, 4)

    STAGES_UNFUSED = ("seed", "seed_long", "lookup", "nams", "nams_warp", "rescue", "rescue_sort")

    def set_fuse_limit(self, index_bytes):
        """Largest index (entry bytes) seeded and looked up in one kernel; 0: never."""
        _check(lib().gbsa_mapper_set_fuse_limit(self.h, int(index_bytes)))

    def set_l2_window(self, on=True):
        """Bucket table held in L2 (access-policy window); returns the window's bytes."""
        b = C.c_uint64()
        _check(lib().gbsa_mapper_set_l2_window(self.h, 1 if on else 0, C.byref(b)))
        return b.value

    def set_rescue_block(self, hits):
        """Rescued reads with at least `hits` estimated merge hits are merged by a block
        each (0: every rescued read by one warp)."""
        _check(lib().gbsa_mapper_set_rescue_block(self.h, int(hits)))

    def fused_lookup(self):
        """Whether the last batch ran seeding and lookup as one kernel."""
        return bool(lib().gbsa_mapper_fused_lookup(self.h))

    def stage_ms(self):
        a = np.zeros(7, np.float32)
        lib().gbsa_mapper_stage_ms(self.h, a.ctypes.data, 7)
        return dict(zip(self.STAGES if self.fused_lookup() else self.STAGES_UNFUSED, a.tolist()))

    def map_reads(self, reads, capacity=None):
        n = reads.n
        cap = capacity or max(1024, 24 * n)
        seq = _u8(reads.seq)
        offs_in = np.ascontiguousarray(reads.offsets, np.uint64)
        lens = np.ascontiguousarray(reads.lengths, np.uint32)
        while True:
            nams = np.zeros(cap, abi.NAM)
            offs = np.zeros(n + 1, np.uint64)
            frac = np.zeros(max(1, n), np.float32)
            resc = np.zeros(max(1, n), np.uint8)
            rc = lib().gbsa_map_reads(self.h, seq.ctypes.data, offs_in.ctypes.data, lens.ctypes.data, n,
                                      nams.ctypes.data, cap, offs.ctypes.data, frac.ctypes.data, resc.ctypes.data)
            if rc == abi.GBSA_ERR_CAPACITY:
                cap = int(offs[-1]) + 16
                continue
            _check(rc)
            return nams[: int(offs[-1])], offs, frac[:n], resc[:n]

    def map_reads_device(self, d_seq, d_offsets, d_lengths, n, d_nams, nam_capacity, d_nam_offsets, d_frac=None,
                         d_rescued=None, stream=None):
        """All arguments are device pointers (ints); returns the NAM total."""
        tot = C.c_uint64()
        rc = lib().gbsa_map_reads_device(self.h, d_seq, d_offsets, d_lengths, n, d_nams, nam_capacity, d_nam_offsets,
                                         d_frac, d_rescued, C.byref(tot), stream)
        if rc == abi.GBSA_ERR_CAPACITY:
            return tot.value
        _check(rc)
        return tot.value

    def find_nams(self, queries, q_offsets, rescue=False, rescue_cutoff=0):
        q = np.ascontiguousarray(queries)
        qo = np.ascontiguousarray(q_offsets, np.uint64)
        n = len(qo) - 1
        cap = max(1024, 4 * len(q))
        while True:
            nams = np.zeros(cap, abi.NAM)
            offs = np.zeros(n + 1, np.uint64)
            frac = np.zeros(max(1, n), np.float32)
            rc = lib().gbsa_find_nams(self.h, q.ctypes.data if len(q) else None, qo.ctypes.data, n,
                                      1 if rescue else 0, rescue_cutoff, nams.ctypes.data, cap, offs.ctypes.data,
                                      frac.ctypes.data)
            if rc == abi.GBSA_ERR_CAPACITY:
                cap = int(offs[-1]) + 16
                continue
            _check(rc)
            return nams[: int(offs[-1])], offs, frac[:n]


def batch_config_default():
    """The committed tuned batched-form configuration: (config, loaded from the file)."""
    c, f = abi.BatchConfig(), C.c_int()
    _check(lib().gbsa_batch_config_default(C.byref(c), C.byref(f)))
    return c, bool(f.value)


class Batcher:
    """The batched form: each batch one launch of a captured CUDA graph, seeding and
    lookup in one persistent kernel pulling work items (a read, or both mates of a pair)
    from a device queue."""

    def __init__(self, index, opt=None, config=None, max_reads=1 << 20, max_bases=None):
        self.index = index
        self.opt = opt or abi.map_options()
        h = C.c_void_p()
        _check(lib().gbsa_batcher_create(index.h, C.byref(self.opt), C.byref(config) if config is not None else None,
                                         max_reads, max_bases or max_reads * 160, C.byref(h)))
        self.h = h

    def free(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().gbsa_batcher_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def config(self):
        c = abi.BatchConfig()
        _check(lib().gbsa_batcher_get_config(self.h, C.byref(c)))
        return c

    def stats(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().gbsa_batcher_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"graph_launches": a.value, "captures": b.value, "eager_runs": c.value}

    def set_profile(self, on=True):
        """Stage events inside the batch graph (the graph is captured anew)."""
        _check(lib().gbsa_batcher_set_profile(self.h, 1 if on else 0))

    def stage_ms(self):
        """Stage times of the last device-entry batch (fused seeding + lookup names)."""
        a = np.zeros(7, np.float32)
        lib().gbsa_batcher_stage_ms(self.h, a.ctypes.data, 7)
        return dict(zip(Mapper.STAGES, a.tolist()))

    def map_reads(self, reads, items=None, capacity=None):
        """Host entry point; items (n_items + 1 read starts) may be None."""
        n = reads.n
        cap = capacity or max(1024, 24 * n)
        seq = _u8(reads.seq)
        offs_in = np.ascontiguousarray(reads.offsets, np.uint64)
        lens = np.ascontiguousarray(reads.lengths, np.uint32)
        it = None if items is None else np.ascontiguousarray(items, np.uint32)
        while True:
            nams = np.zeros(cap, abi.NAM)
            offs = np.zeros(n + 1, np.uint64)
            frac = np.zeros(max(1, n), np.float32)
            resc = np.zeros(max(1, n), np.uint8)
            rc = lib().gbsa_batcher_map(self.h, seq.ctypes.data, offs_in.ctypes.data, lens.ctypes.data, n,
                                        None if it is None else it.ctypes.data, 0 if it is None else len(it) - 1,
                                        nams.ctypes.data, cap, offs.ctypes.data, frac.ctypes.data, resc.ctypes.data)
            if rc == abi.GBSA_ERR_CAPACITY:
                cap = int(offs[-1]) + 16
                continue
            _check(rc)
            return nams[: int(offs[-1])], offs, frac[:n], resc[:n]

    def map_reads_device(self, d_seq, d_offsets, d_lengths, n, d_nams, nam_capacity, d_nam_offsets, d_frac=None,
                         d_rescued=None, d_items=None, n_items=0, stream=None):
        """All buffers are device pointers (ints); returns the NAM total."""
        tot = C.c_uint64()
        rc = lib().gbsa_batcher_map_device(self.h, d_seq, d_offsets, d_lengths, n, d_items, n_items, d_nams,
                                           nam_capacity, d_nam_offsets, d_frac, d_rescued, C.byref(tot), stream)
        if rc == abi.GBSA_ERR_CAPACITY:
            return tot.value
        _check(rc)
        return tot.value


class Server:
    """The served form (gbsa_server_*): continuous batching of queued requests onto batch
    slots (batchers) created against a device-memory budget."""

    def __init__(self, index, opt=None, workers=4, max_reads=100_000, max_bases=None, memory_budget=0):
        self.index = index
        self.opt = opt or abi.map_options()
        cfg = abi.ServerConfig(workers, max_reads, max_bases or max_reads * 256, memory_budget)
        h = C.c_void_p()
        _check(lib().gbsa_server_create_ex(index.h, C.byref(self.opt), C.byref(cfg), C.byref(h)))
        self.h = h

    def replay(self, seq_ptr, offsets, lengths, reqs, bufs, nam_cap, max_reads, expected=None):
        """gbsa_server_replay: reqs is an abi.REPLAY_REQUEST array, bufs a list of
        (nams, nam_offsets, frac, rescued) pointer tuples, expected None or pointers
        (nams, nam_offsets, frac, rescued) of the pool's results.  Returns (submit_us,
        done_us, status, mismatch) arrays."""
        n = len(reqs)
        P = C.c_void_p * len(bufs)
        nb = [P(*[b[k] for b in bufs]) for k in range(4)]
        sub, done = np.zeros(n), np.zeros(n)
        st, mis = np.zeros(n, np.int32), np.zeros(n, np.uint8)
        ex = expected or (None, None, None, None)
        rc = lib().gbsa_server_replay(self.h, seq_ptr, offsets.ctypes.data, lengths.ctypes.data, reqs.ctypes.data, n,
                                      len(bufs), nb[0], nam_cap, nb[1], nb[2], nb[3], max_reads, ex[0], ex[1], ex[2],
                                      ex[3], sub.ctypes.data, done.ctypes.data, st.ctypes.data, mis.ctypes.data)
        _check(rc)
        return sub, done, st, mis

    def stats(self):
        """Graph launches, captures and eager batches over all slots since creation."""
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().gbsa_server_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"graph_launches": a.value, "captures": b.value, "eager_runs": c.value}

    def info(self):
        a, b, c, d, e = C.c_uint32(), C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().gbsa_server_info(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d), C.byref(e)))
        return {"slots": a.value, "slot_bytes": b.value, "budget": c.value, "batches": d.value, "requests": e.value}

    def submit(self, seq_ptr, offsets_ptr, lengths_ptr, n, nams_ptr, cap, nam_offsets_ptr, frac_ptr, resc_ptr, tag):
        """All buffers are host pointers kept alive until poll reports `tag`."""
        _check(lib().gbsa_server_submit(self.h, seq_ptr, offsets_ptr, lengths_ptr, n, nams_ptr, cap, nam_offsets_ptr,
                                        frac_ptr, resc_ptr, tag))

    def poll(self, cap=64, wait_ms=-1):
        """Completed requests: list of (tag, status, nam_total)."""
        tags = (C.c_uint64 * cap)()
        st = (C.c_int * cap)()
        tot = (C.c_uint64 * cap)()
        k = lib().gbsa_server_poll(self.h, tags, st, tot, cap, wait_ms)
        return [(int(tags[i]), int(st[i]), int(tot[i])) for i in range(k)]

    def free(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().gbsa_server_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        self.free()


def _fastq_out(total_len):
    seqs = np.zeros(max(1, total_len), np.uint8)
    cap_reads = total_len // 8 + 2
    return seqs, np.zeros(cap_reads + 1, np.uint64), np.zeros(max(1, cap_reads), np.uint32), cap_reads


def fastq_parse(buf, final=True):
    """Complete FASTQ records of a chunk: (Reads, consumed bytes)."""
    from .synth import Reads
    b = np.frombuffer(buf, np.uint8) if isinstance(buf, (bytes, bytearray)) else np.ascontiguousarray(buf, np.uint8)
    seqs, offs, lens, cap = _fastq_out(len(b))
    n, nb, used = C.c_uint32(), C.c_uint64(), C.c_uint64()
    _check(lib().gbsa_fastq_parse(b.ctypes.data if len(b) else None, len(b), 1 if final else 0, seqs.ctypes.data,
                                  len(seqs), offs.ctypes.data, lens.ctypes.data, cap, C.byref(n), C.byref(nb),
                                  C.byref(used)))
    k = n.value
    return Reads(seqs[: nb.value].copy(), offs[:k].copy(), lens[:k].copy()), used.value


def fastq_parse_pairs(buf1, buf2, final=True, out=None):
    """Complete pairs of two mate-file chunks, mates interleaved: (Reads, consumed1, consumed2).
    out = (seqs u8, offsets u64, lengths u32) arrays to parse into (e.g. views of pinned
    memory); the returned Reads then views them."""
    from .synth import Reads
    b1 = np.frombuffer(buf1, np.uint8) if isinstance(buf1, (bytes, bytearray)) else np.ascontiguousarray(buf1, np.uint8)
    b2 = np.frombuffer(buf2, np.uint8) if isinstance(buf2, (bytes, bytearray)) else np.ascontiguousarray(buf2, np.uint8)
    if out is None:
        seqs, offs, lens, cap = _fastq_out(len(b1) + len(b2))
    else:
        seqs, offs, lens = out
        cap = min(len(lens), len(offs) - 1)
    n, nb, u1, u2 = C.c_uint32(), C.c_uint64(), C.c_uint64(), C.c_uint64()
    _check(lib().gbsa_fastq_parse_pairs(b1.ctypes.data if len(b1) else None, len(b1),
                                        b2.ctypes.data if len(b2) else None, len(b2), 1 if final else 0,
                                        seqs.ctypes.data, len(seqs), offs.ctypes.data, lens.ctypes.data, cap,
                                        C.byref(n), C.byref(nb), C.byref(u1), C.byref(u2)))
    k = n.value
    if out is not None:
        return Reads(seqs[: nb.value], offs[:k], lens[:k]), u1.value, u2.value
    return Reads(seqs[: nb.value].copy(), offs[:k].copy(), lens[:k].copy()), u1.value, u2.value

