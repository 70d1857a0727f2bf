"""ctypes mirrors of the records declared in include/gbsa.h.

The layouts are byte-identical to the reference structs (RefRandstrobe,
step2/randstrobes.hpp:65-94; QueryRandstrobe, step2/randstrobes.hpp:96-101; Nam,
step2/my_struct.hpp:48-62) so numpy views of these arrays can be handed to either
side without conversion.
"""
import ctypes as C

import numpy as np

GBSA_OK = 0
GBSA_ERR_PARAM = 1
GBSA_ERR_CUDA = 2
GBSA_ERR_NOMEM = 3
GBSA_ERR_INDEX_FILE = 4
GBSA_ERR_CAPACITY = 5
GBSA_ERR_READ_TOO_LONG = 6
GBSA_ERR_NO_DEVICE = 7
GBSA_ERR_DEVICE_STATUS = 8

GBSA_DEFAULT = -2147483648
GBSA_MAX_READ_LEN = 4096

GBSA_SORT_SCORE = 0
GBSA_SORT_REF_MATE2 = 1
GBSA_SORT_REF_MATE1 = 2
GBSA_PAIRS_INTERLEAVED = 0
GBSA_PAIRS_HALVES = 1


class Params(C.Structure):
    _fields_ = [
        ("canonical_read_length", C.c_int32),
        ("k", C.c_int32),
        ("s", C.c_int32),
        ("t_syncmer", C.c_int32),
        ("l", C.c_int32),
        ("u", C.c_int32),
        ("q", C.c_uint64),
        ("max_dist", C.c_int32),
        ("w_min", C.c_uint32),
        ("w_max", C.c_uint32),
        ("_pad", C.c_int32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("_")}


class IndexInfo(C.Structure):
    _fields_ = [
        ("size", C.c_uint64),
        ("bits", C.c_int32),
        ("filter_cutoff", C.c_uint32),
        ("tot_strobemer_count", C.c_uint64),
        ("tot_occur_once", C.c_uint64),
        ("tot_high_ab", C.c_uint64),
        ("tot_mid_ab", C.c_uint64),
        ("index_cutoff", C.c_uint64),
        ("distinct_strobemers", C.c_uint64),
    ]


class MapOptions(C.Structure):
    _fields_ = [
        ("rescue_level", C.c_int32),
        ("rescue_count_cap", C.c_uint32),
        ("sort_mode", C.c_int32),
        ("_pad", C.c_int32),
    ]


class BatchConfig(C.Structure):
    """gbsa_batch_config: shape of the batched form's kernels (see include/gbsa.h)."""
    _fields_ = [
        ("seed_variant", C.c_int32),
        ("lane_max_hits", C.c_uint32),
        ("sort_variant", C.c_int32),
        ("chunk_reads", C.c_uint32),
        ("lane_variant", C.c_int32),
        ("warp_variant", C.c_int32),
        ("rescue_block_hits", C.c_uint32),
        ("_reserved", C.c_uint32),
    ]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class ReplayRequest(C.Structure):
    """gbsa_replay_request: reads [start, start + n_reads) of the pool at at_us."""
    _fields_ = [("at_us", C.c_double), ("start", C.c_uint64), ("n_reads", C.c_uint32), ("_pad", C.c_uint32)]


REPLAY_REQUEST = np.dtype([("at_us", "<f8"), ("start", "<u8"), ("n_reads", "<u4"), ("_pad", "<u4")])


class ServerConfig(C.Structure):
    """gbsa_server_config."""
    _fields_ = [
        ("slots", C.c_uint32),
        ("batch_reads", C.c_uint32),
        ("batch_bases", C.c_uint64),
        ("memory_budget", C.c_uint64),
    ]


SEED_VARIANTS = 6   # shapes of the batched form's seeding + lookup kernel


def batch_config(seed_variant=0, lane_max_hits=160, sort_variant=0, chunk_reads=1 << 19, lane_variant=0,
                 warp_variant=0, rescue_block_hits=4000):
    return BatchConfig(seed_variant, lane_max_hits, sort_variant, chunk_reads, lane_variant, warp_variant,
                       rescue_block_hits, 0)


REF_RANDSTROBE = np.dtype([("hash", "<u8"), ("position", "<u4"), ("packed", "<u4")])
QUERY_RANDSTROBE = np.dtype(
    [("hash", "<u8"), ("start", "<u4"), ("end", "<u4"), ("is_reverse", "u1"), ("_pad", "u1", (7,))]
)
NAM = np.dtype(
    [
        ("nam_id", "<i4"),
        ("query_start", "<i4"),
        ("query_end", "<i4"),
        ("query_prev_hit_startpos", "<i4"),
        ("ref_start", "<i4"),
        ("ref_end", "<i4"),
        ("ref_prev_hit_startpos", "<i4"),
        ("n_hits", "<i4"),
        ("ref_id", "<i4"),
        ("score", "<f4"),
        ("is_rc", "u1"),
        ("_pad", "u1", (3,)),
    ]
)
assert REF_RANDSTROBE.itemsize == 16 and QUERY_RANDSTROBE.itemsize == 24 and NAM.itemsize == 44
# gbsa_nam_pair: a scored pair of NAMs (indices into the mates' NAM lists, -1: absent)
NAM_PAIR = np.dtype([("score", "<i4"), ("i1", "<i4"), ("i2", "<i4")])
GBSA_NAM_PAIRS_TOP_K = 40

# gbsa_align_params (AlignmentParameters, step2/aligner.hpp:11-18) and its command-line
# defaults -A 2 -B 8 -O 12 -E 1 --end-bonus 10 (step2/cmdline.hpp:46-50).
ALIGN_PARAMS = np.dtype([("match", "<i4"), ("mismatch", "<i4"), ("gap_open", "<i4"), ("gap_extend", "<i4"),
                         ("end_bonus", "<i4")])
DEFAULT_ALIGN = (2, 8, 12, 1, 10)

# gbsa_seed_alignment: one NAM's seed extension.
SEED_ALIGNMENT = np.dtype([("ref_id", "<i4"), ("ref_start", "<i4"), ("edit_distance", "<i4"), ("global_ed", "<i4"),
                           ("score", "<i4"), ("length", "<i4"), ("query_start", "<i4"), ("query_end", "<i4"),
                           ("is_rc", "u1"), ("done", "u1"), ("consistent", "u1"), ("_pad", "u1")])
assert SEED_ALIGNMENT.itemsize == 36 and ALIGN_PARAMS.itemsize == 20

# gbsa_mate_rescue: one mate-rescue decision.
MATE_RESCUE = np.dtype([("ref_id", "<i4"), ("window_start", "<i4"), ("window_end", "<i4"), ("edit_distance", "<i4"),
                        ("is_rc", "u1"), ("done", "u1"), ("is_unaligned", "u1"), ("_pad", "u1")])
assert MATE_RESCUE.itemsize == 20

# gbsa_align_step / gbsa_pair_plan: the alignment orchestration's step lists
GBSA_STEP_EXTEND, GBSA_STEP_RESCUE = 0, 1
ALIGN_STEP = np.dtype([("pair", "<u4"), ("read", "<u4"), ("nam_read", "<u4"), ("nam", "<u4"), ("kind", "u1"),
                       ("is_read1", "u1"), ("_pad", "u1", (2,))])
PAIR_PLAN = np.dtype([("type", "u1"), ("mapq1", "u1"), ("mapq2", "u1"), ("_pad", "u1"), ("type4_loop_size", "<i4"),
                      ("first_step", "<u4"), ("n_steps", "<u4")])
assert ALIGN_STEP.itemsize == 20 and PAIR_PLAN.itemsize == 16


def align_params(match=2, mismatch=8, gap_open=12, gap_extend=1, end_bonus=10):
    return np.array([(match, mismatch, gap_open, gap_extend, end_bonus)], ALIGN_PARAMS)

# Fields of a NAM that results are compared on (nam_id and the two prev-hit
# positions are internal to the merge).
NAM_COMPARED = ("ref_id", "query_start", "query_end", "ref_start", "ref_end", "n_hits", "score", "is_rc")


def ptr(a, ctype=C.c_void_p):
    """Pointer to a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return C.cast(a.ctypes.data, ctype)


def map_options(rescue_level=2, rescue_count_cap=1000, sort_mode=GBSA_SORT_SCORE):
    o = MapOptions()
    o.rescue_level = rescue_level
    o.rescue_count_cap = rescue_count_cap
    o.sort_mode = sort_mode
    return o
