"""Loaders for the committed golden fixtures (tests/golden/*.npz)."""
import os

import numpy as np

from gpu_index_test_gb300 import abi, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASE_NAMES = ("c1mini", "c2mini", "c4mini")


def unpack_acgt(packed, n):
    codes = np.stack([(packed >> s) & 3 for s in (0, 2, 4, 6)], axis=1).reshape(-1)[:n]
    return np.ascontiguousarray(np.frombuffer(b"ACGT", np.uint8)[codes])


class Case:
    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        self.name = name
        lengths = z["genome_lengths"].astype(np.uint64)
        offsets = np.zeros(len(lengths), np.uint64)
        offsets[1:] = np.cumsum(lengths[:-1])
        self.genome = synth.Genome(unpack_acgt(z["genome_2bit"], int(lengths.sum())), lengths, offsets)
        self.reads = synth.Reads(z["read_seq"], z["read_offsets"].astype(np.uint64), z["read_lengths"].astype(np.uint32))
        self.read_length_param = int(z["read_length_param"])
        self.rescue_level = int(z["rescue_level"])
        self.index_sha256 = bytes(z["index_sha256"]).decode()
        self.sti_sha256 = bytes(z["sti_sha256"]).decode()
        self.bits = int(z["bits"])
        self.filter_cutoff = int(z["filter_cutoff"])
        self.index_size = int(z["index_size"])
        self.ref_queries = z["ref_queries"]
        self.ref_query_offsets = z["ref_query_offsets"]
        self.ref_frac = z["ref_frac"]
        self.ref_rescued = z["ref_rescued"]
        self.ref_nams = z["ref_nams"]
        self.ref_nam_offsets = z["ref_nam_offsets"]

    def read(self, i):
        o, n = int(self.reads.offsets[i]), int(self.reads.lengths[i])
        return bytes(self.reads.seq[o : o + n])


def nams_equal(a, b):
    if len(a) != len(b):
        return False
    return all((a[f] == b[f]).all() for f in abi.NAM_COMPARED)


def kat():
    z = np.load(os.path.join(GOLDEN, "xxh64_kat.npz"))
    return z["inputs"], z["outputs"]


# ---- read-pair rows: the reference's own code after the NAM stage ---------------------
# tests/golden/align_ref.npz holds the outputs of oracle/_ref/ref_align (the reference's
# gpu_sort_nams, gpu_pre_cal_type, get_best_scoring_nam_pairs_sort3 and gpu_align_PE0..4
# from its main.cu, run on the host) for the variants below; the inputs are rebuilt here
# from the NAM fixtures above, so only the outputs are stored.

# Each variant: the source fixture whose first n_pairs read pairs (mates interleaved) and
# reference NAMs are the input, k, max_tries and dropoff.  Pair i loses mate 2's NAMs when
# i % 10 == 3, mate 1's when i % 10 == 7 and both when i % 50 == 25; it keeps only each
# end's best NAM when i % 10 == 5, and when i % 10 == 9 its best NAM and a decoy (the best
# moved 2 kb along its contig, same strand, a third of its hits and score: a second NAM
# that sorts after the best in both mate orders, so that get_mapq's formula runs), so
# that all five pair types occur (the reference classifies on lists sorted by strand
# first, so that with all NAMs both first NAMs are mostly forward and rarely a proper
# pair, type 3); min_span
# drops NAMs shorter than that on the read or on the contig (for k = 32: the reference
# reads k-mers at both ends of a NAM).
ALIGN_VARIANTS = (
    dict(src="c2mini", n_pairs=600, k=20, max_tries=20, dropoff=0.5, min_span=0),
    dict(src="c2mini", n_pairs=600, k=20, max_tries=3, dropoff=0.3, min_span=0),
    dict(src="c2mini", n_pairs=600, k=9, max_tries=20, dropoff=0.5, min_span=0),
    dict(src="c2mini", n_pairs=600, k=32, max_tries=20, dropoff=0.5, min_span=32),
    dict(src="c4mini", n_pairs=1000, k=20, max_tries=20, dropoff=0.5, min_span=0),
)

# One record of the reference's GPUAlignTmpRes lists (is_read1, is_extend_seed,
# done_align, todo_nams, align_res; step2/main.cu:418-477), as oracle/_ref/ref_align
# writes it.
REF_ALIGN_RECORD = np.dtype([("is_read1", "<i4"), ("is_extend_seed", "<i4"), ("done_align", "<i4"), ("nam", abi.NAM),
                             ("ref_id", "<i4"), ("ref_start", "<i4"), ("edit_distance", "<i4"), ("global_ed", "<i4"),
                             ("score", "<i4"), ("length", "<i4"), ("is_rc", "u1"), ("is_unaligned", "u1"),
                             ("gapped", "u1"), ("_pad", "u1")])
ALIGN_FIXTURE = os.path.join(GOLDEN, "align_ref.npz")


def align_inputs(case, v):
    """The variant's input: the NAM lists of its 2 n_pairs read ends in the reference's
    score order (end 2i mate 1 of pair i, end 2i + 1 mate 2) as (nams, offsets), and the
    reads of those ends."""
    lists = []
    for e in range(2 * v["n_pairs"]):
        p, mate = divmod(e, 2)
        a = case.ref_nams[int(case.ref_nam_offsets[e]) : int(case.ref_nam_offsets[e + 1])]
        if p % 50 == 25 or (p % 10 == 3 and mate == 1) or (p % 10 == 7 and mate == 0):
            a = a[:0]
        elif p % 10 == 5:
            a = a[:1]
        elif p % 10 == 9 and len(a):
            a = np.concatenate([a[:1], a[:1]])
            shift = 2000 if int(a[1]["ref_end"]) + 2000 <= int(case.genome.lengths[int(a[1]["ref_id"])]) else -2000
            a[1]["ref_start"] += shift
            a[1]["ref_end"] += shift
            a[1]["n_hits"] //= 3
            a[1]["score"] = np.float32(a[1]["score"] / np.float32(3))
        if v["min_span"]:
            keep = (a["query_end"] - a["query_start"] >= v["min_span"]) & (a["ref_end"] - a["ref_start"] >= v["min_span"])
            a = a[keep]
        lists.append(a)
    offs = np.zeros(len(lists) + 1, np.uint64)
    offs[1:] = np.cumsum([len(a) for a in lists])
    nams = np.ascontiguousarray(np.concatenate(lists))
    return nams, offs, case.reads.subset(np.arange(2 * v["n_pairs"]))


class AlignRef:
    """The reference's outputs for variant i of ALIGN_VARIANTS."""

    def __init__(self, i):
        z = np.load(ALIGN_FIXTURE)
        v = ALIGN_VARIANTS[i]
        pre = f"v{i}_"
        got = tuple(int(x) for x in z[pre + "params"])
        assert got == (v["n_pairs"], v["k"], v["max_tries"], v["min_span"]), "fixture made for other variants"
        assert float(z[pre + "dropoff"]) == np.float32(v["dropoff"])
        self.v = v
        self.sort_perm = z[pre + "sort_perm"].astype(np.int64)   # per end: the sorted list as input indices
        self.types = z[pre + "types"]
        self.joint_counts = z[pre + "joint_counts"].astype(np.int64)
        self.joint = z[pre + "joint"]                             # (score, i1, i2) rows, pair after pair
        self.plan = z[pre + "plan"]                               # (type, mapq1, mapq2, type4_loop_size) per pair
        self.rec_counts = z[pre + "rec_counts"].astype(np.int64)
        self.records = z[pre + "records"]
        self.t4_counts = z[pre + "t4_counts"].astype(np.int64)
        self.t4_nams = z[pre + "t4_nams"]

    def sorted_lists(self, nams, offs):
        """The input lists in the order the reference's NAM sort left them."""
        out = np.empty_like(nams)
        for e in range(len(offs) - 1):
            a, b = int(offs[e]), int(offs[e + 1])
            out[a:b] = nams[a:b][self.sort_perm[a:b]]
        return out


def _nam_rows_equal(a, b):
    return all((a[f] == b[f]).all() for f in abi.NAM_COMPARED + ("nam_id",))


def check_align(ref, nams, offs, types, jp, jc, plans, steps, ext, resc):
    """Compares one variant's pair types, joint NAM pairs, plans and step records with the
    reference's (ref: an AlignRef; nams / offs: the sorted lists).  Returns a list of
    differences, empty when all agree."""
    bad = []
    P = ref.v["n_pairs"]
    if not (np.asarray(types) == ref.types).all():
        bad.append(f"types differ at pairs {np.nonzero(np.asarray(types) != ref.types)[0][:10]}")
    jstart = np.concatenate([[0], np.cumsum(ref.joint_counts)])
    for p in range(P):
        rj = ref.joint[jstart[p] : jstart[p + 1]]
        mine = jp[p][: int(jc[p])]
        if len(mine) != len(rj) or not ((mine["score"] == rj[:, 0]).all() and (mine["i1"] == rj[:, 1]).all()
                                        and (mine["i2"] == rj[:, 2]).all()):
            bad.append(f"pair {p}: joint NAM pairs differ")
    for col, f in enumerate(("type", "mapq1", "mapq2", "type4_loop_size")):
        if not (plans[f].astype(np.int64) == ref.plan[:, col]).all():
            bad.append(f"plan field {f} differs at pairs {np.nonzero(plans[f] != ref.plan[:, col])[0][:10]}")
    if not (plans["n_steps"].astype(np.int64) == ref.rec_counts).all():
        bad.append("step counts differ")
        return bad
    r = ref.records
    kind_ext = steps["kind"] == abi.GBSA_STEP_EXTEND
    if not (kind_ext == (r["is_extend_seed"] != 0)).all():
        bad.append("extension / rescue order differs")
    if not (steps["is_read1"] == r["is_read1"]).all():
        bad.append("is_read1 tags differ")
    # the NAM each record names, after reverse_nam_if_needed
    idx = (offs[steps["nam_read"].astype(np.int64)] + steps["nam"].astype(np.uint64)).astype(np.int64)
    todo = nams[idx].copy()
    todo["query_start"], todo["query_end"], todo["is_rc"] = ext["query_start"], ext["query_end"], ext["is_rc"]
    if not _nam_rows_equal(todo, r["nam"]):
        bad.append("the steps' NAMs (after reverse_nam_if_needed) differ")
    done = np.where(kind_ext, ext["done"], resc["done"])
    if not (done == r["done_align"]).all():
        bad.append(f"done_align differs at records {np.nonzero(done != r['done_align'])[0][:10]}")
    # an extension the ungapped path aligned: its GPUAlignment; a pending one: all zero
    e_done = kind_ext & (ext["done"] == 1)
    for f in ("ref_id", "ref_start", "edit_distance", "global_ed", "score", "length", "is_rc"):
        if not (ext[f][e_done] == r[f][e_done]).all():
            bad.append(f"extension field {f} differs")
    if (r["gapped"][kind_ext] != 0).any() or (r["is_unaligned"][kind_ext] != 0).any():
        bad.append("an extension record is gapped or unaligned")
    # a rescue that left the mate unaligned: edit distance = read length, the NAM's contig
    # and orientation; a pending one: all zero
    rs_done = ~kind_ext & (resc["done"] == 1)
    for f in ("ref_id", "edit_distance", "is_rc", "is_unaligned"):
        if not (resc[f][rs_done] == r[f][rs_done]).all():
            bad.append(f"rescue field {f} differs")
    pending = ~(e_done | rs_done)
    for f in ("ref_id", "ref_start", "edit_distance", "global_ed", "score", "length", "is_rc", "is_unaligned", "gapped"):
        if (r[f][pending] != 0).any():
            bad.append(f"a pending reference record has {f} set")
    for f in ("ref_start", "edit_distance", "global_ed", "score", "length"):
        if (ext[f][pending & kind_ext] != 0).any():
            bad.append(f"a pending extension has {f} set")
    if (resc["edit_distance"][pending & ~kind_ext] != 0).any() or (resc["is_unaligned"][pending & ~kind_ext] != 0).any():
        bad.append("a pending rescue is marked unaligned")
    # type4_nams: the NAMs of each joint pair the type-4 loop visited (absent end: an
    # all-zero Nam with ref_start -1)
    tstart = np.concatenate([[0], np.cumsum(ref.t4_counts)])
    dummy = np.zeros(1, abi.NAM)
    dummy["ref_start"] = -1
    for p in range(P):
        loop = int(ref.plan[p, 3])
        got = ref.t4_nams[tstart[p] : tstart[p + 1]]
        if len(got) != 2 * loop:
            bad.append(f"pair {p}: type4_nams hold {len(got)} NAMs for {loop} loop steps")
            continue
        for i in range(loop):
            for end, col in ((0, "i1"), (1, "i2")):
                j = int(jp[p][i][col])
                want = dummy[0] if j < 0 else nams[int(offs[2 * p + end]) + j]
                if not _nam_rows_equal(np.array([want]), got[2 * i + end : 2 * i + end + 1]):
                    bad.append(f"pair {p}: type4_nams[{2 * i + end}] differs")
    return bad


def oracle_pair_rows(ref, case, nams, offs, reads):
    """The oracle's restatement of the pair rows on the reference-sorted lists:
    (sorted lists, types, joint pairs, joint counts, plans, steps, extension records,
    rescue records)."""
    from oracle import oracle_py

    v = ref.v
    P = v["n_pairs"]
    s = ref.sorted_lists(nams, offs)
    types = oracle_py.classify_pairs(s, offs, P, abi.GBSA_PAIRS_INTERLEAVED, v["dropoff"], 300.0, 100.0)
    jp, jc = oracle_py.nam_pairs(s, offs, P, abi.GBSA_PAIRS_INTERLEAVED, 300.0, 100.0, v["max_tries"])
    plans, steps = oracle_py.plan_pairs(s, offs, P, types, jp, jc, max_tries=v["max_tries"], dropoff=v["dropoff"])
    g = case.genome
    ext, resc = oracle_py.run_align_steps(g.seq, g.offsets, g.lengths, reads.seq, reads.offsets, reads.lengths, s,
                                          offs, steps, v["k"])
    return s, types, jp, jc, plans, steps, ext, resc


def oracle_sort_mismatches(ref, nams, offs):
    """Read ends whose oracle mate sort (GBSA_SORT_REF_MATE1 for mate 1, GBSA_SORT_REF_MATE2
    for mate 2) differs from the reference's gpu_sort_nams."""
    from oracle import oracle_py

    want = ref.sorted_lists(nams, offs)
    bad = []
    for e in range(len(offs) - 1):
        a, b = int(offs[e]), int(offs[e + 1])
        mode = abi.GBSA_SORT_REF_MATE1 if e % 2 == 0 else abi.GBSA_SORT_REF_MATE2
        if not nams_equal(oracle_py.sort_nams(nams[a:b], mode), want[a:b]):
            bad.append(e)
    return bad
