"""Generate tests/golden/align_ref.npz from the REFERENCE's own read-pair code.

Run where the reference sources are present (after oracle/build_ref.sh, which builds
oracle/_ref/ref_align from the reference's step2/main.cu):

    python tests/golden/make_align_golden.py [--check-only]

For each variant of golden_cases.ALIGN_VARIANTS it takes the first read pairs of a NAM
fixture (c2mini or c4mini: the reads, the genome and the NAMs the reference's find_nams /
find_nams_rescue produced for them), runs ref_align on them — the reference's
gpu_sort_nams, gpu_pre_cal_type, get_best_scoring_nam_pairs_sort3 and gpu_align_PE0..4 —
and stores its outputs: the order of each sorted NAM list, the pair types, the joint NAM
pairs, each pair's type / mapq / type4_loop_size, the GPUAlignTmpRes records (is_read1,
is_extend_seed, done_align, the NAM after reverse_nam_if_needed, the GPUAlignment) and
type4_nams.  It then checks the oracle's restatement against them (the same check
tests/test_align_plan.py makes) before writing.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

from gpu_index_test_gb300 import abi  # noqa: E402
import golden_cases as gc  # noqa: E402

REF_ALIGN = os.path.join(REPO, "oracle", "_ref", "ref_align")


def run_ref_align(case, v, nams, offs, reads, workdir):
    """Writes ref_align's input (read ends in main.cu's order: mate 1 of every pair, then
    mate 2 of every pair) and parses its output back into the interleaved layout."""
    P = v["n_pairs"]
    ap = np.asarray(abi.align_params()).reshape(-1)[0]
    inp, outp = os.path.join(workdir, "in.bin"), os.path.join(workdir, "out.bin")
    order = [2 * p for p in range(P)] + [2 * p + 1 for p in range(P)]
    with open(inp, "wb") as f:
        np.array([v["k"], v["max_tries"], ap["match"], ap["mismatch"], ap["gap_open"], ap["gap_extend"],
                  ap["end_bonus"]], np.int32).tofile(f)
        np.array([v["dropoff"]], np.float32).tofile(f)
        g = case.genome
        np.array([len(g.lengths)], np.uint32).tofile(f)
        g.lengths.astype(np.uint64).tofile(f)
        g.seq.tofile(f)
        np.array([P], np.uint32).tofile(f)
        reads.lengths[0::2].astype(np.uint32).tofile(f)
        reads.lengths[1::2].astype(np.uint32).tofile(f)
        for p in range(P):
            for e in (2 * p, 2 * p + 1):
                o, n = int(reads.offsets[e]), int(reads.lengths[e])
                f.write(bytes(reads.seq[o : o + n]))
        np.array([int(offs[e + 1] - offs[e]) for e in order], np.uint32).tofile(f)
        for e in order:
            nams[int(offs[e]) : int(offs[e + 1])].tofile(f)
    subprocess.run([REF_ALIGN, inp, outp], check=True)
    raw = open(outp, "rb").read()
    pos = 0

    def take(dtype, n=1):
        nonlocal pos
        a = np.frombuffer(raw, dtype, n, pos)
        pos += a.nbytes
        return a

    sorted_lists = [None] * (2 * P)
    for e in order:
        n = int(take(np.uint32)[0])
        sorted_lists[e] = take(abi.NAM, n)
    types = take(np.int32, P).astype(np.uint8)
    joint_counts, joint, plan, rec_counts, records, t4_counts, t4_nams = [], [], [], [], [], [], []
    for _ in range(P):
        n = int(take(np.uint32)[0])
        joint_counts.append(n)
        joint.append(take(np.int32, 3 * n).reshape(n, 3))
        plan.append(take(np.int32, 4))
        n = int(take(np.uint32)[0])
        rec_counts.append(n)
        records.append(take(gc.REF_ALIGN_RECORD, n))
        n = int(take(np.uint32)[0])
        t4_counts.append(n)
        t4_nams.append(take(abi.NAM, n))
    assert pos == len(raw), "ref_align output not fully read"
    # each sorted list as indices into its input list (every NAM used once; equal NAMs
    # are interchangeable)
    perm = np.zeros(len(nams), np.int16)
    for e in range(2 * P):
        a = nams[int(offs[e]) : int(offs[e + 1])]
        s = sorted_lists[e]
        assert len(a) == len(s)
        used = np.zeros(len(a), bool)
        for j in range(len(s)):
            hit = np.nonzero(~used & (a.view(np.uint8).reshape(len(a), -1) == s[j : j + 1].view(np.uint8)).all(1))[0]
            assert len(hit), "a sorted NAM is not in its input list"
            used[hit[0]] = True
            perm[int(offs[e]) + j] = hit[0]
    return dict(sort_perm=perm, types=types, joint_counts=np.array(joint_counts, np.uint8),
                joint=np.concatenate(joint).astype(np.int32), plan=np.array(plan, np.int32),
                rec_counts=np.array(rec_counts, np.uint16), records=np.concatenate(records),
                t4_counts=np.array(t4_counts, np.uint8), t4_nams=np.concatenate(t4_nams))


def main(check_only=False):
    assert os.path.exists(REF_ALIGN), "build oracle/_ref first (oracle/build_ref.sh)"
    arrays = {}
    outs = []
    for i, v in enumerate(gc.ALIGN_VARIANTS):
        case = gc.Case(v["src"])
        nams, offs, reads = gc.align_inputs(case, v)
        with tempfile.TemporaryDirectory() as td:
            out = run_ref_align(case, v, nams, offs, reads, td)
        pre = f"v{i}_"
        arrays[pre + "params"] = np.array([v["n_pairs"], v["k"], v["max_tries"], v["min_span"]], np.int32)
        arrays[pre + "dropoff"] = np.float32(v["dropoff"])
        for key, val in out.items():
            arrays[pre + key] = val
        outs.append((case, nams, offs, reads))
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "align_ref.npz")
        np.savez_compressed(path, **arrays)
        saved, gc.ALIGN_FIXTURE = gc.ALIGN_FIXTURE, path
        try:
            for i, (case, nams, offs, reads) in enumerate(outs):
                ref = gc.AlignRef(i)
                bad = gc.oracle_sort_mismatches(ref, nams, offs)
                s, types, jp, jc, plans, steps, ext, resc = gc.oracle_pair_rows(ref, case, nams, offs, reads)
                bad += gc.check_align(ref, s, offs, types, jp, jc, plans, steps, ext, resc)
                counts = np.bincount(ref.types, minlength=5)
                print(f"variant {i} {ref.v}: pair types {counts.tolist()}, joint pairs {int(ref.joint_counts.sum())}, "
                      f"records {len(ref.records)} (done {int(ref.records['done_align'].sum())}), "
                      f"oracle differences: {len(bad)} {bad[:5]}")
                assert not bad, "oracle disagrees with the reference"
        finally:
            gc.ALIGN_FIXTURE = saved
        if not check_only:
            os.replace(path, gc.ALIGN_FIXTURE)


if __name__ == "__main__":
    main(check_only="--check-only" in sys.argv)
