"""The read-pair rows after the NAM stage: pair classification (gpu_pre_cal_type), NAM-pair
scoring (get_best_scoring_nam_pairs_sort3) and the alignment orchestration of
align_PE_part0..4 (step2/main.cu:1857-2165) as step lists with their seed extensions and
mate rescues.

The oracle is pinned to the reference's own code of these rows: main.cu as a whole does
not build, but these functions' lines compile as host C++ (oracle/cut_ref_align.py,
oracle/ref_align.cpp), and tests/golden/align_ref.npz holds their outputs on 3,600 read
pairs (all five pair types, k = 9, 20 and 32, two max_tries / dropoff settings).  The CPU
tests check the oracle against those outputs and work the reference's rules through by
hand on small pairs; the GPU tests check the device planner and step runner against the
reference's outputs and against the oracle on mapped read pairs (GB300).
"""
import os
import sys

import numpy as np
import pytest

from gpu_index_test_gb300 import abi, native, synth
from oracle import oracle_py

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_cases import (ALIGN_VARIANTS, AlignRef, Case, align_inputs, check_align,  # noqa: E402
                          oracle_pair_rows, oracle_sort_mismatches)


def _nam(ref_id, qs, qe, rs, re, n_hits, score, is_rc=0):
    n = np.zeros(1, abi.NAM)[0]
    n["ref_id"], n["query_start"], n["query_end"], n["ref_start"], n["ref_end"] = ref_id, qs, qe, rs, re
    n["n_hits"], n["score"], n["is_rc"] = n_hits, score, is_rc
    return n


def _lists(ends):
    nams = np.array([n for e in ends for n in e], abi.NAM) if any(len(e) for e in ends) else np.zeros(0, abi.NAM)
    offs = np.zeros(len(ends) + 1, np.uint64)
    offs[1:] = np.cumsum([len(e) for e in ends])
    return nams, offs


def _steps(steps):
    return [(int(s["kind"]), int(s["is_read1"]), int(s["read"]), int(s["nam_read"]), int(s["nam"])) for s in steps]


E, R = abi.GBSA_STEP_EXTEND, abi.GBSA_STEP_RESCUE


def test_plan_rescue_read_dropoff_and_tries():
    """Type 1: mate 1's NAMs in order, each extended then the mate rescued from it, until
    n_hits / the first's falls below the dropoff or max_tries were tried; type 2 mirrors
    it with the is_read1 tags swapped; type 0 plans nothing."""
    m1 = [_nam(0, 0, 150, 1000, 1150, 10, 100), _nam(0, 0, 150, 5000, 5150, 6, 60), _nam(0, 0, 150, 9000, 9150, 4, 40)]
    nams, offs = _lists([m1, [], [], m1[:2], [], []])
    types = np.array([1, 2, 0], np.uint8)
    jp = np.zeros((3, 20), abi.NAM_PAIR)
    jc = np.zeros(3, np.uint32)
    plans, steps = oracle_py.plan_pairs(nams, offs, 3, types, jp, jc, max_tries=20, dropoff=0.5)
    # pair 0: 10, 6 pass (6/10 >= 0.5), 4 stops (0.4)
    assert _steps(steps[plans[0]["first_step"]:plans[0]["first_step"] + plans[0]["n_steps"]]) == [
        (E, 1, 0, 0, 0), (R, 0, 1, 0, 0), (E, 1, 0, 0, 1), (R, 0, 1, 0, 1)]
    # pair 1: mate 2 mapped (read 3): extensions tagged read 2, rescues of read 2 tagged read 1
    assert _steps(steps[plans[1]["first_step"]:plans[1]["first_step"] + plans[1]["n_steps"]]) == [
        (E, 0, 3, 3, 0), (R, 1, 2, 3, 0), (E, 0, 3, 3, 1), (R, 1, 2, 3, 1)]
    assert plans[2]["n_steps"] == 0 and plans[2]["type"] == 0
    plans, steps = oracle_py.plan_pairs(nams, offs, 3, types, jp, jc, max_tries=1, dropoff=0.5)
    assert plans[0]["n_steps"] == 2 and plans[1]["n_steps"] == 2


def test_plan_type3_mapq():
    """Type 3: both first NAMs extended; get_mapq: 60 for a single NAM, else
    40 (1 - s2/s1) min(1, n_hits/10) log(s1) truncated, capped at 60, as a uint8 (a
    second NAM scoring above the first wraps)."""
    a = [_nam(0, 0, 150, 1000, 1150, 20, 200.0), _nam(0, 0, 150, 3000, 3150, 5, 50.0)]
    b = [_nam(0, 0, 150, 1300, 1450, 5, 80.0, 1)]
    c = [_nam(0, 0, 150, 1000, 1150, 5, 30.0), _nam(0, 0, 150, 3000, 3150, 5, 60.0)]
    nams, offs = _lists([a, b, c, b])
    plans, steps = oracle_py.plan_pairs(nams, offs, 2, np.array([3, 3], np.uint8), np.zeros((2, 20), abi.NAM_PAIR),
                                        np.zeros(2, np.uint32))
    assert _steps(steps[:2]) == [(E, 1, 0, 0, 0), (E, 0, 1, 1, 0)]
    f = np.float32(40.0) * (np.float32(1.0) - np.float32(50.0) / np.float32(200.0))
    f = np.float32(f * np.float32(1.0)) * np.float32(np.log(np.float32(200.0)))
    assert plans[0]["mapq1"] == min(int(f), 60) and plans[0]["mapq2"] == 60
    g = np.float32(40.0) * (np.float32(1.0) - np.float32(60.0) / np.float32(30.0))
    g = np.float32(g * np.float32(0.5)) * np.float32(np.log(np.float32(30.0)))
    assert plans[1]["mapq1"] == (int(g) % 256)


def test_plan_type4_pairs_and_rescues():
    """Type 4: the best-scoring NAM of each end first (the first of equal maxima), then the
    joint pairs while score / the first pair's >= dropoff: present NAMs extended once,
    absent ends rescued from the other end's NAM."""
    m1 = [_nam(0, 0, 150, 1000, 1150, 8, 90.0), _nam(0, 0, 150, 2000, 2150, 9, 90.0), _nam(1, 0, 150, 10, 160, 3, 30.0)]
    m2 = [_nam(0, 0, 150, 1200, 1350, 7, 70.0, 1), _nam(0, 0, 150, 2200, 2350, 9, 95.0, 1)]
    nams, offs = _lists([m1, m2])
    jp = np.zeros((1, 20), abi.NAM_PAIR)
    jp[0][:4] = [(18, 1, 1), (15, 0, 0), (9, -1, 1), (3, 2, -1)]
    plans, steps = oracle_py.plan_pairs(nams, offs, 1, np.array([4], np.uint8), jp, np.array([4], np.uint32),
                                        max_tries=20, dropoff=0.5)
    # firsts: mate 1's first maximum score is NAM 0 (90 = 90), mate 2's NAM 1
    # pair (18: 1, 1): mate 1 NAM 1 extended, mate 2 NAM 1 done already
    # pair (15: 0, 0): mate 1 NAM 0 done, mate 2 NAM 0 extended
    # pair (9: -, 1): 9 / 18 is not below 0.5: mate 1 rescued from mate 2's NAM 1
    # pair (3: 2, -) is below 18 * 0.5: the loop stops
    assert _steps(steps) == [(E, 1, 0, 0, 0), (E, 0, 1, 1, 1), (E, 1, 0, 0, 1), (E, 0, 1, 1, 0), (R, 1, 0, 1, 1)]
    assert plans[0]["type4_loop_size"] == 3
    plans, steps = oracle_py.plan_pairs(nams, offs, 1, np.array([4], np.uint8), jp, np.array([4], np.uint32),
                                        max_tries=20, dropoff=0.1)
    assert _steps(steps)[5:] == [(E, 1, 0, 0, 2), (R, 0, 1, 0, 2)]
    assert plans[0]["type4_loop_size"] == 4
    plans, steps = oracle_py.plan_pairs(nams, offs, 1, np.array([4], np.uint8), jp, np.array([4], np.uint32),
                                        max_tries=2, dropoff=0.1)
    assert plans[0]["type4_loop_size"] == 2 and len(steps) == 4


@pytest.mark.parametrize("i", range(len(ALIGN_VARIANTS)))
def test_pair_rows_match_the_reference_code(i):
    """The oracle's mate sorts, pair types, joint NAM pairs, plans (type, mapq,
    type4_loop_size) and step records (is_read1, extension or rescue, the NAM after
    reverse_nam_if_needed, done_align, the GPUAlignment fields) against the reference's own
    gpu_sort_nams, gpu_pre_cal_type, get_best_scoring_nam_pairs_sort3 and gpu_align_PE0..4
    on the variant's read pairs."""
    ref = AlignRef(i)
    case = Case(ref.v["src"])
    nams, offs, reads = align_inputs(case, ref.v)
    assert oracle_sort_mismatches(ref, nams, offs) == []
    s, types, jp, jc, plans, steps, ext, resc = oracle_pair_rows(ref, case, nams, offs, reads)
    assert check_align(ref, s, offs, types, jp, jc, plans, steps, ext, resc) == []
    assert set(np.unique(ref.types).tolist()) == {0, 1, 2, 3, 4}


def test_reference_pair_check_catches_planted_differences():
    """check_align reports a changed pair type, joint pair, mapq, is_read1 tag, extension
    score and rescue edit distance (each planted in a copy of the oracle's output)."""
    ref = AlignRef(0)
    case = Case(ref.v["src"])
    nams, offs, reads = align_inputs(case, ref.v)
    s, types, jp, jc, plans, steps, ext, resc = oracle_pair_rows(ref, case, nams, offs, reads)
    assert check_align(ref, s, offs, types, jp, jc, plans, steps, ext, resc) == []
    t3 = int(np.nonzero(types == 3)[0][0])
    t = types.copy()
    t[t3] = 4
    assert any("types" in b for b in check_align(ref, s, offs, t, jp, jc, plans, steps, ext, resc))
    j = jp.copy()
    j4 = int(np.nonzero(jc > 0)[0][0])
    j[j4][0]["score"] += 1
    assert any("joint" in b for b in check_align(ref, s, offs, types, j, jc, plans, steps, ext, resc))
    pl = plans.copy()
    pl[t3]["mapq1"] -= 1
    assert any("mapq1" in b for b in check_align(ref, s, offs, types, jp, jc, pl, steps, ext, resc))
    st = steps.copy()
    st[0]["is_read1"] ^= 1
    assert any("is_read1" in b for b in check_align(ref, s, offs, types, jp, jc, plans, st, ext, resc))
    e = ext.copy()
    d = int(np.nonzero((steps["kind"] == abi.GBSA_STEP_EXTEND) & (ext["done"] == 1))[0][0])
    e[d]["score"] += 1
    assert any("score" in b for b in check_align(ref, s, offs, types, jp, jc, plans, steps, e, resc))
    r = resc.copy()
    u = int(np.nonzero(resc["is_unaligned"] == 1)[0][0])
    r[u]["edit_distance"] -= 1
    assert any("edit_distance" in b for b in check_align(ref, s, offs, types, jp, jc, plans, steps, ext, r))


@pytest.mark.gpu
@pytest.mark.parametrize("i", range(len(ALIGN_VARIANTS)))
def test_pair_rows_on_the_gpu_match_the_reference_code(i):
    """gbsa_classify_pairs_device, gbsa_nam_pairs_device, gbsa_plan_pairs_device and
    gbsa_run_align_steps_device on the reference-sorted NAM lists of the variant's read pairs
    against the reference's own outputs, record by record."""
    import torch

    ref = AlignRef(i)
    v = ref.v
    P, tries = v["n_pairs"], v["max_tries"]
    case = Case(v["src"])
    nams, offs, reads = align_inputs(case, v)
    s = ref.sorted_lists(nams, offs)
    g = case.genome
    dev = torch.device("cuda:0")
    up = lambda x: torch.from_numpy(np.ascontiguousarray(x).view(np.uint8).copy()).to(dev)
    d_n, d_o = up(s), up(offs.astype(np.uint64))
    d_t = torch.zeros(P, dtype=torch.uint8, device=dev)
    native.classify_pairs_device(d_n.data_ptr(), d_o.data_ptr(), P, d_t.data_ptr(), 0, v["dropoff"], 300.0, 100.0)
    d_p = torch.zeros(P * tries * 3, dtype=torch.int32, device=dev)
    d_c = torch.zeros(P, dtype=torch.int32, device=dev)
    native.nam_pairs_device(d_n.data_ptr(), d_o.data_ptr(), P, d_p.data_ptr(), d_c.data_ptr(), 0, 300.0, 100.0, tries)
    cap = P * (2 + 2 * tries)
    d_plans = torch.zeros(P * abi.PAIR_PLAN.itemsize, dtype=torch.uint8, device=dev)
    d_steps = torch.zeros(cap * abi.ALIGN_STEP.itemsize, dtype=torch.uint8, device=dev)
    n = native.plan_pairs_device(d_n.data_ptr(), d_o.data_ptr(), P, d_t.data_ptr(), d_p.data_ptr(), d_c.data_ptr(),
                                 d_plans.data_ptr(), d_steps.data_ptr(), cap, 0, tries, v["dropoff"])
    d_ref = up(g.seq)
    d_roff, d_rlen = up(g.offsets.astype(np.uint64)), up(g.lengths.astype(np.uint64))
    d_seq, d_qoff, d_qlen = up(reads.seq), up(reads.offsets.astype(np.uint64)), up(reads.lengths.astype(np.uint32))
    d_ext = torch.zeros(max(1, n) * abi.SEED_ALIGNMENT.itemsize, dtype=torch.uint8, device=dev)
    d_res = torch.zeros(max(1, n) * abi.MATE_RESCUE.itemsize, dtype=torch.uint8, device=dev)
    native.run_align_steps_device(d_ref.data_ptr(), d_roff.data_ptr(), d_rlen.data_ptr(), len(g.lengths),
                                  d_seq.data_ptr(), d_qoff.data_ptr(), d_qlen.data_ptr(), reads.n, d_n.data_ptr(),
                                  d_o.data_ptr(), d_steps.data_ptr(), n, v["k"], d_ext.data_ptr(), d_res.data_ptr())
    torch.cuda.synchronize()
    types = d_t.cpu().numpy()
    jp = d_p.cpu().numpy().view(abi.NAM_PAIR).reshape(P, tries)
    jc = d_c.cpu().numpy().astype(np.uint32)
    plans = d_plans.cpu().numpy().view(abi.PAIR_PLAN)
    steps = d_steps.cpu().numpy().view(abi.ALIGN_STEP)[:n]
    ext = d_ext.cpu().numpy().view(abi.SEED_ALIGNMENT)[:n]
    resc = d_res.cpu().numpy().view(abi.MATE_RESCUE)[:n]
    assert check_align(ref, s, offs, types, jp, jc, plans, steps, ext, resc) == []


@pytest.mark.gpu
def test_plan_and_steps_against_oracle():
    """Mapped read pairs (mate 1 in GBSA_SORT_REF_MATE1 order, mate 2 in GBSA_SORT_REF_MATE2
    order, as the reference's NAM sort leaves them) through pair classification, NAM-pair
    scoring, the planner and the step runner on the GPU: plans, steps, extension and
    rescue records equal the oracle's."""
    import torch

    g = synth.make_genome(synth.genome_params("C2", scale=0.01, seed=141))
    reads = synth.make_reads(g, synth.read_params("C2", n_units=4000, seed=142))
    p = native.params_from_read_length(150)
    idx = native.Index.build(p, g)
    n_pairs = reads.n // 2
    a = native.Mapper(idx, abi.map_options(rescue_level=2, sort_mode=abi.GBSA_SORT_REF_MATE1)).map_reads(
        reads.subset(np.arange(0, reads.n, 2)))
    b = native.Mapper(idx, abi.map_options(rescue_level=2, sort_mode=abi.GBSA_SORT_REF_MATE2)).map_reads(
        reads.subset(np.arange(1, reads.n, 2)))
    ends = []
    for i in range(n_pairs):
        ends.append(a[0][int(a[1][i]):int(a[1][i + 1])])
        ends.append(b[0][int(b[1][i]):int(b[1][i + 1])])
    nams, offs = _lists(ends)
    tries = 20
    types = oracle_py.classify_pairs(nams, offs, n_pairs, abi.GBSA_PAIRS_INTERLEAVED, 0.5, 300.0, 100.0)
    jp, jc = oracle_py.nam_pairs(nams, offs, n_pairs, abi.GBSA_PAIRS_INTERLEAVED, 300.0, 100.0, tries)
    plans, steps = oracle_py.plan_pairs(nams, offs, n_pairs, types, jp, jc, max_tries=tries, dropoff=0.5)
    assert set(np.unique(plans["type"])) >= {1, 2, 3, 4}
    assert (steps["kind"] == abi.GBSA_STEP_RESCUE).sum() > 0

    dev = torch.device("cuda:0")
    up = lambda x: torch.from_numpy(np.ascontiguousarray(x).view(np.uint8).copy()).to(dev)
    d_n, d_o = up(nams), up(offs.astype(np.uint64))
    d_t = torch.zeros(n_pairs, dtype=torch.uint8, device=dev)
    native.classify_pairs_device(d_n.data_ptr(), d_o.data_ptr(), n_pairs, d_t.data_ptr(), 0, 0.5, 300.0, 100.0)
    d_p = torch.zeros(n_pairs * tries * 3, dtype=torch.int32, device=dev)
    d_c = torch.zeros(n_pairs, dtype=torch.int32, device=dev)
    native.nam_pairs_device(d_n.data_ptr(), d_o.data_ptr(), n_pairs, d_p.data_ptr(), d_c.data_ptr(), 0, 300.0, 100.0,
                            tries)
    cap = len(steps) + 16
    d_plans = torch.zeros(n_pairs * abi.PAIR_PLAN.itemsize, dtype=torch.uint8, device=dev)
    d_steps = torch.zeros(cap * abi.ALIGN_STEP.itemsize, dtype=torch.uint8, device=dev)
    n = native.plan_pairs_device(d_n.data_ptr(), d_o.data_ptr(), n_pairs, d_t.data_ptr(), d_p.data_ptr(),
                                 d_c.data_ptr(), d_plans.data_ptr(), d_steps.data_ptr(), cap, 0, tries, 0.5)
    torch.cuda.synchronize()
    assert n == len(steps)
    got_plans = d_plans.cpu().numpy().view(abi.PAIR_PLAN)
    got_steps = d_steps.cpu().numpy().view(abi.ALIGN_STEP)[:n]
    assert (got_plans == plans).all() and (got_steps == steps).all()
    with pytest.raises(native.GbsaError):   # too small a step list
        native.plan_pairs_device(d_n.data_ptr(), d_o.data_ptr(), n_pairs, d_t.data_ptr(), d_p.data_ptr(),
                                 d_c.data_ptr(), d_plans.data_ptr(), d_steps.data_ptr(), n - 1, 0, tries, 0.5)
    d_ref = up(g.seq)
    d_roff, d_rlen = up(g.offsets.astype(np.uint64)), up(g.lengths.astype(np.uint64))
    # the reads in the NAM lists' order (mates interleaved, as generated)
    d_seq, d_qoff, d_qlen = up(reads.seq), up(reads.offsets.astype(np.uint64)), up(reads.lengths.astype(np.uint32))
    d_ext = torch.zeros(n * abi.SEED_ALIGNMENT.itemsize, dtype=torch.uint8, device=dev)
    d_res = torch.zeros(n * abi.MATE_RESCUE.itemsize, dtype=torch.uint8, device=dev)
    native.run_align_steps_device(d_ref.data_ptr(), d_roff.data_ptr(), d_rlen.data_ptr(), len(g.lengths),
                                  d_seq.data_ptr(), d_qoff.data_ptr(), d_qlen.data_ptr(), reads.n, d_n.data_ptr(),
                                  d_o.data_ptr(), d_steps.data_ptr(), n, p.k, d_ext.data_ptr(), d_res.data_ptr())
    ext, resc = oracle_py.run_align_steps(g.seq, g.offsets, g.lengths, reads.seq, reads.offsets, reads.lengths, nams,
                                          offs, steps, p.k)
    assert (d_ext.cpu().numpy().view(abi.SEED_ALIGNMENT) == ext).all()
    assert (d_res.cpu().numpy().view(abi.MATE_RESCUE) == resc).all()
