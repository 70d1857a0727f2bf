"""The alignment orchestration of align_PE_part0..4 (step2/main.cu:1857-2165) as step
lists: the oracle's planner on hand-made pairs (CPU), and the GPU planner and step
runner against the oracle on mapped read pairs (GB300).

The reference's versions are device code of its main.cu, which does not build (the
Gallatin allocator it needs is not vendored), so the planner is pinned to the
restatement: the CPU tests below work the reference's rules through by hand.
"""
import numpy as np
import pytest

from gpu_index_test_gb300 import abi, native, synth
from oracle import oracle_py


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
