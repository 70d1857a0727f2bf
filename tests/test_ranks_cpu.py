"""The multi-rank form of bench.py on CPU: two gloo ranks (spawned processes) each map
their own shard of reads with no exchange in the data path, then agree on the slowest
rank's time with one all-reduce; the whole-job throughput counts every rank's reads.
The GPU form differs only in the backend (NCCL, device tensors) and the mapper."""
import hashlib
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.join(os.path.dirname(__file__), "..")
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import time

    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle_py

    g, reads, _, _, _ = bench.workload(0.001, rank)
    t0 = time.perf_counter()
    idx = oracle_py.Index.build(oracle_py.params_from_read_length(150), g)
    nams, offs, frac, resc = idx.map_reads(reads)
    seconds = time.perf_counter() - t0
    slowest = bench.max_over_ranks(seconds, world)
    rec = {"rank": rank, "seconds": seconds, "slowest": slowest, "n": int(reads.n), "nams": int(len(nams)),
           "genome": hashlib.sha1(g.seq.tobytes()).hexdigest(), "reads": hashlib.sha1(reads.seq.tobytes()).hexdigest(),
           "value": bench.job_throughput(reads.n, world, slowest)}
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(rec, f)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_reads_and_take_the_slowest_time(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    recs = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(world)]
    assert recs[0]["genome"] == recs[1]["genome"]          # one index, replicated
    assert recs[0]["reads"] != recs[1]["reads"]            # a shard of reads per rank (weak scaling)
    slowest = max(r["seconds"] for r in recs)
    for r in recs:
        assert r["slowest"] == pytest.approx(slowest)
        assert r["value"] == pytest.approx(world * r["n"] / slowest)
        assert r["nams"] > 0


def test_one_rank_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(1000, 1, 0.5) == 2000
    assert np.isclose(bench.job_throughput(1000, 4, 0.5), 8000)
