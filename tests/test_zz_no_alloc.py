"""The allocation-free seeding entry point (gbsa_randstrobes_query_noalloc).

Some callers cannot allocate device memory while they work: a host framework that
owns the device memory pool, or a serving loop that must not call cudaMalloc /
cudaFree.  This entry point takes device buffers for inputs and outputs and uses a
fixed file-scope device array as its only scratch.  The test calls it through the
C-ABI twice in a row (the array keeps the previous call's contents) and checks
both results against the regular entry point gbsa_randstrobes_query, bit for bit.
This file is collected last so that a failure here stops a -x run only after every
other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_index_test_gb300 import abi, native, synth

pytestmark = pytest.mark.gpu


def _reads():
    g = synth.make_genome(synth.GenomeParams(seed=31, total_len=300_000, n_contigs=3, str_frac=0.01))
    a = synth.make_reads(g, synth.ReadParams(seed=32, n_units=700, len_min=50, len_max=1500, paired_frac=0.5,
                                             insert_mean=1600, insert_sd=100))
    b = synth.make_reads(g, synth.ReadParams(seed=33, n_units=300, len_min=150, len_max=150))
    seqs = [bytes(r.seq[int(o):int(o) + int(n)]) for r in (a, b) for o, n in zip(r.offsets, r.lengths)]
    seqs += [b"", b"ACGT", b"A" * 300, b"AC" * 200, b"N" * 40 + bytes(a.seq[:200]), bytes(a.seq[:4096])]
    lens = np.array([len(s) for s in seqs], np.uint32)
    offs = np.zeros(len(seqs), np.uint64)
    offs[1:] = np.cumsum(lens[:-1].astype(np.uint64))
    return synth.Reads(np.frombuffer(b"".join(seqs), np.uint8).copy(), offs, lens)


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    reads = _reads()
    p = native.params_from_read_length(150)
    ref_q, ref_off = native.randstrobes_query(p, reads)

    n = reads.n
    d_seq = torch.from_numpy(reads.seq).to(dev)
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).to(dev)
    d_len = torch.from_numpy(reads.lengths.view(np.int32)).to(dev)
    cap = len(ref_q) + 8
    d_out = torch.zeros(cap * 24, dtype=torch.uint8, device=dev)
    d_qoff = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    L = native.lib()
    for call in range(2):
        d_out.fill_(0xAB)
        tot = C.c_uint64()
        rc = L.gbsa_randstrobes_query_noalloc(C.byref(p), d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), n,
                                              d_out.data_ptr(), cap, d_qoff.data_ptr(), C.byref(tot),
                                              stream.cuda_stream)
        assert rc == abi.GBSA_OK, L.gbsa_last_error()
        torch.cuda.synchronize()
        assert tot.value == len(ref_q), call
        offs = d_qoff.cpu().numpy().view(np.uint64)
        assert (offs == ref_off).all(), call
        got = d_out[: tot.value * 24].cpu().numpy().view(abi.QUERY_RANDSTROBE)
        for f in ("hash", "start", "end", "is_reverse"):
            assert (got[f] == ref_q[f]).all(), (call, f)


def test_noalloc_rejects_small_capacity_and_long_reads():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    p = native.params_from_read_length(150)
    L = native.lib()
    seq = np.frombuffer(b"ACGTTGCA" * 700, np.uint8).copy()   # 5600 bases
    for lens, cap, code in (([150], 4, abi.GBSA_ERR_CAPACITY), ([5000], 10000, abi.GBSA_ERR_READ_TOO_LONG)):
        lens = np.array(lens, np.uint32)
        d_seq = torch.from_numpy(seq).to(dev)
        d_off = torch.zeros(1, dtype=torch.int64, device=dev)
        d_len = torch.from_numpy(lens.view(np.int32)).to(dev)
        d_out = torch.zeros(max(1, cap) * 24, dtype=torch.uint8, device=dev)
        d_qoff = torch.zeros(2, dtype=torch.int64, device=dev)
        tot = C.c_uint64()
        rc = L.gbsa_randstrobes_query_noalloc(C.byref(p), d_seq.data_ptr(), d_off.data_ptr(), d_len.data_ptr(), 1,
                                              d_out.data_ptr(), cap, d_qoff.data_ptr(), C.byref(tot),
                                              torch.cuda.current_stream(dev).cuda_stream)
        assert rc == code, (rc, L.gbsa_last_error())
