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
