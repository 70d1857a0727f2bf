"""Seeded synthetic genomes and reads (host C++ generator, csrc/synth.cpp).

The reference ships no data; its pipeline reads user FASTA/FASTQ files.  The
workloads below stand in for them with the shapes the benchmark configurations
describe:

  C1  5 Mbp single contig of i.i.d. uniform ACGT; 100k single-end 150 bp reads,
      1% substitutions and 0.1% 1-3 bp indels per base.
  C2  100 Mbp in 20 contigs; 5% of bases in duplicated 1-10 kb segments copied
      2-20x at 0.5-2% divergence, plus short tandem repeats (unit 2-6 bp,
      20-200 copies); 1M paired-end 2x150 bp pairs, insert ~Normal(300, 30).
  C3  the C1 reference; 2M units of log-uniform length in [50, 500] bp, half
      single-end and half paired-end.
  C4  3.1 Gbp in 24 contigs of 50-250 Mbp, ~45% interspersed repeat families
      (300 bp-6 kb elements at 5-20% divergence) plus 5% segmental duplications;
      10M paired-end 2x150 bp pairs, insert ~Normal(350, 50), 0.5-1.5% substitutions.

Every generator is a pure function of its seed.
"""
import ctypes as C
import os
from dataclasses import dataclass, field, replace

import numpy as np

from . import _build_paths


class GenomeSpec(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("total_len", C.c_uint64),
        ("n_contigs", C.c_uint32),
        ("_pad0", C.c_uint32),
        ("min_contig", C.c_uint64),
        ("max_contig", C.c_uint64),
        ("dup_frac", C.c_double),
        ("dup_min", C.c_uint32),
        ("dup_max", C.c_uint32),
        ("dup_copies_min", C.c_uint32),
        ("dup_copies_max", C.c_uint32),
        ("dup_div_min", C.c_double),
        ("dup_div_max", C.c_double),
        ("fam_frac", C.c_double),
        ("n_families", C.c_uint32),
        ("fam_min", C.c_uint32),
        ("fam_max", C.c_uint32),
        ("_pad1", C.c_uint32),
        ("fam_div_min", C.c_double),
        ("fam_div_max", C.c_double),
        ("str_frac", C.c_double),
        ("str_unit_min", C.c_uint32),
        ("str_unit_max", C.c_uint32),
        ("str_copies_min", C.c_uint32),
        ("str_copies_max", C.c_uint32),
    ]


class ReadSpec(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("n_units", C.c_uint32),
        ("len_min", C.c_uint32),
        ("len_max", C.c_uint32),
        ("_pad0", C.c_uint32),
        ("paired_frac", C.c_double),
        ("insert_mean", C.c_double),
        ("insert_sd", C.c_double),
        ("sub_min", C.c_double),
        ("sub_max", C.c_double),
        ("indel_rate", C.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build_paths.SYNTH_SO
        if not os.path.exists(path):
            raise RuntimeError(f"synthetic-data library missing: {path} (run __graft_entry__.build())")
        L = C.CDLL(path)
        L.gbsa_synth_contig_lengths.restype = C.c_uint64
        L.gbsa_synth_contig_lengths.argtypes = [C.POINTER(GenomeSpec), C.c_void_p]
        L.gbsa_synth_genome.restype = C.c_int
        L.gbsa_synth_genome.argtypes = [C.POINTER(GenomeSpec), C.c_void_p, C.c_void_p]
        L.gbsa_synth_reads_size.restype = C.c_int
        L.gbsa_synth_reads_size.argtypes = [C.POINTER(ReadSpec), C.c_void_p, C.c_void_p]
        L.gbsa_synth_read_items.restype = C.c_int
        L.gbsa_synth_read_items.argtypes = [C.POINTER(ReadSpec), C.c_void_p]
        L.gbsa_synth_reads.restype = C.c_int
        L.gbsa_synth_reads.argtypes = [
            C.POINTER(ReadSpec), C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
        ]
        _lib = L
    return _lib


@dataclass
class Genome:
    seq: np.ndarray        # uint8 ASCII, contigs back to back
    lengths: np.ndarray    # uint64 per contig
    offsets: np.ndarray    # uint64 per contig

    @property
    def total_length(self):
        return int(self.lengths.sum())


@dataclass
class Reads:
    seq: np.ndarray        # uint8 ASCII, reads back to back
    offsets: np.ndarray    # uint64 per read
    lengths: np.ndarray    # uint32 per read
    truth: np.ndarray = None

    @property
    def n(self):
        return int(self.lengths.shape[0])

    def subset(self, idx):
        idx = np.asarray(idx)
        lens = self.lengths[idx]
        offs = np.zeros(len(idx), np.uint64)
        if len(idx):
            offs[1:] = np.cumsum(lens[:-1].astype(np.uint64))
        parts = [self.seq[int(self.offsets[i]) : int(self.offsets[i]) + int(self.lengths[i])] for i in idx]
        seq = np.concatenate(parts) if parts else np.zeros(0, np.uint8)
        return Reads(np.ascontiguousarray(seq), offs, np.ascontiguousarray(lens))


@dataclass
class GenomeParams:
    seed: int = 1
    total_len: int = 5_000_000
    n_contigs: int = 1
    min_contig: int = 0
    max_contig: int = 0
    dup_frac: float = 0.0
    dup_len: tuple = (1000, 10000)
    dup_copies: tuple = (2, 20)
    dup_div: tuple = (0.005, 0.02)
    fam_frac: float = 0.0
    n_families: int = 0
    fam_len: tuple = (300, 6000)
    fam_div: tuple = (0.05, 0.20)
    str_frac: float = 0.0
    str_unit: tuple = (2, 6)
    str_copies: tuple = (20, 200)


@dataclass
class ReadParams:
    seed: int = 11
    n_units: int = 100_000
    len_min: int = 150
    len_max: int = 150
    paired_frac: float = 0.0
    insert_mean: float = 300.0
    insert_sd: float = 30.0
    sub: tuple = (0.01, 0.01)
    indel_rate: float = 0.001


def make_genome(gp: GenomeParams) -> Genome:
    s = GenomeSpec()
    s.seed = gp.seed
    s.total_len = gp.total_len
    s.n_contigs = gp.n_contigs
    s.min_contig = gp.min_contig or gp.total_len // gp.n_contigs
    s.max_contig = gp.max_contig or gp.total_len // gp.n_contigs
    s.dup_frac = gp.dup_frac
    s.dup_min, s.dup_max = gp.dup_len
    s.dup_copies_min, s.dup_copies_max = gp.dup_copies
    s.dup_div_min, s.dup_div_max = gp.dup_div
    s.fam_frac = gp.fam_frac
    s.n_families = gp.n_families
    s.fam_min, s.fam_max = gp.fam_len
    s.fam_div_min, s.fam_div_max = gp.fam_div
    s.str_frac = gp.str_frac
    s.str_unit_min, s.str_unit_max = gp.str_unit
    s.str_copies_min, s.str_copies_max = gp.str_copies
    L = lib()
    lengths = np.zeros(gp.n_contigs, np.uint64)
    L.gbsa_synth_contig_lengths(C.byref(s), lengths.ctypes.data)
    seq = np.empty(int(lengths.sum()), np.uint8)
    L.gbsa_synth_genome(C.byref(s), lengths.ctypes.data, seq.ctypes.data)
    offsets = np.zeros(gp.n_contigs, np.uint64)
    offsets[1:] = np.cumsum(lengths[:-1])
    return Genome(seq, lengths, offsets)


def make_reads(genome: Genome, rp: ReadParams, with_truth=False) -> Reads:
    s = ReadSpec()
    s.seed = rp.seed
    s.n_units = rp.n_units
    s.len_min = rp.len_min
    s.len_max = rp.len_max
    s.paired_frac = rp.paired_frac
    s.insert_mean = rp.insert_mean
    s.insert_sd = rp.insert_sd
    s.sub_min, s.sub_max = rp.sub
    s.indel_rate = rp.indel_rate
    L = lib()
    nr = C.c_uint64()
    nb = C.c_uint64()
    L.gbsa_synth_reads_size(C.byref(s), C.byref(nr), C.byref(nb))
    seq = np.empty(nb.value, np.uint8)
    offsets = np.empty(nr.value, np.uint64)
    lengths = np.empty(nr.value, np.uint32)
    truth = np.empty((nr.value, 3), np.uint64) if with_truth else None
    L.gbsa_synth_reads(
        C.byref(s), genome.seq.ctypes.data, genome.lengths.ctypes.data, len(genome.lengths),
        seq.ctypes.data, offsets.ctypes.data, lengths.ctypes.data,
        truth.ctypes.data if truth is not None else None,
    )
    return Reads(seq, offsets, lengths, truth)


def read_items(rp: ReadParams) -> np.ndarray:
    """Work items of make_reads(genome, rp): item u is reads [items[u], items[u + 1]), a
    single-end read or the two mates of a pair (n_units + 1 entries)."""
    s = ReadSpec()
    s.seed = rp.seed
    s.n_units = rp.n_units
    s.len_min = rp.len_min
    s.len_max = rp.len_max
    s.paired_frac = rp.paired_frac
    out = np.empty(rp.n_units + 1, np.uint32)
    lib().gbsa_synth_read_items(C.byref(s), out.ctypes.data)
    return out


# ---- benchmark configurations -------------------------------------------------

def genome_params(config: str, scale: float = 1.0, seed: int = 1) -> GenomeParams:
    """Genome shape of a configuration; scale < 1 shrinks it for tests."""
    if config in ("C1", "C3", "C5"):
        return GenomeParams(seed=seed, total_len=max(50_000, int(5_000_000 * scale)), n_contigs=1)
    if config == "C2":
        tot = max(200_000, int(100_000_000 * scale))
        return GenomeParams(
            seed=seed, total_len=tot, n_contigs=20, min_contig=int(tot / 20 * 0.6), max_contig=int(tot / 20 * 1.4),
            dup_frac=0.05, str_frac=0.005,
        )
    if config == "C4":
        tot = max(1_000_000, int(3_100_000_000 * scale))
        return GenomeParams(
            seed=seed, total_len=tot, n_contigs=24, min_contig=int(tot * 50 / 3100), max_contig=int(tot * 250 / 3100),
            fam_frac=0.45, n_families=2000, dup_frac=0.05, str_frac=0.003,
        )
    raise ValueError(config)


def read_params(config: str, n_units=None, seed: int = 11) -> ReadParams:
    if config == "C1":
        return ReadParams(seed=seed, n_units=n_units or 100_000, len_min=150, len_max=150, paired_frac=0.0)
    if config == "C2":
        return ReadParams(seed=seed, n_units=n_units or 1_000_000, len_min=150, len_max=150, paired_frac=1.0,
                          insert_mean=300, insert_sd=30)
    if config == "C3":
        return ReadParams(seed=seed, n_units=n_units or 2_000_000, len_min=50, len_max=500, paired_frac=0.5,
                          insert_mean=600, insert_sd=60)
    if config == "C4":
        return ReadParams(seed=seed, n_units=n_units or 10_000_000, len_min=150, len_max=150, paired_frac=1.0,
                          insert_mean=350, insert_sd=50, sub=(0.005, 0.015))
    if config == "C5":
        return ReadParams(seed=seed, n_units=n_units or 10_000, len_min=100, len_max=250, paired_frac=1.0,
                          insert_mean=400, insert_sd=50)
    raise ValueError(config)
