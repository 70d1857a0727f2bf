"""Generate the golden fixtures of tests/golden/ from the REFERENCE's own CPU code.

Run where the reference sources are present (after oracle/build_ref.sh):

    python tests/golden/make_golden.py [--check-only]

For each case it generates a small seeded genome and read set, builds the index
with the oracle and writes it as a .sti file (the reference cannot build an index:
its populate() is commented out, step2/index.cu:143-244), then runs
oracle/_ref/ref_driver — the reference's StrobemerIndex::read, SyncmerIterator,
RandstrobeIterator, find_nams and find_nams_rescue — on every read.  It checks the
oracle against those outputs and stores inputs + reference outputs as compressed
.npz fixtures, together with xxh64 known answers from the reference's hash.hpp.
The fixtures carry the reference's results to machines without the reference.
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from gpu_index_test_gb300 import abi, synth  # noqa: E402
from oracle import oracle_py  # noqa: E402

REF_DRIVER = os.path.join(REPO, "oracle", "_ref", "ref_driver")
READ_LENGTH = 150
RESCUE_LEVEL = 2


def edge_reads(genome, seed=5):
    """Hand-made reads: empty, short, N runs, lowercase, homopolymers, tandem repeats, long."""
    rng = np.random.default_rng(seed)
    g = genome.seq
    out = []

    def frag(n):
        a = int(rng.integers(0, len(g) - n))
        return bytes(g[a : a + n])

    out += [b"", b"ACGTA", b"ACGTACGTACGTACG", frag(20), frag(21), frag(24), frag(25), frag(31)]
    out += [b"A" * 150, b"C" * 60, b"AC" * 75, b"ACG" * 50, b"ACGT" * 40, b"ACGTA" * 30, b"AACCG" * 30]
    out += [b"AT" * 20 + frag(110), frag(60) + b"TTTTTTTTTTTTTTTTTTTTTTTTTT" + frag(64)]
    out += [b"N" * 150, frag(70) + b"N" + frag(79), frag(40) + b"NNNN" + frag(106), b"N" + frag(149), frag(149) + b"N"]
    r = bytearray(frag(150))
    for i in range(0, 150, 17):
        r[i] = ord("N")
    out.append(bytes(r))
    out += [frag(150).lower(), frag(150).replace(b"T", b"U"), frag(75) + b"RYKM" + frag(71)]
    out += [frag(500), frag(1000), frag(4000)]
    s = bytearray(frag(300))
    for i in range(0, 300, 50):
        s[i : i + 8] = b"ACACACAC"
    out.append(bytes(s))
    # a read equal to the start / end of the first contig, and its reverse complement
    comp = bytes.maketrans(b"ACGT", b"TGCA")
    out += [bytes(g[:150]), bytes(g[len(g) - 150 :]), bytes(g[:150]).translate(comp)[::-1]]
    return out


def to_reads(seqs):
    lens = np.array([len(s) for s in seqs], np.uint32)
    offs = np.zeros(len(seqs), np.uint64)
    if len(seqs) > 1:
        offs[1:] = np.cumsum(lens[:-1].astype(np.uint64))
    buf = np.frombuffer(b"".join(seqs), np.uint8).copy() if sum(lens) else np.zeros(0, np.uint8)
    return synth.Reads(buf, offs, lens)


def concat_reads(a, b):
    seqs = [bytes(a.seq[int(o) : int(o) + int(n)]) for o, n in zip(a.offsets, a.lengths)]
    seqs += [bytes(b.seq[int(o) : int(o) + int(n)]) for o, n in zip(b.offsets, b.lengths)]
    return to_reads(seqs)


def run_reference(reads, sti_path, workdir):
    case = os.path.join(workdir, "case.bin")
    out = os.path.join(workdir, "out.bin")
    with open(case, "wb") as f:
        np.array([READ_LENGTH, RESCUE_LEVEL], np.int32).tofile(f)
        np.array([reads.n], np.uint32).tofile(f)
        reads.lengths.astype(np.uint32).tofile(f)
        for o, n in zip(reads.offsets, reads.lengths):
            f.write(bytes(reads.seq[int(o) : int(o) + int(n)]))
    subprocess.run([REF_DRIVER, case, sti_path, out], check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    raw = open(out, "rb").read()
    p = 0
    q_all, q_off, frac, resc, nam_all, nam_off = [], [0], [], [], [], [0]
    qdt = np.dtype([("hash", "<u8"), ("start", "<u4"), ("end", "<u4"), ("is_reverse", "u1")])
    ndt = np.dtype([("query_start", "<i4"), ("query_end", "<i4"), ("ref_start", "<i4"), ("ref_end", "<i4"),
                    ("n_hits", "<i4"), ("ref_id", "<i4"), ("score", "<f4"), ("is_rc", "u1")])
    for _ in range(reads.n):
        nq = int(np.frombuffer(raw, np.uint32, 1, p)[0]); p += 4
        q = np.frombuffer(raw, qdt, nq, p); p += nq * qdt.itemsize
        fr = float(np.frombuffer(raw, np.float32, 1, p)[0]); p += 4
        rs = raw[p]; p += 1
        nn = int(np.frombuffer(raw, np.uint32, 1, p)[0]); p += 4
        nm = np.frombuffer(raw, ndt, nn, p); p += nn * ndt.itemsize
        q_all.append(q); q_off.append(q_off[-1] + nq)
        frac.append(fr); resc.append(rs)
        full = np.zeros(nn, abi.NAM)
        for f in ndt.names:
            full[f] = nm[f]
        nam_all.append(oracle_py.sort_nams(full))
        nam_off.append(nam_off[-1] + nn)
    assert p == len(raw)
    qcat = np.concatenate(q_all) if q_all else np.zeros(0, qdt)
    ncat = np.concatenate(nam_all) if nam_all else np.zeros(0, abi.NAM)
    return qcat, np.array(q_off, np.uint64), np.array(frac, np.float32), np.array(resc, np.uint8), ncat, np.array(nam_off, np.uint64)


def pack_acgt(seq):
    """ACGT bytes → 2-bit codes, 4 per byte (the synthetic genomes hold no other symbols)."""
    lut = np.full(256, 255, np.uint8)
    for i, c in enumerate(b"ACGT"):
        lut[c] = i
    codes = lut[seq]
    assert (codes < 4).all()
    pad = (-len(codes)) % 4
    codes = np.concatenate([codes, np.zeros(pad, np.uint8)]).reshape(-1, 4)
    return (codes[:, 0] | (codes[:, 1] << 2) | (codes[:, 2] << 4) | (codes[:, 3] << 6)).astype(np.uint8)


def unpack_acgt(packed, n):
    codes = np.stack([(packed >> s) & 3 for s in (0, 2, 4, 6)], axis=1).reshape(-1)[:n]
    return np.frombuffer(b"ACGT", np.uint8)[codes]


def index_digest(idx):
    h = hashlib.sha256()
    h.update(idx.randstrobes().tobytes())
    h.update(idx.starts().tobytes())
    return h.hexdigest()


CASES = {
    # name: (genome params, list of read params)
    "c1mini": (synth.GenomeParams(seed=101, total_len=300_000, n_contigs=1),
               [synth.ReadParams(seed=7, n_units=1500, len_min=150, len_max=150)]),
    "c2mini": (synth.GenomeParams(seed=202, total_len=1_000_000, n_contigs=20, min_contig=30_000, max_contig=70_000,
                                  dup_frac=0.05, str_frac=0.005),
               [synth.ReadParams(seed=8, n_units=600, len_min=150, len_max=150, paired_frac=1.0),
                synth.ReadParams(seed=9, n_units=400, len_min=50, len_max=500, paired_frac=0.5, insert_mean=600,
                                 insert_sd=60)]),
    "c4mini": (synth.GenomeParams(seed=404, total_len=2_000_000, n_contigs=24, min_contig=40_000, max_contig=120_000,
                                  fam_frac=0.45, n_families=6, fam_div=(0.01, 0.20), dup_frac=0.05, str_frac=0.003),
               [synth.ReadParams(seed=10, n_units=1000, len_min=150, len_max=150, paired_frac=1.0, insert_mean=350,
                                 insert_sd=50, sub=(0.005, 0.015))]),
}


def main(check_only=False):
    assert os.path.exists(REF_DRIVER), "build oracle/_ref first (oracle/build_ref.sh)"
    p = oracle_py.params_from_read_length(READ_LENGTH)
    # xxh64 known answers from the reference's hash.hpp
    kat_in = np.array([0, 1, 2, 3, 0xFFFFFFFF, 0xFFFFFFFFFFFFFFFF, 0x123456789ABCDEF0, 12345678901234567890,
                       0xAAAAAAAA, 0x55555555, 1 << 40, (1 << 63) + 17], np.uint64)
    r = subprocess.run([REF_DRIVER, "xxh64"], input=" ".join(str(int(x)) for x in kat_in), capture_output=True,
                       text=True, check=True)
    kat_out = np.array([int(x) for x in r.stdout.split()], np.uint64)
    assert all(oracle_py.xxh64(int(a)) == int(b) for a, b in zip(kat_in, kat_out)), "oracle xxh64 differs"
    if not check_only:
        np.savez_compressed(os.path.join(HERE, "xxh64_kat.npz"), inputs=kat_in, outputs=kat_out)

    for name, (gp, rps) in CASES.items():
        genome = synth.make_genome(gp)
        reads = None
        for rp in rps:
            rr = synth.make_reads(genome, rp)
            reads = rr if reads is None else concat_reads(reads, rr)
        reads = concat_reads(reads, to_reads(edge_reads(genome)))
        idx = oracle_py.Index.build(p, genome)
        info = idx.info()
        with tempfile.TemporaryDirectory() as td:
            sti = os.path.join(td, "idx.sti")
            idx.write_sti(sti)
            sti_bytes = open(sti, "rb").read()
            q, qoff, frac, resc, nams, noff = run_reference(reads, sti, td)
        # oracle against the reference
        onams, ooff, ofrac, oresc = idx.map_reads(reads, abi.map_options(rescue_level=RESCUE_LEVEL))
        bad_q = bad_n = 0
        for i in range(reads.n):
            s = bytes(reads.seq[int(reads.offsets[i]) : int(reads.offsets[i]) + int(reads.lengths[i])])
            oq = oracle_py.randstrobes_query(p, s)
            rq = q[int(qoff[i]) : int(qoff[i + 1])]
            if len(oq) != len(rq) or any((oq[f] != rq[f]).any() for f in ("hash", "start", "end", "is_reverse")):
                bad_q += 1
            a = nams[int(noff[i]) : int(noff[i + 1])]
            b = onams[int(ooff[i]) : int(ooff[i + 1])]
            if len(a) != len(b) or any((a[f] != b[f]).any() for f in abi.NAM_COMPARED):
                bad_n += 1
        bad_f = int((frac != ofrac).sum())
        bad_r = int((resc != oresc).sum())
        print(f"{name}: reads={reads.n} entries={info.size} bits={info.bits} filter_cutoff={info.filter_cutoff} "
              f"queries={len(q)} nams={len(nams)} rescued={int(resc.sum())} | oracle mismatches: "
              f"queries={bad_q} nams={bad_n} frac={bad_f} rescued={bad_r}")
        assert bad_q == bad_n == bad_f == bad_r == 0, "oracle disagrees with the reference"
        if check_only:
            continue
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            genome_2bit=pack_acgt(genome.seq), genome_lengths=genome.lengths,
            read_seq=reads.seq, read_offsets=reads.offsets, read_lengths=reads.lengths,
            read_length_param=np.int32(READ_LENGTH), rescue_level=np.int32(RESCUE_LEVEL),
            index_sha256=np.bytes_(index_digest(idx).encode()), sti_sha256=np.bytes_(hashlib.sha256(sti_bytes).hexdigest().encode()),
            bits=np.int32(info.bits), filter_cutoff=np.int32(info.filter_cutoff), index_size=np.uint64(info.size),
            ref_queries=q, ref_query_offsets=qoff, ref_frac=frac, ref_rescued=resc, ref_nams=nams, ref_nam_offsets=noff,
        )


if __name__ == "__main__":
    main(check_only="--check-only" in sys.argv)
