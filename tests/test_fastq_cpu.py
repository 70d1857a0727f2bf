"""FASTQ chunk parsing (host code of the C-ABI, no GPU needed) against a plain
Python reading of the same text: sequences, offsets, lengths, chunk carry-over,
mate interleaving and the format errors."""
import numpy as np
import pytest

from gpu_index_test_gb300 import native


def records_of(text):
    """Plain reading: 4-line records, CR stripped, blank lines between records skipped."""
    lines = [l[:-1] if l.endswith("\r") else l for l in text.split("\n")]
    out, i = [], 0
    while i < len(lines):
        if lines[i] == "":
            i += 1
            continue
        assert lines[i].startswith("@") and lines[i + 2].startswith("+")
        out.append(lines[i + 1])
        i += 4
    return out


def fastq(seqs, rng, crlf=False, at_quality=False):
    nl = "\r\n" if crlf else "\n"
    alphabet = np.frombuffer(b"@IJ#5+", np.uint8)
    parts = []
    for i, s in enumerate(seqs):
        q = alphabet[rng.integers(0, len(alphabet), len(s))].tobytes().decode() if at_quality else "I" * len(s)
        parts.append(f"@read{i} extra{nl}{s}{nl}+{nl}{q}{nl}")
    return "".join(parts)


def random_seqs(rng, n, lo=1, hi=300):
    alphabet = np.frombuffer(b"ACGTNacgt", np.uint8)
    lens = rng.integers(lo, hi, n)
    codes = alphabet[rng.integers(0, len(alphabet), int(lens.sum()))].tobytes().decode()
    ends = np.cumsum(lens)
    return [codes[e - l:e] for e, l in zip(ends, lens)]


def check(reads, expected):
    assert reads.n == len(expected)
    got = [bytes(reads.seq[int(o):int(o) + int(l)]).decode() for o, l in zip(reads.offsets, reads.lengths)]
    assert got == expected


@pytest.mark.parametrize("crlf", [False, True])
def test_parse_whole_file(crlf):
    rng = np.random.default_rng(1)
    seqs = random_seqs(rng, 500)
    text = fastq(seqs, rng, crlf=crlf)
    reads, used = native.fastq_parse(text.encode())
    check(reads, seqs)
    assert used == len(text)


def test_blank_lines_and_no_final_newline():
    text = "@a\nACGT\n+\nIIII\n\n\n@b\nGG\n+b\n!!"
    reads, used = native.fastq_parse(text.encode(), final=True)
    check(reads, ["ACGT", "GG"])
    assert used == len(text)


def test_chunks_carry_cut_records():
    """Fed in chunks cut at arbitrary bytes, with the unconsumed tail passed again."""
    rng = np.random.default_rng(2)
    seqs = random_seqs(rng, 2000)
    data = fastq(seqs, rng).encode()
    got, pos, carry = [], 0, b""
    cuts = sorted(rng.integers(0, len(data), size=40).tolist()) + [len(data)]
    for c in cuts:
        chunk = carry + data[pos:c]
        pos = c
        final = c == len(data)
        reads, used = native.fastq_parse(chunk, final=final)
        got += [bytes(reads.seq[int(o):int(o) + int(l)]).decode() for o, l in zip(reads.offsets, reads.lengths)]
        carry = chunk[used:]
    assert got == seqs and carry == b""


def test_large_chunk_split_among_threads():
    """Several MB are parsed by several threads; quality strings that start with '@'
    must not be taken for record starts."""
    rng = np.random.default_rng(3)
    seqs = random_seqs(rng, 40000, 50, 250)
    text = fastq(seqs, rng, at_quality=True)
    assert len(text) > 8 << 20
    reads, used = native.fastq_parse(text.encode())
    check(reads, seqs)
    assert used == len(text)


def test_pairs_interleaved_and_carried():
    rng = np.random.default_rng(4)
    s1, s2 = random_seqs(rng, 300), random_seqs(rng, 300)
    t1, t2 = fastq(s1, rng).encode(), fastq(s2, rng).encode()
    # first chunks: 100 records of file 1, a cut part of file 2
    c1 = t1[: t1.index(b"@read100 ")]
    c2 = t2[: t2.index(b"@read80 ") + 7]
    reads, u1, u2 = native.fastq_parse_pairs(c1, c2, final=False)
    check(reads, [x for p in zip(s1[:80], s2[:80]) for x in p])
    assert u1 == t1.index(b"@read80 ") and u2 == t2.index(b"@read80 ")
    reads, u1b, u2b = native.fastq_parse_pairs(t1[u1:], t2[u2:], final=True)
    check(reads, [x for p in zip(s1[80:], s2[80:]) for x in p])


@pytest.mark.parametrize("text", [
    "ACGT\n+\nIIII\n",              # no '@' header
    "@a\nACGT\nIIII\n+\n",          # no '+' line in third place
    "@a\nACGT\n+\nIII\n",           # quality shorter than the sequence
])
def test_format_errors(text):
    with pytest.raises(native.GbsaError) as e:
        native.fastq_parse(text.encode())
    assert e.value.code == 9


def test_pairs_of_different_lengths_rejected():
    rng = np.random.default_rng(5)
    with pytest.raises(native.GbsaError):
        native.fastq_parse_pairs(fastq(random_seqs(rng, 5), rng).encode(), fastq(random_seqs(rng, 4), rng).encode())
