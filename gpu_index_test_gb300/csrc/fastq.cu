// fastq.cu — FASTQ chunk parsing into the reads layout of the mapping entry points.
//
// The reference stages its input on the host: a producer thread reads paired FASTQ
// in chunks, the records are formatted, and their sequence bytes are copied back to
// back into a host buffer with lengths and prefix sums before the copy to the device
// (step2/main.cu:63-81, 4212-4240, 4404-4430).  Here one call parses a chunk of a
// FASTQ file (or of a pair of files, mates interleaved) straight into caller buffers
// (pinned, to be passed on to gbsa_map_reads): the chunk is split at record starts
// among host threads, each thread parses its records (4-line records; CR before LF
// and blank lines between records are accepted), and the sequences are copied to
// their final places in parallel.  A record cut by the end of a chunk that is not the
// last is left for the next call (`consumed` tells where it starts).
#include <algorithm>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "runtime.h"

namespace gbsa {
namespace {

struct RecPos {
    uint64_t seq;    // first sequence byte in the chunk
    uint32_t len;    // sequence length
    uint64_t end;    // one past the record (after its last newline, or the chunk end)
};

// One line [p, *line_end) of b[0, len) without its CR; *next is the byte after the
// LF (len if the chunk ends first).  Returns false when no LF follows and the chunk
// is not the last one (the line may continue in the next chunk).
inline bool take_line(const char* b, uint64_t len, uint64_t p, bool final, uint64_t* line_end, uint64_t* next) {
    const void* nl = p < len ? std::memchr(b + p, '\n', len - p) : nullptr;
    uint64_t e;
    if (nl) {
        e = (uint64_t)(static_cast<const char*>(nl) - b);
        *next = e + 1;
    } else {
        if (!final) return false;
        e = len;
        *next = len;
    }
    *line_end = (e > p && b[e - 1] == '\r') ? e - 1 : e;
    return true;
}

// Whether a record starts at line start p: "@" header, sequence, "+" line, quality
// of the sequence's length.  Used to find split points.
bool record_at(const char* b, uint64_t len, uint64_t p) {
    if (p >= len || b[p] != '@') return false;
    uint64_t e1, n1, e2, n2, e3, n3, e4, n4;
    if (!take_line(b, len, p, false, &e1, &n1) || !take_line(b, len, n1, false, &e2, &n2)) return false;
    if (!take_line(b, len, n2, false, &e3, &n3) || n2 >= len || b[n2] != '+') return false;
    if (!take_line(b, len, n3, true, &e4, &n4)) return false;
    return e4 - n3 == e2 - n1;
}

// Parses the records starting in [s, e) of b[0, len).  On a record cut by the chunk
// end (not final) stops before it.  Returns "" or an error message.
std::string parse_range(const char* b, uint64_t len, uint64_t s, uint64_t e, bool final, std::vector<RecPos>& out) {
    uint64_t p = s;
    while (p < e) {
        if (b[p] == '\n' || b[p] == '\r') {
            ++p;
            continue;
        }
        if (b[p] != '@') return "FASTQ record does not start with '@' at byte " + std::to_string(p);
        uint64_t e1, n1, e2, n2, e3, n3, e4, n4;
        if (!take_line(b, len, p, final, &e1, &n1) || !take_line(b, len, n1, final, &e2, &n2) ||
            !take_line(b, len, n2, final, &e3, &n3) || !take_line(b, len, n3, final, &e4, &n4))
            return "";   // cut by the chunk end: left for the next call
        if (n1 >= len && final) return "FASTQ record truncated at byte " + std::to_string(p);
        if (n2 >= len || b[n2] != '+') return "FASTQ record without '+' line at byte " + std::to_string(p);
        if (e4 - n3 != e2 - n1)
            return "FASTQ quality length differs from the sequence length at byte " + std::to_string(p);
        if (e2 - n1 > 0xFFFFFFFFull) return "FASTQ sequence too long at byte " + std::to_string(p);
        out.push_back(RecPos{n1, (uint32_t)(e2 - n1), n4});
        p = n4;
    }
    return "";
}

// All complete records of a chunk, in order, parsed by up to 16 host threads.
std::vector<RecPos> parse_chunk(const char* b, uint64_t len, bool final) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const uint64_t parts = std::max<uint64_t>(1, std::min<uint64_t>(std::min(16u, hw), len / (1 << 20)));
    std::vector<uint64_t> split(parts + 1, len);
    split[0] = 0;
    for (uint64_t t = 1; t < parts; ++t) {
        uint64_t p = len * t / parts;
        while (p < len && b[p - 1] != '\n') ++p;                 // next line start
        while (p < len && !record_at(b, len, p)) {                // next record start
            const void* nl = std::memchr(b + p, '\n', len - p);
            p = nl ? (uint64_t)(static_cast<const char*>(nl) - b) + 1 : len;
        }
        split[t] = std::max(p, split[t - 1]);
    }
    std::vector<std::vector<RecPos>> recs(parts);
    std::vector<std::string> errs(parts);
    host_parallel_tasks(parts, [&](size_t t) {
        errs[t] = parse_range(b, len, split[t], split[t + 1], final && t + 1 == parts, recs[t]);
    });
    std::vector<RecPos> all;
    for (uint64_t t = 0; t < parts; ++t) {
        if (!errs[t].empty()) throw Error(GBSA_ERR_FORMAT, errs[t]);
        // parts meet at record starts: a part's last record ends where the next begins
        // (a part that stopped early, at a record cut by the chunk end, is the last one)
        if (t + 1 < parts && !recs[t].empty() && recs[t].back().end > split[t + 1])
            throw Error(GBSA_ERR_FORMAT, "malformed FASTQ record before byte " + std::to_string(split[t + 1]));
        if (t + 1 < parts && !recs[t].empty() && recs[t].back().end < split[t + 1]) {
            uint64_t q = recs[t].back().end;
            while (q < split[t + 1] && (b[q] == '\n' || b[q] == '\r')) ++q;
            if (q < split[t + 1]) throw Error(GBSA_ERR_FORMAT, "malformed FASTQ record at byte " + std::to_string(q));
        }
        all.insert(all.end(), recs[t].begin(), recs[t].end());
    }
    return all;
}

// Writes records (in the order given) to seqs / offsets / lengths, in parallel.
void write_records(const char* const* src, const RecPos* const* rec, size_t n, char* seqs, uint64_t* offsets,
                   uint32_t* lengths) {
    uint64_t acc = 0;
    for (size_t i = 0; i < n; ++i) {
        offsets[i] = acc;
        lengths[i] = rec[i]->len;
        acc += rec[i]->len;
    }
    host_parallel_for(n, [&](size_t b0, size_t e0) {
        for (size_t i = b0; i < e0; ++i) std::memcpy(seqs + offsets[i], src[i] + rec[i]->seq, rec[i]->len);
    });
}

template <class F>
int guarded_fastq(F&& f) {
    try {
        f();
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_NOMEM;
    }
}

}  // namespace
}  // namespace gbsa

using namespace gbsa;

extern "C" {

int gbsa_fastq_parse(const char* buf, uint64_t len, int final, char* seqs, uint64_t seq_capacity, uint64_t* offsets,
                     uint32_t* lengths, uint32_t read_capacity, uint32_t* n_reads, uint64_t* n_bases,
                     uint64_t* consumed) {
    return guarded_fastq([&] {
        const std::vector<RecPos> r = parse_chunk(buf, len, final != 0);
        uint64_t bases = 0;
        for (const RecPos& x : r) bases += x.len;
        *n_reads = (uint32_t)std::min<size_t>(r.size(), 0xFFFFFFFFu);
        *n_bases = bases;
        uint64_t end = r.empty() ? 0 : r.back().end;
        if (final) end = len;
        else if (r.empty()) {
            uint64_t q = 0;   // blank lines before a cut record
            while (q < len && (buf[q] == '\n' || buf[q] == '\r')) ++q;
            end = q < len ? q : len;
        }
        *consumed = end;
        if (r.size() > read_capacity || bases > seq_capacity)
            throw Error(GBSA_ERR_CAPACITY, "FASTQ chunk holds " + std::to_string(r.size()) + " reads / " +
                                               std::to_string(bases) + " bases");
        std::vector<const char*> src(r.size(), buf);
        std::vector<const RecPos*> rp(r.size());
        for (size_t i = 0; i < r.size(); ++i) rp[i] = &r[i];
        write_records(src.data(), rp.data(), r.size(), seqs, offsets, lengths);
        offsets[r.size()] = bases;
    });
}

int gbsa_fastq_parse_pairs(const char* buf1, uint64_t len1, const char* buf2, uint64_t len2, int final, char* seqs,
                           uint64_t seq_capacity, uint64_t* offsets, uint32_t* lengths, uint32_t read_capacity,
                           uint32_t* n_reads, uint64_t* n_bases, uint64_t* consumed1, uint64_t* consumed2) {
    return guarded_fastq([&] {
        const std::vector<RecPos> r1 = parse_chunk(buf1, len1, final != 0);
        const std::vector<RecPos> r2 = parse_chunk(buf2, len2, final != 0);
        if (final && r1.size() != r2.size())
            throw Error(GBSA_ERR_FORMAT, "paired FASTQ files hold " + std::to_string(r1.size()) + " and " +
                                             std::to_string(r2.size()) + " records");
        const size_t k = std::min(r1.size(), r2.size());
        uint64_t bases = 0;
        for (size_t i = 0; i < k; ++i) bases += (uint64_t)r1[i].len + r2[i].len;
        *n_reads = (uint32_t)std::min<size_t>(2 * k, 0xFFFFFFFFu);
        *n_bases = bases;
        *consumed1 = final ? len1 : (k ? r1[k - 1].end : 0);
        *consumed2 = final ? len2 : (k ? r2[k - 1].end : 0);
        if (2 * k > read_capacity || bases > seq_capacity)
            throw Error(GBSA_ERR_CAPACITY, "paired FASTQ chunks hold " + std::to_string(2 * k) + " reads / " +
                                               std::to_string(bases) + " bases");
        std::vector<const char*> src(2 * k);
        std::vector<const RecPos*> rp(2 * k);
        for (size_t i = 0; i < k; ++i) {
            src[2 * i] = buf1;
            rp[2 * i] = &r1[i];
            src[2 * i + 1] = buf2;
            rp[2 * i + 1] = &r2[i];
        }
        write_records(src.data(), rp.data(), 2 * k, seqs, offsets, lengths);
        offsets[2 * k] = bases;
    });
}

}  // extern "C"
