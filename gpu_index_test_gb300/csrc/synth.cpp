/*
 * synth.cpp — seeded synthetic reference genomes and sequencing reads.
 *
 * The reference project ships no data; its pipeline reads user FASTA/FASTQ files
 * (step2/main.cu:4190-4240).  These generators stand in for them with inputs of the
 * documented shapes: i.i.d. uniform contigs, duplicated segments at a chosen
 * divergence, repeat families, short tandem repeats, and single-end or paired-end
 * reads with substitutions and short indels.  Everything is a pure function of the
 * seed (xoshiro256** seeded through splitmix64), and contigs are generated in
 * parallel with per-contig streams so the output does not depend on thread count.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto& v : s) v = splitmix64(x);
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    inline uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    inline double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    inline uint64_t below(uint64_t n) { return n ? (uint64_t)(uniform() * (double)n) % n : 0; }
    inline int64_t range(int64_t lo, int64_t hi) { return lo + (int64_t)below((uint64_t)(hi - lo + 1)); }
    inline double normal() {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

const char kBases[4] = {'A', 'C', 'G', 'T'};

inline char comp(char c) {
    switch (c) {
        case 'A': return 'T';
        case 'C': return 'G';
        case 'G': return 'C';
        case 'T': return 'A';
        default: return 'N';
    }
}

void fill_random(Rng& r, char* out, uint64_t n) {
    uint64_t i = 0;
    while (i < n) {
        uint64_t x = r.next();
        for (int j = 0; j < 32 && i < n; ++j, ++i) {
            out[i] = kBases[x & 3];
            x >>= 2;
        }
    }
}

/* copy src → dst with per-base substitution probability `div` */
void copy_diverged(Rng& r, const char* src, char* dst, uint64_t n, double div) {
    for (uint64_t i = 0; i < n; ++i) {
        char c = src[i];
        if (r.uniform() < div) {
            char d;
            do {
                d = kBases[r.next() & 3];
            } while (d == c);
            c = d;
        }
        dst[i] = c;
    }
}

template <class Fn>
void par_for(uint32_t n, Fn&& fn) {
    const uint32_t nt = std::max(1u, std::min(n, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (uint32_t t = 0; t < nt; ++t) {
        th.emplace_back([&, t]() {
            for (uint32_t i = t; i < n; i += nt) fn(i);
        });
    }
    for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

/*
 * Genome specification.  Contig lengths are drawn uniformly in
 * [min_contig, max_contig] and scaled to sum to total_len (a single contig when
 * n_contigs == 1).  Repeat content is written over the i.i.d. background:
 *   dup_frac    fraction of bases in segmental duplications: segments of
 *               dup_min..dup_max bp copied dup_copies_min..dup_copies_max times at
 *               divergence dup_div_min..dup_div_max;
 *   fam_frac    fraction of bases in interspersed repeat families: n_families
 *               consensus elements of fam_min..fam_max bp, copies at divergence
 *               fam_div_min..fam_div_max;
 *   str_frac    fraction of bases in short tandem repeats: unit str_unit_min..
 *               str_unit_max bp, str_copies_min..str_copies_max copies.
 */
typedef struct gbsa_genome_spec {
    uint64_t seed;
    uint64_t total_len;
    uint32_t n_contigs;
    uint32_t _pad0;
    uint64_t min_contig, max_contig;
    double dup_frac;
    uint32_t dup_min, dup_max, dup_copies_min, dup_copies_max;
    double dup_div_min, dup_div_max;
    double fam_frac;
    uint32_t n_families, fam_min, fam_max, _pad1;
    double fam_div_min, fam_div_max;
    double str_frac;
    uint32_t str_unit_min, str_unit_max, str_copies_min, str_copies_max;
} gbsa_genome_spec;

/* Writes the contig lengths (n_contigs) and returns their sum. */
uint64_t gbsa_synth_contig_lengths(const gbsa_genome_spec* sp, uint64_t* lengths) {
    Rng r(sp->seed ^ 0xC0A7161ULL);
    const uint32_t n = sp->n_contigs;
    if (n == 1) {
        lengths[0] = sp->total_len;
        return sp->total_len;
    }
    std::vector<double> w(n);
    double sum = 0;
    for (uint32_t i = 0; i < n; ++i) {
        w[i] = (double)r.range((int64_t)sp->min_contig, (int64_t)sp->max_contig);
        sum += w[i];
    }
    uint64_t tot = 0;
    for (uint32_t i = 0; i < n; ++i) {
        lengths[i] = (uint64_t)((double)sp->total_len * w[i] / sum);
        tot += lengths[i];
    }
    lengths[n - 1] += sp->total_len - tot;
    return sp->total_len;
}

/* Fills out[0 .. total_len) with the contigs back to back (lengths from
 * gbsa_synth_contig_lengths).  Returns 0. */
int gbsa_synth_genome(const gbsa_genome_spec* sp, const uint64_t* lengths, char* out) {
    const uint32_t n = sp->n_contigs;
    std::vector<uint64_t> off(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i) off[i + 1] = off[i] + lengths[i];

    /* repeat-family consensus sequences, shared by all contigs */
    std::vector<std::string> fam;
    {
        Rng r(sp->seed ^ 0xFA111E5ULL);
        for (uint32_t f = 0; f < sp->n_families; ++f) {
            const uint64_t len = (uint64_t)r.range(sp->fam_min, sp->fam_max);
            std::string s(len, 'A');
            fill_random(r, &s[0], len);
            fam.push_back(std::move(s));
        }
    }

    par_for(n, [&](uint32_t c) {
        Rng r(sp->seed * 0x100000001B3ULL + c + 1);
        char* seq = out + off[c];
        const uint64_t len = lengths[c];
        fill_random(r, seq, len);
        if (len < 20000) return;

        /* interspersed repeat families */
        if (sp->fam_frac > 0 && !fam.empty()) {
            uint64_t budget = (uint64_t)(sp->fam_frac * (double)len), done = 0;
            while (done < budget) {
                const std::string& e = fam[r.below(fam.size())];
                const uint64_t el = std::min<uint64_t>(e.size(), len / 4);
                const uint64_t at = r.below(len - el);
                const double div = sp->fam_div_min + (sp->fam_div_max - sp->fam_div_min) * r.uniform();
                if (r.next() & 1) {
                    copy_diverged(r, e.data(), seq + at, el, div);
                } else {
                    std::string rc(el, 'A');
                    for (uint64_t i = 0; i < el; ++i) rc[i] = comp(e[el - 1 - i]);
                    copy_diverged(r, rc.data(), seq + at, el, div);
                }
                done += el;
            }
        }
        /* segmental duplications within the contig */
        if (sp->dup_frac > 0) {
            uint64_t budget = (uint64_t)(sp->dup_frac * (double)len), done = 0;
            std::string buf;
            while (done < budget) {
                const uint64_t sl = std::min<uint64_t>((uint64_t)r.range(sp->dup_min, sp->dup_max), len / 8);
                const uint64_t src = r.below(len - sl);
                buf.assign(seq + src, sl);
                const int copies = (int)r.range(sp->dup_copies_min, sp->dup_copies_max);
                for (int k = 0; k < copies && done < budget; ++k) {
                    const uint64_t dst = r.below(len - sl);
                    const double div = sp->dup_div_min + (sp->dup_div_max - sp->dup_div_min) * r.uniform();
                    copy_diverged(r, buf.data(), seq + dst, sl, div);
                    done += sl;
                }
            }
        }
        /* short tandem repeats */
        if (sp->str_frac > 0) {
            uint64_t budget = (uint64_t)(sp->str_frac * (double)len), done = 0;
            char unit[16];
            while (done < budget) {
                const int ul = (int)r.range(sp->str_unit_min, sp->str_unit_max);
                const int copies = (int)r.range(sp->str_copies_min, sp->str_copies_max);
                fill_random(r, unit, (uint64_t)ul);
                const uint64_t tl = std::min<uint64_t>((uint64_t)ul * (uint64_t)copies, len / 8);
                const uint64_t at = r.below(len - tl);
                for (uint64_t i = 0; i < tl; ++i) seq[at + i] = unit[i % (uint64_t)ul];
                done += tl;
            }
        }
    });
    return 0;
}

/*
 * Read specification.  Each read (or pair) picks a contig with probability
 * proportional to its length and a uniform start.  Read length is fixed
 * (len_min == len_max) or drawn log-uniformly in [len_min, len_max].  A fraction
 * paired_frac of units are pairs: a fragment of length ~Normal(insert_mean,
 * insert_sd) (at least the read length), mate 1 from its start and mate 2 the
 * reverse complement of its end; the fragment comes from either strand with equal
 * probability, as do single-end reads.  Each base then gets a substitution with
 * probability sub_rate (drawn per read in [sub_min, sub_max]) and an indel (1-3 bp,
 * insertion or deletion with equal probability) with probability indel_rate.
 * Mates are stored next to each other (mate 1 first).
 */
typedef struct gbsa_read_spec {
    uint64_t seed;
    uint32_t n_units;       /* reads (single-end) or pairs */
    uint32_t len_min, len_max;
    uint32_t _pad0;
    double paired_frac;
    double insert_mean, insert_sd;
    double sub_min, sub_max;
    double indel_rate;
} gbsa_read_spec;

/* Pass 1: number of reads and total bases of the read set (deterministic). */
int gbsa_synth_reads_size(const gbsa_read_spec* sp, uint64_t* n_reads, uint64_t* n_bases) {
    Rng r(sp->seed ^ 0x5EED5ULL);
    uint64_t nr = 0, nb = 0;
    for (uint32_t u = 0; u < sp->n_units; ++u) {
        uint32_t L = sp->len_min;
        if (sp->len_max > sp->len_min) {
            const double a = std::log((double)sp->len_min), b = std::log((double)sp->len_max);
            L = (uint32_t)std::lround(std::exp(a + (b - a) * r.uniform()));
            L = std::min(std::max(L, sp->len_min), sp->len_max);
        }
        const bool paired = r.uniform() < sp->paired_frac;
        nr += paired ? 2 : 1;
        nb += paired ? 2 * (uint64_t)L : L;
    }
    *n_reads = nr;
    *n_bases = nb;
    return 0;
}

/* Pass 2: writes the reads.  truth (may be NULL) receives per read
 * (contig, start of the source window, strand). */
/* The unit layout of gbsa_synth_reads: items[u] = first read of unit u (a single-end
 * read, or mate 1 of a pair, mate 2 following), items[n_units] = the read count. */
int gbsa_synth_read_items(const gbsa_read_spec* sp, uint32_t* items) {
    Rng shape(sp->seed ^ 0x5EED5ULL);
    uint32_t nr = 0;
    for (uint32_t u = 0; u < sp->n_units; ++u) {
        if (sp->len_max > sp->len_min) shape.uniform();   /* the length draw */
        const bool paired = shape.uniform() < sp->paired_frac;
        items[u] = nr;
        nr += paired ? 2 : 1;
    }
    items[sp->n_units] = nr;
    return 0;
}

int gbsa_synth_reads(const gbsa_read_spec* sp, const char* genome, const uint64_t* lengths, uint32_t n_contigs,
                     char* out, uint64_t* offsets, uint32_t* out_lengths, uint64_t* truth) {
    Rng shape(sp->seed ^ 0x5EED5ULL);
    std::vector<uint64_t> coff(n_contigs + 1, 0);
    for (uint32_t i = 0; i < n_contigs; ++i) coff[i + 1] = coff[i] + lengths[i];
    const uint64_t glen = coff[n_contigs];

    struct Unit {
        uint32_t L;
        bool paired;
        uint64_t read0, base0;
    };
    std::vector<Unit> units(sp->n_units);
    uint64_t nr = 0, nb = 0;
    for (uint32_t u = 0; u < sp->n_units; ++u) {
        uint32_t L = sp->len_min;
        if (sp->len_max > sp->len_min) {
            const double a = std::log((double)sp->len_min), b = std::log((double)sp->len_max);
            L = (uint32_t)std::lround(std::exp(a + (b - a) * shape.uniform()));
            L = std::min(std::max(L, sp->len_min), sp->len_max);
        }
        const bool paired = shape.uniform() < sp->paired_frac;
        units[u] = Unit{L, paired, nr, nb};
        nr += paired ? 2 : 1;
        nb += paired ? 2 * (uint64_t)L : L;
    }

    const uint32_t n_chunks = std::max(1u, std::min(sp->n_units / 1024 + 1, 4096u));
    par_for(n_chunks, [&](uint32_t ch) {
        const uint32_t a = (uint32_t)((uint64_t)sp->n_units * ch / n_chunks);
        const uint32_t b = (uint32_t)((uint64_t)sp->n_units * (ch + 1) / n_chunks);
        std::string frag, mate;
        for (uint32_t u = a; u < b; ++u) {
            Rng r(sp->seed * 0x9E3779B97F4A7C15ULL + u + 7);
            const Unit& un = units[u];
            const uint32_t L = un.L;
            uint64_t flen = L;
            if (un.paired) {
                double f = sp->insert_mean + sp->insert_sd * r.normal();
                flen = (uint64_t)std::max<double>((double)L, std::round(f));
            }
            const uint64_t need = flen + 64;   /* slack for deletions */
            /* pick a contig long enough */
            uint32_t c = 0;
            uint64_t start = 0;
            for (int tries = 0; tries < 1000; ++tries) {
                const uint64_t g = r.below(glen);
                c = (uint32_t)(std::upper_bound(coff.begin(), coff.end(), g) - coff.begin() - 1);
                if (lengths[c] > need) {
                    start = r.below(lengths[c] - need);
                    break;
                }
            }
            const char* src = genome + coff[c] + start;
            const uint64_t avail = std::min<uint64_t>(need, lengths[c] - start);
            frag.assign(src, avail);
            const bool minus = r.next() & 1;
            if (minus) {
                std::string rc(frag.size(), 'A');
                for (size_t i = 0; i < frag.size(); ++i) rc[i] = comp(frag[frag.size() - 1 - i]);
                frag.swap(rc);
            }
            const double sub = sp->sub_min + (sp->sub_max - sp->sub_min) * r.uniform();
            auto mutate = [&](const char* s, uint64_t n_avail, char* dst) {
                uint64_t i = 0, o = 0;
                while (o < L) {
                    if (i >= n_avail) {
                        dst[o++] = kBases[r.next() & 3];
                        continue;
                    }
                    if (r.uniform() < sp->indel_rate) {
                        const int n = (int)r.range(1, 3);
                        if (r.next() & 1) {
                            for (int j = 0; j < n && o < L; ++j) dst[o++] = kBases[r.next() & 3];
                        } else {
                            i += (uint64_t)n;
                        }
                        continue;
                    }
                    char ch = s[i++];
                    if (r.uniform() < sub) {
                        char d;
                        do {
                            d = kBases[r.next() & 3];
                        } while (d == ch);
                        ch = d;
                    }
                    dst[o++] = ch;
                }
            };
            const uint64_t r0 = un.read0;
            offsets[r0] = un.base0;
            out_lengths[r0] = L;
            mutate(frag.data(), frag.size(), out + un.base0);
            if (truth) {
                truth[3 * r0] = c;
                truth[3 * r0 + 1] = start;
                truth[3 * r0 + 2] = minus ? 1 : 0;
            }
            if (un.paired) {
                /* mate 2: reverse complement of the fragment end */
                const uint64_t fe = std::min<uint64_t>(flen, frag.size());
                mate.clear();
                for (uint64_t i = fe; i-- > 0;) mate.push_back(comp(frag[i]));
                offsets[r0 + 1] = un.base0 + L;
                out_lengths[r0 + 1] = L;
                mutate(mate.data(), mate.size(), out + un.base0 + L);
                if (truth) {
                    truth[3 * (r0 + 1)] = c;
                    truth[3 * (r0 + 1) + 1] = start;
                    truth[3 * (r0 + 1) + 2] = minus ? 0 : 1;
                }
            }
        }
    });
    return 0;
}

}  // extern "C"
