/* ref_align.cpp — runs the reference's own read-pair code after the NAM stage on the
 * host CPU.  Test infrastructure, built by oracle/build_ref.sh into oracle/_ref/ref_align
 * where the reference sources are present; tests/golden/make_align_golden.py runs it to
 * make the golden fixture that the oracle's restatement (and through it the GPU kernels)
 * of these rows is checked against.
 *
 * The code is the reference's step2/main.cu, cut unchanged by oracle/cut_ref_align.py into
 * oracle/_ref/main_align.inc: gpu_sort_nams (mate 1 by sort_nams_single2, mate 2 by
 * sort_nams_single), the pair classification gpu_pre_cal_type, and gpu_align_PE0..4 with
 * align_PE_part0..4, get_best_scoring_nam_pairs_sort3, rescue_read_part,
 * reverse_nam_if_needed, extend_seed_part, my_hamming_align, rescue_mate_part,
 * has_shared_substring and get_mapq.  It compiles as host C++: with cuda_runtime.h and a
 * host compiler the CUDA qualifiers are attributes the compiler ignores, a __shared__
 * array becomes a local one, my_malloc / my_free are malloc / free here, and the launch
 * index variables are set by this file for every thread of the launches main.cu makes (32
 * threads per block, GPU_thread_task_size tasks per thread), run one thread after another.
 * Each thread touches only its own tasks' data, so the order changes no result.
 *
 * This file replays the host side of main.cu:4592-4720: the sort over the 2n read ends,
 * the classification, the pairs grouped by type and each group's align launch.  Beside it,
 * for every pair with NAMs on both ends, it records get_best_scoring_nam_pairs_sort3's list
 * cut to max_tries as align_PE_part4 cuts it (main.cu:2059-2061), taken on the sorted lists
 * before the align launches (rescue_read_part reverses NAMs inside the lists).
 *
 * Usage: ref_align IN OUT
 * IN (little-endian): int32 k, max_tries, match, mismatch, gap_open, gap_extend, end_bonus;
 *   float dropoff; uint32 n_refs, uint64 ref_length[n_refs], the contigs' bytes; uint32
 *   n_pairs, uint32 len1[n_pairs], uint32 len2[n_pairs], the reads' bytes (mate 1 then
 *   mate 2, pair after pair); uint32 n_nams[2 n_pairs] for the read ends in main.cu's order
 *   (mate 1 of every pair, then mate 2 of every pair), then their NAMs as gbsa_nam records.
 * OUT: the 2 n_pairs sorted NAM lists (uint32 count + gbsa_nam records each); int32
 *   type[n_pairs]; then per pair: uint32 count + (int32 score, i1, i2) of the joint list
 *   (0 when an end has no NAMs); int32 type, mapq1, mapq2, type4_loop_size; uint32 count +
 *   records (int32 is_read1, is_extend_seed, done_align; the todo NAM as gbsa_nam; int32
 *   ref_id, ref_start, edit_distance, global_ed, score, length; uint8 is_rc, is_unaligned,
 *   gapped, 0); uint32 count + type4_nams as gbsa_nam records.
 */
#include <cstdint>
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "my_struct.hpp"
#include "randstrobes.hpp"
#include "indexparameters.hpp"
#include "aln.hpp"

#include "gbsa.h"

void* my_malloc(size_t n) { return std::malloc(n ? n : 1); }
void my_free(void* p) { std::free(p); }

// acquire_lock / release_lock (main.cu:388-397) are in the cut range but never called
static int atomicCAS(int* p, int compare, int value) {
    const int old = *p;
    if (old == compare) *p = value;
    return old;
}
static int atomicExch(int* p, int value) {
    const int old = *p;
    *p = value;
    return old;
}
static uint3 threadIdx, blockIdx;
static dim3 blockDim;

#include "main_align.inc"

namespace {

// One launch of `threads_per_block` threads per block over num_tasks tasks, as main.cu
// sizes them (blocks_per_grid = ceil(num_tasks / (32 * GPU_thread_task_size))).
template <class Body>
void launch(int num_tasks, Body&& body) {
    const int threads = 32;
    const int per_block = threads * GPU_thread_task_size;
    const int blocks = (num_tasks + per_block - 1) / per_block;
    blockDim.x = threads;
    blockDim.y = blockDim.z = 1;
    for (int b = 0; b < blocks; ++b) {
        for (int t = 0; t < threads; ++t) {
            blockIdx.x = b;
            threadIdx.x = t;
            body();
        }
    }
}

struct Reader {
    std::vector<char> buf;
    size_t p = 0;
    template <class T>
    T get() {
        T v;
        if (p + sizeof(T) > buf.size()) throw std::runtime_error("input truncated");
        std::memcpy(&v, buf.data() + p, sizeof(T));
        p += sizeof(T);
        return v;
    }
    const char* bytes(size_t n) {
        if (p + n > buf.size()) throw std::runtime_error("input truncated");
        const char* s = buf.data() + p;
        p += n;
        return s;
    }
};

Nam to_nam(const gbsa_nam& r) {
    Nam n;
    n.nam_id = r.nam_id;
    n.query_start = r.query_start;
    n.query_end = r.query_end;
    n.query_prev_hit_startpos = r.query_prev_hit_startpos;
    n.ref_start = r.ref_start;
    n.ref_end = r.ref_end;
    n.ref_prev_hit_startpos = r.ref_prev_hit_startpos;
    n.n_hits = r.n_hits;
    n.ref_id = r.ref_id;
    n.score = r.score;
    n.is_rc = r.is_rc != 0;
    return n;
}

gbsa_nam to_rec(const Nam& n) {
    gbsa_nam r;
    std::memset(&r, 0, sizeof r);
    r.nam_id = n.nam_id;
    r.query_start = n.query_start;
    r.query_end = n.query_end;
    r.query_prev_hit_startpos = n.query_prev_hit_startpos;
    r.ref_start = n.ref_start;
    r.ref_end = n.ref_end;
    r.ref_prev_hit_startpos = n.ref_prev_hit_startpos;
    r.n_hits = n.n_hits;
    r.ref_id = n.ref_id;
    r.score = n.score;
    r.is_rc = n.is_rc ? 1 : 0;
    return r;
}

struct Writer {
    std::ofstream o;
    template <class T>
    void put(const T& v) {
        o.write(reinterpret_cast<const char*>(&v), sizeof(T));
    }
    void nams(const my_vector<Nam>& v) {
        put<uint32_t>((uint32_t)v.size());
        for (int i = 0; i < v.size(); ++i) put(to_rec(v[i]));
    }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
        return 2;
    }
    Reader in;
    {
        std::ifstream f(argv[1], std::ios::binary);
        in.buf.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    }
    const int k = in.get<int32_t>();
    const int max_tries = in.get<int32_t>();
    AlignmentParameters ap;
    ap.match = in.get<int32_t>();
    ap.mismatch = in.get<int32_t>();
    ap.gap_open = in.get<int32_t>();
    ap.gap_extend = in.get<int32_t>();
    ap.end_bonus = in.get<int32_t>();
    const float dropoff = in.get<float>();

    const uint32_t n_refs = in.get<uint32_t>();
    std::vector<uint64_t> ref_len(n_refs);
    for (auto& x : ref_len) x = in.get<uint64_t>();
    GPUReferences refs;
    for (uint32_t j = 0; j < n_refs; ++j) {
        char* s = const_cast<char*>(in.bytes(ref_len[j]));
        refs.sequences.push_back(my_string(s, (int)ref_len[j]));
        refs.lengths.push_back((int)ref_len[j]);
    }
    refs.num_refs = (int)n_refs;

    const int s_len = (int)in.get<uint32_t>();
    std::vector<int> lens(s_len), lens2(s_len), pre_sum(s_len), pre_sum2(s_len);
    for (auto& x : lens) x = (int)in.get<uint32_t>();
    for (auto& x : lens2) x = (int)in.get<uint32_t>();
    std::string seqs, seqs2;
    for (int i = 0; i < s_len; ++i) {
        pre_sum[i] = (int)seqs.size();
        seqs.append(in.bytes(lens[i]), lens[i]);
        pre_sum2[i] = (int)seqs2.size();
        seqs2.append(in.bytes(lens2[i]), lens2[i]);
    }
    std::vector<my_vector<Nam>> global_nams(2 * s_len);
    std::vector<uint32_t> counts(2 * s_len);
    for (auto& c : counts) c = in.get<uint32_t>();
    for (int e = 0; e < 2 * s_len; ++e) {
        for (uint32_t i = 0; i < counts[e]; ++i) global_nams[e].push_back(to_nam(in.get<gbsa_nam>()));
    }
    if (in.p != in.buf.size()) throw std::runtime_error("trailing input");

    IndexParameters index_para = IndexParameters::from_read_length(150, k);
    MappingParameters map_param;
    map_param.dropoff_threshold = dropoff;
    map_param.max_tries = max_tries;
    map_param.max_secondary = 0;

    Writer out{std::ofstream(argv[2], std::ios::binary)};

    // main.cu:4592-4597: the NAM sort over the 2 s_len read ends
    launch(s_len * 2, [&] { gpu_sort_nams(s_len * 2, global_nams.data(), &map_param); });
    for (int e = 0; e < 2 * s_len; ++e) out.nams(global_nams[e]);

    // main.cu:4634-4644: the classification, then the pairs grouped by type
    std::vector<int> todo(s_len);
    launch(s_len, [&] { gpu_pre_cal_type(s_len, map_param.dropoff_threshold, global_nams.data(), todo.data()); });
    std::vector<int> types[5];
    for (int i = 0; i < s_len; ++i) {
        if (todo[i] < 0 || todo[i] > 4) throw std::runtime_error("pair type out of range");
        out.put<int32_t>(todo[i]);
        types[todo[i]].push_back(i);
    }

    // the joint NAM pairs of every pair with NAMs on both ends, as align_PE_part4 takes
    // them (fresh insert-size estimate, cut to max_tries)
    std::vector<std::vector<NamPair>> joint(s_len);
    for (int i = 0; i < s_len; ++i) {
        if (global_nams[i].empty() || global_nams[i + s_len].empty()) continue;
        GPUInsertSizeDistribution isize_est;
        my_vector<NamPair> j(global_nams[i].size() + global_nams[i + s_len].size());
        get_best_scoring_nam_pairs_sort3(j, global_nams[i], global_nams[i + s_len], isize_est.mu, isize_est.sigma,
                                         map_param.max_tries, 0);
        if (j.size() > map_param.max_tries) j.length = map_param.max_tries;
        for (int x = 0; x < j.size(); ++x) joint[i].push_back(j[x]);
    }

    // main.cu:4646-4720: each type's align launch over its pairs
    std::vector<uint64_t> align_info(s_len, 0);
    GPUAlignTmpRes* res = static_cast<GPUAlignTmpRes*>(std::calloc(s_len ? s_len : 1, sizeof(GPUAlignTmpRes)));
    for (int t = 0; t < 5; ++t) {
        const int n = (int)types[t].size();
        for (int i = 0; i < n; ++i) todo[i] = types[t][i];
        auto body = [&] {
            switch (t) {
            case 0:
                gpu_align_PE0(n, s_len, &index_para, align_info.data(), &ap, pre_sum.data(), lens.data(), &seqs[0],
                              pre_sum2.data(), lens2.data(), &seqs2[0], &refs, &map_param, global_nams.data(),
                              todo.data(), res);
                break;
            case 1:
                gpu_align_PE1(n, s_len, &index_para, align_info.data(), &ap, pre_sum.data(), lens.data(), &seqs[0],
                              pre_sum2.data(), lens2.data(), &seqs2[0], &refs, &map_param, global_nams.data(),
                              todo.data(), res);
                break;
            case 2:
                gpu_align_PE2(n, s_len, &index_para, align_info.data(), &ap, pre_sum.data(), lens.data(), &seqs[0],
                              pre_sum2.data(), lens2.data(), &seqs2[0], &refs, &map_param, global_nams.data(),
                              todo.data(), res);
                break;
            case 3:
                gpu_align_PE3(n, s_len, &index_para, align_info.data(), &ap, pre_sum.data(), lens.data(), &seqs[0],
                              pre_sum2.data(), lens2.data(), &seqs2[0], &refs, &map_param, global_nams.data(),
                              todo.data(), res);
                break;
            default:
                gpu_align_PE4(n, s_len, &index_para, align_info.data(), &ap, pre_sum.data(), lens.data(), &seqs[0],
                              pre_sum2.data(), lens2.data(), &seqs2[0], &refs, &map_param, global_nams.data(),
                              todo.data(), res);
            }
        };
        launch(n, body);
    }

    for (int i = 0; i < s_len; ++i) {
        out.put<uint32_t>((uint32_t)joint[i].size());
        for (const NamPair& p : joint[i]) {
            out.put<int32_t>(p.score);
            out.put<int32_t>(p.i1);
            out.put<int32_t>(p.i2);
        }
        const GPUAlignTmpRes& r = res[i];
        out.put<int32_t>(r.type);
        out.put<int32_t>(r.mapq1);
        out.put<int32_t>(r.mapq2);
        out.put<int32_t>(r.type4_loop_size);
        const int n = r.todo_nams.size();
        if (r.is_read1.size() != n || r.is_extend_seed.size() != n || r.done_align.size() != n ||
            r.align_res.size() != n)
            throw std::runtime_error("record lists of unequal length");
        out.put<uint32_t>((uint32_t)n);
        for (int x = 0; x < n; ++x) {
            out.put<int32_t>(r.is_read1[x]);
            out.put<int32_t>(r.is_extend_seed[x]);
            out.put<int32_t>(r.done_align[x]);
            out.put(to_rec(r.todo_nams[x]));
            const GPUAlignment& a = r.align_res[x];
            out.put<int32_t>(a.ref_id);
            out.put<int32_t>(a.ref_start);
            out.put<int32_t>(a.edit_distance);
            out.put<int32_t>(a.global_ed);
            out.put<int32_t>(a.score);
            out.put<int32_t>(a.length);
            const uint8_t flags[4] = {(uint8_t)a.is_rc, (uint8_t)a.is_unaligned, (uint8_t)a.gapped, 0};
            out.o.write(reinterpret_cast<const char*>(flags), 4);
        }
        out.nams(r.type4_nams);
    }
    return out.o.good() ? 0 : 1;
}
