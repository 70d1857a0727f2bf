"""Cuts the reference's post-NAM read-pair code out of its step2/main.cu, unchanged, into
oracle/_ref/main_align.inc (git-ignored; never part of this repository), for
oracle/ref_align.cpp to compile as host C++.  Test infrastructure: the binary it makes
generates the golden fixture of the pair rows (tests/golden/make_align_golden.py).

main.cu as a whole does not build here (its FASTQ reader, allocator and thrust code
need libraries that are not vendored), but the functions of the read-pair path after
the NAM sort use only my_vector / my_string (step2/my_struct.hpp) and integer and
float arithmetic.  Cut, by their first lines:
  * main.cu:194-2166, from the quick-sort helpers through align_PE_part4 (every
    function of the range, whether used or not, so that nothing is picked by hand);
  * the GPU_thread_task_size definition (main.cu:2789);
  * sort_nams_single / sort_nams_single2 (main.cu:2264-2290);
  * the launch bodies gpu_sort_nams (main.cu:3449-3470), gpu_pre_cal_type
    (main.cu:3552-3580) and gpu_align_PE0..4 (main.cu:3583-3899, without
    gpu_align_PE4_single, which the main loop does not launch).

Usage: python oracle/cut_ref_align.py MAIN_CU OUT_INC
"""
import sys


def cut(main_cu: str, out_inc: str) -> None:
    src = open(main_cu).read().split("\n")

    def first(prefix):
        hits = [i for i, line in enumerate(src) if line.startswith(prefix)]
        if len(hits) != 1:
            raise SystemExit(f"{prefix!r}: {len(hits)} matches in {main_cu}")
        return hits[0]

    def function(prefix):
        s = first(prefix)
        e = next(i for i in range(s, len(src)) if src[i] == "}")   # the closing brace at column 0
        return src[s : e + 1]

    start = first("__device__ int partition(T* data")
    if not src[start - 1].startswith("template <typename T>"):
        raise SystemExit("partition's template line not found")
    end = first("#define BLOCK_SIZE 32")
    out = src[start - 1 : end]
    out.append(src[first("#define GPU_thread_task_size")])
    for prefix in ["__device__ void sort_nams_single(", "__device__ void sort_nams_single2(",
                   "__global__ void gpu_sort_nams(", "__global__ void gpu_pre_cal_type("] + [
                      f"__global__ void gpu_align_PE{i}(" for i in range(5)]:
        out += function(prefix)
    with open(out_inc, "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 3:
        raise SystemExit(__doc__)
    cut(sys.argv[1], sys.argv[2])
