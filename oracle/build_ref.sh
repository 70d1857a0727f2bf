#!/usr/bin/env bash
# Builds oracle/_ref/ref_driver from the reference's own CPU sources: where they lie in
# the reference tree (never copied into this repository) on x86-64 hosts, or from the
# staged copy of oracle/stage_ref.sh (baseline/_ref/src, git-ignored) on any host.  Test
# and benchmark infrastructure: the binary runs the reference's find_nams /
# find_nams_rescue / StrobemerIndex / syncmer code so that the oracle restatement can
# be checked against it (tests/golden/make_golden.py) and the reference's CPU path can
# be timed (bench.py --impl reference).
#
# Usage: oracle/build_ref.sh [SOURCE_DIR]
#   SOURCE_DIR: the reference's step2/ directory (default /root/reference/step2), or a
#   staged copy.  Needs g++ and the CUDA headers (the reference headers include
#   cuda_runtime.h).  The reference's nam.cu times its stages with x86 rdtsc, so an
#   unstaged tree builds on x86-64 hosts only.
set -euo pipefail
SRC="${1:-/root/reference/step2}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$SRC/nam.cu" ]; then
  echo "reference sources not found under $SRC" >&2
  exit 3
fi
if [ "$(uname -m)" != "x86_64" ] && grep -q rdtsc "$SRC/nam.cu"; then
  echo "reference nam.cu uses x86 rdtsc; stage it with oracle/stage_ref.sh to build on $(uname -m)" >&2
  exit 4
fi
mkdir -p "$OUT"
# The CPU sources are compiled as plain C++ (see oracle/ref_shim.h for why): compiled
# by nvcc, their host code reads an uninitialised shadow of the device-qualified
# nucleotide table.
FLAGS=(-std=c++17 -w -O2 -x c++ -include "$HERE/ref_shim.h" -I"$SRC" -I/usr/local/cuda/include)
pids=()
for f in nam index randstrobes; do
  g++ "${FLAGS[@]}" -c "$SRC/$f.cu" -o "$OUT/$f.o" & pids+=($!)
done
g++ -std=c++17 -w -O2 -I"$SRC" -I/usr/local/cuda/include -c "$SRC/indexparameters.cpp" -o "$OUT/indexparameters.o" & pids+=($!)
g++ -std=c++17 -w -O2 -I"$SRC" -c "$SRC/io.cpp" -o "$OUT/io.o" & pids+=($!)
g++ "${FLAGS[@]}" -c "$HERE/ref_driver.cu" -o "$OUT/ref_driver.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -pthread -o "$OUT/ref_driver" "$OUT"/ref_driver.o "$OUT"/nam.o "$OUT"/index.o \
  "$OUT"/randstrobes.o "$OUT"/indexparameters.o "$OUT"/io.o
echo "built $OUT/ref_driver"
# the reference's read-pair code after the NAM stage (main.cu's own lines, cut by
# oracle/cut_ref_align.py into oracle/_ref, compiled as host C++ by oracle/ref_align.cpp);
# only where main.cu is present (the staged copy carries the NAM path's sources alone)
if [ -f "$SRC/main.cu" ]; then
  # only tests/golden/make_align_golden.py needs it: a failure here stops nothing below
  if python3 "$HERE/cut_ref_align.py" "$SRC/main.cu" "$OUT/main_align.inc" &&
     g++ "${FLAGS[@]}" -I"$OUT" -I"$HERE/../include" -c "$HERE/ref_align.cpp" -o "$OUT/ref_align.o" &&
     g++ -o "$OUT/ref_align" "$OUT"/ref_align.o "$OUT"/indexparameters.o "$OUT"/io.o; then
    echo "built $OUT/ref_align"
  else
    echo "oracle/_ref/ref_align not built" >&2
  fi
fi
# the reference-side binding (include/gbsa_shim.hpp) checked against the reference's own
# find_nams: needs the library built first
GBSA_DIR="$(cd "$HERE/../gpu_index_test_gb300" && pwd)"
if [ -f "$GBSA_DIR/libgbsa.so" ]; then
  g++ "${FLAGS[@]}" -I"$HERE/../include" -c "$HERE/shim_check.cu" -o "$OUT/shim_check.o"
  g++ -pthread -o "$OUT/shim_check" "$OUT"/shim_check.o "$OUT"/nam.o "$OUT"/index.o "$OUT"/randstrobes.o \
    "$OUT"/indexparameters.o "$OUT"/io.o -L"$GBSA_DIR" -lgbsa -Wl,-rpath,"$GBSA_DIR" \
    -L/usr/local/cuda/lib64 -Wl,-rpath-link,/usr/local/cuda/lib64
  echo "built $OUT/shim_check"
fi
