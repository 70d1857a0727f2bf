#!/usr/bin/env bash
# Builds oracle/_ref/ref_driver from the reference's own CPU sources where they lie
# (never copied into this repository).  Test infrastructure: the binary runs the
# reference's find_nams / find_nams_rescue / StrobemerIndex / syncmer code so that
# the oracle restatement can be checked against it (tests/golden/make_golden.py).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: /root/reference)
# Needs g++ and the CUDA headers (the reference headers include cuda_runtime.h).
# The reference's nam.cu times its stages with x86 rdtsc, so this builds on x86-64
# hosts only.
set -euo pipefail
REF="${1:-/root/reference}"
SRC="$REF/step2"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$SRC/nam.cu" ]; then
  echo "reference sources not found under $SRC" >&2
  exit 3
fi
if [ "$(uname -m)" != "x86_64" ]; then
  echo "reference nam.cu uses x86 rdtsc; not buildable on $(uname -m)" >&2
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
g++ -o "$OUT/ref_driver" "$OUT"/ref_driver.o "$OUT"/nam.o "$OUT"/index.o \
  "$OUT"/randstrobes.o "$OUT"/indexparameters.o "$OUT"/io.o
echo "built $OUT/ref_driver"
