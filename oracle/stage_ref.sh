#!/usr/bin/env bash
# Stages the reference's CPU sources of the seeding -> lookup -> NAM path for the
# reference arm of the benchmark on hosts without the reference tree (the GPU host is
# arm64): copies them, unchanged but for one line, into baseline/_ref/src/ (git-ignored;
# never part of this repository), from where oracle/build_ref.sh builds the reference's
# own CPU code there.
#
# The one change: step2/nam.cu times its stages with the x86 instruction rdtsc
# (nam.cu:86-90, GetTime), which does not assemble on arm64; its inline-assembly line
# is replaced by a read of std::chrono::steady_clock.  The timers only feed the
# reference's own progress prints; the path's arithmetic is untouched.
#
# Usage: oracle/stage_ref.sh [REFERENCE_ROOT] [DEST]   (default /root/reference, baseline/_ref/src)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
DEST="${2:-$HERE/../baseline/_ref/src}"
SRC="$REF/step2"
if [ ! -f "$SRC/nam.cu" ]; then
  echo "reference sources not found under $SRC" >&2
  exit 3
fi
mkdir -p "$DEST/pdqsort"
for f in nam.cu nam.hpp index.cu index.hpp randstrobes.cu randstrobes.hpp indexparameters.cpp indexparameters.hpp \
         io.cpp io.hpp my_struct.hpp hash.hpp exceptions.hpp refs.hpp logger.hpp timer.hpp robin_hood.h; do
  cp "$SRC/$f" "$DEST/$f"
done
cp "$SRC/pdqsort/pdqsort.h" "$DEST/pdqsort/pdqsort.h"
# GetTime: the rdtsc line becomes a steady_clock read (hi:lo of its tick count)
python3 - "$DEST/nam.cu" <<'PY'
import sys
p = sys.argv[1]
s = open(p).read()
old = 'asm volatile ("rdtsc" : "=a" (lo), "=d" (hi));'
assert s.count(old) == 1, "GetTime's rdtsc line not found"
new = ('{ const unsigned long long t = (unsigned long long)std::chrono::steady_clock::now().time_since_epoch().count(); '
       'lo = (unsigned int)t; hi = (unsigned int)(t >> 32); }')
s = s.replace(old, new)
s = '#include <chrono>\n' + s
open(p, 'w').write(s)
PY
echo "staged reference CPU sources in $DEST (GetTime made portable)"
