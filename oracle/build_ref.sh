#!/usr/bin/env bash
# Builds the les-model reference into oracle/_ref/libles_ref.so, compiling
# its sources where they lie (read-only) together with oracle/ref_harness.cpp.
# Test infrastructure only: used to generate tests/golden/ and to check the
# C restatement oracle/les_oracle.c.  Needs the reference checkout; skipped
# (exit 0, nothing built) when REF is unset or holds no sources.
#
#   REF=<path to a les-model checkout> bash oracle/build_ref.sh
#
# Flags follow the reference Makefile (Makefile:2-3: g++ -std=c++17 -O2
# -fopenmp).  Two additions: -include cstdint, because src/io.cpp uses
# std::uint64_t without including <cstdint> and does not compile with GCC 13
# otherwise; and -Dmain=ref_main, so src/main.cpp's step functions link into
# the harness without its interactive main().  -ffp-contract=off keeps the
# build FMA-free on every host (x86-64 without -march has no FMA; aarch64
# GCC would otherwise contract a*b+c).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
REF="${REF:-}"
if [ -z "$REF" ] || [ ! -f "$REF/src/pressure.cpp" ]; then
  echo "build_ref: REF does not name a les-model checkout (REF='$REF'); skipping" >&2
  exit 0
fi
mkdir -p "$here/_ref"
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -shared -w \
    -include cstdint -Dmain=ref_main -I"$REF/src" \
    "$here/ref_harness.cpp" \
    "$REF/src/main.cpp" "$REF/src/pressure.cpp" "$REF/src/io.cpp" "$REF/src/statistics.cpp" \
    -o "$here/_ref/libles_ref.so"
echo "build_ref: built $here/_ref/libles_ref.so"
