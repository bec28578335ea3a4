#!/bin/sh
# Test infrastructure, not product code: builds the UNMODIFIED reference umcx (fangq/umcx, src/umcx.cpp plus the
# two third-party headers it includes) as a CPU OpenMP binary, oracle/_ref/umcx.  The flags are those of the
# reference's own `make multi` target (src/Makefile:8,17,63-65): -std=c++11 -O3 -fopenmp -foffload=disable.
#
# The reference tree exists only on the development container.  The GPU host is a different architecture, so the
# three source files are staged (unchanged) into oracle/_ref/src/, which is git-ignored but travels with the
# working copy, and the binary is rebuilt there from that staged copy.  Nothing under oracle/_ref/ is committed.
#
# usage: sh oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT: the reference checkout; default $UMCX_REFERENCE_ROOT, else a `reference` directory beside this
#   repository.  Without one, the staged copy in oracle/_ref/src/ is built.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${UMCX_REFERENCE_ROOT:-$(dirname "$(dirname "$HERE")")/reference}}
OUT="$HERE/_ref"
mkdir -p "$OUT/src/nlohmann" "$OUT/src/zmat"
if [ -f "$REF/src/umcx.cpp" ]; then
    cp -p "$REF/src/umcx.cpp" "$OUT/src/umcx.cpp"
    cp -p "$REF/src/nlohmann/json.hpp" "$OUT/src/nlohmann/json.hpp"
    cp -p "$REF/src/zmat/zmat.h" "$OUT/src/zmat/zmat.h"
fi
if [ ! -f "$OUT/src/umcx.cpp" ]; then
    echo "build_ref: reference sources not found (neither $REF/src nor $OUT/src)" >&2
    exit 3
fi
ARCH=$(uname -m)
BIN="$OUT/umcx.$ARCH"
if [ -x "$BIN" ] && [ "$BIN" -nt "$OUT/src/umcx.cpp" ]; then
    ln -sf "umcx.$ARCH" "$OUT/umcx"
    exit 0
fi
${CXX:-g++} -std=c++11 -O3 -fopenmp -foffload=disable -w -o "$BIN.tmp" "$OUT/src/umcx.cpp"
mv "$BIN.tmp" "$BIN"
ln -sf "umcx.$ARCH" "$OUT/umcx"
echo "build_ref: built $BIN"
