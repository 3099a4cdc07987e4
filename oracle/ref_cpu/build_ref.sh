#!/bin/sh
# TEST INFRASTRUCTURE ONLY (oracle).
#
# Builds the unmodified reference program (IsidoroGlez/micSA-EA-MC, PROGRAM/)
# for the HOST CPU, so that its own kernels and host code produce golden
# outputs in a container without a GPU.
#
#   usage: MICSA_REFERENCE_DIR=<reference checkout> build_ref.sh L NR [MAXNSAMPLES] [OUTDIR]
#
# Compile-time settings follow PROGRAM/Makefile:1-6 (-DNBETAS=1
# -DNUMBITSPREBUSQUEDAS=10 -DJANUS -DWALK) with L from the command line.
# NR (header.h:17) and MAXNSAMPLES (header.h:20) are plain #defines in the
# reference; a copy of header.h with those two lines substituted is written to
# a temporary directory under /tmp, used for the compile and deleted again.
# main.cu is streamed through sed to turn the `<<<...>>>` launch syntax into a
# call of the serial launcher in cuda_emu.h; no reference source is stored.
# The result is oracle/_ref/micsa_ref_L<L>_NR<NR>_MS<MS> (git-ignored).
set -eu
L=$1
NR=$2
MS=${3:-2}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=${4:-$HERE/../_ref}
[ -n "${MICSA_REFERENCE_DIR:-}" ] || { echo "MICSA_REFERENCE_DIR (the reference sources) is not set" >&2; exit 3; }
REF=$MICSA_REFERENCE_DIR/PROGRAM
[ -f "$REF/src/main.cu" ] || { echo "reference sources not found at $REF" >&2; exit 3; }
mkdir -p "$OUT"
OUT=$(cd "$OUT" && pwd)
BIN="$OUT/micsa_ref_L${L}_NR${NR}_MS${MS}"
TMP=$(mktemp -d /tmp/micsa_refcpu.XXXXXX)
trap 'rm -rf "$TMP"' EXIT
mkdir -p "$TMP/include" "$TMP/src" "$TMP/obj"

sed -e "s|^#define NR 16\$|#define NR ${NR}|" \
    -e "s|^#define MAXNSAMPLES 2\$|#define MAXNSAMPLES ${MS}|" \
    -e "s|^#include \"random_generator.h\"|#include \"$REF/include/random_generator.h\"|" \
    "$REF/include/header.h" > "$TMP/include/header.h"
grep -q "^#define NR ${NR}\$" "$TMP/include/header.h"
grep -q "^#define MAXNSAMPLES ${MS}\$" "$TMP/include/header.h"

DEFS="-DL=${L} -DNBETAS=1 -DNUMBITSPREBUSQUEDAS=10 -DJANUS -DWALK"
CXX="g++ -O2 -m64 -mcmodel=large -w -x c++"

# Host C files: compiled from stdin inside $TMP/src so that their
# "../include/header.h" resolves to the substituted copy.
for f in ini io med timing; do
  (cd "$TMP/src" && $CXX $DEFS -c - -o "$TMP/obj/$f.o" < "$REF/src/$f.c")
done
# random_generator.cu holds host code only and does not depend on NR.
$CXX $DEFS -include string.h -c "$REF/src/random_generator.cu" -o "$TMP/obj/random_generator.o"
# main.cu: launch syntax rewritten in the pipe, CUDA runtime emulated.
sed -E \
    -e 's/([A-Za-z_][A-Za-z0-9_]*)<<<([^>]*)>>>\(/EMU_LAUNCH(\1, \2)(/' \
    -e "s|\"\\.\\./include/cudamacro\\.h\"|\"$REF/include/cudamacro.h\"|" \
    -e "s|\"\\.\\./include/fill_bits\\.h\"|\"$REF/include/fill_bits.h\"|" \
    "$REF/src/main.cu" | \
  (cd "$TMP/src" && $CXX -std=c++17 $DEFS -include "$HERE/cuda_emu.h" -c - -o "$TMP/obj/main.o")
g++ -m64 -mcmodel=large "$TMP"/obj/*.o -o "$BIN" -lquadmath -lpthread -lm
echo "$BIN"
