#!/bin/sh
# TEST INFRASTRUCTURE ONLY (oracle).
#
# Compiles the unmodified device code of the reference program
# (IsidoroGlez/micSA-EA-MC, PROGRAM/src/main.cu: d_oneMCstepBN_multisample,
# d_Walk, d_computeEne, d_gen_rndbits_cuda) for sm_103a into a cubin, so that
# the reference's own CUDA kernels can be timed and checked on the GPU host,
# which has no copy of the reference sources.  ref_gpu_harness.cu loads the
# cubin and drives the kernels the way Monte_Carlo (main.cu:197-313) does.
#
#   usage: MICSA_REFERENCE_DIR=<reference checkout> build_ref_gpu.sh L NR [MAXNSAMPLES] [OUTDIR]
#
# Compile-time settings follow PROGRAM/Makefile:1-6 (-DNBETAS=1
# -DNUMBITSPREBUSQUEDAS=10 -DJANUS -DWALK) with L from the command line; NR
# (header.h:17) and MAXNSAMPLES (header.h:20) are substituted in a copy of
# header.h, and main.cu is compiled from a copy beside it (so that its
# "../include/header.h" finds the copy), both in a temporary directory under
# /tmp that is deleted afterwards.  No reference source is stored.  The
# result is oracle/_ref/micsa_ref_gpu_L<L>_NR<NR>_MS<MS>.cubin (git-ignored).
set -eu
L=$1
NR=$2
MS=${3:-2}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=${4:-$HERE/../_ref}
[ -n "${MICSA_REFERENCE_DIR:-}" ] || { echo "MICSA_REFERENCE_DIR (the reference sources) is not set" >&2; exit 3; }
REF=$MICSA_REFERENCE_DIR/PROGRAM
[ -f "$REF/src/main.cu" ] || { echo "reference sources not found at $REF" >&2; exit 3; }
NVCC=${NVCC:-nvcc}
command -v "$NVCC" >/dev/null 2>&1 || NVCC=/usr/local/cuda/bin/nvcc
mkdir -p "$OUT"
OUT=$(cd "$OUT" && pwd)
CUBIN="$OUT/micsa_ref_gpu_L${L}_NR${NR}_MS${MS}.cubin"
TMP=$(mktemp -d /tmp/micsa_refgpu.XXXXXX)
trap 'rm -rf "$TMP"' EXIT
mkdir -p "$TMP/include" "$TMP/src"
sed -e "s|^#define NR 16\$|#define NR ${NR}|" \
    -e "s|^#define MAXNSAMPLES 2\$|#define MAXNSAMPLES ${MS}|" \
    -e "s|^#include \"random_generator.h\"|#include \"$REF/include/random_generator.h\"|" \
    "$REF/include/header.h" > "$TMP/include/header.h"
grep -q "^#define NR ${NR}\$" "$TMP/include/header.h"
grep -q "^#define MAXNSAMPLES ${MS}\$" "$TMP/include/header.h"
cp "$REF/include/cudamacro.h" "$REF/include/fill_bits.h" "$TMP/include/"
cp "$REF/src/main.cu" "$TMP/src/main.cu"
(cd "$TMP/src" && "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 \
    -DL="${L}" -DNBETAS=1 -DNUMBITSPREBUSQUEDAS=10 -DJANUS -DWALK -o "$CUBIN" main.cu)
echo "$CUBIN"
