#!/bin/sh
# Builds the reference project's own solver sources into executables under oracle/_ref/.
# TEST INFRASTRUCTURE ONLY: the executables pin the CPU restatement (shll_oracle.c) bit for bit
# and generate the golden fixtures in tests/golden/.  They are never committed (oracle/_ref/ is
# git-ignored) and nothing in the product runs them.
#
# The sources are read where they lie: the reference's root directory is the first argument (or
# REF_ROOT).  Each variant is a
# stream edit into a temporary directory that changes only:
#   * the compile-time problem size (const int N / NX / NY),
#   * optionally the end time (const float TOTAL_TIME),
#   * float -> double for the FP64 variants,
#   * the results.dat format %e -> %.17g (so values round-trip exactly), and
#   * Save_Results() enabled where the reference commented it out, and
#   * base-omp only: the hard-coded omp_set_num_threads(16) -> 2 threads.
# Compiler flags follow the reference makefiles (gcc -O3 -lm; -fopenmp for base-omp).
# Usage: oracle/make_ref.sh <reference root>   (builds the fixed set used by the tests)
set -eu
REF=${1:-${REF_ROOT:-}}
if [ -z "$REF" ]; then
    echo "make_ref: usage: make_ref.sh <reference root> (or REF_ROOT=...); nothing built" >&2
    exit 0
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/base-c/base_shll.c" ]; then
    echo "make_ref: reference sources not found under $REF; nothing built" >&2
    exit 0
fi
mkdir -p "$OUT"
TMP=$(mktemp -d "$OUT/tmp.XXXXXX")
trap 'rm -rf "$TMP"' EXIT

# patch <src> <dst> <prec:32|64> <sed expressions...>
patch_src() {
    src=$1; dst=$2; prec=$3; shift 3
    tr -d '\r' < "$src" > "$TMP/in.c"
    sed -e 's/%e/%.17g/g' \
        -e 's#^\( *\)// *Save_Results();#\1Save_Results();#' \
        -e 's#^\( *\)//Save_Results();#\1Save_Results();#' \
        "$@" "$TMP/in.c" > "$TMP/p.c"
    if [ "$prec" = 64 ]; then sed -e 's/float/double/g' "$TMP/p.c" > "$dst"; else cp "$TMP/p.c" "$dst"; fi
}

# 1D first order (base-c/base_shll.c)
for n in 8 64 256 1024 2048; do
    for prec in 32 64; do
        patch_src "$REF/base-c/base_shll.c" "$TMP/b1d.c" $prec -e "s/^const int N = 256;/const int N = $n;/"
        gcc -O3 -o "$OUT/base_shll_f${prec}_n${n}" "$TMP/b1d.c" -lm 2>/dev/null
    done
done

# 2D first order (base-c/base_shll_2d.c); 32x24 checks a non-square grid
for sz in 16x16 32x24 64x64 256x256; do
    nx=${sz%x*}; ny=${sz#*x}
    for prec in 32 64; do
        patch_src "$REF/base-c/base_shll_2d.c" "$TMP/b2d.c" $prec \
            -e "s/^const int NX = 256;/const int NX = $nx;/" -e "s/^const int NY = 256;/const int NY = $ny;/"
        gcc -O3 -o "$OUT/base_shll_2d_f${prec}_${sz}" "$TMP/b2d.c" -lm 2>/dev/null
    done
done

# 2D second order, minmod, outflow walls (base-c/2nd_order_base_shll.c); end time 0.2
for sz in 16x16 32x24 64x64; do
    nx=${sz%x*}; ny=${sz#*x}
    for prec in 32 64; do
        patch_src "$REF/base-c/2nd_order_base_shll.c" "$TMP/o2.c" $prec \
            -e "s/^const int NX = 256;/const int NX = $nx;/" -e "s/^const int NY = 256;/const int NY = $ny;/" \
            -e "s/^const float TOTAL_TIME = 0.8;/const float TOTAL_TIME = 0.2;/"
        gcc -O3 -o "$OUT/o2_2d_f${prec}_${sz}" "$TMP/o2.c" -lm 2>/dev/null
    done
done

# 2D second order with the MC limiter (base-omp/2nd_order_base_shll.c), 2 threads, end time 0.05
for sz in 32x32; do
    nx=${sz%x*}; ny=${sz#*x}
    for prec in 32 64; do
        patch_src "$REF/base-omp/2nd_order_base_shll.c" "$TMP/omp.c" $prec \
            -e "s/^const int NX = 1024;/const int NX = $nx;/" -e "s/^const int NY = 1024;/const int NY = $ny;/" \
            -e "s/^const float TOTAL_TIME = 0.3;/const float TOTAL_TIME = 0.05;/" \
            -e "s/omp_set_num_threads(16);/omp_set_num_threads(2);/"
        gcc -O3 -fopenmp -o "$OUT/omp_mc_2d_f${prec}_${sz}" "$TMP/omp.c" -lm 2>/dev/null
    done
done
echo "make_ref: built $(ls "$OUT" | wc -l) reference executables in $OUT"
