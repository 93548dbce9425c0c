#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure only).
#
#   oracle/liboracle.so      the C restatement (bsm_oracle.c) + deterministic
#                            BLAS shim; built anywhere (also on the GPU host).
#   oracle/_ref/libref.so    the UNMODIFIED reference headers, compiled where
#                            they lie, behind ref_wrapper.cpp's C entry points,
#                            linked against the same BLAS shim.
#   oracle/_ref/occ_ri_k_step
#                            the reference's own live driver (all of its .cpp
#                            files, as its Makefile links them) on the shim.
#
# The reference part is built only when REF_DIR (default: a checkout named
# "reference" beside this repository) holds the reference sources;
# outputs go to oracle/_ref/ (git-ignored).  Parity flags: -O2
# -ffp-contract=off (the reference's -Ofast would let the compiler reorder
# and fuse the Winograd sums; no -march=native so it builds on any host).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_DIR="${REF_DIR:-$HERE/../../reference}"
CC="${CC:-gcc}"
CXX="${CXX:-g++}"
FLAGS="-O2 -ffp-contract=off -fPIC -fopenmp"

"$CC" $FLAGS -std=c11 -shared -o "$HERE/liboracle.so" "$HERE/bsm_oracle.c" "$HERE/naive_blas.c" -lm -ldl

if [ -f "$REF_DIR/strassen.hpp" ] && [ -f "$REF_DIR/occ_ri_k_step.cpp" ]; then
    mkdir -p "$HERE/_ref"
    CXXF="$FLAGS -std=c++20 -w -I$REF_DIR -I$HERE"
    "$CXX" $CXXF -shared -o "$HERE/_ref/libref.so" "$HERE/ref_wrapper.cpp" \
        "$REF_DIR/blaslapack.cpp" "$REF_DIR/matrix.cpp" -x c "$HERE/naive_blas.c" -lm -ldl
    # the reference's Makefile links every .cpp into one binary (Makefile:7-13)
    "$CXX" $CXXF -o "$HERE/_ref/occ_ri_k_step" "$REF_DIR/occ_ri_k_step.cpp" "$REF_DIR/main.cpp" \
        "$REF_DIR/3c_2c_transform.cpp" "$REF_DIR/matrix.cpp" "$REF_DIR/blaslapack.cpp" \
        -x c "$HERE/naive_blas.c" -lm -ldl
fi
