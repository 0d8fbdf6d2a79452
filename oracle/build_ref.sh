#!/usr/bin/env bash
# Builds the reference's own CPU programs for the solve stage from their
# sources where they lie (read-only), into oracle/_ref/.  Nothing is copied
# and no reference file is edited: Windows-only names come from the
# force-included shims in oracle/ref_shim/.
#
# Test infrastructure only.  The binaries are the pinning oracle for
# tests/golden/make_golden.py; the product never links or runs them.
#
#   COCR_FP      Code/COCR_FP/*.cpp      the reference solver (PCOCR_2x2_Folded)
#   BuildMatrix  Code/BuildMatrix/*.cpp  the reference SLAE assembly
#   Harm1D       Code/Harm1D/*.cpp       the reference 1-D normal field
#   RegularMeshBuilder  Code/RegularMeshBuilder/*.cpp (two fixes streamed in, ref_fix_rmb.py)
#   ref_receivers  Code/OutputNu/{T_Brick,OutputArbitrary,For_Solvers,in_out}.cpp
#                plus ref_receivers_main.cpp: the receiver evaluation
#   ref_smoothing  Code/OutputNu/{OutputResultant3d,Subdomain,Hex_Local_Matrix,
#                Portret,ElemNeib,FormatConverter,T_Brick,For_Solvers,in_out,
#                iobinary}.cpp (Subdomain.cpp through ref_fix_subdomain.py)
#                plus ref_smoothing_main.cpp and ref_shim/pardiso_shim.cpp:
#                the default (smoothing) receiver output
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default $MTCALC_REFERENCE_ROOT, else a `reference` directory beside the repository)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${MTCALC_REFERENCE_ROOT:-$HERE/../../reference}}"
OUT="$HERE/_ref"
SHIM="$HERE/ref_shim"
mkdir -p "$OUT"

if [ ! -d "$REF/Code/COCR_FP" ]; then
    echo "build_ref: no reference sources at $REF; nothing to build" >&2
    exit 0
fi

CXX="${CXX:-g++}"
# `intn` is a typo for `int n` in COCR_FP/rci.h:63 and COCR_FP/T_Mapping.h:40;
# the macro restores the declaration without touching the file.
COMMON=(-O2 -fopenmp -fpermissive -w -std=gnu++14 -D'intn=int n'
        -include "$SHIM/msvc_compat.h" -I "$SHIM/include")

build_prog() {
    local name="$1"; shift
    local src="$REF/Code/$name"
    local objdir="$OUT/obj_$name"
    mkdir -p "$objdir"
    local objs=()
    for f in "$src"/*.cpp; do
        local o="$objdir/$(basename "${f%.cpp}").o"
        "$CXX" "${COMMON[@]}" "$@" -I "$src" -c "$f" -o "$o" &
        objs+=("$o")
    done
    wait
    "$CXX" -fopenmp -o "$OUT/$name" "${objs[@]}"
    echo "build_ref: $OUT/$name"
}

build_prog COCR_FP
build_prog BuildMatrix -include "$SHIM/llp64.h"
build_prog Harm1D -include "$SHIM/llp64.h"

# Receiver evaluation (direct path) of Code/OutputNu: four of its sources plus
# the harness oracle/ref_receivers_main.cpp.  Only those four are compiled: the
# rest of OutputNu needs MKL PARDISO.
build_receivers() {
    local src="$REF/Code/OutputNu"
    local objdir="$OUT/obj_OutputNu"
    mkdir -p "$objdir"
    local flags=("${COMMON[@]}" -I "$SHIM/mkl" -I "$src")
    local objs=()
    for n in T_Brick OutputArbitrary For_Solvers in_out; do
        "$CXX" "${flags[@]}" -c "$src/$n.cpp" -o "$objdir/$n.o" &
        objs+=("$objdir/$n.o")
    done
    "$CXX" "${flags[@]}" -c "$HERE/ref_receivers_main.cpp" -o "$objdir/main.o" &
    objs+=("$objdir/main.o")
    wait
    "$CXX" -fopenmp -o "$OUT/ref_receivers" "${objs[@]}"
    echo "build_ref: $OUT/ref_receivers"
}
build_receivers

# Receiver output by subdomain smoothing (the reference's default path):
# the OutputNu classes it needs, built as for Windows' 4-byte `long`
# (llp64.h: Subdomain passes int arrays through `long*`), with PARDISO
# replaced by oracle/ref_shim/pardiso_shim.cpp.  iobinary.cpp defines both
# the int and the long binary readers, so it is built without llp64.h.
build_smoothing() {
    local src="$REF/Code/OutputNu"
    local objdir="$OUT/obj_OutputNu_smoothing"
    mkdir -p "$objdir"
    local flags=("${COMMON[@]}" -include "$SHIM/llp64.h" -I "$SHIM/mkl" -I "$src")
    local objs=()
    for n in OutputResultant3d Hex_Local_Matrix Portret ElemNeib FormatConverter T_Brick \
             For_Solvers in_out; do
        "$CXX" "${flags[@]}" -c "$src/$n.cpp" -o "$objdir/$n.o" &
        objs+=("$objdir/$n.o")
    done
    python3 "$HERE/ref_fix_subdomain.py" "$REF" |
        "$CXX" "${flags[@]}" -x c++ -c - -o "$objdir/Subdomain.o" &
    objs+=("$objdir/Subdomain.o")
    "$CXX" "${COMMON[@]}" -I "$SHIM/mkl" -I "$src" -c "$src/iobinary.cpp" -o "$objdir/iobinary.o" &
    objs+=("$objdir/iobinary.o")
    "$CXX" "${flags[@]}" -c "$SHIM/pardiso_shim.cpp" -o "$objdir/pardiso_shim.o" &
    objs+=("$objdir/pardiso_shim.o")
    "$CXX" "${flags[@]}" -c "$HERE/ref_smoothing_main.cpp" -o "$objdir/main.o" &
    objs+=("$objdir/main.o")
    wait
    "$CXX" -fopenmp -o "$OUT/ref_smoothing" "${objs[@]}"
    echo "build_ref: $OUT/ref_smoothing"
}
build_smoothing

# RegularMeshBuilder (Code/RegularMeshBuilder): main.cpp passes through
# oracle/ref_fix_rmb.py (two compile/run fixes, streamed into the compiler;
# no copy is written) and is built with BasicOperations.cpp.
build_meshbuilder() {
    local src="$REF/Code/RegularMeshBuilder"
    local objdir="$OUT/obj_RegularMeshBuilder"
    mkdir -p "$objdir"
    local flags=("${COMMON[@]}" -include cmath -include cfloat -I "$src")
    python3 "$HERE/ref_fix_rmb.py" "$REF" | "$CXX" "${flags[@]}" -x c++ -c - -o "$objdir/main.o" &
    "$CXX" "${flags[@]}" -c "$src/BasicOperations.cpp" -o "$objdir/BasicOperations.o" &
    wait
    "$CXX" -o "$OUT/RegularMeshBuilder" "$objdir/main.o" "$objdir/BasicOperations.o"
    echo "build_ref: $OUT/RegularMeshBuilder"
}
build_meshbuilder
