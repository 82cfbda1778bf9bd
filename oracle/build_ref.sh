#!/bin/sh
# build_ref.sh -- compile the reference's own CPU scattering integral, CPU
# moments and direction partition from the reference source text, for the
# development container only (the reference tree is not present elsewhere).
#
# The reference's translation units cannot be compiled as they stand: every
# one includes global_headers.h, which includes Eigen from a Windows vcpkg
# path or an absolute cluster path, plus MPI.  This recipe therefore takes the
# function bodies by line range, prepends oracle/ref_standin/standin.hpp
# (plain stand-ins for Vector3, grid_t, grid_directions_t, MPI_GET_INF) and
# appends extern "C" wrappers.  The text is piped straight into g++; no
# reference source is written into this repository.  Output:
# oracle/_ref/libref_scatter.so (git-ignored).
#
#   Illum_async.cpp:201-256   GetS, CalculateIntCPU
#   Illum_async.cpp:1101-1122 GET_FACE_TO_CELL, IntegarteDirection
#   Illum_async.cpp:1156-1178 IntegarteDirection3
#   Illum_async.cpp:1179-1247 MakeStream (flux and its divergence)
#   Illum_async.cpp:1250-1349 IntegarteDirection9, MakeDivImpuls (impulse
#                             tensor and its divergence)
#   solve_utils.cpp:177-202   GetSend, GetDisp
set -eu
REF=${RTS_REFERENCE_ROOT:-/root/reference}/solver_hllc_illum_cuda
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF" ]; then
    echo "reference tree not found at $REF; nothing to build" >&2
    exit 3
fi
mkdir -p "$OUT"
ILL="$REF/solve_module/illum/Illum_async.cpp"
UTL="$REF/solve_module/solve_utils.cpp"
{
    cat "$HERE/ref_standin/standin.hpp"
    echo '#line 201 "solve_module/illum/Illum_async.cpp"'
    iconv -f cp1251 -t utf-8 "$ILL" | sed -n '201,256p'
    echo '#line 1101 "solve_module/illum/Illum_async.cpp"'
    iconv -f cp1251 -t utf-8 "$ILL" | sed -n '1101,1122p'
    echo '#line 1156 "solve_module/illum/Illum_async.cpp"'
    iconv -f cp1251 -t utf-8 "$ILL" | sed -n '1156,1178p'
    echo '#line 1179 "solve_module/illum/Illum_async.cpp"'
    iconv -f cp1251 -t utf-8 "$ILL" | sed -n '1179,1247p'
    echo '#line 1250 "solve_module/illum/Illum_async.cpp"'
    iconv -f cp1251 -t utf-8 "$ILL" | sed -n '1250,1349p'
    echo '#line 177 "solve_module/solve_utils.cpp"'
    iconv -f cp1251 -t utf-8 "$UTL" | sed -n '177,202p'
    echo '#line 1 "oracle/ref_standin/entry.cpp"'
    cat "$HERE/ref_standin/entry.cpp"
} | g++ -x c++ -std=c++17 -O2 -ffp-contract=off -fopenmp -fPIC -shared -w -o "$OUT/libref_scatter.so" -
echo "built $OUT/libref_scatter.so"
