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
#
# A second library, oracle/_ref/libref_sweep.so, holds the reference's
# transport sweep and the structures it reads, with
# oracle/ref_standin/sweep_standin.hpp in front and the harness of
# sweep_entry_head.cpp / sweep_entry_tail.cpp around the sweep loop:
#   make_illum_struct/struct_short_characteristics_calculations.cpp:102-118,
#       124-128, 146-183  FromLocalToGlobalTetra, FromPlaneToTetra, BaseTetra_t
#   utils/grid_geometry/geometry_solve.cpp:8-56, 109-159, 212-227
#       SetBasis, Make2dPoint, IntersectionWithPlane, InTriangle, GetInAndOutFaces
#   make_illum_struct/struct_short_characteristics_logic_function.cpp:10-73,
#       222-297  MakeArrayX, CalculateNodeValue, GetNodes
#   build_graph/build_graph_calculation.cpp:92-121, 347-391, 482-510
#       FindInAndOutFaces, InitFacesState, FindNumberOfAllInnerFaceAndKnew,
#       FindCurCell, NewStep
#   solve_module/illum/illum_utils.cpp:407-474  BoundaryConditions
#   solve_module/illum/Illum_async.cpp:172-199, 259-510, 726-784
#       CalculateIllumeOnInnerFace, GetCurIllum, ReCalcIllum, the sweep loop
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
# the reference tree: RTS_REFERENCE_ROOT, else "reference" beside the repository root
REF=${RTS_REFERENCE_ROOT:-$HERE/../../reference}/solver_hllc_illum_cuda
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

piece() {  # piece FILE FIRST LAST: the reference's lines FIRST..LAST, with their origin
    echo "#line $2 \"$1\""
    iconv -f cp1251 -t utf-8 "$REF/$1" | sed -n "$2,$3p"
}
{
    cat "$HERE/ref_standin/sweep_standin.hpp"
    piece make_illum_struct/struct_short_characteristics_calculations.cpp 102 118
    piece make_illum_struct/struct_short_characteristics_calculations.cpp 124 128
    piece make_illum_struct/struct_short_characteristics_calculations.cpp 146 183
    echo 'static const BaseTetra_t base_tetra_geo;'
    piece utils/grid_geometry/geometry_solve.cpp 8 56
    piece utils/grid_geometry/geometry_solve.cpp 109 159
    piece utils/grid_geometry/geometry_solve.cpp 212 227
    piece make_illum_struct/struct_short_characteristics_logic_function.cpp 10 73
    piece make_illum_struct/struct_short_characteristics_logic_function.cpp 222 297
    piece build_graph/build_graph_calculation.cpp 92 121
    piece build_graph/build_graph_calculation.cpp 347 391
    piece build_graph/build_graph_calculation.cpp 482 510
    piece solve_module/illum/illum_utils.cpp 407 474
    piece solve_module/illum/Illum_async.cpp 172 199
    piece solve_module/illum/Illum_async.cpp 259 510
    echo '#line 1 "oracle/ref_standin/sweep_entry_head.cpp"'
    cat "$HERE/ref_standin/sweep_entry_head.cpp"
    piece solve_module/illum/Illum_async.cpp 726 784
    echo '#line 1 "oracle/ref_standin/sweep_entry_tail.cpp"'
    cat "$HERE/ref_standin/sweep_entry_tail.cpp"
} | g++ -x c++ -std=c++14 -O2 -ffp-contract=off -fPIC -shared -w -o "$OUT/libref_sweep.so" -
echo "built $OUT/libref_sweep.so"
