#!/bin/sh
# Builds oracle/_ref/libgplsaco_ref.so from the reference's own CPU sources
# (cpp/src/faco_cpu.cpp, program_cpu.cpp, control_cpu.cpp, prepared_problem.cpp
# and sparse_graph.cpp of LinHuanli/GPLSACO, read in place, never copied) plus
# oracle/ref_shim.cpp.  Test infrastructure only.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The reference checkout is the argument, else $GPLSACO_REFERENCE, else the
# location this recipe was written against (/root/reference).
set -e
REF=${1:-${GPLSACO_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/cpp/src/faco_cpu.cpp" ]; then
    echo "reference sources not found under $REF; oracle/_ref not built" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -fPIC -shared -ffp-contract=off -I"$REF/cpp/include" \
    "$REF/cpp/src/faco_cpu.cpp" "$REF/cpp/src/program_cpu.cpp" "$REF/cpp/src/control_cpu.cpp" \
    "$REF/cpp/src/prepared_problem.cpp" "$REF/cpp/src/sparse_graph.cpp" "$HERE/ref_shim.cpp" \
    -o "$HERE/_ref/libgplsaco_ref.so"
echo "built $HERE/_ref/libgplsaco_ref.so"
