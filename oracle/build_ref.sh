#!/usr/bin/env bash
# Builds the reference's own thermal-path code (headers under
# <reference>/libraries, plus its logger and parallel .cpp files) against the
# Eigen API shim in oracle/eigen_shim, into oracle/_ref/ref_driver.
# Test infrastructure only; needs the reference sources (default
# /root/reference), which exist only in the development container.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${NONLOCAL_REFERENCE:-/root/reference}"
lib="$ref/libraries"
[ -d "$lib" ] || { echo "reference sources not found at $ref" >&2; exit 2; }
mkdir -p "$here/_ref"
out="$here/_ref/ref_driver"
if [ -x "$out" ] && [ "$out" -nt "$here/ref_driver.cpp" ] && [ "$out" -nt "$here/eigen_shim/Eigen/src/shim.hpp" ]; then
    echo "up to date: $out"
    exit 0
fi
g++ -std=c++23 -O3 -fopenmp -ffp-contract=off -w \
    -I "$here/eigen_shim" -I "$lib" -I "$lib/parallel" -I "$lib/logger" \
    "$here/ref_driver.cpp" "$lib/logger/logger.cpp" "$lib/parallel/MPI_utils.cpp" \
    "$lib/parallel/OMP_utils.cpp" "$lib/parallel/uniform_ranges.cpp" \
    -o "$here/_ref/ref_driver"
echo "built $here/_ref/ref_driver"
