#!/usr/bin/env bash
# Compiles include/nlgpu_reference_adapters.hpp against the reference's own
# solver headers (preconditioner_base, the conjugate gradient and its
# init_preconditioner plug-in call) and the Eigen API shim in
# oracle/eigen_shim, and links the result against libnlgpu.so, so the adapters
# INTEGRATION.md shows are checked C++.  Test infrastructure only; needs the
# reference sources (default /root/reference, which exist only in the
# development container): exits 2 without them.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="$(cd "$here/.." && pwd)"
ref="${NONLOCAL_REFERENCE:-/root/reference}"
lib="$ref/libraries"
[ -d "$lib/solvers/slae" ] || { echo "reference sources not found at $ref" >&2; exit 2; }
so="$root/nonlocal_gb300/lib/libnlgpu.so"
[ -f "$so" ] || { echo "libnlgpu.so not built" >&2; exit 3; }
tmp="$(mktemp -d)"
trap 'rm -rf "$tmp"' EXIT
cat > "$tmp/adapters.cpp" <<'CPP'
#include <iostream>
#include <memory>          // the solver headers use std::unique_ptr and the logger without including them
#include <logger/logger.hpp>
#include <solvers/slae/conjugate_gradient.hpp>
#include "nlgpu_reference_adapters.hpp"

using namespace nonlocal::slae;
using matrix_t = Eigen::SparseMatrix<double, Eigen::RowMajor, int64_t>;
using vector_t = Eigen::Matrix<double, Eigen::Dynamic, 1>;

template class nonlocal::slae::gpu_ILLT_preconditioner<double, int64_t>;

// the reference's own plug-in call (stationary_heat_equation_solver_2d.hpp:96)
void plug_in(conjugate_gradient<double, int64_t>& solver, matrix_t& local) {
    solver.template init_preconditioner<gpu_ILLT_preconditioner>(local);
}

vector_t whole_cg(const matrix_t& A, const matrix_t& local, const vector_t& b) {
    nlgpu_solve_report report{};
    return gpu_conjugate_gradient_solve<double, int64_t>(A, &local, b, 1e-10, 10000, &report);
}

int main() { return 0; }
CPP
g++ -std=c++23 -O0 -w -I "$here/eigen_shim" -I "$lib" -I "$lib/parallel" -I "$lib/logger" -I "$root/include" \
    "$tmp/adapters.cpp" "$lib/logger/logger.cpp" "$lib/parallel/MPI_utils.cpp" "$lib/parallel/OMP_utils.cpp" \
    "$lib/parallel/uniform_ranges.cpp" -o "$tmp/adapters" -L "$(dirname "$so")" -lnlgpu -Wl,-rpath,"$(dirname "$so")" -fopenmp
echo "adapters compile and link against libnlgpu.so"
