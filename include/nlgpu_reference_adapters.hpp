/* C++ adapters that put libnlgpu behind the reference's own interfaces
 * (NonLocFEM).  Header-only; include it after the reference's
 * solvers/slae/preconditioner_base.hpp (it needs Eigen's sparse/dense types and
 * nonlocal::slae::preconditioner_base).
 *
 *   nlgpu_check                     status code -> the reference's exceptions
 *                                   (std::domain_error for bad input,
 *                                   std::runtime_error otherwise)
 *   gpu_ILLT_preconditioner<T, I>   the GPU ILLT behind the plug-in point
 *                                   preconditioner_base<T, I>
 *                                   (preconditioner_base.hpp:8-15); selected
 *                                   where the reference selects Eigen's, e.g.
 *                                   stationary_heat_equation_solver_2d.hpp:96:
 *       solver.template init_preconditioner<slae::gpu_ILLT_preconditioner>(local.matrix().inner());
 *   gpu_conjugate_gradient_solve    one call for the whole CG loop
 *                                   (conjugate_gradient.hpp:48-79) with the ILLT
 *                                   of a second matrix, stopped on the true
 *                                   residual |b - Ax| / |b|
 *
 * The reference's matrices are Eigen::SparseMatrix<double, RowMajor, int64_t>
 * (NonLocFEM/main.cpp:14-15): their index arrays are passed as int64_t. */
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "nlgpu.h"

namespace nonlocal::slae {

inline void nlgpu_check(int status) {
    if (status == NLGPU_OK) return;
    const std::string msg = std::string{nlgpu_status_string(status)} + ": " + nlgpu_last_error();
    if (status == NLGPU_ERR_ARG) throw std::domain_error{msg};
    throw std::runtime_error{msg};
}

template<class T, class I>
class gpu_ILLT_preconditioner final : public preconditioner_base<T, I> {
    static_assert(std::is_same_v<T, double> && sizeof(I) == sizeof(int64_t) && std::is_integral_v<I>,
                  "libnlgpu takes FP64 values and 64-bit indices");
    nlgpu_ctx* _ctx = nullptr;
    int _info = int(Eigen::NumericalIssue);

    static const int64_t* indices(const I* p) noexcept { return reinterpret_cast<const int64_t*>(p); }

public:
    explicit gpu_ILLT_preconditioner(const Eigen::SparseMatrix<T, Eigen::RowMajor, I>& matrix) {
        nlgpu_check(nlgpu_create(&_ctx, nullptr));
        try {
            compute(matrix);
        } catch (...) {
            nlgpu_destroy(_ctx);
            throw;
        }
    }

    gpu_ILLT_preconditioner(const gpu_ILLT_preconditioner&) = delete;
    gpu_ILLT_preconditioner& operator=(const gpu_ILLT_preconditioner&) = delete;

    ~gpu_ILLT_preconditioner() noexcept override { nlgpu_destroy(_ctx); }

    preconditioner_base<T, I>& analyze_pattern(const Eigen::SparseMatrix<T, Eigen::RowMajor, I>&) override {
        return *this;
    }

    preconditioner_base<T, I>& factorize(const Eigen::SparseMatrix<T, Eigen::RowMajor, I>& matrix) override {
        return compute(matrix);
    }

    preconditioner_base<T, I>& compute(const Eigen::SparseMatrix<T, Eigen::RowMajor, I>& matrix) override {
        nlgpu_check(nlgpu_illt_compute(_ctx, int64_t(matrix.rows()), indices(matrix.outerIndexPtr()),
                                       indices(matrix.innerIndexPtr()), matrix.valuePtr(), &_info));
        return *this;
    }

    Eigen::Matrix<T, Eigen::Dynamic, 1> solve(const Eigen::Matrix<T, Eigen::Dynamic, 1>& x) const override {
        Eigen::Matrix<T, Eigen::Dynamic, 1> y(x.size());
        nlgpu_check(nlgpu_illt_solve(_ctx, int64_t(x.size()), x.data(), y.data()));
        return y;
    }

    Eigen::ComputationInfo computation_info() const override { return Eigen::ComputationInfo(_info); }
};

// A: the system in the reference's storage (upper part for a symmetric
// problem, diagonal first in every row); local: the matrix whose ILLT
// preconditions (p1 K_local in the stationary driver) or nullptr for none.
// Like the reference's CG, the last iterate comes back when the iteration
// limit is reached (report->converged tells).
template<class T, class I>
Eigen::Matrix<T, Eigen::Dynamic, 1> gpu_conjugate_gradient_solve(const Eigen::SparseMatrix<T, Eigen::RowMajor, I>& A,
                                                                 const Eigen::SparseMatrix<T, Eigen::RowMajor, I>* local,
                                                                 const Eigen::Matrix<T, Eigen::Dynamic, 1>& b,
                                                                 T tolerance, uintmax_t max_iterations,
                                                                 nlgpu_solve_report* report = nullptr) {
    static_assert(std::is_same_v<T, double> && sizeof(I) == sizeof(int64_t) && std::is_integral_v<I>,
                  "libnlgpu takes FP64 values and 64-bit indices");
    auto p64 = [](const I* p) { return reinterpret_cast<const int64_t*>(p); };
    nlgpu_ctx* ctx = nullptr;
    nlgpu_check(nlgpu_create(&ctx, nullptr));
    Eigen::Matrix<T, Eigen::Dynamic, 1> x(b.size());
    const int rc = nlgpu_cg_solve(ctx, int64_t(A.rows()), p64(A.outerIndexPtr()), p64(A.innerIndexPtr()),
                                  A.valuePtr(), local ? p64(local->outerIndexPtr()) : nullptr,
                                  local ? p64(local->innerIndexPtr()) : nullptr, local ? local->valuePtr() : nullptr,
                                  b.data(), nullptr, tolerance, int64_t(max_iterations), x.data(), report);
    nlgpu_destroy(ctx);
    if (rc != NLGPU_ERR_NO_CONVERGENCE) nlgpu_check(rc);
    return x;
}

}  // namespace nonlocal::slae
