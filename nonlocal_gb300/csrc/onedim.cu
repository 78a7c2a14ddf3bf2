// 1D stationary nonlocal heat conduction (stationary_heat_equation_solver_1d.hpp:43-122).
//
//   mesh: one segment [0, length], `elements` Lagrange elements of order 1 or 2,
//     neighbours e +- round(r / h) inside the segment (mesh_1d.hpp:119-122, 221-232);
//   assembly: p1 * local + (1 - p1) * nonlocal element blocks
//     (thermal_conductivity_assembler.hpp:64-125, assebmler_base.hpp:112-155),
//     upper band, node 0 Dirichlet: its row goes to the bound vector, entries
//     of column 0 in other rows are dropped, unit diagonal;
//   right-hand side: flux at the right end, source integral, first-kind step;
//   solve: LDL^T of the band matrix in natural order (the reference's
//     Eigen::SimplicialCholesky<..., Upper, NaturalOrdering>).
//
// Assembly: one thread per (element, neighbour element) pair computes the
// (order+1)^2 block.  Factorisation: one CTA walks the diagonal; at step k
// every thread updates part of the trailing (bandwidth x bandwidth) window.
//
// 1D nonstationary (nonstationary_heat_equation_solver_1d.hpp:24-259):
// compute() assembles A = dt K + C (C the local capacity matrix c rho int N_i N_j,
// heat_capacity_assembler.hpp:30-58) with either end a temperature (its row and
// column routed out, unit diagonal, K's row kept as dt x bound) or a flux, and
// factors A once (LDL^T of the band).  calc_step() forms
// f = dt (flux + source) + C T_prev (inner entries of C only, as the
// reference's product), applies the first kind and solves with the factor: the
// solution the reference's ConjugateGradient reaches at machine tolerance.
#include "common.cuh"

#include <cmath>
#include <numbers>

namespace nlgpu {

namespace {

struct Line {
    int nen, nq;
    double qN[3 * 3], qNxi[3 * 3], w[3], x[3];
};

Line make_line(int order) {
    Line L{};
    L.nen = order + 1;
    L.nq = order == 1 ? 2 : 3;
    if (L.nq == 2) { L.x[0] = -1.0 / std::sqrt(3.0); L.x[1] = 1.0 / std::sqrt(3.0); L.w[0] = L.w[1] = 1.0; }
    else { L.x[0] = -std::sqrt(3.0 / 5.0); L.x[1] = 0.0; L.x[2] = std::sqrt(3.0 / 5.0); L.w[0] = 5.0 / 9.0; L.w[1] = 8.0 / 9.0; L.w[2] = 5.0 / 9.0; }
    for (int q = 0; q < L.nq; ++q) L.w[q] = L.w[q] * 1.0;
    for (int i = 0; i < L.nen; ++i)
        for (int q = 0; q < L.nq; ++q) {
            const double x = -1.0 + (L.x[q] - (-1.0)) * 1.0;
            double N, Nx;
            if (order == 1) { N = i == 0 ? (1 - x) / 2 : (1 + x) / 2; Nx = i == 0 ? -0.5 : 0.5; }
            else if (i == 0) { N = x * (x - 1) / 2; Nx = (2 * x - 1) / 2; }
            else if (i == 1) { N = (1 - x) * (1 + x); Nx = -2 * x; }
            else { N = x * (x + 1) / 2; Nx = (2 * x + 1) / 2; }
            L.qN[i * L.nq + q] = N; L.qNxi[i * L.nq + q] = Nx;
        }
    return L;
}

struct Problem1d {
    i64 E, n, nb, bw;          // elements, nodes, neighbour count, half bandwidth
    int order;
    double h, jac, r, p1, lambda, norm;
    int kind;                  // 0 bell, 1 triangle, 2 normal, 3 constant
    int fk0, fk1;              // temperature (first kind) at the left / right end
    int cv0, cv1;              // convection at the left / right end
    double h0, h1;             // their heat transfer coefficients
};

// influence_functions_1d.hpp:10-75
__device__ __forceinline__ double influence_1d(const Problem1d& P, double x, double y) {
    const double d = fabs(x - y);
    if (P.kind == 0) { const double t = d / P.r; return d < P.r ? P.norm * (1 - t * t) : 0.0; }
    if (P.kind == 1) { return d < P.r ? P.norm * (1 - d / P.r) : 0.0; }
    if (P.kind == 2) { return P.norm * exp((-0.5 / (P.r * P.r)) * ((x - y) * (x - y))); }
    return d < P.r ? P.norm : 0.0;
}

// assembler_base_1d::calc_matrix (assebmler_base.hpp:121-154): entries in the
// row or column of a first-kind end go to that end's bound vector (its row's
// entries; the diagonal becomes 1 later) or are dropped; the rest fill the
// upper band.  bound0 / boundN may be null (dropped).
__device__ __forceinline__ void band_add(const Problem1d& P, double* band, double* bound0, double* boundN, i64 row,
                                         i64 col, double v) {
    const i64 last = P.n - 1;
    if (P.fk0 && (row == 0 || col == 0)) {
        if (row == 0 && col != 0 && bound0) atomicAdd(bound0 + col, v);
        return;
    }
    if (P.fk1 && (row == last || col == last)) {
        if (row == last && col != last && boundN) atomicAdd(boundN + col, v);
        return;
    }
    if (row <= col) atomicAdd(band + row * (P.bw + 1) + (col - row), v);
}

__global__ void k_assemble_1d(Problem1d P, Line L, double* __restrict__ band, double* __restrict__ bound0,
                              double* __restrict__ boundN) {
    const i64 width = 2 * P.nb + 1;
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < P.E * width; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / width, f = e - P.nb + t % width;
        if (f < 0 || f >= P.E) continue;
        const bool nonlocal = P.p1 < 0.999;
        double xl[3], xn[3];
        for (int q = 0; q < L.nq; ++q) {
            xl[q] = P.h * double(e) + (L.x[q] - (-1.0)) * P.jac;
            xn[q] = P.h * double(f) + (L.x[q] - (-1.0)) * P.jac;
        }
        for (int i = 0; i < L.nen; ++i) {
            const i64 row = e * P.order + i;
            for (int j = 0; j < L.nen; ++j) {
                const i64 col = f * P.order + j;
                if (nonlocal) {
                    double integral = 0.0;
                    for (int qL = 0; qL < L.nq; ++qL) {
                        double inner = 0.0;
                        for (int qNL = 0; qNL < L.nq; ++qNL)
                            inner += influence_1d(P, xl[qL], xn[qNL]) * P.lambda * L.w[qNL] * L.qNxi[j * L.nq + qNL];
                        integral += L.w[qL] * L.qNxi[i * L.nq + qL] * inner;
                    }
                    band_add(P, band, bound0, boundN, row, col, (1.0 - P.p1) * integral);
                }
                if (f == e) {
                    double integral = 0.0;
                    for (int q = 0; q < L.nq; ++q) integral += P.lambda * L.w[q] * L.qNxi[i * L.nq + q] * L.qNxi[j * L.nq + q];
                    band_add(P, band, bound0, boundN, row, col, P.p1 * (integral / P.jac));
                }
            }
        }
    }
}

__global__ void k_rhs_1d(Problem1d P, Line L, double q_right, bool sin_source, double* __restrict__ f) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < P.E * L.nen; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / L.nen;
        const int i = int(t % L.nen);
        if (!sin_source) continue;
        double integral = 0.0;
        for (int q = 0; q < L.nq; ++q)
            integral += L.w[q] * L.qN[i * L.nq + q] * sin(std::numbers::pi * (P.h * double(e) + (L.x[q] - (-1.0)) * P.jac));
        atomicAdd(f + e * P.order + i, integral * P.jac);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(f + P.n - 1, q_right);
}

__global__ void k_first_kind_1d(i64 n, const double* __restrict__ bound0, double t_left, double* __restrict__ f,
                                double* __restrict__ band) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        if (i == 0) { f[0] = t_left; band[0] = 1.0; }
        else f[i] -= bound0[i] * t_left;
    }
}

// In-place band LDL^T (upper band: band[i*(bw+1) + (j-i)]) in one CTA.  Step
// k scales row k by 1/d_k after using it to update the trailing window.
// Returns false (and raises *failed) on a zero pivot.
__device__ bool band_ldlt(i64 n, i64 bw, double* __restrict__ band, int* __restrict__ failed) {
    const i64 w = bw + 1;
    __shared__ double dk;
    for (i64 k = 0; k < n; ++k) {
        if (threadIdx.x == 0) {
            dk = band[k * w];
            if (dk == 0.0) *failed = 1;
        }
        __syncthreads();
        if (dk == 0.0) return false;
        const i64 m = min(bw, n - 1 - k);   // rows k+1 .. k+m
        for (i64 t = threadIdx.x; t < m * m; t += blockDim.x) {
            const i64 a = t / m + 1, b = t % m + 1;   // row k+a, col k+b
            if (b < a) continue;
            const double uka = band[k * w + a], ukb = band[k * w + b];
            band[(k + a) * w + (b - a)] -= uka * ukb / dk;
        }
        __syncthreads();
        for (i64 t = threadIdx.x + 1; t <= m; t += blockDim.x) band[k * w + t] /= dk;
        __syncthreads();
    }
    return true;
}

__global__ void __launch_bounds__(1024) k_band_ldlt(i64 n, i64 bw, double* __restrict__ band, int* __restrict__ failed) {
    band_ldlt(n, bw, band, failed);
}

// U^T D U x = f with the factor of k_band_ldlt (unit upper U), by one warp:
// forward U^T y = f, y /= d, backward U x = y.  Every row's dot product is
// spread over the lanes and reduced by shuffles; __syncwarp orders each
// solved value before the next row reads it.
__global__ void __launch_bounds__(32) k_band_solve_warp(i64 n, i64 bw, const double* __restrict__ band,
                                                        double* __restrict__ f) {
    const i64 w = bw + 1;
    const int lane = threadIdx.x;
    for (i64 i = 1; i < n; ++i) {
        double s = 0.0;
        for (i64 k = max(i64(0), i - bw) + lane; k < i; k += 32) s += band[k * w + (i - k)] * f[k];
        s = warp_sum(s);
        if (lane == 0) f[i] -= s;
        __syncwarp();
    }
    for (i64 i = lane; i < n; i += 32) f[i] /= band[i * w];
    __syncwarp();
    for (i64 i = n - 2; i >= 0; --i) {
        double s = 0.0;
        for (i64 j = i + 1 + lane; j <= min(n - 1, i + bw); j += 32) s += band[i * w + (j - i)] * f[j];
        s = warp_sum(s);
        if (lane == 0) f[i] -= s;
        __syncwarp();
    }
}

// heat_capacity_assembler_1d::integrate: c rho sum_q w_q N_i N_j |J| per
// (element, i, j), routed as the conductivity (bound entries dropped)
__global__ void k_capacity_1d(Problem1d P, Line L, double factor, double* __restrict__ band) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < P.E * L.nen * L.nen; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / (L.nen * L.nen);
        const int i = int(t / L.nen % L.nen), j = int(t % L.nen);
        double integral = 0.0;
        for (int q = 0; q < L.nq; ++q) integral += L.w[q] * L.qN[i * L.nq + q] * L.qN[j * L.nq + q];
        band_add(P, band, nullptr, nullptr, e * P.order + i, e * P.order + j, factor * (integral * P.jac));
    }
}

// A = dt K + C over the band, unit diagonal at first-kind ends (C too), bound
// vectors x dt; a convection end adds dt h to its diagonal (K gets h before the
// time step factor: convection_condition_1d.hpp:10-14,
// nonstationary_heat_equation_solver_1d.hpp:167-178).  The ends' diagonals are
// set by the thread of their band element.
__global__ void k_combine_1d(Problem1d P, double dt, double* __restrict__ a, double* __restrict__ c,
                             double* __restrict__ bound0, double* __restrict__ boundN) {
    const i64 w = P.bw + 1, last = P.n - 1;
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < P.n * w; t += i64(gridDim.x) * blockDim.x) {
        double v = dt * a[t] + c[t];
        if (t == 0) {
            if (P.fk0) { v = 1.0; c[0] = 1.0; }
            else if (P.cv0) v += dt * P.h0;
        }
        if (t == last * w) {
            if (P.fk1) { v = 1.0; c[t] = 1.0; }
            else if (P.cv1) v += dt * P.h1;
        }
        a[t] = v;
        if (t < P.n) { bound0[t] *= dt; boundN[t] *= dt; }
    }
}

// f = second-kind ends + source integral (before the time step factor)
__global__ void k_step_loads_1d(Problem1d P, Line L, double q_left, double q_right, bool sin_source,
                                double* __restrict__ f) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < P.E * L.nen; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / L.nen;
        const int i = int(t % L.nen);
        if (!sin_source) continue;
        double integral = 0.0;
        for (int q = 0; q < L.nq; ++q)
            integral += L.w[q] * L.qN[i * L.nq + q] * sin(std::numbers::pi * (P.h * double(e) + (L.x[q] - (-1.0)) * P.jac));
        atomicAdd(f + e * P.order + i, integral * P.jac);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // a convection end's value is its ambient temperature
        if (!P.fk0) atomicAdd(f, P.cv0 ? P.h0 * q_left : q_left);
        if (!P.fk1) atomicAdd(f + P.n - 1, P.cv1 ? P.h1 * q_right : q_right);
    }
}

// f = dt f + C T_prev (symmetric band product), then the first kind of each
// temperature end: f -= bound T_end, f[end] = T_end (boundary_condition_first_kind_1d.hpp)
__global__ void k_step_rhs_1d(Problem1d P, double dt, const double* __restrict__ c, const double* __restrict__ t_prev,
                              const double* __restrict__ bound0, const double* __restrict__ boundN, double t_left,
                              double t_right, double* __restrict__ f) {
    const i64 w = P.bw + 1, last = P.n - 1;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < P.n; i += i64(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (i64 j = max(i64(0), i - P.bw); j < i; ++j) s += c[j * w + (i - j)] * t_prev[j];
        for (i64 j = i; j <= min(last, i + P.bw); ++j) s += c[i * w + (j - i)] * t_prev[j];
        double v = dt * f[i] + s;
        if (P.fk0) v -= bound0[i] * t_left;
        if (P.fk1) v -= boundN[i] * t_right;
        if (P.fk0 && i == 0) v = t_left;
        if (P.fk1 && i == last) v = t_right;
        f[i] = v;
    }
}

// One CTA: band LDL^T and both triangular solves (the stationary solve).
__global__ void __launch_bounds__(1024) k_band_ldlt_solve(i64 n, i64 bw, double* __restrict__ band, double* __restrict__ f,
                                                          int* __restrict__ failed) {
    const i64 w = bw + 1;
    if (!band_ldlt(n, bw, band, failed)) return;
    // U^T D U x = f with unit upper U: forward U^T y = f
    for (i64 i = 1; i < n; ++i) {
        double s = 0.0;
        for (i64 k = max(i64(0), i - bw) + threadIdx.x; k < i; k += blockDim.x) s += band[k * w + (i - k)] * f[k];
        s = warp_sum(s);
        __shared__ double red[32];
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) { double tsum = 0.0; for (int q = 0; q < int(blockDim.x >> 5); ++q) tsum += red[q]; f[i] -= tsum; }
        __syncthreads();
    }
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) f[i] /= band[i * w];
    __syncthreads();
    for (i64 i = n - 2; i >= 0; --i) {
        double s = 0.0;
        for (i64 j = i + 1 + threadIdx.x; j <= min(n - 1, i + bw); j += blockDim.x) s += band[i * w + (j - i)] * f[j];
        s = warp_sum(s);
        __shared__ double red2[32];
        if ((threadIdx.x & 31) == 0) red2[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) { double tsum = 0.0; for (int q = 0; q < int(blockDim.x >> 5); ++q) tsum += red2[q]; f[i] -= tsum; }
        __syncthreads();
    }
}

// mesh, model and band geometry of one segment [0, length]
Problem1d make_problem_1d(i64 elements, int order, double length, double radius, double local_weight, int influence,
                          double conductivity) {
    NL_REQUIRE(influence >= 0 && influence <= 3, NLGPU_ERR_ARG, "unknown 1D influence kind");
    Problem1d P{};
    P.E = elements; P.order = order; P.n = elements * order + 1;
    P.h = length / double(elements);
    P.jac = P.h / (1.0 - (-1.0));
    P.r = radius; P.p1 = local_weight; P.lambda = conductivity; P.kind = influence;
    const bool nonlocal = local_weight < 0.999;
    NL_REQUIRE(!nonlocal || radius > 0.0, NLGPU_ERR_ARG, "nonlocal radius must be positive");
    P.nb = nonlocal ? i64(std::round(radius / P.h)) : 0;
    P.bw = nonlocal ? (P.nb + 1) * order : order;
    if (influence == 0) P.norm = 2.0 / (2 * radius * std::beta(0.5, 2.0));
    else if (influence == 1) P.norm = 1.0 / (2 * radius * std::beta(1.0, 2.0));
    else if (influence == 2) P.norm = 1.0 / (radius * std::sqrt(2 * std::numbers::pi));
    else P.norm = 0.5 / radius;
    NL_REQUIRE(double(P.n) * double(P.bw + 1) * 8.0 < 64e9, NLGPU_ERR_UNSUPPORTED, "1D band too large");
    return P;
}

}  // namespace

// Device state of nonstationary_heat_equation_solver_1d between compute and the steps.
struct OneDimState {
    Problem1d P{};
    Line L{};
    double dt = 0.0;
    dbuf<double> a, c, bound0, boundN, t, f;
};

void nonstationary_1d_compute(Ctx& ctx, i64 elements, int order, double length, double radius, double local_weight,
                              int influence, double conductivity, double capacity, double density, double time_step,
                              int left_kind, int right_kind, const double* initial) {
    NL_REQUIRE(elements > 0 && (order == 1 || order == 2) && length > 0.0 && time_step > 0.0, NLGPU_ERR_ARG,
               "invalid 1D mesh or time step");
    for (const int k : {left_kind, right_kind})
        NL_REQUIRE(k == NLGPU_BC_TEMPERATURE || k == NLGPU_BC_FLUX || k == NLGPU_BC_CONVECTION, NLGPU_ERR_UNSUPPORTED,
                   "1D ends take a temperature, a flux or a convection");
    auto st = std::make_shared<OneDimState>();
    Problem1d& P = st->P;
    P = make_problem_1d(elements, order, length, radius, local_weight, influence, conductivity);
    P.fk0 = left_kind == NLGPU_BC_TEMPERATURE;
    P.fk1 = right_kind == NLGPU_BC_TEMPERATURE;
    P.cv0 = left_kind == NLGPU_BC_CONVECTION;
    P.cv1 = right_kind == NLGPU_BC_CONVECTION;
    P.h0 = P.cv0 ? ctx.od_heat_transfer[0] : 0.0;
    P.h1 = P.cv1 ? ctx.od_heat_transfer[1] : 0.0;
    st->L = make_line(order);
    st->dt = time_step;
    const size_t n = size_t(P.n), nb = size_t(P.n * (P.bw + 1));
    st->a.resize(nb); st->a.zero(ctx.stream);
    st->c.resize(nb); st->c.zero(ctx.stream);
    st->bound0.resize(n); st->bound0.zero(ctx.stream);
    st->boundN.resize(n); st->boundN.zero(ctx.stream);
    st->t.resize(n);
    st->f.resize(n);
    if (initial) st->t.upload(initial, n, ctx.stream);
    else st->t.zero(ctx.stream);
    dbuf<int> failed;
    failed.resize(1); failed.zero(ctx.stream);
    NL_LAUNCH(k_assemble_1d, grid_for(P.E * (2 * P.nb + 1), 128), 128, 0, ctx.stream, P, st->L, st->a.p, st->bound0.p,
              st->boundN.p);
    NL_LAUNCH(k_capacity_1d, grid_for(P.E * st->L.nen * st->L.nen, 256), 256, 0, ctx.stream, P, st->L,
              capacity * density, st->c.p);
    NL_LAUNCH(k_combine_1d, grid_for(i64(nb), 256), 256, 0, ctx.stream, P, time_step, st->a.p, st->c.p, st->bound0.p,
              st->boundN.p);
    NL_LAUNCH(k_band_ldlt, 1, 1024, 0, ctx.stream, P.n, P.bw, st->a.p, failed.p);
    int hf = 0;
    NL_CUDA(cudaMemcpyAsync(&hf, failed.p, sizeof hf, cudaMemcpyDeviceToHost, ctx.stream));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    NL_REQUIRE(!hf, NLGPU_ERR_NUMERICAL, "zero pivot in the 1D LDL^T factorisation");
    ctx.od = st;
}

void nonstationary_1d_step(Ctx& ctx, double left_value, double right_value, bool sin_source, double* temperature) {
    NL_REQUIRE(ctx.od, NLGPU_ERR_STATE, "call nlgpu_nonstationary_1d_compute first");
    OneDimState& st = *ctx.od;
    const Problem1d& P = st.P;
    const size_t n = size_t(P.n);
    st.f.zero(ctx.stream);
    NL_LAUNCH(k_step_loads_1d, grid_for(P.E * st.L.nen, 256), 256, 0, ctx.stream, P, st.L, left_value, right_value,
              sin_source, st.f.p);
    NL_LAUNCH(k_step_rhs_1d, grid_for(P.n, 256), 256, 0, ctx.stream, P, st.dt, st.c.p, st.t.p, st.bound0.p,
              st.boundN.p, left_value, right_value, st.f.p);
    NL_LAUNCH(k_band_solve_warp, 1, 32, 0, ctx.stream, P.n, P.bw, st.a.p, st.f.p);
    std::swap(st.t, st.f);
    if (temperature) st.t.download(temperature, n, ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
}

void nonstationary_1d_temperature(Ctx& ctx, double* temperature) {
    NL_REQUIRE(ctx.od, NLGPU_ERR_STATE, "call nlgpu_nonstationary_1d_compute first");
    ctx.od->t.download(temperature, size_t(ctx.od->P.n), ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
}

i64 nonstationary_1d_nodes(const Ctx& ctx) { return ctx.od ? ctx.od->P.n : 0; }

void stationary_1d(Ctx& ctx, i64 elements, int order, double length, double radius, double local_weight, int influence,
                   double conductivity, double t_left, double q_right, bool sin_source, double* temperature) {
    const Line L = make_line(order);
    Problem1d P = make_problem_1d(elements, order, length, radius, local_weight, influence, conductivity);
    P.fk0 = 1; P.fk1 = 0;   // temperature on the left, flux on the right
    dbuf<double> band, bound0, f;
    dbuf<int> failed;
    band.resize(size_t(P.n * (P.bw + 1))); band.zero(ctx.stream);
    bound0.resize(size_t(P.n)); bound0.zero(ctx.stream);
    f.resize(size_t(P.n)); f.zero(ctx.stream);
    failed.resize(1); failed.zero(ctx.stream);
    NL_LAUNCH(k_assemble_1d, grid_for(P.E * (2 * P.nb + 1), 128), 128, 0, ctx.stream, P, L, band.p, bound0.p,
              static_cast<double*>(nullptr));
    NL_LAUNCH(k_rhs_1d, grid_for(P.E * L.nen, 256), 256, 0, ctx.stream, P, L, q_right, sin_source, f.p);
    NL_LAUNCH(k_first_kind_1d, grid_for(P.n, 256), 256, 0, ctx.stream, P.n, bound0.p, t_left, f.p, band.p);
    NL_LAUNCH(k_band_ldlt_solve, 1, 1024, 0, ctx.stream, P.n, P.bw, band.p, f.p, failed.p);
    int hf = 0;
    NL_CUDA(cudaMemcpyAsync(&hf, failed.p, sizeof hf, cudaMemcpyDeviceToHost, ctx.stream));
    f.download(temperature, size_t(P.n), ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    NL_REQUIRE(!hf, NLGPU_ERR_NUMERICAL, "zero pivot in the 1D LDL^T factorisation");
}

}  // namespace nlgpu
