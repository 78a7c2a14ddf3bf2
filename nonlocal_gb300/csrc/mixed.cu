// Mixed-precision solve: FP64 iterative refinement around an FP32 inner solve.
//
// The plain path runs slae::conjugate_gradient (conjugate_gradient.hpp:48-79)
// in FP64.  This form keeps FP64 only where accuracy is decided -- the outer
// residual b - A x (FP64 matrix, FP64 SpMV), the solution update, every
// global dot product and norm (FP64 partial sums), and the IC(0) pivots (the
// factor is computed in FP64) -- and runs the inner solve in FP32:
//
//   x = x0;  repeat
//     r = b - A x                                   FP64
//     stop when |r| <= tol |b|
//     r32 = r / |r|                                  scaled into FP32
//     d32 ~ A^-1 r32 by flexible CG in FP32 with the FP32 ILLT sweeps,
//           until |r_inner| <= eta |r32|
//     x += |r| d32                                   FP64
//
// The inner iteration is flexible CG (beta = -(z.q)/(p.q) with q = A p),
// which stays correct when the preconditioner is not exactly symmetric (FP32
// rounding in the sweeps, or a learned correction added to the ILLT output).
// The inner matrix is the FP32 copy of the solver's full-row matrix (values
// rounded once), so each inner SpMV moves 8 bytes per entry instead of 12.
// Scalars stay on the device (block partials re-summed by each consuming
// block); the host reads the done flag once per GRAPH_ITERS iterations.
#include "common.cuh"

#include <cmath>

namespace nlgpu {

namespace {

constexpr int MX_THREADS = 256;
constexpr int MX_ITERS = 16;
// partial slots (P_PQ, P_RR, P_RZ_A, P_RZ_B as in the FP64 solver, so the
// sweeps' early exit reads the inner residual) and one more for z.q
enum { M_ZQ = P_COUNT, M_SLOTS = P_COUNT + 1 };

__device__ __forceinline__ double mx_block_sum(double v, double* sh) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += sh[w];
    __syncthreads();
    return s;
}

__device__ __forceinline__ double mx_partials(const double* part, double* sh) {
    double v = 0.0;
    for (int k = threadIdx.x; k < RED_BLOCKS; k += blockDim.x) v += part[k];
    v = mx_block_sum(v, sh);
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    const double s = sh[32];
    __syncthreads();
    return s;
}

__device__ __forceinline__ bool mx_converged(const double* part, const double* flags, double tol2, double* sh) {
    return mx_partials(part + P_RR * RED_BLOCKS, sh) <= tol2 * flags[S_BB];
}

// q = A32 p (FP32 values, FP32 accumulation), warp per padded full row; partial of p.q in FP64
__global__ void __launch_bounds__(MX_THREADS) k_spmv32(i64 n, const i64* __restrict__ rp, const int4* __restrict__ col4,
                                                       const float4* __restrict__ val4, const float* __restrict__ x,
                                                       float* __restrict__ y, double* __restrict__ dot_partial,
                                                       const double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags && flags[S_DONE] != 0.0) return;
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    double dot = 0.0;
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        const i64 b4 = rp[r] >> 2, e4 = rp[r + 1] >> 2;
        float s = 0.0f;
        for (i64 k = b4 + lane; k < e4; k += 32) {
            const int4 c = __ldg(col4 + k);
            const float4 v = __ldg(val4 + k);
            s += v.x * x[c.x] + v.y * x[c.y] + v.z * x[c.z] + v.w * x[c.w];
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) { y[r] = s; dot += double(s) * double(x[r]); }
    }
    if (dot_partial) {
        const double t = mx_block_sum(dot, sh);
        if (threadIdx.x == 0) dot_partial[blockIdx.x] = t;
    }
}

// FP64 outer kernels: partial of a.b; r = b - q with the partial of r.r
__global__ void __launch_bounds__(MX_THREADS) k_dot_f64(i64 n, const double* __restrict__ a, const double* __restrict__ b,
                                                        double* __restrict__ partial) {
    __shared__ double sh[40];
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) s += a[i] * b[i];
    const double t = mx_block_sum(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void __launch_bounds__(MX_THREADS) k_residual_f64(i64 n, const double* __restrict__ b,
                                                             const double* __restrict__ q, double* __restrict__ r,
                                                             double* __restrict__ partial) {
    __shared__ double sh[40];
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double v = b[i] - q[i];
        r[i] = v;
        s += v * v;
    }
    const double t = mx_block_sum(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void k_to_f32(i64 n, const double* __restrict__ a, float* __restrict__ b) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = float(a[i]);
}

// partial of a.b
__global__ void __launch_bounds__(MX_THREADS) k_dot32(i64 n, const float* __restrict__ a, const float* __restrict__ b,
                                                      double* __restrict__ partial) {
    __shared__ double sh[40];
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        s += double(a[i]) * double(b[i]);
    const double t = mx_block_sum(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void __launch_bounds__(MX_THREADS) k_sum_to(const double* __restrict__ part, double* __restrict__ dst) {
    __shared__ double sh[40];
    const double s = mx_partials(part, sh);
    if (threadIdx.x == 0) *dst = s;
}

// r32 = r * s (s = 1 / |r| read from the device), d32 = 0
__global__ void k_scale_to_f32(i64 n, const double* __restrict__ r, const double* __restrict__ rr,
                               float* __restrict__ r32, float* __restrict__ d32) {
    const double s = *rr > 0.0 ? 1.0 / sqrt(*rr) : 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        r32[i] = float(r[i] * s);
        d32[i] = 0.0f;
    }
}

// x += |r| d32 in FP64
__global__ void k_refine(i64 n, double* __restrict__ x, const float* __restrict__ d32, const double* __restrict__ rr) {
    const double s = sqrt(*rr);
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        x[i] += s * double(d32[i]);
}

__global__ void k_copy32(i64 n, const float* __restrict__ a, float* __restrict__ b, const double* __restrict__ part,
                         const double* __restrict__ flags, double tol2) {
    __shared__ double sh[40];
    if (flags && (flags[S_DONE] != 0.0 || mx_converged(part, flags, tol2, sh))) return;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = a[i];
}

// alpha = rz / pq; d += alpha p; r -= alpha q; partial of r.r; counts the iteration
__global__ void __launch_bounds__(MX_THREADS) k_update_dr32(i64 n, float* __restrict__ d, float* __restrict__ r,
                                                            const float* __restrict__ p, const float* __restrict__ q,
                                                            double* __restrict__ part, int parity,
                                                            double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const double pq = mx_partials(part + P_PQ * RED_BLOCKS, sh);
    const double rz = mx_partials(part + (parity ? P_RZ_A : P_RZ_B) * RED_BLOCKS, sh);
    const float alpha = float(rz / pq);
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        d[i] += alpha * p[i];
        const float v = r[i] - alpha * q[i];
        r[i] = v;
        s += double(v) * double(v);
    }
    const double t = mx_block_sum(s, sh);
    if (threadIdx.x == 0) part[P_RR * RED_BLOCKS + blockIdx.x] = t;
    if (blockIdx.x == 0 && threadIdx.x == 0) flags[S_ITERS] += 1.0;
}

// partials of z.r (the next iteration's rz) and z.q
__global__ void __launch_bounds__(MX_THREADS) k_dot2_32(i64 n, const float* __restrict__ z, const float* __restrict__ r,
                                                        const float* __restrict__ q, double* __restrict__ part, int parity,
                                                        const double* __restrict__ flags, double tol2) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0 || mx_converged(part, flags, tol2, sh)) return;
    double zr = 0.0, zq = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double zi = z[i];
        zr += zi * double(r[i]);
        zq += zi * double(q[i]);
    }
    const double t1 = mx_block_sum(zr, sh);
    const double t2 = mx_block_sum(zq, sh);
    if (threadIdx.x == 0) {
        part[(parity ? P_RZ_B : P_RZ_A) * RED_BLOCKS + blockIdx.x] = t1;
        part[M_ZQ * RED_BLOCKS + blockIdx.x] = t2;
    }
}

// beta = -(z.q) / (p.q); p = z + beta p; raises the done flag
__global__ void __launch_bounds__(MX_THREADS) k_update_p32(i64 n, float* __restrict__ p, const float* __restrict__ z,
                                                           const double* __restrict__ part, double* __restrict__ flags,
                                                           double tol2, double max_iterations) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    if (mx_converged(part, flags, tol2, sh) || flags[S_ITERS] >= max_iterations) {
        __syncthreads();
        if (blockIdx.x == 0 && threadIdx.x == 0) flags[S_DONE] = 1.0;
        return;
    }
    const double zq = mx_partials(part + M_ZQ * RED_BLOCKS, sh);
    const double pq = mx_partials(part + P_PQ * RED_BLOCKS, sh);
    const float beta = float(-zq / pq);
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

__global__ void k_widen(i64 n, const float* __restrict__ a, double* __restrict__ b) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = a[i];
}

void precondition32(Ctx& ctx, IncompleteCholesky* M, const float* r, float* z, const double* part, const double* flags,
                    double tol2) {
    const i64 n = ctx.mx.n;
    if (!M) {
        NL_LAUNCH(k_copy32, RED_BLOCKS, MX_THREADS, 0, ctx.stream, n, r, z, part, flags, tol2);
    } else if (M->fwd_plan.ok && M->bwd_plan.ok && !ctx.force_global_sweeps) {
        sweep_apply32(ctx, *M, r, z, part, flags, tol2);
    } else {
        // no shared-memory sweep plan (a dependency too far back for the ring):
        // the FP64 global-memory sweeps on widened copies
        MixedWork& w = ctx.mx;
        NL_LAUNCH(k_widen, grid_for(n, 256), 256, 0, ctx.stream, n, r, w.r64.p);
        ilt_apply(ctx, *M, w.r64.p, w.q64.p);
        NL_LAUNCH(k_to_f32, grid_for(n, 256), 256, 0, ctx.stream, n, w.q64.p, z);
    }
}

}  // namespace

void spmv32(Ctx& ctx, const Csr& A, const float* x, float* y) {
    NL_LAUNCH(k_spmv32, RED_BLOCKS, MX_THREADS, 0, ctx.stream, A.rows, A.rowptr.p, reinterpret_cast<const int4*>(A.col.p),
              reinterpret_cast<const float4*>(A.val32.p), x, y, static_cast<double*>(nullptr),
              static_cast<const double*>(nullptr));
}

void ilt_apply32(Ctx& ctx, IncompleteCholesky& ic, const float* r, float* z) {
    ctx.mx.n = ic.n;
    ctx.mx.r64.reserve(size_t(ic.n)); ctx.mx.q64.reserve(size_t(ic.n));
    precondition32(ctx, &ic, r, z, nullptr, nullptr, 0.0);
}

void matrix_to_f32(Ctx& ctx, Csr& A) {
    A.val32.resize(size_t(A.nnz));
    NL_LAUNCH(k_to_f32, grid_for(A.nnz, 256), 256, 0, ctx.stream, A.nnz, A.val.p, A.val32.p);
}

CgResult mixed_solve(Ctx& ctx, const Csr& A, IncompleteCholesky* M, const double* b, double* x, double tolerance,
                     i64 max_iterations, double inner_tolerance, bool x_is_initial_guess) {
    NL_REQUIRE(A.val32.n == size_t(A.nnz), NLGPU_ERR_STATE, "the FP32 copy of the matrix is missing");
    const i64 n = A.rows;
    MixedWork& w = ctx.mx;
    w.n = n;
    w.r64.reserve(size_t(n)); w.q64.reserve(size_t(n));
    w.r.reserve(size_t(n)); w.z.reserve(size_t(n)); w.p.reserve(size_t(n)); w.q.reserve(size_t(n)); w.d.reserve(size_t(n));
    w.partial.reserve(size_t(M_SLOTS) * RED_BLOCKS);
    w.outer.reserve(size_t(2) * RED_BLOCKS + 8);
    w.flags.reserve(8);
    double* part = w.partial.p;
    double* flags = w.flags.p;
    double* outer_part = w.outer.p;
    double* outer_sc = w.outer.p + 2 * RED_BLOCKS;   // [0] |b|^2, [1] |r|^2
    const unsigned G = RED_BLOCKS;
    if (!x_is_initial_guess) NL_CUDA(cudaMemsetAsync(x, 0, size_t(n) * sizeof(double), ctx.stream));
    const double eta2 = inner_tolerance * inner_tolerance;
    CgResult res;
    // |b|^2
    NL_LAUNCH(k_dot_f64, G, MX_THREADS, 0, ctx.stream, n, b, b, outer_part);
    NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, outer_part, outer_sc);
    i64 inner_total = 0;
    for (int outer = 0; outer < 64; ++outer) {
        // r = b - A x in FP64
        spmv_full(ctx, A, x, w.q64.p);
        NL_LAUNCH(k_residual_f64, G, MX_THREADS, 0, ctx.stream, n, b, w.q64.p, w.r64.p, outer_part + RED_BLOCKS);
        NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, outer_part + RED_BLOCKS, outer_sc + 1);
        double hs[2];
        NL_CUDA(cudaMemcpyAsync(hs, outer_sc, sizeof hs, cudaMemcpyDeviceToHost, ctx.stream));
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
        res.residual = hs[0] > 0.0 ? std::sqrt(hs[1] / hs[0]) : 0.0;
        res.outer_iterations = outer;
        if (hs[0] == 0.0 || hs[1] <= tolerance * tolerance * hs[0]) { res.converged = true; break; }
        if (inner_total >= max_iterations || !std::isfinite(hs[1])) break;
        // inner flexible CG in FP32 on A d = r / |r|
        NL_LAUNCH(k_scale_to_f32, G, MX_THREADS, 0, ctx.stream, n, w.r64.p, outer_sc + 1, w.r.p, w.d.p);
        NL_CUDA(cudaMemsetAsync(flags, 0, 8 * sizeof(double), ctx.stream));
        NL_LAUNCH(k_dot32, G, MX_THREADS, 0, ctx.stream, n, w.r.p, w.r.p, part + P_RR * RED_BLOCKS);
        NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, part + P_RR * RED_BLOCKS, flags + S_BB);
        precondition32(ctx, M, w.r.p, w.z.p, nullptr, nullptr, 0.0);
        NL_CUDA(cudaMemcpyAsync(w.p.p, w.z.p, size_t(n) * sizeof(float), cudaMemcpyDeviceToDevice, ctx.stream));
        NL_LAUNCH(k_dot32, G, MX_THREADS, 0, ctx.stream, n, w.r.p, w.z.p, part + P_RZ_B * RED_BLOCKS);
        const double cap = double(max_iterations - inner_total);
        for (;;) {
            for (int it = 0; it < MX_ITERS; ++it) {   // even: every chunk starts at parity 0
                const int parity = it & 1;
                NL_LAUNCH(k_spmv32, G, MX_THREADS, 0, ctx.stream, n, A.rowptr.p, reinterpret_cast<const int4*>(A.col.p),
                          reinterpret_cast<const float4*>(A.val32.p), w.p.p, w.q.p, part + P_PQ * RED_BLOCKS, flags);
                NL_LAUNCH(k_update_dr32, G, MX_THREADS, 0, ctx.stream, n, w.d.p, w.r.p, w.p.p, w.q.p, part, parity, flags);
                precondition32(ctx, M, w.r.p, w.z.p, part, flags, eta2);
                NL_LAUNCH(k_dot2_32, G, MX_THREADS, 0, ctx.stream, n, w.z.p, w.r.p, w.q.p, part, parity, flags, eta2);
                NL_LAUNCH(k_update_p32, G, MX_THREADS, 0, ctx.stream, n, w.p.p, w.z.p, part, flags, eta2, cap);
            }
            double hf[8];
            NL_CUDA(cudaMemcpyAsync(hf, flags, sizeof hf, cudaMemcpyDeviceToHost, ctx.stream));
            NL_CUDA(cudaStreamSynchronize(ctx.stream));
            if (hf[S_DONE] != 0.0) { inner_total += i64(hf[S_ITERS]); break; }
        }
        NL_LAUNCH(k_refine, G, MX_THREADS, 0, ctx.stream, n, x, w.d.p, outer_sc + 1);
    }
    res.iterations = inner_total;
    return res;
}

}  // namespace nlgpu
