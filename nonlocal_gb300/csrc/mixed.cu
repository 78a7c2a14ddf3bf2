// Mixed-precision solve: flexible CG in FP32 with FP64 reliable updates.
//
// The plain path runs slae::conjugate_gradient (conjugate_gradient.hpp:48-79)
// in FP64.  This form keeps FP64 only where accuracy is decided -- the
// residual b - A x (FP64 matrix, FP64 SpMV), the solution, every global dot
// product and norm (FP64 partial sums), and the IC(0) pivots (the factor is
// computed in FP64) -- and runs the iteration itself in FP32:
//
//   r = b - A x (FP64); r32 = r / s0; d32 = 0; p_0 = z = P(r32)
//   repeat k   (FP32 vectors, FP32 matrix copy, FP32 ILLT sweeps)
//     q_k = A32 p_k;  alpha = p_k.r / p_k.q_k;  d += alpha p_k;  r32 -= alpha q_k
//     z = P(r32);  p_k+1 = z - sum_i (z.q_i / p_i.q_i) p_i   (last MX_M directions)
//     when |r32| has dropped by update_factor since the last update (or after
//     MX_UPDATE_MAX iterations):
//       x += s0 d (FP64), d = 0;  r = b - A x (FP64);  stop when |r| <= tol |b|;
//       r32 = r / s0 replaces the recurrence residual; the directions are kept
//
// Flexible CG with a few stored directions (Notay's FCG(m)) stays correct when
// the preconditioner is not exactly symmetric or not linear (FP32 rounding in
// the sweeps, the learned correction added to the ILLT output).  The reliable
// updates keep the directions, so no Krylov restart is paid per update.  The
// FP32 SpMV runs in difference form against the FP64 row sums (see k_spmv32)
// and moves 8 bytes per entry instead of 12.  Scalars stay on the device
// (block partials re-summed by each consuming block); the host reads the done
// flag once per MX_ITERS iterations.
#include "common.cuh"

#include <cmath>

namespace nlgpu {

namespace {

constexpr int MX_THREADS = 256;
constexpr int MX_ITERS = 16;
constexpr int MX_M = 4;   // directions kept for the A-orthogonalisation (flexible CG truncation)
constexpr i64 MX_UPDATE_MAX = 64;   // iterations between reliable updates at most
// partial slots: P_RR, P_RZ_A, P_RZ_B as in the FP64 solver (the sweeps' early
// exit reads the residual there), then p_i.q_i and z.q_i of the stored directions
enum { M_PQ = P_COUNT, M_ZQ = P_COUNT + MX_M, M_SLOTS = P_COUNT + 2 * MX_M };
// scalar slots after the solver's (S_BB .. S_RR_FINAL): alpha and the betas
enum { S_ALPHA = 8, S_BETA = 9, S_MIXED_COUNT = 9 + MX_M };

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

// q = A32 p (FP32 values, FP32 accumulation), warp per padded full row, in
// difference form  y_i = sum_j a_ij (x_j - x_i) + s_i x_i  with s_i the row sum
// of the FP64 matrix: the rows of the conductivity matrix sum to (nearly) zero,
// so for smooth x the plain FP32 sum would cancel to a result far below the
// rounding error of its terms, while here each FP32 entry multiplies a small
// difference.  Partial of p.q in FP64.
__global__ void __launch_bounds__(MX_THREADS) k_spmv32(i64 n, const i64* __restrict__ rp, const int4* __restrict__ col4,
                                                       const float4* __restrict__ val4,
                                                       const float* __restrict__ rowsum, const float* __restrict__ x,
                                                       float* __restrict__ y, double* __restrict__ dot_partial,
                                                       const double* __restrict__ flags, i64 ring) {
    __shared__ double sh[40];
    if (flags && flags[S_DONE] != 0.0) return;
    if (ring) {   // direction slot of the current iteration in the rings of x, y and the partials
        const i64 slot = i64(flags[S_ITERS]) % MX_M;
        x += slot * ring; y += slot * ring; dot_partial += slot * RED_BLOCKS;
    }
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    double dot = 0.0;
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        const i64 b4 = rp[r] >> 2, e4 = rp[r + 1] >> 2;
        const float xr = x[r];
        float s = 0.0f;
        for (i64 k = b4 + lane; k < e4; k += 32) {
            const int4 c = __ldg(col4 + k);
            const float4 v = __ldg(val4 + k);
            s += v.x * (x[c.x] - xr) + v.y * (x[c.y] - xr) + v.z * (x[c.z] - xr) + v.w * (x[c.w] - xr);
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            s += rowsum[r] * xr;
            y[r] = s;
            dot += double(s) * double(xr);
        }
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

__global__ void k_rowsum(i64 n, const i64* __restrict__ rp, const double* __restrict__ val, float* __restrict__ out) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (i64 k = rp[r]; k < rp[r + 1]; ++k) s += val[k];
        out[r] = float(s);
    }
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

// x += s d32 in FP64 (s^2 read from the device), d32 = 0
__global__ void k_refine(i64 n, double* __restrict__ x, float* __restrict__ d32, const double* __restrict__ rr) {
    const double s = sqrt(*rr);
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        x[i] += s * double(d32[i]);
        d32[i] = 0.0f;
    }
}

__global__ void k_copy32(i64 n, const float* __restrict__ a, float* __restrict__ b, const double* __restrict__ part,
                         const double* __restrict__ flags, double tol2) {
    __shared__ double sh[40];
    if (flags && (flags[S_DONE] != 0.0 || mx_converged(part, flags, tol2, sh))) return;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = a[i];
}

// one block: alpha = p_j.r / p_j.q_j into the scalars
__global__ void __launch_bounds__(MX_THREADS) k_alpha32(const double* __restrict__ part, double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const i64 k = i64(flags[S_ITERS]);
    const int parity = int(k & 1), slot = int(k % MX_M);
    const double pq = mx_partials(part + (M_PQ + slot) * RED_BLOCKS, sh);
    const double pr = mx_partials(part + (parity ? P_RZ_A : P_RZ_B) * RED_BLOCKS, sh);
    if (threadIdx.x == 0) flags[S_ALPHA] = pr / pq;
}

// one block: counts the iteration; the done flag when |r| <= tol |r_update| or
// the iteration cap is reached.  The kernels after it in the iteration read
// the new count (k + 1).
__global__ void __launch_bounds__(MX_THREADS) k_check32(const double* __restrict__ part, double* __restrict__ flags,
                                                        double tol2, double max_iterations) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const bool converged = mx_converged(part, flags, tol2, sh);
    if (threadIdx.x == 0) {
        const double it = flags[S_ITERS] + 1.0;
        flags[S_ITERS] = it;
        if (converged || it >= max_iterations) flags[S_DONE] = 1.0;
    }
}

// directions stored after k iterations
__device__ __forceinline__ int mx_count(const double* flags) {
    return int(min(i64(flags[S_ITERS]), i64(MX_M)));
}

// one block: beta_i = -(z.q_i) / (p_i.q_i) into the scalars
__global__ void __launch_bounds__(MX_THREADS) k_betas32(const double* __restrict__ part, double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const int count = mx_count(flags);
    for (int s = 0; s < count; ++s) {
        const double b = -mx_partials(part + (M_ZQ + s) * RED_BLOCKS, sh) / mx_partials(part + (M_PQ + s) * RED_BLOCKS, sh);
        if (threadIdx.x == 0) flags[S_BETA + s] = b;
    }
}

// d += alpha p_j; r -= alpha q_j (j the current direction slot); partial of r.r
__global__ void __launch_bounds__(MX_THREADS) k_update_dr32(i64 n, float* __restrict__ d, float* __restrict__ r,
                                                            const float* __restrict__ p, const float* __restrict__ q,
                                                            double* __restrict__ part, const double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const i64 slot = i64(flags[S_ITERS]) % MX_M;
    p += slot * n;
    q += slot * n;
    const float alpha = float(flags[S_ALPHA]);
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        d[i] += alpha * p[i];
        const float v = r[i] - alpha * q[i];
        r[i] = v;
        s += double(v) * double(v);
    }
    const double t = mx_block_sum(s, sh);
    if (threadIdx.x == 0) part[P_RR * RED_BLOCKS + blockIdx.x] = t;
}

// partials of z.q_i for the stored directions
__global__ void __launch_bounds__(MX_THREADS) k_dotm32(i64 n, const float* __restrict__ z, const float* __restrict__ qring,
                                                       double* __restrict__ part, const double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const int count = mx_count(flags);
    double zq[MX_M] = {};
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double zi = z[i];
#pragma unroll
        for (int s = 0; s < MX_M; ++s)
            if (s < count) zq[s] += zi * double(qring[i64(s) * n + i]);
    }
#pragma unroll
    for (int s = 0; s < MX_M; ++s) {
        if (s >= count) break;
        const double ts = mx_block_sum(zq[s], sh);
        if (threadIdx.x == 0) part[(M_ZQ + s) * RED_BLOCKS + blockIdx.x] = ts;
    }
}

// p_k = z + sum_i beta_i p_i over the stored directions (A-orthogonal to the
// last MX_M directions), k the iteration count, and the partial of p_k.r (the
// next alpha's numerator, slot by the parity of k - 1)
__global__ void __launch_bounds__(MX_THREADS) k_update_pm32(i64 n, float* __restrict__ pring, const float* __restrict__ z,
                                                            const float* __restrict__ r, double* __restrict__ part,
                                                            const double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const i64 k = i64(flags[S_ITERS]);
    const int count = mx_count(flags), next = int(k % MX_M), parity = int((k - 1) & 1);
    float beta[MX_M];
#pragma unroll
    for (int s = 0; s < MX_M; ++s) beta[s] = s < count ? float(flags[S_BETA + s]) : 0.0f;
    float* pn = pring + i64(next) * n;
    double pr = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        float v = z[i];
#pragma unroll
        for (int s = 0; s < MX_M; ++s)
            if (s < count) v += beta[s] * pring[i64(s) * n + i];
        pn[i] = v;   // may overwrite the oldest direction: element i was read above
        pr += double(v) * double(r[i]);
    }
    const double t = mx_block_sum(pr, sh);
    if (threadIdx.x == 0) part[(parity ? P_RZ_B : P_RZ_A) * RED_BLOCKS + blockIdx.x] = t;
}

__global__ void k_widen(i64 n, const float* __restrict__ a, double* __restrict__ b) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = a[i];
}

void precondition32(Ctx& ctx, IncompleteCholesky* M, const float* r, float* z, const double* part, const double* flags,
                    double tol2, int sweeps) {
    const i64 n = ctx.mx.n;
    if (!M) {
        NL_LAUNCH(k_copy32, RED_BLOCKS, MX_THREADS, 0, ctx.stream, n, r, z, part, flags, tol2);
    } else if (sweeps > 0) {
        jacobi_apply32(ctx, *M, sweeps, r, z, flags);
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
              reinterpret_cast<const float4*>(A.val32.p), A.rowsum32.p, x, y, static_cast<double*>(nullptr),
              static_cast<const double*>(nullptr), i64(0));
}

void ilt_apply32(Ctx& ctx, IncompleteCholesky& ic, const float* r, float* z, int sweeps) {
    ctx.mx.n = ic.n;
    ctx.mx.r64.reserve(size_t(ic.n)); ctx.mx.q64.reserve(size_t(ic.n));
    precondition32(ctx, &ic, r, z, nullptr, nullptr, 0.0, sweeps);
}

void matrix_to_f32(Ctx& ctx, Csr& A) {
    A.val32.resize(size_t(A.nnz));
    A.rowsum32.resize(size_t(A.rows));
    NL_LAUNCH(k_to_f32, grid_for(A.nnz, 256), 256, 0, ctx.stream, A.nnz, A.val.p, A.val32.p);
    NL_LAUNCH(k_rowsum, grid_for(A.rows, 256), 256, 0, ctx.stream, A.rows, A.rowptr.p, A.val.p, A.rowsum32.p);
}

// One flexible CG in FP32 with reliable updates: the FP32 recurrence runs
// until its residual has dropped by `update_factor` since the last update;
// then the FP32 correction d is added to x in FP64, the residual is replaced
// by the true FP64 residual b - A x, and the iteration continues with the
// same search direction (no Krylov restart).  Every vector keeps the scale
// s0 = |r0| of the first residual (FP32 precision is scale-free).  Every
// index an iteration needs (direction slot, partial slot) is derived on the
// device from the iteration count, so all iterations launch the same kernels
// with the same arguments: after the first chunk, a chunk of MX_ITERS
// iterations is captured once per solve and replayed as one CUDA graph (not
// with the learned correction, whose network runs outside graphs).
CgResult mixed_solve(Ctx& ctx, const Csr& A, IncompleteCholesky* M, const double* b, double* x, double tolerance,
                     i64 max_iterations, double update_factor, bool x_is_initial_guess, bool learned, int sweeps) {
    NL_REQUIRE(A.val32.n == size_t(A.nnz), NLGPU_ERR_STATE, "the FP32 copy of the matrix is missing");
    NL_REQUIRE(!learned || (M && ctx.mp.ready && ctx.mp.n == A.rows), NLGPU_ERR_STATE,
               "the learned correction needs ILLT and a prepared network");
    const i64 n = A.rows;
    MixedWork& w = ctx.mx;
    w.n = n;
    w.r64.reserve(size_t(n)); w.q64.reserve(size_t(n));
    w.r.reserve(size_t(n)); w.z.reserve(size_t(n)); w.d.reserve(size_t(n));
    w.p.reserve(size_t(MX_M) * size_t(n)); w.q.reserve(size_t(MX_M) * size_t(n));   // direction rings
    w.partial.reserve(size_t(M_SLOTS) * RED_BLOCKS);
    w.outer.reserve(size_t(2) * RED_BLOCKS + 8);
    w.flags.reserve(S_MIXED_COUNT);
    double* part = w.partial.p;
    double* flags = w.flags.p;
    double* outer_part = w.outer.p;
    double* outer_sc = w.outer.p + 2 * RED_BLOCKS;   // [0] |b|^2, [1] |r|^2, [2] s0^2
    const unsigned G = RED_BLOCKS;
    if (!x_is_initial_guess) NL_CUDA(cudaMemsetAsync(x, 0, size_t(n) * sizeof(double), ctx.stream));
    const double eta2 = update_factor * update_factor;
    CgResult res;
    auto precondition = [&](const double* pt, const double* fl, double t2) {
        precondition32(ctx, M, w.r.p, w.z.p, pt, fl, t2, sweeps);
        if (learned) mpnn_apply(ctx, w.r.p, w.z.p, w.z.p, false);
    };
    // |b|^2 and the first residual
    NL_LAUNCH(k_dot_f64, G, MX_THREADS, 0, ctx.stream, n, b, b, outer_part);
    NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, outer_part, outer_sc);
    auto true_residual = [&](double* hs) {
        spmv_full(ctx, A, x, w.q64.p);
        NL_LAUNCH(k_residual_f64, G, MX_THREADS, 0, ctx.stream, n, b, w.q64.p, w.r64.p, outer_part + RED_BLOCKS);
        NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, outer_part + RED_BLOCKS, outer_sc + 1);
        NL_CUDA(cudaMemcpyAsync(hs, outer_sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
    };
    double hs[2];
    true_residual(hs);
    if (hs[0] == 0.0 || hs[1] <= tolerance * tolerance * hs[0] || !std::isfinite(hs[1])) {
        res.residual = hs[0] > 0.0 ? std::sqrt(hs[1] / hs[0]) : 0.0;
        res.converged = std::isfinite(hs[1]);
        return res;
    }
    NL_CUDA(cudaMemcpyAsync(outer_sc + 2, outer_sc + 1, sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
    // r32 = r / s0, d = 0, p_0 = z = P(r) in ring slot 0, rz -> the slot iteration 0 reads
    NL_LAUNCH(k_scale_to_f32, G, MX_THREADS, 0, ctx.stream, n, w.r64.p, outer_sc + 2, w.r.p, w.d.p);
    NL_CUDA(cudaMemsetAsync(flags, 0, 8 * sizeof(double), ctx.stream));
    NL_LAUNCH(k_dot32, G, MX_THREADS, 0, ctx.stream, n, w.r.p, w.r.p, part + P_RR * RED_BLOCKS);
    NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, part + P_RR * RED_BLOCKS, flags + S_BB);
    precondition(nullptr, nullptr, 0.0);
    NL_CUDA(cudaMemcpyAsync(w.p.p, w.z.p, size_t(n) * sizeof(float), cudaMemcpyDeviceToDevice, ctx.stream));
    NL_LAUNCH(k_dot32, G, MX_THREADS, 0, ctx.stream, n, w.r.p, w.z.p, part + P_RZ_B * RED_BLOCKS);
    const double cap = double(std::min<i64>(max_iterations, i64(1) << 40));
    double last_rr = hs[1];
    i64 k = 0;
    i64 iters_at_update = 0;
    // one iteration k (k read on the device): q_j = A p_j (j = k mod MX_M),
    // alpha, d and r, the count and stop test, z = P(r), the betas, p_k+1
    auto iteration = [&] {
        NL_LAUNCH(k_spmv32, G, MX_THREADS, 0, ctx.stream, n, A.rowptr.p, reinterpret_cast<const int4*>(A.col.p),
                  reinterpret_cast<const float4*>(A.val32.p), A.rowsum32.p, w.p.p, w.q.p, part + M_PQ * RED_BLOCKS,
                  flags, n);
        NL_LAUNCH(k_alpha32, 1, MX_THREADS, 0, ctx.stream, part, flags);
        NL_LAUNCH(k_update_dr32, G, MX_THREADS, 0, ctx.stream, n, w.d.p, w.r.p, w.p.p, w.q.p, part, flags);
        NL_LAUNCH(k_check32, 1, MX_THREADS, 0, ctx.stream, part, flags, eta2, cap);
        precondition(part, flags, eta2);
        NL_LAUNCH(k_dotm32, G, MX_THREADS, 0, ctx.stream, n, w.z.p, w.q.p, part, flags);
        NL_LAUNCH(k_betas32, 1, MX_THREADS, 0, ctx.stream, part, flags);
        NL_LAUNCH(k_update_pm32, G, MX_THREADS, 0, ctx.stream, n, w.p.p, w.z.p, w.r.p, part, flags);
    };
    bool eager_done = false, captured = false;
    auto run_chunk = [&] {
        if (learned || !eager_done) {   // the first chunk also makes every lazy allocation
            for (int it = 0; it < MX_ITERS; ++it) iteration();
            eager_done = true;
            return;
        }
        if (!captured) {
            cudaGraph_t g = nullptr;
            const i64 before = g_launches.load();
            NL_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
            for (int it = 0; it < MX_ITERS; ++it) iteration();
            NL_CUDA(cudaStreamEndCapture(ctx.stream, &g));
            w.chunk_kernels = int(g_launches.load() - before);
            g_launches.fetch_sub(w.chunk_kernels);   // counted when the graph is launched
            cudaError_t e = cudaErrorGraphExecUpdateFailure;
            if (w.chunk) {
                cudaGraphExecUpdateResultInfo info;
                e = cudaGraphExecUpdate(w.chunk, g, &info);
                if (e != cudaSuccess) {
                    (void)cudaGetLastError();
                    cudaGraphExecDestroy(w.chunk);
                    w.chunk = nullptr;
                }
            }
            if (e != cudaSuccess) e = cudaGraphInstantiate(&w.chunk, g, 0);
            cudaGraphDestroy(g);
            NL_CUDA(e);
            captured = true;
        }
        NL_CUDA(cudaGraphLaunch(w.chunk, ctx.stream));
        g_launches.fetch_add(w.chunk_kernels);
    };
    for (;;) {
        bool forced = false;
        for (;;) {
            run_chunk();
            double hf[8];
            NL_CUDA(cudaMemcpyAsync(hf, flags, sizeof hf, cudaMemcpyDeviceToHost, ctx.stream));
            NL_CUDA(cudaStreamSynchronize(ctx.stream));
            res.iterations = i64(hf[S_ITERS]);
            if (hf[S_DONE] != 0.0) break;
            // a recurrence that stalls still gets an update (and the progress check below)
            if (res.iterations - iters_at_update >= MX_UPDATE_MAX) { forced = true; break; }
        }
        k = res.iterations;   // the iterations after the one that stopped were skipped
        iters_at_update = res.iterations;
        // reliable update: x += s0 d (FP64), r = b - A x (FP64)
        NL_LAUNCH(k_refine, G, MX_THREADS, 0, ctx.stream, n, x, w.d.p, outer_sc + 2);
        true_residual(hs);
        ++res.outer_iterations;
        res.residual = std::sqrt(hs[1] / hs[0]);
        if (hs[1] <= tolerance * tolerance * hs[0]) { res.converged = true; break; }
        if (res.iterations >= max_iterations || !std::isfinite(hs[1])) break;
        // the learned correction must buy at least a factor 10 per update interval,
        // or the rest of the solve runs with ILLT alone
        if (learned && hs[1] > 1e-2 * last_rr) { learned = false; res.learned_fallback = true; }
        last_rr = hs[1];
        // r32 = r / s0 replaces the recurrence residual; the stored directions are kept
        NL_LAUNCH(k_scale_to_f32, G, MX_THREADS, 0, ctx.stream, n, w.r64.p, outer_sc + 2, w.r.p, w.d.p);
        NL_CUDA(cudaMemsetAsync(flags + S_DONE, 0, sizeof(double), ctx.stream));
        NL_LAUNCH(k_dot32, G, MX_THREADS, 0, ctx.stream, n, w.r.p, w.r.p, part + P_RR * RED_BLOCKS);
        NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, part + P_RR * RED_BLOCKS, flags + S_BB);
        const int next = int(k % MX_M);
        if (forced) {
            // the last chunk already formed p_k: only its alpha numerator p_k.r changes
            NL_LAUNCH(k_dot32, G, MX_THREADS, 0, ctx.stream, n, w.p.p + i64(next) * n, w.r.p,
                      part + ((k & 1) ? P_RZ_A : P_RZ_B) * RED_BLOCKS);
        } else {
            // the stop skipped p_k: z = P(r), p_k = z - sum_i (z.q_i / p_i.q_i) p_i as at
            // the end of iteration k - 1 (the kernels read k from the count)
            precondition(nullptr, nullptr, 0.0);
            NL_LAUNCH(k_dotm32, G, MX_THREADS, 0, ctx.stream, n, w.z.p, w.q.p, part, flags);
            NL_LAUNCH(k_betas32, 1, MX_THREADS, 0, ctx.stream, part, flags);
            NL_LAUNCH(k_update_pm32, G, MX_THREADS, 0, ctx.stream, n, w.p.p, w.z.p, w.r.p, part, flags);
        }
    }
    return res;
}

}  // namespace nlgpu
