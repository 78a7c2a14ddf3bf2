// BiCGSTAB for the non-symmetric systems (variable conductivity with a
// nonlocal model): stationary_heat_equation_solver_2d.hpp:105-108 solves them
// with Eigen::BiCGSTAB and its default diagonal (Jacobi) preconditioner.
//
// Right-preconditioned BiCGSTAB (van der Vorst 1992), M = diag(A):
//   rho = r0.r;  beta = (rho / rho_old)(alpha / omega);  p = r + beta (p - omega v)
//   y = M^-1 p;  v = A y;  alpha = rho / r0.v;  s = r - alpha v
//   z = M^-1 s;  t = A z;  omega = t.s / t.t;  x += alpha y + omega z;  r = s - omega t
// FP64 throughout, on the solver's full-row matrix.  Scalars live on the
// device in slots alternating with the iteration parity (a kernel never
// overwrites a scalar that other blocks of the same kernel still read); every
// reduction writes one partial per block, re-summed in a fixed order by the
// consumers, so every iteration launches the same kernels with the same
// arguments: BI_ITERS iterations are captured once per solve and replayed as
// one CUDA graph (eight launches an iteration made small systems
// launch-bound).  The host checks the done flag every BI_ITERS iterations and
// restarts from the true residual when the shadow residual becomes orthogonal
// to the residual (rho ~ 0), as the documented Eigen solver does.
#include "common.cuh"

#include <cmath>

namespace nlgpu {

namespace {

constexpr int BI_THREADS = 256;
constexpr int BI_ITERS = 16;
enum { B_RHO = 0, B_R0V = 1, B_TS = 2, B_TT = 3, B_RR = 4, B_SLOTS = 5 };   // partial slots
// scalars: |b|^2, done, iterations, rho[2], alpha[2], omega[2], |r|^2 (host check)
enum { SB_BB = 0, SB_DONE = 1, SB_ITERS = 2, SB_RHO = 3, SB_ALPHA = 5, SB_OMEGA = 7, SB_RR = 9, SB_COUNT = 10 };

__device__ __forceinline__ double bi_block_sum(double v, double* sh) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += sh[w];
    __syncthreads();
    return s;
}

// sum of the partials of a reduction made by a launch of gridDim.x blocks
// (every reducing kernel of one solve runs with the same grid)
__device__ __forceinline__ double bi_partials(const double* part, double* sh, int nb) {
    double v = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) v += part[k];
    v = bi_block_sum(v, sh);
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    const double s = sh[32];
    __syncthreads();
    return s;
}

#define BI_LOOP(i) for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)

// dinv = 1 / diagonal (1 where it is zero)
__global__ void k_bi_jacobi(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                            const double* __restrict__ val, double* __restrict__ dinv) {
    BI_LOOP(r) {
        double d = 0.0;
        for (i64 k = rp[r]; k < rp[r + 1]; ++k)
            if (col[k] == int32_t(r)) d += val[k];
        dinv[r] = d != 0.0 ? 1.0 / d : 1.0;
    }
}

// r = b - q; r0 = r; p = v = 0; partial of r.r
__global__ void __launch_bounds__(BI_THREADS) k_bi_start(i64 n, const double* __restrict__ b, const double* __restrict__ q,
                                                         double* __restrict__ r, double* __restrict__ r0,
                                                         double* __restrict__ p, double* __restrict__ v,
                                                         double* __restrict__ part) {
    __shared__ double sh[40];
    double s = 0.0;
    BI_LOOP(i) {
        const double x = b[i] - q[i];
        r[i] = x; r0[i] = x; p[i] = 0.0; v[i] = 0.0;
        s += x * x;
    }
    const double t = bi_block_sum(s, sh);
    if (threadIdx.x == 0) part[B_RR * RED_BLOCKS + blockIdx.x] = t;
}

// rho = r0.r partials; stops (done flag) when |r| <= tol |b|
__global__ void __launch_bounds__(BI_THREADS) k_bi_rho(i64 n, const double* __restrict__ r0, const double* __restrict__ r,
                                                       double* __restrict__ part, double* __restrict__ sc, double tol2,
                                                       double max_iterations) {
    __shared__ double sh[40];
    if (sc[SB_DONE] != 0.0) return;
    const double rr = bi_partials(part + B_RR * RED_BLOCKS, sh, gridDim.x);
    if (rr <= tol2 * sc[SB_BB] || sc[SB_ITERS] >= max_iterations || !(rr == rr)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) { sc[SB_DONE] = 1.0; sc[SB_RR] = rr; }
        return;
    }
    double s = 0.0;
    BI_LOOP(i) s += r0[i] * r[i];
    const double t = bi_block_sum(s, sh);
    if (threadIdx.x == 0) part[B_RHO * RED_BLOCKS + blockIdx.x] = t;
}

// beta = (rho / rho_old)(alpha_old / omega_old); p = r + beta (p - omega_old v); y = dinv p
__global__ void __launch_bounds__(BI_THREADS) k_bi_p(i64 n, const double* __restrict__ r, double* __restrict__ p,
                                                     const double* __restrict__ v, const double* __restrict__ dinv,
                                                     double* __restrict__ y, const double* __restrict__ part,
                                                     double* __restrict__ sc, int q) {
    __shared__ double sh[40];
    if (sc[SB_DONE] != 0.0) return;
    const int o = q ^ 1;
    const double rho = bi_partials(part + B_RHO * RED_BLOCKS, sh, gridDim.x);
    const double beta = (rho / sc[SB_RHO + o]) * (sc[SB_ALPHA + o] / sc[SB_OMEGA + o]);
    const double w = sc[SB_OMEGA + o];
    BI_LOOP(i) {
        const double pi = r[i] + beta * (p[i] - w * v[i]);
        p[i] = pi;
        y[i] = dinv[i] * pi;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[SB_RHO + q] = rho;
}

// partials of a.b (skipped once done)
__global__ void __launch_bounds__(BI_THREADS) k_bi_dot(i64 n, const double* __restrict__ a, const double* __restrict__ b,
                                                       double* __restrict__ part, const double* __restrict__ sc) {
    __shared__ double sh[40];
    if (sc[SB_DONE] != 0.0) return;
    double s = 0.0;
    BI_LOOP(i) s += a[i] * b[i];
    const double t = bi_block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// alpha = rho / r0.v; s = r - alpha v; z = dinv s
__global__ void __launch_bounds__(BI_THREADS) k_bi_s(i64 n, const double* __restrict__ r, const double* __restrict__ v,
                                                     const double* __restrict__ dinv, double* __restrict__ s,
                                                     double* __restrict__ z, const double* __restrict__ part,
                                                     double* __restrict__ sc, int q) {
    __shared__ double sh[40];
    if (sc[SB_DONE] != 0.0) return;
    const double alpha = sc[SB_RHO + q] / bi_partials(part + B_R0V * RED_BLOCKS, sh, gridDim.x);
    BI_LOOP(i) {
        const double si = r[i] - alpha * v[i];
        s[i] = si;
        z[i] = dinv[i] * si;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[SB_ALPHA + q] = alpha;
}

// partials of t.s and t.t
__global__ void __launch_bounds__(BI_THREADS) k_bi_ts(i64 n, const double* __restrict__ t, const double* __restrict__ s,
                                                      double* __restrict__ part, const double* __restrict__ sc) {
    __shared__ double sh[40];
    if (sc[SB_DONE] != 0.0) return;
    double a = 0.0, b = 0.0;
    BI_LOOP(i) { a += t[i] * s[i]; b += t[i] * t[i]; }
    const double ta = bi_block_sum(a, sh), tb = bi_block_sum(b, sh);
    if (threadIdx.x == 0) { part[B_TS * RED_BLOCKS + blockIdx.x] = ta; part[B_TT * RED_BLOCKS + blockIdx.x] = tb; }
}

// omega = t.s / t.t; x += alpha y + omega z; r = s - omega t; partial of r.r
__global__ void __launch_bounds__(BI_THREADS) k_bi_x(i64 n, double* __restrict__ x, const double* __restrict__ y,
                                                     const double* __restrict__ z, const double* __restrict__ s,
                                                     const double* __restrict__ t, double* __restrict__ r,
                                                     double* __restrict__ part, double* __restrict__ sc, int q) {
    __shared__ double sh[40];
    if (sc[SB_DONE] != 0.0) return;
    const double ts = bi_partials(part + B_TS * RED_BLOCKS, sh, gridDim.x);
    const double tt = bi_partials(part + B_TT * RED_BLOCKS, sh, gridDim.x);
    const double omega = tt > 0.0 ? ts / tt : 0.0;
    const double alpha = sc[SB_ALPHA + q];
    double acc = 0.0;
    BI_LOOP(i) {
        x[i] += alpha * y[i] + omega * z[i];
        const double ri = s[i] - omega * t[i];
        r[i] = ri;
        acc += ri * ri;
    }
    const double tr = bi_block_sum(acc, sh);
    if (threadIdx.x == 0) part[B_RR * RED_BLOCKS + blockIdx.x] = tr;
    if (blockIdx.x == 0 && threadIdx.x == 0) { sc[SB_OMEGA + q] = omega; sc[SB_ITERS] += 1.0; }
}

__global__ void __launch_bounds__(BI_THREADS) k_bi_sum(const double* __restrict__ part, int nb, double* __restrict__ dst) {
    __shared__ double sh[40];
    const double s = bi_partials(part, sh, nb);
    if (threadIdx.x == 0) *dst = s;
}

}  // namespace

CgResult bicgstab_solve(Ctx& ctx, const Csr& A, const double* b, double* x, double tolerance, i64 max_iterations) {
    const i64 n = A.rows;
    BicgWork& w = ctx.bi;
    for (auto* v : {&w.r, &w.r0, &w.p, &w.v, &w.s, &w.t, &w.y, &w.z, &w.dinv}) v->reserve(size_t(n));
    w.part.reserve(size_t(B_SLOTS) * RED_BLOCKS);
    w.sc.reserve(SB_COUNT);
    double* part = w.part.p;
    double* sc = w.sc.p;
    // one block per 256 rows up to RED_BLOCKS: small systems leave the GPU to
    // the solves of other contexts on other streams
    const unsigned G = unsigned(std::min<i64>(RED_BLOCKS, std::max<i64>(1, (n + BI_THREADS - 1) / BI_THREADS)));
    NL_LAUNCH(k_bi_jacobi, grid_for(n, 256), 256, 0, ctx.stream, n, A.rowptr.p, A.col.p, A.val.p, w.dinv.p);
    NL_CUDA(cudaMemsetAsync(x, 0, size_t(n) * sizeof(double), ctx.stream));
    NL_CUDA(cudaMemsetAsync(sc, 0, SB_COUNT * sizeof(double), ctx.stream));
    NL_LAUNCH(k_bi_dot, G, BI_THREADS, 0, ctx.stream, n, b, b, part + B_RR * RED_BLOCKS, sc);
    NL_LAUNCH(k_bi_sum, 1, BI_THREADS, 0, ctx.stream, part + B_RR * RED_BLOCKS, int(G), sc + SB_BB);
    const double tol2 = tolerance * tolerance;
    const double cap = double(std::min<i64>(max_iterations, i64(1) << 40));
    CgResult res;
    auto chunk = [&] {
        for (int it = 0; it < BI_ITERS; ++it) {
            const int q = it & 1;
            NL_LAUNCH(k_bi_rho, G, BI_THREADS, 0, ctx.stream, n, w.r0.p, w.r.p, part, sc, tol2, cap);
            NL_LAUNCH(k_bi_p, G, BI_THREADS, 0, ctx.stream, n, w.r.p, w.p.p, w.v.p, w.dinv.p, w.y.p, part, sc, q);
            spmv_full(ctx, A, w.y.p, w.v.p);
            NL_LAUNCH(k_bi_dot, G, BI_THREADS, 0, ctx.stream, n, w.r0.p, w.v.p, part + B_R0V * RED_BLOCKS, sc);
            NL_LAUNCH(k_bi_s, G, BI_THREADS, 0, ctx.stream, n, w.r.p, w.v.p, w.dinv.p, w.s.p, w.z.p, part, sc, q);
            spmv_full(ctx, A, w.z.p, w.t.p);
            NL_LAUNCH(k_bi_ts, G, BI_THREADS, 0, ctx.stream, n, w.t.p, w.s.p, part, sc);
            NL_LAUNCH(k_bi_x, G, BI_THREADS, 0, ctx.stream, n, x, w.y.p, w.z.p, w.s.p, w.t.p, w.r.p, part, sc, q);
        }
    };
    bool eager_done = false, captured = false;
    auto run_chunk = [&] {
        if (!eager_done) {   // the first chunk runs eagerly (the SpMV's lazy set-up happens outside a capture)
            chunk();
            eager_done = true;
            return;
        }
        if (!captured) {
            cudaGraph_t g = nullptr;
            {
                CountCaptured counted;
                NL_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
                chunk();
                NL_CUDA(cudaStreamEndCapture(ctx.stream, &g));
                w.chunk_kernels = int(counted.kernels);   // counted when the graph is launched
            }
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
    for (int restart = 0; restart < 16; ++restart) {
        // r = r0 = b - A x, p = v = 0, rho_old = alpha = omega = 1 (the slots iteration 0 reads)
        spmv_full(ctx, A, x, w.t.p);
        NL_LAUNCH(k_bi_start, G, BI_THREADS, 0, ctx.stream, n, b, w.t.p, w.r.p, w.r0.p, w.p.p, w.v.p, part);
        const double ones[3] = {1.0, 1.0, 1.0};
        NL_CUDA(cudaMemcpyAsync(sc + SB_RHO + 1, &ones[0], sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
        NL_CUDA(cudaMemcpyAsync(sc + SB_ALPHA + 1, &ones[1], sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
        NL_CUDA(cudaMemcpyAsync(sc + SB_OMEGA + 1, &ones[2], sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
        NL_CUDA(cudaMemsetAsync(sc + SB_DONE, 0, sizeof(double), ctx.stream));
        double h[SB_COUNT];
        for (;;) {
            run_chunk();
            NL_CUDA(cudaMemcpyAsync(h, sc, sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
            NL_CUDA(cudaStreamSynchronize(ctx.stream));
            res.iterations = i64(h[SB_ITERS]);
            if (h[SB_DONE] != 0.0) break;
            // shadow residual orthogonal to the residual, or a non-finite scalar: restart
            const double rho = h[SB_RHO + 1], rr_b = h[SB_BB];
            if (!std::isfinite(h[SB_ALPHA]) || !std::isfinite(h[SB_ALPHA + 1]) || !std::isfinite(h[SB_OMEGA + 1]) ||
                std::fabs(rho) < 1e-30 * rr_b)
                break;
        }
        // the true residual decides
        spmv_full(ctx, A, x, w.t.p);
        NL_LAUNCH(k_bi_start, G, BI_THREADS, 0, ctx.stream, n, b, w.t.p, w.s.p, w.z.p, w.y.p, w.y.p, part);
        NL_LAUNCH(k_bi_sum, 1, BI_THREADS, 0, ctx.stream, part + B_RR * RED_BLOCKS, int(G), sc + SB_RR);
        NL_CUDA(cudaMemcpyAsync(h, sc, sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
        res.residual = h[SB_BB] > 0.0 ? std::sqrt(h[SB_RR] / h[SB_BB]) : 0.0;
        res.converged = res.residual <= tolerance;
        if (res.converged || res.iterations >= max_iterations || !std::isfinite(res.residual)) break;
    }
    return res;
}

}  // namespace nlgpu
