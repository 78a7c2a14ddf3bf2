// Conjugate gradient that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they need a
// solve: code running under an external memory budget or a fixed memory
// pool, a real-time loop that must not touch the allocator, or a caller that
// only holds device buffers handed to it by another framework.  For them this
// entry point runs the identity-preconditioned CG of slae::conjugate_gradient
// (conjugate_gradient.hpp:48-79) on a matrix, right-hand side and solution
// that already live in device memory, with all of its own work vectors and
// reduction partials in one fixed scratch array that is part of the library:
//
//   * the scratch array is a file-scope static __device__ array sized for at
//     most NLGPU_NOALLOC_MAX_ROWS rows (three vectors plus the partial sums,
//     about 1.6 MB); every GPU on which the library is loaded holds it until
//     the process exits;
//   * the host never uses the array's name as an address: on the first call
//     on a device, with that device current, cudaGetSymbolAddress gives the
//     device address, which is kept per device and passed to the kernels;
//     that first call therefore does the set-up and should come before any
//     stream capture;
//   * every call shares the one array and leaves the last call's contents in
//     it; the call clears what must start at zero, and calls that overlap on
//     the GPU (on different streams) race on the array.
// No cudaMalloc, cudaFree or allocating library routine is called.
#include "common.cuh"

#include <mutex>

namespace nlgpu {

namespace {

constexpr i64 NA_MAX_ROWS = NLGPU_NOALLOC_MAX_ROWS;
constexpr int NA_BLOCKS = 152 * 2;
constexpr int NA_THREADS = 256;
constexpr int NA_ITERS = 16;
// layout (doubles): r, p, q [NA_MAX_ROWS each], partials [4][NA_BLOCKS], scalars [8]
constexpr i64 NA_PARTIALS = 3 * NA_MAX_ROWS;
constexpr i64 NA_SCALARS = NA_PARTIALS + 4 * NA_BLOCKS;
constexpr i64 NA_DOUBLES = NA_SCALARS + 8;
// partial slots; r.r alternates between RR0 and RR1 by iteration parity so that
// no kernel overwrites partials that its own blocks still read
enum { NA_PQ = 0, NA_RR0 = 1, NA_RR1 = 2, NA_BB = 3 };
enum { NA_DONE = 0, NA_ITS = 1, NA_BB_S = 2, NA_RR_S = 3 };       // scalar slots

static __device__ __align__(256) double g_noalloc_scratch[NA_DOUBLES];

__device__ __forceinline__ double block_total(double v, double* sh) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += sh[w];
    __syncthreads();
    return s;
}

__device__ __forceinline__ double partial_sum(const double* part, double* sh) {
    double v = 0.0;
    for (int k = threadIdx.x; k < NA_BLOCKS; k += blockDim.x) v += part[k];
    v = block_total(v, sh);
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    const double s = sh[32];
    __syncthreads();
    return s;
}

// y = A x, warp per row, plain CSR; optional partial of dot(x, y)
__global__ void __launch_bounds__(NA_THREADS) na_spmv(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                                                       const double* __restrict__ val, const double* __restrict__ x,
                                                       double* __restrict__ y, double* __restrict__ part,
                                                       const double* __restrict__ sc) {
    __shared__ double sh[40];
    if (sc && sc[NA_DONE] != 0.0) return;
    const int lane = threadIdx.x & 31;
    double dot = 0.0;
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += i64(gridDim.x) * (blockDim.x >> 5)) {
        double s = 0.0;
        for (i64 k = rp[r] + lane; k < rp[r + 1]; k += 32) s += val[k] * x[col[k]];
        s = warp_sum(s);
        if (lane == 0) { y[r] = s; dot += s * x[r]; }
    }
    if (part) {
        const double t = block_total(dot, sh);
        if (threadIdx.x == 0) part[blockIdx.x] = t;
    }
}

// r = b - r (r holds A x), p = r, partials of r.r and b.b
__global__ void __launch_bounds__(NA_THREADS) na_start(i64 n, const double* __restrict__ b, double* __restrict__ r,
                                                        double* __restrict__ p, double* __restrict__ part) {
    __shared__ double sh[40];
    double rr = 0.0, bb = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double v = b[i] - r[i];
        r[i] = v; p[i] = v;
        rr += v * v; bb += b[i] * b[i];
    }
    const double t1 = block_total(rr, sh), t2 = block_total(bb, sh);
    if (threadIdx.x == 0) { part[NA_RR0 * NA_BLOCKS + blockIdx.x] = t1; part[NA_BB * NA_BLOCKS + blockIdx.x] = t2; }
}

__global__ void __launch_bounds__(NA_THREADS) na_scalars(const double* __restrict__ part, double* __restrict__ sc) {
    __shared__ double sh[40];
    const double rr = partial_sum(part + NA_RR0 * NA_BLOCKS, sh), bb = partial_sum(part + NA_BB * NA_BLOCKS, sh);
    if (threadIdx.x == 0) { sc[NA_BB_S] = bb; sc[NA_RR_S] = rr; }
}

// alpha = rr / pq; x += alpha p; r -= alpha q; the new r.r partials go to the
// other parity's buffer (read by na_update_p and the next iteration)
__global__ void __launch_bounds__(NA_THREADS) na_update_xr(i64 n, double* __restrict__ x, double* __restrict__ r,
                                                            const double* __restrict__ p, const double* __restrict__ q,
                                                            double* __restrict__ part, double* __restrict__ sc,
                                                            int parity) {
    __shared__ double sh[40];
    if (sc[NA_DONE] != 0.0) return;
    const double pq = partial_sum(part + NA_PQ * NA_BLOCKS, sh);
    const double rr = partial_sum(part + (parity ? NA_RR1 : NA_RR0) * NA_BLOCKS, sh);
    const double alpha = rr / pq;
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        x[i] += alpha * p[i];
        const double v = r[i] - alpha * q[i];
        r[i] = v;
        s += v * v;
    }
    const double t = block_total(s, sh);
    if (threadIdx.x == 0) part[(parity ? NA_RR0 : NA_RR1) * NA_BLOCKS + blockIdx.x] = t;
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[NA_ITS] += 1.0;
}

// beta = rr_new / rr_old; p = r + beta p; done when |r| <= tol |b| or the iteration cap is reached
__global__ void __launch_bounds__(NA_THREADS) na_update_p(i64 n, double* __restrict__ p, const double* __restrict__ r,
                                                           const double* __restrict__ part, double* __restrict__ sc,
                                                           double tol2, double max_iterations, int parity) {
    __shared__ double sh[40];
    if (sc[NA_DONE] != 0.0) return;
    const double rr_new = partial_sum(part + (parity ? NA_RR0 : NA_RR1) * NA_BLOCKS, sh);
    const double rr_old = partial_sum(part + (parity ? NA_RR1 : NA_RR0) * NA_BLOCKS, sh);
    // written so that a NaN (breakdown) also stops
    const bool stop = !(rr_new > tol2 * sc[NA_BB_S]) || sc[NA_ITS] >= max_iterations;
    if (!stop) {
        const double beta = rr_new / rr_old;
        for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
            p[i] = r[i] + beta * p[i];
    } else if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc[NA_DONE] = 1.0;
        sc[NA_RR_S] = rr_new;
    }
}

// partial of |b - q|^2 (q holds A x) into the PQ slot, for the final residual
__global__ void __launch_bounds__(NA_THREADS) na_true_residual(i64 n, const double* __restrict__ b,
                                                                const double* __restrict__ q, double* __restrict__ part) {
    __shared__ double sh[40];
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double v = b[i] - q[i];
        s += v * v;
    }
    const double t = block_total(s, sh);
    if (threadIdx.x == 0) part[NA_PQ * NA_BLOCKS + blockIdx.x] = t;
}

__global__ void __launch_bounds__(NA_THREADS) na_final(const double* __restrict__ part, double* __restrict__ sc) {
    __shared__ double sh[40];
    const double rr = partial_sum(part + NA_PQ * NA_BLOCKS, sh);
    if (threadIdx.x == 0) sc[NA_RR_S] = rr;
}

struct DeviceScratch {
    std::mutex lock;
    double* ptr[64] = {};
};
DeviceScratch g_scratch;

double* scratch_for_current_device() {
    int dev = 0;
    NL_CUDA(cudaGetDevice(&dev));
    NL_REQUIRE(dev >= 0 && dev < 64, NLGPU_ERR_UNSUPPORTED, "device index beyond 63");
    std::lock_guard<std::mutex> guard(g_scratch.lock);
    if (!g_scratch.ptr[dev]) {
        void* p = nullptr;
        NL_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch.ptr[dev] = static_cast<double*>(p);
    }
    return g_scratch.ptr[dev];
}

}  // namespace

bool cg_solve_noalloc(cudaStream_t s, i64 n, const i64* rp, const int32_t* col, const double* val, const double* b,
                      double* x, double tolerance, i64 max_iterations, i64* iterations, double* residual) {
    NL_REQUIRE(n > 0 && n <= NA_MAX_ROWS, NLGPU_ERR_ARG, "n must be in 1 .. NLGPU_NOALLOC_MAX_ROWS");
    NL_REQUIRE(rp && col && val && b && x && tolerance > 0.0 && max_iterations > 0, NLGPU_ERR_ARG, "invalid argument");
    double* base = scratch_for_current_device();
    double* r = base;
    double* p = base + NA_MAX_ROWS;
    double* q = base + 2 * NA_MAX_ROWS;
    double* part = base + NA_PARTIALS;
    double* sc = base + NA_SCALARS;
    const double tol2 = tolerance * tolerance;
    const double maxit = double(std::min<i64>(max_iterations, i64(1) << 40));
    NL_CUDA(cudaMemsetAsync(sc, 0, 8 * sizeof(double), s));   // the previous call's state is cleared
    NL_LAUNCH(na_spmv, NA_BLOCKS, NA_THREADS, 0, s, n, rp, col, val, x, r, static_cast<double*>(nullptr),
              static_cast<const double*>(nullptr));
    NL_LAUNCH(na_start, NA_BLOCKS, NA_THREADS, 0, s, n, b, r, p, part);
    NL_LAUNCH(na_scalars, 1, NA_THREADS, 0, s, part, sc);
    double host[8];
    NL_CUDA(cudaMemcpyAsync(host, sc, sizeof host, cudaMemcpyDeviceToHost, s));
    NL_CUDA(cudaStreamSynchronize(s));
    if (host[NA_BB_S] == 0.0) {
        // b = 0: the solution is x = 0 whatever the starting guess held
        NL_CUDA(cudaMemsetAsync(x, 0, size_t(n) * sizeof(double), s));
        NL_CUDA(cudaStreamSynchronize(s));
        *iterations = 0;
        *residual = 0.0;
        return true;
    }
    // a starting guess that already meets the tolerance skips the iteration and
    // goes straight to the recomputed residual below
    if (host[NA_RR_S] > tol2 * host[NA_BB_S]) {
        for (;;) {
            for (int it = 0; it < NA_ITERS; ++it) {   // NA_ITERS is even: every chunk starts at parity 0
                const int parity = it & 1;
                NL_LAUNCH(na_spmv, NA_BLOCKS, NA_THREADS, 0, s, n, rp, col, val, p, q, part + NA_PQ * NA_BLOCKS, sc);
                NL_LAUNCH(na_update_xr, NA_BLOCKS, NA_THREADS, 0, s, n, x, r, p, q, part, sc, parity);
                NL_LAUNCH(na_update_p, NA_BLOCKS, NA_THREADS, 0, s, n, p, r, part, sc, tol2, maxit, parity);
            }
            NL_CUDA(cudaMemcpyAsync(host, sc, sizeof host, cudaMemcpyDeviceToHost, s));
            NL_CUDA(cudaStreamSynchronize(s));
            if (host[NA_DONE] != 0.0) break;
        }
    }
    // |b - A x| / |b| recomputed from the final x
    NL_LAUNCH(na_spmv, NA_BLOCKS, NA_THREADS, 0, s, n, rp, col, val, x, q, static_cast<double*>(nullptr),
              static_cast<const double*>(nullptr));
    NL_LAUNCH(na_true_residual, NA_BLOCKS, NA_THREADS, 0, s, n, b, q, part);
    NL_LAUNCH(na_final, 1, NA_THREADS, 0, s, part, sc);
    NL_CUDA(cudaMemcpyAsync(host, sc, sizeof host, cudaMemcpyDeviceToHost, s));
    NL_CUDA(cudaStreamSynchronize(s));
    *iterations = i64(host[NA_ITS]);
    *residual = std::sqrt(host[NA_RR_S] / host[NA_BB_S]);
    NL_REQUIRE(std::isfinite(*residual), NLGPU_ERR_NUMERICAL, "CG broke down (non-finite residual)");
    // a stop before the iteration cap means the recurrence met the tolerance;
    // at the cap, the residual recomputed from x decides
    return !(host[NA_ITS] >= maxit && host[NA_RR_S] > tol2 * host[NA_BB_S]);
}

}  // namespace nlgpu
