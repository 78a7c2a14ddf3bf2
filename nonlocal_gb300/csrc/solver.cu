// Conjugate gradient with the ILLT preconditioner.
//
// Reference: slae::conjugate_gradient::solve (conjugate_gradient.hpp:48-79) with
// the symmetric product of independent_symmetric_matrix_vector_product.hpp:55-79,
// and eigen_ILLT_preconditioner = Eigen::IncompleteCholesky<T, Upper,
// NaturalOrdering> (eigen_preconditioner.hpp:57) built from p1*K_local
// (stationary_heat_equation_solver_2d.hpp:91-101).
//
// GB300 form:
//   * SpMV on full-row CSR (both triangles, rows padded to multiples of 4):
//     one warp per row, 16-byte loads of 4 columns and 2x2 values, no atomics;
//   * all CG scalars stay on the device: reductions write one partial per
//     block, and every block of the consuming kernel re-adds the partials in a
//     fixed order (deterministic, no extra launch);
//   * iterations are enqueued in chunks of GRAPH_ITERS iterations; each
//     kernel returns at once after convergence, the host reads the flag once
//     per chunk;
//   * ILLT: Lin-More scaling S = diag(|a_j|_2)^(-1/2) and diagonal shift retry
//     (alpha_S = 1e-3, doubled, at most 10 attempts) around IC(0) on the
//     pattern of the upper local matrix, factored level by level in one CTA;
//     the triangular solves run level by level in one CTA over a per-level
//     column-major (ELL) copy of the factor, so consecutive threads read
//     consecutive entries.  Eigen's factorisation additionally admits fill
//     entries larger than the dropped originals; this one keeps the original
//     pattern (the converged solution is the same to the tolerance).
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace nlgpu {

namespace {

constexpr int RED_THREADS = 256;
constexpr int GRAPH_ITERS = 16;
constexpr int TRI_THREADS = 1024;

__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += sh[w];
    __syncthreads();
    return s;   // valid in thread 0
}

// Sum of RED_BLOCKS partials in a fixed order, computed by every block.
__device__ __forceinline__ double sum_partials(const double* part, double* sh) {
    double v = 0.0;
    for (int k = threadIdx.x; k < RED_BLOCKS; k += blockDim.x) v += part[k];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    const double s = sh[32];
    __syncthreads();
    return s;
}

// y = A x on padded full rows; optional partial of dot(x, y)
__global__ void __launch_bounds__(RED_THREADS) k_spmv(i64 n, const i64* __restrict__ rp, const int4* __restrict__ col4,
                                                      const double2* __restrict__ val2, const double* __restrict__ x,
                                                      double* __restrict__ y, double* __restrict__ dot_partial,
                                                      const double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags && flags[S_DONE] != 0.0) return;
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    double dot = 0.0;
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        const i64 b4 = rp[r] >> 2, e4 = rp[r + 1] >> 2;
        double s = 0.0, s2 = 0.0;
        for (i64 k = b4 + lane; k < e4; k += 32) {
            const int4 c = __ldg(col4 + k);
            const double2 v0 = __ldg(val2 + 2 * k), v1 = __ldg(val2 + 2 * k + 1);
            // two FMA chains: written as one sum of products the group cost a multiply
            // and an add besides its FMAs on the FP64 pipe, which bounds this product
            s = fma(v0.x, x[c.x], s);
            s2 = fma(v0.y, x[c.y], s2);
            s = fma(v1.x, x[c.z], s);
            s2 = fma(v1.y, x[c.w], s2);
        }
        s = warp_sum(s + s2);
        if (lane == 0) { y[r] = s; dot += s * x[r]; }
    }
    if (dot_partial) {
        const double t = block_sum(dot, sh);
        if (threadIdx.x == 0) dot_partial[blockIdx.x] = t;
    }
}

// partial of dot(a, b)
__global__ void __launch_bounds__(RED_THREADS) k_dot(i64 n, const double* __restrict__ a, const double* __restrict__ b,
                                                     double* __restrict__ partial, const double* __restrict__ flags) {
    __shared__ double sh[40];
    if (flags && flags[S_DONE] != 0.0) return;
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) s += a[i] * b[i];
    const double t = block_sum(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// r = b - r (r holds A x0 on entry); partial of dot(r, r)
__global__ void __launch_bounds__(RED_THREADS) k_residual(i64 n, const double* __restrict__ b, double* __restrict__ r,
                                                          double* __restrict__ rr_partial) {
    __shared__ double sh[40];
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double v = b[i] - r[i];
        r[i] = v;
        s += v * v;
    }
    const double t = block_sum(s, sh);
    if (threadIdx.x == 0) rr_partial[blockIdx.x] = t;
}

// alpha = rz / pq; x += alpha p; r -= alpha q; partial of r.r; counts the iteration
__global__ void __launch_bounds__(RED_THREADS) k_update_xr(i64 n, double* __restrict__ x, double* __restrict__ r,
                                                           const double* __restrict__ p, const double* __restrict__ q,
                                                           double* __restrict__ partials, int parity,
                                                           double* __restrict__ flags, i64 max_iterations) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const double pq = sum_partials(partials + P_PQ * RED_BLOCKS, sh);
    const double rz = sum_partials(partials + (parity ? P_RZ_A : P_RZ_B) * RED_BLOCKS, sh);
    const double alpha = rz / pq;
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        x[i] += alpha * p[i];
        const double v = r[i] - alpha * q[i];
        r[i] = v;
        s += v * v;
    }
    const double t = block_sum(s, sh);
    if (threadIdx.x == 0) partials[P_RR * RED_BLOCKS + blockIdx.x] = t;
    if (blockIdx.x == 0 && threadIdx.x == 0) flags[S_ITERS] += 1.0;
    (void)max_iterations;
}

// converged when |r| <= tol |b| (every block decides the same way)
__device__ __forceinline__ bool converged(const double* partials, const double* flags, double tol2, double* sh) {
    const double rr = sum_partials(partials + P_RR * RED_BLOCKS, sh);
    return rr <= tol2 * flags[S_BB];
}

// z = r (identity preconditioner), skipped after convergence
__global__ void __launch_bounds__(RED_THREADS) k_copy_if_running(i64 n, const double* __restrict__ r, double* __restrict__ z,
                                                                 const double* __restrict__ partials,
                                                                 const double* __restrict__ flags, double tol2) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0 || converged(partials, flags, tol2, sh)) return;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) z[i] = r[i];
}

// beta = rz_new / rz_old; p = z + beta p; raises the done flag on convergence
__global__ void __launch_bounds__(RED_THREADS) k_update_p(i64 n, double* __restrict__ p, const double* __restrict__ z,
                                                          double* __restrict__ partials, int parity,
                                                          double* __restrict__ flags, double tol2, i64 max_iterations) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    if (converged(partials, flags, tol2, sh) || flags[S_ITERS] >= double(max_iterations)) {
        __syncthreads();
        if (blockIdx.x == 0 && threadIdx.x == 0) flags[S_DONE] = 1.0;
        return;
    }
    const double rz_new = sum_partials(partials + (parity ? P_RZ_B : P_RZ_A) * RED_BLOCKS, sh);
    const double rz_old = sum_partials(partials + (parity ? P_RZ_A : P_RZ_B) * RED_BLOCKS, sh);
    const double beta = rz_new / rz_old;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

__global__ void k_copy(i64 n, const double* __restrict__ a, double* __restrict__ b) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = a[i];
}

// ---------------------------------------------------------------- IC(0)
// column 2-norms of the full symmetric matrix given by its upper part
__global__ void k_colnorm2(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                           const double* __restrict__ val, double* __restrict__ norm2) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x)
        for (i64 k = rp[r]; k < rp[r + 1]; ++k) {
            const double v2 = val[k] * val[k];
            atomicAdd(norm2 + r, v2);
            if (col[k] != int32_t(r)) atomicAdd(norm2 + col[k], v2);
        }
}

__global__ void k_scale(i64 n, double* __restrict__ s) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double root = sqrt(sqrt(s[i]));
        s[i] = root > 2.2250738585072014e-308 ? 1.0 / root : 1.0;
    }
}

// scaled copy of the matrix and the minimum scaled diagonal (ordered bits)
__global__ void k_scaled(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col, const double* __restrict__ val,
                         const double* __restrict__ s, double* __restrict__ out, unsigned long long* __restrict__ mindiag) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x)
        for (i64 k = rp[r]; k < rp[r + 1]; ++k) {
            const double v = val[k] * s[col[k]] * s[r];
            out[k] = v;
            if (col[k] == int32_t(r)) {
                const unsigned long long b = __double_as_longlong(v);
                atomicMin(mindiag, (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull));
            }
        }
}

// Up-looking IC(0): U has the pattern of the upper matrix; row i subtracts
// u_ki * row k for every k < i with u_ki != 0 (L row i, with its U position in
// l_to_u), then divides by the root of its pivot.
//
// Synchronisation-free schedule (after Liu, Li, Hou and Vinter, "A
// synchronization-free algorithm for parallel sparse triangular solves",
// Euro-Par 2016): one launch for the whole factorisation; each warp takes the
// next row from a ticket counter over the rows in dependency-level order,
// loads the row's structure, waits until every row k of L row i has
// published its U row (done[k], stored with release semantics after the
// row's values; the wait is bounded by %globaltimer and reports a timeout),
// reads those rows through L2, computes and publishes its own.  A row's
// dependencies come earlier in the level order, so their tickets went to
// warps that are already running: the oldest unfinished row can always
// proceed, and rows of consecutive levels overlap instead of waiting for a
// launch boundary.
//
// Inside a row: lane y owns entry y of row i (rows of up to 32 entries;
// longer rows run the sequential merge on lane 0).  For up to IC_MAXS rows k
// of L row i at a time, the lanes spread over the entries of those rows'
// segments (columns >= i), each finds its column among row i's (binary search
// in shared memory) and stores u_ki u_kj in a table; lane y then subtracts
// the table's column y in the order of k, as the sequential form does
// (product and subtraction rounded separately), so the result does not depend
// on the schedule.
//
// SWEEP: one sweep of the fixed-point form of the same equations (Chow and
// Patel, "Fine-grained parallel incomplete LU factorization", SISC 2015): every
// row at once, reading the other rows' values of the previous sweep (uin) and
// writing its own (u), with no order and no waits.  Started from the scaled
// matrix's rows divided by the root of their diagonal, a few sweeps give a
// factor that serves the FP32 Jacobi-sweep application as well as the exact
// one, without the exact form's dependency chain (2 401 levels on the
// 300x300 serendipity mesh, at a few microseconds each).
constexpr int IC_WARPS = 8;
constexpr int IC_SWEEPS = 3;
constexpr int IC_MAXS = 16;
constexpr unsigned long long IC_WAIT_LIMIT_NS = 2000000000ull;

__device__ __forceinline__ unsigned long long ic_globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// rows of other warps are read through L2 (__ldcg): they were written after
// this SM may have cached the lines
__device__ void ic0_row_sequential(int32_t i, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                                   const double* __restrict__ a, double shift, const i64* __restrict__ lrp,
                                   const int32_t* __restrict__ lcol, const i64* __restrict__ l_to_u,
                                   const double* uin, double* u, int* __restrict__ failed) {
    const i64 b = rp[i], e = rp[i + 1];
    for (i64 s = b; s < e; ++s) u[s] = a[s];
    u[b] += shift;
    for (i64 s = lrp[i]; s < lrp[i + 1] - 1; ++s) {
        const int32_t k = lcol[s];
        const i64 pk = l_to_u[s];
        const double uki = __ldcg(uin + pk);
        i64 x = pk, y = b;
        const i64 ke = rp[k + 1];
        while (x < ke && y < e) {
            const int32_t cx = col[x], cy = col[y];
            if (cx < cy) ++x;
            else if (cx > cy) ++y;
            else { u[y] = __dsub_rn(u[y], __dmul_rn(uki, __ldcg(uin + x))); ++x; ++y; }
        }
    }
    const double d = u[b];
    if (!(d > 0.0)) { atomicExch(failed, 1); return; }
    const double rd = sqrt(d);
    u[b] = rd;
    for (i64 s = b + 1; s < e; ++s) u[s] /= rd;
}

template<bool SWEEP>
__global__ void __launch_bounds__(IC_WARPS * 32) k_ic0_rows(i64 n, const int32_t* __restrict__ order,
                                                            const i64* __restrict__ rp, const int32_t* __restrict__ col,
                                                            const double* __restrict__ a, double shift,
                                                            const i64* __restrict__ lrp,
                                                            const int32_t* __restrict__ lcol,
                                                            const i64* __restrict__ l_to_u, const double* uin,
                                                            double* u, int* __restrict__ ticket, int* done,
                                                            int* __restrict__ failed, int* __restrict__ timed_out) {
    __shared__ double table[IC_WARPS][IC_MAXS][32];
    __shared__ int32_t rowcol[IC_WARPS][32];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(ticket, 1);
        t = __shfl_sync(full, t, 0);
        if (t >= n) break;
        const int32_t i = SWEEP ? int32_t(t) : order[t];
        const i64 b = rp[i], e = rp[i + 1];
        const int m = int(e - b);
        const i64 lb = lrp[i], le = lrp[i + 1] - 1;   // L row i without its diagonal (its last entry)
        const bool own = lane < m;
        double acc = 0.0;
        if (m <= 32) {
            rowcol[wb][lane] = own ? col[b + lane] : 0x7fffffff;
            acc = own ? a[b + lane] : 0.0;
            if (lane == 0) acc += shift;
        }
        // the first chunk's structure does not depend on other rows: load it
        // before waiting, so only the values are read after the wait
        const int ns_first = le - lb < IC_MAXS ? int(le - lb) : IC_MAXS;
        i64 pk_first = 0;
        int len_first = 0;
        if (m <= 32 && lane < ns_first) {
            pk_first = l_to_u[lb + lane];
            len_first = int(rp[lcol[lb + lane] + 1] - pk_first);
        }
        if constexpr (!SWEEP) {   // wait for the rows this row reads
            bool gave_up = false;
            for (i64 s = lb + lane; s < le && !gave_up; s += 32) {
                const int* flag = done + lcol[s];
                if (ld_acquire_gpu(flag) == 0) {
                    const unsigned long long t0 = ic_globaltimer();
                    while (ld_acquire_gpu(flag) == 0) {
                        if (ic_globaltimer() - t0 > IC_WAIT_LIMIT_NS) { gave_up = true; break; }
                        __nanosleep(32);
                    }
                }
            }
            if (__any_sync(full, gave_up) && lane == 0) atomicExch(timed_out, 1);
        }
        __syncwarp();
        if (m > 32) {
            if (lane == 0) ic0_row_sequential(i, rp, col, a, shift, lrp, lcol, l_to_u, uin, u, failed);
        } else {
            for (i64 s0 = lb; s0 < le; s0 += IC_MAXS) {
                const int ns = le - s0 < IC_MAXS ? int(le - s0) : IC_MAXS;
                const bool first_chunk = s0 == lb;
                i64 pk = first_chunk ? pk_first : 0;
                double uki = 0.0;
                int len = first_chunk ? len_first : 0;
                if (!first_chunk && lane < ns) {
                    pk = l_to_u[s0 + lane];   // (k, i) in U: row k's segment from column i on
                    len = int(rp[lcol[s0 + lane] + 1] - pk);
                }
                if (lane < ns) uki = __ldcg(uin + pk);
                int incl = len;
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(full, incl, o);
                    if (lane >= o) incl += v;
                }
                const int total = __shfl_sync(full, incl, 31);
                for (int q = 0; q < ns; ++q) table[wb][q][lane] = 0.0;
                __syncwarp();
                for (int base = 0; base < total; base += 32) {
                    const int idx = base + lane;
                    int s = 0;
                    for (int q = 0; q < ns; ++q) s += __shfl_sync(full, incl, q) <= idx ? 1 : 0;
                    const int sc = min(s, ns - 1);
                    const int start = __shfl_sync(full, incl, max(sc - 1, 0)) * (sc > 0 ? 1 : 0);
                    const i64 pks = __shfl_sync(full, pk, sc);
                    const double ukis = __shfl_sync(full, uki, sc);
                    if (idx < total) {
                        const i64 x = pks + (idx - start);
                        const int32_t cx = col[x];
                        int lo = 0, hi = m;   // column cx among row i's
                        while (lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            if (rowcol[wb][mid] < cx) lo = mid + 1; else hi = mid;
                        }
                        if (lo < m && rowcol[wb][lo] == cx) table[wb][s][lo] = __dmul_rn(ukis, __ldcg(uin + x));
                    }
                }
                __syncwarp();
                for (int q = 0; q < ns; ++q) acc = __dsub_rn(acc, table[wb][q][lane]);
                __syncwarp();
            }
            const double d = __shfl_sync(full, acc, 0);
            if (!(d > 0.0)) {
                if (lane == 0) atomicExch(failed, 1);
            } else {
                const double rd = sqrt(d);
                if (lane == 0) u[b] = rd;
                else if (own) u[b + lane] = acc / rd;
            }
        }
        // publish row i (a failed pivot publishes too: the attempt is retried
        // with a larger shift, and no row may wait for ever)
        if constexpr (!SWEEP) {
            __threadfence();
            __syncwarp();
            if (lane == 0) st_release_gpu(done + i, 1);
        }
    }
}

// Starting factor of the fixed-point form: row i of the scaled matrix divided
// by the root of its (shifted) diagonal
__global__ void k_ic0_start(i64 n, const i64* __restrict__ rp, const double* __restrict__ a, double shift,
                            double* __restrict__ u, int* __restrict__ failed) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double d = a[rp[i]] + shift;
        if (!(d > 0.0)) { atomicExch(failed, 1); continue; }
        const double rd = sqrt(d);
        u[rp[i]] = rd;
        for (i64 k = rp[i] + 1; k < rp[i + 1]; ++k) u[k] = a[k] / rd;
    }
}

__global__ void k_slab_values(i64 count, const i64* __restrict__ src, const double* __restrict__ u,
                              double* __restrict__ v, float* __restrict__ v32) {
    for (i64 k = blockIdx.x * i64(blockDim.x) + threadIdx.x; k < count; k += i64(gridDim.x) * blockDim.x) {
        const double x = src[k] >= 0 ? u[src[k]] : 0.0;
        v[k] = x;
        v32[k] = float(x);
    }
}
__global__ void k_slab_diag(i64 count, const i64* __restrict__ src, const double* __restrict__ u,
                            double* __restrict__ inv, float* __restrict__ inv32) {
    for (i64 k = blockIdx.x * i64(blockDim.x) + threadIdx.x; k < count; k += i64(gridDim.x) * blockDim.x) {
        const double x = 1.0 / u[src[k]];
        inv[k] = x;
        inv32[k] = float(x);
    }
}
__global__ void k_to_float(i64 n, const double* __restrict__ a, float* __restrict__ b) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = float(a[i]);
}

// One level-scheduled sweep in one CTA:
//   y[row] = (scale_in[row] * in[row] - sum_k val * y[col]) * inv_diag
// (y has n + 1 entries, y[n] = 0 serves the padding); out[row] = scale_out * y[row].
// After convergence (flags) the sweep is skipped.
template<class T>
__global__ void __launch_bounds__(TRI_THREADS) k_trisolve(i64 n, i64 n_levels, const i64* __restrict__ lev_ptr,
                                                          const i64* __restrict__ slab_base, const int32_t* __restrict__ width,
                                                          const int32_t* __restrict__ rows, const int32_t* __restrict__ col,
                                                          const T* __restrict__ val, const T* __restrict__ inv_diag,
                                                          const double* __restrict__ in, const T* __restrict__ scale_in,
                                                          T* __restrict__ y, const T* __restrict__ scale_out,
                                                          double* __restrict__ out, const double* __restrict__ partials,
                                                          const double* __restrict__ flags, double tol2) {
    __shared__ double sh[40];
    if (flags) {
        if (flags[S_DONE] != 0.0 || converged(partials, flags, tol2, sh)) return;
    }
    if (threadIdx.x == 0) y[n] = T(0);
    __syncthreads();
    for (i64 l = 0; l < n_levels; ++l) {
        const i64 b = lev_ptr[l], cnt = lev_ptr[l + 1] - b;
        const i64 base = slab_base[l];
        const int w = width[l];
        for (i64 t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int32_t row = rows[b + t];
            T s = scale_in ? scale_in[row] * T(in[row]) : T(in[row]);
            for (int k = 0; k < w; ++k) {
                const i64 e = base + i64(k) * cnt + t;
                s -= val[e] * y[col[e]];
            }
            const T v = s * inv_diag[b + t];
            y[row] = v;
            if (out) out[row] = scale_out ? double(scale_out[row] * v) : double(v);
        }
        __syncthreads();
    }
}

// levels of a triangular dependency graph: forward rows depend on smaller
// columns, backward rows on larger ones
i64 build_levels(const std::vector<i64>& rp, const std::vector<int32_t>& col, bool forward, std::vector<i64>& level_of) {
    const i64 n = i64(rp.size()) - 1;
    level_of.assign(size_t(n), 0);
    i64 max_level = -1;
    for (i64 it = 0; it < n; ++it) {
        const i64 i = forward ? it : n - 1 - it;
        i64 lv = 0;
        for (i64 k = rp[size_t(i)]; k < rp[size_t(i) + 1]; ++k) {
            const i64 c = col[size_t(k)];
            if (forward ? c < i : c > i) lv = std::max(lv, level_of[size_t(c)] + 1);
        }
        level_of[size_t(i)] = lv;
        max_level = std::max(max_level, lv);
    }
    return max_level + 1;
}

// Level-ELL slab of the triangular matrix with rows rp/col whose value of
// entry s is factor[val_index[s]] and whose diagonal sits at diag_pos[row].
void build_slab(Ctx& ctx, const std::vector<i64>& rp, const std::vector<int32_t>& col, const std::vector<i64>& val_index,
                const std::vector<i64>& diag_pos, bool forward, TriSlab& slab, std::vector<i64>* lev_ptr_out,
                std::vector<int32_t>* rows_out) {
    const i64 n = i64(rp.size()) - 1;
    std::vector<i64> level_of;
    const i64 L = build_levels(rp, col, forward, level_of);
    std::vector<i64> lev_ptr(size_t(L + 1), 0);
    for (i64 i = 0; i < n; ++i) ++lev_ptr[size_t(level_of[size_t(i)]) + 1];
    for (i64 l = 0; l < L; ++l) lev_ptr[size_t(l) + 1] += lev_ptr[size_t(l)];
    std::vector<int32_t> rows(static_cast<size_t>(n));
    {
        std::vector<i64> cur(lev_ptr.begin(), lev_ptr.end() - 1);
        for (i64 i = 0; i < n; ++i) rows[size_t(cur[size_t(level_of[size_t(i)])]++)] = int32_t(i);
    }
    std::vector<i64> base(static_cast<size_t>(L));
    std::vector<int32_t> width(static_cast<size_t>(L));
    i64 total = 0;
    for (i64 l = 0; l < L; ++l) {
        int w = 0;
        for (i64 t = lev_ptr[size_t(l)]; t < lev_ptr[size_t(l) + 1]; ++t) {
            const int32_t r = rows[size_t(t)];
            w = std::max(w, int(rp[size_t(r) + 1] - rp[size_t(r)] - 1));
        }
        base[size_t(l)] = total;
        width[size_t(l)] = w;
        total += i64(w) * (lev_ptr[size_t(l) + 1] - lev_ptr[size_t(l)]);
    }
    std::vector<int32_t> scol(static_cast<size_t>(total), int32_t(n));
    std::vector<i64> ssrc(static_cast<size_t>(total), -1), dsrc(static_cast<size_t>(n));
    for (i64 l = 0; l < L; ++l) {
        const i64 cnt = lev_ptr[size_t(l) + 1] - lev_ptr[size_t(l)];
        for (i64 t = 0; t < cnt; ++t) {
            const int32_t r = rows[size_t(lev_ptr[size_t(l)] + t)];
            int k = 0;
            for (i64 s = rp[size_t(r)]; s < rp[size_t(r) + 1]; ++s) {
                if (s == diag_pos[size_t(r)]) continue;
                const i64 e = base[size_t(l)] + i64(k) * cnt + t;
                scol[size_t(e)] = col[size_t(s)];
                ssrc[size_t(e)] = val_index[size_t(s)];
                ++k;
            }
            dsrc[size_t(lev_ptr[size_t(l)] + t)] = val_index[size_t(diag_pos[size_t(r)])];
        }
    }
    slab.n_levels = L;
    slab.entries = total;
    slab.lev_ptr.upload(lev_ptr.data(), lev_ptr.size(), ctx.stream);
    slab.slab_base.upload(base.data(), base.size(), ctx.stream);
    slab.width.upload(width.data(), width.size(), ctx.stream);
    slab.rows.upload(rows.data(), rows.size(), ctx.stream);
    slab.col.upload(scol.data(), scol.size(), ctx.stream);
    slab.src.upload(ssrc.data(), ssrc.size(), ctx.stream);
    slab.diag_src.upload(dsrc.data(), dsrc.size(), ctx.stream);
    slab.val.resize(size_t(total)); slab.val32.resize(size_t(total));
    slab.inv_diag.resize(size_t(n)); slab.inv_diag32.resize(size_t(n));
    if (lev_ptr_out) *lev_ptr_out = lev_ptr;
    if (rows_out) *rows_out = rows;
    NL_CUDA(cudaStreamSynchronize(ctx.stream));   // host staging vectors end here
}

void finalize_scalar(Ctx& ctx, const double* partials, double* dst);

__global__ void k_finalize(const double* __restrict__ partials, double* __restrict__ dst) {
    __shared__ double sh[40];
    const double s = sum_partials(partials, sh);
    if (threadIdx.x == 0) *dst = s;
}

void finalize_scalar(Ctx& ctx, const double* partials, double* dst) {
    NL_LAUNCH(k_finalize, 1, RED_THREADS, 0, ctx.stream, partials, dst);
}

void precondition(Ctx& ctx, const IncompleteCholesky* M, const double* r, double* z, const double* partials,
                  const double* flags, double tol2) {
    const i64 n = ctx.cg.n;
    if (M && M->fwd_plan.ok && M->bwd_plan.ok && !ctx.force_global_sweeps) {
        sweep_apply(ctx, const_cast<IncompleteCholesky&>(*M), r, z, partials, flags, tol2);
        return;
    }
    if (!M) {
        if (flags) NL_LAUNCH(k_copy_if_running, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, r, z, partials, flags, tol2);
        else NL_LAUNCH(k_copy, grid_for(n, 256), 256, 0, ctx.stream, n, r, z);
        return;
    }
    // y = U^-T (S r); z = S U^-1 y
    NL_LAUNCH(k_trisolve<double>, 1, TRI_THREADS, 0, ctx.stream, n, M->fwd.n_levels, M->fwd.lev_ptr.p, M->fwd.slab_base.p,
              M->fwd.width.p, M->fwd.rows.p, M->fwd.col.p, M->fwd.val.p, M->fwd.inv_diag.p, r, M->scale.p, M->y.p,
              static_cast<const double*>(nullptr), static_cast<double*>(nullptr), partials, flags, tol2);
    NL_LAUNCH(k_trisolve<double>, 1, TRI_THREADS, 0, ctx.stream, n, M->bwd.n_levels, M->bwd.lev_ptr.p, M->bwd.slab_base.p,
              M->bwd.width.p, M->bwd.rows.p, M->bwd.col.p, M->bwd.val.p, M->bwd.inv_diag.p, M->y.p,
              static_cast<const double*>(nullptr), M->w.p, M->scale.p, z, partials, flags, tol2);
}

}  // namespace

// ------------------------------------------------------------------ API
void spmv_full(Ctx& ctx, const Csr& A, const double* x, double* y) {
    NL_LAUNCH(k_spmv, grid_for(A.rows * 32, RED_THREADS, i64(RED_BLOCKS) * 4), RED_THREADS, 0, ctx.stream, A.rows,
              A.rowptr.p, reinterpret_cast<const int4*>(A.col.p), reinterpret_cast<const double2*>(A.val.p), x, y,
              static_cast<double*>(nullptr), static_cast<const double*>(nullptr));
}

// The exact level-scheduled sweeps' layouts from the factor's structure (host):
// level-ELL slabs of both triangles and the TMA-fed shared-memory plans when
// every dependency fits the ring, with the factor's values.  Built once per
// factorisation, the first time a solve uses exact sweeps (FP64 ILLT-CG, or
// the mixed solve with exact FP32 sweeps); not inside a stream capture.
void ilt_exact_layouts(Ctx& ctx, IncompleteCholesky& ic) {
    if (ic.exact_ready || !ic.ok) return;
    const i64 n = ic.n, nnz = ic.nnz;
    PhaseTimer timer(ctx.stream, "ilt_exact_layouts");
    std::vector<i64> rp(size_t(n + 1)), lrp(size_t(n + 1)), l_to_u(static_cast<size_t>(nnz));
    std::vector<int32_t> col(static_cast<size_t>(nnz)), lcol(static_cast<size_t>(nnz));
    ic.rp.download(rp.data(), rp.size(), ctx.stream);
    ic.col.download(col.data(), col.size(), ctx.stream);
    ic.lrp.download(lrp.data(), lrp.size(), ctx.stream);
    ic.lcol.download(lcol.data(), lcol.size(), ctx.stream);
    ic.l_to_u.download(l_to_u.data(), l_to_u.size(), ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    std::vector<i64> ident(static_cast<size_t>(nnz)), u_diag(static_cast<size_t>(n)), l_diag(static_cast<size_t>(n));
    std::iota(ident.begin(), ident.end(), i64(0));
    for (i64 r = 0; r < n; ++r) { u_diag[size_t(r)] = rp[size_t(r)]; l_diag[size_t(r)] = lrp[size_t(r) + 1] - 1; }
    std::vector<i64> fwd_lev_ptr, bwd_lev_ptr;
    std::vector<int32_t> fwd_rows, bwd_rows;
    build_slab(ctx, lrp, lcol, l_to_u, l_diag, true, ic.fwd, &fwd_lev_ptr, &fwd_rows);
    build_slab(ctx, rp, col, ident, u_diag, false, ic.bwd, &bwd_lev_ptr, &bwd_rows);
    if (sweep_plan_build(ctx, fwd_lev_ptr, fwd_rows, lrp, lcol, l_to_u, l_diag, ic.fwd_plan))
        sweep_plan_build(ctx, bwd_lev_ptr, bwd_rows, rp, col, ident, u_diag, ic.bwd_plan);
    timer.mark("layouts");
    if (ic.fwd_plan.ok && ic.bwd_plan.ok) {
        sweep_plan_fill(ctx, ic.fwd_plan, ic.u.p);
        sweep_plan_fill(ctx, ic.bwd_plan, ic.u.p);
    }
    for (TriSlab* sl : {&ic.fwd, &ic.bwd}) {
        if (sl->entries)
            NL_LAUNCH(k_slab_values, grid_for(sl->entries, 256), 256, 0, ctx.stream, sl->entries, sl->src.p, ic.u.p,
                      sl->val.p, sl->val32.p);
        NL_LAUNCH(k_slab_diag, grid_for(n, 256), 256, 0, ctx.stream, n, sl->diag_src.p, ic.u.p, sl->inv_diag.p,
                  sl->inv_diag32.p);
    }
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    ic.exact_ready = true;
    timer.mark("value fills");
}

void ilt_build(Ctx& ctx, const Csr& upper, IncompleteCholesky& ic, bool tma_plans, bool approximate) {
    const i64 n = upper.rows, nnz = upper.nnz;
    ic.n = n; ic.nnz = nnz;
    ic.approximate = approximate;
    PhaseTimer timer(ctx.stream, "ilt_build");
    // U^T, the factorisation's levels (exact form) and the Jacobi layouts on the device
    ilt_structure_gpu(ctx, upper, ic, !approximate);
    timer.mark("structure");
    ctx.sweep_error.resize(1);
    ctx.sweep_error.zero(ctx.stream);
    ic.fwd_plan = SweepPlan{};
    ic.bwd_plan = SweepPlan{};
    for (TriSlab* sl : {&ic.fwd, &ic.bwd}) { sl->n_levels = 0; sl->entries = 0; }
    ic.exact_ready = false;
    ic.y.resize(size_t(n + 1)); ic.w.resize(size_t(n + 1));
    ic.y32.resize(size_t(n + 1)); ic.w32.resize(size_t(n + 1));
    // Lin-More scaling and the shifted factorisation
    ic.scale.resize(size_t(n)); ic.scale.zero(ctx.stream);
    ic.scale32.resize(size_t(n));
    NL_LAUNCH(k_colnorm2, grid_for(n, 256), 256, 0, ctx.stream, n, upper.rowptr.p, upper.col.p, upper.val.p, ic.scale.p);
    NL_LAUNCH(k_scale, grid_for(n, 256), 256, 0, ctx.stream, n, ic.scale.p);
    NL_LAUNCH(k_to_float, grid_for(n, 256), 256, 0, ctx.stream, n, ic.scale.p, ic.scale32.p);
    ic.a_scaled.resize(size_t(nnz)); ic.u.resize(size_t(nnz));
    dbuf<unsigned long long> mind;
    dbuf<int> failed, sync;   // failed: [pivot, timeout]; sync: [ticket, done flags per row]
    mind.resize(1); failed.resize(2); sync.resize(size_t(n + 1));
    // resident warps well above the widest level, so the rows of the next
    // levels are taken while the current one finishes
    const unsigned ic_grid = unsigned(std::max<i64>(1, std::min<i64>((n + IC_WARPS - 1) / IC_WARPS, 152 * 2)));
    const unsigned long long init = ~0ull;
    NL_CUDA(cudaMemcpyAsync(mind.p, &init, sizeof init, cudaMemcpyHostToDevice, ctx.stream));
    NL_LAUNCH(k_scaled, grid_for(n, 256), 256, 0, ctx.stream, n, upper.rowptr.p, upper.col.p, upper.val.p, ic.scale.p,
              ic.a_scaled.p, mind.p);
    unsigned long long mbits = 0;
    NL_CUDA(cudaMemcpyAsync(&mbits, mind.p, sizeof mbits, cudaMemcpyDeviceToHost, ctx.stream));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    const unsigned long long raw = (mbits & 0x8000000000000000ull) ? (mbits & 0x7fffffffffffffffull) : ~mbits;
    double mindiag;
    std::memcpy(&mindiag, &raw, sizeof mindiag);
    const double initial_shift = 1e-3;
    double shift = mindiag <= 0.0 ? initial_shift - mindiag : 0.0;
    ic.ok = false;
    dbuf<double> u_prev;
    if (approximate) u_prev.resize(size_t(nnz));
    for (ic.attempts = 1; ic.attempts <= 10; ++ic.attempts) {
        failed.zero(ctx.stream);
        if (approximate) {
            // the sweeps alternate between the two buffers and end in ic.u
            double* buf[2] = {IC_SWEEPS % 2 ? u_prev.p : ic.u.p, IC_SWEEPS % 2 ? ic.u.p : u_prev.p};
            NL_LAUNCH(k_ic0_start, grid_for(n, 256), 256, 0, ctx.stream, n, ic.rp.p, ic.a_scaled.p, shift, buf[0],
                      failed.p);
            const unsigned sweep_grid = unsigned(std::max<i64>(1, std::min<i64>((n + IC_WARPS - 1) / IC_WARPS, 152 * 16)));
            for (int sw = 0; sw < IC_SWEEPS; ++sw) {
                sync.zero(ctx.stream);   // the sweep's row ticket
                NL_LAUNCH(k_ic0_rows<true>, sweep_grid, IC_WARPS * 32, 0, ctx.stream, n,
                          static_cast<const int32_t*>(nullptr), ic.rp.p, ic.col.p, ic.a_scaled.p, shift, ic.lrp.p,
                          ic.lcol.p, ic.l_to_u.p, buf[sw & 1], buf[(sw + 1) & 1], sync.p, sync.p + 1, failed.p,
                          failed.p + 1);
            }
        } else {
            sync.zero(ctx.stream);
            NL_LAUNCH(k_ic0_rows<false>, ic_grid, IC_WARPS * 32, 0, ctx.stream, n, ic.ic_rows.p, ic.rp.p, ic.col.p,
                      ic.a_scaled.p, shift, ic.lrp.p, ic.lcol.p, ic.l_to_u.p, ic.u.p, ic.u.p, sync.p, sync.p + 1,
                      failed.p, failed.p + 1);
        }
        int hf[2] = {0, 0};
        NL_CUDA(cudaMemcpyAsync(hf, failed.p, sizeof hf, cudaMemcpyDeviceToHost, ctx.stream));
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
        NL_REQUIRE(!hf[1], NLGPU_ERR_TIMEOUT, "the factorisation's wait for a dependency row timed out");
        if (!hf[0]) { ic.ok = true; break; }
        shift = std::max(initial_shift, 2.0 * shift);
    }
    ic.shift = shift;
    timer.mark("scaling, factorisation");
    if (!ic.ok) return;
    jacobi_fill(ctx, ic);
    timer.mark("value fills");
    if (tma_plans) ilt_exact_layouts(ctx, ic);
}

void ilt_apply(Ctx& ctx, const IncompleteCholesky& ic, const double* r, double* z) {
    ilt_exact_layouts(ctx, const_cast<IncompleteCholesky&>(ic));
    ctx.cg.n = ic.n;
    precondition(ctx, &ic, r, z, nullptr, nullptr, 0.0);
}

CgResult cg_solve(Ctx& ctx, const Csr& A, const IncompleteCholesky* M, const double* b, double* x,
                  double tolerance, i64 max_iterations, bool x_is_initial_guess, const CgChunkHook& on_chunk) {
    if (M) ilt_exact_layouts(ctx, const_cast<IncompleteCholesky&>(*M));
    const i64 n = A.rows;
    CgWork& w = ctx.cg;
    w.n = n;
    w.r.reserve(size_t(n)); w.z.reserve(size_t(n)); w.p.reserve(size_t(n)); w.q.reserve(size_t(n));
    w.partial.reserve(size_t(P_COUNT) * RED_BLOCKS);
    w.scalars.reserve(8);
    if (!x_is_initial_guess) NL_CUDA(cudaMemsetAsync(x, 0, size_t(n) * sizeof(double), ctx.stream));
    double* part = w.partial.p;
    double* flags = w.scalars.p;
    const double tol2 = tolerance * tolerance;
    CgResult res;
    // |b|^2
    NL_LAUNCH(k_dot, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, b, b, part + P_BB * RED_BLOCKS,
              static_cast<const double*>(nullptr));
    NL_CUDA(cudaMemsetAsync(flags, 0, 8 * sizeof(double), ctx.stream));
    finalize_scalar(ctx, part + P_BB * RED_BLOCKS, flags + S_BB);
    for (int restart = 0; restart < 4; ++restart) {
        // r = b - A x; z = M^-1 r; p = z; rz -> P_RZ_B (the "current" buffer of an even iteration)
        spmv_full(ctx, A, x, w.r.p);
        NL_LAUNCH(k_residual, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, b, w.r.p, part + P_RR * RED_BLOCKS);
        precondition(ctx, M, w.r.p, w.z.p, nullptr, nullptr, 0.0);
        NL_LAUNCH(k_copy, grid_for(n, 256), 256, 0, ctx.stream, n, w.z.p, w.p.p);
        NL_LAUNCH(k_dot, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, w.r.p, w.z.p, part + P_RZ_B * RED_BLOCKS,
                  static_cast<const double*>(nullptr));
        double host[8];
        NL_CUDA(cudaMemsetAsync(flags + S_DONE, 0, sizeof(double), ctx.stream));
        finalize_scalar(ctx, part + P_RR * RED_BLOCKS, flags + S_RR_FINAL);
        NL_CUDA(cudaMemcpyAsync(host, flags, 8 * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
        const double bb = host[S_BB];
        if (bb == 0.0) { NL_CUDA(cudaMemsetAsync(x, 0, size_t(n) * sizeof(double), ctx.stream)); res.converged = true; break; }
        if (host[S_RR_FINAL] <= tol2 * bb) { res.converged = true; break; }
        // the iteration counter carries over restarts
        NL_CUDA(cudaMemcpyAsync(flags + S_ITERS, &host[S_ITERS], sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
        i64 done_iters = i64(host[S_ITERS]);
        bool done = false;
        max_iterations = std::min<i64>(max_iterations, i64(1) << 40);
        while (!done) {
            for (int it = 0; it < GRAPH_ITERS; ++it) {
                const int parity = it & 1;
                NL_LAUNCH(k_spmv, grid_for(n * 32, RED_THREADS, RED_BLOCKS), RED_THREADS, 0, ctx.stream, n, A.rowptr.p,
                          reinterpret_cast<const int4*>(A.col.p), reinterpret_cast<const double2*>(A.val.p), w.p.p,
                          w.q.p, static_cast<double*>(nullptr), flags);
                NL_LAUNCH(k_dot, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, w.p.p, w.q.p, part + P_PQ * RED_BLOCKS, flags);
                NL_LAUNCH(k_update_xr, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, x, w.r.p, w.p.p, w.q.p, part, parity,
                          flags, max_iterations);
                precondition(ctx, M, w.r.p, w.z.p, part, flags, tol2);
                NL_LAUNCH(k_dot, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, w.r.p, w.z.p,
                          part + (parity ? P_RZ_B : P_RZ_A) * RED_BLOCKS, flags);
                NL_LAUNCH(k_update_p, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, w.p.p, w.z.p, part, parity, flags, tol2,
                          max_iterations);
            }
            NL_CUDA(cudaMemcpyAsync(host, flags, 8 * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
            NL_CUDA(cudaStreamSynchronize(ctx.stream));
            done_iters = i64(host[S_ITERS]);
            done = host[S_DONE] != 0.0 || done_iters >= max_iterations;
            if (on_chunk && !done) on_chunk(done_iters, x);
        }
        res.iterations = done_iters;
        // reference measure sqrt(r.z)/|b| from the last r.z partials
        finalize_scalar(ctx, part + ((done_iters & 1) ? P_RZ_A : P_RZ_B) * RED_BLOCKS, flags + S_RZ0);
        // true residual
        spmv_full(ctx, A, x, w.q.p);
        NL_LAUNCH(k_copy, grid_for(n, 256), 256, 0, ctx.stream, n, w.q.p, w.z.p);
        NL_LAUNCH(k_residual, RED_BLOCKS, RED_THREADS, 0, ctx.stream, n, b, w.z.p, part + P_RR * RED_BLOCKS);
        finalize_scalar(ctx, part + P_RR * RED_BLOCKS, flags + S_RR_FINAL);
        NL_CUDA(cudaMemcpyAsync(host, flags, 8 * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
        res.residual = std::sqrt(host[S_RR_FINAL] / host[S_BB]);
        res.reference_residual = std::sqrt(std::fabs(host[S_RZ0]) / host[S_BB]);
        res.converged = res.residual <= tolerance;
        if (res.converged || done_iters >= max_iterations) break;
        x_is_initial_guess = true;   // recurrence drifted from the true residual: restart from x
    }
    return res;
}

}  // namespace nlgpu
