// Mixed-precision solve: flexible CG in FP32 with FP64 reliable updates.
//
// The plain path runs slae::conjugate_gradient (conjugate_gradient.hpp:48-79)
// in FP64.  This form keeps FP64 only where accuracy is decided -- the
// residual b - A x (FP64 matrix, FP64 SpMV), the solution, every global dot
// product and norm (FP64 block and global sums; the inner iteration's
// products and each thread's one or two elements in FP32, since a warp-wide
// FP64 instruction costs GB300 16 issue cycles of its FP64 pipe), and the IC(0)
// pivots (the factor is computed in FP64) -- and runs the iteration itself in FP32:
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
// and moves 8 bytes per entry instead of 12 (6 with 16-bit column offsets).
// Scalars stay on the device: the block that finishes last in each reducing
// kernel sums the block partials and forms alpha, the betas and the stop test
// (no separate scalar kernels); the host reads the done flag once per
// MX_ITERS iterations.
#include "common.cuh"

#include <cmath>

namespace nlgpu {

namespace {

constexpr int MX_THREADS = 256;
constexpr int MX_ITERS = 16;
constexpr int MX_M = 4;   // directions kept for the A-orthogonalisation (flexible CG truncation)
constexpr i64 MX_UPDATE_MAX = 64;   // iterations between reliable updates at most
// partial slots: P_RR as in the FP64 solver (the exact sweeps' early exit reads
// the residual there), P_RZ_A / P_RZ_B for p.r, then the SpMV's p.q partials
// (MX_M slots of room: the SpMV runs SPMV_BLOCKS blocks) and z.q_i
constexpr int SPMV_BLOCKS = 2 * RED_BLOCKS;
static_assert(SPMV_BLOCKS <= MX_M * RED_BLOCKS, "the SpMV partials overflow their slots");
enum { M_PQ = P_COUNT, M_ZQ = P_COUNT + MX_M, M_SLOTS = P_COUNT + 2 * MX_M };
// scalar slots after the solver's (S_BB .. S_RR_FINAL): alpha, the betas, p_k.r
// (the next alpha's numerator) and p_i.q_i of the stored directions
enum { S_ALPHA = 8, S_BETA = 9, S_PR = 9 + MX_M, S_PQ = 10 + MX_M, S_MIXED_COUNT = 10 + 2 * MX_M };

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

// N block sums in one pass (sh: at least 33 N doubles); every thread gets them
template<int N>
__device__ __forceinline__ void mx_block_sums(double (&v)[N], double* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = int(blockDim.x >> 5);
#pragma unroll
    for (int s = 0; s < N; ++s) v[s] = warp_sum(v[s]);
    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < N; ++s) sh[s * 32 + warp] = v[s];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int s = 0; s < N; ++s) {
            const double t = warp_sum(lane < nw ? sh[s * 32 + lane] : 0.0);
            if (lane == 0) sh[32 * N + s] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < N; ++s) v[s] = sh[32 * N + s];
    __syncthreads();
}

// Publishes this block's N sums as partials (slot s at part + s RED_BLOCKS) and
// returns true in the block that finished last, with v replaced by the totals
// over all blocks; that block also re-arms the ticket for the next kernel.
// (Every later kernel of the stream starts after this one has ended.)
template<int N>
__device__ __forceinline__ bool mx_reduce_last(double (&v)[N], double* part, unsigned* ticket, double* sh) {
    __shared__ unsigned last;
    mx_block_sums<N>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < N; ++s) part[s * RED_BLOCKS + blockIdx.x] = v[s];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1 ? 1u : 0u;
    }
    __syncthreads();
    if (!last) return false;
#pragma unroll
    for (int s = 0; s < N; ++s) v[s] = 0.0;
    for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
#pragma unroll
        for (int s = 0; s < N; ++s) v[s] += __ldcg(part + s * RED_BLOCKS + k);
    }
    mx_block_sums<N>(v, sh);
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// q = A32 p (FP32 values, FP32 accumulation), warp per padded full row, in
// difference form  y_i = sum_j a_ij (x_j - x_i) + s_i x_i  with s_i the row sum
// of the FP64 matrix: the rows of the conductivity matrix sum to (nearly) zero,
// so for smooth x the plain FP32 sum would cancel to a result far below the
// rounding error of its terms, while here each FP32 entry multiplies a small
// difference.  p.q in FP64; in the solve the last block stores it and forms
// alpha.  Columns are int32 (C = int32_t) or, when every |column - row| fits
// 16 bits, int16 offsets from the row (C = int16_t): 6 instead of 8 bytes per
// entry.  Lane l takes entries l, l + 32, ... of its warp's row, so each
// gather instruction of the warp reads 32 neighbouring columns (few cache
// lines) rather than 32 columns four entries apart; four entries per lane are
// loaded before their gathers.  Launched with SPMV_BLOCKS blocks of 256
// threads: with at most 32 registers per thread, 8 blocks fill an SM.
template<class C>
__global__ void __launch_bounds__(MX_THREADS) k_spmv32(i64 n, const i64* __restrict__ rp, const C* __restrict__ col,
                                                       const float* __restrict__ val,
                                                       const float* __restrict__ rowsum, const float* __restrict__ x,
                                                       float* __restrict__ y, double* __restrict__ dot_partial,
                                                       double* __restrict__ flags, i64 ring, unsigned* ticket) {
    __shared__ double sh[40];
    if (flags && flags[S_DONE] != 0.0) return;
    i64 slot = 0;
    if (ring) {   // direction slot of the current iteration in the rings of x and y
        slot = i64(flags[S_ITERS]) % MX_M;
        x += slot * ring; y += slot * ring;
    }
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    float dot = 0.0f;   // this warp's few rows in FP32; block and global sums in FP64
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        const i64 e = rp[r + 1];
        const float xr = x[r];
        const float* xo = sizeof(C) == 4 ? x : x + r;   // int16 offsets count from the row
        float s = 0.0f;
        i64 q = rp[r] + lane;
        for (; q + 96 < e; q += 128) {
            const C c0 = __ldg(col + q), c1 = __ldg(col + q + 32), c2 = __ldg(col + q + 64), c3 = __ldg(col + q + 96);
            const float v0 = __ldg(val + q), v1 = __ldg(val + q + 32), v2 = __ldg(val + q + 64),
                        v3 = __ldg(val + q + 96);
            s += v0 * (xo[c0] - xr) + v1 * (xo[c1] - xr) + v2 * (xo[c2] - xr) + v3 * (xo[c3] - xr);
        }
        for (; q < e; q += 32) s += __ldg(val + q) * (xo[__ldg(col + q)] - xr);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            s += rowsum[r] * xr;
            y[r] = s;
            dot = fmaf(s, xr, dot);
        }
    }
    if (dot_partial) {   // p_j.q_j: the last block stores it and alpha = (p_j.r) / (p_j.q_j)
        double v[1] = {double(dot)};
        if (mx_reduce_last<1>(v, dot_partial, ticket, sh) && threadIdx.x == 0) {
            flags[S_PQ + slot] = v[0];
            flags[S_ALPHA] = flags[S_PR] / v[0];
        }
    }
}

// q = A32 p from the strictly upper part of the symmetric matrix (half the
// bytes of the full rows; NLGPU_OPTION_FP32_SYMMETRIC).  Measured on the
// 300x300 serendipity problem it is no faster than the full-row kernel (0.77
// against 0.79 ms per product; one more launch for p.q): the shared-memory
// atomics, not the bytes, bound it, so full rows stay the default.  In the same difference form, an upper entry a_rc
// (c > r) gives t = a_rc (p_c - p_r) to row r and -t to row c.  Each CTA (one
// per SM, so that the x values of its rows' reach stay in L1 beside the
// window) owns a contiguous range of rows with equal entry counts and
// accumulates every contribution with shared-memory atomics into a window of
// the columns its rows reach (its first row up to the farthest column); the
// window is then added to q with global atomics, so q must be zero before the
// launch (the kernel that forms the next direction clears its slot).  Warp per
// row, entry per lane, four entries in flight per lane.  Summation order is
// not fixed (atomics); the flexible FP32 iteration absorbs that.  p.q is taken
// afterwards from the finished q (k_pq32): alpha must match the q the residual
// update uses, or the recurrence loses its local orthogonality.
constexpr int UP_THREADS = 1024;

__global__ void __launch_bounds__(UP_THREADS, 1) k_spmv32_up(const i64* __restrict__ rp, const uint16_t* __restrict__ off,
                                                             const float* __restrict__ val,
                                                             const float* __restrict__ rowsum,
                                                             const int32_t* __restrict__ part_rows,
                                                             const int32_t* __restrict__ window,
                                                             const float* __restrict__ x, float* __restrict__ y,
                                                             const double* __restrict__ flags, i64 ring) {
    extern __shared__ float acc[];
    if (flags && flags[S_DONE] != 0.0) return;
    if (ring) {
        const i64 slot = i64(flags[S_ITERS]) % MX_M;
        x += slot * ring; y += slot * ring;
    }
    const int r0 = part_rows[blockIdx.x], r1 = part_rows[blockIdx.x + 1], W = window[blockIdx.x];
    for (int k = threadIdx.x; k < W; k += blockDim.x) acc[k] = 0.0f;
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = int(blockDim.x >> 5);
    for (int r = r0 + int(threadIdx.x >> 5); r < r1; r += nw) {
        const float xr = x[r];
        const float* xo = x + r;
        float* ao = acc + (r - r0);
        const i64 b = rp[r];
        const uint16_t* orow = off + b;
        const float* vrow = val + b;
        const int len = int(rp[r + 1] - b);
        float s = 0.0f;
        int q = lane;
        for (; q + 96 < len; q += 128) {
            const int o0 = __ldg(orow + q), o1 = __ldg(orow + q + 32), o2 = __ldg(orow + q + 64),
                      o3 = __ldg(orow + q + 96);
            const float v0 = __ldg(vrow + q), v1 = __ldg(vrow + q + 32), v2 = __ldg(vrow + q + 64),
                        v3 = __ldg(vrow + q + 96);
            const float t0 = v0 * (xo[o0] - xr), t1 = v1 * (xo[o1] - xr), t2 = v2 * (xo[o2] - xr),
                        t3 = v3 * (xo[o3] - xr);
            s += (t0 + t1) + (t2 + t3);
            atomicAdd(ao + o0, -t0); atomicAdd(ao + o1, -t1); atomicAdd(ao + o2, -t2); atomicAdd(ao + o3, -t3);
        }
        for (; q < len; q += 32) {
            const int o = __ldg(orow + q);
            const float t = __ldg(vrow + q) * (xo[o] - xr);
            s += t;
            atomicAdd(ao + o, -t);
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) atomicAdd(ao, s + rowsum[r] * xr);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < W; k += blockDim.x) {
        const float v = acc[k];
        if (v != 0.0f) atomicAdd(y + r0 + k, v);
    }
}

// p_j.q_j of the current direction slot j (after the symmetric SpMV); the last
// block stores it and forms alpha = (p_j.r) / (p_j.q_j)
__global__ void __launch_bounds__(MX_THREADS) k_pq32(i64 n, const float* __restrict__ pring,
                                                     const float* __restrict__ qring, double* __restrict__ part,
                                                     double* __restrict__ flags, unsigned* ticket) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const i64 slot = i64(flags[S_ITERS]) % MX_M;
    const float* p = pring + slot * n;
    const float* q = qring + slot * n;
    float s = 0.0f;   // a thread's one or two elements in FP32; block and global sums in FP64
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        s = fmaf(p[i], q[i], s);
    double v[1] = {double(s)};
    if (mx_reduce_last<1>(v, part, ticket, sh) && threadIdx.x == 0) {
        flags[S_PQ + slot] = v[0];
        flags[S_ALPHA] = flags[S_PR] / v[0];
    }
}

// strictly upper entries per row of an upper-stored matrix (warp per row);
// an entry below the diagonal marks the matrix unusable here
__global__ void k_up_count(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col, i64* __restrict__ cnt,
                           int* __restrict__ bad) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        int c = 0, below = 0;
        for (i64 k = rp[r] + lane; k < rp[r + 1]; k += 32) {
            c += col[k] > r;
            below |= col[k] < r;
        }
        for (int o = 16; o > 0; o >>= 1) {
            c += __shfl_xor_sync(0xffffffffu, c, o);
            below |= __shfl_xor_sync(0xffffffffu, below, o);
        }
        if (lane == 0) {
            cnt[r] = c;
            if (below) *bad = 1;
        }
    }
}

// offsets column - row (16 bits) and FP32 values of the strictly upper entries,
// which are the tail of each sorted upper row
__global__ void k_up_fill(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                          const double* __restrict__ val, const i64* __restrict__ up_rp, uint16_t* __restrict__ off,
                          float* __restrict__ v32, int* __restrict__ bad) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        const i64 len = up_rp[r + 1] - up_rp[r], src = rp[r + 1] - len;
        int wide = 0;
        for (i64 k = lane; k < len; k += 32) {
            const i64 o = i64(col[src + k]) - r;
            wide |= o > 65535;
            off[up_rp[r] + k] = uint16_t(o);
            v32[up_rp[r] + k] = float(val[src + k]);
        }
        if (__any_sync(0xffffffffu, wide) && lane == 0) *bad = 1;
    }
}

// first row of each of `blocks` row ranges with equal entry counts
__global__ void k_up_partition(i64 n, const i64* __restrict__ up_rp, int blocks, int32_t* __restrict__ part) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > blocks) return;
    if (c == blocks) { part[c] = int32_t(n); return; }
    const i64 target = i64(double(up_rp[n]) * c / blocks);
    i64 lo = 0, hi = n;   // first row r with up_rp[r] >= target
    while (lo < hi) {
        const i64 mid = (lo + hi) / 2;
        if (up_rp[mid] < target) lo = mid + 1; else hi = mid;
    }
    part[c] = int32_t(lo);
}

// columns reached by each range: from its first row to the farthest column of its rows
__global__ void k_up_window(const i64* __restrict__ up_rp, const uint16_t* __restrict__ off,
                            const int32_t* __restrict__ part, int32_t* __restrict__ window, int* __restrict__ wmax) {
    __shared__ int sh[32];
    const int r0 = part[blockIdx.x], r1 = part[blockIdx.x + 1];
    int far = r0 - 1;
    for (int r = r0 + int(threadIdx.x); r < r1; r += blockDim.x) {
        const i64 e = up_rp[r + 1];
        far = max(far, e > up_rp[r] ? r + int(off[e - 1]) : r);
    }
    for (int o = 16; o > 0; o >>= 1) far = max(far, __shfl_xor_sync(0xffffffffu, far, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = far;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < int(blockDim.x >> 5); ++w) far = max(far, sh[w]);
        window[blockIdx.x] = far - r0 + 1;
        atomicMax(wmax, far - r0 + 1);
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

// The FP32 copy in one pass over the FP64 rows (warp per row): float values,
// 16-bit offsets column - row (written clamped; kept only when the widest
// offset fits), the row sums of the FP64 values and the widest offset.
__global__ void k_fp32_copy(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                            const double* __restrict__ val, float* __restrict__ val32, int16_t* __restrict__ col16,
                            float* __restrict__ rowsum, unsigned long long* __restrict__ widest) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    unsigned long long m = 0;
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        double s = 0.0;
        for (i64 k = rp[r] + lane; k < rp[r + 1]; k += 32) {
            const double v = val[k];
            const i64 d = i64(col[k]) - r;
            s += v;
            val32[k] = float(v);
            col16[k] = int16_t(d < -32768 ? -32768 : (d > 32767 ? 32767 : d));
            m = max(m, static_cast<unsigned long long>(d < 0 ? -d : d));
        }
        s = warp_sum(s);
        if (lane == 0) rowsum[r] = float(s);
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m) atomicMax(widest, m);
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

__global__ void k_copy32(i64 n, const float* __restrict__ a, float* __restrict__ b, const double* __restrict__ flags) {
    if (flags && flags[S_DONE] != 0.0) return;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = a[i];
}

// directions stored after k iterations
__device__ __forceinline__ int mx_count(const double* flags) {
    return int(min(i64(flags[S_ITERS]), i64(MX_M)));
}

// d += alpha p_j; r -= alpha q_j (j the current direction slot); r.r.  The last
// block counts the iteration and sets the done flag when |r| <= tol |r_update|
// or the iteration cap is reached; the kernels after it read the new count.
__global__ void __launch_bounds__(MX_THREADS) k_update_dr32(i64 n, float* __restrict__ d, float* __restrict__ r,
                                                            const float* __restrict__ p, const float* __restrict__ q,
                                                            double* __restrict__ part, double* __restrict__ flags,
                                                            unsigned* ticket, double tol2, double max_iterations) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const i64 slot = i64(flags[S_ITERS]) % MX_M;
    p += slot * n;
    q += slot * n;
    const float alpha = float(flags[S_ALPHA]);
    if (!isfinite(alpha)) {   // p.q vanished in FP32 (breakdown): end the cycle, the reliable update restarts it
        if (blockIdx.x == 0 && threadIdx.x == 0) flags[S_DONE] = 1.0;
        return;
    }
    float s = 0.0f;   // a thread's one or two elements in FP32; block and global sums in FP64
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        d[i] += alpha * p[i];
        const float v = r[i] - alpha * q[i];
        r[i] = v;
        s = fmaf(v, v, s);
    }
    double v[1] = {double(s)};
    if (mx_reduce_last<1>(v, part + P_RR * RED_BLOCKS, ticket, sh) && threadIdx.x == 0) {
        const double it = flags[S_ITERS] + 1.0;
        flags[S_ITERS] = it;
        if (v[0] <= tol2 * flags[S_BB] || it >= max_iterations) flags[S_DONE] = 1.0;
    }
}

// z.q_i for the stored directions; the last block forms beta_i = -(z.q_i) / (p_i.q_i)
__global__ void __launch_bounds__(MX_THREADS) k_dotm32(i64 n, const float* __restrict__ z, const float* __restrict__ qring,
                                                       double* __restrict__ part, double* __restrict__ flags,
                                                       unsigned* ticket) {
    __shared__ double sh[33 * MX_M];
    if (flags[S_DONE] != 0.0) return;
    const int count = mx_count(flags);
    float zq32[MX_M] = {};
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const float zi = z[i];
#pragma unroll
        for (int s = 0; s < MX_M; ++s)
            if (s < count) zq32[s] = fmaf(zi, qring[i64(s) * n + i], zq32[s]);
    }
    double zq[MX_M];
#pragma unroll
    for (int s = 0; s < MX_M; ++s) zq[s] = zq32[s];
    if (mx_reduce_last<MX_M>(zq, part + M_ZQ * RED_BLOCKS, ticket, sh) && threadIdx.x == 0)
        for (int s = 0; s < count; ++s) flags[S_BETA + s] = -zq[s] / flags[S_PQ + s];
}

// p_k = z + sum_i beta_i p_i over the stored directions (A-orthogonal to the
// last MX_M directions), k the iteration count, and p_k.r (the next alpha's
// numerator, stored by the last block)
__global__ void __launch_bounds__(MX_THREADS) k_update_pm32(i64 n, float* __restrict__ pring, const float* __restrict__ z,
                                                            const float* __restrict__ r, double* __restrict__ part,
                                                            double* __restrict__ flags, unsigned* ticket,
                                                            float* __restrict__ qring_clear) {
    __shared__ double sh[40];
    if (flags[S_DONE] != 0.0) return;
    const i64 k = i64(flags[S_ITERS]);
    const int count = mx_count(flags), next = int(k % MX_M);
    float beta[MX_M];
#pragma unroll
    for (int s = 0; s < MX_M; ++s) beta[s] = s < count ? float(flags[S_BETA + s]) : 0.0f;
    float* pn = pring + i64(next) * n;
    // the symmetric SpMV accumulates q_k into its slot: clear it (its old
    // direction was last read by k_dotm32 of this iteration)
    float* qn = qring_clear ? qring_clear + i64(next) * n : nullptr;
    float pr = 0.0f;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        if (qn) qn[i] = 0.0f;
        float v = z[i];
#pragma unroll
        for (int s = 0; s < MX_M; ++s)
            if (s < count) v += beta[s] * pring[i64(s) * n + i];
        pn[i] = v;   // may overwrite the oldest direction: element i was read above
        pr = fmaf(v, r[i], pr);
    }
    double v[1] = {double(pr)};
    if (mx_reduce_last<1>(v, part + P_RZ_A * RED_BLOCKS, ticket, sh) && threadIdx.x == 0) flags[S_PR] = v[0];
}

__global__ void k_widen(i64 n, const float* __restrict__ a, double* __restrict__ b) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) b[i] = a[i];
}

void precondition32(Ctx& ctx, IncompleteCholesky* M, const float* r, float* z, const double* part, const double* flags,
                    double tol2, int sweeps) {
    const i64 n = ctx.mx.n;
    if (!M) {
        NL_LAUNCH(k_copy32, RED_BLOCKS, MX_THREADS, 0, ctx.stream, n, r, z, flags);
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

void launch_spmv32(Ctx& ctx, const Csr& A, const float* x, float* y, double* dot_partial, double* flags, i64 ring,
                   unsigned* ticket) {
    if (A.up_ok) {
        NL_LAUNCH(k_spmv32_up, A.up_blocks, UP_THREADS, size_t(A.up_window_max) * sizeof(float), ctx.stream,
                  A.up_rp.p, A.up_off.p, A.up_val.p, A.rowsum32.p, A.up_part.p, A.up_window.p, x, y, flags, ring);
        if (dot_partial) {
            const unsigned G = unsigned(std::min<i64>(RED_BLOCKS, std::max<i64>(1, (A.rows + MX_THREADS - 1) / MX_THREADS)));
            NL_LAUNCH(k_pq32, G, MX_THREADS, 0, ctx.stream, A.rows, x, y, dot_partial, flags, ticket);
        }
    } else if (A.col16_ok)
        NL_LAUNCH(k_spmv32<int16_t>, SPMV_BLOCKS, MX_THREADS, 0, ctx.stream, A.rows, A.rowptr.p, A.col16.p, A.val32.p,
                  A.rowsum32.p, x, y, dot_partial, flags, ring, ticket);
    else
        NL_LAUNCH(k_spmv32<int32_t>, SPMV_BLOCKS, MX_THREADS, 0, ctx.stream, A.rows, A.rowptr.p, A.col.p, A.val32.p,
                  A.rowsum32.p, x, y, dot_partial, flags, ring, ticket);
}

}  // namespace

void spmv32(Ctx& ctx, const Csr& A, const float* x, float* y) {
    if (A.up_ok) NL_CUDA(cudaMemsetAsync(y, 0, size_t(A.rows) * sizeof(float), ctx.stream));
    launch_spmv32(ctx, A, x, y, nullptr, nullptr, 0, nullptr);
}

void ilt_apply32(Ctx& ctx, IncompleteCholesky& ic, const float* r, float* z, int sweeps) {
    if (sweeps <= 0) ilt_exact_layouts(ctx, ic);
    ctx.mx.n = ic.n;
    ctx.mx.r64.reserve(size_t(ic.n)); ctx.mx.q64.reserve(size_t(ic.n));
    precondition32(ctx, &ic, r, z, nullptr, nullptr, 0.0, sweeps);
}

namespace {

// The strictly upper part of `upper` in FP32 with 16-bit offsets and the row
// ranges of the symmetric SpMV's CTAs (one per SM); false (full rows are used)
// when an offset exceeds 16 bits or a window exceeds one CTA's shared memory.
bool upper_to_f32(Ctx& ctx, Csr& A, const Csr& upper) {
    const i64 n = upper.rows;
    if (n <= 0 || n != A.rows || n >= (i64(1) << 31)) return false;
    int dev = 0, sms = 0, smem_optin = 0, smem_sm = 0;
    NL_CUDA(cudaGetDevice(&dev));
    NL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    NL_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    NL_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    A.up_rp.resize(size_t(n) + 1);
    dbuf<int> flags;   // [0] bad, [1] widest window
    flags.resize(2);
    flags.zero(ctx.stream);
    NL_LAUNCH(k_up_count, RED_BLOCKS, 256, 0, ctx.stream, n, upper.rowptr.p, upper.col.p, A.up_rp.p, flags.p);
    NL_CUDA(cudaMemsetAsync(A.up_rp.p + n, 0, sizeof(i64), ctx.stream));
    i64 total = 0;
    exclusive_scan(ctx, A.up_rp.p, A.up_rp.p, n + 1, &total);
    A.up_nnz = total;
    A.up_off.resize(size_t(std::max<i64>(total, 1)));
    A.up_val.resize(size_t(std::max<i64>(total, 1)));
    NL_LAUNCH(k_up_fill, RED_BLOCKS, 256, 0, ctx.stream, n, upper.rowptr.p, upper.col.p, upper.val.p, A.up_rp.p,
              A.up_off.p, A.up_val.p, flags.p);
    const int blocks = sms;
    A.up_part.resize(size_t(blocks) + 1);
    A.up_window.resize(size_t(blocks));
    NL_LAUNCH(k_up_partition, grid_for(blocks + 1, 256), 256, 0, ctx.stream, n, A.up_rp.p, blocks, A.up_part.p);
    NL_LAUNCH(k_up_window, blocks, 256, 0, ctx.stream, A.up_rp.p, A.up_off.p, A.up_part.p, A.up_window.p, flags.p + 1);
    int h[2] = {0, 0};
    flags.download(h, 2, ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    const size_t bytes = size_t(std::max(h[1], 1)) * sizeof(float);
    if (h[0] || bytes + 2048 > size_t(std::min(smem_optin, smem_sm))) return false;
    NL_CUDA(cudaFuncSetAttribute(k_spmv32_up, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
    A.up_blocks = blocks;
    A.up_window_max = std::max(h[1], 1);
    return true;
}

}  // namespace

// FP64 row sums of the solver matrix in FP32, and FP32 values: the strictly
// upper part of `upper` for the symmetric SpMV when it applies, else the full
// rows with 16-bit column offsets when the pattern's bandwidth allows
void matrix_to_f32(Ctx& ctx, Csr& A, const Csr* upper) {
    A.rowsum32.resize(size_t(A.rows));
    A.up_ok = upper && upper_to_f32(ctx, A, *upper);
    if (A.up_ok) {
        NL_LAUNCH(k_rowsum, grid_for(A.rows, 256), 256, 0, ctx.stream, A.rows, A.rowptr.p, A.val.p, A.rowsum32.p);
        // the full-row FP32 copy is not needed (and not kept up to date)
        A.val32.release();
        A.col16.release();
        A.col16_ok = false;
        return;
    }
    A.up_rp.release(); A.up_off.release(); A.up_val.release();
    A.val32.resize(size_t(A.nnz));
    A.col16.resize(size_t(A.nnz));
    dbuf<unsigned long long> widest;
    widest.resize(1);
    widest.zero(ctx.stream);
    NL_LAUNCH(k_fp32_copy, grid_for(A.rows * 32, 256, 152 * 64), 256, 0, ctx.stream, A.rows, A.rowptr.p, A.col.p,
              A.val.p, A.val32.p, A.col16.p, A.rowsum32.p, widest.p);
    unsigned long long w = 0;
    widest.download(&w, 1, ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    A.col16_ok = w <= 32767;
    if (!A.col16_ok) A.col16.release();
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
                     i64 max_iterations, double update_factor, bool x_is_initial_guess, bool learned, int sweeps,
                     bool coarse) {
    NL_REQUIRE(!coarse || ctx.co.ready, NLGPU_ERR_STATE, "the coarse correction is not built");
    if (M && sweeps <= 0) ilt_exact_layouts(ctx, *M);   // exact FP32 sweeps (before any capture)
    NL_REQUIRE(A.up_ok || A.val32.n == size_t(A.nnz), NLGPU_ERR_STATE, "the FP32 copy of the matrix is missing");
    NL_REQUIRE(!learned || (M && ctx.mp.ready && ctx.mp.n == A.rows), NLGPU_ERR_STATE,
               "the learned correction needs ILLT and a prepared network");
    const i64 n = A.rows;
    PhaseTimer timer(ctx.stream, "mixed_solve");
    MixedWork& w = ctx.mx;
    w.n = n;
    w.r64.reserve(size_t(n)); w.q64.reserve(size_t(n));
    w.r.reserve(size_t(n)); w.z.reserve(size_t(n)); w.d.reserve(size_t(n));
    w.p.reserve(size_t(MX_M) * size_t(n)); w.q.reserve(size_t(MX_M) * size_t(n));   // direction rings
    w.partial.reserve(size_t(M_SLOTS) * RED_BLOCKS);
    w.outer.reserve(size_t(2) * RED_BLOCKS + 8);
    w.flags.reserve(S_MIXED_COUNT);
    w.ticket.reserve(1);
    w.ticket.zero(ctx.stream);
    double* part = w.partial.p;
    double* flags = w.flags.p;
    unsigned* ticket = w.ticket.p;
    double* outer_part = w.outer.p;
    double* outer_sc = w.outer.p + 2 * RED_BLOCKS;   // [0] |b|^2, [1] |r|^2, [2] s0^2
    // vector kernels: one element per thread up to RED_BLOCKS blocks (a small
    // system runs fewer blocks and fewer partials); partial entries of blocks
    // that do not run stay zero, so every consumer may sum all RED_BLOCKS
    const unsigned G = unsigned(std::min<i64>(RED_BLOCKS, std::max<i64>(1, (n + MX_THREADS - 1) / MX_THREADS)));
    NL_CUDA(cudaMemsetAsync(part, 0, size_t(M_SLOTS) * RED_BLOCKS * sizeof(double), ctx.stream));
    NL_CUDA(cudaMemsetAsync(outer_part, 0, size_t(2) * RED_BLOCKS * sizeof(double), ctx.stream));
    if (!x_is_initial_guess) NL_CUDA(cudaMemsetAsync(x, 0, size_t(n) * sizeof(double), ctx.stream));
    // the symmetric SpMV adds into q's ring slot: slot 0 starts at zero, the
    // later slots are cleared by the kernel that forms their direction
    float* qclear = A.up_ok ? w.q.p : nullptr;
    if (qclear) NL_CUDA(cudaMemsetAsync(w.q.p, 0, size_t(n) * sizeof(float), ctx.stream));
    const double eta2 = update_factor * update_factor;
    CgResult res;
    auto precondition = [&](const double* pt, const double* fl, double t2) {
        if (coarse) {   // z = M^-1 (r - A Q r) + Q r
            coarse_before(ctx, w.r.p, fl);
            precondition32(ctx, M, ctx.co.w.p, w.z.p, pt, fl, t2, sweeps);
            coarse_after(ctx, w.z.p, fl);
        } else {
            precondition32(ctx, M, w.r.p, w.z.p, pt, fl, t2, sweeps);
        }
        if (learned) mpnn_apply(ctx, w.r.p, w.z.p, w.z.p, false);
    };
    // |b|^2 and the first residual
    NL_LAUNCH(k_dot_f64, G, MX_THREADS, 0, ctx.stream, n, b, b, outer_part);
    NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, outer_part, outer_sc);
    bool x_zero = !x_is_initial_guess;   // A 0 = 0: the first residual needs no product
    auto true_residual = [&](double* hs) {
        if (x_zero) NL_CUDA(cudaMemsetAsync(w.q64.p, 0, size_t(n) * sizeof(double), ctx.stream));
        else spmv_full(ctx, A, x, w.q64.p);
        x_zero = false;
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
    // r32 = r / s0, d = 0, p_0 = z = P(r) in ring slot 0, p_0.r for the first alpha
    NL_LAUNCH(k_scale_to_f32, G, MX_THREADS, 0, ctx.stream, n, w.r64.p, outer_sc + 2, w.r.p, w.d.p);
    NL_CUDA(cudaMemsetAsync(flags, 0, 8 * sizeof(double), ctx.stream));
    NL_LAUNCH(k_dot32, G, MX_THREADS, 0, ctx.stream, n, w.r.p, w.r.p, part + P_RR * RED_BLOCKS);
    NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, part + P_RR * RED_BLOCKS, flags + S_BB);
    precondition(nullptr, nullptr, 0.0);
    NL_CUDA(cudaMemcpyAsync(w.p.p, w.z.p, size_t(n) * sizeof(float), cudaMemcpyDeviceToDevice, ctx.stream));
    NL_LAUNCH(k_dot32, G, MX_THREADS, 0, ctx.stream, n, w.r.p, w.z.p, part + P_RZ_B * RED_BLOCKS);
    NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, part + P_RZ_B * RED_BLOCKS, flags + S_PR);
    const double cap = double(std::min<i64>(max_iterations, i64(1) << 40));
    double last_rr = hs[1];
    int stalled = 0;
    i64 k = 0;
    i64 iters_at_update = 0;
    // one iteration k (k read on the device): q_j = A p_j (j = k mod MX_M) and
    // alpha; d, r, the count and the stop test; z = P(r); the betas; p_k+1 and
    // its alpha numerator.  Each reducing kernel's last block forms the scalars.
    auto iteration = [&] {
        launch_spmv32(ctx, A, w.p.p, w.q.p, part + M_PQ * RED_BLOCKS, flags, n, ticket);
        NL_LAUNCH(k_update_dr32, G, MX_THREADS, 0, ctx.stream, n, w.d.p, w.r.p, w.p.p, w.q.p, part, flags, ticket,
                  eta2, cap);
        precondition(part, flags, eta2);
        NL_LAUNCH(k_dotm32, G, MX_THREADS, 0, ctx.stream, n, w.z.p, w.q.p, part, flags, ticket);
        NL_LAUNCH(k_update_pm32, G, MX_THREADS, 0, ctx.stream, n, w.p.p, w.z.p, w.r.p, part, flags, ticket, qclear);
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
            {
                CountCaptured counted;
                NL_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
                for (int it = 0; it < MX_ITERS; ++it) iteration();
                NL_CUDA(cudaStreamEndCapture(ctx.stream, &g));
                w.chunk_kernels = int(counted.kernels);   // counted when the graph is launched
            }
            timer.mark("first chunk, capture");
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
            timer.mark(captured ? "graph chunk" : "eager chunk");
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
        timer.mark("reliable update");
        ++res.outer_iterations;
        res.residual = std::sqrt(hs[1] / hs[0]);
        if (hs[1] <= tolerance * tolerance * hs[0]) { res.converged = true; break; }
        if (res.iterations >= max_iterations || !std::isfinite(hs[1])) break;
        // five updates in a row without progress: the recurrence has stalled
        stalled = hs[1] >= last_rr ? stalled + 1 : 0;
        if (stalled >= 5) break;
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
                      part + P_RZ_B * RED_BLOCKS);
            NL_LAUNCH(k_sum_to, 1, MX_THREADS, 0, ctx.stream, part + P_RZ_B * RED_BLOCKS, flags + S_PR);
        } else {
            // the stop skipped p_k: z = P(r), p_k = z - sum_i (z.q_i / p_i.q_i) p_i as at
            // the end of iteration k - 1 (the kernels read k from the count)
            precondition(nullptr, nullptr, 0.0);
            NL_LAUNCH(k_dotm32, G, MX_THREADS, 0, ctx.stream, n, w.z.p, w.q.p, part, flags, ticket);
            NL_LAUNCH(k_update_pm32, G, MX_THREADS, 0, ctx.stream, n, w.p.p, w.z.p, w.r.p, part, flags, ticket, qclear);
        }
    }
    timer.mark("remaining iterations");
    return res;
}

}  // namespace nlgpu
