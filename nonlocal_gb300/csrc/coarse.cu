// Coarse-space correction for the mixed-precision solve (deflation on top of
// the FP32 ILLT application).  Not part of the reference, whose
// preconditioner is ILLT alone (eigen_preconditioner.hpp:57): an optional
// preconditioner component of the flexible CG, for comparison with and on top
// of the reference's method.
//
//   aggregates  nodes grouped by the cells of a uniform grid over the inner
//               nodes' bounding box (about `target` non-empty cells); rows
//               that are not inner (Dirichlet) belong to none.  P is the
//               n x nc indicator matrix of the aggregates; each aggregate's
//               node list is kept sorted (deterministic restriction).
//   AP          per row the sums of the row's entries by column aggregate,
//               one entry per aggregate in increasing order (float-float
//               segmented warp sums over the row's sorted columns), from the
//               FP32 rows the inner iteration applies, the own aggregate's
//               entry completing the FP64 row sum
//   A_c = P^T A P  from AP, a row per aggregate summed in shared memory, FP64
//   A_c^-1      blocked Gauss-Jordan in FP64 (A_c is SPD, no pivoting), 32
//               pivots per panel, three launches per panel ping-ponging two
//               copies; stored in FP32 for the solve
//   apply       Q r = P A_c^-1 P^T r, then z = M^-1 (r - A Q r) + Q r with
//               A Q r = AP (A_c^-1 P^T r)  (A-DEF1 of Tang, Nabben, Vuik and
//               Erlangga 2009); flexible CG absorbs its non-symmetry.
// Per application: a warp-per-aggregate restriction, a dense FP32 matvec of
// nc x nc, one pass over AP and r before the ILLT application and one add
// after it.
#include "common.cuh"
#include "ff.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace nlgpu {

namespace {

constexpr int CO_THREADS = 256;
constexpr int CO_SORT_MAX = 4096;   // aggregate sizes sorted in shared memory

// bounding box of the inner nodes: atomic min / max on an order-preserving
// integer image of the coordinates
__device__ __forceinline__ unsigned long long order_key(double v) {
    const unsigned long long b = __double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double from_key(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
#ifdef __CUDA_ARCH__
    return __longlong_as_double(static_cast<long long>(b));
#else
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
#endif
}

__global__ void k_bbox(i64 n, const double* __restrict__ xy, const uint8_t* __restrict__ is_inner,
                       unsigned long long* __restrict__ box) {
    unsigned long long lo0 = ~0ull, lo1 = ~0ull, hi0 = 0ull, hi1 = 0ull;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        if (is_inner && !is_inner[i]) continue;
        const unsigned long long kx = order_key(xy[2 * i]), ky = order_key(xy[2 * i + 1]);
        lo0 = min(lo0, kx); hi0 = max(hi0, kx); lo1 = min(lo1, ky); hi1 = max(hi1, ky);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo0 = min(lo0, __shfl_xor_sync(0xffffffffu, lo0, o)); hi0 = max(hi0, __shfl_xor_sync(0xffffffffu, hi0, o));
        lo1 = min(lo1, __shfl_xor_sync(0xffffffffu, lo1, o)); hi1 = max(hi1, __shfl_xor_sync(0xffffffffu, hi1, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(box + 0, lo0); atomicMin(box + 1, lo1);
        atomicMax(box + 2, hi0); atomicMax(box + 3, hi1);
    }
}

// aggregate cell of every node (-1 for rows that are not inner)
__global__ void k_cell_of_node(i64 n, const double* __restrict__ xy, const uint8_t* __restrict__ is_inner, double x0,
                               double y0, double inv_hx, double inv_hy, int cx, int cy, int32_t* __restrict__ cell,
                               i64* __restrict__ used) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        if (is_inner && !is_inner[i]) { cell[i] = -1; continue; }
        const int a = min(cx - 1, max(0, int((xy[2 * i] - x0) * inv_hx)));
        const int b = min(cy - 1, max(0, int((xy[2 * i + 1] - y0) * inv_hy)));
        const int c = b * cx + a;
        cell[i] = c;
        used[c] = 1;
    }
}

// cell -> aggregate number (exclusive scan of the used flags), node counts
__global__ void k_renumber_cells(i64 n, const i64* __restrict__ cell_index, int32_t* __restrict__ agg,
                                 unsigned long long* __restrict__ count) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        if (agg[i] >= 0) {
            const int32_t a = int32_t(cell_index[agg[i]]);
            agg[i] = a;
            atomicAdd(count + a, 1ull);
        }
}

// node lists of the aggregates (positions by atomics, sorted afterwards)
__global__ void k_agg_scatter(i64 n, const int32_t* __restrict__ agg, const i64* __restrict__ ptr,
                              unsigned* __restrict__ fill, int32_t* __restrict__ nodes) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        if (agg[i] >= 0) nodes[ptr[agg[i]] + atomicAdd(fill + agg[i], 1u)] = int32_t(i);
}

// sorts each aggregate's node list (CTA per aggregate, bitonic in shared memory)
__global__ void __launch_bounds__(CO_THREADS) k_agg_sort(i64 nc, const i64* __restrict__ ptr, int32_t* __restrict__ nodes) {
    __shared__ int32_t s[CO_SORT_MAX];
    for (i64 a = blockIdx.x; a < nc; a += gridDim.x) {
        const i64 b = ptr[a];
        const int len = int(ptr[a + 1] - b);
        if (len > CO_SORT_MAX) continue;   // left in scatter order (still a valid list)
        int m = 1;
        while (m < len) m <<= 1;
        for (int t = threadIdx.x; t < m; t += blockDim.x) s[t] = t < len ? nodes[b + t] : 0x7fffffff;
        __syncthreads();
        for (int k = 2; k <= m; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = threadIdx.x; t < m; t += blockDim.x) {
                    const int u = t ^ j;
                    if (u > t) {
                        const bool up = (t & k) == 0;
                        const int32_t x = s[t], y = s[u];
                        if ((x > y) == up) { s[t] = y; s[u] = x; }
                    }
                }
                __syncthreads();
            }
        for (int t = threadIdx.x; t < len; t += blockDim.x) nodes[b + t] = s[t];
        __syncthreads();
    }
}

// AP = A P: entry (r, J) = sum of row r's entries over the columns in
// aggregate J (Dirichlet columns belong to none).  Warp per row.  A first
// sweep over the row marks its aggregates in the warp's shared-memory bitmap
// (nc bits) and counts the runs of equal aggregates in column order; a row
// with at most AP_MAXD distinct aggregates gets one entry per aggregate, in
// increasing order, each the sum of its runs in column order (a run's sum by a
// segmented warp scan, the runs added one after another by lane 0, so the
// result does not depend on the schedule); a row with more keeps one entry
// per run.  The count pass (FILL = false) makes the same choice.  The sums run
// in float-float on the FP32 pipes (each FP64 entry split by integer
// operations): a warp-wide FP64 add occupies GB300's FP64 pipe for 16 cycles,
// and five of them per entry made this kernel FP64-bound.
constexpr int AP_WARPS = 8;
constexpr int AP_MAXD = 128;

inline size_t ap_smem_bytes(i64 nc) {
    const size_t words = size_t((nc + 31) / 32);
    return size_t(AP_WARPS) * (2 * words * sizeof(uint32_t) + AP_MAXD * sizeof(double));
}

// The matrix rows AP reads: the FP32 copy of the mixed-precision solve (float
// values, 16-bit column offsets, FP64 row sums), so that AP is that of the
// difference-form operator the FP32 iteration applies (its entries sum to the
// row sum: the own aggregate takes s_r minus the others), or the FP64 rows
// (values split into float-float by integer operations).
struct ApInput {
    const i64* rp;
    const int32_t* col;     // FP64 form
    const double* val;
    const int16_t* off;     // FP32 form: column - row
    const float* val32;
    const float* rowsum;
};

template<bool F32>
__device__ __forceinline__ int32_t ap_col_of(const ApInput& in, i64 r, i64 k) {
    if constexpr (F32) return int32_t(r + in.off[k]);
    else return in.col[k];
}

template<bool F32>
__device__ __forceinline__ ff ap_val_of(const ApInput& in, i64 k) {
    if constexpr (F32) return ff{in.val32[k], 0.0f};
    else return ff_split(in.val[k]);
}

template<bool FILL, bool F32>
__global__ void __launch_bounds__(AP_WARPS * 32) k_ap(i64 n, int nc, ApInput in, const int32_t* __restrict__ agg,
                                                      i64* __restrict__ cnt, const i64* __restrict__ ap_rp,
                                                      int32_t* __restrict__ ap_col, double* __restrict__ ap_val) {
    extern __shared__ __align__(8) unsigned char ap_smem[];
    const unsigned full = 0xffffffffu;
    const int words = (nc + 31) >> 5;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    ff* slot = reinterpret_cast<ff*>(ap_smem) + wid * AP_MAXD;
    uint32_t* bm = reinterpret_cast<uint32_t*>(ap_smem + AP_WARPS * AP_MAXD * sizeof(double)) + wid * 2 * words;
    int* pre = reinterpret_cast<int*>(bm + words);
    const i64 warps = i64(gridDim.x) * AP_WARPS;
    for (i64 r = i64(blockIdx.x) * AP_WARPS + wid; r < n; r += warps) {
        const int32_t own = agg[r];
        if (own < 0) {
            if (!FILL && lane == 0) cnt[r] = 0;
            continue;
        }
        const i64 rb = in.rp[r], re = in.rp[r + 1];
        for (int w = lane; w < words; w += 32) bm[w] = 0u;
        __syncwarp();
        int runs = 0;
        for (i64 k0 = rb; k0 < re; k0 += 32) {
            const i64 k = k0 + lane;
            const int32_t J = k < re ? agg[ap_col_of<F32>(in, r, k)] : -1;
            const int32_t Jn = __shfl_down_sync(full, J, 1);
            const bool end = J >= 0 && (lane == 31 || Jn != J);
            // one mark per run: neighbouring lanes mostly share an aggregate,
            // and their atomics on one word would serialise
            if (end) atomicOr(&bm[J >> 5], 1u << (J & 31));
            runs += __popc(__ballot_sync(full, end));
        }
        __syncwarp();
        int D = 0;   // distinct aggregates; pre[w] = set bits before word w
        for (int w0 = 0; w0 < words; w0 += 32) {
            const int w = w0 + lane;
            const int c = w < words ? __popc(bm[w]) : 0;
            int incl = c;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(full, incl, o);
                if (lane >= o) incl += t;
            }
            if (w < words) pre[w] = D + incl - c;
            D += __shfl_sync(full, incl, 31);
        }
        const bool merge = D <= AP_MAXD;
        if constexpr (!FILL) {
            if (lane == 0) cnt[r] = merge ? D : runs;
        } else {
            for (int t = lane; t < AP_MAXD; t += 32) slot[t] = ff{0.0f, 0.0f};
            __syncwarp();
            i64 out = ap_rp[r], own_pos = -1;
            ff lane_total{0.0f, 0.0f};   // this lane's entries (FP32 form: the row-sum correction)
            for (i64 k0 = rb; k0 < re; k0 += 32) {
                const i64 k = k0 + lane;
                const bool valid = k < re;
                const int32_t J = valid ? agg[ap_col_of<F32>(in, r, k)] : -1;
                ff v = J >= 0 ? ap_val_of<F32>(in, k) : ff{0.0f, 0.0f};
                if constexpr (F32) lane_total = ff_add(lane_total, v);
                const int32_t Jp = __shfl_up_sync(full, J, 1);
                bool head = lane == 0 || Jp != J;
                for (int o = 1; o < 32; o <<= 1) {
                    const ff vu{__shfl_up_sync(full, v.h, o), __shfl_up_sync(full, v.l, o)};
                    const bool hu = __shfl_up_sync(full, head, o);
                    if (lane >= o) {
                        if (!head) v = ff_add(v, vu);
                        head = head || hu;
                    }
                }
                const int32_t Jn = __shfl_down_sync(full, J, 1);
                const bool end = J >= 0 && (lane == 31 || Jn != J);
                const unsigned ends = __ballot_sync(full, end);
                if (merge) {
                    for (unsigned m = ends; m; m &= m - 1) {
                        const int src = __ffs(m) - 1;
                        const ff vs{__shfl_sync(full, v.h, src), __shfl_sync(full, v.l, src)};
                        const int32_t Js = __shfl_sync(full, J, src);
                        if (lane == 0) {
                            ff& t = slot[pre[Js >> 5] + __popc(bm[Js >> 5] & ((1u << (Js & 31)) - 1u))];
                            t = ff_add(t, vs);
                        }
                    }
                } else {
                    if (end) {
                        const i64 pos = out + __popc(ends & ((1u << lane) - 1u));
                        ap_col[pos] = J;
                        ap_val[pos] = ff_to(v);
                    }
                    const unsigned owns = __ballot_sync(full, end && J == own);
                    if (own_pos < 0 && owns) own_pos = out + __popc(ends & ((1u << (__ffs(owns) - 1)) - 1u));
                    out += __popc(ends);
                }
            }
            __syncwarp();
            if constexpr (F32) {   // the own aggregate takes s_r - (everything else)
                for (int o = 16; o > 0; o >>= 1)
                    lane_total = ff_add(lane_total, ff{__shfl_xor_sync(full, lane_total.h, o),
                                                       __shfl_xor_sync(full, lane_total.l, o)});
                if (lane == 0) {
                    const ff d = ff_sub(ff{in.rowsum[r], 0.0f}, lane_total);
                    if (merge) {
                        ff& t = slot[pre[own >> 5] + __popc(bm[own >> 5] & ((1u << (own & 31)) - 1u))];
                        t = ff_add(t, d);
                    } else if (own_pos >= 0) {
                        ap_val[own_pos] += ff_to(d);
                    }
                }
                __syncwarp();
            }
            if (merge)
                for (int w = lane; w < words; w += 32) {
                    int p = pre[w];
                    for (uint32_t m = bm[w]; m; m &= m - 1, ++p) {
                        ap_col[out + p] = w * 32 + __ffs(m) - 1;
                        ap_val[out + p] = ff_to(slot[p]);
                    }
                }
        }
        __syncwarp();
    }
}

// Row I of A_c = sum over the nodes r of aggregate I of AP row r: a CTA per
// aggregate accumulates the row in shared memory (nc doubles), then writes it
// whole.  Dynamic shared memory: nc doubles.
__global__ void __launch_bounds__(CO_THREADS) k_coarse_rows(i64 nc, const i64* __restrict__ ptr,
                                                            const int32_t* __restrict__ nodes,
                                                            const i64* __restrict__ ap_rp,
                                                            const int32_t* __restrict__ ap_col,
                                                            const double* __restrict__ ap_val, double* __restrict__ ac) {
    extern __shared__ double row[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = int(blockDim.x >> 5);
    for (i64 I = blockIdx.x; I < nc; I += gridDim.x) {
        for (i64 j = threadIdx.x; j < nc; j += blockDim.x) row[j] = 0.0;
        __syncthreads();
        for (i64 t = ptr[I] + warp; t < ptr[I + 1]; t += nw) {
            const int32_t r = nodes[t];
            for (i64 k = ap_rp[r] + lane; k < ap_rp[r + 1]; k += 32) atomicAdd(row + ap_col[k], ap_val[k]);
        }
        __syncthreads();
        for (i64 j = threadIdx.x; j < nc; j += blockDim.x) ac[I * nc + j] = row[j];
        __syncthreads();
    }
}

// A_c^-1 by blocked Gauss-Jordan without pivoting (A_c is SPD), in panels of
// GJ_B pivots on a copy padded to a multiple of GJ_B with an identity block
// (blockdiag(A_c, I)^-1 = blockdiag(A_c^-1, I)).  For panel P, with
// D = src[P][P]^-1 and R = D src[P][:], one out-of-place pass writes
//   dst[P][P] = D,   dst[P][j] = R[j],   dst[i][P] = -src[i][P] D,
//   dst[i][j] = src[i][j] - src[i][P] R[j]      (i, j outside P),
// the Gauss-Jordan step of a whole panel: three launches per panel instead
// of one per pivot, the rank-GJ_B update run as 32x32 tiles from shared memory.
constexpr int GJ_B = 32;

__global__ void k_gj_pad(int nc, int ncp, const double* __restrict__ a, double* __restrict__ dst) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < i64(ncp) * ncp; t += i64(gridDim.x) * blockDim.x) {
        const int i = int(t / ncp), j = int(t % ncp);
        dst[t] = (i < nc && j < nc) ? a[i64(i) * nc + j] : (i == j ? 1.0 : 0.0);
    }
}

// D = src[P][P]^-1 by unblocked Gauss-Jordan in shared memory (one CTA, 32x32)
__global__ void __launch_bounds__(GJ_B * GJ_B) k_gj_diag(int ncp, int k0, const double* __restrict__ src,
                                                         double* __restrict__ dinv) {
    __shared__ double d[GJ_B][GJ_B + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    d[ty][tx] = src[i64(k0 + ty) * ncp + k0 + tx];
    __syncthreads();
    for (int k = 0; k < GJ_B; ++k) {
        const double inv = 1.0 / d[k][k];
        const double dik = d[ty][k], dkj = d[k][tx];
        double v;
        if (ty == k) v = tx == k ? inv : dkj * inv;
        else if (tx == k) v = -dik * inv;
        else v = d[ty][tx] - dik * (dkj * inv);
        __syncthreads();
        d[ty][tx] = v;
        __syncthreads();
    }
    dinv[ty * GJ_B + tx] = d[ty][tx];
}

// R = D src[P][:] (GJ_B x ncp), a 32-column tile per CTA
__global__ void __launch_bounds__(GJ_B * GJ_B) k_gj_rows(int ncp, int k0, const double* __restrict__ src,
                                                         const double* __restrict__ dinv, double* __restrict__ R) {
    __shared__ double D[GJ_B][GJ_B + 1], S[GJ_B][GJ_B + 1];
    const int tx = threadIdx.x, ty = threadIdx.y, j = blockIdx.x * GJ_B + tx;
    D[ty][tx] = dinv[ty * GJ_B + tx];
    S[ty][tx] = src[i64(k0 + ty) * ncp + j];
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < GJ_B; ++q) s = fma(D[ty][q], S[q][tx], s);
    R[i64(ty) * ncp + j] = s;
}

// one 32x32 tile of dst per CTA
__global__ void __launch_bounds__(GJ_B * GJ_B) k_gj_update(int ncp, int k0, const double* __restrict__ src,
                                                           const double* __restrict__ dinv,
                                                           const double* __restrict__ R, double* __restrict__ dst) {
    __shared__ double C[GJ_B][GJ_B + 1], T[GJ_B][GJ_B + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.y * GJ_B, j0 = blockIdx.x * GJ_B, i = i0 + ty, j = j0 + tx;
    const bool pj = j0 == k0;
    if (i0 == k0) {   // the panel's rows (uniform over the CTA)
        dst[i64(i) * ncp + j] = pj ? dinv[ty * GJ_B + tx] : R[i64(ty) * ncp + j];
        return;
    }
    C[ty][tx] = src[i64(i) * ncp + k0 + tx];
    T[ty][tx] = pj ? dinv[ty * GJ_B + tx] : R[i64(ty) * ncp + j];
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < GJ_B; ++q) s = fma(C[ty][q], T[q][tx], s);
    dst[i64(i) * ncp + j] = pj ? -s : src[i64(i) * ncp + j] - s;
}

// the nc x nc part of the padded inverse as FP32
__global__ void k_inverse_to_f32(int nc, int ncp, const double* __restrict__ a, float* __restrict__ b,
                                 int* __restrict__ bad) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < i64(nc) * nc; t += i64(gridDim.x) * blockDim.x) {
        const double v = a[(t / nc) * ncp + t % nc];
        if (!isfinite(v)) *bad = 1;
        b[t] = float(v);
    }
}

__global__ void k_to_f32_co(i64 n, const double* __restrict__ a, float* __restrict__ b, int* __restrict__ bad) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        const double v = a[i];
        if (!isfinite(v)) *bad = 1;
        b[i] = float(v);
    }
}

// ---- application (FP32; every kernel returns at once once the solve is done)
// rc[J] = sum of r over aggregate J's nodes (warp per aggregate, fixed order)
__global__ void k_restrict(i64 nc, const i64* __restrict__ ptr, const int32_t* __restrict__ nodes,
                           const float* __restrict__ r, float* __restrict__ rc, const double* __restrict__ flags) {
    if (flags && flags[S_DONE] != 0.0) return;
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 a = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; a < nc; a += warps) {
        float s = 0.0f;
        for (i64 k = ptr[a] + lane; k < ptr[a + 1]; k += 32) s += r[nodes[k]];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) rc[a] = s;
    }
}

// ec = A_c^-1 rc (warp per row)
__global__ void k_coarse_solve(i64 nc, const float* __restrict__ ainv, const float* __restrict__ rc,
                               float* __restrict__ ec, const double* __restrict__ flags) {
    if (flags && flags[S_DONE] != 0.0) return;
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 i = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; i < nc; i += warps) {
        float s = 0.0f;
        for (i64 j = lane; j < nc; j += 32) s = fmaf(ainv[i * nc + j], rc[j], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) ec[i] = s;
    }
}

// w = r - AP ec (the residual left after the coarse correction), y = P ec (warp per row)
__global__ void k_deflate(i64 n, const i64* __restrict__ ap_rp, const int32_t* __restrict__ ap_col,
                          const float* __restrict__ ap_val, const int32_t* __restrict__ agg,
                          const float* __restrict__ ec, const float* __restrict__ r, float* __restrict__ w,
                          float* __restrict__ y, const double* __restrict__ flags) {
    if (flags && flags[S_DONE] != 0.0) return;
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 i = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; i < n; i += warps) {
        float s = 0.0f;
        for (i64 k = ap_rp[i] + lane; k < ap_rp[i + 1]; k += 32) s = fmaf(ap_val[k], ec[ap_col[k]], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            w[i] = r[i] - s;
            y[i] = agg[i] >= 0 ? ec[agg[i]] : 0.0f;
        }
    }
}

__global__ void k_add_coarse(i64 n, const float* __restrict__ y, float* __restrict__ z, const double* __restrict__ flags) {
    if (flags && flags[S_DONE] != 0.0) return;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) z[i] += y[i];
}

}  // namespace

void coarse_build(Ctx& ctx, const Csr& A, int target, double aspect) {
    Coarse& co = ctx.co;
    const i64 n = A.rows;
    NL_REQUIRE(n == ctx.n_nodes && ctx.is_inner.n == size_t(n), NLGPU_ERR_STATE,
               "the coarse correction needs the mesh's nodes and boundary flags");
    NL_REQUIRE(target >= 4 && target <= 8192, NLGPU_ERR_ARG, "coarse aggregates: 4 .. 8192");
    NL_REQUIRE(ctx.nodes.n >= size_t(2 * n), NLGPU_ERR_STATE, "no node coordinates");
    PhaseTimer timer(ctx.stream, "coarse_build");
    co.ready = false;
    // ---- aggregates: cells of a uniform grid over the inner nodes' bounding box
    dbuf<unsigned long long> box;
    box.resize(4);
    const unsigned long long init[4] = {~0ull, ~0ull, 0ull, 0ull};
    NL_CUDA(cudaMemcpyAsync(box.p, init, sizeof init, cudaMemcpyHostToDevice, ctx.stream));
    NL_LAUNCH(k_bbox, grid_for(n, CO_THREADS, 152 * 4), CO_THREADS, 0, ctx.stream, n, ctx.nodes.p, ctx.is_inner.p, box.p);
    unsigned long long hb[4];
    box.download(hb, 4, ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    if (hb[0] == ~0ull) return;   // no inner node
    const double x0 = from_key(hb[0]), y0 = from_key(hb[1]), x1 = from_key(hb[2]), y1 = from_key(hb[3]);
    const double wx = std::max(x1 - x0, 1e-300), wy = std::max(y1 - y0, 1e-300);
    // cells of area wx wy / target, `aspect` times wider than high (elongated
    // along the stronger conductivity, where the error is smoothest)
    const double a = std::min(std::max(aspect > 0.0 ? aspect : 1.0, 1.0 / 64.0), 64.0);
    const double h = std::max(std::sqrt(wx * wy / double(target)), std::max(wx, wy) / 4096.0);
    const double hx = h * std::sqrt(a), hy = h / std::sqrt(a);
    const int cx = std::max(1, int(std::ceil(wx / hx * (1.0 + 1e-12)))), cy = std::max(1, int(std::ceil(wy / hy * (1.0 + 1e-12))));
    const i64 cells = i64(cx) * cy;
    co.agg.resize(size_t(n));
    dbuf<i64> used;
    used.resize(size_t(cells) + 1);
    used.zero(ctx.stream);
    NL_LAUNCH(k_cell_of_node, grid_for(n, CO_THREADS), CO_THREADS, 0, ctx.stream, n, ctx.nodes.p, ctx.is_inner.p, x0, y0,
              1.0 / hx, 1.0 / hy, cx, cy, co.agg.p, used.p);
    i64 nc = 0;
    exclusive_scan(ctx, used.p, used.p, cells + 1, &nc);
    co.nc = nc;
    // a mesh whose nodes leave most cells empty (strongly graded or elongated)
    // may still give far more aggregates than asked for: no coarse correction
    // (the coarse rows are accumulated in shared memory: at most 24 Ki aggregates)
    if (nc < 1 || nc > std::min<i64>(2 * i64(target) + 64, 24 * 1024)) return;
    dbuf<unsigned long long> count;
    count.resize(size_t(nc) + 1);
    count.zero(ctx.stream);
    NL_LAUNCH(k_renumber_cells, grid_for(n, CO_THREADS), CO_THREADS, 0, ctx.stream, n, used.p, co.agg.p, count.p);
    co.ptr.resize(size_t(nc) + 1);
    exclusive_scan(ctx, reinterpret_cast<const i64*>(count.p), co.ptr.p, nc + 1, nullptr);
    co.nodes.resize(size_t(std::max<i64>(n, 1)));
    dbuf<unsigned> fill;
    fill.resize(size_t(nc));
    fill.zero(ctx.stream);
    NL_LAUNCH(k_agg_scatter, grid_for(n, CO_THREADS), CO_THREADS, 0, ctx.stream, n, co.agg.p, co.ptr.p, fill.p,
              co.nodes.p);
    NL_LAUNCH(k_agg_sort, unsigned(std::min<i64>(nc, 152 * 8)), CO_THREADS, 0, ctx.stream, nc, co.ptr.p, co.nodes.p);
    timer.mark("aggregates");
    // ---- AP (count, scan, fill) and A_c = P^T A P
    dbuf<i64> cnt;
    cnt.resize(size_t(n) + 1);
    NL_CUDA(cudaMemsetAsync(cnt.p + n, 0, sizeof(i64), ctx.stream));
    const unsigned gw = unsigned(std::max<i64>(1, std::min<i64>((n + AP_WARPS - 1) / AP_WARPS, 152 * 8)));
    const size_t ap_smem = ap_smem_bytes(nc);
    // the FP32 rows of the mixed-precision solve when they are there
    const bool f32 = A.col16_ok && A.col16.n == size_t(A.nnz) && A.val32.n == size_t(A.nnz) &&
                     A.rowsum32.n == size_t(A.rows);
    const ApInput in{A.rowptr.p, A.col.p, A.val.p, A.col16.p, A.val32.p, A.rowsum32.p};
    auto launch_ap = [&](bool fill, const i64* rp_out, int32_t* col_out, double* val_out) {
        auto kernel = fill ? (f32 ? k_ap<true, true> : k_ap<true, false>) : (f32 ? k_ap<false, true> : k_ap<false, false>);
        NL_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(ap_smem)));
        NL_LAUNCH(kernel, gw, AP_WARPS * 32, ap_smem, ctx.stream, n, int(nc), in, co.agg.p, cnt.p, rp_out, col_out,
                  val_out);
    };
    launch_ap(false, nullptr, nullptr, nullptr);
    co.ap_rp.resize(size_t(n) + 1);
    i64 nap = 0;
    exclusive_scan(ctx, cnt.p, co.ap_rp.p, n + 1, &nap);
    co.ap_nnz = nap;
    co.ap_col.resize(size_t(std::max<i64>(nap, 1)));
    dbuf<double> ap64;
    ap64.resize(size_t(std::max<i64>(nap, 1)));
    launch_ap(true, co.ap_rp.p, co.ap_col.p, ap64.p);
    co.ap_val.resize(size_t(std::max<i64>(nap, 1)));
    dbuf<int> bad;
    bad.resize(1);
    bad.zero(ctx.stream);
    NL_LAUNCH(k_to_f32_co, grid_for(nap, CO_THREADS), CO_THREADS, 0, ctx.stream, nap, ap64.p, co.ap_val.p, bad.p);
    dbuf<double> m0;
    m0.resize(size_t(nc * nc));
    const size_t row_bytes = size_t(nc) * sizeof(double);
    NL_CUDA(cudaFuncSetAttribute(k_coarse_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, int(row_bytes)));
    NL_LAUNCH(k_coarse_rows, unsigned(std::min<i64>(nc, 152 * 8)), CO_THREADS, row_bytes, ctx.stream, nc, co.ptr.p,
              co.nodes.p, co.ap_rp.p, co.ap_col.p, ap64.p, m0.p);
    timer.mark("AP and A_c");
    // ---- A_c^-1 by blocked Gauss-Jordan (ping-pong), then FP32
    const int ncp = int((nc + GJ_B - 1) / GJ_B * GJ_B);
    dbuf<double> p0, p1, dinv, R;
    p0.resize(size_t(ncp) * ncp);
    p1.resize(size_t(ncp) * ncp);
    dinv.resize(size_t(GJ_B) * GJ_B);
    R.resize(size_t(GJ_B) * ncp);
    NL_LAUNCH(k_gj_pad, grid_for(i64(ncp) * ncp, CO_THREADS), CO_THREADS, 0, ctx.stream, int(nc), ncp, m0.p, p0.p);
    double* src = p0.p;
    double* dst = p1.p;
    const dim3 tb(GJ_B, GJ_B), gr(unsigned(ncp / GJ_B)), gt(unsigned(ncp / GJ_B), unsigned(ncp / GJ_B));
    for (int k0 = 0; k0 < ncp; k0 += GJ_B) {
        NL_LAUNCH(k_gj_diag, 1, tb, 0, ctx.stream, ncp, k0, src, dinv.p);
        NL_LAUNCH(k_gj_rows, gr, tb, 0, ctx.stream, ncp, k0, src, dinv.p, R.p);
        NL_LAUNCH(k_gj_update, gt, tb, 0, ctx.stream, ncp, k0, src, dinv.p, R.p, dst);
        std::swap(src, dst);
    }
    co.ainv.resize(size_t(nc * nc));
    NL_LAUNCH(k_inverse_to_f32, grid_for(nc * nc, CO_THREADS), CO_THREADS, 0, ctx.stream, int(nc), ncp, src, co.ainv.p,
              bad.p);
    int hbad = 0;
    NL_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof hbad, cudaMemcpyDeviceToHost, ctx.stream));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    timer.mark("coarse inverse");
    NL_REQUIRE(!hbad, NLGPU_ERR_NUMERICAL, "the coarse matrix is singular or its inverse overflowed");
    co.rc.resize(size_t(nc));
    co.ec.resize(size_t(nc));
    co.w.resize(size_t(n));
    co.y.resize(size_t(n));
    co.ready = true;
}

void coarse_before(Ctx& ctx, const float* r, const double* flags) {
    Coarse& co = ctx.co;
    const i64 n = ctx.n_nodes;
    NL_LAUNCH(k_restrict, grid_for(co.nc * 32, CO_THREADS, 152 * 16), CO_THREADS, 0, ctx.stream, co.nc, co.ptr.p,
              co.nodes.p, r, co.rc.p, flags);
    NL_LAUNCH(k_coarse_solve, grid_for(co.nc * 32, CO_THREADS, 152 * 16), CO_THREADS, 0, ctx.stream, co.nc, co.ainv.p,
              co.rc.p, co.ec.p, flags);
    NL_LAUNCH(k_deflate, grid_for(n * 32, CO_THREADS, 152 * 64), CO_THREADS, 0, ctx.stream, n, co.ap_rp.p, co.ap_col.p,
              co.ap_val.p, co.agg.p, co.ec.p, r, co.w.p, co.y.p, flags);
}

void coarse_after(Ctx& ctx, float* z, const double* flags) {
    NL_LAUNCH(k_add_coarse, grid_for(ctx.n_nodes, CO_THREADS), CO_THREADS, 0, ctx.stream, ctx.n_nodes, ctx.co.y.p, z,
              flags);
}

}  // namespace nlgpu
