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
//   AP          per row the sums of the row's entries by column aggregate
//               (segmented warp sums over the row's sorted columns; a row may
//               hold an aggregate more than once, only the sum matters)
//   A_c = P^T A P  from AP, a row per aggregate summed in shared memory, FP64
//   A_c^-1      Gauss-Jordan in FP64 (A_c is SPD, no pivoting), one launch per
//               pivot ping-ponging two copies; stored in FP32 for the solve
//   apply       Q r = P A_c^-1 P^T r, then z = M^-1 (r - A Q r) + Q r with
//               A Q r = AP (A_c^-1 P^T r)  (A-DEF1 of Tang, Nabben, Vuik and
//               Erlangga 2009); flexible CG absorbs its non-symmetry.
// Per application: a warp-per-aggregate restriction, a dense FP32 matvec of
// nc x nc, one pass over AP and r before the ILLT application and one add
// after it.
#include "common.cuh"

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
                               double y0, double inv_h, int cx, int cy, int32_t* __restrict__ cell,
                               i64* __restrict__ used) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        if (is_inner && !is_inner[i]) { cell[i] = -1; continue; }
        const int a = min(cx - 1, max(0, int((xy[2 * i] - x0) * inv_h)));
        const int b = min(cy - 1, max(0, int((xy[2 * i + 1] - y0) * inv_h)));
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

// Segmented sums of one row's entries by column aggregate: lanes hold 32
// consecutive entries; a segment is a run of equal aggregates over
// neighbouring lanes (head flags, segmented inclusive scan), its last lane
// holds the sum.  Count pass (ap_col null): segments per row; fill pass:
// (J, sum) in row order.  Rows outside every aggregate get none.
__global__ void k_ap(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col, const double* __restrict__ val,
                     const int32_t* __restrict__ agg, i64* __restrict__ cnt, const i64* __restrict__ ap_rp,
                     int32_t* __restrict__ ap_col, double* __restrict__ ap_val) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        i64 out = ap_col ? ap_rp[r] : 0, count = 0;
        if (agg[r] >= 0) {
            for (i64 k0 = rp[r]; k0 < rp[r + 1]; k0 += 32) {
                const i64 k = k0 + lane;
                const bool valid = k < rp[r + 1];
                const int32_t J = valid ? agg[col[k]] : -1;   // Dirichlet columns: no aggregate
                double v = J >= 0 ? val[k] : 0.0;
                const int32_t Jp = __shfl_up_sync(0xffffffffu, J, 1);
                bool head = lane == 0 || Jp != J;
                for (int o = 1; o < 32; o <<= 1) {
                    const double vu = __shfl_up_sync(0xffffffffu, v, o);
                    const bool hu = __shfl_up_sync(0xffffffffu, head, o);
                    if (lane >= o) {
                        if (!head) v += vu;
                        head = head || hu;
                    }
                }
                const int32_t Jn = __shfl_down_sync(0xffffffffu, J, 1);
                const bool end = J >= 0 && (lane == 31 || Jn != J);
                const unsigned ends = __ballot_sync(0xffffffffu, end);
                if (ap_col && end) {
                    const i64 pos = out + __popc(ends & ((1u << lane) - 1u));
                    ap_col[pos] = J;
                    ap_val[pos] = v;
                }
                out += __popc(ends);
                count += __popc(ends);
            }
        }
        if (!ap_col && lane == 0) cnt[r] = count;
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

// one Gauss-Jordan step at pivot k, from src into dst (in-place inversion
// without pivoting for an SPD matrix); block (32, 8): a warp covers 32
// columns of one row, so the row's pivot-column entry is a broadcast load
// The pivot's reciprocal comes from pinv[k & 1] (one FP64 division per step,
// not per entry): the thread that writes the next pivot's entry also stores
// its reciprocal in the other slot.
constexpr int GJ_X = 32, GJ_Y = 8;
__global__ void __launch_bounds__(GJ_X * GJ_Y) k_gauss_jordan(int nc, int k, const double* __restrict__ src,
                                                              double* __restrict__ dst, double* __restrict__ pinv) {
    const int j = blockIdx.x * GJ_X + threadIdx.x, i = blockIdx.y * GJ_Y + threadIdx.y;
    if (i >= nc || j >= nc) return;
    const double inv_p = pinv[k & 1];
    const i64 t = i64(i) * nc + j;
    double v;
    if (i == k) v = j == k ? inv_p : src[i64(k) * nc + j] * inv_p;
    else if (j == k) v = -src[i64(i) * nc + k] * inv_p;
    else v = src[t] - src[i64(i) * nc + k] * (src[i64(k) * nc + j] * inv_p);
    dst[t] = v;
    if (i == k + 1 && j == k + 1) pinv[(k + 1) & 1] = 1.0 / v;
}

__global__ void k_first_pivot(const double* __restrict__ a, double* __restrict__ pinv) { pinv[0] = 1.0 / a[0]; }

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

void coarse_build(Ctx& ctx, const Csr& A, int target) {
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
    const double h = std::max(std::sqrt(wx * wy / double(target)), std::max(wx, wy) / 4096.0);
    const int cx = std::max(1, int(std::ceil(wx / h * (1.0 + 1e-12)))), cy = std::max(1, int(std::ceil(wy / h * (1.0 + 1e-12))));
    const i64 cells = i64(cx) * cy;
    co.agg.resize(size_t(n));
    dbuf<i64> used;
    used.resize(size_t(cells) + 1);
    used.zero(ctx.stream);
    NL_LAUNCH(k_cell_of_node, grid_for(n, CO_THREADS), CO_THREADS, 0, ctx.stream, n, ctx.nodes.p, ctx.is_inner.p, x0, y0,
              1.0 / h, cx, cy, co.agg.p, used.p);
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
    const unsigned gw = grid_for(n * 32, CO_THREADS, 152 * 64);
    NL_LAUNCH(k_ap, gw, CO_THREADS, 0, ctx.stream, n, A.rowptr.p, A.col.p, A.val.p, co.agg.p, cnt.p,
              static_cast<const i64*>(nullptr), static_cast<int32_t*>(nullptr), static_cast<double*>(nullptr));
    co.ap_rp.resize(size_t(n) + 1);
    i64 nap = 0;
    exclusive_scan(ctx, cnt.p, co.ap_rp.p, n + 1, &nap);
    co.ap_nnz = nap;
    co.ap_col.resize(size_t(std::max<i64>(nap, 1)));
    dbuf<double> ap64;
    ap64.resize(size_t(std::max<i64>(nap, 1)));
    NL_LAUNCH(k_ap, gw, CO_THREADS, 0, ctx.stream, n, A.rowptr.p, A.col.p, A.val.p, co.agg.p, cnt.p, co.ap_rp.p,
              co.ap_col.p, ap64.p);
    co.ap_val.resize(size_t(std::max<i64>(nap, 1)));
    dbuf<int> bad;
    bad.resize(1);
    bad.zero(ctx.stream);
    NL_LAUNCH(k_to_f32_co, grid_for(nap, CO_THREADS), CO_THREADS, 0, ctx.stream, nap, ap64.p, co.ap_val.p, bad.p);
    dbuf<double> m0, m1;
    m0.resize(size_t(nc * nc));
    m1.resize(size_t(nc * nc));
    const size_t row_bytes = size_t(nc) * sizeof(double);
    NL_CUDA(cudaFuncSetAttribute(k_coarse_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, int(row_bytes)));
    NL_LAUNCH(k_coarse_rows, unsigned(std::min<i64>(nc, 152 * 8)), CO_THREADS, row_bytes, ctx.stream, nc, co.ptr.p,
              co.nodes.p, co.ap_rp.p, co.ap_col.p, ap64.p, m0.p);
    timer.mark("AP and A_c");
    // ---- A_c^-1 by Gauss-Jordan (ping-pong), then FP32
    double* src = m0.p;
    double* dst = m1.p;
    const dim3 gb(unsigned((nc + GJ_X - 1) / GJ_X), unsigned((nc + GJ_Y - 1) / GJ_Y)), tb(GJ_X, GJ_Y);
    dbuf<double> pinv;
    pinv.resize(2);
    NL_LAUNCH(k_first_pivot, 1, 1, 0, ctx.stream, src, pinv.p);
    for (int k = 0; k < int(nc); ++k) {
        NL_LAUNCH(k_gauss_jordan, gb, tb, 0, ctx.stream, int(nc), k, src, dst, pinv.p);
        std::swap(src, dst);
    }
    co.ainv.resize(size_t(nc * nc));
    NL_LAUNCH(k_to_f32_co, grid_for(nc * nc, CO_THREADS), CO_THREADS, 0, ctx.stream, nc * nc, src, co.ainv.p, bad.p);
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
