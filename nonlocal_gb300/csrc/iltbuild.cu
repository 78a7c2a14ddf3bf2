// Structure of the ILLT factor built on the GPU (the preconditioner of
// eigen_ILLT_preconditioner, eigen_preconditioner.hpp:57, restated as IC(0) on
// the pattern of the local matrix's upper part):
//   * the transpose U^T as lower CSR (diagonal last) with the U position of
//     every entry: column counts, scan, atomic placement, then each row
//     sorted by column (thread per row; rows of a local matrix are short);
//   * the dependency levels of the factorisation (row i waits for the rows j < i
//     of its lower row): Kahn's algorithm in one CTA, one barrier per level --
//     each level's rows are the frontier appended after the previous one, so
//     the rows come out grouped by level with the level offsets;
//   * the sliced-ELL layouts of both triangles for the Jacobi sweeps
//     (slice widths, scan, fill).
// The exact level-scheduled sweeps still build their layouts on the host from
// these arrays, only when a solve uses them.
#include "common.cuh"

#include <algorithm>

namespace nlgpu {

namespace {

constexpr int IB_THREADS = 256;
constexpr int IB_LEVEL_THREADS = 1024;

// every row of the upper pattern starts with its diagonal
__global__ void k_check_diag_first(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                                   int* __restrict__ bad) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x)
        if (rp[r + 1] <= rp[r] || col[rp[r]] != int32_t(r)) *bad = 1;
}

__global__ void k_col_count(i64 nnz, const int32_t* __restrict__ col, unsigned long long* __restrict__ cnt) {
    for (i64 k = blockIdx.x * i64(blockDim.x) + threadIdx.x; k < nnz; k += i64(gridDim.x) * blockDim.x)
        atomicAdd(cnt + col[k], 1ull);
}

// entry k of U row r goes to lower row col[k] (any order, sorted below)
__global__ void k_transpose_place(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                                  const i64* __restrict__ lrp, unsigned* __restrict__ cursor, int32_t* __restrict__ lcol,
                                  i64* __restrict__ l_to_u) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x)
        for (i64 k = rp[r]; k < rp[r + 1]; ++k) {
            const int32_t c = col[k];
            const i64 pos = lrp[c] + atomicAdd(cursor + c, 1u);
            lcol[pos] = int32_t(r);
            l_to_u[pos] = k;
        }
}

// each lower row in increasing column order (insertion sort; the diagonal,
// the largest column, ends last)
__global__ void k_sort_rows(i64 n, const i64* __restrict__ lrp, int32_t* __restrict__ lcol, i64* __restrict__ l_to_u) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x) {
        const i64 b = lrp[r], e = lrp[r + 1];
        for (i64 i = b + 1; i < e; ++i) {
            const int32_t c = lcol[i];
            const i64 u = l_to_u[i];
            i64 j = i - 1;
            while (j >= b && lcol[j] > c) { lcol[j + 1] = lcol[j]; l_to_u[j + 1] = l_to_u[j]; --j; }
            lcol[j + 1] = c;
            l_to_u[j + 1] = u;
        }
    }
}

// Kahn's algorithm in one CTA: in-degree of row i = off-diagonal entries of
// its lower row; a finished row releases the rows of its U row.  rows[] holds
// the levels one after another; lev_ptr[L] their starts.  LV_SUB threads share
// a frontier row, so the releases of a whole level (about a hundred rows of a
// dozen entries on an 8-node mesh) go out as one round of independent
// atomics.  Every row is finished once and each level finishes at least one
// row, so the loop ends after at most n levels.  The order of the rows inside
// a level is that of the atomics; nothing downstream depends on it.
constexpr int LV_SUB = 8;
__global__ void __launch_bounds__(IB_LEVEL_THREADS) k_levels(i64 n, const i64* __restrict__ lrp,
                                                             const i64* __restrict__ rp, const int32_t* __restrict__ col,
                                                             int* __restrict__ indeg, int32_t* __restrict__ rows,
                                                             i64* __restrict__ lev_ptr, i64* __restrict__ out) {
    __shared__ int count;
    if (threadIdx.x == 0) count = 0;
    __syncthreads();
    for (i64 i = threadIdx.x; i < n; i += blockDim.x) {
        const int d = int(lrp[i + 1] - lrp[i] - 1);
        indeg[i] = d;
        if (d == 0) rows[atomicAdd(&count, 1)] = int32_t(i);
    }
    __syncthreads();
    i64 s = 0, e = count;
    i64 L = 0;
    if (threadIdx.x == 0) lev_ptr[0] = 0;
    while (e > s) {
        if (threadIdx.x == 0) lev_ptr[L + 1] = e;
        for (i64 t = s * LV_SUB + threadIdx.x; t < e * LV_SUB; t += blockDim.x) {
            const int32_t i = rows[t / LV_SUB];
            const i64 re = rp[i + 1];
            for (i64 k = rp[i] + 1 + t % LV_SUB; k < re; k += LV_SUB) {
                const int32_t c = col[k];
                if (atomicSub(indeg + c, 1) == 1) rows[atomicAdd(&count, 1)] = c;
            }
        }
        __syncthreads();
        s = e;
        e = count;
        ++L;
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = L; out[1] = e; }
}

// Jacobi slab: entry range [first, last) of row r in a CSR; `lower` selects
// the U^T rows (lrp, without the trailing diagonal) or the U rows (rp,
// without the leading diagonal)
struct TriRows {
    const i64* rp;
    bool lower;
    __device__ __forceinline__ i64 first(i64 r) const { return lower ? rp[r] : rp[r] + 1; }
    __device__ __forceinline__ i64 last(i64 r) const { return lower ? rp[r + 1] - 1 : rp[r + 1]; }
};

__global__ void k_slice_width(i64 n, TriRows tr, i64* __restrict__ cnt) {
    const i64 slices = (n + 31) / 32;
    for (i64 sl = blockIdx.x * i64(blockDim.x) + threadIdx.x; sl < slices; sl += i64(gridDim.x) * blockDim.x) {
        i64 w = 0;
        for (i64 r = sl * 32; r < min(n, sl * 32 + 32); ++r) w = max(w, tr.last(r) - tr.first(r));
        cnt[sl] = 32 * w;
    }
}

// entry k of row r (slice s, lane l) at slice[s] + 32 k + l; padding entries
// point at the row itself with no source (value 0)
__global__ void k_slice_fill(i64 n, TriRows tr, const int32_t* __restrict__ cols, const i64* __restrict__ src_of,
                             const i64* __restrict__ slice, int32_t* __restrict__ col, i64* __restrict__ src) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x) {
        const i64 sl = r >> 5, lane = r & 31, w = (slice[sl + 1] - slice[sl]) >> 5;
        const i64 f = tr.first(r), l = tr.last(r);
        for (i64 k = 0; k < w; ++k) {
            const i64 e = slice[sl] + 32 * k + lane, pos = f + k;
            if (pos < l) {
                col[e] = cols[pos];
                src[e] = src_of ? src_of[pos] : pos;
            } else {
                col[e] = int32_t(r);
                src[e] = -1;
            }
        }
    }
}

void jacobi_slab_gpu(Ctx& ctx, i64 n, TriRows tr, const int32_t* cols, const i64* src_of, JacobiSlab& s) {
    const i64 slices = (n + 31) / 32;
    s.slice.resize(size_t(slices + 1));
    NL_CUDA(cudaMemsetAsync(s.slice.p + slices, 0, sizeof(i64), ctx.stream));
    NL_LAUNCH(k_slice_width, grid_for(slices, IB_THREADS), IB_THREADS, 0, ctx.stream, n, tr, s.slice.p);
    i64 total = 0;
    exclusive_scan(ctx, s.slice.p, s.slice.p, slices + 1, &total);
    s.entries = total;
    const size_t m = size_t(std::max<i64>(total, 1));
    s.col.resize(m);
    s.src.resize(m);
    // the padding rows past n in the last slice: column 0, no source
    NL_CUDA(cudaMemsetAsync(s.col.p, 0, m * sizeof(int32_t), ctx.stream));
    NL_CUDA(cudaMemsetAsync(s.src.p, 0xff, m * sizeof(i64), ctx.stream));
    NL_LAUNCH(k_slice_fill, grid_for(n, IB_THREADS), IB_THREADS, 0, ctx.stream, n, tr, cols, src_of, s.slice.p, s.col.p,
              s.src.p);
    s.val.resize(m);
    s.val.zero(ctx.stream);
}

}  // namespace

// U pattern copies, U^T, the factorisation's rows in level order and the
// Jacobi layouts, all on the device
void ilt_structure_gpu(Ctx& ctx, const Csr& upper, IncompleteCholesky& ic, bool levels) {
    const i64 n = upper.rows, nnz = upper.nnz;
    dbuf<int> bad;
    bad.resize(1);
    bad.zero(ctx.stream);
    NL_LAUNCH(k_check_diag_first, grid_for(n, IB_THREADS), IB_THREADS, 0, ctx.stream, n, upper.rowptr.p, upper.col.p,
              bad.p);
    ic.rp.resize(size_t(n + 1));
    ic.col.resize(size_t(nnz));
    NL_CUDA(cudaMemcpyAsync(ic.rp.p, upper.rowptr.p, size_t(n + 1) * sizeof(i64), cudaMemcpyDeviceToDevice, ctx.stream));
    NL_CUDA(cudaMemcpyAsync(ic.col.p, upper.col.p, size_t(nnz) * sizeof(int32_t), cudaMemcpyDeviceToDevice, ctx.stream));
    // U^T
    ic.lrp.resize(size_t(n + 1));
    ic.lrp.zero(ctx.stream);
    NL_LAUNCH(k_col_count, grid_for(nnz, IB_THREADS), IB_THREADS, 0, ctx.stream, nnz, upper.col.p,
              reinterpret_cast<unsigned long long*>(ic.lrp.p));
    exclusive_scan(ctx, ic.lrp.p, ic.lrp.p, n + 1, nullptr);
    ic.lcol.resize(size_t(nnz));
    ic.l_to_u.resize(size_t(nnz));
    dbuf<unsigned> cursor;
    cursor.resize(size_t(n));
    cursor.zero(ctx.stream);
    NL_LAUNCH(k_transpose_place, grid_for(n, IB_THREADS), IB_THREADS, 0, ctx.stream, n, upper.rowptr.p, upper.col.p,
              ic.lrp.p, cursor.p, ic.lcol.p, ic.l_to_u.p);
    NL_LAUNCH(k_sort_rows, grid_for(n, IB_THREADS), IB_THREADS, 0, ctx.stream, n, ic.lrp.p, ic.lcol.p, ic.l_to_u.p);
    // levels of the exact factorisation's schedule
    i64 ho[2] = {0, n};
    int hbad = 0;
    dbuf<int> indeg;
    dbuf<i64> out;
    if (levels) {
        indeg.resize(size_t(n));
        ic.ic_rows.resize(size_t(n));
        ic.ic_lev_ptr.resize(size_t(n + 1));
        out.resize(2);
        NL_LAUNCH(k_levels, 1, IB_LEVEL_THREADS, 0, ctx.stream, n, ic.lrp.p, upper.rowptr.p, upper.col.p, indeg.p,
                  ic.ic_rows.p, ic.ic_lev_ptr.p, out.p);
        out.download(ho, 2, ctx.stream);
    }
    NL_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof hbad, cudaMemcpyDeviceToHost, ctx.stream));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    NL_REQUIRE(!hbad, NLGPU_ERR_ARG, "every row of the preconditioner matrix needs its diagonal first");
    NL_REQUIRE(ho[1] == n, NLGPU_ERR_STATE, "the factor's dependency graph does not reach every row");
    ic.ic_levels = levels ? ho[0] : 0;
    // Jacobi layouts of U^T (values u[l_to_u]) and U
    jacobi_slab_gpu(ctx, n, TriRows{ic.lrp.p, true}, ic.lcol.p, ic.l_to_u.p, ic.jlo);
    jacobi_slab_gpu(ctx, n, TriRows{ic.rp.p, false}, ic.col.p, nullptr, ic.jup);
    ic.jc.resize(size_t(n)); ic.jdinv.resize(size_t(n));
    ic.jt0.resize(size_t(n)); ic.jt1.resize(size_t(n)); ic.jy.resize(size_t(n));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
}

}  // namespace nlgpu
