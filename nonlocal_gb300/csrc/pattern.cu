// Sparsity patterns of the assembled matrices.
//
// The reference builds them in two mesh_run sweeps (shift_initializer counts
// distinct columns per row, matrix_index_initializer writes them, then
// sort_indices; matrix_assembler_2d.hpp:144-176, conductivity_matrix_2d.hpp:39-72)
// with the split of matrix_separator_base::part (matrix_separator_base.hpp:51-58):
//   INNER  column and row inner, and row <= column when symmetric;
//   BOUND  column Dirichlet and row != column (full rows);
//   NO     otherwise; a Dirichlet row holds only its unit diagonal.
// The candidate columns of row r are the nodes of every neighbour eNL of every
// element eL containing r (nodes of eL itself for the local part).
//
// Here one CTA owns a row.  Candidates are OR-ed into a shared-memory bitmap
// over a window of node numbers (windows repeat when the row spans more
// nodes than a window holds, so any numbering works), then the set bits are
// classified and emitted in increasing order with per-thread counts and block
// scans: the result is the reference's sorted column list without any sort.
// Three lists come out at once: the inner part (upper or full), the bound
// part, and the full-row inner pattern the solver's SpMV reads (rows padded
// to a multiple of 4 entries).
#include "common.cuh"

namespace nlgpu {

namespace {

constexpr int PT_THREADS = 256;
constexpr int PT_WORDS = 10048;                // 321536 node numbers per window (39.3 KB)
constexpr i64 PT_WINDOW = i64(PT_WORDS) * 32;
constexpr int PT_ELEM_WORDS = 2048;            // 65536 element numbers for the element bitmap (8 KB)
constexpr int PT_MAX_ELEMS = 16;               // elements sharing one node

struct PatternArgs {
    i64 n;
    int nen;
    bool local_only, symmetric;
    const int32_t* elems;
    const i64* ne_off;
    const int32_t* ne_elem;
    const i64* noff;
    const int32_t* nlist;
    const uint8_t* is_inner;
    const int32_t* emin;   // smallest / largest node number of every element
    const int32_t* emax;
    // count pass outputs
    i64* cnt_inner;
    i64* cnt_bound;
    i64* cnt_full;
    // fill pass outputs (null in the count pass)
    const i64* rp_inner;
    const i64* rp_bound;
    const i64* rp_full;
    int32_t* col_inner;
    int32_t* col_bound;
    int32_t* col_full;
    int* error;
};

__device__ __forceinline__ i64 block_scan_excl(i64 v, i64* sh, i64* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    i64 incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const i64 t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        i64 s = lane < PT_THREADS / 32 ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const i64 t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        if (lane < PT_THREADS / 32) sh[lane] = s;
    }
    __syncthreads();
    const i64 off = warp ? sh[warp - 1] : 0;
    *total = sh[PT_THREADS / 32 - 1];
    __syncthreads();
    return off + incl - v;
}

// One CTA per row.  Every candidate column goes into one shared-memory
// bitmap over a window of node numbers; the set bits are then classified
// (inner / bound / full) and emitted in increasing order with per-thread
// counts and block scans.  The window's node range comes from the candidate
// elements' smallest and largest node numbers, and NEN is a template
// parameter, so a candidate costs two loads and one shared-memory OR.
// The elements of a node share most of their neighbours: each candidate
// element is expanded into its nodes once per row, the first time it is met
// (an element bitmap over a window of element numbers from the smallest
// candidate; candidates beyond the window are expanded every time).
template<int NEN>
__global__ void __launch_bounds__(PT_THREADS) k_pattern(PatternArgs a) {
    __shared__ uint32_t bm[PT_WORDS];
    __shared__ uint32_t ebm[PT_ELEM_WORDS];
    __shared__ int32_t seg_elem[PT_MAX_ELEMS];
    __shared__ i64 seg_noff[PT_MAX_ELEMS], seg_len[PT_MAX_ELEMS];
    __shared__ i64 sh_scan[PT_THREADS / 32];
    __shared__ int red_min[PT_THREADS / 32], red_max[PT_THREADS / 32], red_emin[PT_THREADS / 32],
        red_emax[PT_THREADS / 32];
    const bool fill = a.col_inner != nullptr;

    for (i64 r = blockIdx.x; r < a.n; r += gridDim.x) {
        const i64 eb = a.ne_off[r], ee = a.ne_off[r + 1];
        const int ne = int(ee - eb);
        if (ne > PT_MAX_ELEMS) { if (threadIdx.x == 0) atomicExch(a.error, 1); continue; }
        if (threadIdx.x < ne) {
            const int32_t e = a.ne_elem[eb + threadIdx.x];
            seg_elem[threadIdx.x] = e;
            seg_noff[threadIdx.x] = a.local_only ? 0 : a.noff[e];
            seg_len[threadIdx.x] = a.local_only ? 1 : a.noff[e + 1] - a.noff[e];
        }
        __syncthreads();
        const bool row_inner = a.is_inner[r];
        auto cand_elem = [&](int s, i64 k) -> int32_t {
            return a.local_only ? seg_elem[s] : a.nlist[seg_noff[s] + k];
        };

        // node range of the candidates from their elements' extreme nodes, and
        // the smallest candidate element
        int lo = 0x7fffffff, hi = -1, elo = 0x7fffffff, ehi = -1;
        for (int s = 0; s < ne; ++s)
            for (i64 k = threadIdx.x; k < seg_len[s]; k += PT_THREADS) {
                const int32_t e = cand_elem(s, k);
                lo = min(lo, a.emin[e]);
                hi = max(hi, a.emax[e]);
                elo = min(elo, e);
                ehi = max(ehi, e);
            }
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            elo = min(elo, __shfl_xor_sync(0xffffffffu, elo, o));
            ehi = max(ehi, __shfl_xor_sync(0xffffffffu, ehi, o));
        }
        if ((threadIdx.x & 31) == 0) {
            red_min[threadIdx.x >> 5] = lo; red_max[threadIdx.x >> 5] = hi;
            red_emin[threadIdx.x >> 5] = elo; red_emax[threadIdx.x >> 5] = ehi;
        }
        __syncthreads();
        lo = red_min[0]; hi = red_max[0]; elo = red_emin[0]; ehi = red_emax[0];
        for (int w = 1; w < PT_THREADS / 32; ++w) {
            lo = min(lo, red_min[w]); hi = max(hi, red_max[w]); elo = min(elo, red_emin[w]); ehi = max(ehi, red_emax[w]);
        }
        __syncthreads();

        i64 n_inner = 0, n_bound = 0, n_full = 0;
        if (!row_inner) {   // Dirichlet row: unit diagonal only in the inner parts
            n_inner = 1; n_full = 1;
            if (fill && threadIdx.x == 0) { a.col_inner[a.rp_inner[r]] = int32_t(r); a.col_full[a.rp_full[r]] = int32_t(r); }
        }
        for (i64 base = lo; hi >= 0 && base <= hi; base += PT_WINDOW) {
            // clear only the words the candidates can reach
            const int node_words = int(min(i64(hi) - base, PT_WINDOW - 1) >> 5) + 1;
            for (int w = threadIdx.x; w < node_words; w += PT_THREADS) bm[w] = 0u;
            if (ne > 1) {
                const int elem_words = int(min(i64(ehi) - elo, i64(PT_ELEM_WORDS) * 32 - 1) >> 5) + 1;
                for (int w = threadIdx.x; w < elem_words; w += PT_THREADS) ebm[w] = 0u;
            }
            __syncthreads();
            for (int s = 0; s < ne; ++s)
                for (i64 k = threadIdx.x; k < seg_len[s]; k += PT_THREADS) {
                    const int32_t e = cand_elem(s, k);
                    if (ne > 1) {   // an element met before in this row adds nothing new
                        const i64 eo = i64(e) - elo;
                        if (eo < i64(PT_ELEM_WORDS) * 32) {
                            const uint32_t bit = 1u << (eo & 31);
                            if (atomicOr(&ebm[eo >> 5], bit) & bit) continue;
                        }
                    }
#pragma unroll
                    for (int j = 0; j < NEN; ++j) {
                        const i64 off = i64(a.elems[i64(e) * NEN + j]) - base;
                        if (off < 0 || off >= PT_WINDOW) continue;
                        atomicOr(&bm[off >> 5], 1u << (off & 31));
                    }
                }
            __syncthreads();
            const i64 span = min(i64(hi) - base + 1, PT_WINDOW);
            const int words = int((span + 31) >> 5);
            const int per = (words + PT_THREADS - 1) / PT_THREADS;
            const int w0 = threadIdx.x * per, w1 = min(words, w0 + per);
            // matrix_separator_base::part on every distinct candidate column
            auto classify = [&](int32_t c, bool& in_inner, bool& in_bound, bool& in_full) {
                const bool c_in = a.is_inner[c];
                in_full = c_in && row_inner;
                in_inner = in_full && (!a.symmetric || r <= c);
                in_bound = !c_in && c != r;
            };
            i64 ci = 0, cb = 0, cf = 0;
            for (int w = w0; w < w1; ++w)
                for (uint32_t m = bm[w]; m; m &= m - 1) {
                    bool ii, bb, ff;
                    classify(int32_t(base + i64(w) * 32 + __ffs(m) - 1), ii, bb, ff);
                    ci += ii; cb += bb; cf += ff;
                }
            i64 ti, tb, tf;
            const i64 oi = block_scan_excl(ci, sh_scan, &ti);
            const i64 ob = block_scan_excl(cb, sh_scan, &tb);
            const i64 of = block_scan_excl(cf, sh_scan, &tf);
            if (fill) {
                i64 pi = a.rp_inner[r] + n_inner + oi, pb = a.rp_bound[r] + n_bound + ob, pf = a.rp_full[r] + n_full + of;
                for (int w = w0; w < w1; ++w)
                    for (uint32_t m = bm[w]; m; m &= m - 1) {
                        const int32_t c = int32_t(base + i64(w) * 32 + __ffs(m) - 1);
                        bool ii, bb, ff;
                        classify(c, ii, bb, ff);
                        if (ii) a.col_inner[pi++] = c;
                        if (bb) a.col_bound[pb++] = c;
                        if (ff) a.col_full[pf++] = c;
                    }
            }
            n_inner += ti; n_bound += tb; n_full += tf;
            __syncthreads();
        }
        if (!fill) {
            if (threadIdx.x == 0) { a.cnt_inner[r] = n_inner; a.cnt_bound[r] = n_bound; a.cnt_full[r] = (n_full + 3) & ~i64(3); }
        } else {   // pad the solver row to a multiple of 4 with (r, 0) entries
            const i64 end = a.rp_full[r + 1];
            for (i64 k = a.rp_full[r] + n_full + threadIdx.x; k < end; k += PT_THREADS) a.col_full[k] = int32_t(r);
        }
        __syncthreads();
    }
}

void launch_pattern(Ctx& ctx, unsigned grid, const PatternArgs& a) {
    if (a.nen == 4) NL_LAUNCH(k_pattern<4>, grid, PT_THREADS, 0, ctx.stream, a);
    else if (a.nen == 8) NL_LAUNCH(k_pattern<8>, grid, PT_THREADS, 0, ctx.stream, a);
    else NL_REQUIRE(false, NLGPU_ERR_UNSUPPORTED, "elements of 4 or 8 nodes");
}

// full-row entry -> index of the same value in the upper storage (or -1 for padding)
__global__ void k_full_map(i64 n, const i64* __restrict__ up_rp, const int32_t* __restrict__ up_col,
                           const i64* __restrict__ full_rp, const int32_t* __restrict__ full_col,
                           const uint8_t* __restrict__ is_inner, bool symmetric, i64* __restrict__ map) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        const i64 fb = full_rp[r], fe = full_rp[r + 1];
        const i64 ub = up_rp[r], ue = up_rp[r + 1];
        for (i64 k = fb + lane; k < fe; k += 32) {
            const int32_t c = full_col[k];
            i64 target = -1;
            // real entries are strictly increasing; padding (col r) breaks the order
            if (k > fb && c <= full_col[k - 1]) target = -1;
            else if (!symmetric || c >= int32_t(r)) {
                i64 lo = ub, hi = ue;   // search c in row r
                while (lo < hi) { const i64 mid = (lo + hi) >> 1; if (up_col[mid] < c) lo = mid + 1; else hi = mid; }
                target = (lo < ue && up_col[lo] == c) ? lo : -1;
            } else {
                i64 lo = up_rp[c], hi = up_rp[c + 1];   // transpose: search r in row c
                while (lo < hi) { const i64 mid = (lo + hi) >> 1; if (up_col[mid] < int32_t(r)) lo = mid + 1; else hi = mid; }
                target = (lo < up_rp[c + 1] && up_col[lo] == int32_t(r)) ? lo : -1;
            }
            map[k] = target;
        }
        (void)is_inner;
    }
}

}  // namespace

void full_map(Ctx& ctx, const Csr& upper, const Csr& full, dbuf<i64>& map, bool symmetric) {
    map.resize(size_t(full.nnz));
    NL_LAUNCH(k_full_map, grid_for(full.rows * 32, 256, 152 * 64), 256, 0, ctx.stream, full.rows, upper.rowptr.p,
              upper.col.p, full.rowptr.p, full.col.p, static_cast<const uint8_t*>(nullptr), symmetric, map.p);
}

void build_patterns(Ctx& ctx, bool local_only, bool symmetric, Csr& inner, Csr* bound, Csr* full,
                    dbuf<i64>* full_from_upper, const uint8_t* is_inner) {
    const i64 n = ctx.n_nodes;
    NL_REQUIRE(local_only || ctx.neighbours_ready, NLGPU_ERR_STATE, "neighbour search must run before a nonlocal assembly");
    for (Csr* m : {&inner, bound, full})   // 16-bit column offsets belong to the old pattern
        if (m) m->col16_ok = false;
    dbuf<i64> ci, cb, cf;
    ci.resize(size_t(n + 1)); cb.resize(size_t(n + 1)); cf.resize(size_t(n + 1));
    ci.zero(ctx.stream); cb.zero(ctx.stream); cf.zero(ctx.stream);
    dbuf<int> err;
    err.resize(1); err.zero(ctx.stream);
    PatternArgs a{};
    a.n = n; a.nen = ctx.basis.nen; a.local_only = local_only; a.symmetric = symmetric;
    a.elems = ctx.elems.p; a.ne_off = ctx.ne_off.p; a.ne_elem = ctx.ne_elem.p;
    a.noff = local_only ? nullptr : ctx.noff.p; a.nlist = local_only ? nullptr : ctx.nlist.p;
    a.is_inner = is_inner ? is_inner : ctx.is_inner.p;
    a.emin = ctx.elem_minnode.p; a.emax = ctx.elem_maxnode.p;
    a.cnt_inner = ci.p; a.cnt_bound = cb.p; a.cnt_full = cf.p; a.error = err.p;
    const unsigned grid = unsigned(std::min<i64>(n, 152 * 8));
    launch_pattern(ctx, grid, a);
    int herr = 0;
    NL_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof herr, cudaMemcpyDeviceToHost, ctx.stream));
    i64 nnz_i = 0, nnz_b = 0, nnz_f = 0;
    inner.rows = n; inner.rowptr.resize(size_t(n + 1));
    exclusive_scan(ctx, ci.p, inner.rowptr.p, n + 1, &nnz_i);
    NL_REQUIRE(herr == 0, NLGPU_ERR_UNSUPPORTED, "a node belongs to more than 16 elements");
    Csr tmp_bound, tmp_full;
    Csr& B = bound ? *bound : tmp_bound;
    Csr& F = full ? *full : tmp_full;
    B.rows = n; B.rowptr.resize(size_t(n + 1));
    F.rows = n; F.rowptr.resize(size_t(n + 1));
    exclusive_scan(ctx, cb.p, B.rowptr.p, n + 1, &nnz_b);
    exclusive_scan(ctx, cf.p, F.rowptr.p, n + 1, &nnz_f);
    inner.nnz = nnz_i; B.nnz = nnz_b; F.nnz = nnz_f;
    inner.col.resize(size_t(nnz_i)); B.col.resize(size_t(nnz_b)); F.col.resize(size_t(nnz_f));
    a.rp_inner = inner.rowptr.p; a.rp_bound = B.rowptr.p; a.rp_full = F.rowptr.p;
    a.col_inner = inner.col.p; a.col_bound = B.col.p; a.col_full = F.col.p;
    // count pointers stay set but are not written in the fill pass
    launch_pattern(ctx, grid, a);
    inner.val.resize(size_t(nnz_i)); inner.val.zero(ctx.stream);
    B.val.resize(size_t(nnz_b)); B.val.zero(ctx.stream);
    if (full && full_from_upper) {
        full_from_upper->resize(size_t(nnz_f));
        NL_LAUNCH(k_full_map, grid_for(n * 32, 256, 152 * 64), 256, 0, ctx.stream, n, inner.rowptr.p, inner.col.p,
                  F.rowptr.p, F.col.p, a.is_inner, symmetric, full_from_upper->p);
        F.val.resize(size_t(nnz_f));
    }
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
}

}  // namespace nlgpu
