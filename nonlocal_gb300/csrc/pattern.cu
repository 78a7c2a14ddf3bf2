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
// Here one warp owns a row.  Candidates are OR-ed into the warp's
// shared-memory bitmap over a window of node numbers (windows repeat when the
// row spans more nodes than a window holds, so any numbering works), then the
// set bits are classified a word at a time and emitted in increasing order
// with warp scans: the result is the reference's sorted column list without
// any sort.
// Three lists come out at once: the inner part (upper or full), the bound
// part, and the full-row inner pattern the solver's SpMV reads (rows padded
// to a multiple of 4 entries).
#include "common.cuh"

namespace nlgpu {

namespace {

constexpr int PT_MAX_ELEMS = 16;               // elements sharing one node
constexpr int PW_WARPS = 8;                    // rows (warps) per CTA
constexpr int PW_WORDS = 1024;                 // node bitmap per warp: 32768 node numbers (4 KB)
constexpr i64 PW_WINDOW = i64(PW_WORDS) * 32;
constexpr int PW_EWORDS = 512;                 // element bitmap per warp: 16384 element numbers (2 KB)
constexpr int PW_UNROLL = 4;                   // candidate elements in flight per lane
constexpr size_t PW_SMEM = size_t(PW_WARPS) * (PW_WORDS + PW_EWORDS) * sizeof(uint32_t);

struct PatternArgs {
    i64 n;
    bool local_only, symmetric;
    const int32_t* elems;
    const i64* ne_off;
    const int32_t* ne_elem;
    const i64* noff;
    const int32_t* nlist;
    const uint8_t* is_inner;
    const uint32_t* inner_bits;   // is_inner as a bitmap (bit c of word c / 32)
    const int32_t* emin;          // smallest / largest node number of every element
    const int32_t* emax;
    const int4* nb_range;         // per element: the extreme node and element numbers of its neighbours
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

__global__ void k_inner_bits(i64 n, const uint8_t* __restrict__ is_inner, uint32_t* __restrict__ bits) {
    const i64 words = (n + 31) / 32;
    for (i64 w = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; w < words; w += (i64(gridDim.x) * blockDim.x) >> 5) {
        const i64 c = w * 32 + (threadIdx.x & 31);
        const unsigned b = __ballot_sync(0xffffffffu, c < n && is_inner[c]);
        if ((threadIdx.x & 31) == 0) bits[w] = b;
    }
}

// per element e: (smallest node, largest node, smallest element, largest
// element) over its neighbour list (warp per element)
__global__ void k_neighbour_range(i64 E, const i64* __restrict__ noff, const int32_t* __restrict__ nlist,
                                  const int32_t* __restrict__ emin, const int32_t* __restrict__ emax,
                                  int4* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const i64 warps = (i64(gridDim.x) * blockDim.x) >> 5;
    for (i64 e = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; e < E; e += warps) {
        int lo = 0x7fffffff, hi = -1, elo = 0x7fffffff, ehi = -1;
        for (i64 k = noff[e] + lane; k < noff[e + 1]; k += 32) {
            const int32_t f = nlist[k];
            lo = min(lo, emin[f]); hi = max(hi, emax[f]);
            elo = min(elo, f); ehi = max(ehi, f);
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            elo = min(elo, __shfl_xor_sync(0xffffffffu, elo, o));
            ehi = max(ehi, __shfl_xor_sync(0xffffffffu, ehi, o));
        }
        if (lane == 0) out[e] = make_int4(lo, hi, elo, ehi);
    }
}

// bits b of the word of node numbers [nb, nb + 32) with nb + b >= r
__device__ __forceinline__ uint32_t mask_from(i64 r, i64 nb) {
    if (r <= nb) return 0xffffffffu;
    if (r >= nb + 32) return 0u;
    return ~((1u << unsigned(r - nb)) - 1u);
}

__device__ __forceinline__ uint32_t bit_of(i64 r, i64 nb) {
    return (r >= nb && r < nb + 32) ? (1u << unsigned(r - nb)) : 0u;
}

template<int NEN>
__device__ __forceinline__ void load_nodes(const int32_t* __restrict__ elems, int32_t e, int32_t (&v)[NEN]) {
    const int4* p = reinterpret_cast<const int4*>(elems + i64(e) * NEN);
#pragma unroll
    for (int h = 0; h < NEN / 4; ++h) {
        const int4 q = __ldg(p + h);
        v[4 * h] = q.x; v[4 * h + 1] = q.y; v[4 * h + 2] = q.z; v[4 * h + 3] = q.w;
    }
}

// One warp per row.  The candidate columns go into the warp's shared-memory
// bitmap over a window of node numbers (from the precomputed extreme node
// numbers of the row's elements' neighbours; rows spanning more than one
// window take several, so any numbering works).  The elements of a node share
// most of their neighbours: a second bitmap over element numbers lets each
// candidate element be expanded into its nodes once per row (candidates
// beyond that window are expanded every time).  The set bits are then
// classified a word at a time against the inner-node bitmap and emitted in
// increasing order, 32 words per round with a warp scan of the counts: the
// reference's sorted column list without a sort.
template<int NEN>
__global__ void __launch_bounds__(PW_WARPS * 32) k_pattern(PatternArgs a) {
    extern __shared__ uint32_t pw_smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t* bm = pw_smem + wid * PW_WORDS;
    uint32_t* ebm = pw_smem + PW_WARPS * PW_WORDS + wid * PW_EWORDS;
    const unsigned full = 0xffffffffu;
    const bool fill = a.col_inner != nullptr;
    const i64 warps = i64(gridDim.x) * PW_WARPS;

    for (i64 r = i64(blockIdx.x) * PW_WARPS + wid; r < a.n; r += warps) {
        const i64 eb = a.ne_off[r];
        const int ne = int(a.ne_off[r + 1] - eb);
        if (ne > PT_MAX_ELEMS) { if (lane == 0) atomicExch(a.error, 1); continue; }
        int32_t my_e = -1;
        i64 my_off = 0;
        int my_len = 0, lo = 0x7fffffff, hi = -1, elo = 0x7fffffff, ehi = -1;
        if (lane < ne) {
            my_e = a.ne_elem[eb + lane];
            if (a.local_only) {
                lo = a.emin[my_e]; hi = a.emax[my_e];
            } else {
                my_off = a.noff[my_e];
                my_len = int(a.noff[my_e + 1] - my_off);
                const int4 g = a.nb_range[my_e];
                lo = g.x; hi = g.y; elo = g.z; ehi = g.w;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(full, lo, o));
            hi = max(hi, __shfl_xor_sync(full, hi, o));
            elo = min(elo, __shfl_xor_sync(full, elo, o));
            ehi = max(ehi, __shfl_xor_sync(full, ehi, o));
        }
        const bool row_inner = a.is_inner[r];
        i64 n_inner = 0, n_bound = 0, n_full = 0;
        if (!row_inner) {   // Dirichlet row: unit diagonal only in the inner parts
            n_inner = 1; n_full = 1;
            if (fill && lane == 0) { a.col_inner[a.rp_inner[r]] = int32_t(r); a.col_full[a.rp_full[r]] = int32_t(r); }
        }
        const bool dedupe = !a.local_only && ne > 1;
        const i64 elem_span = min(i64(ehi) - elo, i64(PW_EWORDS) * 32 - 1);
        for (i64 base = i64(lo) & ~i64(31); hi >= 0 && base <= hi; base += PW_WINDOW) {
            const int nw = int(min(i64(hi) - base, PW_WINDOW - 1) >> 5) + 1;
            for (int w = lane; w < nw; w += 32) bm[w] = 0u;
            if (dedupe)
                for (int w = lane; w <= int(elem_span >> 5); w += 32) ebm[w] = 0u;
            __syncwarp();
            auto expand = [&](int32_t e) {
                int32_t v[NEN];
                load_nodes<NEN>(a.elems, e, v);
#pragma unroll
                for (int j = 0; j < NEN; ++j) {
                    const i64 off = i64(v[j]) - base;
                    if (off >= 0 && off < PW_WINDOW) atomicOr(&bm[off >> 5], 1u << (off & 31));
                }
            };
            if (a.local_only) {
                if (lane < ne) expand(my_e);
            } else {
                for (int s = 0; s < ne; ++s) {
                    const i64 off = __shfl_sync(full, my_off, s);
                    const int len = __shfl_sync(full, my_len, s);
                    for (int k0 = 0; k0 < len; k0 += 32 * PW_UNROLL) {
                        int32_t e[PW_UNROLL];
#pragma unroll
                        for (int u = 0; u < PW_UNROLL; ++u) {
                            const int k = k0 + u * 32 + lane;
                            e[u] = k < len ? a.nlist[off + k] : -1;
                        }
                        if (dedupe) {   // an element met before in this row adds nothing new
#pragma unroll
                            for (int u = 0; u < PW_UNROLL; ++u) {
                                const i64 eo = i64(e[u]) - elo;
                                if (e[u] >= 0 && eo < i64(PW_EWORDS) * 32) {
                                    const uint32_t bit = 1u << (eo & 31);
                                    if (atomicOr(&ebm[eo >> 5], bit) & bit) e[u] = -1;
                                }
                            }
                        }
#pragma unroll
                        for (int u = 0; u < PW_UNROLL; ++u)
                            if (e[u] >= 0) expand(e[u]);
                    }
                }
            }
            __syncwarp();
            // matrix_separator_base::part a word at a time, 32 words per round
            for (int w0 = 0; w0 < nw; w0 += 32) {
                const int w = w0 + lane;
                const i64 nb = base + i64(w) * 32;
                uint32_t m = 0u, iw = 0u;
                if (w < nw) {
                    m = bm[w];
                    if (m) iw = a.inner_bits[nb >> 5];
                }
                const uint32_t mf = row_inner ? (m & iw) : 0u;
                const uint32_t mi = a.symmetric ? (mf & mask_from(r, nb)) : mf;
                const uint32_t mb = m & ~iw & ~bit_of(r, nb);
                // three counts (each <= 1024 per round) packed in 21-bit fields
                const unsigned long long c = (unsigned long long)__popc(mi) |
                                             ((unsigned long long)__popc(mb) << 21) |
                                             ((unsigned long long)__popc(mf) << 42);
                unsigned long long incl = c;
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned long long t = __shfl_up_sync(full, incl, o);
                    if (lane >= o) incl += t;
                }
                const unsigned long long tot = __shfl_sync(full, incl, 31);
                if (fill) {
                    const unsigned long long ex = incl - c;
                    const unsigned long long f21 = (1ull << 21) - 1;
                    i64 pi = a.rp_inner[r] + n_inner + i64(ex & f21);
                    i64 pb = a.rp_bound[r] + n_bound + i64((ex >> 21) & f21);
                    i64 pf = a.rp_full[r] + n_full + i64(ex >> 42);
                    for (uint32_t t = mi; t; t &= t - 1) a.col_inner[pi++] = int32_t(nb + __ffs(t) - 1);
                    for (uint32_t t = mb; t; t &= t - 1) a.col_bound[pb++] = int32_t(nb + __ffs(t) - 1);
                    for (uint32_t t = mf; t; t &= t - 1) a.col_full[pf++] = int32_t(nb + __ffs(t) - 1);
                }
                n_inner += i64(tot & ((1ull << 21) - 1));
                n_bound += i64((tot >> 21) & ((1ull << 21) - 1));
                n_full += i64(tot >> 42);
            }
            __syncwarp();
        }
        if (!fill) {
            if (lane == 0) { a.cnt_inner[r] = n_inner; a.cnt_bound[r] = n_bound; a.cnt_full[r] = (n_full + 3) & ~i64(3); }
        } else {   // pad the solver row to a multiple of 4 with (r, 0) entries
            const i64 end = a.rp_full[r + 1];
            for (i64 k = a.rp_full[r] + n_full + lane; k < end; k += 32) a.col_full[k] = int32_t(r);
        }
    }
}

void launch_pattern(Ctx& ctx, int nen, unsigned grid, const PatternArgs& a) {
    if (nen == 4) {
        NL_CUDA(cudaFuncSetAttribute(k_pattern<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(PW_SMEM)));
        NL_LAUNCH(k_pattern<4>, grid, PW_WARPS * 32, PW_SMEM, ctx.stream, a);
    } else if (nen == 8) {
        NL_CUDA(cudaFuncSetAttribute(k_pattern<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(PW_SMEM)));
        NL_LAUNCH(k_pattern<8>, grid, PW_WARPS * 32, PW_SMEM, ctx.stream, a);
    } else {
        NL_REQUIRE(false, NLGPU_ERR_UNSUPPORTED, "elements of 4 or 8 nodes");
    }
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
    a.n = n; a.local_only = local_only; a.symmetric = symmetric;
    a.elems = ctx.elems.p; a.ne_off = ctx.ne_off.p; a.ne_elem = ctx.ne_elem.p;
    a.noff = local_only ? nullptr : ctx.noff.p; a.nlist = local_only ? nullptr : ctx.nlist.p;
    a.is_inner = is_inner ? is_inner : ctx.is_inner.p;
    a.emin = ctx.elem_minnode.p; a.emax = ctx.elem_maxnode.p;
    a.cnt_inner = ci.p; a.cnt_bound = cb.p; a.cnt_full = cf.p; a.error = err.p;
    dbuf<uint32_t> bits;
    bits.resize(size_t((n + 31) / 32 + 1));
    NL_LAUNCH(k_inner_bits, grid_for((n + 31) / 32 * 32, 256), 256, 0, ctx.stream, n, a.is_inner, bits.p);
    a.inner_bits = bits.p;
    dbuf<int4> range;
    if (!local_only) {
        const i64 E = ctx.n_elems;
        range.resize(size_t(std::max<i64>(E, 1)));
        NL_LAUNCH(k_neighbour_range, grid_for(E * 32, 256, 152 * 64), 256, 0, ctx.stream, E, ctx.noff.p, ctx.nlist.p,
                  ctx.elem_minnode.p, ctx.elem_maxnode.p, range.p);
        a.nb_range = range.p;
    }
    const int nen = ctx.basis.nen;
    const unsigned grid = unsigned(std::max<i64>(1, std::min<i64>((n + PW_WARPS - 1) / PW_WARPS, 152 * 4 * 8)));
    launch_pattern(ctx, nen, grid, a);
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
    launch_pattern(ctx, nen, grid, a);
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
