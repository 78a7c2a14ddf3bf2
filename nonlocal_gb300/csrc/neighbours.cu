// Neighbour search of mesh::find_neighbours (libraries/mesh/mesh_2d/find_neighbours.hpp:120-160)
// for a mesh whose elements form one group.
//
//   1. radius widening by the element-centre distance between elements that
//      share a node (increase_influence, :399-434);
//   2. bucket grid of square cells of the widened radius over the bounding
//      rectangle of the nodes (split_elements_by_subareas, :436-457), each
//      cell listing its elements by increasing number;
//   3. per element, a scan of the 3x3 surrounding cells in the reference's
//      order (subareas_ids, :459-467) keeping elements whose normalised
//      powered centre distance is <= 1.
//
// One warp per element in step 3; lanes test consecutive elements of a cell
// and a ballot keeps the reference's list order.  Built with --fmad=false so
// every distance rounds as the reference's host code, which makes the lists
// bit-exact.
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace nlgpu {

namespace {

__device__ __forceinline__ unsigned long long ordered_bits(double v) {
    const unsigned long long b = __double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
double from_ordered_bits(unsigned long long b) {
    const unsigned long long raw = (b & 0x8000000000000000ull) ? (b & 0x7fffffffffffffffull) : ~b;
    double v;
    std::memcpy(&v, &raw, sizeof v);
    return v;
}

struct WidenOut {
    unsigned long long dmax, dmin, count;
    double sum;
    unsigned long long bbox[4];   // ordered bits: min x, min y, max x, max y
};

constexpr int WIDEN_THREADS = 256;

// min / max of 64-bit keys over the block, then one atomic per block
__device__ void block_min_max(unsigned long long (&v)[6], unsigned long long* out_min[3],
                              unsigned long long* out_max[3]) {
    __shared__ unsigned long long sh[6][WIDEN_THREADS / 32];
    for (int k = 0; k < 6; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k] = k < 3 ? (w < v[k] ? w : v[k]) : (w > v[k] ? w : v[k]);
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 6; ++k) sh[k][threadIdx.x >> 5] = v[k];
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        unsigned long long r = sh[k][0];
        for (int w = 1; w < WIDEN_THREADS / 32; ++w) r = k < 3 ? (sh[k][w] < r ? sh[k][w] : r) : (sh[k][w] > r ? sh[k][w] : r);
        if (k < 3) { if (out_min[k]) atomicMin(out_min[k], r); }
        else if (out_max[k - 3]) atomicMax(out_max[k - 3], r);
    }
}

// Squared centre distance over elements sharing a node (diameter_between_elements_centers),
// and the bounding rectangle of the nodes; extremes reduced per block.
__global__ void __launch_bounds__(WIDEN_THREADS) k_widen(i64 E, int nen, const int32_t* __restrict__ elems,
                                                         const double* __restrict__ centres,
                                                         const double* __restrict__ nodes,
                                                         const i64* __restrict__ ne_off,
                                                         const int32_t* __restrict__ ne_elem, int strategy,
                                                         WidenOut* out) {
    // min x, min y, min d, max x, max y, max d
    unsigned long long v[6] = {~0ull, ~0ull, ~0ull, 0ull, 0ull, 0ull};
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < E * nen; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / nen;
        const int i = int(t % nen);
        const int32_t node = elems[t];
        const unsigned long long bx = ordered_bits(nodes[2 * i64(node)]), by = ordered_bits(nodes[2 * i64(node) + 1]);
        v[0] = bx < v[0] ? bx : v[0];
        v[1] = by < v[1] ? by : v[1];
        v[3] = bx > v[3] ? bx : v[3];
        v[4] = by > v[4] ? by : v[4];
        if (strategy == NLGPU_EXPAND_NO) continue;
        const double cx = centres[2 * e], cy = centres[2 * e + 1];
        for (i64 k = ne_off[node]; k < ne_off[node + 1]; ++k) {
            const int32_t a = ne_elem[k];
            const double zx = cx - centres[2 * i64(a)], zy = cy - centres[2 * i64(a) + 1];
            const double d = zx * zx + zy * zy;
            const unsigned long long db = (unsigned long long)__double_as_longlong(d);   // d >= 0: bits order as values
            if (strategy == NLGPU_EXPAND_MAX) v[5] = db > v[5] ? db : v[5];
            else if (strategy == NLGPU_EXPAND_MIN) v[2] = db < v[2] ? db : v[2];
            else if (a >= e) {
                // count the unordered pair once: at the first local node of e shared with a
                bool first = true;
                for (int i2 = 0; i2 < i && first; ++i2) {
                    const int32_t n2 = elems[e * nen + i2];
                    for (i64 k2 = ne_off[n2]; k2 < ne_off[n2 + 1]; ++k2)
                        if (ne_elem[k2] == a) { first = false; break; }
                }
                if (first) { atomicAdd(&out->sum, sqrt(d)); atomicAdd(&out->count, 1ull); }
            }
        }
    }
    unsigned long long* mins[3] = {&out->bbox[0], &out->bbox[1], strategy == NLGPU_EXPAND_MIN ? &out->dmin : nullptr};
    unsigned long long* maxs[3] = {&out->bbox[2], &out->bbox[3], strategy == NLGPU_EXPAND_MAX ? &out->dmax : nullptr};
    block_min_max(v, mins, maxs);
}

struct Grid {
    double left, down, inv_dummy;
    double maxr, R0, R1;
    i64 rows, cols;
    int n;   // powered-distance exponent
    // FP32 pre-test (n = 2): a candidate whose FP32 distance is farther than
    // tau from 1 is decided by it; the others by the FP64 test
    int filter;
    float inv_r0, inv_r1, tau;
};

// centres rounded to FP32 for the pre-test
__global__ void k_centres32(i64 E, const double* __restrict__ centres, float2* __restrict__ c32) {
    for (i64 e = blockIdx.x * i64(blockDim.x) + threadIdx.x; e < E; e += i64(gridDim.x) * blockDim.x)
        c32[e] = make_float2(float(centres[2 * e]), float(centres[2 * e + 1]));
}

__device__ __forceinline__ void cell_of(const Grid& g, double cx, double cy, i64& row, i64& col) {
    const double fx = (cx - g.left) / g.maxr, fy = (cy - g.down) / g.maxr;
    row = fx > 0.0 ? i64((unsigned long long)fx) : 0;   // centres lie inside the node box
    col = fy > 0.0 ? i64((unsigned long long)fy) : 0;
    row = row < g.rows ? row : g.rows - 1;
    col = col < g.cols ? col : g.cols - 1;
}

__global__ void k_cell_count(i64 E, const double* __restrict__ centres, Grid g, int32_t* __restrict__ cell,
                             i64* __restrict__ count) {
    for (i64 e = blockIdx.x * i64(blockDim.x) + threadIdx.x; e < E; e += i64(gridDim.x) * blockDim.x) {
        i64 r, c;
        cell_of(g, centres[2 * e], centres[2 * e + 1], r, c);
        const i64 id = r * g.cols + c;
        cell[e] = int32_t(id);
        atomicAdd(reinterpret_cast<unsigned long long*>(count + id), 1ull);
    }
}

__global__ void k_cell_fill(i64 E, const int32_t* __restrict__ cell, const i64* __restrict__ off,
                            i64* __restrict__ cursor, int32_t* __restrict__ unsorted) {
    for (i64 e = blockIdx.x * i64(blockDim.x) + threadIdx.x; e < E; e += i64(gridDim.x) * blockDim.x) {
        const int32_t id = cell[e];
        const i64 slot = atomicAdd(reinterpret_cast<unsigned long long*>(cursor + id), 1ull);
        unsorted[off[id] + slot] = int32_t(e);
    }
}

// Each cell's elements by increasing number: rank = number of smaller ids.
__global__ void k_cell_rank(i64 n_cells, const i64* __restrict__ off, const int32_t* __restrict__ unsorted,
                            int32_t* __restrict__ sorted) {
    for (i64 c = blockIdx.x; c < n_cells; c += gridDim.x) {
        const i64 b = off[c], e = off[c + 1];
        for (i64 k = b + threadIdx.x; k < e; k += blockDim.x) {
            const int32_t v = unsorted[k];
            i64 rank = 0;
            for (i64 m = b; m < e; ++m) rank += unsorted[m] < v;
            sorted[b + rank] = v;
        }
    }
}

__device__ __forceinline__ double powered(double z0, double z1, int n) {
    if (n == 2) return z0 * z0 + z1 * z1;
    if (n == 1) return fabs(z0) + fabs(z1);
    return pow(fabs(z0), double(n)) + pow(fabs(z1), double(n));
}

// Warp per element: count (list == nullptr) or write the neighbour list.
// The reference's test -- sum of ((c_e - c_f) / R)^n <= 1 in FP64 -- is
// applied to the candidates whose FP32 distance lies within tau of 1 (with
// n = 2; tau bounds the FP32 error from above, so the lists are the FP64
// test's); GB300's FP64 pipe made the two FP64 divisions per candidate the
// kernel's bound.
__global__ void k_neighbours(i64 E, const double* __restrict__ centres, const float2* __restrict__ c32, Grid g,
                             const int32_t* __restrict__ cell, const i64* __restrict__ cell_off,
                             const int32_t* __restrict__ cell_elems, i64* __restrict__ counts,
                             const i64* __restrict__ offsets, int32_t* __restrict__ list) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 e = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; e < E; e += warps) {
        const double cx = centres[2 * e], cy = centres[2 * e + 1];
        const float2 me = c32[e];
        const i64 id = cell[e];
        const i64 row = id / g.cols, col = id % g.cols;
        i64 found = 0;
        i64 out = list ? offsets[e] : 0;
        const i64 r0 = row ? row - 1 : row, r1 = row != g.rows - 1 ? row + 2 : row + 1;
        const i64 c0 = col ? col - 1 : col, c1 = col != g.cols - 1 ? col + 2 : col + 1;
        for (i64 i = r0; i < r1; ++i)
            for (i64 j = c0; j < c1; ++j) {
                const i64 cb = cell_off[i * g.cols + j], ce = cell_off[i * g.cols + j + 1];
                for (i64 k = cb; k < ce; k += 32) {
                    bool hit = false;
                    int32_t f = -1;
                    if (k + lane < ce) {
                        f = cell_elems[k + lane];
                        bool decided = false;
                        if (g.filter) {
                            const float2 cf = c32[f];
                            const float z0 = (me.x - cf.x) * g.inv_r0, z1 = (me.y - cf.y) * g.inv_r1;
                            const float d32 = z0 * z0 + z1 * z1;
                            if (d32 < 1.0f - g.tau) { hit = true; decided = true; }
                            else if (d32 > 1.0f + g.tau) { hit = false; decided = true; }
                        }
                        if (!decided) {
                            const double z0 = (cx - centres[2 * i64(f)]) / g.R0;
                            const double z1 = (cy - centres[2 * i64(f) + 1]) / g.R1;
                            hit = powered(z0, z1, g.n) <= 1.0;
                        }
                    }
                    const unsigned mask = __ballot_sync(0xffffffffu, hit);
                    if (list && hit) list[out + __popc(mask & ((1u << lane) - 1u))] = f;
                    out += __popc(mask);
                    found += __popc(mask);
                }
            }
        if (!list && lane == 0) counts[e] = found;
    }
}

}  // namespace

void find_neighbours(Ctx& ctx, int strategy) {
    NL_REQUIRE(ctx.mesh_ready && ctx.model_ready, NLGPU_ERR_STATE, "mesh and model must be set before the neighbour search");
    NL_REQUIRE(strategy >= NLGPU_EXPAND_NO && strategy <= NLGPU_EXPAND_MEAN, NLGPU_ERR_ARG, "unknown expanding strategy");
    const i64 E = ctx.n_elems;
    const int nen = ctx.basis.nen;
    WidenOut init{};
    init.dmax = 0ull;
    init.dmin = 0x7ff0000000000000ull;   // +inf
    init.bbox[0] = init.bbox[1] = ~0ull;
    init.bbox[2] = init.bbox[3] = 0ull;
    auto* dw = reinterpret_cast<WidenOut*>(ctx.scratch_bytes(sizeof(WidenOut)));
    NL_CUDA(cudaMemcpyAsync(dw, &init, sizeof init, cudaMemcpyHostToDevice, ctx.stream));
    NL_LAUNCH(k_widen, grid_for(E * nen, 256), 256, 0, ctx.stream, E, nen, ctx.elems.p, ctx.centres.p, ctx.nodes.p,
              ctx.ne_off.p, ctx.ne_elem.p, strategy, dw);
    WidenOut w{};
    NL_CUDA(cudaMemcpyAsync(&w, dw, sizeof w, cudaMemcpyDeviceToHost, ctx.stream));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    double add = 0.0;
    if (strategy == NLGPU_EXPAND_MAX) { double d; std::memcpy(&d, &w.dmax, sizeof d); add = std::sqrt(d); }
    else if (strategy == NLGPU_EXPAND_MIN) { double d; std::memcpy(&d, &w.dmin, sizeof d); add = std::sqrt(d); }
    else if (strategy == NLGPU_EXPAND_MEAN) add = w.count ? w.sum / double(w.count) : 0.0;
    const double R0 = ctx.model.r[0] + add, R1 = ctx.model.r[1] + add;
    ctx.search_r[0] = R0; ctx.search_r[1] = R1;
    ctx.strategy = strategy;
    ctx.noff.resize(size_t(E + 1));
    if (R0 <= 0.0 || R1 <= 0.0) {   // the reference skips the group with a warning
        ctx.noff.zero(ctx.stream);
        ctx.nlist.resize(0);
        ctx.pairs = 0;
        ctx.neighbours_ready = true;
        return;
    }
    Grid g{};
    g.left = from_ordered_bits(w.bbox[0]);
    g.down = from_ordered_bits(w.bbox[1]);
    const double right = from_ordered_bits(w.bbox[2]), up = from_ordered_bits(w.bbox[3]);
    g.maxr = std::max(R0, R1);
    g.R0 = R0; g.R1 = R1; g.n = ctx.model.n;
    g.rows = i64(size_t((right - g.left) / g.maxr) + 1);
    g.cols = i64(size_t((up - g.down) / g.maxr) + 1);
    // FP32 pre-test bound: centres rounded to FP32 (|c| <= M), the
    // difference, the scaling by 1/R and the square sum each add relative
    // errors of 2^-24; near the boundary (|z| <= 1) the FP32 distance is
    // within (19 + 8 M / R) 2^-24 of the exact one, doubled here
    const double M = std::max(std::max(std::fabs(g.left), std::fabs(right)), std::max(std::fabs(g.down), std::fabs(up)));
    const double tau = (32.0 + 16.0 * M / std::min(R0, R1)) * std::ldexp(1.0, -24);
    g.filter = ctx.model.n == 2 && tau < 0.25;
    g.inv_r0 = float(1.0 / R0);
    g.inv_r1 = float(1.0 / R1);
    g.tau = float(tau);
    ctx.centres32.reserve(size_t(E));
    NL_LAUNCH(k_centres32, grid_for(E, 256), 256, 0, ctx.stream, E, ctx.centres.p, ctx.centres32.p);
    const i64 n_cells = g.rows * g.cols;
    // scratch: cell id per element, cell offsets, cursors, unsorted and sorted cell lists
    dbuf<int32_t> cell, unsorted, sorted;
    dbuf<i64> cell_off, cursor;
    cell.resize(size_t(E)); unsorted.resize(size_t(E)); sorted.resize(size_t(E));
    cell_off.resize(size_t(n_cells + 1)); cursor.resize(size_t(n_cells));
    cell_off.zero(ctx.stream); cursor.zero(ctx.stream);
    NL_LAUNCH(k_cell_count, grid_for(E, 256), 256, 0, ctx.stream, E, ctx.centres.p, g, cell.p, cell_off.p);
    exclusive_scan(ctx, cell_off.p, cell_off.p, n_cells + 1, nullptr);
    NL_LAUNCH(k_cell_fill, grid_for(E, 256), 256, 0, ctx.stream, E, cell.p, cell_off.p, cursor.p, unsorted.p);
    NL_LAUNCH(k_cell_rank, unsigned(std::min<i64>(n_cells, 65535)), 256, 0, ctx.stream, n_cells, cell_off.p,
              unsorted.p, sorted.p);
    // count, scan, fill
    ctx.i64_scratch_b.reserve(size_t(E + 1));
    i64* counts = ctx.i64_scratch_b.p;
    NL_CUDA(cudaMemsetAsync(counts + E, 0, sizeof(i64), ctx.stream));
    const unsigned blocks = grid_for(E * 32, 256, 152 * 64);
    NL_LAUNCH(k_neighbours, blocks, 256, 0, ctx.stream, E, ctx.centres.p, ctx.centres32.p, g, cell.p, cell_off.p,
              sorted.p, counts, nullptr, nullptr);
    i64 total = 0;
    exclusive_scan(ctx, counts, ctx.noff.p, E + 1, &total);
    ctx.nlist.resize(size_t(total));
    NL_LAUNCH(k_neighbours, blocks, 256, 0, ctx.stream, E, ctx.centres.p, ctx.centres32.p, g, cell.p, cell_off.p,
              sorted.p, nullptr, ctx.noff.p, ctx.nlist.p);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));   // scratch buffers are freed on return
    ctx.pairs = total;
    ctx.neighbours_ready = true;
}

}  // namespace nlgpu
