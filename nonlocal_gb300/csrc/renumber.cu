// Node renumbering: the Cuthill-McKee order of the node graph
// (mesh::utils::cuthill_mckee, libraries/mesh/mesh_2d/cuthill_mckee.hpp) and
// the renumbering of a mesh by a permutation (mesh_2d::renumbering,
// mesh_container_2d.hpp:333-350).
//
// Node graph.  In the reference, node r's adjacency lists the nodes met by
// the mesh_run sweep of r (for every element eL containing r, in element
// order; for every neighbour eNL of eL, in neighbour-list order, or eL itself
// for a local graph; for every node of that element, in local order), each
// once and without r, in order of first meeting.  Here a warp owns a node:
// it walks the same sequence 32 candidates at a time, keeps the first lane of
// equal candidates (__match_any_sync), tests and sets a bitmap of the node
// numbers seen (shared memory over the node's window of numbers, or a global
// per-warp bitmap when the window is too wide), and emits new nodes in order
// with a ballot.  Two passes: degrees, then the lists at scanned offsets.
//
// Order.  The reference visits each layer of the breadth-first search in the
// iteration order of a std::unordered_set and gives the unvisited neighbours
// of each node numbers in order of degree (a std::multimap: equal degrees in
// adjacency order).  The layer order is a property of the standard library's
// hashed container, so the ordering loop runs on the host with the same
// container and the same sequence of operations (construct from the start
// node, clear, insert in numbering order, swap), which gives the reference's
// permutation exactly; its cost is one pass over the adjacency lists.
#include "common.cuh"

#include <algorithm>
#include <unordered_set>

namespace nlgpu {

namespace {

constexpr int NG_WARPS = 4;                    // warps (nodes in flight) per CTA
constexpr int NG_SMEM_WORDS = 12288;           // bitmap words per warp in shared memory (48 KB)

struct GraphArgs {
    i64 n;
    bool local_graph;
    const int32_t* elems;
    const i64* ne_off;
    const int32_t* ne_elem;
    const i64* noff;
    const int32_t* nlist;
    const int32_t* emin;
    const int32_t* emax;
    const int32_t* lo;        // window start per node
    int words;                // bitmap words per warp
    uint32_t* global_bits;    // per-warp bitmaps when the window does not fit shared memory
    i64* degree;              // count pass
    const i64* offsets;       // fill pass
    int32_t* adjacency;
};

// smallest / largest node number over the elements a node's candidates come
// from: per element (over its neighbours, or itself), then per node
__global__ void k_graph_element_window(GraphArgs a, i64 E, int32_t* elo, int32_t* ehi) {
    const i64 e = i64(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int32_t l = a.emin[e], h = a.emax[e];
    if (!a.local_graph)
        for (i64 m = a.noff[e]; m < a.noff[e + 1]; ++m) {
            const int32_t o = a.nlist[m];
            l = min(l, a.emin[o]); h = max(h, a.emax[o]);
        }
    elo[e] = l; ehi[e] = h;
}

__global__ void k_graph_window(GraphArgs a, const int32_t* elo, const int32_t* ehi, int32_t* lo, int* max_width) {
    const i64 r = i64(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= a.n) return;
    int32_t l = int32_t(r), h = int32_t(r);
    for (i64 k = a.ne_off[r]; k < a.ne_off[r + 1]; ++k) {
        const int32_t e = a.ne_elem[k];
        l = min(l, elo[e]); h = max(h, ehi[e]);
    }
    lo[r] = l;
    atomicMax(max_width, h - l + 1);
}

template<int NEN, bool FILL>
__global__ void __launch_bounds__(NG_WARPS * 32) k_node_graph(GraphArgs a) {
    extern __shared__ uint32_t sh_bits[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const i64 gwarp = i64(blockIdx.x) * NG_WARPS + warp, nwarps = i64(gridDim.x) * NG_WARPS;
    uint32_t* bits = a.global_bits ? a.global_bits + gwarp * a.words : sh_bits + size_t(warp) * a.words;
    if (!a.global_bits)
        for (int w = lane; w < a.words; w += 32) bits[w] = 0u;
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    for (i64 r = gwarp; r < a.n; r += nwarps) {
        const int32_t lo = a.lo[r];
        i64 pos = FILL ? a.offsets[r] : 0;
        const i64 start = pos;
        int32_t hi = lo;
        for (i64 k = a.ne_off[r]; k < a.ne_off[r + 1]; ++k) {
            const int32_t eL = a.ne_elem[k];
            const i64 first = a.local_graph ? 0 : a.noff[eL];
            const i64 total = (a.local_graph ? 1 : a.noff[eL + 1] - first) * NEN;
            for (i64 base = 0; base < total; base += 32) {
                const i64 f = base + lane;
                const bool valid = f < total;
                int32_t v = -1 - lane;
                if (valid) {
                    const int32_t e = a.local_graph ? eL : a.nlist[first + f / NEN];
                    v = a.elems[i64(e) * NEN + f % NEN];
                }
                const unsigned same = __match_any_sync(0xffffffffu, v);
                bool fresh = false;
                uint32_t word = 0, bit = 0;
                if (valid && __ffs(same) - 1 == lane && v != int32_t(r)) {
                    word = uint32_t(v - lo) >> 5;
                    bit = 1u << ((v - lo) & 31);
                    fresh = !(bits[word] & bit);
                }
                const unsigned ballot = __ballot_sync(0xffffffffu, fresh);
                if (fresh) {
                    atomicOr(&bits[word], bit);
                    if (FILL) a.adjacency[pos + __popc(ballot & lt)] = v;
                    hi = max(hi, v);
                }
                pos += __popc(ballot);
                __syncwarp();
            }
        }
        if (!FILL && lane == 0) a.degree[r] = pos - start;
        // clear the words this node may have touched
        hi = __reduce_max_sync(0xffffffffu, hi);
        for (int32_t w = lane; w <= (hi - lo) >> 5; w += 32) bits[w] = 0u;
        __syncwarp();
    }
}

__global__ void k_renumber_nodes(i64 n, const int32_t* __restrict__ perm, const double* __restrict__ in,
                                 double* __restrict__ out) {
    const i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[2 * i64(perm[i])] = in[2 * i];
    out[2 * i64(perm[i]) + 1] = in[2 * i + 1];
}

__global__ void k_renumber_values(i64 n, const int32_t* __restrict__ perm, const double* __restrict__ in,
                                  double* __restrict__ out) {
    const i64 i = i64(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[perm[i]] = in[i];
}

__global__ void k_renumber_indices(i64 count, const int32_t* __restrict__ perm, int32_t* __restrict__ idx) {
    const i64 k = i64(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < count) idx[k] = perm[idx[k]];
}

template<int NEN>
void launch_graph(Ctx& ctx, const GraphArgs& a, bool fill, unsigned grid, size_t smem) {
    if (fill) NL_LAUNCH((k_node_graph<NEN, true>), grid, NG_WARPS * 32, smem, ctx.stream, a);
    else NL_LAUNCH((k_node_graph<NEN, false>), grid, NG_WARPS * 32, smem, ctx.stream, a);
}

}  // namespace

void node_graph(Ctx& ctx, bool local_graph, std::vector<i64>& offsets, std::vector<int32_t>& adjacency) {
    const i64 n = ctx.n_nodes;
    const int nen = ctx.basis.nen;
    GraphArgs a{};
    a.n = n; a.local_graph = local_graph;
    a.elems = ctx.elems.p; a.ne_off = ctx.ne_off.p; a.ne_elem = ctx.ne_elem.p;
    a.noff = ctx.noff.p; a.nlist = ctx.nlist.p;
    a.emin = ctx.elem_minnode.p; a.emax = ctx.elem_maxnode.p;
    const i64 E = ctx.n_elems;
    dbuf<int32_t> lo, elo, ehi;
    dbuf<int> width;
    lo.resize(size_t(n)); elo.resize(size_t(E)); ehi.resize(size_t(E));
    width.resize(1);
    width.zero(ctx.stream);
    a.lo = lo.p;
    NL_LAUNCH(k_graph_element_window, grid_for(E, 256, i64(1) << 30), 256, 0, ctx.stream, a, E, elo.p, ehi.p);
    NL_LAUNCH(k_graph_window, grid_for(n, 256, i64(1) << 30), 256, 0, ctx.stream, a, elo.p, ehi.p, lo.p, width.p);
    int max_width = 0;
    width.download(&max_width, 1, ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    a.words = (max_width + 31) / 32 + 1;
    const unsigned grid = unsigned(std::min<i64>((n + NG_WARPS - 1) / NG_WARPS, 152 * 8));
    dbuf<uint32_t> gbits;
    size_t smem = 0;
    if (a.words <= NG_SMEM_WORDS) {
        smem = size_t(a.words) * NG_WARPS * sizeof(uint32_t);
    } else {
        gbits.resize(size_t(grid) * NG_WARPS * size_t(a.words));
        gbits.zero(ctx.stream);
        a.global_bits = gbits.p;
    }
    auto set_smem = [&](auto kernel) {
        if (smem > 48 * 1024) NL_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    };
    if (nen == 4) { set_smem(k_node_graph<4, false>); set_smem(k_node_graph<4, true>); }
    else { set_smem(k_node_graph<8, false>); set_smem(k_node_graph<8, true>); }
    dbuf<i64> deg;
    deg.resize(size_t(n + 1));
    deg.zero(ctx.stream);
    a.degree = deg.p;
    if (nen == 4) launch_graph<4>(ctx, a, false, grid, smem); else launch_graph<8>(ctx, a, false, grid, smem);
    i64 total = 0;
    exclusive_scan(ctx, deg.p, deg.p, n + 1, &total);
    NL_REQUIRE(total < (i64(1) << 40), NLGPU_ERR_UNSUPPORTED, "node graph too large");
    dbuf<int32_t> adj;
    adj.resize(size_t(std::max<i64>(total, 1)));
    a.offsets = deg.p;
    a.adjacency = adj.p;
    if (nen == 4) launch_graph<4>(ctx, a, true, grid, smem); else launch_graph<8>(ctx, a, true, grid, smem);
    offsets.resize(size_t(n + 1));
    adjacency.resize(size_t(total));
    deg.download(offsets.data(), size_t(n + 1), ctx.stream);
    if (total) adj.download(adjacency.data(), size_t(total), ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
}

std::vector<i64> cuthill_mckee_order(const std::vector<i64>& off, const std::vector<int32_t>& adj) {
    const i64 n = i64(off.size()) - 1;
    std::vector<i64> perm(size_t(n), -1);
    if (n == 0) return perm;
    auto degree = [&](i64 v) { return off[size_t(v) + 1] - off[size_t(v)]; };
    // the first node of smallest degree (cuthill_mckee.hpp:118-127)
    i64 start = 0;
    for (i64 v = 1; v < n; ++v)
        if (degree(v) < degree(start)) start = v;
    i64 next_number = 0;
    perm[size_t(start)] = next_number++;
    std::unordered_set<i64> layer{start}, next_layer;
    std::vector<std::pair<i64, i64>> fresh;   // (degree, node) in adjacency order
    while (next_number < n) {
        NL_REQUIRE(!layer.empty(), NLGPU_ERR_UNSUPPORTED, "node graph is not connected");
        next_layer.clear();
        for (const i64 v : layer) {
            fresh.clear();
            for (i64 k = off[size_t(v)]; k < off[size_t(v) + 1]; ++k)
                if (const i64 w = adj[size_t(k)]; perm[size_t(w)] < 0) fresh.emplace_back(degree(w), w);
            std::stable_sort(fresh.begin(), fresh.end(),
                             [](const auto& x, const auto& y) { return x.first < y.first; });
            for (const auto& [d, w] : fresh) {
                next_layer.emplace(w);
                perm[size_t(w)] = next_number++;
            }
        }
        std::swap(layer, next_layer);
    }
    return perm;
}

void renumber_mesh(Ctx& ctx, const std::vector<int32_t>& perm) {
    const i64 n = ctx.n_nodes;
    dbuf<int32_t> p;
    p.upload(perm.data(), perm.size(), ctx.stream);
    dbuf<double> nodes;
    nodes.resize(size_t(2 * n));
    NL_LAUNCH(k_renumber_nodes, grid_for(n, 256, i64(1) << 30), 256, 0, ctx.stream, n, p.p, ctx.nodes.p, nodes.p);
    NL_CUDA(cudaMemcpyAsync(ctx.nodes.p, nodes.p, size_t(2 * n) * sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
    const i64 ne = ctx.n_elems * ctx.basis.nen;
    NL_LAUNCH(k_renumber_indices, grid_for(ne, 256, i64(1) << 30), 256, 0, ctx.stream, ne, p.p, ctx.elems.p);
    for (BoundaryGroup& g : ctx.groups) {
        const i64 m = g.n_edges * g.nen;
        if (m) NL_LAUNCH(k_renumber_indices, grid_for(m, 256, i64(1) << 30), 256, 0, ctx.stream, m, p.p, g.edges.p);
    }
    if (ctx.dirichlet_override.n) {
        NL_LAUNCH(k_renumber_values, grid_for(n, 256, i64(1) << 30), 256, 0, ctx.stream, n, p.p,
                  ctx.dirichlet_override.p, nodes.p);
        NL_CUDA(cudaMemcpyAsync(ctx.dirichlet_override.p, nodes.p, size_t(n) * sizeof(double),
                                cudaMemcpyDeviceToDevice, ctx.stream));
    }
    mesh_init(ctx);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
}

}  // namespace nlgpu
