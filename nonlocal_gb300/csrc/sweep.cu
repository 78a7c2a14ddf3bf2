// Level-scheduled triangular sweep fed by TMA bulk copies, with the solved
// values kept in a shared-memory ring.
//
// A sweep solves y[row] = (in[row] - sum_k L[row][k] y[k]) / L[row][row] level
// by level (rows of one level depend only on earlier levels).  Everything the
// sweep reads is laid out per level, contiguously, in level order:
//   * a "level block": off-diagonal values [w][cntp], inverse diagonal [cntp]
//     and dependency positions [w][cntp] (int32 padded level-order position,
//     -1 for padding), padded to 16 bytes;
//   * the right-hand side, pre-gathered into level order (padded positions).
// One CTA walks the levels.  Thread 0 keeps STAGES levels in flight with
// cp.async.bulk (one copy per block, one per right-hand-side chunk) completing
// on an mbarrier per stage; the other threads wait on the stage's barrier
// (bounded spin), solve their row and put the value into a ring of RING
// values in shared memory at (padded position mod RING; RING = 16384 FP32 or
// 4096 FP64 entries) and into the level-ordered output in global memory.
// The block stores, per entry, the shared-memory slot its value is read from:
// the ring slot for a dependency within RING positions of the end of its
// level, the zero slot RING for padding, or a per-stage "far" slot after the
// ring for the few older dependencies, whose values the producer warp copies
// from the global output (finished levels earlier) when it issues the stage.
// So the compute threads only ever read shared memory.  Small gather/scatter
// kernels convert between level order and node order around the sweeps.
#include "common.cuh"

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace nlgpu {

namespace {

constexpr int SW_THREADS = 256;
constexpr int SW_STAGES = 6;
// shared-memory ring of solved values: 16384 FP32 or 4096 FP64 entries (64 / 32 KB)
constexpr int ring_for_bytes(int es) { return es == 4 ? 16384 : 4096; }
template<class T> constexpr int ring_size() { return ring_for_bytes(int(sizeof(T))); }
constexpr int SW_MAX_WIDTH = 16;          // widest level the unrolled row loop handles
constexpr unsigned long long SW_WAIT_LIMIT_NS = 2000000000ull;   // a stage wait gives up after 2 s

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

template<class T>
struct SweepArgs {
    i64 n_levels;
    const ushort4* meta;      // [L] rows, padded rows (multiple of 8), width, 0
    const unsigned char* blocks;
    const T* in;              // right-hand side in padded level order
    T* out;                   // solution in padded level order
    int stage_bytes;          // bytes of one stage (block + rhs chunk)
    int nct;                  // compute threads (a multiple of 32, <= SW_THREADS)
    int farmax;               // far slots per stage after the ring
    const int32_t* far_off;   // [L + 1]
    const int32_t* far_pos;   // positions of the far dependencies, level by level
    int* error;
    const double* partials;   // optional CG state: skip after convergence
    const double* flags;
    double tol2;
};

// nct compute threads (one row each per pass) plus one producer warp
// that only issues the copies: a stage is refilled once the compute threads
// have released it (empty barrier), so the copy issue is off the critical
// path of the level chain.  MAXW bounds the level width so the dependency
// loads of a row are unrolled and issued together.
template<class T, int MAXW>
__global__ void __launch_bounds__(SW_THREADS + 32) k_sweep_tma(SweepArgs<T> a) {
    extern __shared__ __align__(128) unsigned char smem[];
    T* ring = reinterpret_cast<T*>(smem);
    constexpr int RING = ring_size<T>();
    unsigned char* stage_base = smem + ((sizeof(T) * (RING + 1 + SW_STAGES * a.farmax) + 127) / 128) * 128;
    uint64_t* bars = reinterpret_cast<uint64_t*>(stage_base + size_t(a.stage_bytes) * SW_STAGES);
    uint64_t* empty = bars + SW_STAGES;
    __shared__ double sh[40];
    __shared__ int skip;
    if (a.flags) {
        // converged CG state: every thread takes the same early return
        double v = 0.0;
        for (int k = threadIdx.x; k < RED_BLOCKS; k += blockDim.x) v += a.partials[P_RR * RED_BLOCKS + k];
        v = warp_sum(v);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double rr = 0.0;
            for (int w = 0; w < int(blockDim.x >> 5); ++w) rr += sh[w];
            skip = (a.flags[S_DONE] != 0.0) || (rr <= a.tol2 * a.flags[S_BB]);
        }
        __syncthreads();
        if (skip) return;
    }
    // per-level (rows, padded rows, width) for every level, read once
    ushort4* meta = reinterpret_cast<ushort4*>(empty + SW_STAGES);
    __shared__ int abort_flag;
    for (i64 l = threadIdx.x; l < a.n_levels; l += blockDim.x) meta[l] = a.meta[l];
    for (int k = threadIdx.x; k <= RING; k += blockDim.x) ring[k] = T(0);
    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < SW_STAGES; ++s) { mbar_init(&bars[s], 1); mbar_init(&empty[s], 1); }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    const int L = int(a.n_levels);
    if (int(threadIdx.x) >= a.nct) {
        // producer warp: lane 0 walks the level blocks and right-hand-side chunks in order
        if (int(threadIdx.x) != a.nct) return;
        i64 issue_block = 0, issue_pos = 0;
        for (int l = 0; l < L; ++l) {
            const int s = l % SW_STAGES;
            if (l >= SW_STAGES) {   // wait until the compute threads released level l - STAGES
                const uint32_t par = uint32_t((l / SW_STAGES - 1) & 1);
                if (!mbar_try_wait(&empty[s], par)) {
                    const unsigned long long t0 = globaltimer_ns();
                    while (!mbar_try_wait(&empty[s], par))
                        if (globaltimer_ns() - t0 > SW_WAIT_LIMIT_NS) { atomicExch(a.error, 1); return; }
                }
            }
            // dependencies older than the ring: prefetch their (long finished) values
            // from the global output into this stage's far slots; the arrive below
            // publishes them with the stage
            for (int j = a.far_off[l], f = 0; j < a.far_off[l + 1]; ++j, ++f)
                ring[RING + 1 + s * a.farmax + f] = __ldcg(a.out + a.far_pos[j]);
            unsigned char* dst = stage_base + size_t(s) * a.stage_bytes;
            const int cp = meta[l].y, w = meta[l].z;
            const uint32_t block_bytes = uint32_t((size_t(w) * cp * (sizeof(T) + 4) + size_t(cp) * sizeof(T) + 15) / 16 * 16);
            const uint32_t rhs_bytes = uint32_t(size_t(cp) * sizeof(T));
            mbar_expect_tx(&bars[s], block_bytes + rhs_bytes);
            bulk_g2s(dst, a.blocks + issue_block, block_bytes, &bars[s]);
            bulk_g2s(dst + block_bytes, a.in + issue_pos, rhs_bytes, &bars[s]);
            issue_block += block_bytes;
            issue_pos += cp;
        }
        return;
    }
    int p0 = 0;
    for (int l = 0; l < L; ++l) {
        const int s = l % SW_STAGES;
        const uint32_t parity = uint32_t((l / SW_STAGES) & 1);
        if (!mbar_try_wait(&bars[s], parity)) {
            const unsigned long long t0 = globaltimer_ns();
            while (!mbar_try_wait(&bars[s], parity)) {
                // a wait that gives up still reaches the level barrier below, where
                // every compute thread sees the flag and returns
                if (globaltimer_ns() - t0 > SW_WAIT_LIMIT_NS) { abort_flag = 1; atomicExch(a.error, 1); break; }
            }
        }
        const ushort4 mt = meta[l];
        const int c = mt.x, cp = mt.y, w = mt.z;
        const unsigned char* blk = stage_base + size_t(s) * a.stage_bytes;
        const T* vals = reinterpret_cast<const T*>(blk);
        const T* inv = vals + size_t(w) * cp;
        const int32_t* dep = reinterpret_cast<const int32_t*>(inv + cp);
        const uint32_t block_bytes = uint32_t((size_t(w) * cp * (sizeof(T) + 4) + size_t(cp) * sizeof(T) + 15) / 16 * 16);
        const T* rhs = reinterpret_cast<const T*>(blk + block_bytes);
        for (int t = threadIdx.x; t < c; t += a.nct) {
            // all dependency slots first (ring, prefetched far slot, or the zero slot
            // RING for padding), then the values, then the products
            int32_t d[MAXW];
#pragma unroll
            for (int k = 0; k < MAXW; ++k) d[k] = k < w ? dep[k * cp + t] : RING;
            T y[MAXW];
#pragma unroll
            for (int k = 0; k < MAXW; ++k) y[k] = ring[d[k]];
            T acc = rhs[t];
#pragma unroll
            for (int k = 0; k < MAXW; ++k)
                if (k < w) acc -= vals[k * cp + t] * y[k];
            const T v = acc * inv[t];
            ring[(p0 + t) & (RING - 1)] = v;
            a.out[p0 + t] = v;
        }
        p0 += cp;
        // the level's ring values are visible and stage s is consumed: release it
        asm volatile("bar.sync 1, %0;" ::"r"(a.nct) : "memory");
        if (abort_flag) return;
        if (threadIdx.x == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&empty[s])) : "memory");
        }
    }
}

// level order <-> node order
template<class T, class R>
__global__ void k_gather_scaled(i64 P, const int32_t* __restrict__ row_of, const double* __restrict__ scale,
                                const R* __restrict__ r, T* __restrict__ out) {
    for (i64 p = blockIdx.x * i64(blockDim.x) + threadIdx.x; p < P; p += i64(gridDim.x) * blockDim.x) {
        const int32_t row = row_of[p];
        out[p] = row >= 0 ? T(scale[row] * double(r[row])) : T(0);
    }
}

template<class T>
__global__ void k_transfer(i64 P, const int32_t* __restrict__ row_of_b, const int32_t* __restrict__ ppos_of_row_f,
                           const T* __restrict__ in_f, T* __restrict__ out_b) {
    for (i64 p = blockIdx.x * i64(blockDim.x) + threadIdx.x; p < P; p += i64(gridDim.x) * blockDim.x) {
        const int32_t row = row_of_b[p];
        out_b[p] = row >= 0 ? in_f[ppos_of_row_f[row]] : T(0);
    }
}

template<class T, class Z>
__global__ void k_scatter_scaled(i64 P, const int32_t* __restrict__ row_of, const double* __restrict__ scale,
                                 const T* __restrict__ in, Z* __restrict__ z) {
    for (i64 p = blockIdx.x * i64(blockDim.x) + threadIdx.x; p < P; p += i64(gridDim.x) * blockDim.x) {
        const int32_t row = row_of[p];
        if (row >= 0) z[row] = Z(scale[row] * double(in[p]));
    }
}

// factor values (FP64) into the level blocks, as T; the inverse diagonal is
// formed in FP64 before the conversion
template<class T>
__global__ void k_fill_blocks(i64 count, const i64* __restrict__ dst_off, const i64* __restrict__ src,
                              const double* __restrict__ u, bool invert, unsigned char* __restrict__ blocks) {
    for (i64 k = blockIdx.x * i64(blockDim.x) + threadIdx.x; k < count; k += i64(gridDim.x) * blockDim.x) {
        double v = src[k] >= 0 ? u[src[k]] : 0.0;
        if (invert) v = src[k] >= 0 ? 1.0 / v : 0.0;
        *reinterpret_cast<T*>(blocks + dst_off[k]) = T(v);
    }
}

}  // namespace

// Host construction of a sweep plan from the level structure of a triangular
// matrix (rows by level, entries with their factor value indices).
bool sweep_plan_build(Ctx& ctx, const std::vector<i64>& lev_ptr, const std::vector<int32_t>& rows,
                      const std::vector<i64>& rp, const std::vector<int32_t>& col, const std::vector<i64>& val_index,
                      const std::vector<i64>& diag_pos, SweepPlan& plan) {
    const i64 L = i64(lev_ptr.size()) - 1;
    const i64 n = i64(rows.size());
    std::vector<int32_t> cnt(static_cast<size_t>(L)), cntp(static_cast<size_t>(L)), width(static_cast<size_t>(L));
    std::vector<i64> ppos(static_cast<size_t>(L + 1), 0), block_off(static_cast<size_t>(L));
    std::vector<int32_t> ppos_of_row(static_cast<size_t>(n));
    for (i64 l = 0; l < L; ++l) {
        const int c = int(lev_ptr[size_t(l) + 1] - lev_ptr[size_t(l)]);
        int w = 0;
        for (i64 t = lev_ptr[size_t(l)]; t < lev_ptr[size_t(l) + 1]; ++t) {
            const int32_t r = rows[size_t(t)];
            w = std::max(w, int(rp[size_t(r) + 1] - rp[size_t(r)] - 1));
        }
        cnt[size_t(l)] = c;
        cntp[size_t(l)] = (c + 7) / 8 * 8;
        width[size_t(l)] = w;
        ppos[size_t(l) + 1] = ppos[size_t(l)] + cntp[size_t(l)];
        for (int t = 0; t < c; ++t) ppos_of_row[size_t(rows[size_t(lev_ptr[size_t(l)] + t)])] = int32_t(ppos[size_t(l)] + t);
    }
    const i64 P = ppos[size_t(L)];
    // Level blocks for one value size es (8: FP64 sweeps, 4: FP32 sweeps); the
    // factor-value sources (val_src, inv_src) are the same for both.
    std::vector<i64> val_src, inv_src;
    // farthest dependency, counted from the end of its level (reported), and the
    // widest level (compute threads)
    i64 max_dist = 0;
    int max_rows = 0;
    for (i64 l = 0; l < L; ++l) {
        max_rows = std::max(max_rows, cnt[size_t(l)]);
        for (i64 t = lev_ptr[size_t(l)]; t < lev_ptr[size_t(l) + 1]; ++t) {
            const int32_t r = rows[size_t(t)];
            for (i64 s = rp[size_t(r)]; s < rp[size_t(r) + 1]; ++s)
                if (s != diag_pos[size_t(r)])
                    max_dist = std::max(max_dist, ppos[size_t(l) + 1] - ppos_of_row[size_t(col[size_t(s)])]);
        }
    }
    plan.threads = std::min(SW_THREADS, std::max(32, (max_rows + 31) / 32 * 32));
    auto layout = [&](int es, SweepLayout& out, std::vector<unsigned char>& dep_bytes, std::vector<i64>& val_dst,
                      std::vector<i64>& inv_dst, std::vector<i64>& block_off_out, bool record_src) {
        i64 bytes = 0;
        int max_stage = 0;
        const int ring = ring_for_bytes(es);
        // dependencies beyond the ring (counted from the end of their level): per
        // level the distinct positions the producer prefetches into far slots
        std::vector<int32_t> far_off(static_cast<size_t>(L + 1), 0), far_pos;
        std::vector<std::vector<i64>> far_of(static_cast<size_t>(L));
        out.farmax = 0;
        for (i64 l = 0; l < L; ++l) {
            auto& f = far_of[size_t(l)];
            for (i64 t = lev_ptr[size_t(l)]; t < lev_ptr[size_t(l) + 1]; ++t) {
                const int32_t r = rows[size_t(t)];
                for (i64 s = rp[size_t(r)]; s < rp[size_t(r) + 1]; ++s) {
                    if (s == diag_pos[size_t(r)]) continue;
                    const i64 dp = ppos_of_row[size_t(col[size_t(s)])];
                    if (ppos[size_t(l) + 1] - dp > ring) f.push_back(dp);
                }
            }
            std::sort(f.begin(), f.end());
            f.erase(std::unique(f.begin(), f.end()), f.end());
            out.farmax = std::max(out.farmax, int(f.size()));
            far_off[size_t(l) + 1] = far_off[size_t(l)] + int32_t(f.size());
            for (const i64 dp : f) far_pos.push_back(int32_t(dp));
        }
        if (far_pos.empty()) far_pos.push_back(0);   // never read; keeps the buffer non-empty
        out.far_off.upload(far_off.data(), far_off.size(), ctx.stream);
        out.far_pos.upload(far_pos.data(), far_pos.size(), ctx.stream);
        for (i64 l = 0; l < L; ++l) {
            const i64 cp = cntp[size_t(l)], w = width[size_t(l)];
            const i64 blk = (w * cp * (es + 4) + cp * es + 15) / 16 * 16;
            block_off_out[size_t(l)] = bytes;
            bytes += blk;
            max_stage = std::max<int>(max_stage, int(blk + cp * es));
        }
        dep_bytes.assign(static_cast<size_t>(bytes), 0);
        for (i64 l = 0; l < L; ++l) {
            const int c = cnt[size_t(l)], cp = cntp[size_t(l)], w = width[size_t(l)];
            const i64 vbase = block_off_out[size_t(l)];
            const i64 ibase = vbase + i64(w) * cp * es;
            const i64 dbase = ibase + i64(cp) * es;
            for (int t = 0; t < cp; ++t) {
                const bool real = t < c;
                const int32_t r = real ? rows[size_t(lev_ptr[size_t(l)] + t)] : -1;
                inv_dst.push_back(ibase + i64(t) * es);
                if (record_src) inv_src.push_back(real ? val_index[size_t(diag_pos[size_t(r)])] : -1);
                int k = 0;
                if (real)
                    for (i64 s = rp[size_t(r)]; s < rp[size_t(r) + 1]; ++s) {
                        if (s == diag_pos[size_t(r)]) continue;
                        const i64 dp = ppos_of_row[size_t(col[size_t(s)])];
                        int32_t slot = int32_t(dp & (ring - 1));
                        if (ppos[size_t(l) + 1] - dp > ring) {
                            const auto& f = far_of[size_t(l)];
                            const i64 idx = std::lower_bound(f.begin(), f.end(), dp) - f.begin();
                            slot = int32_t(ring + 1 + (l % SW_STAGES) * out.farmax + idx);
                        }
                        std::memcpy(&dep_bytes[size_t(dbase + (i64(k) * cp + t) * 4)], &slot, 4);
                        val_dst.push_back(vbase + (i64(k) * cp + t) * es);
                        if (record_src) val_src.push_back(val_index[size_t(s)]);
                        ++k;
                    }
                for (; k < w; ++k) {
                    const int32_t slot = ring;   // ring slot RING holds 0
                    std::memcpy(&dep_bytes[size_t(dbase + (i64(k) * cp + t) * 4)], &slot, 4);
                    val_dst.push_back(vbase + (i64(k) * cp + t) * es);
                    if (record_src) val_src.push_back(-1);
                }
            }
        }
        out.stage_bytes = max_stage;
        out.smem_bytes = ((size_t(es) * (ring + 1 + SW_STAGES * out.farmax) + 127) / 128) * 128 +
                         size_t(max_stage) * SW_STAGES +
                         2 * SW_STAGES * sizeof(uint64_t) + size_t(L) * sizeof(ushort4);
    };
    std::vector<unsigned char> dep64, dep32;
    std::vector<i64> val_dst64, inv_dst64, val_dst32, inv_dst32;
    std::vector<i64> block_off32(static_cast<size_t>(L));
    layout(8, plan.f64, dep64, val_dst64, inv_dst64, block_off, true);
    layout(4, plan.f32, dep32, val_dst32, inv_dst32, block_off32, false);
    std::vector<ushort4> meta(static_cast<size_t>(L));
    bool small = true;
    plan.max_width = 0;
    for (i64 l = 0; l < L; ++l) {
        small = small && cntp[size_t(l)] < 65536 && width[size_t(l)] <= SW_MAX_WIDTH;
        plan.max_width = std::max(plan.max_width, int(width[size_t(l)]));
        meta[size_t(l)] = make_ushort4(uint16_t(cnt[size_t(l)]), uint16_t(cntp[size_t(l)]), uint16_t(width[size_t(l)]), 0);
    }
    // level widths within the unrolled bound, stages within shared memory
    plan.ok = small && plan.f64.smem_bytes <= 220 * 1024 && plan.f32.smem_bytes <= 220 * 1024 && P < (i64(1) << 31);
    if (std::getenv("NLGPU_DEBUG_SWEEPS"))
        for (int ring : {4096, 16384}) {   // dependencies beyond the ring: total, unique per level (max)
            i64 total = 0, max_unique = 0;
            for (i64 l = 0; l < L; ++l) {
                std::vector<i64> far;
                for (i64 t = lev_ptr[size_t(l)]; t < lev_ptr[size_t(l) + 1]; ++t) {
                    const int32_t r = rows[size_t(t)];
                    for (i64 s = rp[size_t(r)]; s < rp[size_t(r) + 1]; ++s) {
                        if (s == diag_pos[size_t(r)]) continue;
                        const i64 dp = ppos_of_row[size_t(col[size_t(s)])];
                        if (ppos[size_t(l) + 1] - dp > ring) far.push_back(dp);
                    }
                }
                total += i64(far.size());
                std::sort(far.begin(), far.end());
                max_unique = std::max<i64>(max_unique, i64(std::unique(far.begin(), far.end()) - far.begin()));
            }
            std::fprintf(stderr, "  ring %d: far dependencies %lld, max unique per level %lld\n", ring,
                         static_cast<long long>(total), static_cast<long long>(max_unique));
        }
    if (std::getenv("NLGPU_DEBUG_SWEEPS"))
        std::fprintf(stderr, "sweep plan: levels %lld positions %lld max distance %lld smem %zu/%zu far slots %d/%d "
                     "threads %d -> %s\n", static_cast<long long>(L), static_cast<long long>(P),
                     static_cast<long long>(max_dist), plan.f64.smem_bytes, plan.f32.smem_bytes, plan.f64.farmax,
                     plan.f32.farmax, plan.threads, plan.ok ? "ring" : "global");
    if (!plan.ok) return false;
    plan.meta.upload(meta.data(), meta.size(), ctx.stream);
    std::vector<int32_t> row_of(static_cast<size_t>(P), -1);
    for (i64 l = 0; l < L; ++l)
        for (int t = 0; t < cnt[size_t(l)]; ++t) row_of[size_t(ppos[size_t(l)] + t)] = rows[size_t(lev_ptr[size_t(l)] + t)];
    plan.n_levels = L;
    plan.P = P;
    plan.cnt.upload(cnt.data(), cnt.size(), ctx.stream);
    plan.cntp.upload(cntp.data(), cntp.size(), ctx.stream);
    plan.width.upload(width.data(), width.size(), ctx.stream);
    plan.ppos.upload(ppos.data(), ppos.size(), ctx.stream);
    plan.block_off.upload(block_off.data(), block_off.size(), ctx.stream);
    plan.row_of.upload(row_of.data(), row_of.size(), ctx.stream);
    plan.ppos_of_row.upload(ppos_of_row.data(), ppos_of_row.size(), ctx.stream);
    plan.val_src.upload(val_src.data(), val_src.size(), ctx.stream);
    plan.inv_src.upload(inv_src.data(), inv_src.size(), ctx.stream);
    // dependency slots now, values by sweep_plan_fill
    plan.f64.blocks.upload(dep64.data(), dep64.size(), ctx.stream);
    plan.f64.val_dst.upload(val_dst64.data(), val_dst64.size(), ctx.stream);
    plan.f64.inv_dst.upload(inv_dst64.data(), inv_dst64.size(), ctx.stream);
    plan.f32.blocks.upload(dep32.data(), dep32.size(), ctx.stream);
    plan.f32.val_dst.upload(val_dst32.data(), val_dst32.size(), ctx.stream);
    plan.f32.inv_dst.upload(inv_dst32.data(), inv_dst32.size(), ctx.stream);
    plan.in.resize(size_t(P)); plan.out.resize(size_t(P));
    plan.in32.resize(size_t(P)); plan.out32.resize(size_t(P));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    return true;
}

void sweep_plan_fill(Ctx& ctx, SweepPlan& plan, const double* u) {
    const i64 nv = i64(plan.val_src.n), ni = i64(plan.inv_src.n);
    if (nv) {
        NL_LAUNCH(k_fill_blocks<double>, grid_for(nv, 256), 256, 0, ctx.stream, nv, plan.f64.val_dst.p, plan.val_src.p, u,
                  false, plan.f64.blocks.p);
        NL_LAUNCH(k_fill_blocks<float>, grid_for(nv, 256), 256, 0, ctx.stream, nv, plan.f32.val_dst.p, plan.val_src.p, u,
                  false, plan.f32.blocks.p);
    }
    NL_LAUNCH(k_fill_blocks<double>, grid_for(ni, 256), 256, 0, ctx.stream, ni, plan.f64.inv_dst.p, plan.inv_src.p, u, true,
              plan.f64.blocks.p);
    NL_LAUNCH(k_fill_blocks<float>, grid_for(ni, 256), 256, 0, ctx.stream, ni, plan.f32.inv_dst.p, plan.inv_src.p, u, true,
              plan.f32.blocks.p);
}

template<class T, int MAXW>
static void launch_sweep_w(Ctx& ctx, int threads, size_t smem, const SweepArgs<T>& a) {
    static bool attr_set = false;
    if (!attr_set) {
        NL_CUDA(cudaFuncSetAttribute(k_sweep_tma<T, MAXW>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
        attr_set = true;
    }
    NL_LAUNCH((k_sweep_tma<T, MAXW>), 1, threads, smem, ctx.stream, a);
}

template<class T>
static void launch_sweep(Ctx& ctx, int max_width, int threads, size_t smem, const SweepArgs<T>& a) {
    if (max_width <= 4) launch_sweep_w<T, 4>(ctx, threads, smem, a);
    else if (max_width <= 8) launch_sweep_w<T, 8>(ctx, threads, smem, a);
    else if (max_width <= 12) launch_sweep_w<T, 12>(ctx, threads, smem, a);
    else launch_sweep_w<T, 16>(ctx, threads, smem, a);
}

template<class T>
static void run_sweep(Ctx& ctx, SweepPlan& plan, const double* partials, const double* flags, double tol2) {
    const SweepLayout& lay = sizeof(T) == 8 ? plan.f64 : plan.f32;
    SweepArgs<T> a{};
    a.n_levels = plan.n_levels; a.meta = plan.meta.p;
    a.blocks = lay.blocks.p;
    if constexpr (sizeof(T) == 8) { a.in = plan.in.p; a.out = plan.out.p; }
    else { a.in = plan.in32.p; a.out = plan.out32.p; }
    a.stage_bytes = lay.stage_bytes; a.partials = partials; a.flags = flags; a.tol2 = tol2;
    ctx.sweep_error.reserve(1);
    a.error = ctx.sweep_error.p;
    a.nct = plan.threads;
    a.farmax = lay.farmax;
    a.far_off = lay.far_off.p;
    a.far_pos = lay.far_pos.p;
    launch_sweep<T>(ctx, plan.max_width, plan.threads + 32, lay.smem_bytes, a);
}

// z = S U^-1 U^-T S r with the TMA sweeps (forward plan on U^T, backward on U)
void sweep_apply(Ctx& ctx, IncompleteCholesky& ic, const double* r, double* z, const double* partials,
                 const double* flags, double tol2) {
    SweepPlan& F = ic.fwd_plan;
    SweepPlan& B = ic.bwd_plan;
    NL_LAUNCH((k_gather_scaled<double, double>), grid_for(F.P, 256), 256, 0, ctx.stream, F.P, F.row_of.p, ic.scale.p, r,
              F.in.p);
    run_sweep<double>(ctx, F, partials, flags, tol2);
    NL_LAUNCH(k_transfer<double>, grid_for(B.P, 256), 256, 0, ctx.stream, B.P, B.row_of.p, F.ppos_of_row.p, F.out.p, B.in.p);
    run_sweep<double>(ctx, B, partials, flags, tol2);
    NL_LAUNCH((k_scatter_scaled<double, double>), grid_for(B.P, 256), 256, 0, ctx.stream, B.P, B.row_of.p, ic.scale.p,
              B.out.p, z);
}

// The same with FP32 factor values, right-hand side and solution (the inner
// solve of the mixed-precision form); the scaling S stays FP64.
void sweep_apply32(Ctx& ctx, IncompleteCholesky& ic, const float* r, float* z, const double* partials,
                   const double* flags, double tol2) {
    SweepPlan& F = ic.fwd_plan;
    SweepPlan& B = ic.bwd_plan;
    NL_LAUNCH((k_gather_scaled<float, float>), grid_for(F.P, 256), 256, 0, ctx.stream, F.P, F.row_of.p, ic.scale.p, r,
              F.in32.p);
    run_sweep<float>(ctx, F, partials, flags, tol2);
    NL_LAUNCH(k_transfer<float>, grid_for(B.P, 256), 256, 0, ctx.stream, B.P, B.row_of.p, F.ppos_of_row.p, F.out32.p,
              B.in32.p);
    run_sweep<float>(ctx, B, partials, flags, tol2);
    NL_LAUNCH((k_scatter_scaled<float, float>), grid_for(B.P, 256), 256, 0, ctx.stream, B.P, B.row_of.p, ic.scale.p,
              B.out32.p, z);
}

}  // namespace nlgpu
