// BF16 tensor-core GEMM on the 5th-generation tensor cores (tcgen05) for the
// learned preconditioner's dense layers.
//
//   C[M x N] = A[M x K] . B[N x K]^T      A, B: BF16, K contiguous (K-major)
//
// A CTA (128 threads) takes 128-row tiles of C (all N <= 128 columns) in
// turn, and each tile's K steps of 64:
//   * the A tile (128 x 64) and B tile (N x 64) of a step are copied by the
//     threads with 16-byte cp.async (asynchronous, zero-filled past the ends)
//     into shared memory in the canonical no-swizzle K-major layout: 8x8 "core
//     matrices" of 128 contiguous bytes, K-adjacent core matrices 128 B apart
//     (LBO), 8-row groups 1024 B apart (SBO); consecutive threads fill
//     consecutive 16-byte rows of a core matrix, so the stores do not collide
//     in the banks.  Two stages: the copies of the next step are in flight
//     while the tensor cores run the current one;
//   * one thread issues four tcgen05.mma.cta_group::1.kind::f16 (M = 128,
//     N, K = 16 each) accumulating in FP32 in tensor memory, and commits them
//     to an mbarrier that every thread waits on (bounded by %globaltimer);
//   * after a tile's last step the epilogue reads the accumulator with
//     tcgen05.ld (warp w reads lanes 32w..32w+31, i.e. rows) and applies one
//     of the epilogues below.
// Split-K launches (gridDim.y > 1) add their partial products with FP32
// atomics.
#include "common.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace nlgpu {

namespace {

constexpr int TG_THREADS = 128;
constexpr int TG_KT = 64;                                  // K per step
constexpr uint32_t TG_LBO = 128, TG_SBO = 1024;
constexpr unsigned long long TG_WAIT_LIMIT_NS = 2000000000ull;

__device__ __forceinline__ uint32_t tg_smem(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ unsigned long long tg_time() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// shared-memory matrix descriptor: start, LBO, SBO (all >> 4), version 1, no swizzle
__device__ __forceinline__ uint64_t tg_desc(uint32_t saddr) {
    return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((TG_LBO >> 4) & 0x3FFFu) << 16) |
           (uint64_t((TG_SBO >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: D F32, A and B BF16, both K-major, N, M = 128
__host__ __device__ constexpr uint32_t tg_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(128 >> 4) << 24);
}

__device__ __forceinline__ bool tg_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(tg_smem(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// starts the copies of rows [row0, row0 + rows) x K range [k0, k0 + 64) of a
// K-major BF16 matrix (leading dimension ld elements) into the core-matrix
// layout; zeros outside [0, nrows) x [0, kmax) (cp.async zero-fills what its
// source size leaves out)
__device__ __forceinline__ void tg_load_tile(unsigned char* dst, const __nv_bfloat16* __restrict__ src, i64 ld,
                                             i64 row0, int rows, i64 nrows, i64 k0, i64 kmax) {
    const int chunks = rows * (TG_KT / 8);
    for (int c = threadIdx.x; c < chunks; c += TG_THREADS) {
        const int rl = c & 7, kg = (c >> 3) & 7, rh = c >> 6;   // row rh * 8 + rl, K group kg
        const int r = rh * 8 + rl;
        const i64 gr = row0 + r, gk = k0 + kg * 8;
        int bytes = 0;
        if (gr < nrows && gk < kmax) bytes = int(kmax - gk >= 8 ? 16 : (kmax - gk) * 2);
        const __nv_bfloat16* g = bytes ? src + gr * ld + gk : src;
        const uint32_t d = tg_smem(dst + rh * TG_SBO + kg * TG_LBO + rl * 16);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(g), "r"(bytes) : "memory");
    }
}

}  // namespace

// epilogue kinds
enum TgEpilogue : int {
    TG_TANH_BF16 = 0,   // out_bf16[row * ld_out + col] = bf16(tanh(acc)); optional transposed copy outT[col * ldT + row]
    TG_STORE_F32 = 1,   // out_f32[row * ld_out + col] = acc
    TG_ATOMIC_F32 = 2,  // out_f32[row * ld_out + col] += acc (split-K)
};

struct TgArgs {
    const __nv_bfloat16* A; i64 lda; i64 M;
    const __nv_bfloat16* B; i64 ldb;
    i64 K, k_per_split;
    __nv_bfloat16* out_bf16; __nv_bfloat16* outT; i64 ldT;
    float* out_f32; i64 ld_out;
    int* error;
};

template<int N, int EPI>
__global__ void __launch_bounds__(TG_THREADS) k_tc_gemm(TgArgs a) {
    static_assert(N % 16 == 0 && N >= 16 && N <= 128, "N");
    constexpr int STAGE = (128 + N) * TG_KT * 2;          // A tile then B tile
    extern __shared__ __align__(1024) unsigned char tg_smem_buf[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base_slot;
    __shared__ int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr uint32_t TMEM_COLS = N <= 32 ? 32 : (N <= 64 ? 64 : 128);
    if (threadIdx.x == 0) {
        failed = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tg_smem(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(tg_smem(&tmem_base_slot)), "r"(TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_slot;
    const i64 kbeg = i64(blockIdx.y) * a.k_per_split;
    const i64 kend = kbeg + a.k_per_split < a.K ? kbeg + a.k_per_split : a.K;
    const i64 steps = kend > kbeg ? (kend - kbeg + TG_KT - 1) / TG_KT : 0;
    const i64 tiles = (a.M + 127) / 128;
    const i64 my_tiles = i64(blockIdx.x) < tiles ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const i64 items = my_tiles * steps;   // (tile, step) pairs of this CTA, tile-major
    auto load = [&](i64 item) {
        const i64 tile = i64(blockIdx.x) + (item / steps) * gridDim.x;
        const i64 k0 = kbeg + (item % steps) * TG_KT;
        unsigned char* st = tg_smem_buf + (item & 1) * STAGE;
        tg_load_tile(st, a.A, a.lda, tile * 128, 128, a.M, k0, kend);
        tg_load_tile(st + 128 * TG_KT * 2, a.B, a.ldb, 0, N, N, k0, kend);
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    uint32_t phase = 0;
    if (items > 0) load(0);
    for (i64 it = 0; it < items && !failed; ++it) {
        // the next step's copies go out before this step's wait
        if (it + 1 < items) {
            load(it + 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        const i64 step = it % steps;
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = tg_smem(tg_smem_buf + (it & 1) * STAGE), sb = sa + 128 * TG_KT * 2;
#pragma unroll
            for (int j = 0; j < TG_KT / 16; ++j) {
                const uint64_t da = tg_desc(sa + uint32_t(j) * 2 * TG_LBO);
                const uint64_t db = tg_desc(sb + uint32_t(j) * 2 * TG_LBO);
                const uint32_t acc = (step == 0 && j == 0) ? 0u : 1u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                    ::"r"(tmem), "l"(da), "l"(db), "r"(tg_idesc(N)), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(tg_smem(&bar)) : "memory");
        }
        // every thread waits for the MMAs: their stage is refilled two steps on
        if (!tg_try_wait(&bar, phase)) {
            const unsigned long long t0 = tg_time();
            while (!tg_try_wait(&bar, phase)) {
                if (tg_time() - t0 > TG_WAIT_LIMIT_NS) { failed = 1; break; }
            }
        }
        phase ^= 1u;
        __syncthreads();
        if (failed) break;
        if (step != steps - 1) continue;
        // the tile's epilogue
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const i64 tile = i64(blockIdx.x) + (it / steps) * gridDim.x;
        const i64 row = tile * 128 + warp * 32 + lane;
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < a.M) {
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const float f = __uint_as_float(v[e]);
                    const int col = c0 + e;
                    if constexpr (EPI == TG_TANH_BF16) {
                        const __nv_bfloat16 h = __float2bfloat16(tanhf(f));
                        a.out_bf16[row * a.ld_out + col] = h;
                        if (a.outT) a.outT[i64(col) * a.ldT + row] = h;
                    } else if constexpr (EPI == TG_STORE_F32) {
                        a.out_f32[row * a.ld_out + col] = f;
                    } else {
                        atomicAdd(a.out_f32 + row * a.ld_out + col, f);
                    }
                }
            }
        }
        // the accumulator is read before the next tile's first MMA overwrites it
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    if (threadIdx.x == 0 && failed && a.error) atomicExch(a.error, 1);
}

template<int N, int EPI>
static void launch_tc_gemm(Ctx& ctx, const TgArgs& a, int splits) {
    const size_t smem = 2 * size_t(128 + N) * TG_KT * 2;   // two stages
    static bool attr = false;
    if (!attr) {
        NL_CUDA(cudaFuncSetAttribute(k_tc_gemm<N, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        attr = true;
    }
    // at most four CTAs per SM (tensor memory and shared memory), taking the tiles in turn
    const i64 tiles = (a.M + 127) / 128;
    const dim3 grid(unsigned(std::min<i64>(tiles, i64(152) * 4 / std::max(1, splits) + 1)), unsigned(splits));
    NL_LAUNCH((k_tc_gemm<N, EPI>), grid, TG_THREADS, smem, ctx.stream, a);
}

// C = A . B^T.  N in {64, 128}; epi as TgEpilogue; splits > 1 only with TG_ATOMIC_F32.
void tc_gemm(Ctx& ctx, int N, int epi, const __nv_bfloat16* A, i64 lda, i64 M, const __nv_bfloat16* B, i64 ldb, i64 K,
             int splits, __nv_bfloat16* out_bf16, __nv_bfloat16* outT, i64 ldT, float* out_f32, i64 ld_out, int* err) {
    NL_REQUIRE(lda % 8 == 0 && ldb % 8 == 0 && K > 0 && M > 0 && splits >= 1, NLGPU_ERR_ARG, "tc_gemm shape");
    TgArgs a{};
    a.A = A; a.lda = lda; a.M = M; a.B = B; a.ldb = ldb; a.K = K;
    a.k_per_split = (K + splits - 1) / splits;
    a.k_per_split = (a.k_per_split + TG_KT - 1) / TG_KT * TG_KT;
    a.out_bf16 = out_bf16; a.outT = outT; a.ldT = ldT; a.out_f32 = out_f32; a.ld_out = ld_out; a.error = err;
    NL_REQUIRE(splits == 1 || epi == TG_ATOMIC_F32, NLGPU_ERR_ARG, "split-K needs the atomic epilogue");
    if (N == 64 && epi == TG_TANH_BF16) launch_tc_gemm<64, TG_TANH_BF16>(ctx, a, splits);
    else if (N == 64 && epi == TG_STORE_F32) launch_tc_gemm<64, TG_STORE_F32>(ctx, a, splits);
    else if (N == 64 && epi == TG_ATOMIC_F32) launch_tc_gemm<64, TG_ATOMIC_F32>(ctx, a, splits);
    else if (N == 128 && epi == TG_STORE_F32) launch_tc_gemm<128, TG_STORE_F32>(ctx, a, splits);
    else if (N == 128 && epi == TG_ATOMIC_F32) launch_tc_gemm<128, TG_ATOMIC_F32>(ctx, a, splits);
    else throw error{NLGPU_ERR_UNSUPPORTED, "tc_gemm: unsupported N / epilogue"};
}

}  // namespace nlgpu

// C ABI check of the GEMM itself (host BF16 bit patterns in, FP32 out).
extern "C" int nlgpu_gemm_bf16(int64_t M, int N, int64_t K, int splits, const uint16_t* A, const uint16_t* B,
                               float* C) {
    using namespace nlgpu;
    if (!A || !B || !C || M <= 0 || K <= 0 || K % 8 || (N != 64 && N != 128) || splits < 1) return NLGPU_ERR_ARG;
    try {
        Ctx ctx;
        NL_CUDA(cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking));
        dbuf<uint16_t> a, b;
        dbuf<float> c;
        dbuf<int> err;
        a.upload(A, size_t(M * K), ctx.stream);
        b.upload(B, size_t(N) * size_t(K), ctx.stream);
        c.resize(size_t(M) * size_t(N));
        c.zero(ctx.stream);
        err.resize(1);
        err.zero(ctx.stream);
        tc_gemm(ctx, N, splits > 1 ? TG_ATOMIC_F32 : TG_STORE_F32, reinterpret_cast<const __nv_bfloat16*>(a.p), K, M,
                reinterpret_cast<const __nv_bfloat16*>(b.p), K, K, splits, nullptr, nullptr, 0, c.p, N, err.p);
        c.download(C, size_t(M) * size_t(N), ctx.stream);
        int h = 0;
        err.download(&h, 1, ctx.stream);
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
        cudaStreamDestroy(ctx.stream);
        ctx.stream = nullptr;
        return h ? NLGPU_ERR_TIMEOUT : NLGPU_OK;
    } catch (const nlgpu::error& e) {
        return e.code;
    }
}
