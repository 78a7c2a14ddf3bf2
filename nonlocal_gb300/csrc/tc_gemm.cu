// BF16 tensor-core GEMM on the 5th-generation tensor cores (tcgen05) for the
// learned preconditioner's dense layers.
//
//   C[M x N] = A[M x K] . B[N x K]^T      A, B: BF16, K contiguous (K-major)
//
// One CTA (128 threads) owns a 128-row tile of C and all N <= 128 columns:
//   * the A tile (128 x 64) and B tile (N x 64) of each K step are copied by
//     the threads (16-byte loads) into shared memory in the canonical
//     no-swizzle K-major layout: 8x8 "core matrices" of 128 contiguous bytes,
//     K-adjacent core matrices 128 B apart (LBO), 8-row groups 1024 B apart
//     (SBO);
//   * one thread issues four tcgen05.mma.cta_group::1.kind::f16 (M = 128,
//     N, K = 16 each) accumulating in FP32 in tensor memory, and commits them
//     to an mbarrier that every thread waits on (bounded by %globaltimer);
//   * the epilogue reads the accumulator with tcgen05.ld (warp w reads lanes
//     32w..32w+31, i.e. rows) and applies one of the epilogues below.
// Rows beyond M and K beyond the end are loaded as zeros.  Split-K launches
// (gridDim.y > 1) add their partial products with FP32 atomics.
#include "common.cuh"

#include <cuda_bf16.h>

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

// copies rows [row0, row0 + rows) x K range [k0, k0 + 64) of a K-major BF16
// matrix (leading dimension ld elements) into the core-matrix layout; zeros
// outside [0, nrows) x [0, kmax)
__device__ __forceinline__ void tg_load_tile(unsigned char* dst, const __nv_bfloat16* __restrict__ src, i64 ld,
                                             i64 row0, int rows, i64 nrows, i64 k0, i64 kmax) {
    const int chunks = rows * (TG_KT / 8);
    for (int c = threadIdx.x; c < chunks; c += TG_THREADS) {
        const int r = c >> 3, kg = c & 7;
        const i64 gr = row0 + r, gk = k0 + kg * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gr < nrows && gk + 8 <= kmax) v = *reinterpret_cast<const uint4*>(src + gr * ld + gk);
        else if (gr < nrows && gk < kmax) {
            __nv_bfloat16 tmp[8];
            for (int e = 0; e < 8; ++e) tmp[e] = gk + e < kmax ? src[gr * ld + gk + e] : __float2bfloat16(0.0f);
            v = *reinterpret_cast<const uint4*>(tmp);
        }
        *reinterpret_cast<uint4*>(dst + (r >> 3) * TG_SBO + kg * TG_LBO + (r & 7) * 16) = v;
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
    extern __shared__ __align__(1024) unsigned char tg_smem_buf[];
    unsigned char* tileA = tg_smem_buf;                    // 16 KB
    unsigned char* tileB = tg_smem_buf + 128 * TG_KT * 2;  // N x 64 x 2 B
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
    const i64 row0 = i64(blockIdx.x) * 128;
    const i64 kbeg = i64(blockIdx.y) * a.k_per_split;
    const i64 kend = kbeg + a.k_per_split < a.K ? kbeg + a.k_per_split : a.K;
    uint32_t phase = 0;
    bool first = true;
    for (i64 k0 = kbeg; k0 < kend; k0 += TG_KT) {
        tg_load_tile(tileA, a.A, a.lda, row0, 128, a.M, k0, kend);
        tg_load_tile(tileB, a.B, a.ldb, 0, N, N, k0, kend);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = tg_smem(tileA), sb = tg_smem(tileB);
#pragma unroll
            for (int j = 0; j < TG_KT / 16; ++j) {
                const uint64_t da = tg_desc(sa + uint32_t(j) * 2 * TG_LBO);
                const uint64_t db = tg_desc(sb + uint32_t(j) * 2 * TG_LBO);
                const uint32_t acc = (first && j == 0) ? 0u : 1u;
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
        first = false;
        // every thread waits for the MMAs (the tiles are rewritten next step)
        if (!tg_try_wait(&bar, phase)) {
            const unsigned long long t0 = tg_time();
            while (!tg_try_wait(&bar, phase)) {
                if (tg_time() - t0 > TG_WAIT_LIMIT_NS) { failed = 1; break; }
            }
        }
        phase ^= 1u;
        __syncthreads();
        if (failed) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!failed && kend > kbeg) {
        const i64 row = row0 + warp * 32 + lane;
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
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    if (threadIdx.x == 0 && failed && a.error) atomicExch(a.error, 1);
}

template<int N, int EPI>
static void launch_tc_gemm(Ctx& ctx, const TgArgs& a, int splits) {
    const size_t smem = size_t(128 + N) * TG_KT * 2;
    static bool attr = false;
    if (!attr) {
        NL_CUDA(cudaFuncSetAttribute(k_tc_gemm<N, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        attr = true;
    }
    const dim3 grid(unsigned((a.M + 127) / 128), unsigned(splits));
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
