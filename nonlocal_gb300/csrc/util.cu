// Prefix sums and small helpers shared by the pattern, neighbour and solver
// stages.
#include "common.cuh"

namespace nlgpu {

std::atomic<int64_t> g_launches{0};
thread_local int64_t* t_capture_sink = nullptr;

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ i64 block_exclusive_scan(i64 v, i64* sh, i64* total) {
    // sh: SCAN_THREADS / 32 entries
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    i64 incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const i64 t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        i64 s = lane < SCAN_THREADS / 32 ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const i64 t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        if (lane < SCAN_THREADS / 32) sh[lane] = s;
    }
    __syncthreads();
    const i64 warp_off = warp ? sh[warp - 1] : 0;
    if (total) *total = sh[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return warp_off + incl - v;
}

__global__ void k_tile_sums(const i64* in, i64 n, i64* sums) {
    __shared__ i64 sh[SCAN_THREADS / 32];
    const i64 base = i64(blockIdx.x) * SCAN_TILE;
    i64 s = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const i64 i = base + i64(threadIdx.x) * SCAN_ITEMS + k;
        if (i < n) s += in[i];
    }
    i64 total;
    block_exclusive_scan(s, sh, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(i64* sums, i64 nb, i64* grand_total) {
    __shared__ i64 sh[SCAN_THREADS / 32];
    i64 carry = 0;
    for (i64 base = 0; base < nb; base += SCAN_THREADS) {
        const i64 i = base + threadIdx.x;
        const i64 v = i < nb ? sums[i] : 0;
        i64 total;
        const i64 ex = block_exclusive_scan(v, sh, &total);
        if (i < nb) sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *grand_total = carry;
}

__global__ void k_scan_tiles(const i64* in, i64* out, i64 n, const i64* offsets) {
    __shared__ i64 sh[SCAN_THREADS / 32];
    const i64 base = i64(blockIdx.x) * SCAN_TILE;
    i64 v[SCAN_ITEMS];
    i64 s = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const i64 i = base + i64(threadIdx.x) * SCAN_ITEMS + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    i64 run = block_exclusive_scan(s, sh, nullptr) + offsets[blockIdx.x];
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const i64 i = base + i64(threadIdx.x) * SCAN_ITEMS + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

}  // namespace

void exclusive_scan(Ctx& ctx, const i64* in, i64* out, i64 n, i64* total_host) {
    const i64 nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    ctx.i64_scratch_a.reserve(size_t(nb + 2));
    i64* sums = ctx.i64_scratch_a.p;
    i64* grand = sums + nb + 1;
    if (n > 0) {
        NL_LAUNCH(k_tile_sums, unsigned(nb), SCAN_THREADS, 0, ctx.stream, in, n, sums);
        NL_LAUNCH(k_scan_sums, 1, SCAN_THREADS, 0, ctx.stream, sums, nb, grand);
        NL_LAUNCH(k_scan_tiles, unsigned(nb), SCAN_THREADS, 0, ctx.stream, in, out, n, sums);
    } else {
        NL_CUDA(cudaMemsetAsync(grand, 0, sizeof(i64), ctx.stream));
    }
    if (total_host) {
        NL_CUDA(cudaMemcpyAsync(total_host, grand, sizeof(i64), cudaMemcpyDeviceToHost, ctx.stream));
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
    }
}

i64 device_read_i64(Ctx& ctx, const i64* p) {
    i64 v = 0;
    NL_CUDA(cudaMemcpyAsync(&v, p, sizeof(i64), cudaMemcpyDeviceToHost, ctx.stream));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    return v;
}

}  // namespace nlgpu
