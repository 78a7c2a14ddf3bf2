// Learned correction on top of ILLT: a 4-layer message-passing network over
// the graph of the local stiffness pattern (no counterpart in the reference;
// it sits behind the same preconditioner slot as ILLT).
//
//   A_hat = D^-1/2 |offdiag(K_local)| D^-1/2      symmetric, zero diagonal, FP32
//   X0    = [r / rms(r), z / rms(z)],  z = ILLT^-1 r
//   U0    = [X0, A_hat X0]               n x 4     FP32
//   H1    = tanh(U0 W1)                  W1 4 x 64 (CUDA cores)
//   Ul    = [Hl, A_hat Hl]               n x 128   BF16
//   Hl+1  = tanh(Ul Wl+1)                W2, W3 128 x 64: tcgen05 BF16 GEMM, FP32 accumulation
//   y     = U3 w4                        w4 128
//   P(r)  = z + rms(z) y
//
// Training minimises L = (P(r) - e)^T A (P(r) - e) / (e^T A e) over (r, e)
// pairs harvested from plain ILLT-CG runs (e = x* - x_k, r = A e); the
// backward pass uses the same GEMM kernel for dU = dP W^T and, split over K,
// for dW = U^T dP; Adam keeps FP32 master weights and refreshes the BF16
// copies.  Every kernel here is the project's own; the CPU FP64 restatement
// checks forward values and gradients.
#include "common.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <random>

namespace nlgpu {

void tc_gemm(Ctx& ctx, int N, int epi, const __nv_bfloat16* A, i64 lda, i64 M, const __nv_bfloat16* B, i64 ldb, i64 K,
             int splits, __nv_bfloat16* out_bf16, __nv_bfloat16* outT, i64 ldT, float* out_f32, i64 ld_out, int* err);

namespace {

constexpr int HID = MPNN_HIDDEN;           // 64
constexpr int U_LD = 2 * HID;              // 128
constexpr int MP_THREADS = 256;
enum { TG_TANH_BF16 = 0, TG_STORE_F32 = 1, TG_ATOMIC_F32 = 2 };
// scalars: [0] 1/rms(r), [1] 1/rms(z), [2] rms(z), [3] loss numerator, [4] e.A.e
enum { SC_IR = 0, SC_IZ = 1, SC_SZ = 2, SC_LOSS = 3, SC_EE = 4 };

using bf16 = __nv_bfloat16;

__device__ __forceinline__ double mp_block_sum(double v, double* sh) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += sh[w];
    __syncthreads();
    return s;
}

// partials of r.r and z.z
__global__ void __launch_bounds__(MP_THREADS) k_mp_norms(i64 n, const float* __restrict__ r, const float* __restrict__ z,
                                                         double* __restrict__ part) {
    __shared__ double sh[40];
    double a = 0.0, b = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        a += double(r[i]) * r[i];
        b += double(z[i]) * z[i];
    }
    const double ta = mp_block_sum(a, sh), tb = mp_block_sum(b, sh);
    if (threadIdx.x == 0) { part[blockIdx.x] = ta; part[RED_BLOCKS + blockIdx.x] = tb; }
}

__global__ void __launch_bounds__(MP_THREADS) k_mp_scalars(i64 n, const double* __restrict__ part, float* __restrict__ sc) {
    __shared__ double sh[40];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < RED_BLOCKS; k += blockDim.x) { a += part[k]; b += part[RED_BLOCKS + k]; }
    a = mp_block_sum(a, sh);
    b = mp_block_sum(b, sh);
    if (threadIdx.x == 0) {
        const double rr = sqrt(a / double(n)), rz = sqrt(b / double(n));
        sc[SC_IR] = rr > 0.0 ? float(1.0 / rr) : 0.0f;
        sc[SC_IZ] = rz > 0.0 ? float(1.0 / rz) : 0.0f;
        sc[SC_SZ] = float(rz);
    }
}

// layer 1: U0 = [X0, A_hat X0] (kept for training), H1 = tanh(U0 W1) into U1[:, 0:64]
__global__ void __launch_bounds__(MP_THREADS) k_mp_layer1(i64 n, const i64* __restrict__ arp, const int32_t* __restrict__ acol,
                                                          const float* __restrict__ aw, const float* __restrict__ r,
                                                          const float* __restrict__ z, const float* __restrict__ sc,
                                                          const float* __restrict__ w1, float* __restrict__ u0,
                                                          bf16* __restrict__ u1) {
    __shared__ float W[4 * HID];
    for (int k = threadIdx.x; k < 4 * HID; k += blockDim.x) W[k] = w1[k];
    __syncthreads();
    const float ir = sc[SC_IR], iz = sc[SC_IZ];
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        float x0 = r[i] * ir, x1 = z[i] * iz, a0 = 0.0f, a1 = 0.0f;
        for (i64 k = arp[i]; k < arp[i + 1]; ++k) {
            const int32_t j = acol[k];
            a0 += aw[k] * (r[j] * ir);
            a1 += aw[k] * (z[j] * iz);
        }
        if (u0) { u0[4 * i] = x0; u0[4 * i + 1] = x1; u0[4 * i + 2] = a0; u0[4 * i + 3] = a1; }
        bf16* out = u1 + i * U_LD;
#pragma unroll 8
        for (int c = 0; c < HID; ++c)
            out[c] = __float2bfloat16(tanhf(x0 * W[c] + x1 * W[HID + c] + a0 * W[2 * HID + c] + a1 * W[3 * HID + c]));
    }
}

// U[:, 64:128] = A_hat U[:, 0:64]; warp per node, two features per lane;
// optional transposed copy Ut[c][i] of all 128 columns (training)
__global__ void __launch_bounds__(MP_THREADS) k_mp_aggregate(i64 n, const i64* __restrict__ arp,
                                                             const int32_t* __restrict__ acol, const float* __restrict__ aw,
                                                             bf16* __restrict__ u, bf16* __restrict__ ut, i64 ldt) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 i = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; i < n; i += warps) {
        float s0 = 0.0f, s1 = 0.0f;
        for (i64 k = arp[i]; k < arp[i + 1]; ++k) {
            const int32_t j = acol[k];
            const float2 h = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(u + i64(j) * U_LD + 2 * lane));
            s0 += aw[k] * h.x;
            s1 += aw[k] * h.y;
        }
        const __nv_bfloat162 o = __floats2bfloat162_rn(s0, s1);
        *reinterpret_cast<__nv_bfloat162*>(u + i * U_LD + HID + 2 * lane) = o;
        if (ut) {
            const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(u + i * U_LD + 2 * lane);
            ut[i64(2 * lane) * ldt + i] = h.x;
            ut[i64(2 * lane + 1) * ldt + i] = h.y;
            ut[i64(HID + 2 * lane) * ldt + i] = o.x;
            ut[i64(HID + 2 * lane + 1) * ldt + i] = o.y;
        }
    }
}

// out = z + rms(z) (U3 w4); warp per node
__global__ void __launch_bounds__(MP_THREADS) k_mp_output(i64 n, const bf16* __restrict__ u3, const float* __restrict__ w4,
                                                          const float* __restrict__ sc, const float* __restrict__ z,
                                                          float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    const float sz = sc[SC_SZ];
    for (i64 i = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; i < n; i += warps) {
        const bf16* row = u3 + i * U_LD + 4 * lane;
        const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(row));
        const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(row + 2));
        float s = a.x * w4[4 * lane] + a.y * w4[4 * lane + 1] + b.x * w4[4 * lane + 2] + b.y * w4[4 * lane + 3];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[i] = z[i] + sz * s;
    }
}

// ---------------------------------------------------------------- training
// d = p - e; partial of d.(A d) is formed after the SpMV (k_mp_loss)
__global__ void k_mp_diff(i64 n, const float* __restrict__ p, const float* __restrict__ e, float* __restrict__ d) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) d[i] = p[i] - e[i];
}

__global__ void __launch_bounds__(MP_THREADS) k_mp_dot(i64 n, const float* __restrict__ a, const float* __restrict__ b,
                                                       double* __restrict__ part) {
    __shared__ double sh[40];
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        s += double(a[i]) * b[i];
    const double t = mp_block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void __launch_bounds__(MP_THREADS) k_mp_finish(const double* __restrict__ part, float* __restrict__ sc, int slot,
                                                          double* __restrict__ out64) {
    __shared__ double sh[40];
    double a = 0.0;
    for (int k = threadIdx.x; k < RED_BLOCKS; k += blockDim.x) a += part[k];
    a = mp_block_sum(a, sh);
    if (threadIdx.x == 0) { sc[slot] = float(a); if (out64) *out64 = a; }
}

// gy = 2 sz (A d) / eAe; g4 += U3^T gy; dH3 = gy w4[0:64] + (A_hat gy) w4[64:128];
// dP3 = dH3 (1 - H3^2) into dp [n][64] and dpt [64][ldt]
__global__ void __launch_bounds__(MP_THREADS) k_mp_back_out(i64 n, const i64* __restrict__ arp,
                                                            const int32_t* __restrict__ acol, const float* __restrict__ aw,
                                                            const float* __restrict__ ad, const float* __restrict__ sc,
                                                            const double* __restrict__ ee, const bf16* __restrict__ u3,
                                                            const float* __restrict__ w4, float* __restrict__ g4,
                                                            bf16* __restrict__ dp, bf16* __restrict__ dpt, i64 ldt) {
    __shared__ float acc[U_LD];
    for (int k = threadIdx.x; k < U_LD; k += blockDim.x) acc[k] = 0.0f;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    const float scale = float(2.0 * double(sc[SC_SZ]) / *ee);
    float g[4] = {0, 0, 0, 0};
    for (i64 i = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; i < n; i += warps) {
        const float gy = scale * ad[i];
        float agy = 0.0f;
        for (i64 k = arp[i]; k < arp[i + 1]; ++k) agy += aw[k] * (scale * ad[acol[k]]);
        const bf16* row = u3 + i * U_LD;
        // lanes own features 2*lane, 2*lane+1 of each half
        const float2 h = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(row + 2 * lane));
        const float2 ah = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(row + HID + 2 * lane));
        g[0] += h.x * gy; g[1] += h.y * gy; g[2] += ah.x * gy; g[3] += ah.y * gy;
        const float d0 = (gy * w4[2 * lane] + agy * w4[HID + 2 * lane]) * (1.0f - h.x * h.x);
        const float d1 = (gy * w4[2 * lane + 1] + agy * w4[HID + 2 * lane + 1]) * (1.0f - h.y * h.y);
        const __nv_bfloat162 o = __floats2bfloat162_rn(d0, d1);
        *reinterpret_cast<__nv_bfloat162*>(dp + i * HID + 2 * lane) = o;
        dpt[i64(2 * lane) * ldt + i] = o.x;
        dpt[i64(2 * lane + 1) * ldt + i] = o.y;
    }
    atomicAdd(&acc[2 * lane], g[0]); atomicAdd(&acc[2 * lane + 1], g[1]);
    atomicAdd(&acc[HID + 2 * lane], g[2]); atomicAdd(&acc[HID + 2 * lane + 1], g[3]);
    __syncthreads();
    for (int k = threadIdx.x; k < U_LD; k += blockDim.x) atomicAdd(g4 + k, acc[k]);
}

// dH = dU[:, 0:64] + A_hat dU[:, 64:128]; dP = dH (1 - H^2) into dp / dpt
__global__ void __launch_bounds__(MP_THREADS) k_mp_back_hidden(i64 n, const i64* __restrict__ arp,
                                                               const int32_t* __restrict__ acol, const float* __restrict__ aw,
                                                               const float* __restrict__ du, const bf16* __restrict__ u,
                                                               bf16* __restrict__ dp, bf16* __restrict__ dpt, i64 ldt,
                                                               float* __restrict__ dp32) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 i = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; i < n; i += warps) {
        float s0 = du[i * U_LD + 2 * lane], s1 = du[i * U_LD + 2 * lane + 1];
        for (i64 k = arp[i]; k < arp[i + 1]; ++k) {
            const i64 j = acol[k];
            s0 += aw[k] * du[j * U_LD + HID + 2 * lane];
            s1 += aw[k] * du[j * U_LD + HID + 2 * lane + 1];
        }
        const float2 h = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(u + i * U_LD + 2 * lane));
        const float d0 = s0 * (1.0f - h.x * h.x), d1 = s1 * (1.0f - h.y * h.y);
        if (dp32) { dp32[i * HID + 2 * lane] = d0; dp32[i * HID + 2 * lane + 1] = d1; }
        const __nv_bfloat162 o = __floats2bfloat162_rn(d0, d1);
        *reinterpret_cast<__nv_bfloat162*>(dp + i * HID + 2 * lane) = o;
        dpt[i64(2 * lane) * ldt + i] = o.x;
        dpt[i64(2 * lane + 1) * ldt + i] = o.y;
    }
}

// g1 += U0^T dP1 (4 x 64); block partials in shared memory, then atomics
__global__ void __launch_bounds__(MP_THREADS) k_mp_grad1(i64 n, const float* __restrict__ u0, const float* __restrict__ dp32,
                                                         float* __restrict__ g1) {
    __shared__ float acc[4 * HID];
    for (int k = threadIdx.x; k < 4 * HID; k += blockDim.x) acc[k] = 0.0f;
    __syncthreads();
    const int c = threadIdx.x & (HID - 1), slot = threadIdx.x / HID;   // 4 node slots x 64 features
    float a[4] = {0, 0, 0, 0};
    for (i64 i = blockIdx.x * i64(4) + slot; i < n; i += i64(gridDim.x) * 4) {
        const float d = dp32[i * HID + c];
        for (int f = 0; f < 4; ++f) a[f] += u0[4 * i + f] * d;
    }
    for (int f = 0; f < 4; ++f) atomicAdd(&acc[f * HID + c], a[f]);
    __syncthreads();
    for (int k = threadIdx.x; k < 4 * HID; k += blockDim.x) atomicAdd(g1 + k, acc[k]);
}

// Adam on the FP32 masters (bias-corrected step size passed in), gradients zeroed
__global__ void k_mp_adam(i64 count, float* __restrict__ w, float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, float lr_t, float b1, float b2, float eps, float inv_batch) {
    for (i64 k = blockIdx.x * i64(blockDim.x) + threadIdx.x; k < count; k += i64(gridDim.x) * blockDim.x) {
        const float gk = g[k] * inv_batch;
        m[k] = b1 * m[k] + (1.0f - b1) * gk;
        v[k] = b2 * v[k] + (1.0f - b2) * gk * gk;
        w[k] -= lr_t * m[k] / (sqrtf(v[k]) + eps);
        g[k] = 0.0f;
    }
}

// BF16 copies of W (in x out, 128 x 64): wt [out][in] (forward B operand) and wb [in][out]
__global__ void k_mp_refresh(const float* __restrict__ w, bf16* __restrict__ wt, bf16* __restrict__ wb) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < U_LD * HID; k += gridDim.x * blockDim.x) {
        const int in = k / HID, out = k % HID;
        const bf16 b = __float2bfloat16(w[k]);
        wt[out * U_LD + in] = b;
        wb[k] = b;
    }
}

bf16* B16(dbuf<uint16_t>& b) { return reinterpret_cast<bf16*>(b.p); }
const bf16* B16(const dbuf<uint16_t>& b) { return reinterpret_cast<const bf16*>(b.p); }

// layer offsets inside the packed FP32 parameter vector
constexpr i64 OFF_W1 = 0, OFF_W2 = 4 * HID, OFF_W3 = OFF_W2 + U_LD * HID, OFF_W4 = OFF_W3 + U_LD * HID;

}  // namespace

void mpnn_prepare(Ctx& ctx, const Csr& local_upper) {
    Mpnn& m = ctx.mp;
    const i64 n = local_upper.rows;
    // A_hat from the upper local matrix on the host (a once-per-mesh step)
    std::vector<i64> rp(size_t(n + 1));
    std::vector<int32_t> col(static_cast<size_t>(local_upper.nnz));
    std::vector<double> val(static_cast<size_t>(local_upper.nnz));
    local_upper.rowptr.download(rp.data(), rp.size(), ctx.stream);
    local_upper.col.download(col.data(), col.size(), ctx.stream);
    local_upper.val.download(val.data(), val.size(), ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    std::vector<double> diag(static_cast<size_t>(n), 1.0);
    for (i64 r = 0; r < n; ++r)
        for (i64 k = rp[size_t(r)]; k < rp[size_t(r) + 1]; ++k)
            if (col[size_t(k)] == r && val[size_t(k)] != 0.0) diag[size_t(r)] = std::fabs(val[size_t(k)]);
    std::vector<i64> cnt(static_cast<size_t>(n + 1), 0);
    for (i64 r = 0; r < n; ++r)
        for (i64 k = rp[size_t(r)]; k < rp[size_t(r) + 1]; ++k)
            if (col[size_t(k)] != r) { ++cnt[size_t(r) + 1]; ++cnt[size_t(col[size_t(k)]) + 1]; }
    for (i64 r = 0; r < n; ++r) cnt[size_t(r) + 1] += cnt[size_t(r)];
    std::vector<int32_t> acol(static_cast<size_t>(cnt[size_t(n)]));
    std::vector<float> aw(static_cast<size_t>(cnt[size_t(n)]));
    std::vector<i64> cur(cnt.begin(), cnt.end() - 1);
    for (i64 r = 0; r < n; ++r)
        for (i64 k = rp[size_t(r)]; k < rp[size_t(r) + 1]; ++k) {
            const i64 c = col[size_t(k)];
            if (c == r) continue;
            const float w = float(std::fabs(val[size_t(k)]) / std::sqrt(diag[size_t(r)] * diag[size_t(c)]));
            acol[size_t(cur[size_t(r)])] = int32_t(c); aw[size_t(cur[size_t(r)]++)] = w;
            acol[size_t(cur[size_t(c)])] = int32_t(r); aw[size_t(cur[size_t(c)]++)] = w;
        }
    m.n = n;
    m.ldt = (n + 7) / 8 * 8;
    m.arp.upload(cnt.data(), cnt.size(), ctx.stream);
    m.acol.upload(acol.data(), acol.size(), ctx.stream);
    m.aw.upload(aw.data(), aw.size(), ctx.stream);
    m.u0.resize(size_t(n) * 4);
    for (auto* u : {&m.u1, &m.u2, &m.u3}) u->resize(size_t(n) * U_LD);
    m.part.resize(size_t(2) * RED_BLOCKS);
    m.sc.resize(8);
    m.sc.zero(ctx.stream);
    m.error.resize(1);
    m.error.zero(ctx.stream);
    if (!m.params.n) {
        mpnn_init_weights(ctx, 0);
        m.weights_set = false;
    }
    m.ready = true;
}

void mpnn_init_weights(Ctx& ctx, unsigned seed) {
    Mpnn& m = ctx.mp;
    std::vector<float> w(static_cast<size_t>(MPNN_PARAMS));
    std::mt19937_64 gen(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    auto fill = [&](i64 off, i64 fan_in, i64 count, double scale) {
        for (i64 k = 0; k < count; ++k) w[size_t(off + k)] = float(nd(gen) * scale / std::sqrt(double(fan_in)));
    };
    fill(OFF_W1, 4, 4 * HID, 1.0);
    fill(OFF_W2, U_LD, U_LD * HID, 1.0);
    fill(OFF_W3, U_LD, U_LD * HID, 1.0);
    fill(OFF_W4, U_LD, U_LD, 0.1);
    mpnn_set_weights(ctx, w.data());
}

void mpnn_set_weights(Ctx& ctx, const float* host) {
    Mpnn& m = ctx.mp;
    m.params.upload(host, size_t(MPNN_PARAMS), ctx.stream);
    m.weights_set = true;
    m.use = true;
    m.grads.resize(size_t(MPNN_PARAMS)); m.grads.zero(ctx.stream);
    m.adam_m.resize(size_t(MPNN_PARAMS)); m.adam_m.zero(ctx.stream);
    m.adam_v.resize(size_t(MPNN_PARAMS)); m.adam_v.zero(ctx.stream);
    m.adam_t = 0;
    for (auto* b : {&m.w2t, &m.w3t, &m.w2b, &m.w3b}) b->resize(size_t(U_LD) * HID);
    NL_LAUNCH(k_mp_refresh, 32, 256, 0, ctx.stream, m.params.p + OFF_W2, B16(m.w2t), B16(m.w2b));
    NL_LAUNCH(k_mp_refresh, 32, 256, 0, ctx.stream, m.params.p + OFF_W3, B16(m.w3t), B16(m.w3b));
}

void mpnn_get_weights(Ctx& ctx, float* host) {
    ctx.mp.params.download(host, size_t(MPNN_PARAMS), ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
}

// out = P(r) given r and z = ILLT^-1 r (out may alias z); training keeps the
// transposed activations
void mpnn_apply(Ctx& ctx, const float* r, const float* z, float* out, bool training) {
    Mpnn& m = ctx.mp;
    NL_REQUIRE(m.ready, NLGPU_ERR_STATE, "the learned preconditioner is not prepared");
    const i64 n = m.n;
    const float* W = m.params.p;
    if (training) { m.u1t.resize(size_t(U_LD) * m.ldt); m.u2t.resize(size_t(U_LD) * m.ldt); }
    bf16* u1t = training ? B16(m.u1t) : nullptr;
    bf16* u2t = training ? B16(m.u2t) : nullptr;
    NL_LAUNCH(k_mp_norms, RED_BLOCKS, MP_THREADS, 0, ctx.stream, n, r, z, m.part.p);
    NL_LAUNCH(k_mp_scalars, 1, MP_THREADS, 0, ctx.stream, n, m.part.p, m.sc.p);
    NL_LAUNCH(k_mp_layer1, grid_for(n, MP_THREADS), MP_THREADS, 0, ctx.stream, n, m.arp.p, m.acol.p, m.aw.p, r, z, m.sc.p,
              W + OFF_W1, training ? m.u0.p : static_cast<float*>(nullptr), B16(m.u1));
    const unsigned gw = grid_for(n * 32, MP_THREADS);
    NL_LAUNCH(k_mp_aggregate, gw, MP_THREADS, 0, ctx.stream, n, m.arp.p, m.acol.p, m.aw.p, B16(m.u1), u1t, m.ldt);
    tc_gemm(ctx, HID, TG_TANH_BF16, B16(m.u1), U_LD, n, B16(m.w2t), U_LD, U_LD, 1, B16(m.u2), nullptr, 0, nullptr, U_LD,
            m.error.p);
    NL_LAUNCH(k_mp_aggregate, gw, MP_THREADS, 0, ctx.stream, n, m.arp.p, m.acol.p, m.aw.p, B16(m.u2), u2t, m.ldt);
    tc_gemm(ctx, HID, TG_TANH_BF16, B16(m.u2), U_LD, n, B16(m.w3t), U_LD, U_LD, 1, B16(m.u3), nullptr, 0, nullptr, U_LD,
            m.error.p);
    NL_LAUNCH(k_mp_aggregate, gw, MP_THREADS, 0, ctx.stream, n, m.arp.p, m.acol.p, m.aw.p, B16(m.u3),
              static_cast<bf16*>(nullptr), m.ldt);
    NL_LAUNCH(k_mp_output, gw, MP_THREADS, 0, ctx.stream, n, B16(m.u3), W + OFF_W4, m.sc.p, z, out);
}

// One training sample: forward, loss, gradients accumulated into m.grads.
// A is the full-row system matrix with its FP32 copy; ee_out gets e.A.e and
// loss_out the loss (device doubles, may be null).
void mpnn_backward(Ctx& ctx, const Csr& A, const float* r, const float* z, const float* e, float* p_out,
                   double* loss_num, double* ee_out) {
    Mpnn& m = ctx.mp;
    const i64 n = m.n;
    m.d.resize(size_t(n)); m.ad.resize(size_t(n));
    m.dp.resize(size_t(n) * HID); m.dpt.resize(size_t(HID) * m.ldt);
    m.du.resize(size_t(n) * U_LD); m.dp32.resize(size_t(n) * HID);
    m.part2.resize(size_t(RED_BLOCKS));
    m.ee64.resize(2);
    if (m.ldt > n) {   // transposed buffers: the padding columns stay zero
        NL_CUDA(cudaMemsetAsync(m.dpt.p, 0, m.dpt.bytes(), ctx.stream));
    }
    mpnn_apply(ctx, r, z, p_out, true);
    // e.A.e and d.A d
    spmv32(ctx, A, e, m.ad.p);
    NL_LAUNCH(k_mp_dot, RED_BLOCKS, MP_THREADS, 0, ctx.stream, n, e, m.ad.p, m.part2.p);
    NL_LAUNCH(k_mp_finish, 1, MP_THREADS, 0, ctx.stream, m.part2.p, m.sc.p, SC_EE, m.ee64.p);
    NL_LAUNCH(k_mp_diff, grid_for(n, 256), 256, 0, ctx.stream, n, p_out, e, m.d.p);
    spmv32(ctx, A, m.d.p, m.ad.p);
    NL_LAUNCH(k_mp_dot, RED_BLOCKS, MP_THREADS, 0, ctx.stream, n, m.d.p, m.ad.p, m.part2.p);
    NL_LAUNCH(k_mp_finish, 1, MP_THREADS, 0, ctx.stream, m.part2.p, m.sc.p, SC_LOSS, m.ee64.p + 1);
    if (ee_out) NL_CUDA(cudaMemcpyAsync(ee_out, m.ee64.p, sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
    if (loss_num) NL_CUDA(cudaMemcpyAsync(loss_num, m.ee64.p + 1, sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
    float* G = m.grads.p;
    const unsigned gw = grid_for(n * 32, MP_THREADS);
    // output layer
    NL_LAUNCH(k_mp_back_out, gw, MP_THREADS, 0, ctx.stream, n, m.arp.p, m.acol.p, m.aw.p, m.ad.p, m.sc.p, m.ee64.p,
              B16(m.u3), m.params.p + OFF_W4, G + OFF_W4, B16(m.dp), B16(m.dpt), m.ldt);
    const int splits = int(std::min<i64>(148, std::max<i64>(1, n / 512)));
    // layer 3: dW3 = U2^T dP3, dU2 = dP3 W3^T
    tc_gemm(ctx, HID, TG_ATOMIC_F32, B16(m.u2t), m.ldt, U_LD, B16(m.dpt), m.ldt, n, splits, nullptr, nullptr, 0,
            G + OFF_W3, HID, m.error.p);
    tc_gemm(ctx, U_LD, TG_STORE_F32, B16(m.dp), HID, n, B16(m.w3b), HID, HID, 1, nullptr, nullptr, 0, m.du.p, U_LD,
            m.error.p);
    NL_LAUNCH(k_mp_back_hidden, gw, MP_THREADS, 0, ctx.stream, n, m.arp.p, m.acol.p, m.aw.p, m.du.p, B16(m.u2), B16(m.dp),
              B16(m.dpt), m.ldt, static_cast<float*>(nullptr));
    // layer 2: dW2 = U1^T dP2, dU1 = dP2 W2^T
    tc_gemm(ctx, HID, TG_ATOMIC_F32, B16(m.u1t), m.ldt, U_LD, B16(m.dpt), m.ldt, n, splits, nullptr, nullptr, 0,
            G + OFF_W2, HID, m.error.p);
    tc_gemm(ctx, U_LD, TG_STORE_F32, B16(m.dp), HID, n, B16(m.w2b), HID, HID, 1, nullptr, nullptr, 0, m.du.p, U_LD,
            m.error.p);
    NL_LAUNCH(k_mp_back_hidden, gw, MP_THREADS, 0, ctx.stream, n, m.arp.p, m.acol.p, m.aw.p, m.du.p, B16(m.u1), B16(m.dp),
              B16(m.dpt), m.ldt, m.dp32.p);
    // layer 1: dW1 = U0^T dP1
    NL_LAUNCH(k_mp_grad1, 304, MP_THREADS, 0, ctx.stream, n, m.u0.p, m.dp32.p, G + OFF_W1);
}

void mpnn_adam_step(Ctx& ctx, float lr, int batch) {
    Mpnn& m = ctx.mp;
    m.adam_t += 1;
    const double b1 = 0.9, b2 = 0.999;
    const double lr_t = lr * std::sqrt(1.0 - std::pow(b2, m.adam_t)) / (1.0 - std::pow(b1, m.adam_t));
    NL_LAUNCH(k_mp_adam, grid_for(MPNN_PARAMS, 256), 256, 0, ctx.stream, i64(MPNN_PARAMS), m.params.p, m.grads.p,
              m.adam_m.p, m.adam_v.p, float(lr_t), float(b1), float(b2), 1e-8f, 1.0f / float(batch));
    NL_LAUNCH(k_mp_refresh, 32, 256, 0, ctx.stream, m.params.p + OFF_W2, B16(m.w2t), B16(m.w2b));
    NL_LAUNCH(k_mp_refresh, 32, 256, 0, ctx.stream, m.params.p + OFF_W3, B16(m.w3t), B16(m.w3b));
}

namespace {

__global__ void k_mp_sub64(i64 n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) out[i] = a[i] - b[i];
}

__global__ void __launch_bounds__(MP_THREADS) k_mp_norm64(i64 n, const double* __restrict__ v, double* __restrict__ part) {
    __shared__ double sh[40];
    double s = 0.0;
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) s += v[i] * v[i];
    const double t = mp_block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// out = float(v / sqrt(sum of partials)) for two vectors scaled by the same norm
__global__ void __launch_bounds__(MP_THREADS) k_mp_pair_f32(i64 n, const double* __restrict__ r, const double* __restrict__ e,
                                                            const double* __restrict__ part, float* __restrict__ r32,
                                                            float* __restrict__ e32) {
    __shared__ double sh[40];
    double a = 0.0;
    for (int k = threadIdx.x; k < RED_BLOCKS; k += blockDim.x) a += part[k];
    a = mp_block_sum(a, sh);
    if (threadIdx.x == 0) sh[32] = a > 0.0 ? 1.0 / sqrt(a) : 0.0;
    __syncthreads();
    const double s = sh[32];
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) {
        r32[i] = float(r[i] * s);
        e32[i] = float(e[i] * s);
    }
}

}  // namespace

// Harvests (r, e) pairs from plain FP64 ILLT-CG runs on the assembled system
// (the given right-hand side and random ones): snapshots x_k every chunk of
// iterations, e = x* - x_k, r = A e, both divided by |r|.  Then trains the
// network with Adam on minibatches of pairs.
void mpnn_train(Ctx& ctx, const Csr& A, IncompleteCholesky& M, const double* b_given, const MpnnTrainOptions& o,
                MpnnTrainResult& out) {
    Mpnn& m = ctx.mp;
    NL_REQUIRE(m.ready && m.n == A.rows && M.ok, NLGPU_ERR_STATE, "training needs the assembled system and ILLT");
    NL_REQUIRE(o.right_hand_sides >= 1 && o.epochs >= 1 && o.batch >= 1, NLGPU_ERR_ARG, "training options");
    const i64 n = A.rows;
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<dbuf<float>> R, E;
    dbuf<double> b, xs, xk, e64, r64, part;
    b.resize(size_t(n)); xs.resize(size_t(n)); xk.resize(size_t(n)); e64.resize(size_t(n)); r64.resize(size_t(n));
    part.resize(RED_BLOCKS);
    std::mt19937_64 gen(o.seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    std::vector<double> hb(static_cast<size_t>(n));
    for (int s = 0; s < o.right_hand_sides; ++s) {
        if (s == 0 && b_given) {
            NL_CUDA(cudaMemcpyAsync(b.p, b_given, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
        } else {
            for (auto& v : hb) v = nd(gen);
            b.upload(hb.data(), hb.size(), ctx.stream);
        }
        cg_solve(ctx, A, &M, b.p, xs.p, 1e-12, 100000, false);
        const CgChunkHook hook = [&](i64, const double* x) {
            NL_LAUNCH(k_mp_sub64, grid_for(n, 256), 256, 0, ctx.stream, n, xs.p, x, e64.p);
            spmv_full(ctx, A, e64.p, r64.p);
            NL_LAUNCH(k_mp_norm64, RED_BLOCKS, MP_THREADS, 0, ctx.stream, n, r64.p, part.p);
            R.emplace_back(); E.emplace_back();
            R.back().resize(size_t(n)); E.back().resize(size_t(n));
            NL_LAUNCH(k_mp_pair_f32, RED_BLOCKS, MP_THREADS, 0, ctx.stream, n, r64.p, e64.p, part.p, R.back().p, E.back().p);
        };
        cg_solve(ctx, A, &M, b.p, xk.p, 1e-12, 100000, false, hook);
    }
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    out.samples = i64(R.size());
    out.seconds_harvest = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    NL_REQUIRE(out.samples > 0, NLGPU_ERR_STATE, "no training pairs (the solves converged within one chunk)");
    const auto t1 = std::chrono::steady_clock::now();
    const i64 S = out.samples;
    dbuf<float> z, p;
    dbuf<double> num, ee;
    z.resize(size_t(n)); p.resize(size_t(n));
    num.resize(size_t(S)); ee.resize(size_t(S));
    std::vector<double> hnum(static_cast<size_t>(S)), hee(static_cast<size_t>(S));
    auto mean_loss = [&]() {
        num.download(hnum.data(), size_t(S), ctx.stream);
        ee.download(hee.data(), size_t(S), ctx.stream);
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
        double l = 0.0;
        for (i64 k = 0; k < S; ++k) l += hnum[size_t(k)] / hee[size_t(k)];
        return l / double(S);
    };
    // the plain ILLT error on the same pairs: (z - e)^T A (z - e) / e^T A e
    m.d.reserve(size_t(n)); m.ad.reserve(size_t(n)); m.part2.reserve(RED_BLOCKS);
    for (i64 k = 0; k < S; ++k) {
        ilt_apply32(ctx, M, R[size_t(k)].p, z.p, ctx.ilt_sweeps);
        spmv32(ctx, A, E[size_t(k)].p, m.ad.p);
        NL_LAUNCH(k_mp_dot, RED_BLOCKS, MP_THREADS, 0, ctx.stream, n, E[size_t(k)].p, m.ad.p, m.part2.p);
        NL_LAUNCH(k_mp_finish, 1, MP_THREADS, 0, ctx.stream, m.part2.p, m.sc.p, SC_EE, ee.p + k);
        NL_LAUNCH(k_mp_diff, grid_for(n, 256), 256, 0, ctx.stream, n, z.p, E[size_t(k)].p, m.d.p);
        spmv32(ctx, A, m.d.p, m.ad.p);
        NL_LAUNCH(k_mp_dot, RED_BLOCKS, MP_THREADS, 0, ctx.stream, n, m.d.p, m.ad.p, m.part2.p);
        NL_LAUNCH(k_mp_finish, 1, MP_THREADS, 0, ctx.stream, m.part2.p, m.sc.p, SC_LOSS, num.p + k);
    }
    out.loss_illt = mean_loss();
    std::vector<i64> order(static_cast<size_t>(S));
    for (i64 k = 0; k < S; ++k) order[size_t(k)] = k;
    out.steps = 0;
    for (int ep = 0; ep < o.epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), gen);
        for (i64 k0 = 0; k0 < S; k0 += o.batch) {
            const i64 k1 = std::min<i64>(S, k0 + o.batch);
            for (i64 k = k0; k < k1; ++k) {
                const i64 s = order[size_t(k)];
                ilt_apply32(ctx, M, R[size_t(s)].p, z.p, ctx.ilt_sweeps);
                mpnn_backward(ctx, A, R[size_t(s)].p, z.p, E[size_t(s)].p, p.p, num.p + s, ee.p + s);
            }
            mpnn_adam_step(ctx, float(o.learning_rate), int(k1 - k0));
            ++out.steps;
        }
        const double l = mean_loss();
        if (ep == 0) out.loss_first = l;
        out.loss_last = l;
    }
    mpnn_check(ctx);
    out.seconds_train = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    m.weights_set = true;
    // validation gate: the system's own right-hand side solved with and without
    // the correction; it stays enabled only when it is faster
    if (b_given) {
        dbuf<double> xv;
        xv.resize(size_t(n));
        auto timed = [&](bool learned, double& secs) {
            const auto s0 = std::chrono::steady_clock::now();
            const CgResult r = mixed_solve(ctx, A, &M, b_given, xv.p, 1e-10, 20 * n + 1000, 1e-2, false, learned,
                                           ctx.ilt_sweeps);
            NL_CUDA(cudaStreamSynchronize(ctx.stream));
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - s0).count();
            return r;
        };
        m.use = true;
        const CgResult with = timed(true, out.validation_seconds_learned);
        const CgResult without = timed(false, out.validation_seconds_illt);
        out.validation_iterations_learned = with.iterations;
        out.validation_iterations_illt = without.iterations;
        m.use = with.converged && !with.learned_fallback && out.validation_seconds_learned < out.validation_seconds_illt;
    } else {
        m.use = true;
    }
    out.learned_enabled = m.use;
}

void mpnn_check(Ctx& ctx) {
    int err = 0;
    ctx.mp.error.download(&err, 1, ctx.stream);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    NL_REQUIRE(err == 0, NLGPU_ERR_TIMEOUT, "a tensor-core GEMM gave up waiting for its MMAs");
}

}  // namespace nlgpu
