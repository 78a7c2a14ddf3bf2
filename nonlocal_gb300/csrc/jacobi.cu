// ILLT applied by Jacobi sweeps on the triangles of the factor (FP32).
//
// The preconditioner is the same incomplete Cholesky factor U (S A S ~ U^T U,
// eigen_preconditioner.hpp:56-57 through the Lin-More restatement of
// solver.cu); only the way its two triangular systems are solved changes.
// Instead of the exact level-scheduled substitution -- one dependent step per
// level, a few hundred to a few thousand per sweep on these meshes -- each
// triangle is solved approximately by k Jacobi iterations (Anzt, Chow and
// Dongarra, "Iterative sparse triangular solves for preconditioning",
// Euro-Par 2015):
//
//   U^T y = S r:  y_0 = D^-1 S r,  y_t+1 = D^-1 S r - (D^-1 N) y_t
//   U z = y_k:    z_0 = D^-1 y_k,  z_t+1 = D^-1 y_k - (D^-1 N^T) z_t,  result S z_k
//
// with D the diagonal of U and N the strict lower part of U^T.  D^-1 N is
// nilpotent, so k sweeps give the first k + 1 terms of the Neumann series of
// each triangular inverse, and k >= the level count reproduces the exact
// solve.  The truncated operator is S F^T F S with F lower triangular and
// nonsingular: symmetric positive definite, so it is a valid CG
// preconditioner; FP32 rounding makes it slightly non-symmetric, which the
// flexible CG of mixed.cu absorbs.  Every sweep is one fully parallel pass
// over one triangle (thread per row, sliced ELL), so a preconditioner
// application costs 2 k short bandwidth-bound launches instead of two chains
// of per-level barriers.
#include "common.cuh"

#include <algorithm>

namespace nlgpu {

namespace {

constexpr int JB_THREADS = 256;

// val = u[src] / u_ii of the entry's row (0 for padding); the sliced-ELL
// layouts themselves are built by iltbuild.cu
__global__ void k_jacobi_values(i64 n, const i64* __restrict__ slice, const i64* __restrict__ src,
                                const i64* __restrict__ u_rp, const double* __restrict__ u, float* __restrict__ val) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x) {
        const i64 sl = r >> 5, lane = r & 31, beg = slice[sl], w = (slice[sl + 1] - beg) >> 5;
        const double inv = 1.0 / u[u_rp[r]];
        for (i64 k = 0; k < w; ++k) {
            const i64 e = beg + 32 * k + lane;
            val[e] = src[e] >= 0 ? float(u[src[e]] * inv) : 0.0f;
        }
    }
}

// c_i = s_i / u_ii, dinv_i = 1 / u_ii
__global__ void k_jacobi_diag(i64 n, const i64* __restrict__ u_rp, const double* __restrict__ u,
                              const double* __restrict__ scale, float* __restrict__ c, float* __restrict__ dinv) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x) {
        const double inv = 1.0 / u[u_rp[r]];
        c[r] = float(scale[r] * inv);
        dinv[r] = float(inv);
    }
}

// One Jacobi sweep on a scaled triangle T (thread per row):
//   out_i = o_i (bs_i base_i - sum_j T_ij ys_j y_j)
// where bs, ys and o are optional per-row scales (nullptr: 1).  Skipped once
// the solver has stopped (flags[S_DONE]).
__global__ void __launch_bounds__(JB_THREADS) k_jacobi32(i64 n, const i64* __restrict__ slice,
                                                          const int32_t* __restrict__ col, const float* __restrict__ val,
                                                          const float* __restrict__ base, const float* __restrict__ bs,
                                                          const float* __restrict__ y, const float* __restrict__ ys,
                                                          const float* __restrict__ o, float* __restrict__ out,
                                                          const double* __restrict__ flags) {
    if (flags && flags[S_DONE] != 0.0) return;
    const i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x;
    if (r >= n) return;
    const i64 sl = r >> 5, beg = slice[sl] + (r & 31), w = (slice[sl + 1] - slice[sl]) >> 5;
    float acc = 0.0f;
    if (ys) {
        for (i64 k = 0; k < w; ++k) {
            const int32_t j = __ldg(col + beg + 32 * k);
            acc += __ldg(val + beg + 32 * k) * (y[j] * __ldg(ys + j));
        }
    } else {
        for (i64 k = 0; k < w; ++k) {
            const int32_t j = __ldg(col + beg + 32 * k);
            acc += __ldg(val + beg + 32 * k) * y[j];
        }
    }
    float b = base[r];
    if (bs) b *= bs[r];
    float v = b - acc;
    if (o) v *= o[r];
    out[r] = v;
}

void sweep(Ctx& ctx, i64 n, const JacobiSlab& s, const float* base, const float* bs, const float* y, const float* ys,
           const float* o, float* out, const double* flags) {
    NL_LAUNCH(k_jacobi32, unsigned((n + JB_THREADS - 1) / JB_THREADS), JB_THREADS, 0, ctx.stream, n, s.slice.p,
              s.col.p, s.val.p, base, bs, y, ys, o, out, flags);
}

}  // namespace

void jacobi_fill(Ctx& ctx, IncompleteCholesky& ic) {
    const i64 n = ic.n;
    for (JacobiSlab* s : {&ic.jlo, &ic.jup})
        NL_LAUNCH(k_jacobi_values, grid_for(n, 256), 256, 0, ctx.stream, n, s->slice.p, s->src.p, ic.rp.p, ic.u.p,
                  s->val.p);
    NL_LAUNCH(k_jacobi_diag, grid_for(n, 256), 256, 0, ctx.stream, n, ic.rp.p, ic.u.p, ic.scale.p, ic.jc.p, ic.jdinv.p);
}

void jacobi_apply32(Ctx& ctx, IncompleteCholesky& ic, int sweeps, const float* r, float* z, const double* flags) {
    NL_REQUIRE(sweeps >= 1, NLGPU_ERR_ARG, "at least one Jacobi sweep per triangle");
    const i64 n = ic.n;
    float* t[2] = {ic.jt0.p, ic.jt1.p};
    // forward: y_t+1 = c r - L y_t from y_0 = c r; the last sweep scales by 1 / u_ii
    const float* prev = r;
    const float* prev_scale = ic.jc.p;
    for (int s = 1; s <= sweeps; ++s) {
        float* out = s == sweeps ? ic.jy.p : t[s & 1];
        sweep(ctx, n, ic.jlo, r, ic.jc.p, prev, prev_scale, s == sweeps ? ic.jdinv.p : nullptr, out, flags);
        prev = out;
        prev_scale = nullptr;
    }
    // backward: z_t+1 = y~ - U z_t from z_0 = y~; the last sweep scales by s_i
    prev = ic.jy.p;
    for (int s = 1; s <= sweeps; ++s) {
        float* out = s == sweeps ? z : t[s & 1];
        sweep(ctx, n, ic.jup, ic.jy.p, nullptr, prev, nullptr, s == sweeps ? ic.scale32.p : nullptr, out, flags);
        prev = out;
    }
}

}  // namespace nlgpu
