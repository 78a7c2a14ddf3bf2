// Values of the conductivity (and capacity) matrices.
//
// Reference: conductivity_matrix_2d::compute (conductivity_matrix_2d.hpp:166-193)
// runs integrator::operator() (integrator.hpp:62-91) for every
// (row node, eL containing it, eNL in neighbours(eL), jNL), recomputing
//   K_ij += (1 - p1) * sum_qL w_qL G_i(qL) . sum_qNL w_qNL phi(x_qL, x_qNL) Lambda(qNL) G_j(qNL)
//         + p1 * [eL == eNL] * sum_q w_q G_i(q) . Lambda(q) G_j(q) / |J(q)|
// (integrate_nonlocal :132-164, integrate_local :106-130) for each entry.
//
// Here the work is organised by element pair.  A CTA owns element eL: the CSR
// segments of its node rows (column numbers and value accumulators) sit in
// shared memory.  Each warp takes one neighbour eNL at a time, stages eNL's
// quadrature data in shared memory and evaluates the pair's whole block once,
// factorised as
//   Phi[qL][qNL] = c_qNL * shape(x_qL, x_qNL)       c_qNL = w_qNL norm (1 - p1) [lambda]
//   H[qL][j]     = sum_qNL Phi[qL][qNL] Lambda G_j(qNL)
//   K[i][j]      = sum_qL (w_qL G_i(qL)) . H[qL][j]
// and adds every entry the reference keeps (matrix_separator_base::part) to
// the shared accumulators; BOUND entries go to global memory.  When the
// problem is symmetric (constant conductivity) each unordered pair is
// evaluated once: the CTA of the element with the smaller (first node, number)
// key takes it, and the block's transposed entries -- which the reference
// computes from the swapped pair, the same value mathematically -- go to the
// other element's rows through global atomics (few with a banded numbering).
// When the CTA is done its accumulators are added to the global values.  Rows
// too long for shared memory fall back to global atomics with a binary search.
#include "common.cuh"
#include "ff.cuh"
#include "influence.cuh"

#include <cmath>

namespace nlgpu {

namespace {

constexpr int AS_THREADS = 256;
constexpr int AS_WARPS = AS_THREADS / 32;

struct AssembleArgs {
    i64 E;
    i64 e0;                   // first element (the float-float kernel's tuning samples start later)
    const int32_t* elems;
    const double* qcoord;     // [e][q][2]
    const double* jac;        // [e][q]
    const double* deriv;      // [e][i][q][2]
    const i64* noff;
    const int32_t* nlist;
    const int32_t* minnode;
    const uint8_t* is_inner;
    const double* cond_field; // isotropic conductivity per quadrature point, or null
    const i64* in_rp; const int32_t* in_col; double* in_val;
    const i64* bd_rp; const int32_t* bd_col; double* bd_val;
    bool symmetric;
    int cap;                  // accumulator entries in shared memory
    int* error;               // set when an entry is missing from its pattern
};

__device__ __forceinline__ i64 find_col(const int32_t* col, i64 lo, i64 hi, int32_t c) {
    while (lo < hi) {
        const i64 mid = (lo + hi) >> 1;
        if (col[mid] < c) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void add_global(const i64* rp, const int32_t* col, double* val, int32_t r, int32_t c, double v,
                                           int* error) {
    const i64 pos = find_col(col, rp[r], rp[r + 1], c);
    if (pos < rp[r + 1] && col[pos] == c) atomicAdd(val + pos, v);
    else atomicExch(error, 1);
}

template<int NEN, int NQ>
struct PairSmem {
    double qx[NQ], qy[NQ];
    double gx[NEN * NQ], gy[NEN * NQ];
    double phi[NQ * NQ];
    double hx[NQ * NEN], hy[NQ * NEN];
    double c[NQ];             // c_qNL
    int32_t nodes[NEN];
};

template<int NEN, int NQ, int INF, bool SYM>
__global__ void __launch_bounds__(AS_THREADS) k_assemble_pairs(AssembleArgs a, Model m, Basis b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double eqx[NQ], eqy[NQ], egx[NEN * NQ], egy[NEN * NQ], ewx[NEN * NQ], ewy[NEN * NQ], ejac[NQ], elam[NQ];
    __shared__ int32_t enodes[NEN];
    __shared__ i64 row_start[NEN];
    __shared__ int row_len[NEN], row_off[NEN + 1];
    __shared__ int use_smem;

    auto* pairs = reinterpret_cast<PairSmem<NEN, NQ>*>(smem_raw);
    double* acc = reinterpret_cast<double*>(smem_raw + sizeof(PairSmem<NEN, NQ>) * AS_WARPS);
    int32_t* cols = reinterpret_cast<int32_t*>(acc + a.cap);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    PairSmem<NEN, NQ>& ps = pairs[warp];
    const double cnl = m.norm * (1.0 - m.p1);
    const bool iso = m.cond_kind == NLGPU_CONDUCTIVITY_ISOTROPIC;

    for (i64 eL = blockIdx.x; eL < a.E; eL += gridDim.x) {
        // ---- element eL: quadrature data, weighted gradients and its node rows
        for (int t = threadIdx.x; t < NEN * NQ; t += AS_THREADS) {
            const double gx = a.deriv[2 * (eL * NEN * NQ + t)], gy = a.deriv[2 * (eL * NEN * NQ + t) + 1];
            egx[t] = gx; egy[t] = gy;
            ewx[t] = b.w[t % NQ] * gx; ewy[t] = b.w[t % NQ] * gy;
        }
        for (int t = threadIdx.x; t < NQ; t += AS_THREADS) {
            eqx[t] = a.qcoord[2 * (eL * NQ + t)];
            eqy[t] = a.qcoord[2 * (eL * NQ + t) + 1];
            ejac[t] = a.jac[eL * NQ + t];
            elam[t] = a.cond_field ? a.cond_field[eL * NQ + t] : m.cond[0];
        }
        if (threadIdx.x < NEN) {
            const int32_t r = a.elems[eL * NEN + threadIdx.x];
            enodes[threadIdx.x] = r;
            row_start[threadIdx.x] = a.in_rp[r];
            row_len[threadIdx.x] = a.is_inner[r] ? int(a.in_rp[r + 1] - a.in_rp[r]) : 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int off = 0;
            for (int i = 0; i < NEN; ++i) { row_off[i] = off; off += row_len[i]; }
            row_off[NEN] = off;
            use_smem = off <= a.cap;
        }
        __syncthreads();
        const bool smem_rows = use_smem;
        if (smem_rows) {
            for (int i = 0; i < NEN; ++i)
                for (int t = threadIdx.x; t < row_len[i]; t += AS_THREADS) {
                    cols[row_off[i] + t] = a.in_col[row_start[i] + t];
                    acc[row_off[i] + t] = 0.0;
                }
        }
        __syncthreads();
        const int32_t key_l = SYM ? a.minnode[eL] : 0;

        // ---- pairs (eL, eNL): one warp each
        const i64 kb = a.noff[eL], ke = a.noff[eL + 1];
        for (i64 k = kb + warp; k < ke; k += AS_WARPS) {
            const int32_t eNL = a.nlist[k];
            if constexpr (SYM) {   // the pair belongs to the element with the smaller key
                const int32_t key_n = a.minnode[eNL];
                if (key_n < key_l || (key_n == key_l && eNL < int32_t(eL))) continue;
            }
            for (int t = lane; t < NEN * NQ; t += 32) {
                ps.gx[t] = a.deriv[2 * (i64(eNL) * NEN * NQ + t)];
                ps.gy[t] = a.deriv[2 * (i64(eNL) * NEN * NQ + t) + 1];
            }
            if (lane < NQ) {
                ps.qx[lane] = a.qcoord[2 * (i64(eNL) * NQ + lane)];
                ps.qy[lane] = a.qcoord[2 * (i64(eNL) * NQ + lane) + 1];
                const double lam = a.cond_field ? a.cond_field[i64(eNL) * NQ + lane] : m.cond[0];
                ps.c[lane] = b.w[lane] * cnl * (iso ? lam : 1.0);
            }
            if (lane < NEN) ps.nodes[lane] = a.elems[i64(eNL) * NEN + lane];
            __syncwarp();
            for (int t = lane; t < NQ * NQ; t += 32) {
                const int qL = t / NQ, qNL = t % NQ;
                ps.phi[t] = ps.c[qNL] * shape<INF>(m, eqx[qL] - ps.qx[qNL], eqy[qL] - ps.qy[qNL]);
            }
            __syncwarp();
            for (int t = lane; t < NQ * NEN; t += 32) {
                const int qL = t / NEN, j = t % NEN;
                double h0 = 0.0, h1 = 0.0;
                #pragma unroll
                for (int qNL = 0; qNL < NQ; ++qNL) {
                    const double f = ps.phi[qL * NQ + qNL];
                    const double gx = ps.gx[j * NQ + qNL], gy = ps.gy[j * NQ + qNL];
                    if (m.cond_kind != NLGPU_CONDUCTIVITY_ANISOTROPIC) { h0 += f * gx; h1 += f * gy; }
                    else { h0 += f * (m.cond[0] * gx + m.cond[2] * gy); h1 += f * (m.cond[2] * gx + m.cond[1] * gy); }
                }
                if (m.cond_kind == NLGPU_CONDUCTIVITY_ORTHOTROPIC) { h0 *= m.cond[0]; h1 *= m.cond[1]; }
                ps.hx[t] = h0; ps.hy[t] = h1;
            }
            __syncwarp();
            const bool self = eNL == int32_t(eL);
            for (int t = lane; t < NEN * NEN; t += 32) {
                const int i = t / NEN, j = t % NEN;
                const int32_t r = enodes[i], c = ps.nodes[j];
                const bool r_in = a.is_inner[r], c_in = a.is_inner[c];
                // (r, c) from this pair; (c, r) from the swapped pair when it is folded into this one
                const bool fwd_inner = c_in && r_in && (!a.symmetric || r <= c);
                const bool fwd_bound = !c_in && r != c;
                const bool tr = SYM && !self;
                const bool bwd_inner = tr && c_in && r_in && c <= r;
                const bool bwd_bound = tr && !r_in && c != r;
                if (!fwd_inner && !fwd_bound && !bwd_inner && !bwd_bound) continue;
                double v = 0.0;
                #pragma unroll
                for (int qL = 0; qL < NQ; ++qL)
                    v = fma(ewy[i * NQ + qL], ps.hy[qL * NEN + j], fma(ewx[i * NQ + qL], ps.hx[qL * NEN + j], v));
                if (self) {
                    double loc = 0.0;
                    #pragma unroll
                    for (int q = 0; q < NQ; ++q) {
                        const double ax = egx[i * NQ + q], ay = egy[i * NQ + q];
                        const double bx = egx[j * NQ + q], by = egy[j * NQ + q];
                        double val;
                        if (iso) val = elam[q] * (ax * bx + ay * by);
                        else if (m.cond_kind == NLGPU_CONDUCTIVITY_ORTHOTROPIC) val = m.cond[0] * ax * bx + m.cond[1] * ay * by;
                        else val = ax * (m.cond[0] * bx + m.cond[2] * by) + ay * (m.cond[2] * bx + m.cond[1] * by);
                        loc += b.w[q] * val / ejac[q];
                    }
                    v += m.p1 * loc;
                }
                if (fwd_inner) {
                    if (smem_rows) {
                        const i64 pos = find_col(cols, row_off[i], row_off[i + 1], c);
                        if (pos < row_off[i + 1] && cols[pos] == c) atomicAdd(acc + pos, v);
                        else atomicExch(a.error, 1);
                    } else {
                        add_global(a.in_rp, a.in_col, a.in_val, r, c, v, a.error);
                    }
                }
                if (fwd_bound) add_global(a.bd_rp, a.bd_col, a.bd_val, r, c, v, a.error);
                if (bwd_inner) add_global(a.in_rp, a.in_col, a.in_val, c, r, v, a.error);
                if (bwd_bound) add_global(a.bd_rp, a.bd_col, a.bd_val, c, r, v, a.error);
            }
            __syncwarp();
        }
        __syncthreads();
        if (smem_rows)
            for (int i = 0; i < NEN; ++i)
                for (int t = threadIdx.x; t < row_len[i]; t += AS_THREADS) {
                    const double v = acc[row_off[i] + t];
                    if (v != 0.0) atomicAdd(a.in_val + row_start[i] + t, v);
                }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- float-float
// The same pair blocks with the influence values and both contractions in
// float-float arithmetic (ff.cuh) on the FP32 pipes -- the mixed-precision
// form's FP32 nonlocal blocks, carried to about 48 bits so that the matrix
// stays within the FP64 entries' tolerance and the FP64 refinement converges
// to the FP64 solution.  Only the rows' accumulators, the rare self term and
// the index work stay FP64 / integer.  Element data is staged once per
// assembly as float-float (k_ff_stage), so the pair loop converts nothing.
// 16 or 32 warps per CTA (the FP64 kernel's 8 leave the FP32 pipes idle),
// chosen per problem by timing both on a sample of elements (ff_warps).

struct FFArgs {
    const float4* deriv;    // [e][i][q]: (gx.h, gx.l, gy.h, gy.l)
    const float4* qcoord;   // [e][q]: (x/r0 .h, .l, y/r1 .h, .l), coordinates in units of the radii
    const float2* cw;       // [e][q]: c_q = w_q norm (1 - p1) [lambda_q]
    FFExpTable exp_table;   // exp(k / 256), copied to shared memory by each CTA
};

__global__ void k_ff_stage(i64 E, int nen, int nq, const double* __restrict__ deriv, const double* __restrict__ qcoord,
                           const double* __restrict__ cond_field, Model m, Basis b, float4* __restrict__ dff,
                           float4* __restrict__ qff, float2* __restrict__ cw) {
    const double cnl = m.norm * (1.0 - m.p1);
    const bool iso = m.cond_kind == NLGPU_CONDUCTIVITY_ISOTROPIC;
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < E * nen * nq; t += i64(gridDim.x) * blockDim.x) {
        const ff gx = ff_from(deriv[2 * t]), gy = ff_from(deriv[2 * t + 1]);
        dff[t] = make_float4(gx.h, gx.l, gy.h, gy.l);
        if (t < E * nq) {
            const ff x = ff_from(qcoord[2 * t] * m.inv_r[0]), y = ff_from(qcoord[2 * t + 1] * m.inv_r[1]);
            qff[t] = make_float4(x.h, x.l, y.h, y.l);
            const double lam = cond_field ? cond_field[t] : m.cond[0];
            const ff c = ff_from(b.w[t % nq] * cnl * (iso ? lam : 1.0));
            cw[t] = make_float2(c.h, c.l);
        }
    }
}

// per warp: eNL's data; g holds eNL's gradients (x then y) for H = Phi (Lambda
// G) and then H itself (x then y), which the lanes keep in registers until
// every lane has read G
template<int NEN, int NQ>
struct PairFF {
    ff qx[NQ], qy[NQ];
    ff g[2 * NEN * NQ];
    ff phi[NQ * NQ];
    ff c[NQ];
    int32_t nodes[NEN];
    int32_t inner[NEN];   // whether each of eNL's nodes is inner (read once per pair, not per entry)
};

// shape<INF> in float-float (fast polynomial, polynomial and exponential with
// p divisible by n; the host sends the other kinds to the FP64 kernel)
// z0, z1: the coordinate differences in units of the radii
template<int INF>
__device__ __forceinline__ ff shape_ff(const Model& m, ff z0, ff z1, ff q, const ff* exp_table) {
    ff d;
    if (m.n == 2) d = ff_add(ff_mul(z0, z0), ff_mul(z1, z1));
    else if (m.n == 1) d = ff_add(ff_abs(z0), ff_abs(z1));
    else d = ff_add(ff_ipow(ff_abs(z0), m.n), ff_ipow(ff_abs(z1), m.n));
    if constexpr (INF == NLGPU_INFLUENCE_FAST_POLYNOMIAL) {
        return ff_lt(d, 1.0f) ? ff_sub(ff_make(1.0f), d) : ff_make(0.0f);
    } else {
        const ff dp = ff_ipow(d, m.p / m.n);
        if constexpr (INF == NLGPU_INFLUENCE_POLYNOMIAL)
            return ff_lt(d, 1.0f) ? ff_ipow(ff_sub(ff_make(1.0f), dp), int(m.q)) : ff_make(0.0f);
        else
            return ff_exp_nonpositive(ff_neg(ff_mul(q, dp)), exp_table);
    }
}

template<int NEN, int NQ, int INF, bool SYM, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_assemble_pairs_ff(AssembleArgs a, FFArgs f, Model m, Basis b) {
    constexpr int THREADS = WARPS * 32;
    constexpr int HN = 2 * NQ * NEN, HR = (HN + 31) / 32;   // H outputs and lane rounds
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ ff eqx[NQ], eqy[NQ], ewx[NEN * NQ], ewy[NEN * NQ];
    __shared__ double egx[NEN * NQ], egy[NEN * NQ], ejac[NQ], elam[NQ];   // the self term stays FP64
    __shared__ int32_t enodes[NEN], einner[NEN];   // eL's nodes and whether each is inner
    __shared__ i64 row_start[NEN];
    __shared__ int row_len[NEN], row_off[NEN + 1];
    __shared__ int use_smem;
    __shared__ ff etab[2 * FF_EXP_K + 1];
    for (int t = threadIdx.x; t < 2 * FF_EXP_K + 1; t += blockDim.x)
        etab[t] = ff{f.exp_table.v[t].x, f.exp_table.v[t].y};

    auto* pairs = reinterpret_cast<PairFF<NEN, NQ>*>(smem_raw);
    double* acc = reinterpret_cast<double*>(smem_raw + sizeof(PairFF<NEN, NQ>) * WARPS);
    int32_t* cols = reinterpret_cast<int32_t*>(acc + a.cap);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    PairFF<NEN, NQ>& ps = pairs[warp];
    const bool iso = m.cond_kind == NLGPU_CONDUCTIVITY_ISOTROPIC;
    const ff qf = ff_from(m.q);
    const ff k0 = ff_from(m.cond[0]), k1 = ff_from(m.cond[1]), k2 = ff_from(m.cond[2]);

    for (i64 eL = a.e0 + blockIdx.x; eL < a.E; eL += gridDim.x) {
        // ---- element eL: quadrature data, weighted gradients and its node rows
        for (int t = threadIdx.x; t < NEN * NQ; t += THREADS) {
            egx[t] = a.deriv[2 * (eL * NEN * NQ + t)];
            egy[t] = a.deriv[2 * (eL * NEN * NQ + t) + 1];
            const float4 g = f.deriv[eL * NEN * NQ + t];
            const ff w = ff_from(b.w[t % NQ]);
            ewx[t] = ff_mul(w, ff{g.x, g.y});
            ewy[t] = ff_mul(w, ff{g.z, g.w});
        }
        for (int t = threadIdx.x; t < NQ; t += THREADS) {
            const float4 q = f.qcoord[eL * NQ + t];
            eqx[t] = ff{q.x, q.y};
            eqy[t] = ff{q.z, q.w};
            ejac[t] = a.jac[eL * NQ + t];
            elam[t] = a.cond_field ? a.cond_field[eL * NQ + t] : m.cond[0];
        }
        if (threadIdx.x < NEN) {
            const int32_t r = a.elems[eL * NEN + threadIdx.x];
            const bool r_in = a.is_inner[r];
            enodes[threadIdx.x] = r;
            einner[threadIdx.x] = r_in;
            row_start[threadIdx.x] = a.in_rp[r];
            row_len[threadIdx.x] = r_in ? int(a.in_rp[r + 1] - a.in_rp[r]) : 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int off = 0;
            for (int i = 0; i < NEN; ++i) { row_off[i] = off; off += row_len[i]; }
            row_off[NEN] = off;
            use_smem = off <= a.cap;
        }
        __syncthreads();
        const bool smem_rows = use_smem;
        if (smem_rows) {
            for (int i = 0; i < NEN; ++i)
                for (int t = threadIdx.x; t < row_len[i]; t += THREADS) {
                    cols[row_off[i] + t] = a.in_col[row_start[i] + t];
                    acc[row_off[i] + t] = 0.0;
                }
        }
        __syncthreads();
        const int32_t key_l = SYM ? a.minnode[eL] : 0;

        // ---- pairs (eL, eNL): one warp each
        const i64 kb = a.noff[eL], ke = a.noff[eL + 1];
        for (i64 k = kb + warp; k < ke; k += WARPS) {
            const int32_t eNL = a.nlist[k];
            if constexpr (SYM) {   // the pair belongs to the element with the smaller key
                const int32_t key_n = a.minnode[eNL];
                if (key_n < key_l || (key_n == key_l && eNL < int32_t(eL))) continue;
            }
            for (int t = lane; t < NEN * NQ; t += 32) {
                const float4 g = f.deriv[i64(eNL) * NEN * NQ + t];
                ps.g[t] = ff{g.x, g.y};
                ps.g[NEN * NQ + t] = ff{g.z, g.w};
            }
            if (lane < NQ) {
                const float4 q = f.qcoord[i64(eNL) * NQ + lane];
                ps.qx[lane] = ff{q.x, q.y};
                ps.qy[lane] = ff{q.z, q.w};
                const float2 c = f.cw[i64(eNL) * NQ + lane];
                ps.c[lane] = ff{c.x, c.y};
            }
            if (lane < NEN) {
                const int32_t c = a.elems[i64(eNL) * NEN + lane];
                ps.nodes[lane] = c;
                ps.inner[lane] = a.is_inner[c];
            }
            __syncwarp();
            for (int t = lane; t < NQ * NQ; t += 32) {
                const int qL = t / NQ, qNL = t % NQ;
                ps.phi[t] = ff_mul(ps.c[qNL], shape_ff<INF>(m, ff_sub(eqx[qL], ps.qx[qNL]), ff_sub(eqy[qL], ps.qy[qNL]),
                                                             qf, etab));
            }
            __syncwarp();
            // one lane per (direction, qL, j): 2 NQ NEN dots of NQ terms fill
            // the lanes better than NQ NEN pairs of dots (144 = 4.5 rounds of
            // 32 against 72 = 2.25 rounds of double work for the 8-node element)
            ff hv[HR];
#pragma unroll
            for (int rnd = 0; rnd < HR; ++rnd) {
                const int t = lane + 32 * rnd;
                if (t < HN) {
                    const int dir = t >= NQ * NEN, u = dir ? t - NQ * NEN : t;
                    const int qL = u / NEN, j = u % NEN;
                    const ff* gd = ps.g + dir * NEN * NQ;
                    ffdot d;
#pragma unroll
                    for (int qNL = 0; qNL < NQ; ++qNL) {
                        const ff fq = ps.phi[qL * NQ + qNL];
                        if (m.cond_kind != NLGPU_CONDUCTIVITY_ANISOTROPIC) {
                            ffdot_add(d, fq, gd[j * NQ + qNL]);
                        } else {
                            const ff gx = ps.g[j * NQ + qNL], gy = ps.g[NEN * NQ + j * NQ + qNL];
                            ffdot_add(d, fq, dir ? ff_add(ff_mul(k2, gx), ff_mul(k1, gy))
                                                 : ff_add(ff_mul(k0, gx), ff_mul(k2, gy)));
                        }
                    }
                    hv[rnd] = ffdot_value(d);
                    if (m.cond_kind == NLGPU_CONDUCTIVITY_ORTHOTROPIC) hv[rnd] = ff_mul(hv[rnd], dir ? k1 : k0);
                }
            }
            __syncwarp();   // every lane has read G: H (x then y, [qL][j]) replaces it
#pragma unroll
            for (int rnd = 0; rnd < HR; ++rnd)
                if (lane + 32 * rnd < HN) ps.g[lane + 32 * rnd] = hv[rnd];
            __syncwarp();
            const bool self = eNL == int32_t(eL);
            for (int t = lane; t < NEN * NEN; t += 32) {
                const int i = t / NEN, j = t % NEN;
                const int32_t r = enodes[i], c = ps.nodes[j];
                const bool r_in = einner[i] != 0, c_in = ps.inner[j] != 0;
                const bool fwd_inner = c_in && r_in && (!a.symmetric || r <= c);
                const bool fwd_bound = !c_in && r != c;
                const bool tr = SYM && !self;
                const bool bwd_inner = tr && c_in && r_in && c <= r;
                const bool bwd_bound = tr && !r_in && c != r;
                if (!fwd_inner && !fwd_bound && !bwd_inner && !bwd_bound) continue;
                ffdot dv;
#pragma unroll
                for (int qL = 0; qL < NQ; ++qL) {
                    ffdot_add(dv, ewx[i * NQ + qL], ps.g[qL * NEN + j]);
                    ffdot_add(dv, ewy[i * NQ + qL], ps.g[NQ * NEN + qL * NEN + j]);
                }
                double v = ff_to(ffdot_value(dv));
                if (self) {
                    double loc = 0.0;
#pragma unroll
                    for (int q = 0; q < NQ; ++q) {
                        const double ax = egx[i * NQ + q], ay = egy[i * NQ + q];
                        const double bx = egx[j * NQ + q], by = egy[j * NQ + q];
                        double val;
                        if (iso) val = elam[q] * (ax * bx + ay * by);
                        else if (m.cond_kind == NLGPU_CONDUCTIVITY_ORTHOTROPIC) val = m.cond[0] * ax * bx + m.cond[1] * ay * by;
                        else val = ax * (m.cond[0] * bx + m.cond[2] * by) + ay * (m.cond[2] * bx + m.cond[1] * by);
                        loc += b.w[q] * val / ejac[q];
                    }
                    v += m.p1 * loc;
                }
                if (fwd_inner) {
                    if (smem_rows) {
                        const i64 pos = find_col(cols, row_off[i], row_off[i + 1], c);
                        if (pos < row_off[i + 1] && cols[pos] == c) atomicAdd(acc + pos, v);
                        else atomicExch(a.error, 1);
                    } else {
                        add_global(a.in_rp, a.in_col, a.in_val, r, c, v, a.error);
                    }
                }
                if (fwd_bound) add_global(a.bd_rp, a.bd_col, a.bd_val, r, c, v, a.error);
                if (bwd_inner) add_global(a.in_rp, a.in_col, a.in_val, c, r, v, a.error);
                if (bwd_bound) add_global(a.bd_rp, a.bd_col, a.bd_val, c, r, v, a.error);
            }
            __syncwarp();
        }
        __syncthreads();
        if (smem_rows)
            for (int i = 0; i < NEN; ++i)
                for (int t = threadIdx.x; t < row_len[i]; t += THREADS) {
                    const double v = acc[row_off[i] + t];
                    if (v != 0.0) atomicAdd(a.in_val + row_start[i] + t, v);
                }
        __syncthreads();
    }
}

// Local integrands, one thread per (e, i, j): conductivity
// (integrate_local, conductivity_matrix_2d.hpp:106-130) or capacity
// (integrate_basic_pair, heat_capacity_matrix_2d.hpp:30-37).
__global__ void k_assemble_local(i64 E, int nen, int nq, const int32_t* __restrict__ elems,
                                 const double* __restrict__ jac, const double* __restrict__ deriv,
                                 const uint8_t* __restrict__ is_inner, const double* __restrict__ cond_field,
                                 Model m, Basis b, int integrand, double weight, bool symmetric,
                                 const i64* __restrict__ rp, const int32_t* __restrict__ col, double* __restrict__ val,
                                 const i64* __restrict__ bd_rp, const int32_t* __restrict__ bd_col, double* __restrict__ bd_val) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < E * nen * nen; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / (nen * nen);
        const int i = int((t / nen) % nen), j = int(t % nen);
        const int32_t r = elems[e * nen + i], c = elems[e * nen + j];
        const bool keep_inner = is_inner[c] && is_inner[r] && (!symmetric || r <= c);
        const bool keep_bound = !is_inner[c] && r != c && bd_rp != nullptr;
        if (!keep_inner && !keep_bound) continue;
        double integral = 0.0;
        for (int q = 0; q < nq; ++q) {
            if (integrand == 1) {
                integral += b.w[q] * b.qN[i * nq + q] * b.qN[j * nq + q] * jac[e * nq + q];
            } else {
                const double* di = deriv + 2 * ((e * nen + i) * nq + q);
                const double* dj = deriv + 2 * ((e * nen + j) * nq + q);
                double v;
                if (m.cond_kind == NLGPU_CONDUCTIVITY_ISOTROPIC)
                    v = (cond_field ? cond_field[e * nq + q] : m.cond[0]) * (di[0] * dj[0] + di[1] * dj[1]);
                else if (m.cond_kind == NLGPU_CONDUCTIVITY_ORTHOTROPIC) v = m.cond[0] * di[0] * dj[0] + m.cond[1] * di[1] * dj[1];
                else v = di[0] * (m.cond[0] * dj[0] + m.cond[2] * dj[1]) + di[1] * (m.cond[2] * dj[0] + m.cond[1] * dj[1]);
                integral += b.w[q] * v / jac[e * nq + q];
            }
        }
        integral *= weight;
        if (keep_inner) {
            const i64 pos = find_col(col, rp[r], rp[r + 1], c);
            if (pos < rp[r + 1] && col[pos] == c) atomicAdd(val + pos, integral);
        } else {
            const i64 pos = find_col(bd_col, bd_rp[r], bd_rp[r + 1], c);
            if (pos < bd_rp[r + 1] && bd_col[pos] == c) atomicAdd(bd_val + pos, integral);
        }
    }
}

__global__ void k_dirichlet_diagonal(i64 n, const uint8_t* __restrict__ is_inner, const i64* __restrict__ rp,
                                     double* __restrict__ val, double value) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x)
        if (!is_inner[r]) val[rp[r]] = value;
}

__global__ void k_gather_full(i64 nnz, const i64* __restrict__ map, const double* __restrict__ upper,
                              double* __restrict__ full, float* __restrict__ full32) {
    for (i64 k = blockIdx.x * i64(blockDim.x) + threadIdx.x; k < nnz; k += i64(gridDim.x) * blockDim.x) {
        const i64 s = map[k];
        const double v = s >= 0 ? upper[s] : 0.0;
        full[k] = v;
        if (full32) full32[k] = float(v);
    }
}

template<int NEN, int NQ, int INF>
void launch_pairs(Ctx& ctx, const AssembleArgs& a, bool sym) {
    const size_t fixed = sizeof(PairSmem<NEN, NQ>) * AS_WARPS;
    const size_t dyn = fixed + size_t(a.cap) * (sizeof(double) + sizeof(int32_t));
    const unsigned grid = unsigned(std::min<i64>(a.E, 152 * 16));
    if (sym) {
        auto kernel = k_assemble_pairs<NEN, NQ, INF, true>;
        NL_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dyn)));
        NL_LAUNCH(kernel, grid, AS_THREADS, dyn, ctx.stream, a, ctx.model, ctx.basis);
    } else {
        auto kernel = k_assemble_pairs<NEN, NQ, INF, false>;
        NL_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dyn)));
        NL_LAUNCH(kernel, grid, AS_THREADS, dyn, ctx.stream, a, ctx.model, ctx.basis);
    }
}

template<int NEN, int NQ>
void dispatch_influence(Ctx& ctx, const AssembleArgs& a, bool sym) {
    switch (ctx.model.influence) {
    case NLGPU_INFLUENCE_FAST_POLYNOMIAL: launch_pairs<NEN, NQ, NLGPU_INFLUENCE_FAST_POLYNOMIAL>(ctx, a, sym); break;
    case NLGPU_INFLUENCE_POLYNOMIAL: launch_pairs<NEN, NQ, NLGPU_INFLUENCE_POLYNOMIAL>(ctx, a, sym); break;
    case NLGPU_INFLUENCE_EXPONENTIAL: launch_pairs<NEN, NQ, NLGPU_INFLUENCE_EXPONENTIAL>(ctx, a, sym); break;
    default: launch_pairs<NEN, NQ, NLGPU_INFLUENCE_CONSTANT>(ctx, a, sym); break;
    }
}

template<int NEN, int NQ, int INF, int WARPS>
void launch_pairs_ff_w(Ctx& ctx, AssembleArgs a, const FFArgs& f, bool sym) {
    auto kernel = sym ? k_assemble_pairs_ff<NEN, NQ, INF, true, WARPS> : k_assemble_pairs_ff<NEN, NQ, INF, false, WARPS>;
    // the row accumulators take what shared memory the per-warp blocks leave
    int dev = 0, optin = 0;
    NL_CUDA(cudaGetDevice(&dev));
    NL_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa{};
    NL_CUDA(cudaFuncGetAttributes(&fa, kernel));
    const size_t fixed = sizeof(PairFF<NEN, NQ>) * WARPS;
    const size_t avail = size_t(optin) - fa.sharedSizeBytes;
    NL_REQUIRE(avail > fixed + 4096, NLGPU_ERR_UNSUPPORTED, "not enough shared memory for the pair assembly");
    a.cap = int((avail - fixed) / 12);
    const size_t dyn = fixed + size_t(a.cap) * (sizeof(double) + sizeof(int32_t));
    const unsigned grid = unsigned(std::max<i64>(1, std::min<i64>(a.E - a.e0, 152 * 16)));
    NL_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dyn)));
    NL_LAUNCH(kernel, grid, WARPS * 32, dyn, ctx.stream, a, f, ctx.model, ctx.basis);
}

// Warps per CTA: forced by NLGPU_OPTION_ASSEMBLY_WARPS, else tuned once per
// (element type, influence kind, pair mode) and context by timing both forms
// on the same sample of elements from the middle of the mesh (their
// contributions are cleared afterwards: the matrices are zeroed again).
template<int NEN, int NQ, int INF>
void launch_pairs_ff(Ctx& ctx, AssembleArgs a, const FFArgs& f, bool sym) {
    int warps = ctx.ff_warps_option;
    if (warps == 0) {
        const int key = NEN * 1000 + INF * 10 + (sym ? 1 : 0);
        auto it = ctx.ff_warps_tuned.find(key);
        if (it != ctx.ff_warps_tuned.end()) {
            warps = it->second;
        } else {
            const i64 sample = std::min<i64>(a.E, 152 * 8);
            AssembleArgs s = a;
            s.e0 = (a.E - sample) / 2;
            s.E = s.e0 + sample;
            double ms[2] = {0.0, 0.0};
            cudaEvent_t ev[2] = {};
            NL_CUDA(cudaEventCreate(&ev[0]));
            NL_CUDA(cudaEventCreate(&ev[1]));
            for (int rep = 0; rep < 2; ++rep)   // the first round warms up
                for (int v = 0; v < 2; ++v) {
                    NL_CUDA(cudaEventRecord(ev[0], ctx.stream));
                    if (v == 0) launch_pairs_ff_w<NEN, NQ, INF, 16>(ctx, s, f, sym);
                    else launch_pairs_ff_w<NEN, NQ, INF, 32>(ctx, s, f, sym);
                    NL_CUDA(cudaEventRecord(ev[1], ctx.stream));
                    NL_CUDA(cudaEventSynchronize(ev[1]));
                    float t = 0.0f;
                    NL_CUDA(cudaEventElapsedTime(&t, ev[0], ev[1]));
                    ms[v] = double(t);
                }
            cudaEventDestroy(ev[0]);
            cudaEventDestroy(ev[1]);
            ctx.inner.val.zero(ctx.stream);
            ctx.bound.val.zero(ctx.stream);
            warps = ms[1] < ms[0] ? 32 : 16;
            ctx.ff_warps_tuned[key] = warps;
            ctx.ff_tune_ms[0] = ms[0];
            ctx.ff_tune_ms[1] = ms[1];
        }
    }
    ctx.ff_warps_used = warps;
    if (warps == 32) launch_pairs_ff_w<NEN, NQ, INF, 32>(ctx, a, f, sym);
    else launch_pairs_ff_w<NEN, NQ, INF, 16>(ctx, a, f, sym);
}

template<int NEN, int NQ>
void dispatch_influence_ff(Ctx& ctx, const AssembleArgs& a, const FFArgs& f, bool sym) {
    switch (ctx.model.influence) {
    case NLGPU_INFLUENCE_FAST_POLYNOMIAL: launch_pairs_ff<NEN, NQ, NLGPU_INFLUENCE_FAST_POLYNOMIAL>(ctx, a, f, sym); break;
    case NLGPU_INFLUENCE_POLYNOMIAL: launch_pairs_ff<NEN, NQ, NLGPU_INFLUENCE_POLYNOMIAL>(ctx, a, f, sym); break;
    default: launch_pairs_ff<NEN, NQ, NLGPU_INFLUENCE_EXPONENTIAL>(ctx, a, f, sym); break;
    }
}

// float-float covers the continuous influence kinds with an integral power
// p / n and constant conductivity; the rest runs the FP64 kernel
bool ff_supported(const Ctx& ctx) {
    const Model& m = ctx.model;
    if (m.n < 1) return false;
    if (m.influence == NLGPU_INFLUENCE_FAST_POLYNOMIAL) return true;
    if (m.influence == NLGPU_INFLUENCE_POLYNOMIAL || m.influence == NLGPU_INFLUENCE_EXPONENTIAL)
        return m.p >= 0 && m.p % m.n == 0;
    return false;
}

}  // namespace

// Assembles p1*K_local + (1-p1)*K_nonlocal (or p1*K_local for a local model)
// into ctx.inner / ctx.bound, whose patterns are already built.
void assemble_full(Ctx& ctx) {
    ctx.inner.val.zero(ctx.stream);
    ctx.bound.val.zero(ctx.stream);
    const Model& m = ctx.model;
    if (!m.nonlocal()) {
        assemble_local(ctx, ctx.inner, m.p1, 0);
        return;
    }
    AssembleArgs a{};
    a.E = ctx.n_elems; a.elems = ctx.elems.p; a.qcoord = ctx.qcoord.p; a.jac = ctx.jac.p; a.deriv = ctx.deriv.p;
    a.noff = ctx.noff.p; a.nlist = ctx.nlist.p; a.minnode = ctx.elem_minnode.p; a.is_inner = ctx.is_inner.p;
    a.cond_field = ctx.cond_field.n ? ctx.cond_field.p : nullptr;
    a.in_rp = ctx.inner.rowptr.p; a.in_col = ctx.inner.col.p; a.in_val = ctx.inner.val.p;
    a.bd_rp = ctx.bound.rowptr.p; a.bd_col = ctx.bound.col.p; a.bd_val = ctx.bound.val.p;
    a.symmetric = ctx.symmetric;
    dbuf<int> err;
    err.resize(1);
    err.zero(ctx.stream);
    a.error = err.p;
    // unordered pairs need a symmetric influence and constant conductivity
    const bool sym = ctx.symmetric && !ctx.cond_field.n && !ctx.ordered_pairs;
    ctx.ff_assembled = ctx.ff_assembly && ff_supported(ctx);
    if (ctx.ff_assembled) {
        const int nen = ctx.basis.nen, nq = ctx.basis.nq;
        ctx.deriv_ff.reserve(size_t(ctx.n_elems * nen * nq));
        ctx.qcoord_ff.reserve(size_t(ctx.n_elems * nq));
        ctx.cw_ff.reserve(size_t(ctx.n_elems * nq));
        NL_LAUNCH(k_ff_stage, grid_for(ctx.n_elems * nen * nq, 256), 256, 0, ctx.stream, ctx.n_elems, nen, nq,
                  ctx.deriv.p, ctx.qcoord.p, a.cond_field, ctx.model, ctx.basis, ctx.deriv_ff.p, ctx.qcoord_ff.p,
                  ctx.cw_ff.p);
        FFArgs f{ctx.deriv_ff.p, ctx.qcoord_ff.p, ctx.cw_ff.p, {}};
        for (int k = -FF_EXP_K; k <= FF_EXP_K; ++k) {
            const double x = std::exp(double(k) / double(FF_EXP_STEPS));
            const float hi = float(x);
            f.exp_table.v[k + FF_EXP_K] = make_float2(hi, float(x - double(hi)));
        }
        if (nen == 4) dispatch_influence_ff<4, 4>(ctx, a, f, sym);
        else dispatch_influence_ff<8, 9>(ctx, a, f, sym);
    } else if (ctx.basis.nen == 4) {
        a.cap = int((200 * 1024 - sizeof(PairSmem<4, 4>) * AS_WARPS) / 12);
        dispatch_influence<4, 4>(ctx, a, sym);
    } else {
        a.cap = int((200 * 1024 - sizeof(PairSmem<8, 9>) * AS_WARPS) / 12);
        dispatch_influence<8, 9>(ctx, a, sym);
    }
    set_dirichlet_diagonal(ctx, ctx.inner, 1.0);
    int herr = 0;
    NL_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof herr, cudaMemcpyDeviceToHost, ctx.stream));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    NL_REQUIRE(herr == 0, NLGPU_ERR_STATE, "assembly met an entry outside the sparsity pattern");
}

void assemble_local(Ctx& ctx, Csr& mtx, double weight, int integrand) {
    const int nen = ctx.basis.nen, nq = ctx.basis.nq;
    const i64 work = ctx.n_elems * nen * nen;
    const bool with_bound = &mtx == &ctx.inner;
    NL_LAUNCH(k_assemble_local, grid_for(work, 256), 256, 0, ctx.stream, ctx.n_elems, nen, nq, ctx.elems.p, ctx.jac.p,
              ctx.deriv.p, ctx.is_inner.p, ctx.cond_field.n ? ctx.cond_field.p : nullptr, ctx.model, ctx.basis,
              integrand, weight, ctx.symmetric || integrand == 1, mtx.rowptr.p, mtx.col.p, mtx.val.p,
              with_bound ? ctx.bound.rowptr.p : nullptr, with_bound ? ctx.bound.col.p : nullptr,
              with_bound ? ctx.bound.val.p : nullptr);
    set_dirichlet_diagonal(ctx, mtx, 1.0);
}

void set_dirichlet_diagonal(Ctx& ctx, Csr& mtx, double value) {
    NL_LAUNCH(k_dirichlet_diagonal, grid_for(mtx.rows, 256), 256, 0, ctx.stream, mtx.rows, ctx.is_inner.p,
              mtx.rowptr.p, mtx.val.p, value);
}

void fill_full_from_upper(Ctx& ctx, const Csr& upper, Csr& full, const dbuf<i64>& map) {
    full.val.resize(size_t(full.nnz));
    NL_LAUNCH(k_gather_full, grid_for(full.nnz, 256), 256, 0, ctx.stream, full.nnz, map.p, upper.val.p, full.val.p,
              full.val32.n ? full.val32.p : nullptr);
}

// ---------------------------------------------------------------- nonstationary
namespace {

// K <- dt K + C row by row (C's pattern is contained in K's), unit Dirichlet
// diagonal; bound <- dt bound (nonstationary_heat_equation_solver_2d.hpp:77-82).
__global__ void k_combine(i64 n, double dt, const uint8_t* __restrict__ is_inner, const i64* __restrict__ krp,
                          const int32_t* __restrict__ kcol, double* __restrict__ kval, const i64* __restrict__ crp,
                          const int32_t* __restrict__ ccol, const double* __restrict__ cval, const i64* __restrict__ brp,
                          double* __restrict__ bval) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < n; r += i64(gridDim.x) * blockDim.x) {
        for (i64 k = krp[r]; k < krp[r + 1]; ++k) kval[k] *= dt;
        for (i64 k = brp[r]; k < brp[r + 1]; ++k) bval[k] *= dt;
        i64 k = krp[r];
        for (i64 s = crp[r]; s < crp[r + 1]; ++s) {
            while (k < krp[r + 1] && kcol[k] != ccol[s]) ++k;
            if (k < krp[r + 1]) kval[k] += cval[s];
        }
        if (!is_inner[r]) kval[krp[r]] = 1.0;
    }
}

// Dirichlet vector of a step: value on every Dirichlet node (or the uploaded per-node values)
__global__ void k_step_dirichlet(i64 n, const uint8_t* __restrict__ is_inner, double value, bool per_node,
                                 double* __restrict__ xd) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)
        xd[i] = is_inner[i] ? 0.0 : (per_node ? xd[i] : value);
}

__global__ void k_axpy_into(i64 n, double a, const double* __restrict__ x, double* __restrict__ y) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x) y[i] += a * x[i];
}

}  // namespace

void combine_nonstationary(Ctx& ctx, double dt) {
    NL_LAUNCH(k_combine, grid_for(ctx.n_nodes, 256), 256, 0, ctx.stream, ctx.n_nodes, dt, ctx.is_inner.p,
              ctx.inner.rowptr.p, ctx.inner.col.p, ctx.inner.val.p, ctx.capacity_m.rowptr.p, ctx.capacity_m.col.p,
              ctx.capacity_m.val.p, ctx.bound.rowptr.p, ctx.bound.val.p);
}

// rhs = dt * rhs_init + C T_prev, then the first-kind step with the step's Dirichlet values
void nonstationary_rhs(Ctx& ctx, double dirichlet_value, bool per_node_values, const double* radiation) {
    const i64 n = ctx.n_nodes;
    NL_LAUNCH(k_step_dirichlet, grid_for(n, 256), 256, 0, ctx.stream, n, ctx.is_inner.p, dirichlet_value,
              per_node_values, ctx.step_xd.p);
    spmv_full(ctx, ctx.capacity_full, ctx.temperature.p, ctx.step_tmp.p);
    NL_LAUNCH(k_axpy_into, grid_for(n, 256), 256, 0, ctx.stream, n, ctx.time_step, ctx.rhs_init.p, ctx.step_tmp.p);
    if (radiation)
        NL_LAUNCH(k_axpy_into, grid_for(n, 256), 256, 0, ctx.stream, n, ctx.time_step, radiation, ctx.step_tmp.p);
    apply_first_kind(ctx, ctx.bound, ctx.step_tmp.p, ctx.rhs.p, ctx.step_xd.p);
}

}  // namespace nlgpu
