// Nonlocal plane elasticity: the stiffness system of equilibrium_equation
// (mechanical/equilibrium_equation_2d.hpp:19-60) with two degrees of freedom
// per node, row and column 2 node + component as matrix_assembler_2d<.., 2>
// numbers them (matrix_assembler_2d.hpp, integrator.hpp:42-91).
//
// Reference: stiffness_matrix::compute (stiffness_matrix_2d.hpp:176-197) runs
// the same mesh_run as the conductivity matrix; per (row node, eL, eNL, jNL) it
// integrates a 2x2 block
//   local     sum_q (w_q / |J_q|) C(G_i(q), G_j(q))             (:45-79)
//   nonlocal  sum_qL w_qL sum_qNL w_qNL phi(x_qL, x_qNL) C(G_i(qL), G_j(qNL))   (:81-121)
// with the Hooke combination C of (a, b) = (w dN_i, w dN_j):
//   XX = h11 a_x b_x + h16 (a_x b_y + a_y b_x) + h66 a_y b_y
//   XY = h12 a_x b_y + h16 a_x b_x + h66 a_y b_x + h26 a_y b_y
//   YX = h12 a_y b_x + h16 a_x b_x + h66 a_x b_y + h26 a_y b_y
//   YY = h22 a_y b_y + h26 (a_x b_y + a_y b_x) + h66 a_x b_x
// (isotropic: h22 = h11, h16 = h26 = 0; orthotropic: h16 = h26 = 0), mixed as
// p1 local + (1 - p1) nonlocal, and splits each entry by
// matrix_separator_base::part on the degree-of-freedom indices.
//
// Here the patterns come from the node adjacency (the same candidate columns
// as the thermal pattern) expanded to 2x2 blocks and classified per degree of
// freedom; the values are integrated by element pair with a warp per ordered
// pair (eL, eNL): Phi[qL][qNL] once, then H_b[qL][j] = sum_qNL Phi G_j,b(qNL)
// and the four products P_ab[i][j] = sum_qL w_qL G_i,a(qL) H_b[qL][j], from
// which the block follows; entries are added to the CSR rows with FP64
// atomics (binary search for the column).  FP64 throughout.
#include "common.cuh"
#include "influence.cuh"

#include <cmath>

namespace nlgpu {

namespace {

constexpr int EL_THREADS = 256;
constexpr int EL_WARPS = EL_THREADS / 32;

// ------------------------------------------------------------ boundaries
// displacement components: not inner, value (first non-zero wins:
// boundary_condition_first_kind_2d.hpp:16-26); per degree of freedom
__global__ void k_el_dirichlet(i64 count, const int32_t* __restrict__ nodes, int component, double value,
                               uint8_t* __restrict__ is_inner, double* __restrict__ x) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < count; t += i64(gridDim.x) * blockDim.x) {
        const i64 d = 2 * i64(nodes[t]) + component;
        is_inner[d] = 0;
        if (x[d] == 0.0) x[d] = value;
    }
}

// pressure component: int N_i p |J| over the boundary line elements
// (boundary_condition_second_kind_2d.hpp:12-33), into row 2 node + component
__global__ void k_el_pressure(i64 n_edges, int nen, const int32_t* __restrict__ edges, const double* __restrict__ nodes,
                              Basis1d b, int component, double p, double* __restrict__ f) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < n_edges * nen; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / nen;
        const int i = int(t % nen);
        double integral = 0.0;
        for (int q = 0; q < b.nq; ++q) {
            double J0 = 0.0, J1 = 0.0;
            for (int k = 0; k < nen; ++k) {
                const int32_t v = edges[e * nen + k];
                J0 += nodes[2 * i64(v)] * b.qNxi[k * b.nq + q];
                J1 += nodes[2 * i64(v) + 1] * b.qNxi[k * b.nq + q];
            }
            integral += b.w[q] * b.qN[i * b.nq + q] * p * sqrt(J0 * J0 + J1 * J1);
        }
        atomicAdd(f + 2 * i64(edges[t]) + component, integral);
    }
}

// ------------------------------------------------------------ patterns
__device__ __forceinline__ int warp_excl_scan(int v, int lane, int* total) {
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    *total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - v;
}

// Degree-of-freedom rows from the node adjacency (sorted node columns b of
// node a): row R = 2 a + r, candidate columns 2 b, 2 b + 1 in increasing order,
// classified by matrix_separator_base::part (matrix_separator_base.hpp:51-58):
// INNER if the column and the row are inner and R <= column; BOUND if the
// column is not inner and differs from R.  A row that is not inner holds its
// unit diagonal only (matrix_assembler_2d.hpp first_kind_filler).  The
// full-row solver pattern keeps both triangles of INNER, padded to a
// multiple of 4 entries with (R, 0).  Warp per row; count pass when the
// column outputs are null.
__global__ void k_dof_pattern(i64 rows, const i64* __restrict__ arp, const int32_t* __restrict__ acol,
                              const uint8_t* __restrict__ inner2, i64* __restrict__ cnt_in, i64* __restrict__ cnt_bd,
                              i64* __restrict__ cnt_full, const i64* __restrict__ rp_in, const i64* __restrict__ rp_bd,
                              const i64* __restrict__ rp_full, int32_t* __restrict__ c_in, int32_t* __restrict__ c_bd,
                              int32_t* __restrict__ c_full) {
    const int lane = threadIdx.x & 31;
    const bool fill = c_in != nullptr;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 R = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; R < rows; R += warps) {
        const i64 a = R >> 1;
        const bool row_inner = inner2[R];
        i64 ni = 0, nb = 0, nf = 0;
        if (!row_inner) {
            ni = 1; nf = 1;
            if (fill && lane == 0) { c_in[rp_in[R]] = int32_t(R); c_full[rp_full[R]] = int32_t(R); }
        }
        for (i64 k0 = arp[a]; k0 < arp[a + 1]; k0 += 32) {
            const i64 k = k0 + lane;
            const bool valid = k < arp[a + 1];
            const int32_t b = valid ? acol[k] : 0;
            bool fi[2] = {false, false}, fb[2] = {false, false}, ff[2] = {false, false};
            int ci = 0, cb = 0, cf = 0;
#pragma unroll
            for (int cl = 0; cl < 2; ++cl) {
                if (!valid) continue;
                const i64 col = 2 * i64(b) + cl;
                const bool cin = inner2[col];
                ff[cl] = cin && row_inner;
                fi[cl] = ff[cl] && R <= col;
                fb[cl] = !cin && col != R;
                ci += fi[cl]; cb += fb[cl]; cf += ff[cl];
            }
            int ti, tb, tf;
            const int oi = warp_excl_scan(ci, lane, &ti), ob = warp_excl_scan(cb, lane, &tb),
                      of = warp_excl_scan(cf, lane, &tf);
            if (fill && valid) {
                i64 pi = rp_in[R] + ni + oi, pb = rp_bd[R] + nb + ob, pf = rp_full[R] + nf + of;
#pragma unroll
                for (int cl = 0; cl < 2; ++cl) {
                    const int32_t col = 2 * b + cl;
                    if (fi[cl]) c_in[pi++] = col;
                    if (fb[cl]) c_bd[pb++] = col;
                    if (ff[cl]) c_full[pf++] = col;
                }
            }
            ni += ti; nb += tb; nf += tf;
        }
        if (!fill) {
            if (lane == 0) { cnt_in[R] = ni; cnt_bd[R] = nb; cnt_full[R] = (nf + 3) & ~i64(3); }
        } else {
            for (i64 k = rp_full[R] + nf + lane; k < rp_full[R + 1]; k += 32) c_full[k] = int32_t(R);
        }
    }
}

// ------------------------------------------------------------ values
struct ElasticArgs {
    i64 E;
    const int32_t* elems;
    const double* qcoord;     // [e][q][2]
    const double* jac;        // [e][q]
    const double* deriv;      // [e][i][q][2]  (grad N . adj J)
    const i64* noff;          // neighbours (null: local part, eNL = eL only)
    const int32_t* nlist;
    const uint8_t* inner2;
    const i64* in_rp; const int32_t* in_col; double* in_val;
    const i64* bd_rp; const int32_t* bd_col; double* bd_val;   // null: BOUND entries dropped
    double h[6];              // h11 h12 h66 h22 h16 h26
    double local_weight;      // p1 (the local part's weight)
    double cnl;               // norm (1 - p1) (0 for the local part)
    int* error;               // set when an entry is missing from its pattern
};

template<int NEN, int NQ>
struct ElasticSmem {
    double aLx[NEN * NQ], aLy[NEN * NQ];   // w_qL G_L
    double qLx[NQ], qLy[NQ];
    double gx[NEN * NQ], gy[NEN * NQ];     // G_NL
    double qx[NQ], qy[NQ];
    double phi[NQ * NQ];
    double hx[NQ * NEN], hy[NQ * NEN];
    int32_t nL[NEN], nNL[NEN];
};

__device__ __forceinline__ i64 el_find(const int32_t* col, i64 lo, i64 hi, int32_t c) {
    while (lo < hi) {
        const i64 mid = (lo + hi) >> 1;
        if (col[mid] < c) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void el_add(const i64* rp, const int32_t* col, double* val, i64 r, int32_t c, double v,
                                       int* error) {
    const i64 pos = el_find(col, rp[r], rp[r + 1], c);
    if (pos < rp[r + 1] && col[pos] == c) atomicAdd(val + pos, v);
    else atomicExch(error, 1);
}

// the Hooke combination of the four products P_ab = sum a_a b_b
__device__ __forceinline__ void hooke_block(const double* h, double pxx, double pxy, double pyx, double pyy,
                                            double (&blk)[2][2]) {
    blk[0][0] = h[0] * pxx + h[4] * (pxy + pyx) + h[2] * pyy;
    blk[0][1] = h[1] * pxy + h[4] * pxx + h[2] * pyx + h[5] * pyy;
    blk[1][0] = h[1] * pyx + h[4] * pxx + h[2] * pxy + h[5] * pyy;
    blk[1][1] = h[3] * pyy + h[5] * (pxy + pyx) + h[2] * pxx;
}

// Warp per element eL (grid-stride), looping over its ordered pairs (eL, eNL).
template<int NEN, int NQ, int INF>
__global__ void __launch_bounds__(EL_THREADS) k_elastic_pairs(ElasticArgs a, Model m, Basis b) {
    __shared__ ElasticSmem<NEN, NQ> smem[EL_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ElasticSmem<NEN, NQ>& s = smem[warp];
    const i64 warps = i64(gridDim.x) * EL_WARPS;
    for (i64 eL = blockIdx.x * i64(EL_WARPS) + warp; eL < a.E; eL += warps) {
        for (int t = lane; t < NEN * NQ; t += 32) {
            const double w = b.w[t % NQ];
            s.aLx[t] = w * a.deriv[2 * (eL * NEN * NQ + t)];
            s.aLy[t] = w * a.deriv[2 * (eL * NEN * NQ + t) + 1];
        }
        if (lane < NQ) {
            s.qLx[lane] = a.qcoord[2 * (eL * NQ + lane)];
            s.qLy[lane] = a.qcoord[2 * (eL * NQ + lane) + 1];
        }
        if (lane < NEN) s.nL[lane] = a.elems[eL * NEN + lane];
        __syncwarp();
        const i64 kb = a.noff ? a.noff[eL] : 0, ke = a.noff ? a.noff[eL + 1] : 1;
        for (i64 k = kb; k < ke; ++k) {
            const i64 eNL = a.noff ? i64(a.nlist[k]) : eL;
            const bool self = eNL == eL;
            for (int t = lane; t < NEN * NQ; t += 32) {
                s.gx[t] = a.deriv[2 * (eNL * NEN * NQ + t)];
                s.gy[t] = a.deriv[2 * (eNL * NEN * NQ + t) + 1];
            }
            if (lane < NQ) {
                s.qx[lane] = a.qcoord[2 * (eNL * NQ + lane)];
                s.qy[lane] = a.qcoord[2 * (eNL * NQ + lane) + 1];
            }
            if (lane < NEN) s.nNL[lane] = a.elems[eNL * NEN + lane];
            __syncwarp();
            const bool nonlocal = a.cnl != 0.0;
            if (nonlocal) {
                for (int t = lane; t < NQ * NQ; t += 32) {
                    const int qL = t / NQ, qNL = t % NQ;
                    s.phi[t] = b.w[qNL] * a.cnl * shape<INF>(m, s.qLx[qL] - s.qx[qNL], s.qLy[qL] - s.qy[qNL]);
                }
                __syncwarp();
                for (int t = lane; t < NQ * NEN; t += 32) {
                    const int qL = t / NEN, j = t % NEN;
                    double h0 = 0.0, h1 = 0.0;
#pragma unroll
                    for (int qNL = 0; qNL < NQ; ++qNL) {
                        const double f = s.phi[qL * NQ + qNL];
                        h0 += f * s.gx[j * NQ + qNL];
                        h1 += f * s.gy[j * NQ + qNL];
                    }
                    s.hx[t] = h0; s.hy[t] = h1;
                }
                __syncwarp();
            }
            for (int t = lane; t < NEN * NEN; t += 32) {
                const int i = t / NEN, j = t % NEN;
                double blk[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
                if (nonlocal) {
                    double pxx = 0.0, pxy = 0.0, pyx = 0.0, pyy = 0.0;
#pragma unroll
                    for (int qL = 0; qL < NQ; ++qL) {
                        const double ax = s.aLx[i * NQ + qL], ay = s.aLy[i * NQ + qL];
                        const double bx = s.hx[qL * NEN + j], by = s.hy[qL * NEN + j];
                        pxx += ax * bx; pxy += ax * by; pyx += ay * bx; pyy += ay * by;
                    }
                    hooke_block(a.h, pxx, pxy, pyx, pyy, blk);
                }
                if (self) {   // p1 x the local block, weights w_q / |J_q| (stiffness_matrix_2d.hpp:45-79)
                    double pxx = 0.0, pxy = 0.0, pyx = 0.0, pyy = 0.0;
#pragma unroll
                    for (int q = 0; q < NQ; ++q) {
                        const double inv = 1.0 / a.jac[eL * NQ + q];
                        const double ax = s.aLx[i * NQ + q] * inv, ay = s.aLy[i * NQ + q] * inv;
                        const double bx = s.gx[j * NQ + q], by = s.gy[j * NQ + q];
                        pxx += ax * bx; pxy += ax * by; pyx += ay * bx; pyy += ay * by;
                    }
                    double loc[2][2];
                    hooke_block(a.h, pxx, pxy, pyx, pyy, loc);
                    for (int r = 0; r < 2; ++r)
                        for (int c = 0; c < 2; ++c) blk[r][c] += a.local_weight * loc[r][c];
                }
                const i64 row0 = 2 * i64(s.nL[i]), col0 = 2 * i64(s.nNL[j]);
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    const i64 row = row0 + r;
                    const bool r_in = a.inner2[row];
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const i64 col = col0 + c;
                        const bool c_in = a.inner2[col];
                        if (c_in) {
                            if (r_in && row <= col)
                                el_add(a.in_rp, a.in_col, a.in_val, row, int32_t(col), blk[r][c], a.error);
                        } else if (row != col && a.bd_rp) {
                            el_add(a.bd_rp, a.bd_col, a.bd_val, row, int32_t(col), blk[r][c], a.error);
                        }
                    }
                }
            }
            __syncwarp();
        }
    }
}

// a row that is not inner holds 1 on its diagonal (its only inner entry)
__global__ void k_el_unit_rows(i64 rows, const uint8_t* __restrict__ inner2, const i64* __restrict__ rp,
                               double* __restrict__ val) {
    for (i64 r = blockIdx.x * i64(blockDim.x) + threadIdx.x; r < rows; r += i64(gridDim.x) * blockDim.x)
        if (!inner2[r]) val[rp[r]] = 1.0;
}

template<int NEN, int NQ>
void launch_pairs_inf(Ctx& ctx, const ElasticArgs& a, unsigned grid) {
    const Model& m = ctx.model;
    switch (m.influence) {
    case NLGPU_INFLUENCE_CONSTANT:
        NL_LAUNCH((k_elastic_pairs<NEN, NQ, NLGPU_INFLUENCE_CONSTANT>), grid, EL_THREADS, 0, ctx.stream, a, m, ctx.basis);
        break;
    case NLGPU_INFLUENCE_POLYNOMIAL:
        NL_LAUNCH((k_elastic_pairs<NEN, NQ, NLGPU_INFLUENCE_POLYNOMIAL>), grid, EL_THREADS, 0, ctx.stream, a, m, ctx.basis);
        break;
    case NLGPU_INFLUENCE_EXPONENTIAL:
        NL_LAUNCH((k_elastic_pairs<NEN, NQ, NLGPU_INFLUENCE_EXPONENTIAL>), grid, EL_THREADS, 0, ctx.stream, a, m, ctx.basis);
        break;
    default:
        NL_LAUNCH((k_elastic_pairs<NEN, NQ, NLGPU_INFLUENCE_FAST_POLYNOMIAL>), grid, EL_THREADS, 0, ctx.stream, a, m,
                  ctx.basis);
    }
}

// patterns of one part (FULL: nonlocal candidates when the model is nonlocal;
// LOCAL: the element's own nodes) over the degree-of-freedom rows
void dof_patterns(Ctx& ctx, bool local_only, Csr& inner, Csr* bound, Csr* full, dbuf<i64>* map) {
    Elastic& el = ctx.el;
    const i64 n = ctx.n_nodes, rows = 2 * n;
    // node adjacency: every candidate node column of each node row (all rows
    // inner, no triangle), sorted
    dbuf<uint8_t> ones;
    ones.resize(size_t(n));
    NL_CUDA(cudaMemsetAsync(ones.p, 1, size_t(n), ctx.stream));
    Csr adj;
    build_patterns(ctx, local_only, false, adj, nullptr, nullptr, nullptr, ones.p);
    dbuf<i64> ci, cb, cf;
    ci.resize(size_t(rows + 1)); cb.resize(size_t(rows + 1)); cf.resize(size_t(rows + 1));
    ci.zero(ctx.stream); cb.zero(ctx.stream); cf.zero(ctx.stream);
    const unsigned grid = grid_for(rows * 32, 256, 152 * 64);
    NL_LAUNCH(k_dof_pattern, grid, 256, 0, ctx.stream, rows, adj.rowptr.p, adj.col.p, el.is_inner.p, ci.p, cb.p, cf.p,
              static_cast<const i64*>(nullptr), static_cast<const i64*>(nullptr), static_cast<const i64*>(nullptr),
              static_cast<int32_t*>(nullptr), static_cast<int32_t*>(nullptr), static_cast<int32_t*>(nullptr));
    Csr tmp_b, tmp_f;
    Csr& B = bound ? *bound : tmp_b;
    Csr& F = full ? *full : tmp_f;
    for (Csr* m : {&inner, &B, &F}) { m->rows = rows; m->rowptr.resize(size_t(rows + 1)); m->col16_ok = false; }
    exclusive_scan(ctx, ci.p, inner.rowptr.p, rows + 1, &inner.nnz);
    exclusive_scan(ctx, cb.p, B.rowptr.p, rows + 1, &B.nnz);
    exclusive_scan(ctx, cf.p, F.rowptr.p, rows + 1, &F.nnz);
    inner.col.resize(size_t(inner.nnz)); B.col.resize(size_t(B.nnz)); F.col.resize(size_t(F.nnz));
    NL_LAUNCH(k_dof_pattern, grid, 256, 0, ctx.stream, rows, adj.rowptr.p, adj.col.p, el.is_inner.p, ci.p, cb.p, cf.p,
              inner.rowptr.p, B.rowptr.p, F.rowptr.p, inner.col.p, B.col.p, F.col.p);
    inner.val.resize(size_t(inner.nnz)); inner.val.zero(ctx.stream);
    B.val.resize(size_t(B.nnz)); B.val.zero(ctx.stream);
    if (full && map) {
        full_map(ctx, inner, F, *map, true);
        F.val.resize(size_t(F.nnz));
    }
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
}

void assemble_values(Ctx& ctx, bool local_part, Csr& inner, Csr* bound) {
    Elastic& el = ctx.el;
    const Model& m = ctx.model;
    const bool nonlocal = !local_part && m.nonlocal();
    dbuf<int> err;
    err.resize(1); err.zero(ctx.stream);
    ElasticArgs a{};
    a.E = ctx.n_elems; a.elems = ctx.elems.p; a.qcoord = ctx.qcoord.p; a.jac = ctx.jac.p; a.deriv = ctx.deriv.p;
    a.noff = nonlocal ? ctx.noff.p : nullptr; a.nlist = nonlocal ? ctx.nlist.p : nullptr;
    a.inner2 = el.is_inner.p;
    a.in_rp = inner.rowptr.p; a.in_col = inner.col.p; a.in_val = inner.val.p;
    a.bd_rp = bound ? bound->rowptr.p : nullptr; a.bd_col = bound ? bound->col.p : nullptr;
    a.bd_val = bound ? bound->val.p : nullptr;
    for (int k = 0; k < 6; ++k) a.h[k] = el.h[k];
    // the LOCAL part and a local model integrate p1 x the local block only
    // (local_theories; stiffness_matrix_2d.hpp:183-188)
    a.local_weight = m.p1;
    a.cnl = nonlocal ? m.norm * (1.0 - m.p1) : 0.0;
    a.error = err.p;
    const unsigned grid = grid_for(ctx.n_elems, EL_WARPS, 152 * 16);
    if (ctx.basis.nen == 4) launch_pairs_inf<4, 4>(ctx, a, grid);
    else if (ctx.basis.nen == 8) launch_pairs_inf<8, 9>(ctx, a, grid);
    else NL_REQUIRE(false, NLGPU_ERR_UNSUPPORTED, "elements of 4 or 8 nodes");
    NL_LAUNCH(k_el_unit_rows, grid_for(inner.rows, 256), 256, 0, ctx.stream, inner.rows, el.is_inner.p, inner.rowptr.p,
              inner.val.p);
    int herr = 0;
    NL_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof herr, cudaMemcpyDeviceToHost, ctx.stream));
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    NL_REQUIRE(herr == 0, NLGPU_ERR_STATE, "a stiffness entry is missing from its pattern");
}

}  // namespace

// is_inner per degree of freedom (solvers_utils.hpp inner_nodes), the
// displacement vector and the pressure integrals (the right-hand side before
// the first kind)
void elastic_boundaries(Ctx& ctx) {
    Elastic& el = ctx.el;
    const i64 rows = 2 * ctx.n_nodes;
    el.is_inner.resize(size_t(rows));
    NL_CUDA(cudaMemsetAsync(el.is_inner.p, 1, size_t(rows), ctx.stream));
    el.x_dirichlet.resize(size_t(rows)); el.x_dirichlet.zero(ctx.stream);
    el.rhs_init.resize(size_t(rows)); el.rhs_init.zero(ctx.stream);
    for (const MechanicalGroup& g : el.groups) {
        const i64 cnt = g.n_edges * g.nen;
        for (int d = 0; d < 2; ++d) {
            if (g.kind[d] == NLGPU_MECH_DISPLACEMENT)
                NL_LAUNCH(k_el_dirichlet, grid_for(cnt, 256), 256, 0, ctx.stream, cnt, g.edges.p, d, g.value[d],
                          el.is_inner.p, el.x_dirichlet.p);
            else if (g.kind[d] == NLGPU_MECH_PRESSURE)
                NL_LAUNCH(k_el_pressure, grid_for(cnt, 256), 256, 0, ctx.stream, g.n_edges, g.nen, g.edges.p,
                          ctx.nodes.p, make_basis_1d(g.nen), d, g.value[d], el.rhs_init.p);
        }
    }
}

// stiffness_matrix::compute (FULL into inner / bound and the solver's full
// rows, with the right-hand side; LOCAL into `local`, the ILLT's matrix)
void elastic_assemble(Ctx& ctx, bool local_part) {
    Elastic& el = ctx.el;
    NL_REQUIRE(ctx.mesh_ready && ctx.model_ready && el.hooke_set, NLGPU_ERR_STATE,
               "mesh, model and elastic parameters must be set before the stiffness assembly");
    elastic_boundaries(ctx);
    if (local_part) {
        dof_patterns(ctx, true, el.local, nullptr, nullptr, nullptr);
        assemble_values(ctx, true, el.local, nullptr);
        el.local_ready = true;
        return;
    }
    NL_REQUIRE(!ctx.model.nonlocal() || ctx.neighbours_ready, NLGPU_ERR_STATE,
               "neighbour search must run before a nonlocal assembly");
    dof_patterns(ctx, !ctx.model.nonlocal(), el.inner, &el.bound, &el.full, &el.full_from_upper);
    assemble_values(ctx, false, el.inner, &el.bound);
    fill_full_from_upper(ctx, el.inner, el.full, el.full_from_upper);
    // f = pressure integrals; f -= K_bound x_D, f[D] = x_D (equilibrium_equation_2d.hpp:28-33)
    el.rhs.resize(size_t(2 * ctx.n_nodes));
    apply_first_kind(ctx, el.bound, el.rhs_init.p, el.rhs.p, el.x_dirichlet.p, el.is_inner.p);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));
    el.assembled = true;
    el.local_ready = false;
}

// equilibrium_equation_2d.hpp:34-56: CG on the stiffness system with ILLT of the
// LOCAL stiffness for a nonlocal model (identity when the factorisation fails
// or for a local model, as the reference's default preconditioner)
CgResult elastic_solve(Ctx& ctx, const nlgpu_solve_options& o, nlgpu_solve_report* rep) {
    Elastic& el = ctx.el;
    NL_REQUIRE(el.assembled, NLGPU_ERR_STATE, "assemble the stiffness matrix first");
    NL_REQUIRE(o.precision == NLGPU_PRECISION_FP64 || o.precision == NLGPU_PRECISION_MIXED, NLGPU_ERR_ARG,
               "unknown precision");
    NL_REQUIRE(o.preconditioner == NLGPU_PRECONDITIONER_IDENTITY || o.preconditioner == NLGPU_PRECONDITIONER_ILLT,
               NLGPU_ERR_ARG, "the stiffness solve takes the identity or the ILLT preconditioner");
    const auto t0 = std::chrono::steady_clock::now();
    const IncompleteCholesky* M = nullptr;
    const bool mixed = o.precision == NLGPU_PRECISION_MIXED;
    const int sweeps = o.triangular_sweeps == 0 ? NLGPU_DEFAULT_TRIANGULAR_SWEEPS : std::max(o.triangular_sweeps, 0);
    if (o.preconditioner == NLGPU_PRECONDITIONER_ILLT) {
        if (!el.local_ready) elastic_assemble(ctx, true);
        ilt_build(ctx, el.local, el.ilt, !(mixed && sweeps > 0), mixed && sweeps > 0);
        if (el.ilt.ok) M = &el.ilt;
    } else {
        el.ilt.ok = false;
    }
    const i64 rows = 2 * ctx.n_nodes;
    el.displacement.resize(size_t(rows));
    CgResult r;
    if (mixed) {
        matrix_to_f32(ctx, el.full);
        r = mixed_solve(ctx, el.full, M ? &el.ilt : nullptr, el.rhs.p, el.displacement.p, o.tolerance,
                        o.max_iterations, o.inner_tolerance > 0.0 ? o.inner_tolerance : MIXED_UPDATE_FACTOR, false, false, sweeps);
    } else {
        r = cg_solve(ctx, el.full, M, el.rhs.p, el.displacement.p, o.tolerance, o.max_iterations, false);
    }
    if (M && ctx.sweep_error.n) {
        int err = 0;
        NL_CUDA(cudaMemcpyAsync(&err, ctx.sweep_error.p, sizeof err, cudaMemcpyDeviceToHost, ctx.stream));
        NL_CUDA(cudaStreamSynchronize(ctx.stream));
        NL_REQUIRE(err == 0, NLGPU_ERR_TIMEOUT, "a triangular sweep stage wait gave up");
    }
    if (rep) {
        rep->iterations = r.iterations;
        rep->residual = r.residual;
        rep->reference_residual = r.reference_residual;
        rep->preconditioner_ok = el.ilt.ok ? 1 : 0;
        rep->preconditioner_shifts = el.ilt.attempts;
        rep->nnz_inner = el.inner.nnz;
        rep->nnz_solver = el.full.nnz;
        rep->element_pairs = ctx.model.nonlocal() ? ctx.pairs : ctx.n_elems;
        rep->outer_iterations = r.outer_iterations;
        rep->seconds_solve = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        rep->nnz_fp32 = mixed ? el.full.nnz : 0;
    }
    return r;
}

}  // namespace nlgpu
