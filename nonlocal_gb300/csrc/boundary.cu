// Boundary conditions and the right-hand side of the stationary problem:
//   * is_inner: nodes of temperature groups are Dirichlet (solvers_utils.hpp:31-40);
//   * Dirichlet values, first non-zero value wins (boundary_condition_first_kind_2d.hpp:16-26);
//   * flux integrals over boundary line elements (boundary_condition_second_kind_2d.hpp:12-33);
//   * volume source integrals (right_part_2d.hpp:10-35);
//   * f -= K_bound x_D, f[D] = x_D (boundary_condition_first_kind_2d.hpp:50-59).
#include "common.cuh"

namespace nlgpu {

namespace {

__global__ void k_mark_dirichlet(i64 count, const int32_t* __restrict__ nodes, uint8_t* __restrict__ is_inner) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < count; t += i64(gridDim.x) * blockDim.x)
        is_inner[nodes[t]] = 0;
}

__global__ void k_dirichlet_values(i64 count, const int32_t* __restrict__ nodes, double value,
                                   const double* __restrict__ node_values, double* __restrict__ x) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < count; t += i64(gridDim.x) * blockDim.x) {
        const int32_t v = nodes[t];
        if (x[v] == 0.0) x[v] = node_values ? node_values[t] : value;
    }
}

__global__ void k_dirichlet_override(i64 n, const uint8_t* __restrict__ is_inner, const double* __restrict__ values,
                                     double* __restrict__ x) {
    for (i64 v = blockIdx.x * i64(blockDim.x) + threadIdx.x; v < n; v += i64(gridDim.x) * blockDim.x)
        if (!is_inner[v]) x[v] = values[v];
}

// flux integral of one boundary line element per thread and local node
__global__ void k_flux(i64 n_edges, int nen, const int32_t* __restrict__ edges, const double* __restrict__ nodes,
                       Basis1d b, double flux, double* __restrict__ f) {
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
            integral += b.w[q] * b.qN[i * b.nq + q] * flux * sqrt(J0 * J0 + J1 * J1);
        }
        atomicAdd(f + edges[t], integral);
    }
}

// source integral: one thread per (element, local node)
__global__ void k_source(i64 E, int nen, int nq, const int32_t* __restrict__ elems, const double* __restrict__ jac,
                         Basis b, double value, const double* __restrict__ per_q, double* __restrict__ f) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < E * nen; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / nen;
        const int i = int(t % nen);
        double integral = 0.0;
        for (int q = 0; q < nq; ++q)
            integral += b.w[q] * b.qN[i * nq + q] * jac[e * nq + q] * (per_q ? per_q[e * nq + q] : value);
        atomicAdd(f + elems[t], integral);
    }
}

// out = in - bound * x_D on every row, then out[D] = x_D.  Warp per row.
__global__ void k_first_kind(i64 n, const i64* __restrict__ rowptr, const int32_t* __restrict__ col,
                             const double* __restrict__ val, const double* __restrict__ in,
                             const double* __restrict__ xd, const uint8_t* __restrict__ is_inner,
                             double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        double s = 0.0;
        for (i64 k = rowptr[r] + lane; k < rowptr[r + 1]; k += 32) s += val[k] * xd[col[k]];
        s = warp_sum(s);
        if (lane == 0) out[r] = is_inner[r] ? in[r] - s : xd[r];
    }
}

}  // namespace

void boundary_vectors(Ctx& ctx) {
    const i64 n = ctx.n_nodes;
    ctx.is_inner.resize(size_t(n));
    NL_CUDA(cudaMemsetAsync(ctx.is_inner.p, 1, size_t(n), ctx.stream));
    ctx.x_dirichlet.resize(size_t(n)); ctx.x_dirichlet.zero(ctx.stream);
    ctx.rhs_init.resize(size_t(n)); ctx.rhs_init.zero(ctx.stream);
    for (const BoundaryGroup& g : ctx.groups) {
        const i64 cnt = g.n_edges * g.nen;
        if (g.kind == NLGPU_BC_TEMPERATURE) {
            NL_LAUNCH(k_mark_dirichlet, grid_for(cnt, 256), 256, 0, ctx.stream, cnt, g.edges.p, ctx.is_inner.p);
            NL_LAUNCH(k_dirichlet_values, grid_for(cnt, 256), 256, 0, ctx.stream, cnt, g.edges.p, g.value,
                      g.node_values.n ? g.node_values.p : nullptr, ctx.x_dirichlet.p);
        } else {
            NL_LAUNCH(k_flux, grid_for(cnt, 256), 256, 0, ctx.stream, g.n_edges, g.nen, g.edges.p, ctx.nodes.p,
                      make_basis_1d(g.nen), g.value, ctx.rhs_init.p);
        }
    }
    if (ctx.source != 0.0 || ctx.source_q.n)
        NL_LAUNCH(k_source, grid_for(ctx.n_elems * ctx.basis.nen, 256), 256, 0, ctx.stream, ctx.n_elems, ctx.basis.nen,
                  ctx.basis.nq, ctx.elems.p, ctx.jac.p, ctx.basis, ctx.source, ctx.source_q.n ? ctx.source_q.p : nullptr,
                  ctx.rhs_init.p);
    if (ctx.dirichlet_override.n)
        NL_LAUNCH(k_dirichlet_override, grid_for(n, 256), 256, 0, ctx.stream, n, ctx.is_inner.p,
                  ctx.dirichlet_override.p, ctx.x_dirichlet.p);
    ctx.bc_ready = true;
}

void apply_first_kind(Ctx& ctx, const Csr& bound, const double* rhs_in, double* rhs_out, const double* x_dirichlet,
                      const uint8_t* is_inner) {
    NL_LAUNCH(k_first_kind, grid_for(bound.rows * 32, 256, 152 * 64), 256, 0, ctx.stream, bound.rows, bound.rowptr.p,
              bound.col.p, bound.val.p, rhs_in, x_dirichlet, is_inner ? is_inner : ctx.is_inner.p, rhs_out);
}

}  // namespace nlgpu
