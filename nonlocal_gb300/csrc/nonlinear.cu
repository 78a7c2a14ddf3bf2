// Convection, radiation and the integral condition of pure Neumann problems.
//
//   * convection (convection_condition_2d.hpp:11-31): alpha int_edge N_i N_j |J|
//     added to the entries (row, col >= row) of the assembled matrix for every
//     pair of nodes of a convection edge;
//   * radiation: with the previous temperature T_q = sum_k N_k(q) T_k on the
//     edge, stationary (radiation_condition_2d.hpp:59-104)
//     K(row, col >= row) -= 4 sigma eps int T_q^3 N_i N_j |J| and
//     r_rad[row] -= sigma eps int T_q^4 N_i |J|; nonstationary
//     (radiation_condition_2d.hpp:43-88) K += dt 4 sigma eps int T_q^3 N_i N_j |J|
//     (kept from step to step) and f[row] += 3 sigma eps int T_q^4 N_i |J|;
//   * pure Neumann problems (conductivity_matrix_2d.hpp:83-104): the Lagrange
//     column int N_i over the node's elements.
// Rows of temperature nodes are skipped: the reference resets them
// afterwards (first_kind_matrix_fill_2d), and edges that would couple a
// temperature node to another node are rejected before any of this runs.
// Edges hold 2 or 3 nodes; one thread per (edge, i) or (edge, i, j).
#include "common.cuh"

#include <array>

namespace nlgpu {

namespace {

constexpr double STEFAN_BOLTZMANN = 5.67036713e-8;   // metamath::constants (utils/constants.hpp:12)

__device__ double edge_jacobian(const int32_t* e, int nen, const double* nodes, const Basis1d& b, int q) {
    double J0 = 0.0, J1 = 0.0;
    for (int k = 0; k < nen; ++k) {
        J0 += nodes[2 * i64(e[k])] * b.qNxi[k * b.nq + q];
        J1 += nodes[2 * i64(e[k]) + 1] * b.qNxi[k * b.nq + q];
    }
    return sqrt(J0 * J0 + J1 * J1);
}

// entry (row, col) with col >= row of every node pair of every edge, found in
// the sorted rows of the assembled (upper or full-storage) inner matrix; -1 for
// a temperature row or a pair below the diagonal.  Counts edges touching a
// temperature node.
__global__ void k_edge_index(i64 n_edges, int nen, const int32_t* __restrict__ edges,
                             const uint8_t* __restrict__ is_inner, const i64* __restrict__ rp,
                             const int32_t* __restrict__ col, i64* __restrict__ index, int* touching) {
    const i64 per = i64(nen) * nen;
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < n_edges * per; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / per;
        const int i = int(t % per) / nen, j = int(t % per) % nen;
        const int32_t row = edges[e * nen + i], c = edges[e * nen + j];
        if (i == 0 && j == 0) {
            bool any = false;
            for (int k = 0; k < nen; ++k) any |= !is_inner[edges[e * nen + k]];
            if (any) atomicAdd(touching, 1);
        }
        i64 found = -1;
        if (c >= row && is_inner[row] && is_inner[c]) {
            i64 lo = rp[row], hi = rp[row + 1];
            while (lo < hi) { const i64 mid = (lo + hi) >> 1; if (col[mid] < c) lo = mid + 1; else hi = mid; }
            if (lo < rp[row + 1] && col[lo] == c) found = lo;
        }
        index[t] = found;
    }
}

__global__ void k_convection(i64 n_edges, int nen, const int32_t* __restrict__ edges, const double* __restrict__ nodes,
                             Basis1d b, double heat_transfer, const i64* __restrict__ index, double* __restrict__ val) {
    const i64 per = i64(nen) * nen;
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < n_edges * per; t += i64(gridDim.x) * blockDim.x) {
        if (index[t] < 0) continue;
        const i64 e = t / per;
        const int i = int(t % per) / nen, j = int(t % per) % nen;
        double integral = 0.0;
        for (int q = 0; q < b.nq; ++q)
            integral += b.w[q] * b.qN[i * b.nq + q] * b.qN[j * b.nq + q] * edge_jacobian(edges + e * nen, nen, nodes, b, q);
        atomicAdd(val + index[t], heat_transfer * integral);
    }
}

__device__ double edge_temperature(const int32_t* e, int nen, const Basis1d& b, int q, const double* T) {
    double s = 0.0;
    for (int k = 0; k < nen; ++k) s += b.qN[k * b.nq + q] * T[e[k]];
    return s;
}

// val[entry] += coef int T_q^3 N_i N_j |J|
__global__ void k_radiation_matrix(i64 n_edges, int nen, const int32_t* __restrict__ edges,
                                   const double* __restrict__ nodes, Basis1d b, double coef,
                                   const double* __restrict__ T, const i64* __restrict__ index,
                                   double* __restrict__ val) {
    const i64 per = i64(nen) * nen;
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < n_edges * per; t += i64(gridDim.x) * blockDim.x) {
        if (index[t] < 0) continue;
        const i64 e = t / per;
        const int i = int(t % per) / nen, j = int(t % per) % nen;
        const int32_t* ed = edges + e * nen;
        double integral = 0.0;
        for (int q = 0; q < b.nq; ++q) {
            const double tq = edge_temperature(ed, nen, b, q, T);
            integral += b.w[q] * (tq * tq * tq) * b.qN[i * b.nq + q] * b.qN[j * b.nq + q] *
                        edge_jacobian(ed, nen, nodes, b, q);
        }
        atomicAdd(val + index[t], coef * integral);
    }
}

// rad[row] += coef int T_q^4 N_i |J| on the rows of non-temperature nodes
__global__ void k_radiation_vector(i64 n_edges, int nen, const int32_t* __restrict__ edges,
                                   const double* __restrict__ nodes, Basis1d b, double coef,
                                   const double* __restrict__ T, const uint8_t* __restrict__ is_inner,
                                   double* __restrict__ rad) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < n_edges * nen; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / nen;
        const int i = int(t % nen);
        const int32_t* ed = edges + e * nen;
        if (!is_inner[ed[i]]) continue;
        double integral = 0.0;
        for (int q = 0; q < b.nq; ++q) {
            const double tq = edge_temperature(ed, nen, b, q, T);
            const double t2 = tq * tq;
            integral += b.w[q] * b.qN[i * b.nq + q] * (t2 * t2) * edge_jacobian(ed, nen, nodes, b, q);
        }
        atomicAdd(rad + ed[i], coef * integral);
    }
}

// int N_i |J| over the elements of each node, in element order
// (conductivity_matrix_2d.hpp:75-104, integrate_basic)
__global__ void k_node_integral(i64 n, int nq, const i64* __restrict__ ne_off, const int32_t* __restrict__ ne_elem,
                                const int8_t* __restrict__ ne_local, const double* __restrict__ jac, Basis b,
                                double* __restrict__ out) {
    for (i64 v = blockIdx.x * i64(blockDim.x) + threadIdx.x; v < n; v += i64(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (i64 k = ne_off[v]; k < ne_off[v + 1]; ++k) {
            const i64 e = ne_elem[k];
            const int i = ne_local[k];
            double integral = 0.0;
            for (int q = 0; q < nq; ++q) integral += b.w[q] * b.qN[i * nq + q] * jac[e * nq + q];
            s += integral;
        }
        out[v] = s;
    }
}

// y = a - b - c (the radiation step's residual K T_prev - r_rad - f)
__global__ void k_sub3(i64 n, const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                       double* __restrict__ y) {
    for (i64 v = blockIdx.x * i64(blockDim.x) + threadIdx.x; v < n; v += i64(gridDim.x) * blockDim.x)
        y[v] = a[v] - b[v] - c[v];
}

// T = T_prev - dT in place of dT; block partials of |r|^2, |T - T_prev|^2, |T|^2
constexpr int NORM_BLOCKS = 152;
__global__ void k_step_norms(i64 n, const double* __restrict__ residual, const double* __restrict__ prev,
                             double* __restrict__ x, double* __restrict__ partial) {
    double s[3] = {0.0, 0.0, 0.0};
    for (i64 v = blockIdx.x * i64(blockDim.x) + threadIdx.x; v < n; v += i64(gridDim.x) * blockDim.x) {
        const double t = prev[v] - x[v];
        x[v] = t;
        s[0] += residual[v] * residual[v];
        s[1] += (t - prev[v]) * (t - prev[v]);
        s[2] += t * t;
    }
    __shared__ double sh[3][32];
    for (int k = 0; k < 3; ++k) {
        double w = warp_sum(s[k]);
        if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = w;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double w = 0.0;
        for (int k = 0; k < int(blockDim.x >> 5); ++k) w += sh[threadIdx.x][k];
        partial[threadIdx.x * NORM_BLOCKS + blockIdx.x] = w;
    }
}

__global__ void k_add_scaled(i64 n, double a, const double* __restrict__ x, double* __restrict__ y) {
    for (i64 v = blockIdx.x * i64(blockDim.x) + threadIdx.x; v < n; v += i64(gridDim.x) * blockDim.x) y[v] += a * x[v];
}

__global__ void k_add_constant(i64 n, double a, double* __restrict__ y) {
    for (i64 v = blockIdx.x * i64(blockDim.x) + threadIdx.x; v < n; v += i64(gridDim.x) * blockDim.x) y[v] += a;
}

}  // namespace

bool has_convection(const Ctx& c) {
    for (const BoundaryGroup& g : c.groups) if (g.convection()) return true;
    return false;
}

bool has_radiation(const Ctx& c) {
    for (const BoundaryGroup& g : c.groups) if (g.radiation()) return true;
    return false;
}

bool pure_neumann(const Ctx& c) {   // init_problem_settings.hpp:18-21,43
    for (const BoundaryGroup& g : c.groups) if (g.kind != NLGPU_BC_FLUX) return false;
    return true;
}

void boundary_matrix_index(Ctx& c) {
    dbuf<int> touching;
    touching.resize(1);
    touching.zero(c.stream);
    for (BoundaryGroup& g : c.groups) {
        if (!g.convection() && !g.radiation()) continue;
        const i64 cnt = g.n_edges * g.nen * g.nen;
        g.upper_index.resize(size_t(std::max<i64>(cnt, 1)));
        if (cnt)
            NL_LAUNCH(k_edge_index, grid_for(cnt, 256), 256, 0, c.stream, g.n_edges, g.nen, g.edges.p, c.is_inner.p,
                      c.inner.rowptr.p, c.inner.col.p, g.upper_index.p, touching.p);
    }
    int t = 0;
    touching.download(&t, 1, c.stream);
    NL_CUDA(cudaStreamSynchronize(c.stream));
    NL_REQUIRE(t == 0, NLGPU_ERR_UNSUPPORTED,
               "a convection or radiation edge shares a node with a temperature boundary");
}

void add_convection(Ctx& c) {
    for (const BoundaryGroup& g : c.groups) {
        if (!g.convection() || g.n_edges == 0) continue;
        const i64 cnt = g.n_edges * g.nen * g.nen;
        NL_LAUNCH(k_convection, grid_for(cnt, 256), 256, 0, c.stream, g.n_edges, g.nen, g.edges.p, c.nodes.p,
                  make_basis_1d(g.nen), g.heat_transfer, g.upper_index.p, c.inner.val.p);
    }
}

void add_radiation(Ctx& c, const double* T, double* rad, double matrix_factor, double vector_factor) {
    for (const BoundaryGroup& g : c.groups) {
        if (!g.radiation() || g.n_edges == 0) continue;
        const Basis1d b = make_basis_1d(g.nen);
        const i64 cnt = g.n_edges * g.nen * g.nen;
        const double se = STEFAN_BOLTZMANN * g.emissivity;
        NL_LAUNCH(k_radiation_matrix, grid_for(cnt, 256), 256, 0, c.stream, g.n_edges, g.nen, g.edges.p, c.nodes.p, b,
                  matrix_factor * se, T, g.upper_index.p, c.inner.val.p);
        NL_LAUNCH(k_radiation_vector, grid_for(g.n_edges * g.nen, 256), 256, 0, c.stream, g.n_edges, g.nen, g.edges.p,
                  c.nodes.p, b, vector_factor * se, T, c.is_inner.p, rad);
    }
}

void neumann_integrals(Ctx& c) {
    c.node_integral.resize(size_t(c.n_nodes));
    NL_LAUNCH(k_node_integral, grid_for(c.n_nodes, 256), 256, 0, c.stream, c.n_nodes, c.basis.nq, c.ne_off.p,
              c.ne_elem.p, c.ne_local.p, c.jac.p, c.basis, c.node_integral.p);
}

void subtract3(Ctx& c, const double* a, const double* b, const double* d, double* y) {
    NL_LAUNCH(k_sub3, grid_for(c.n_nodes, 256), 256, 0, c.stream, c.n_nodes, a, b, d, y);
}

std::array<double, 3> step_norms(Ctx& c, const double* residual, const double* prev, double* x) {
    dbuf<double> partial;
    partial.resize(3 * NORM_BLOCKS);
    NL_LAUNCH(k_step_norms, NORM_BLOCKS, 256, 0, c.stream, c.n_nodes, residual, prev, x, partial.p);
    std::vector<double> h(3 * NORM_BLOCKS);
    partial.download(h.data(), h.size(), c.stream);
    NL_CUDA(cudaStreamSynchronize(c.stream));
    std::array<double, 3> s{0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k)
        for (int b = 0; b < NORM_BLOCKS; ++b) s[size_t(k)] += h[size_t(k * NORM_BLOCKS + b)];
    return s;
}

void add_scaled(Ctx& c, double a, const double* x, double* y) {
    NL_LAUNCH(k_add_scaled, grid_for(c.n_nodes, 256), 256, 0, c.stream, c.n_nodes, a, x, y);
}

void add_constant(Ctx& c, double a, double* y) {
    NL_LAUNCH(k_add_constant, grid_for(c.n_nodes, 256), 256, 0, c.stream, c.n_nodes, a, y);
}

}  // namespace nlgpu
