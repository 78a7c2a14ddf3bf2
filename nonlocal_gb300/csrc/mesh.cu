// Element tables and the per-quadrature-point mesh data of mesh_2d::init
// (libraries/mesh/mesh_2d/mesh_2d.hpp:97-108).  Built with --fmad=false so the
// coordinates, Jacobians and element centres round exactly as the reference's
// host code does; the neighbour search compares distances computed from them.
#include "common.cuh"

#include <cmath>
#include <limits>

namespace nlgpu {

namespace {

// Gauss rules (libraries/metamath/finite_elements/finite_elements_1d/quadrature/gaussian_quadrature.hpp:22-40)
void gauss_rule(int n, double* x, double* w) {
    if (n == 1) { x[0] = 0.0; w[0] = 2.0; return; }
    if (n == 2) { x[0] = -1.0 / std::sqrt(3.0); x[1] = 1.0 / std::sqrt(3.0); w[0] = w[1] = 1.0; return; }
    x[0] = -std::sqrt(3.0 / 5.0); x[1] = 0.0; x[2] = std::sqrt(3.0 / 5.0);
    w[0] = 5.0 / 9.0; w[1] = 8.0 / 9.0; w[2] = 5.0 / 9.0;
}

// Shape function i and its derivatives at (x, y).
// Bilinear: serendipity<T,1> (serendipity_2d.hpp:144-175).
// 8-node: serendipity<T,2> with parameter p = 2/9 (serendipity_2d.hpp:177-222),
//   N_corner = (1 +- x)(1 +- y) (a(1 +- x +- y) +- b x y) / 16,
//   N_mid    = -(1 - x^2)(1 +- y)(c +- b y) / 16 (and the x <-> y counterparts),
//   a = 9p - 1, b = 9p + 3, c = 9p - 5; derivatives by the product rule.
void shape(int type, int i, double x, double y, double& N, double& Nx, double& Ny) {
    if (type == NLGPU_BILINEAR) {
        const double sx = (i == 1 || i == 2) ? 1.0 : -1.0, sy = (i >= 2) ? 1.0 : -1.0;
        N = (1 + sx * x) * (1 + sy * y) / 4;
        Nx = sx * (1 + sy * y) / 4;
        Ny = sy * (1 + sx * x) / 4;
        return;
    }
    const double p = 2.0 / 9.0, a = 9 * p - 1, b = 9 * p + 3, c = 9 * p - 5;
    if (i % 2 == 0) {   // corners 0, 2, 4, 6 at (sx, sy)
        const double sx = (i == 2 || i == 4) ? 1.0 : -1.0, sy = (i >= 4) ? 1.0 : -1.0;
        const double fx = 1 + sx * x, fy = 1 + sy * y;
        // inner factor g = a (1 - sx x - sy y) + sx sy b x y, written per corner as the reference does
        const double g = a * (1 - sx * x - sy * y) + sx * sy * b * x * y;
        N = fx * fy * g / 16;
        Nx = (sx * fy * g + fx * fy * (-sx * a + sx * sy * b * y)) / 16;
        Ny = (sy * fx * g + fx * fy * (-sy * a + sx * sy * b * x)) / 16;
        return;
    }
    if (i == 1 || i == 5) {   // mid-sides (0, -1) and (0, 1): -(1 - x^2)(1 + sy y)(c - sy b y) / 16
        const double sy = i == 5 ? 1.0 : -1.0;
        const double h = c - sy * b * y, dh = -sy * b;
        N = -(1 - x * x) * (1 + sy * y) * h / 16;
        Nx = 2 * x * (1 + sy * y) * h / 16;
        Ny = -(1 - x * x) * (sy * h + (1 + sy * y) * dh) / 16;
        return;
    }
    // mid-sides (1, 0) and (-1, 0): -(1 - y^2)(1 + sx x)(c - sx b x) / 16
    const double sx = i == 3 ? 1.0 : -1.0;
    const double h = c - sx * b * x, dh = -sx * b;
    N = -(1 - y * y) * (1 + sx * x) * h / 16;
    Nx = -(1 - y * y) * (sx * h + (1 + sx * x) * dh) / 16;
    Ny = 2 * y * (1 + sx * x) * h / 16;
}

__global__ void k_quadrature(i64 E, int nen, int nq, const double* __restrict__ nodes,
                             const int32_t* __restrict__ elems, Basis b, double* __restrict__ qcoord,
                             double* __restrict__ jac, double* __restrict__ deriv, double* __restrict__ centres) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < E * (nq + 1); t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / (nq + 1);
        const int q = int(t % (nq + 1));
        const int32_t* en = elems + e * nen;
        if (q == nq) {   // element centre, sum_i x_i N_i(0,0) (mesh_container_2d.hpp:131-139)
            double cx = 0.0, cy = 0.0;
            for (int i = 0; i < nen; ++i) {
                cx += nodes[2 * i64(en[i])] * b.centre[i];
                cy += nodes[2 * i64(en[i]) + 1] * b.centre[i];
            }
            centres[2 * e] = cx; centres[2 * e + 1] = cy;
            continue;
        }
        // quad_coord and jacobi_matrix (mesh_container_2d.hpp:141-160)
        double cx = 0.0, cy = 0.0, J00 = 0.0, J01 = 0.0, J10 = 0.0, J11 = 0.0;
        for (int i = 0; i < nen; ++i) {
            const double x = nodes[2 * i64(en[i])], y = nodes[2 * i64(en[i]) + 1];
            const double n = b.qN[i * nq + q], dxi = b.qNxi[i * nq + q], deta = b.qNeta[i * nq + q];
            cx += x * n; cy += y * n;
            J00 += x * dxi; J01 += x * deta; J10 += y * dxi; J11 += y * deta;
        }
        qcoord[2 * (e * nq + q)] = cx; qcoord[2 * (e * nq + q) + 1] = cy;
        jac[e * nq + q] = fabs(J00 * J11 - J01 * J10);   // mesh_container_2d_utils.hpp:88-91
        for (int i = 0; i < nen; ++i) {   // derivatives_in_quad (mesh_container_2d_utils.hpp:101-123)
            const double dxi = b.qNxi[i * nq + q], deta = b.qNeta[i * nq + q];
            double* d = deriv + 2 * ((e * nen + i) * nq + q);
            d[0] = dxi * J11 - deta * J10;
            d[1] = -dxi * J01 + deta * J00;
        }
    }
}

// smallest node number of each element: orders element pairs for the
// symmetric assembly (assemble.cu)
// smallest and largest node number of every element
__global__ void k_elem_minnode(i64 E, int nen, const int32_t* __restrict__ elems, int32_t* __restrict__ out,
                               int32_t* __restrict__ out_max) {
    for (i64 e = blockIdx.x * i64(blockDim.x) + threadIdx.x; e < E; e += i64(gridDim.x) * blockDim.x) {
        int32_t m = elems[e * nen], x = m;
        for (int i = 1; i < nen; ++i) { m = min(m, elems[e * nen + i]); x = max(x, elems[e * nen + i]); }
        out[e] = m;
        out_max[e] = x;
    }
}

__global__ void k_count_node_elements(i64 E, int nen, const int32_t* __restrict__ elems, i64* __restrict__ count) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < E * nen; t += i64(gridDim.x) * blockDim.x)
        atomicAdd(reinterpret_cast<unsigned long long*>(count + elems[t]), 1ull);
}

__global__ void k_fill_node_elements(i64 E, int nen, const int32_t* __restrict__ elems, const i64* __restrict__ off,
                                     i64* __restrict__ cursor, int32_t* __restrict__ ne_elem) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < E * nen; t += i64(gridDim.x) * blockDim.x) {
        const int32_t node = elems[t];
        const i64 slot = atomicAdd(reinterpret_cast<unsigned long long*>(cursor + node), 1ull);
        ne_elem[off[node] + slot] = int32_t(t / nen);
    }
}

// Orders each node's element list by element number (node_elements_2d,
// mesh_container_2d_utils.hpp:18-26) and records the node's local index.
__global__ void k_sort_node_elements(i64 n, int nen, const int32_t* __restrict__ elems, const i64* __restrict__ off,
                                     int32_t* __restrict__ ne_elem, int8_t* __restrict__ ne_local) {
    for (i64 v = blockIdx.x * i64(blockDim.x) + threadIdx.x; v < n; v += i64(gridDim.x) * blockDim.x) {
        const i64 b = off[v], e = off[v + 1];
        for (i64 i = b + 1; i < e; ++i) {   // insertion sort, lists are short
            const int32_t key = ne_elem[i];
            i64 j = i - 1;
            while (j >= b && ne_elem[j] > key) { ne_elem[j + 1] = ne_elem[j]; --j; }
            ne_elem[j + 1] = key;
        }
        for (i64 i = b; i < e; ++i) {
            const int32_t* en = elems + i64(ne_elem[i]) * nen;
            int8_t loc = 0;
            while (loc < nen && en[loc] != int32_t(v)) ++loc;
            ne_local[i] = loc;
        }
    }
}

}  // namespace

Basis make_basis(int element_type) {
    NL_REQUIRE(element_type == NLGPU_BILINEAR || element_type == NLGPU_QUADRATIC_SERENDIPITY, NLGPU_ERR_UNSUPPORTED,
               "only bilinear (2) and 8-node serendipity (3) elements are supported");
    Basis b{};
    b.type = element_type;
    b.nen = element_type == NLGPU_BILINEAR ? 4 : 8;
    const int n1 = element_type == NLGPU_BILINEAR ? 2 : 3;   // vtk_elements_set.hpp:54-72
    b.nq = n1 * n1;
    double g[3], gw[3];
    gauss_rule(n1, g, gw);
    // set_quadrature on the rectangle [-1,1]^2: mapped nodes and weights
    const double jx = (1.0 - (-1.0)) / (1.0 - (-1.0));
    double x[3], y[3];
    for (int i = 0; i < n1; ++i) {
        x[i] = -1.0 + (g[i] - (-1.0)) * jx;
        const double jy = (1.0 - (-1.0)) / (1.0 - (-1.0));
        for (int j = 0; j < n1; ++j) {
            y[j] = -1.0 + (g[j] - (-1.0)) * jy;
            b.w[i * n1 + j] = gw[i] * jx * gw[j] * jy;
        }
    }
    for (int i = 0; i < b.nen; ++i)
        for (int a = 0; a < n1; ++a)
            for (int c = 0; c < n1; ++c) {
                const int k = i * b.nq + a * n1 + c;
                shape(element_type, i, x[a], y[c], b.qN[k], b.qNxi[k], b.qNeta[k]);
            }
    for (int i = 0; i < b.nen; ++i) { double dx, dy; shape(element_type, i, 0.0, 0.0, b.centre[i], dx, dy); }
    // local node coordinates on [-1,1]^2: corners counterclockwise from (-1,-1);
    // the 8-node element interleaves the mid-sides
    const double bx[4] = {-1, 1, 1, -1}, by[4] = {-1, -1, 1, 1};
    const double sx[8] = {-1, 0, 1, 1, 1, 0, -1, -1}, sy[8] = {-1, -1, -1, 0, 1, 1, 1, 0};
    for (int i = 0; i < b.nen; ++i) {
        const double nx = b.nen == 4 ? bx[i] : sx[i], ny = b.nen == 4 ? by[i] : sy[i];
        double best = std::numeric_limits<double>::max();
        b.nearest[i] = 0;
        for (int a = 0; a < n1; ++a)
            for (int c = 0; c < n1; ++c)
                if (const double d = std::sqrt((nx - x[a]) * (nx - x[a]) + (ny - y[c]) * (ny - y[c])); best > d) {
                    best = d;
                    b.nearest[i] = a * n1 + c;
                }
    }
    return b;
}

Basis1d make_basis_1d(int nodes) {
    NL_REQUIRE(nodes == 2 || nodes == 3, NLGPU_ERR_UNSUPPORTED, "boundary line elements have 2 or 3 nodes");
    Basis1d b{};
    b.nen = nodes;
    double g[3], gw[3];
    gauss_rule(nodes == 2 ? 1 : 2, g, gw);
    b.nq = nodes == 2 ? 1 : 2;
    for (int q = 0; q < b.nq; ++q) b.w[q] = gw[q] * 1.0;
    for (int i = 0; i < nodes; ++i)
        for (int q = 0; q < b.nq; ++q) {
            const double x = -1.0 + (g[q] - (-1.0)) * 1.0;
            double N, Nx;
            if (nodes == 2) { N = i == 0 ? (1 - x) / 2 : (1 + x) / 2; Nx = i == 0 ? -0.5 : 0.5; }
            else if (i == 0) { N = x * (x - 1) / 2; Nx = (2 * x - 1) / 2; }   // Lagrange on (-1, 0, 1)
            else if (i == 1) { N = (1 - x) * (1 + x); Nx = -2 * x; }
            else { N = x * (x + 1) / 2; Nx = (2 * x + 1) / 2; }
            b.qN[i * b.nq + q] = N; b.qNxi[i * b.nq + q] = Nx;
        }
    return b;
}

void mesh_init(Ctx& ctx) {
    const int nen = ctx.basis.nen, nq = ctx.basis.nq;
    const i64 E = ctx.n_elems, n = ctx.n_nodes;
    ctx.qcoord.resize(size_t(E * nq * 2));
    ctx.jac.resize(size_t(E * nq));
    ctx.deriv.resize(size_t(E * nen * nq * 2));
    ctx.centres.resize(size_t(E * 2));
    NL_LAUNCH(k_quadrature, grid_for(E * (nq + 1), 256), 256, 0, ctx.stream, E, nen, nq, ctx.nodes.p, ctx.elems.p,
              ctx.basis, ctx.qcoord.p, ctx.jac.p, ctx.deriv.p, ctx.centres.p);
    ctx.elem_minnode.resize(size_t(E));
    ctx.elem_maxnode.resize(size_t(E));
    NL_LAUNCH(k_elem_minnode, grid_for(E, 256), 256, 0, ctx.stream, E, nen, ctx.elems.p, ctx.elem_minnode.p,
              ctx.elem_maxnode.p);
    // node -> elements
    ctx.ne_off.resize(size_t(n + 1));
    ctx.ne_off.zero(ctx.stream);
    NL_LAUNCH(k_count_node_elements, grid_for(E * nen, 256), 256, 0, ctx.stream, E, nen, ctx.elems.p, ctx.ne_off.p);
    i64 total = 0;
    exclusive_scan(ctx, ctx.ne_off.p, ctx.ne_off.p, n + 1, &total);
    NL_REQUIRE(total == E * nen, NLGPU_ERR_ARG, "element connectivity references nodes out of range");
    ctx.ne_elem.resize(size_t(E * nen));
    ctx.ne_local.resize(size_t(E * nen));
    ctx.i64_scratch_b.reserve(size_t(n));
    NL_CUDA(cudaMemsetAsync(ctx.i64_scratch_b.p, 0, size_t(n) * sizeof(i64), ctx.stream));
    NL_LAUNCH(k_fill_node_elements, grid_for(E * nen, 256), 256, 0, ctx.stream, E, nen, ctx.elems.p, ctx.ne_off.p,
              ctx.i64_scratch_b.p, ctx.ne_elem.p);
    NL_LAUNCH(k_sort_node_elements, grid_for(n, 128), 128, 0, ctx.stream, n, nen, ctx.elems.p, ctx.ne_off.p,
              ctx.ne_elem.p, ctx.ne_local.p);
    ctx.mesh_ready = true;
}

}  // namespace nlgpu
