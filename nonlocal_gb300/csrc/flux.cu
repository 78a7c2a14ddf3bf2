// Heat flux of a solution: heat_equation_solution_2d::calc_flux
// (heat_equation_solution_2d.hpp:99-137).
//
//   1. local flux at every quadrature point, -Lambda grad T with
//      grad T = sum_i T_i (grad N_i . adj J) / |J| (gradient_in_qnodes,
//      mesh_2d_utils.hpp:40-60; local_flux_in_qnodes, heat_equation_solution_2d.hpp:72-96);
//   2. for a nonlocal model, at every quadrature point x of element eL the
//      influence-weighted average of the local flux over the neighbours'
//      quadrature points, flux = p1 local + (1 - p1) sum w |J| phi(x, x') local(x');
//   3. nodal values: the element-area-weighted mean, over the elements of a
//      node, of the flux at the Gauss point nearest to the node
//      (qnodes_to_nodes, mesh_2d_utils.hpp:82-101; mesh_2d::area, mesh_2d.hpp:225-234).
//
// Step 2 is the same pair loop as the assembly (every ordered neighbour pair,
// nq x nq influence evaluations): one warp per element eL, the lanes spread
// over the (eNL, qNL) points of its neighbour list, each accumulating the
// contributions to all of eL's quadrature points in registers, then a warp
// reduction.  FP64 throughout (post-processing of the FP64 solution).
#include "common.cuh"
#include "influence.cuh"

namespace nlgpu {

namespace {

constexpr int FX_THREADS = 256;

__global__ void k_flux_local(i64 E, int nen, int nq, const int32_t* __restrict__ elems, const double* __restrict__ deriv,
                             const double* __restrict__ jac, const double* __restrict__ cond_field, Model m,
                             const double* __restrict__ T, double* __restrict__ lx, double* __restrict__ ly) {
    for (i64 t = blockIdx.x * i64(blockDim.x) + threadIdx.x; t < E * nq; t += i64(gridDim.x) * blockDim.x) {
        const i64 e = t / nq;
        const int q = int(t % nq);
        double gx = 0.0, gy = 0.0;
        for (int i = 0; i < nen; ++i) {
            const double v = T[elems[e * nen + i]];
            const double* d = deriv + 2 * ((e * nen + i) * nq + q);
            gx += v * d[0];
            gy += v * d[1];
        }
        gx /= jac[t];
        gy /= jac[t];
        double fx, fy;
        if (m.cond_kind == NLGPU_CONDUCTIVITY_ISOTROPIC) {
            const double c = cond_field ? cond_field[t] : m.cond[0];
            fx = gx * -c;
            fy = gy * -c;
        } else if (m.cond_kind == NLGPU_CONDUCTIVITY_ORTHOTROPIC) {
            fx = gx * -m.cond[0];
            fy = gy * -m.cond[1];
        } else {
            fx = -m.cond[0] * gx - m.cond[2] * gy;
            fy = -m.cond[2] * gx - m.cond[1] * gy;
        }
        lx[t] = fx;
        ly[t] = fy;
    }
}

template<int NQ, int INF>
__global__ void __launch_bounds__(FX_THREADS) k_flux_nonlocal(i64 E, const double* __restrict__ qcoord,
                                                              const double* __restrict__ jac, const i64* __restrict__ noff,
                                                              const int32_t* __restrict__ nlist, Model m, Basis b,
                                                              const double* __restrict__ lx,
                                                              const double* __restrict__ ly, double* __restrict__ fx,
                                                              double* __restrict__ fy) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 eL = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; eL < E; eL += warps) {
        double xq[NQ], yq[NQ], ax[NQ], ay[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            xq[q] = qcoord[2 * (eL * NQ + q)];
            yq[q] = qcoord[2 * (eL * NQ + q) + 1];
            ax[q] = 0.0;
            ay[q] = 0.0;
        }
        const i64 kb = noff[eL], items = (noff[eL + 1] - kb) * NQ;
        for (i64 it = lane; it < items; it += 32) {
            const int32_t eNL = nlist[kb + it / NQ];
            const int qn = int(it % NQ);
            const i64 s = i64(eNL) * NQ + qn;
            const double wj = b.w[qn] * jac[s];
            const double xs = qcoord[2 * s], ys = qcoord[2 * s + 1], vx = lx[s], vy = ly[s];
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const double w = wj * (m.norm * shape<INF>(m, xq[q] - xs, yq[q] - ys));
                ax[q] += w * vx;
                ay[q] += w * vy;
            }
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            ax[q] = warp_sum(ax[q]);
            ay[q] = warp_sum(ay[q]);
        }
        if (lane < NQ) {
            double sx = 0.0, sy = 0.0;
#pragma unroll
            for (int q = 0; q < NQ; ++q)
                if (q == lane) { sx = ax[q]; sy = ay[q]; }
            const i64 t = eL * NQ + lane;
            const double nw = 1.0 - m.p1;
            fx[t] = lx[t] * m.p1 + sx * nw;
            fy[t] = ly[t] * m.p1 + sy * nw;
        }
    }
}

__global__ void k_element_area(i64 E, int nen, int nq, const double* __restrict__ jac, Basis b, double* __restrict__ area) {
    for (i64 e = blockIdx.x * i64(blockDim.x) + threadIdx.x; e < E; e += i64(gridDim.x) * blockDim.x) {
        double a = 0.0;
        for (int q = 0; q < nq; ++q) {
            const double factor = b.w[q] * jac[e * nq + q];
            for (int i = 0; i < nen; ++i) a += factor * b.qN[i * nq + q];
        }
        area[e] = a;
    }
}

__global__ void k_flux_nodes(i64 n, const i64* __restrict__ ne_off, const int32_t* __restrict__ ne_elem,
                             const int8_t* __restrict__ ne_local, int nq, Basis b, const double* __restrict__ area,
                             const double* __restrict__ fx, const double* __restrict__ fy, double* __restrict__ ox,
                             double* __restrict__ oy) {
    for (i64 node = blockIdx.x * i64(blockDim.x) + threadIdx.x; node < n; node += i64(gridDim.x) * blockDim.x) {
        double sx = 0.0, sy = 0.0, s = 0.0;
        for (i64 k = ne_off[node]; k < ne_off[node + 1]; ++k) {
            const i64 e = ne_elem[k];
            const double a = area[e];
            const i64 q = e * nq + b.nearest[ne_local[k]];
            sx += a * fx[q];
            sy += a * fy[q];
            s += a;
        }
        ox[node] = sx / s;
        oy[node] = sy / s;
    }
}

template<int NQ>
void launch_nonlocal(Ctx& ctx, const double* lx, const double* ly, double* fx, double* fy) {
    const i64 E = ctx.n_elems;
    const unsigned grid = grid_for(E * 32, FX_THREADS, 152 * 64);
    switch (ctx.model.influence) {
    case NLGPU_INFLUENCE_FAST_POLYNOMIAL:
        NL_LAUNCH((k_flux_nonlocal<NQ, NLGPU_INFLUENCE_FAST_POLYNOMIAL>), grid, FX_THREADS, 0, ctx.stream, E,
                  ctx.qcoord.p, ctx.jac.p, ctx.noff.p, ctx.nlist.p, ctx.model, ctx.basis, lx, ly, fx, fy);
        break;
    case NLGPU_INFLUENCE_POLYNOMIAL:
        NL_LAUNCH((k_flux_nonlocal<NQ, NLGPU_INFLUENCE_POLYNOMIAL>), grid, FX_THREADS, 0, ctx.stream, E,
                  ctx.qcoord.p, ctx.jac.p, ctx.noff.p, ctx.nlist.p, ctx.model, ctx.basis, lx, ly, fx, fy);
        break;
    case NLGPU_INFLUENCE_EXPONENTIAL:
        NL_LAUNCH((k_flux_nonlocal<NQ, NLGPU_INFLUENCE_EXPONENTIAL>), grid, FX_THREADS, 0, ctx.stream, E,
                  ctx.qcoord.p, ctx.jac.p, ctx.noff.p, ctx.nlist.p, ctx.model, ctx.basis, lx, ly, fx, fy);
        break;
    default:
        NL_LAUNCH((k_flux_nonlocal<NQ, NLGPU_INFLUENCE_CONSTANT>), grid, FX_THREADS, 0, ctx.stream, E,
                  ctx.qcoord.p, ctx.jac.p, ctx.noff.p, ctx.nlist.p, ctx.model, ctx.basis, lx, ly, fx, fy);
        break;
    }
}

}  // namespace

void calc_flux(Ctx& ctx, const double* temperature, double* flux_x, double* flux_y) {
    const i64 E = ctx.n_elems, n = ctx.n_nodes;
    const int nen = ctx.basis.nen, nq = ctx.basis.nq;
    dbuf<double> lx, ly, fx, fy, area;
    lx.resize(size_t(E * nq)); ly.resize(size_t(E * nq));
    area.resize(size_t(E));
    NL_LAUNCH(k_flux_local, grid_for(E * nq, FX_THREADS), FX_THREADS, 0, ctx.stream, E, nen, nq, ctx.elems.p,
              ctx.deriv.p, ctx.jac.p, ctx.cond_field.n ? ctx.cond_field.p : nullptr, ctx.model, temperature, lx.p, ly.p);
    const double* qx = lx.p;
    const double* qy = ly.p;
    if (ctx.model.nonlocal()) {
        fx.resize(size_t(E * nq)); fy.resize(size_t(E * nq));
        if (nq == 4) launch_nonlocal<4>(ctx, lx.p, ly.p, fx.p, fy.p);
        else launch_nonlocal<9>(ctx, lx.p, ly.p, fx.p, fy.p);
        qx = fx.p;
        qy = fy.p;
    }
    NL_LAUNCH(k_element_area, grid_for(E, FX_THREADS), FX_THREADS, 0, ctx.stream, E, nen, nq, ctx.jac.p, ctx.basis,
              area.p);
    NL_LAUNCH(k_flux_nodes, grid_for(n, FX_THREADS), FX_THREADS, 0, ctx.stream, n, ctx.ne_off.p, ctx.ne_elem.p,
              ctx.ne_local.p, nq, ctx.basis, area.p, qx, qy, flux_x, flux_y);
    NL_CUDA(cudaStreamSynchronize(ctx.stream));   // the scratch buffers are freed on return
}

}  // namespace nlgpu
