// CPU restatement of NonLocFEM's nonlocal thermal hot path (the "port" oracle).
//
// TEST INFRASTRUCTURE ONLY.  Used by tests/ as the checker of the CUDA path, by
// __graft_entry__.smoke() as its checker and by bench.py as the timed CPU
// baseline ("port").  The shipped library never links or calls it.
//
// Every function follows the reference implementation step by step and cites
// the file:line it restates (paths relative to the reference project root).
// The loop structure of the assembly is the reference's own
// (mesh_run -> integrator -> integrate_nonlocal per matrix entry, OpenMP
// dynamic over node rows), so that timing it on the host cores is a fair
// stand-in for timing the reference.  Third-party pieces the reference calls
// (Eigen's IncompleteCholesky and SimplicialCholesky) come from the
// restatements in eigen_shim/Eigen/src/shim.hpp.
//
// Build: oracle/build.py (g++ -O3 -fopenmp -ffp-contract=off, no ISA flags).

#include "eigen_shim/Eigen/src/shim.hpp"

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <numbers>
#include <string>
#include <unordered_set>
#include <vector>

namespace {

using i64 = int64_t;
using vec2 = std::array<double, 2>;

enum { ORC_BILINEAR = 2, ORC_SERENDIPITY = 3 };   // element_2d_t numbering (elements_set.hpp:22-28)
enum { INF_CONSTANT = 0, INF_POLYNOMIAL = 1, INF_EXPONENTIAL = 2, INF_FAST_POLYNOMIAL = 3 };
enum { COND_ISO = 0, COND_ORTHO = 1, COND_ANISO = 2 };
// temperature_2d, flux_2d, convection_2d, radiation_2d, combined_flux_2d
// (thermal_boundary_conditions_2d.hpp:9-98)
enum { BC_TEMPERATURE = 0, BC_FLUX = 1, BC_CONVECTION = 2, BC_RADIATION = 3, BC_COMBINED = 4 };
constexpr double STEFAN_BOLTZMANN = 5.67036713e-8;   // metamath/utils/constants.hpp:12

// ------------------------------------------------------------------ elements
// Gauss nodes/weights: gaussian_quadrature.hpp:22-40.
struct Gauss { std::vector<double> x, w; };
Gauss gauss(int n) {
    if (n == 1) return {{0.0}, {2.0}};
    if (n == 2) return {{-1.0 / std::sqrt(3.0), 1.0 / std::sqrt(3.0)}, {1.0, 1.0}};
    return {{-std::sqrt(3.0 / 5.0), 0.0, std::sqrt(3.0 / 5.0)}, {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0}};
}

// Basis of serendipity<T,1> (serendipity_2d.hpp:144-175) and serendipity<T,2>
// with parameter p = 2/9 (serendipity_2d.hpp:177-222); derivatives by hand.
void basis2d(int type, int i, double x, double y, double& N, double& Nx, double& Ny) {
    if (type == ORC_BILINEAR) {
        const double sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
        N = (1 + sx[i] * x) * (1 + sy[i] * y) / 4;
        Nx = sx[i] * (1 + sy[i] * y) / 4;
        Ny = sy[i] * (1 + sx[i] * x) / 4;
        return;
    }
    const double p = 2.0 / 9.0;
    const double a = 9 * p - 1, b = 9 * p + 3, c = 9 * p - 5;
    switch (i) {
    case 0: { const double g = a * (1 + x + y) + b * x * y;
        N = (1 - x) * (1 - y) * g / 16;
        Nx = (-(1 - y) * g + (1 - x) * (1 - y) * (a + b * y)) / 16;
        Ny = (-(1 - x) * g + (1 - x) * (1 - y) * (a + b * x)) / 16; break; }
    case 1: N = -(1 - x * x) * (1 - y) * (c + b * y) / 16;
        Nx = 2 * x * (1 - y) * (c + b * y) / 16;
        Ny = (1 - x * x) * ((c + b * y) - (1 - y) * b) / 16; break;
    case 2: { const double g = a * (1 - x + y) - b * x * y;
        N = (1 + x) * (1 - y) * g / 16;
        Nx = ((1 - y) * g + (1 + x) * (1 - y) * (-a - b * y)) / 16;
        Ny = (-(1 + x) * g + (1 + x) * (1 - y) * (a - b * x)) / 16; break; }
    case 3: N = -(1 - y * y) * (1 + x) * (c - b * x) / 16;
        Nx = -((1 - y * y) * (c - b * x) - (1 - y * y) * (1 + x) * b) / 16;
        Ny = 2 * y * (1 + x) * (c - b * x) / 16; break;
    case 4: { const double g = a * (1 - x - y) + b * x * y;
        N = (1 + x) * (1 + y) * g / 16;
        Nx = ((1 + y) * g + (1 + x) * (1 + y) * (-a + b * y)) / 16;
        Ny = ((1 + x) * g + (1 + x) * (1 + y) * (-a + b * x)) / 16; break; }
    case 5: N = -(1 - x * x) * (1 + y) * (c - b * y) / 16;
        Nx = 2 * x * (1 + y) * (c - b * y) / 16;
        Ny = -((1 - x * x) * (c - b * y) - (1 - x * x) * (1 + y) * b) / 16; break;
    case 6: { const double g = a * (1 + x - y) - b * x * y;
        N = (1 - x) * (1 + y) * g / 16;
        Nx = (-(1 + y) * g + (1 - x) * (1 + y) * (a - b * y)) / 16;
        Ny = ((1 - x) * g + (1 - x) * (1 + y) * (-a - b * x)) / 16; break; }
    default: N = -(1 - y * y) * (1 - x) * (c + b * x) / 16;
        Nx = (1 - y * y) * ((c + b * x) - (1 - x) * b) / 16;
        Ny = 2 * y * (1 - x) * (c + b * x) / 16; break;
    }
}

struct Element2d {
    int type = ORC_BILINEAR, nen = 4, nq = 4;
    std::vector<double> qN, qNxi, qNeta, w, centre;   // [i*nq + q], centre N_i(0,0)
};

// element_2d_integrate::set_quadrature (element_2d_integrate.hpp:69-106) on the
// rectangle [-1,1]^2 with the element's Gauss rule (vtk_elements_set.hpp:54-72).
Element2d make_element2d(int type) {
    Element2d el;
    el.type = type;
    el.nen = type == ORC_BILINEAR ? 4 : 8;
    const Gauss g = gauss(type == ORC_BILINEAR ? 2 : 3);
    const int n1 = int(g.x.size());
    el.nq = n1 * n1;
    const double jx = (1.0 - (-1.0)) / (1.0 - (-1.0));
    std::vector<double> x(static_cast<size_t>(n1)), y(static_cast<size_t>(n1)), jy(static_cast<size_t>(n1));
    el.w.resize(size_t(el.nq));
    for (int i = 0; i < n1; ++i) {
        x[size_t(i)] = -1.0 + (g.x[size_t(i)] - (-1.0)) * jx;
        jy[size_t(i)] = (1.0 - (-1.0)) / (1.0 - (-1.0));
        for (int j = 0; j < n1; ++j) {
            y[size_t(j)] = -1.0 + (g.x[size_t(j)] - (-1.0)) * jy[size_t(i)];
            el.w[size_t(i * n1 + j)] = g.w[size_t(i)] * jx * g.w[size_t(j)] * jy[size_t(i)];
        }
    }
    el.qN.resize(size_t(el.nen * el.nq)); el.qNxi.resize(el.qN.size()); el.qNeta.resize(el.qN.size());
    for (int i = 0; i < el.nen; ++i)
        for (int a = 0; a < n1; ++a)
            for (int b = 0; b < n1; ++b) {
                const size_t k = size_t(i * el.nq + a * n1 + b);
                basis2d(type, i, x[size_t(a)], y[size_t(b)], el.qN[k], el.qNxi[k], el.qNeta[k]);
            }
    el.centre.resize(size_t(el.nen));
    for (int i = 0; i < el.nen; ++i) { double dx, dy; basis2d(type, i, 0.0, 0.0, el.centre[size_t(i)], dx, dy); }
    return el;
}

// 1D boundary elements: lagrangian order 1 with Gauss-1, order 2 with Gauss-2
// (vtk_elements_set.hpp:43-52, element_1d_integrate.hpp:60-80).
struct Element1d { int nen = 2, nq = 1; std::vector<double> qN, qNxi, w; };
Element1d make_element1d(int nen) {
    Element1d el; el.nen = nen;
    const Gauss g = gauss(nen == 2 ? 1 : 2);
    el.nq = int(g.x.size());
    for (int q = 0; q < el.nq; ++q) el.w.push_back(g.w[size_t(q)]);
    el.qN.resize(size_t(nen * el.nq)); el.qNxi.resize(el.qN.size());
    for (int i = 0; i < nen; ++i)
        for (int q = 0; q < el.nq; ++q) {
            const double x = -1.0 + (g.x[size_t(q)] - (-1.0)) * 1.0;
            double N, Nx;
            if (nen == 2) { N = i == 0 ? (1 - x) / 2 : (1 + x) / 2; Nx = i == 0 ? -0.5 : 0.5; }
            else if (i == 0) { N = x * (x - 1) / 2; Nx = (2 * x - 1) / 2; }
            else if (i == 1) { N = (1 - x) * (1 + x); Nx = -2 * x; }
            else { N = x * (x + 1) / 2; Nx = (2 * x + 1) / 2; }
            el.qN[size_t(i * el.nq + q)] = N; el.qNxi[size_t(i * el.nq + q)] = Nx;
        }
    return el;
}

// ---------------------------------------------------------------- CSR helpers
struct Csr {
    i64 rows = 0, cols = 0;
    std::vector<i64> rowptr{0}, col;
    std::vector<double> val;
    i64 nnz() const { return rowptr.empty() ? 0 : rowptr.back(); }
    double* find(i64 r, i64 c) {
        auto b = col.begin() + rowptr[size_t(r)], e = col.begin() + rowptr[size_t(r) + 1];
        auto it = std::lower_bound(b, e, c);
        return (it != e && *it == c) ? &val[size_t(it - col.begin())] : nullptr;
    }
};

// value: the temperature, or the second-kind flux (operator() of the condition)
struct Boundary {
    int kind; int nen; std::vector<i64> edges; double value; std::vector<double> node_values;
    double heat_transfer = 0.0, emissivity = 0.0;
    bool convection() const { return kind == BC_CONVECTION || kind == BC_COMBINED; }
    bool radiation() const { return kind == BC_RADIATION || kind == BC_COMBINED; }
};

struct Problem {
    Element2d el;
    i64 n_nodes = 0, n_elems = 0;
    std::vector<double> nodes;           // [n][2]
    std::vector<i64> elems;              // [e][nen]
    std::vector<std::vector<i64>> node_elements;
    std::vector<double> qcoord, jac, deriv;   // [e][q][2], [e][q], [e][i][q][2]
    std::vector<double> centres;
    // model
    int influence = INF_FAST_POLYNOMIAL, inf_n = 2, inf_p = 2;
    double inf_q = 1, r[2] = {0, 0}, p1 = 1.0, norm = 1.0;
    int cond_kind = COND_ISO; double cond[3] = {1, 0, 0};
    std::vector<double> cond_q;          // optional per-quadrature conductivity (iso) [e][q]
    double capacity = 1.0, density = 1.0;
    // neighbours
    std::vector<i64> noff, nlist;
    double search_r[2] = {0, 0};
    // boundaries / source
    std::vector<Boundary> bnds;
    double source = 0.0;
    std::vector<double> source_q;        // optional per-quadrature source [e][q]
    std::vector<double> dirichlet_override;   // optional per-node Dirichlet values
    std::vector<uint8_t> is_inner;
    std::vector<double> x_dirichlet;
    // matrices
    Csr K_inner, K_bound, K_local, C_inner;
    bool symmetric = true;
    std::vector<double> rhs, rhs_init, solution;
    // solver outputs
    long iterations = 0; double residual = 0, true_residual = 0, ilt_shift = 0; int ilt_ok = 0, ilt_attempts = 0;
    std::vector<i64> L_colptr, L_rowidx; std::vector<double> L_val, L_scale;
    std::vector<double> history;
    // stationary_equation_parameters_2d (stationary_heat_equation_solver_2d.hpp:19-26)
    double nl_tolerance = 1e-8, energy = 0.0;
    long nl_max_iterations = 100, nonlinear_iterations = 0;
    std::vector<double> initial;
    std::map<std::string, double> timings;
    // optional checkpoint of a solve run past a looser tolerance: the CG time
    // and iterations at which the stopping measure first reached record_tol
    double record_tol = 0.0;
    long record_iterations = -1;
};

bool nonlocal_model(const Problem& p) { return p.p1 < 0.999; }   // nonlocal_constants.hpp:22-37

// influence_functions_2d.hpp:39-148 with powered_distance (search_function.hpp:29-73)
double powered_dist(const Problem& p, const vec2& a, const vec2& b, const double* r) {
    const double z0 = (a[0] - b[0]) / r[0], z1 = (a[1] - b[1]) / r[1];
    if (p.inf_n == 2) return z0 * z0 + z1 * z1;
    if (p.inf_n == 1) return std::abs(z0) + std::abs(z1);
    return std::pow(std::abs(z0), p.inf_n) + std::pow(std::abs(z1), p.inf_n);
}
double ipow(double x, int n) {   // power.hpp:25-40
    double res = 1.0;
    while (n > 0) { if (n & 1) { res *= x; --n; } else { x *= x; n >>= 1; } }
    return res;
}
void init_norm(Problem& p) {
    const double n = p.inf_n;
    switch (p.influence) {
    case INF_FAST_POLYNOMIAL: p.norm = 2.0 / (std::numbers::pi * p.r[0] * p.r[1]); break;
    case INF_POLYNOMIAL: p.norm = n * p.inf_p / (4 * p.r[0] * p.r[1] * std::beta(1 / n, 1 / n) * std::beta(2.0 / p.inf_p, p.inf_q + 1)); break;
    case INF_EXPONENTIAL: p.norm = (n * p.inf_p * std::pow(4.0, 1 / n) * std::pow(p.inf_q, 2.0 / p.inf_p)) /
                                   (8 * p.r[0] * p.r[1] * std::tgamma(2.0 / p.inf_p) * std::beta(0.5, 1 / n)); break;
    default: p.norm = std::tgamma(1 + 2 / n) / (4 * p.r[0] * p.r[1] * ipow(std::tgamma(1 + 1 / n), 2)); break;
    }
}
double influence(const Problem& p, const vec2& a, const vec2& b) {
    const double d = powered_dist(p, a, b, p.r);
    switch (p.influence) {
    case INF_FAST_POLYNOMIAL: return d < 1.0 ? p.norm * (1.0 - d) : 0.0;
    case INF_POLYNOMIAL: {   // exponent p/n on the powered distance (influence_functions_2d.hpp:84-91)
        const bool integral = p.inf_p % p.inf_n == 0;
        const double dp = integral ? (p.inf_p / p.inf_n == 1 ? d : ipow(d, p.inf_p / p.inf_n)) : std::pow(d, double(p.inf_p) / p.inf_n);
        const int q = int(p.inf_q);
        return d < 1.0 ? p.norm * (q == 1 ? 1.0 - dp : ipow(1.0 - dp, q)) : 0.0;
    }
    case INF_EXPONENTIAL: {
        const bool integral = p.inf_p % p.inf_n == 0;
        const double dp = integral ? (p.inf_p / p.inf_n == 1 ? d : ipow(d, p.inf_p / p.inf_n)) : std::pow(d, double(p.inf_p) / p.inf_n);
        return p.norm * std::exp(-p.inf_q * dp);
    }
    default: return d <= 1.0 ? p.norm : 0.0;
    }
}

vec2 qc(const Problem& p, i64 e, int q) { const double* c = &p.qcoord[size_t((e * p.el.nq + q) * 2)]; return {c[0], c[1]}; }
const double* dN(const Problem& p, i64 e, int i, int q) { return &p.deriv[size_t(((e * p.el.nen + i) * p.el.nq + q) * 2)]; }
i64 node_of(const Problem& p, i64 e, int i) { return p.elems[size_t(e * p.el.nen + i)]; }

// mesh_2d::init (mesh_2d.hpp:97-108): node_elements_2d, quad coords, Jacobi
// matrices, |J| and derivatives_in_quad (mesh_container_2d_utils.hpp:18-123).
void mesh_init(Problem& p) {
    const int nen = p.el.nen, nq = p.el.nq;
    p.node_elements.assign(size_t(p.n_nodes), {});
    for (i64 e = 0; e < p.n_elems; ++e)
        for (int i = 0; i < nen; ++i) p.node_elements[size_t(node_of(p, e, i))].push_back(e);
    p.qcoord.assign(size_t(p.n_elems * nq * 2), 0.0);
    p.jac.assign(size_t(p.n_elems * nq), 0.0);
    p.deriv.assign(size_t(p.n_elems * nen * nq * 2), 0.0);
    p.centres.assign(size_t(p.n_elems * 2), 0.0);
    for (i64 e = 0; e < p.n_elems; ++e) {
        for (int q = 0; q < nq; ++q) {
            double cx = 0, cy = 0, J00 = 0, J01 = 0, J10 = 0, J11 = 0;
            for (int i = 0; i < nen; ++i) {
                const double* x = &p.nodes[size_t(node_of(p, e, i) * 2)];
                const double n = p.el.qN[size_t(i * nq + q)];
                cx += x[0] * n; cy += x[1] * n;
                const double dxi = p.el.qNxi[size_t(i * nq + q)], deta = p.el.qNeta[size_t(i * nq + q)];
                J00 += x[0] * dxi; J01 += x[0] * deta; J10 += x[1] * dxi; J11 += x[1] * deta;
            }
            p.qcoord[size_t((e * nq + q) * 2)] = cx; p.qcoord[size_t((e * nq + q) * 2 + 1)] = cy;
            p.jac[size_t(e * nq + q)] = std::abs(J00 * J11 - J01 * J10);
            for (int i = 0; i < nen; ++i) {
                const double dxi = p.el.qNxi[size_t(i * nq + q)], deta = p.el.qNeta[size_t(i * nq + q)];
                double* d = &p.deriv[size_t(((e * nen + i) * nq + q) * 2)];
                d[0] = dxi * J11 - deta * J10;
                d[1] = -dxi * J01 + deta * J00;
            }
        }
        double cx = 0, cy = 0;   // element_data_2d::center (mesh_container_2d.hpp:131-139)
        for (int i = 0; i < nen; ++i) {
            const double* x = &p.nodes[size_t(node_of(p, e, i) * 2)];
            cx += x[0] * p.el.centre[size_t(i)]; cy += x[1] * p.el.centre[size_t(i)];
        }
        p.centres[size_t(e * 2)] = cx; p.centres[size_t(e * 2 + 1)] = cy;
    }
}

// find_neighbours (find_neighbours.hpp:120-160) for one group holding every
// element, with increase_influence (:424-434) and the bucket grid (:436-467).
void find_neighbours(Problem& p, int strategy) {
    const i64 E = p.n_elems;
    auto cen = [&](i64 e) { return vec2{p.centres[size_t(2 * e)], p.centres[size_t(2 * e + 1)]}; };
    double add = 0.0;
    if (strategy != 0) {   // diameter_between_elements_centers (:399-422)
        double d = strategy == 2 ? std::numeric_limits<double>::max() : 0.0;
        double mean_sum = 0.0; size_t pairs = 0;
        std::vector<std::pair<i64, i64>> seen;
        for (i64 e = 0; e < E; ++e)
            for (int i = 0; i < p.el.nen; ++i)
                for (const i64 a : p.node_elements[size_t(node_of(p, e, i))]) {
                    const vec2 ce = cen(e), ca = cen(a);
                    const double z0 = ce[0] - ca[0], z1 = ce[1] - ca[1];
                    const double dist = z0 * z0 + z1 * z1;
                    if (strategy == 1) d = std::max(d, dist);
                    else if (strategy == 2) d = std::min(d, dist);
                    else {
                        const auto key = std::minmax(e, a);
                        if (std::find(seen.begin(), seen.end(), std::pair<i64, i64>{key.first, key.second}) == seen.end()) {
                            seen.push_back({key.first, key.second}); mean_sum += std::sqrt(dist); ++pairs;
                        }
                    }
                }
        add = strategy == 3 ? mean_sum / double(pairs) : std::sqrt(d);
    }
    const double R[2] = {p.r[0] + add, p.r[1] + add};
    p.search_r[0] = R[0]; p.search_r[1] = R[1];
    double left = std::numeric_limits<double>::max(), down = left;
    double right = std::numeric_limits<double>::lowest(), up = right;
    for (i64 e = 0; e < E; ++e)
        for (int i = 0; i < p.el.nen; ++i) {
            const double* x = &p.nodes[size_t(node_of(p, e, i) * 2)];
            left = std::min(left, x[0]); down = std::min(down, x[1]);
            right = std::max(right, x[0]); up = std::max(up, x[1]);
        }
    const double maxr = std::max(R[0], R[1]);
    const size_t rows = size_t((right - left) / maxr) + 1, cols = size_t((up - down) / maxr) + 1;
    std::vector<std::vector<i64>> cells(rows * cols);
    auto cell_of = [&](const vec2& c) { return std::pair<size_t, size_t>{size_t((c[0] - left) / maxr), size_t((c[1] - down) / maxr)}; };
    for (i64 e = 0; e < E; ++e) { const auto [a, b] = cell_of(cen(e)); cells[a * cols + b].push_back(e); }
    p.noff.assign(size_t(E) + 1, 0); p.nlist.clear();
    for (i64 e = 0; e < E; ++e) {
        const auto [row, col] = cell_of(cen(e));
        for (size_t i = row ? row - 1 : row; i < (row != rows - 1 ? row + 2 : row + 1); ++i)
            for (size_t j = col ? col - 1 : col; j < (col != cols - 1 ? col + 2 : col + 1); ++j)
                for (const i64 f : cells[i * cols + j])
                    if (powered_dist(p, cen(e), cen(f), R) <= 1.0) p.nlist.push_back(f);
        p.noff[size_t(e) + 1] = i64(p.nlist.size());
    }
}

double cond_at(const Problem& p, i64 e, int q, int comp) {
    if (!p.cond_q.empty()) return p.cond_q[size_t(e * p.el.nq + q)];
    return p.cond[comp];
}

// conductivity_matrix_2d::integrate_local (conductivity_matrix_2d.hpp:106-130)
double integrate_local(const Problem& p, i64 e, int i, int j) {
    double integral = 0.0;
    for (int q = 0; q < p.el.nq; ++q) {
        const double* a = dN(p, e, i, q); const double* b = dN(p, e, j, q);
        double value;
        if (p.cond_kind == COND_ISO) value = cond_at(p, e, q, 0) * (a[0] * b[0] + a[1] * b[1]);
        else if (p.cond_kind == COND_ORTHO) value = p.cond[0] * a[0] * b[0] + p.cond[1] * a[1] * b[1];
        else value = a[0] * (p.cond[0] * b[0] + p.cond[2] * b[1]) + a[1] * (p.cond[2] * b[0] + p.cond[1] * b[1]);
        integral += p.el.w[size_t(q)] * value / p.jac[size_t(e * p.el.nq + q)];
    }
    return integral;
}

// conductivity_matrix_2d::integrate_nonlocal (conductivity_matrix_2d.hpp:132-164)
double integrate_nonlocal(const Problem& p, i64 eL, i64 eNL, int iL, int jNL) {
    double integral = 0.0;
    for (int qL = 0; qL < p.el.nq; ++qL) {
        double in0 = 0.0, in1 = 0.0;
        const vec2 xL = qc(p, eL, qL);
        const double* a = dN(p, eL, iL, qL);
        for (int qNL = 0; qNL < p.el.nq; ++qNL) {
            const double* b = dN(p, eNL, jNL, qNL);
            const double iw = p.el.w[size_t(qNL)] * influence(p, xL, qc(p, eNL, qNL));
            if (p.cond_kind == COND_ISO) { const double s = iw * cond_at(p, eNL, qNL, 0); in0 += s * b[0]; in1 += s * b[1]; }
            else if (p.cond_kind == COND_ORTHO) { in0 += iw * p.cond[0] * b[0]; in1 += iw * p.cond[1] * b[1]; }
            else { in0 += iw * (p.cond[0] * b[0] + p.cond[2] * b[1]); in1 += iw * (p.cond[2] * b[0] + p.cond[1] * b[1]); }
        }
        integral += p.el.w[size_t(qL)] * (a[0] * in0 + a[1] * in1);
    }
    return integral;
}

// matrix_separator_base::part (matrix_separator_base.hpp:51-58): 0 INNER, 1 BOUND, 2 NO
int part(const Problem& p, i64 row, i64 col, bool symmetric) {
    if (p.is_inner[size_t(col)]) {
        if ((!symmetric || row <= col) && p.is_inner[size_t(row)]) return 0;
    } else if (row != col) return 1;
    return 2;
}

// Portrait (shift_initializer/matrix_index_initializer, matrix_assembler_2d.hpp:144-176)
// and values (integrator, integrator.hpp:62-91; calc_coeffs :463-475) of
// conductivity_matrix_2d::compute (conductivity_matrix_2d.hpp:166-193).
// The three mesh_run passes (mesh_2d_utils.hpp:13-37) run over node rows with
// OpenMP dynamic scheduling; a per-thread flag array marks visited columns.
void assemble(Problem& p, bool local_only, bool symmetric, Csr& inner, Csr& bound,
              double (*local_fn)(const Problem&, i64, int, int), double local_scale, double nonlocal_scale) {
    const i64 n = p.n_nodes;
    const bool nonlocal = !local_only && nonlocal_model(p);
    inner = Csr{}; bound = Csr{};
    inner.rows = bound.rows = n; inner.cols = bound.cols = n;
    inner.rowptr.assign(size_t(n) + 1, 0); bound.rowptr.assign(size_t(n) + 1, 0);
    std::vector<std::vector<i64>> icols(static_cast<size_t>(n)), bcols(static_cast<size_t>(n));
    #pragma omp parallel
    {
        std::vector<uint8_t> fi(static_cast<size_t>(n), 0), fb(static_cast<size_t>(n), 0);
        #pragma omp for schedule(dynamic)
        for (i64 row = 0; row < n; ++row) {
            auto visit = [&](i64 col) {
                const int pt = part(p, row, col, symmetric);
                if (pt == 0 && !fi[size_t(col)]) { fi[size_t(col)] = 1; icols[size_t(row)].push_back(col); }
                if (pt == 1 && !fb[size_t(col)]) { fb[size_t(col)] = 1; bcols[size_t(row)].push_back(col); }
            };
            for (const i64 eL : p.node_elements[size_t(row)]) {
                if (!nonlocal) { for (int j = 0; j < p.el.nen; ++j) visit(node_of(p, eL, j)); }
                else for (i64 k = p.noff[size_t(eL)]; k < p.noff[size_t(eL) + 1]; ++k)
                    for (int j = 0; j < p.el.nen; ++j) visit(node_of(p, p.nlist[size_t(k)], j));
            }
            if (!p.is_inner[size_t(row)]) icols[size_t(row)].push_back(row);   // first_kind_filler
            for (const i64 c : icols[size_t(row)]) fi[size_t(c)] = 0;
            for (const i64 c : bcols[size_t(row)]) fb[size_t(c)] = 0;
            std::sort(icols[size_t(row)].begin(), icols[size_t(row)].end());
            std::sort(bcols[size_t(row)].begin(), bcols[size_t(row)].end());
        }
    }
    for (i64 r = 0; r < n; ++r) {
        inner.rowptr[size_t(r) + 1] = inner.rowptr[size_t(r)] + i64(icols[size_t(r)].size());
        bound.rowptr[size_t(r) + 1] = bound.rowptr[size_t(r)] + i64(bcols[size_t(r)].size());
    }
    inner.col.resize(size_t(inner.nnz())); inner.val.assign(size_t(inner.nnz()), 0.0);
    bound.col.resize(size_t(bound.nnz())); bound.val.assign(size_t(bound.nnz()), 0.0);
    for (i64 r = 0; r < n; ++r) {
        std::copy(icols[size_t(r)].begin(), icols[size_t(r)].end(), inner.col.begin() + inner.rowptr[size_t(r)]);
        std::copy(bcols[size_t(r)].begin(), bcols[size_t(r)].end(), bound.col.begin() + bound.rowptr[size_t(r)]);
    }
    icols.clear(); bcols.clear();
    #pragma omp parallel for schedule(dynamic)
    for (i64 row = 0; row < n; ++row) {
        for (const i64 eL : p.node_elements[size_t(row)]) {
            int iL = 0;
            while (node_of(p, eL, iL) != row) ++iL;
            auto add = [&](i64 col, double v) {
                const int pt = part(p, row, col, symmetric);
                if (pt == 2) return;
                double* slot = pt == 0 ? inner.find(row, col) : bound.find(row, col);
                *slot += v;
            };
            if (!nonlocal) {
                for (int j = 0; j < p.el.nen; ++j) {
                    const i64 col = node_of(p, eL, j);
                    if (part(p, row, col, symmetric) == 2) continue;
                    add(col, local_scale * local_fn(p, eL, iL, j));
                }
            } else {
                for (i64 k = p.noff[size_t(eL)]; k < p.noff[size_t(eL) + 1]; ++k) {
                    const i64 eNL = p.nlist[size_t(k)];
                    for (int j = 0; j < p.el.nen; ++j) {
                        const i64 col = node_of(p, eNL, j);
                        if (part(p, row, col, symmetric) == 2) continue;
                        double v = nonlocal_scale * integrate_nonlocal(p, eL, eNL, iL, j);
                        if (eL == eNL) v += local_scale * local_fn(p, eL, iL, j);
                        add(col, v);
                    }
                }
            }
        }
        if (!p.is_inner[size_t(row)]) inner.val[size_t(inner.rowptr[size_t(row)])] = 1.0;
    }
}

// heat_capacity_matrix_2d::integrate_basic_pair (heat_capacity_matrix_2d.hpp:30-35)
double integrate_capacity(const Problem& p, i64 e, int i, int j) {
    double integral = 0.0;
    for (int q = 0; q < p.el.nq; ++q)
        integral += p.el.w[size_t(q)] * p.el.qN[size_t(i * p.el.nq + q)] * p.el.qN[size_t(j * p.el.nq + q)] * p.jac[size_t(e * p.el.nq + q)];
    return integral;
}

// 1D boundary element data (mesh_container_2d.hpp:110-128) and the flux
// integral of boundary_condition_second_kind_2d (boundary_condition_second_kind_2d.hpp:12-33).
void boundary_vectors(Problem& p) {
    const i64 n = p.n_nodes;
    p.is_inner.assign(size_t(n), 1);
    p.x_dirichlet.assign(size_t(n), 0.0);
    for (const Boundary& b : p.bnds)   // inner_nodes (solvers_utils.hpp:31-40)
        if (b.kind == BC_TEMPERATURE)
            for (const i64 v : b.edges) p.is_inner[size_t(v)] = 0;
    p.rhs_init.assign(size_t(n), 0.0);
    for (const Boundary& b : p.bnds) {
        if (b.kind == BC_TEMPERATURE) continue;
        const Element1d el = make_element1d(b.nen);
        const i64 ne = i64(b.edges.size()) / b.nen;
        for (i64 e = 0; e < ne; ++e)
            for (int i = 0; i < b.nen; ++i) {
                double integral = 0.0;
                for (int q = 0; q < el.nq; ++q) {
                    double J0 = 0, J1 = 0;
                    for (int k = 0; k < b.nen; ++k) {
                        const double* x = &p.nodes[size_t(b.edges[size_t(e * b.nen + k)] * 2)];
                        J0 += x[0] * el.qNxi[size_t(k * el.nq + q)]; J1 += x[1] * el.qNxi[size_t(k * el.nq + q)];
                    }
                    integral += el.w[size_t(q)] * el.qN[size_t(i * el.nq + q)] * b.value * std::sqrt(J0 * J0 + J1 * J1);
                }
                p.rhs_init[size_t(b.edges[size_t(e * b.nen + i)])] += integral;
            }
    }
    if (p.source != 0.0 || !p.source_q.empty())   // integrate_right_part (right_part_2d.hpp:10-35)
        for (i64 node = 0; node < n; ++node)
            for (const i64 e : p.node_elements[size_t(node)]) {
                int i = 0;
                while (node_of(p, e, i) != node) ++i;
                double integral = 0.0;
                for (int q = 0; q < p.el.nq; ++q)
                    integral += p.el.w[size_t(q)] * p.el.qN[size_t(i * p.el.nq + q)] * p.jac[size_t(e * p.el.nq + q)] *
                                (p.source_q.empty() ? p.source : p.source_q[size_t(e * p.el.nq + q)]);
                p.rhs_init[size_t(node)] += integral;
            }
    // calc_vector (boundary_condition_first_kind_2d.hpp:16-26): first non-zero wins
    for (const Boundary& b : p.bnds)
        if (b.kind == BC_TEMPERATURE)
            for (size_t k = 0; k < b.edges.size(); ++k) {
                const i64 v = b.edges[k];
                const double value = b.node_values.empty() ? b.value : b.node_values[k];
                if (p.x_dirichlet[size_t(v)] == 0.0) p.x_dirichlet[size_t(v)] = value;
            }
    if (!p.dirichlet_override.empty())
        for (i64 v = 0; v < n; ++v) if (!p.is_inner[size_t(v)]) p.x_dirichlet[size_t(v)] = p.dirichlet_override[size_t(v)];
}

// boundary_condition_first_kind_2d (boundary_condition_first_kind_2d.hpp:50-59)
void apply_first_kind(const Problem& p, const Csr& bound, std::vector<double>& f) {
    for (i64 r = 0; r < bound.rows; ++r) {
        double s = 0.0;
        for (i64 k = bound.rowptr[size_t(r)]; k < bound.rowptr[size_t(r) + 1]; ++k) s += bound.val[size_t(k)] * p.x_dirichlet[size_t(bound.col[size_t(k)])];
        f[size_t(r)] -= s;
    }
    for (i64 r = 0; r < p.n_nodes; ++r) if (!p.is_inner[size_t(r)]) f[size_t(r)] = p.x_dirichlet[size_t(r)];
}

// |J| of boundary edge e of group b at its quadrature point q (element_1d_data::jacobi_matrix)
double edge_jacobian(const Problem& p, const Boundary& b, const Element1d& el, i64 e, int q) {
    double J0 = 0, J1 = 0;
    for (int k = 0; k < b.nen; ++k) {
        const double* x = &p.nodes[size_t(b.edges[size_t(e * b.nen + k)] * 2)];
        J0 += x[0] * el.qNxi[size_t(k * el.nq + q)]; J1 += x[1] * el.qNxi[size_t(k * el.nq + q)];
    }
    return std::sqrt(J0 * J0 + J1 * J1);
}

// the stored entry (row, col) of A (sorted rows), or -1
i64 find_entry(const Csr& A, i64 row, i64 col) {
    for (i64 k = A.rowptr[size_t(row)]; k < A.rowptr[size_t(row) + 1]; ++k)
        if (A.col[size_t(k)] == col) return k;
    return -1;
}

// run_by_boundaries over the edges of every group of one kind (solvers_utils.hpp:11-29):
// f(group, edge, i, row) for each local node i of each edge
template<class Pred, class F>
void for_boundary_rows(const Problem& p, Pred pred, F&& f) {
    for (const Boundary& b : p.bnds) {
        if (!pred(b)) continue;
        const i64 ne = i64(b.edges.size()) / b.nen;
        for (i64 e = 0; e < ne; ++e)
            for (int i = 0; i < b.nen; ++i) f(b, e, i, b.edges[size_t(e * b.nen + i)]);
    }
}

// convection_condition_2d (convection_condition_2d.hpp:11-31): alpha int N_i N_j |J|
// into the entries (row, col >= row); rows of temperature nodes are skipped (the
// reference resets them afterwards)
void convection_condition(const Problem& p, Csr& K) {
    for_boundary_rows(p, [](const Boundary& b) { return b.convection(); },
        [&](const Boundary& b, i64 e, int i, i64 row) {
            if (!p.is_inner[size_t(row)]) return;
            const Element1d el = make_element1d(b.nen);
            for (int j = 0; j < b.nen; ++j) {
                const i64 col = b.edges[size_t(e * b.nen + j)];
                if (col < row || !p.is_inner[size_t(col)]) continue;
                double integral = 0.0;
                for (int q = 0; q < el.nq; ++q)
                    integral += el.w[size_t(q)] * el.qN[size_t(i * el.nq + q)] * el.qN[size_t(j * el.nq + q)] *
                                edge_jacobian(p, b, el, e, q);
                const i64 k = find_entry(K, row, col);
                if (k >= 0) K.val[size_t(k)] += b.heat_transfer * integral;
            }
        });
}

// radiation_condition_2d, stationary overload (radiation_condition_2d.hpp:59-104):
// K(row, col >= row) -= 4 sigma eps int T^3 N_i N_j |J|, r[row] -= sigma eps int T^4 N_i |J|
// with T the previous temperature at the edge's quadrature points
void radiation_condition(const Problem& p, Csr& K, std::vector<double>& r, const std::vector<double>& T) {
    for_boundary_rows(p, [](const Boundary& b) { return b.radiation(); },
        [&](const Boundary& b, i64 e, int i, i64 row) {
            if (!p.is_inner[size_t(row)]) return;
            const Element1d el = make_element1d(b.nen);
            auto tq = [&](int q) {
                double s = 0.0;
                for (int k = 0; k < b.nen; ++k) s += el.qN[size_t(k * el.nq + q)] * T[size_t(b.edges[size_t(e * b.nen + k)])];
                return s;
            };
            for (int j = 0; j < b.nen; ++j) {
                const i64 col = b.edges[size_t(e * b.nen + j)];
                if (col < row || !p.is_inner[size_t(col)]) continue;
                double integral = 0.0;
                for (int q = 0; q < el.nq; ++q)
                    integral += el.w[size_t(q)] * std::pow(tq(q), 3) * el.qN[size_t(i * el.nq + q)] *
                                el.qN[size_t(j * el.nq + q)] * edge_jacobian(p, b, el, e, q);
                const i64 k = find_entry(K, row, col);
                if (k >= 0) K.val[size_t(k)] -= 4.0 * STEFAN_BOLTZMANN * b.emissivity * integral;
            }
            double integral = 0.0;
            for (int q = 0; q < el.nq; ++q)
                integral += el.w[size_t(q)] * el.qN[size_t(i * el.nq + q)] * std::pow(tq(q), 4) * edge_jacobian(p, b, el, e, q);
            r[size_t(row)] -= STEFAN_BOLTZMANN * b.emissivity * integral;
        });
}

bool pure_neumann(const Problem& p) {   // init_problem_settings.hpp:18-21,43
    for (const Boundary& b : p.bnds) if (b.kind != BC_FLUX) return false;
    return true;
}
bool nonlinear_boundary(const Problem& p) {
    for (const Boundary& b : p.bnds) if (b.radiation()) return true;
    return false;
}

// The bordered matrix of a pure Neumann problem (conductivity_matrix_2d.hpp:39-104):
// each row ends with the column n holding int N_i over the node's elements
// (integral_condition), and row n holds its zero diagonal.
Csr bordered(const Problem& p, const Csr& A) {
    const i64 n = A.rows;
    Csr B;
    B.rows = B.cols = n + 1;
    B.rowptr.assign(size_t(n) + 2, 0);
    for (i64 r = 0; r < n; ++r) {
        for (i64 k = A.rowptr[size_t(r)]; k < A.rowptr[size_t(r) + 1]; ++k) {
            B.col.push_back(A.col[size_t(k)]); B.val.push_back(A.val[size_t(k)]);
        }
        double integral = 0.0;
        for (const i64 e : p.node_elements[size_t(r)]) {
            int i = 0;
            while (node_of(p, e, i) != r) ++i;
            double s = 0.0;
            for (int q = 0; q < p.el.nq; ++q) s += p.el.w[size_t(q)] * p.el.qN[size_t(i * p.el.nq + q)] * p.jac[size_t(e * p.el.nq + q)];
            integral += s;
        }
        B.col.push_back(n); B.val.push_back(integral);
        B.rowptr[size_t(r) + 1] = i64(B.col.size());
    }
    B.col.push_back(n); B.val.push_back(0.0);
    B.rowptr[size_t(n) + 1] = i64(B.col.size());
    return B;
}

// Symmetric product from upper storage, first stored entry of a row being the
// diagonal (independent_symmetric_matrix_vector_product.hpp:55-79; a thread
// scatters into a private column, then the columns are summed).
void sym_spmv(const Csr& A, const std::vector<double>& x, std::vector<double>& y) {
    const int T = omp_get_max_threads();
    const i64 n = A.rows;
    std::vector<double> priv(static_cast<size_t>(n) * size_t(T), 0.0);
    #pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num();
        double* py = &priv[size_t(n) * size_t(t)];
        #pragma omp for schedule(static)
        for (i64 r = 0; r < n; ++r) {
            const i64 k0 = A.rowptr[size_t(r)];
            py[r] += A.val[size_t(k0)] * x[size_t(A.col[size_t(k0)])];
            for (i64 k = k0 + 1; k < A.rowptr[size_t(r) + 1]; ++k) {
                py[r] += A.val[size_t(k)] * x[size_t(A.col[size_t(k)])];
                py[A.col[size_t(k)]] += A.val[size_t(k)] * x[size_t(r)];
            }
        }
    }
    y.assign(size_t(n), 0.0);
    for (int t = 0; t < T; ++t) for (i64 i = 0; i < n; ++i) y[size_t(i)] += priv[size_t(n) * size_t(t) + size_t(i)];
}

Eigen::SparseMatrix<double, Eigen::RowMajor, i64> to_eigen(const Csr& A) {
    Eigen::SparseMatrix<double, Eigen::RowMajor, i64> m(A.rows, A.cols);
    std::copy(A.rowptr.begin(), A.rowptr.end(), m.outerIndexPtr());
    m.data().resize(size_t(A.nnz()));
    std::copy(A.col.begin(), A.col.end(), m.innerIndexPtr());
    std::copy(A.val.begin(), A.val.end(), m.valuePtr());
    return m;
}

// Fixed-pattern IC(0) on the same Lin-More scaled and shifted matrix as the
// Eigen restatement: the factor the CUDA path computes.
struct IC0 {
    i64 n = 0; std::vector<i64> rp, ci; std::vector<double> v, scale; double shift = 0; int attempts = 0; bool ok = false;
    void compute(const Csr& A) {
        n = A.rows; rp = A.rowptr; ci = A.col; v = A.val;   // upper CSR == lower CSC
        scale.assign(size_t(n), 0.0);
        for (i64 r = 0; r < n; ++r)
            for (i64 k = rp[size_t(r)]; k < rp[size_t(r) + 1]; ++k) {
                scale[size_t(r)] += v[size_t(k)] * v[size_t(k)];
                if (ci[size_t(k)] != r) scale[size_t(ci[size_t(k)])] += v[size_t(k)] * v[size_t(k)];
            }
        for (double& s : scale) { const double root = std::sqrt(std::sqrt(s)); s = root > std::numeric_limits<double>::min() ? 1.0 / root : 1.0; }
        double mindiag = std::numeric_limits<double>::max();
        for (i64 r = 0; r < n; ++r) {
            for (i64 k = rp[size_t(r)]; k < rp[size_t(r) + 1]; ++k) v[size_t(k)] *= scale[size_t(ci[size_t(k)])] * scale[size_t(r)];
            mindiag = std::min(mindiag, v[size_t(rp[size_t(r)])]);
        }
        const std::vector<double> a = v;
        shift = mindiag <= 0 ? 1e-3 - mindiag : 0.0;
        for (attempts = 1; attempts <= 10; ++attempts) {
            if (factor(a)) { ok = true; return; }
            shift = std::max(1e-3, 2 * shift);
        }
    }
    // Up-looking row form of U = L^T: row i of U needs rows k < i with U(k,i) != 0.
    bool factor(const std::vector<double>& a) {
        v = a;
        for (i64 i = 0; i < n; ++i) v[size_t(rp[size_t(i)])] += shift;
        std::vector<std::vector<std::pair<i64, i64>>> colpos(static_cast<size_t>(n));   // col -> (row k, slot) of U
        for (i64 k = 0; k < n; ++k)
            for (i64 s = rp[size_t(k)] + 1; s < rp[size_t(k) + 1]; ++s) colpos[size_t(ci[size_t(s)])].push_back({k, s});
        for (i64 i = 0; i < n; ++i) {
            // subtract sum_k U(k,i) U(k,j) for j >= i in row i's pattern
            for (const auto& [k, s] : colpos[size_t(i)]) {
                const double uki = v[size_t(s)];
                i64 a1 = s, b1 = rp[size_t(i)];
                while (a1 < rp[size_t(k) + 1] && b1 < rp[size_t(i) + 1]) {
                    if (ci[size_t(a1)] < ci[size_t(b1)]) ++a1;
                    else if (ci[size_t(a1)] > ci[size_t(b1)]) ++b1;
                    else { v[size_t(b1)] -= uki * v[size_t(a1)]; ++a1; ++b1; }
                }
            }
            const double d = v[size_t(rp[size_t(i)])];
            if (!(d > 0)) return false;
            const double rd = std::sqrt(d);
            v[size_t(rp[size_t(i)])] = rd;
            for (i64 s = rp[size_t(i)] + 1; s < rp[size_t(i) + 1]; ++s) v[size_t(s)] /= rd;
        }
        return true;
    }
    void solve(const std::vector<double>& b, std::vector<double>& x) const {
        x.resize(size_t(n));
        for (i64 i = 0; i < n; ++i) x[size_t(i)] = scale[size_t(i)] * b[size_t(i)];
        for (i64 i = 0; i < n; ++i) {   // U^T y = x  (column sweep of U^T == row sweep of U)
            x[size_t(i)] /= v[size_t(rp[size_t(i)])];
            for (i64 s = rp[size_t(i)] + 1; s < rp[size_t(i) + 1]; ++s) x[size_t(ci[size_t(s)])] -= v[size_t(s)] * x[size_t(i)];
        }
        for (i64 i = n - 1; i >= 0; --i) {   // U z = y
            double s = x[size_t(i)];
            for (i64 k = rp[size_t(i)] + 1; k < rp[size_t(i) + 1]; ++k) s -= v[size_t(k)] * x[size_t(ci[size_t(k)])];
            x[size_t(i)] = s / v[size_t(rp[size_t(i)])];
        }
        for (i64 i = 0; i < n; ++i) x[size_t(i)] *= scale[size_t(i)];
    }
};

// conjugate_gradient::solve (conjugate_gradient.hpp:48-79).  stop_true_residual
// switches the stopping measure from the reference's sqrt(r.z)/|b| to |r|/|b|.
template<class Prec>
void cg(Problem& p, const Csr& A, const std::vector<double>& b, std::vector<double>& x, const Prec& prec,
        double tol, long maxit, bool stop_true_residual) {
    const size_t n = size_t(A.rows);
    if (x.size() != n) x.assign(n, 0.0);
    std::vector<double> r, z(n), pv, tmp;
    sym_spmv(A, x, r);
    for (size_t i = 0; i < n; ++i) r[i] = b[i] - r[i];
    prec(r, pv);
    auto dot = [n](const std::vector<double>& u, const std::vector<double>& w) { double s = 0; for (size_t i = 0; i < n; ++i) s += u[i] * w[i]; return s; };
    double rho = dot(r, pv);
    const double bnorm = std::sqrt(dot(b, b));
    auto measure = [&](double rho_) { return stop_true_residual ? std::sqrt(dot(r, r)) / bnorm : std::sqrt(rho_) / bnorm; };
    p.iterations = 0;
    p.residual = measure(rho);
    const double t_start = omp_get_wtime();
    p.record_iterations = -1;
    auto checkpoint = [&] {
        if (p.record_tol > 0.0 && p.record_iterations < 0 && p.residual <= p.record_tol) {
            p.record_iterations = p.iterations;
            p.timings["cg_to_record"] = omp_get_wtime() - t_start;
        }
    };
    checkpoint();
    while (p.iterations < maxit && p.residual > tol) {
        sym_spmv(A, pv, z);
        const double nu = rho / dot(pv, z);
        for (size_t i = 0; i < n; ++i) { x[i] += nu * pv[i]; r[i] -= nu * z[i]; }
        prec(r, z);
        const double rho_prev = rho;
        rho = dot(r, z);
        const double mu = rho / rho_prev;
        for (size_t i = 0; i < n; ++i) pv[i] = z[i] + mu * pv[i];
        ++p.iterations;
        p.residual = measure(rho);
        checkpoint();
    }
    sym_spmv(A, x, tmp);
    double s = 0; for (size_t i = 0; i < n; ++i) s += (b[i] - tmp[i]) * (b[i] - tmp[i]);
    p.true_residual = std::sqrt(s) / bnorm;
}

// y = A x over full (non-symmetric) rows
void full_spmv(const Csr& A, const std::vector<double>& x, std::vector<double>& y) {
    const i64 n = A.rows;
    y.assign(size_t(n), 0.0);
    #pragma omp parallel for schedule(static)
    for (i64 r = 0; r < n; ++r) {
        double s = 0.0;
        for (i64 k = A.rowptr[size_t(r)]; k < A.rowptr[size_t(r) + 1]; ++k) s += A.val[size_t(k)] * x[size_t(A.col[size_t(k)])];
        y[size_t(r)] = s;
    }
}

// Jacobi-preconditioned BiCGSTAB (van der Vorst 1992, right preconditioning by
// the diagonal, as Eigen's BiCGSTAB with its default diagonal preconditioner)
// from x = 0 for the reference's non-symmetric systems (a conductivity field
// with a nonlocal model, stationary_heat_equation_solver_2d.hpp:105-108);
// restarts with r0^ = r when (r0^, r) vanishes; stops on |b - A x| / |b|.
void bicgstab(Problem& p, const Csr& A, const std::vector<double>& b, std::vector<double>& x, double tol, long maxit) {
    const size_t n = size_t(A.rows);
    auto dot = [n](const std::vector<double>& u, const std::vector<double>& w) {
        double s = 0.0;
        for (size_t i = 0; i < n; ++i) s += u[i] * w[i];
        return s;
    };
    std::vector<double> dinv(n, 1.0);
    for (size_t r = 0; r < n; ++r) {
        const double* d = const_cast<Csr&>(A).find(i64(r), i64(r));
        if (d && *d != 0.0) dinv[r] = 1.0 / *d;
    }
    x.assign(n, 0.0);
    const double bnorm = std::sqrt(dot(b, b));
    p.iterations = 0;
    if (bnorm == 0.0) { p.residual = p.true_residual = 0.0; return; }
    std::vector<double> r = b, rhat = b, pv(n, 0.0), v(n, 0.0), y(n), sv(n), z(n), t(n);
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    p.residual = 1.0;
    while (p.iterations < maxit && p.residual > tol) {
        const double rho_new = dot(rhat, r);
        if (rho_new == 0.0) {   // breakdown: restart the shadow residual
            rhat = r;
            rho = alpha = omega = 1.0;
            std::fill(pv.begin(), pv.end(), 0.0);
            std::fill(v.begin(), v.end(), 0.0);
            continue;
        }
        const double beta = (rho_new / rho) * (alpha / omega);
        rho = rho_new;
        for (size_t i = 0; i < n; ++i) pv[i] = r[i] + beta * (pv[i] - omega * v[i]);
        for (size_t i = 0; i < n; ++i) y[i] = dinv[i] * pv[i];
        full_spmv(A, y, v);
        alpha = rho / dot(rhat, v);
        for (size_t i = 0; i < n; ++i) sv[i] = r[i] - alpha * v[i];
        for (size_t i = 0; i < n; ++i) z[i] = dinv[i] * sv[i];
        full_spmv(A, z, t);
        const double tt = dot(t, t);
        omega = tt > 0.0 ? dot(t, sv) / tt : 0.0;
        for (size_t i = 0; i < n; ++i) {
            x[i] += alpha * y[i] + omega * z[i];
            r[i] = sv[i] - omega * t[i];
        }
        ++p.iterations;
        p.residual = std::sqrt(dot(r, r)) / bnorm;
    }
    full_spmv(A, x, t);
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += (b[i] - t[i]) * (b[i] - t[i]);
    p.true_residual = std::sqrt(s) / bnorm;
}

double now() { return omp_get_wtime(); }

} // namespace

extern "C" {

void* orc_create(int elem_type, i64 n_nodes, const double* nodes, i64 n_elems, const i64* elems) {
    if (elem_type != ORC_BILINEAR && elem_type != ORC_SERENDIPITY) return nullptr;
    auto* p = new Problem;
    p->el = make_element2d(elem_type);
    p->n_nodes = n_nodes; p->n_elems = n_elems;
    p->nodes.assign(nodes, nodes + 2 * n_nodes);
    p->elems.assign(elems, elems + n_elems * p->el.nen);
    const double t0 = now();
    mesh_init(*p);
    p->timings["mesh"] = now() - t0;
    p->is_inner.assign(size_t(n_nodes), 1);
    return p;
}

void orc_destroy(void* h) { delete static_cast<Problem*>(h); }

void orc_set_model(void* h, int influence, int n, int pp, double q, double r1, double r2, double local_weight,
                   int cond_kind, double c0, double c1, double c2) {
    auto& p = *static_cast<Problem*>(h);
    p.influence = influence; p.inf_n = n; p.inf_p = pp; p.inf_q = q; p.r[0] = r1; p.r[1] = r2; p.p1 = local_weight;
    p.cond_kind = cond_kind; p.cond[0] = c0; p.cond[1] = c1; p.cond[2] = c2;
    init_norm(p);
}

void orc_set_conductivity_field(void* h, const double* values) {   // isotropic, per quadrature point [e][q]
    auto& p = *static_cast<Problem*>(h);
    p.cond_q.assign(values, values + p.n_elems * p.el.nq);
    p.symmetric = !nonlocal_model(p);   // problem_settings::is_symmetric (problem_settings.hpp:32-34)
}

void orc_set_capacity(void* h, double capacity, double density) {
    auto& p = *static_cast<Problem*>(h); p.capacity = capacity; p.density = density;
}

void orc_add_boundary(void* h, int kind, i64 n_edges, int nen, const i64* edges, double value) {
    auto& p = *static_cast<Problem*>(h);
    p.bnds.push_back({kind, nen, std::vector<i64>(edges, edges + n_edges * nen), value, {}});
}

// flux-type groups: the second-kind flux is operator() of the condition
// (flux q, convection alpha T_a, radiation 0, combined q + alpha T_a)
void orc_add_flux_boundary(void* h, int kind, i64 n_edges, int nen, const i64* edges, double flux,
                           double heat_transfer, double ambient, double emissivity) {
    auto& p = *static_cast<Problem*>(h);
    Boundary b{kind, nen, std::vector<i64>(edges, edges + n_edges * nen), 0.0, {}};
    b.value = kind == BC_FLUX ? flux : kind == BC_CONVECTION ? heat_transfer * ambient :
              kind == BC_COMBINED ? flux + heat_transfer * ambient : 0.0;
    b.heat_transfer = (kind == BC_CONVECTION || kind == BC_COMBINED) ? heat_transfer : 0.0;
    b.emissivity = (kind == BC_RADIATION || kind == BC_COMBINED) ? emissivity : 0.0;
    p.bnds.push_back(std::move(b));
}

void orc_set_stationary(void* h, double tolerance, long max_iterations, double energy, const double* initial) {
    auto& p = *static_cast<Problem*>(h);
    p.nl_tolerance = tolerance; p.nl_max_iterations = max_iterations; p.energy = energy;
    if (initial) p.initial.assign(initial, initial + p.n_nodes);
    else p.initial.clear();
}

void orc_set_source(void* h, double value) { static_cast<Problem*>(h)->source = value; }

void orc_set_source_field(void* h, const double* values) {   // [e][q]
    auto& p = *static_cast<Problem*>(h);
    p.source_q.assign(values, values + p.n_elems * p.el.nq);
}

void orc_set_dirichlet_values(void* h, const double* values) {   // [node], used on Dirichlet nodes
    auto& p = *static_cast<Problem*>(h);
    p.dirichlet_override.assign(values, values + p.n_nodes);
}

void orc_find_neighbours(void* h, int strategy) {
    auto& p = *static_cast<Problem*>(h);
    const double t0 = now();
    if (nonlocal_model(p)) find_neighbours(p, strategy);
    else { p.noff.assign(size_t(p.n_elems) + 1, 0); p.nlist.clear(); }
    p.timings["neighbours"] = now() - t0;
}

// stationary_heat_equation_solver_2d steps up to the right-hand side
// (stationary_heat_equation_solver_2d.hpp:52-84): BC vectors, full assembly,
// first-kind condition on the right-hand side.
void orc_assemble_stationary(void* h) {
    auto& p = *static_cast<Problem*>(h);
    boundary_vectors(p);
    const double t0 = now();
    assemble(p, false, p.symmetric, p.K_inner, p.K_bound, integrate_local, p.p1, 1.0 - p.p1);
    convection_condition(p, p.K_inner);   // stationary_heat_equation_solver_2d.hpp:76
    p.timings["assembly"] = now() - t0;
    p.rhs = p.rhs_init;
    apply_first_kind(p, p.K_bound, p.rhs);
}

// local part p1*K_local used for the preconditioner (stationary_heat_equation_solver_2d.hpp:91-93)
void orc_assemble_local(void* h) {
    auto& p = *static_cast<Problem*>(h);
    Csr unused;
    const double t0 = now();
    assemble(p, true, p.symmetric, p.K_local, unused, integrate_local, p.p1, 0.0);
    p.timings["assembly_local"] = now() - t0;
}

// ILLT-preconditioned CG (stationary_heat_equation_solver_2d.hpp:94-102).
// variant 0: Eigen-style Lin-More ICF (reference); 1: fixed-pattern IC(0); 2: identity.
// Pure Neumann problems (stationary_heat_equation_solver_2d.hpp:29-44, 52-103 with
// is_neumann): the flux balance check, then CG with the ILLT of the bordered
// local matrix on the bordered system [K b; b^T 0] [T; lambda] = [f; energy].
// Returns -2 for an unbalanced problem.
static int solve_neumann(Problem& p, double tol, long maxit, bool stop_true_residual) {
    double s = 0.0;
    for (const double v : p.rhs) s += v;
    if (std::abs(s) > 1e-10) return -2;
    const Csr K = bordered(p, p.K_inner), Kl = bordered(p, p.K_local);
    std::vector<double> f = p.rhs, x;
    f.push_back(p.energy);
    const auto E = to_eigen(Kl);
    Eigen::IncompleteCholesky<double, Eigen::Upper, Eigen::NaturalOrdering<i64>> ilt(E);
    p.ilt_ok = ilt.info() == Eigen::Success;
    if (p.ilt_ok)
        cg(p, K, f, x, [&](const std::vector<double>& r, std::vector<double>& z) {
            Eigen::Matrix<double, Eigen::Dynamic, 1> rr(long(r.size()));
            std::copy(r.begin(), r.end(), rr.data());
            const auto zz = ilt.solve(rr);
            z.assign(zz.begin(), zz.end());
        }, tol, maxit, stop_true_residual);
    else
        cg(p, K, f, x, [](const std::vector<double>& r, std::vector<double>& z) { z = r; }, tol, maxit, stop_true_residual);
    p.solution.assign(x.begin(), x.begin() + p.n_nodes);
    return p.ilt_ok;
}

// The radiation loop (stationary_heat_equation_solver_2d.hpp:66-116): from the
// initial temperature, K_T dT = K T_prev - r_rad - f with K_T = K - 4 sigma eps
// int T^3 N_i N_j, solved by CG with the diagonal preconditioner to machine
// precision (Eigen::ConjugateGradient's defaults), T = T_prev - dT, until
// max_iterations or until |T - T_prev| / |T| or |residual| is at most the tolerance.
static int solve_radiation(Problem& p) {
    const size_t n = size_t(p.n_nodes);
    std::vector<double> curr = p.initial.empty() ? std::vector<double>(n, 0.0) : p.initial, prev = curr;
    double difference = 1.0, norm = 1.0;
    long it = 0;
    while (it < p.nl_max_iterations && p.nl_tolerance < difference && p.nl_tolerance < norm) {
        std::swap(curr, prev);
        Csr K = p.K_inner;
        std::vector<double> residual, rad(n, 0.0), dx;
        sym_spmv(K, prev, residual);
        radiation_condition(p, K, rad, prev);
        for (size_t i = 0; i < n; ++i) residual[i] -= rad[i] + p.rhs[i];
        std::vector<double> inv(n);
        for (size_t r = 0; r < n; ++r) {
            const double d = K.val[size_t(K.rowptr[r])];
            inv[r] = d != 0.0 ? 1.0 / d : 1.0;
        }
        cg(p, K, residual, dx, [&](const std::vector<double>& r, std::vector<double>& z) {
            z.resize(r.size());
            for (size_t i = 0; i < r.size(); ++i) z[i] = inv[i] * r[i];
        }, std::numeric_limits<double>::epsilon(), long(2 * n), true);
        double rr = 0.0, dd = 0.0, tt = 0.0;
        for (size_t i = 0; i < n; ++i) {
            curr[i] = prev[i] - dx[i];
            rr += residual[i] * residual[i];
            dd += (curr[i] - prev[i]) * (curr[i] - prev[i]);
            tt += curr[i] * curr[i];
        }
        ++it;
        norm = std::sqrt(rr);
        difference = std::sqrt(dd) / (tt != 0.0 ? std::sqrt(tt) : 1.0);
    }
    p.nonlinear_iterations = it;
    p.solution = curr;
    return 1;
}

int orc_solve(void* h, int variant, double tol, long maxit, int stop_true_residual) {
    auto& p = *static_cast<Problem*>(h);
    if (nonlinear_boundary(p)) return solve_radiation(p);
    if (pure_neumann(p)) return solve_neumann(p, tol, maxit, stop_true_residual);
    double t0 = now();
    std::vector<double> x;
    if (!p.symmetric) {   // full storage: BiCGSTAB, as the reference
        bicgstab(p, p.K_inner, p.rhs, x, tol, maxit);
        p.timings["cg"] = now() - t0;
        p.solution = x;
        return 1;
    }
    if (variant == 0) {
        const auto Kl = to_eigen(p.K_local);
        Eigen::IncompleteCholesky<double, Eigen::Upper, Eigen::NaturalOrdering<i64>> ilt(Kl);
        p.ilt_ok = ilt.info() == Eigen::Success; p.ilt_attempts = ilt.attempts(); p.ilt_shift = ilt.shift();
        p.timings["ilt"] = now() - t0;
        t0 = now();
        if (p.ilt_ok) {
            p.L_colptr.assign(ilt.colptr().begin(), ilt.colptr().end());
            p.L_rowidx.assign(ilt.rowidx().begin(), ilt.rowidx().end());
            p.L_val = ilt.values(); p.L_scale = ilt.scale();
            cg(p, p.K_inner, p.rhs, x, [&](const std::vector<double>& r, std::vector<double>& z) {
                Eigen::Matrix<double, Eigen::Dynamic, 1> rr(long(r.size()));
                std::copy(r.begin(), r.end(), rr.data());
                const auto zz = ilt.solve(rr);
                z.assign(zz.begin(), zz.end());
            }, tol, maxit, stop_true_residual);
        } else
            cg(p, p.K_inner, p.rhs, x, [](const std::vector<double>& r, std::vector<double>& z) { z = r; }, tol, maxit, stop_true_residual);
    } else if (variant == 1) {
        IC0 ic; ic.compute(p.K_local);
        p.ilt_ok = ic.ok; p.ilt_attempts = ic.attempts; p.ilt_shift = ic.shift;
        p.L_colptr = ic.rp; p.L_rowidx = ic.ci; p.L_val = ic.v; p.L_scale = ic.scale;
        p.timings["ilt"] = now() - t0;
        t0 = now();
        if (ic.ok)
            cg(p, p.K_inner, p.rhs, x, [&](const std::vector<double>& r, std::vector<double>& z) { ic.solve(r, z); }, tol, maxit, stop_true_residual);
        else
            cg(p, p.K_inner, p.rhs, x, [](const std::vector<double>& r, std::vector<double>& z) { z = r; }, tol, maxit, stop_true_residual);
    } else {
        cg(p, p.K_inner, p.rhs, x, [](const std::vector<double>& r, std::vector<double>& z) { z = r; }, tol, maxit, stop_true_residual);
    }
    p.timings["cg"] = now() - t0;
    p.solution = x;
    return p.ilt_ok;
}

// heat_equation_solution_2d::calc_flux (heat_equation_solution_2d.hpp:99-137):
// -Lambda grad T at the quadrature points (gradient_in_qnodes,
// mesh_2d_utils.hpp:40-60; local_flux_in_qnodes, :72-96), the nonlocal mix
// p1 local + (1 - p1) sum_eNL sum_qNL w |J| phi local, and the nodal values of
// qnodes_to_nodes (mesh_2d_utils.hpp:82-101) with mesh_2d::area (mesh_2d.hpp:225-234)
// and the nearest Gauss point of each local node (element_2d_integrate.hpp:87-105).
void orc_calc_flux(void* h, const double* T, double* fx_out, double* fy_out) {
    auto& p = *static_cast<Problem*>(h);
    const int nen = p.el.nen, nq = p.el.nq;
    const size_t E = size_t(p.n_elems);
    std::vector<double> lx(E * size_t(nq)), ly(E * size_t(nq));
    for (size_t e = 0; e < E; ++e)
        for (int q = 0; q < nq; ++q) {
            const size_t s = e * size_t(nq) + size_t(q);
            double gx = 0, gy = 0;
            for (int i = 0; i < nen; ++i) {
                const double v = T[node_of(p, i64(e), i)];
                const double* d = &p.deriv[2 * ((e * size_t(nen) + size_t(i)) * size_t(nq) + size_t(q))];
                gx += v * d[0];
                gy += v * d[1];
            }
            gx /= p.jac[s];
            gy /= p.jac[s];
            if (p.cond_kind == COND_ISO) {
                const double c = p.cond_q.empty() ? p.cond[0] : p.cond_q[s];
                lx[s] = gx * -c; ly[s] = gy * -c;
            } else if (p.cond_kind == COND_ORTHO) {
                lx[s] = gx * -p.cond[0]; ly[s] = gy * -p.cond[1];
            } else {
                lx[s] = -p.cond[0] * gx - p.cond[2] * gy;
                ly[s] = -p.cond[2] * gx - p.cond[1] * gy;
            }
        }
    std::vector<double> fx = lx, fy = ly;
    if (nonlocal_model(p)) {
        const double nw = 1.0 - p.p1;
#pragma omp parallel for schedule(dynamic)
        for (i64 eL = 0; eL < i64(E); ++eL)
            for (int qL = 0; qL < nq; ++qL) {
                const size_t sL = size_t(eL) * size_t(nq) + size_t(qL);
                const vec2 xL{p.qcoord[2 * sL], p.qcoord[2 * sL + 1]};
                double ngx = 0, ngy = 0;
                for (i64 k = p.noff[size_t(eL)]; k < p.noff[size_t(eL) + 1]; ++k) {
                    const size_t eNL = size_t(p.nlist[size_t(k)]);
                    for (int qN = 0; qN < nq; ++qN) {
                        const size_t s = eNL * size_t(nq) + size_t(qN);
                        const double iw = p.el.w[size_t(qN)] * p.jac[s] *
                                          influence(p, xL, vec2{p.qcoord[2 * s], p.qcoord[2 * s + 1]});
                        ngx += iw * lx[s];
                        ngy += iw * ly[s];
                    }
                }
                ngx *= nw; ngy *= nw;
                fx[sL] = lx[sL] * p.p1 + ngx;
                fy[sL] = ly[sL] * p.p1 + ngy;
            }
    }
    // nearest Gauss point of each local node on [-1,1]^2
    const Gauss g = gauss(p.el.type == ORC_BILINEAR ? 2 : 3);
    const int n1 = int(g.x.size());
    const double bx[4] = {-1, 1, 1, -1}, by[4] = {-1, -1, 1, 1};
    const double sx[8] = {-1, 0, 1, 1, 1, 0, -1, -1}, sy[8] = {-1, -1, -1, 0, 1, 1, 1, 0};
    std::vector<int> nearest(size_t(nen), 0);
    for (int i = 0; i < nen; ++i) {
        const double nx = nen == 4 ? bx[i] : sx[i], ny = nen == 4 ? by[i] : sy[i];
        double best = std::numeric_limits<double>::max();
        for (int a = 0; a < n1; ++a)
            for (int c = 0; c < n1; ++c)
                if (const double d = std::sqrt((nx - g.x[size_t(a)]) * (nx - g.x[size_t(a)]) +
                                               (ny - g.x[size_t(c)]) * (ny - g.x[size_t(c)])); best > d) {
                    best = d;
                    nearest[size_t(i)] = a * n1 + c;
                }
    }
    std::vector<double> area(E, 0.0);
    for (size_t e = 0; e < E; ++e)
        for (int q = 0; q < nq; ++q) {
            const double factor = p.el.w[size_t(q)] * p.jac[e * size_t(nq) + size_t(q)];
            for (int i = 0; i < nen; ++i) area[e] += factor * p.el.qN[size_t(i * nq + q)];
        }
    for (i64 node = 0; node < p.n_nodes; ++node) {
        double ax = 0, ay = 0, s = 0;
        for (const i64 e : p.node_elements[size_t(node)]) {
            int i = 0;
            while (node_of(p, e, i) != node) ++i;
            const size_t q = size_t(e) * size_t(nq) + size_t(nearest[size_t(i)]);
            ax += area[size_t(e)] * fx[q];
            ay += area[size_t(e)] * fy[q];
            s += area[size_t(e)];
        }
        fx_out[node] = ax / s;
        fy_out[node] = ay / s;
    }
}

// nonstationary_heat_equation_solver_2d::compute + calc_step
// (nonstationary_heat_equation_solver_2d.hpp:63-106): K <- dt*K + C with unit
// Dirichlet diagonal, CG with the identity preconditioner and x0 = T_prev,
// Dirichlet value amp*sin(omega*t) on the temperature groups.
void orc_nonstationary(void* h, double dt, long steps, double omega, double tol, long maxit) {
    auto& p = *static_cast<Problem*>(h);
    boundary_vectors(p);
    assemble(p, false, true, p.K_inner, p.K_bound, integrate_local, p.p1, 1.0 - p.p1);
    Csr Cb;
    const double rc = p.capacity * p.density;
    assemble(p, true, true, p.C_inner, Cb,
             [](const Problem& pr, i64 e, int i, int j) { return integrate_capacity(pr, e, i, j); }, rc, 0.0);
    for (double& v : p.K_inner.val) v *= dt;
    for (double& v : p.K_bound.val) v *= dt;
    // K_inner += C_inner (capacity pattern is a subset of the nonlocal pattern)
    for (i64 r = 0; r < p.n_nodes; ++r)
        for (i64 k = p.C_inner.rowptr[size_t(r)]; k < p.C_inner.rowptr[size_t(r) + 1]; ++k)
            *p.K_inner.find(r, p.C_inner.col[size_t(k)]) += p.C_inner.val[size_t(k)];
    for (i64 r = 0; r < p.n_nodes; ++r) if (!p.is_inner[size_t(r)]) p.K_inner.val[size_t(p.K_inner.rowptr[size_t(r)])] = 1.0;
    std::vector<double> T(static_cast<size_t>(p.n_nodes), 0.0), f, CT;
    p.history.clear();
    long total_it = 0;
    const double t_steps = now();
    for (long s = 1; s <= steps; ++s) {
        const double value = std::sin(omega * double(s) * dt);
        f = p.rhs_init;
        for (double& v : f) v *= dt;
        sym_spmv(p.C_inner, T, CT);
        for (size_t i = 0; i < f.size(); ++i) f[i] += CT[i];
        for (i64 i = 0; i < p.n_nodes; ++i) p.x_dirichlet[size_t(i)] = p.is_inner[size_t(i)] ? 0.0 : value;
        apply_first_kind(p, p.K_bound, f);
        std::vector<double> x = T;
        cg(p, p.K_inner, f, x, [](const std::vector<double>& r, std::vector<double>& z) { z = r; }, tol, maxit, false);
        total_it += p.iterations;
        T = x;
        p.history.insert(p.history.end(), T.begin(), T.end());
    }
    p.timings["steps"] = now() - t_steps;
    p.iterations = total_it;
    p.solution = T;
}

// ------------------------------------------------------------- accessors
i64 orc_size(void* h, const char* name) {
    auto& p = *static_cast<Problem*>(h);
    const std::string s{name};
    if (s == "qcoords") return i64(p.qcoord.size());
    if (s == "jacobians") return i64(p.jac.size());
    if (s == "derivatives") return i64(p.deriv.size());
    if (s == "centres") return i64(p.centres.size());
    if (s == "neigh_offsets") return i64(p.noff.size());
    if (s == "neigh_list") return i64(p.nlist.size());
    if (s == "is_inner") return i64(p.is_inner.size());
    if (s == "rhs") return i64(p.rhs.size());
    if (s == "rhs_init") return i64(p.rhs_init.size());
    if (s == "solution") return i64(p.solution.size());
    if (s == "history") return i64(p.history.size());
    if (s == "basis_qN" || s == "basis_qNxi" || s == "basis_qNeta") return i64(p.el.qN.size());
    if (s == "basis_weights") return i64(p.el.w.size());
    if (s == "basis_centre") return i64(p.el.centre.size());
    const auto csr = [&](const std::string& pre, const Csr& A) -> i64 {
        if (s == pre + "_rowptr") return i64(A.rowptr.size());
        if (s == pre + "_col" || s == pre + "_val") return i64(A.col.size());
        return -1;
    };
    for (const auto& [pre, A] : {std::pair<std::string, const Csr*>{"K_inner", &p.K_inner}, {"K_bound", &p.K_bound},
                                 {"K_local", &p.K_local}, {"C_inner", &p.C_inner}})
        if (const i64 k = csr(pre, *A); k >= 0) return k;
    if (s == "L_rowptr") return i64(p.L_colptr.size());
    if (s == "L_col" || s == "L_val") return i64(p.L_rowidx.size());
    if (s == "L_scale") return i64(p.L_scale.size());
    return -1;
}

// mesh::utils::cuthill_mckee (cuthill_mckee.hpp:107-171).  The node graph of
// init_graph: mesh_run over the nodes (mesh_2d_utils.hpp:13-37), local
// theory (only_local or a local model: the nodes of each element of the node)
// or nonlocal (the nodes of each neighbour of each element of the node), each
// other node once in order of first meeting (neighbour_checker).  Then
// calculate_permutation from the first node of smallest degree: layers in a
// std::unordered_set, unvisited neighbours numbered in std::multimap order of
// degree.  reverse returns the inverse permutation (reverse_permutation).
// Returns -1 when the graph is not connected (the reference loops forever).
int orc_cuthill_mckee(void* h, int only_local, int reverse, i64* out) {
    auto& p = *static_cast<Problem*>(h);
    const bool local = only_local || !nonlocal_model(p);
    const i64 n = p.n_nodes;
    const int nen = p.el.nen;
    const size_t count = size_t(n);
    std::vector<std::vector<i64>> graph(count);
#pragma omp parallel
    {
        std::vector<bool> included(count, false);
#pragma omp for schedule(dynamic)
        for (i64 node = 0; node < n; ++node) {
            auto& adj = graph[size_t(node)];
            auto check = [&](const i64 neighbour) {
                if (node != neighbour && !included[size_t(neighbour)]) {
                    included[size_t(neighbour)] = true;
                    adj.push_back(neighbour);
                }
            };
            for (const i64 eL : p.node_elements[size_t(node)]) {
                if (local) {
                    for (int j = 0; j < nen; ++j) check(p.elems[size_t(eL * nen + j)]);
                } else {
                    for (i64 k = p.noff[size_t(eL)]; k < p.noff[size_t(eL) + 1]; ++k) {
                        const i64 eNL = p.nlist[size_t(k)];
                        for (int j = 0; j < nen; ++j) check(p.elems[size_t(eNL * nen + j)]);
                    }
                }
            }
            for (const i64 v : adj) included[size_t(v)] = false;
        }
    }
    i64 init = 0, min_count = std::numeric_limits<i64>::max();
    for (i64 node = 0; node < n; ++node)
        if (const i64 c = i64(graph[size_t(node)].size()); c < min_count) { init = node; min_count = c; }
    std::vector<i64> permutation(size_t(n), -1);
    i64 curr_index = 0;
    permutation[size_t(init)] = curr_index++;
    std::unordered_set<i64> curr_layer{init}, next_layer;
    while (curr_index < n) {
        if (curr_layer.empty()) return -1;
        next_layer.clear();
        for (const i64 node : curr_layer) {
            std::multimap<i64, i64> neighbours;
            for (const i64 nb : graph[size_t(node)])
                if (permutation[size_t(nb)] == -1) neighbours.emplace(i64(graph[size_t(nb)].size()), nb);
            for (const auto& [count, nb] : neighbours) {
                next_layer.emplace(nb);
                permutation[size_t(nb)] = curr_index++;
            }
        }
        std::swap(curr_layer, next_layer);
    }
    if (reverse)
        for (i64 i = 0; i < n; ++i) out[size_t(permutation[size_t(i)])] = i;
    else
        std::copy(permutation.begin(), permutation.end(), out);
    return 0;
}

int orc_get_f64(void* h, const char* name, double* out) {
    auto& p = *static_cast<Problem*>(h);
    const std::string s{name};
    const std::vector<double>* v = nullptr;
    if (s == "qcoords") v = &p.qcoord; else if (s == "jacobians") v = &p.jac; else if (s == "derivatives") v = &p.deriv;
    else if (s == "centres") v = &p.centres; else if (s == "rhs") v = &p.rhs; else if (s == "rhs_init") v = &p.rhs_init;
    else if (s == "solution") v = &p.solution; else if (s == "history") v = &p.history;
    else if (s == "basis_qN") v = &p.el.qN; else if (s == "basis_qNxi") v = &p.el.qNxi; else if (s == "basis_qNeta") v = &p.el.qNeta;
    else if (s == "basis_weights") v = &p.el.w; else if (s == "basis_centre") v = &p.el.centre;
    else if (s == "K_inner_val") v = &p.K_inner.val; else if (s == "K_bound_val") v = &p.K_bound.val;
    else if (s == "K_local_val") v = &p.K_local.val; else if (s == "C_inner_val") v = &p.C_inner.val;
    else if (s == "L_val") v = &p.L_val; else if (s == "L_scale") v = &p.L_scale;
    if (!v) return -1;
    std::memcpy(out, v->data(), v->size() * sizeof(double));
    return 0;
}

int orc_get_i64(void* h, const char* name, i64* out) {
    auto& p = *static_cast<Problem*>(h);
    const std::string s{name};
    const std::vector<i64>* v = nullptr;
    if (s == "neigh_offsets") v = &p.noff; else if (s == "neigh_list") v = &p.nlist;
    else if (s == "K_inner_rowptr") v = &p.K_inner.rowptr; else if (s == "K_inner_col") v = &p.K_inner.col;
    else if (s == "K_bound_rowptr") v = &p.K_bound.rowptr; else if (s == "K_bound_col") v = &p.K_bound.col;
    else if (s == "K_local_rowptr") v = &p.K_local.rowptr; else if (s == "K_local_col") v = &p.K_local.col;
    else if (s == "C_inner_rowptr") v = &p.C_inner.rowptr; else if (s == "C_inner_col") v = &p.C_inner.col;
    else if (s == "L_rowptr") v = &p.L_colptr; else if (s == "L_col") v = &p.L_rowidx;
    if (s == "is_inner") { for (size_t i = 0; i < p.is_inner.size(); ++i) out[i] = p.is_inner[i]; return 0; }
    if (!v) return -1;
    std::memcpy(out, v->data(), v->size() * sizeof(i64));
    return 0;
}

double orc_scalar(void* h, const char* name) {
    auto& p = *static_cast<Problem*>(h);
    const std::string s{name};
    if (s == "iterations") return double(p.iterations);
    if (s == "residual") return p.residual;
    if (s == "true_residual") return p.true_residual;
    if (s == "search_radius") return p.search_r[0];
    if (s == "search_radius2") return p.search_r[1];
    if (s == "ilt_ok") return p.ilt_ok;
    if (s == "ilt_attempts") return p.ilt_attempts;
    if (s == "ilt_shift") return p.ilt_shift;
    if (s == "threads") return omp_get_max_threads();
    if (s == "nonlinear_iterations") return double(p.nonlinear_iterations);
    if (s == "record_iterations") return double(p.record_iterations);
    const auto it = p.timings.find(s);
    return it == p.timings.end() ? -1.0 : it->second;
}

// ------------------------------------------------------------------ 1D
// stationary_heat_equation_solver_1d (stationary_heat_equation_solver_1d.hpp:43-122)
// for one segment [0, length], quadratic (order 2, Gauss-3) or linear
// (order 1, Gauss-2) Lagrange elements, T(0) = t_left, flux q_right at the
// right end, source sin(pi x) when sin_source != 0, influence kind
// 0 = polynomial_1d<2,1> (bell), 1 = polynomial_1d<1,1>, 2 = normal, 3 = constant
// (influence_functions_1d.hpp:10-75).  Mesh: mesh_1d.hpp:119-300; assembly:
// thermal_conductivity_assembler.hpp:64-125 and assebmler_base.hpp:112-155;
// direct LDL^T solve (the restated SimplicialCholesky).
int orc_stationary_1d(i64 elements, int order, double length, double r, double p1, int kind, double conductivity,
                      double t_left, double q_right, int sin_source, double* temperature_out) {
    const int nen = order + 1;
    const Gauss g = gauss(order == 2 ? 3 : 2);
    const int nq = int(g.x.size());
    std::vector<double> qN(static_cast<size_t>(nen * nq)), qNxi(qN.size()), w(static_cast<size_t>(nq));
    for (int q = 0; q < nq; ++q) w[size_t(q)] = g.w[size_t(q)] * 1.0;
    for (int i = 0; i < nen; ++i)
        for (int q = 0; q < nq; ++q) {
            const double x = -1.0 + (g.x[size_t(q)] - (-1.0)) * 1.0;
            double N, Nx;
            if (order == 1) { N = i == 0 ? (1 - x) / 2 : (1 + x) / 2; Nx = i == 0 ? -0.5 : 0.5; }
            else if (i == 0) { N = x * (x - 1) / 2; Nx = (2 * x - 1) / 2; }
            else if (i == 1) { N = (1 - x) * (1 + x); Nx = -2 * x; }
            else { N = x * (x + 1) / 2; Nx = (2 * x + 1) / 2; }
            qN[size_t(i * nq + q)] = N; qNxi[size_t(i * nq + q)] = Nx;
        }
    const i64 nodes = elements * order + 1;
    const double h = length / double(elements), jac = h / 2.0;
    const i64 nb = i64(std::round(r / h));
    auto qcoord = [&](i64 e, int q) { return h * double(e) + (g.x[size_t(q)] - (-1.0)) * jac; };
    auto infl = [&](double x, double y) {
        const double d = std::abs(x - y);
        if (kind == 0) { const double nrm = 2.0 / (2 * r * std::beta(0.5, 2.0)); return d < r ? nrm * (1 - (d / r) * (d / r)) : 0.0; }
        if (kind == 1) { const double nrm = 1.0 / (2 * r * std::beta(1.0, 2.0)); return d < r ? nrm * (1 - d / r) : 0.0; }
        if (kind == 2) { const double nrm = 1 / (r * std::sqrt(2 * std::numbers::pi)); return nrm * std::exp((-0.5 / (r * r)) * ((x - y) * (x - y))); }
        return d < r ? 0.5 / r : 0.0;
    };
    const bool nonlocal = p1 < 0.999;
    // dense upper band, bandwidth (nb+1)*order
    const i64 bw = nonlocal ? (nb + 1) * order : order;
    std::vector<double> band(static_cast<size_t>(nodes * (bw + 1)), 0.0), bound_row0;
    std::map<i64, double> bound0;
    auto add = [&](i64 row, i64 col, double v) {
        if (row == 0 || col == 0) { if (row == 0 && col != 0) bound0[col] += v; return; }
        if (row <= col) band[size_t(row * (bw + 1) + (col - row))] += v;
    };
    for (i64 e = 0; e < elements; ++e) {
        const i64 lo = std::max<i64>(0, e - nb), hi = std::min<i64>(elements, e + nb + 1);
        for (int i = 0; i < nen; ++i) {
            const i64 row = e * order + i;
            if (nonlocal)
                for (i64 f = lo; f < hi; ++f)
                    for (int j = 0; j < nen; ++j) {
                        double integral = 0.0;
                        for (int qL = 0; qL < nq; ++qL) {
                            double inner = 0.0;
                            for (int qNL = 0; qNL < nq; ++qNL)
                                inner += infl(qcoord(e, qL), qcoord(f, qNL)) * conductivity * w[size_t(qNL)] * qNxi[size_t(j * nq + qNL)];
                            integral += w[size_t(qL)] * qNxi[size_t(i * nq + qL)] * inner;
                        }
                        add(row, f * order + j, (1 - p1) * integral);
                    }
            for (int j = 0; j < nen; ++j) {
                double integral = 0.0;
                for (int q = 0; q < nq; ++q) integral += conductivity * w[size_t(q)] * qNxi[size_t(i * nq + q)] * qNxi[size_t(j * nq + q)];
                add(row, e * order + j, p1 * (integral / jac));
            }
        }
    }
    band[0] = 1.0;   // Dirichlet row: unit diagonal
    std::vector<double> f(static_cast<size_t>(nodes), 0.0);
    f[size_t(nodes - 1)] += q_right;   // boundary_condition_second_kind_1d
    if (sin_source)
        for (i64 e = 0; e < elements; ++e)
            for (int i = 0; i < nen; ++i) {
                double integral = 0.0;
                for (int q = 0; q < nq; ++q) integral += w[size_t(q)] * qN[size_t(i * nq + q)] * std::sin(std::numbers::pi * qcoord(e, q));
                f[size_t(e * order + i)] += integral * jac;
            }
    for (const auto& [col, v] : bound0) f[size_t(col)] -= v * t_left;   // K_bound column of node 0 (symmetric)
    f[0] = t_left;
    // band LDL^T
    Eigen::SparseMatrix<double, Eigen::RowMajor, i64> K(nodes, nodes);
    std::vector<i64> cols; std::vector<double> vals;
    for (i64 rr = 0; rr < nodes; ++rr) {
        for (i64 c = rr; c <= std::min(nodes - 1, rr + bw); ++c) {
            const double v = band[size_t(rr * (bw + 1) + (c - rr))];
            if (c == rr || v != 0.0) { cols.push_back(c); vals.push_back(v); }
        }
        K.outerIndexPtr()[rr + 1] = i64(cols.size());
    }
    K.data().resize(cols.size());
    std::copy(cols.begin(), cols.end(), K.innerIndexPtr());
    std::copy(vals.begin(), vals.end(), K.valuePtr());
    Eigen::SimplicialCholesky<Eigen::SparseMatrix<double, Eigen::RowMajor, i64>, Eigen::Upper> llt(K);
    if (llt.info() != Eigen::Success) return -1;
    Eigen::Matrix<double, Eigen::Dynamic, 1> fb(nodes);
    std::copy(f.begin(), f.end(), fb.data());
    const auto T = llt.solve(fb);
    std::copy(T.begin(), T.end(), temperature_out);
    return 0;
}

int orc_threads() { return omp_get_max_threads(); }
void orc_set_threads(int n) { omp_set_num_threads(n); }

// records the CG time and iteration count at which the next solves' stopping
// measure first reaches `tol` (0 switches it off)
void orc_set_record_tolerance(void* h, double tol) { static_cast<Problem*>(h)->record_tol = tol; }

} // extern "C"
