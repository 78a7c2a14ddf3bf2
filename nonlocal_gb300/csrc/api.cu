// C ABI of the library (include/nlgpu.h): argument checks, call order,
// host <-> device copies, and the stationary / nonstationary drivers.
#include "common.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numbers>

using namespace nlgpu;

struct nlgpu_ctx : Ctx {};

namespace {

thread_local std::string g_last_error;

template<class F>
int guarded(F&& f) {
    g_last_error.clear();
    try {
        f();
        return NLGPU_OK;
    } catch (const nlgpu::error& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return NLGPU_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return NLGPU_ERR_ARG;
    }
}

// the status of a solve entry: its error, else NLGPU_ERR_NO_CONVERGENCE (with a
// message) when the solve ended before the tolerance
int solve_status(int rc, int conv_status) {
    if (rc != NLGPU_OK) return rc;
    if (conv_status == NLGPU_ERR_NO_CONVERGENCE)
        g_last_error = "the solve stopped before the tolerance (iteration limit or a stalled recurrence)";
    return conv_status;
}

double ipow_host(double x, int n) {
    double r = 1.0;
    while (n > 0) { if (n & 1) { r *= x; --n; } else { x *= x; n >>= 1; } }
    return r;
}

double seconds(std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
}

void reset_from_model(Ctx& c) {
    c.neighbours_ready = false;
    c.inner_ready = c.local_ready = c.nonstationary_ready = false;
}

void reset_from_boundary(Ctx& c) {
    c.bc_ready = false;
    c.inner_ready = c.local_ready = c.nonstationary_ready = false;
}

void ensure_neighbours(Ctx& c) {
    if (!c.neighbours_ready) find_neighbours(c, c.strategy);
}

void ensure_boundary(Ctx& c) {
    if (!c.bc_ready) boundary_vectors(c);
}

// convection edges into the assembled matrix (convection_condition_2d.hpp:11-31),
// and the index of every convection / radiation edge pair in it
void boundary_matrix_terms(Ctx& c) {
    if (!has_convection(c) && !has_radiation(c)) return;
    NL_REQUIRE(c.symmetric || !has_radiation(c), NLGPU_ERR_UNSUPPORTED,
               "radiation with a non-symmetric system (variable conductivity and a nonlocal model)");
    boundary_matrix_index(c);
    add_convection(c);
}

// pure Neumann problems: the Lagrange column int N_i, the balance check of the
// fluxes (stationary_heat_equation_solver_2d.hpp:38-41) and the right-hand side
// f - lambda b, lambda = sum f / sum b, the multiplier the bordered system has
// (its first n rows sum to lambda sum b = sum f, as the rows of K sum to zero)
void neumann_prepare(Ctx& c) {
    c.neumann = pure_neumann(c);
    if (!c.neumann) return;
    NL_REQUIRE(c.symmetric, NLGPU_ERR_UNSUPPORTED, "a pure Neumann problem with a non-symmetric system");
    neumann_integrals(c);
    const size_t n = size_t(c.n_nodes);
    std::vector<double> f(n), b(n);
    c.rhs.download(f.data(), n, c.stream);
    c.node_integral.download(b.data(), n, c.stream);
    NL_CUDA(cudaStreamSynchronize(c.stream));
    double sf = 0.0, sb = 0.0;
    for (size_t i = 0; i < n; ++i) { sf += f[i]; sb += b[i]; }
    NL_REQUIRE(std::abs(sf) <= 1e-10, NLGPU_ERR_ARG, "It's unsolvable Neumann problem.");
    add_scaled(c, -sf / sb, c.node_integral.p, c.rhs.p);
}

// conductivity_matrix_2d::compute(FULL) into inner/bound, and the solver's full rows
void build_inner(Ctx& c) {
    NL_REQUIRE(c.mesh_ready && c.model_ready, NLGPU_ERR_STATE, "mesh and model must be set before assembly");
    ensure_boundary(c);
    c.symmetric = !(c.model.nonlocal() && c.cond_field.n);   // problem_settings::is_symmetric (problem_settings.hpp:32-34)
    if (c.model.nonlocal()) ensure_neighbours(c);
    build_patterns(c, !c.model.nonlocal(), c.symmetric, c.inner, &c.bound, &c.full, &c.full_from_upper);
    c.ff_assembly = c.assembly_precision == NLGPU_ASSEMBLY_FF;
    assemble_full(c);
    boundary_matrix_terms(c);
    fill_full_from_upper(c, c.inner, c.full, c.full_from_upper);
    c.rhs.resize(size_t(c.n_nodes));
    apply_first_kind(c, c.bound, c.rhs_init.p, c.rhs.p, c.x_dirichlet.p);
    neumann_prepare(c);
    c.inner_ready = true;
}

// CSR of n rows copied out as the reference stores a pure Neumann problem's
// matrix: each row ends with the Lagrange column n (int N_i), and row n holds
// its zero diagonal (conductivity_matrix_2d.hpp:39-72)
void download_csr_bordered(Ctx& c, const Csr& m, const double* lagrange, int64_t* rowptr, int64_t* col, double* val) {
    const size_t n = size_t(m.rows), nnz = size_t(m.nnz);
    std::vector<int64_t> rp(n + 1);
    std::vector<double> vl(val ? nnz : 0), b(n, 0.0);
    m.rowptr.download(rp.data(), n + 1, c.stream);
    std::vector<int32_t> c32(col ? nnz : 0);
    if (col) m.col.download(c32.data(), nnz, c.stream);
    if (val) m.val.download(vl.data(), nnz, c.stream);
    if (lagrange && val) NL_CUDA(cudaMemcpyAsync(b.data(), lagrange, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    NL_CUDA(cudaStreamSynchronize(c.stream));
    if (rowptr) {
        for (size_t r = 0; r <= n; ++r) rowptr[r] = rp[r] + int64_t(r);
        rowptr[n + 1] = rp[n] + int64_t(n) + 1;
    }
    for (size_t r = 0; r < n; ++r) {
        const size_t out = size_t(rp[r]) + r;
        const size_t len = size_t(rp[r + 1] - rp[r]);
        for (size_t k = 0; k < len; ++k) {
            if (col) col[out + k] = c32[size_t(rp[r]) + k];
            if (val) val[out + k] = vl[size_t(rp[r]) + k];
        }
        if (col) col[out + len] = int64_t(n);
        if (val) val[out + len] = b[r];
    }
    if (col) col[size_t(rp[n]) + n] = int64_t(n);
    if (val) val[size_t(rp[n]) + n] = 0.0;
}

// p1 * K_local with the reference's LOCAL theories (stationary_heat_equation_solver_2d.hpp:91-93)
void build_local(Ctx& c) {
    ensure_boundary(c);
    build_patterns(c, true, true, c.local, nullptr, nullptr, nullptr);
    assemble_local(c, c.local, c.model.p1, 0);
    c.local_ready = true;
}

void download_csr(Ctx& c, const Csr& m, int64_t* rowptr, int64_t* col, double* val) {
    if (rowptr) m.rowptr.download(rowptr, size_t(m.rows + 1), c.stream);
    std::vector<int32_t> tmp;
    if (col) { tmp.resize(size_t(m.nnz)); m.col.download(tmp.data(), tmp.size(), c.stream); }
    if (val) m.val.download(val, size_t(m.nnz), c.stream);
    NL_CUDA(cudaStreamSynchronize(c.stream));
    if (col) for (size_t k = 0; k < tmp.size(); ++k) col[k] = tmp[k];
}

void fill_report(Ctx& c, nlgpu_solve_report* rep, const CgResult& r) {
    if (!rep) return;
    rep->iterations = r.iterations;
    rep->residual = r.residual;
    rep->reference_residual = r.reference_residual;
    rep->preconditioner_ok = c.ilt.ok ? 1 : 0;
    rep->preconditioner_shifts = c.ilt.attempts;
    rep->nnz_inner = c.inner.nnz;
    rep->nnz_solver = c.full.nnz;
    rep->element_pairs = c.pairs;
    rep->outer_iterations = r.outer_iterations;
    rep->learned_fallback = r.learned_fallback ? 1 : 0;
    rep->column_bytes = c.full.up_ok || c.full.col16_ok ? 2 : 4;
    rep->nnz_fp32 = c.full.up_ok ? c.full.up_nnz : c.full.nnz;
    rep->fp32_symmetric = c.full.up_ok ? 1 : 0;
}

// One linear solve of the assembled system with right-hand side rhs (default
// ctx.rhs) into ctx.temperature.  keep_preconditioner reuses the ILLT factor
// of the previous call (the radiation loop changes only boundary entries).
CgResult solve_system(Ctx& c, const nlgpu_solve_options& o, nlgpu_solve_report* rep, const double* rhs = nullptr,
                      bool keep_preconditioner = false) {
    NL_REQUIRE(c.inner_ready, NLGPU_ERR_STATE, "the system must be assembled first");
    const double* b = rhs ? rhs : c.rhs.p;
    if (!c.symmetric) {
        // variable conductivity with a nonlocal model: full storage, BiCGSTAB with
        // the diagonal preconditioner (stationary_heat_equation_solver_2d.hpp:105-108);
        // MIXED: preconditioned by the FP32 ILLT of the local part instead
        const auto t0 = std::chrono::steady_clock::now();
        c.temperature.resize(size_t(c.n_nodes));
        CgResult r = o.precision == NLGPU_PRECISION_MIXED && !rhs
                         ? batch_bicgstab({&c}, o.tolerance, o.max_iterations, true).front()
                         : bicgstab_solve(c, c.full, b, c.temperature.p, o.tolerance, o.max_iterations);
        if (rep) rep->seconds_solve = seconds(t0);
        fill_report(c, rep, r);
        return r;
    }
    NL_REQUIRE(o.preconditioner >= NLGPU_PRECONDITIONER_IDENTITY && o.preconditioner <= NLGPU_PRECONDITIONER_ILLT_LEARNED,
               NLGPU_ERR_ARG, "unknown preconditioner");
    NL_REQUIRE(o.precision == NLGPU_PRECISION_FP64 || o.precision == NLGPU_PRECISION_MIXED, NLGPU_ERR_ARG,
               "unknown precision");
    NL_REQUIRE(o.triangular_sweeps <= 4096, NLGPU_ERR_ARG, "at most 4096 Jacobi sweeps per triangle");
    const bool learned = o.preconditioner == NLGPU_PRECONDITIONER_ILLT_LEARNED;
    NL_REQUIRE(!learned || c.mp.weights_set, NLGPU_ERR_STATE, "train the learned correction or set its weights first");
    const IncompleteCholesky* M = nullptr;
    auto t0 = std::chrono::steady_clock::now();
    PhaseTimer timer(c.stream, "solve_system");
    const bool mixed = o.precision == NLGPU_PRECISION_MIXED || learned;
    const int sweeps = o.triangular_sweeps == 0 ? NLGPU_DEFAULT_TRIANGULAR_SWEEPS : std::max(o.triangular_sweeps, 0);
    if (o.preconditioner != NLGPU_PRECONDITIONER_IDENTITY) {
        if (!c.local_ready) build_local(c);
        timer.mark("local matrix");
        // the exact sweeps' shared-memory plans only when this solve uses them
        if (!keep_preconditioner) ilt_build(c, c.local, c.ilt, !(mixed && sweeps > 0), mixed && sweeps > 0);
        timer.mark("preconditioner");
        if (c.ilt.ok) M = &c.ilt;   // identity fallback (stationary_heat_equation_solver_2d.hpp:97-101)
        if (learned && M && !(c.mp.ready && c.mp.n == c.local.rows)) mpnn_prepare(c, c.local);
    } else {
        c.ilt.ok = false;
    }
    NL_CUDA(cudaStreamSynchronize(c.stream));
    if (rep) rep->seconds_preconditioner = seconds(t0);
    t0 = std::chrono::steady_clock::now();
    c.temperature.resize(size_t(c.n_nodes));
    CgResult r;
    if (mixed) {
        matrix_to_f32(c, c.full, c.symmetric && c.fp32_symmetric ? &c.inner : nullptr);
        timer.mark("FP32 matrix");
        NL_REQUIRE(o.coarse_aggregates >= 0, NLGPU_ERR_ARG, "coarse_aggregates must be >= 0");
        const bool coarse = o.coarse_aggregates > 0 && M && !c.neumann;
        if (coarse) {
            double aspect = o.coarse_aspect;
            // (lambda_x / lambda_y)^0.7: on the 300x300 orthotropic (1, 0.1) problem the
            // FCG took 87 iterations with square cells, 67 at ratio^0.5, 62 at
            // ratio^0.7 (aspect 5), 72 at the ratio itself
            if (!(aspect > 0.0))
                aspect = c.model.cond_kind == NLGPU_CONDUCTIVITY_ORTHOTROPIC && c.model.cond[0] > 0.0 && c.model.cond[1] > 0.0
                             ? std::pow(c.model.cond[0] / c.model.cond[1], 0.7) : 1.0;
            coarse_build(c, c.full, o.coarse_aggregates, aspect);
        }
        timer.mark("coarse correction");
        c.ilt_sweeps = sweeps;
        r = mixed_solve(c, c.full, M ? &c.ilt : nullptr, b, c.temperature.p, o.tolerance, o.max_iterations,
                        o.inner_tolerance > 0.0 ? o.inner_tolerance : MIXED_UPDATE_FACTOR, false, learned && M && c.mp.use,
                        c.ilt_sweeps, coarse && c.co.ready);
        if (learned && M && c.mp.use) mpnn_check(c);
        if (learned && !(M && c.mp.use)) r.learned_fallback = true;   // gated off: ILLT alone
    } else {
        r = cg_solve(c, c.full, M, b, c.temperature.p, o.tolerance, o.max_iterations, false);
    }
    if (rep) rep->seconds_solve = seconds(t0);
    if (M && c.sweep_error.n) {
        int err = 0;
        NL_CUDA(cudaMemcpyAsync(&err, c.sweep_error.p, sizeof err, cudaMemcpyDeviceToHost, c.stream));
        NL_CUDA(cudaStreamSynchronize(c.stream));
        NL_REQUIRE(err == 0, NLGPU_ERR_TIMEOUT, "a triangular sweep stage wait gave up");
    }
    fill_report(c, rep, r);
    return r;
}

// stationary_heat_equation_solver_2d.hpp:66-116 with radiation edges: from the
// initial temperature, each step solves K_T dT = K T_prev - r_rad - f, where K
// holds conductivity and convection, K_T = K - 4 sigma eps int T_prev^3 N_i N_j
// and r_rad = -sigma eps int T_prev^4 N_i, then T = T_prev - dT; it stops after
// max_iterations or once |T - T_prev| / |T| or |residual| is at most the
// tolerance.  The linear solves are this library's ILLT-CG (the reference uses
// Jacobi-preconditioned CG to machine precision; both solve the same system).
CgResult radiation_loop(Ctx& c, const nlgpu_solve_options& o, nlgpu_solve_report* rep) {
    const i64 n = c.n_nodes;
    c.nl_work.resize(size_t(4 * n));
    double* kt = c.nl_work.p;            // K T_prev
    double* rad = kt + n;                // r_rad
    double* prev = rad + n;              // T_prev
    double* residual = prev + n;
    if (c.initial_temperature.n) {
        NL_CUDA(cudaMemcpyAsync(prev, c.initial_temperature.p, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    } else {
        NL_CUDA(cudaMemsetAsync(prev, 0, size_t(n) * sizeof(double), c.stream));
    }
    c.upper_base.resize(size_t(c.inner.nnz));
    NL_CUDA(cudaMemcpyAsync(c.upper_base.p, c.inner.val.p, size_t(c.inner.nnz) * sizeof(double),
                            cudaMemcpyDeviceToDevice, c.stream));
    c.temperature.resize(size_t(n));
    NL_CUDA(cudaMemcpyAsync(c.temperature.p, prev, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    CgResult total;
    total.converged = true;
    double difference = 1.0, norm = 1.0;
    i64 it = 0;
    while (it < c.nl_max_iterations && c.nl_tolerance < difference && c.nl_tolerance < norm) {
        NL_CUDA(cudaMemcpyAsync(c.inner.val.p, c.upper_base.p, size_t(c.inner.nnz) * sizeof(double),
                                cudaMemcpyDeviceToDevice, c.stream));
        fill_full_from_upper(c, c.inner, c.full, c.full_from_upper);
        spmv_full(c, c.full, prev, kt);
        NL_CUDA(cudaMemsetAsync(rad, 0, size_t(n) * sizeof(double), c.stream));
        add_radiation(c, prev, rad, -4.0, -1.0);
        fill_full_from_upper(c, c.inner, c.full, c.full_from_upper);
        subtract3(c, kt, rad, c.rhs.p, residual);
        const CgResult r = solve_system(c, o, rep, residual, it > 0);
        total.iterations += r.iterations;
        total.outer_iterations += r.outer_iterations;
        total.residual = r.residual;
        total.reference_residual = r.reference_residual;
        total.converged = total.converged && r.converged;
        const std::array<double, 3> s = step_norms(c, residual, prev, c.temperature.p);
        ++it;
        norm = std::sqrt(s[0]);
        const double tn = std::sqrt(s[2]);
        difference = std::sqrt(s[1]) / (tn != 0.0 ? tn : 1.0);
        NL_CUDA(cudaMemcpyAsync(prev, c.temperature.p, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    }
    // leave the assembled matrix (conductivity and convection) in place
    NL_CUDA(cudaMemcpyAsync(c.inner.val.p, c.upper_base.p, size_t(c.inner.nnz) * sizeof(double),
                            cudaMemcpyDeviceToDevice, c.stream));
    fill_full_from_upper(c, c.inner, c.full, c.full_from_upper);
    NL_CUDA(cudaStreamSynchronize(c.stream));
    fill_report(c, rep, total);
    if (rep) rep->nonlinear_iterations = it;
    return total;
}

// The stationary solve of the assembled system: one linear solve, or the
// radiation loop; a pure Neumann problem's temperature is then shifted to
// int T = energy (the bordered system's last row)
CgResult stationary_solve(Ctx& c, const nlgpu_solve_options& o, nlgpu_solve_report* rep) {
    const CgResult r = has_radiation(c) ? radiation_loop(c, o, rep) : solve_system(c, o, rep);
    if (c.neumann) {
        const size_t n = size_t(c.n_nodes);
        std::vector<double> t(n), b(n);
        c.temperature.download(t.data(), n, c.stream);
        c.node_integral.download(b.data(), n, c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        double bt = 0.0, sb = 0.0;
        for (size_t i = 0; i < n; ++i) { bt += b[i] * t[i]; sb += b[i]; }
        add_constant(c, (c.energy - bt) / sb, c.temperature.p);
    }
    if (rep) rep->neumann = c.neumann ? 1 : 0;
    return r;
}

}  // namespace

extern "C" {

const char* nlgpu_status_string(int status) {
    switch (status) {
    case NLGPU_OK: return "ok";
    case NLGPU_ERR_ARG: return "invalid argument";
    case NLGPU_ERR_CUDA: return "CUDA error";
    case NLGPU_ERR_UNSUPPORTED: return "unsupported";
    case NLGPU_ERR_STATE: return "call order violated";
    case NLGPU_ERR_NUMERICAL: return "numerical breakdown";
    case NLGPU_ERR_NO_CONVERGENCE: return "no convergence";
    case NLGPU_ERR_OUT_OF_MEMORY: return "out of device memory";
    case NLGPU_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

const char* nlgpu_last_error(void) { return g_last_error.c_str(); }

int nlgpu_device_count(int* count) {
    if (!count) return NLGPU_ERR_ARG;
    int n = 0;
    const cudaError_t e = cudaGetDeviceCount(&n);
    *count = e == cudaSuccess ? n : 0;
    if (e != cudaSuccess) cudaGetLastError();
    return NLGPU_OK;
}

int64_t nlgpu_kernel_launches(void) { return g_launches.load(); }

int nlgpu_set_device(int device) {
    return guarded([&] { NL_CUDA(cudaSetDevice(device)); });
}

int nlgpu_create(nlgpu_ctx** ctx, void* stream) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        int n = 0;
        NL_CUDA(cudaGetDeviceCount(&n));
        NL_REQUIRE(n > 0, NLGPU_ERR_CUDA, "no CUDA device");
        auto* c = new nlgpu_ctx{};
        if (stream) c->stream = static_cast<cudaStream_t>(stream);
        else {
            if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; NL_CUDA(cudaGetLastError()); }
            c->own_stream = true;
        }
        *ctx = c;
    });
}

int nlgpu_destroy(nlgpu_ctx* ctx) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        cudaStreamSynchronize(ctx->stream);
        const bool own = ctx->own_stream;
        cudaStream_t s = ctx->stream;
        delete ctx;
        if (own) cudaStreamDestroy(s);
    });
}

int nlgpu_synchronize(nlgpu_ctx* ctx) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] { NL_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

int nlgpu_mesh_2d(nlgpu_ctx* ctx, int element_type, int64_t n_nodes, const double* nodes, int64_t n_elements,
                  const int64_t* elements) {
    if (!ctx || !nodes || !elements || n_nodes <= 0 || n_elements <= 0) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        c.basis = make_basis(element_type);
        NL_REQUIRE(n_nodes < (int64_t(1) << 31) && n_elements * c.basis.nen < (int64_t(1) << 40), NLGPU_ERR_UNSUPPORTED,
                   "mesh too large for 32-bit node numbers");
        std::vector<int32_t> el(size_t(n_elements * c.basis.nen));
        for (size_t k = 0; k < el.size(); ++k) {
            NL_REQUIRE(elements[k] >= 0 && elements[k] < n_nodes, NLGPU_ERR_ARG, "element node out of range");
            el[k] = int32_t(elements[k]);
        }
        c.element_type = element_type;
        c.n_nodes = n_nodes; c.n_elems = n_elements;
        c.nodes.upload(nodes, size_t(2 * n_nodes), c.stream);
        c.elems.upload(el.data(), el.size(), c.stream);
        mesh_init(c);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        c.cond_field.release(); c.source_q.release(); c.dirichlet_override.release();
        c.groups.clear();
        reset_from_model(c);
        reset_from_boundary(c);
    });
}

int nlgpu_cuthill_mckee(nlgpu_ctx* ctx, int only_local, int reverse, int64_t* permutation) {
    if (!ctx || !permutation) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
        const bool local_graph = only_local || !(c.model_ready && c.model.nonlocal());
        if (!local_graph) ensure_neighbours(c);
        std::vector<i64> off;
        std::vector<int32_t> adj;
        node_graph(c, local_graph, off, adj);
        const std::vector<i64> perm = cuthill_mckee_order(off, adj);
        if (reverse)   // reverse_permutation (cuthill_mckee.hpp:157-164): the inverse
            for (size_t i = 0; i < perm.size(); ++i) permutation[perm[i]] = int64_t(i);
        else
            std::copy(perm.begin(), perm.end(), permutation);
    });
}

int nlgpu_renumbering(nlgpu_ctx* ctx, const int64_t* permutation) {
    if (!ctx || !permutation) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
        const size_t n = size_t(c.n_nodes);
        std::vector<int32_t> perm(n);
        std::vector<char> seen(n, 0);
        for (size_t i = 0; i < n; ++i) {
            NL_REQUIRE(permutation[i] >= 0 && permutation[i] < c.n_nodes, NLGPU_ERR_ARG,
                       "Permutation entry out of range.");
            NL_REQUIRE(!seen[size_t(permutation[i])], NLGPU_ERR_ARG, "Incorrect permutation, some of the nodes are the same.");
            seen[size_t(permutation[i])] = 1;
            perm[i] = int32_t(permutation[i]);
        }
        renumber_mesh(c, perm);
        reset_from_boundary(c);   // element-based neighbour lists stay valid
    });
}

int nlgpu_get_quadrature(nlgpu_ctx* ctx, double* qcoords, double* jacobians, double* derivatives) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
        if (qcoords) c.qcoord.download(qcoords, c.qcoord.n, c.stream);
        if (jacobians) c.jac.download(jacobians, c.jac.n, c.stream);
        if (derivatives) c.deriv.download(derivatives, c.deriv.n, c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int nlgpu_get_basis(nlgpu_ctx* ctx, int* nodes_per_element, int* qnodes, double* qN, double* qNxi, double* qNeta,
                    double* weights, double* centre) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        const Basis& b = ctx->basis;
        NL_REQUIRE(ctx->mesh_ready, NLGPU_ERR_STATE, "no mesh");
        if (nodes_per_element) *nodes_per_element = b.nen;
        if (qnodes) *qnodes = b.nq;
        const size_t m = size_t(b.nen * b.nq);
        if (qN) std::memcpy(qN, b.qN, m * sizeof(double));
        if (qNxi) std::memcpy(qNxi, b.qNxi, m * sizeof(double));
        if (qNeta) std::memcpy(qNeta, b.qNeta, m * sizeof(double));
        if (weights) std::memcpy(weights, b.w, size_t(b.nq) * sizeof(double));
        if (centre) std::memcpy(centre, b.centre, size_t(b.nen) * sizeof(double));
    });
}

int nlgpu_set_model_2d(nlgpu_ctx* ctx, const nlgpu_model_2d* model) {
    if (!ctx || !model) return NLGPU_ERR_ARG;
    return guarded([&] {
        ctx->model = make_model(*model);
        ctx->model_ready = true;
        reset_from_model(*ctx);
    });
}

int nlgpu_set_conductivity_field(nlgpu_ctx* ctx, const double* values) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
        if (values) c.cond_field.upload(values, size_t(c.n_elems * c.basis.nq), c.stream);
        else c.cond_field.release();
        c.inner_ready = c.local_ready = c.nonstationary_ready = false;
    });
}

int nlgpu_set_capacity(nlgpu_ctx* ctx, double capacity, double density) {
    if (!ctx) return NLGPU_ERR_ARG;
    ctx->capacity = capacity; ctx->density = density; ctx->nonstationary_ready = false;
    return NLGPU_OK;
}

int nlgpu_find_neighbours(nlgpu_ctx* ctx, int strategy, double* search_radius, int64_t* pairs) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        find_neighbours(*ctx, strategy);
        if (search_radius) { search_radius[0] = ctx->search_r[0]; search_radius[1] = ctx->search_r[1]; }
        if (pairs) *pairs = ctx->pairs;
        ctx->inner_ready = ctx->nonstationary_ready = false;
    });
}

int nlgpu_get_neighbours(nlgpu_ctx* ctx, int64_t* offsets, int64_t* list) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.neighbours_ready, NLGPU_ERR_STATE, "no neighbour search yet");
        if (offsets) c.noff.download(offsets, size_t(c.n_elems + 1), c.stream);
        std::vector<int32_t> tmp(static_cast<size_t>(c.pairs));
        if (list) c.nlist.download(tmp.data(), tmp.size(), c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        if (list) for (size_t k = 0; k < tmp.size(); ++k) list[k] = tmp[k];
    });
}

namespace {

// one boundary group; value is the temperature or the second-kind flux
// (operator() of the condition classes, thermal_boundary_conditions_2d.hpp:20-97)
void add_group(Ctx& c, int kind, int64_t n_edges, int nodes_per_edge, const int64_t* edges, double value,
               const double* node_values, double heat_transfer, double emissivity) {
    NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
    NL_REQUIRE(nodes_per_edge == 2 || nodes_per_edge == 3, NLGPU_ERR_UNSUPPORTED, "boundary edges have 2 or 3 nodes");
    BoundaryGroup g;
    g.kind = kind; g.nen = nodes_per_edge; g.n_edges = n_edges; g.value = value;
    g.heat_transfer = heat_transfer; g.emissivity = emissivity;
    std::vector<int32_t> e(size_t(n_edges * nodes_per_edge));
    for (size_t k = 0; k < e.size(); ++k) {
        NL_REQUIRE(edges[k] >= 0 && edges[k] < c.n_nodes, NLGPU_ERR_ARG, "boundary node out of range");
        e[k] = int32_t(edges[k]);
    }
    g.edges.upload(e.data(), e.size(), c.stream);
    if (node_values) g.node_values.upload(node_values, e.size(), c.stream);
    NL_CUDA(cudaStreamSynchronize(c.stream));
    c.groups.push_back(std::move(g));
    reset_from_boundary(c);
}

}  // namespace

int nlgpu_add_boundary_2d(nlgpu_ctx* ctx, int kind, int64_t n_edges, int nodes_per_edge, const int64_t* edges,
                          double value, const double* node_values) {
    if (!ctx || !edges || n_edges < 0) return NLGPU_ERR_ARG;
    return guarded([&] {
        NL_REQUIRE(kind == NLGPU_BC_TEMPERATURE || kind == NLGPU_BC_FLUX, NLGPU_ERR_ARG,
                   "unknown boundary kind (convection and radiation: nlgpu_add_flux_boundary_2d)");
        add_group(*ctx, kind, n_edges, nodes_per_edge, edges, value, node_values, 0.0, 0.0);
    });
}

int nlgpu_add_flux_boundary_2d(nlgpu_ctx* ctx, int kind, int64_t n_edges, int nodes_per_edge, const int64_t* edges,
                               double flux, double heat_transfer, double ambient_temperature, double emissivity) {
    if (!ctx || !edges || n_edges < 0) return NLGPU_ERR_ARG;
    return guarded([&] {
        double value = 0.0;
        switch (kind) {
        case NLGPU_BC_FLUX: value = flux; heat_transfer = emissivity = 0.0; break;
        case NLGPU_BC_CONVECTION: value = heat_transfer * ambient_temperature; emissivity = 0.0; break;
        case NLGPU_BC_RADIATION: value = 0.0; heat_transfer = 0.0; break;
        case NLGPU_BC_COMBINED_FLUX: value = flux + heat_transfer * ambient_temperature; break;
        default: throw nlgpu::error{NLGPU_ERR_ARG, "unknown flux boundary kind"};
        }
        NL_REQUIRE(std::isfinite(value) && std::isfinite(heat_transfer) && std::isfinite(emissivity), NLGPU_ERR_ARG,
                   "boundary coefficients must be finite");
        add_group(*ctx, kind, n_edges, nodes_per_edge, edges, value, nullptr, heat_transfer, emissivity);
    });
}

int nlgpu_set_stationary_parameters(nlgpu_ctx* ctx, double tolerance, int64_t max_iterations, double energy,
                                    const double* initial_temperature) {
    if (!ctx || max_iterations < 0 || !std::isfinite(energy)) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
        c.nl_tolerance = tolerance;
        c.nl_max_iterations = max_iterations;
        c.energy = energy;
        if (initial_temperature) c.initial_temperature.upload(initial_temperature, size_t(c.n_nodes), c.stream);
        else c.initial_temperature.release();
        NL_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int nlgpu_get_system_rows(nlgpu_ctx* ctx, int64_t* rows) {
    if (!ctx || !rows) return NLGPU_ERR_ARG;
    return guarded([&] {
        NL_REQUIRE(ctx->inner_ready, NLGPU_ERR_STATE, "FULL part not assembled");
        *rows = ctx->n_nodes + (ctx->neumann ? 1 : 0);
    });
}

int nlgpu_set_source(nlgpu_ctx* ctx, double value, const double* per_qnode) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
        c.source = value;
        if (per_qnode) c.source_q.upload(per_qnode, size_t(c.n_elems * c.basis.nq), c.stream);
        else c.source_q.release();
        reset_from_boundary(c);
    });
}

int nlgpu_set_dirichlet_values(nlgpu_ctx* ctx, const double* values) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
        if (values) c.dirichlet_override.upload(values, size_t(c.n_nodes), c.stream);
        else c.dirichlet_override.release();
        reset_from_boundary(c);
    });
}

int nlgpu_clear_boundaries(nlgpu_ctx* ctx) {
    if (!ctx) return NLGPU_ERR_ARG;
    ctx->groups.clear();
    ctx->source = 0.0;
    ctx->source_q.release();
    ctx->dirichlet_override.release();
    reset_from_boundary(*ctx);
    return NLGPU_OK;
}

int nlgpu_conductivity_matrix_2d(nlgpu_ctx* ctx, int part, int64_t* nnz_inner, int64_t* nnz_bound) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(part == NLGPU_PART_FULL || part == NLGPU_PART_LOCAL, NLGPU_ERR_ARG, "part is LOCAL or FULL");
        NL_REQUIRE(c.mesh_ready && c.model_ready, NLGPU_ERR_STATE, "mesh and model must be set before assembly");
        if (part == NLGPU_PART_FULL) {
            build_inner(c);
            // a pure Neumann problem is copied out with the Lagrange column and row
            if (nnz_inner) *nnz_inner = c.inner.nnz + (c.neumann ? c.n_nodes + 1 : 0);
            if (nnz_bound) *nnz_bound = c.neumann ? 0 : c.bound.nnz;
        } else {
            build_local(c);
            if (nnz_inner) *nnz_inner = c.local.nnz + (c.neumann && c.node_integral.n ? c.n_nodes + 1 : 0);
            if (nnz_bound) *nnz_bound = 0;
        }
        NL_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int nlgpu_get_matrix(nlgpu_ctx* ctx, int which, int64_t* rowptr, int64_t* col, double* val) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        if (which == NLGPU_MATRIX_INNER || which == NLGPU_MATRIX_BOUND) {
            NL_REQUIRE(c.inner_ready, NLGPU_ERR_STATE, "FULL part not assembled");
            if (c.neumann && which == NLGPU_MATRIX_INNER) {
                download_csr_bordered(c, c.inner, c.node_integral.p, rowptr, col, val);
            } else if (c.neumann) {   // no temperature nodes: an empty bound part of n + 1 rows
                if (rowptr) std::fill(rowptr, rowptr + c.n_nodes + 2, int64_t{0});
            } else {
                download_csr(c, which == NLGPU_MATRIX_INNER ? c.inner : c.bound, rowptr, col, val);
            }
        } else if (which == NLGPU_MATRIX_LOCAL) {
            NL_REQUIRE(c.local_ready, NLGPU_ERR_STATE, "LOCAL part not assembled");
            if (c.neumann && c.node_integral.n) download_csr_bordered(c, c.local, c.node_integral.p, rowptr, col, val);
            else download_csr(c, c.local, rowptr, col, val);
        } else {
            throw nlgpu::error{NLGPU_ERR_ARG, "unknown matrix"};
        }
    });
}

int nlgpu_get_rhs(nlgpu_ctx* ctx, double* rhs, double* rhs_init) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.inner_ready, NLGPU_ERR_STATE, "FULL part not assembled");
        if (rhs_init) c.rhs_init.download(rhs_init, size_t(c.n_nodes), c.stream);
        if (rhs && c.neumann) {   // the reference's f: the fluxes (not shifted by lambda b) and the energy row
            c.rhs_init.download(rhs, size_t(c.n_nodes), c.stream);
            rhs[c.n_nodes] = c.energy;
        } else if (rhs) {
            c.rhs.download(rhs, size_t(c.n_nodes), c.stream);
        }
        if (rhs_init && c.neumann) rhs_init[c.n_nodes] = c.energy;
        NL_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int nlgpu_calc_flux(nlgpu_ctx* ctx, const double* temperature, double* flux_x, double* flux_y) {
    if (!ctx || !temperature || !flux_x || !flux_y) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready && c.model_ready, NLGPU_ERR_STATE, "mesh and model must be set");
        if (c.model.nonlocal()) ensure_neighbours(c);
        const size_t n = size_t(c.n_nodes);
        dbuf<double> t, fx, fy;
        t.upload(temperature, n, c.stream);
        fx.resize(n);
        fy.resize(n);
        calc_flux(c, t.p, fx.p, fy.p);
        fx.download(flux_x, n, c.stream);
        fy.download(flux_y, n, c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int nlgpu_solve_assembled(nlgpu_ctx* ctx, const nlgpu_solve_options* options, double* temperature,
                          nlgpu_solve_report* report) {
    if (!ctx || !options || !temperature) return NLGPU_ERR_ARG;
    int conv_status = NLGPU_OK;
    const int rc = guarded([&] {
        Ctx& c = *ctx;
        const auto t0 = std::chrono::steady_clock::now();
        const CgResult r = stationary_solve(c, *options, report);
        c.temperature.download(temperature, size_t(c.n_nodes), c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        if (report) report->seconds_total = seconds(t0);
        if (!r.converged) conv_status = NLGPU_ERR_NO_CONVERGENCE;
    });
    return solve_status(rc, conv_status);
}

int nlgpu_solve_assembled_batch(int64_t count, nlgpu_ctx* const* instances, const nlgpu_solve_options* options,
                                double* const* temperatures, nlgpu_solve_report* reports) {
    if (count < 0 || (count > 0 && (!instances || !temperatures)) || !options) return NLGPU_ERR_ARG;
    for (int64_t k = 0; k < count; ++k)
        if (!instances[k] || !temperatures[k]) return NLGPU_ERR_ARG;
    int conv_status = NLGPU_OK;
    const int rc = guarded([&] {
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<Ctx*> batched;
        std::vector<int64_t> index;
        for (int64_t k = 0; k < count; ++k) {
            Ctx& c = *instances[k];
            NL_REQUIRE(c.inner_ready, NLGPU_ERR_STATE, "the system must be assembled first");
            if (!c.symmetric && !has_radiation(c) && !c.neumann) {
                batched.push_back(&c);
                index.push_back(k);
            }
        }
        std::vector<CgResult> res;
        if (!batched.empty())
            res = batch_bicgstab(batched, options->tolerance, options->max_iterations,
                                 options->precision == NLGPU_PRECISION_MIXED);
        const double batch_seconds = seconds(t0);
        size_t next = 0;
        for (int64_t k = 0; k < count; ++k) {
            Ctx& c = *instances[k];
            nlgpu_solve_report* rep = reports ? reports + k : nullptr;
            if (rep) std::memset(rep, 0, sizeof *rep);
            CgResult r;
            const auto t1 = std::chrono::steady_clock::now();
            if (next < index.size() && index[next] == k) {
                r = res[next++];
                fill_report(c, rep, r);
                if (rep) rep->seconds_solve = batch_seconds;
            } else {
                r = stationary_solve(c, *options, rep);
            }
            c.temperature.download(temperatures[k], size_t(c.n_nodes), c.stream);
            NL_CUDA(cudaStreamSynchronize(c.stream));
            if (rep) rep->seconds_total = (rep->seconds_solve > 0.0 ? rep->seconds_solve : 0.0) + seconds(t1);
            if (!r.converged) conv_status = NLGPU_ERR_NO_CONVERGENCE;
        }
    });
    return solve_status(rc, conv_status);
}

int nlgpu_stationary_2d(nlgpu_ctx* ctx, const nlgpu_solve_options* options, double* temperature,
                        nlgpu_solve_report* report) {
    if (!ctx || !options || !temperature) return NLGPU_ERR_ARG;
    int conv_status = NLGPU_OK;
    const int rc = guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready && c.model_ready, NLGPU_ERR_STATE, "mesh and model must be set");
        nlgpu_solve_report local_rep{};
        nlgpu_solve_report* rep = report ? report : &local_rep;
        std::memset(rep, 0, sizeof *rep);
        const auto t_all = std::chrono::steady_clock::now();
        auto t0 = t_all;
        ensure_boundary(c);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        rep->seconds_boundary = seconds(t0);
        t0 = std::chrono::steady_clock::now();
        if (c.model.nonlocal()) ensure_neighbours(c);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        rep->seconds_neighbours = seconds(t0);
        t0 = std::chrono::steady_clock::now();
        c.symmetric = !(c.model.nonlocal() && c.cond_field.n);
        build_patterns(c, !c.model.nonlocal(), c.symmetric, c.inner, &c.bound, &c.full, &c.full_from_upper);
        // the local matrix feeds the ILLT; the non-symmetric systems' BiCGSTAB uses the diagonal
        if (c.symmetric) build_patterns(c, true, true, c.local, nullptr, nullptr, nullptr);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        rep->seconds_pattern = seconds(t0);
        t0 = std::chrono::steady_clock::now();
        // the mixed-precision form computes its nonlocal blocks on the FP32 pipes (float-float)
        const bool mixed = options->precision == NLGPU_PRECISION_MIXED ||
                           options->preconditioner == NLGPU_PRECONDITIONER_ILLT_LEARNED;
        c.ff_assembly = c.assembly_precision == NLGPU_ASSEMBLY_FF ||
                        (c.assembly_precision == NLGPU_ASSEMBLY_AUTO && mixed);
        assemble_full(c);
        boundary_matrix_terms(c);
        fill_full_from_upper(c, c.inner, c.full, c.full_from_upper);
        if (c.symmetric) {
            assemble_local(c, c.local, c.model.p1, 0);
            c.local_ready = true;
        }
        NL_CUDA(cudaStreamSynchronize(c.stream));
        rep->seconds_assembly = seconds(t0);
        t0 = std::chrono::steady_clock::now();
        c.rhs.resize(size_t(c.n_nodes));
        apply_first_kind(c, c.bound, c.rhs_init.p, c.rhs.p, c.x_dirichlet.p);
        neumann_prepare(c);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        rep->seconds_boundary += seconds(t0);
        c.inner_ready = true;
        const CgResult r = stationary_solve(c, *options, rep);
        c.temperature.download(temperature, size_t(c.n_nodes), c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        rep->seconds_total = seconds(t_all);
        if (!r.converged) conv_status = NLGPU_ERR_NO_CONVERGENCE;
    });
    return solve_status(rc, conv_status);
}

int nlgpu_cg_solve(nlgpu_ctx* ctx, int64_t n, const int64_t* a_rowptr, const int64_t* a_col, const double* a_val,
                   const int64_t* p_rowptr, const int64_t* p_col, const double* p_val, const double* b, const double* x0,
                   double tolerance, int64_t max_iterations, double* x, nlgpu_solve_report* report) {
    if (!ctx || n <= 0 || !a_rowptr || !a_col || !a_val || !b || !x) return NLGPU_ERR_ARG;
    int conv_status = NLGPU_OK;
    const int rc = guarded([&] {
        Ctx& c = *ctx;
        const auto t0 = std::chrono::steady_clock::now();
        // full padded rows from the upper storage (both triangles)
        std::vector<std::vector<std::pair<int32_t, double>>> rows(static_cast<size_t>(n));
        for (int64_t r = 0; r < n; ++r)
            for (int64_t k = a_rowptr[r]; k < a_rowptr[r + 1]; ++k) {
                const int64_t cc = a_col[k];
                NL_REQUIRE(cc >= r && cc < n, NLGPU_ERR_ARG, "A must be the upper triangle with columns in range");
                rows[size_t(r)].push_back({int32_t(cc), a_val[k]});
                if (cc != r) rows[size_t(cc)].push_back({int32_t(r), a_val[k]});
            }
        std::vector<i64> rp(size_t(n + 1), 0);
        std::vector<int32_t> col;
        std::vector<double> val;
        for (int64_t r = 0; r < n; ++r) {
            auto& row = rows[size_t(r)];
            std::sort(row.begin(), row.end(), [](const auto& u, const auto& v) { return u.first < v.first; });
            for (const auto& [cc, v] : row) { col.push_back(cc); val.push_back(v); }
            while (col.size() % 4) { col.push_back(int32_t(r)); val.push_back(0.0); }
            rp[size_t(r) + 1] = i64(col.size());
        }
        rows.clear();
        Csr A;
        A.rows = n; A.nnz = i64(col.size());
        A.rowptr.upload(rp.data(), rp.size(), c.stream);
        A.col.upload(col.data(), col.size(), c.stream);
        A.val.upload(val.data(), val.size(), c.stream);
        dbuf<double> db, dx;
        db.upload(b, size_t(n), c.stream);
        dx.resize(size_t(n));
        if (x0) dx.upload(x0, size_t(n), c.stream);
        const IncompleteCholesky* M = nullptr;
        IncompleteCholesky ic;
        if (p_rowptr && p_col && p_val) {
            Csr P;
            P.rows = n; P.nnz = p_rowptr[n];
            std::vector<int32_t> pc(static_cast<size_t>(P.nnz));
            for (int64_t k = 0; k < P.nnz; ++k) {
                NL_REQUIRE(p_col[k] >= 0 && p_col[k] < n, NLGPU_ERR_ARG, "P column out of range");
                pc[size_t(k)] = int32_t(p_col[k]);
            }
            std::vector<i64> prp(p_rowptr, p_rowptr + n + 1);
            P.rowptr.upload(prp.data(), prp.size(), c.stream);
            P.col.upload(pc.data(), pc.size(), c.stream);
            P.val.upload(p_val, size_t(P.nnz), c.stream);
            ilt_build(c, P, ic);
            if (ic.ok) M = &ic;
        }
        const CgResult r = cg_solve(c, A, M, db.p, dx.p, tolerance, max_iterations, x0 != nullptr);
        dx.download(x, size_t(n), c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        if (report) {
            std::memset(report, 0, sizeof *report);
            report->iterations = r.iterations;
            report->residual = r.residual;
            report->reference_residual = r.reference_residual;
            report->preconditioner_ok = M ? 1 : 0;
            report->preconditioner_shifts = ic.attempts;
            report->nnz_solver = A.nnz;
            report->seconds_total = seconds(t0);
        }
        if (!r.converged) conv_status = NLGPU_ERR_NO_CONVERGENCE;
    });
    return solve_status(rc, conv_status);
}

int nlgpu_illt_compute(nlgpu_ctx* ctx, int64_t n, const int64_t* rowptr, const int64_t* col, const double* val,
                       int* computation_info) {
    if (!ctx || n <= 0 || n >= (int64_t(1) << 31) || !rowptr || !col || !val || !computation_info) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        c.plugin_ilt_ready = false;
        NL_REQUIRE(rowptr[0] == 0 && rowptr[n] >= n, NLGPU_ERR_ARG, "row pointers must start at 0 and hold a diagonal per row");
        Csr P;
        P.rows = n; P.nnz = rowptr[n];
        std::vector<int32_t> pc(static_cast<size_t>(P.nnz));
        for (int64_t r = 0; r < n; ++r) {
            NL_REQUIRE(rowptr[r + 1] > rowptr[r], NLGPU_ERR_ARG, "every row needs its diagonal");
            for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
                NL_REQUIRE(col[k] >= r && col[k] < n && (k == rowptr[r] || col[k] > col[k - 1]), NLGPU_ERR_ARG,
                           "columns must be upper, sorted and in range");
                pc[size_t(k)] = int32_t(col[k]);
            }
        }
        std::vector<i64> prp(rowptr, rowptr + n + 1);
        P.rowptr.upload(prp.data(), prp.size(), c.stream);
        P.col.upload(pc.data(), pc.size(), c.stream);
        P.val.upload(val, size_t(P.nnz), c.stream);
        ilt_build(c, P, c.plugin_ilt);
        c.plugin_ilt_ready = c.plugin_ilt.ok;
        *computation_info = c.plugin_ilt.ok ? 0 : 1;
    });
}

int nlgpu_illt_solve(nlgpu_ctx* ctx, int64_t n, const double* x, double* y) {
    if (!ctx || !x || !y) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.plugin_ilt_ready, NLGPU_ERR_STATE, "nlgpu_illt_compute has not succeeded on this context");
        NL_REQUIRE(n == c.plugin_ilt.n, NLGPU_ERR_ARG, "vector size differs from the factorised matrix");
        dbuf<double> dx, dy;
        dx.upload(x, size_t(n), c.stream);
        dy.resize(size_t(n));
        c.sweep_error.zero(c.stream);
        ilt_apply(c, c.plugin_ilt, dx.p, dy.p);
        dy.download(y, size_t(n), c.stream);
        int err = 0;
        c.sweep_error.download(&err, 1, c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        NL_REQUIRE(err == 0, NLGPU_ERR_TIMEOUT, "a triangular sweep gave up waiting for its data");
    });
}

int nlgpu_illt_solve_f32(nlgpu_ctx* ctx, int64_t n, int sweeps, const float* x, float* y) {
    if (!ctx || !x || !y || sweeps == 0 || sweeps > 4096) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.plugin_ilt_ready, NLGPU_ERR_STATE, "nlgpu_illt_compute has not succeeded on this context");
        NL_REQUIRE(n == c.plugin_ilt.n, NLGPU_ERR_ARG, "vector size differs from the factorised matrix");
        dbuf<float> dx, dy;
        dx.upload(x, size_t(n), c.stream);
        dy.resize(size_t(n));
        c.sweep_error.zero(c.stream);
        ilt_apply32(c, c.plugin_ilt, dx.p, dy.p, std::max(sweeps, 0));
        dy.download(y, size_t(n), c.stream);
        int err = 0;
        c.sweep_error.download(&err, 1, c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        NL_REQUIRE(err == 0, NLGPU_ERR_TIMEOUT, "a triangular sweep gave up waiting for its data");
    });
}

namespace {
// assembled system + ILLT + FP32 matrix + prepared network, for training and gradient checks
void ensure_learning_state(Ctx& c) {
    NL_REQUIRE(c.inner_ready, NLGPU_ERR_STATE, "assemble the system first (nlgpu_conductivity_matrix_2d)");
    NL_REQUIRE(c.symmetric, NLGPU_ERR_UNSUPPORTED, "the learned correction needs a symmetric system");
    if (!c.local_ready) build_local(c);
    if (!c.ilt.ok || c.ilt.n != c.local.rows || c.ilt.approximate) ilt_build(c, c.local, c.ilt);
    NL_REQUIRE(c.ilt.ok, NLGPU_ERR_NUMERICAL, "ILLT failed on the local matrix");
    if (!c.full.up_ok && c.full.val32.n != size_t(c.full.nnz))
        matrix_to_f32(c, c.full, c.fp32_symmetric ? &c.inner : nullptr);
    if (!(c.mp.ready && c.mp.n == c.local.rows)) mpnn_prepare(c, c.local);
}
}  // namespace

int nlgpu_mpnn_set_weights(nlgpu_ctx* ctx, const float* params) {
    if (!ctx || !params) return NLGPU_ERR_ARG;
    return guarded([&] { mpnn_set_weights(*ctx, params); NL_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

int nlgpu_mpnn_set_enabled(nlgpu_ctx* ctx, int enabled) {
    if (!ctx) return NLGPU_ERR_ARG;
    ctx->mp.use = enabled != 0;
    return NLGPU_OK;
}

int nlgpu_mpnn_get_weights(nlgpu_ctx* ctx, float* params) {
    if (!ctx || !params) return NLGPU_ERR_ARG;
    return guarded([&] {
        NL_REQUIRE(ctx->mp.params.n == size_t(MPNN_PARAMS), NLGPU_ERR_STATE, "no weights yet");
        mpnn_get_weights(*ctx, params);
    });
}

int nlgpu_mpnn_train(nlgpu_ctx* ctx, const nlgpu_train_options* options, nlgpu_train_report* report) {
    if (!ctx || !options) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        ensure_learning_state(c);
        MpnnTrainOptions o;
        o.right_hand_sides = options->right_hand_sides;
        o.epochs = options->epochs;
        o.batch = options->batch;
        o.learning_rate = options->learning_rate;
        o.seed = options->seed;
        MpnnTrainResult r;
        mpnn_train(c, c.full, c.ilt, c.rhs.p, o, r);
        c.mp.weights_set = true;
        if (report) {
            report->samples = r.samples; report->steps = r.steps;
            report->loss_illt = r.loss_illt; report->loss_first = r.loss_first; report->loss_last = r.loss_last;
            report->seconds_harvest = r.seconds_harvest; report->seconds_train = r.seconds_train;
            report->validation_iterations_learned = r.validation_iterations_learned;
            report->validation_iterations_illt = r.validation_iterations_illt;
            report->validation_seconds_learned = r.validation_seconds_learned;
            report->validation_seconds_illt = r.validation_seconds_illt;
            report->learned_enabled = r.learned_enabled ? 1 : 0;
        }
    });
}

int nlgpu_mpnn_loss_grad(nlgpu_ctx* ctx, const float* r, const float* e, float* z, float* p, double* loss,
                         float* grad) {
    if (!ctx || !r || !e) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        ensure_learning_state(c);
        const i64 n = c.full.rows;
        dbuf<float> dr, de, dz, dp;
        dbuf<double> num_ee;
        dr.upload(r, size_t(n), c.stream);
        de.upload(e, size_t(n), c.stream);
        dz.resize(size_t(n)); dp.resize(size_t(n)); num_ee.resize(2);
        c.mp.grads.zero(c.stream);
        ilt_apply32(c, c.ilt, dr.p, dz.p, c.ilt_sweeps);
        mpnn_backward(c, c.full, dr.p, dz.p, de.p, dp.p, num_ee.p, num_ee.p + 1);
        double h[2];
        num_ee.download(h, 2, c.stream);
        if (z) dz.download(z, size_t(n), c.stream);
        if (p) dp.download(p, size_t(n), c.stream);
        if (grad) c.mp.grads.download(grad, size_t(MPNN_PARAMS), c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        c.mp.grads.zero(c.stream);
        mpnn_check(c);
        if (loss) *loss = h[0] / h[1];
    });
}

int nlgpu_nonstationary_2d_compute(nlgpu_ctx* ctx, double time_step, const double* initial) {
    if (!ctx || !(time_step > 0.0)) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready && c.model_ready, NLGPU_ERR_STATE, "mesh and model must be set");
        // nonstationary_heat_equation_solver_2d::compute (nonstationary_heat_equation_solver_2d.hpp:63-88)
        NL_REQUIRE(!(c.model.nonlocal() && c.cond_field.n), NLGPU_ERR_UNSUPPORTED, "variable conductivity with a nonlocal model");
        ensure_boundary(c);
        c.symmetric = true;
        if (c.model.nonlocal()) ensure_neighbours(c);
        build_patterns(c, !c.model.nonlocal(), true, c.inner, &c.bound, &c.full, &c.full_from_upper);
        c.ff_assembly = c.assembly_precision == NLGPU_ASSEMBLY_FF;
        assemble_full(c);
        boundary_matrix_terms(c);   // convection before the time-step scaling (nonstationary_heat_equation_solver_2d.hpp:74)
        c.neumann = false;
        build_patterns(c, true, true, c.capacity_m, nullptr, &c.capacity_full, &c.capacity_map);
        assemble_local(c, c.capacity_m, c.capacity * c.density, 1);
        fill_full_from_upper(c, c.capacity_m, c.capacity_full, c.capacity_map);
        c.time_step = time_step;
        combine_nonstationary(c, time_step);   // K <- dt K + C, unit Dirichlet diagonal, bound <- dt bound
        fill_full_from_upper(c, c.inner, c.full, c.full_from_upper);
        c.temperature.resize(size_t(c.n_nodes));
        if (initial) c.temperature.upload(initial, size_t(c.n_nodes), c.stream);
        else c.temperature.zero(c.stream);
        c.rhs.resize(size_t(c.n_nodes));
        c.step_tmp.resize(size_t(c.n_nodes));
        c.step_xd.resize(size_t(c.n_nodes));
        NL_CUDA(cudaStreamSynchronize(c.stream));
        c.inner_ready = false;   // inner now holds dt K + C
        c.nonstationary_ready = true;
    });
}

int nlgpu_nonstationary_2d_step(nlgpu_ctx* ctx, double dirichlet_value, const double* dirichlet_values,
                                double tolerance, int64_t max_iterations, double* temperature, int64_t* iterations) {
    if (!ctx) return NLGPU_ERR_ARG;
    int conv_status = NLGPU_OK;
    const int rc = guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.nonstationary_ready, NLGPU_ERR_STATE, "nonstationary_2d_compute must run first");
        // calc_step (nonstationary_heat_equation_solver_2d.hpp:90-106):
        // f = dt * (flux + source) + C T_prev; f -= dt K_bound x_D; f[D] = x_D; CG from T_prev
        if (dirichlet_values) c.step_xd.upload(dirichlet_values, size_t(c.n_nodes), c.stream);
        const double* radiation = nullptr;
        if (has_radiation(c)) {
            // radiation_condition_2d (radiation_condition_2d.hpp:43-88) on the previous
            // temperature: dt 4 sigma eps int T^3 N_i N_j is added to the system matrix
            // and stays there for the following steps, as in the reference; the
            // vector 3 sigma eps int T^4 N_i joins the fluxes
            c.nl_work.resize(size_t(c.n_nodes));
            c.nl_work.zero(c.stream);
            add_radiation(c, c.temperature.p, c.nl_work.p, 4.0 * c.time_step, 3.0);
            fill_full_from_upper(c, c.inner, c.full, c.full_from_upper);
            radiation = c.nl_work.p;
        }
        nonstationary_rhs(c, dirichlet_value, dirichlet_values != nullptr, radiation);
        const CgResult r = cg_solve(c, c.full, nullptr, c.rhs.p, c.temperature.p, tolerance, max_iterations, true);
        if (temperature) c.temperature.download(temperature, size_t(c.n_nodes), c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        if (iterations) *iterations = r.iterations;
        if (!r.converged) conv_status = NLGPU_ERR_NO_CONVERGENCE;
    });
    return solve_status(rc, conv_status);
}

struct nlgpu_batch {
    nlgpu::Batch* impl = nullptr;
    int64_t count = 0;
};

int nlgpu_batch_create(nlgpu_batch** batch, int64_t count, nlgpu_ctx* const* instances) {
    if (!batch || count <= 0 || !instances) return NLGPU_ERR_ARG;
    return guarded([&] {
        std::vector<Ctx*> v;
        for (int64_t k = 0; k < count; ++k) {
            NL_REQUIRE(instances[k], NLGPU_ERR_ARG, "null instance");
            NL_REQUIRE(!has_radiation(*instances[k]), NLGPU_ERR_UNSUPPORTED,
                       "radiation edges change the matrix every step: step such problems one by one");
            v.push_back(instances[k]);
        }
        auto* b = new nlgpu_batch{};
        try {
            b->impl = batch_create(v);
        } catch (...) {
            delete b;
            throw;
        }
        b->count = count;
        *batch = b;
    });
}

int nlgpu_batch_destroy(nlgpu_batch* batch) {
    if (!batch) return NLGPU_ERR_ARG;
    return guarded([&] {
        batch_destroy(batch->impl);
        delete batch;
    });
}

int nlgpu_batch_step(nlgpu_batch* batch, const double* dirichlet_values, double tolerance, int64_t max_iterations,
                     int64_t* iterations) {
    if (!batch || !dirichlet_values || !(tolerance > 0.0) || max_iterations <= 0) return NLGPU_ERR_ARG;
    return guarded([&] { batch_step(*batch->impl, dirichlet_values, tolerance, max_iterations, iterations); });
}

int nlgpu_batch_temperature(nlgpu_batch* batch, int64_t index, double* temperature) {
    if (!batch || !temperature) return NLGPU_ERR_ARG;
    return guarded([&] { batch_temperature(*batch->impl, index, temperature); });
}

int nlgpu_batch_last_solve(nlgpu_batch* batch, int64_t* inner_iterations, int64_t* outer_iterations, int* fallback) {
    if (!batch || !inner_iterations || !outer_iterations || !fallback) return NLGPU_ERR_ARG;
    return guarded([&] { batch_last_solve(*batch->impl, inner_iterations, outer_iterations, fallback); });
}

int nlgpu_batch_set_method(nlgpu_batch* batch, int method) {
    if (!batch) return NLGPU_ERR_ARG;
    return guarded([&] { batch_set_method(*batch->impl, method); });
}

int nlgpu_batch_sizes(nlgpu_batch* batch, int64_t* rows, int64_t* system_entries) {
    if (!batch || !rows || !system_entries) return NLGPU_ERR_ARG;
    return guarded([&] { batch_sizes(*batch->impl, rows, system_entries); });
}

int nlgpu_stationary_1d(nlgpu_ctx* ctx, int64_t elements, int order, double length, double radius, double local_weight,
                        int influence, double conductivity, double t_left, double q_right, int sin_source,
                        double* temperature) {
    if (!ctx || elements <= 0 || (order != 1 && order != 2) || !(length > 0.0) || !temperature) return NLGPU_ERR_ARG;
    return guarded([&] {
        stationary_1d(*ctx, elements, order, length, radius, local_weight, influence, conductivity, t_left, q_right,
                      sin_source != 0, temperature);
    });
}

int nlgpu_nonstationary_1d_compute(nlgpu_ctx* ctx, int64_t elements, int order, double length, double radius,
                                   double local_weight, int influence, double conductivity, double capacity,
                                   double density, double time_step, int left_kind, int right_kind,
                                   const double* initial_temperature, int64_t* nodes) {
    if (!ctx || elements <= 0 || (order != 1 && order != 2) || !(length > 0.0) || !(time_step > 0.0))
        return NLGPU_ERR_ARG;
    return guarded([&] {
        nonstationary_1d_compute(*ctx, elements, order, length, radius, local_weight, influence, conductivity,
                                 capacity, density, time_step, left_kind, right_kind, initial_temperature);
        if (nodes) *nodes = nonstationary_1d_nodes(*ctx);
    });
}

int nlgpu_nonstationary_1d_convection(nlgpu_ctx* ctx, double heat_transfer_left, double heat_transfer_right) {
    if (!ctx || !(heat_transfer_left >= 0.0) || !(heat_transfer_right >= 0.0)) return NLGPU_ERR_ARG;
    ctx->od_heat_transfer[0] = heat_transfer_left;
    ctx->od_heat_transfer[1] = heat_transfer_right;
    return NLGPU_OK;
}

int nlgpu_nonstationary_1d_step(nlgpu_ctx* ctx, double left_value, double right_value, int sin_source,
                                double* temperature) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] { nonstationary_1d_step(*ctx, left_value, right_value, sin_source != 0, temperature); });
}

int nlgpu_nonstationary_1d_temperature(nlgpu_ctx* ctx, double* temperature) {
    if (!ctx || !temperature) return NLGPU_ERR_ARG;
    return guarded([&] { nonstationary_1d_temperature(*ctx, temperature); });
}

int nlgpu_set_elastic_2d(nlgpu_ctx* ctx, int kind, const double* prm, double* hooke_out) {
    if (!ctx || !prm) return NLGPU_ERR_ARG;
    return guarded([&] {
        Elastic& el = ctx->el;
        double h[6] = {0, 0, 0, 0, 0, 0};   // h11 h12 h66 h22 h16 h26
        if (kind == NLGPU_ELASTIC_ISOTROPIC) {
            // isotropic_elastic_parameters::hooke (elastic_parameters.hpp:64-70)
            const double E = prm[0], nu = prm[1];
            NL_REQUIRE(E > 0.0 && nu > -1.0 && nu < 1.0, NLGPU_ERR_ARG, "isotropic: E > 0, -1 < nu < 1");
            const double v = E / (1.0 - nu * nu);
            h[0] = v; h[1] = nu * v; h[2] = 0.5 * v * (1.0 - nu); h[3] = v;
        } else if (kind == NLGPU_ELASTIC_ORTHOTROPIC || kind == NLGPU_ELASTIC_ANISOTROPIC) {
            // orthotropic_elastic_parameters::hooke (elastic_parameters.hpp:84-90)
            const double Ex = prm[0], Ey = prm[1], nux = prm[2], nuy = prm[3], G = prm[4];
            NL_REQUIRE(Ex > 0.0 && Ey > 0.0 && G > 0.0 && nux * nuy < 1.0, NLGPU_ERR_ARG,
                       "orthotropic: E_x, E_y, G > 0 and nu_x nu_y < 1");
            const double v = 1.0 / (1.0 - nux * nuy);
            const double o11 = Ex * v, o12 = Ex * nuy * v, o66 = G, o22 = Ey * v;
            if (kind == NLGPU_ELASTIC_ORTHOTROPIC) {
                h[0] = o11; h[1] = o12; h[2] = o66; h[3] = o22;
            } else {
                // anisotropic_elastic_parameters::rotate (elastic_parameters.hpp:100-122)
                const double a2 = 2.0 * prm[5];
                const double s2 = std::sin(a2), c2 = std::cos(a2);
                const double c4 = 0.125 * (c2 * c2 - s2 * s2);
                const double diff = o11 - o22, core = o11 + o22 - 2.0 * o12 - 4.0 * o66;
                const double plus = core * (c4 + 0.125), minus = core * (0.125 - c4);
                const double cdiff = diff * (c2 + 0.5), minor = core * c2, s2q = 0.25 * s2;
                h[0] = plus + 0.5 * (o12 + o22 + cdiff) + o66;
                h[1] = minus + o12;
                h[2] = minus + o66;
                h[3] = plus + 0.5 * (o12 + o11 - cdiff) + o66;
                h[4] = s2q * (diff + minor);
                h[5] = s2q * (diff - minor);
            }
        } else {
            NL_REQUIRE(false, NLGPU_ERR_ARG, "unknown elastic parameters kind");
        }
        el.kind = kind;
        for (int k = 0; k < 6; ++k) el.h[k] = h[k];
        if (hooke_out) for (int k = 0; k < 6; ++k) hooke_out[k] = h[k];
        el.hooke_set = true;
        el.assembled = false;
        el.local_ready = false;
    });
}

int nlgpu_add_mechanical_boundary_2d(nlgpu_ctx* ctx, int64_t n_edges, int nodes_per_edge, const int64_t* edges,
                                     int kind_x, double value_x, int kind_y, double value_y) {
    if (!ctx || !edges || n_edges < 0) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.mesh_ready, NLGPU_ERR_STATE, "no mesh");
        NL_REQUIRE(nodes_per_edge == 2 || nodes_per_edge == 3, NLGPU_ERR_UNSUPPORTED, "boundary edges have 2 or 3 nodes");
        for (const int k : {kind_x, kind_y})
            NL_REQUIRE(k >= NLGPU_MECH_NONE && k <= NLGPU_MECH_PRESSURE, NLGPU_ERR_ARG, "unknown mechanical condition");
        MechanicalGroup g;
        g.nen = nodes_per_edge; g.n_edges = n_edges;
        g.kind[0] = kind_x; g.kind[1] = kind_y; g.value[0] = value_x; g.value[1] = value_y;
        std::vector<int32_t> e(size_t(n_edges * nodes_per_edge));
        for (size_t k = 0; k < e.size(); ++k) {
            NL_REQUIRE(edges[k] >= 0 && edges[k] < c.n_nodes, NLGPU_ERR_ARG, "boundary node out of range");
            e[k] = int32_t(edges[k]);
        }
        g.edges.upload(e.data(), e.size(), c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        c.el.groups.push_back(std::move(g));
        c.el.assembled = false;
        c.el.local_ready = false;
    });
}

int nlgpu_clear_mechanical_boundaries(nlgpu_ctx* ctx) {
    if (!ctx) return NLGPU_ERR_ARG;
    ctx->el.groups.clear();
    ctx->el.assembled = false;
    ctx->el.local_ready = false;
    return NLGPU_OK;
}

int nlgpu_stiffness_matrix_2d(nlgpu_ctx* ctx, int part, int64_t* nnz_inner, int64_t* nnz_bound) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(part == NLGPU_PART_FULL || part == NLGPU_PART_LOCAL, NLGPU_ERR_ARG, "part FULL or LOCAL");
        if (part == NLGPU_PART_FULL && c.model.nonlocal()) ensure_neighbours(c);
        elastic_assemble(c, part == NLGPU_PART_LOCAL);
        const Csr& m = part == NLGPU_PART_LOCAL ? c.el.local : c.el.inner;
        if (nnz_inner) *nnz_inner = m.nnz;
        if (nnz_bound) *nnz_bound = part == NLGPU_PART_LOCAL ? 0 : c.el.bound.nnz;
    });
}

int nlgpu_get_stiffness_matrix(nlgpu_ctx* ctx, int which, int64_t* rowptr, int64_t* col, double* val) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(which >= NLGPU_MATRIX_INNER && which <= NLGPU_MATRIX_LOCAL, NLGPU_ERR_ARG, "unknown matrix");
        if (which == NLGPU_MATRIX_LOCAL) {
            NL_REQUIRE(c.el.local_ready, NLGPU_ERR_STATE, "LOCAL stiffness not assembled");
            download_csr(c, c.el.local, rowptr, col, val);
        } else {
            NL_REQUIRE(c.el.assembled, NLGPU_ERR_STATE, "FULL stiffness not assembled");
            download_csr(c, which == NLGPU_MATRIX_INNER ? c.el.inner : c.el.bound, rowptr, col, val);
        }
    });
}

int nlgpu_get_mechanical_rhs(nlgpu_ctx* ctx, double* rhs, double* rhs_init) {
    if (!ctx) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.el.assembled, NLGPU_ERR_STATE, "FULL stiffness not assembled");
        const size_t rows = size_t(2 * c.n_nodes);
        if (rhs) c.el.rhs.download(rhs, rows, c.stream);
        if (rhs_init) c.el.rhs_init.download(rhs_init, rows, c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int nlgpu_equilibrium_equation_2d(nlgpu_ctx* ctx, const nlgpu_solve_options* options, double* displacement,
                                  nlgpu_solve_report* report) {
    if (!ctx || !options || !displacement) return NLGPU_ERR_ARG;
    int conv_status = NLGPU_OK;
    const int rc = guarded([&] {
        Ctx& c = *ctx;
        const auto t0 = std::chrono::steady_clock::now();
        if (report) *report = nlgpu_solve_report{};
        if (c.model.nonlocal()) ensure_neighbours(c);
        elastic_assemble(c, false);
        if (report) report->seconds_assembly = seconds(t0);
        const CgResult r = elastic_solve(c, *options, report);
        c.el.displacement.download(displacement, size_t(2 * c.n_nodes), c.stream);
        NL_CUDA(cudaStreamSynchronize(c.stream));
        if (report) report->seconds_total = seconds(t0);
        if (!r.converged) conv_status = NLGPU_ERR_NO_CONVERGENCE;
    });
    return solve_status(rc, conv_status);
}

int nlgpu_cg_solve_noalloc(void* stream, int64_t n, const int64_t* d_rowptr, const int32_t* d_col, const double* d_val,
                           const double* d_b, double* d_x, double tolerance, int64_t max_iterations, int64_t* iterations,
                           double* residual) {
    if (!iterations || !residual) return NLGPU_ERR_ARG;
    int conv_status = NLGPU_OK;
    const int rc = guarded([&] {
        if (!cg_solve_noalloc(static_cast<cudaStream_t>(stream), n, d_rowptr, d_col, d_val, d_b, d_x, tolerance,
                              max_iterations, iterations, residual))
            conv_status = NLGPU_ERR_NO_CONVERGENCE;
    });
    return solve_status(rc, conv_status);
}

int nlgpu_set_option(nlgpu_ctx* ctx, int option, int value) {
    if (!ctx) return NLGPU_ERR_ARG;
    if (option == NLGPU_OPTION_GLOBAL_SWEEPS) { ctx->force_global_sweeps = value != 0; return NLGPU_OK; }
    if (option == NLGPU_OPTION_ORDERED_PAIRS) { ctx->ordered_pairs = value != 0; return NLGPU_OK; }
    if (option == NLGPU_OPTION_FP32_SYMMETRIC) {
        ctx->fp32_symmetric = value != 0;
        ctx->full.up_ok = false;   // the next mixed solve or stage timing rebuilds the FP32 copy
        ctx->full.val32.release();
        return NLGPU_OK;
    }
    if (option == NLGPU_OPTION_ASSEMBLY_WARPS) {
        if (value != 0 && value != 16 && value != 32) return NLGPU_ERR_ARG;
        ctx->ff_warps_option = value;
        return NLGPU_OK;
    }
    if (option == NLGPU_OPTION_ASSEMBLY_PRECISION) {
        if (value < NLGPU_ASSEMBLY_AUTO || value > NLGPU_ASSEMBLY_FP64) return NLGPU_ERR_ARG;
        ctx->assembly_precision = value;
        ctx->inner_ready = false;   // the next use re-assembles
        return NLGPU_OK;
    }
    return NLGPU_ERR_ARG;
}

int nlgpu_assembly_tuning(nlgpu_ctx* ctx, int* warps, double* sample_ms) {
    if (!ctx || !warps || !sample_ms) return NLGPU_ERR_ARG;
    *warps = ctx->ff_warps_used;
    sample_ms[0] = ctx->ff_tune_ms[0];
    sample_ms[1] = ctx->ff_tune_ms[1];
    return NLGPU_OK;
}

int nlgpu_event_record(nlgpu_ctx* ctx, int slot) {
    if (!ctx || slot < 0 || slot >= 64) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        if (!c.events[slot]) NL_CUDA(cudaEventCreate(&c.events[slot]));
        NL_CUDA(cudaEventRecord(c.events[slot], c.stream));
    });
}

int nlgpu_event_elapsed(nlgpu_ctx* ctx, int a, int b, double* ms) {
    if (!ctx || !ms || a < 0 || b < 0 || a >= 64 || b >= 64) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        NL_REQUIRE(c.events[a] && c.events[b], NLGPU_ERR_STATE, "event slot not recorded");
        NL_CUDA(cudaEventSynchronize(c.events[b]));
        float f = 0.0f;
        NL_CUDA(cudaEventElapsedTime(&f, c.events[a], c.events[b]));
        *ms = double(f);
    });
}

int nlgpu_flush_l2(nlgpu_ctx* ctx, int64_t bytes) {
    if (!ctx || bytes <= 0) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        c.flush.reserve(size_t(bytes));
        NL_CUDA(cudaMemsetAsync(c.flush.p, int(c.flush_value++ & 0xff), size_t(bytes), c.stream));
    });
}

int nlgpu_time_stage(nlgpu_ctx* ctx, int stage, int reps, double* ms) {
    if (!ctx || !ms || reps <= 0) return NLGPU_ERR_ARG;
    return guarded([&] {
        Ctx& c = *ctx;
        cudaEvent_t e0, e1;
        NL_CUDA(cudaEventCreate(&e0));
        NL_CUDA(cudaEventCreate(&e1));
        dbuf<double> x, y;
        dbuf<float> x32, y32;
        NL_REQUIRE(stage >= 0 && stage <= 8, NLGPU_ERR_ARG, "unknown stage");
        dbuf<double> flux_x, flux_y;
        if (stage == 8) {
            NL_REQUIRE(c.temperature.n == size_t(c.n_nodes), NLGPU_ERR_STATE, "solve first (the flux of its temperature)");
            if (c.model.nonlocal()) ensure_neighbours(c);
            flux_x.resize(size_t(c.n_nodes)); flux_y.resize(size_t(c.n_nodes));
        }
        const bool ff_before = c.ff_assembly;
        if (stage == 1 || stage == 7) c.ff_assembly = stage == 7;
        if (stage == 0 || stage == 2 || (stage >= 4 && stage <= 6)) {
            NL_REQUIRE(c.full.nnz > 0, NLGPU_ERR_STATE, "assemble the system first");
            x.resize(size_t(c.n_nodes)); y.resize(size_t(c.n_nodes));
            x32.resize(size_t(c.n_nodes)); y32.resize(size_t(c.n_nodes));
            NL_CUDA(cudaMemsetAsync(x.p, 0, x.bytes(), c.stream));
            NL_CUDA(cudaMemsetAsync(x32.p, 0, x32.bytes(), c.stream));
            if (stage == 2 || stage >= 5) NL_REQUIRE(c.ilt.ok, NLGPU_ERR_STATE, "no ILLT factor");
            if (stage == 4 && !c.full.up_ok && (c.full.val32.n != size_t(c.full.nnz) || !c.full.col16_ok))
                matrix_to_f32(c, c.full, c.symmetric && c.fp32_symmetric ? &c.inner : nullptr);
        }
        if (stage == 1 || stage == 7)
            NL_REQUIRE(c.inner.nnz > 0 && c.model.nonlocal(), NLGPU_ERR_STATE, "no nonlocal pattern");
        if (stage == 3) NL_REQUIRE(c.mesh_ready && c.model_ready, NLGPU_ERR_STATE, "no mesh/model");
        NL_CUDA(cudaEventRecord(e0, c.stream));
        for (int k = 0; k < reps; ++k) {
            if (stage == 0) spmv_full(c, c.full, x.p, y.p);
            else if (stage == 1 || stage == 7) assemble_full(c);
            else if (stage == 2) ilt_apply(c, c.ilt, x.p, y.p);
            else if (stage == 3) find_neighbours(c, c.strategy);
            else if (stage == 4) spmv32(c, c.full, x32.p, y32.p);
            else if (stage == 5) ilt_apply32(c, c.ilt, x32.p, y32.p, 0);
            else if (stage == 6) ilt_apply32(c, c.ilt, x32.p, y32.p, std::max(c.ilt_sweeps, 1));
            else calc_flux(c, c.temperature.p, flux_x.p, flux_y.p);
        }
        NL_CUDA(cudaEventRecord(e1, c.stream));
        NL_CUDA(cudaEventSynchronize(e1));
        float f = 0.0f;
        NL_CUDA(cudaEventElapsedTime(&f, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        c.ff_assembly = ff_before;
        *ms = double(f) / reps;
    });
}

}  // extern "C"

namespace nlgpu {

Model make_model(const nlgpu_model_2d& m) {
    NL_REQUIRE(m.influence >= NLGPU_INFLUENCE_CONSTANT && m.influence <= NLGPU_INFLUENCE_FAST_POLYNOMIAL, NLGPU_ERR_ARG,
               "unknown influence kind");
    NL_REQUIRE(m.conductivity_kind >= 0 && m.conductivity_kind <= 2, NLGPU_ERR_ARG, "unknown conductivity kind");
    NL_REQUIRE(m.n >= 1, NLGPU_ERR_ARG, "powered-distance exponent must be positive");
    Model o{};
    o.influence = m.influence; o.n = m.n; o.p = m.p; o.q = m.q;
    o.r[0] = m.radius[0]; o.r[1] = m.radius[1];
    o.p1 = m.local_weight;
    o.cond_kind = m.conductivity_kind;
    for (int k = 0; k < 3; ++k) o.cond[k] = m.conductivity[k];
    if (o.nonlocal()) {
        NL_REQUIRE(o.r[0] > 0.0 && o.r[1] > 0.0, NLGPU_ERR_ARG, "nonlocal radii must be positive");
        o.inv_r[0] = 1.0 / o.r[0]; o.inv_r[1] = 1.0 / o.r[1];
        const double n = m.n;
        switch (m.influence) {   // normalisations of influence_functions_2d.hpp:44-142
        case NLGPU_INFLUENCE_FAST_POLYNOMIAL:
            o.norm = 2.0 / (std::numbers::pi * o.r[0] * o.r[1]); break;
        case NLGPU_INFLUENCE_POLYNOMIAL:
            NL_REQUIRE(m.p > 0 && m.q >= 1.0 && m.q == std::floor(m.q), NLGPU_ERR_UNSUPPORTED, "polynomial: integer q >= 1");
            o.norm = n * m.p / (4 * o.r[0] * o.r[1] * std::beta(1 / n, 1 / n) * std::beta(2.0 / m.p, m.q + 1)); break;
        case NLGPU_INFLUENCE_EXPONENTIAL:
            NL_REQUIRE(m.p > 0 && m.q > 0.0, NLGPU_ERR_ARG, "exponential: p > 0, q > 0");
            o.norm = (n * m.p * std::pow(4.0, 1 / n) * std::pow(m.q, 2.0 / m.p)) /
                     (8 * o.r[0] * o.r[1] * std::tgamma(2.0 / m.p) * std::beta(0.5, 1 / n)); break;
        default:
            o.norm = std::tgamma(1 + 2 / n) / (4 * o.r[0] * o.r[1] * ipow_host(std::tgamma(1 + 1 / n), 2)); break;
        }
    }
    return o;
}

}  // namespace nlgpu
