// Drives the reference implementation (NonLocFEM's own headers, compiled
// against the Eigen API shim in eigen_shim/) on one problem and dumps every
// intermediate of the thermal hot path as raw little-endian arrays, for the
// golden fixtures under tests/golden/.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into oracle/_ref/ in a
// container that has the reference sources; never shipped, never timed as the
// product.
//
// Usage: ref_driver key=value ...   (see parse() below)
//   mode=stationary2d | nonstationary2d | stationary1d | nonstationary1d | mechanical2d
//
// The stationary 2D branch restates the ten driver lines of
// libraries/solvers/solver_2d/thermal/stationary_heat_equation_solver_2d.hpp:72-103
// (symmetric, linear boundary) so that the CG tolerance can be set; every
// numerical step is the reference's own code.

#include <mesh/mesh_2d/find_neighbours.hpp>
#include <mesh/mesh_2d/mesh_2d_utils.hpp>
#include <solvers/solver_2d/influence_functions_2d.hpp>
#include <solvers/solver_2d/thermal/stationary_heat_equation_solver_2d.hpp>
#include <solvers/solver_2d/thermal/nonstationary_heat_equation_solver_2d.hpp>
#include <solvers/solver_2d/mechanical/equilibrium_equation_2d.hpp>
#include <solvers/solver_1d/influence_functions_1d.hpp>
#include <solvers/solver_1d/thermal/stationary_heat_equation_solver_1d.hpp>
#include <solvers/solver_1d/thermal/nonstationary_heat_equation_solver_1d.hpp>
#include <metamath/finite_elements/finite_elements_1d/element/element_1d_integrate.hpp>
#include <map>            // cuthill_mckee.hpp uses std::multimap without including <map>
#include <unordered_set>
#include <mesh/mesh_2d/cuthill_mckee.hpp>

#include <chrono>
#include <cstdio>
#include <fstream>
#include <map>
#include <numbers>
#include <sstream>
#include <string>

namespace {

using T = double;
using I = int64_t;   // mesh index (the reference's tests use int64_t)
using J = int64_t;   // matrix index (NonLocFEM/main.cpp:15)

std::map<std::string, std::string> cfg;

std::string get(const std::string& k, const std::string& d = "") {
    const auto it = cfg.find(k);
    return it == cfg.end() ? d : it->second;
}
double getd(const std::string& k, double d) { const auto s = get(k); return s.empty() ? d : std::stod(s); }

std::string outdir;
std::ofstream manifest;

template<class U>
void dump(const std::string& name, const U* data, size_t count, const std::string& shape) {
    std::ofstream f{outdir + "/" + name + ".bin", std::ios::binary};
    f.write(reinterpret_cast<const char*>(data), std::streamsize(sizeof(U) * count));
    const char* dt = std::is_same_v<U, double> ? "f8" : std::is_same_v<U, int64_t> ? "i8" :
                     std::is_same_v<U, uint8_t> ? "u1" : "??";
    manifest << name << ' ' << dt << ' ' << shape << '\n';
}
template<class U>
void dumpv(const std::string& name, const std::vector<U>& v) { dump(name, v.data(), v.size(), std::to_string(v.size())); }
void dumps(const std::string& name, double v) { dump(name, &v, 1, "1"); }

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

template<class Matrix>
void dump_csr(const std::string& name, const Matrix& m) {
    std::vector<int64_t> rp(m.outerIndexPtr(), m.outerIndexPtr() + m.rows() + 1);
    std::vector<int64_t> ci(m.innerIndexPtr(), m.innerIndexPtr() + m.nonZeros());
    std::vector<double> va(m.valuePtr(), m.valuePtr() + m.nonZeros());
    dumpv(name + "_rowptr", rp); dumpv(name + "_col", ci); dumpv(name + "_val", va);
}

std::function<T(const std::array<T, 2>&, const std::array<T, 2>&)> make_influence(const std::array<T, 2>& r) {
    namespace inf = nonlocal::solver_2d::influence;
    const std::string kind = get("influence", "fast_polynomial");
    const size_t n = size_t(getd("n", 2)), p = size_t(getd("p", 2));
    if (kind == "fast_polynomial") return inf::fast_polynomial<T>{r};
    if (kind == "polynomial") return inf::polynomial<T>{r, n, p, size_t(getd("q", 1))};
    if (kind == "exponential") return inf::exponential<T>{r, n, p, getd("q", 0.5)};
    if (kind == "constant") return inf::constant<T>{r, n};
    throw std::domain_error{"unknown influence " + kind};
}

// lambda(x, y) = 1 + 0.5 sin(2 pi x) cos(pi y): with a nonlocal model this makes
// the reference's system non-symmetric (problem_settings::is_symmetric)
T conductivity_wave(const std::array<T, 2>& x) {
    return 1.0 + 0.5 * std::sin(2.0 * std::numbers::pi * x[0]) * std::cos(std::numbers::pi * x[1]);
}

nonlocal::solver_2d::thermal::raw_conductivity_t<T> make_conductivity() {
    const std::string c = get("conductivity", "1");
    std::stringstream s{c};
    std::vector<T> v; std::string tok;
    while (std::getline(s, tok, ',')) v.push_back(std::stod(tok));
    using namespace nonlocal;
    if (get("conductivity_field") == "wave")   // a spatially varying isotropic conductivity
        return solver_2d::thermal::raw_conductivity_t<T>{coefficient_t<T, 2>{spatial_dependency<T, 2>{conductivity_wave}}};
    if (v.size() == 1) return solver_2d::thermal::raw_conductivity_t<T>{coefficient_t<T, 2>{v[0]}};
    if (v.size() == 2) return solver_2d::thermal::raw_orthotropic_conductivity_t<T>{coefficient_t<T, 2>{v[0]}, coefficient_t<T, 2>{v[1]}};
    return solver_2d::thermal::raw_anisotropic_conductivity_t<T>{coefficient_t<T, 2>{v[0]}, coefficient_t<T, 2>{v[1]}, coefficient_t<T, 2>{v[2]}};
}

// Manufactured solution of the reference's own 2D test
// (tests/solvers_2d/thermal_2d/boundary_conditions_2d.cpp:28-85, mult = 1):
// T = f(x) g(y), f = (-3 alpha (x - 1.01))^(-1/3), g = exp(-(y - 0.5)^2 / 0.1),
// conductivity 10, source chosen so that div(k grad T) + q = 0.
struct manufactured {
    static constexpr T sigma = 5.670374419e-8;   // metamath::constants::Stefan_Boltzmann_Constant
    static constexpr T lambda = 10.0, emissivity = 0.7, A = 1.0, m = 0.5, d = 0.1;
    static T alpha() { return emissivity * sigma / lambda; }
    static T f(T x) { return std::pow(-3. * alpha() * (x - 1.01), -1. / 3.); }
    static T g(T y) { return A * std::exp(-(y - m) * (y - m) / d); }
    static T solution(const std::array<T, 2>& x) { return f(x[0]) * g(x[1]); }
    static T source(const std::array<T, 2>& x) {
        const T a1 = 4 * alpha() * alpha() * lambda;
        constexpr T a2 = 2 * lambda / d;
        const T fx = f(x[0]);
        return -solution(x) * (a1 * (fx * fx * fx * fx * fx * fx) + a2 * (2. / d * ((x[1] - m) * (x[1] - m)) - 1.));
    }
};

// bc.<group>=temperature:<v> | flux:<v> | temperature:manufactured |
//            convection:<heat transfer>,<ambient T> | radiation:<emissivity> |
//            combined:<flux>,<heat transfer>,<ambient T>,<emissivity>
nonlocal::solver_2d::thermal::thermal_boundaries_conditions_2d<T> make_bcs_2d() {
    using namespace nonlocal::solver_2d::thermal;
    thermal_boundaries_conditions_2d<T> bcs;
    for (const auto& [k, v] : cfg) {
        if (k.rfind("bc.", 0) != 0) continue;
        const std::string group = k.substr(3);
        const auto colon = v.find(':');
        const std::string kind = v.substr(0, colon);
        if (v.substr(colon + 1) == "manufactured") {
            bcs[group] = std::make_unique<temperature_2d<T>>([](const std::array<T, 2>& x) { return manufactured::solution(x); });
            continue;
        }
        std::vector<T> a;
        std::stringstream s{v.substr(colon + 1)};
        for (std::string tok; std::getline(s, tok, ',');) a.push_back(std::stod(tok));
        if (kind == "temperature") bcs[group] = std::make_unique<temperature_2d<T>>(a.at(0));
        else if (kind == "flux") bcs[group] = std::make_unique<flux_2d<T>>(a.at(0));
        else if (kind == "convection") bcs[group] = std::make_unique<convection_2d<T>>(a.at(0), a.at(1));
        else if (kind == "radiation") bcs[group] = std::make_unique<radiation_2d<T>>(a.at(0));
        else if (kind == "combined") bcs[group] = std::make_unique<combined_flux_2d<T>>(a.at(0), a.at(1), a.at(2), a.at(3));
        else throw std::domain_error{"unknown bc " + kind};
    }
    return bcs;
}

void dump_mesh(const nonlocal::mesh::mesh_2d<T, I>& mesh) {
    const auto& c = mesh.container();
    std::vector<double> nodes;
    for (const size_t n : c.nodes()) { nodes.push_back(c.node_coord(n)[0]); nodes.push_back(c.node_coord(n)[1]); }
    dump("nodes", nodes.data(), nodes.size(), std::to_string(c.nodes_count()) + ",2");
    const size_t nen = c.nodes_count(0);
    std::vector<int64_t> el;
    for (const size_t e : c.elements_2d()) for (const size_t i : std::ranges::iota_view{0u, nen}) el.push_back(c.node_number(e, i));
    dump("elements", el.data(), el.size(), std::to_string(c.elements_2d_count()) + "," + std::to_string(nen));
    // 1D boundary groups, local node order, as (group_id, nodes...)
    std::vector<std::string> groups(c.groups_1d().begin(), c.groups_1d().end());
    std::sort(groups.begin(), groups.end());
    std::ofstream g{outdir + "/groups_1d.txt"};
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        g << groups[gi] << '\n';
        std::vector<int64_t> be;
        for (const size_t e : c.elements(groups[gi])) for (const size_t n : c.nodes(e)) be.push_back(int64_t(n));
        const size_t nb = c.elements(groups[gi]).size();
        dump("bnd_" + groups[gi], be.data(), be.size(), std::to_string(nb) + "," + std::to_string(nb ? be.size() / nb : 0));
    }
    // quadrature data (A1)
    const size_t E = c.elements_2d_count();
    const auto& el0 = c.element_2d(0);
    const size_t nq = el0.qnodes_count();
    std::vector<double> qc, jac, der;
    for (size_t e = 0; e < E; ++e)
        for (size_t q = 0; q < nq; ++q) { qc.push_back(mesh.quad_coord(e, q)[0]); qc.push_back(mesh.quad_coord(e, q)[1]); jac.push_back(mesh.jacobian(e, q)); }
    for (size_t e = 0; e < E; ++e)
        for (size_t i = 0; i < nen; ++i)
            for (size_t q = 0; q < nq; ++q) { der.push_back(mesh.derivatives(e, i, q)[0]); der.push_back(mesh.derivatives(e, i, q)[1]); }
    dump("qcoords", qc.data(), qc.size(), std::to_string(E) + "," + std::to_string(nq) + ",2");
    dump("jacobians", jac.data(), jac.size(), std::to_string(E) + "," + std::to_string(nq));
    dump("derivatives", der.data(), der.size(), std::to_string(E) + "," + std::to_string(nen) + "," + std::to_string(nq) + ",2");
    // element basis tables (A2)
    std::vector<double> qN, qNxi, qNeta, w, centre_weights;
    for (size_t i = 0; i < nen; ++i) for (size_t q = 0; q < nq; ++q) {
        qN.push_back(el0.qN(i, q)); qNxi.push_back(el0.qNxi(i, q)); qNeta.push_back(el0.qNeta(i, q));
    }
    for (size_t q = 0; q < nq; ++q) w.push_back(el0.weight(q));
    for (size_t i = 0; i < nen; ++i) centre_weights.push_back(el0.N(i, {0.0, 0.0}));
    dump("basis_qN", qN.data(), qN.size(), std::to_string(nen) + "," + std::to_string(nq));
    dump("basis_qNxi", qNxi.data(), qNxi.size(), std::to_string(nen) + "," + std::to_string(nq));
    dump("basis_qNeta", qNeta.data(), qNeta.size(), std::to_string(nen) + "," + std::to_string(nq));
    dumpv("basis_weights", w);
    dumpv("basis_centre", centre_weights);
    const auto centres = nonlocal::mesh::utils::approx_centers_of_elements(c);
    std::vector<double> cc;
    for (const auto& x : centres) { cc.push_back(x[0]); cc.push_back(x[1]); }
    dump("centres", cc.data(), cc.size(), std::to_string(E) + ",2");
}

void dump_neighbours(const nonlocal::mesh::mesh_2d<T, I>& mesh) {
    std::vector<int64_t> off{0}, lst;
    for (const size_t e : mesh.container().elements_2d()) {
        for (const I n : mesh.neighbours(e)) lst.push_back(n);
        off.push_back(int64_t(lst.size()));
    }
    dumpv("neigh_offsets", off); dumpv("neigh_list", lst);
    const auto& inf = mesh.get_influences();
    if (!inf.empty()) dump("search_radius", inf.begin()->second.radius.data(), 2, "2");
}

// mesh::utils::cuthill_mckee (cuthill_mckee.hpp:166-171) for the local and,
// when the mesh has neighbours, the nonlocal node graph, plain and with
// reverse = true; then, with renumber=local|nonlocal[_reverse], the mesh is
// renumbered by that permutation (mesh_2d::renumbering, mesh_2d.hpp:258-262)
// and everything after this point runs on the renumbered mesh.
void cuthill_mckee_and_renumber(nonlocal::mesh::mesh_2d<T, I>& mesh, const bool nonlocal_graph) {
    std::map<std::string, std::vector<size_t>> perms;
    for (const bool only_local : {true, false}) {
        if (!only_local && !nonlocal_graph) continue;
        for (const bool reverse : {false, true}) {
            const std::string name = std::string{"cm_"} + (only_local ? "local" : "nonlocal") + (reverse ? "_reverse" : "");
            perms[name] = nonlocal::mesh::utils::cuthill_mckee(mesh, only_local, reverse);
            std::vector<int64_t> p(perms[name].begin(), perms[name].end());
            dumpv(name, p);
        }
    }
    const std::string rn = get("renumber");
    if (rn.empty()) return;
    const auto& c = mesh.container();
    std::vector<double> nodes;
    for (const size_t n : c.nodes()) { nodes.push_back(c.node_coord(n)[0]); nodes.push_back(c.node_coord(n)[1]); }
    dump("nodes_before_renumbering", nodes.data(), nodes.size(), std::to_string(c.nodes_count()) + ",2");
    mesh.renumbering(perms.at("cm_" + rn));
}

// heat_equation_solution_2d::calc_flux (heat_equation_solution_2d.hpp:99-137):
// the nodal heat flux of a solution, local part -lambda grad T and the
// influence-weighted nonlocal part, averaged from the nearest quadrature
// points to the nodes
template<class Conductivity, class Vector>
void dump_flux(const std::shared_ptr<nonlocal::mesh::mesh_2d<T, I>>& mesh, const Conductivity& conductivity,
               const Vector& temperature) {
    nonlocal::solver_2d::thermal::heat_equation_solution_2d<T, I> solution{mesh, conductivity, temperature};
    const auto& flux = solution.calc_flux();
    dumpv("flux_x", flux[0]);
    dumpv("flux_y", flux[1]);
}

int stationary2d() {
    using namespace nonlocal;
    using namespace nonlocal::solver_2d;
    using namespace nonlocal::solver_2d::thermal;
    auto t0 = std::chrono::steady_clock::now();
    auto mesh = std::make_shared<mesh::mesh_2d<T, I>>(std::filesystem::path{get("mesh")});
    dumps("t_mesh", seconds_since(t0));
    const std::array<T, 2> r = {getd("radius", 0.1), getd("radius2", getd("radius", 0.1))};
    const T p1 = getd("local_weight", 1.0);
    t0 = std::chrono::steady_clock::now();
    if (theory_type(p1) == theory_t::NONLOCAL) {
        mesh::influences<T> infl;
        for (const std::string& g : mesh->container().groups_2d())
            infl[g] = {mesh::powered_distance<T>{size_t(getd("n", 2))}, r};
        const std::string strat = get("strategy", "MAX");
        const auto s = strat == "NO" ? mesh::diameter_expanding_strategy::NO :
                       strat == "MIN" ? mesh::diameter_expanding_strategy::MIN :
                       strat == "MEAN" ? mesh::diameter_expanding_strategy::MEAN : mesh::diameter_expanding_strategy::MAX;
        mesh->neighbours(mesh::find_neighbours(*mesh, infl, s));
    }
    dumps("t_neighbours", seconds_since(t0));
    cuthill_mckee_and_renumber(*mesh, theory_type(p1) == theory_t::NONLOCAL);
    dump_mesh(*mesh);
    dump_neighbours(*mesh);

    parameters_2d<T> parameters;
    for (const std::string& g : mesh->container().groups_2d()) {
        parameters[g].model.local_weight = p1;
        parameters[g].model.influence = make_influence(r);
        parameters[g].physical.conductivity = make_conductivity();
    }
    const auto bcs = make_bcs_2d();
    stationary_equation_parameters_2d<T> aux;
    aux.energy = getd("energy", 0.0);   // the Lagrange row's right-hand side (pure Neumann problems)
    if (get("source") == "manufactured") {
        aux.right_part = [](const std::array<T, 2>& x) { return manufactured::source(x); };
        std::vector<double> sq, exact;
        const size_t nq_total = mesh->quad_shift(mesh->container().elements_2d_count());
        for (size_t q = 0; q < nq_total; ++q) sq.push_back(manufactured::source(mesh->quad_coord(q)));
        for (const size_t n : mesh->container().nodes()) exact.push_back(manufactured::solution(mesh->container().node_coord(n)));
        dumpv("source_q", sq);
        dumpv("exact_solution", exact);
    } else if (const T source = getd("source", 0.0); source != 0.0)
        aux.right_part = [source](const std::array<T, 2>&) { return source; };

    // stationary_heat_equation_solver_2d.hpp:52-84 (linear, Dirichlet present)
    const auto settings = init_problem_settings(mesh->container(), parameters, bcs, true);
    Eigen::Matrix<T, Eigen::Dynamic, 1> f = init_right_part(*mesh, bcs, aux, settings.is_neumann);
    dumpv("rhs_init", std::vector<double>(f.begin(), f.end()));
    std::vector<uint8_t> inner(settings.is_inner_nodes.begin(), settings.is_inner_nodes.end());
    dumpv("is_inner", inner);
    {   // Dirichlet node values as calc_vector forms them (boundary_condition_first_kind_2d.hpp:16-26)
        std::vector<double> xd(mesh->container().nodes_count(), 0.0);
        nonlocal::solver_2d::utils::run_by_boundaries<first_kind_2d, physics_t::THERMAL>(mesh->container(), bcs,
            [&](const first_kind_2d<T, physics_t::THERMAL>& c, const size_t, const size_t node, const size_t) {
                if (xd[node] == T{0}) xd[node] = c(mesh->container().node_coord(node));
            });
        dumpv("dirichlet_values", xd);
    }
    const auto conductivity_parameters = evaluate_conductivity(*mesh, parameters, std::vector<T>(mesh->quad_shift(mesh->container().elements_2d_count()), T{0}));
    t0 = std::chrono::steady_clock::now();
    conductivity_matrix_2d<T, I, J> conductivity{mesh};
    conductivity.compute(conductivity_parameters, settings.is_inner_nodes, settings.is_symmetric(), settings.is_neumann);
    convection_condition_2d(conductivity.matrix().inner(), *mesh, bcs);   // a no-op without convection groups
    dumps("t_assembly", seconds_since(t0));
    const size_t rows = mesh->container().nodes_count() + settings.is_neumann;
    Eigen::Matrix<T, Eigen::Dynamic, 1> temperature_prev = Eigen::Matrix<T, Eigen::Dynamic, 1>::Zero(rows);
    Eigen::Matrix<T, Eigen::Dynamic, 1> residual = conductivity.matrix().inner().template selfadjointView<Eigen::Upper>() * temperature_prev;
    Eigen::Matrix<T, Eigen::Dynamic, 1> residual_rad = Eigen::Matrix<T, Eigen::Dynamic, 1>::Zero(rows);
    if (!settings.is_neumann) {
        first_kind_matrix_fill_2d(conductivity.matrix().inner(), residual_rad, *mesh, bcs);
        boundary_condition_first_kind_2d(f, *mesh, bcs, conductivity.matrix().bound());
    }
    dump_csr("K_inner", conductivity.matrix().inner());
    dump_csr("K_bound", conductivity.matrix().bound());
    dumpv("rhs", std::vector<double>(f.begin(), f.end()));
    residual -= residual_rad + f;
    if (settings.is_nonlinear_boundary) {
        // radiation: the reference's own fixed-point loop
        // (stationary_heat_equation_solver_2d.hpp:66-116, Eigen::ConjugateGradient per step)
        stationary_equation_parameters_2d<T> nl = aux;
        nl.tolerance = getd("nonlinear_tolerance", nl.tolerance);
        nl.max_iterations = size_t(getd("nonlinear_max_iterations", double(nl.max_iterations)));
        t0 = std::chrono::steady_clock::now();
        auto solution = stationary_heat_equation_solver_2d<J>(mesh, parameters, bcs, nl);
        dumps("t_cg", seconds_since(t0));
        dumpv("temperature", solution.temperature());
        dumpv("flux_x", solution.flux()[0]);
        dumpv("flux_y", solution.flux()[1]);
        return 0;
    }
    if (!settings.is_symmetric()) {
        // stationary_heat_equation_solver_2d.hpp:105-108: full storage, Eigen::BiCGSTAB
        std::vector<double> lq;
        const size_t nq_total = mesh->quad_shift(mesh->container().elements_2d_count());
        for (size_t q = 0; q < nq_total; ++q) lq.push_back(conductivity_wave(mesh->quad_coord(q)));
        dumpv("conductivity_q", lq);
        t0 = std::chrono::steady_clock::now();
        const Eigen::BiCGSTAB<Eigen::SparseMatrix<T, Eigen::RowMajor, J>> solver{conductivity.matrix().inner()};
        const Eigen::Matrix<T, Eigen::Dynamic, 1> delta = solver.solve(residual);
        dumps("t_cg", seconds_since(t0));
        const Eigen::Matrix<T, Eigen::Dynamic, 1> temperature = temperature_prev - delta;
        dumpv("temperature", std::vector<double>(temperature.begin(), temperature.end()));
        dumps("cg_iterations", double(solver.iterations()));
        dumps("cg_residual", double(solver.error()));
        const auto Ax = conductivity.matrix().inner() * temperature;
        dumps("true_residual", (f - Ax).norm() / f.norm());
        dump_flux(mesh, conductivity_parameters, temperature);
        return 0;
    }

    t0 = std::chrono::steady_clock::now();
    conductivity_matrix_2d<T, I, J> conductivity_local{mesh};
    conductivity_local.nodes_for_processing(std::ranges::iota_view<size_t, size_t>{0u, mesh->container().nodes_count()});
    conductivity_local.compute(conductivity_parameters, settings.is_inner_nodes, settings.is_symmetric(), settings.is_neumann, assemble_part::LOCAL);
    dumps("t_assembly_local", seconds_since(t0));
    dump_csr("K_local", conductivity_local.matrix().inner());

    slae::conjugate_gradient<T, J> solver{conductivity.matrix().inner()};
    solver.set_tolerance(getd("tolerance", 1e-13));
    t0 = std::chrono::steady_clock::now();
    solver.template init_preconditioner<slae::eigen_ILLT_preconditioner>(conductivity_local.matrix().inner());
    const bool illt_ok = solver.preconditioner().computation_info() == Eigen::Success;
    if (!illt_ok) solver.template init_preconditioner<slae::eigen_identity_preconditioner>();
    dumps("t_illt", seconds_since(t0));
    dumps("illt_ok", illt_ok ? 1.0 : 0.0);
    t0 = std::chrono::steady_clock::now();
    const Eigen::Matrix<T, Eigen::Dynamic, 1> delta = solver.solve(residual);
    dumps("t_cg", seconds_since(t0));
    const Eigen::Matrix<T, Eigen::Dynamic, 1> temperature = temperature_prev - delta;
    dumpv("temperature", std::vector<double>(temperature.begin(), temperature.end()));
    dumps("cg_iterations", double(solver.iterations()));
    dumps("cg_residual", double(solver.residual()));
    const auto Ax = conductivity.matrix().inner().template selfadjointView<Eigen::Upper>() * temperature;
    dumps("true_residual", (f - Ax).norm() / f.norm());
    dump_flux(mesh, conductivity_parameters, temperature);
    return 0;
}

// Nonlocal plane elasticity, DoF = 2 (equilibrium_equation_2d.hpp:19-60): the
// stiffness matrices, the right-hand side and the displacement of the
// reference's own code, restated around its solve so the CG tolerance can be
// set.  mbc.<group>=<x>,<y> with d:<value> (displacement_2d) or p:<value>
// (pressure_2d) per component, e.g. mbc.left=d:0,d:0 mbc.right=p:1,p:0.
int mechanical2d() {
    using namespace nonlocal;
    using namespace nonlocal::solver_2d;
    using namespace nonlocal::solver_2d::mechanical;
    auto mesh = std::make_shared<mesh::mesh_2d<T, I>>(std::filesystem::path{get("mesh")});
    const std::array<T, 2> r = {getd("radius", 0.1), getd("radius2", getd("radius", 0.1))};
    const T p1 = getd("local_weight", 1.0);
    if (theory_type(p1) == theory_t::NONLOCAL) {
        mesh::influences<T> infl;
        for (const std::string& g : mesh->container().groups_2d())
            infl[g] = {mesh::powered_distance<T>{size_t(getd("n", 2))}, r};
        mesh->neighbours(mesh::find_neighbours(*mesh, infl, mesh::diameter_expanding_strategy::MAX));
    }
    dump_mesh(*mesh);
    dump_neighbours(*mesh);
    raw_mechanical_parameters<T> parameters;
    for (const std::string& g : mesh->container().groups_2d()) {
        parameters[g].model.local_weight = p1;
        parameters[g].model.influence = make_influence(r);
        isotropic_elastic_parameters<T> elastic;
        elastic.young_modulus = getd("young_modulus", 210.0);
        elastic.poissons_ratio = getd("poissons_ratio", 0.3);
        parameters[g].physical.elastic = elastic;
    }
    mechanical_boundaries_conditions_2d<T> bcs;
    for (const auto& [k, v] : cfg) {
        if (k.rfind("mbc.", 0) != 0) continue;
        auto& cond = bcs[k.substr(4)];
        std::stringstream s{v};
        std::string part;
        for (size_t d = 0; d < 2 && std::getline(s, part, ','); ++d) {
            const T value = std::stod(part.substr(2));
            if (part[0] == 'd') cond[d] = std::make_unique<displacement_2d<T>>(value);
            else cond[d] = std::make_unique<pressure_2d<T>>(value);
        }
    }
    // equilibrium_equation_2d.hpp:26-45
    const auto settings = init_problem_settings(mesh->container(), parameters, bcs);
    std::vector<uint8_t> inner(settings.is_inner_nodes.begin(), settings.is_inner_nodes.end());
    dumpv("is_inner", inner);
    const auto evaluated = evaluate_mechanical_parameters(*mesh, parameters);
    stiffness_matrix<T, I, J> stiffness{mesh};
    stiffness.compute(evaluated, settings);
    Eigen::Matrix<T, Eigen::Dynamic, 1> f = Eigen::Matrix<T, Eigen::Dynamic, 1>::Zero(stiffness.matrix().inner().cols());
    boundary_condition_second_kind_2d(f, *mesh, bcs);
    dumpv("rhs_init", std::vector<double>(f.begin(), f.end()));
    boundary_condition_first_kind_2d(f, *mesh, bcs, stiffness.matrix().bound());
    dump_csr("K_inner", stiffness.matrix().inner());
    dump_csr("K_bound", stiffness.matrix().bound());
    dumpv("rhs", std::vector<double>(f.begin(), f.end()));
    stiffness_matrix<T, I, J> local{mesh};
    local.nodes_for_processing(std::ranges::iota_view<size_t, size_t>{0u, mesh->container().nodes_count()});
    local.compute(evaluated, settings, assemble_part::LOCAL);
    dump_csr("K_local", local.matrix().inner());
    slae::conjugate_gradient<T, J> solver{stiffness.matrix().inner()};
    solver.set_tolerance(getd("tolerance", 1e-13));
    solver.template init_preconditioner<slae::eigen_ILLT_preconditioner>(local.matrix().inner());
    const bool illt_ok = solver.preconditioner().computation_info() == Eigen::Success;
    if (!illt_ok) solver.template init_preconditioner<slae::eigen_identity_preconditioner>();
    dumps("illt_ok", illt_ok ? 1.0 : 0.0);
    const Eigen::Matrix<T, Eigen::Dynamic, 1> u = solver.solve(f);
    dumpv("displacement", std::vector<double>(u.begin(), u.end()));
    dumps("cg_iterations", double(solver.iterations()));
    const auto Ku = stiffness.matrix().inner().template selfadjointView<Eigen::Upper>() * u;
    dumps("true_residual", (f - Ku).norm() / f.norm());
    return 0;
}

int nonstationary2d() {
    using namespace nonlocal;
    using namespace nonlocal::solver_2d;
    using namespace nonlocal::solver_2d::thermal;
    auto mesh = std::make_shared<mesh::mesh_2d<T, I>>(std::filesystem::path{get("mesh")});
    const std::array<T, 2> r = {getd("radius", 0.1), getd("radius2", getd("radius", 0.1))};
    const T p1 = getd("local_weight", 1.0);
    if (theory_type(p1) == theory_t::NONLOCAL) {
        mesh::influences<T> infl;
        for (const std::string& g : mesh->container().groups_2d())
            infl[g] = {mesh::powered_distance<T>{size_t(getd("n", 2))}, r};
        mesh->neighbours(mesh::find_neighbours(*mesh, infl, mesh::diameter_expanding_strategy::MAX));
    }
    dump_mesh(*mesh);
    dump_neighbours(*mesh);
    parameters_2d<T> parameters;
    for (const std::string& g : mesh->container().groups_2d()) {
        parameters[g].model.local_weight = p1;
        parameters[g].model.influence = make_influence(r);
        parameters[g].physical.conductivity = make_conductivity();
        parameters[g].physical.capacity = getd("capacity", 1.0);
        parameters[g].physical.density = getd("density", 1.0);
    }
    const T dt = getd("dt", 1e-3);
    const size_t steps = size_t(getd("steps", 10));
    const T omega = getd("omega", 10.0);           // Dirichlet value amp*sin(omega*t) on `dirichlet_group`
    const std::string dgroup = get("dirichlet_group", "left");
    nonstationary_heat_equation_solver_2d<T, I, J> solver{mesh, dt};
    const auto bcs_at = [&](const T t) {   // the bc.<group> entries, plus the time-dependent temperature
        thermal_boundaries_conditions_2d<T> bcs = make_bcs_2d();
        bcs[dgroup] = std::make_unique<temperature_2d<T>>(std::sin(omega * t));
        return bcs;
    };
    const T initial = getd("initial", 0.0);
    solver.compute(parameters, bcs_at(0), [initial](const std::array<T, 2>&) { return initial; });
    std::vector<double> history;
    for (size_t s = 1; s <= steps; ++s) {
        solver.calc_step(bcs_at(T(s) * dt), [](const std::array<T, 2>&) { return T{0}; });
        history.insert(history.end(), solver.temperature().begin(), solver.temperature().end());
    }
    dump("temperature_history", history.data(), history.size(), std::to_string(steps) + "," + std::to_string(mesh->container().nodes_count()));
    return 0;
}

int stationary1d() {
    using namespace nonlocal;
    using namespace nonlocal::solver_1d;
    using namespace nonlocal::solver_1d::thermal;
    const size_t elements = size_t(getd("elements", 1000));
    const size_t order = size_t(getd("order", 2));
    const T r = getd("radius", 0.1);
    const T p1 = getd("local_weight", 0.5);
    std::unique_ptr<metamath::finite_element::element_1d_integrate<T>> element;
    using metamath::finite_element::element_1d_integrate;
    using metamath::finite_element::element_1d;
    using metamath::finite_element::lagrangian_element_1d;
    using metamath::finite_element::quadrature_1d;
    using metamath::finite_element::gauss;
    const size_t qn = size_t(getd("quadrature", double(order + 1)));
    if (order == 1 && qn == 2) element = std::make_unique<element_1d_integrate<T>>(std::make_unique<element_1d<T, lagrangian_element_1d, 1>>(), quadrature_1d<T, gauss, 2>{});
    else if (order == 2 && qn == 3) element = std::make_unique<element_1d_integrate<T>>(std::make_unique<element_1d<T, lagrangian_element_1d, 2>>(), quadrature_1d<T, gauss, 3>{});
    else throw std::domain_error{"unsupported 1D element/quadrature"};
    auto mesh = std::make_shared<mesh::mesh_1d<T>>(std::move(element), std::vector<mesh::segment_data<T>>{{.length = 1, .search_radius = r, .elements = elements}});
    parameters_1d<T> parameters(1);
    parameters[0].model.local_weight = p1;
    const std::string kind = get("influence", "bell");
    if (kind == "bell") parameters[0].model.influence = influence::polynomial_1d<T, 2, 1>{r};
    else if (kind == "triangle") parameters[0].model.influence = influence::polynomial_1d<T, 1, 1>{r};
    else if (kind == "normal") parameters[0].model.influence = influence::normal_distribution_1d<T>{r};
    else parameters[0].model.influence = influence::constant_1d<T>{r};
    parameters[0].physical.conductivity = getd("conductivity", 1.0);
    thermal_boundaries_conditions_1d<T> bcs;
    bcs.front() = std::make_unique<temperature_1d<T>>(getd("left_temperature", 0.0));
    bcs.back() = std::make_unique<flux_1d<T>>(getd("right_flux", 1.0));
    stationary_equation_parameters_1d<T> aux;
    if (get("source", "sin") == "sin") aux.right_part = [](const T x) { return std::sin(std::numbers::pi_v<T> * x); };
    const auto t0 = std::chrono::steady_clock::now();
    const auto solution = stationary_heat_equation_solver_1d<T, J>(mesh, parameters, bcs, aux);
    dumps("t_solve", seconds_since(t0));
    dumpv("temperature", solution.temperature());
    return 0;
}

// nonstationary_heat_equation_solver_1d (nonstationary_heat_equation_solver_1d.hpp:24-259):
// one segment [0, 1], constant conductivity, capacity and density; each end a
// temperature, a flux or a convection (left=t:<v> | f:<v> | c:<h>,<T_ambient>,
// right=...), source sin(pi x) or
// none, initial temperature 0 or sin(pi x); `steps` calls of calc_step, the
// temperature after each dumped as history (steps x n).
int nonstationary1d() {
    using namespace nonlocal;
    using namespace nonlocal::solver_1d;
    using namespace nonlocal::solver_1d::thermal;
    const size_t elements = size_t(getd("elements", 200));
    const size_t order = size_t(getd("order", 2));
    const T r = getd("radius", 0.1);
    const T p1 = getd("local_weight", 0.5);
    using metamath::finite_element::element_1d_integrate;
    using metamath::finite_element::element_1d;
    using metamath::finite_element::lagrangian_element_1d;
    using metamath::finite_element::quadrature_1d;
    using metamath::finite_element::gauss;
    std::unique_ptr<element_1d_integrate<T>> element;
    if (order == 1) element = std::make_unique<element_1d_integrate<T>>(std::make_unique<element_1d<T, lagrangian_element_1d, 1>>(), quadrature_1d<T, gauss, 2>{});
    else if (order == 2) element = std::make_unique<element_1d_integrate<T>>(std::make_unique<element_1d<T, lagrangian_element_1d, 2>>(), quadrature_1d<T, gauss, 3>{});
    else throw std::domain_error{"unsupported 1D element"};
    auto mesh = std::make_shared<mesh::mesh_1d<T>>(std::move(element), std::vector<mesh::segment_data<T>>{{.length = 1, .search_radius = r, .elements = elements}});
    parameters_1d<T> parameters(1);
    parameters[0].model.local_weight = p1;
    const std::string kind = get("influence", "bell");
    if (kind == "bell") parameters[0].model.influence = influence::polynomial_1d<T, 2, 1>{r};
    else if (kind == "triangle") parameters[0].model.influence = influence::polynomial_1d<T, 1, 1>{r};
    else if (kind == "normal") parameters[0].model.influence = influence::normal_distribution_1d<T>{r};
    else parameters[0].model.influence = influence::constant_1d<T>{r};
    parameters[0].physical.conductivity = getd("conductivity", 1.0);
    parameters[0].physical.capacity = getd("capacity", 1.0);
    parameters[0].physical.density = getd("density", 1.0);
    const auto side = [](const std::string& spec) -> std::unique_ptr<thermal_boundary_condition_1d<T>> {
        const T v = std::stod(spec.substr(2));
        if (spec[0] == 't') return std::make_unique<temperature_1d<T>>(v);
        if (spec[0] == 'c') {   // c:<heat transfer>,<ambient temperature>
            const size_t comma = spec.find(',');
            return std::make_unique<convection_1d<T>>(v, std::stod(spec.substr(comma + 1)));
        }
        return std::make_unique<flux_1d<T>>(v);
    };
    thermal_boundaries_conditions_1d<T> bcs;
    bcs.front() = side(get("left", "t:0"));
    bcs.back() = side(get("right", "f:1"));
    const T dt = getd("dt", 1e-3);
    nonstationary_heat_equation_solver_1d<T, J> solver{mesh, parameters, dt};
    if (get("initial", "zero") == "sin")
        solver.initialize_temperature(std::function<T(const T)>{[](const T x) { return std::sin(std::numbers::pi_v<T> * x); }});
    solver.compute(bcs);
    std::optional<std::function<T(const T)>> source;
    if (get("source", "sin") == "sin") source = [](const T x) { return std::sin(std::numbers::pi_v<T> * x); };
    const size_t steps = size_t(getd("steps", 5));
    std::vector<double> history;
    for (size_t s = 0; s < steps; ++s) {
        solver.calc_step(bcs, source);
        const auto& t = solver.temperature();
        history.insert(history.end(), t.begin(), t.end());
    }
    dump("history", history.data(), history.size(), std::to_string(steps) + "," + std::to_string(mesh->nodes_count()));
    return 0;
}

} // namespace

int main(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        const auto eq = a.find('=');
        if (eq != std::string::npos) cfg[a.substr(0, eq)] = a.substr(eq + 1);
    }
    outdir = get("out", ".");
    std::filesystem::create_directories(outdir);
    manifest.open(outdir + "/manifest.txt");
    try {
        const std::string mode = get("mode", "stationary2d");
        if (mode == "stationary2d") return stationary2d();
        if (mode == "nonstationary2d") return nonstationary2d();
        if (mode == "mechanical2d") return mechanical2d();
        if (mode == "stationary1d") return stationary1d();
        if (mode == "nonstationary1d") return nonstationary1d();
        std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "ref_driver: %s\n", e.what());
    }
    return 1;
}
