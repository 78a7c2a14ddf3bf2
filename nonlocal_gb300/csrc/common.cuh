// Shared definitions of the nlgpu library: error handling, device buffers,
// element tables, the per-problem context and small device utilities.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <array>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/nlgpu.h"

namespace nlgpu {

using i64 = int64_t;

// ------------------------------------------------------------------ errors
struct error : std::runtime_error {
    int code;
    error(int c, const std::string& what) : std::runtime_error{what}, code{c} {}
};

[[noreturn]] inline void cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    const int code = e == cudaErrorMemoryAllocation ? NLGPU_ERR_OUT_OF_MEMORY : NLGPU_ERR_CUDA;
    throw error{code, std::string{what} + ": " + cudaGetErrorString(e) + " (" + file + ":" + std::to_string(line) + ")"};
}

#define NL_CUDA(call)                                                          \
    do {                                                                       \
        const cudaError_t nl_e_ = (call);                                      \
        if (nl_e_ != cudaSuccess) ::nlgpu::cuda_fail(nl_e_, #call, __FILE__, __LINE__); \
    } while (0)

#define NL_REQUIRE(cond, code, msg)                                            \
    do {                                                                       \
        if (!(cond)) throw ::nlgpu::error{(code), (msg)};                      \
    } while (0)

// Kernel launches issued by the library (all host threads).  A launch made
// while this thread captures a stream into a graph counts into the capture's
// own counter instead, and the graph's kernels count when the graph launches.
extern std::atomic<int64_t> g_launches;
extern thread_local int64_t* t_capture_sink;

struct CountCaptured {
    int64_t kernels = 0;
    int64_t* prev;
    CountCaptured() : prev{t_capture_sink} { t_capture_sink = &kernels; }
    ~CountCaptured() { t_capture_sink = prev; }
    CountCaptured(const CountCaptured&) = delete;
    CountCaptured& operator=(const CountCaptured&) = delete;
};

inline void count_launch() {
    if (t_capture_sink) ++*t_capture_sink;
    else g_launches.fetch_add(1, std::memory_order_relaxed);
}

#define NL_LAUNCH(kernel, grid, block, smem, stream, ...)                      \
    do {                                                                       \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);            \
        ::nlgpu::count_launch();                                               \
        NL_CUDA(cudaGetLastError());                                           \
    } while (0)

// Diagnostics: with NLGPU_DEBUG_TIMING set in the environment, mark() prints
// the wall time since the previous mark (after synchronising the stream).
struct PhaseTimer {
    cudaStream_t stream;
    const char* scope;
    bool on;
    std::chrono::steady_clock::time_point t;
    PhaseTimer(cudaStream_t s, const char* name)
        : stream{s}, scope{name}, on{std::getenv("NLGPU_DEBUG_TIMING") != nullptr}, t{std::chrono::steady_clock::now()} {}
    void mark(const char* what) {
        if (!on) return;
        cudaStreamSynchronize(stream);
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[nlgpu timing] %s/%s %.3f ms\n", scope, what,
                     std::chrono::duration<double, std::milli>(now - t).count());
        t = now;
    }
};

inline unsigned grid_for(i64 n, int block, i64 cap = 152 * 32) {
    i64 g = (n + block - 1) / block;
    if (g > cap) g = cap;
    return unsigned(g < 1 ? 1 : g);
}

// --------------------------------------------------------- device buffers
template<class T>
struct dbuf {
    T* p = nullptr;
    size_t n = 0;
    dbuf() = default;
    dbuf(const dbuf&) = delete;
    dbuf& operator=(const dbuf&) = delete;
    dbuf(dbuf&& o) noexcept : p{o.p}, n{o.n} { o.p = nullptr; o.n = 0; }
    dbuf& operator=(dbuf&& o) noexcept { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; return *this; }
    ~dbuf() { release(); }
    void release() noexcept { if (p) cudaFree(p); p = nullptr; n = 0; }
    void resize(size_t count) {
        if (count == n && p) return;
        release();
        if (count) NL_CUDA(cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T)));
        n = count;
    }
    // grows only; keeps the allocation when it is already large enough
    void reserve(size_t count) { if (count > n) resize(count); }
    void zero(cudaStream_t s) { if (n) NL_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s)); }
    void upload(const T* host, size_t count, cudaStream_t s) {
        resize(count);
        if (count) NL_CUDA(cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T* host, size_t count, cudaStream_t s) const {
        if (count) NL_CUDA(cudaMemcpyAsync(host, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    size_t bytes() const noexcept { return n * sizeof(T); }
};

// ------------------------------------------------------ element tables
constexpr int MAX_NEN = 8;
constexpr int MAX_NQ = 9;

// Shape functions and derivatives at the Gauss points of the reference
// element, q = ix * ny + iy (element_2d_integrate.hpp:69-106), and N_i(0,0).
struct Basis {
    int type = 0, nen = 0, nq = 0;
    double qN[MAX_NEN * MAX_NQ], qNxi[MAX_NEN * MAX_NQ], qNeta[MAX_NEN * MAX_NQ];
    double w[MAX_NQ];
    double centre[MAX_NEN];
    int nearest[MAX_NEN];        // Gauss point nearest to each local node (element_2d_integrate.hpp:87-105)
};
Basis make_basis(int element_type);

// Line elements of boundary groups: 2 nodes / Gauss-1, 3 nodes / Gauss-2
// (vtk_elements_set.hpp:43-52).
struct Basis1d {
    int nen = 0, nq = 0;
    double qN[3 * 2], qNxi[3 * 2], w[2];
};
Basis1d make_basis_1d(int nodes);

// Nonlocal model with the influence normalisation precomputed on the host.
struct Model {
    int influence = NLGPU_INFLUENCE_FAST_POLYNOMIAL, n = 2, p = 2;
    double q = 1.0, r[2] = {0.1, 0.1}, inv_r[2] = {10.0, 10.0}, p1 = 1.0, norm = 1.0;
    int cond_kind = NLGPU_CONDUCTIVITY_ISOTROPIC;
    double cond[3] = {1.0, 0.0, 0.0};
    bool nonlocal() const noexcept { return p1 < 0.999; }   // nonlocal_constants.hpp:22-37
};
Model make_model(const nlgpu_model_2d& m);

// CSR on the device: int64 row pointers, int32 columns.
struct Csr {
    i64 rows = 0, nnz = 0;
    dbuf<i64> rowptr;
    dbuf<int32_t> col;
    dbuf<double> val;
    dbuf<float> val32;
    dbuf<float> rowsum32;        // row sums of the FP64 values (difference-form FP32 SpMV)
    dbuf<int16_t> col16;         // column - row, when every entry's offset fits 16 bits
    bool col16_ok = false;
    // the strictly upper part in FP32 for the symmetric FP32 SpMV (mixed.cu):
    // row pointers, 16-bit offsets column - row and values; each CTA of that
    // SpMV owns a contiguous row range and accumulates into a shared-memory
    // window of the columns its rows reach
    dbuf<i64> up_rp;
    dbuf<uint16_t> up_off;
    dbuf<float> up_val;
    dbuf<int32_t> up_part;       // [up_blocks + 1] first row of each CTA's range
    dbuf<int32_t> up_window;     // [up_blocks] columns from the range's first row to the farthest column
    i64 up_nnz = 0;
    int up_blocks = 0, up_window_max = 0;
    bool up_ok = false;
};

struct BoundaryGroup {
    int kind = NLGPU_BC_TEMPERATURE, nen = 2;
    i64 n_edges = 0;
    double value = 0.0;                 // temperature, or the flux of the second-kind integral
    double heat_transfer = 0.0;         // convection: alpha int N_i N_j in the matrix
    double emissivity = 0.0;            // radiation: sigma eps T^4 (nonlinear)
    dbuf<int32_t> edges;
    dbuf<double> node_values;   // optional, per listed node
    dbuf<i64> upper_index;      // [edge][i][j]: entry (row, col >= row) in the upper inner matrix, or -1
    bool convection() const { return kind == NLGPU_BC_CONVECTION || kind == NLGPU_BC_COMBINED_FLUX; }
    bool radiation() const { return kind == NLGPU_BC_RADIATION || kind == NLGPU_BC_COMBINED_FLUX; }
    bool flux_kind() const { return kind != NLGPU_BC_TEMPERATURE; }
};

// One triangular sweep, level scheduled: rows grouped by level, each level's
// off-diagonal entries in a column-major (ELL) slab so that consecutive
// threads read consecutive entries; padding points at the zero slot n.
struct TriSlab {
    i64 n_levels = 0, entries = 0;
    dbuf<i64> lev_ptr;           // [n_levels + 1] positions in `rows`
    dbuf<i64> slab_base;         // [n_levels]
    dbuf<int32_t> width;         // [n_levels]
    dbuf<int32_t> rows;          // row of each level position
    dbuf<int32_t> col;           // slab columns
    dbuf<i64> src;               // slab entry -> factor value (-1: padding)
    dbuf<i64> diag_src;          // level position -> factor diagonal value
    dbuf<double> val, inv_diag;
    dbuf<float> val32, inv_diag32;
};

// One triangle of the factor for Jacobi sweeps (jacobi.cu): the off-diagonal
// entries of each row divided by the row's diagonal, FP32, in sliced ELL with
// 32-row slices (entry k of row 32 s + l at slice[s] + 32 k + l), so that the
// thread of a row and its 31 neighbours read consecutive words.  Padding
// entries point at their own row with value 0.
struct JacobiSlab {
    i64 entries = 0;
    dbuf<i64> slice;             // [slices + 1] entry offsets
    dbuf<int32_t> col;
    dbuf<i64> src;               // entry -> factor value (-1: padding)
    dbuf<float> val;
};

// Level blocks of a sweep plan for one value type (FP64 or FP32).
struct SweepLayout {
    int farmax = 0;              // most dependencies of one level that lie beyond the ring
    dbuf<int32_t> far_off, far_pos;   // per level: level-order positions the producer prefetches
    int stage_bytes = 0;
    size_t smem_bytes = 0;
    dbuf<unsigned char> blocks;  // per level: values, inverse diagonal, ring slots
    dbuf<i64> val_dst, inv_dst;  // block byte offset of each factor value source
};

// Triangular sweep fed by TMA bulk copies with a shared-memory ring (sweep.cu).
struct SweepPlan {
    bool ok = false;
    i64 n_levels = 0, P = 0;     // levels, padded positions
    int max_width = 0;           // off-diagonal entries of the widest row
    int threads = 0;             // compute threads (widest level rounded up to a warp)
    dbuf<int32_t> cnt, cntp, width;
    dbuf<ushort4> meta;          // per level: rows, padded rows, width
    dbuf<i64> ppos, block_off;
    dbuf<int32_t> row_of;        // padded position -> row (-1 padding)
    dbuf<int32_t> ppos_of_row;
    dbuf<i64> val_src, inv_src;  // factor value index of each block entry (-1 padding)
    SweepLayout f64, f32;
    dbuf<double> in, out;        // right-hand side / solution in padded level order
    dbuf<float> in32, out32;
};

// CG reduction layout shared by the solver kernels
constexpr int RED_BLOCKS = 152 * 4;   // blocks of every reducing kernel (one partial each)
// default drop of the FP32 residual between the mixed solve's FP64 reliable updates
// (1e-3 saved two updates and 5 ms on the 300x300 serendipity problem but
// stalled the FP32 recurrence of a pure Neumann problem)
constexpr double MIXED_UPDATE_FACTOR = 1e-2;
enum { S_BB = 0, S_RZ0 = 1, S_DONE = 2, S_ITERS = 3, S_RR_FINAL = 4 };   // scalar slots
enum { P_PQ = 0, P_RR = 1, P_RZ_A = 2, P_RZ_B = 3, P_BB = 4, P_COUNT = 5 };   // partial buffers

// ILLT preconditioner: IC(0) of S A S + alpha I on the pattern of A's upper part.
struct IncompleteCholesky {
    SweepPlan fwd_plan, bwd_plan;
    i64 n = 0, nnz = 0;
    dbuf<i64> rp;                // upper pattern (diagonal first)
    dbuf<int32_t> col;
    dbuf<double> a_scaled, u;    // S A S and the factor values
    dbuf<i64> lrp, l_to_u;       // U^T as lower CSR (diagonal last) and its U positions
    dbuf<int32_t> lcol;
    dbuf<i64> ic_lev_ptr;        // forward levels for the factorisation
    dbuf<int32_t> ic_rows;
    i64 ic_levels = 0;
    dbuf<double> scale;          // S
    dbuf<float> scale32;
    TriSlab fwd, bwd;
    dbuf<double> y, w;           // sweep buffers, n + 1 entries
    dbuf<float> y32, w32;
    JacobiSlab jlo, jup;         // U^T and U for Jacobi sweeps, rows scaled by 1 / u_ii
    dbuf<float> jc, jdinv;       // s_i / u_ii and 1 / u_ii
    dbuf<float> jt0, jt1, jy;    // Jacobi iterates and the scaled forward result
    bool ok = false;
    bool approximate = false;    // factor from the fixed-point sweeps (ilt_build), not the exact IC(0)
    bool exact_ready = false;    // fwd / bwd slabs and plans built and filled (ilt_exact_layouts)
    int attempts = 0;
    double shift = 0.0;
};

// Persistent device state of CG.
struct CgWork {
    i64 n = 0;
    dbuf<double> r, z, p, q, x, tmp;
    dbuf<double> partial;        // block partial sums
    dbuf<double> scalars;        // see solver.cu
    dbuf<int> flags;
};

// Learned correction on top of ILLT (mpnn.cu): a 4-layer message-passing
// network of width 64 over the local stiffness graph.  Parameters are packed
// FP32 [W1 4x64 | W2 128x64 | W3 128x64 | w4 128]; BF16 copies feed the
// tensor-core GEMMs (stored as uint16_t bit patterns).
constexpr int MPNN_HIDDEN = 64;
constexpr long long MPNN_PARAMS = 4 * 64 + 2 * 128 * 64 + 128;
struct Mpnn {
    bool ready = false, weights_set = false;
    bool use = true;             // validation gate: the correction beat ILLT alone on its own system
    i64 n = 0, ldt = 0;          // nodes; leading dimension of transposed copies (n rounded up to 8)
    dbuf<i64> arp;               // A_hat: symmetric, zero diagonal, FP32 weights
    dbuf<int32_t> acol;
    dbuf<float> aw;
    dbuf<float> params, grads, adam_m, adam_v;
    long long adam_t = 0;
    dbuf<uint16_t> w2t, w3t, w2b, w3b;   // BF16: [out][in] and [in][out]
    dbuf<float> u0;              // [n][4]
    dbuf<uint16_t> u1, u2, u3;   // [n][128] BF16: [H | A_hat H]
    dbuf<uint16_t> u1t, u2t;     // [128][ldt] transposed (training)
    dbuf<uint16_t> dp, dpt;      // [n][64] and [64][ldt] BF16 (training)
    dbuf<float> du, dp32, d, ad; // training work
    dbuf<double> part, part2, ee64;
    dbuf<float> sc;              // scalars (1/rms r, 1/rms z, rms z, ...)
    dbuf<int> error;
};

// Coarse-space correction of the mixed solve (coarse.cu): aggregates, AP,
// the FP32 inverse of A_c = P^T A P and the application's work vectors.
struct Coarse {
    bool ready = false;
    i64 nc = 0, ap_nnz = 0;
    dbuf<int32_t> agg;           // [n] aggregate of each node (-1: none)
    dbuf<i64> ptr;               // [nc + 1] node lists of the aggregates
    dbuf<int32_t> nodes;
    dbuf<i64> ap_rp;             // AP: per row (aggregate, sum of the row's entries over it)
    dbuf<int32_t> ap_col;
    dbuf<float> ap_val;
    dbuf<float> ainv;            // [nc][nc]
    dbuf<float> rc, ec, w, y;
};

// Device state of BiCGSTAB (bicgstab.cu).
struct BicgWork {
    dbuf<double> r, r0, p, v, s, t, y, z, dinv, part, sc;
    cudaGraphExec_t chunk = nullptr;   // BI_ITERS iterations, captured per solve
    int chunk_kernels = 0;
    ~BicgWork() { if (chunk) cudaGraphExecDestroy(chunk); }
};

// Device state of the mixed-precision solve (mixed.cu).
struct MixedWork {
    i64 n = 0;
    dbuf<double> r64, q64;       // outer residual and A x
    dbuf<float> r, z, p, q, d;   // inner vectors
    dbuf<double> partial, outer, flags;
    dbuf<unsigned> ticket;             // blocks done in the current reducing kernel
    cudaGraphExec_t chunk = nullptr;   // a chunk of inner iterations, re-captured per solve
    int chunk_kernels = 0;
    MixedWork() = default;
    MixedWork(const MixedWork&) = delete;
    MixedWork& operator=(const MixedWork&) = delete;
    ~MixedWork() { if (chunk) cudaGraphExecDestroy(chunk); }
};

// Nonlocal plane elasticity, DoF = 2 (elastic.cu): Hooke coefficients, the
// boundary groups per component, and the stiffness system over 2 n rows
// (row 2 node + component, as the reference numbers them).
struct MechanicalGroup {
    int nen = 2;
    i64 n_edges = 0;
    dbuf<int32_t> edges;
    int kind[2] = {0, 0};        // NLGPU_MECH_NONE / DISPLACEMENT / PRESSURE per component
    double value[2] = {0.0, 0.0};
};
struct Elastic {
    bool hooke_set = false;
    int kind = 0;
    double h[6] = {0, 0, 0, 0, 0, 0};   // h11 h12 h66 h22 h16 h26
    std::vector<MechanicalGroup> groups;
    dbuf<uint8_t> is_inner;      // [2n] per degree of freedom
    dbuf<double> x_dirichlet, rhs_init, rhs, displacement;
    Csr inner, bound, full, local;
    dbuf<i64> full_from_upper;
    IncompleteCholesky ilt;
    bool assembled = false, local_ready = false;
};

struct OneDimState;   // nonstationary 1D solver state (onedim.cu)

struct Ctx {
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // mesh
    int element_type = 0;
    Basis basis{};
    i64 n_nodes = 0, n_elems = 0;
    dbuf<double> nodes;          // [n][2]
    dbuf<int32_t> elems;         // [e][nen]
    dbuf<double> qcoord, jac, deriv, centres;
    dbuf<float2> centres32;             // FP32 copies for the neighbour search's pre-test
    dbuf<i64> ne_off;            // node -> elements CSR
    dbuf<int32_t> ne_elem;
    dbuf<int8_t> ne_local;
    dbuf<int32_t> elem_minnode;  // smallest node number per element
    dbuf<int32_t> elem_maxnode;  // largest node number per element
    bool mesh_ready = false;
    // model
    Model model{};
    bool model_ready = false;
    dbuf<double> cond_field;     // optional isotropic conductivity [e][q]
    double capacity = 1.0, density = 1.0;
    // neighbours
    bool neighbours_ready = false;
    int strategy = NLGPU_EXPAND_MAX;
    double search_r[2] = {0, 0};
    i64 pairs = 0;
    dbuf<i64> noff;
    dbuf<int32_t> nlist;
    // boundary
    std::vector<BoundaryGroup> groups;
    double source = 0.0;
    dbuf<double> source_q;
    dbuf<double> dirichlet_override;
    dbuf<uint8_t> is_inner;
    dbuf<double> x_dirichlet, rhs_init, rhs;
    bool bc_ready = false;
    // stationary_equation_parameters_2d: the radiation loop's stop test, the
    // Lagrange row's energy (pure Neumann problems) and the initial temperature
    double nl_tolerance = 1e-8, energy = 0.0;
    i64 nl_max_iterations = 100;
    dbuf<double> initial_temperature;
    bool neumann = false;        // stationary and every group a plain flux: integral condition
    dbuf<double> node_integral;  // Neumann: int N_i over the node's elements (the Lagrange column)
    dbuf<double> upper_base;     // radiation: the upper values before the temperature-dependent part
    dbuf<double> nl_work;        // radiation: K T_prev, the radiation vector, T_prev, partial norms
    // matrices (reference storage) and the solver's full-row copy
    bool symmetric = true;
    Csr inner, bound, local, full;
    dbuf<i64> full_from_upper;   // full entry -> upper entry (lower part via transpose)
    bool inner_ready = false, local_ready = false;
    IncompleteCholesky ilt;
    IncompleteCholesky plugin_ilt;   // nlgpu_illt_compute / nlgpu_illt_solve
    bool plugin_ilt_ready = false;
    CgWork cg;
    Coarse co;
    Elastic el;
    std::shared_ptr<OneDimState> od;
    double od_heat_transfer[2] = {0.0, 0.0};   // 1D convection ends (nlgpu_nonstationary_1d_convection)
    MixedWork mx;
    BicgWork bi;
    Mpnn mp;
    // nonstationary
    Csr capacity_m, capacity_full;
    dbuf<i64> capacity_map;
    dbuf<double> step_tmp, step_xd;
    double time_step = 0.0;
    dbuf<double> temperature;
    bool nonstationary_ready = false;
    dbuf<int> sweep_error;
    bool force_global_sweeps = false;   // use the global-memory sweeps (for comparison)
    int ilt_sweeps = NLGPU_DEFAULT_TRIANGULAR_SWEEPS;   // FP32 ILLT: Jacobi sweeps per triangle (0: exact)
    bool ordered_pairs = false;         // evaluate every ordered element pair (for comparison)
    bool fp32_symmetric = false;        // FP32 SpMV from the strictly upper part (for comparison)
    int assembly_precision = NLGPU_ASSEMBLY_AUTO;
    bool ff_assembly = false;           // pair blocks in float-float on the FP32 pipes (mixed precision)
    bool ff_assembled = false;          // the last assembly ran in float-float
    int ff_warps_option = 0;            // warps per CTA of the float-float pair assembly (0: tuned)
    int ff_warps_used = 0;              // ... of its last launch
    double ff_tune_ms[2] = {0.0, 0.0};  // the last tuning's sample times with 16 and 32 warps
    std::map<int, int> ff_warps_tuned;  // tuned choice per (element type, influence kind, pair mode)
    dbuf<float4> deriv_ff, qcoord_ff;   // float-float copies: (gx, gy) / (x, y) as (hi, lo, hi, lo)
    dbuf<float2> cw_ff;                 // w_q norm (1 - p1) [lambda_q] per element and point
    // measurement
    cudaEvent_t events[64] = {};
    dbuf<unsigned char> flush;
    unsigned flush_value = 0;
    ~Ctx() { for (cudaEvent_t& e : events) if (e) cudaEventDestroy(e); }
    // scratch
    dbuf<unsigned char> scratch;
    dbuf<i64> i64_scratch_a, i64_scratch_b;
    unsigned char* scratch_bytes(size_t bytes) { scratch.reserve(bytes); return scratch.p; }
};

// ------------------------------------------------------------ utilities
// Exclusive prefix sum of n int64 values (in may alias out); writes the total
// to *total_host when not null (synchronises the stream).
void exclusive_scan(Ctx& ctx, const i64* in, i64* out, i64 n, i64* total_host);
i64 device_read_i64(Ctx& ctx, const i64* p);

// mesh.cu
void mesh_init(Ctx& ctx);
// neighbours.cu
void find_neighbours(Ctx& ctx, int strategy);
// boundary.cu
void boundary_vectors(Ctx& ctx);
// is_inner: per-row inner flags (default ctx.is_inner)
void apply_first_kind(Ctx& ctx, const Csr& bound, const double* rhs_in, double* rhs_out, const double* x_dirichlet,
                      const uint8_t* is_inner = nullptr);
// pattern.cu
// is_inner: per-row inner flags (default ctx.is_inner)
void build_patterns(Ctx& ctx, bool local_only, bool symmetric, Csr& inner, Csr* bound, Csr* full,
                    dbuf<i64>* full_from_upper, const uint8_t* is_inner = nullptr);
// full-row entry -> entry of the same value in the upper storage (-1 for padding)
void full_map(Ctx& ctx, const Csr& upper, const Csr& full, dbuf<i64>& map, bool symmetric);
// assemble.cu
void assemble_full(Ctx& ctx);
void assemble_local(Ctx& ctx, Csr& m, double weight, int integrand);   // integrand 0 conductivity, 1 capacity
void fill_full_from_upper(Ctx& ctx, const Csr& upper, Csr& full, const dbuf<i64>& map);
void set_dirichlet_diagonal(Ctx& ctx, Csr& m, double value);
void combine_nonstationary(Ctx& ctx, double dt);
// f = dt (flux + source [+ radiation]) + C T_prev, then the first kind
void nonstationary_rhs(Ctx& ctx, double dirichlet_value, bool per_node_values, const double* radiation = nullptr);
// solver.cu
void spmv_full(Ctx& ctx, const Csr& A, const double* x, double* y);
// tma_plans: also build the TMA-fed shared-memory sweep plans of the exact
// triangular solves (without them exact solves use the global-memory sweeps)
// approximate: the factor from a few fixed-point sweeps (for the FP32 Jacobi-sweep application)
void ilt_build(Ctx& ctx, const Csr& upper, IncompleteCholesky& ic, bool tma_plans = true, bool approximate = false);
void ilt_apply(Ctx& ctx, const IncompleteCholesky& ic, const double* r, double* z);
// the exact sweeps' layouts of a factorised ILLT (once; before any stream capture)
void ilt_exact_layouts(Ctx& ctx, IncompleteCholesky& ic);
struct CgResult {
    i64 iterations = 0, outer_iterations = 0;
    double residual = 0, reference_residual = 0;
    bool converged = false;
    bool learned_fallback = false;   // the learned correction stalled and was switched off
};
// on_chunk (optional) is called with the iteration count and x after every
// chunk of iterations the host checks (used to harvest training snapshots)
using CgChunkHook = std::function<void(i64 iterations, const double* x)>;
CgResult cg_solve(Ctx& ctx, const Csr& A_full, const IncompleteCholesky* M, const double* b, double* x,
                  double tolerance, i64 max_iterations, bool x_is_initial_guess, const CgChunkHook& on_chunk = {});
// sweep.cu
bool sweep_plan_build(Ctx& ctx, const std::vector<i64>& lev_ptr, const std::vector<int32_t>& rows,
                      const std::vector<i64>& rp, const std::vector<int32_t>& col, const std::vector<i64>& val_index,
                      const std::vector<i64>& diag_pos, SweepPlan& plan);
void sweep_plan_fill(Ctx& ctx, SweepPlan& plan, const double* u);
void sweep_apply(Ctx& ctx, IncompleteCholesky& ic, const double* r, double* z, const double* partials,
                 const double* flags, double tol2);
void sweep_apply32(Ctx& ctx, IncompleteCholesky& ic, const float* r, float* z, const double* partials,
                   const double* flags, double tol2);
// flux.cu: nodal heat flux of a temperature field (device vectors)
void calc_flux(Ctx& ctx, const double* temperature, double* flux_x, double* flux_y);
// renumber.cu: the node graph (adjacency in the reference's order, CSR on the
// host), its Cuthill-McKee order (perm[old] = new), and the renumbering of
// the context's mesh by a checked permutation
void node_graph(Ctx& ctx, bool local_graph, std::vector<i64>& offsets, std::vector<int32_t>& adjacency);
std::vector<i64> cuthill_mckee_order(const std::vector<i64>& offsets, const std::vector<int32_t>& adjacency);
void renumber_mesh(Ctx& ctx, const std::vector<int32_t>& perm);
// nonlinear.cu: convection and radiation edges, pure Neumann problems
bool has_convection(const Ctx& ctx);
bool has_radiation(const Ctx& ctx);
bool pure_neumann(const Ctx& ctx);
// entries of the edge node pairs in ctx.inner; throws when an edge touches a temperature node
void boundary_matrix_index(Ctx& ctx);
void add_convection(Ctx& ctx);                                  // into ctx.inner.val
// ctx.inner.val += matrix_factor sigma eps int T^3 N_i N_j, rad += vector_factor sigma eps int T^4 N_i
void add_radiation(Ctx& ctx, const double* T, double* rad, double matrix_factor, double vector_factor);
void neumann_integrals(Ctx& ctx);                               // ctx.node_integral
void subtract3(Ctx& ctx, const double* a, const double* b, const double* d, double* y);
// x <- prev - x; returns |residual|^2, |x - prev|^2, |x|^2 (deterministic order)
std::array<double, 3> step_norms(Ctx& ctx, const double* residual, const double* prev, double* x);
void add_scaled(Ctx& ctx, double a, const double* x, double* y);
void add_constant(Ctx& ctx, double a, double* y);
// iltbuild.cu: U pattern copies, U^T, the factorisation's levels (offsets on the
// host too) and the Jacobi sweeps' layouts, built on the device
void ilt_structure_gpu(Ctx& ctx, const Csr& upper, IncompleteCholesky& ic, bool levels = true);
// jacobi.cu: the factor applied by Jacobi sweeps on its two triangles
void jacobi_fill(Ctx& ctx, IncompleteCholesky& ic);
void jacobi_apply32(Ctx& ctx, IncompleteCholesky& ic, int sweeps, const float* r, float* z, const double* flags);
// mixed.cu
// FP32 copy of the solver matrix A (full rows) for the mixed solve; with the
// upper storage of a symmetric A given, only its strictly upper part is copied
// (symmetric FP32 SpMV) when every row's reach fits the SpMV's shared memory
void matrix_to_f32(Ctx& ctx, Csr& A, const Csr* upper = nullptr);
void spmv32(Ctx& ctx, const Csr& A, const float* x, float* y);
// sweeps 0: level-scheduled triangular solves; > 0: that many Jacobi sweeps per triangle
void ilt_apply32(Ctx& ctx, IncompleteCholesky& ic, const float* r, float* z, int sweeps = 0);
CgResult mixed_solve(Ctx& ctx, const Csr& A_full, IncompleteCholesky* M, const double* b, double* x, double tolerance,
                     i64 max_iterations, double update_factor, bool x_is_initial_guess, bool learned, int sweeps,
                     bool coarse = false);
// coarse.cu: the coarse-space correction around the FP32 ILLT application
void coarse_build(Ctx& ctx, const Csr& A_full, int target, double aspect = 1.0);
void coarse_before(Ctx& ctx, const float* r, const double* flags);   // ctx.co.w = r - A Q r, ctx.co.y = Q r
void coarse_after(Ctx& ctx, float* z, const double* flags);          // z += Q r
// batch.cu: many nonstationary instances stepped together (block-diagonal system)
struct Batch;
Batch* batch_create(const std::vector<Ctx*>& instances);
void batch_destroy(Batch* bt);
i64 batch_step(Batch& bt, const double* dirichlet_values, double tolerance, i64 max_iterations, i64* iterations);
void batch_temperature(Batch& bt, i64 index, double* out);
cudaStream_t batch_stream(Batch& bt);
void batch_sizes(const Batch& bt, i64* rows, i64* system_entries);
void batch_set_method(Batch& bt, int method);
void batch_last_solve(const Batch& bt, i64* inner, i64* outer, int* fallback);
std::vector<CgResult> batch_bicgstab(const std::vector<Ctx*>& instances, double tolerance, i64 max_iterations,
                                     bool illt);
// bicgstab.cu: Jacobi-preconditioned BiCGSTAB on a full-row (non-symmetric) matrix, zero start
CgResult bicgstab_solve(Ctx& ctx, const Csr& A_full, const double* b, double* x, double tolerance, i64 max_iterations);
// mpnn.cu
void mpnn_prepare(Ctx& ctx, const Csr& local_upper);
void mpnn_init_weights(Ctx& ctx, unsigned seed);
void mpnn_set_weights(Ctx& ctx, const float* host);
void mpnn_get_weights(Ctx& ctx, float* host);
void mpnn_apply(Ctx& ctx, const float* r, const float* z, float* out, bool training);
void mpnn_backward(Ctx& ctx, const Csr& A, const float* r, const float* z, const float* e, float* p_out,
                   double* loss_num, double* ee_out);
void mpnn_adam_step(Ctx& ctx, float lr, int batch);
void mpnn_check(Ctx& ctx);
struct MpnnTrainOptions {
    int right_hand_sides = 4, epochs = 20, batch = 8;
    double learning_rate = 1e-3;
    unsigned seed = 0;
};
struct MpnnTrainResult {
    i64 samples = 0, steps = 0;
    double loss_illt = 0, loss_first = 0, loss_last = 0, seconds_harvest = 0, seconds_train = 0;
    i64 validation_iterations_learned = 0, validation_iterations_illt = 0;
    double validation_seconds_learned = 0, validation_seconds_illt = 0;
    bool learned_enabled = false;
};
void mpnn_train(Ctx& ctx, const Csr& A, IncompleteCholesky& M, const double* b, const MpnnTrainOptions& o,
                MpnnTrainResult& out);
// noalloc.cu
bool cg_solve_noalloc(cudaStream_t s, i64 n, const i64* rp, const int32_t* col, const double* val, const double* b,
                      double* x, double tolerance, i64 max_iterations, i64* iterations, double* residual);
// elastic.cu: nonlocal plane elasticity (equilibrium_equation_2d.hpp:19-60)
void elastic_boundaries(Ctx& ctx);
void elastic_assemble(Ctx& ctx, bool local_part);
CgResult elastic_solve(Ctx& ctx, const nlgpu_solve_options& o, nlgpu_solve_report* rep);
// onedim.cu
void nonstationary_1d_compute(Ctx& ctx, i64 elements, int order, double length, double radius, double local_weight,
                              int influence, double conductivity, double capacity, double density, double time_step,
                              int left_kind, int right_kind, const double* initial);
void nonstationary_1d_step(Ctx& ctx, double left_value, double right_value, bool sin_source, double* temperature);
void nonstationary_1d_temperature(Ctx& ctx, double* temperature);
i64 nonstationary_1d_nodes(const Ctx& ctx);
void stationary_1d(Ctx& ctx, i64 elements, int order, double length, double radius, double local_weight, int influence,
                   double conductivity, double t_left, double q_right, bool sin_source, double* temperature);

// device helpers --------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace nlgpu
