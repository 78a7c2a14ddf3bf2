// Batched nonstationary stepping: many instances of uneven size advanced by
// one implicit-Euler step together.
//
// The reference steps one problem at a time (nonstationary_heat_equation_
// solver_2d::calc_step, nonstationary_heat_equation_solver_2d.hpp:90-106: the
// right-hand side C T_prev + dt f - dt K_bound x_D with f[D] = x_D, then CG with
// the identity preconditioner from x0 = T_prev).  Here the instances'
// matrices are concatenated into one block-diagonal system, so every stage of
// every instance runs in one launch that covers all rows:
//   * the right-hand side: one SpMV with the concatenated capacity matrices,
//     one with the Dirichlet columns, elementwise kernels;
//   * CG: one SpMV over the concatenated system matrices per iteration, the
//     vector updates over all rows, each instance with its own alpha, beta,
//     residual and stop flag; per-instance dot products are reduced by warps
//     whose rows belong to one instance, then one FP64 atomic per warp;
//   * a converged instance's rows are skipped from then on;
//   * a chunk of CG_ITERS iterations is captured once as a CUDA graph and
//     replayed; the host reads how many instances are still running once per
//     chunk.
// That identity FP64 CG is the reference's per-step solve.  The other method
// (NLGPU_BATCH_MIXED_ILLT) solves the whole block-diagonal system with the
// single-system mixed-precision FCG (FP32 difference-form SpMV, FP32 ILLT by
// Jacobi sweeps, FP64 reliable updates) preconditioned by the ILLT of
// C + dt p1 K_local of every instance (the block-diagonal local part, factored
// once), to a global tolerance tol sqrt(min_k |b_k|^2 / sum_k |b_k|^2) that
// gives every instance |b_k - A_k x_k| <= tol |b_k|; the FP64 ILLT-CG is its
// fallback when the FCG does not converge.
#include "common.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>

namespace nlgpu {

namespace {

constexpr int BT_THREADS = 256;
constexpr int BT_ITERS = 16;   // iterations per captured chunk (even: the parity pattern repeats)
constexpr int BT_RUN_SLOT = 0; // count of running instances (int scalar area)

// per-instance scalar arrays (double [K] each)
enum { BS_BB = 0, BS_RR0 = 1, BS_RR1 = 2, BS_PQ = 3, BS_DONE = 4, BS_ITERS = 5, BS_COUNT = 6 };

__device__ __forceinline__ void seg_add(double v, int inst, double* acc) {
    // lanes of one instance: one warp sum and one atomic; mixed warps: one atomic per lane
    const unsigned full = 0xffffffffu;
    const int inst0 = __shfl_sync(full, inst, 0);
    if (__all_sync(full, inst == inst0)) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(full, v, o);
        if ((threadIdx.x & 31) == 0 && inst0 >= 0) atomicAdd(acc + inst0, v);
    } else if (inst >= 0 && v != 0.0) {
        atomicAdd(acc + inst, v);
    }
}

#define BT_ROWS(i) for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i < n; i += i64(gridDim.x) * blockDim.x)

// x_D: the instance's Dirichlet value on Dirichlet rows, 0 elsewhere
__global__ void k_bt_xd(i64 n, const int32_t* __restrict__ inst, const uint8_t* __restrict__ is_inner,
                        const double* __restrict__ value, double* __restrict__ xd) {
    BT_ROWS(i) xd[i] = is_inner[i] ? 0.0 : value[inst[i]];
}

__global__ void k_bt_axpy(i64 n, const double* __restrict__ a, double* __restrict__ y) {
    BT_ROWS(i) y[i] += a[i];
}

// y = A x over padded full rows in row blocks: a block holds 32 / g
// consecutive rows of one instance, each taken by g lanes (g a power of two
// from the instance's mean row length, so that every lane reads a few int4
// groups), and the warps take blocks in turn (grid stride).  The instances'
// rows differ in length by two orders of magnitude (r/h from 2 to 26): a
// whole warp per short row left most lanes idle and spent a five-step FP64
// warp reduction per row, which on GB300's two-lane FP64 pipe cost more than
// the row.  Blocks of stopped instances are skipped.  Optional per-instance
// partials of x.y: one warp sum per block, kept by lane 0 while its blocks stay
// in one instance and added with one FP64 atomic when the instance changes.
// desc: first row (bits 0-31), log2 g (bits 32-34), rows in the block (35-40).
__global__ void __launch_bounds__(BT_THREADS) k_bt_spmv(i64 nblocks, const unsigned long long* __restrict__ desc,
                                                        const i64* __restrict__ rp, const int4* __restrict__ col4,
                                                        const double2* __restrict__ val2, const double* __restrict__ x,
                                                        double* __restrict__ y, const int32_t* __restrict__ inst,
                                                        const double* __restrict__ sc, i64 K, double* __restrict__ dot) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    double acc = 0.0;
    int acc_inst = -1;
    for (i64 bk = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; bk < nblocks; bk += warps) {
        const unsigned long long d = desc[bk];
        const i64 first = i64(d & 0xffffffffull);
        const int lg = int((d >> 32) & 7), cnt = int((d >> 35) & 63);
        const int k = inst[first];
        if (sc[BS_DONE * K + k] != 0.0) continue;
        const int g = 1 << lg, sub = lane & (g - 1), slot = lane >> lg;
        const i64 r = first + slot;
        const bool active = slot < cnt;
        double s = 0.0;
        if (active) {
            const i64 b4 = rp[r] >> 2, e4 = rp[r + 1] >> 2;
            for (i64 q = b4 + sub; q < e4; q += g) {
                const int4 c = __ldg(col4 + q);
                const double2 v0 = __ldg(val2 + 2 * q), v1 = __ldg(val2 + 2 * q + 1);
                s += v0.x * x[c.x] + v0.y * x[c.y] + v1.x * x[c.z] + v1.y * x[c.w];
            }
        }
        for (int o = g >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(full, s, o);   // within the lane group
        double contrib = 0.0;
        if (active && sub == 0) {
            y[r] = s;
            contrib = s * x[r];
        }
        if (dot) {
            contrib = warp_sum(contrib);
            if (lane == 0) {
                if (k != acc_inst) {
                    if (acc_inst >= 0) atomicAdd(dot + acc_inst, acc);
                    acc = 0.0;
                    acc_inst = k;
                }
                acc += contrib;
            }
        }
    }
    if (dot && lane == 0 && acc_inst >= 0) atomicAdd(dot + acc_inst, acc);
}

// per-instance |v|^2 into acc (zeroed by the caller)
__global__ void __launch_bounds__(BT_THREADS) k_bt_norm2(i64 n, const double* __restrict__ v,
                                                         const int32_t* __restrict__ inst, double* __restrict__ acc) {
    BT_ROWS(i) seg_add(v[i] * v[i], inst[i], acc);
}

// out = in - B x_D on inner rows, x_D on Dirichlet rows (warp per row of the
// concatenated Dirichlet-column matrices; boundary_condition_first_kind_2d.hpp:50-59)
__global__ void k_bt_first_kind(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                                const double* __restrict__ val, const double* __restrict__ in,
                                const double* __restrict__ xd, const uint8_t* __restrict__ is_inner,
                                double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    for (i64 r = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; r < n; r += warps) {
        double s = 0.0;
        for (i64 k = rp[r] + lane; k < rp[r + 1]; k += 32) s += val[k] * xd[col[k]];
        s = warp_sum(s);
        if (lane == 0) out[r] = is_inner[r] ? in[r] - s : xd[r];
    }
}

__global__ void k_bt_scale(i64 n, double h, double* __restrict__ v) {
    BT_ROWS(i) v[i] *= h;
}

// r = b - q, p = r; partials of r.r and b.b (grid-stride rows: a warp's 32
// consecutive rows are almost always one instance)
__global__ void __launch_bounds__(BT_THREADS) k_bt_start(i64 n, const double* __restrict__ b, const double* __restrict__ q,
                                                         double* __restrict__ r, double* __restrict__ p,
                                                         const int32_t* __restrict__ inst, double* __restrict__ sc, i64 K) {
    BT_ROWS(i) {
        const double v = b[i] - q[i];
        r[i] = v; p[i] = v;
        seg_add(v * v, inst[i], sc + BS_RR0 * K);
        seg_add(b[i] * b[i], inst[i], sc + BS_BB * K);
    }
}

// alpha = rr / pq per instance; x += alpha p; r -= alpha q; partial of the new r.r
__global__ void __launch_bounds__(BT_THREADS) k_bt_update_xr(i64 n, double* __restrict__ x, double* __restrict__ r,
                                                             const double* __restrict__ p, const double* __restrict__ q,
                                                             const int32_t* __restrict__ inst, double* __restrict__ sc,
                                                             i64 K, int parity) {
    const double* rr_cur = sc + (parity ? BS_RR1 : BS_RR0) * K;
    double* rr_new = sc + (parity ? BS_RR0 : BS_RR1) * K;
    BT_ROWS(i) {
        const int k = inst[i];
        double v2 = 0.0;
        int kk = -1;
        if (sc[BS_DONE * K + k] == 0.0) {
            const double alpha = rr_cur[k] / sc[BS_PQ * K + k];
            x[i] += alpha * p[i];
            const double v = r[i] - alpha * q[i];
            r[i] = v;
            v2 = v * v;
            kk = k;
        }
        seg_add(v2, kk, rr_new);
    }
}

// beta = rr_new / rr_cur per instance; p = r + beta p
__global__ void k_bt_update_p(i64 n, double* __restrict__ p, const double* __restrict__ r,
                              const int32_t* __restrict__ inst, const double* __restrict__ sc, i64 K, int parity) {
    const double* rr_cur = sc + (parity ? BS_RR1 : BS_RR0) * K;
    const double* rr_new = sc + (parity ? BS_RR0 : BS_RR1) * K;
    BT_ROWS(i) {
        const int k = inst[i];
        if (sc[BS_DONE * K + k] != 0.0) continue;
        p[i] = r[i] + (rr_new[k] / rr_cur[k]) * p[i];
    }
}

// per instance: count the iteration, stop on |r| <= tol |b| or the cap; clear the
// accumulators the next iteration adds into; count the running instances
__global__ void k_bt_check(i64 K, double* __restrict__ sc, int parity, double tol2, double max_iterations,
                           int* __restrict__ running) {
    __shared__ int cnt;
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    for (i64 k = threadIdx.x; k < K; k += blockDim.x) {
        if (sc[BS_DONE * K + k] == 0.0) {
            sc[BS_ITERS * K + k] += 1.0;
            const double rr = sc[(parity ? BS_RR0 : BS_RR1) * K + k];
            if (rr <= tol2 * sc[BS_BB * K + k] || sc[BS_ITERS * K + k] >= max_iterations) sc[BS_DONE * K + k] = 1.0;
            else atomicAdd(&cnt, 1);
        }
        sc[BS_PQ * K + k] = 0.0;
        sc[(parity ? BS_RR1 : BS_RR0) * K + k] = 0.0;   // the slot the next iteration's residual goes to
    }
    __syncthreads();
    if (threadIdx.x == 0) running[BT_RUN_SLOT] = cnt;
}

// before the first iteration: stop instances that already satisfy the tolerance
__global__ void k_bt_first(i64 K, double* __restrict__ sc, double tol2) {
    for (i64 k = threadIdx.x; k < K; k += blockDim.x) {
        sc[BS_ITERS * K + k] = 0.0;
        sc[BS_DONE * K + k] = (sc[BS_BB * K + k] == 0.0 || sc[BS_RR0 * K + k] <= tol2 * sc[BS_BB * K + k]) ? 1.0 : 0.0;
        sc[BS_PQ * K + k] = 0.0;
        sc[BS_RR1 * K + k] = 0.0;
    }
}

// concatenation: row pointers shifted by the entries before, columns by the rows before
__global__ void k_bt_shift(i64 rows, const i64* __restrict__ rp_in, const int32_t* __restrict__ col_in, i64 nnz,
                           i64 row_off, i64 nnz_off, i64* __restrict__ rp_out, int32_t* __restrict__ col_out,
                           int32_t* __restrict__ inst_out, int inst) {
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i <= rows; i += i64(gridDim.x) * blockDim.x) {
        rp_out[i] = rp_in[i] + nnz_off;
        if (i < rows && inst_out) inst_out[i] = inst;
    }
    for (i64 k = blockIdx.x * i64(blockDim.x) + threadIdx.x; k < nnz; k += i64(gridDim.x) * blockDim.x)
        col_out[k] = col_in[k] + int32_t(row_off);
}

}  // namespace

struct Batch {
    cudaStream_t stream = nullptr;
    std::vector<Ctx*> inst;
    i64 K = 0, N = 0;
    std::vector<i64> row_off;
    dbuf<int32_t> inst_of_row;
    Csr A, C, B;
    dbuf<unsigned long long> blocks_A, blocks_C;   // SpMV row blocks (k_bt_spmv)
    i64 nblocks_A = 0, nblocks_C = 0;
    dbuf<double> rhs_dt, x, b, r, p, q, tmp, xd, dval, sc;
    dbuf<uint8_t> is_inner;
    dbuf<int> running;
    cudaGraphExec_t chunk = nullptr;
    double chunk_tol2 = -1.0, chunk_cap = -1.0;
    int chunk_kernels = 0;
    // NLGPU_BATCH_MIXED_ILLT: the single-system solvers' work buffers on this
    // stream, the block-diagonal local matrix and its ILLT (built at the first
    // mixed step)
    int method = NLGPU_BATCH_IDENTITY_FP64;
    Ctx solver;
    Csr M;
    IncompleteCholesky ic;
    bool mixed_ready = false;
    i64 last_inner = 0, last_outer = 0;
    bool last_fallback = false;
};

namespace {

// concatenates one matrix of every instance (sel picks it) into `out`
template<class Sel>
void concat(Batch& bt, Csr& out, Sel sel, bool with_inst) {
    i64 nnz = 0;
    for (Ctx* c : bt.inst) nnz += sel(*c).nnz;
    out.rows = bt.N; out.nnz = nnz;
    out.rowptr.resize(size_t(bt.N + 1));
    out.col.resize(size_t(std::max<i64>(nnz, 1)));
    out.val.resize(size_t(std::max<i64>(nnz, 1)));
    i64 nnz_off = 0;
    for (size_t k = 0; k < bt.inst.size(); ++k) {
        const Csr& m = sel(*bt.inst[k]);
        NL_REQUIRE(m.rows == bt.row_off[k + 1] - bt.row_off[k], NLGPU_ERR_STATE, "instance matrix size");
        NL_LAUNCH(k_bt_shift, grid_for(std::max<i64>(m.nnz, m.rows + 1), 256), 256, 0, bt.stream, m.rows, m.rowptr.p, m.col.p,
                  m.nnz, bt.row_off[k], nnz_off, out.rowptr.p + bt.row_off[k], out.col.p + nnz_off,
                  with_inst ? bt.inst_of_row.p + bt.row_off[k] : static_cast<int32_t*>(nullptr), int(k));
        if (m.nnz)
            NL_CUDA(cudaMemcpyAsync(out.val.p + nnz_off, m.val.p, size_t(m.nnz) * sizeof(double), cudaMemcpyDeviceToDevice,
                                    bt.stream));
        nnz_off += m.nnz;
    }
}

// row blocks of a concatenated matrix for k_bt_spmv: per instance g lanes per
// row, g the smallest power of two (2 .. 32) with g * 12 >= the mean padded
// row length (about three int4 groups per lane)
void row_blocks(Batch& bt, const Csr& M, dbuf<unsigned long long>& out, i64& count) {
    std::vector<i64> rp(size_t(bt.N + 1));
    M.rowptr.download(rp.data(), rp.size(), bt.stream);
    NL_CUDA(cudaStreamSynchronize(bt.stream));
    std::vector<unsigned long long> desc;
    for (i64 k = 0; k < bt.K; ++k) {
        const i64 r0 = bt.row_off[size_t(k)], r1 = bt.row_off[size_t(k) + 1];
        if (r1 <= r0) continue;
        const double mean = double(rp[size_t(r1)] - rp[size_t(r0)]) / double(r1 - r0);
        int lg = 1;
        while (lg < 5 && double(1 << lg) * 12.0 < mean) ++lg;
        const i64 per = 32 >> lg;
        for (i64 r = r0; r < r1; r += per)
            desc.push_back((unsigned long long)r | ((unsigned long long)lg << 32) |
                           ((unsigned long long)std::min<i64>(per, r1 - r) << 35));
    }
    count = i64(desc.size());
    out.resize(std::max<size_t>(desc.size(), 1));
    if (!desc.empty()) out.upload(desc.data(), desc.size(), bt.stream);
}

// y = M x over every row; with skip_done the rows of stopped instances are left
// alone (the second half of the scalar array stays zero: "nothing stopped")
void bt_spmv(Batch& bt, const Csr& M, const double* x, double* y, double* dot, bool skip_done) {
    const bool is_a = &M == &bt.A;
    const i64 nb = is_a ? bt.nblocks_A : bt.nblocks_C;
    NL_LAUNCH(k_bt_spmv, grid_for(nb * 32, BT_THREADS, 152 * 8), BT_THREADS, 0, bt.stream, nb,
              (is_a ? bt.blocks_A : bt.blocks_C).p, M.rowptr.p, reinterpret_cast<const int4*>(M.col.p),
              reinterpret_cast<const double2*>(M.val.p), x, y, bt.inst_of_row.p,
              skip_done ? bt.sc.p : bt.sc.p + bt.K * BS_COUNT, bt.K, dot);
}

}  // namespace

Batch* batch_create(const std::vector<Ctx*>& instances) {
    auto* bt = new Batch{};
    try {
        NL_CUDA(cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking));
        bt->inst = instances;
        bt->K = i64(instances.size());
        bt->row_off.assign(size_t(bt->K + 1), 0);
        for (i64 k = 0; k < bt->K; ++k) {
            Ctx& c = *instances[size_t(k)];
            NL_REQUIRE(c.nonstationary_ready, NLGPU_ERR_STATE, "every instance needs nlgpu_nonstationary_2d_compute");
            NL_CUDA(cudaStreamSynchronize(c.stream));
            bt->row_off[size_t(k) + 1] = bt->row_off[size_t(k)] + c.n_nodes;
        }
        bt->N = bt->row_off.back();
        NL_REQUIRE(bt->N < (i64(1) << 31), NLGPU_ERR_UNSUPPORTED, "more than 2^31 rows in one batch");
        bt->inst_of_row.resize(size_t(bt->N));
        concat(*bt, bt->A, [](Ctx& c) -> const Csr& { return c.full; }, true);
        concat(*bt, bt->C, [](Ctx& c) -> const Csr& { return c.capacity_full; }, false);
        concat(*bt, bt->B, [](Ctx& c) -> const Csr& { return c.bound; }, false);
        row_blocks(*bt, bt->A, bt->blocks_A, bt->nblocks_A);
        row_blocks(*bt, bt->C, bt->blocks_C, bt->nblocks_C);
        // the instances' upper-storage copies of dt K + C and their full -> upper
        // maps are read again only by the radiation update of a single-instance
        // step, and batches hold no radiation: release them (a third of the
        // memory of a large batch)
        NL_CUDA(cudaStreamSynchronize(bt->stream));
        for (Ctx* c : instances) {
            c->full_from_upper.release();
            c->inner.col.release();
            c->inner.val.release();
            c->inner.nnz = 0;
        }
        for (auto* v : {&bt->rhs_dt, &bt->x, &bt->b, &bt->r, &bt->p, &bt->q, &bt->tmp, &bt->xd}) v->resize(size_t(bt->N));
        bt->is_inner.resize(size_t(bt->N));
        for (i64 k = 0; k < bt->K; ++k) {
            Ctx& c = *instances[size_t(k)];
            const size_t off = size_t(bt->row_off[size_t(k)]), n = size_t(c.n_nodes);
            NL_CUDA(cudaMemcpyAsync(bt->x.p + off, c.temperature.p, n * sizeof(double), cudaMemcpyDeviceToDevice, bt->stream));
            NL_CUDA(cudaMemcpyAsync(bt->is_inner.p + off, c.is_inner.p, n, cudaMemcpyDeviceToDevice, bt->stream));
            NL_CUDA(cudaMemcpyAsync(bt->rhs_dt.p + off, c.rhs_init.p, n * sizeof(double), cudaMemcpyDeviceToDevice,
                                    bt->stream));
            // dt * (flux + source) with the instance's own time step
            NL_LAUNCH(k_bt_scale, grid_for(i64(n), 256), 256, 0, bt->stream, i64(n), c.time_step, bt->rhs_dt.p + off);
        }
        bt->dval.resize(size_t(bt->K));
        bt->sc.resize(size_t(bt->K) * BS_COUNT * 2);   // the second half: all zero ("nothing done")
        bt->sc.zero(bt->stream);
        bt->running.resize(1);
        NL_CUDA(cudaStreamSynchronize(bt->stream));
        return bt;
    } catch (...) {
        if (bt->stream) cudaStreamDestroy(bt->stream);
        delete bt;
        throw;
    }
}

void batch_destroy(Batch* bt) {
    if (!bt) return;
    if (bt->chunk) cudaGraphExecDestroy(bt->chunk);
    if (bt->stream) { cudaStreamSynchronize(bt->stream); cudaStreamDestroy(bt->stream); }
    delete bt;
}

namespace {

// the block-diagonal local matrix C + dt p1 K_local (upper, Dirichlet rows a
// unit diagonal), its ILLT and the FP32 copy of the system matrix
void batch_prepare_mixed(Batch& bt) {
    if (bt.mixed_ready) return;
    std::vector<Csr> local(bt.inst.size());
    for (size_t k = 0; k < bt.inst.size(); ++k) {
        Ctx& c = *bt.inst[k];
        build_patterns(c, true, true, local[k], nullptr, nullptr, nullptr);
        assemble_local(c, local[k], c.capacity * c.density, 1);
        assemble_local(c, local[k], c.time_step * c.model.p1, 0);
        NL_CUDA(cudaStreamSynchronize(c.stream));
    }
    concat(bt, bt.M, [&](Ctx& c) -> const Csr& {
        const size_t k = size_t(std::find(bt.inst.begin(), bt.inst.end(), &c) - bt.inst.begin());
        return local[k];
    }, false);
    bt.solver.stream = bt.stream;
    bt.solver.n_nodes = bt.N;
    ilt_build(bt.solver, bt.M, bt.ic, false);
    NL_REQUIRE(bt.ic.ok, NLGPU_ERR_NUMERICAL, "the ILLT of the batched local matrix failed");
    matrix_to_f32(bt.solver, bt.A, nullptr);
    NL_REQUIRE(bt.A.col16_ok, NLGPU_ERR_UNSUPPORTED, "an instance's band is wider than 16-bit column offsets");
    NL_CUDA(cudaStreamSynchronize(bt.stream));
    bt.mixed_ready = true;
}

i64 batch_solve_mixed(Batch& bt, double tolerance, i64 max_iterations, i64* iterations) {
    const i64 N = bt.N, K = bt.K;
    batch_prepare_mixed(bt);
    double* bb = bt.sc.p + BS_BB * K;
    NL_CUDA(cudaMemsetAsync(bb, 0, size_t(K) * sizeof(double), bt.stream));
    NL_LAUNCH(k_bt_norm2, RED_BLOCKS, BT_THREADS, 0, bt.stream, N, bt.b.p, bt.inst_of_row.p, bb);
    std::vector<double> h(static_cast<size_t>(K));
    NL_CUDA(cudaMemcpyAsync(h.data(), bb, size_t(K) * sizeof(double), cudaMemcpyDeviceToHost, bt.stream));
    NL_CUDA(cudaStreamSynchronize(bt.stream));
    double total = 0.0, smallest = 0.0;
    for (double v : h) {
        total += v;
        if (v > 0.0 && (smallest == 0.0 || v < smallest)) smallest = v;
    }
    if (total == 0.0) {   // every right-hand side zero: x = 0 everywhere
        NL_CUDA(cudaMemsetAsync(bt.x.p, 0, size_t(N) * sizeof(double), bt.stream));
        if (iterations) for (i64 k = 0; k < K; ++k) iterations[k] = 0;
        return 0;
    }
    const double tol_g = tolerance * std::sqrt(smallest / total);
    CgResult r = mixed_solve(bt.solver, bt.A, &bt.ic, bt.b.p, bt.x.p, tol_g, max_iterations, 1e-2, true, false,
                             NLGPU_DEFAULT_TRIANGULAR_SWEEPS, false);
    bt.last_fallback = !r.converged;
    if (!r.converged) r = cg_solve(bt.solver, bt.A, &bt.ic, bt.b.p, bt.x.p, tol_g, max_iterations, true);
    bt.last_inner = r.iterations;
    bt.last_outer = r.outer_iterations;
    NL_REQUIRE(r.converged, NLGPU_ERR_NO_CONVERGENCE, "the batched step did not converge");
    if (iterations) for (i64 k = 0; k < K; ++k) iterations[k] = r.iterations;
    return r.iterations;
}

}  // namespace

void batch_last_solve(const Batch& bt, i64* inner, i64* outer, int* fallback) {
    *inner = bt.method == NLGPU_BATCH_MIXED_ILLT ? bt.last_inner : 0;
    *outer = bt.method == NLGPU_BATCH_MIXED_ILLT ? bt.last_outer : 0;
    *fallback = bt.method == NLGPU_BATCH_MIXED_ILLT && bt.last_fallback ? 1 : 0;
}

void batch_set_method(Batch& bt, int method) {
    NL_REQUIRE(method == NLGPU_BATCH_IDENTITY_FP64 || method == NLGPU_BATCH_MIXED_ILLT, NLGPU_ERR_ARG,
               "batch method: NLGPU_BATCH_IDENTITY_FP64 or NLGPU_BATCH_MIXED_ILLT");
    bt.method = method;
}

// one implicit-Euler step of every instance; returns the largest iteration count
i64 batch_step(Batch& bt, const double* dirichlet_values, double tolerance, i64 max_iterations, i64* iterations) {
    const i64 N = bt.N, K = bt.K;
    const double tol2 = tolerance * tolerance;
    const double cap = double(std::min<i64>(max_iterations, i64(1) << 40));
    double* sc = bt.sc.p;
    bt.dval.upload(dirichlet_values, size_t(K), bt.stream);
    // right-hand side: C T_prev + dt f, minus dt K_bound x_D, x_D on Dirichlet rows
    NL_LAUNCH(k_bt_xd, grid_for(N, 256), 256, 0, bt.stream, N, bt.inst_of_row.p, bt.is_inner.p, bt.dval.p, bt.xd.p);
    bt_spmv(bt, bt.C, bt.x.p, bt.tmp.p, nullptr, false);
    NL_LAUNCH(k_bt_axpy, grid_for(N, 256), 256, 0, bt.stream, N, bt.rhs_dt.p, bt.tmp.p);
    NL_LAUNCH(k_bt_first_kind, grid_for(N * 32, 256, 152 * 64), 256, 0, bt.stream, N, bt.B.rowptr.p, bt.B.col.p,
              bt.B.val.p, bt.tmp.p, bt.xd.p, bt.is_inner.p, bt.b.p);
    if (bt.method == NLGPU_BATCH_MIXED_ILLT) return batch_solve_mixed(bt, tolerance, max_iterations, iterations);
    // CG from x0 = T_prev: r = b - A x, p = r, |r|^2 and |b|^2 per instance
    NL_CUDA(cudaMemsetAsync(sc, 0, size_t(K) * BS_COUNT * sizeof(double), bt.stream));
    bt_spmv(bt, bt.A, bt.x.p, bt.q.p, nullptr, false);
    NL_LAUNCH(k_bt_start, RED_BLOCKS, BT_THREADS, 0, bt.stream, N, bt.b.p, bt.q.p, bt.r.p, bt.p.p, bt.inst_of_row.p, sc, K);
    NL_LAUNCH(k_bt_first, 1, 256, 0, bt.stream, K, sc, tol2);
    // the iteration chunk as a graph (captured once per tolerance / cap)
    if (!bt.chunk || bt.chunk_tol2 != tol2 || bt.chunk_cap != cap) {
        if (bt.chunk) { cudaGraphExecDestroy(bt.chunk); bt.chunk = nullptr; }
        cudaGraph_t g = nullptr;
        const i64 before = g_launches.load();
        NL_CUDA(cudaStreamBeginCapture(bt.stream, cudaStreamCaptureModeThreadLocal));
        for (int it = 0; it < BT_ITERS; ++it) {
            const int parity = it & 1;
            bt_spmv(bt, bt.A, bt.p.p, bt.q.p, sc + BS_PQ * K, true);
            NL_LAUNCH(k_bt_update_xr, RED_BLOCKS, BT_THREADS, 0, bt.stream, N, bt.x.p, bt.r.p, bt.p.p, bt.q.p,
                      bt.inst_of_row.p, sc, K, parity);
            NL_LAUNCH(k_bt_update_p, RED_BLOCKS, BT_THREADS, 0, bt.stream, N, bt.p.p, bt.r.p, bt.inst_of_row.p, sc, K,
                      parity);
            NL_LAUNCH(k_bt_check, 1, 256, 0, bt.stream, K, sc, parity, tol2, cap, bt.running.p);
        }
        NL_CUDA(cudaStreamEndCapture(bt.stream, &g));
        bt.chunk_kernels = int(g_launches.load() - before);
        g_launches.fetch_sub(bt.chunk_kernels);   // counted when the graph is launched
        const cudaError_t e = cudaGraphInstantiate(&bt.chunk, g, 0);
        cudaGraphDestroy(g);
        NL_CUDA(e);
        bt.chunk_tol2 = tol2;
        bt.chunk_cap = cap;
    }
    i64 chunks = 0;
    for (;;) {
        NL_CUDA(cudaGraphLaunch(bt.chunk, bt.stream));
        g_launches.fetch_add(bt.chunk_kernels);
        ++chunks;
        int running = 0;
        NL_CUDA(cudaMemcpyAsync(&running, bt.running.p, sizeof running, cudaMemcpyDeviceToHost, bt.stream));
        NL_CUDA(cudaStreamSynchronize(bt.stream));
        if (running == 0 || double(chunks * BT_ITERS) >= cap + BT_ITERS) break;
    }
    std::vector<double> host(static_cast<size_t>(K));
    NL_CUDA(cudaMemcpyAsync(host.data(), sc + BS_ITERS * K, size_t(K) * sizeof(double), cudaMemcpyDeviceToHost, bt.stream));
    NL_CUDA(cudaStreamSynchronize(bt.stream));
    i64 worst = 0;
    for (i64 k = 0; k < K; ++k) {
        if (iterations) iterations[k] = i64(host[size_t(k)]);
        worst = std::max(worst, i64(host[size_t(k)]));
    }
    return worst;
}

void batch_temperature(Batch& bt, i64 index, double* out) {
    NL_REQUIRE(index >= 0 && index < bt.K, NLGPU_ERR_ARG, "instance index out of range");
    const size_t off = size_t(bt.row_off[size_t(index)]), n = size_t(bt.row_off[size_t(index) + 1]) - off;
    NL_CUDA(cudaMemcpyAsync(out, bt.x.p + off, n * sizeof(double), cudaMemcpyDeviceToHost, bt.stream));
    NL_CUDA(cudaStreamSynchronize(bt.stream));
}

cudaStream_t batch_stream(Batch& bt) { return bt.stream; }

void batch_sizes(const Batch& bt, i64* rows, i64* system_entries) {
    for (size_t k = 0; k < bt.inst.size(); ++k) {
        rows[k] = bt.row_off[k + 1] - bt.row_off[k];
        system_entries[k] = bt.inst[k]->full.nnz;
    }
}

}  // namespace nlgpu
