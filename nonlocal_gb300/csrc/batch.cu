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
// the same rows, but every lane of a warp stays in the loop while any lane has
// a row (i - lane is the warp's first row): for loops that call seg_add, whose
// shuffles need the whole warp; lanes past the end pass instance -1
#define BT_WARP_ROWS(i)                                                                          \
    for (i64 i = blockIdx.x * i64(blockDim.x) + threadIdx.x; i - i64(threadIdx.x & 31) < n; \
         i += i64(gridDim.x) * blockDim.x)

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
// from the instance's mean row length, so that every lane reads about twelve
// int4 groups), and the warps take blocks in turn (grid stride).  The
// instances' rows differ in length by two orders of magnitude (r/h from 2 to
// 26).  On GB300's two-lane FP64 pipe every warp-wide FP64 add costs as much
// as a warp of FMAs, so the reductions are kept rare: a row's g partial sums
// meet in log2 g shuffle steps, and the optional per-instance products w.y
// (w = x when w is null) and y.y (dot2) stay in the lanes' registers while a
// warp's blocks belong to one instance; one warp sum and one FP64 atomic each
// when the instance changes (with one FP64 add per row in the loop, the
// pipe spent more on the sums than on the products).  Blocks of stopped
// instances (done[k] != 0) are skipped.
// desc: first row (bits 0-31), log2 g (bits 32-34), rows in the block (35-40).
__global__ void __launch_bounds__(BT_THREADS) k_bt_spmv(i64 nblocks, const unsigned long long* __restrict__ desc,
                                                        const i64* __restrict__ rp, const int4* __restrict__ col4,
                                                        const double2* __restrict__ val2, const double* __restrict__ x,
                                                        double* __restrict__ y, const int32_t* __restrict__ inst,
                                                        const double* __restrict__ done, double* __restrict__ dot,
                                                        const double* __restrict__ w, double* __restrict__ dot2) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const i64 warps = i64(gridDim.x) * (blockDim.x >> 5);
    const double* wv = w ? w : x;
    double acc = 0.0, acc2 = 0.0;
    int acc_inst = -1;
    auto flush = [&]() {   // warp-uniform: called by every lane
        const double a = warp_sum(acc);
        const double a2 = dot2 ? warp_sum(acc2) : 0.0;
        if (lane == 0 && acc_inst >= 0) {
            atomicAdd(dot + acc_inst, a);
            if (dot2) atomicAdd(dot2 + acc_inst, a2);
        }
        acc = acc2 = 0.0;
    };
    for (i64 bk = (blockIdx.x * i64(blockDim.x) + threadIdx.x) >> 5; bk < nblocks; bk += warps) {
        const unsigned long long d = desc[bk];
        const i64 first = i64(d & 0xffffffffull);
        const int lg = int((d >> 32) & 7), cnt = int((d >> 35) & 63);
        const int k = inst[first];
        if (done[k] != 0.0) continue;
        if (dot && k != acc_inst) {
            flush();
            acc_inst = k;
        }
        const int g = 1 << lg, sub = lane & (g - 1), slot = lane >> lg;
        const i64 r = first + slot;
        const bool active = slot < cnt;
        double s = 0.0, s2 = 0.0;
        if (active) {
            const i64 b4 = rp[r] >> 2, e4 = rp[r + 1] >> 2;
            for (i64 q = b4 + sub; q < e4; q += g) {
                const int4 c = __ldg(col4 + q);
                const double2 v0 = __ldg(val2 + 2 * q), v1 = __ldg(val2 + 2 * q + 1);
                // two FMA chains: written as one sum of products the group cost a multiply
                // and an add besides its FMAs on the FP64 pipe, which bounds this product
                s = fma(v0.x, x[c.x], s);
                s2 = fma(v0.y, x[c.y], s2);
                s = fma(v1.x, x[c.z], s);
                s2 = fma(v1.y, x[c.w], s2);
            }
            s += s2;
        }
        for (int o = g >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(full, s, o);   // within the lane group
        if (active && sub == 0) {
            y[r] = s;
            if (dot) {
                acc += s * wv[r];
                acc2 += s * s;
            }
        }
    }
    if (dot) flush();
}

// per-instance |v|^2 into acc (zeroed by the caller)
__global__ void __launch_bounds__(BT_THREADS) k_bt_norm2(i64 n, const double* __restrict__ v,
                                                         const int32_t* __restrict__ inst, double* __restrict__ acc) {
    BT_WARP_ROWS(i) seg_add(i < n ? v[i] * v[i] : 0.0, i < n ? inst[i] : -1, acc);
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
    BT_WARP_ROWS(i) {
        double v = 0.0, bi = 0.0;
        int k = -1;
        if (i < n) {
            bi = b[i];
            v = bi - q[i];
            r[i] = v; p[i] = v;
            k = inst[i];
        }
        seg_add(v * v, k, sc + BS_RR0 * K);
        seg_add(bi * bi, k, sc + BS_BB * K);
    }
}

// alpha = rr / pq per instance; x += alpha p; r -= alpha q; partial of the new r.r
__global__ void __launch_bounds__(BT_THREADS) k_bt_update_xr(i64 n, double* __restrict__ x, double* __restrict__ r,
                                                             const double* __restrict__ p, const double* __restrict__ q,
                                                             const int32_t* __restrict__ inst, double* __restrict__ sc,
                                                             i64 K, int parity) {
    const double* rr_cur = sc + (parity ? BS_RR1 : BS_RR0) * K;
    double* rr_new = sc + (parity ? BS_RR0 : BS_RR1) * K;
    BT_WARP_ROWS(i) {
        const int k = i < n ? inst[i] : -1;
        double v2 = 0.0;
        int kk = -1;
        if (k >= 0 && sc[BS_DONE * K + k] == 0.0) {
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
// row, g the smallest power of two (1 .. 32) with g * 48 >= the mean padded
// row length (about twelve int4 groups per lane)
void row_blocks(Batch& bt, const Csr& M, dbuf<unsigned long long>& out, i64& count) {
    std::vector<i64> rp(size_t(bt.N + 1));
    M.rowptr.download(rp.data(), rp.size(), bt.stream);
    NL_CUDA(cudaStreamSynchronize(bt.stream));
    std::vector<unsigned long long> desc;
    for (i64 k = 0; k < bt.K; ++k) {
        const i64 r0 = bt.row_off[size_t(k)], r1 = bt.row_off[size_t(k) + 1];
        if (r1 <= r0) continue;
        const double mean = double(rp[size_t(r1)] - rp[size_t(r0)]) / double(r1 - r0);
        int lg = 0;
        while (lg < 5 && double(1 << lg) * 48.0 < mean) ++lg;
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
              (skip_done ? bt.sc.p : bt.sc.p + bt.K * BS_COUNT) + BS_DONE * bt.K, dot, static_cast<const double*>(nullptr),
              static_cast<double*>(nullptr));
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
    // the exact IC(0): factored once for every step (the fixed-point factor,
    // cheaper to build, took 41 instead of 31 to 41 FCG iterations a step)
    ilt_build(bt.solver, bt.M, bt.ic, false, false);
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
    CgResult r = mixed_solve(bt.solver, bt.A, &bt.ic, bt.b.p, bt.x.p, tol_g, max_iterations, MIXED_UPDATE_FACTOR, true, false,
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
        CountCaptured counted;
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
        bt.chunk_kernels = int(counted.kernels);   // counted when the graph is launched
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

// ------------------------------------------------------------ stationary batch
// The stationary solves of many assembled non-symmetric systems (variable
// conductivity with a nonlocal model) at once.  The reference solves each with
// Eigen's BiCGSTAB and its diagonal preconditioner
// (stationary_heat_equation_solver_2d.hpp:105-108); here the instances' full
// matrices are concatenated into one block-diagonal system and every
// instance runs the right-preconditioned BiCGSTAB of the single-system solver
// (van der Vorst 1992) with its own scalars, from x0 = 0:
//   beta = (rho / rho_old)(alpha / omega);  p = r + beta (p - omega v);  y = D^-1 p
//   v = A y                      (one SpMV over all rows; r0.v per instance)
//   alpha = rho / r0.v;  s = r - alpha v;  z = D^-1 s
//   t = A z                      (one SpMV; t.s and t.t per instance)
//   omega = t.s / t.t;  x += alpha y + omega z;  r = s - omega t   (|r|^2, r0.r)
// Six launches an iteration for all instances, captured as CUDA-graph chunks;
// a stopped instance's rows are skipped.  An instance stops when its
// recurrence residual meets the tolerance, at the iteration cap, or when the
// recurrence breaks down (rho or omega vanishing, a non-finite scalar); then
// the true residuals decide, and the instances that miss the tolerance start
// again from their x with r0 = b - A x (at most 16 rounds), as the
// single-system solver does.  With `illt` the preconditioner is instead the
// ILLT of every instance's p1 K_local (this library's addition: the local
// part is symmetric also with a conductivity field), applied in FP32 by the
// single-system Jacobi sweeps and widened; the products, vectors and scalars
// stay FP64.

namespace {

constexpr int BB_ITERS = 16;   // iterations per captured chunk (even)
constexpr int BB_ROUNDS = 16;  // starts from the true residual
// per-instance scalars (double [K] each); RHO0 / RHO1 alternate with the parity;
// FIN marks an instance whose true residual met the tolerance (or the cap)
enum { BB_BB = 0, BB_RHO0, BB_RHO1, BB_R0V, BB_TS, BB_TT, BB_RR, BB_ALPHA, BB_OMEGA, BB_DONE, BB_ITERS_S, BB_FIN,
       BB_COUNT };

// r = r0 = b - q (q = A x); p = v = 0; r0.r per instance into RHO0 (zeroed
// by the caller), and |b|^2 into BB on the first start
__global__ void __launch_bounds__(BT_THREADS) k_bb_start(i64 n, const double* __restrict__ b, const double* __restrict__ q,
                                                         double* __restrict__ r, double* __restrict__ r0,
                                                         double* __restrict__ p, double* __restrict__ v,
                                                         const int32_t* __restrict__ inst, double* __restrict__ sc, i64 K,
                                                         int first) {
    BT_WARP_ROWS(i) {
        double bi = 0.0, ri = 0.0;
        int k = -1;
        if (i < n) {
            bi = b[i];
            ri = bi - q[i];
            r[i] = ri; r0[i] = ri; p[i] = 0.0; v[i] = 0.0;
            k = inst[i];
        }
        seg_add(ri * ri, k, sc + BB_RHO0 * K);
        if (first) seg_add(bi * bi, k, sc + BB_BB * K);
    }
}

// the scalars of a start: rho = r0.r, |r|^2 = rho, rho_old = alpha = omega = 1;
// the instances marked final stay stopped (on the first start: b = 0)
__global__ void k_bb_first(i64 K, double* __restrict__ sc, int first) {
    for (i64 k = threadIdx.x; k < K; k += blockDim.x) {
        if (first) {
            sc[BB_ITERS_S * K + k] = 0.0;
            sc[BB_FIN * K + k] = sc[BB_BB * K + k] == 0.0 ? 1.0 : 0.0;
        }
        sc[BB_RR * K + k] = sc[BB_RHO0 * K + k];
        sc[BB_RHO1 * K + k] = 1.0;
        sc[BB_ALPHA * K + k] = 1.0;
        sc[BB_OMEGA * K + k] = 1.0;
        sc[BB_R0V * K + k] = 0.0;
        sc[BB_TS * K + k] = 0.0;
        sc[BB_TT * K + k] = 0.0;
        sc[BB_DONE * K + k] = sc[BB_FIN * K + k];
    }
}

// dinv = 1 / diagonal (1 where it is zero) of the concatenated full rows
__global__ void k_bb_jacobi(i64 n, const i64* __restrict__ rp, const int32_t* __restrict__ col,
                            const double* __restrict__ val, double* __restrict__ dinv) {
    BT_ROWS(r) {
        double d = 0.0;
        for (i64 k = rp[r]; k < rp[r + 1]; ++k)
            if (col[k] == int32_t(r)) d += val[k];
        dinv[r] = d != 0.0 ? 1.0 / d : 1.0;
    }
}

// p = r + beta (p - omega v); y = dinv p, or p32 = p for the ILLT (which then writes y)
__global__ void k_bb_p(i64 n, const double* __restrict__ r, double* __restrict__ p, const double* __restrict__ v,
                       const double* __restrict__ dinv, double* __restrict__ y, float* __restrict__ p32,
                       const int32_t* __restrict__ inst, const double* __restrict__ sc, i64 K, int q) {
    const double* rho = sc + (q ? BB_RHO1 : BB_RHO0) * K;
    const double* rho_old = sc + (q ? BB_RHO0 : BB_RHO1) * K;
    BT_ROWS(i) {
        const int k = inst[i];
        if (sc[BB_DONE * K + k] != 0.0) continue;
        const double w = sc[BB_OMEGA * K + k];
        const double beta = (rho[k] / rho_old[k]) * (sc[BB_ALPHA * K + k] / w);
        const double pi = r[i] + beta * (p[i] - w * v[i]);
        p[i] = pi;
        if (p32) p32[i] = float(pi);
        else y[i] = dinv[i] * pi;
    }
}

// alpha = rho / r0.v; s = r - alpha v; z = dinv s, or s32 = s for the ILLT.
// Block 0 clears the accumulators the x / r update adds into (nothing reads
// them here).
__global__ void k_bb_s(i64 n, const double* __restrict__ r, const double* __restrict__ v, const double* __restrict__ dinv,
                       double* __restrict__ s, double* __restrict__ z, float* __restrict__ s32,
                       const int32_t* __restrict__ inst, double* __restrict__ sc, i64 K, int q) {
    const double* rho = sc + (q ? BB_RHO1 : BB_RHO0) * K;
    BT_ROWS(i) {
        const int k = inst[i];
        if (sc[BB_DONE * K + k] != 0.0) continue;
        const double alpha = rho[k] / sc[BB_R0V * K + k];
        const double si = r[i] - alpha * v[i];
        s[i] = si;
        if (s32) s32[i] = float(si);
        else z[i] = dinv[i] * si;
    }
    if (blockIdx.x == 0)
        for (i64 k = threadIdx.x; k < K; k += blockDim.x) {
            sc[(q ? BB_RHO0 : BB_RHO1) * K + k] = 0.0;
            sc[BB_RR * K + k] = 0.0;
        }
}

// omega = t.s / t.t; x += alpha y + omega z; r = s - omega t; |r|^2 and r0.r per instance
__global__ void __launch_bounds__(BT_THREADS) k_bb_xr(i64 n, double* __restrict__ x, const double* __restrict__ y,
                                                      const double* __restrict__ z, const double* __restrict__ s,
                                                      const double* __restrict__ t, double* __restrict__ r,
                                                      const double* __restrict__ r0, const int32_t* __restrict__ inst,
                                                      double* __restrict__ sc, i64 K, int q) {
    const double* rho = sc + (q ? BB_RHO1 : BB_RHO0) * K;
    double* rho_new = sc + (q ? BB_RHO0 : BB_RHO1) * K;
    BT_WARP_ROWS(i) {
        const int k = i < n ? inst[i] : -1;
        double rr = 0.0, r0r = 0.0;
        int kk = -1;
        if (k >= 0 && sc[BB_DONE * K + k] == 0.0) {
            const double alpha = rho[k] / sc[BB_R0V * K + k];
            const double tt = sc[BB_TT * K + k];
            const double omega = tt > 0.0 ? sc[BB_TS * K + k] / tt : 0.0;
            x[i] += alpha * y[i] + omega * z[i];
            const double ri = s[i] - omega * t[i];
            r[i] = ri;
            rr = ri * ri;
            r0r = r0[i] * ri;
            kk = k;
        }
        seg_add(rr, kk, sc + BB_RR * K);
        seg_add(r0r, kk, rho_new);
    }
}

// per instance: keep alpha and omega, count the iteration, stop on
// |r| <= tol |b|, the cap or a breakdown; clear the SpMV accumulators and
// count the running instances
__global__ void k_bb_check(i64 K, double* __restrict__ sc, int q, double tol2, double max_iterations,
                           int* __restrict__ running) {
    __shared__ int cnt;
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    for (i64 k = threadIdx.x; k < K; k += blockDim.x) {
        if (sc[BB_DONE * K + k] == 0.0) {
            const double rho_new = sc[(q ? BB_RHO0 : BB_RHO1) * K + k];
            const double alpha = sc[(q ? BB_RHO1 : BB_RHO0) * K + k] / sc[BB_R0V * K + k];
            const double tt = sc[BB_TT * K + k];
            const double omega = tt > 0.0 ? sc[BB_TS * K + k] / tt : 0.0;
            const double rr = sc[BB_RR * K + k], bb = sc[BB_BB * K + k];
            sc[BB_ALPHA * K + k] = alpha;
            sc[BB_OMEGA * K + k] = omega;
            sc[BB_ITERS_S * K + k] += 1.0;
            const bool broke = !isfinite(alpha) || !isfinite(omega) || omega == 0.0 || !isfinite(rr) ||
                               !(fabs(rho_new) >= 1e-30 * bb);
            if (rr <= tol2 * bb || broke || sc[BB_ITERS_S * K + k] >= max_iterations) sc[BB_DONE * K + k] = 1.0;
            else atomicAdd(&cnt, 1);
        }
        sc[BB_R0V * K + k] = 0.0;
        sc[BB_TS * K + k] = 0.0;
        sc[BB_TT * K + k] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) running[BT_RUN_SLOT] = cnt;
}

// y = the FP32 preconditioner output, widened
__global__ void k_bb_widen(i64 n, const float* __restrict__ a, double* __restrict__ y) {
    BT_ROWS(i) y[i] = double(a[i]);
}

// per instance |b - q|^2 into acc (zeroed by the caller)
__global__ void __launch_bounds__(BT_THREADS) k_bb_residual(i64 n, const double* __restrict__ b, const double* __restrict__ q,
                                                            const int32_t* __restrict__ inst, double* __restrict__ acc) {
    BT_WARP_ROWS(i) {
        const double d = i < n ? b[i] - q[i] : 0.0;
        seg_add(d * d, i < n ? inst[i] : -1, acc);
    }
}

}  // namespace

std::vector<CgResult> batch_bicgstab(const std::vector<Ctx*>& instances, double tolerance, i64 max_iterations,
                                     bool illt) {
    Batch bt;
    NL_CUDA(cudaStreamCreateWithFlags(&bt.stream, cudaStreamNonBlocking));
    struct StreamGuard {
        Batch& b;
        ~StreamGuard() {
            if (b.chunk) cudaGraphExecDestroy(b.chunk);
            cudaStreamSynchronize(b.stream);
            cudaStreamDestroy(b.stream);
        }
    } guard{bt};
    bt.inst = instances;
    bt.K = i64(instances.size());
    bt.row_off.assign(size_t(bt.K + 1), 0);
    PhaseTimer timer(bt.stream, "batch_bicgstab");
    for (i64 k = 0; k < bt.K; ++k) {
        Ctx& c = *instances[size_t(k)];
        NL_REQUIRE(c.inner_ready && !c.symmetric && c.full.rows == c.n_nodes, NLGPU_ERR_STATE,
                   "every instance needs its assembled non-symmetric system");
        NL_CUDA(cudaStreamSynchronize(c.stream));
        bt.row_off[size_t(k) + 1] = bt.row_off[size_t(k)] + c.n_nodes;
    }
    const i64 N = bt.row_off.back(), K = bt.K;
    bt.N = N;
    NL_REQUIRE(N < (i64(1) << 31), NLGPU_ERR_UNSUPPORTED, "more than 2^31 rows in one batch");
    bt.inst_of_row.resize(size_t(N));
    concat(bt, bt.A, [](Ctx& c) -> const Csr& { return c.full; }, true);
    row_blocks(bt, bt.A, bt.blocks_A, bt.nblocks_A);
    timer.mark("concatenation, row blocks");
    // the local ILLT preconditioner: p1 K_local of every instance (symmetric also with a
    // conductivity field: the field enters at the element's own quadrature points),
    // block-diagonal, factored by the fixed-point form of IC(0) (rebuilt with every
    // batch) and applied by FP32 Jacobi sweeps
    if (illt) {
        std::vector<Csr> local(instances.size());
        for (size_t k = 0; k < instances.size(); ++k) {
            Ctx& c = *instances[k];
            build_patterns(c, true, true, local[k], nullptr, nullptr, nullptr);
            assemble_local(c, local[k], c.model.p1, 0);
            NL_CUDA(cudaStreamSynchronize(c.stream));
        }
        concat(bt, bt.M, [&](Ctx& c) -> const Csr& {
            const size_t k = size_t(std::find(bt.inst.begin(), bt.inst.end(), &c) - bt.inst.begin());
            return local[k];
        }, false);
        bt.solver.stream = bt.stream;
        bt.solver.n_nodes = N;
        ilt_build(bt.solver, bt.M, bt.ic, false, true);
        illt = bt.ic.ok;   // the diagonal otherwise (as the reference)
        timer.mark("local matrices, ILLT");
    }
    dbuf<double> r0, v, s, t, y, z, dinv, acc;
    dbuf<float> in32, out32;
    for (auto* b : {&bt.x, &bt.b, &bt.r, &bt.p, &r0, &v, &s, &t, &y, &z, &dinv}) b->resize(size_t(N));
    if (illt) {
        in32.resize(size_t(N));
        out32.resize(size_t(N));
    }
    const int sweeps = NLGPU_DEFAULT_TRIANGULAR_SWEEPS;
    auto precondition = [&](double* out) {   // out = M^-1 in32 (FP32 sweeps), widened
        ilt_apply32(bt.solver, bt.ic, in32.p, out32.p, sweeps);
        NL_LAUNCH(k_bb_widen, grid_for(N, 256), 256, 0, bt.stream, N, out32.p, out);
    };
    if (illt) {   // the first application outside the capture (lazy set-up)
        in32.zero(bt.stream);
        precondition(y.p);
    }
    timer.mark("vectors");
    for (i64 k = 0; k < K; ++k) {
        Ctx& c = *instances[size_t(k)];
        NL_CUDA(cudaMemcpyAsync(bt.b.p + bt.row_off[size_t(k)], c.rhs.p, size_t(c.n_nodes) * sizeof(double),
                                cudaMemcpyDeviceToDevice, bt.stream));
    }
    bt.sc.resize(size_t(K) * BB_COUNT);
    bt.sc.zero(bt.stream);
    bt.running.resize(1);
    acc.resize(size_t(K));
    double* sc = bt.sc.p;
    const double tol2 = tolerance * tolerance;
    const double cap = double(std::min<i64>(max_iterations, i64(1) << 40));
    NL_LAUNCH(k_bb_jacobi, grid_for(N, 256), 256, 0, bt.stream, N, bt.A.rowptr.p, bt.A.col.p, bt.A.val.p, dinv.p);
    NL_CUDA(cudaMemsetAsync(bt.x.p, 0, size_t(N) * sizeof(double), bt.stream));
    NL_CUDA(cudaMemsetAsync(t.p, 0, size_t(N) * sizeof(double), bt.stream));   // A x for x = 0
    auto spmv = [&](const double* in, double* out, double* dot, const double* w, double* dot2) {
        NL_LAUNCH(k_bt_spmv, grid_for(bt.nblocks_A * 32, BT_THREADS, 152 * 8), BT_THREADS, 0, bt.stream, bt.nblocks_A,
                  bt.blocks_A.p, bt.A.rowptr.p, reinterpret_cast<const int4*>(bt.A.col.p),
                  reinterpret_cast<const double2*>(bt.A.val.p), in, out, bt.inst_of_row.p, sc + BB_DONE * K, dot, w,
                  dot2);
    };
    std::vector<double> h(size_t(K) * BB_COUNT), res2(static_cast<size_t>(K)), fin(static_cast<size_t>(K));
    std::vector<CgResult> out(static_cast<size_t>(K));
    for (int round = 0; round < BB_ROUNDS; ++round) {
        const int first = round == 0 ? 1 : 0;
        NL_CUDA(cudaMemsetAsync(sc + BB_RHO0 * K, 0, size_t(K) * sizeof(double), bt.stream));
        NL_LAUNCH(k_bb_start, RED_BLOCKS, BT_THREADS, 0, bt.stream, N, bt.b.p, t.p, bt.r.p, r0.p, bt.p.p, v.p,
                  bt.inst_of_row.p, sc, K, first);
        NL_LAUNCH(k_bb_first, 1, 256, 0, bt.stream, K, sc, first);
        if (!bt.chunk) {
            cudaGraph_t g = nullptr;
            CountCaptured counted;
            NL_CUDA(cudaStreamBeginCapture(bt.stream, cudaStreamCaptureModeThreadLocal));
            for (int it = 0; it < BB_ITERS; ++it) {
                const int q = it & 1;
                NL_LAUNCH(k_bb_p, grid_for(N, 256, RED_BLOCKS * 4), 256, 0, bt.stream, N, bt.r.p, bt.p.p, v.p, dinv.p,
                          y.p, illt ? in32.p : nullptr, bt.inst_of_row.p, sc, K, q);
                if (illt) precondition(y.p);
                spmv(y.p, v.p, sc + BB_R0V * K, r0.p, static_cast<double*>(nullptr));
                NL_LAUNCH(k_bb_s, grid_for(N, 256, RED_BLOCKS * 4), 256, 0, bt.stream, N, bt.r.p, v.p, dinv.p, s.p, z.p,
                          illt ? in32.p : nullptr, bt.inst_of_row.p, sc, K, q);
                if (illt) precondition(z.p);
                spmv(z.p, t.p, sc + BB_TS * K, s.p, sc + BB_TT * K);
                NL_LAUNCH(k_bb_xr, RED_BLOCKS, BT_THREADS, 0, bt.stream, N, bt.x.p, y.p, z.p, s.p, t.p, bt.r.p, r0.p,
                          bt.inst_of_row.p, sc, K, q);
                NL_LAUNCH(k_bb_check, 1, 256, 0, bt.stream, K, sc, q, tol2, cap, bt.running.p);
            }
            NL_CUDA(cudaStreamEndCapture(bt.stream, &g));
            bt.chunk_kernels = int(counted.kernels);   // counted when the graph is launched
            const cudaError_t e = cudaGraphInstantiate(&bt.chunk, g, 0);
            cudaGraphDestroy(g);
            NL_CUDA(e);
        }
        for (i64 chunks = 1;; ++chunks) {
            NL_CUDA(cudaGraphLaunch(bt.chunk, bt.stream));
            g_launches.fetch_add(bt.chunk_kernels);
            int running = 0;
            NL_CUDA(cudaMemcpyAsync(&running, bt.running.p, sizeof running, cudaMemcpyDeviceToHost, bt.stream));
            NL_CUDA(cudaStreamSynchronize(bt.stream));
            if (running == 0 || double(chunks * BB_ITERS) >= cap + BB_ITERS) break;
        }
        // the true residual of every instance decides (t = A x over every row)
        acc.zero(bt.stream);
        NL_CUDA(cudaMemsetAsync(sc + BB_DONE * K, 0, size_t(K) * sizeof(double), bt.stream));
        spmv(bt.x.p, t.p, nullptr, nullptr, nullptr);
        NL_LAUNCH(k_bb_residual, RED_BLOCKS, BT_THREADS, 0, bt.stream, N, bt.b.p, t.p, bt.inst_of_row.p, acc.p);
        NL_CUDA(cudaMemcpyAsync(h.data(), sc, h.size() * sizeof(double), cudaMemcpyDeviceToHost, bt.stream));
        NL_CUDA(cudaMemcpyAsync(res2.data(), acc.p, res2.size() * sizeof(double), cudaMemcpyDeviceToHost, bt.stream));
        NL_CUDA(cudaStreamSynchronize(bt.stream));
        bool all = true;
        for (i64 k = 0; k < K; ++k) {
            CgResult& r = out[size_t(k)];
            const double bb = h[size_t(BB_BB * K + k)];
            r.iterations = i64(h[size_t(BB_ITERS_S * K + k)]);
            r.residual = bb > 0.0 ? std::sqrt(res2[size_t(k)] / bb) : 0.0;
            r.converged = r.residual <= tolerance;
            const bool final = r.converged || r.iterations >= max_iterations || !std::isfinite(r.residual);
            fin[size_t(k)] = final ? 1.0 : 0.0;
            all = all && final;
        }
        timer.mark("round");
        if (all) break;
        NL_CUDA(cudaMemcpyAsync(sc + BB_FIN * K, fin.data(), size_t(K) * sizeof(double), cudaMemcpyHostToDevice, bt.stream));
    }
    for (i64 k = 0; k < K; ++k) {
        Ctx& c = *instances[size_t(k)];
        c.temperature.resize(size_t(c.n_nodes));
        NL_CUDA(cudaMemcpyAsync(c.temperature.p, bt.x.p + bt.row_off[size_t(k)], size_t(c.n_nodes) * sizeof(double),
                                cudaMemcpyDeviceToDevice, bt.stream));
    }
    NL_CUDA(cudaStreamSynchronize(bt.stream));
    return out;
}

}  // namespace nlgpu
