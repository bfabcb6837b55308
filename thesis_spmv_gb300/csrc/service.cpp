// service.cpp -- the batched power-method service (include/pwmsvc.h).
//
// Host side of the serving loop: a FIFO queue, admission against live-slot
// and HBM budgets, per-solve phase control (FP32 / BF16 bulk, FP64
// refinement), the per-class device tables the batched kernels read
// (batch.h), and one round per pwmsvc_step: the three class branches
// (FP64, FP32, BF16) run as parallel streams inside one captured CUDA graph.
// Matrices are built (generated or uploaded, then planned) on each request's
// own stream, so admissions overlap the previous round on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <system_error>
#include <thread>
#include <vector>

#include "batch.h"
#include "internal.h"
#include "matrix_impl.h"
#include "pwmsvc.h"

using namespace pwmgpu;

namespace {

using Clock = std::chrono::steady_clock;

// Precision classes; the FP32 / BF16 iterations of matrices that fit the
// SELL-32 layout run in their own classes (kernel per layout).
enum { kClsF64 = 0, kClsF32 = 1, kClsBF16 = 2, kClsF32Sell = 3, kClsBF16Sell = 4, kNumCls = 5 };
constexpr int kSides = kNumCls - 1;  // forked streams of a round (the F64 class runs on the service stream)

// Residual at which a mixed solve leaves the FP32 / BF16 phase (as in
// pwmgpu_solve).
constexpr double kSvcSwitchRel = 2e-6;

// Precision tuner of the mixed solves: a MIXED request runs its first round
// in FP64 (the probe); from the residual r after those C steps it projects
// the steps to tol at that rate, C ln(tol) / ln(r).  A matrix that would
// finish within kProbeRounds rounds stays in FP64 -- a low-precision phase
// there costs a phase switch and an extra round for the few steps it would
// cheapen (the service's 128 random Poisson(8)-row matrices: 696 mixed vs
// 861 FP64 solves/s with the phase, the batch-wide figure without the probe);
// slower ones take the FP32 / BF16 bulk phase from the probe's iterate on.
// The choice depends only on the solve's own residual, so a solve gives the
// same bits alone and in any mix.
constexpr int kProbeRounds = 5;

// Requests admitted per step while a round runs: a burst that arrives
// while solves are live is built a slice at a time beside their rounds.
// With nothing live (a batch submitted at once) the step admits all it can:
// there is no round to overlap, and the solves started later would only
// finish later.
constexpr int kAdmitPerStep = 32;
// Host threads that build a step's admissions while its round runs (each on
// its own stream: the builds are chains of short kernels, allocations and
// stream syncs, bound by their latency, not by the GPU).
constexpr int kAdmitThreads = 8;

struct Req {
    int64_t id = 0;
    pwmsvc_request spec{};
    std::vector<int32_t> rs, ci, ri;
    std::vector<double> vals, x0;
    int state = PWMSVC_QUEUED;
    int error = PWMGPU_OK;
    double t_submit = 0, t_admit = 0, t_done = 0;
    pwmgpu_matrix* m = nullptr;
    size_t est = 0, bytes = 0;
    int n = 0;
    int cls = kClsF64;
    bool low = false;
    bool probe = false;  // MIXED: the first round runs in FP64 (the precision tuner's probe)
    int low_cls = kClsF64;
    int slot = -1;
    const void* valp_low = nullptr;
    int iterations = 0, iterations_low = 0, rounds_in_phase = 0, converged = 0;
    double prev_rel = 1.0, rel = INFINITY, lambda = 0.0;
    bool exact_set = false;  // the state asks for the residual's row pass
    std::vector<double> u;
};

struct ClassDev {
    BatchTable* dT = nullptr;
    BatchSlot* d_slots = nullptr;
    size_t slots_cap = 0;
    int* tile_slot = nullptr;
    size_t slot_cap = 0;
    double* row_part = nullptr;
    size_t row_cap = 0;
    double* res_part = nullptr;
    size_t res_cap = 0;
    double* grp_part = nullptr;
    size_t grp_cap = 0;
};

int grow(double** p, size_t* cap, size_t need) {
    if (*cap >= need && *p) return PWMGPU_OK;
    size_t c = std::max(need, *cap * 2);
    dfree(*p);
    *cap = 0;
    TRY(dalloc(p, c));
    *cap = c;
    return PWMGPU_OK;
}

// Device bytes of a solve: CRS row starts, the lane-interleaved plan (columns,
// FP64 values, records, masks, coordinates, carries), the CRS arrays while
// the plan is built, FP64 vectors, and FP32 values + vectors for a
// low-precision phase.
size_t solve_bytes(long long nor, long long nnz, int precision) {
    const long long nsub = (nor + nnz + 32 * kMliIpt - 1) / (32 * kMliIpt);
    const long long elems = nnz + 7 * nsub + 16;
    long long b = 4 * (nor + 1) + 12 * elems + nsub * (32 + 64 + 8 + 8) + 12 * nnz + 2 * 8 * (nor + 16) + 65536;
    // FP32 values and vectors; a SELL-32 copy (at most 1.25 nnz elements of
    // 2-byte columns and 4-byte values) where the matrix fits it
    if (precision != PWMGPU_PREC_F64) b += 4 * elems + 2 * 4 * (nor + 16) + 8 * nnz;
    return (size_t)b;
}

}  // namespace

struct pwmsvc {
    pwmsvc_config cfg{};
    int device = 0, sm_count = 1;
    cudaStream_t stream = nullptr;
    cudaStream_t side[kSides] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[kSides] = {}, ev0 = nullptr, ev1 = nullptr;
    Clock::time_point t0;
    int64_t next_id = 1;
    std::deque<Req*> queue;
    std::vector<Req*> live;
    std::map<int64_t, std::unique_ptr<Req>> all;
    size_t in_use = 0;
    SlotState* d_states = nullptr;
    SlotState* h_states = nullptr;
    std::vector<int> free_states;
    int* d_status = nullptr;
    int* h_status = nullptr;  // pinned: read back while the host admits requests
    std::vector<void*> deferred;  // device frees of the matrix builds, made after the round
    ClassDev cls[kNumCls];
    bool dirty = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int64_t submitted = 0, finished = 0, failed = 0, rounds = 0;
    double gpu_ms = 0.0;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    void release() {
        free_deferred(deferred);
        for (auto& kv : all)
            if (kv.second->m) pwmgpu_destroy(kv.second->m);
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        for (auto& c : cls) {
            dfree(c.dT);
            dfree(c.d_slots);
            dfree(c.tile_slot);
            dfree(c.row_part);
            dfree(c.res_part);
            dfree(c.grp_part);
        }
        dfree(d_states);
        dfree(d_status);
        if (h_states) cudaFreeHost(h_states);
        if (h_status) cudaFreeHost(h_status);
        for (cudaEvent_t e : {fork_ev, ev0, ev1})
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : join_ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
        for (cudaStream_t s : side)
            if (s) cudaStreamDestroy(s);
    }
};

namespace {

// The FP32 / BF16 copies of a request's matrix (values, SELL-32 slices where
// the matrix fits them) and vectors, made on its own stream when its solve
// enters the low-precision phase.
int prepare_low(Req* r) {
    pwmgpu_matrix* m = r->m;
    const pwmsvc_request& q = r->spec;
    int cfg = kCfgF32, pg = 0;
    TRY(ensure_low_values(m, q.precision == PWMGPU_PREC_MIXED, &cfg, &r->valp_low, &pg));
    TRY(ensure_fvectors(m));
    if (sell_for(m, cfg)) {
        r->valp_low = cfg == kCfgBF16 ? m->sell.valbf : (const void*)m->sell.val32;
        r->low_cls = cfg == kCfgBF16 ? kClsBF16Sell : kClsF32Sell;
    } else {
        r->low_cls = cfg == kCfgBF16 ? kClsBF16 : kClsF32;
    }
    CU(cudaStreamSynchronize(m->stream));
    return PWMGPU_OK;
}

// Build the request's matrix and start vector on its own stream.
int admit(pwmsvc* S, Req* r) {
    const pwmsvc_request& q = r->spec;
    TRY(pwmgpu_create(PWMGPU_FMT_MERGE, 1, &r->m));
    pwmgpu_matrix* m = r->m;
    m->skip_tune = true;
    if (q.source == PWMSVC_SRC_POISSON) {
        TRY(pwmgpu_generate_poisson(m, q.grid_m, q.grid_n));
    } else if (q.source == PWMSVC_SRC_RANDOM) {
        TRY(pwmgpu_generate_random(m, q.n, q.seed, q.length_dist, q.mean_len, q.sigma, q.max_len, q.band_permille,
                                   q.band_half));
    } else if (q.source == PWMSVC_SRC_TRIPLETS) {
        TRY(pwmgpu_load_triplets(m, q.nor, q.nor, q.nnz, r->ri.data(), r->ci.data(), r->vals.data()));
        r->ri.clear();
        r->ri.shrink_to_fit();
        r->ci.clear();
        r->ci.shrink_to_fit();
        r->vals.clear();
        r->vals.shrink_to_fit();
    } else {
        TRY(pwmgpu_load_csr(m, q.nor, q.nor, q.nnz, r->rs.data(), r->ci.data(), r->vals.data()));
        r->rs.clear();
        r->rs.shrink_to_fit();
        r->ci.clear();
        r->ci.shrink_to_fit();
        r->vals.clear();
        r->vals.shrink_to_fit();
    }
    r->n = m->M.nor;
    if (r->n == 0) return fail(PWMGPU_ERR_INVALID, "empty matrix");
    TRY(ensure_vectors(m));
    if (!r->x0.empty()) {
        CU(cudaMemcpyAsync(m->dx, r->x0.data(), sizeof(double) * (size_t)r->n, cudaMemcpyHostToDevice, m->stream));
    } else {
        CU(launch_fill_uniform(m->dx, r->n, q.x0_seed, m->sm_count, m->stream));
    }
    r->cls = kClsF64;
    r->low = false;
    // MIXED: the probe round first, the low-precision copies only if the
    // solve takes the low phase
    r->probe = q.precision == PWMGPU_PREC_MIXED;
    if (q.precision == PWMGPU_PREC_F32) {  // FP32 throughout: the low phase from the start
        TRY(prepare_low(r));
        CU(launch_convert_f64_f32(m->dx, m->fx, r->n, m->sm_count, m->stream));
        r->low = true;
        r->cls = r->low_cls;
    }
    CU(cudaStreamSynchronize(m->stream));
    r->bytes = solve_bytes(m->M.nor, m->M.nnz, q.precision);
    return PWMGPU_OK;
}

int reset_state(pwmsvc* S, int slot) {
    CU(cudaMemsetAsync(S->d_states + slot, 0, sizeof(SlotState), S->stream));
    return PWMGPU_OK;
}

int rebuild_tables(pwmsvc* S) {
    for (int c = 0; c < kNumCls; ++c) {
        ClassDev& D = S->cls[c];
        std::vector<BatchSlot> hs;
        int tiles = 0, fix = 0, rows = 0;
        for (Req* r : S->live) {
            if (r->cls != c) continue;
            pwmgpu_matrix* m = r->m;
            BatchSlot b{};
            b.row_start = m->M.row_start;
            b.colp = m->P.colp;
            b.valp = r->low ? r->valp_low : (const void*)m->P.valp;
            b.rec = m->P.rec;
            b.masks = m->P.masks;
            b.subc = m->P.subc;
            b.X = r->low ? (void*)m->fx : (void*)m->dx;
            b.Y = r->low ? (void*)m->fy : (void*)m->dy;
            b.carries = m->carries;
            b.nor = m->M.nor;
            b.nsub = m->P.nsub;
            if (c == kClsF32Sell || c == kClsBF16Sell) {  // slices instead of sub-tiles, no fix-up
                b.soff = m->sell.soff;
                b.col16 = m->sell.col16;
                b.nsub = m->sell.nslices;
            }
            b.tile0 = tiles;
            b.nfix = (c == kClsF32Sell || c == kClsBF16Sell) ? (b.nsub + kSellGroup - 1) / kSellGroup
                                                              : (b.nsub + kFixTiles - 1) / kFixTiles;
            b.fix0 = fix;
            b.nrow = (b.nor + kRowChunk - 1) / kRowChunk;
            b.row0 = rows;
            b.state = r->slot;
            tiles += b.nsub;
            fix += b.nfix;
            rows += b.nrow;
            hs.push_back(b);
        }
        if (D.slots_cap < hs.size() || !D.d_slots) {
            dfree(D.d_slots);
            D.slots_cap = 0;
            TRY(dalloc(&D.d_slots, std::max<size_t>(hs.size(), 64)));
            D.slots_cap = std::max<size_t>(hs.size(), 64);
        }
        if (D.slot_cap < (size_t)tiles + 1 || !D.tile_slot) {
            dfree(D.tile_slot);
            D.slot_cap = 0;
            const size_t cap = std::max<size_t>((size_t)tiles + 1, 2 * D.slot_cap);
            TRY(dalloc(&D.tile_slot, cap));
            D.slot_cap = cap;
        }
        TRY(grow(&D.row_part, &D.row_cap, 2 * (size_t)rows + 2));
        TRY(grow(&D.res_part, &D.res_cap, (size_t)rows + 1));
        if (c == kClsF32Sell || c == kClsBF16Sell) TRY(grow(&D.grp_part, &D.grp_cap, (size_t)fix + 1));
        if (!hs.empty())
            CU(cudaMemcpyAsync(D.d_slots, hs.data(), hs.size() * sizeof(BatchSlot), cudaMemcpyHostToDevice,
                               S->stream));
        BatchTable T{};
        T.nslots = (int)hs.size();
        T.ntiles = tiles;
        T.nfix = fix;
        T.nrow = rows;
        T.slots = D.d_slots;
        T.states = S->d_states;
        T.tile_slot = D.tile_slot;
        T.row_part = D.row_part;
        T.res_part = D.res_part;
        T.grp_part = D.grp_part;
        T.status = S->d_status;
        // pageable source: the copy is staged before the call returns
        CU(cudaMemcpyAsync(D.dT, &T, sizeof T, cudaMemcpyHostToDevice, S->stream));
        CU(launch_tile_slots(D.dT, T.nslots, S->stream));
        CU(cudaStreamSynchronize(S->stream));
    }
    S->dirty = false;
    return PWMGPU_OK;
}

// The round: three class branches forked from S->stream.
int enqueue_round(pwmsvc* S) {
    const int C = S->cfg.round_iterations;
    CU(cudaEventRecord(S->fork_ev, S->stream));
    for (int i = 0; i < kSides; ++i) CU(cudaStreamWaitEvent(S->side[i], S->fork_ev, 0));
    CU(launch_batch_round(kCfgF64, S->cls[kClsF64].dT, C, S->sm_count, S->stream));
    CU(launch_batch_round(kCfgF32, S->cls[kClsF32].dT, C, S->sm_count, S->side[0]));
    CU(launch_batch_round(kCfgBF16, S->cls[kClsBF16].dT, C, S->sm_count, S->side[1]));
    CU(launch_batch_round(kCfgF32, S->cls[kClsF32Sell].dT, C, S->sm_count, S->side[2], true));
    CU(launch_batch_round(kCfgBF16, S->cls[kClsBF16Sell].dT, C, S->sm_count, S->side[3], true));
    for (int i = 0; i < kSides; ++i) {
        CU(cudaEventRecord(S->join_ev[i], S->side[i]));
        CU(cudaStreamWaitEvent(S->stream, S->join_ev[i], 0));
    }
    return PWMGPU_OK;
}

int run_round(pwmsvc* S) {
    if (S->cfg.use_graph && !S->gexec) {
        CU(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_round(S);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(S->stream, &g);
        if (rc != PWMGPU_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return fail(PWMGPU_ERR_CUDA, "round capture: %s", cudaGetErrorString(e));
        S->graph = g;
        CU(cudaGraphInstantiate(&S->gexec, S->graph, 0));
    }
    CU(cudaEventRecord(S->ev0, S->stream));
    if (S->gexec) {
        CU(cudaGraphLaunch(S->gexec, S->stream));
    } else {
        TRY(enqueue_round(S));
    }
    CU(cudaEventRecord(S->ev1, S->stream));
    return PWMGPU_OK;
}

// Normalised u = v_{k-1} / ||v_{k-1}|| (the vector lambda and the residual
// belong to) into the request's host copy, then free the device memory.
int retire(pwmsvc* S, Req* r, int state) {
    pwmgpu_matrix* m = r->m;
    if (state == PWMSVC_DONE && r->spec.keep_vector) {
        const SlotState& st = S->h_states[r->slot];
        const int k = st.k;
        double* prev64;
        if (r->low) {
            float* prev = (k & 1) ? m->fx : m->fy;
            CU(launch_convert_f32_f64(prev, m->dx, r->n, m->sm_count, S->stream));
            prev64 = m->dx;
        } else {
            prev64 = (k & 1) ? m->dx : m->dy;
        }
        CU(launch_power_finalize_f64(prev64, &S->d_states[r->slot].nsq_prev, nullptr, nullptr, r->n, m->sm_count,
                                     S->stream));
        r->u.resize((size_t)r->n);
        CU(cudaMemcpyAsync(r->u.data(), prev64, sizeof(double) * (size_t)r->n, cudaMemcpyDeviceToHost, S->stream));
        CU(cudaStreamSynchronize(S->stream));
    }
    pwmgpu_destroy(m);
    r->m = nullptr;
    S->in_use -= std::min(S->in_use, r->bytes);
    if (r->slot >= 0) S->free_states.push_back(r->slot);
    r->slot = -1;
    r->state = state;
    r->t_done = S->now();
    if (state == PWMSVC_DONE) ++S->finished;
    else ++S->failed;
    S->dirty = true;
    return PWMGPU_OK;
}

// Per-solve decisions after a round (the stopping and phase rules of
// pwmgpu_solve, at round granularity).
int after_round(pwmsvc* S, int* finished) {
    const int C = S->cfg.round_iterations;
    std::vector<Req*> keep;
    for (Req* r : S->live) {
        const SlotState& st = S->h_states[r->slot];
        const pwmsvc_request& q = r->spec;
        r->iterations += C;
        if (r->low) r->iterations_low += C;
        ++r->rounds_in_phase;
        const double nsq = st.nsq_prev;
        const bool finite = std::isfinite(st.lambda) && std::isfinite(st.res2) && nsq > 0.0 && std::isfinite(nsq);
        if (!finite || st.lambda == 0.0) {
            r->error = PWMGPU_ERR_NUMERIC;
            TRY(retire(S, r, PWMSVC_FAILED));
            ++*finished;
            continue;
        }
        r->lambda = st.lambda;
        r->rel = std::sqrt(st.res2 / nsq) / std::fabs(st.lambda);
        if (r->probe) {
            r->probe = false;
            // projected steps to tol at this round's rate (r starts near 1)
            const bool fast = r->rel <= q.tol ||
                              (r->rel < 1.0 && q.tol > 0.0 &&
                               C * std::log(q.tol) / std::log(r->rel) <= (double)(kProbeRounds * C));
            const int reserve = std::max(2, std::min(64, q.max_it / 4));
            if (!fast && r->iterations < q.max_it - reserve) {
                // the bulk in FP32 / BF16 from the newest FP64 iterate on,
                // normalised first (an FP64 iterate may lie outside FP32's range)
                TRY(prepare_low(r));
                pwmgpu_matrix* m = r->m;
                double* newest = (st.k & 1) ? m->dy : m->dx;
                CU(launch_power_finalize_f64(newest, &S->d_states[r->slot].nsq, nullptr, nullptr, r->n, m->sm_count,
                                             S->stream));
                CU(launch_convert_f64_f32(newest, m->fx, r->n, m->sm_count, S->stream));
                TRY(reset_state(S, r->slot));
                r->exact_set = false;
                r->low = true;
                r->cls = r->low_cls;
                r->rounds_in_phase = 0;
                r->prev_rel = r->rel;
                S->dirty = true;
                keep.push_back(r);
                continue;
            }
        }
        bool done = false;
        if (!r->low || q.precision == PWMGPU_PREC_F32) {
            if (r->rel <= q.tol) {
                r->converged = 1;
                done = true;
            } else if (r->iterations >= q.max_it) {
                done = true;
            }
        } else {
            // mixed: leave the low-precision phase at the switch residual, when
            // it stops falling, or when only the FP64 reserve is left
            const int reserve = std::max(2, std::min(64, q.max_it / 4));
            const bool stalled = r->rounds_in_phase >= 2 && low_precision_floor(r->rel, r->prev_rel);
            if (r->rel <= std::max(q.tol, kSvcSwitchRel) || stalled || r->iterations >= q.max_it - reserve) {
                pwmgpu_matrix* m = r->m;
                float* newest = (st.k & 1) ? m->fy : m->fx;
                CU(launch_convert_f32_f64(newest, m->dx, r->n, m->sm_count, S->stream));
                TRY(reset_state(S, r->slot));
                r->exact_set = false;
                r->low = false;
                r->cls = kClsF64;
                r->rounds_in_phase = 0;
                S->dirty = true;
            }
        }
        r->prev_rel = r->rel;
        if (done) {
            TRY(retire(S, r, PWMSVC_DONE));
            ++*finished;
        } else {
            keep.push_back(r);
        }
    }
    S->live.swap(keep);
    return PWMGPU_OK;
}

}  // namespace

extern "C" {

int pwmsvc_create(const pwmsvc_config* cfg, pwmsvc** out) {
    if (!out) return fail(PWMGPU_ERR_INVALID, "null output handle");
    *out = nullptr;
    pwmsvc_config c = cfg ? *cfg : pwmsvc_config{};
    if (c.max_live <= 0) c.max_live = 1024;
    if (c.round_iterations == 0) c.round_iterations = 8;
    if (c.round_iterations < 2) return fail(PWMGPU_ERR_INVALID, "round_iterations must be >= 2");
    std::unique_ptr<pwmsvc> S(new pwmsvc());
    S->cfg = c;
    S->t0 = Clock::now();
    int rc = PWMGPU_OK;
    do {
        cudaError_t e = cudaGetDevice(&S->device);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&S->sm_count, cudaDevAttrMultiProcessorCount, S->device);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking);
        for (int i = 0; i < kSides && e == cudaSuccess; ++i)
            e = cudaStreamCreateWithFlags(&S->side[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->fork_ev, cudaEventDisableTiming);
        for (int i = 0; i < kSides && e == cudaSuccess; ++i)
            e = cudaEventCreateWithFlags(&S->join_ev[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreate(&S->ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&S->ev1);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "pwmsvc_create: %s", cudaGetErrorString(e)); break; }
        if (S->cfg.hbm_budget_bytes == 0) {
            size_t f = 0, t = 0;
            e = cudaMemGetInfo(&f, &t);
            if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "cudaMemGetInfo: %s", cudaGetErrorString(e)); break; }
            S->cfg.hbm_budget_bytes = (size_t)(0.9 * (double)f);
        }
        if ((rc = dalloc(&S->d_states, (size_t)c.max_live)) != PWMGPU_OK) break;
        if ((rc = dalloc(&S->d_status, 4)) != PWMGPU_OK) break;
        e = cudaMallocHost((void**)&S->h_states, sizeof(SlotState) * (size_t)c.max_live);
        if (e != cudaSuccess) { S->h_states = nullptr; rc = fail(PWMGPU_ERR_NOMEM, "cudaMallocHost failed"); break; }
        e = cudaMallocHost((void**)&S->h_status, sizeof(int));
        if (e != cudaSuccess) { S->h_status = nullptr; rc = fail(PWMGPU_ERR_NOMEM, "cudaMallocHost failed"); break; }
        *S->h_status = 0;
        for (auto& D : S->cls)
            if ((rc = dalloc(&D.dT, 1)) != PWMGPU_OK) break;
        if (rc != PWMGPU_OK) break;
        for (int i = c.max_live - 1; i >= 0; --i) S->free_states.push_back(i);
        e = cudaMemsetAsync(S->d_states, 0, sizeof(SlotState) * (size_t)c.max_live, S->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(S->d_status, 0, 4 * sizeof(int), S->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(S->stream);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "pwmsvc_create: %s", cudaGetErrorString(e)); break; }
        batch_prepare(S->sm_count);
        warm_launch_caches(S->sm_count);  // before builds run on several threads
        if ((rc = rebuild_tables(S.get())) != PWMGPU_OK) break;
    } while (0);
    if (rc != PWMGPU_OK) {
        S->release();
        return rc;
    }
    *out = S.release();
    return PWMGPU_OK;
}

int pwmsvc_destroy(pwmsvc* s) {
    if (!s) return PWMGPU_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->release();
    delete s;
    return PWMGPU_OK;
}

int pwmsvc_submit(pwmsvc* s, const pwmsvc_request* q, int64_t* id) {
    if (!s || !q) return fail(PWMGPU_ERR_INVALID, "null service or request");
    if (q->max_it < 2) return fail(PWMGPU_ERR_INVALID, "max_it must be at least 2");
    if (!(q->tol >= 0.0)) return fail(PWMGPU_ERR_INVALID, "tol must be >= 0");
    if (q->precision != PWMGPU_PREC_F64 && q->precision != PWMGPU_PREC_F32 && q->precision != PWMGPU_PREC_MIXED)
        return fail(PWMGPU_ERR_INVALID, "unknown precision %d", q->precision);
    std::unique_ptr<Req> r(new Req());
    r->spec = *q;
    long long nor = 0, nnz = 0;
    switch (q->source) {
        case PWMSVC_SRC_CSR:
            if (q->nor < 1 || q->nnz < 0 || !q->row_start || (q->nnz > 0 && (!q->col_ind || !q->vals)))
                return fail(PWMGPU_ERR_INVALID, "bad CSR request");
            nor = q->nor;
            nnz = q->nnz;
            r->rs.assign(q->row_start, q->row_start + nor + 1);
            r->ci.assign(q->col_ind, q->col_ind + nnz);
            r->vals.assign(q->vals, q->vals + nnz);
            break;
        case PWMSVC_SRC_TRIPLETS:
            if (q->nor < 1 || q->nnz < 0 || (q->nnz > 0 && (!q->row_ind || !q->col_ind || !q->vals)))
                return fail(PWMGPU_ERR_INVALID, "bad triplet request");
            nor = q->nor;
            nnz = q->nnz;
            r->ri.assign(q->row_ind, q->row_ind + nnz);
            r->ci.assign(q->col_ind, q->col_ind + nnz);
            r->vals.assign(q->vals, q->vals + nnz);
            break;
        case PWMSVC_SRC_POISSON:
            if (q->grid_m < 1 || q->grid_n < 1) return fail(PWMGPU_ERR_INVALID, "bad Poisson grid");
            nor = (long long)q->grid_m * q->grid_n;
            nnz = (long long)q->grid_n * (q->grid_m + 2LL * (q->grid_m - 1)) + 2LL * (q->grid_n - 1) * q->grid_m;
            break;
        case PWMSVC_SRC_RANDOM:
            if (q->n < 1 || !(q->mean_len > 0.0)) return fail(PWMGPU_ERR_INVALID, "bad random-matrix request");
            nor = q->n;
            nnz = (long long)std::ceil(q->n * std::min((double)q->n, q->mean_len) * 1.1) + 64;
            break;
        default:
            return fail(PWMGPU_ERR_INVALID, "unknown source %d", q->source);
    }
    r->spec.row_start = nullptr;
    r->spec.row_ind = nullptr;
    r->spec.col_ind = nullptr;
    r->spec.vals = nullptr;
    if (q->x0) r->x0.assign(q->x0, q->x0 + nor);
    r->spec.x0 = nullptr;
    r->n = (int)nor;
    r->est = solve_bytes(nor, nnz, q->precision);
    if (r->est > s->cfg.hbm_budget_bytes)
        return fail(PWMGPU_ERR_BUDGET, "request needs about %zu bytes, more than the service's HBM budget (%zu)",
                    r->est, s->cfg.hbm_budget_bytes);
    r->id = s->next_id++;
    r->t_submit = s->now();
    if (id) *id = r->id;
    s->queue.push_back(r.get());
    s->all[r->id] = std::move(r);
    ++s->submitted;
    return PWMGPU_OK;
}

int pwmsvc_step(pwmsvc* s, int32_t* live, int32_t* queued, int32_t* finished) {
    if (!s) return fail(PWMGPU_ERR_INVALID, "null service");
    int fin = 0;
    // the round of the solves already live goes to the GPU first; the queue's
    // matrices are built while it runs (on their own streams) and join the
    // next round
    const bool ran = !s->live.empty();
    if (ran) {
        if (s->dirty) TRY(rebuild_tables(s));
        // a solve's last possible round reports its residual from the row
        // pass (earlier rounds may take it from the round's sums while it is
        // large)
        for (Req* r : s->live) {
            const bool result_phase = !r->low || r->spec.precision == PWMGPU_PREC_F32;
            if (result_phase && !r->exact_set && r->iterations + s->cfg.round_iterations >= r->spec.max_it) {
                static const int one = 1;
                CU(cudaMemcpyAsync(&s->d_states[r->slot].exact_res, &one, sizeof(int), cudaMemcpyHostToDevice,
                                   s->stream));
                r->exact_set = true;
            }
        }
        TRY(run_round(s));
        CU(cudaMemcpyAsync(s->h_states, s->d_states, sizeof(SlotState) * (size_t)s->cfg.max_live,
                           cudaMemcpyDeviceToHost, s->stream));
        CU(cudaMemcpyAsync(s->h_status, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    }
    // admission: FIFO while slots and the HBM budget allow (by the requests'
    // estimates), the builds on up to kAdmitThreads host threads; their
    // device frees wait until the round is done (a cudaFree now would wait
    // for the round)
    std::vector<Req*> batch;
    size_t planned = s->in_use;
    const int cap = ran ? kAdmitPerStep : s->cfg.max_live;
    while (!s->queue.empty() && (int)(s->live.size() + batch.size()) < s->cfg.max_live &&
           !s->free_states.empty() && (int)batch.size() < cap) {
        Req* r = s->queue.front();
        if (!(s->live.empty() && batch.empty()) && planned + r->est > s->cfg.hbm_budget_bytes) break;
        s->queue.pop_front();
        r->t_admit = s->now();
        r->slot = s->free_states.back();
        s->free_states.pop_back();
        planned += r->est;
        batch.push_back(r);
    }
    std::vector<int> built(batch.size(), PWMGPU_OK);
    // several builders only beside a round: with the device idle (a batch
    // submitted at once) one thread built the 256-matrix batch faster (178
    // vs 170 solves/s; its 128 small random matrices 870 vs 760)
    const int nt = ran ? (int)std::min<size_t>((size_t)kAdmitThreads, batch.size()) : 1;
    if (nt <= 1) {
        defer_frees(&s->deferred);
        for (size_t i = 0; i < batch.size(); ++i) built[i] = admit(s, batch[i]);
        defer_frees(nullptr);
    } else {
        std::vector<std::vector<void*>> frees((size_t)nt + 1);
        std::atomic<int> next{0};
        auto work = [&](size_t slot) {
            cudaSetDevice(s->device);
            defer_frees(&frees[slot]);
            for (int i; (i = next.fetch_add(1)) < (int)batch.size();) built[(size_t)i] = admit(s, batch[(size_t)i]);
            defer_frees(nullptr);
        };
        std::vector<std::thread> th;
        try {
            for (int t = 0; t < nt; ++t) th.emplace_back(work, (size_t)t);
        } catch (const std::system_error&) {
            // no more threads: the ones started and this one share the rest
        }
        work((size_t)nt);
        for (auto& t : th) t.join();
        for (auto& f : frees) s->deferred.insert(s->deferred.end(), f.begin(), f.end());
    }
    std::vector<Req*> admitted;
    for (size_t i = 0; i < batch.size(); ++i) {
        Req* r = batch[i];
        int rc = built[i];
        if (rc == PWMGPU_OK) rc = reset_state(s, r->slot);
        if (rc != PWMGPU_OK) {
            r->error = rc;
            if (r->m) pwmgpu_destroy(r->m);
            r->m = nullptr;
            s->free_states.push_back(r->slot);
            r->slot = -1;
            r->state = PWMSVC_FAILED;
            r->t_done = s->now();
            ++s->failed;
            ++fin;
            continue;
        }
        r->state = PWMSVC_RUNNING;
        s->in_use += r->bytes;
        admitted.push_back(r);
    }
    if (ran) {
        const cudaError_t se = cudaStreamSynchronize(s->stream);
        free_deferred(s->deferred);
        CU(se);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess) s->gpu_ms += ms;
        ++s->rounds;
        const int status = *s->h_status;
        if (status != PWMGPU_OK) {
            for (Req* r : admitted) s->live.push_back(r);
            if (!admitted.empty()) s->dirty = true;
            return fail(status, "a bounded device wait timed out in a service round");
        }
        // the round's solves only: the new ones have no state yet
        TRY(after_round(s, &fin));
    }
    for (Req* r : admitted) s->live.push_back(r);
    if (!admitted.empty()) s->dirty = true;
    free_deferred(s->deferred);
    if (live) *live = (int32_t)s->live.size();
    if (queued) *queued = (int32_t)s->queue.size();
    if (finished) *finished = fin;
    return PWMGPU_OK;
}

int pwmsvc_result(pwmsvc* s, int64_t id, pwmsvc_result_info* out, double* u) {
    if (!s || !out) return fail(PWMGPU_ERR_INVALID, "null service or output");
    auto it = s->all.find(id);
    if (it == s->all.end()) return fail(PWMGPU_ERR_INVALID, "unknown request %lld", (long long)id);
    const Req* r = it->second.get();
    std::memset(out, 0, sizeof *out);
    out->state = r->state;
    out->n = r->n;
    out->iterations = r->iterations;
    out->iterations_low = r->iterations_low;
    out->converged = r->converged;
    out->precision = r->spec.precision;
    out->error = r->error;
    out->lambda = r->lambda;
    out->residual = r->rel;
    out->t_submit = r->t_submit;
    out->t_admit = r->t_admit;
    out->t_done = r->t_done;
    if (u) {
        if (r->state != PWMSVC_DONE || r->u.empty())
            return fail(PWMGPU_ERR_STATE, "request %lld has no eigenvector (not finished or keep_vector = 0)",
                        (long long)id);
        std::memcpy(u, r->u.data(), sizeof(double) * r->u.size());
    }
    return PWMGPU_OK;
}

int pwmsvc_release(pwmsvc* s, int64_t id) {
    if (!s) return fail(PWMGPU_ERR_INVALID, "null service");
    auto it = s->all.find(id);
    if (it == s->all.end()) return fail(PWMGPU_ERR_INVALID, "unknown request %lld", (long long)id);
    if (it->second->state != PWMSVC_DONE && it->second->state != PWMSVC_FAILED)
        return fail(PWMGPU_ERR_STATE, "request %lld is still queued or running", (long long)id);
    s->all.erase(it);
    return PWMGPU_OK;
}

int pwmsvc_stats(pwmsvc* s, pwmsvc_stats_info* out) {
    if (!s || !out) return fail(PWMGPU_ERR_INVALID, "null service or output");
    std::memset(out, 0, sizeof *out);
    out->submitted = s->submitted;
    out->finished = s->finished;
    out->failed = s->failed;
    out->rounds = s->rounds;
    out->live = (int32_t)s->live.size();
    out->queued = (int32_t)s->queue.size();
    out->hbm_in_use = s->in_use;
    out->hbm_budget = s->cfg.hbm_budget_bytes;
    out->gpu_round_ms = s->gpu_ms;
    return PWMGPU_OK;
}

}  // extern "C"
