// matrix_impl.h -- the pwmgpu_matrix handle and the host helpers shared by
// the C ABI (pwmgpu.cpp) and the batched service (service.cpp).  Not part of
// the public ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "internal.h"
#include "pwmgpu.h"

namespace pwmgpu {

// Record a failure for pwmgpu_last_error() and return `code`.
int fail(int code, const char* fmt, ...);

#define CU(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(e_ == cudaErrorMemoryAllocation ? PWMGPU_ERR_NOMEM : PWMGPU_ERR_CUDA,     \
                        "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

#define TRY(expr)                 \
    do {                          \
        int r_ = (expr);          \
        if (r_ != PWMGPU_OK) return r_; \
    } while (0)

constexpr int kPad = 16;  // kArrayPad in merge.cuh

template <typename T>
inline int dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(PWMGPU_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
    }
    return PWMGPU_OK;
}

template <typename T>
inline void dfree(T*& p) {
    if (p) dev_free((void*)p);
    p = nullptr;
}

}  // namespace pwmgpu

struct pwmgpu_matrix {
    using DevMatrix = pwmgpu::DevMatrix;
    using MliPlan = pwmgpu::MliPlan;
    int format = PWMGPU_FMT_MERGE;
    int partitions = 1;
    int device = 0;
    int sm_count = 1;
    int pageable_access = -1;  // the device reads / writes pageable host memory (-1: not asked yet)
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool loaded = false;
    // No load-time launch tuning (the serving loop's matrices: its batched
    // kernels do not use the handle's launch variant).
    bool skip_tune = false;

    DevMatrix M;

    // merge-path plan: sub-tiles of tm merge items (num_tiles of them), the
    // lane-interleaved arrays, and launch geometry
    int cfg = pwmgpu::kCfgF64;
    int tm = 0, num_tiles = 0, grid = 1, fix_grid = 1;
    // persistent power kernel grids per configuration (0: not launchable)
    int pgrid = 0, pgrid32 = 0, pgridbf = 0;
    // launch variant picked by the load-time tuner (0: most resident CTAs,
    // 1: more L1), and the timings it compared (ms per SpMV)
    int l1 = 0;
    float tune_ms[2] = {0.f, 0.f};
    int power_mode = PWMGPU_POWER_AUTO;
    // grid barrier budget of the persistent power kernel (pwmgpu_test_grid_wait)
    pwmgpu::GridWait grid_wait{pwmgpu::kWaitCycles, 0u};
    // format autotuner (PWMGPU_FMT_AUTO handles, tuned on every load): the
    // format whose FP64 SpMV runs (-1: the handle's own), the CSB kernel
    // variant, and what the tuner saw
    bool auto_fmt = false;
    int tuned_fmt = -1;
    int csb_var = 0;
    pwmgpu_tuning tuning{};
    MliPlan P;
    // lane-interleaved FP32 / BF16 copies of the values (lazy)
    float* val32 = nullptr;
    void* valbf = nullptr;
    int bf16_exact = -1;
    // SELL-32 copy for the FP32 / BF16 iterations (lazy), and whether they
    // may use it (PWMGPU_LOWFMT_*)
    pwmgpu::SellPlan sell;
    int low_format = PWMGPU_LOWFMT_AUTO;

    // scratch
    double* carries = nullptr;  // max(num_tiles, num_tiles32) doubles (also used as floats)
    size_t carries_cap = 0;
    double* partials = nullptr;  // spmv partials
    size_t partials_cap = 0;
    double* npart = nullptr;  // per-CTA shares of a power step's ||y||^2 (SpMV CTAs, then fix-up CTAs)
    size_t npart_cap = 0;
    unsigned int* counter = nullptr;
    double* nsq = nullptr;
    size_t nsq_cap = 0;
    unsigned int* mxk = nullptr;  // mxk[k]: largest magnitude key of iterate k (power steps in MODE_SCALE)
    size_t mxk_cap = 0;
    double* small = nullptr;  // 16 doubles of reduction outputs
    int* status = nullptr;
    unsigned int* barrier = nullptr;  // grid barrier words of the persistent kernel
    double* hres = nullptr;           // pinned host copy of a solve chunk's results

    // CSB format (csb.cu): the reference's arrays plus the window / unit plan
    struct {
        int beta = 0, bits = 0, hb = 0, vb = 0, S = 0, nwin = 0;
        uint32_t* ind = nullptr;
        int32_t* kcol = nullptr;  // global columns of the flat (merged sparse) units
        double* data = nullptr;
        int32_t* blk_ptr = nullptr;
        int* win_ptr = nullptr;
        int* units = nullptr;
        std::vector<uint32_t> h_ind;
        std::vector<double> h_data;
        std::vector<int32_t> h_blk_ptr;
    } csb;
    // CO-H format (coh.cu): the reference's arrays (host) and the tiles the
    // tile kernel runs (device; same layout as the CSB handle's)
    struct {
        int parts = 0;
        long long nblocks = 0;
        int S = 0, nwin = 0;
        uint32_t* ind = nullptr;
        int32_t* kcol = nullptr;
        double* data = nullptr;
        int* win_ptr = nullptr;
        int* units = nullptr;
        std::vector<int32_t> part_info, block_nnz;
        std::vector<uint16_t> h_row_jump, h_col_jump;
        std::vector<double> h_data;
        std::vector<int16_t> row_jump_block, col_jump_block;
    } coh;

    // pipelined host-array SpMV (pwmgpu_mv): chunk records, streams, events
    struct {
        int K = 0;          // chunks (0: not planned yet, -1: not pipelined)
        std::vector<int> rec;  // 4 per chunk: first sub-tile, first row, split flag, prefix max column
        std::vector<int> fpre; // K + 1: fix-up descriptors of the runs starting before each chunk
        cudaStream_t in = nullptr, out = nullptr;
        std::vector<cudaEvent_t> ev_x, ev_y;
        cudaEvent_t ev_start = nullptr;
    } pipe;

    // host-facing vector buffers
    double* dx = nullptr;
    double* dy = nullptr;
    size_t vec_cap = 0;
    float* fx = nullptr;
    float* fy = nullptr;
    size_t fvec_cap = 0;

    void release_csb() {
        pwmgpu::dfree(csb.ind);
        pwmgpu::dfree(csb.kcol);
        pwmgpu::dfree(csb.data);
        pwmgpu::dfree(csb.blk_ptr);
        pwmgpu::dfree(csb.win_ptr);
        pwmgpu::dfree(csb.units);
        csb = decltype(csb)();
    }
    void release_coh() {
        pwmgpu::dfree(coh.ind);
        pwmgpu::dfree(coh.kcol);
        pwmgpu::dfree(coh.data);
        pwmgpu::dfree(coh.win_ptr);
        pwmgpu::dfree(coh.units);
        coh = decltype(coh)();
    }
    void release_matrix() {
        pwmgpu::dfree(M.row_start);
        pwmgpu::dfree(M.col);
        pwmgpu::dfree(M.val);
        pwmgpu::dfree(P.subc);
        pwmgpu::dfree(P.rec);
        pwmgpu::dfree(P.masks);
        pwmgpu::dfree(P.colp);
        pwmgpu::dfree(P.colp16);
        pwmgpu::dfree(P.runs);
        pwmgpu::dfree(P.run_pre);
        pwmgpu::dfree(P.valp);
        P = MliPlan();
        pwmgpu::dfree(val32);
        release_csb();
        release_coh();
        tuned_fmt = -1;
        tuning = pwmgpu_tuning{};
        pipe.K = 0;
        pipe.rec.clear();
        if (valbf) pwmgpu::dev_free(valbf);
        valbf = nullptr;
        bf16_exact = -1;
        sell.release();
        M = DevMatrix();
        num_tiles = 0;
        loaded = false;
    }
    void release_all() {
        release_matrix();
        for (cudaEvent_t e : pipe.ev_x) cudaEventDestroy(e);
        for (cudaEvent_t e : pipe.ev_y) cudaEventDestroy(e);
        if (pipe.ev_start) cudaEventDestroy(pipe.ev_start);
        if (pipe.in) cudaStreamDestroy(pipe.in);
        if (pipe.out) cudaStreamDestroy(pipe.out);
        pipe.ev_x.clear();
        pipe.ev_y.clear();
        pipe.ev_start = nullptr;
        pipe.in = pipe.out = nullptr;
        pwmgpu::dfree(carries);
        pwmgpu::dfree(partials);
        pwmgpu::dfree(npart);
        pwmgpu::dfree(counter);
        pwmgpu::dfree(nsq);
        pwmgpu::dfree(mxk);
        pwmgpu::dfree(small);
        pwmgpu::dfree(status);
        pwmgpu::dfree(barrier);
        if (hres) cudaFreeHost(hres);
        hres = nullptr;
        pwmgpu::dfree(dx);
        pwmgpu::dfree(dy);
        pwmgpu::dfree(fx);
        pwmgpu::dfree(fy);
        carries_cap = partials_cap = npart_cap = nsq_cap = mxk_cap = vec_cap = fvec_cap = 0;
    }
};


namespace pwmgpu {

// Host helpers of a handle (pwmgpu.cpp).
int check_status(pwmgpu_matrix* m);
int check_sizes(long long nor, long long noc, long long nnz);
int build_plan(pwmgpu_matrix* m);
int ensure_vectors(pwmgpu_matrix* m);
int ensure_fvectors(pwmgpu_matrix* m);
int ensure_low_values(pwmgpu_matrix* m, bool allow_bf16, int* cfg, const void** valp, int* pgrid);
bool low_precision_floor(double rel, double prev_rel);
bool sell_for(pwmgpu_matrix* m, int cfg);

}  // namespace pwmgpu
