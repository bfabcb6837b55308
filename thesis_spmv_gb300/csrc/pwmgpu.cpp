// pwmgpu.cpp -- host side of the C ABI (include/pwmgpu.h).
//
// A pwmgpu_matrix owns the device copy of one sparse matrix plus the plan
// its kernels need (merge-path tile coordinates, scratch for carries and
// reductions) and a CUDA stream.  It mirrors pwm::SparseMatrix
// (Matrix/SparseMatrix.hpp:13-68): load / generate, mv, powerIteration.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <map>
#include <mutex>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "matrix_impl.h"
#include "pwmgpu.h"

using namespace pwmgpu;

namespace {
thread_local std::string g_err;
}  // namespace

namespace pwmgpu {
int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
}  // namespace pwmgpu

namespace {

int ensure_cap(double** p, size_t* cap, size_t need) {
    if (*cap >= need && *p) return PWMGPU_OK;
    dfree(*p);
    *cap = 0;
    TRY(dalloc(p, need));
    *cap = need;
    return PWMGPU_OK;
}

}  // namespace
namespace pwmgpu {
namespace {
thread_local std::vector<void*>* g_deferred_frees = nullptr;
}

void dev_free(void* p) {
    if (!p) return;
    if (g_deferred_frees) g_deferred_frees->push_back(p);
    else cudaFree(p);
}

void defer_frees(std::vector<void*>* list) { g_deferred_frees = list; }

void free_deferred(std::vector<void*>& list) {
    for (void* p : list) cudaFree(p);
    list.clear();
}

int check_status(pwmgpu_matrix* m) {
    int st = 0;
    CU(cudaMemcpyAsync(&st, m->status, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    CU(cudaStreamSynchronize(m->stream));
    if (st != PWMGPU_OK) {
        cudaMemsetAsync(m->status, 0, sizeof(int), m->stream);
        cudaStreamSynchronize(m->stream);
        return fail(st, "device kernel reported status %d (a bounded wait timed out)", st);
    }
    return PWMGPU_OK;
}
}  // namespace pwmgpu
namespace {

// Build the merge-path plan from the CRS arrays in M: sub-tile boundaries at
// diagonals s*WM (k_merge_partition), then the lane-interleaved columns and
// values, row-end masks and metadata (k_mli_plan).  The CRS column / value
// arrays are released afterwards; row_start stays (fix-up, general path).
}  // namespace
namespace pwmgpu {
// CSB / CO-H formats: build the format's arrays on the host from the CRS
// arrays (which stay on the device for pwmgpu_get_csr), upload them.
int build_format(pwmgpu_matrix* m) {
    const int nor = m->M.nor, noc = m->M.noc;
    const long long nnz = m->M.nnz;
    std::vector<int32_t> rs((size_t)nor + 1), ci((size_t)std::max(nnz, 1LL));
    std::vector<double> va((size_t)std::max(nnz, 1LL));
    CU(cudaMemcpyAsync(rs.data(), m->M.row_start, sizeof(int32_t) * ((size_t)nor + 1), cudaMemcpyDeviceToHost,
                       m->stream));
    if (nnz > 0) {
        CU(cudaMemcpyAsync(ci.data(), m->M.col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToHost, m->stream));
        CU(cudaMemcpyAsync(va.data(), m->M.val, sizeof(double) * (size_t)nnz, cudaMemcpyDeviceToHost, m->stream));
    }
    CU(cudaStreamSynchronize(m->stream));
    if (m->format == PWMGPU_FMT_CSB) {
        auto& c = m->csb;
        csb_params(std::max(nor, 1), std::max(noc, 1), &c.beta, &c.bits);
        c.hb = (noc + c.beta - 1) / c.beta;
        c.vb = (nor + c.beta - 1) / c.beta;
        c.S = csb_window(nor, c.beta, m->sm_count);
        c.nwin = (nor + c.S - 1) / c.S;
        std::vector<int> win_ptr, units;
        csb_build_host(nor, noc, nnz, rs.data(), ci.data(), va.data(), c.beta, c.bits, c.h_ind, c.h_data,
                       c.h_blk_ptr, c.S, win_ptr, units);
        // the kernel's copy: dense sub-squares row-major (csb.cu); the
        // reference's arrays stay on the host for pwmgpu_get_csb
        std::vector<uint32_t> kind;
        std::vector<double> kdata;
        std::vector<int32_t> kcol;
        if (!csb_kernel_layout(c.h_ind, c.h_data, c.S, win_ptr, units, kind, kdata, kcol))
            return fail(PWMGPU_ERR_INVALID, "CSB: the padded device copy exceeds 32-bit element offsets");
        TRY(dalloc(&c.ind, kind.size()));
        TRY(dalloc(&c.kcol, kcol.size()));
        TRY(dalloc(&c.data, kdata.size()));
        CU(cudaMemcpyAsync(c.kcol, kcol.data(), sizeof(int32_t) * kcol.size(), cudaMemcpyHostToDevice, m->stream));
        TRY(dalloc(&c.blk_ptr, c.h_blk_ptr.size()));
        TRY(dalloc(&c.win_ptr, win_ptr.size()));
        TRY(dalloc(&c.units, units.size() + 4));
        CU(cudaMemcpyAsync(c.ind, kind.data(), sizeof(uint32_t) * kind.size(), cudaMemcpyHostToDevice, m->stream));
        CU(cudaMemcpyAsync(c.data, kdata.data(), sizeof(double) * kdata.size(), cudaMemcpyHostToDevice, m->stream));
        CU(cudaMemcpyAsync(c.blk_ptr, c.h_blk_ptr.data(), sizeof(int32_t) * c.h_blk_ptr.size(),
                           cudaMemcpyHostToDevice, m->stream));
        CU(cudaMemcpyAsync(c.win_ptr, win_ptr.data(), sizeof(int) * win_ptr.size(), cudaMemcpyHostToDevice,
                           m->stream));
        if (!units.empty())
            CU(cudaMemcpyAsync(c.units, units.data(), sizeof(int) * units.size(), cudaMemcpyHostToDevice, m->stream));
    } else {
        auto& c = m->coh;
        std::vector<int> parts, blocks;
        c.parts = coh_build_host(nor, noc, nnz, rs.data(), ci.data(), va.data(), m->partitions, c.part_info,
                                 c.h_row_jump, c.h_col_jump, c.h_data, c.block_nnz, c.row_jump_block,
                                 c.col_jump_block, parts, blocks);
        c.nblocks = (long long)c.block_nnz.size();
        // the kernel's copy: the blocks as tiles of the tile kernel (windows
        // of S rows, Hilbert block order per partition; csb.cu / coh.cu)
        c.S = csb_window(nor, 1024, m->sm_count);
        c.nwin = (nor + c.S - 1) / c.S;
        std::vector<uint32_t> tind, kind;
        std::vector<double> tdata, kdata;
        std::vector<int32_t> kcol;
        std::vector<int> win_ptr, units;
        coh_tile_units(nor, noc, nnz, rs.data(), ci.data(), va.data(), parts, c.S, tind, tdata, win_ptr, units);
        if (!csb_kernel_layout(tind, tdata, c.S, win_ptr, units, kind, kdata, kcol))
            return fail(PWMGPU_ERR_INVALID, "CO-H: the padded device copy exceeds 32-bit element offsets");
        TRY(dalloc(&c.ind, kind.size()));
        TRY(dalloc(&c.kcol, kcol.size()));
        TRY(dalloc(&c.data, kdata.size()));
        TRY(dalloc(&c.win_ptr, win_ptr.size()));
        TRY(dalloc(&c.units, units.size() + 4));
        CU(cudaMemcpyAsync(c.ind, kind.data(), sizeof(uint32_t) * kind.size(), cudaMemcpyHostToDevice, m->stream));
        CU(cudaMemcpyAsync(c.kcol, kcol.data(), sizeof(int32_t) * kcol.size(), cudaMemcpyHostToDevice, m->stream));
        CU(cudaMemcpyAsync(c.data, kdata.data(), sizeof(double) * kdata.size(), cudaMemcpyHostToDevice, m->stream));
        CU(cudaMemcpyAsync(c.win_ptr, win_ptr.data(), sizeof(int) * win_ptr.size(), cudaMemcpyHostToDevice,
                           m->stream));
        if (!units.empty())
            CU(cudaMemcpyAsync(c.units, units.data(), sizeof(int) * units.size(), cudaMemcpyHostToDevice, m->stream));
    }
    CU(cudaStreamSynchronize(m->stream));
    TRY(ensure_cap(&m->partials, &m->partials_cap, (size_t)2 * dot_grid(m->M.nor, m->sm_count) + 64));
    m->loaded = true;
    return PWMGPU_OK;
}

// Load-time tuner of the merge kernels' launch variant: with enough work to
// measure (at least 8 sub-tiles per resident warp), time a few SpMVs in each
// variant (x = 0: the timing does not depend on the values) and keep the
// faster.  The variants compute the same bits; only the shared-memory / L1
// split and the resident CTA count differ (a Poisson-like matrix gains from
// more CTAs, gathers spread over a large x from more L1).
void apply_merge_variant(pwmgpu_matrix* m, int v) {
    m->l1 = v;
    m->grid = merge_grid(m->cfg, m->num_tiles, m->sm_count, v);
    m->pgrid = power_persistent_grid(kCfgF64, m->num_tiles, m->sm_count, v);
    m->pgrid32 = power_persistent_grid(kCfgF32, m->num_tiles, m->sm_count, v);
    m->pgridbf = power_persistent_grid(kCfgBF16, m->num_tiles, m->sm_count, v);
}

int tune(pwmgpu_matrix* m) {
    const MergeGeom g = merge_geometry(kCfgF64, 0);
    if (m->num_tiles < 8 * g.occ * g.w * m->sm_count) return PWMGPU_OK;
    TRY(ensure_vectors(m));
    CU(cudaMemsetAsync(m->dx, 0, sizeof(double) * (size_t)std::max(m->M.nor, m->M.noc), m->stream));
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    int rc = PWMGPU_OK;
    const int c16 = m->P.colp16 ? 2 : 0;
    // variants: carveout (bit 0) x gathers through L1 or around it (bit 2)
    const int cand[4] = {0, 1, 4, 5};
    float ms[4] = {0.f, 0.f, 0.f, 0.f};
    for (int c = 0; c < 4 && rc == PWMGPU_OK; ++c) {
        const int v = cand[c] | c16;
        const int grid = merge_grid(kCfgF64, m->num_tiles, m->sm_count, v);
        cudaError_t e = cudaSuccess;
        for (int r = 0; r < 9 && e == cudaSuccess; ++r) {  // one warm-up, eight timed
            if (r == 1) e = cudaEventRecord(e0, m->stream);
            if (e == cudaSuccess)
                e = launch_merge_spmv(kCfgF64, kModeSpmv, m->M, m->P.valp, m->P, grid, m->dx, m->dy, m->carries,
                                      nullptr, m->status, m->stream, v);
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, m->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[c], e0, e1);
        if (e != cudaSuccess) rc = fail(PWMGPU_ERR_CUDA, "launch tuning: %s", cudaGetErrorString(e));
        ms[c] /= 8.f;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    TRY(rc);
    TRY(check_status(m));
    m->tune_ms[0] = ms[0];
    m->tune_ms[1] = ms[1];
    int best = 0;  // another variant only for a clear (3 %) gain
    for (int c = 1; c < 4; ++c)
        if (ms[c] < 0.97f * ms[best]) best = c;
    apply_merge_variant(m, cand[best] | c16);
    return PWMGPU_OK;
}

// 16-bit columns for the merge kernels when every sub-tile's columns span
// less than 2^16 (then the SpMV streams 10 bytes per FP64 nonzero instead of
// 12).  Skipped, not an error, when the span is wider or the extra array does
// not fit.
int build_col16(pwmgpu_matrix* m) {
    MliPlan& P = m->P;
    if (P.nsub == 0 || m->M.nnz == 0) return PWMGPU_OK;
    int* cbase = nullptr;
    int* flag = nullptr;
    TRY(dalloc(&cbase, (size_t)P.nsub));
    int rc = dalloc(&flag, 1);
    int wide = 1;
    cudaError_t e = cudaSuccess;
    if (rc == PWMGPU_OK) {
        e = cudaMemsetAsync(flag, 0, sizeof(int), m->stream);
        if (e == cudaSuccess) e = launch_mli_colspan(P, cbase, flag, m->sm_count, m->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&wide, flag, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    }
    if (rc == PWMGPU_OK && e == cudaSuccess && !wide) {
        const size_t elems = (size_t)mli_storage_elems(m->M.nnz, P.nsub);
        if (cudaMalloc((void**)&P.colp16, elems * sizeof(uint16_t)) != cudaSuccess) {
            (void)cudaGetLastError();
            P.colp16 = nullptr;
        } else {
            e = cudaMemsetAsync(P.colp16, 0, elems * sizeof(uint16_t), m->stream);
            if (e == cudaSuccess) e = launch_mli_col16(P, cbase, m->sm_count, m->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        }
    }
    dfree(cbase);
    dfree(flag);
    if (rc != PWMGPU_OK) return rc;
    if (e != cudaSuccess) return fail(PWMGPU_ERR_CUDA, "16-bit column plan: %s", cudaGetErrorString(e));
    return PWMGPU_OK;
}

// The merge-path plan (and, with run_tuner, the load-time launch tuner).
int build_merge(pwmgpu_matrix* m, bool run_tuner) {
    const long long total = (long long)m->M.nor + m->M.nnz;
    const MergeGeom g = merge_geometry(m->cfg);
    m->tm = g.wm;
    m->num_tiles = (int)((total + m->tm - 1) / m->tm);
    MliPlan& P = m->P;
    P.nsub = m->num_tiles;
    const long long elems = mli_storage_elems(m->M.nnz, P.nsub);
    TRY(dalloc(&P.subc, (size_t)P.nsub + 1));
    TRY(dalloc(&P.rec, 2 * (size_t)P.nsub + 2));
    TRY(dalloc(&P.masks, (size_t)P.nsub * 32 + 32));
    TRY(dalloc(&P.colp, (size_t)elems));
    TRY(dalloc(&P.valp, (size_t)elems));
    // gaps between sub-tiles are never read by the kernels; keep them defined
    CU(cudaMemsetAsync(P.colp, 0, sizeof(int32_t) * (size_t)elems, m->stream));
    CU(cudaMemsetAsync(P.valp, 0, sizeof(double) * (size_t)elems, m->stream));
    if (P.nsub > 0) {
        CU(launch_merge_partition(m->M.row_start, m->M.nor, m->M.nnz, m->tm, P.nsub, P.subc, m->stream));
        CU(launch_mli_plan(m->M.row_start, m->M.col, m->M.val, P, m->sm_count, m->stream));
    }
    CU(cudaStreamSynchronize(m->stream));
    TRY(build_col16(m));
    // fix-up descriptors; without them (no memory) the search-based fix-up runs
    (void)build_fix_runs(m->P, m->M.row_start, m->M.nor, m->sm_count, m->stream);
    dfree(m->M.col);
    dfree(m->M.val);
    m->l1 = m->P.colp16 ? 2 : 0;
    m->grid = merge_grid(m->cfg, m->num_tiles, m->sm_count, m->l1);
    m->fix_grid = fixup_grid(m->num_tiles, m->sm_count);
    m->pgrid = power_persistent_grid(kCfgF64, m->num_tiles, m->sm_count, m->l1);
    m->pgrid32 = power_persistent_grid(kCfgF32, m->num_tiles, m->sm_count, m->l1);
    m->pgridbf = power_persistent_grid(kCfgBF16, m->num_tiles, m->sm_count, m->l1);
    const int pmax = std::max(m->pgrid, std::max(m->pgrid32, m->pgridbf));
    TRY(ensure_cap(&m->carries, &m->carries_cap, (size_t)m->num_tiles + 1));
    TRY(ensure_cap(&m->partials, &m->partials_cap,
                   (size_t)std::max(std::max(m->grid, 2 * pmax), 2 * dot_grid(m->M.nor, m->sm_count)) + 64));
    // shares of a power step's ||y||^2: at most one per SpMV CTA (16 resident
    // CTAs per SM at most, 4 warps per CTA) and one per fix-up CTA
    TRY(ensure_cap(&m->npart, &m->npart_cap,
                   (size_t)power_norm_parts(m->P, (int)std::min<long long>(((long long)m->num_tiles + 3) / 4,
                                                                           16LL * m->sm_count)) + 64));
    CU(cudaStreamSynchronize(m->stream));
    m->loaded = true;
    return run_tuner ? tune(m) : PWMGPU_OK;
}

int build_auto(pwmgpu_matrix* m);

int tune_csb(pwmgpu_matrix* m);

int build_plan(pwmgpu_matrix* m) {
    if (m->auto_fmt) return build_auto(m);
    if (m->format == PWMGPU_FMT_CSB || m->format == PWMGPU_FMT_COH) {
        TRY(build_format(m));
        return tune_csb(m);
    }
    return build_merge(m, !m->skip_tune);
}
}  // namespace pwmgpu
namespace {

}  // namespace
namespace pwmgpu {
int ensure_vectors(pwmgpu_matrix* m) {
    size_t need = (size_t)std::max(m->M.nor, m->M.noc) + kPad;
    if (m->vec_cap >= need) return PWMGPU_OK;
    dfree(m->dx);
    dfree(m->dy);
    m->vec_cap = 0;
    TRY(dalloc(&m->dx, need));
    TRY(dalloc(&m->dy, need));
    m->vec_cap = need;
    return PWMGPU_OK;
}
}  // namespace pwmgpu
namespace {

int ensure_nsq(pwmgpu_matrix* m, size_t need) { return ensure_cap(&m->nsq, &m->nsq_cap, need + 1); }

// Magnitude keys of `need` iterates, zeroed (the steps atomicMax into them).
int ensure_mxk(pwmgpu_matrix* m, size_t need) {
    if (m->mxk_cap < need || !m->mxk) {
        dfree(m->mxk);
        m->mxk_cap = 0;
        TRY(dalloc(&m->mxk, need));
        m->mxk_cap = need;
    }
    CU(cudaMemsetAsync(m->mxk, 0, sizeof(unsigned int) * need, m->stream));
    return PWMGPU_OK;
}

int alloc_matrix(pwmgpu_matrix* m, int32_t nor, int32_t noc, long long nnz) {
    m->release_matrix();
    m->M.nor = nor;
    m->M.noc = noc;
    m->M.nnz = nnz;
    TRY(dalloc(&m->M.row_start, (size_t)nor + 1 + kPad));
    TRY(dalloc(&m->M.col, (size_t)nnz + kPad));
    TRY(dalloc(&m->M.val, (size_t)nnz + kPad));
    // the TMA windows may read the padding: keep it defined
    CU(cudaMemsetAsync(m->M.row_start + nor + 1, 0, kPad * sizeof(int32_t), m->stream));
    CU(cudaMemsetAsync(m->M.col + nnz, 0, kPad * sizeof(int32_t), m->stream));
    CU(cudaMemsetAsync(m->M.val + nnz, 0, kPad * sizeof(double), m->stream));
    return PWMGPU_OK;
}

}  // namespace
namespace pwmgpu {
int check_sizes(long long nor, long long noc, long long nnz) {
    if (nor < 0 || noc < 0 || nnz < 0) return fail(PWMGPU_ERR_INVALID, "negative size");
    if (nor + nnz >= (1LL << 31) - 4096)
        return fail(PWMGPU_ERR_INVALID, "nor + nnz = %lld exceeds the 32-bit merge-path range", nor + nnz);
    if (noc >= (1LL << 31)) return fail(PWMGPU_ERR_INVALID, "noc too large");
    return PWMGPU_OK;
}

// Host CRS arrays a host-side builder may index: row_start runs from 0 to
// nnz without decreasing, every column lies in [0, noc).
static int check_host_crs(int nor, int noc, long long nnz, const int32_t* row_start, const int32_t* col_ind) {
    if (row_start[0] != 0 || row_start[nor] != nnz)
        return fail(PWMGPU_ERR_INVALID, "row_start must run from 0 to nnz (got %d..%d, nnz %lld)", row_start[0],
                    row_start[nor], nnz);
    for (int i = 0; i < nor; ++i)
        if (row_start[i + 1] < row_start[i]) return fail(PWMGPU_ERR_INVALID, "row_start decreases at row %d", i);
    for (long long k = 0; k < nnz; ++k)
        if (col_ind[k] < 0 || col_ind[k] >= noc)
            return fail(PWMGPU_ERR_INVALID, "column index %d at nonzero %lld out of range [0,%d)", col_ind[k], k,
                        noc);
    return PWMGPU_OK;
}
}  // namespace pwmgpu
namespace {

// y = 2^e(nsq_in) A x with the CSB or CO-H kernel (nsq_in null: e = 0).
int spmv_format(pwmgpu_matrix* m, int fmt, const double* dx, double* dy, const double* nsq_in) {
    if (m->M.nor == 0) return PWMGPU_OK;
    if (fmt == PWMGPU_FMT_CSB) {
        const auto& c = m->csb;
        CU(launch_csb_spmv(c.ind, c.kcol, c.data, c.win_ptr, c.units, c.nwin, c.S, m->M.nor, m->M.noc, dx, dy, nsq_in,
                           m->status, m->sm_count, m->stream, m->csb_var));
    } else {
        const auto& c = m->coh;
        CU(launch_csb_spmv(c.ind, c.kcol, c.data, c.win_ptr, c.units, c.nwin, c.S, m->M.nor, m->M.noc, dx, dy, nsq_in,
                           m->status, m->sm_count, m->stream, m->csb_var));
    }
    return PWMGPU_OK;
}

// The format whose FP64 SpMV a handle runs: its own, or the autotuner's
// choice on a PWMGPU_FMT_AUTO handle.
int fp64_format(const pwmgpu_matrix* m) {
    if (m->format != PWMGPU_FMT_MERGE) return m->format;
    return m->tuned_fmt > 0 ? m->tuned_fmt : PWMGPU_FMT_MERGE;
}

int spmv_f64(pwmgpu_matrix* m, const double* dx, double* dy) {
    if (fp64_format(m) != PWMGPU_FMT_MERGE) return spmv_format(m, fp64_format(m), dx, dy, nullptr);
    if (m->num_tiles == 0) return PWMGPU_OK;
    CU(launch_merge_spmv(kCfgF64, kModeSpmv, m->M, m->P.valp, m->P, m->grid, dx, dy, m->carries, nullptr, m->status,
                         m->stream, m->l1));
    if (m->P.runs)
        CU(launch_fix_runs_f64(kModeSpmv, m->P, 0, m->P.nruns, dy, m->carries, nullptr, m->stream));
    else
        CU(launch_merge_fixup_f64(kModeSpmv, m->M, m->P.subc, m->num_tiles, dy, m->carries, nullptr, m->fix_grid,
                                  m->stream));
    return PWMGPU_OK;
}

// ||y||^2 of a power step taken inside its SpMV and fix-up kernels (needs the
// fix-up run descriptors and room for the shares of a `grid`-CTA SpMV).
bool norm_in_step(const pwmgpu_matrix* m, int grid) {
    return m->P.runs && m->npart && (size_t)power_norm_parts(m->P, grid) <= m->npart_cap;
}

// One power-method step on device vectors: out = 2^e(nsq_in) * A in (SpMV +
// fix-up), and nsq_out = ||out||^2 (deterministic): summed by the two kernels
// from the rows they store, or a row pass where the plan has no run
// descriptors.
int power_step_f64(pwmgpu_matrix* m, const double* in, double* out, const double* nsq_in, double* nsq_out,
                   const unsigned int* mx_in = nullptr) {
    if (norm_in_step(m, m->grid)) {
        CU(launch_merge_spmv(kCfgF64, kModePower, m->M, m->P.valp, m->P, m->grid, in, out, m->carries, nsq_in,
                             m->status, m->stream, m->l1, m->npart, mx_in));
        CU(launch_fix_runs_norm(false, m->P, out, m->carries, nsq_in, m->npart, m->grid, m->counter + 1, nsq_out,
                                m->stream, mx_in));
        return PWMGPU_OK;
    }
    CU(launch_merge_spmv(kCfgF64, kModePower, m->M, m->P.valp, m->P, m->grid, in, out, m->carries, nsq_in,
                         m->status, m->stream, m->l1));
    if (m->P.runs)
        CU(launch_fix_runs_f64(kModePower, m->P, 0, m->P.nruns, out, m->carries, nsq_in, m->stream));
    else
        CU(launch_merge_fixup_f64(kModePower, m->M, m->P.subc, m->num_tiles, out, m->carries, nsq_in,
                                  m->fix_grid, m->stream));
    CU(launch_power_norm_f64(out, nullptr, m->M.nor, m->partials, m->counter, nsq_out,
                             dot_grid(m->M.nor, m->sm_count), m->stream));
    return PWMGPU_OK;
}

// A power step whose norm only decides the exact power-of-two rescale: out =
// 2^e A in (e from the input's largest magnitude key *mx_in, or its squared
// norm *nsq_in, or 0), and atomicMax(*mx_out) of out's magnitude keys (an
// integer max on the stored rows -- no FP64 square per row, no norm shares).
// Scaling by powers of two is exact, so an iterate differs from the one an
// exact-norm step would give by a power of two only, which the final
// normalisation (by the exact norms of the last two iterates) removes.
// Needs the plan's run descriptors (norm_in_step).
int scale_step_f64(pwmgpu_matrix* m, const double* in, double* out, const double* nsq_in, const unsigned int* mx_in,
                   unsigned int* mx_out) {
    CU(launch_merge_spmv(kCfgF64, kModeScale, m->M, m->P.valp, m->P, m->grid, in, out, m->carries, nsq_in,
                         m->status, m->stream, m->l1, nullptr, mx_in, mx_out));
    CU(launch_fix_runs_scale(false, m->P, out, m->carries, nsq_in, mx_in, mx_out, m->stream));
    return PWMGPU_OK;
}

// POWER_AUTO runs the two-kernel step at every size: its kernel boundaries
// (programmatic dependent launch) cost less than the persistent kernel's
// grid barriers, and its SpMV keeps the most resident CTAs.  Per iteration,
// Poisson grids: 256^2 6.5 vs 11.0 us, 512^2 10.7 vs 19.7 us, 1024^2 21.7 vs
// 30.4 us, 2048^2 63.2 vs 72.3 us, 4096^2 0.223 vs 0.240 ms; the irregular 4M
// matrix 0.393 vs 0.425 ms.  POWER_FUSED selects the persistent kernel.
bool use_fused(const pwmgpu_matrix* m, int pgrid) {
    return m->power_mode == PWMGPU_POWER_FUSED && pgrid > 0;
}

int power_device(pwmgpu_matrix* m, double* dx, double* dy, int32_t it) {
    if (it <= 0 || m->M.nor == 0) return PWMGPU_OK;
    TRY(ensure_nsq(m, (size_t)it + 1));
    if (fp64_format(m) != PWMGPU_FMT_MERGE) {
        // the format's SpMV (with the rescale) and the row-pass norm per step
        for (int k = 0; k < it; ++k) {
            const double* in = (k % 2 == 0) ? dx : dy;
            double* out = (k % 2 == 0) ? dy : dx;
            TRY(spmv_format(m, fp64_format(m), in, out, k ? m->nsq + k : nullptr));
            CU(launch_power_norm_f64(out, nullptr, m->M.nor, m->partials, m->counter, m->nsq + k + 1,
                                     dot_grid(m->M.nor, m->sm_count), m->stream));
        }
        double* last = (it % 2 == 1) ? dy : dx;
        double* prev = (it % 2 == 1) ? dx : dy;
        CU(launch_power_finalize_f64(last, m->nsq + it, it >= 2 ? prev : nullptr, m->nsq + it - 1, m->M.nor,
                                     m->sm_count, m->stream));
        return PWMGPU_OK;
    }
    if (m->power_mode == PWMGPU_POWER_FUSED && m->pgrid == 0)
        return fail(PWMGPU_ERR_UNSUPPORTED, "the fused power kernel cannot be made co-resident on this device");
    if (use_fused(m, m->pgrid)) {
        // K5: all `it` iterations in one persistent launch (the iterations
        // before the last two track only the rescale's magnitude keys)
        TRY(ensure_mxk(m, (size_t)it + 1));
        CU(launch_power_persistent(kCfgF64, m->M, m->P.valp, m->P, m->pgrid, dx, dy, m->carries, 0, it, m->nsq,
                                   nullptr, m->partials, m->barrier, m->status, m->stream, m->l1, m->grid_wait,
                                   m->mxk));
    } else {
        // The last two steps compute the exact norms the final normalisation
        // uses; the steps before them only need the rescale exponent, from
        // their input's largest magnitude key (MODE_SCALE).
        const bool scale = norm_in_step(m, m->grid);
        if (scale) TRY(ensure_mxk(m, (size_t)it + 1));
        for (int k = 0; k < it; ++k) {
            const double* in = (k % 2 == 0) ? dx : dy;
            double* out = (k % 2 == 0) ? dy : dx;
            const bool prev_scale = scale && k >= 1 && k - 1 < it - 2;  // step k-1 tracked keys only
            const double* nsq_in = (k > 0 && !prev_scale) ? m->nsq + k : nullptr;
            const unsigned int* mx_in = prev_scale ? m->mxk + k : nullptr;
            if (scale && k < it - 2)
                TRY(scale_step_f64(m, in, out, nsq_in, mx_in, m->mxk + k + 1));
            else
                TRY(power_step_f64(m, in, out, nsq_in, m->nsq + k + 1, mx_in));
        }
    }
    double* last = (it % 2 == 1) ? dy : dx;
    double* prev = (it % 2 == 1) ? dx : dy;
    CU(launch_power_finalize_f64(last, m->nsq + it, it >= 2 ? prev : nullptr, m->nsq + it - 1, m->M.nor,
                                 m->sm_count, m->stream));
    return PWMGPU_OK;
}

// Lane-interleaved FP32 or (when every value is exactly a BF16 number, as the
// Poisson 4 / -1 stencil is) BF16 copy of the values, made on first use.
}  // namespace
namespace pwmgpu {
int ensure_low_values(pwmgpu_matrix* m, bool allow_bf16, int* cfg, const void** valp, int* pgrid) {
    const long long elems = mli_storage_elems(m->M.nnz, m->P.nsub);
    if (allow_bf16) {
        if (m->bf16_exact < 0) {
            int* flag = reinterpret_cast<int*>(m->barrier + 2);
            int h = 0;
            CU(cudaMemsetAsync(flag, 0, sizeof(int), m->stream));
            CU(launch_bf16_exact(m->P.valp, elems, flag, m->sm_count, m->stream));
            CU(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
            CU(cudaStreamSynchronize(m->stream));
            m->bf16_exact = h == 0 ? 1 : 0;
        }
        if (m->bf16_exact == 1) {
            if (!m->valbf) {
                CU(cudaMalloc(&m->valbf, 2 * (size_t)elems + 16));
                CU(cudaMemsetAsync(m->valbf, 0, 2 * (size_t)elems + 16, m->stream));
                CU(launch_mli_convert(m->P, kCfgBF16, m->valbf, m->sm_count, m->stream));
            }
            *cfg = kCfgBF16;
            *valp = m->valbf;
            *pgrid = m->pgridbf;
            return PWMGPU_OK;
        }
    }
    if (!m->val32) {
        TRY(dalloc(&m->val32, (size_t)elems + 4));
        CU(cudaMemsetAsync(m->val32, 0, sizeof(float) * ((size_t)elems + 4), m->stream));
        CU(launch_mli_convert(m->P, kCfgF32, m->val32, m->sm_count, m->stream));
    }
    *cfg = kCfgF32;
    *valp = m->val32;
    *pgrid = m->pgrid32;
    return PWMGPU_OK;
}

// The SELL-32 copy with values of configuration cfg (FP32 or BF16), built on
// first use from the CRS order of the merge plan; false where the matrix does
// not fit the format, the handle asks for the merge layout, or the iterations
// run in the persistent merge kernel.
bool sell_for(pwmgpu_matrix* m, int cfg) {
    if (cfg == kCfgF64 || m->low_format != PWMGPU_LOWFMT_AUTO || m->power_mode == PWMGPU_POWER_FUSED) return false;
    SellPlan& S = m->sell;
    const bool bf = cfg == kCfgBF16;
    if (S.state < 0) return false;
    if (S.state == 1 && (bf ? S.valbf != nullptr : S.val32 != nullptr)) return true;
    const long long nnz = m->M.nnz;
    int32_t* tcol = nullptr;
    double* tval = nullptr;
    const int32_t* col = m->M.col;
    const double* val = m->M.val;
    int rc = 2;
    if (!col || !val) {
        // the merge format keeps only its lane-interleaved copy: CRS order back
        if (dalloc(&tcol, (size_t)nnz + 1) == PWMGPU_OK && dalloc(&tval, (size_t)nnz + 1) == PWMGPU_OK &&
            launch_mli_unpermute(m->P, tcol, tval, m->sm_count, m->stream) == cudaSuccess) {
            col = tcol;
            val = tval;
        }
    }
    if (col && val) rc = sell_build(S, m->M.row_start, col, val, m->M.nor, nnz, bf, m->sm_count, m->stream);
    (void)cudaStreamSynchronize(m->stream);
    dfree(tcol);
    dfree(tval);
    (void)cudaGetLastError();
    return rc == 0;
}
}  // namespace pwmgpu
namespace {

}  // namespace
namespace pwmgpu {
int ensure_fvectors(pwmgpu_matrix* m) {
    size_t need = (size_t)std::max(m->M.nor, m->M.noc) + kPad;
    if (m->fvec_cap >= need) return PWMGPU_OK;
    dfree(m->fx);
    dfree(m->fy);
    m->fvec_cap = 0;
    TRY(dalloc(&m->fx, need));
    TRY(dalloc(&m->fy, need));
    m->fvec_cap = need;
    return PWMGPU_OK;
}
}  // namespace pwmgpu
namespace {

// One chunk of the persistent power kernel (iterations k0 .. k0+nk-1 of the
// current phase, k0 + nk >= 2) with the Rayleigh quotient and eigen-residual
// of its last iterate v_k, k = k0 + nk - 1.
struct ChunkOut {
    double lambda, rel;
};
// Iterations k0 .. k0+nk-1 of a solve and the Rayleigh quotient / residual of
// the last: in the persistent kernel, or (where the two-kernel step is the
// faster, see use_fused) as SpMV, fix-up and norm kernels per iteration plus
// a result pass -- the same steps; only the order of the reductions' sums
// differs.
int solve_chunk(pwmgpu_matrix* m, int cfg, const void* valp, int pgrid, void* X, void* Y, int k0, int nk,
                ChunkOut* o) {
    if (sell_for(m, cfg)) {
        // SELL-32: one kernel per step (no fix-up; ||y||^2 summed in it), the
        // chunk's last step with the norm pass for the Rayleigh dot
        const bool bf = cfg == kCfgBF16;
        const int dg = dot_grid(m->M.nor, m->sm_count);
        for (int k = k0; k < k0 + nk; ++k) {
            const float* in = static_cast<const float*>((k & 1) ? Y : X);
            float* out = static_cast<float*>((k & 1) ? X : Y);
            const double* nsq_in = k > 0 ? m->nsq + k : nullptr;
            const bool last = k == k0 + nk - 1;
            CU(launch_sell_spmv(m->sell, bf, m->M.row_start, m->M.nor, in, out, nsq_in, last ? nullptr : m->nsq + k + 1,
                                m->counter + 2, m->sm_count, m->stream));
            if (last) {
                CU(launch_power_norm_f32(out, in, m->M.nor, m->partials, m->counter, m->small + 6, dg, m->stream));
                CU(launch_solve_result(true, in, out, m->M.nor, m->nsq + k, m->small + 6, m->nsq + k + 1, m->small,
                                       m->partials, m->counter, dg, m->stream));
            }
        }
    } else if (use_fused(m, pgrid)) {
        TRY(ensure_mxk(m, (size_t)(k0 + nk) + 1));
        CU(launch_power_persistent(cfg, m->M, valp, m->P, pgrid, X, Y, m->carries, k0, nk, m->nsq, m->small,
                                   m->partials, m->barrier, m->status, m->stream, m->l1, m->grid_wait, m->mxk));
    } else {
        const bool f32 = cfg != kCfgF64;
        const int grid = merge_grid(cfg, m->num_tiles, m->sm_count, m->l1);
        const int dg = dot_grid(m->M.nor, m->sm_count);
        // steps before the chunk's last two track only the rescale's
        // magnitude keys (scale_step_f64); the last two sum ||v||^2
        const bool keys = norm_in_step(m, grid) && nk > 2;
        if (keys) TRY(ensure_mxk(m, (size_t)(k0 + nk) + 1));
        for (int k = k0; k < k0 + nk; ++k) {
            void* in = (k & 1) ? Y : X;
            void* out = (k & 1) ? X : Y;
            const bool prev_keys = keys && k > k0 && k - 1 < k0 + nk - 2;
            const double* nsq_in = (k > 0 && !prev_keys) ? m->nsq + k : nullptr;
            const unsigned int* mx_in = prev_keys ? m->mxk + k : nullptr;
            const bool last = k == k0 + nk - 1;
            if (keys && k < k0 + nk - 2) {
                CU(launch_merge_spmv(cfg, kModeScale, m->M, valp, m->P, grid, in, out, m->carries, nsq_in, m->status,
                                     m->stream, m->l1, nullptr, mx_in, m->mxk + k + 1));
                CU(launch_fix_runs_scale(f32, m->P, out, m->carries, nsq_in, mx_in, m->mxk + k + 1, m->stream));
                continue;
            }
            if (!last && norm_in_step(m, grid)) {
                CU(launch_merge_spmv(cfg, kModePower, m->M, valp, m->P, grid, in, out, m->carries, nsq_in, m->status,
                                     m->stream, m->l1, m->npart, mx_in));
                CU(launch_fix_runs_norm(f32, m->P, out, m->carries, nsq_in, m->npart, grid, m->counter + 1,
                                        m->nsq + k + 1, m->stream, mx_in));
                continue;
            }
            CU(launch_merge_spmv(cfg, kModePower, m->M, valp, m->P, grid, in, out, m->carries, nsq_in, m->status,
                                 m->stream, m->l1));
            if (f32) {
                if (m->P.runs)
                    CU(launch_fix_runs_f32(kModePower, m->P, 0, m->P.nruns, (float*)out, (const float*)m->carries,
                                           nsq_in, m->stream));
                else
                    CU(launch_merge_fixup_f32(kModePower, m->M, m->P.subc, m->num_tiles, (float*)out,
                                              (const float*)m->carries, nsq_in, m->fix_grid, m->stream));
                CU(launch_power_norm_f32((const float*)out, last ? (const float*)in : nullptr, m->M.nor, m->partials,
                                         m->counter, last ? m->small + 6 : m->nsq + k + 1, dg, m->stream));
            } else {
                if (m->P.runs)
                    CU(launch_fix_runs_f64(kModePower, m->P, 0, m->P.nruns, (double*)out, m->carries, nsq_in,
                                           m->stream));
                else
                    CU(launch_merge_fixup_f64(kModePower, m->M, m->P.subc, m->num_tiles, (double*)out, m->carries,
                                              nsq_in, m->fix_grid, m->stream));
                CU(launch_power_norm_f64((const double*)out, last ? (const double*)in : nullptr, m->M.nor,
                                         m->partials, m->counter, last ? m->small + 6 : m->nsq + k + 1, dg,
                                         m->stream));
            }
            if (last)
                CU(launch_solve_result(f32, in, out, m->M.nor, m->nsq + k, m->small + 6, m->nsq + k + 1, m->small,
                                       m->partials, m->counter, dg, m->stream));
        }
    }
    CU(cudaMemcpyAsync(m->hres, m->small, 5 * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    TRY(check_status(m));
    const double lam = m->hres[0], r2 = m->hres[1], nsq = m->hres[2];
    if (!(nsq > 0.0) || !std::isfinite(nsq) || !std::isfinite(lam) || !std::isfinite(r2))
        return fail(PWMGPU_ERR_NUMERIC, "power solve met a zero or non-finite iterate (||v||^2 = %g)", nsq);
    o->lambda = lam;
    o->rel = lam != 0.0 ? std::sqrt(r2 / nsq) / std::fabs(lam) : INFINITY;
    return PWMGPU_OK;
}

// Length of the next chunk: the iterations the residual's observed rate
// needs to reach `target`, within [8, 512].  Before the first chunk the
// residual is taken as 1 (a generic start vector).
int next_chunk(double rel, double prev_rel, int nk, double target) {
    if (std::isfinite(prev_rel) && rel < prev_rel && rel > 0.0 && target > 0.0) {
        const double rate = std::log(rel / prev_rel) / nk;  // < 0
        const double need = std::log(target / rel) / rate;
        if (need <= 0.0) return 8;
        return (int)std::min(512.0, std::max(8.0, std::ceil(need * 1.05) + 1.0));
    }
    return std::min(2 * nk, 512);
}

// Residual at which the mixed solve leaves the FP32 / BF16 phase: above the
// FP32 rounding floor of the residual (about nnz_row * 2^-24).
constexpr double kSwitchRel = 2e-6;

}  // namespace
namespace pwmgpu {
// The FP32 / BF16 phase has hit its rounding floor: the residual is small
// (below 1e-4) and no longer falls (less than 10 % over the last check).  A
// slowly converging solve (residual still large) stays in the fast phase.
bool low_precision_floor(double rel, double prev_rel) { return rel < 1e-4 && rel >= 0.9 * prev_rel; }
}  // namespace pwmgpu
namespace {

int solve(pwmgpu_matrix* m, double* x, int32_t max_it, double tol, int precision, pwmgpu_solve_info* info) {
    const int N = m->M.nor;
    TRY(ensure_vectors(m));
    TRY(ensure_nsq(m, (size_t)max_it + 2));
    CU(cudaMemcpyAsync(m->dx, x, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, m->stream));
    int k = 0, low = 0;
    bool conv = false;
    ChunkOut o{0.0, INFINITY};
    double* result = nullptr;  // device vector holding the final (unnormalised) iterate

    // the mixed solve leaves at least 2 (at most 64) iterations for the FP64 phase
    const int budget = precision == PWMGPU_PREC_F32 ? max_it : max_it - std::max(2, std::min(64, max_it / 4));
    if (precision == PWMGPU_PREC_F32 || (precision == PWMGPU_PREC_MIXED && budget >= 2)) {
        int cfg = kCfgF32, pg = 0;
        const void* valp = nullptr;
        TRY(ensure_low_values(m, precision == PWMGPU_PREC_MIXED, &cfg, &valp, &pg));
        if (pg == 0 && m->power_mode == PWMGPU_POWER_FUSED)
            return fail(PWMGPU_ERR_UNSUPPORTED, "the fused power kernel cannot be made co-resident");
        TRY(ensure_fvectors(m));
        CU(launch_convert_f64_f32(m->dx, m->fx, N, m->sm_count, m->stream));
        int kl = 0, chunk = 16, nchunks = 0;
        double prev = 1.0;
        const double target = precision == PWMGPU_PREC_F32 ? tol : std::max(tol, kSwitchRel);
        while (true) {
            int nk = std::min(chunk, budget - k);
            if (kl + nk < 2) nk = 2 - kl;
            TRY(solve_chunk(m, cfg, valp, pg, m->fx, m->fy, kl, nk, &o));
            kl += nk;
            k += nk;
            low += nk;
            ++nchunks;
            if (o.rel <= target) {
                conv = precision == PWMGPU_PREC_F32;
                break;
            }
            if (k >= budget) break;
            // FP32 has reached its rounding floor: refine in FP64 from here
            if (precision == PWMGPU_PREC_MIXED && nchunks >= 2 && low_precision_floor(o.rel, prev)) break;
            chunk = next_chunk(o.rel, prev, nk, target);
            prev = o.rel;
        }
        if (precision == PWMGPU_PREC_F32) {
            // v_{kl-1} is the iterate whose Rayleigh quotient was measured
            float* last = ((kl - 1) & 1) ? m->fy : m->fx;
            CU(launch_convert_f32_f64(last, m->dx, N, m->sm_count, m->stream));
            result = m->dx;
        } else {
            // the newest iterate v_kl starts the FP64 phase
            float* newest = (kl & 1) ? m->fy : m->fx;
            CU(launch_convert_f32_f64(newest, m->dx, N, m->sm_count, m->stream));
        }
    }
    if (precision != PWMGPU_PREC_F32) {
        if (m->pgrid == 0 && m->power_mode == PWMGPU_POWER_FUSED)
            return fail(PWMGPU_ERR_UNSUPPORTED, "the fused power kernel cannot be made co-resident");
        int kl = 0, chunk = precision == PWMGPU_PREC_MIXED ? 8 : 16;
        double prev = precision == PWMGPU_PREC_MIXED ? o.rel : 1.0;
        while (true) {
            int nk = std::min(chunk, max_it - k);
            if (kl + nk < 2) nk = 2 - kl;
            TRY(solve_chunk(m, kCfgF64, m->P.valp, m->pgrid, m->dx, m->dy, kl, nk, &o));
            kl += nk;
            k += nk;
            if (o.rel <= tol) {
                conv = true;
                break;
            }
            if (k >= max_it) break;
            chunk = next_chunk(o.rel, prev, nk, tol);
            prev = o.rel;
        }
        result = ((kl - 1) & 1) ? m->dy : m->dx;
    }
    // u = v / ||v|| (||v||^2 = result[2] of the last chunk, still on the device)
    CU(launch_power_finalize_f64(result, m->small + 2, nullptr, nullptr, N, m->sm_count, m->stream));
    CU(cudaMemcpyAsync(x, result, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost, m->stream));
    TRY(check_status(m));
    info->iterations = k;
    info->iterations_low = low;
    info->converged = conv ? 1 : 0;
    info->precision = precision;
    info->lambda = o.lambda;
    info->residual = o.rel;
    return PWMGPU_OK;
}

// ---- pipelined host-array SpMV -------------------------------------------
// x goes up in kPipeX pieces on one stream, y comes down per chunk on
// another; chunk c's SpMV waits only for the x pieces holding the columns
// chunks 0..c read, and chunk c's rows go down once the fix-up of the runs
// starting in chunk c has run (after chunk c+1's SpMV: such a run ends in
// chunk c+1 at the latest, checked at plan time).  Upload, compute and
// download overlap; the result is the same as the one-shot path (the same
// sub-tiles and fix-ups, in the same arithmetic).
constexpr int kPipeChunks = 16;
constexpr int kPipeX = 16;

int plan_pipeline(pwmgpu_matrix* m) {
    auto& p = m->pipe;
    if (p.K != 0) return PWMGPU_OK;
    p.K = -1;
    const int K = kPipeChunks;
    if (m->num_tiles < 64 * K) return PWMGPU_OK;  // too small to gain from it
    int* d = nullptr;
    TRY(dalloc(&d, 4 * (size_t)K));
    p.rec.assign(4 * (size_t)K, 0);
    cudaError_t e = launch_pipeline_plan(m->M.row_start, m->P, K, d, m->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p.rec.data(), d, sizeof(int) * 4 * K, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    dfree(d);
    if (e != cudaSuccess) return fail(PWMGPU_ERR_CUDA, "pipeline plan: %s", cudaGetErrorString(e));
    // a run of sub-tiles may cross at most one chunk boundary: chunk first
    // rows must increase strictly
    for (int c = 1; c < K; ++c)
        if (p.rec[4 * c + 1] <= p.rec[4 * (c - 1) + 1]) return PWMGPU_OK;
    for (int c = 1; c < K; ++c) p.rec[4 * c + 3] = std::max(p.rec[4 * c + 3], p.rec[4 * (c - 1) + 3]);
    p.fpre.assign(K + 1, 0);
    if (m->P.runs) {
        for (int c = 0; c < K; ++c)
            CU(cudaMemcpy(&p.fpre[(size_t)c], m->P.run_pre + p.rec[4 * c], sizeof(int), cudaMemcpyDeviceToHost));
        p.fpre[(size_t)K] = m->P.nruns;
    }
    // streams and events outlive a reload of the matrix: create them once
    // highest priority: their copy kernels (pageable arrays) go ahead of SpMV CTAs
    int lo_prio = 0, hi_prio = 0;
    CU(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    if (!p.in) CU(cudaStreamCreateWithPriority(&p.in, cudaStreamNonBlocking, hi_prio));
    if (!p.out) CU(cudaStreamCreateWithPriority(&p.out, cudaStreamNonBlocking, hi_prio));
    if (!p.ev_start) CU(cudaEventCreateWithFlags(&p.ev_start, cudaEventDisableTiming));
    for (auto* v : {&p.ev_x, &p.ev_y}) {
        const size_t want = v == &p.ev_x ? (size_t)kPipeX : (size_t)K;
        while (v->size() < want) {
            cudaEvent_t ev = nullptr;
            CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            v->push_back(ev);
        }
    }
    p.K = K;
    return PWMGPU_OK;
}

// A caller array the copy engines would have to stage (pageable memory) but
// the SMs can reach directly: copied by launch_host_copy instead.
bool sm_reachable_pageable(pwmgpu_matrix* m, const void* h) {
    if (m->pageable_access < 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess)
            v = 0;
        m->pageable_access = v ? 1 : 0;
    }
    if (!m->pageable_access) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

int mv_pipelined(pwmgpu_matrix* m, const double* x, double* y) {
    auto& p = m->pipe;
    const int K = p.K, noc = m->M.noc, nor = m->M.nor, nsub = m->num_tiles;
    const bool x_sm = sm_reachable_pageable(m, x), y_sm = sm_reachable_pageable(m, y);
    // the streams start after earlier work on the handle's stream
    CU(cudaEventRecord(p.ev_start, m->stream));
    CU(cudaStreamWaitEvent(p.in, p.ev_start, 0));
    CU(cudaStreamWaitEvent(p.out, p.ev_start, 0));
    for (int q = 0; q < kPipeX; ++q) {
        const long long a = (long long)noc * q / kPipeX, b = (long long)noc * (q + 1) / kPipeX;
        if (b > a && x_sm)
            CU(launch_host_copy(x + a, m->dx + a, b - a, p.in));
        else if (b > a)
            CU(cudaMemcpyAsync(m->dx + a, x + a, sizeof(double) * (size_t)(b - a), cudaMemcpyHostToDevice, p.in));
        CU(cudaEventRecord(p.ev_x[(size_t)q], p.in));
    }
    auto piece_of = [&](int col) {  // the x piece holding column col
        int q = 0;
        while (q + 1 < kPipeX && (long long)noc * (q + 1) / kPipeX <= col) ++q;
        return q;
    };
    auto chunk_tiles = [&](int c, int* t0, int* t1) {
        *t0 = p.rec[4 * c];
        *t1 = c + 1 < K ? p.rec[4 * (c + 1)] : nsub;
    };
    // rows chunk c downloads: [lo_c, lo_{c+1})
    auto row_lo = [&](int c) { return c == 0 ? 0 : (c >= K ? nor : p.rec[4 * c + 1] + p.rec[4 * c + 2]); };
    int waited = -1;
    for (int c = 0; c <= K; ++c) {
        if (c < K) {
            const int need = piece_of(p.rec[4 * c + 3]);
            for (int q = waited + 1; q <= need; ++q) CU(cudaStreamWaitEvent(m->stream, p.ev_x[(size_t)q], 0));
            waited = std::max(waited, need);
            int t0, t1;
            chunk_tiles(c, &t0, &t1);
            const int grid = merge_grid(kCfgF64, t1 - t0, m->sm_count, m->l1);
            CU(launch_merge_spmv_range(m->M, m->P, t0, t1, grid, m->dx, m->dy, m->carries, m->status, m->stream,
                                       m->l1));
        }
        if (c >= 1) {
            // chunk c-1: fix-up of its runs (they end by chunk c), then its rows go down
            int t0, t1;
            chunk_tiles(c - 1, &t0, &t1);
            if (m->P.runs)
                CU(launch_fix_runs_f64(kModeSpmv, m->P, p.fpre[(size_t)c - 1], p.fpre[(size_t)c], m->dy, m->carries,
                                       nullptr, m->stream));
            else
                CU(launch_merge_fixup_range(m->M, m->P.subc, nsub, t0, t1, m->dy, m->carries, m->stream,
                                            m->sm_count));
            CU(cudaEventRecord(p.ev_y[(size_t)c - 1], m->stream));
            CU(cudaStreamWaitEvent(p.out, p.ev_y[(size_t)c - 1], 0));
            const int r0 = row_lo(c - 1), r1 = row_lo(c);
            if (r1 > r0 && y_sm)
                CU(launch_host_copy(m->dy + r0, y + r0, r1 - r0, p.out));
            else if (r1 > r0)
                CU(cudaMemcpyAsync(y + r0, m->dy + r0, sizeof(double) * (size_t)(r1 - r0), cudaMemcpyDeviceToHost,
                                   p.out));
        }
    }
    CU(cudaStreamSynchronize(p.out));
    CU(cudaStreamSynchronize(p.in));
    return check_status(m);
}

}  // namespace

namespace pwmgpu {
void record_error(const char* msg) { g_err = msg ? msg : ""; }

long long poisson_row_start_host(long long row, long long m, long long n) {
    long long mn = m * n;
    long long below = row > m ? row - m : 0;
    long long left = row - (row + m - 1) / m;
    long long right = row - row / m;
    long long above = row < mn - m ? row : (mn - m > 0 ? mn - m : 0);
    return below + left + row + right + above;
}
}  // namespace pwmgpu

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* pwmgpu_last_error(void) { return g_err.c_str(); }

int pwmgpu_device_info(int* sm_count, size_t* free_bytes, size_t* total_bytes) {
    int dev = 0;
    CU(cudaGetDevice(&dev));
    int sms = 0;
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    size_t f = 0, t = 0;
    CU(cudaMemGetInfo(&f, &t));
    if (sm_count) *sm_count = sms;
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return PWMGPU_OK;
}

int pwmgpu_create(int format, int partitions, pwmgpu_matrix** out) {
    if (!out) return fail(PWMGPU_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (format != PWMGPU_FMT_MERGE && format != PWMGPU_FMT_CSB && format != PWMGPU_FMT_COH &&
        format != PWMGPU_FMT_AUTO)
        return fail(PWMGPU_ERR_INVALID, "unknown format %d", format);
    pwmgpu_matrix* m = new pwmgpu_matrix();
    m->auto_fmt = format == PWMGPU_FMT_AUTO;
    m->format = m->auto_fmt ? PWMGPU_FMT_MERGE : format;
    m->partitions = partitions > 0 ? partitions : 1;
    int rc = PWMGPU_OK;
    do {
        cudaError_t e = cudaGetDevice(&m->device);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e)); break; }
        e = cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, m->device);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "cudaDeviceGetAttribute: %s", cudaGetErrorString(e)); break; }
        e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); break; }
        m->own_stream = true;
        if ((rc = dalloc(&m->counter, 4)) != PWMGPU_OK) break;
        if ((rc = dalloc(&m->status, 4)) != PWMGPU_OK) break;
        if ((rc = dalloc(&m->small, 16)) != PWMGPU_OK) break;
        if ((rc = dalloc(&m->barrier, 4)) != PWMGPU_OK) break;
        e = cudaMallocHost((void**)&m->hres, 16 * sizeof(double));
        if (e != cudaSuccess) { m->hres = nullptr; rc = fail(PWMGPU_ERR_NOMEM, "cudaMallocHost: %s", cudaGetErrorString(e)); break; }
        cudaMemsetAsync(m->counter, 0, 4 * sizeof(unsigned int), m->stream);
        cudaMemsetAsync(m->status, 0, 4 * sizeof(int), m->stream);
        e = cudaStreamSynchronize(m->stream);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "init: %s", cudaGetErrorString(e)); break; }
    } while (0);
    if (rc != PWMGPU_OK) {
        m->release_all();
        if (m->own_stream && m->stream) cudaStreamDestroy(m->stream);
        delete m;
        return rc;
    }
    *out = m;
    return PWMGPU_OK;
}

int pwmgpu_destroy(pwmgpu_matrix* m) {
    if (!m) return PWMGPU_OK;
    if (m->stream) cudaStreamSynchronize(m->stream);
    m->release_all();
    if (m->own_stream && m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return PWMGPU_OK;
}

int pwmgpu_set_stream(pwmgpu_matrix* m, void* stream) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    CU(cudaStreamSynchronize(m->stream));
    if (m->own_stream) cudaStreamDestroy(m->stream);
    m->stream = (cudaStream_t)stream;
    m->own_stream = false;
    return PWMGPU_OK;
}

int pwmgpu_generate_poisson(pwmgpu_matrix* m, int32_t mx, int32_t ny) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (mx < 1 || ny < 1) return fail(PWMGPU_ERR_INVALID, "Poisson grid must be at least 1x1 (got %d x %d)", mx, ny);
    long long N = (long long)mx * ny;
    long long nnz = (long long)ny * (mx + 2LL * (mx - 1)) + 2LL * (ny - 1) * mx;  // CRS.hpp:64
    TRY(check_sizes(N, N, nnz));
    TRY(alloc_matrix(m, (int32_t)N, (int32_t)N, nnz));
    CU(launch_poisson_crs(mx, ny, m->M.row_start, m->M.col, m->M.val, m->sm_count, m->stream));
    return build_plan(m);
}

int pwmgpu_generate_random(pwmgpu_matrix* m, int32_t n, uint64_t seed, int length_dist, double mean_len,
                           double sigma, int32_t max_len, int32_t band_permille, int32_t band_half) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (n < 1) return fail(PWMGPU_ERR_INVALID, "n must be >= 1");
    if (length_dist != PWMGPU_RAND_LOGNORMAL && length_dist != PWMGPU_RAND_POISSON)
        return fail(PWMGPU_ERR_INVALID, "unknown length distribution %d", length_dist);
    if (!(mean_len > 0.0) || !std::isfinite(mean_len)) return fail(PWMGPU_ERR_INVALID, "mean_len must be > 0");
    if (length_dist == PWMGPU_RAND_LOGNORMAL && !(sigma > 0.0 && std::isfinite(sigma)))
        return fail(PWMGPU_ERR_INVALID, "sigma must be > 0");
    if (max_len < 1 || max_len > (1 << 20)) return fail(PWMGPU_ERR_INVALID, "max_len must be in [1, 2^20]");
    if (band_permille < 0 || band_permille > 1000) return fail(PWMGPU_ERR_INVALID, "band_permille in [0, 1000]");
    if (band_half < 0 || band_half > (1 << 30)) return fail(PWMGPU_ERR_INVALID, "band_half in [0, 2^30]");
    std::vector<uint64_t> thr;
    random_length_table(length_dist == PWMGPU_RAND_LOGNORMAL ? 0 : 1, mean_len, sigma, max_len, thr);
    m->release_matrix();
    uint64_t* dthr = nullptr;
    unsigned long long* dtotal = nullptr;
    int32_t* scratch = nullptr;
    int rc = PWMGPU_OK;
    do {
        if ((rc = dalloc(&dthr, thr.size())) != PWMGPU_OK) break;
        if ((rc = dalloc(&dtotal, 1)) != PWMGPU_OK) break;
        if ((rc = dalloc(&scratch, (size_t)scan_scratch_elems(n))) != PWMGPU_OK) break;
        if ((rc = dalloc(&m->M.row_start, (size_t)n + 1 + kPad)) != PWMGPU_OK) break;
        m->M.nor = m->M.noc = n;
        cudaError_t e = cudaMemcpyAsync(dthr, thr.data(), thr.size() * sizeof(uint64_t), cudaMemcpyHostToDevice,
                                        m->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(dtotal, 0, sizeof(unsigned long long), m->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(m->M.row_start + n + 1, 0, kPad * sizeof(int32_t), m->stream);
        if (e == cudaSuccess)
            e = launch_random_count(dthr, max_len, n, seed, band_permille, band_half, m->M.row_start, dtotal,
                                    m->sm_count, m->stream);
        unsigned long long total = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&total, dtotal, sizeof total, cudaMemcpyDeviceToHost, m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "random generator: %s", cudaGetErrorString(e)); break; }
        if ((rc = check_sizes(n, n, (long long)total)) != PWMGPU_OK) break;
        m->M.nnz = (long long)total;
        e = launch_inclusive_scan(m->M.row_start + 1, n, scratch, m->stream);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "scan: %s", cudaGetErrorString(e)); break; }
        if ((rc = dalloc(&m->M.col, (size_t)total + kPad)) != PWMGPU_OK) break;
        if ((rc = dalloc(&m->M.val, (size_t)total + kPad)) != PWMGPU_OK) break;
        e = cudaMemsetAsync(m->M.col + total, 0, kPad * sizeof(int32_t), m->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(m->M.val + total, 0, kPad * sizeof(double), m->stream);
        if (e == cudaSuccess)
            e = launch_random_fill(dthr, max_len, n, seed, band_permille, band_half, m->M.row_start, m->M.col,
                                   m->M.val, m->sm_count, m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "random generator: %s", cudaGetErrorString(e)); break; }
    } while (0);
    dfree(dthr);
    dfree(dtotal);
    dfree(scratch);
    if (rc != PWMGPU_OK) {
        m->release_matrix();
        return rc;
    }
    return build_plan(m);
}

}  // extern "C"
namespace {

struct TripletIn {
    int32_t* rows = nullptr;
    int32_t* cols = nullptr;
    double* vals = nullptr;
    void release() {
        dfree(rows);
        dfree(cols);
        dfree(vals);
    }
};

// Util/TripletToCRS.hpp:135-172 on the device: CRS with rows ascending and
// columns ascending within a row (duplicates in input order) from device
// triplet arrays, which are not modified.  With host arrays h_* the sorted
// triplet is also written back there, as the reference sorts its caller's
// triplet in place (TripletToCRS.hpp:139-142).  Entries are range-checked
// before anything of the previous matrix is released.
int load_triplets_dev(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, const int32_t* rows,
                      const int32_t* cols, const double* vals, int32_t* h_rows, int32_t* h_cols, double* h_vals) {
    int32_t* cnt = nullptr;
    int32_t* scan_scratch = nullptr;
    TripletScan* dflags = nullptr;
    unsigned long long *keys_a = nullptr, *keys_b = nullptr;
    int32_t *src_a = nullptr, *src_b = nullptr, *tab = nullptr;
    bool matrix_touched = false;
    int rc = PWMGPU_OK;
    do {
        const long long tab_elems = triplet_sort_table_elems(nnz);
        const long long scan_n = std::max<long long>(nor, tab_elems);
        if ((rc = dalloc(&cnt, (size_t)nor + 1)) != PWMGPU_OK) break;
        if ((rc = dalloc(&scan_scratch, (size_t)scan_scratch_elems(scan_n))) != PWMGPU_OK) break;
        if ((rc = dalloc(&dflags, 1)) != PWMGPU_OK) break;
        TripletScan flags{~0ull, 0u, 0u};
        cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)nor + 1), m->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dflags, &flags, sizeof flags, cudaMemcpyHostToDevice, m->stream);
        if (e == cudaSuccess) e = launch_triplet_scan(rows, cols, nnz, nor, noc, cnt, dflags, m->sm_count, m->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, dflags, sizeof flags, cudaMemcpyDeviceToHost, m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "triplet scan: %s", cudaGetErrorString(e)); break; }
        if (flags.bad != ~0ull) {
            const long long k = (long long)flags.bad;
            int32_t r = 0, c = 0;
            e = cudaMemcpy(&r, rows + k, sizeof r, cudaMemcpyDeviceToHost);
            if (e == cudaSuccess) e = cudaMemcpy(&c, cols + k, sizeof c, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "triplet check: %s", cudaGetErrorString(e)); break; }
            if (r < 0 || r >= nor)
                rc = fail(PWMGPU_ERR_INVALID, "row %d at entry %lld out of range", r, k);
            else
                rc = fail(PWMGPU_ERR_INVALID, "column %d at entry %lld out of range", c, k);
            break;
        }
        e = launch_inclusive_scan(cnt + 1, nor, scan_scratch, m->stream);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "row scan: %s", cudaGetErrorString(e)); break; }
        matrix_touched = true;
        if ((rc = alloc_matrix(m, nor, noc, nnz)) != PWMGPU_OK) break;
        e = cudaMemcpyAsync(m->M.row_start, cnt, sizeof(int32_t) * ((size_t)nor + 1), cudaMemcpyDeviceToDevice,
                            m->stream);
        if (e == cudaSuccess && nnz > 0 && !flags.unsorted_rc) {
            // already in CRS order: the columns and values are the input
            e = cudaMemcpyAsync(m->M.col, cols, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToDevice, m->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(m->M.val, vals, sizeof(double) * (size_t)nnz, cudaMemcpyDeviceToDevice,
                                    m->stream);
        } else if (e == cudaSuccess && nnz > 0) {
            if ((rc = dalloc(&keys_a, (size_t)nnz)) != PWMGPU_OK) break;
            if ((rc = dalloc(&keys_b, (size_t)nnz)) != PWMGPU_OK) break;
            if ((rc = dalloc(&src_a, (size_t)nnz)) != PWMGPU_OK) break;
            if ((rc = dalloc(&src_b, (size_t)nnz)) != PWMGPU_OK) break;
            if ((rc = dalloc(&tab, (size_t)tab_elems)) != PWMGPU_OK) break;
            unsigned long long* keys = nullptr;
            int32_t* src = nullptr;
            e = launch_triplet_sort(rows, cols, nnz, nor, noc, flags.unsorted_c != 0, keys_a, src_a, keys_b, src_b,
                                    tab, scan_scratch, &keys, &src, m->sm_count, m->stream);
            // the sorted rows (for the caller's triplet) overwrite the source indices
            if (e == cudaSuccess)
                e = launch_triplet_gather(keys, src, vals, nnz, m->M.col, m->M.val, h_rows ? src : nullptr,
                                          m->sm_count, m->stream);
            if (e == cudaSuccess && h_rows)
                e = cudaMemcpyAsync(h_rows, src, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToHost, m->stream);
            if (e == cudaSuccess && h_cols)
                e = cudaMemcpyAsync(h_cols, m->M.col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToHost,
                                    m->stream);
            if (e == cudaSuccess && h_vals)
                e = cudaMemcpyAsync(h_vals, m->M.val, sizeof(double) * (size_t)nnz, cudaMemcpyDeviceToHost,
                                    m->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "triplet to CRS: %s", cudaGetErrorString(e)); break; }
    } while (0);
    dfree(cnt);
    dfree(scan_scratch);
    dfree(dflags);
    dfree(keys_a);
    dfree(keys_b);
    dfree(src_a);
    dfree(src_b);
    dfree(tab);
    if (rc != PWMGPU_OK) {
        if (matrix_touched) m->release_matrix();
        return rc;
    }
    return build_plan(m);
}

}  // namespace
extern "C" {

int pwmgpu_load_csr(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, const int32_t* row_start,
                    const int32_t* col_ind, const double* vals) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    TRY(check_sizes(nor, noc, nnz));
    if (!row_start || (nnz > 0 && (!col_ind || !vals))) return fail(PWMGPU_ERR_INVALID, "null CRS array");
    if (row_start[0] != 0 || row_start[nor] != nnz)
        return fail(PWMGPU_ERR_INVALID, "row_start must run from 0 to nnz (got %d..%d, nnz %d)", row_start[0],
                    row_start[nor], nnz);
    for (int32_t i = 0; i < nor; ++i)
        if (row_start[i + 1] < row_start[i]) return fail(PWMGPU_ERR_INVALID, "row_start decreases at row %d", i);
    for (int32_t k = 0; k < nnz; ++k)
        if (col_ind[k] < 0 || col_ind[k] >= noc)
            return fail(PWMGPU_ERR_INVALID, "column index %d at nonzero %d out of range [0,%d)", col_ind[k], k, noc);
    TRY(alloc_matrix(m, nor, noc, nnz));
    CU(cudaMemcpyAsync(m->M.row_start, row_start, sizeof(int32_t) * ((size_t)nor + 1), cudaMemcpyHostToDevice,
                       m->stream));
    if (nnz > 0) {
        CU(cudaMemcpyAsync(m->M.col, col_ind, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, m->stream));
        CU(cudaMemcpyAsync(m->M.val, vals, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, m->stream));
    }
    return build_plan(m);
}

int pwmgpu_load_triplets(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, int32_t* rows, int32_t* cols,
                         double* vals) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    TRY(check_sizes(nor, noc, nnz));
    if (nnz > 0 && (!rows || !cols || !vals)) return fail(PWMGPU_ERR_INVALID, "null triplet array");
    // the triplet goes up, is sorted on the device and comes back sorted
    TripletIn in;
    int rc = PWMGPU_OK;
    do {
        if ((rc = dalloc(&in.rows, (size_t)nnz)) != PWMGPU_OK) break;
        if ((rc = dalloc(&in.cols, (size_t)nnz)) != PWMGPU_OK) break;
        if ((rc = dalloc(&in.vals, (size_t)nnz)) != PWMGPU_OK) break;
        cudaError_t e = cudaSuccess;
        if (nnz > 0) {
            e = cudaMemcpyAsync(in.rows, rows, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, m->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(in.cols, cols, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, m->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(in.vals, vals, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, m->stream);
        }
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "triplet upload: %s", cudaGetErrorString(e)); break; }
        rc = load_triplets_dev(m, nor, noc, nnz, in.rows, in.cols, in.vals, rows, cols, vals);
    } while (0);
    in.release();
    return rc;
}

int pwmgpu_load_triplets_device(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, const int32_t* d_rows,
                                const int32_t* d_cols, const double* d_vals) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    TRY(check_sizes(nor, noc, nnz));
    if (nnz > 0 && (!d_rows || !d_cols || !d_vals)) return fail(PWMGPU_ERR_INVALID, "null triplet array");
    return load_triplets_dev(m, nor, noc, nnz, d_rows, d_cols, d_vals, nullptr, nullptr, nullptr);
}

int pwmgpu_stats(pwmgpu_matrix* m, pwmgpu_matrix_stats* out) {
    if (!m || !out) return fail(PWMGPU_ERR_INVALID, "null handle or output");
    const long long n = m->M.nor, nnz = m->M.nnz;
    if (!m->loaded || n <= 0 || !m->M.row_start)
        return fail(PWMGPU_ERR_INVALID, "statistics need a loaded, non-empty matrix");
    // Util_Scripts/calc_stats.cpp:45-58
    const double avg = (double)nnz / (double)n;
    const int lg = (int)std::ceil(std::log2(std::sqrt((double)n)));
    const int bits = std::min(16, 3 + lg);
    const long long nbw = n >> bits;  // whole blocks (the script's nb_blocks after :70-73)
    unsigned int* blocks = nullptr;
    long long* brow = nullptr;
    double *rp = nullptr, *bp = nullptr;
    StatsDev* dst = nullptr;
    int32_t* tcol = nullptr;
    double* tval = nullptr;
    const int32_t* col = m->M.col;
    int rc = PWMGPU_OK;
    StatsDev h{};
    do {
        if (nbw > 0 && nnz > 0 && !col) {
            // the merge format keeps only its lane-interleaved copy of the
            // columns: bring them back to CRS order for the block pass
            if ((rc = dalloc(&tcol, (size_t)nnz)) != PWMGPU_OK) break;
            if ((rc = dalloc(&tval, (size_t)nnz)) != PWMGPU_OK) break;
            cudaError_t e = launch_mli_unpermute(m->P, tcol, tval, m->sm_count, m->stream);
            if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "matrix statistics: %s", cudaGetErrorString(e)); break; }
            col = tcol;
        }
        if ((rc = dalloc(&blocks, (size_t)(nbw * nbw))) != PWMGPU_OK) break;
        if ((rc = dalloc(&brow, (size_t)nbw)) != PWMGPU_OK) break;
        if ((rc = dalloc(&rp, (size_t)stats_row_ctas((int)n))) != PWMGPU_OK) break;
        if ((rc = dalloc(&bp, (size_t)nbw)) != PWMGPU_OK) break;
        if ((rc = dalloc(&dst, 1)) != PWMGPU_OK) break;
        cudaError_t e = cudaMemsetAsync(blocks, 0, sizeof(unsigned int) * (size_t)(nbw * nbw), m->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(dst, 0, sizeof(StatsDev), m->stream);
        if (e == cudaSuccess)
            e = launch_matrix_stats(m->M.row_start, col, (int)n, avg, bits, (int)nbw, blocks, brow, rp, bp, dst,
                                    m->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h, dst, sizeof h, cudaMemcpyDeviceToHost, m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        if (e != cudaSuccess) rc = fail(PWMGPU_ERR_CUDA, "matrix statistics: %s", cudaGetErrorString(e));
    } while (0);
    dfree(blocks);
    dfree(brow);
    dfree(rp);
    dfree(bp);
    dfree(dst);
    dfree(tcol);
    dfree(tval);
    if (rc != PWMGPU_OK) return rc;
    out->size = n;
    out->nnz = nnz;
    out->rows_avg = avg;
    out->rows_var = h.rows_var;
    out->block_avg = h.block_avg;
    out->block_var = h.block_var;
    out->balanced = h.balanced;
    out->block_bits = bits;
    out->nb_blocks = (int32_t)nbw;
    out->max_row_nnz = h.max_row_nnz;
    return PWMGPU_OK;
}

int pwmgpu_dims(const pwmgpu_matrix* m, int32_t* nor, int32_t* noc, int64_t* nnz) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (nor) *nor = m->M.nor;
    if (noc) *noc = m->M.noc;
    if (nnz) *nnz = m->M.nnz;
    return PWMGPU_OK;
}

int pwmgpu_get_csr(pwmgpu_matrix* m, int32_t* row_start, int32_t* col_ind, double* vals) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (!row_start || (m->M.nnz > 0 && (!col_ind || !vals))) return fail(PWMGPU_ERR_INVALID, "null output array");
    CU(cudaMemcpyAsync(row_start, m->M.row_start, sizeof(int32_t) * ((size_t)m->M.nor + 1), cudaMemcpyDeviceToHost,
                       m->stream));
    if (m->M.nnz > 0 && m->format != PWMGPU_FMT_MERGE) {
        // the CSB / CO-H handles keep the CRS arrays
        CU(cudaMemcpyAsync(col_ind, m->M.col, sizeof(int32_t) * (size_t)m->M.nnz, cudaMemcpyDeviceToHost, m->stream));
        CU(cudaMemcpyAsync(vals, m->M.val, sizeof(double) * (size_t)m->M.nnz, cudaMemcpyDeviceToHost, m->stream));
    } else if (m->M.nnz > 0) {
        // back from the lane-interleaved storage to CRS order
        int32_t* dc = nullptr;
        double* dv = nullptr;
        TRY(dalloc(&dc, (size_t)m->M.nnz));
        int rc = dalloc(&dv, (size_t)m->M.nnz);
        cudaError_t e = cudaSuccess;
        if (rc == PWMGPU_OK) e = launch_mli_unpermute(m->P, dc, dv, m->sm_count, m->stream);
        if (rc == PWMGPU_OK && e == cudaSuccess)
            e = cudaMemcpyAsync(col_ind, dc, sizeof(int32_t) * (size_t)m->M.nnz, cudaMemcpyDeviceToHost, m->stream);
        if (rc == PWMGPU_OK && e == cudaSuccess)
            e = cudaMemcpyAsync(vals, dv, sizeof(double) * (size_t)m->M.nnz, cudaMemcpyDeviceToHost, m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        dfree(dc);
        dfree(dv);
        if (rc != PWMGPU_OK) return rc;
        if (e != cudaSuccess) return fail(PWMGPU_ERR_CUDA, "get_csr: %s", cudaGetErrorString(e));
    }
    CU(cudaStreamSynchronize(m->stream));
    return PWMGPU_OK;
}

int pwmgpu_mv_device(pwmgpu_matrix* m, const double* dx, double* dy) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (m->M.nor > 0 && (!dx || !dy)) return fail(PWMGPU_ERR_INVALID, "null vector");
    return spmv_f64(m, dx, dy);
}

int pwmgpu_mv(pwmgpu_matrix* m, const double* x, double* y) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (m->M.nor == 0) return PWMGPU_OK;
    if (!y || (m->M.noc > 0 && !x)) return fail(PWMGPU_ERR_INVALID, "null vector");
    TRY(ensure_vectors(m));
    if (fp64_format(m) == PWMGPU_FMT_MERGE) {
        int rc = plan_pipeline(m);
        if (rc != PWMGPU_OK) return rc;
        if (m->pipe.K > 0) return mv_pipelined(m, x, y);
    }
    if (m->M.noc > 0)
        CU(cudaMemcpyAsync(m->dx, x, sizeof(double) * (size_t)m->M.noc, cudaMemcpyHostToDevice, m->stream));
    TRY(spmv_f64(m, m->dx, m->dy));
    CU(cudaMemcpyAsync(y, m->dy, sizeof(double) * (size_t)m->M.nor, cudaMemcpyDeviceToHost, m->stream));
    return check_status(m);
}

int pwmgpu_power_device(pwmgpu_matrix* m, double* dx, double* dy, int32_t it) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (m->M.nor != m->M.noc) return fail(PWMGPU_ERR_NOT_SQUARE, "power method needs a square matrix");
    if (it < 0) return fail(PWMGPU_ERR_INVALID, "negative iteration count");
    if (m->M.nor > 0 && (!dx || !dy)) return fail(PWMGPU_ERR_INVALID, "null vector");
    return power_device(m, dx, dy, it);
}

int pwmgpu_power(pwmgpu_matrix* m, double* x, double* y, int32_t it) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (m->M.nor != m->M.noc) return fail(PWMGPU_ERR_NOT_SQUARE, "power method needs a square matrix");
    if (it < 0) return fail(PWMGPU_ERR_INVALID, "negative iteration count");
    if (it == 0 || m->M.nor == 0) return PWMGPU_OK;
    if (!x || !y) return fail(PWMGPU_ERR_INVALID, "null vector");
    TRY(ensure_vectors(m));
    const size_t bytes = sizeof(double) * (size_t)m->M.nor;
    CU(cudaMemcpyAsync(m->dx, x, bytes, cudaMemcpyHostToDevice, m->stream));
    TRY(power_device(m, m->dx, m->dy, it));
    CU(cudaMemcpyAsync(x, m->dx, bytes, cudaMemcpyDeviceToHost, m->stream));
    CU(cudaMemcpyAsync(y, m->dy, bytes, cudaMemcpyDeviceToHost, m->stream));
    return check_status(m);
}

int pwmgpu_merge_partition(pwmgpu_matrix* m, int32_t parts, int32_t* coords) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (parts < 1 || !coords) return fail(PWMGPU_ERR_INVALID, "parts must be >= 1 and coords non-null");
    const long long total = (long long)m->M.nor + m->M.nnz;
    const long long ipt = (total + parts - 1) / parts;  // CRS_Merge.hpp:98
    int2* d = nullptr;
    TRY(dalloc(&d, (size_t)parts + 1));
    cudaError_t e = launch_merge_partition(m->M.row_start, m->M.nor, m->M.nnz, ipt, parts, d, m->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(coords, d, sizeof(int2) * ((size_t)parts + 1), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    dev_free(d);
    if (e != cudaSuccess) return fail(PWMGPU_ERR_CUDA, "merge partition: %s", cudaGetErrorString(e));
    return PWMGPU_OK;
}

int pwmgpu_tile_info(const pwmgpu_matrix* m, int32_t* items_per_tile, int32_t* num_tiles, int32_t* grid) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (items_per_tile) *items_per_tile = m->tm;
    if (num_tiles) *num_tiles = m->num_tiles;
    if (grid) *grid = m->grid;
    return PWMGPU_OK;
}

int pwmgpu_mv_device_f32(pwmgpu_matrix* m, const float* dx, float* dy) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (m->format != PWMGPU_FMT_MERGE) return fail(PWMGPU_ERR_UNSUPPORTED, "FP32 SpMV runs on the merge format");
    if (m->M.nor > 0 && (!dx || !dy)) return fail(PWMGPU_ERR_INVALID, "null vector");
    if (m->num_tiles == 0) return PWMGPU_OK;
    if (sell_for(m, kCfgF32)) {
        CU(launch_sell_spmv(m->sell, false, m->M.row_start, m->M.nor, dx, dy, nullptr, nullptr, m->counter + 2,
                            m->sm_count, m->stream));
        return PWMGPU_OK;
    }
    int cfg = kCfgF32, pg = 0;
    const void* valp = nullptr;
    TRY(ensure_low_values(m, false, &cfg, &valp, &pg));
    CU(launch_merge_spmv(kCfgF32, kModeSpmv, m->M, valp, m->P, merge_grid(kCfgF32, m->num_tiles, m->sm_count, m->l1),
                         dx, dy, m->carries, nullptr, m->status, m->stream, m->l1));
    if (m->P.runs)
        CU(launch_fix_runs_f32(kModeSpmv, m->P, 0, m->P.nruns, dy, reinterpret_cast<float*>(m->carries), nullptr,
                               m->stream));
    else
        CU(launch_merge_fixup_f32(kModeSpmv, m->M, m->P.subc, m->num_tiles, dy, reinterpret_cast<float*>(m->carries),
                                  nullptr, m->fix_grid, m->stream));
    return PWMGPU_OK;
}

int pwmgpu_set_low_format(pwmgpu_matrix* m, int fmt) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (fmt != PWMGPU_LOWFMT_AUTO && fmt != PWMGPU_LOWFMT_MERGE)
        return fail(PWMGPU_ERR_INVALID, "unknown low-precision format %d", fmt);
    m->low_format = fmt;
    return PWMGPU_OK;
}

int pwmgpu_set_power_mode(pwmgpu_matrix* m, int mode) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (mode != PWMGPU_POWER_AUTO && mode != PWMGPU_POWER_FUSED && mode != PWMGPU_POWER_MULTI)
        return fail(PWMGPU_ERR_INVALID, "unknown power mode %d", mode);
    m->power_mode = mode;
    return PWMGPU_OK;
}

int pwmgpu_row_blocks(int32_t nor, int32_t parts, int32_t* first_rows, int32_t* thread_rows) {
    if (nor < 0 || parts < 1 || !first_rows || !thread_rows)
        return fail(PWMGPU_ERR_INVALID, "row blocks: nor >= 0, parts >= 1 and non-null outputs");
    // Util/TripletToCRS.hpp:318-327: round(nor / partitions) on integers
    const int32_t am = nor / parts;
    int32_t last = 0;
    for (int32_t i = 0; i < parts; ++i) {
        first_rows[i] = last;
        last = (i == parts - 1) ? nor : first_rows[i] + am;
        thread_rows[i] = last - first_rows[i];
    }
    return PWMGPU_OK;
}

int pwmgpu_generate_poisson_rows(pwmgpu_matrix* m, int32_t mx, int32_t ny, int32_t first_row, int32_t last_row) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (mx < 1 || ny < 1) return fail(PWMGPU_ERR_INVALID, "Poisson grid must be at least 1x1 (got %d x %d)", mx, ny);
    const long long N = (long long)mx * ny;
    TRY(check_sizes(N, N, (long long)ny * (mx + 2LL * (mx - 1)) + 2LL * (ny - 1) * mx));
    if (first_row < 0 || last_row < first_row || last_row > N)
        return fail(PWMGPU_ERR_INVALID, "row block [%d, %d) outside the %lld rows", first_row, last_row, N);
    const long long nnz = poisson_rows_nnz(mx, ny, first_row, last_row);
    TRY(alloc_matrix(m, last_row - first_row, (int32_t)N, nnz));
    if (last_row > first_row)
        CU(launch_poisson_crs(mx, ny, m->M.row_start, m->M.col, m->M.val, m->sm_count, m->stream, first_row,
                              last_row));
    else
        CU(cudaMemsetAsync(m->M.row_start, 0, sizeof(int32_t), m->stream));
    return build_plan(m);
}

int pwmgpu_load_triplets_rows(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, const int32_t* rows,
                              const int32_t* cols, const double* vals, int32_t first_row, int32_t last_row) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    TRY(check_sizes(nor, noc, nnz));
    if (nnz > 0 && (!rows || !cols || !vals)) return fail(PWMGPU_ERR_INVALID, "null triplet array");
    if (first_row < 0 || last_row < first_row || last_row > nor)
        return fail(PWMGPU_ERR_INVALID, "row block [%d, %d) outside the %d rows", first_row, last_row, nor);
    // the block's entries, rows counted from first_row (TripletToCRS.hpp:328-345)
    std::vector<int32_t> r, c;
    std::vector<double> v;
    for (int32_t i = 0; i < nnz; ++i) {
        if (rows[i] < 0 || rows[i] >= nor)
            return fail(PWMGPU_ERR_INVALID, "triplet entry %d: row %d outside [0, %d)", i, rows[i], nor);
        if (rows[i] >= first_row && rows[i] < last_row) {
            r.push_back(rows[i] - first_row);
            c.push_back(cols[i]);
            v.push_back(vals[i]);
        }
    }
    const int32_t bn = (int32_t)r.size();
    TripletIn in;
    int rc = PWMGPU_OK;
    do {
        if ((rc = dalloc(&in.rows, (size_t)bn)) != PWMGPU_OK) break;
        if ((rc = dalloc(&in.cols, (size_t)bn)) != PWMGPU_OK) break;
        if ((rc = dalloc(&in.vals, (size_t)bn)) != PWMGPU_OK) break;
        cudaError_t e = cudaSuccess;
        if (bn > 0) {
            e = cudaMemcpyAsync(in.rows, r.data(), sizeof(int32_t) * (size_t)bn, cudaMemcpyHostToDevice, m->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(in.cols, c.data(), sizeof(int32_t) * (size_t)bn, cudaMemcpyHostToDevice,
                                    m->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(in.vals, v.data(), sizeof(double) * (size_t)bn, cudaMemcpyHostToDevice, m->stream);
        }
        if (e != cudaSuccess) { rc = fail(PWMGPU_ERR_CUDA, "triplet upload: %s", cudaGetErrorString(e)); break; }
        rc = load_triplets_dev(m, last_row - first_row, noc, bn, in.rows, in.cols, in.vals, nullptr, nullptr, nullptr);
    } while (0);
    in.release();
    return rc;
}

int pwmgpu_rows_step_device(pwmgpu_matrix* m, const double* dx_full, double* dy_loc, double* dnsq_loc) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (!dnsq_loc || (m->M.nor > 0 && (!dx_full || !dy_loc))) return fail(PWMGPU_ERR_INVALID, "null vector");
    if (m->M.nor == 0) {
        CU(cudaMemsetAsync(dnsq_loc, 0, sizeof(double), m->stream));
        return PWMGPU_OK;
    }
    if (fp64_format(m) != PWMGPU_FMT_MERGE || m->num_tiles == 0) {
        TRY(spmv_f64(m, dx_full, dy_loc));
        CU(launch_power_norm_f64(dy_loc, nullptr, m->M.nor, m->partials, m->counter, dnsq_loc,
                                 dot_grid(m->M.nor, m->sm_count), m->stream));
        return PWMGPU_OK;
    }
    return power_step_f64(m, dx_full, dy_loc, nullptr, dnsq_loc);
}

int pwmgpu_rows_normalize_device(pwmgpu_matrix* m, double* dy_loc, const double* dnsq_total) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (m->M.nor == 0) return PWMGPU_OK;
    if (!dy_loc || !dnsq_total) return fail(PWMGPU_ERR_INVALID, "null vector");
    CU(launch_power_finalize_f64(dy_loc, dnsq_total, nullptr, nullptr, m->M.nor, m->sm_count, m->stream));
    return PWMGPU_OK;
}

int pwmgpu_test_grid_wait(pwmgpu_matrix* m, int64_t cycles, int32_t extra) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (cycles == 0 && extra == 0) {
        m->grid_wait = GridWait{kWaitCycles, 0u};
        return PWMGPU_OK;
    }
    if (cycles < 10000 || cycles > kWaitCycles || (extra != 0 && extra != 1))
        return fail(PWMGPU_ERR_INVALID, "grid wait: cycles in [1e4, %lld] and extra 0 or 1 (got %lld, %d)",
                    (long long)kWaitCycles, (long long)cycles, extra);
    m->grid_wait = GridWait{(long long)cycles, (unsigned int)extra};
    return PWMGPU_OK;
}

int pwmgpu_solve(pwmgpu_matrix* m, double* x, int32_t max_it, double tol, int precision, pwmgpu_solve_info* info) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (m->M.nor != m->M.noc) return fail(PWMGPU_ERR_NOT_SQUARE, "power method needs a square matrix");
    if (m->M.nor == 0) return fail(PWMGPU_ERR_INVALID, "empty matrix");
    if (!x || !info) return fail(PWMGPU_ERR_INVALID, "null vector or info");
    if (max_it < 2) return fail(PWMGPU_ERR_INVALID, "max_it must be at least 2 (got %d)", max_it);
    if (!(tol >= 0.0)) return fail(PWMGPU_ERR_INVALID, "tol must be >= 0");
    if (precision != PWMGPU_PREC_F64 && precision != PWMGPU_PREC_F32 && precision != PWMGPU_PREC_MIXED)
        return fail(PWMGPU_ERR_INVALID, "unknown precision %d", precision);
    if (m->format != PWMGPU_FMT_MERGE) return fail(PWMGPU_ERR_UNSUPPORTED, "the solve runs on the merge format");
    std::memset(info, 0, sizeof *info);
    return solve(m, x, max_it, tol, precision, info);
}

int pwmgpu_csb_info(const pwmgpu_matrix* m, int32_t* beta, int32_t* block_bits, int32_t* hb, int32_t* vb,
                    int64_t* nnz) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded || m->format != PWMGPU_FMT_CSB) return fail(PWMGPU_ERR_STATE, "no CSB matrix loaded");
    if (beta) *beta = m->csb.beta;
    if (block_bits) *block_bits = m->csb.bits;
    if (hb) *hb = m->csb.hb;
    if (vb) *vb = m->csb.vb;
    if (nnz) *nnz = m->M.nnz;
    return PWMGPU_OK;
}

int pwmgpu_get_csb(pwmgpu_matrix* m, uint32_t* ind, double* data, int32_t* blk_ptr) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded || m->format != PWMGPU_FMT_CSB) return fail(PWMGPU_ERR_STATE, "no CSB matrix loaded");
    const auto& c = m->csb;
    if (!blk_ptr || (m->M.nnz > 0 && (!ind || !data))) return fail(PWMGPU_ERR_INVALID, "null output array");
    // the host copies are the reference's arrays (the device copy orders
    // dense sub-squares row-major for the kernel)
    if (m->M.nnz > 0) {
        std::memcpy(ind, c.h_ind.data(), sizeof(uint32_t) * (size_t)m->M.nnz);
        std::memcpy(data, c.h_data.data(), sizeof(double) * (size_t)m->M.nnz);
    }
    std::memcpy(blk_ptr, c.h_blk_ptr.data(), sizeof(int32_t) * c.h_blk_ptr.size());
    return PWMGPU_OK;
}

int pwmgpu_coh_info(const pwmgpu_matrix* m, int32_t* partitions, int64_t* row_jumps, int64_t* blocks,
                    int64_t* block_row_jumps, int64_t* nnz) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded || m->format != PWMGPU_FMT_COH) return fail(PWMGPU_ERR_STATE, "no CO-H matrix loaded");
    const auto& c = m->coh;
    if (partitions) *partitions = c.parts;
    if (row_jumps) *row_jumps = (int64_t)c.h_row_jump.size();
    if (blocks) *blocks = c.nblocks;
    if (block_row_jumps) *block_row_jumps = (int64_t)c.row_jump_block.size();
    if (nnz) *nnz = m->M.nnz;
    return PWMGPU_OK;
}

int pwmgpu_get_coh(pwmgpu_matrix* m, int32_t* part_info, uint16_t* row_jump, uint16_t* col_jump, double* data,
                   int32_t* block_nnz, int16_t* row_jump_block, int16_t* col_jump_block) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded || m->format != PWMGPU_FMT_COH) return fail(PWMGPU_ERR_STATE, "no CO-H matrix loaded");
    const auto& c = m->coh;
    if (!part_info) return fail(PWMGPU_ERR_INVALID, "null output array");
    auto put = [](auto* dst, const auto& v) {
        if (dst && !v.empty()) std::memcpy(dst, v.data(), sizeof(v[0]) * v.size());
    };
    put(part_info, c.part_info);
    // the reference's arrays, kept on the host (the device holds the tiles)
    put(row_jump, c.h_row_jump);
    put(col_jump, c.h_col_jump);
    put(data, c.h_data);
    put(block_nnz, c.block_nnz);
    put(row_jump_block, c.row_jump_block);
    put(col_jump_block, c.col_jump_block);
    return PWMGPU_OK;
}

int pwmgpu_csb_params(int32_t nor, int32_t noc, int32_t* beta, int32_t* block_bits) {
    if (nor < 1 || noc < 1) return fail(PWMGPU_ERR_INVALID, "empty matrix");
    int b = 0, bits = 0;
    csb_params(nor, noc, &b, &bits);
    if (beta) *beta = b;
    if (block_bits) *block_bits = bits;
    return PWMGPU_OK;
}

int pwmgpu_csb_build_host(int32_t nor, int32_t noc, int64_t nnz, const int32_t* row_start, const int32_t* col_ind,
                          const double* vals, uint32_t* ind, double* data, int32_t* blk_ptr) {
    TRY(check_sizes(nor, noc, nnz));
    if (nor < 1 || noc < 1) return fail(PWMGPU_ERR_INVALID, "empty matrix");
    if (!row_start || !blk_ptr || (nnz > 0 && (!col_ind || !vals || !ind || !data)))
        return fail(PWMGPU_ERR_INVALID, "null array");
    TRY(check_host_crs(nor, noc, nnz, row_start, col_ind));
    int beta = 0, bits = 0;
    csb_params(nor, noc, &beta, &bits);
    std::vector<uint32_t> vi;
    std::vector<double> vd;
    std::vector<int32_t> vb;
    std::vector<int> wp, un;
    csb_build_host(nor, noc, nnz, row_start, col_ind, vals, beta, bits, vi, vd, vb, std::min(beta, 1024), wp, un);
    if (nnz > 0) {
        std::memcpy(ind, vi.data(), sizeof(uint32_t) * (size_t)nnz);
        std::memcpy(data, vd.data(), sizeof(double) * (size_t)nnz);
    }
    std::memcpy(blk_ptr, vb.data(), sizeof(int32_t) * vb.size());
    return PWMGPU_OK;
}

int pwmgpu_coh_build_host(int32_t nor, int32_t noc, int64_t nnz, const int32_t* row_start, const int32_t* col_ind,
                          const double* vals, int32_t threads, int32_t* partitions, int64_t* row_jumps,
                          int64_t* blocks, int64_t* block_row_jumps, int32_t* part_info, uint16_t* row_jump,
                          uint16_t* col_jump, double* data, int32_t* block_nnz, int16_t* row_jump_block,
                          int16_t* col_jump_block) {
    TRY(check_sizes(nor, noc, nnz));
    if (nor < 1 || noc < 1) return fail(PWMGPU_ERR_INVALID, "empty matrix");
    if (!row_start || !part_info || (nnz > 0 && (!col_ind || !vals)))
        return fail(PWMGPU_ERR_INVALID, "null array");
    TRY(check_host_crs(nor, noc, nnz, row_start, col_ind));
    std::vector<int32_t> pi, bn;
    std::vector<uint16_t> rj, cj;
    std::vector<double> d;
    std::vector<int16_t> rjb, cjb;
    std::vector<int> parts, blks;
    const int T = coh_build_host(nor, noc, nnz, row_start, col_ind, vals, std::max(threads, 1), pi, rj, cj, d, bn,
                                 rjb, cjb, parts, blks);
    if (partitions) *partitions = T;
    if (row_jumps) *row_jumps = (int64_t)rj.size();
    if (blocks) *blocks = (int64_t)bn.size();
    if (block_row_jumps) *block_row_jumps = (int64_t)rjb.size();
    auto put = [](auto* dst, const auto& v) {
        if (dst && !v.empty()) std::memcpy(dst, v.data(), sizeof(v[0]) * v.size());
    };
    put(part_info, pi);
    put(row_jump, rj);
    put(col_jump, cj);
    put(data, d);
    put(block_nnz, bn);
    put(row_jump_block, rjb);
    put(col_jump_block, cjb);
    return PWMGPU_OK;
}

int pwmgpu_tile_layout_host(int32_t format, int32_t nor, int32_t noc, int64_t nnz, const int32_t* row_start,
                            const int32_t* col_ind, const double* vals, int32_t partitions, int32_t window,
                            int64_t* sizes, int32_t* win_ptr, int32_t* units, uint32_t* ind, double* data,
                            int32_t* col) {
    TRY(check_sizes(nor, noc, nnz));
    if (nor < 1 || noc < 1) return fail(PWMGPU_ERR_INVALID, "empty matrix");
    if (format != PWMGPU_FMT_CSB && format != PWMGPU_FMT_COH) return fail(PWMGPU_ERR_INVALID, "format: CSB or CO-H");
    if (!row_start || !sizes || (nnz > 0 && (!col_ind || !vals))) return fail(PWMGPU_ERR_INVALID, "null array");
    TRY(check_host_crs(nor, noc, nnz, row_start, col_ind));
    int beta = 1024, bits = 0;
    if (format == PWMGPU_FMT_CSB) csb_params(nor, noc, &beta, &bits);
    if (window < 64 || window > std::min(beta, 1024) || (window & (window - 1)) != 0)
        return fail(PWMGPU_ERR_INVALID, "window: a power of two in [64, min(beta, 1024)]");
    std::vector<uint32_t> eind, kind;
    std::vector<double> edata, kdata;
    std::vector<int32_t> blk, kcol;
    std::vector<int> wp, un;
    if (format == PWMGPU_FMT_CSB) {
        csb_build_host(nor, noc, nnz, row_start, col_ind, vals, beta, bits, eind, edata, blk, window, wp, un);
    } else {
        std::vector<int32_t> pi, bn;
        std::vector<uint16_t> rj, cj;
        std::vector<double> d;
        std::vector<int16_t> rjb, cjb;
        std::vector<int> parts, blks;
        coh_build_host(nor, noc, nnz, row_start, col_ind, vals, std::max(partitions, 1), pi, rj, cj, d, bn, rjb, cjb,
                       parts, blks);
        coh_tile_units(nor, noc, nnz, row_start, col_ind, vals, parts, window, eind, edata, wp, un);
    }
    if (!csb_kernel_layout(eind, edata, window, wp, un, kind, kdata, kcol))
        return fail(PWMGPU_ERR_INVALID, "the padded device copy exceeds 32-bit element offsets");
    sizes[0] = (int64_t)wp.size();
    sizes[1] = (int64_t)un.size();
    sizes[2] = (int64_t)kind.size();
    if (win_ptr && units && ind && data && col) {
        std::memcpy(win_ptr, wp.data(), sizeof(int32_t) * wp.size());
        if (!un.empty()) std::memcpy(units, un.data(), sizeof(int32_t) * un.size());
        std::memcpy(ind, kind.data(), sizeof(uint32_t) * kind.size());
        std::memcpy(data, kdata.data(), sizeof(double) * kdata.size());
        std::memcpy(col, kcol.data(), sizeof(int32_t) * kcol.size());
    }
    return PWMGPU_OK;
}

int pwmgpu_launch_config(const pwmgpu_matrix* m, int32_t* prefer_l1, int32_t* grid, int32_t* power_grid,
                         float* tuned_ms) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (prefer_l1) *prefer_l1 = m->l1 & 1;
    if (grid) *grid = m->grid;
    if (power_grid) *power_grid = m->pgrid;
    if (tuned_ms) {
        tuned_ms[0] = m->tune_ms[0];
        tuned_ms[1] = m->tune_ms[1];
    }
    return PWMGPU_OK;
}

int pwmgpu_launch_variant(const pwmgpu_matrix* m, int32_t* variant) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!variant) return fail(PWMGPU_ERR_INVALID, "null output");
    *variant = m->l1;
    return PWMGPU_OK;
}

int pwmgpu_set_launch_variant(pwmgpu_matrix* m, int32_t variant) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (variant != 0 && variant != 1 && variant != 4 && variant != 5)
        return fail(PWMGPU_ERR_INVALID, "launch variant must be 0, 1, 4 or 5");
    if (!m->loaded || m->format != PWMGPU_FMT_MERGE) return fail(PWMGPU_ERR_STATE, "no merge-format matrix loaded");
    CU(cudaStreamSynchronize(m->stream));
    m->l1 = variant | (m->P.colp16 ? 2 : 0);
    m->grid = merge_grid(m->cfg, m->num_tiles, m->sm_count, m->l1);
    m->pgrid = power_persistent_grid(kCfgF64, m->num_tiles, m->sm_count, m->l1);
    m->pgrid32 = power_persistent_grid(kCfgF32, m->num_tiles, m->sm_count, m->l1);
    m->pgridbf = power_persistent_grid(kCfgBF16, m->num_tiles, m->sm_count, m->l1);
    return PWMGPU_OK;
}

int pwmgpu_plan_info(const pwmgpu_matrix* m, int32_t* column_bytes, int32_t* gathers_bypass_l1) {
    if (!m) return fail(PWMGPU_ERR_INVALID, "null handle");
    if (!m->loaded) return fail(PWMGPU_ERR_STATE, "no matrix loaded");
    const bool merge = m->format == PWMGPU_FMT_MERGE;
    if (column_bytes) *column_bytes = merge && m->P.colp16 ? 2 : 4;
    if (gathers_bypass_l1) *gathers_bypass_l1 = merge && (m->l1 & 4) ? 1 : 0;
    return PWMGPU_OK;
}

}  // extern "C"

// ---- format autotuner (PWMGPU_FMT_AUTO) ------------------------------------
namespace pwmgpu {
namespace {

constexpr int kCohPartsDefault = 24;  // CO-H partitions per SM

struct TuneChoice {
    int fmt = PWMGPU_FMT_MERGE;
    int csb_var = 0;
    int merge_var = 0;
    int coh_pps = kCohPartsDefault;  // CO-H partitions per SM
};
using ClassKey = std::array<int32_t, 7>;
std::mutex g_tune_mu;
std::map<ClassKey, TuneChoice> g_tune_table;  // one entry per matrix class, process-wide

void class_key_of(const pwmgpu_matrix_stats& st, int sm_count, int32_t* key) {
    auto flog2 = [](double v) { return v > 0.0 ? (int32_t)std::floor(std::log2(v)) : -1; };
    const double cv_rows = st.rows_avg > 0.0 ? std::sqrt(std::max(st.rows_var, 0.0)) / st.rows_avg : 0.0;
    const double cv_blocks = st.block_avg > 0.0 ? std::sqrt(std::max(st.block_var, 0.0)) / st.block_avg : 0.0;
    key[0] = flog2((double)st.size);
    key[1] = st.rows_avg > 0.0 ? (int32_t)std::floor(2.0 * std::log2(st.rows_avg)) : -1;
    key[2] = flog2(1.0 + 8.0 * cv_rows);
    key[3] = flog2(1.0 + cv_blocks);
    key[4] = st.balanced;
    key[5] = flog2(1.0 + (double)st.max_row_nnz);
    key[6] = sm_count;
}

// ms per FP64 SpMV of the handle with format `fmt` (x = 0: the kernels'
// time does not depend on the values): two warm-ups, then 8 timed on the
// handle's stream.
int time_format(pwmgpu_matrix* m, int fmt, float* ms) {
    TRY(ensure_vectors(m));
    CU(cudaMemsetAsync(m->dx, 0, sizeof(double) * (size_t)std::max(m->M.nor, m->M.noc), m->stream));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CU(cudaEventCreate(&e0));
    cudaError_t e = cudaEventCreate(&e1);
    int rc = e == cudaSuccess ? PWMGPU_OK : fail(PWMGPU_ERR_CUDA, "cudaEventCreate: %s", cudaGetErrorString(e));
    const int saved = m->tuned_fmt;
    m->tuned_fmt = fmt;
    for (int r = 0; r < 10 && rc == PWMGPU_OK; ++r) {
        if (r == 2 && (e = cudaEventRecord(e0, m->stream)) != cudaSuccess) rc = fail(PWMGPU_ERR_CUDA, "event");
        if (rc == PWMGPU_OK) rc = spmv_f64(m, m->dx, m->dy);
    }
    m->tuned_fmt = saved;
    if (rc == PWMGPU_OK) e = cudaEventRecord(e1, m->stream);
    if (rc == PWMGPU_OK && e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (rc == PWMGPU_OK && e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    if (rc == PWMGPU_OK && e != cudaSuccess) rc = fail(PWMGPU_ERR_CUDA, "format timing: %s", cudaGetErrorString(e));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms /= 8.f;
    TRY(rc);
    return check_status(m);
}

// Build one of the CSB / CO-H formats beside the CRS arrays (still on the
// device); a CO-H candidate has coh_pps partitions (warps) per SM.
int build_candidate(pwmgpu_matrix* m, int fmt, int coh_pps = kCohPartsDefault) {
    const int saved_fmt = m->format, saved_parts = m->partitions;
    m->format = fmt;
    if (fmt == PWMGPU_FMT_COH) {
        m->release_coh();
        m->partitions = coh_pps * m->sm_count;
    }
    const int rc = build_format(m);
    m->format = saved_fmt;
    m->partitions = saved_parts;
    m->loaded = false;
    return rc;
}

}  // namespace

// Load-time variant tuner of a CSB or CO-H handle (both run the tile
// kernel): with enough work to measure (the merge tuner's threshold), time
// the four kernel variants and keep the fastest (pwmgpu_set_csb_variant
// overrides it).  4096^2 stencil: 4 elements per lane, 128 threads;
// irregular matrix: 256 threads.
int tune_csb(pwmgpu_matrix* m) {
    m->csb_var = 0;
    const MergeGeom g = merge_geometry(kCfgF64, 0);
    const long long tiles = ((long long)m->M.nor + m->M.nnz + g.wm - 1) / g.wm;
    if (m->M.nor == 0 || tiles < 8LL * g.occ * g.w * m->sm_count) return PWMGPU_OK;
    float ms[kCsbVariants];
    int best = 0;
    for (int v = 0; v < kCsbVariants; ++v) {
        m->csb_var = v;
        TRY(time_format(m, m->format, &ms[v]));
        if (ms[v] < 0.97f * ms[best]) best = v;  // another variant only for a clear (3 %) gain
    }
    m->csb_var = best;
    return PWMGPU_OK;
}

int build_auto(pwmgpu_matrix* m) {
    const auto t0 = std::chrono::steady_clock::now();
    pwmgpu_tuning T{};
    T.format = PWMGPU_FMT_MERGE;
    m->format = PWMGPU_FMT_MERGE;
    m->tuned_fmt = -1;
    m->csb_var = 0;
    // matrices below the merge tuner's threshold (and non-square ones: the
    // reference's CSB indexes blocks for square matrices) run merge, untimed
    const MergeGeom g = merge_geometry(kCfgF64, 0);
    const long long tiles = ((long long)m->M.nor + m->M.nnz + g.wm - 1) / g.wm;
    if (m->M.nor == 0 || m->M.nnz == 0 || m->M.nor != m->M.noc || tiles < 8LL * g.occ * g.w * m->sm_count) {
        TRY(build_merge(m, true));
        T.merge_variant = m->l1;
        m->tuning = T;
        return PWMGPU_OK;
    }
    // class key from the statistics of the CRS arrays (still on the device)
    pwmgpu_matrix_stats st{};
    m->loaded = true;  // the statistics want a loaded handle
    int rc = pwmgpu_stats(m, &st);
    m->loaded = false;
    TRY(rc);
    ClassKey key{};
    class_key_of(st, m->sm_count, key.data());
    std::copy(key.begin(), key.end(), T.class_key);
    TuneChoice choice;
    bool hit = false;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_table.find(key);
        if (it != g_tune_table.end()) {
            choice = it->second;
            hit = true;
        }
    }
    if (hit) {
        T.cache_hit = 1;
        if (choice.fmt != PWMGPU_FMT_MERGE) TRY(build_candidate(m, choice.fmt, choice.coh_pps));
        TRY(build_merge(m, false));
        apply_merge_variant(m, choice.merge_var | (m->P.colp16 ? 2 : 0));
    } else {
        T.timed = 1;
        // CSB: all four kernel variants
        TRY(build_candidate(m, PWMGPU_FMT_CSB));
        m->loaded = true;
        for (int v = 0; v < kCsbVariants; ++v) {
            m->csb_var = v;
            TRY(time_format(m, PWMGPU_FMT_CSB, &T.csb_ms[v]));
        }
        m->loaded = false;
        // CO-H (the default partition count): the tile kernel's four variants
        // on its tiles
        int coh_best = 0;
        TRY(build_candidate(m, PWMGPU_FMT_COH, kCohPartsDefault));
        m->loaded = true;
        for (int v = 0; v < kCsbVariants; ++v) {
            m->csb_var = v;
            TRY(time_format(m, PWMGPU_FMT_COH, &T.coh_ms[v]));
            if (T.coh_ms[v] < T.coh_ms[coh_best]) coh_best = v;
        }
        m->loaded = false;
        // merge: plan and launch-variant tuner, then the same timing
        TRY(build_merge(m, true));
        TRY(time_format(m, PWMGPU_FMT_MERGE, &T.merge_ms));
        choice.merge_var = m->l1 & ~2;  // the column width is the plan's, not a choice
        float best = T.merge_ms;
        for (int v = 0; v < kCsbVariants; ++v)
            if (T.csb_ms[v] < best) {
                best = T.csb_ms[v];
                choice.fmt = PWMGPU_FMT_CSB;
                choice.csb_var = v;
            }
        if (T.coh_ms[coh_best] < best) {
            best = T.coh_ms[coh_best];
            choice.fmt = PWMGPU_FMT_COH;
            choice.csb_var = coh_best;
        }
        choice.coh_pps = kCohPartsDefault;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_table[key] = choice;
    }
    // keep the chosen format's arrays (and the merge plan); drop the others
    if (choice.fmt != PWMGPU_FMT_CSB) m->release_csb();
    if (choice.fmt != PWMGPU_FMT_COH) m->release_coh();
    m->tuned_fmt = choice.fmt;
    m->csb_var = choice.fmt == PWMGPU_FMT_MERGE ? 0 : choice.csb_var;
    T.format = choice.fmt;
    T.coh_partitions = choice.fmt == PWMGPU_FMT_COH ? choice.coh_pps * m->sm_count : 0;
    T.csb_variant = m->csb_var;
    T.merge_variant = m->l1;
    T.tune_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    m->tuning = T;
    m->loaded = true;
    return PWMGPU_OK;
}

}  // namespace pwmgpu

extern "C" {

int pwmgpu_tuning_info(const pwmgpu_matrix* m, pwmgpu_tuning* out) {
    if (!m || !out) return pwmgpu::fail(PWMGPU_ERR_INVALID, "null handle or output");
    if (!m->loaded) return pwmgpu::fail(PWMGPU_ERR_STATE, "no matrix loaded");
    if (!m->auto_fmt) return pwmgpu::fail(PWMGPU_ERR_STATE, "not a PWMGPU_FMT_AUTO handle");
    *out = m->tuning;
    return PWMGPU_OK;
}

int pwmgpu_class_key(const pwmgpu_matrix_stats* st, int32_t sm_count, int32_t key[7]) {
    if (!st || !key) return pwmgpu::fail(PWMGPU_ERR_INVALID, "null statistics or key");
    pwmgpu::class_key_of(*st, sm_count, key);
    return PWMGPU_OK;
}

int pwmgpu_tuner_reset(void) {
    std::lock_guard<std::mutex> lk(pwmgpu::g_tune_mu);
    pwmgpu::g_tune_table.clear();
    return PWMGPU_OK;
}

int pwmgpu_tuner_size(void) {
    std::lock_guard<std::mutex> lk(pwmgpu::g_tune_mu);
    return (int)pwmgpu::g_tune_table.size();
}

int pwmgpu_tuner_record(const int32_t key[7], int32_t format, int32_t csb_variant, int32_t merge_variant,
                        int32_t coh_parts_per_sm) {
    if (!key) return pwmgpu::fail(PWMGPU_ERR_INVALID, "null key");
    if (format != PWMGPU_FMT_MERGE && format != PWMGPU_FMT_CSB && format != PWMGPU_FMT_COH)
        return pwmgpu::fail(PWMGPU_ERR_INVALID, "format must be merge, CSB or CO-H");
    if (csb_variant < 0 || csb_variant >= pwmgpu::kCsbVariants)
        return pwmgpu::fail(PWMGPU_ERR_INVALID, "CSB variant 0..3");
    if (merge_variant != 0 && merge_variant != 1 && merge_variant != 4 && merge_variant != 5)
        return pwmgpu::fail(PWMGPU_ERR_INVALID, "merge variant 0, 1, 4 or 5");
    if (coh_parts_per_sm < 0 || coh_parts_per_sm > 64)
        return pwmgpu::fail(PWMGPU_ERR_INVALID, "CO-H partitions per SM 0..64");
    pwmgpu::ClassKey k{};
    std::copy(key, key + 7, k.begin());
    pwmgpu::TuneChoice c;
    c.fmt = format;
    c.csb_var = format == PWMGPU_FMT_MERGE ? 0 : csb_variant;
    c.merge_var = merge_variant;
    c.coh_pps = coh_parts_per_sm ? coh_parts_per_sm : pwmgpu::kCohPartsDefault;
    std::lock_guard<std::mutex> lk(pwmgpu::g_tune_mu);
    pwmgpu::g_tune_table[k] = c;
    return PWMGPU_OK;
}

int pwmgpu_tuner_entries(int32_t max, int32_t* keys, int32_t* choices) {
    if (max < 0 || (max > 0 && (!keys || !choices)))
        return -pwmgpu::fail(PWMGPU_ERR_INVALID, "null output arrays or negative count");
    std::lock_guard<std::mutex> lk(pwmgpu::g_tune_mu);
    int n = 0;
    for (const auto& kv : pwmgpu::g_tune_table) {
        if (n >= max) break;
        std::copy(kv.first.begin(), kv.first.end(), keys + 7 * (size_t)n);
        choices[4 * (size_t)n] = kv.second.fmt;
        choices[4 * (size_t)n + 1] = kv.second.csb_var;
        choices[4 * (size_t)n + 2] = kv.second.merge_var;
        choices[4 * (size_t)n + 3] = kv.second.coh_pps;
        ++n;
    }
    return n;
}

int pwmgpu_get_csb_variant(const pwmgpu_matrix* m, int32_t* variant) {
    if (!m || !variant) return pwmgpu::fail(PWMGPU_ERR_INVALID, "null handle or output");
    if (m->format != PWMGPU_FMT_CSB && m->format != PWMGPU_FMT_COH)
        return pwmgpu::fail(PWMGPU_ERR_STATE, "not a CSB or CO-H handle");
    *variant = m->csb_var;
    return PWMGPU_OK;
}

int pwmgpu_set_csb_variant(pwmgpu_matrix* m, int32_t variant) {
    if (!m) return pwmgpu::fail(PWMGPU_ERR_INVALID, "null handle");
    if (variant < 0 || variant >= pwmgpu::kCsbVariants) return pwmgpu::fail(PWMGPU_ERR_INVALID, "CSB variant 0..3");
    if (m->format != PWMGPU_FMT_CSB && m->format != PWMGPU_FMT_COH)
        return pwmgpu::fail(PWMGPU_ERR_STATE, "not a CSB or CO-H handle");
    m->csb_var = variant;
    return PWMGPU_OK;
}

}  // extern "C"
