// internal.h -- declarations shared by the host side (pwmgpu.cpp) and the
// kernel translation units.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "pwmgpu.h"

namespace pwmgpu {

// Device CRS view (row_start[nor+1], col[nnz], val[nnz]; each array padded by
// kArrayPad elements past its end).
struct DevMatrix {
    int32_t nor = 0, noc = 0;
    long long nnz = 0;
    int32_t* row_start = nullptr;
    int32_t* col = nullptr;
    double* val = nullptr;
};

// Merge kernel modes (merge.cuh MergeMode): plain SpMV; a power step with its
// squared norm; a power step tracking only the largest magnitude key.
enum { kModeSpmv = 0, kModePower = 1, kModeScale = 2 };

// Largest clock64 interval any spin-wait may take before it reports
// PWMGPU_ERR_TIMEOUT (about 2 s at the 2.07 GHz maximum SM clock).
constexpr long long kWaitCycles = 4000000000LL;

// merge.cu
// Items per lane of a merge-path sub-tile (a sub-tile is 32 * kMliIpt merge
// items, one warp); the lane-interleaved storage is laid out for this size.
constexpr int kMliIpt = 12;

// Merge-path kernel configurations (value / vector / accumulation types).
enum { kCfgF64 = 0, kCfgF32 = 2, kCfgBF16 = 3 };
struct MergeGeom {
    int wm;    // merge items per sub-tile (one warp)
    int w;     // warps per CTA
    int smem;  // dynamic shared memory per CTA
    int occ;   // resident CTAs per SM
    int nt;    // threads per CTA
};

// Per-matrix plan of the merge-path kernel: sub-tile boundaries, metadata,
// row-end masks and the lane-interleaved column / FP64 value arrays.
// Device frees.  cudaFree waits for all work on the device, so a build that
// runs beside other kernels (the serving loop builds admitted matrices while
// its round runs) would wait for them at every free.  defer_frees(&list)
// makes this thread's dev_free calls append to `list` instead, until
// defer_frees(nullptr); free_deferred(list) then frees them (after the caller
// has synchronised the work that used them).
void dev_free(void* p);
void defer_frees(std::vector<void*>* list);
void free_deferred(std::vector<void*>& list);

struct MliPlan {
    int nsub = 0;
    int2* subc = nullptr;       // nsub + 1 merge coordinates (row, nonzero)
    int4* rec = nullptr;        // 2 x nsub: {rw0, kw0, rw1, kw1}, {first row, flags, base, nkw}
    uint16_t* masks = nullptr;  // nsub x 32 row-end masks
    int32_t* colp = nullptr;    // lane-interleaved column indices
    double* valp = nullptr;     // lane-interleaved FP64 values
    uint16_t* colp16 = nullptr; // or null: the same columns as offsets from the sub-tile's base (rec0.w)
    // fix-up runs with a carry to add: {first sub-tile t, completing sub-tile n, row r, 0},
    // ordered by t; run_pre[t] = runs whose first sub-tile is < t (nsub + 1 entries)
    int4* runs = nullptr;
    int* run_pre = nullptr;
    int nruns = 0;
};
long long mli_storage_elems(long long nnz, long long nsub);

// sell.cu: SELL-32 copy of a matrix for the FP32 / BF16 iterations (slices
// of 32 rows, column-major in the slice, 16-bit column offsets from
// 32 s - 32768, padding skipped); built when every column fits and the
// padding is within a quarter of the nonzeros.
struct SellPlan {
    int state = 0;  // 0: not built, 1: built, -1: the matrix does not fit the format
    int nslices = 0;
    long long stored = 0;        // padded elements
    int32_t* soff = nullptr;     // nslices + 1 element offsets
    uint16_t* col16 = nullptr;   // column - (32 s - 32768)
    float* val32 = nullptr;      // FP32 values (built on first use)
    void* valbf = nullptr;       // BF16 values (built on first use)
    double* npart = nullptr;     // per-CTA shares of ||y||^2
    void release();
};
int sell_grid(int nslices, int sm_count);
// Fill the launch-geometry caches (occupancies) of the merge and SELL kernels
// once, so that matrix builds on several host threads only read them.
void warm_launch_caches(int sm_count);
// Build the slices (first call) and the value array of the requested type
// from CRS arrays; 0 = built, 1 = the matrix does not fit (state -1), 2 = a
// CUDA error or no memory (state 0).
int sell_build(SellPlan& S, const int32_t* row_start, const int32_t* col, const double* val, int nor, long long nnz,
               bool bf16, int sm_count, cudaStream_t st);
// y = 2^e A x (e from nsq_in, or 0 when null) on FP32 vectors; with nsq_out,
// also *nsq_out = ||y||^2 (deterministic; counter zero between launches).
cudaError_t launch_sell_spmv(const SellPlan& S, bool bf16, const int32_t* row_start, int nor, const float* x, float* y,
                             const double* nsq_in, double* nsq_out, unsigned int* counter, int sm_count,
                             cudaStream_t st);

// l1: launch variant of the merge kernels.  Bit 0: 0 = most resident CTAs,
// 1 = a smaller shared-memory carveout, more L1 for irregular gathers; bit 1:
// stream the plan's 16-bit column offsets (set only when the plan has them);
// bit 2: the FP64 SpMV's x gathers bypass L1 (the persistent and the
// low-precision kernels ignore it).
MergeGeom merge_geometry(int cfg, int l1 = 0);
int merge_grid(int cfg, int nsub, int sm_count, int l1 = 0);
int fixup_grid(int num_tiles, int sm_count);
int dot_grid(long long n, int sm_count);
// Persistent power-method kernel (cooperative launch): grid size for a
// matrix with nsub sub-tiles, 0 if the kernel cannot be made co-resident.
int power_persistent_grid(int cfg, int nsub, int sm_count, int l1 = 0);
// Iterations k0 .. k0+nk-1 on X/Y (ping-pong; v_k in X for even k), nsq[k]
// = ||v_k||^2 (nsq[k0] read when k0 > 0), result (5 doubles, or null):
// {lambda, residual^2, ||v_k||^2, v_k.v_{k+1}, e_k} of the last iteration.
// partials: 2 doubles per CTA; barrier: 2 words (zeroed here).
// wait: the grid barrier's budget (clock64 cycles) before it records
// PWMGPU_ERR_TIMEOUT, and extra arrivals it waits for beyond the grid (0;
// pwmgpu_test_grid_wait sets 1 to make every barrier run out of budget).
struct GridWait {
    long long cycles;
    unsigned int extra;
};
// mxk: k0 + nk + 1 zeroed words (or null): iterations before the last two
// of the launch track only the iterate's largest magnitude key (mxk[k+1]) for
// the rescale instead of summing ||v||^2 (nsq[k+1] is then not written).
cudaError_t launch_power_persistent(int cfg, const DevMatrix& M, const void* valp, const MliPlan& P, int grid,
                                    void* X, void* Y, void* carries, int k0, int nk, double* nsq, double* result,
                                    double* partials, unsigned int* barrier, int* status, cudaStream_t st,
                                    int l1, GridWait wait, unsigned int* mxk = nullptr);
cudaError_t launch_merge_partition(const int32_t* row_start, int nor, long long nnz, long long ipt, int parts,
                                   int2* out, cudaStream_t st);
cudaError_t launch_mli_plan(const int32_t* row_start, const int32_t* col, const double* val, const MliPlan& P,
                            int sm_count, cudaStream_t st);
cudaError_t launch_mli_convert(const MliPlan& P, int cfg, void* out, int sm_count, cudaStream_t st);
// the separate-kernel form of a solve chunk: FP32 norm pass and the result pass
cudaError_t launch_power_norm_f32(const float* y, const float* x, int n, double* partials, unsigned int* counter,
                                  double* out, int grid, cudaStream_t st);
cudaError_t launch_solve_result(bool f32, const void* in, const void* out, int n, const double* nsq_k,
                                const double* nd, double* nsq_next, double* result, double* partials,
                                unsigned int* counter, int grid, cudaStream_t st);
// fix-up run descriptors of a plan (P.runs, P.run_pre, P.nruns; scratch: 2 *
// (nsub + 1) ints and nsub int4) and the fix-up over descriptors [k0, k1)
int build_fix_runs(MliPlan& P, const int32_t* row_start, int nor, int sm_count, cudaStream_t st);
cudaError_t launch_fix_runs_f64(int mode, const MliPlan& P, int k0, int k1, double* y, const double* carries,
                                const double* nsq_in, cudaStream_t st);
cudaError_t launch_fix_runs_f32(int mode, const MliPlan& P, int k0, int k1, float* y, const float* carries,
                                const double* nsq_in, cudaStream_t st);
// ||y||^2 of a power step inside its kernels: the MODE_POWER SpMV launched
// with `npart` writes one share per CTA (spmv_grid of them), this fix-up over
// all runs adds one per CTA after them and its last CTA writes the ordered
// total to *nsq_out.  npart holds power_norm_parts(P, spmv_grid) doubles;
// counter is zero between launches.
int power_norm_parts(const MliPlan& P, int spmv_grid);
// mx_in (optional): the step's rescale from its input's largest magnitude key
// instead of nsq_in.
cudaError_t launch_fix_runs_norm(bool f32, const MliPlan& P, void* y, const void* carries, const double* nsq_in,
                                 double* npart, int spmv_grid, unsigned int* counter, double* nsq_out,
                                 cudaStream_t st, const unsigned int* mx_in = nullptr);
// The fix-up of a MODE_SCALE step: carries times 2^e (e from *mx_in, else
// from *nsq_in, else 0 -- the same source as the step's SpMV), and atomicMax
// of the fixed rows' magnitude keys into *mx_out.
cudaError_t launch_fix_runs_scale(bool f32, const MliPlan& P, void* y, const void* carries, const double* nsq_in,
                                  const unsigned int* mx_in, unsigned int* mx_out, cudaStream_t st);
cudaError_t launch_mli_colspan(const MliPlan& P, int* cbase, int* flag, int sm_count, cudaStream_t st);
cudaError_t launch_mli_col16(const MliPlan& P, const int* cbase, int sm_count, cudaStream_t st);
cudaError_t launch_mli_unpermute(const MliPlan& P, int32_t* col, double* val, int sm_count, cudaStream_t st);
// mode kModeScale: mx_in (or nsq_in, or neither: e = 0) sets the rescale,
// the stored rows' magnitude keys go to atomicMax(*mx_out); kModePower may
// take its rescale from mx_in as well.
cudaError_t launch_merge_spmv(int cfg, int mode, const DevMatrix& M, const void* valp, const MliPlan& P, int grid,
                              const void* x, void* y, void* carries, const double* nsq_in, int* status,
                              cudaStream_t st, int l1 = 0, double* npart = nullptr,
                              const unsigned int* mx_in = nullptr, unsigned int* mx_out = nullptr);
// Carries of the merge SpMV into y (MODE_POWER: times the rescale factor of
// nsq_in).
cudaError_t launch_merge_fixup_f64(int mode, const DevMatrix& M, const int2* tiles, int num_tiles, double* y,
                                   const double* carries, const double* nsq_in, int fix_grid, cudaStream_t st);
cudaError_t launch_merge_fixup_f32(int mode, const DevMatrix& M, const int2* tiles, int num_tiles, float* y,
                                   const float* carries, const double* nsq_in, int fix_grid, cudaStream_t st);
// out[0] = ||y||^2 and, when x is given, out[1] = x . y (deterministic;
// partials: 2 per CTA of `grid`; counter zero between launches).
cudaError_t launch_power_norm_f64(const double* y, const double* x, int n, double* partials, unsigned int* counter,
                                  double* out, int grid, cudaStream_t st);
cudaError_t launch_power_finalize_f64(double* last, const double* nsq_last, double* prev, const double* nsq_prev,
                                      int n, int sm_count, cudaStream_t st);
// Rows [first_row, last_row) of the Poisson matrix (last_row < 0: all m*n).
cudaError_t launch_poisson_crs(int m, int n, int32_t* row_start, int32_t* col, double* val, int sm_count,
                               cudaStream_t st, int first_row = 0, int last_row = -1);
long long poisson_rows_nnz(int m, int n, int first_row, int last_row);
cudaError_t launch_dot2_f64(const double* a, const double* b, int n, double* partials, unsigned int* counter,
                            double* out, int grid, cudaStream_t st);
cudaError_t launch_dot2_f32(const float* a, const float* b, int n, double* partials, unsigned int* counter,
                            double* out, int grid, cudaStream_t st);
cudaError_t launch_resid_f64(const double* a, double sa, const double* b, double sb, int n, double* partials,
                             unsigned int* counter, double* out, int grid, cudaStream_t st);
cudaError_t launch_resid_f32(const float* a, double sa, const float* b, double sb, int n, double* partials,
                             unsigned int* counter, double* out, int grid, cudaStream_t st);
cudaError_t launch_convert_f64_f32(const double* s, float* d, long long n, int sm_count, cudaStream_t st);
cudaError_t launch_convert_f32_f64(const float* s, double* d, long long n, int sm_count, cudaStream_t st);
cudaError_t launch_convert_f64_bf16(const double* s, void* d, long long n, int sm_count, cudaStream_t st);
cudaError_t launch_bf16_exact(const double* v, long long n, int* flag, int sm_count, cudaStream_t st);

// gen.cu: seeded random sparse matrices and an in-place int32 inclusive scan
void random_length_table(int kind, double mean, double sigma, int max_len, std::vector<uint64_t>& thr);
cudaError_t launch_random_count(const uint64_t* thr, int max_len, int n, uint64_t seed, int band_permille,
                                int band_half, int32_t* row_start, unsigned long long* total, int sm_count,
                                cudaStream_t st);
cudaError_t launch_random_fill(const uint64_t* thr, int max_len, int n, uint64_t seed, int band_permille,
                               int band_half, const int32_t* row_start, int32_t* col, double* val, int sm_count,
                               cudaStream_t st);
long long scan_scratch_elems(long long n);
cudaError_t launch_inclusive_scan(int32_t* a, long long n, int32_t* scratch, cudaStream_t st);

// triplet.cu: triplet -> CRS on the device (stable LSD radix sort by (row, col))
struct TripletScan {
    unsigned long long bad;   // first entry with a row or column out of range (~0 when none)
    unsigned int unsorted_rc; // input not sorted by (row, col)
    unsigned int unsorted_c;  // input not sorted by column
};
cudaError_t launch_triplet_scan(const int32_t* rows, const int32_t* cols, long long nnz, int32_t nor, int32_t noc,
                                int32_t* cnt, TripletScan* flags, int sm_count, cudaStream_t st);
long long triplet_sort_table_elems(long long nnz);
int triplet_sort_passes(int32_t nor, int32_t noc, bool col_passes);
cudaError_t launch_triplet_sort(const int32_t* rows, const int32_t* cols, long long nnz, int32_t nor, int32_t noc,
                                bool col_passes, unsigned long long* keys_a, int32_t* src_a,
                                unsigned long long* keys_b, int32_t* src_b, int32_t* tab, int32_t* scan_scratch,
                                unsigned long long** keys_sorted, int32_t** src_sorted, int sm_count,
                                cudaStream_t st);
cudaError_t launch_triplet_gather(const unsigned long long* keys, const int32_t* src, const double* vals,
                                  long long nnz, int32_t* col, double* val, int32_t* rows_out, int sm_count,
                                  cudaStream_t st);

// stats.cu: Util_Scripts/calc_stats.cpp figures on the device
struct StatsDev {
    double rows_var, block_avg, block_var;
    int max_row_nnz, balanced;
};
int stats_row_ctas(int n);
cudaError_t launch_matrix_stats(const int32_t* row_start, const int32_t* col, int n, double avg, int bits, int nbw,
                                unsigned int* blocks, long long* brow, double* row_partials, double* blk_partials,
                                StatsDev* out, cudaStream_t st);

// hostcopy.cu: SM-driven copy between pageable host memory and the device
// (only where the device reaches pageable memory)
cudaError_t launch_host_copy(const double* src, double* dst, long long n, cudaStream_t st);

// batch.cu: one round (`steps` power steps + the residual pass) of every slot
// of a class table; seeded uniform start vectors
struct BatchTable;
void batch_prepare(int sm_count);
// sell: the class's slots are SELL-32 copies (FP32 / BF16 values).
cudaError_t launch_batch_round(int cfg, const BatchTable* T, int steps, int sm_count, cudaStream_t st,
                               bool sell = false);
cudaError_t launch_tile_slots(const BatchTable* T, int nslots, cudaStream_t st);
cudaError_t launch_fill_uniform(double* x, int n, uint64_t seed, int sm_count, cudaStream_t st);

// The tile kernel (k_csb_spmv) runs both blocked formats: rows in windows of
// S, each window's tiles ("units", elements of one block in an S-column
// window) from a list; tiles of at least kTileDenseUnit elements stage their
// x window in shared memory, the rest are merged into one gathered unit.
constexpr int kTileDenseUnit = 256;

// csb.cu: CSB (CSB.hpp) parameters, host build and SpMV
void csb_params(int nor, int noc, int* beta, int* bits);
int csb_window(int nor, int beta, int sm_count);
int csb_build_host(int nor, int noc, long long nnz, const int32_t* row_start, const int32_t* col, const double* val,
                   int beta, int bits, std::vector<uint32_t>& ind, std::vector<double>& data,
                   std::vector<int32_t>& blk_ptr, int S, std::vector<int>& win_ptr, std::vector<int>& unit_data);
bool csb_kernel_layout(const std::vector<uint32_t>& ind, const std::vector<double>& data, int S,
                       std::vector<int>& win_ptr, std::vector<int>& units, std::vector<uint32_t>& kind,
                       std::vector<double>& kdata, std::vector<int32_t>& kcol);
cudaError_t launch_csb_spmv(const uint32_t* ind, const int32_t* kcol, const double* data, const int* win_ptr, const int* units, int nwin,
                            int S, int nor, int noc, const double* x, double* y, const double* nsq_in, int* status,
                            int sm_count, cudaStream_t st, int variant = 0);
constexpr int kCsbVariants = 4;

// coh.cu: CO-H (BlockCOH.hpp) host build and SpMV
int coh_build_host(int nor, int noc, long long nnz, const int32_t* row_start, const int32_t* col, const double* val,
                   int threads, std::vector<int32_t>& part_info, std::vector<uint16_t>& row_jump,
                   std::vector<uint16_t>& col_jump, std::vector<double>& data, std::vector<int32_t>& block_nnz,
                   std::vector<int16_t>& row_jump_block, std::vector<int16_t>& col_jump_block,
                   std::vector<int>& parts, std::vector<int>& blocks);
// The CO-H matrix as tiles for the tile kernel: per window of S rows, the
// tiles of its rows' CO-H blocks -- partitions in row order, each
// partition's blocks in its Hilbert order, a block's tiles by column window
// -- with elements row-major inside a tile (columns ascending per row, as
// in the block's ICRS order).  Outputs as csb_build_host's (ind = local row
// << 16 | column - tile column, win_ptr: sparse tiles then dense ones).
// parts: 8 ints per partition as coh_build_host writes them.
void coh_tile_units(int nor, int noc, long long nnz, const int32_t* row_start, const int32_t* col, const double* val,
                    const std::vector<int>& parts, int S, std::vector<uint32_t>& ind, std::vector<double>& data,
                    std::vector<int>& win_ptr, std::vector<int>& unit_data);

// Pipelined host-array SpMV: chunk records (4 ints per chunk: first
// sub-tile, its first row, row-split flag, largest column read), and the
// SpMV / fix-up over sub-tile ranges.
cudaError_t launch_pipeline_plan(const int32_t* row_start, const MliPlan& P, int K, int* out, cudaStream_t st);
cudaError_t launch_merge_spmv_range(const DevMatrix& M, const MliPlan& P, int t0, int t1, int grid, const double* x,
                                    double* y, double* carries, int* status, cudaStream_t st, int l1);
cudaError_t launch_merge_fixup_range(const DevMatrix& M, const int2* tiles, int num_tiles, int f0, int f1, double* y,
                                     const double* carries, cudaStream_t st, int sm_count);

// Record the calling thread's last error message (pwmgpu_last_error).
void record_error(const char* msg);

// Poisson row start closed form (shared with the host checker of the
// device generator).
long long poisson_row_start_host(long long row, long long m, long long n);

}  // namespace pwmgpu
