/*
 * pwmgpu.h -- C ABI of the GB300 (sm_103a) SpMV / power-method library.
 *
 * This is the drop-in boundary for KobeBergmans/Thesis_SPMV's operator
 * interface pwm::SparseMatrix<T,int_type> (Matrix/SparseMatrix.hpp:13-68).
 * Each entry point names the reference interface it replaces.  All entry
 * points are extern "C", take plain pointers and sizes, return an int status
 * (PWMGPU_OK == 0) and never abort; pwmgpu_last_error() gives the message of
 * the calling thread's last failure.
 *
 * Index arrays are 32-bit.  The reference instantiates int_type as int,
 * unsigned int and uint32_t (Util/Constants.hpp:38, Tests/poisson.cpp:28,146);
 * all three have the same bits for sizes below 2^31, which the library
 * enforces (nor + nnz < 2^31).
 *
 * Host-array calls (pwmgpu_mv, pwmgpu_power, pwmgpu_solve) are synchronous:
 * results are final on return, as in the reference.  *_device calls take
 * device pointers and are asynchronous on the handle's stream.
 */
#ifndef PWMGPU_H
#define PWMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PWMGPU_OK 0
#define PWMGPU_ERR_INVALID 1    /* bad argument: null pointer, bad size, index out of range */
#define PWMGPU_ERR_CUDA 2       /* a CUDA runtime call failed */
#define PWMGPU_ERR_NOMEM 3      /* device allocation failed */
#define PWMGPU_ERR_TIMEOUT 4    /* a bounded device-side wait gave up */
#define PWMGPU_ERR_STATE 5      /* no matrix loaded / call out of order */
#define PWMGPU_ERR_NOT_SQUARE 6 /* power method on a non-square matrix (CRS.hpp:119 asserts) */
#define PWMGPU_ERR_BUDGET 7     /* service admission refused: over the HBM budget */
#define PWMGPU_ERR_NUMERIC 8    /* zero or non-finite norm met by the power method */
#define PWMGPU_ERR_UNSUPPORTED 9

/* ---- storage formats (the reference's method numbers 8, 9, 10 in
 *      Util/DriverUtil.hpp:67-74 selectType) ---- */
#define PWMGPU_FMT_MERGE 0 /* CRS, merge-path SpMV (SOA_Implementations/CRS_Merge.hpp) */
#define PWMGPU_FMT_CSB 1   /* compressed sparse blocks (SOA_Implementations/CSB.hpp) */
#define PWMGPU_FMT_COH 2   /* row-distributed Hilbert block CO-H (SOA_Implementations/BlockCOH.hpp) */
/* Format autotuner (no counterpart in the reference, whose drivers pick the
 * method by number): the handle keeps the merge-path plan (solves, FP32 and
 * host-array paths) and runs its FP64 mv / powerIteration with whichever of
 * merge, CSB or CO-H, and which kernel variant, the tuner found fastest for
 * the matrix's class (pwmgpu_tuning_info). */
#define PWMGPU_FMT_AUTO 3

/* ---- precision of a power solve ---- */
#define PWMGPU_PREC_F64 0   /* FP64 values, vectors and accumulation */
#define PWMGPU_PREC_F32 1   /* FP32 values and vectors, FP32 accumulation, FP64 reductions */
#define PWMGPU_PREC_MIXED 2 /* FP32 (or exact BF16) bulk phase, then FP64 refinement */

typedef struct pwmgpu_matrix pwmgpu_matrix;

/* Message of the calling thread's last failing call ("" if none). */
const char* pwmgpu_last_error(void);

/* Device facts for the current device. */
int pwmgpu_device_info(int* sm_count, size_t* free_bytes, size_t* total_bytes);

/* Replaces the reference constructors `CRS_Merge(int threads)`,
 * `CSB(int threads)`, `BlockCOH(int threads)` (SparseMatrix.hpp:30).
 * `partitions` is the reference's thread count where the format's layout
 * depends on it (CO-H row partitions, BlockCOH.hpp:325-355); the GPU kernels
 * do not depend on it otherwise.  The handle owns a CUDA stream. */
int pwmgpu_create(int format, int partitions, pwmgpu_matrix** out);
/* Replaces the virtual destructor (SparseMatrix.hpp:33). */
int pwmgpu_destroy(pwmgpu_matrix* m);
/* Use `stream` (a cudaStream_t, may be NULL for the legacy stream) for all
 * later work of this handle instead of its own stream. */
int pwmgpu_set_stream(pwmgpu_matrix* m, void* stream);

/* Seeded random square matrix generated on the device (no counterpart in
 * the reference: the benchmarks' irregular and batch workloads).  Row
 * lengths: PWMGPU_RAND_LOGNORMAL -- clip(round(exp(mu + sigma Z)), 1,
 * max_len) with mu = ln(mean_len) - sigma^2/2; PWMGPU_RAND_POISSON --
 * Poisson(mean_len) clipped to max_len.  band_permille / 1000 of a row's
 * columns fall within +-band_half of the diagonal, the rest anywhere in
 * [0, n); each part is stratified (sorted, no duplicates) and a column drawn
 * by both is kept once.  Values in (0, 1].  Every array is a deterministic
 * function of the arguments (integer hashing), reproduced bit for bit by the
 * host restatement in the test oracle. */
#define PWMGPU_RAND_LOGNORMAL 0
#define PWMGPU_RAND_POISSON 1
int pwmgpu_generate_random(pwmgpu_matrix* m, int32_t n, uint64_t seed, int length_dist, double mean_len,
                           double sigma, int32_t max_len, int32_t band_permille, int32_t band_half);

/* Replaces generatePoissonMatrix(m, n, partitions) (SparseMatrix.hpp:41,
 * CRS.hpp:60-74, CSB.hpp:576-582, BlockCOH.hpp:464-470).  The merge format
 * writes the CRS arrays on the device in Util/Poisson.hpp:32-83 order. */
int pwmgpu_generate_poisson(pwmgpu_matrix* m, int32_t mx, int32_t ny);
/* Upload a host CRS matrix (rows sorted, columns ascending within a row). */
int pwmgpu_load_csr(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, const int32_t* row_start,
                    const int32_t* col_ind, const double* vals);
/* Replaces loadFromTriplets(input, partitions) (SparseMatrix.hpp:48).  Like
 * the reference (Util/TripletToCRS.hpp:139-142) it sorts the caller's
 * triplet arrays in place (by row, then column; entries with equal
 * coordinates keep their input order).  The sort runs on the device. */
int pwmgpu_load_triplets(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, int32_t* rows, int32_t* cols,
                         double* vals);
/* The same CRS from triplet arrays already on the device (d_rows[nnz],
 * d_cols[nnz], d_vals[nnz]), which are left unchanged; synchronous. */
int pwmgpu_load_triplets_device(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, const int32_t* d_rows,
                                const int32_t* d_cols, const double* d_vals);
int pwmgpu_dims(const pwmgpu_matrix* m, int32_t* nor, int32_t* noc, int64_t* nnz);
/* Copy the device CRS arrays back (row_start[nor+1], col_ind[nnz], vals[nnz]);
 * the reference's protected row_start / col_ind / data_arr (CRS.hpp:30-37). */
int pwmgpu_get_csr(pwmgpu_matrix* m, int32_t* row_start, int32_t* col_ind, double* vals);

/* Matrix statistics of Util_Scripts/calc_stats.cpp:45-98, computed on the
 * device from the loaded matrix (any format).  Blocks are squares of side
 * 2^block_bits, block_bits = min(16, 3 + ceil(log2 sqrt(nor))); the block
 * figures cover the nb_blocks x nb_blocks whole blocks (columns beyond them
 * are not counted).  Counts are exact; rows_var, block_avg and block_var are
 * summed in a fixed parallel order (deterministic; the script sums
 * sequentially), balanced uses the script's own order for the average block
 * row. */
typedef struct {
    int64_t size;        /* nor */
    int64_t nnz;
    double rows_avg;     /* nonzeros per row: mean */
    double rows_var;     /* nonzeros per row: population variance */
    double block_avg;    /* nonzeros per whole block: mean */
    double block_var;    /* nonzeros per whole block: population variance */
    int32_t balanced;    /* 1: no block row holds more than twice the average block row */
    int32_t block_bits;
    int32_t nb_blocks;   /* whole blocks per side */
    int32_t max_row_nnz; /* longest row */
} pwmgpu_matrix_stats;
int pwmgpu_stats(pwmgpu_matrix* m, pwmgpu_matrix_stats* out);

/* ---- format autotuner (PWMGPU_FMT_AUTO handles; no counterpart in the
 *      reference) ----
 * A matrix class is a key of the statistics above (Util_Scripts/
 * calc_stats.cpp:45-98 features) and the SM count: floor(log2 nor),
 * floor(2 log2 rows_avg), floor(log2(1 + 8 cv_rows)) with cv_rows =
 * sqrt(rows_var) / rows_avg, floor(log2(1 + cv_blocks)) with cv_blocks =
 * sqrt(block_var) / block_avg, balanced, floor(log2(1 + max_row_nnz)),
 * sm_count.  The first matrix of a class loaded into an AUTO handle times
 * every candidate -- the merge kernels' 4 launch variants (shared-memory /
 * L1 carveout x gathers through or around L1), CSB with 4 or 8 elements
 * per lane and 128 or 256 threads per CTA, and CO-H with a warp per
 * partition and 8, 16, 24 or 32 partitions per SM -- on a few SpMVs each
 * and records the fastest in a process-wide table; later matrices of the
 * class take the recorded choice without timing.  Matrices too small to time
 * (the merge tuner's threshold) run merge. */
typedef struct {
    int32_t format;          /* PWMGPU_FMT_MERGE / _CSB / _COH: the FP64 SpMV in use */
    int32_t csb_variant;     /* tile kernel variant of a CSB or CO-H choice: bit 0 = 8 elements per lane,
                                bit 1 = 256 threads */
    int32_t merge_variant;   /* merge launch variant (pwmgpu_launch_config) */
    int32_t cache_hit;       /* 1: taken from the class table without timing */
    int32_t timed;           /* 1: candidates were timed for this matrix */
    int32_t class_key[7];
    int32_t coh_partitions;  /* CO-H partitions when CO-H is the format */
    float merge_ms;          /* ms per SpMV of the best merge variant (0 if not timed) */
    float csb_ms[4];         /* per CSB variant */
    float coh_ms[4];         /* per tile kernel variant on the CO-H tiles (24 partitions per SM) */
    double tune_seconds;     /* wall time of the tuning (builds and timings) */
} pwmgpu_tuning;
int pwmgpu_tuning_info(const pwmgpu_matrix* m, pwmgpu_tuning* out);
/* The class key of a statistics record for `sm_count` SMs (host only). */
int pwmgpu_class_key(const pwmgpu_matrix_stats* st, int32_t sm_count, int32_t key[7]);
/* Forget every recorded class choice (the next matrix of each class is
 * timed again). */
int pwmgpu_tuner_reset(void);
/* Number of classes recorded. */
int pwmgpu_tuner_size(void);
/* Record a class choice (to carry tunings between processes): format
 * PWMGPU_FMT_MERGE / _CSB / _COH, csb_variant 0..3 (the tile kernel variant
 * of CSB and CO-H), merge_variant one of
 * the merge launch variants (0, 1, 4, 5), coh_parts_per_sm 1..64 (CO-H
 * partitions per SM; 0: 24). */
int pwmgpu_tuner_record(const int32_t key[7], int32_t format, int32_t csb_variant, int32_t merge_variant,
                        int32_t coh_parts_per_sm);
/* Copy up to `max` recorded entries: keys[7 i ..], choices[4 i ..] =
 * {format, csb_variant, merge_variant, coh_parts_per_sm}; returns the number
 * copied (or a negative status). */
int pwmgpu_tuner_entries(int32_t max, int32_t* keys, int32_t* choices);
/* Tile kernel variant of a PWMGPU_FMT_CSB or PWMGPU_FMT_COH handle (both
 * formats run as tiles of one kernel; 0..3, as csb_variant above).  Loading
 * a matrix large enough to time (the merge tuner's threshold) picks the
 * fastest of the four; smaller ones get 0. */
int pwmgpu_set_csb_variant(pwmgpu_matrix* m, int32_t variant);
int pwmgpu_get_csb_variant(const pwmgpu_matrix* m, int32_t* variant);

/* Replaces mv(x, y) (SparseMatrix.hpp:57, CRS.hpp:99-109): y = A x with
 * caller-owned host arrays x[noc], y[nor]; synchronous. */
int pwmgpu_mv(pwmgpu_matrix* m, const double* x, double* y);
/* y = A x with device arrays (x[noc], y[nor] must not overlap);
 * asynchronous on the handle's stream. */
int pwmgpu_mv_device(pwmgpu_matrix* m, const double* dx, double* dy);
/* FP32 SpMV with device arrays: values converted to FP32 once, FP32
 * accumulation. */
int pwmgpu_mv_device_f32(pwmgpu_matrix* m, const float* dx, float* dy);

/* Replaces powerIteration(x, y, it) (SparseMatrix.hpp:66, CRS.hpp:118-130):
 * `it` times y = A x, y /= ||y||, roles swapped; the result is in x when `it`
 * is even and in y when it is odd, the other array holds the previous
 * iterate (the untouched input for it == 1), as in the reference.  Host
 * arrays of length nor; synchronous.  FP64. */
int pwmgpu_power(pwmgpu_matrix* m, double* x, double* y, int32_t it);
/* Same on device arrays; the kernel sequence is asynchronous. */
int pwmgpu_power_device(pwmgpu_matrix* m, double* dx, double* dy, int32_t it);

/* How pwmgpu_power / pwmgpu_power_device run the iterations:
 * FUSED uses one persistent cooperative kernel for all iterations (SpMV pass,
 * grid barrier, fix-up pass, grid barrier per iteration, the norms of the
 * last two iterations folded in; fails with PWMGPU_ERR_UNSUPPORTED where it
 * cannot be co-resident); MULTI launches the SpMV and fix-up kernels per
 * iteration with programmatic dependent launch; AUTO (default) takes MULTI,
 * which measured faster at every size on GB300 (256^2 to 4096^2 Poisson
 * grids, the 4M-row irregular matrix).  Results are equal within the power
 * method's tolerance. */
#define PWMGPU_POWER_AUTO 0
#define PWMGPU_POWER_FUSED 1
#define PWMGPU_POWER_MULTI 2
int pwmgpu_set_power_mode(pwmgpu_matrix* m, int mode);

/* Failure-path testing hook (not in the reference): the grid barriers of the
 * persistent power kernel wait at most `cycles` clock64 cycles (the default is
 * about 2 s, 4e9 cycles) and open once every CTA of the grid plus `extra`
 * more have arrived (extra = 0 normally).  With extra = 1 no barrier can
 * open: every CTA gives up after `cycles`, lets its copies in flight land,
 * records PWMGPU_ERR_TIMEOUT and returns, and the call reports that status;
 * the handle stays usable.  cycles in [1e4, 4e9], extra 0 or 1; pass
 * (0, 0) to restore the default. */
int pwmgpu_test_grid_wait(pwmgpu_matrix* m, int64_t cycles, int32_t extra);

/* Storage the FP32 / BF16 iterations (pwmgpu_solve's low-precision phase,
 * pwmgpu_mv_device_f32) stream (not in the reference).  AUTO (default): a
 * SELL-32 copy (slices of 32 rows, one row per lane, 16-bit column offsets;
 * built on first use) for matrices whose columns all lie within 32768 rows
 * of their row's slice and whose padding is within a quarter of the
 * nonzeros -- stencils and banded matrices -- the merge-path layout
 * otherwise; MERGE: always the merge-path layout.  The SELL kernel sums each
 * row left to right in CRS order; results differ from the merge layout's
 * only by rounding (within the FP32 row bound either way).  The power modes
 * above apply to the merge layout; POWER_FUSED keeps the low-precision
 * iterations on it too. */
#define PWMGPU_LOWFMT_AUTO 0
#define PWMGPU_LOWFMT_MERGE 1
int pwmgpu_set_low_format(pwmgpu_matrix* m, int fmt);

/* Power solve with an eigenvalue estimate, the eigen-residual and a stopping
 * test (not in the reference: an extension of the power method).  x (host, length nor)
 * holds the start vector on entry and the normalised eigenvector estimate on
 * return.  Iterates until ||A u - lambda u|| / |lambda| <= tol or max_it
 * iterations (max_it >= 2; tol = 0 runs exactly max_it SpMVs).  precision:
 * PWMGPU_PREC_*.  lambda is the Rayleigh quotient u^T A u of the returned u
 * (||u|| = 1), the normalised iterate after iterations - 1 SpMVs (the last
 * SpMV computes A u for lambda and the residual).  The residual test runs
 * after every chunk of iterations (FP64 reductions), the chunk executed as
 * pwmgpu_set_power_mode selects (the persistent kernel, or separate kernels);
 * MIXED runs FP32 (BF16 values where exact) until the residual reaches 2e-6,
 * stops falling below 1e-4 (the FP32 rounding floor), or only the FP64
 * reserve of min(64, max_it/4) iterations is left; then FP64 to tol. */
typedef struct {
    int32_t iterations;     /* total SpMVs performed */
    int32_t iterations_low; /* of which in the FP32/BF16 phase */
    int32_t converged;      /* 1 if the residual test was met */
    int32_t precision;      /* the PWMGPU_PREC_* used */
    double lambda;          /* Rayleigh quotient of the returned vector */
    double residual;        /* ||A u - lambda u|| / |lambda| of the returned vector */
} pwmgpu_solve_info;
int pwmgpu_solve(pwmgpu_matrix* m, double* x, int32_t max_it, double tol, int precision, pwmgpu_solve_info* info);

/* The merge-path coordinates the reference's CRS_Merge::mv uses for `parts`
 * threads (CRS_Merge.hpp:96-107 diagonals, :42-62 searchPathOnDiag),
 * computed on the device by the kernel that partitions the merge path:
 * coords[2*t], coords[2*t+1] = (row, nonzero) for t = 0..parts. */
int pwmgpu_merge_partition(pwmgpu_matrix* m, int32_t parts, int32_t* coords);
/* y = A x for a CRS matrix whose arrays are already on the device and owned
 * by the caller (row_start[nor+1], col_ind[nnz], vals[nnz], x[noc], y[nor]),
 * without allocating anything.  No counterpart in the reference: it is for
 * callers that cannot allocate device memory at call time -- a host runtime
 * whose allocator owns all device memory, a serving loop that must not hit
 * cudaMalloc / cudaFree (both may synchronise the device), a plug-in that is
 * handed device pointers only.  Its scratch (merge-path sub-tile coordinates
 * and carries) lives in one fixed 8 MiB array in device memory that every GPU
 * loading the library keeps until the process exits; this limits a call to
 * nor + nnz <= 134,217,472 (larger sizes return PWMGPU_ERR_INVALID).
 * Asynchronous on `stream` (a cudaStream_t, NULL for the legacy stream).
 * The first call on each device looks up the array's device address; make
 * that first call before any stream capture.  Every call shares the one
 * array, so calls that overlap on the GPU (other streams, other host threads)
 * race: order them on one stream. */
int pwmgpu_mv_csr_device_noalloc(int32_t nor, int32_t noc, int32_t nnz, const int32_t* row_start,
                                 const int32_t* col_ind, const double* vals, const double* x, double* y,
                                 void* stream);

/* ---- Row-sharded power method (one rank per GPU) ----
 * The reference's distributed power method (MPI_driver_poisson.cpp:38-63)
 * gives each rank a block of consecutive rows: y_loc = A_loc x, the sum of
 * squares of y_loc, an allreduce of those sums (:50), y_loc /= ||y||, and
 * an allgather of the blocks into x (:61).  These entry points are the
 * per-rank device work; the host mirror (thesis_spmv_gb300/sharded.py) runs
 * the two collectives with torch.distributed between them.
 *
 * Row blocks of the reference's 1D split (Util/TripletToCRS.hpp:318-327,
 * MPI_driver_poisson.cpp:84-89): nor / parts rows per block (integer
 * division), the last block takes the rest.  Host only; parts >= 1. */
int pwmgpu_row_blocks(int32_t nor, int32_t parts, int32_t* first_rows, int32_t* thread_rows);
/* Rows [first_row, last_row) of the mx x ny Poisson matrix as a
 * (last_row - first_row) x (mx * ny) matrix with global columns: the
 * reference's fillPoisson with first_row / last_row (Util/Poisson.hpp:33-83),
 * built on the device. */
int pwmgpu_generate_poisson_rows(pwmgpu_matrix* m, int32_t mx, int32_t ny, int32_t first_row, int32_t last_row);
/* Rows [first_row, last_row) of an nor x noc triplet matrix as a
 * (last_row - first_row) x noc CRS matrix with global columns: one block of
 * the reference's TripletToMultipleCRS (Util/TripletToCRS.hpp:309-385),
 * sorted on the device like pwmgpu_load_triplets.  Every row index must lie
 * in [0, nor); the caller's arrays are left unchanged (the reference sorts
 * the whole triplet by row in place). */
int pwmgpu_load_triplets_rows(pwmgpu_matrix* m, int32_t nor, int32_t noc, int32_t nnz, const int32_t* rows,
                              const int32_t* cols, const double* vals, int32_t first_row, int32_t last_row);
/* A rank's part of one step (MPI_driver_poisson.cpp:41-47): dy_loc = A_loc
 * dx_full (dx_full: all noc entries), and *dnsq_loc = sum of dy_loc[i]^2 in a
 * fixed order (a device double).  Asynchronous on the handle's stream. */
int pwmgpu_rows_step_device(pwmgpu_matrix* m, const double* dx_full, double* dy_loc, double* dnsq_loc);
/* dy_loc[i] *= 1 / sqrt(*dnsq_total) for the handle's rows (the reference
 * divides by the norm, MPI_driver_poisson.cpp:53-57; the reciprocal is within
 * one ulp of the quotient).  Asynchronous on the handle's stream. */
int pwmgpu_rows_normalize_device(pwmgpu_matrix* m, double* dy_loc, const double* dnsq_total);

/* The CSB arrays of a PWMGPU_FMT_CSB handle, as CSB.hpp:464-567 builds them
 * (for checks against the reference): beta, block bits, horizontal and
 * vertical block counts, then ind[nnz] (local row << 16 | local column),
 * data[nnz], blk_ptr[hb * vb + 1] (block_row * hb + block_col). */
int pwmgpu_csb_info(const pwmgpu_matrix* m, int32_t* beta, int32_t* block_bits, int32_t* hb, int32_t* vb,
                    int64_t* nnz);
int pwmgpu_get_csb(pwmgpu_matrix* m, uint32_t* ind, double* data, int32_t* blk_ptr);
/* The CO-H arrays of a PWMGPU_FMT_COH handle, as BlockCOH.hpp:319-455 builds
 * them for `partitions` threads: part_info[9 * partitions] = {first row,
 * beta, block bits, hb, vb, nnz, blocks, row jumps, block-row jumps} per
 * partition, then the concatenated row_jump, col_jump[nnz], data[nnz],
 * block_nnz[blocks], row_jump_block, col_jump_block[blocks]. */
int pwmgpu_coh_info(const pwmgpu_matrix* m, int32_t* partitions, int64_t* row_jumps, int64_t* blocks,
                    int64_t* block_row_jumps, int64_t* nnz);
int pwmgpu_get_coh(pwmgpu_matrix* m, int32_t* part_info, uint16_t* row_jump, uint16_t* col_jump, double* data,
                   int32_t* block_nnz, int16_t* row_jump_block, int16_t* col_jump_block);

/* Host-side format builders (no device work), the constructions of
 * CSB.hpp:96-113,464-567 and BlockCOH.hpp:319-455 from CRS arrays.  CSB:
 * pwmgpu_csb_params gives beta and the block bits (blk_ptr holds
 * ceil(noc/beta) * ceil(nor/beta) + 1 entries).  CO-H: every output array has
 * room for nnz entries (part_info for 9 * threads); the counts come back in
 * partitions, row_jumps, blocks and block_row_jumps. */
int pwmgpu_csb_params(int32_t nor, int32_t noc, int32_t* beta, int32_t* block_bits);
int pwmgpu_csb_build_host(int32_t nor, int32_t noc, int64_t nnz, const int32_t* row_start, const int32_t* col_ind,
                          const double* vals, uint32_t* ind, double* data, int32_t* blk_ptr);
int pwmgpu_coh_build_host(int32_t nor, int32_t noc, int64_t nnz, const int32_t* row_start, const int32_t* col_ind,
                          const double* vals, int32_t threads, int32_t* partitions, int64_t* row_jumps,
                          int64_t* blocks, int64_t* block_row_jumps, int32_t* part_info, uint16_t* row_jump,
                          uint16_t* col_jump, double* data, int32_t* block_nnz, int16_t* row_jump_block,
                          int16_t* col_jump_block);
/* Layout inspection (no device work; no reference counterpart): the device
 * copy the CSB (format PWMGPU_FMT_CSB) or CO-H (PWMGPU_FMT_COH, with
 * `partitions`) kernel reads, for windows of `window` rows (a power of two in
 * [64, min(beta, 1024)]).  sizes[3] = entries of win_ptr, of units and of
 * ind / data / col; the arrays are filled when all five pointers are
 * non-null.  win_ptr[2w], win_ptr[2w+1], win_ptr[2w+2]: window w's first
 * unit, its first dense unit, the next window's first unit.  units: 4 ints
 * per unit {lo, hi, c0, kind}: c0 = -1 for the window's flat unit (col holds
 * each element's global column), else the first column of the unit's x
 * window; kind 0 = row-major elements, 2 = one element per row (rows
 * ascending).  ind = row << 16 | column within the block (CSB.hpp:89-91)
 * or the tile (CO-H); the kernel reads both modulo the window. */
int pwmgpu_tile_layout_host(int32_t format, int32_t nor, int32_t noc, int64_t nnz, const int32_t* row_start,
                            const int32_t* col_ind, const double* vals, int32_t partitions, int32_t window,
                            int64_t* sizes, int32_t* win_ptr, int32_t* units, uint32_t* ind, double* data,
                            int32_t* col);

/* The merge kernels' launch variant the load-time tuner picked for this
 * matrix (prefer_l1: 0 = most resident CTAs, 1 = a smaller shared-memory
 * carveout leaving more L1 for the x gathers; both compute the same bits),
 * the SpMV and persistent-power grids, and the two timings compared
 * (tuned_ms[2], ms per SpMV; 0 when the matrix was too small to tune). */
int pwmgpu_launch_config(const pwmgpu_matrix* m, int32_t* prefer_l1, int32_t* grid, int32_t* power_grid,
                         float* tuned_ms);
/* The merge kernels' full launch variant: bit 0 = the smaller shared-memory
 * carveout, bit 1 = 16-bit columns, bit 2 = x gathers that bypass L1. */
int pwmgpu_launch_variant(const pwmgpu_matrix* m, int32_t* variant);
/* Override the tuner's choice for later launches: 0 or 1 (carveout), 4 or 5
 * (the same with x gathers that bypass L1, on FP64 iterations).  16-bit
 * columns are used wherever the plan has them. */
int pwmgpu_set_launch_variant(pwmgpu_matrix* m, int32_t variant);
/* Bytes per column index the merge kernels stream: 2 when every merge
 * sub-tile's columns span less than 2^16 (banded and stencil matrices: the
 * plan then keeps 16-bit offsets from a per-sub-tile base), else 4; and
 * whether the load-time tuner chose x gathers that bypass L1 (1) or not (0).
 * Either pointer may be null. */
int pwmgpu_plan_info(const pwmgpu_matrix* m, int32_t* column_bytes, int32_t* gathers_bypass_l1);

/* Tile size (merge items per tile) and tile count used by the SpMV kernel. */
int pwmgpu_tile_info(const pwmgpu_matrix* m, int32_t* items_per_tile, int32_t* num_tiles, int32_t* grid);

#ifdef __cplusplus
}
#endif
#endif /* PWMGPU_H */
