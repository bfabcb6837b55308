/*
 * oracle.h -- CPU restatement of the reference's SpMV / power-method path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: only tests/, the smoke()
 * entry and bench.py's CPU-baseline leg may load it.  The product library
 * (libpwmgpu.so) never links or calls it.
 *
 * Every function restates one function of KobeBergmans/Thesis_SPMV (cited
 * file:line).  It is pinned two ways: against the reference's own known-answer
 * vectors (Tests/poisson.cpp, Tests/input.cpp, extracted into tests/golden/)
 * and against the unmodified reference headers compiled by oracle/build_ref.sh
 * (tests/test_oracle_vs_ref.py, run where the reference tree is present).
 *
 * Types: indices are int32 (the reference's int / uint32 instantiations are
 * identical for N < 2^31); values are double (data_t, Util/Constants.hpp:32).
 * Built with -ffp-contract=off so `y = y + a*x` rounds as written.
 */
#ifndef PWM_ORACLE_H
#define PWM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Matrix/CRS.hpp:64 -- nnz of the m x n 5-point Poisson matrix. */
int64_t orc_poisson_nnz(int32_t m, int32_t n);
/* Util/Poisson.hpp:32-83 (fillPoisson, whole matrix). */
void orc_fill_poisson(int32_t m, int32_t n, int32_t* row_start, int32_t* col_ind, double* data);
/* Matrix/Triplet.hpp:226-278 (Triplet::generatePoisson; COO order differs). */
void orc_triplet_poisson(int32_t m, int32_t n, int32_t* rows, int32_t* cols, double* vals);

/* Util/TripletToCRS.hpp:135-172.  Sorts the triplet in place (by row, then
 * column) and writes CRS.  For unique coordinates the reference's randomised
 * quicksort yields exactly this order. */
void orc_triplet_to_crs(int32_t nnz, int32_t nor, int32_t* rows, int32_t* cols, double* vals,
                        int32_t* row_start, int32_t* col_ind, double* crs_data);

/* Row blocks of the reference's 1D split (Util/TripletToCRS.hpp:318-327,
 * MPI_driver_poisson.cpp:84-89): am = nor / parts rows per block (integer
 * division), the last block takes the rest. */
void orc_row_blocks(int32_t nor, int32_t parts, int32_t* first_rows, int32_t* thread_rows);
/* Util/TripletToCRS.hpp:309-385 (TripletToMultipleCRS): the triplet sorted
 * in place like TripletToCRS, then one CRS per row block with local row
 * starts and global columns.  Outputs are concatenated: block p's row starts
 * (thread_rows[p] + 1 entries) follow block p-1's; columns and values of the
 * blocks are consecutive (nnz in total).  A block without nonzeros gets all
 * row starts 0 (the reference reads into the next block there). */
void orc_triplet_to_multi_crs(int32_t nnz, int32_t nor, int32_t parts, int32_t* rows, int32_t* cols, double* vals,
                              int32_t* first_rows, int32_t* thread_rows, int32_t* row_start_all, int32_t* col_all,
                              double* data_all);
/* Util/Poisson.hpp:33-83 with first_row / last_row: rows [first_row,
 * last_row) of the m x n Poisson matrix, local row starts, global columns. */
void orc_fill_poisson_rows(int32_t m, int32_t n, int32_t first_row, int32_t last_row, int32_t* row_start,
                           int32_t* col_ind, double* data);
/* MPI_driver_poisson.cpp:38-63 (powerIteration over `parts` ranks), in one
 * process: per iteration every block's mv (:24-35, a row sum from 0), every
 * block's sum of squares in row order (:44-47), the blocks' sums added in
 * rank order (the MPI_Allreduce of :50), norm = sqrt, y /= norm per element
 * (:53-57) and the full x assembled from the blocks (MPI_Allgatherv, :61).
 * rs_all / ci / d: the blocks as orc_triplet_to_multi_crs writes them; x:
 * all nor entries in, the normalised iterate after `it` iterations out. */
void orc_power_rows(int32_t nor, int32_t parts, const int32_t* rs_all, const int32_t* ci, const double* d, double* x,
                    int32_t it);

/* SOA_Implementations/CRS_Merge.hpp:95-141 with one merge-path partition per
 * OpenMP thread, as the reference runs it (the CPU baseline's timing;
 * orc_merge_mv is the same arithmetic, partitions in sequence). */
void orc_merge_omp_mv(int32_t nor, int32_t nnz, const int32_t* row_start, const int32_t* col_ind,
                      const double* data, const double* x, double* y, int32_t threads);
/* Matrix/CRS.hpp:99-109 (sequential CRS::mv). */
void orc_crs_mv(int32_t nor, const int32_t* row_start, const int32_t* col_ind, const double* data,
                const double* x, double* y);
/* Env_Implementations/CRSOMP.hpp:110-123 (OpenMP, schedule(dynamic,512)). */
void orc_crs_omp_mv(int32_t nor, const int32_t* row_start, const int32_t* col_ind, const double* data,
                    const double* x, double* y, int threads);

/* SOA_Implementations/CRS_Merge.hpp:42-62 (searchPathOnDiag). */
void orc_merge_search(int32_t diagonal, int32_t nor, int32_t nnz, const int32_t* row_end_offsets,
                      int32_t* a_coord, int32_t* b_coord);
/* CRS_Merge.hpp:95-141: the thread coordinates for `threads` partitions
 * (coords has 2*(threads+1) entries: a0,b0,a1,b1,...). */
void orc_merge_partition(int32_t nor, int32_t nnz, const int32_t* row_start, int32_t threads, int32_t* coords);
/* CRS_Merge.hpp:95-141 (merge-path mv; partitions run one after another,
 * giving the same result as the OpenMP version, carries fixed in tid order). */
void orc_merge_mv(int32_t nor, int32_t nnz, const int32_t* row_start, const int32_t* col_ind,
                  const double* data, const double* x, double* y, int32_t threads);

/* Util/VectorUtill.hpp:23-26 and :34-41. */
double orc_norm2(const double* x, int64_t n);
void orc_normalize(double* x, int64_t n);

/* powerIteration: Matrix/CRS.hpp:118-130 (kind 0, sequential mv),
 * Env_Implementations/CRSOMP.hpp:135-157 (kind 1, OpenMP mv + static divide),
 * CRS_Merge (kind 2: merge mv with `threads` partitions, CRSOMP's loop).
 * The result is in x when `it` is even and in y when it is odd. */
void orc_power(int kind, int32_t nor, int32_t nnz, const int32_t* row_start, const int32_t* col_ind,
               const double* data, double* x, double* y, int32_t it, int threads);

/* ---- CSB (SOA_Implementations/CSB.hpp) ---- */
/* :96-113 setBlockSizeParam for T=double. */
/* Eigenvalue estimate (Rayleigh quotient) and relative eigen-residual of u
 * (harness arithmetic; the reference has none). */
void orc_rayleigh(int32_t nor, const int32_t* row_start, const int32_t* col_ind, const double* data,
                  const double* u, double* lambda, double* residual);

void orc_csb_params(int32_t nor, int32_t noc, int32_t* beta, int32_t* block_bits);
/* :464-567 loadFromTriplets.  ind[nnz], data[nnz], blk_ptr[H*V+1].
 * The triplet is sorted in place (row, then column).  Returns the balanced
 * flag (:549-559). */
int orc_csb_build(int32_t nor, int32_t noc, int32_t nnz, int32_t* rows, int32_t* cols, double* vals,
                  uint32_t* ind, double* data, int32_t* blk_ptr);
/* :593-642 mv in block-row / block / Z-Morton storage order (the balanced
 * path's summation order). */
void orc_csb_mv(int32_t nor, int32_t noc, const uint32_t* ind, const double* data, const int32_t* blk_ptr,
                const double* x, double* y);

/* ---- Block CO-H (SOA_Implementations/BlockCOH.hpp) ---- */
/* :79-114 rowColToHilbert. */
int32_t orc_hilbert(int32_t size, int32_t row, int32_t col);
/* :319-455 loadFromTriplets, returned as a flat description.  Per partition
 * p (p < *threads_out): part_info[p*9 + k] = {row_start, beta, block_bits,
 * hblocks, vblocks, nnz, blocks, n_row_jump, n_row_jump_block}; the per-
 * partition arrays are concatenated in partition order (the caller sizes
 * them with orc_coh_sizes first).  The triplet is sorted in place. */
int orc_coh_sizes(int32_t nor, int32_t noc, int32_t nnz, const int32_t* rows, const int32_t* cols,
                  int32_t threads, int64_t* total_row_jump, int64_t* total_blocks);
int orc_coh_build(int32_t nor, int32_t noc, int32_t nnz, int32_t* rows, int32_t* cols, double* vals,
                  int32_t threads, int32_t* part_info, uint16_t* row_jump, uint16_t* col_jump, double* data,
                  int32_t* block_nnz, int16_t* row_jump_block, int16_t* col_jump_block);
/* :479-510 mv over the flat description produced above. */
void orc_coh_mv(int32_t nor, int32_t threads, const int32_t* part_info, const uint16_t* row_jump,
                const uint16_t* col_jump, const double* data, const int32_t* block_nnz,
                const int16_t* row_jump_block, const int16_t* col_jump_block, const double* x, double* y);

/* ---- Loaders (Matrix/Triplet.hpp:75-154, :164-216) ----
 * Two-pass: call with out arrays NULL to get the capacity, then again. */
int64_t orc_load_mm(const char* filename, int has_data, int symmetric, int32_t* nor, int32_t* noc,
                    int32_t* rows, int32_t* cols, double* vals, int64_t capacity);
int64_t orc_load_bin(const char* filename, int32_t mat_size, int symmetric, int32_t* rows, int32_t* cols,
                     double* vals, int64_t capacity);

/* Seeded random matrices: restatement of the library's device generator
 * (benchmark inputs, no reference counterpart).  Call with NULL arrays to
 * get nnz, then with row_start[n+1], col_ind[nnz], data[nnz]. */
void orc_random_table(int kind, double mean, double sigma, int32_t max_len, uint64_t* thr);
int64_t orc_random_crs(int32_t n, uint64_t seed, int kind, double mean, double sigma, int32_t max_len,
                       int32_t band_permille, int32_t band_half, int32_t* row_start, int32_t* col_ind,
                       double* data);

/* The batched service's seeded start vector (uniform in [0, 1)). */
void orc_uniform_vector(int32_t n, uint64_t seed, double* x);

/* Matrix statistics (Util_Scripts/calc_stats.cpp:45-98), in the script's
 * order of operations.  out: size, nnz, rows_avg, rows_var, block_avg,
 * block_var, balanced (1/0), block_bits, whole blocks per side (the script's
 * nb_blocks after its "whole blocks only" decrement).  Square matrices (the
 * script indexes column blocks by the row count); returns -1 if a column block
 * falls outside, or the block table cannot be allocated. */
int orc_calc_stats(int64_t nnz, int32_t nor, const int32_t* rows, const int32_t* cols, double* out);

#ifdef __cplusplus
}
#endif
#endif
