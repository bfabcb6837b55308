/*
 * pwmsvc.h -- C ABI of the batched power-method service (GB300, sm_103a).
 *
 * No counterpart in the reference (KobeBergmans/Thesis_SPMV serves one matrix
 * per powerIteration call, Matrix/CRS.hpp:118-130); this is the serving loop
 * around the same path.  Requests -- power solves on matrices of any size --
 * are queued on submit, admitted while live slots and the HBM budget allow,
 * and advanced together: each round runs `round_iterations` power steps of
 * every live solve, one launch per step for all of them (their merge-path
 * sub-tiles form one list: the block-diagonal matrix of the live solves, cut
 * at the matrix boundaries), followed by a residual pass; with use_graph the
 * round is one CUDA graph.  Each solve keeps its matrix and iterates resident
 * in HBM until it retires.  Mixed precision starts with one FP64 round
 * (the precision tuner's probe): a matrix whose residual after it projects
 * to tol within five rounds stays in FP64; the others run the FP32 (BF16
 * values where exact) phase as pwmgpu_solve does (to a residual of 2e-6,
 * the FP32 floor, or the FP64 reserve), then FP64.
 * Sums over a solve's rows run in a fixed order over its own sub-tiles, so a
 * solve gives the same bits alone and in any mix.
 *
 * All entry points return a PWMGPU_* status (pwmgpu.h) and record a message
 * for pwmgpu_last_error().  One host thread per service.
 */
#ifndef PWMSVC_H
#define PWMSVC_H

#include <stddef.h>
#include <stdint.h>

#include "pwmgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pwmsvc pwmsvc;

typedef struct {
    size_t hbm_budget_bytes;  /* admission budget for matrices + vectors (0: 90 % of free memory) */
    int32_t max_live;         /* live solves at most (0: 1024) */
    int32_t round_iterations; /* power steps per round, >= 2 (0: 8) */
    int32_t use_graph;        /* 1: each round replays one captured CUDA graph */
} pwmsvc_config;

/* matrix sources */
#define PWMSVC_SRC_CSR 0     /* host CRS arrays, copied at submit */
#define PWMSVC_SRC_POISSON 1 /* grid_m x grid_n 5-point Poisson (Util/Poisson.hpp:32-83), built on the device */
#define PWMSVC_SRC_RANDOM 2  /* pwmgpu_generate_random's matrix, built on the device */
#define PWMSVC_SRC_TRIPLETS 3 /* host triplets (row_ind, col_ind, vals; square nor), copied at submit,
                                 * turned into CRS on the device at admission (pwmgpu_load_triplets) */

typedef struct {
    int32_t source;
    /* PWMSVC_SRC_CSR (square) */
    int32_t nor, nnz;
    const int32_t* row_start;
    const int32_t* col_ind;
    const double* vals;
    /* PWMSVC_SRC_POISSON */
    int32_t grid_m, grid_n;
    /* PWMSVC_SRC_RANDOM */
    int32_t n;
    uint64_t seed;
    int32_t length_dist;
    double mean_len, sigma;
    int32_t max_len, band_permille, band_half;
    /* start vector: x0 (host, copied at submit) or, when NULL, x0[i] uniform
     * in [0, 1) from a hash of (x0_seed, i) */
    const double* x0;
    uint64_t x0_seed;
    /* stopping rule: ||A u - lambda u|| / |lambda| <= tol, checked at the end
     * of each round, or max_it steps (rounded up to whole rounds) */
    int32_t max_it;
    double tol;
    int32_t precision;   /* PWMGPU_PREC_* */
    int32_t keep_vector; /* 1: keep the eigenvector on the host for pwmsvc_result */
    /* PWMSVC_SRC_TRIPLETS: the row of each of the nnz entries (col_ind and
     * vals as for PWMSVC_SRC_CSR, in the same entry order) */
    const int32_t* row_ind;
} pwmsvc_request;

#define PWMSVC_QUEUED 0
#define PWMSVC_RUNNING 1
#define PWMSVC_DONE 2
#define PWMSVC_FAILED 3

typedef struct {
    int32_t state;          /* PWMSVC_* */
    int32_t n;              /* matrix order */
    int32_t iterations;     /* power steps (SpMVs) done */
    int32_t iterations_low; /* of which in the FP32 / BF16 phase */
    int32_t converged;
    int32_t precision;
    int32_t error;          /* PWMGPU_* status of a failed request */
    int32_t pad;
    double lambda;          /* Rayleigh quotient of the returned u (||u|| = 1) */
    double residual;        /* ||A u - lambda u|| / |lambda| */
    double t_submit, t_admit, t_done; /* seconds since pwmsvc_create */
} pwmsvc_result_info;

typedef struct {
    int64_t submitted, finished, failed, rounds;
    int32_t live, queued;
    size_t hbm_in_use, hbm_budget;
    double gpu_round_ms; /* device time of all rounds so far (events around each round) */
} pwmsvc_stats_info;

int pwmsvc_create(const pwmsvc_config* cfg, pwmsvc** out);
int pwmsvc_destroy(pwmsvc* s);
/* Queue a request (a request that alone exceeds the budget fails with
 * PWMGPU_ERR_BUDGET here). */
int pwmsvc_submit(pwmsvc* s, const pwmsvc_request* r, int64_t* id);
/* Admit what fits, run one round of every live solve, retire the finished
 * ones.  Outputs (each may be NULL): live and queued requests after the
 * round, requests finished by this round. */
int pwmsvc_step(pwmsvc* s, int32_t* live, int32_t* queued, int32_t* finished);
/* Result of a request; u (nor doubles, may be NULL) receives the eigenvector
 * of a finished request submitted with keep_vector. */
int pwmsvc_result(pwmsvc* s, int64_t id, pwmsvc_result_info* out, double* u);
/* Forget a finished request (its host copy of u). */
int pwmsvc_release(pwmsvc* s, int64_t id);
int pwmsvc_stats(pwmsvc* s, pwmsvc_stats_info* out);

#ifdef __cplusplus
}
#endif
#endif /* PWMSVC_H */
