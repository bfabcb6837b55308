/*
 * oracle.c -- CPU restatement of KobeBergmans/Thesis_SPMV's SpMV and
 * power-method path.  TEST INFRASTRUCTURE ONLY (see oracle.h): the checker
 * for the GPU library and the CPU baseline of bench.py, never the product.
 *
 * Each function names the reference function it restates (file:line).  The
 * reference sorts with a randomised quicksort (Util/TripletToCRS.hpp:107-120);
 * for unique coordinates its output is fully determined by the keys, so the
 * restatement sorts with a deterministic comparison on the same keys.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Poisson                                                              */
/* ------------------------------------------------------------------ */

int64_t orc_poisson_nnz(int32_t m, int32_t n) {
    /* Matrix/CRS.hpp:64: nnz = n*(m+2*(m-1)) + 2*(n-1)*m */
    return (int64_t)n * (m + 2 * (int64_t)(m - 1)) + 2 * (int64_t)(n - 1) * m;
}

void orc_fill_poisson(int32_t m, int32_t n, int32_t* row_start, int32_t* col_ind, double* data) {
    /* Util/Poisson.hpp:32-83: per row, ascending columns row-m, row-1, row,
     * row+1, row+m with the boundary guards of :46, :54, :67, :75. */
    int32_t last_row = m * n;
    int32_t k = 0;
    row_start[0] = 0;
    for (int32_t row = 0; row < last_row; ++row) {
        if (row >= m) { data[k] = -1; col_ind[k] = row - m; ++k; }
        if (row % m != 0) { data[k] = -1; col_ind[k] = row - 1; ++k; }
        data[k] = 4; col_ind[k] = row; ++k;
        if (row % m != m - 1) { data[k] = -1; col_ind[k] = row + 1; ++k; }
        if (row < m * n - m) { data[k] = -1; col_ind[k] = m + row; ++k; }
        row_start[row + 1] = k;
    }
}

void orc_triplet_poisson(int32_t m, int32_t n, int32_t* rows, int32_t* cols, double* vals) {
    /* Matrix/Triplet.hpp:226-278 */
    int32_t size = m * n;
    int64_t k = 0;
    for (int32_t i = 0; i < size; ++i) {
        rows[k] = i; cols[k] = i; vals[k] = 4.; ++k;
        if (i < size - 1) {
            if (i % m != m - 1) { rows[k] = i; cols[k] = i + 1; vals[k] = -1.; ++k; }
            if ((i + 1) % m != 0) { rows[k] = i + 1; cols[k] = i; vals[k] = -1.; ++k; }
        }
        if (i < size - m) {
            rows[k] = i + m; cols[k] = i; vals[k] = -1.; ++k;
            rows[k] = i; cols[k] = i + m; vals[k] = -1.; ++k;
        }
    }
}

/* ------------------------------------------------------------------ */
/* Sorting helpers                                                      */
/* ------------------------------------------------------------------ */

typedef struct { uint64_t key; int64_t idx; } keyed_t;

static int cmp_keyed(const void* a, const void* b) {
    const keyed_t* x = (const keyed_t*)a;
    const keyed_t* y = (const keyed_t*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    if (x->idx != y->idx) return x->idx < y->idx ? -1 : 1;
    return 0;
}

/* Apply the permutation in kv[lo..hi) to rows/cols/vals (in place). */
static void permute_triplets(keyed_t* kv, int64_t lo, int64_t hi, int32_t* rows, int32_t* cols, double* vals) {
    int64_t n = hi - lo;
    int32_t* r = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? (size_t)n : 1));
    int32_t* c = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? (size_t)n : 1));
    double* v = (double*)malloc(sizeof(double) * (n > 0 ? (size_t)n : 1));
    for (int64_t i = 0; i < n; ++i) {
        int64_t s = kv[lo + i].idx;
        r[i] = rows[s]; c[i] = cols[s]; v[i] = vals[s];
    }
    memcpy(rows + lo, r, sizeof(int32_t) * n);
    memcpy(cols + lo, c, sizeof(int32_t) * n);
    memcpy(vals + lo, v, sizeof(double) * n);
    free(r); free(c); free(v);
}

/* Sort triplets by (row, col). */
static void sort_row_col(int32_t nnz, int32_t* rows, int32_t* cols, double* vals) {
    keyed_t* kv = (keyed_t*)malloc(sizeof(keyed_t) * (nnz > 0 ? (size_t)nnz : 1));
    for (int64_t i = 0; i < nnz; ++i) {
        kv[i].key = ((uint64_t)(uint32_t)rows[i] << 32) | (uint32_t)cols[i];
        kv[i].idx = i;
    }
    qsort(kv, nnz, sizeof(keyed_t), cmp_keyed);
    permute_triplets(kv, 0, nnz, rows, cols, vals);
    free(kv);
}

/* ------------------------------------------------------------------ */
/* Triplet -> CRS                                                       */
/* ------------------------------------------------------------------ */

void orc_triplet_to_crs(int32_t nnz, int32_t nor, int32_t* rows, int32_t* cols, double* vals,
                        int32_t* row_start, int32_t* col_ind, double* crs_data) {
    /* Util/TripletToCRS.hpp:135-172: sort on rows, copy, fill row_start with
     * the index of each row's first entry (empty rows repeat it), trailing
     * rows get nnz, then sort each row's columns. */
    sort_row_col(nnz, rows, cols, vals);
    int32_t row_index = 0;
    row_start[0] = 0;
    for (int32_t i = 0; i < nnz; ++i) {
        col_ind[i] = cols[i];
        crs_data[i] = vals[i];
        while (rows[i] != row_index) {
            row_index++;
            row_start[row_index] = i;
        }
    }
    while (row_index < nor) {
        row_index++;
        row_start[row_index] = nnz;
    }
}

void orc_row_blocks(int32_t nor, int32_t parts, int32_t* first_rows, int32_t* thread_rows) {
    /* Util/TripletToCRS.hpp:318-327: am_rows = round(nor / partitions) on
     * integers (the division already truncates), first_rows[i] = previous
     * last row, the last partition ends at nor. */
    const int32_t am = nor / parts;
    int32_t last = 0;
    for (int32_t i = 0; i < parts; ++i) {
        first_rows[i] = last;
        last = (i == parts - 1) ? nor : first_rows[i] + am;
        thread_rows[i] = last - first_rows[i];
    }
}

void orc_triplet_to_multi_crs(int32_t nnz, int32_t nor, int32_t parts, int32_t* rows, int32_t* cols, double* vals,
                              int32_t* first_rows, int32_t* thread_rows, int32_t* row_start_all, int32_t* col_all,
                              double* data_all) {
    /* Util/TripletToCRS.hpp:309-385: sort on rows (columns follow), then per
     * partition copy its entries, fill the local row starts (empty rows
     * repeat the index, trailing rows get the partition's count) and sort
     * each row's columns.  Sorting the whole triplet by (row, column) first
     * gives the same arrays for unique coordinates. */
    sort_row_col(nnz, rows, cols, vals);
    orc_row_blocks(nor, parts, first_rows, thread_rows);
    int32_t k = 0, base = 0;
    for (int32_t p = 0; p < parts; ++p) {
        int32_t* rs = row_start_all + base;
        const int32_t last = first_rows[p] + thread_rows[p];
        const int32_t k0 = k;
        int32_t row_index = 0;
        rs[0] = 0;
        while (k < nnz && rows[k] < last) {
            col_all[k] = cols[k];
            data_all[k] = vals[k];
            while (rows[k] != row_index + first_rows[p]) {
                row_index++;
                rs[row_index] = k - k0;
            }
            ++k;
        }
        while (row_index < thread_rows[p]) {
            row_index++;
            rs[row_index] = k - k0;
        }
        base += thread_rows[p] + 1;
    }
}

void orc_fill_poisson_rows(int32_t m, int32_t n, int32_t first_row, int32_t last_row, int32_t* row_start,
                           int32_t* col_ind, double* data) {
    /* Util/Poisson.hpp:33-83 with a row range: the same per-row entries as
     * orc_fill_poisson, row starts counted from the block's first row. */
    int32_t k = 0;
    row_start[0] = 0;
    for (int32_t row = first_row; row < last_row; ++row) {
        if (row >= m) { data[k] = -1; col_ind[k] = row - m; ++k; }
        if (row % m != 0) { data[k] = -1; col_ind[k] = row - 1; ++k; }
        data[k] = 4; col_ind[k] = row; ++k;
        if (row % m != m - 1) { data[k] = -1; col_ind[k] = row + 1; ++k; }
        if (row < m * n - m) { data[k] = -1; col_ind[k] = m + row; ++k; }
        row_start[row - first_row + 1] = k;
    }
}

void orc_power_rows(int32_t nor, int32_t parts, const int32_t* rs_all, const int32_t* ci, const double* d, double* x,
                    int32_t it) {
    /* MPI_driver_poisson.cpp:38-63, every rank in turn */
    int32_t* first = (int32_t*)malloc(sizeof(int32_t) * (size_t)parts);
    int32_t* nrow = (int32_t*)malloc(sizeof(int32_t) * (size_t)parts);
    double* part = (double*)malloc(sizeof(double) * (size_t)parts);
    double* y = (double*)malloc(sizeof(double) * (size_t)(nor > 0 ? nor : 1));
    orc_row_blocks(nor, parts, first, nrow);
    for (int32_t i = 0; i < it; ++i) {
        int32_t base = 0, k0 = 0;
        for (int32_t p = 0; p < parts; ++p) {
            const int32_t* rs = rs_all + base;
            double* yp = y + first[p];
            for (int32_t l = 0; l < nrow[p]; ++l) {  /* mv, :24-35 */
                double sum = 0;
                for (int32_t k = rs[l]; k < rs[l + 1]; ++k) sum += d[k0 + k] * x[ci[k0 + k]];
                yp[l] = sum;
            }
            double np = 0;  /* :44-47 */
            for (int32_t l = 0; l < nrow[p]; ++l) np += yp[l] * yp[l];
            part[p] = np;
            k0 += rs[nrow[p]];
            base += nrow[p] + 1;
        }
        double norm = 0;  /* :50, rank order */
        for (int32_t p = 0; p < parts; ++p) norm += part[p];
        norm = sqrt(norm);
        for (int32_t r = 0; r < nor; ++r) x[r] = y[r] / norm;  /* :53-61 */
    }
    free(first);
    free(nrow);
    free(part);
    free(y);
}

/* ------------------------------------------------------------------ */
/* CRS mv                                                               */
/* ------------------------------------------------------------------ */

void orc_crs_mv(int32_t nor, const int32_t* row_start, const int32_t* col_ind, const double* data,
                const double* x, double* y) {
    /* Matrix/CRS.hpp:99-109 */
    for (int32_t i = 0; i < nor; ++i) y[i] = 0.;
    for (int32_t i = 0; i < nor; ++i)
        for (int32_t k = row_start[i]; k < row_start[i + 1]; ++k)
            y[i] = y[i] + data[k] * x[col_ind[k]];
}

void orc_crs_omp_mv(int32_t nor, const int32_t* row_start, const int32_t* col_ind, const double* data,
                    const double* x, double* y, int threads) {
    /* Env_Implementations/CRSOMP.hpp:110-123 (Constants.hpp:13 chunk 512) */
#pragma omp parallel for schedule(dynamic, 512) num_threads(threads)
    for (int32_t i = 0; i < nor; ++i) {
        double sum = 0.;
        for (int32_t k = row_start[i]; k < row_start[i + 1]; ++k) sum += data[k] * x[col_ind[k]];
        y[i] = sum;
    }
    (void)threads;
}

/* ------------------------------------------------------------------ */
/* Merge path                                                           */
/* ------------------------------------------------------------------ */

void orc_merge_search(int32_t diagonal, int32_t nor, int32_t nnz, const int32_t* list_a,
                      int32_t* a_coord, int32_t* b_coord) {
    /* SOA_Implementations/CRS_Merge.hpp:42-62 */
    int32_t lo = 0;
    if (diagonal > nnz) lo = diagonal - nnz;
    int32_t hi = diagonal < nor ? diagonal : nor;
    while (lo < hi) {
        int32_t pivot = (int32_t)(((uint32_t)lo + (uint32_t)hi) >> 1);
        if (list_a[pivot] <= diagonal - pivot - 1) lo = pivot + 1;
        else hi = pivot;
    }
    *a_coord = lo < nor ? lo : nor;
    *b_coord = diagonal - lo;
}

void orc_merge_partition(int32_t nor, int32_t nnz, const int32_t* row_start, int32_t threads, int32_t* coords) {
    /* CRS_Merge.hpp:96-107: diagonal_t = min(ipt*t, total), ipt = ceil(total/threads) */
    int32_t total = nor + nnz;
    int32_t ipt = (total + threads - 1) / threads;
    for (int32_t t = 0; t <= threads; ++t) {
        int64_t d = (int64_t)ipt * t;
        int32_t diag = d < total ? (int32_t)d : total;
        orc_merge_search(diag, nor, nnz, row_start + 1, &coords[2 * t], &coords[2 * t + 1]);
    }
}

void orc_merge_mv(int32_t nor, int32_t nnz, const int32_t* row_start, const int32_t* col_ind,
                  const double* data, const double* x, double* y, int32_t threads) {
    /* CRS_Merge.hpp:95-141.  Partitions are independent; running them in
     * sequence gives the OpenMP result bit for bit. */
    const int32_t* row_end = row_start + 1;
    int32_t* coords = (int32_t*)malloc(sizeof(int32_t) * 2 * (threads + 1));
    int32_t* carry_row = (int32_t*)malloc(sizeof(int32_t) * threads);
    double* carry_val = (double*)malloc(sizeof(double) * threads);
    orc_merge_partition(nor, nnz, row_start, threads, coords);
    for (int32_t t = 0; t < threads; ++t) {
        int32_t a = coords[2 * t], b = coords[2 * t + 1];
        int32_t a_end = coords[2 * t + 2], b_end = coords[2 * t + 3];
        double running = 0.;
        for (; a < a_end; ++a) {
            for (; b < row_end[a]; ++b) running += data[b] * x[col_ind[b]];
            y[a] = running;
            running = 0.;
        }
        for (; b < b_end; ++b) running += data[b] * x[col_ind[b]];
        carry_row[t] = a_end;
        carry_val[t] = running;
    }
    for (int32_t t = 0; t < threads; ++t)
        if (carry_row[t] < nor) y[carry_row[t]] += carry_val[t];
    free(coords); free(carry_row); free(carry_val);
}

void orc_merge_omp_mv(int32_t nor, int32_t nnz, const int32_t* row_start, const int32_t* col_ind,
                      const double* data, const double* x, double* y, int32_t threads) {
    /* CRS_Merge.hpp:95-141 as the reference runs it: one merge-path
     * partition per OpenMP thread (schedule(static), :101), then the serial
     * carry fix-up (:136-140).  Same arithmetic as orc_merge_mv. */
    const int32_t* row_end = row_start + 1;
    int32_t* coords = (int32_t*)malloc(sizeof(int32_t) * 2 * (threads + 1));
    int32_t* carry_row = (int32_t*)malloc(sizeof(int32_t) * threads);
    double* carry_val = (double*)malloc(sizeof(double) * threads);
    orc_merge_partition(nor, nnz, row_start, threads, coords);
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int32_t t = 0; t < threads; ++t) {
        int32_t a = coords[2 * t], b = coords[2 * t + 1];
        const int32_t a_end = coords[2 * t + 2], b_end = coords[2 * t + 3];
        double running = 0.;
        for (; a < a_end; ++a) {
            for (; b < row_end[a]; ++b) running += data[b] * x[col_ind[b]];
            y[a] = running;
            running = 0.;
        }
        for (; b < b_end; ++b) running += data[b] * x[col_ind[b]];
        carry_row[t] = a_end;
        carry_val[t] = running;
    }
    for (int32_t t = 0; t < threads; ++t)
        if (carry_row[t] < nor) y[carry_row[t]] += carry_val[t];
    free(coords); free(carry_row); free(carry_val);
}

/* ------------------------------------------------------------------ */
/* Vector utilities and the power method                                */
/* ------------------------------------------------------------------ */

double orc_norm2(const double* x, int64_t n) {
    /* Util/VectorUtill.hpp:23-26: sqrt(inner_product(x, x, 0.)) in order */
    double s = 0.;
    for (int64_t i = 0; i < n; ++i) s = s + x[i] * x[i];
    return sqrt(s);
}

void orc_normalize(double* x, int64_t n) {
    /* Util/VectorUtill.hpp:34-41: a true divide by the norm */
    double nrm = orc_norm2(x, n);
    for (int64_t i = 0; i < n; ++i) x[i] /= nrm;
}

void orc_power(int kind, int32_t nor, int32_t nnz, const int32_t* row_start, const int32_t* col_ind,
               const double* data, double* x, double* y, int32_t it, int threads) {
    /* CRS.hpp:118-130 / CRSOMP.hpp:135-157: it times y=Ax, y/=||y||, swap roles */
    for (int32_t i = 0; i < it; ++i) {
        const double* in = (i % 2 == 0) ? x : y;
        double* out = (i % 2 == 0) ? y : x;
        if (kind == 0) orc_crs_mv(nor, row_start, col_ind, data, in, out);
        else if (kind == 1) orc_crs_omp_mv(nor, row_start, col_ind, data, in, out, threads);
        else orc_merge_mv(nor, nnz, row_start, col_ind, data, in, out, threads);
        if (kind == 1) {
            double nrm = orc_norm2(out, nor);
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int32_t r = 0; r < nor; ++r) out[r] /= nrm;
        } else {
            orc_normalize(out, nor);
        }
    }
}

void orc_rayleigh(int32_t nor, const int32_t* row_start, const int32_t* col_ind, const double* data,
                  const double* u, double* lambda, double* residual) {
    /* Not in the reference (its powerIteration has no eigenvalue output):
     * the harness's eigenvalue estimate lambda = u.(Au) / u.u with Au from
     * CRS::mv (CRS.hpp:99-109) and sequential FP64 dot products, and the
     * relative eigen-residual ||Au - lambda u|| / (|lambda| ||u||). */
    double* au = (double*)malloc(sizeof(double) * (size_t)(nor > 0 ? nor : 1));
    orc_crs_mv(nor, row_start, col_ind, data, u, au);
    double num = 0., den = 0.;
    for (int32_t i = 0; i < nor; ++i) {
        num = num + u[i] * au[i];
        den = den + u[i] * u[i];
    }
    double lam = num / den, rr = 0.;
    for (int32_t i = 0; i < nor; ++i) {
        double d = au[i] - lam * u[i];
        rr = rr + d * d;
    }
    free(au);
    *lambda = lam;
    *residual = sqrt(rr) / (fabs(lam) * sqrt(den));
}

/* ------------------------------------------------------------------ */
/* CSB                                                                  */
/* ------------------------------------------------------------------ */

void orc_csb_params(int32_t nor, int32_t noc, int32_t* beta, int32_t* block_bits) {
    /* CSB.hpp:96-113 with sizeof(T)=8, L2_CACHE_SIZE_MB=1, L2_CACHE_MULT=0.85
     * (Util/Constants.hpp:27-28). */
    int32_t minimal = nor < noc ? nor : noc;
    int32_t lg = (int32_t)ceil(log2(sqrt((double)minimal)));
    int32_t bits = 3 + lg < 16 ? 3 + lg : 16;
    int32_t b = (int32_t)pow(2, bits);
    while (bits > lg) {
        if ((double)(8 * 8) * b * 2 > 1 * 0.85 * 1e6 * 8) {
            bits -= 1;
            b = (int32_t)pow(2, bits);
        } else {
            break;
        }
    }
    *beta = b;
    *block_bits = bits;
}

/* Z-Morton key of CSB.hpp:147-173: bits interleaved from the top, the row
 * (y) bit before the column (x) bit at every level. */
static uint64_t zmorton_key(uint32_t row, uint32_t col, int32_t bits) {
    uint64_t k = 0;
    for (int32_t b = bits - 1; b >= 0; --b) {
        k = (k << 1) | ((row >> b) & 1u);
        k = (k << 1) | ((col >> b) & 1u);
    }
    return k;
}

int orc_csb_build(int32_t nor, int32_t noc, int32_t nnz, int32_t* rows, int32_t* cols, double* vals,
                  uint32_t* ind, double* data, int32_t* blk_ptr) {
    /* CSB.hpp:464-567 */
    int32_t beta, bits;
    orc_csb_params(nor, noc, &beta, &bits);
    int32_t hb = (noc + beta - 1) / beta;
    int32_t vb = (nor + beta - 1) / beta;
    sort_row_col(nnz, rows, cols, vals);

    /* Within each block row: stable bucket by block column, then Z-Morton
     * order inside each block; blk_ptr indexed block_row*hb + block_col + 1. */
    keyed_t* kv = (keyed_t*)malloc(sizeof(keyed_t) * (nnz > 0 ? (size_t)nnz : 1));
    for (int64_t i = 0; i < nnz; ++i) {
        uint32_t bc = (uint32_t)cols[i] / (uint32_t)beta;
        uint32_t lr = (uint32_t)rows[i] % (uint32_t)beta, lc = (uint32_t)cols[i] % (uint32_t)beta;
        uint32_t br = (uint32_t)rows[i] / (uint32_t)beta;
        /* key: block row, block col, z-morton within the block (2*16 bits) */
        kv[i].key = ((uint64_t)br << 48) | ((uint64_t)bc << 32) | zmorton_key(lr, lc, bits);
        kv[i].idx = i;
    }
    qsort(kv, nnz, sizeof(keyed_t), cmp_keyed);
    double* brnnz = (double*)calloc(vb > 0 ? (size_t)vb : 1, sizeof(double));
    int64_t nblk = (int64_t)hb * vb;
    for (int64_t b = 0; b <= nblk; ++b) blk_ptr[b] = 0;
    for (int64_t i = 0; i < nnz; ++i) {
        int64_t s = kv[i].idx;
        uint32_t r = (uint32_t)rows[s], c = (uint32_t)cols[s];
        ind[i] = ((r % (uint32_t)beta) << 16) | (c % (uint32_t)beta);
        data[i] = vals[s];
        int64_t blk = (int64_t)(r / (uint32_t)beta) * hb + (c / (uint32_t)beta);
        blk_ptr[blk + 1]++;
        brnnz[r / (uint32_t)beta] += 1.;
    }
    for (int64_t b = 0; b < nblk; ++b) blk_ptr[b + 1] += blk_ptr[b];
    free(kv);

    /* :549-559 balanced unless a block row holds more than twice the mean */
    double sum = 0.;
    for (int32_t i = 0; i < vb; ++i) sum += brnnz[i];
    double avg = sum / vb;
    int balanced = 1;
    for (int32_t i = 0; i < vb; ++i)
        if (brnnz[i] > 2 * avg) { balanced = 0; break; }
    free(brnnz);
    return balanced;
}

void orc_csb_mv(int32_t nor, int32_t noc, const uint32_t* ind, const double* data, const int32_t* blk_ptr,
                const double* x, double* y) {
    /* CSB.hpp:593-605 + sparseRowMult :348-364, storage order per block row.
     * (The reference strides blk_ptr by vertical_blocks at :128, which equals
     * horizontal_blocks for the square matrices it supports.) */
    int32_t beta, bits;
    orc_csb_params(nor, noc, &beta, &bits);
    int32_t hb = (noc + beta - 1) / beta;
    int32_t vb = (nor + beta - 1) / beta;
    for (int32_t br = 0; br < vb; ++br) {
        double* yb = y + (int64_t)br * beta;
        int32_t rend = (br + 1) * (int64_t)beta < nor ? (br + 1) * beta : nor;
        for (int32_t r = br * beta; r < rend; ++r) y[r] = 0.;
        for (int32_t bc = 0; bc < hb; ++bc) {
            int64_t blk = (int64_t)br * hb + bc;
            const double* xb = x + (int64_t)bc * beta;
            for (int32_t i = blk_ptr[blk]; i < blk_ptr[blk + 1]; ++i) {
                uint32_t lr = ind[i] >> 16, lc = ind[i] & 0xFFFFu;
                yb[lr] = yb[lr] + data[i] * xb[lc];
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Block CO-H                                                           */
/* ------------------------------------------------------------------ */

int32_t orc_hilbert(int32_t size, int32_t row, int32_t col) {
    /* BlockCOH.hpp:79-114 */
    int32_t index = 0;
    for (int32_t s = size / 2; s > 0; s /= 2) {
        int32_t rr = (row & s) > 0;
        int32_t cr = (col & s) > 0;
        index += s * s * ((3 * cr) ^ rr);
        if (rr == 0) {
            if (cr == 1) {
                col = size - 1 - col;
                row = size - 1 - row;
            }
            int32_t t = col; col = row; row = t;
        }
    }
    return index;
}

/* BlockCOH.hpp:325-355: partition count adjustment and nnz-balanced split.
 * Returns the partition count; fills part_row_start[p] and part_nnz[p]. */
static int32_t coh_split(int32_t nor, int32_t nnz, const int32_t* rows, int32_t threads,
                         int32_t* part_row_start, int32_t* part_nnz) {
    if (nor / threads < 8) threads = nor / 8;
    if (threads < 1) threads = 1; /* the reference divides by zero here */
    /* Partitions the split never reaches are left empty at row nor (the
     * reference leaves them uninitialised). */
    for (int32_t p = 0; p < threads; ++p) { part_row_start[p] = nor; part_nnz[p] = 0; }
    int32_t* row_nnz = (int32_t*)calloc(nor ? nor : 1, sizeof(int32_t));
    for (int32_t i = 0; i < nnz; ++i) row_nnz[rows[i]]++;
    part_row_start[0] = 0;
    int32_t rsi = 1, row_sum = 0, pid = 0;
    for (int32_t i = 0; i < nor; ++i) {
        row_sum += row_nnz[i];
        if (row_sum > nnz / threads && pid != threads - 1) {
            part_nnz[pid++] = row_sum - row_nnz[i];
            part_row_start[rsi++] = i;
            row_sum = row_nnz[i];
        }
    }
    part_nnz[pid] = row_sum;
    free(row_nnz);
    return threads;
}

static int32_t coh_block_bits(int32_t rows_p, int32_t noc) {
    /* BlockCOH.hpp:119-132 */
    int32_t mx = rows_p > noc ? rows_p : noc;
    int32_t lg = (int32_t)ceil(log2(sqrt((double)mx)));
    return 15 < 3 + lg ? 15 : 3 + lg;
}

int orc_coh_sizes(int32_t nor, int32_t noc, int32_t nnz, const int32_t* rows, const int32_t* cols,
                  int32_t threads, int64_t* total_row_jump, int64_t* total_blocks) {
    /* Upper bounds: one row jump per nonzero, one block per nonzero. */
    (void)noc; (void)cols;
    int32_t* prs = (int32_t*)malloc(sizeof(int32_t) * (threads + 1));
    int32_t* pn = (int32_t*)malloc(sizeof(int32_t) * (threads + 1));
    int32_t t = coh_split(nor, nnz, rows, threads, prs, pn);
    *total_row_jump = nnz;
    *total_blocks = nnz;
    free(prs); free(pn);
    return t;
}

int orc_coh_build(int32_t nor, int32_t noc, int32_t nnz, int32_t* rows, int32_t* cols, double* vals,
                  int32_t threads, int32_t* part_info, uint16_t* row_jump, uint16_t* col_jump, double* data,
                  int32_t* block_nnz, int16_t* row_jump_block, int16_t* col_jump_block) {
    /* BlockCOH.hpp:319-455 */
    int32_t* prs = (int32_t*)malloc(sizeof(int32_t) * (threads + 1));
    int32_t* pn = (int32_t*)malloc(sizeof(int32_t) * (threads + 1));
    int32_t T = coh_split(nor, nnz, rows, threads, prs, pn);
    sort_row_col(nnz, rows, cols, vals);

    int64_t off = 0, rj_off = 0, blk_off = 0, rjb_off = 0;
    for (int32_t p = 0; p < T; ++p) {
        int32_t trs = prs[p];
        int32_t rows_p = (p != T - 1) ? prs[p + 1] - prs[p] : nor - prs[p];
        int32_t bits = coh_block_bits(rows_p, noc);
        int32_t beta = (int32_t)pow(2, bits);
        int32_t hb = (noc + beta - 1) / beta;
        int32_t vb = (rows_p + beta - 1) / beta;
        int32_t np = pn[p];
        int32_t mx = rows_p > noc ? rows_p : noc;
        int32_t hsize = (int32_t)pow(2., ceil(log2((double)mx)));

        /* :400-402 order blocks along the Hilbert curve over the block grid
         * (size hsize/beta); within a block, :204-223 + TripletToICRS order
         * rows then columns. */
        keyed_t* kv = (keyed_t*)malloc(sizeof(keyed_t) * (np > 0 ? (size_t)np : 1));
        for (int32_t i = 0; i < np; ++i) {
            int64_t g = off + i;
            uint32_t br = (uint32_t)(rows[g] - trs) / (uint32_t)beta;
            uint32_t bc = (uint32_t)cols[g] / (uint32_t)beta;
            uint64_t h = (uint32_t)orc_hilbert(hsize / beta, (int32_t)br, (int32_t)bc);
            uint32_t lr = (uint32_t)(rows[g] - trs) % (uint32_t)beta;
            uint32_t lc = (uint32_t)cols[g] % (uint32_t)beta;
            kv[i].key = (h << 32) | ((uint64_t)lr << 16) | lc;
            kv[i].idx = g;
        }
        qsort(kv, np, sizeof(keyed_t), cmp_keyed);
        /* gather in sorted order into the triplet slice (the reference leaves
         * the triplet Hilbert-sorted as well) */
        {
            int32_t* r = (int32_t*)malloc(sizeof(int32_t) * (np > 0 ? (size_t)np : 1));
            int32_t* c = (int32_t*)malloc(sizeof(int32_t) * (np > 0 ? (size_t)np : 1));
            double* v = (double*)malloc(sizeof(double) * (np > 0 ? (size_t)np : 1));
            for (int32_t i = 0; i < np; ++i) { r[i] = rows[kv[i].idx]; c[i] = cols[kv[i].idx]; v[i] = vals[kv[i].idx]; }
            memcpy(rows + off, r, sizeof(int32_t) * np);
            memcpy(cols + off, c, sizeof(int32_t) * np);
            memcpy(vals + off, v, sizeof(double) * np);
            free(r); free(c); free(v);
        }
        free(kv);

        /* ICRS per block (TripletToCRS.hpp:402-452) and BICRS between blocks
         * (BlockCOH.hpp:404-445). */
        int32_t nrj = 0, nblk = 0, nrjb = 0;
        int16_t old_br = 0, old_bc = 0;
        int32_t i = 0;
        while (i < np) {
            int64_t g0 = off + i;
            int32_t br = (rows[g0] - trs) / beta, bc = cols[g0] / beta;
            int32_t j = i;
            while (j < np && (rows[off + j] - trs) / beta == br && cols[off + j] / beta == bc) ++j;
            /* block [i, j) */
            int16_t nbr = (int16_t)br, nbc = (int16_t)bc;
            if (nblk == 0) {
                row_jump_block[rjb_off + nrjb++] = nbr;
                col_jump_block[blk_off + nblk] = nbc;
            } else if (nbr == old_br) {
                col_jump_block[blk_off + nblk] = (int16_t)(nbc - old_bc);
            } else {
                row_jump_block[rjb_off + nrjb++] = (int16_t)(nbr - old_br);
                col_jump_block[blk_off + nblk] = (int16_t)(nbc - old_bc + hb);
            }
            old_br = nbr; old_bc = nbc;
            block_nnz[blk_off + nblk] = j - i;
            nblk++;
            uint16_t prev_r = 0, prev_c = 0;
            for (int32_t e = i; e < j; ++e) {
                int64_t g = off + e;
                uint16_t lr = (uint16_t)((rows[g] - trs) % beta);
                uint16_t lc = (uint16_t)(cols[g] % beta);
                if (e == i) {
                    row_jump[rj_off + nrj++] = lr;
                    col_jump[g] = lc;
                } else if (lr != prev_r) {
                    col_jump[g] = (uint16_t)((lc + beta) - prev_c);
                    row_jump[rj_off + nrj++] = (uint16_t)(lr - prev_r);
                } else {
                    col_jump[g] = (uint16_t)(lc - prev_c);
                }
                data[g] = vals[g];
                prev_r = lr; prev_c = lc;
            }
            i = j;
        }
        int32_t* pi = part_info + 9 * p;
        pi[0] = trs; pi[1] = beta; pi[2] = bits; pi[3] = hb; pi[4] = vb;
        pi[5] = np; pi[6] = nblk; pi[7] = nrj; pi[8] = nrjb;
        off += np; rj_off += nrj; blk_off += nblk; rjb_off += nrjb;
    }
    free(prs); free(pn);
    return T;
}

void orc_coh_mv(int32_t nor, int32_t threads, const int32_t* part_info, const uint16_t* row_jump,
                const uint16_t* col_jump, const double* data, const int32_t* block_nnz,
                const int16_t* row_jump_block, const int16_t* col_jump_block, const double* x, double* y) {
    /* BlockCOH.hpp:479-510 with blockMult :235-256 */
    int64_t off = 0, rj_off = 0, blk_off = 0, rjb_off = 0;
    for (int32_t p = 0; p < threads; ++p) {
        const int32_t* pi = part_info + 9 * p;
        int32_t trs = pi[0], beta = pi[1], hb = pi[3], np = pi[5], nblk = pi[6];
        int32_t rows_p = (p != threads - 1) ? part_info[9 * (p + 1)] - trs : nor - trs;
        for (int32_t r = trs; r < trs + rows_p; ++r) y[r] = 0.;
        const uint16_t* rj = row_jump + rj_off;
        const uint16_t* cj = col_jump + off;
        const double* d = data + off;
        const int32_t* bn = block_nnz + blk_off;
        if (nblk == 0) continue;
        int32_t block_row = row_jump_block[rjb_off], block_col = col_jump_block[blk_off];
        int32_t bri = 1, ri = 0, ci = 0;
        for (int32_t b = 0; b < nblk; ++b) {
            if (b > 0) {
                block_col += col_jump_block[blk_off + b];
                if (block_col >= hb) {
                    block_col -= hb;
                    block_row += row_jump_block[rjb_off + bri++];
                }
            }
            const double* xb = x + (int64_t)block_col * beta;
            double* yb = y + trs + (int64_t)block_row * beta;
            int32_t row = rj[ri], col = cj[ci];
            ri++;
            for (int32_t e = 0; e < bn[b] - 1; ++e) {
                yb[row] += d[ci] * xb[col];
                ci++;
                col += cj[ci];
                if (col >= beta) {
                    col -= beta;
                    row += rj[ri];
                    ri++;
                }
            }
            yb[row] += d[ci] * xb[col];
            ci++;
        }
        off += np; rj_off += pi[7]; blk_off += nblk; rjb_off += pi[8];
    }
}

/* ------------------------------------------------------------------ */
/* Loaders                                                              */
/* ------------------------------------------------------------------ */

int64_t orc_load_mm(const char* filename, int has_data, int symmetric, int32_t* nor, int32_t* noc,
                    int32_t* rows, int32_t* cols, double* vals, int64_t capacity) {
    /* Matrix/Triplet.hpp:75-154: skip '%' lines, read the size line, read
     * entries 1-based; explicit zeros are dropped (:132-134); symmetric files
     * add the transposed off-diagonal entry (:143-148).  Pattern files get 1. */
    FILE* f = fopen(filename, "r");
    if (!f) return -1;
    char line[4096];
    long long nr = 0, nc = 0, ne = 0;
    int have_size = 0;
    while (fgets(line, sizeof line, f)) {
        if (line[0] == '%') continue;
        if (sscanf(line, "%lld %lld %lld", &nr, &nc, &ne) == 3) { have_size = 1; break; }
    }
    if (!have_size) { fclose(f); return -1; }
    *nor = (int32_t)nr; *noc = (int32_t)nc;
    int64_t cap_needed = symmetric ? 2 * ne : ne;
    if (!rows) { fclose(f); return cap_needed; }
    int64_t k = 0;
    while (fgets(line, sizeof line, f)) {
        long long r, c; double v = 1.;
        int got;
        if (line[0] == '\n' || line[0] == '\0') break;
        if (has_data) got = sscanf(line, "%lld %lld %lf", &r, &c, &v);
        else got = sscanf(line, "%lld %lld", &r, &c);
        if (got < 2) break;
        if (has_data && v == 0.) continue;
        if (k >= capacity) { fclose(f); return -2; }
        rows[k] = (int32_t)(r - 1); cols[k] = (int32_t)(c - 1); vals[k] = has_data ? v : 1.;
        ++k;
        if (symmetric && r != c) {
            if (k >= capacity) { fclose(f); return -2; }
            rows[k] = (int32_t)(c - 1); cols[k] = (int32_t)(r - 1); vals[k] = vals[k - 1];
            ++k;
        }
    }
    fclose(f);
    return k;
}

int64_t orc_load_bin(const char* filename, int32_t mat_size, int symmetric, int32_t* rows, int32_t* cols,
                     double* vals, int64_t capacity) {
    /* Matrix/Triplet.hpp:164-216: uint32 (row, col) pairs, 0-based, value 1.
     * (The reference keeps reading past the end of a symmetric file that holds
     * diagonal entries; this restatement stops at end of file.) */
    (void)mat_size;
    struct stat st;
    if (stat(filename, &st) != 0) return -1;
    int64_t pairs = (int64_t)st.st_size / 8;
    int64_t cap_needed = symmetric ? 2 * pairs : pairs;
    if (!rows) return cap_needed;
    FILE* f = fopen(filename, "rb");
    if (!f) return -1;
    int64_t k = 0;
    for (int64_t p = 0; p < pairs; ++p) {
        uint32_t rc[2];
        if (fread(rc, sizeof(uint32_t), 2, f) != 2) break;
        if (k >= capacity) { fclose(f); return -2; }
        rows[k] = (int32_t)rc[0]; cols[k] = (int32_t)rc[1]; vals[k] = 1.;
        ++k;
        if (symmetric && rc[0] != rc[1]) {
            if (k >= capacity) { fclose(f); return -2; }
            rows[k] = (int32_t)rc[1]; cols[k] = (int32_t)rc[0]; vals[k] = 1.;
            ++k;
        }
    }
    fclose(f);
    return k;
}

/* ------------------------------------------------------------------ */
/* Seeded random matrices (benchmark inputs; no reference counterpart)  */
/* ------------------------------------------------------------------ */
/* Host restatement of the library's device generator (row lengths from a
 * CDF table scaled by 2^53, stratified uniform and band columns merged
 * without duplicates, values from a hash of (row, column)); the hash is the
 * splitmix64 finaliser (Steele, Lea, Flood 2014) applied twice. */

static uint64_t rg_mix(uint64_t z) {
    z ^= z >> 30;
    z *= 0xbf58476d1ce4e5b9ull;
    z ^= z >> 27;
    z *= 0x94d049bb133111ebull;
    z ^= z >> 31;
    return z;
}

static uint64_t rg_hash(uint64_t seed, uint64_t i, uint64_t k) {
    const uint64_t g = 0x9e3779b97f4a7c15ull;
    return rg_mix(rg_mix(seed + g * (i + 1)) + g * (k + 1));
}

void orc_random_table(int kind, double mean, double sigma, int32_t max_len, uint64_t* thr) {
    const double two53 = 9007199254740992.0;
    double cdf = 0., pmf = 0.;
    double mu = log(mean) - 0.5 * sigma * sigma;
    for (int32_t l = 0; l <= max_len; ++l) thr[l] = (uint64_t)1 << 53;
    for (int32_t l = 0; l < max_len; ++l) {
        if (kind == 0) {
            /* P(round(exp(mu + sigma Z)) <= l) = Phi((ln(l + 1/2) - mu) / sigma) */
            cdf = l == 0 ? 0. : 0.5 * erfc(-((log(l + 0.5) - mu) / sigma) * 0.70710678118654752440);
        } else {
            pmf = l == 0 ? exp(-mean) : pmf * mean / l;
            cdf = cdf + pmf;
        }
        double t = floor(cdf * two53);
        thr[l] = t >= two53 ? ((uint64_t)1 << 53) : (uint64_t)t;
    }
}

typedef struct {
    const uint64_t* thr;
    int32_t max_len, n;
    uint64_t seed;
    int32_t band_permille, band_half;
} orc_rowgen;

static int32_t rg_row(const orc_rowgen* g, int32_t i, int32_t* col, double* val) {
    uint64_t u = rg_hash(g->seed, (uint64_t)i, 0) >> 11;
    int32_t lo = 0, hi = g->max_len;
    while (lo < hi) { /* smallest l with u < thr[l] */
        int32_t mid = (lo + hi) / 2;
        if (u < g->thr[mid]) hi = mid;
        else lo = mid + 1;
    }
    long long L = lo;
    int32_t b0 = i - g->band_half > 0 ? i - g->band_half : 0;
    int32_t b1 = i + (long long)g->band_half < g->n - 1 ? i + g->band_half : g->n - 1;
    long long wb = (long long)b1 - b0 + 1;
    long long lb = 0, lu;
    if (g->band_permille > 0) lb = (L * g->band_permille + (long long)(rg_hash(g->seed, (uint64_t)i, 1) % 1000)) / 1000;
    if (lb > wb) lb = wb;
    lu = L - lb;
    if (lu > g->n) lu = g->n;
    /* the two stratified parts, each sorted, merged */
    long long ju = 0, jb = 0;
    int32_t cnt = 0;
    while (ju < lu || jb < lb) {
        long long cu = 0, cb = 0;
        if (ju < lu) {
            long long l0 = ju * g->n / lu, h0 = (ju + 1) * g->n / lu;
            cu = l0 + (long long)(rg_hash(g->seed, (uint64_t)i, (uint64_t)(2 + 2 * ju)) % (uint64_t)(h0 - l0));
        }
        if (jb < lb) {
            long long l0 = b0 + jb * wb / lb, h0 = b0 + (jb + 1) * wb / lb;
            cb = l0 + (long long)(rg_hash(g->seed, (uint64_t)i, (uint64_t)(3 + 2 * jb)) % (uint64_t)(h0 - l0));
        }
        long long c;
        if (jb >= lb || (ju < lu && cu < cb)) { c = cu; ++ju; }
        else if (ju >= lu || cb < cu) { c = cb; ++jb; }
        else { c = cu; ++ju; ++jb; }
        if (col) {
            col[cnt] = (int32_t)c;
            val[cnt] = (double)((rg_hash(g->seed ^ 0xd6e8feb86659fd93ull, (uint64_t)i, (uint64_t)c) >> 11) + 1) *
                       (1.0 / 9007199254740992.0);
        }
        ++cnt;
    }
    return cnt;
}

int64_t orc_random_crs(int32_t n, uint64_t seed, int kind, double mean, double sigma, int32_t max_len,
                       int32_t band_permille, int32_t band_half, int32_t* row_start, int32_t* col_ind,
                       double* data) {
    uint64_t* thr = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)max_len + 1));
    orc_random_table(kind, mean, sigma, max_len, thr);
    orc_rowgen g = {thr, max_len, n, seed, band_permille, band_half};
    int64_t nnz = 0;
    if (row_start) row_start[0] = 0;
    for (int32_t i = 0; i < n; ++i) {
        int32_t c = rg_row(&g, i, col_ind ? col_ind + nnz : NULL, data ? data + nnz : NULL);
        nnz += c;
        if (row_start) row_start[i + 1] = (int32_t)nnz;
    }
    free(thr);
    return nnz;
}

void orc_uniform_vector(int32_t n, uint64_t seed, double* x) {
    /* the service's seeded start vector: x[i] = (mix(seed + g (i + 1)) >> 11) 2^-53 */
    for (int32_t i = 0; i < n; ++i)
        x[i] = (double)(rg_mix(seed + 0x9e3779b97f4a7c15ull * (uint64_t)(i + 1)) >> 11) * (1.0 / 9007199254740992.0);
}

/* ------------------------------------------------------------------ */
/* Matrix statistics                                                    */
/* ------------------------------------------------------------------ */

int orc_calc_stats(int64_t nnz, int32_t nor, const int32_t* rows, const int32_t* cols, double* out) {
    /* Util_Scripts/calc_stats.cpp:45-98 with index_t = uint32_t
     * (Util/Constants.hpp:38): counters are uint32, each variance term is
     * pow(count - avg, 2) / n (x * x here: both correctly rounded), summed in
     * the script's loop order. */
    const uint32_t n = (uint32_t)nor;
    const double rows_avg = (double)nnz / (double)n;
    const uint32_t lg = (uint32_t)ceil(log2(sqrt((double)n)));
    const uint32_t bits = 3 + lg < 16 ? 3 + lg : 16;
    const uint32_t bs = (uint32_t)1 << bits;
    uint32_t nb = n / bs + (n % bs != 0);
    uint32_t* rows_nnz = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    uint32_t* block_nnz = (uint32_t*)calloc((size_t)nb * nb ? (size_t)nb * nb : 1, sizeof(uint32_t));
    if (!rows_nnz || !block_nnz) {
        free(rows_nnz);
        free(block_nnz);
        return -1;
    }
    for (int64_t k = 0; k < nnz; ++k) {
        const uint32_t r = (uint32_t)rows[k], c = (uint32_t)cols[k];
        if (r / bs >= nb || c / bs >= nb) {
            free(rows_nnz);
            free(block_nnz);
            return -1;
        }
        rows_nnz[r]++;
        block_nnz[(size_t)(r / bs) * nb + c / bs]++;
    }
    double rows_var = 0.;
    for (uint32_t i = 0; i < n; ++i) {
        const double d = (double)rows_nnz[i] - rows_avg;
        rows_var += d * d / (double)n;
    }
    const uint32_t stride = nb;
    if (n % bs != 0) nb--;
    const double nb2 = (double)nb * (double)nb;
    double block_avg = 0., block_row_avg = 0.;
    uint32_t* block_row_nnz = (uint32_t*)calloc(nb ? nb : 1, sizeof(uint32_t));
    for (uint32_t i = 0; i < nb; ++i) {
        for (uint32_t j = 0; j < nb; ++j) {
            block_row_nnz[i] += block_nnz[(size_t)i * stride + j];
            block_avg += (double)block_nnz[(size_t)i * stride + j] / nb2;
        }
        block_row_avg += (double)block_row_nnz[i] / (double)nb;
    }
    double block_var = 0.;
    int balanced = 1;
    for (uint32_t i = 0; i < nb; ++i) {
        if ((double)block_row_nnz[i] > 2 * block_row_avg) balanced = 0;
        for (uint32_t j = 0; j < nb; ++j) {
            const double d = (double)block_nnz[(size_t)i * stride + j] - block_avg;
            block_var += d * d / nb2;
        }
    }
    out[0] = (double)n;
    out[1] = (double)nnz;
    out[2] = rows_avg;
    out[3] = rows_var;
    out[4] = block_avg;
    out[5] = block_var;
    out[6] = balanced;
    out[7] = bits;
    out[8] = nb;
    free(rows_nnz);
    free(block_nnz);
    free(block_row_nnz);
    return 0;
}
