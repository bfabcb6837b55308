// stats.cu -- matrix statistics of Util_Scripts/calc_stats.cpp:45-98 on the
// device, from the CRS arrays: nonzeros per row (mean, population variance),
// nonzeros per block over the whole blocks of a square block grid (block side
// 2^min(16, 3 + ceil(log2 sqrt(n)))), and the "balanced for CSB" flag (no
// block row holds more than twice the average block row).
//
// Integer counts are exact.  The floating-point figures follow the script's
// formulas; sums run in a fixed parallel order (per-CTA tree, then one CTA),
// so they are deterministic but not in the script's sequential order -- except
// the average block row, which one thread sums in the script's order so that
// the balance flag compares the same double.  The block mean is the correctly
// rounded total / nb^2 (the script accumulates total terms of count / nb^2).
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace pwmgpu {

namespace {

constexpr int kStatThreads = 256;
constexpr int kStatRows = 16384;      // rows per CTA of the row pass (fixed: deterministic sums)
constexpr int kStatSegRows = 4096;    // rows per CTA of the block-count pass
constexpr int kStatSmemBlocks = 4096; // block grids up to this side count in shared memory

__device__ double block_sum_f64(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = kStatThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__device__ long long block_sum_i64(long long v, long long* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = kStatThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    const long long r = sh[0];
    __syncthreads();
    return r;
}

// Per CTA: sum over its rows of ((count - avg)^2) / n, and the longest row.
__global__ void __launch_bounds__(kStatThreads) k_stats_rows(const int32_t* __restrict__ row_start, int n,
                                                             double avg, double* partials, StatsDev* out) {
    __shared__ double sh[kStatThreads];
    const long long lo = (long long)blockIdx.x * kStatRows;
    const long long hi = lo + kStatRows < n ? lo + kStatRows : n;
    double acc = 0.0;
    int longest = 0;
    for (long long i = lo + threadIdx.x; i < hi; i += kStatThreads) {
        const int c = row_start[i + 1] - row_start[i];
        const double d = (double)c - avg;
        acc += d * d / (double)n;
        longest = c > longest ? c : longest;
    }
    acc = block_sum_f64(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
    for (int o = 16; o > 0; o >>= 1) longest = max(longest, __shfl_xor_sync(0xffffffffu, longest, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&out->max_row_nnz, longest);
}

// Nonzero counts of the whole blocks: CTA (row block rb, segment of
// kStatSegRows rows); columns outside the whole blocks are not counted.
template <bool SMEM>
__global__ void __launch_bounds__(kStatThreads) k_stats_blocks(const int32_t* __restrict__ row_start,
                                                               const int32_t* __restrict__ col, int bits, int nbw,
                                                               int segs, unsigned int* __restrict__ blocks) {
    extern __shared__ unsigned int hist[];
    const int lane = threadIdx.x & 31;
    const int rb = blockIdx.x / segs, sg = blockIdx.x % segs;
    const long long r0 = ((long long)rb << bits) + (long long)sg * kStatSegRows;
    long long r1 = r0 + kStatSegRows;
    const long long rb_end = (long long)(rb + 1) << bits;
    if (r1 > rb_end) r1 = rb_end;
    if (SMEM) {
        for (int j = threadIdx.x; j < nbw; j += kStatThreads) hist[j] = 0;
        __syncthreads();
    }
    const long long k0 = row_start[r0], k1 = row_start[r1];
    unsigned int* row_blocks = blocks + (size_t)rb * nbw;
    // whole warps walk the range (the match needs every lane)
    const long long span = (k1 - k0 + 31) / 32 * 32;
    for (long long t = threadIdx.x; t < span; t += kStatThreads) {
        const long long k = k0 + t;
        const int cb = k < k1 ? (col[k] >> bits) : nbw;
        const bool in = cb < nbw;
        const int key = in ? cb : -1 - lane;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (in && lane == __ffs(peers) - 1) {
            if (SMEM)
                atomicAdd(&hist[cb], (unsigned)__popc(peers));
            else
                atomicAdd(&row_blocks[cb], (unsigned)__popc(peers));
        }
    }
    if (SMEM) {
        __syncthreads();
        for (int j = threadIdx.x; j < nbw; j += kStatThreads)
            if (hist[j]) atomicAdd(&row_blocks[j], hist[j]);
    }
}

// Per block row: its nonzeros (exact).
__global__ void __launch_bounds__(kStatThreads) k_stats_block_rows(const unsigned int* __restrict__ blocks, int nbw,
                                                                   long long* __restrict__ brow) {
    __shared__ long long sh[kStatThreads];
    const unsigned int* b = blocks + (size_t)blockIdx.x * nbw;
    long long s = 0;
    for (int j = threadIdx.x; j < nbw; j += kStatThreads) s += b[j];
    s = block_sum_i64(s, sh);
    if (threadIdx.x == 0) brow[blockIdx.x] = s;
}

// One CTA: the row variance from the partials, the block mean, the average
// block row (thread 0, the script's order) and the balance flag.
__global__ void __launch_bounds__(kStatThreads) k_stats_mid(const double* __restrict__ row_partials, int nrp,
                                                            const long long* __restrict__ brow, int nbw,
                                                            StatsDev* out) {
    __shared__ double shd[kStatThreads];
    __shared__ long long shl[kStatThreads];
    double v = 0.0;
    for (int i = threadIdx.x; i < nrp; i += kStatThreads) v += row_partials[i];
    v = block_sum_f64(v, shd);
    long long t = 0;
    for (int i = threadIdx.x; i < nbw; i += kStatThreads) t += brow[i];
    t = block_sum_i64(t, shl);
    if (threadIdx.x == 0) {
        out->rows_var = v;
        const double nb = (double)nbw, nb2 = nb * nb;
        out->block_avg = nbw > 0 ? (double)t / nb2 : 0.0;
        double avg_row = 0.0;
        for (int i = 0; i < nbw; ++i) avg_row += (double)brow[i] / nb;
        int balanced = 1;
        for (int i = 0; i < nbw; ++i)
            if ((double)brow[i] > 2 * avg_row) balanced = 0;
        out->balanced = balanced;
    }
}

// Per block row: sum over its whole blocks of (count - mean)^2 / nb^2.
__global__ void __launch_bounds__(kStatThreads) k_stats_block_var(const unsigned int* __restrict__ blocks, int nbw,
                                                                  const StatsDev* st, double* partials) {
    __shared__ double sh[kStatThreads];
    const double avg = st->block_avg;
    const double nb2 = (double)nbw * (double)nbw;
    const unsigned int* b = blocks + (size_t)blockIdx.x * nbw;
    double acc = 0.0;
    for (int j = threadIdx.x; j < nbw; j += kStatThreads) {
        const double d = (double)b[j] - avg;
        acc += d * d / nb2;
    }
    acc = block_sum_f64(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kStatThreads) k_stats_final(const double* __restrict__ partials, int np,
                                                              StatsDev* out) {
    __shared__ double sh[kStatThreads];
    double v = 0.0;
    for (int i = threadIdx.x; i < np; i += kStatThreads) v += partials[i];
    v = block_sum_f64(v, sh);
    if (threadIdx.x == 0) out->block_var = v;
}

}  // namespace

int stats_row_ctas(int n) { return (n + kStatRows - 1) / kStatRows; }

cudaError_t launch_matrix_stats(const int32_t* row_start, const int32_t* col, int n, double avg, int bits, int nbw,
                                unsigned int* blocks, long long* brow, double* row_partials, double* blk_partials,
                                StatsDev* out, cudaStream_t st) {
    const int nrp = stats_row_ctas(n);
    k_stats_rows<<<nrp, kStatThreads, 0, st>>>(row_start, n, avg, row_partials, out);
    if (nbw > 0) {
        const int bs = 1 << bits;
        const int segs = (bs + kStatSegRows - 1) / kStatSegRows;
        const unsigned grid = (unsigned)((long long)nbw * segs);
        if (nbw <= kStatSmemBlocks) {
            k_stats_blocks<true><<<grid, kStatThreads, (size_t)nbw * sizeof(unsigned int), st>>>(row_start, col, bits,
                                                                                               nbw, segs, blocks);
        } else {
            k_stats_blocks<false><<<grid, kStatThreads, 0, st>>>(row_start, col, bits, nbw, segs, blocks);
        }
        k_stats_block_rows<<<nbw, kStatThreads, 0, st>>>(blocks, nbw, brow);
    }
    k_stats_mid<<<1, kStatThreads, 0, st>>>(row_partials, nrp, brow, nbw, out);
    if (nbw > 0) {
        k_stats_block_var<<<nbw, kStatThreads, 0, st>>>(blocks, nbw, out, blk_partials);
        k_stats_final<<<1, kStatThreads, 0, st>>>(blk_partials, nbw, out);
    }
    return cudaGetLastError();
}

}  // namespace pwmgpu
