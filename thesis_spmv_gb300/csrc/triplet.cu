// triplet.cu -- triplet (COO) -> CRS on the device, in the order of
// Util/TripletToCRS.hpp:135-172: rows ascending, columns ascending within a
// row.  For unique coordinates that order is unique; entries with the same
// (row, column) keep their input order (a stable sort), which is also what the
// host counting sort of the previous loader gave.
//
// Plan (all passes are HBM streams; no comparison sort):
//   1. k_trip_scan: one read of rows / cols.  Range check (the first bad entry
//      by atomicMin), per-row counts (warp-aggregated atomics; their scan is
//      row_start), and two order flags: "not sorted by (row, col)" and "not
//      sorted by column".
//   2. Already sorted by (row, col): col / val are the input, copied.
//   3. Otherwise a stable LSD radix sort of the packed key row << 32 | col
//      with 8-bit digits: first the column digits (skipped when the input is
//      already sorted by column -- a stable sort by a key that is already in
//      order is the identity), then the row digits.  Per pass: k_radix_hist
//      counts digits per 4096-item tile into a digit-major table (one
//      inclusive scan makes it the exclusive offsets of every (digit, tile)),
//      and k_radix_scatter ranks each tile's items stably (warp match on the
//      digit, per-warp digit counters in shared memory) and writes key and
//      source index to their places.
//   4. k_trip_gather: col = low word of the sorted key, val = vals[source],
//      and optionally the sorted rows (for callers whose triplet is sorted in
//      place, like the reference's).
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace pwmgpu {

namespace {

constexpr int kRadixBins = 256;
constexpr int kSortWarps = 8;
constexpr int kSortThreads = kSortWarps * 32;
constexpr int kSortRounds = 16;                           // rounds of 32 items per warp
constexpr int kSortTile = kSortThreads * kSortRounds;     // 4096 items per CTA
constexpr int kWarpItems = 32 * kSortRounds;              // 512 consecutive items per warp

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Pass 1.  cnt has nor + 1 zeroed entries; the count of row r goes to
// cnt[r + 1] so that an inclusive scan of cnt + 1 leaves row_start in cnt.
__global__ void k_trip_scan(const int32_t* __restrict__ rows, const int32_t* __restrict__ cols, long long nnz,
                            int32_t nor, int32_t noc, int32_t* __restrict__ cnt, TripletScan* flags) {
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    bool unsorted_rc = false, unsorted_c = false;
    // whole warps walk the array so that the neighbour exchange stays in-warp
    const long long start = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long span = (nnz + 31) / 32 * 32;
    for (long long k = start; k < span; k += stride) {
        const bool in = k < nnz;
        const int32_t r = in ? rows[k] : 0;
        const int32_t c = in ? cols[k] : 0;
        int32_t pr = __shfl_up_sync(0xffffffffu, r, 1);
        int32_t pc = __shfl_up_sync(0xffffffffu, c, 1);
        if (lane == 0 && in && k > 0) {
            pr = rows[k - 1];
            pc = cols[k - 1];
        }
        if (in && k > 0) {
            unsorted_rc |= r < pr || (r == pr && c < pc);
            unsorted_c |= c < pc;
        }
        const bool ok = in && r >= 0 && r < nor && c >= 0 && c < noc;
        if (in && !ok) atomicMin(&flags->bad, (unsigned long long)k);
        // rows of a warp are often equal (sorted input): one atomic per row
        const int key = ok ? r : -1 - lane;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (ok && lane == __ffs(peers) - 1) atomicAdd(&cnt[r + 1], __popc(peers));
    }
    if (__any_sync(0xffffffffu, unsorted_rc) && lane == 0) atomicOr(&flags->unsorted_rc, 1u);
    if (__any_sync(0xffffffffu, unsorted_c) && lane == 0) atomicOr(&flags->unsorted_c, 1u);
}

__global__ void k_trip_pack(const int32_t* __restrict__ rows, const int32_t* __restrict__ cols, long long nnz,
                            unsigned long long* __restrict__ keys, int32_t* __restrict__ src) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += stride) {
        keys[k] = ((unsigned long long)(uint32_t)rows[k] << 32) | (uint32_t)cols[k];
        src[k] = (int32_t)k;
    }
}

__device__ __forceinline__ int digit_of(unsigned long long key, int shift) { return (int)(key >> shift) & 0xff; }

// Digit counts of one tile: tab[1 + d * tiles + tile] (tab[0] = 0 is the
// leading zero of the exclusive offsets).
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const unsigned long long* __restrict__ keys, long long n,
                                                             int shift, int32_t* __restrict__ tab, int tiles) {
    __shared__ int h[kRadixBins];
    const int lane = threadIdx.x & 31;
    h[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kSortTile;
#pragma unroll 4
    for (int r = 0; r < kSortRounds; ++r) {
        const long long k = base + (long long)r * kSortThreads + threadIdx.x;
        const bool in = k < n;
        const int d = in ? digit_of(keys[k], shift) : 0x100 | lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (in && lane == __ffs(peers) - 1) atomicAdd(&h[d & (kRadixBins - 1)], __popc(peers));
    }
    __syncthreads();
    tab[1 + (long long)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
    if (blockIdx.x == 0 && threadIdx.x == 0) tab[0] = 0;
}

// Stable scatter of one tile.  Warp w owns items [base + 512 w, base + 512 (w+1))
// in rounds of 32 consecutive items, so (warp, round, lane) order is the
// items' order; an item's place is the (digit, tile) offset + the same-digit
// items of earlier warps + of earlier rounds of its warp + of lower lanes.
__global__ void __launch_bounds__(kSortThreads, 3) k_radix_scatter(const unsigned long long* __restrict__ keys_in,
                                                                const int32_t* __restrict__ src_in, long long n,
                                                                int shift, const int32_t* __restrict__ tab, int tiles,
                                                                unsigned long long* __restrict__ keys_out,
                                                                int32_t* __restrict__ src_out) {
    __shared__ int wc[kSortWarps][kRadixBins];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < kSortWarps; ++i) wc[i][threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kSortTile + (long long)w * kWarpItems;
    unsigned long long key[kSortRounds];
    int32_t src[kSortRounds];
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        const long long k = base + r * 32 + lane;
        const bool in = k < n;
        key[r] = in ? keys_in[k] : 0ull;
        src[r] = in ? src_in[k] : 0;
        const int d = in ? digit_of(key[r], shift) : 0x100 | lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (in && lane == __ffs(peers) - 1) wc[w][d & (kRadixBins - 1)] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        const int d = threadIdx.x;
        int run = tab[(long long)d * tiles + blockIdx.x];
#pragma unroll
        for (int i = 0; i < kSortWarps; ++i) {
            const int c = wc[i][d];
            wc[i][d] = run;
            run += c;
        }
    }
    __syncthreads();
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        const long long k = base + r * 32 + lane;
        const bool in = k < n;
        const int d = in ? digit_of(key[r], shift) : 0x100 | lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int dd = d & (kRadixBins - 1);  // == d for items in range
        const int at = in ? wc[w][dd] + __popc(peers & lt) : 0;
        __syncwarp();
        if (in && lane == __ffs(peers) - 1) wc[w][dd] += __popc(peers);
        __syncwarp();
        if (in) {
            keys_out[at] = key[r];
            src_out[at] = src[r];
        }
    }
}

__global__ void k_trip_gather(const unsigned long long* __restrict__ keys, const int32_t* src, const double* vals,
                              long long nnz, int32_t* __restrict__ col, double* __restrict__ val, int32_t* rows_out) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += stride) {
        const unsigned long long key = keys[k];
        const int32_t s = src[k];
        col[k] = (int32_t)(uint32_t)key;
        val[k] = vals[s];
        if (rows_out) rows_out[k] = (int32_t)(key >> 32);  // may alias src: same k, read above
    }
}

int bits_for(long long extent) {
    int b = 0;
    while (b < 32 && (1LL << b) < extent) ++b;
    return b;
}

int stream_grid(long long n, int sm_count) {
    long long b = (n + 255) / 256;
    const long long cap = (long long)sm_count * 8;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t launch_triplet_scan(const int32_t* rows, const int32_t* cols, long long nnz, int32_t nor, int32_t noc,
                                int32_t* cnt, TripletScan* flags, int sm_count, cudaStream_t st) {
    if (nnz <= 0) return cudaSuccess;
    k_trip_scan<<<stream_grid(nnz, sm_count), 256, 0, st>>>(rows, cols, nnz, nor, noc, cnt, flags);
    return cudaGetLastError();
}

long long triplet_sort_table_elems(long long nnz) {
    const long long tiles = (nnz + kSortTile - 1) / kSortTile;
    return tiles * kRadixBins + 1;
}

int triplet_sort_passes(int32_t nor, int32_t noc, bool col_passes) {
    return (col_passes ? (bits_for(noc) + 7) / 8 : 0) + (bits_for(nor) + 7) / 8;
}

cudaError_t launch_triplet_sort(const int32_t* rows, const int32_t* cols, long long nnz, int32_t nor, int32_t noc,
                                bool col_passes, unsigned long long* keys_a, int32_t* src_a,
                                unsigned long long* keys_b, int32_t* src_b, int32_t* tab, int32_t* scan_scratch,
                                unsigned long long** keys_sorted, int32_t** src_sorted, int sm_count,
                                cudaStream_t st) {
    *keys_sorted = keys_a;
    *src_sorted = src_a;
    if (nnz <= 0) return cudaSuccess;
    k_trip_pack<<<stream_grid(nnz, sm_count), 256, 0, st>>>(rows, cols, nnz, keys_a, src_a);
    const long long tiles = (nnz + kSortTile - 1) / kSortTile;
    int shifts[8], np = 0;
    if (col_passes)
        for (int s = 0; s < bits_for(noc); s += 8) shifts[np++] = s;
    for (int s = 0; s < bits_for(nor); s += 8) shifts[np++] = 32 + s;
    unsigned long long *ki = keys_a, *ko = keys_b;
    int32_t *si = src_a, *so = src_b;
    for (int p = 0; p < np; ++p) {
        k_radix_hist<<<(unsigned)tiles, kSortThreads, 0, st>>>(ki, nnz, shifts[p], tab, (int)tiles);
        cudaError_t e = launch_inclusive_scan(tab + 1, tiles * kRadixBins, scan_scratch, st);
        if (e != cudaSuccess) return e;
        k_radix_scatter<<<(unsigned)tiles, kSortThreads, 0, st>>>(ki, si, nnz, shifts[p], tab, (int)tiles, ko, so);
        unsigned long long* kt = ki;
        ki = ko;
        ko = kt;
        int32_t* t = si;
        si = so;
        so = t;
    }
    *keys_sorted = ki;
    *src_sorted = si;
    return cudaGetLastError();
}

cudaError_t launch_triplet_gather(const unsigned long long* keys, const int32_t* src, const double* vals,
                                  long long nnz, int32_t* col, double* val, int32_t* rows_out, int sm_count,
                                  cudaStream_t st) {
    if (nnz <= 0) return cudaSuccess;
    k_trip_gather<<<stream_grid(nnz, sm_count), 256, 0, st>>>(keys, src, vals, nnz, col, val, rows_out);
    return cudaGetLastError();
}

}  // namespace pwmgpu
