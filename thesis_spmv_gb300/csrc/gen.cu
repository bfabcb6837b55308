// gen.cu -- device generator of seeded random sparse matrices (the irregular
// and batch workloads of the benchmarks; no counterpart in the reference,
// whose drivers read matrices from files or build Poisson grids).
//
// Row i of an n x n matrix, seed s (all integer arithmetic, so the oracle's
// C restatement reproduces the arrays bit for bit):
//   length   L_i = smallest l with u < thr[l], u = H(s, i, 0) >> 11 (53 bits),
//            thr[] the distribution's CDF scaled by 2^53 (host-built table:
//            lognormal rounded and clipped, or Poisson);
//   band     L_b = (L_i * band_permille + H(s, i, 1) % 1000) / 1000 columns
//            in [i - band_half, i + band_half] (clipped), the rest L_u in
//            [0, n); each part is stratified: stratum j of a range of width
//            W with k strata is [j W / k, (j+1) W / k) and its column is the
//            stratum's start + H(s, i, 2 + 2j (+1 for the band)) mod width --
//            so each part comes out sorted and duplicate-free;
//   columns  the sorted merge of the two parts, a column in both kept once;
//   values   (H(s ^ kValSalt, i, col) >> 11) + 1) * 2^-53, in (0, 1].
// H is the splitmix64 finaliser (Steele, Lea, Flood 2014) applied twice.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "internal.h"

namespace pwmgpu {

namespace {

constexpr uint64_t kGolden = 0x9e3779b97f4a7c15ull;
constexpr uint64_t kValSalt = 0xd6e8feb86659fd93ull;
constexpr uint64_t kTwo53 = 1ull << 53;

__host__ __device__ __forceinline__ uint64_t rg_mix(uint64_t z) {
    z ^= z >> 30;
    z *= 0xbf58476d1ce4e5b9ull;
    z ^= z >> 27;
    z *= 0x94d049bb133111ebull;
    z ^= z >> 31;
    return z;
}

__host__ __device__ __forceinline__ uint64_t rg_hash(uint64_t seed, uint64_t i, uint64_t k) {
    return rg_mix(rg_mix(seed + kGolden * (i + 1)) + kGolden * (k + 1));
}

struct RowGen {
    const uint64_t* thr;
    int max_len;
    int n;
    uint64_t seed;
    int band_permille, band_half;
};

// Column j of the uniform part (Lu strata of [0, n)) or of the band part
// (Lb strata of [b0, b0 + wb)).
__device__ __forceinline__ int ucol(const RowGen& g, int i, long long j, long long lu) {
    const long long lo = j * g.n / lu, hi = (j + 1) * g.n / lu;
    return (int)(lo + (long long)(rg_hash(g.seed, i, 2 + 2 * j) % (uint64_t)(hi - lo)));
}
__device__ __forceinline__ int bcol(const RowGen& g, int i, long long j, long long lb, int b0, long long wb) {
    const long long lo = b0 + j * wb / lb, hi = b0 + (j + 1) * wb / lb;
    return (int)(lo + (long long)(rg_hash(g.seed, i, 3 + 2 * j) % (uint64_t)(hi - lo)));
}

// Generate row i: count its columns, and with WRITE store them (and the
// values) at col[base..], val[base..].
template <bool WRITE>
__device__ int gen_row(const RowGen& g, int i, int32_t* col, double* val, long long base) {
    const uint64_t u = rg_hash(g.seed, i, 0) >> 11;
    int lo = 0, hi = g.max_len;  // smallest l in [0, max_len] with u < thr[l]
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (u < __ldg(g.thr + mid)) hi = mid;
        else lo = mid + 1;
    }
    const long long L = lo;
    const int b0 = i - g.band_half > 0 ? i - g.band_half : 0;
    const int b1 = (long long)i + g.band_half < g.n - 1 ? i + g.band_half : g.n - 1;
    const long long wb = (long long)b1 - b0 + 1;
    long long lb = g.band_permille > 0 ? (L * g.band_permille + (long long)(rg_hash(g.seed, i, 1) % 1000)) / 1000 : 0;
    if (lb > wb) lb = wb;
    long long lu = L - lb;
    if (lu > g.n) lu = g.n;
    long long ju = 0, jb = 0;
    int cu = lu > 0 ? ucol(g, i, 0, lu) : 0;
    int cb = lb > 0 ? bcol(g, i, 0, lb, b0, wb) : 0;
    int cnt = 0;
    while (ju < lu || jb < lb) {
        int c;
        if (jb >= lb || (ju < lu && cu < cb)) {
            c = cu;
            if (++ju < lu) cu = ucol(g, i, ju, lu);
        } else if (ju >= lu || cb < cu) {
            c = cb;
            if (++jb < lb) cb = bcol(g, i, jb, lb, b0, wb);
        } else {  // the same column in both parts: once
            c = cu;
            if (++ju < lu) cu = ucol(g, i, ju, lu);
            if (++jb < lb) cb = bcol(g, i, jb, lb, b0, wb);
        }
        if (WRITE) {
            col[base + cnt] = c;
            val[base + cnt] = (double)((rg_hash(g.seed ^ kValSalt, i, (uint64_t)c) >> 11) + 1) * 0x1.0p-53;
        }
        ++cnt;
    }
    return cnt;
}

__global__ void k_rand_count(RowGen g, int32_t* __restrict__ row_start, unsigned long long* total) {
    unsigned long long local = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const int c = gen_row<false>(g, i, nullptr, nullptr, 0);
        row_start[i + 1] = c;
        local += (unsigned long long)c;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(total, local);
    if (blockIdx.x == 0 && threadIdx.x == 0) row_start[0] = 0;
}

__global__ void k_rand_fill(RowGen g, const int32_t* __restrict__ row_start, int32_t* __restrict__ col,
                            double* __restrict__ val) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x)
        gen_row<true>(g, i, col, val, row_start[i]);
}

// ---- in-place inclusive scan of int32 (three passes: tiles, tile sums, add)
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_incl_scan(int v, int* warp_sums) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[w] = v;
    __syncthreads();
    if (w == 0) {
        int s = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    const int r = v + (w > 0 ? warp_sums[w - 1] : 0);
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(int32_t* a, long long n, int32_t* tile_sums) {
    __shared__ int ws[32];
    const long long t0 = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = t0 + k < n ? a[t0 + k] : 0;
        s += v[k];
    }
    const int incl = block_incl_scan(s, ws);
    int run = incl - s;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        run += v[k];
        if (t0 + k < n) a[t0 + k] = run;
    }
    if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = incl;
}

// Exclusive scan of the tile sums by one CTA (a running carry across chunks).
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int32_t* s, int nt) {
    __shared__ int ws[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nt; base += kScanThreads) {
        const int i = base + threadIdx.x;
        const int v = i < nt ? s[i] : 0;
        const int incl = block_incl_scan(v, ws);
        const int c = carry;
        if (i < nt) s[i] = c + incl - v;
        __syncthreads();
        if (threadIdx.x == kScanThreads - 1) carry = c + incl;
        __syncthreads();
    }
}

__global__ void k_scan_add(int32_t* a, long long n, const int32_t* tile_sums) {
    const long long i = (long long)blockIdx.x * kScanTile + threadIdx.x;
    const int add = tile_sums[blockIdx.x];
    if (add == 0) return;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long j = i + (long long)k * kScanThreads;
        if (j < n) a[j] += add;
    }
}

}  // namespace

// CDF table of the row-length distribution, scaled by 2^53 (see the file
// comment).  kind 0: L = clip(round(exp(mu + sigma Z)), 1, max_len),
// mu = ln(mean) - sigma^2 / 2 (so E exp(mu + sigma Z) = mean); kind 1:
// Poisson(mean) clipped to max_len.
void random_length_table(int kind, double mean, double sigma, int max_len, std::vector<uint64_t>& thr) {
    thr.assign((size_t)max_len + 1, kTwo53);
    double cdf = 0.0, pmf = 0.0;
    const double mu = std::log(mean) - 0.5 * sigma * sigma;
    for (int l = 0; l < max_len; ++l) {
        if (kind == 0) {
            cdf = l == 0 ? 0.0 : 0.5 * std::erfc(-((std::log(l + 0.5) - mu) / sigma) * 0.70710678118654752440);
        } else {
            pmf = l == 0 ? std::exp(-mean) : pmf * mean / l;
            cdf = cdf + pmf;
        }
        double t = std::floor(cdf * 9007199254740992.0);
        thr[(size_t)l] = t >= 9007199254740992.0 ? kTwo53 : (uint64_t)t;
    }
}

cudaError_t launch_random_count(const uint64_t* thr, int max_len, int n, uint64_t seed, int band_permille,
                                int band_half, int32_t* row_start, unsigned long long* total, int sm_count,
                                cudaStream_t st) {
    RowGen g{thr, max_len, n, seed, band_permille, band_half};
    long long blocks = (n + 255) / 256;
    if (blocks > sm_count * 16) blocks = sm_count * 16;
    if (blocks < 1) blocks = 1;
    k_rand_count<<<(int)blocks, 256, 0, st>>>(g, row_start, total);
    return cudaGetLastError();
}

cudaError_t launch_random_fill(const uint64_t* thr, int max_len, int n, uint64_t seed, int band_permille,
                               int band_half, const int32_t* row_start, int32_t* col, double* val, int sm_count,
                               cudaStream_t st) {
    RowGen g{thr, max_len, n, seed, band_permille, band_half};
    long long blocks = (n + 255) / 256;
    if (blocks > sm_count * 16) blocks = sm_count * 16;
    if (blocks < 1) blocks = 1;
    k_rand_fill<<<(int)blocks, 256, 0, st>>>(g, row_start, col, val);
    return cudaGetLastError();
}

long long scan_scratch_elems(long long n) { return (n + kScanTile - 1) / kScanTile + 1; }

cudaError_t launch_inclusive_scan(int32_t* a, long long n, int32_t* scratch, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const long long nt = (n + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<(unsigned)nt, kScanThreads, 0, st>>>(a, n, scratch);
    k_scan_sums<<<1, kScanThreads, 0, st>>>(scratch, (int)nt);
    k_scan_add<<<(unsigned)nt, kScanThreads, 0, st>>>(a, n, scratch);
    return cudaGetLastError();
}

}  // namespace pwmgpu
