// csb.cu -- compressed sparse blocks (CSB) on the GPU.
//
// Storage is the reference's CSB (SOA_Implementations/CSB.hpp): beta x beta
// blocks, beta from setBlockSizeParam (:96-113); blocks in block-column order
// within each block row; elements of a block in Z-Morton order (row bit
// before column bit at every level, zMortonCompare :147-173); ind = local row
// << 16 | local column (:89-91); blk_ptr[block_row * hb + block_col]
// (:464-567).  Built on the host here, bit for bit the reference's arrays.
//
// The GPU kernel (k_csb_spmv) exploits the Z-Morton order: the elements of a
// block inside an aligned S x S sub-square form one contiguous range.  Rows
// are cut into windows of S rows; one CTA owns a window: it zeroes an S-row
// y window in shared memory, walks its sub-squares ("units": every block of
// the block row, every column window) and adds each element's product into
// the y window (shared-memory atomics), then writes its rows of y once.
// Dense units (at least kDenseUnit elements) stage their S-column x window in
// shared memory with a TMA bulk copy (double-buffered, mbarriers) and are
// taken by the whole CTA; sparse units (a random matrix's blocks hold a few
// elements each) are taken one per warp, gathering x through L1/L2 -- staging
// 8 KB of x for a handful of elements would cost more than it saves.  y is
// written once per row and no CTA touches another's rows.  The summation
// order within a row follows the order the atomics land in (the per-row
// error bound holds for any order).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pwmgpu {

namespace {

constexpr int kCsbNT = 256;
constexpr int kCsbMaxS = 1024;
constexpr int kDenseUnit = 256;  // elements from which a unit's x window is staged

// Spread the low 16 bits of v to the even bit positions.
inline uint64_t spread16(uint64_t v) {
    v &= 0xFFFFull;
    v = (v | (v << 8)) & 0x00FF00FFull;
    v = (v | (v << 4)) & 0x0F0F0F0Full;
    v = (v | (v << 2)) & 0x33333333ull;
    v = (v | (v << 1)) & 0x55555555ull;
    return v;
}

// Z-Morton key of a local (row, col): row bit above column bit at each level.
inline uint64_t zmorton(uint32_t lr, uint32_t lc) { return (spread16(lr) << 1) | spread16(lc); }

struct Unit {
    int lo, hi;  // element range (a sub-square of one block)
    int c0;      // first column of the x window
    int pad;
};

// win_ptr[2w] = the window's first unit, win_ptr[2w+1] = its first dense
// unit, win_ptr[2w+2] = the next window's first unit.
__global__ void __launch_bounds__(kCsbNT) k_csb_spmv(const uint32_t* __restrict__ ind, const double* __restrict__ data,
                                                     const int* __restrict__ win_ptr, const int4* __restrict__ units,
                                                     int nwin, int S, int nor, int noc, const double* __restrict__ x,
                                                     double* __restrict__ y, const double* nsq_in, int* status) {
    __shared__ __align__(16) double xs[2][kCsbMaxS];
    __shared__ double ys[kCsbMaxS];
    __shared__ __align__(8) uint64_t bar[2];
    const int tid = threadIdx.x;
    const int e = nsq_in ? pow2_rescale_exponent(*nsq_in, 256) : 0;
    const bool tma_ok = (reinterpret_cast<uintptr_t>(x) & 15u) == 0;
    const uint64_t pol = policy_evict_normal();
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t uses[2] = {0u, 0u};  // completed phases per buffer (same in every thread)
    // stage the x window of unit u into buffer b (thread 0: TMA bulk copy;
    // the odd last element, if any, with a plain load)
    auto stage = [&](int u, int b) {
        const int c0 = __ldg(&units[u].z);
        const int cnt = min(S, noc - c0);
        if (tma_ok) {
            if (tid == 0) {
                const uint32_t bytes = (uint32_t)(cnt & ~1) * 8u;
                mbar_arrive_expect_tx(&bar[b], bytes);
                if (bytes) bulk_g2s(xs[b], x + c0, bytes, &bar[b], pol);
                if (cnt & 1) xs[b][cnt - 1] = __ldg(x + c0 + cnt - 1);
            }
        } else {
            for (int i = tid; i < cnt; i += kCsbNT) xs[b][i] = __ldg(x + c0 + i);
            if (tid == 0) mbar_arrive(&bar[b]);
        }
    };
    const int lane = tid & 31, warp = tid >> 5;
    for (int w = blockIdx.x; w < nwin; w += gridDim.x) {
        const int us = __ldg(win_ptr + 2 * w), u0 = __ldg(win_ptr + 2 * w + 1), u1 = __ldg(win_ptr + 2 * w + 2);
        for (int i = tid; i < S; i += kCsbNT) ys[i] = 0.0;
        if (u0 < u1) stage(u0, 0);
        __syncthreads();  // ys zeroed
        // sparse units: one per warp, x gathered through L1 / L2
        for (int u = us + warp; u < u0; u += kCsbNT / 32) {
            const int4 un = __ldg(units + u);
            const double* xw = x + un.z;
            for (int k = un.x + lane; k < un.y; k += 32) {
                const uint32_t id = __ldg(ind + k);
                const int r = (int)(id >> 16) & (S - 1), c = (int)(id & 0xFFFFu) & (S - 1);
                atomicAdd(&ys[r], __ldg(data + k) * __ldg(xw + c));
            }
        }
        bool ok = true;
        for (int u = u0; u < u1; ++u) {
            const int b = (u - u0) & 1;
            __syncthreads();  // buffer b^1 is free (its unit is done), ys zeroed
            if (u + 1 < u1) stage(u + 1, b ^ 1);
            ok = mbar_wait_bounded(&bar[b], uses[b] & 1u, status);
            uses[b]++;
            if (!__syncthreads_and(ok)) break;
            const int4 un = __ldg(units + u);
            const double* xw = xs[b];
            for (int k = un.x + tid; k < un.y; k += kCsbNT) {
                const uint32_t id = __ldg(ind + k);
                const int r = (int)(id >> 16) & (S - 1), c = (int)(id & 0xFFFFu) & (S - 1);
                atomicAdd(&ys[r], __ldg(data + k) * xw[c]);
            }
        }
        if (!ok) {
            // a wait timed out: let the copies in flight land, then stop
            if (tid == 0)
                for (int b = 0; b < 2; ++b) mbar_wait_bounded(&bar[b], uses[b] & 1u, status, kWaitCycles / 8, false);
            __syncthreads();
            return;
        }
        // an unconsumed prefetch cannot exist: the last unit's stage was waited
        __syncthreads();
        const int r0 = w * S;
        for (int i = tid; i < S && r0 + i < nor; i += kCsbNT) {
            const double v = ys[i];
            y[r0 + i] = e != 0 ? scale_pow2(v, e) : v;
        }
        __syncthreads();
    }
}

}  // namespace

// Host build (CSB.hpp:464-567 semantics): per block row, elements ordered by
// block column then Z-Morton key (ties by CRS position), from CRS arrays.
// Block rows are independent: built by a few host threads.
int csb_build_host(int nor, int noc, long long nnz, const int32_t* row_start, const int32_t* col, const double* val,
                   int beta, int bits, std::vector<uint32_t>& ind, std::vector<double>& data,
                   std::vector<int32_t>& blk_ptr, int S, std::vector<int>& win_ptr, std::vector<int>& unit_data) {
    (void)bits;
    const int hb = (noc + beta - 1) / beta, vb = (nor + beta - 1) / beta;
    ind.resize((size_t)nnz);
    data.resize((size_t)nnz);
    blk_ptr.assign((size_t)hb * vb + 1, 0);
    const int nwin = (nor + S - 1) / S;
    std::vector<std::vector<Unit>> units_per_win(nwin);
    const int wpb = beta / S;  // windows per block row
    auto work = [&](int br0, int br1) {
        std::vector<std::pair<uint64_t, int64_t>> keys;
        std::vector<int> rowof;
        for (int br = br0; br < br1; ++br) {
            const int r0 = br * beta, r1 = std::min(nor, r0 + beta);
            const int64_t e0 = row_start[r0], e1 = row_start[r1];
            keys.clear();
            for (int r = r0; r < r1; ++r)
                for (int64_t k = row_start[r]; k < row_start[r + 1]; ++k) {
                    const uint32_t bc = (uint32_t)col[k] / (uint32_t)beta;
                    const uint32_t lr = (uint32_t)(r - r0), lc = (uint32_t)col[k] % (uint32_t)beta;
                    keys.emplace_back(((uint64_t)bc << 32) | zmorton(lr, lc), k);
                }
            std::sort(keys.begin(), keys.end());
            // local row of each CRS position of the block row
            rowof.resize((size_t)(e1 - e0));
            for (int r = r0; r < r1; ++r)
                for (int64_t k = row_start[r]; k < row_start[r + 1]; ++k) rowof[(size_t)(k - e0)] = r - r0;
            // arrays, block counts, and units (this block row's windows only)
            int cur_key_w = -1, cur_key_c = -1, cur_bc = -1;
            for (size_t q = 0; q < keys.size(); ++q) {
                const int64_t k = keys[q].second;
                const int64_t dst = e0 + (int64_t)q;
                const uint32_t lr = (uint32_t)rowof[(size_t)(k - e0)];
                const uint32_t lc = (uint32_t)col[k] % (uint32_t)beta;
                const int bc = (int)(keys[q].first >> 32);
                ind[(size_t)dst] = (lr << 16) | lc;
                data[(size_t)dst] = val[k];
                blk_ptr[(size_t)br * hb + bc + 1]++;
                const int wi = (int)(lr / (uint32_t)S), ci = (int)(lc / (uint32_t)S);
                const int w = br * wpb + wi;
                if (bc != cur_bc || wi != cur_key_w || ci != cur_key_c) {
                    units_per_win[(size_t)w].push_back(Unit{(int)dst, (int)dst + 1, bc * beta + ci * S, 0});
                    cur_bc = bc;
                    cur_key_w = wi;
                    cur_key_c = ci;
                } else {
                    units_per_win[(size_t)w].back().hi = (int)dst + 1;
                }
            }
        }
    };
    const int nt = std::max(1, std::min<int>(vb, (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        const int a = (int)((long long)vb * t / nt), b = (int)((long long)vb * (t + 1) / nt);
        th.emplace_back(work, a, b);
    }
    for (auto& t : th) t.join();
    for (size_t b = 0; b + 1 < blk_ptr.size(); ++b) blk_ptr[b + 1] += blk_ptr[b];
    // per window: sparse units first, then dense ones (win_ptr holds both starts)
    win_ptr.assign(2 * (size_t)nwin + 1, 0);
    unit_data.clear();
    int o = 0;
    for (int w = 0; w < nwin; ++w) {
        win_ptr[2 * (size_t)w] = o;
        for (int dense = 0; dense < 2; ++dense) {
            if (dense) win_ptr[2 * (size_t)w + 1] = o;
            for (const Unit& u : units_per_win[(size_t)w]) {
                if ((u.hi - u.lo >= kDenseUnit) != (dense == 1)) continue;
                unit_data.insert(unit_data.end(), {u.lo, u.hi, u.c0, 0});
                ++o;
            }
        }
    }
    win_ptr[2 * (size_t)nwin] = o;
    return 0;
}

// CSB.hpp:96-113 with sizeof(T) = 8, L2_CACHE_SIZE_MB = 1, L2_CACHE_MULT =
// 0.85 (Util/Constants.hpp:27-28).
void csb_params(int nor, int noc, int* beta, int* bits) {
    const int minimal = std::min(nor, noc);
    const int lg = (int)std::ceil(std::log2(std::sqrt((double)minimal)));
    int b = std::min(16, 3 + lg);
    int v = 1 << b;
    while (b > lg) {
        if ((double)(8 * 8) * v * 2 > 1 * 0.85 * 1e6 * 8) {
            b -= 1;
            v = 1 << b;
        } else {
            break;
        }
    }
    *beta = v;
    *bits = b;
}

// Window side: the largest power of two <= min(beta, 1024) that still gives
// at least 8 windows per SM (not below 64).
int csb_window(int nor, int beta, int sm_count) {
    int S = std::min(beta, kCsbMaxS);
    while (S > 64 && (nor + S - 1) / S < 8 * sm_count) S >>= 1;
    return S;
}

cudaError_t launch_csb_spmv(const uint32_t* ind, const double* data, const int* win_ptr, const int* units, int nwin,
                            int S, int nor, int noc, const double* x, double* y, const double* nsq_in, int* status,
                            int sm_count, cudaStream_t st) {
    if (nwin <= 0) return cudaSuccess;
    int grid = std::min(nwin, sm_count * 8);
    k_csb_spmv<<<grid, kCsbNT, 0, st>>>(ind, data, win_ptr, reinterpret_cast<const int4*>(units), nwin, S, nor, noc,
                                        x, y, nsq_in, status);
    return cudaGetLastError();
}

}  // namespace pwmgpu
