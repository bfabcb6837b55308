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
// the y window, then writes its rows of y once.  Dense units (at least
// kDenseUnit elements) stage their S-column x window in shared memory with a
// TMA bulk copy (double-buffered, mbarriers) and are taken by the whole CTA;
// a window's sparse units (a random matrix's blocks hold a few elements
// each) are merged into one "flat" unit taken by the whole CTA, gathering x
// through L1/L2 by global column -- staging 8 KB of x for a handful of
// elements would cost more than it saves.  y is written once per row and no
// CTA touches another's rows.
//
// The device copy (csb_kernel_layout) keeps the blocks, their block-column
// order and the Z-Morton order of the dense sub-squares, stores each
// window's flat unit row-major with a global column per element (kcol), and
// stores each dense unit row-major (rows ascending, columns ascending within a row, duplicates
// in build order) from a multiple of 4 elements: the order inside a
// sub-square is free for y += A x, and on this GPU a shared-memory FP64
// atomic add is a compare-and-swap loop that bounded the Z-ordered kernel.
// A warp takes 128 elements of a dense unit (4 per lane: one 16-byte load of
// ind, two of data; 4 rather than 8 keeps the lanes' x / y-window words
// close together in shared memory).  A row that lies inside one lane starts
// from its y-window value and takes one FMA per element (the FP64 pipe, about
// 2 operations per clock per SM here, is the scarce unit); a row split
// across lanes is summed from zero in each lane but the one where it ends,
// which starts from the y-window value, gathers the chain's partials with
// shuffles (a segmented scan for long rows) and stores the total; only a
// row that continues past the warp's chunk (the element just outside has the
// same row) is summed from zero everywhere and added atomically.  The host
// arrays (pwmgpu_get_csb) stay the reference's.  Per row, the summation
// order is the column order inside each dense unit and the order the atomics
// land in elsewhere (the per-row error bound holds for any order).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <thread>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pwmgpu {

namespace {

// Kernel variants (launch_csb_spmv's `variant`): bit 0 = 8 elements of a
// dense unit per lane (else 4), bit 1 = 256 threads per CTA (else 128).
// Every variant is launched with 1024 resident threads per SM (at most 64
// registers; 24.6 KB of shared memory per CTA).  Variant 0 is the default;
// the format autotuner times all four.
constexpr int kCsbThreadsPerSM = 1024;
constexpr int kCsbMaxS = 1024;
constexpr int kDenseUnit = kTileDenseUnit;  // elements from which a unit's x window is staged

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

constexpr unsigned kFull = 0xFFFFFFFFu;

// One lane's K elements of a row-major dense unit (a warp's chunk is 32 K).
template <int K>
struct Oct {
    uint4 id[K / 4];
    uint4 gc[K / 4];  // global columns (flat units only)
    double2 d[K / 2];
    int nv;    // valid elements (0..K)
    int rout;  // lane 0: row of the element before the chunk, lane 1: after it (-1: none)
};

// Lane `lane`'s elements of the chunk at k0 of unit [lo, hi), and the row of
// the element just outside the chunk (lanes 0 and 1).
template <int K, bool GX>
__device__ __forceinline__ Oct<K> load_oct(const uint32_t* __restrict__ ind, const int32_t* __restrict__ kcol,
                                           const double* __restrict__ data, int k0, int lo, int hi, int S, int lane) {
    constexpr int kChunk = 32 * K;
    Oct<K> q;
    const int k = k0 + K * lane;
    q.nv = k < hi ? min(K, hi - k) : 0;
#pragma unroll
    for (int i = 0; i < K / 4; ++i) {
        q.id[i] = q.gc[i] = make_uint4(0u, 0u, 0u, 0u);
        q.d[2 * i] = q.d[2 * i + 1] = make_double2(0.0, 0.0);
    }
    // k is a multiple of 4 and the arrays are padded past the last unit by 8
    const uint4* ip = reinterpret_cast<const uint4*>(ind + k);
    const uint4* cp = reinterpret_cast<const uint4*>(kcol + k);
    const double2* dp = reinterpret_cast<const double2*>(data + k);
    // a flat unit (GX: x gathered by global column through L2) streams its
    // elements with evict-first loads, so they do not push x out of L2; a
    // dense unit's x window is in shared memory and keeps plain loads
#pragma unroll
    for (int i = 0; i < K / 4; ++i)
        if (4 * i < q.nv) {
            if (GX) {
                q.id[i] = __ldcs(ip + i);
                q.gc[i] = __ldcs(cp + i);
                q.d[2 * i] = __ldcs(dp + 2 * i);
                q.d[2 * i + 1] = __ldcs(dp + 2 * i + 1);
            } else {
                q.id[i] = __ldg(ip + i);
                q.d[2 * i] = __ldg(dp + 2 * i);
                q.d[2 * i + 1] = __ldg(dp + 2 * i + 1);
            }
        }
    q.rout = -1;
    if (k0 >= hi) return q;  // a warp past the unit's end
    if (lane == 0 && k0 > lo) q.rout = (int)(__ldg(ind + k0 - 1) >> 16) & (S - 1);
    if (lane == 1 && k0 + kChunk < hi) q.rout = (int)(__ldg(ind + k0 + kChunk) >> 16) & (S - 1);
    return q;
}

// Add a warp's chunk (lane l holds elements 8l..8l+7 of it, rows sorted)
// into the y window with one FMA per element wherever a row lies inside one
// lane: such a row starts from ys[row] and is stored back.  The rest are
// "partial" rows, summed from zero: a lane's first row rf when it continues
// the previous lane's last row ("joins"), its last row rl when the next lane
// joins it, and the chunk's first / last row when the element just outside
// the chunk has the same row (then another warp adds to it as well).  The
// lane where a partial row ends adds the partials of its chain of lanes
// (a few shuffles, or a segmented scan for long chains) -- atomically for
// rows that cross the chunk, with a plain add otherwise.
template <int K, bool GX>
__device__ __forceinline__ void dense_oct(const Oct<K>& q, int S, const double* xw, const double* __restrict__ xg,
                                          double* ys, int lane) {
    // the rows of the elements just before and after the chunk (-1: none)
    const int row_before = __shfl_sync(kFull, q.rout, 0), row_after = __shfl_sync(kFull, q.rout, 1);
    uint32_t ids[K], gcs[K];
    double vs[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const uint4& u4 = q.id[j >> 2];
        ids[j] = (j & 3) == 0 ? u4.x : (j & 3) == 1 ? u4.y : (j & 3) == 2 ? u4.z : u4.w;
        const uint4& g4 = q.gc[j >> 2];
        gcs[j] = (j & 3) == 0 ? g4.x : (j & 3) == 1 ? g4.y : (j & 3) == 2 ? g4.z : g4.w;
        vs[j] = (j & 1) ? q.d[j >> 1].y : q.d[j >> 1].x;
    }
    const int nv = q.nv;
    const int rf = (int)(ids[0] >> 16) & (S - 1);
    int rl = rf;
#pragma unroll
    for (int j = 1; j < K; ++j)
        if (j < nv) rl = (int)(ids[j] >> 16) & (S - 1);
    const int rl_prev = __shfl_up_sync(kFull, rl, 1);
    const int nv_prev = __shfl_up_sync(kFull, nv, 1);
    const bool joins = lane > 0 && nv > 0 && nv_prev > 0 && rl_prev == rf;
    const bool next_joins = __shfl_down_sync(kFull, joins, 1) && lane < 31;
    const int last_lane = __reduce_max_sync(kFull, nv > 0 ? lane : 0);
    const int first_row = __shfl_sync(kFull, rf, 0);
    const int last_row = __shfl_sync(kFull, rl, last_lane);
    const bool cross_lo = row_before == first_row, cross_hi = row_after == last_row;
    const bool one_row = rf == rl;
    const bool bnd_f = (rf == first_row && cross_lo) || (rf == last_row && cross_hi);
    const bool bnd_l = (rl == first_row && cross_lo) || (rl == last_row && cross_hi);
    const bool part_f = nv > 0 && (joins || bnd_f || (one_row && next_joins));
    const bool part_l = nv > 0 && !one_row && (next_joins || bnd_l);
    // the lane where a partial first row ends adds the row once; unless the
    // row continues in another chunk it is the row's only writer, so it
    // starts from the y-window value and stores the total (no extra add)
    const bool add_f = part_f && (!one_row || !next_joins);
    const bool own_f = add_f && !bnd_f;
    // accumulate: rows inside the lane start from ys, partial rows from zero
    double pf = 0.0, pl = 0.0, acc = 0.0;
    int cur = -1;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        if (j < nv) {
            const int r = (int)(ids[j] >> 16) & (S - 1);
            if (r != cur) {
                if (cur >= 0) {
                    if (cur == rf && part_f)
                        pf = acc;
                    else
                        ys[cur] = acc;
                }
                cur = r;
                acc = (r == rf && part_f && !own_f) || (r == rl && part_l) ? 0.0 : ys[r];
            }
            const double xv = GX ? __ldg(xg + gcs[j]) : xw[ids[j] & (uint32_t)(S - 1)];
            acc = fma(vs[j], xv, acc);
        }
    }
    if (cur >= 0) {
        if (cur == rf && part_f)
            pf = acc;
        else if (cur == rl && part_l)
            pl = acc;
        else
            ys[cur] = acc;
    }
    // chains: lane l's tail value is the partial of its last row
    const double t = one_row ? pf : pl;
    // a chain of lanes starts at a lane that is not a one-row lane joining
    // its predecessor; len = the earlier lanes of this lane's chain
    const unsigned starts = __ballot_sync(kFull, !(one_row && joins));
    const int len = joins ? lane - (31 - __clz(starts & ((1u << lane) - 1u))) : 0;
    const int maxlen = __reduce_max_sync(kFull, add_f ? len : 0);
    double tot = pf;
    if (maxlen <= 6) {
        for (int i = 1; i <= maxlen; ++i) {
            const double v = __shfl_up_sync(kFull, t, i);
            if (i <= len) tot += v;
        }
    } else {  // long rows: segmented scan of the tail values
        double a = t;
        bool head = !(one_row && joins);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const double a2 = __shfl_up_sync(kFull, a, d);
            const bool h2 = __shfl_up_sync(kFull, head, d);
            if (lane >= d && !head) {
                a += a2;
                head = h2;
            }
        }
        const double carry = __shfl_up_sync(kFull, a, 1);
        if (joins) tot += carry;
    }
    if (add_f) {
        if (bnd_f)
            atomicAdd(&ys[rf], tot);
        else
            ys[rf] = tot;  // tot started from ys[rf] (own_f)
    }
    if (part_l && !next_joins) atomicAdd(&ys[rl], pl);  // the chunk's last row, continued by another warp
}

// win_ptr[2w] = the window's first unit, win_ptr[2w+1] = its first dense
// unit, win_ptr[2w+2] = the next window's first unit.
template <int NT, int K>
__global__ void __launch_bounds__(NT, kCsbThreadsPerSM / NT) k_csb_spmv(const uint32_t* __restrict__ ind, const int32_t* __restrict__ kcol, const double* __restrict__ data,
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
            for (int i = tid; i < cnt; i += NT) xs[b][i] = __ldg(x + c0 + i);
            if (tid == 0) mbar_arrive(&bar[b]);
        }
    };
    const int lane = tid & 31, warp = tid >> 5;
    for (int w = blockIdx.x; w < nwin; w += gridDim.x) {
        const int us = __ldg(win_ptr + 2 * w), u0 = __ldg(win_ptr + 2 * w + 1), u1 = __ldg(win_ptr + 2 * w + 2);
        for (int i = tid; i < S; i += NT) ys[i] = 0.0;
        if (u0 < u1) stage(u0, 0);
        __syncthreads();  // ys zeroed
        // the window's sparse sub-squares as one flat row-major unit, x
        // gathered through L1 / L2 by global column
        if (u0 > us) {
            const int4 un = __ldg(units + us);
            constexpr int kChunk = 32 * K;
            constexpr int kStep = (NT / 32) * kChunk;
            for (int k = un.x + warp * kChunk; k < un.y; k += kStep) {
                const Oct<K> q = load_oct<K, true>(ind, kcol, data, k, un.x, un.y, S, lane);
                dense_oct<K, true>(q, S, nullptr, x, ys, lane);
            }
        }
        bool ok = true;
        for (int u = u0; u < u1; ++u) {
            const int b = (u - u0) & 1;
            __syncthreads();  // buffer b^1 is free (its unit is done), ys zeroed
            if (u + 1 < u1) stage(u + 1, b ^ 1);
            const int4 un = __ldg(units + u);
            if (un.w == 2) {
                // one element per row: element lo + i to lane i % 32 of warp
                // (i / 32) % W, so a warp's loads, x-window reads and y-window
                // updates are 32 consecutive rows (no bank conflicts), four
                // elements per lane in flight (the first four while the x
                // window lands); one FMA per element from the row's y-window
                // value
                uint32_t id[4];
                double v[4];
                int base = un.x + warp * 128;
                auto load4 = [&](int bs) {
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const int k = bs + 32 * t + lane;
                        id[t] = k < un.y ? __ldg(ind + k) : 0u;
                        v[t] = k < un.y ? __ldg(data + k) : 0.0;
                    }
                };
                load4(base);
                ok = mbar_wait_bounded(&bar[b], uses[b] & 1u, status);
                uses[b]++;
                if (!__syncthreads_and(ok)) break;
                const double* xw = xs[b];
                while (base < un.y) {
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        if (base + 32 * t + lane < un.y) {
                            const int r = (int)(id[t] >> 16) & (S - 1);
                            ys[r] = fma(v[t], xw[id[t] & (uint32_t)(S - 1)], ys[r]);
                        }
                    }
                    base += (NT / 32) * 128;
                    if (base < un.y) load4(base);
                }
                continue;
            }
            // row-major unit: warp chunks of kChunk elements; the first
            // chunk's loads are in flight while the x window lands
            constexpr int kChunk = 32 * K;
            constexpr int kStep = (NT / 32) * kChunk;
            int k = un.x + warp * kChunk;
            Oct<K> q = load_oct<K, false>(ind, kcol, data, k, un.x, un.y, S, lane);
            ok = mbar_wait_bounded(&bar[b], uses[b] & 1u, status);
            uses[b]++;
            if (!__syncthreads_and(ok)) break;
            const double* xw = xs[b];
            while (k < un.y) {
                dense_oct<K, false>(q, S, xw, nullptr, ys, lane);
                k += kStep;
                if (k < un.y) q = load_oct<K, false>(ind, kcol, data, k, un.x, un.y, S, lane);
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
        for (int i = tid; i < S && r0 + i < nor; i += NT) {
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

// Device copy for k_csb_spmv from the built arrays.  Per window: its sparse
// units merged into one "flat" unit, row-major over the window (a stable
// sort by (local row, global column)), with each element's global column in
// kcol (x is gathered from global memory there); then its dense units, each
// row-major (a stable sort by ind = local row << 16 | local column).  Every
// unit starts on a multiple of 4 elements; the gaps hold zeros and are never
// read as elements.  win_ptr and units (4 ints per unit: {lo, hi, c0, kind},
// c0 = -1 for a flat unit; kind 2 for a dense unit whose rows hold one
// element each, else 0) are rewritten: a window has at most one unit before
// its first dense unit.  Windows are independent: filled by a few
// host threads.  Returns false when the copy would not fit 32-bit element
// offsets.
bool csb_kernel_layout(const std::vector<uint32_t>& ind, const std::vector<double>& data, int S,
                       std::vector<int>& win_ptr, std::vector<int>& units, std::vector<uint32_t>& kind,
                       std::vector<double>& kdata, std::vector<int32_t>& kcol) {
    const int nwin = (int)(win_ptr.size() / 2);
    std::vector<int> new_ptr(2 * (size_t)nwin + 1, 0), new_units;
    std::vector<long long> src_first;  // first source unit of each new unit
    std::vector<int> src_last;         // one past its last source unit
    long long o = 0;
    for (int w = 0; w < nwin; ++w) {
        const int us = win_ptr[2 * (size_t)w], ud = win_ptr[2 * (size_t)w + 1], ue = win_ptr[2 * (size_t)w + 2];
        new_ptr[2 * (size_t)w] = (int)(new_units.size() / 4);
        if (ud > us) {
            long long n = 0;
            for (int u = us; u < ud; ++u) n += units[4 * (size_t)u + 1] - units[4 * (size_t)u];
            o = (o + 3) & ~3LL;
            new_units.insert(new_units.end(), {(int)o, (int)(o + n), -1, 0});
            src_first.push_back(us);
            src_last.push_back(ud);
            o += n;
            if (o + 8 > (long long)INT32_MAX) return false;
        }
        new_ptr[2 * (size_t)w + 1] = (int)(new_units.size() / 4);
        for (int u = ud; u < ue; ++u) {
            const int n = units[4 * (size_t)u + 1] - units[4 * (size_t)u];
            o = (o + 3) & ~3LL;
            new_units.insert(new_units.end(), {(int)o, (int)(o + n), units[4 * (size_t)u + 2], 0});
            src_first.push_back(u);
            src_last.push_back(u + 1);
            o += n;
            if (o + 8 > (long long)INT32_MAX) return false;
        }
    }
    new_ptr[2 * (size_t)nwin] = (int)(new_units.size() / 4);
    const size_t total = (size_t)((o + 3) & ~3LL) + 8;
    kind.assign(total, 0u);
    kdata.assign(total, 0.0);
    kcol.assign(total, 0);
    const int nnew = (int)(new_units.size() / 4);
    auto work = [&](int v0, int v1) {
        // (row key, column key, source position)
        std::vector<std::tuple<uint32_t, uint32_t, long long>> key;
        for (int v = v0; v < v1; ++v) {
            const bool flat = new_units[4 * (size_t)v + 2] < 0;
            const int dst = new_units[4 * (size_t)v];
            key.clear();
            for (long long u = src_first[v]; u < src_last[v]; ++u) {
                const int lo = units[4 * (size_t)u], hi = units[4 * (size_t)u + 1], c0 = units[4 * (size_t)u + 2];
                for (int k = lo; k < hi; ++k) {
                    const uint32_t id = ind[(size_t)k];
                    // a flat unit sorts by row, then global column (the unit's
                    // first column + the local column mod S, as the kernel reads x)
                    if (flat)
                        key.emplace_back(id >> 16, (uint32_t)c0 + ((id & 0xFFFFu) & (uint32_t)(S - 1)), k);
                    else
                        key.emplace_back(id, 0u, k);
                }
            }
            std::sort(key.begin(), key.end());  // position last: stable by construction
            bool one_per_row = !flat;
            for (size_t q = 0; q < key.size(); ++q) {
                const long long k = std::get<2>(key[q]);
                kind[(size_t)dst + q] = ind[(size_t)k];
                kdata[(size_t)dst + q] = data[(size_t)k];
                if (flat) kcol[(size_t)dst + q] = (int32_t)std::get<1>(key[q]);
                if (q > 0 && ((std::get<0>(key[q]) ^ std::get<0>(key[q - 1])) >> 16) == 0) one_per_row = false;
            }
            // a dense unit whose rows hold one element each (a stencil's
            // off-diagonal tiles): the kernel's element-per-lane path
            if (one_per_row) new_units[4 * (size_t)v + 3] = 2;
        }
    };
    const int nt = std::max(1, std::min<int>(nnew / 64 + 1, (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        const int a = (int)((long long)nnew * t / nt), b = (int)((long long)nnew * (t + 1) / nt);
        th.emplace_back(work, a, b);
    }
    for (auto& t : th) t.join();

    // A dense unit whose elements lie on at most kTileMaxDiag diagonals of
    // the tile (a banded tile: a stencil's diagonal tiles) is split into one
    // unit per diagonal, each with one element per row -- the kernel's
    // element-per-lane path -- taken in diagonal order, which is column
    // order within each row (the row sums keep CRS order).  The elements
    // are reordered in place: diagonal by diagonal, rows ascending.
    constexpr int kTileMaxDiag = 4;
    std::vector<std::vector<int>> diag_len((size_t)nnew);  // elements per diagonal, or empty: keep the unit
    auto band = [&](int v0, int v1) {
        std::vector<std::tuple<int, uint32_t, uint32_t, double>> el;
        for (int v = v0; v < v1; ++v) {
            const int lo = new_units[4 * (size_t)v], hi = new_units[4 * (size_t)v + 1];
            if (new_units[4 * (size_t)v + 2] < 0 || new_units[4 * (size_t)v + 3] == 2 || hi <= lo) continue;
            int diags[kTileMaxDiag], nd = 0;
            bool ok = true;
            for (int k = lo; k < hi && ok; ++k) {
                const uint32_t id = kind[(size_t)k];
                const int d = (int)(id & (uint32_t)(S - 1)) - (int)((id >> 16) & (uint32_t)(S - 1));
                int j = 0;
                while (j < nd && diags[j] != d) ++j;
                if (j == nd) {
                    if (nd == kTileMaxDiag) ok = false;
                    else diags[nd++] = d;
                }
            }
            if (!ok || nd < 2) continue;
            el.clear();
            for (int k = lo; k < hi; ++k) {
                const uint32_t id = kind[(size_t)k];
                const int d = (int)(id & (uint32_t)(S - 1)) - (int)((id >> 16) & (uint32_t)(S - 1));
                el.emplace_back(d, (id >> 16) & (uint32_t)(S - 1), id, kdata[(size_t)k]);
            }
            std::sort(el.begin(), el.end(), [](const auto& a, const auto& b) {
                return std::get<0>(a) != std::get<0>(b) ? std::get<0>(a) < std::get<0>(b) : std::get<1>(a) < std::get<1>(b);
            });
            // a repeated coordinate puts two elements of one row on one
            // diagonal: such a unit is not one element per row, keep it whole
            bool dup = false;
            for (size_t q = 1; q < el.size() && !dup; ++q)
                dup = std::get<0>(el[q]) == std::get<0>(el[q - 1]) && std::get<1>(el[q]) == std::get<1>(el[q - 1]);
            if (dup) continue;
            std::vector<int>& len = diag_len[(size_t)v];
            for (size_t q = 0; q < el.size(); ++q) {
                kind[(size_t)lo + q] = std::get<2>(el[q]);
                kdata[(size_t)lo + q] = std::get<3>(el[q]);
                if (q == 0 || std::get<0>(el[q]) != std::get<0>(el[q - 1])) len.push_back(0);
                ++len.back();
            }
        }
    };
    th.clear();
    for (int t = 0; t < nt; ++t) {
        const int a = (int)((long long)nnew * t / nt), b = (int)((long long)nnew * (t + 1) / nt);
        th.emplace_back(band, a, b);
    }
    for (auto& t : th) t.join();
    std::vector<int> out_ptr(new_ptr.size(), 0), out_units;
    out_units.reserve(new_units.size());
    for (int w = 0; w < nwin; ++w) {
        for (int part = 0; part < 2; ++part) {
            out_ptr[2 * (size_t)w + part] = (int)(out_units.size() / 4);
            for (int v = new_ptr[2 * (size_t)w + part]; v < new_ptr[2 * (size_t)w + part + 1]; ++v) {
                const int* u = &new_units[4 * (size_t)v];
                if (diag_len[(size_t)v].empty()) {
                    out_units.insert(out_units.end(), {u[0], u[1], u[2], u[3]});
                    continue;
                }
                int a = u[0];
                for (int n : diag_len[(size_t)v]) {
                    out_units.insert(out_units.end(), {a, a + n, u[2], 2});
                    a += n;
                }
            }
        }
    }
    out_ptr[2 * (size_t)nwin] = (int)(out_units.size() / 4);
    win_ptr.swap(out_ptr);
    units.swap(out_units);
    return true;
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

cudaError_t launch_csb_spmv(const uint32_t* ind, const int32_t* kcol, const double* data, const int* win_ptr,
                            const int* units, int nwin,
                            int S, int nor, int noc, const double* x, double* y, const double* nsq_in, int* status,
                            int sm_count, cudaStream_t st, int variant) {
    if (nwin <= 0) return cudaSuccess;
    const int4* un = reinterpret_cast<const int4*>(units);
    const int nt = (variant & 2) ? 256 : 128;
    const int grid = std::min(nwin, sm_count * (kCsbThreadsPerSM / nt));
    switch (variant & 3) {
        case 1: k_csb_spmv<128, 8><<<grid, 128, 0, st>>>(ind, kcol, data, win_ptr, un, nwin, S, nor, noc, x, y, nsq_in, status); break;
        case 2: k_csb_spmv<256, 4><<<grid, 256, 0, st>>>(ind, kcol, data, win_ptr, un, nwin, S, nor, noc, x, y, nsq_in, status); break;
        case 3: k_csb_spmv<256, 8><<<grid, 256, 0, st>>>(ind, kcol, data, win_ptr, un, nwin, S, nor, noc, x, y, nsq_in, status); break;
        default: k_csb_spmv<128, 4><<<grid, 128, 0, st>>>(ind, kcol, data, win_ptr, un, nwin, S, nor, noc, x, y, nsq_in, status); break;
    }
    return cudaGetLastError();
}

}  // namespace pwmgpu
