// merge.cuh -- merge-path CRS SpMV tile machinery (sm_103a).
//
// Restates the merge-based SpMV of SOA_Implementations/CRS_Merge.hpp:95-141
// (after Merrill & Garland, SC'16) for GB300:
//
//  * The merge path (row ends of row_start+1 merged with the nonzero indices,
//    N + nnz items) is cut into tiles of TM = NT*IPT items.  Tile t spans
//    diagonals [t*TM, min((t+1)*TM, N+nnz)); its end points come from the
//    same binary search as CRS_Merge::searchPathOnDiag (:42-62) and are
//    computed once per matrix (k_merge_partition), not per SpMV.
//  * A persistent CTA walks its tiles; one elected thread streams each tile's
//    values, column indices and row-start window into shared memory with TMA
//    bulk copies (16-byte granules, L2 evict-first) STAGES tiles ahead,
//    completing on an mbarrier.
//  * Gather: all threads load x[col] for the tile's nonzeros (coalesced over
//    the nonzeros, many loads in flight) into shared memory.
//  * Consume: thread t re-runs the merge-path search for its diagonal on the
//    shared-memory row window, then walks IPT items exactly as the
//    reference's thread loop does: one FMA per nonzero (the only FP64
//    arithmetic per nonzero -- GB300's FP64 pipe is ~1.9 DFMA/clk/SM), a row
//    end writes the row total to a shared y tile.
//  * Carries: each thread's partial last row is added to the row's total by
//    the first thread of the run of threads ending in that row (fixed order,
//    deterministic); the tile's own partial last row goes to carries[tile]
//    and is added by k_merge_fixup, like the reference's serial fix-up
//    (:136-140).
//  * Store: completed rows leave the shared y tile with coalesced stores;
//    the power-method epilogue rescales by an exact power of two and sums
//    the squares there.
#pragma once
#include "common.cuh"

namespace pwmgpu {

constexpr int a16(long long b) { return (int)((b + 15) / 16 * 16); }

struct TileHdr {
    int r0, k0, r1, k1;  // merge coordinates of the tile's start and end
    int voff, coff, roff;  // offsets of element k0 / k0 / row r0 inside the staged windows
    int pad;
};

template <typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
struct MergeLayout {
    static constexpr int TM = NT * IPT;
    static constexpr int VE = 16 / (int)sizeof(VT);  // elements per 16-byte granule
    static constexpr int VAL_CAP = TM + 2 * VE;
    static constexpr int COL_CAP = TM + 8;
    static constexpr int ROW_CAP = TM + 12;
    static constexpr int VAL_B = a16((long long)VAL_CAP * sizeof(VT));
    static constexpr int COL_B = a16((long long)COL_CAP * 4);
    static constexpr int ROW_B = a16((long long)ROW_CAP * 4);
    static constexpr int STAGE_B = VAL_B + COL_B + ROW_B;
    static constexpr int XG_OFF = STAGES * STAGE_B;
    static constexpr int YS_OFF = XG_OFF + a16((long long)TM * sizeof(XT));
    static constexpr int CO_OFF = YS_OFF + a16((long long)(TM + 1) * sizeof(AT));
    static constexpr int CR_OFF = CO_OFF + a16((long long)(NT + 1) * 8);
    static constexpr int CV_OFF = CR_OFF + a16((long long)NT * 4);
    static constexpr int HDR_OFF = CV_OFF + a16((long long)NT * sizeof(AT));
    static constexpr int BAR_OFF = HDR_OFF + a16((long long)STAGES * sizeof(TileHdr));
    static constexpr int RED_OFF = BAR_OFF + a16((long long)STAGES * 8);
    static constexpr int BYTES = RED_OFF + a16(32 * 8);
};

// Padding (in elements) every device array of a matrix carries past its end,
// so that the 16-byte-rounded TMA windows never leave the allocation.
constexpr int kArrayPad = 16;

// Merge-path search of CRS_Merge.hpp:42-62 on a global row_end array:
// smallest a in [max(0, d - nnz), min(d, nor)) with row_end[a] > d - a - 1.
__device__ __forceinline__ int2 merge_search_global(int d, const int32_t* __restrict__ row_end, int nor, int nnz) {
    int lo = d > nnz ? d - nnz : 0;
    int hi = d < nor ? d : nor;
    while (lo < hi) {
        int pivot = (int)(((unsigned)lo + (unsigned)hi) >> 1);
        if (__ldg(row_end + pivot) <= d - pivot - 1) lo = pivot + 1;
        else hi = pivot;
    }
    return make_int2(lo < nor ? lo : nor, d - lo);
}

// The per-tile shared-memory views of one CTA.
template <typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
struct MergeSmem {
    using L = MergeLayout<VT, XT, AT, NT, IPT, STAGES>;
    unsigned char* base;
    __device__ VT* vals(int s) const { return reinterpret_cast<VT*>(base + s * L::STAGE_B); }
    __device__ int32_t* cols(int s) const { return reinterpret_cast<int32_t*>(base + s * L::STAGE_B + L::VAL_B); }
    __device__ int32_t* rows(int s) const {
        return reinterpret_cast<int32_t*>(base + s * L::STAGE_B + L::VAL_B + L::COL_B);
    }
    __device__ XT* xg() const { return reinterpret_cast<XT*>(base + L::XG_OFF); }
    __device__ AT* ys() const { return reinterpret_cast<AT*>(base + L::YS_OFF); }
    __device__ int2* coords() const { return reinterpret_cast<int2*>(base + L::CO_OFF); }
    __device__ int* carry_row() const { return reinterpret_cast<int*>(base + L::CR_OFF); }
    __device__ AT* carry_val() const { return reinterpret_cast<AT*>(base + L::CV_OFF); }
    __device__ TileHdr* hdr() const { return reinterpret_cast<TileHdr*>(base + L::HDR_OFF); }
    __device__ uint64_t* bar() const { return reinterpret_cast<uint64_t*>(base + L::BAR_OFF); }
    __device__ double* red() const { return reinterpret_cast<double*>(base + L::RED_OFF); }
};

// One elected thread: stage tile `tile` into stage `s` (TMA bulk copies).
// Window arithmetic (all counts in elements):
//   values  [k0 & ~(VE-1), roundup(k1, VE))   <= TM + 2VE - 2 <= VAL_CAP
//   columns [k0 & ~3,      roundup(k1, 4))    <= TM + 6       <= COL_CAP
//   rows    [r0 & ~3,      roundup(rlast+2, 4)) with rlast = min(r1, nor-1);
//           r1 - r0 <= TM, so <= TM + 8 <= ROW_CAP
// The rounded ends stay within the kArrayPad padding of each array, every
// global start is 16-byte aligned (allocations are 256-byte aligned) and
// every size is a multiple of 16 bytes.  A tile always holds r0 <= nor-1, so
// the row window is never empty.
template <typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
__device__ __forceinline__ void issue_tile(const MergeSmem<VT, XT, AT, NT, IPT, STAGES>& sm, int s, int tile,
                                           const int2* __restrict__ tiles, const int32_t* __restrict__ row_start,
                                           const int32_t* __restrict__ col, const VT* __restrict__ val, int nor,
                                           uint64_t pol) {
    using L = MergeLayout<VT, XT, AT, NT, IPT, STAGES>;
    int2 c0 = tiles[tile], c1 = tiles[tile + 1];
    int r0 = c0.x, k0 = c0.y, r1 = c1.x, k1 = c1.y;
    int nk = k1 - k0;
    int rlast = r1 < nor - 1 ? r1 : nor - 1;
    int k0a = k0 & ~(L::VE - 1);
    int k1a = nk ? ((k1 + L::VE - 1) & ~(L::VE - 1)) : k0a;
    int k0c = k0 & ~3;
    int k1c = nk ? ((k1 + 3) & ~3) : k0c;
    int rs = r0 & ~3;
    int re = (rlast + 2 + 3) & ~3;
    uint32_t vb = (uint32_t)(k1a - k0a) * (uint32_t)sizeof(VT);
    uint32_t cb = (uint32_t)(k1c - k0c) * 4u;
    uint32_t rb = (uint32_t)(re - rs) * 4u;
    TileHdr h;
    h.r0 = r0; h.k0 = k0; h.r1 = r1; h.k1 = k1;
    h.voff = k0 - k0a; h.coff = k0 - k0c; h.roff = r0 - rs; h.pad = 0;
    sm.hdr()[s] = h;
    uint64_t* bar = &sm.bar()[s];
    mbar_arrive_expect_tx(bar, vb + cb + rb);
    if (vb) bulk_g2s(sm.vals(s), val + k0a, vb, bar, pol);
    if (cb) bulk_g2s(sm.cols(s), col + k0c, cb, bar, pol);
    bulk_g2s(sm.rows(s), row_start + rs, rb, bar, pol);
}

// Epilogue flavours for the rows a tile completes.
enum MergeMode { MODE_SPMV = 0, MODE_POWER = 1 };

// Process one staged tile.  Returns false if the tile's mbarrier wait timed
// out (every thread of the CTA then returns together).
//
// x, y       : input / output vectors
// carries    : carries[tile] = partial sum of the tile's last (unfinished) row
// e          : power-of-two exponent applied to stored rows (MODE_POWER)
// sumsq      : per-thread running sum of squares of stored rows whose value is
//              final here (MODE_POWER)
template <int MODE, typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
__device__ __forceinline__ bool process_tile(const MergeSmem<VT, XT, AT, NT, IPT, STAGES>& sm, int s,
                                             uint32_t parity, int tile, const XT* __restrict__ x,
                                             XT* __restrict__ y, AT* __restrict__ carries, int nor, int e,
                                             double& sumsq, int* status) {
    const int tid = threadIdx.x;
    bool ok = mbar_wait_bounded(&sm.bar()[s], parity, status);
    const TileHdr h = sm.hdr()[s];
    const int nk = ok ? h.k1 - h.k0 : 0;
    const VT* vals = sm.vals(s) + h.voff;    // vals[j] = value of nonzero k0 + j
    const int32_t* cols = sm.cols(s) + h.coff;
    const int32_t* rstart = sm.rows(s) + h.roff;  // rstart[i] = row_start[r0 + i]
    XT* xg = sm.xg();
    AT* ys = sm.ys();
    int2* co = sm.coords();

    // ---- gather x[col] for the tile's nonzeros ----
    for (int j = tid; j < nk; j += NT) xg[j] = __ldg(x + cols[j]);

    // ---- this thread's start on the merge path (search on the row window) ----
    if (ok) {
        const int d0 = h.r0 + h.k0, d1 = h.r1 + h.k1;
        const int d = d0 + tid * IPT;
        int2 c;
        if (d >= d1) {
            c = make_int2(h.r1, h.k1);
        } else {
            // the answer lies in [max(r0, d - k1), min(r1, d - k0)]; every pivot
            // is < r1, so row_end[pivot] = rstart[pivot + 1 - r0] is staged.
            int lo = d - h.k1 > h.r0 ? d - h.k1 : h.r0;
            int hi = d - h.k0 < h.r1 ? d - h.k0 : h.r1;
            while (lo < hi) {
                int pivot = (lo + hi) >> 1;
                if (rstart[pivot + 1 - h.r0] <= d - pivot - 1) lo = pivot + 1;
                else hi = pivot;
            }
            c = make_int2(lo, d - lo);
        }
        co[tid] = c;
        if (tid == 0) co[NT] = make_int2(h.r1, h.k1);
    }
    if (__syncthreads_or(!ok)) return false;

    // ---- consume IPT merge items (CRS_Merge.hpp:115-128) ----
    {
        int2 c = co[tid], ce = co[tid + 1];
        int a = c.x, b = c.y;
        AT acc = AT(0);
        for (; a < ce.x; ++a) {
            const int re = rstart[a + 1 - h.r0];
            for (; b < re; ++b) acc = fma((AT)vals[b - h.k0], (AT)xg[b - h.k0], acc);
            ys[a - h.r0] = acc;
            acc = AT(0);
        }
        for (; b < ce.y; ++b) acc = fma((AT)vals[b - h.k0], (AT)xg[b - h.k0], acc);
        sm.carry_row()[tid] = ce.x;
        sm.carry_val()[tid] = acc;
    }
    __syncthreads();

    // ---- carries between threads: the first thread of each run of equal
    //      carry rows adds the run (in thread order) to the row total ----
    {
        const int* cr = sm.carry_row();
        const AT* cv = sm.carry_val();
        const int r = cr[tid];
        if (tid == 0 || cr[tid - 1] != r) {
            AT sum = cv[tid];
            for (int u = tid + 1; u < NT && cr[u] == r; ++u) sum += cv[u];
            if (r < h.r1) ys[r - h.r0] += sum;
            else if (r < nor) carries[tile] = sum;  // r == r1: the tile's unfinished row
        }
    }
    __syncthreads();

    // ---- store the rows completed in this tile ----
    {
        const int nr = h.r1 - h.r0;
        // Row r0's total is final here unless the previous tile already
        // consumed some of its nonzeros (k0 > row_start[r0]); k_merge_fixup
        // then completes it.
        const bool r0_open = h.k0 > rstart[0];
        for (int i = tid; i < nr; i += NT) {
            AT v = ys[i];
            if (MODE == MODE_POWER) {
                v = scale_pow2(v, e);
                if (!(i == 0 && r0_open)) sumsq = fma((double)v, (double)v, sumsq);
            }
            y[h.r0 + i] = (XT)v;
        }
    }
    __syncthreads();
    return true;
}

// Deterministic block reduction of one double per thread (fixed tree).
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (l < NT / 32) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;  // valid in thread 0
}

}  // namespace pwmgpu
