// merge.cuh -- merge-path CRS SpMV tile machinery (sm_103a).
//
// Restates the merge-based SpMV of SOA_Implementations/CRS_Merge.hpp:95-141
// (after Merrill & Garland, SC'16) for GB300.
//
// Work decomposition
//  * The merge path (row ends of row_start+1 merged with the nonzero indices,
//    N + nnz items) is cut into SUB-TILES of WM = 32*IPT items, one per warp.
//    Sub-tile s spans diagonals [s*WM, min((s+1)*WM, N+nnz)); its end points
//    come from the binary search of CRS_Merge::searchPathOnDiag (:42-62) and
//    are computed once per matrix (k_merge_partition), not per SpMV.
//  * W = NT/32 consecutive sub-tiles form a TILE, the unit one CTA stages in
//    shared memory: one elected thread streams the tile's values, column
//    indices and row-start window with TMA bulk copies (16-byte granules, L2
//    evict-first), STAGES tiles ahead, completing on a "full" mbarrier.
//  * Each warp then works alone on its sub-tile -- no CTA-wide barrier in the
//    loop; when done it arrives on the stage's "empty" mbarrier, which the
//    producer waits on before refilling the stage.
//
// Inside a sub-tile (rows [rw0, rw1) complete, nonzeros [kw0, kw1)):
//  * the nonzeros are split evenly over the 32 lanes (q = ceil(nnz/32) each),
//    so every FP64 FMA is useful and warp-uniform: on GB300 the FP64 pipe
//    (2 DFMA/clk/SM) is a co-bottleneck with HBM, and a divergent DFMA costs a
//    full warp slot;
//  * a lane first issues all its x[col] gathers (independent loads in
//    registers), then runs q FMAs; a row end stores the row total straight
//    to y (empty rows are written as 0 by the lane that passes them);
//  * each lane's partial last row is its carry; the first lane of each run
//    of lanes with the same carry row adds the run (lane order) to the row's
//    total -- deterministic, like the reference's serial fix-up (:136-140).
//    The sub-tile's own unfinished row goes to carries[sub] for
//    k_merge_fixup;
//  * the power-method epilogue rescales each stored row by an exact power of
//    two and sums squares where the row's final value is known.
#pragma once
#include <climits>

#include "common.cuh"

namespace pwmgpu {

constexpr int a16(long long b) { return (int)((b + 15) / 16 * 16); }

template <int W>
struct TileHdr {
    int r0, k0, r1, k1;    // merge coordinates of the tile's start and end
    int voff, coff, roff;  // offsets of element k0 / k0 / row r0 in the staged windows
    int nsub;              // sub-tiles in this tile (<= W)
    int slow;              // bit w: sub-tile w holds an empty row (general path)
    int2 sub[W + 1];       // sub-tile boundaries
};

template <typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
struct MergeLayout {
    static constexpr int W = NT / 32;
    static constexpr int WM = 32 * IPT;  // merge items per sub-tile (warp)
    static constexpr int TM = W * WM;    // merge items per tile (CTA)
    static constexpr int VE = 16 / (int)sizeof(VT);
    static constexpr int VAL_CAP = TM + 2 * VE;
    static constexpr int COL_CAP = TM + 8;
    static constexpr int ROW_CAP = TM + 12;
    static constexpr int VAL_B = a16((long long)VAL_CAP * sizeof(VT));
    static constexpr int COL_B = a16((long long)COL_CAP * 4);
    static constexpr int ROW_B = a16((long long)ROW_CAP * 4);
    static constexpr int STAGE_B = VAL_B + COL_B + ROW_B;
    static constexpr int CR_OFF = STAGES * STAGE_B;
    static constexpr int CV_OFF = CR_OFF + a16((long long)NT * 4);
    static constexpr int HV_OFF = CV_OFF + a16((long long)NT * sizeof(AT));
    static constexpr int HDR_OFF = HV_OFF + a16((long long)NT * sizeof(AT));
    static constexpr int BAR_OFF = HDR_OFF + a16((long long)STAGES * sizeof(TileHdr<W>));
    static constexpr int RED_OFF = BAR_OFF + a16((long long)2 * STAGES * 8);
    static constexpr int BYTES = RED_OFF + a16(32 * 8);
    // CTAs per SM the shared memory allows (228 KB per SM, 1 KB reserved per
    // CTA), capped by 2048 threads per SM; used as the launch-bounds hint.
    static constexpr int MINB_RAW = 233472 / (BYTES + 1024);
    static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW * NT > 2048 ? 2048 / NT : MINB_RAW);
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

template <typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
struct MergeSmem {
    using L = MergeLayout<VT, XT, AT, NT, IPT, STAGES>;
    unsigned char* base;
    __device__ VT* vals(int s) const { return reinterpret_cast<VT*>(base + s * L::STAGE_B); }
    __device__ int32_t* cols(int s) const { return reinterpret_cast<int32_t*>(base + s * L::STAGE_B + L::VAL_B); }
    __device__ int32_t* rows(int s) const {
        return reinterpret_cast<int32_t*>(base + s * L::STAGE_B + L::VAL_B + L::COL_B);
    }
    __device__ int* carry_row() const { return reinterpret_cast<int*>(base + L::CR_OFF); }
    __device__ AT* carry_val() const { return reinterpret_cast<AT*>(base + L::CV_OFF); }
    __device__ AT* head_val() const { return reinterpret_cast<AT*>(base + L::HV_OFF); }
    __device__ TileHdr<L::W>* hdr() const { return reinterpret_cast<TileHdr<L::W>*>(base + L::HDR_OFF); }
    __device__ uint64_t* full() const { return reinterpret_cast<uint64_t*>(base + L::BAR_OFF); }
    __device__ uint64_t* empty() const { return reinterpret_cast<uint64_t*>(base + L::BAR_OFF) + STAGES; }
    __device__ double* red() const { return reinterpret_cast<double*>(base + L::RED_OFF); }
};

// One elected thread: stage tile `tile` (sub-tiles [tile*W, min((tile+1)*W,
// nsub_total))) into stage `s` with TMA bulk copies.  Window arithmetic (counts
// in elements):
//   values  [k0 & ~(VE-1), roundup(k1, VE))   <= TM + 2VE - 2 <= VAL_CAP
//   columns [k0 & ~3,      roundup(k1, 4))    <= TM + 6       <= COL_CAP
//   rows    [r0 & ~3,      roundup(rlast+2, 4)) with rlast = min(r1, nor-1);
//           r1 - r0 <= TM, so <= TM + 8 <= ROW_CAP
// The rounded ends stay inside the kArrayPad padding of each array, every
// global start is 16-byte aligned (allocations are 256-byte aligned) and
// every size is a multiple of 16 bytes.  A non-empty tile has r0 <= nor-1,
// so the row window is never empty.
template <typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
__device__ __forceinline__ void issue_tile(const MergeSmem<VT, XT, AT, NT, IPT, STAGES>& sm, int s, int tile,
                                           const int2* __restrict__ subc, const uint8_t* __restrict__ subflag,
                                           int nsub_total,
                                           const int32_t* __restrict__ row_start, const int32_t* __restrict__ col,
                                           const VT* __restrict__ val, int nor, uint64_t pol) {
    using L = MergeLayout<VT, XT, AT, NT, IPT, STAGES>;
    const int s0 = tile * L::W;
    const int s1 = s0 + L::W < nsub_total ? s0 + L::W : nsub_total;
    TileHdr<L::W>& h = sm.hdr()[s];
    int slow = 0;
    for (int j = 0; j <= s1 - s0; ++j) h.sub[j] = subc[s0 + j];
    for (int j = 0; j < s1 - s0; ++j) slow |= (subflag[s0 + j] ? 1 : 0) << j;
    h.slow = slow;
    const int r0 = h.sub[0].x, k0 = h.sub[0].y, r1 = h.sub[s1 - s0].x, k1 = h.sub[s1 - s0].y;
    const int nk = k1 - k0;
    const int rlast = r1 < nor - 1 ? r1 : nor - 1;
    const int k0a = k0 & ~(L::VE - 1);
    const int k1a = nk ? ((k1 + L::VE - 1) & ~(L::VE - 1)) : k0a;
    const int k0c = k0 & ~3;
    const int k1c = nk ? ((k1 + 3) & ~3) : k0c;
    const int rs = r0 & ~3;
    const int re = (rlast + 2 + 3) & ~3;
    const uint32_t vb = (uint32_t)(k1a - k0a) * (uint32_t)sizeof(VT);
    const uint32_t cb = (uint32_t)(k1c - k0c) * 4u;
    const uint32_t rb = (uint32_t)(re - rs) * 4u;
    h.r0 = r0; h.k0 = k0; h.r1 = r1; h.k1 = k1;
    h.voff = k0 - k0a; h.coff = k0 - k0c; h.roff = r0 - rs; h.nsub = s1 - s0;
    uint64_t* bar = &sm.full()[s];
    mbar_arrive_expect_tx(bar, vb + cb + rb);
    if (vb) bulk_g2s(sm.vals(s), val + k0a, vb, bar, pol);
    if (cb) bulk_g2s(sm.cols(s), col + k0c, cb, bar, pol);
    bulk_g2s(sm.rows(s), row_start + rs, rb, bar, pol);
}

enum MergeMode { MODE_SPMV = 0, MODE_POWER = 1 };

// Warp `w` processes its sub-tile of the tile staged in stage `s`
// (rows [rw0, rw1) complete here, nonzeros [kw0, kw1)).
//   x, y      input / output vectors
//   carries   carries[sub] = partial sum of the sub-tile's unfinished last row
//   e         power-of-two exponent applied to stored rows (MODE_POWER)
//   sumsq     per-lane running sum of squares (MODE_POWER); every row is
//             counted exactly once, by whoever writes its final value:
//               * the lane that completes it, if the row began in that lane;
//               * the first lane of the carry run, if the row began in an
//                 earlier lane of this sub-tile;
//               * k_merge_fixup, if the row began in an earlier sub-tile.
template <int MODE, typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
__device__ __forceinline__ void process_subtile(const MergeSmem<VT, XT, AT, NT, IPT, STAGES>& sm, int s, int tile,
                                                const XT* __restrict__ x, XT* __restrict__ y,
                                                AT* __restrict__ carries, int nor, int e, double& sumsq) {
    using L = MergeLayout<VT, XT, AT, NT, IPT, STAGES>;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const TileHdr<L::W>& h = sm.hdr()[s];
    if (w >= h.nsub) return;  // the last tile may hold fewer sub-tiles
    const int2 c0 = h.sub[w], c1 = h.sub[w + 1];
    const int rw0 = c0.x, kw0 = c0.y, rw1 = c1.x, kw1 = c1.y;
    const VT* vals = sm.vals(s) + h.voff - h.k0;        // vals[b] for global nonzero b
    const int32_t* cols = sm.cols(s) + h.coff - h.k0;
    const int32_t* rstart = sm.rows(s) + h.roff - h.r0;  // rstart[r] = row_start[r], r in [r0, rlast+1]

    // ---- split the sub-tile's nonzeros over the lanes ----
    const int nkw = kw1 - kw0;
    const int q = (nkw + 31) >> 5;  // <= IPT: a sub-tile holds at most 32*IPT items
    const int b0 = kw0 + lane * q;
    int qe = kw1 - b0;              // this lane's count, in [0, q]
    qe = qe < 0 ? 0 : (qe > q ? q : qe);

    // ---- gathers first (independent loads in flight), then values ----
    AT xv[IPT], vv[IPT];
#pragma unroll
    for (int j = 0; j < IPT; ++j) xv[j] = (j < qe) ? (AT)__ldg(x + cols[b0 + j]) : AT(0);
#pragma unroll
    for (int j = 0; j < IPT; ++j) vv[j] = (j < qe) ? (AT)vals[b0 + j] : AT(0);

    // ---- the row holding the lane's first nonzero ----
    int a = rw1;
    if (qe > 0) {
        int lo = rw0, hi = rw1;  // largest a in [rw0, rw1] with row_start[a] <= b0
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (rstart[mid] <= b0) lo = mid;
            else hi = mid - 1;
        }
        a = lo;
    }
    // Rows >= rw1 never complete here: row rw1's end item belongs to the next
    // sub-tile, so the lane's part of row rw1 leaves as the sub-tile's carry.
    // The lane's first row began in an earlier lane (or an earlier sub-tile).
    const bool head_open = qe > 0 && rstart[a] < b0;

    // rows [rw0, first row of lane 0) have no nonzeros in this sub-tile
    const int a_lane0 = __shfl_sync(0xffffffffu, a, 0);
    for (int r = rw0 + lane; r < a_lane0; r += 32) y[r] = (XT)0;

    AT* hval = sm.head_val() + 32 * w;
    AT acc = AT(0);
    if (!((h.slow >> w) & 1)) {
        // ---- fast path (no empty row in this sub-tile): the positions where
        //      the lane's rows end, as a bit mask; the FMA loop then stores
        //      with a short predicated block instead of a branchy one ----
        uint32_t mask = 0;
        for (int r = a; r < rw1; ++r) {
            const int rr = rstart[r + 1];
            if (rr > b0 + qe) break;
            mask |= 1u << (rr - b0 - 1);
        }
        // The first completed row goes to hval[lane] when it began in an
        // earlier lane of this sub-tile; the carry run's first lane writes it.
        const bool to_head = head_open && lane > 0;
        XT* dst = to_head ? (XT*)(hval + lane) : y + a;
        bool count = !head_open;  // whether this row's square is final here
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            if (j < q) {
                acc = fma(vv[j], xv[j], acc);
                if ((mask >> j) & 1u) {
                    AT v = acc;
                    if (MODE == MODE_POWER) {
                        v = scale_pow2(v, e);
                        if (count) sumsq = fma((double)v, (double)v, sumsq);
                        count = true;
                    }
                    *dst = (XT)v;
                    acc = AT(0);
                    ++a;
                    dst = y + a;
                }
            }
        }
    } else {
        // ---- general path: row ends of the next four rows in registers,
        //      empty rows written as 0 as the lane passes them ----
        auto row_end = [&](int r) { return r < rw1 ? rstart[r + 1] : INT_MAX; };
        int re0 = row_end(a), re1 = row_end(a + 1), re2 = row_end(a + 2), re3 = row_end(a + 3);
        bool first = true;
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            if (j < q) {
                acc = fma(vv[j], xv[j], acc);
                const int bn = b0 + j + 1;
                if (j < qe && bn == re0) {
                    AT v = acc;
                    if (MODE == MODE_POWER) v = scale_pow2(v, e);
                    if (first && head_open && lane > 0) {
                        hval[lane] = v;
                    } else {
                        y[a] = (XT)v;
                        if (MODE == MODE_POWER && !(first && head_open)) sumsq = fma((double)v, (double)v, sumsq);
                    }
                    acc = AT(0);
                    first = false;
                    ++a;
                    re0 = re1; re1 = re2; re2 = re3; re3 = row_end(a + 3);
                    if (re0 == bn) {  // empty rows: their end equals this position
                        do {
                            y[a] = (XT)0;
                            ++a;
                            re0 = re1; re1 = re2; re2 = re3; re3 = row_end(a + 3);
                        } while (re0 == bn);
                    }
                }
            }
        }
    }

    // ---- carries: the first lane of each run of lanes ending in the same
    //      row adds the run (lane order) to the row ----
    int* crow = sm.carry_row() + 32 * w;
    AT* cval = sm.carry_val() + 32 * w;
    crow[lane] = a;
    cval[lane] = acc;
    __syncwarp();
    if (lane == 0 || crow[lane - 1] != a) {
        AT sum = acc;
        int u = lane + 1;
        for (; u < 32 && crow[u] == a; ++u) sum += cval[u];
        if (a < rw1) {
            // Lane u completes row a.  If the row began before lane u, lane u
            // left its part in hval[u] and the total is written here.
            const int rs_a = rstart[a];
            if (rs_a < kw0 + u * q) {
                const AT v = hval[u] + (MODE == MODE_POWER ? scale_pow2(sum, e) : sum);
                y[a] = (XT)v;
                // final now if the row began in this sub-tile; otherwise
                // k_merge_fixup adds the earlier sub-tiles' carries and counts it
                if (MODE == MODE_POWER && rs_a >= kw0) sumsq = fma((double)v, (double)v, sumsq);
            }
        } else if (a < nor) {
            carries[tile * L::W + w] = sum;  // a == rw1: the sub-tile's unfinished row
        }
    }
    __syncwarp();
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
