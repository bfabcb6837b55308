// merge.cuh -- merge-path CRS SpMV for sm_103a: lane-interleaved layout.
//
// Restates the merge-based SpMV of SOA_Implementations/CRS_Merge.hpp:95-141
// (after Merrill & Garland, SC'16) for GB300.
//
// Work decomposition
//  * The merge path (row ends of row_start+1 merged with the nonzero indices,
//    N + nnz items) is cut into SUB-TILES of WM = 32*IPT items, one per warp.
//    Sub-tile s spans diagonals [s*WM, min((s+1)*WM, N+nnz)); its end points
//    come from the binary search of CRS_Merge::searchPathOnDiag (:42-62),
//    computed once per matrix (k_merge_partition).  Rows [rw0, rw1) complete
//    in the sub-tile, which holds nonzeros [kw0, kw1).
//  * The sub-tile's nonzeros are split evenly over the 32 lanes: lane l owns
//    the contiguous range [kw0 + start_l, + cnt_l), qm = nkw/32, rem = nkw%32,
//    cnt_l = qm + (l < rem).  Each lane accumulates its range in order with
//    one FMA per nonzero -- the only FP64 arithmetic per nonzero: GB300's FP64
//    pipe (2 DFMA/clk/SM) is a co-bottleneck with HBM.
//
// Storage (built once per matrix by k_mli_plan, "lane-interleaved")
//  * Each sub-tile's data is contiguous, so a warp stages the sub-tiles it
//    will process with four TMA bulk copies each (record, masks, columns,
//    values) into its own two shared-memory stages -- no CTA-wide
//    coordination at all: while sub-tile i is processed, i+1 is loading.
//  * Values and column indices of sub-tile s are stored from an 8-element-
//    aligned base so that element j of lane l sits at mli_pos(l, j, qm, V)
//    with V = lane_vec<T>() = 2 for every array: pairs of slots (2b, 2b+1)
//    of all 32 lanes form one contiguous block of 2-element vectors (one
//    vector load per lane: 16 bytes for FP64 values, 8 for column indices,
//    conflict-free and consecutive across the warp), then a tail of at most
//    two scalar slots (the partial last one holds lanes < rem only), so the
//    span is exactly nkw elements.  The global reads are the TMA bulk copies
//    of the whole span.  (Wider blocks -- 16 bytes of column indices -- need a
//    tail of up to four scalars per lane that costs more than it saves;
//    scalar-only slots double the loads of full sub-tiles.)
//  * Per lane, a 16-bit mask marks the elements that end a row (precomputed
//    from row_start), so no row-pointer search runs per SpMV: a lane's first
//    row is the sub-tile's first row plus a warp prefix sum of mask popcounts.
//    Sub-tiles that hold an empty row take a general path that walks
//    row_start instead (empty rows are written as 0).
//
// Carries: a lane's partial last row is its carry; the first lane of each run
// of lanes ending in the same row adds the run (lane order) to the row total
// -- deterministic, like the reference's serial fix-up (:136-140).  The
// sub-tile's own unfinished row goes to carries[s] for k_merge_fixup.
#pragma once
#include <climits>
#include <type_traits>

#include "common.cuh"

namespace pwmgpu {

// Padding (in elements) every device array of a matrix carries past its end.
constexpr int kArrayPad = 16;

constexpr int kFlagGeneral = 1;  // the sub-tile holds an empty row
constexpr int kFlagOpen0 = 2;    // the sub-tile's first row began in an earlier sub-tile

// Position of element j of lane l inside a sub-tile with qm = nkw/32, for an
// array of V-element 16-byte vectors.
__host__ __device__ __forceinline__ int mli_pos(int lane, int j, int qm, int V) {
    const int B = qm / V;
    return (j < V * B) ? (j / V) * 32 * V + lane * V + (j % V) : 32 * V * B + (j - V * B) * 32 + lane;
}

// 8-element-aligned storage base of sub-tile s whose nonzeros start at kw0:
// base(s+1) - base(s) >= nkw(s), so sub-tiles never overlap; the arrays hold
// mli_size(nnz, nsub) elements.
__host__ __device__ __forceinline__ long long mli_base(long long kw0, long long s) {
    return 8 * ((kw0 + 7 * s + 7) / 8);
}

__host__ __device__ __forceinline__ long long mli_size(long long nnz, long long nsub) {
    return nnz + 7 * nsub + 16;
}

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

// Largest a in [lo, hi] with row_start[a] <= b (the row holding nonzero b).
__device__ __forceinline__ int row_of(const int32_t* __restrict__ row_start, int b, int lo, int hi) {
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(row_start + mid) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Load this lane's cnt elements of a lane-interleaved sub-tile staged in
// shared memory: 16-byte vector loads for the full blocks (consecutive lanes
// read consecutive 16-byte chunks: conflict-free), scalar loads for the
// tail; zeros beyond cnt.
// Width (elements) of the vector blocks of the lane-interleaved layout for
// element type T: 1 stores element j of lane l at j * 32 + l (every slot one
// conflict-free scalar load, no tail), 16 / sizeof(T) uses 16-byte blocks
// followed by a scalar tail.
#ifndef PWMGPU_LANE_VEC
#define PWMGPU_LANE_VEC 2
#endif
template <typename T>
__host__ __device__ constexpr int lane_vec() {
    return PWMGPU_LANE_VEC;
}

template <typename T, int IPT>
__device__ __forceinline__ void load_lane(const T* p, int qm, int cnt, int lane, T (&out)[IPT]) {
    constexpr int V = lane_vec<T>();
    if (V == 1) {
        const int q = qm + (__any_sync(0xffffffffu, cnt > qm) ? 1 : 0);  // warp-uniform slot count
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            out[j] = T(0);
            if (j < q && j < cnt) out[j] = p[j * 32 + lane];
        }
        return;
    }
    if (V == 2 && IPT % 2 == 0) {
        // block b < B: one 2-element vector load; block b == B: the tail (at
        // most 2 elements, scalar); later blocks: zeros.  B is warp-uniform.
        const int B = qm / 2;
        union Vec2 {
            typename std::conditional<sizeof(T) == 8, uint4, typename std::conditional<sizeof(T) == 4, uint2,
                                                                                        unsigned int>::type>::type u;
            T t[2];
        };
#pragma unroll
        for (int b = 0; b < IPT / 2; ++b) {
            if (b < B) {
                Vec2 v;
                v.u = *reinterpret_cast<const decltype(v.u)*>(p + b * 64 + lane * 2);
                out[2 * b] = v.t[0];
                out[2 * b + 1] = v.t[1];
            } else if (b == B) {
                out[2 * b] = (2 * b < cnt) ? p[64 * B + lane] : T(0);
                out[2 * b + 1] = (2 * b + 1 < cnt) ? p[64 * B + 32 + lane] : T(0);
            } else {
                out[2 * b] = T(0);
                out[2 * b + 1] = T(0);
            }
        }
        return;
    }
    constexpr int NB = (IPT + V - 1) / V;
    const int B = qm / V;
    union Vec {
        uint4 u;
        T t[V];
    };
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        if (b < B) {
            Vec v;
            v.u = *reinterpret_cast<const uint4*>(p + b * 32 * V + lane * V);
#pragma unroll
            for (int k = 0; k < V; ++k)
                if (b * V + k < IPT) out[b * V + k] = v.t[k];
        }
    }
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
        if (j >= V * B) out[j] = (j < cnt) ? p[32 * V * B + (j - V * B) * 32 + lane] : T(0);
    }
}

// Fold a warp's magnitude keys into a max in global memory (one atomic per
// warp; call with the whole warp).
__device__ __forceinline__ void warp_max_out(unsigned mx, unsigned int* out) {
    mx = __reduce_max_sync(0xffffffffu, mx);
    if ((threadIdx.x & 31) == 0 && mx != 0u) atomicMax(out, mx);
}

// The same for a whole CTA of NT threads (call with all of them): one
// atomic per CTA (atomics on one address are serialised where it lives; a
// 4096^2 pass makes 912 instead of 3648).
template <int NT>
__device__ __forceinline__ void block_max_out(unsigned mx, unsigned int* out) {
    __shared__ unsigned wmax[NT / 32];
    mx = __reduce_max_sync(0xffffffffu, mx);
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned m = threadIdx.x < NT / 32 ? wmax[threadIdx.x] : 0u;
        m = __reduce_max_sync(0xffffffffu, m);
        if (threadIdx.x == 0 && m != 0u) atomicMax(out, m);
    }
}

// MODE_SPMV: y = A x.  MODE_POWER: y = 2^e A x with ||y||^2 summed (the power
// method's steps whose norm is used).  MODE_SCALE: y = 2^e A x tracking only
// the largest |y_i| (magnitude keys, integer max) -- the power method's
// intermediate steps, whose norm serves only the exponent of the exact
// power-of-two rescale.
enum MergeMode { MODE_SPMV = 0, MODE_POWER = 1, MODE_SCALE = 2 };

// One warp's shared-memory stage: the staged sub-tile's record, row-end
// masks, lane-interleaved columns and values.  C16: the columns are stored as
// 16-bit offsets from a per-sub-tile base (rec0.w).
template <typename VT, int IPT, bool C16 = false>
struct WarpStage {
    static constexpr int WM = 32 * IPT;
    static constexpr int REC_B = 32;                // int4 rec0, rec1
    static constexpr int MASK_B = 64;               // 32 x uint16
    static constexpr int COL_B = WM * (C16 ? 2 : 4);  // multiple of 16
    static constexpr int VAL_B = WM * (int)sizeof(VT);
    static constexpr int BYTES = REC_B + MASK_B + COL_B + VAL_B;
    static_assert(BYTES % 16 == 0, "stage must keep 16-byte alignment");
};

// Lane 0: stage sub-tile s into `st` with TMA bulk copies.  r1 = rec1 of the
// sub-tile ({fr, flags, base, nkw}), loaded one iteration earlier so the
// issue does not wait on it.  Sizes are rounded up to 16 bytes; the arrays
// carry slack past the last sub-tile, so the rounded copies stay inside.
template <typename VT, int IPT, bool C16 = false>
__device__ __forceinline__ void issue_subtile(unsigned char* st, uint64_t* bar, int s, int4 r1,
                                              const int4* __restrict__ rec, const uint16_t* __restrict__ masks,
                                              const int32_t* __restrict__ colp, const uint16_t* __restrict__ colp16,
                                              const VT* __restrict__ valp, uint64_t pol) {
    using S = WarpStage<VT, IPT, C16>;
    const int base = r1.z, nkw = r1.w;
    const uint32_t cb = (uint32_t)((nkw * (C16 ? 2 : 4) + 15) & ~15);
    const uint32_t vb = (uint32_t)((nkw * (int)sizeof(VT) + 15) & ~15);
    mbar_arrive_expect_tx(bar, S::REC_B + S::MASK_B + cb + vb);
    bulk_g2s(st, rec + 2LL * s, S::REC_B, bar, pol);
    bulk_g2s(st + S::REC_B, masks + 32LL * s, S::MASK_B, bar, pol);
    if (cb) {
        if (C16) bulk_g2s(st + S::REC_B + S::MASK_B, colp16 + base, cb, bar, pol);
        else bulk_g2s(st + S::REC_B + S::MASK_B, colp + base, cb, bar, pol);
    }
    if (vb) bulk_g2s(st + S::REC_B + S::MASK_B + S::COL_B, valp + base, vb, bar, pol);
}

// First half of a sub-tile: the lane's gathers x[col], all issued together
// (read from the staged columns).
// XCOH: x was written earlier in the same launch (persistent power kernel), so
// it is read with ordinary coherent loads (ld.global.ca: L1-cached, and
// ordered after the grid barrier's acquire) instead of the read-only
// non-coherent path.
// CG: gathers of columns far from the sub-tile's rows bypass L1
// (ld.global.cg: where x is spread too widely for L1 to hit), columns within
// kNearRows of its first row use ld.global.ca.  On the irregular
// lognormal-row matrix the split ran 6 % faster than bypassing L1 for all
// gathers (fewer short-scoreboard stalls; the L1 hit rate stayed at 3 %).
// The launch tuner decides per matrix between this and plain read-only
// gathers.
constexpr int kNearRows = 4096;

template <typename VT, typename XT, typename AT, int IPT, bool XCOH = false, bool C16 = false, bool CG = false>
__device__ __forceinline__ void gather_subtile(const unsigned char* st, const XT* __restrict__ x, AT (&xv)[IPT]) {
    using S = WarpStage<VT, IPT, C16>;
    const int lane = threadIdx.x & 31;
    const int nkw = reinterpret_cast<const int4*>(st)[1].w;
    const int qm = nkw >> 5, rem = nkw & 31;
    const int cnt = qm + (lane < rem ? 1 : 0);
    int32_t cv[IPT];
    if (C16) {
        uint16_t c16[IPT];
        load_lane<uint16_t, IPT>(reinterpret_cast<const uint16_t*>(st + S::REC_B + S::MASK_B), qm, cnt, lane, c16);
        const int cbase = reinterpret_cast<const int4*>(st)[0].w;
#pragma unroll
        for (int j = 0; j < IPT; ++j) cv[j] = cbase + (int)c16[j];
    } else {
        load_lane<int32_t, IPT>(reinterpret_cast<const int32_t*>(st + S::REC_B + S::MASK_B), qm, cnt, lane, cv);
    }
    if (XCOH) {
#pragma unroll
        for (int j = 0; j < IPT; ++j) xv[j] = (j < cnt) ? (AT)__ldca(x + cv[j]) : AT(0);
    } else if (CG) {
        const int rw0 = reinterpret_cast<const int4*>(st)[0].x;
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            const bool near = (unsigned)(cv[j] - rw0 + kNearRows) < 2u * kNearRows;
            xv[j] = (j < cnt) ? (near ? (AT)__ldca(x + cv[j]) : (AT)__ldcg(x + cv[j])) : AT(0);
        }
    } else {
#pragma unroll
        for (int j = 0; j < IPT; ++j) xv[j] = (j < cnt) ? (AT)__ldg(x + cv[j]) : AT(0);
    }
}

// Second half: FMAs over the staged values, row completion, carries.
//   x, y      input / output vectors
//   carries   carries[s] = partial sum of the sub-tile's unfinished last row
//   e         MODE_POWER: rows are stored times 2^e (exact rescale of the
//             power method's iterate; a warp-uniform skip when e == 0)
//   crow, cval, hval   this warp's 32-entry shared scratch
//   ss        NORM: += the FP64 squares of the rows this sub-tile completes
//             (as stored), except a row that began in an earlier sub-tile:
//             its value here is a partial that the fix-up completes (and
//             squares)
//   mx        MODE_SCALE: max= the magnitude keys of the same rows
// NORM, common path (no empty row in the sub-tile): the completed rows are
// collected in the stage's column / value area -- free once every lane holds
// its columns and values in registers; the rows [fr, rw1) are consecutive --
// and stored from there with coalesced stores, which is also where the
// squares are taken: about (rw1 - fr) / 32 FP64 FMAs per sub-tile instead of
// one predicated FMA per slot.  Without NORM the rows are stored directly
// (the buffer's extra shared-memory round trip made the plain SpMV ~4 %
// slower on the 4096^2 Poisson matrix).
// SC = false: the caller knows e == 0 (no rescale code in the unrolled loop).
template <int MODE, bool GENERAL, typename VT, typename XT, typename AT, int IPT, bool C16 = false,
          bool NORM = false, bool SC = true>
__device__ __forceinline__ void finish_subtile(int s, unsigned char* st, const AT (&xv)[IPT],
                                               const int32_t* __restrict__ row_start, XT* __restrict__ y,
                                               AT* __restrict__ carries, int nor, int e, int* crow, AT* cval,
                                               AT* hval, double& ss, unsigned* mx = nullptr) {
    using S = WarpStage<VT, IPT, C16>;
    static_assert(S::COL_B + S::VAL_B >= S::WM * (int)sizeof(XT), "row buffer must fit the stage");
    const int lane = threadIdx.x & 31;
    const int4 r0 = reinterpret_cast<const int4*>(st)[0];
    const int4 r1 = reinterpret_cast<const int4*>(st)[1];
    const int rw0 = r0.x, kw0 = r0.y, rw1 = r0.z;
    const int fr = r1.x, flags = r1.y, nkw = r1.w;
    const uint32_t mask = reinterpret_cast<const uint16_t*>(st + S::REC_B)[lane];
    const VT* vals = reinterpret_cast<const VT*>(st + S::REC_B + S::MASK_B + S::COL_B);
    const int qm = nkw >> 5, rem = nkw & 31;
    const int cnt = qm + (lane < rem ? 1 : 0);
    const int q = qm + (rem ? 1 : 0);  // warp-uniform trip count (<= IPT)
    const int b0 = kw0 + lane * qm + (lane < rem ? lane : rem);
    VT vr[IPT];
    load_lane<VT, IPT>(vals, qm, cnt, lane, vr);
    // row buffer (common path): rows fr + i at rbuf[i]; every lane has read
    // the stage's columns (gather) and values before any lane writes it
    constexpr bool BUF = NORM && !GENERAL;
    XT* rbuf = reinterpret_cast<XT*>(st + S::REC_B + S::MASK_B);
    if (BUF) __syncwarp();
    // a row that began in an earlier sub-tile completes here as a partial
    const int open_row = (flags & kFlagOpen0) ? fr : -1;

    // ---- the lane's first row ----
    int a;
    bool head_open;  // the lane's first row began before the lane's range
    if (!GENERAL) {
        const int pc = __popc(mask);
        int incl = pc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        a = fr + incl - pc;
        const int lastbit = cnt > 0 ? (int)((mask >> (cnt - 1)) & 1u) : 1;
        const int prev_last = __shfl_up_sync(0xffffffffu, lastbit, 1);
        head_open = lane == 0 ? ((flags & kFlagOpen0) != 0) : (cnt > 0 && !prev_last);
    } else {
        a = cnt > 0 ? row_of(row_start, b0, rw0, rw1) : rw1;
        head_open = cnt > 0 && __ldg(row_start + a) < b0;
    }
    // rows [rw0, fr) carry no nonzeros in this sub-tile
    for (int r = rw0 + lane; r < fr; r += 32) y[r] = (XT)0;

    // ---- FMAs: one per nonzero, warp-uniform trip count ----
    AT acc = AT(0);
    bool to_head = head_open && lane > 0;  // first completed row goes to hval
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
        if (j < q) {
            acc = fma((AT)vr[j], xv[j], acc);
            if ((mask >> j) & 1u) {
                AT v = acc;
                if (MODE != MODE_SPMV && SC && e != 0) v = scale_pow2(v, e);
                if (to_head) {
                    hval[lane] = v;
                } else if (!BUF) {
                    y[a] = (XT)v;
                    if (NORM && a != open_row) ss = fma((double)(XT)v, (double)(XT)v, ss);
                    if (MODE == MODE_SCALE && a != open_row) *mx = max(*mx, mag_key((XT)v));
                } else {
                    rbuf[a - fr] = (XT)v;
                }
                to_head = false;
                acc = AT(0);
                ++a;
                if (GENERAL) {  // empty rows: written as 0 as the lane passes them
                    while (a < rw1 && __ldg(row_start + a + 1) == __ldg(row_start + a)) {
                        y[a] = (XT)0;
                        ++a;
                    }
                }
            }
        }
    }
    if (cnt == 0) a = rw1;

    // ---- carries: the first lane of each run of lanes ending in the same
    //      row adds the run (lane order) to the row ----
    // crow holds the lane's last row, with the top bit set when the lane's
    // first row began before the lane (head_open): the leader of a run needs
    // that flag of the lane completing the row, and reads it here instead of
    // comparing row_start in global memory.
    crow[lane] = a | (head_open && cnt > 0 ? (int)0x80000000u : 0);
    cval[lane] = acc;
    __syncwarp();
    if (lane == 0 || (crow[lane - 1] & 0x7fffffff) != a) {
        AT sum = acc;
        int u = lane + 1;
        int cu = 0;
        for (; u < 32 && ((cu = crow[u]) & 0x7fffffff) == a; ++u) sum += cval[u];
        if (a < rw1) {
            // Lane u completes row a.  If the row began before lane u, lane u
            // left its part in hval[u] and the total is written here.
            if (cu < 0) {
                const XT t = (XT)(hval[u] + (MODE != MODE_SPMV && SC && e != 0 ? scale_pow2(sum, e) : sum));
                if (!BUF) {
                    y[a] = t;
                    if (NORM && a != open_row) ss = fma((double)t, (double)t, ss);
                    if (MODE == MODE_SCALE && a != open_row) *mx = max(*mx, mag_key(t));
                } else {
                    rbuf[a - fr] = t;
                }
            }
        } else if (a < nor) {
            carries[s] = sum;  // a == rw1: the sub-tile's unfinished row
        }
    }
    __syncwarp();
    if (BUF) {
        // the completed rows [fr, rw1), coalesced (the caller's proxy fence
        // before the stage's next TMA refill follows the warp barrier below)
        for (int i = lane; i < rw1 - fr; i += 32) {
            const XT v = rbuf[i];
            y[fr + i] = v;
            if (fr + i != open_row) ss = fma((double)v, (double)v, ss);
        }
        __syncwarp();
    }
}

// Deterministic block reduction of one double per thread (fixed tree).
// ---------------------------------------------------------------------------
// Fix-up: add each sub-tile's carry to the row the sub-tile left unfinished.
// One thread per sub-tile; the first sub-tile of a run of sub-tiles ending in
// the same row adds the run in order (deterministic).  The run's row r is
// completed (and its partial written) by the first sub-tile after the run; the
// carry is real only if that sub-tile started inside row r.  MODE_POWER adds
// the carries times 2^e.  Threads take the first sub-tiles t = t0, t0 +
// stride, ... < t_end (a run starting before t_end may extend past it).
// ---------------------------------------------------------------------------
// NORM: ss += the FP64 squares of the completed rows (as stored); MODE_SCALE:
// mx max= their magnitude keys.
template <int MODE, typename XT, typename AT, bool NORM = false>
__device__ __forceinline__ void fixup_pass(const int32_t* __restrict__ row_start, const int2* __restrict__ tiles,
                                           int nor, int num_tiles, XT* __restrict__ y, const AT* __restrict__ carries,
                                           int e, int t0, int t_end, int stride, double& ss, unsigned* mx = nullptr) {
    for (int t = t0; t < t_end; t += stride) {
        const int r = tiles[t + 1].x;
        if (r >= nor) continue;
        if (t > 0 && tiles[t].x == r) continue;  // not the first sub-tile of the run
        // carries and y[r] were written by other CTAs: read them through L2
        AT sum = __ldcg(carries + t);
        int n = t + 1;
        while (n < num_tiles && tiles[n + 1].x == r) sum += __ldcg(carries + n++);
        // sub-tile n starts at (r, tiles[n].y) and completes row r
        if (tiles[n].y > row_start[r]) {
            const XT v = (XT)((AT)__ldcg(y + r) + (MODE != MODE_SPMV && e != 0 ? scale_pow2(sum, e) : sum));
            y[r] = v;
            if (NORM) ss = fma((double)v, (double)v, ss);
            if (MODE == MODE_SCALE) *mx = max(*mx, mag_key(v));
        }
    }
}

// Sum of squares of y[i] (and, with DOT, sum of x[i] * y[i]) over rows
// i = lo + t0, lo + t0 + stride, ... < hi, in FP64 (loads through L2: y was
// just written, possibly by other CTAs).
// Four rows per step with independent loads and accumulators (combined as
// (s0 + s1) + (s2 + s3) at the end: a fixed order for a fixed launch shape).
template <typename XT, bool DOT>
__device__ __forceinline__ void norm_rows(const XT* __restrict__ y, const XT* __restrict__ x, int lo, int hi, int t0,
                                          int stride, double& ss, double& dd) {
    double s[4] = {0.0, 0.0, 0.0, 0.0}, d[4] = {0.0, 0.0, 0.0, 0.0};
    int i = lo + t0;
    for (; i + 3 * stride < hi; i += 4 * stride) {
        double v[4], w[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[u] = (double)__ldcg(y + i + u * stride);
            if (DOT) w[u] = (double)__ldcg(x + i + u * stride);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            s[u] = fma(v[u], v[u], s[u]);
            if (DOT) d[u] = fma(w[u], v[u], d[u]);
        }
    }
    double sr = 0.0, dr = 0.0;  // the last (up to 3) rows
    for (; i < hi; i += stride) {
        const double v = (double)__ldcg(y + i);
        sr = fma(v, v, sr);
        if (DOT) dr = fma((double)__ldcg(x + i), v, dr);
    }
    ss += ((s[0] + s[1]) + (s[2] + s[3])) + sr;
    if (DOT) dd += ((d[0] + d[1]) + (d[2] + d[3])) + dr;
}

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
