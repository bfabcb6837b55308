// batch.cu -- one power-method step of many solves per launch (the serving
// loop's rounds; no counterpart in the reference, whose power iteration
// serves one matrix per call: CRS.hpp:118-130).
//
// Per step, for every slot j of a class table (see batch.h):
//   k_batch_spmv    v_{k+1} = 2^{e_k} A_j v_k over all slots' sub-tiles
//                   (merge-path sub-tiles, TMA-staged; e_k is an exact
//                   rescale, nonzero only when the norm leaves a wide window)
//   k_batch_fixup   the carries of each slot's sub-tiles
//   k_batch_norm    ||v_{k+1}||^2 (and v_k . v_{k+1} on a round's last step)
//                   per slot, over fixed row chunks in a fixed order; the
//                   slot's last CTA advances the slot state (k, ||v||^2)
// except on a round's steps before its last two ("key steps"), whose norms
// only choose the next exact rescale: there the SpMV and the fix-up fold the
// largest magnitude key of the rows they store into the slot (one atomic max
// per warp and slot; integer work only) and k_batch_keys advances the state;
// the iterates differ from the norm schedule by powers of two only, which the
// final normalisation removes bit for bit.  Once per round
//   k_batch_resid   lambda and ||A u - lambda u||^2 of u = v_{k-1}/||v_{k-1}||.
// The SpMV keeps one FP64 FMA per nonzero and no other FP64 work (GB300's
// FP64 pipe is 2 operations per clock per SM); the sums are row passes.
// Grids are fixed (graph-captured rounds); the kernels read the table's
// sizes from device memory, so one graph serves every composition.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "batch.h"
#include "internal.h"
#include "merge.cuh"
#include "sell.cuh"

namespace pwmgpu {

namespace {

constexpr int kBatchNT = 128;
constexpr int kBatchStages = 2;

// Largest j with key(j) <= v over the ascending per-slot starts.
template <int FIELD>
__device__ __forceinline__ int find_slot(const BatchSlot* __restrict__ slots, int nslots, int v) {
    int lo = 0, hi = nslots - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int key = FIELD == 0 ? __ldg(&slots[mid].tile0) : FIELD == 1 ? __ldg(&slots[mid].fix0)
                                                                            : __ldg(&slots[mid].row0);
        if (key <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// What a warp needs of a sub-tile's slot, loaded one sub-tile ahead.
struct SlotRegs {
    const int32_t* row_start;
    const void* X;
    const void* Y;
    void* carries;
    unsigned int* mx_next;
    int nor, tile0, k, e;
};

// Exponent of the exact 2^e rescale of step k -> k+1: from the largest key of
// v_k after a key step, else from ||v_k||^2; none on the first step.
template <typename XT>
__device__ __forceinline__ int slot_exponent(const SlotState* st) {
    if (st->k <= 0) return 0;
    return st->keyed ? pow2_rescale_exponent_key<XT>(st->mx) : pow2_rescale_exponent(st->nsq, rescale_window<XT>());
}

template <typename XT>
__device__ __forceinline__ void load_slot(const BatchTable& T, int j, SlotRegs& r) {
    const BatchSlot* d = T.slots + j;
    r.row_start = d->row_start;
    r.X = d->X;
    r.Y = d->Y;
    r.carries = d->carries;
    r.nor = d->nor;
    r.tile0 = d->tile0;
    SlotState* st = T.states + d->state;
    r.k = st->k;
    r.e = slot_exponent<XT>(st);
    r.mx_next = &st->mx_next;
}

// Lane 0: the TMA copies of global sub-tile g (slot j, its record r1).
template <typename VT, int IPT>
__device__ __forceinline__ void issue_global(unsigned char* st, uint64_t* bar, const BatchSlot* slots, int j, int g,
                                             int4 r1, uint64_t pol) {
    const BatchSlot* d = slots + j;
    issue_subtile<VT, IPT>(st, bar, g - d->tile0, r1, d->rec, d->masks, d->colp, nullptr, static_cast<const VT*>(d->valp),
                           pol);
}

// Slot and record of global sub-tile g (for a later issue_global).
__device__ __forceinline__ int4 prefetch_rec(const BatchTable& T, int g, int& j) {
    j = __ldg(T.tile_slot + g);
    const BatchSlot* d = T.slots + j;
    return __ldg(d->rec + 2LL * (g - d->tile0) + 1);
}

// Resident CTAs per SM the kernel is compiled for: the low-precision classes
// are latency-bound (no FP64 pipe limit), so they trade registers for warps.
template <typename VT>
constexpr int batch_min_ctas() {
    return sizeof(VT) == 8 ? 5 : 8;
}

// KEYS: a key step (the largest magnitude key of the stored rows into the
// slot's mx_next, one atomic max per warp and slot), else the rows only.
template <typename VT, typename XT, typename AT, int NT, int IPT, bool KEYS = false>
__global__ void __launch_bounds__(NT, batch_min_ctas<VT>()) k_batch_spmv(const BatchTable* __restrict__ Tp) {
    using S = WarpStage<VT, IPT>;
    constexpr int W = NT / 32;
    constexpr int NS = kBatchStages;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bars[W][NS];
    __shared__ int crow_s[NT];
    __shared__ AT cval_s[NT];
    __shared__ AT hval_s[NT];
    const BatchTable T = *Tp;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * W + w, tw = gridDim.x * W;
    const int n = gw < T.ntiles ? (T.ntiles - 1 - gw) / tw + 1 : 0;
    if (n == 0) return;
    unsigned char* stages = smem_raw + (size_t)w * NS * S::BYTES;
    int* crow = crow_s + 32 * w;
    AT* cval = cval_s + 32 * w;
    AT* hval = hval_s + 32 * w;
    const uint64_t pol = policy_evict_first();
    int pj = 0;
    int4 pref = make_int4(0, 0, 0, 0);
    if (lane == 0) {
        for (int k = 0; k < NS; ++k) mbar_init(&bars[w][k], 1);
        fence_mbar_init();
        for (int k = 0; k < NS && k < n; ++k) {
            int j;
            const int4 r1 = prefetch_rec(T, gw + k * tw, j);
            issue_global<VT, IPT>(stages + k * S::BYTES, &bars[w][k], T.slots, j, gw + k * tw, r1, pol);
        }
        if (n > NS) pref = prefetch_rec(T, gw + NS * tw, pj);
    }
    __syncwarp();
    int jc = __ldg(T.tile_slot + gw);
    int jcur = -1;  // slot whose fields are in `cur` (consecutive sub-tiles of a warp often share it)
    SlotRegs cur;
    unsigned mx = 0u;  // KEYS: largest key of the rows stored for slot jcur
    int i = 0;
    for (; i < n; ++i) {
        const int k = i % NS;
        const int g = gw + i * tw;
        unsigned char* st = stages + k * S::BYTES;
        // the slot's fields (when the slot changes) and the next sub-tile's
        // slot: loads in flight during the wait
        if (jc != jcur) {
            if (KEYS && jcur >= 0) {
                warp_max_out(mx, cur.mx_next);
                mx = 0u;
            }
            load_slot<XT>(T, jc, cur);
            jcur = jc;
        }
        const int jn = i + 1 < n ? __ldg(T.tile_slot + g + tw) : 0;
        const bool ok = mbar_wait_bounded(&bars[w][k], (uint32_t)(i / NS) & 1u, T.status);
        if (!__all_sync(0xffffffffu, ok)) break;
        const int e = cur.e;
        const XT* in = static_cast<const XT*>((cur.k & 1) ? cur.Y : cur.X);
        XT* out = const_cast<XT*>(static_cast<const XT*>((cur.k & 1) ? cur.X : cur.Y));
        const int s = g - cur.tile0;
        AT* car = static_cast<AT*>(cur.carries);
        AT xv[IPT];
        gather_subtile<VT, XT, AT, IPT>(st, in, xv);
        const bool general = reinterpret_cast<const int4*>(st)[1].y & kFlagGeneral;
        double no_ss = 0.0;
        constexpr int MODE = KEYS ? MODE_SCALE : MODE_POWER;
        if (general)
            finish_subtile<MODE, true, VT, XT, AT, IPT>(s, st, xv, cur.row_start, out, car, cur.nor, e, crow, cval,
                                                        hval, no_ss, &mx);
        else
            finish_subtile<MODE, false, VT, XT, AT, IPT>(s, st, xv, cur.row_start, out, car, cur.nor, e, crow, cval,
                                                         hval, no_ss, &mx);
        if (lane == 0) {
            if (i + NS < n) {
                fence_proxy_async();
                issue_global<VT, IPT>(st, &bars[w][k], T.slots, pj, g + NS * tw, pref, pol);
                if (i + NS + 1 < n) pref = prefetch_rec(T, g + (NS + 1) * tw, pj);
            }
        }
        __syncwarp();
        jc = jn;
    }
    if (KEYS && jcur >= 0) warp_max_out(mx, cur.mx_next);
    if (i < n) {  // timed out: let this warp's copies in flight land first
        if (lane == 0)
            for (int t = i; t < n && t < i + NS; ++t)
                mbar_wait_bounded(&bars[w][t % NS], (uint32_t)(t / NS) & 1u, T.status, kWaitCycles / 8, false);
        __syncwarp();
    }
}

// ---- SELL-32 classes ------------------------------------------------------
// What a warp needs of a slice's slot (FP32 vectors).
struct SellSlotRegs {
    const int32_t* soff;
    const uint16_t* col16;
    const void* valp;
    const float* in;
    float* out;
    unsigned int* mx_next;
    int nor, tile0, e;
};

__device__ __forceinline__ void load_sell_slot(const BatchTable& T, int j, SellSlotRegs& r) {
    const BatchSlot* d = T.slots + j;
    SlotState* st = T.states + d->state;
    const int k = st->k;
    r.soff = d->soff;
    r.col16 = d->col16;
    r.valp = d->valp;
    r.in = static_cast<const float*>((k & 1) ? d->Y : d->X);
    r.out = static_cast<float*>((k & 1) ? d->X : d->Y);
    r.mx_next = &st->mx_next;
    r.nor = d->nor;
    r.tile0 = d->tile0;
    r.e = slot_exponent<float>(st);
}

// What a SELL step sums besides the rows: nothing (a round's last step, whose
// row pass follows), the squares per slice group (the step before it), or the
// largest magnitude key per slot (the round's earlier steps).
enum SellSum { kSellNone = 0, kSellSquares = 1, kSellKeys = 2 };

// One power step of every live solve of a SELL-32 class: v_{k+1} =
// 2^{e_k} A_j v_k, one lane per row; with kSellSquares also the sums of
// squares of ||v_{k+1}||^2 per slice group (with kSellKeys the slot's largest
// magnitude key instead: one atomic max per warp and slot).  A slot's slices form groups of kSellGroup,
// in the slot's own slice order; warp w takes the consecutive global groups
// [w K, w K + K) (K = groups / warps, rounded up), two slices at a time, so
// its slot advances by a comparison.  Per group the lanes' FP64 sums of
// their rows (widened on the integer pipes) meet in a fixed shuffle tree and
// land in grp_part; k_batch_grp then sums a slot's groups in order.  Rows
// are one lane's sums in CRS order and the grouping depends only on the
// slot: the same bits in any mix.
template <typename VT, int SUM>
__global__ void __launch_bounds__(256, sizeof(VT) == 2 ? 4 : 3) k_batch_sell(const BatchTable* __restrict__ Tp) {
    constexpr bool NORM = SUM == kSellSquares;
    constexpr bool KEYS = SUM == kSellKeys;
    const BatchTable T = *Tp;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, tw = (gridDim.x * blockDim.x) >> 5;
    const int K = (T.nfix + tw - 1) / tw;
    int q = gw * K;
    const int q1 = min(q + K, T.nfix);
    if (q >= q1) return;
    int j = find_slot<1>(T.slots, T.nslots, q);
    SellSlotRegs A;
    load_sell_slot(T, j, A);
    int fix0 = __ldg(&T.slots[j].fix0), nfix = __ldg(&T.slots[j].nfix), nsub = __ldg(&T.slots[j].nsub);
    unsigned mx = 0u;  // KEYS: largest key of the rows stored for slot j
    for (; q < q1; ++q) {
        while (q >= fix0 + nfix) {  // the next slot (slots own consecutive groups)
            if (KEYS) {
                warp_max_out(mx, A.mx_next);
                mx = 0u;
            }
            ++j;
            load_sell_slot(T, j, A);
            fix0 = __ldg(&T.slots[j].fix0);
            nfix = __ldg(&T.slots[j].nfix);
            nsub = __ldg(&T.slots[j].nsub);
        }
        const int s1 = min((q - fix0 + 1) * kSellGroup, nsub);
        double ss = 0.0;
        for (int s = (q - fix0) * kSellGroup; s < s1; s += 2) {
            const bool two = s + 1 < s1;
            const int oa = __ldg(A.soff + s), ob = __ldg(A.soff + s + 1);
            const int oc = two ? __ldg(A.soff + s + 2) : ob;
            float ya, yb;
            sell_rows2<VT, 5>(A.col16 + oa + lane, static_cast<const VT*>(A.valp) + oa + lane, A.in,
                              s * 32 - 32768, (ob - oa) >> 5, A.col16 + ob + lane,
                              static_cast<const VT*>(A.valp) + ob + lane, A.in, s * 32 + 32 - 32768, (oc - ob) >> 5,
                              ya, yb);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = s * 32 + h * 32 + lane;
                const bool live = (h == 0 || two) && r < A.nor;
                float out = h ? yb : ya;
                if (A.e) out = scale_pow2(out, A.e);
                if (live) A.out[r] = out;
                else out = 0.0f;
                if (NORM) {
                    const double wo = __any_sync(0xffffffffu, widen_special(out)) ? (double)out : widen_normal(out);
                    ss = fma(wo, wo, ss);
                }
                if (KEYS) mx = max(mx, mag_key(out));
            }
        }
        if (NORM) {
            for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
            if (lane == 0) T.grp_part[q] = ss;
        }
    }
    if (KEYS) warp_max_out(mx, A.mx_next);
}

// After a NORM step: per slot (one warp each) ||v_{k+1}||^2 = its groups'
// sums in group order, and the slot's state advanced.
__global__ void __launch_bounds__(256) k_batch_grp(const BatchTable* __restrict__ Tp) {
    const BatchTable T = *Tp;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, tw = (gridDim.x * blockDim.x) >> 5;
    for (int j = gw; j < T.nslots; j += tw) {
        const BatchSlot& d = T.slots[j];
        double s0 = 0.0;
        for (int i = lane; i < d.nfix; i += 32) s0 += T.grp_part[d.fix0 + i];
        for (int o = 16; o > 0; o >>= 1) s0 += __shfl_down_sync(0xffffffffu, s0, o);
        if (lane == 0) {
            SlotState* stt = T.states + d.state;
            stt->nsq_prev = stt->nsq;
            stt->nsq = s0;
            stt->keyed = 0;
            stt->k = stt->k + 1;
        }
    }
}

// After a key step: per slot, the step's largest key becomes v_{k+1}'s and
// the state advances (||v||^2 is not known for v_{k+1}).
__global__ void __launch_bounds__(256) k_batch_keys(const BatchTable* __restrict__ Tp) {
    const BatchTable T = *Tp;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < T.nslots; j += gridDim.x * blockDim.x) {
        SlotState* stt = T.states + T.slots[j].state;
        stt->mx = stt->mx_next;
        stt->mx_next = 0u;
        stt->keyed = 1;
        stt->k = stt->k + 1;
    }
}

// tile_slot[g] = the slot owning global sub-tile g (one CTA per slot).
__global__ void k_tile_slots(const BatchTable* __restrict__ Tp) {
    const BatchTable T = *Tp;
    for (int j = blockIdx.x; j < T.nslots; j += gridDim.x) {
        const int t0 = T.slots[j].tile0, nt = T.slots[j].nsub;
        for (int t = threadIdx.x; t < nt; t += blockDim.x) T.tile_slot[t0 + t] = j;
    }
}

// KEYS: a key step (the fixed rows' largest key into the slot's mx_next).
template <typename XT, typename AT, bool KEYS = false>
__global__ void __launch_bounds__(256) k_batch_fixup(const BatchTable* __restrict__ Tp) {
    const BatchTable T = *Tp;
    for (int c = blockIdx.x; c < T.nfix; c += gridDim.x) {
        const int j = find_slot<1>(T.slots, T.nslots, c);
        const BatchSlot& d = T.slots[j];
        SlotState* stt = T.states + d.state;
        const int kit = stt->k;
        const int e = slot_exponent<XT>(stt);
        XT* out = static_cast<XT*>((kit & 1) ? d.X : d.Y);
        const int lo = (c - d.fix0) * kFixTiles;
        const int hi = min(d.nsub, lo + kFixTiles);
        const AT* car = static_cast<const AT*>(d.carries);
        double no_ss = 0.0;
        unsigned mx = 0u;
        fixup_pass<KEYS ? MODE_SCALE : MODE_POWER, XT, AT>(d.row_start, d.subc, d.nor, d.nsub, out, car, e,
                                                           lo + threadIdx.x, hi, blockDim.x, no_ss, &mx);
        if (KEYS) warp_max_out(mx, &stt->mx_next);
    }
}

// Sum of squares of y[lo, hi) (and, with DOT, sum of x y) by the CTA's
// threads: 16-byte vector loads (lo is a multiple of 4 rows; vectors start
// 16-byte aligned), U vectors per thread in flight, one accumulator per
// vector slot combined in a fixed order, then the scalar tail.
template <typename XT, bool DOT>
__device__ __forceinline__ void chunk_sums(const XT* __restrict__ y, const XT* __restrict__ x, int lo, int hi,
                                           double& ss, double& dd) {
    using VecT = typename std::conditional<sizeof(XT) == 4, float4, double2>::type;
    constexpr int V = 16 / (int)sizeof(XT);
    constexpr int U = 4;
    const int t = threadIdx.x, nt = blockDim.x;
    const int nv = (hi - lo) / V;
    const VecT* yv = reinterpret_cast<const VecT*>(y + lo);
    const VecT* xv = reinterpret_cast<const VecT*>(x + lo);
    double s[U] = {}, d[U] = {};
    for (int b = t; b < nv; b += U * nt) {
        VecT a[U], c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (b + u * nt < nv) {
                a[u] = __ldcg(yv + b + u * nt);
                if (DOT) c[u] = __ldcg(xv + b + u * nt);
            } else {
                a[u] = VecT{};
                c[u] = VecT{};
            }
        }
        // FP32 vectors: widened on the integer pipes unless a lane of the
        // warp holds a subnormal, infinity or NaN (rare: then the conversion
        // instruction, warp-uniformly)
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const XT* av = reinterpret_cast<const XT*>(&a[u]);
            const XT* cv = reinterpret_cast<const XT*>(&c[u]);
            bool special = false;
            if (sizeof(XT) == 4) {
#pragma unroll
                for (int k = 0; k < V; ++k) special |= widen_special((float)av[k]) || (DOT && widen_special((float)cv[k]));
            }
            if (sizeof(XT) == 8 || __any_sync(__activemask(), special)) {
#pragma unroll
                for (int k = 0; k < V; ++k) {
                    const double w = (double)av[k];
                    s[u] = fma(w, w, s[u]);
                    if (DOT) d[u] = fma((double)cv[k], w, d[u]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < V; ++k) {
                    const double w = widen_normal((float)av[k]);
                    s[u] = fma(w, w, s[u]);
                    if (DOT) d[u] = fma(widen_normal((float)cv[k]), w, d[u]);
                }
            }
        }
    }
    double sr = 0.0, dr = 0.0;
    for (int r = lo + nv * V + t; r < hi; r += nt) {
        const double w = (double)__ldcg(y + r);
        sr = fma(w, w, sr);
        if (DOT) dr = fma((double)__ldcg(x + r), w, dr);
    }
    ss += ((s[0] + s[1]) + (s[2] + s[3])) + sr;
    if (DOT) dd += ((d[0] + d[1]) + (d[2] + d[3])) + dr;
}

template <typename XT>
__global__ void __launch_bounds__(256, 3) k_batch_norm(const BatchTable* __restrict__ Tp, int want_dot) {
    __shared__ double red[32];
    __shared__ int last;
    const BatchTable T = *Tp;
    for (int c = blockIdx.x; c < T.nrow; c += gridDim.x) {
        const int j = find_slot<2>(T.slots, T.nslots, c);
        const BatchSlot& d = T.slots[j];
        SlotState* stt = T.states + d.state;
        const int kit = stt->k;
        const XT* in = static_cast<const XT*>((kit & 1) ? d.Y : d.X);
        const XT* out = static_cast<const XT*>((kit & 1) ? d.X : d.Y);
        const int lo = (c - d.row0) * kRowChunk;
        const int hi = min(d.nor, lo + kRowChunk);
        double sq = 0.0, dd = 0.0;
        if (want_dot) chunk_sums<XT, true>(out, in, lo, hi, sq, dd);
        else chunk_sums<XT, false>(out, in, lo, hi, sq, dd);
        sq = block_sum<256>(sq, red);
        if (want_dot) dd = block_sum<256>(dd, red);
        if (threadIdx.x == 0) {
            T.row_part[2LL * c] = sq;
            T.row_part[2LL * c + 1] = dd;
            __threadfence();
            last = atomicAdd(&stt->norm_count, 1u) == (unsigned)d.nrow - 1u;
        }
        __syncthreads();
        if (last && threadIdx.x < 32) {
            __threadfence();
            double s0 = 0.0, s1 = 0.0;
            for (int q = threadIdx.x; q < d.nrow; q += 32) {
                s0 += __ldcg(T.row_part + 2LL * (d.row0 + q));
                s1 += __ldcg(T.row_part + 2LL * (d.row0 + q) + 1);
            }
            for (int o = 16; o > 0; o >>= 1) {
                s0 += __shfl_down_sync(0xffffffffu, s0, o);
                s1 += __shfl_down_sync(0xffffffffu, s1, o);
            }
            if (threadIdx.x == 0) {
                stt->nsq_prev = stt->nsq;
                stt->nsq = s0;
                if (want_dot) stt->dot = s1;
                stt->keyed = 0;
                stt->k = kit + 1;
                stt->norm_count = 0u;
            }
        }
        __syncthreads();
    }
}

template <typename XT>
__global__ void __launch_bounds__(256) k_batch_resid(const BatchTable* __restrict__ Tp) {
    __shared__ double red[32];
    __shared__ int last;
    const BatchTable T = *Tp;
    for (int c = blockIdx.x; c < T.nrow; c += gridDim.x) {
        const int j = find_slot<2>(T.slots, T.nslots, c);
        const BatchSlot& d = T.slots[j];
        SlotState* stt = T.states + d.state;
        const int kit = stt->k;  // >= 2 after a round
        const double nsq_prev = stt->nsq_prev;
        const int e = kit - 1 > 0 ? pow2_rescale_exponent(nsq_prev, rescale_window<XT>()) : 0;
        const double dot = scale_pow2(stt->dot, -e);
        const double lam = dot / nsq_prev;
        // ||2^-e v_k - lam v_{k-1}||^2 = 2^-2e ||v_k||^2 - lam 2^-e (v_{k-1} . v_k)
        // from the round's sums (no pass over the rows): exact in exact
        // arithmetic, and in FP64 good to a few digits while the relative
        // residual is far above the sums' rounding (~1e-7); so it stands in
        // for the row pass while the relative residual is above 1e-3 -- no
        // stopping or phase rule looks at residuals that large -- unless the
        // host asked for the pass (a solve's last round).  The choice depends
        // only on the solve's own state, so it is the same in any mix.
        const double est = fma(-lam, dot, scale_pow2(stt->nsq, -2 * e));
        if (!stt->exact_res && est >= 1e-6 * nsq_prev * lam * lam) {
            if (threadIdx.x == 0) {  // every chunk of the solve writes the same values
                stt->lambda = lam;
                stt->res2 = est;
            }
            continue;
        }
        const XT* cur = static_cast<const XT*>((kit & 1) ? d.Y : d.X);
        const XT* prev = static_cast<const XT*>((kit & 1) ? d.X : d.Y);
        const int lo = (c - d.row0) * kRowChunk;
        const int hi = min(d.nor, lo + kRowChunk);
        double rr = 0.0;
        for (int r = lo + threadIdx.x; r < hi; r += blockDim.x) {
            const double dl = scale_pow2((double)__ldcg(cur + r), -e) - lam * (double)__ldcg(prev + r);
            rr = fma(dl, dl, rr);
        }
        rr = block_sum<256>(rr, red);
        if (threadIdx.x == 0) {
            T.res_part[c] = rr;
            __threadfence();
            last = atomicAdd(&stt->res_count, 1u) == (unsigned)d.nrow - 1u;
        }
        __syncthreads();
        if (last && threadIdx.x < 32) {
            __threadfence();
            double s0 = 0.0;
            for (int q = threadIdx.x; q < d.nrow; q += 32) s0 += __ldcg(T.res_part + d.row0 + q);
            for (int o = 16; o > 0; o >>= 1) s0 += __shfl_down_sync(0xffffffffu, s0, o);
            if (threadIdx.x == 0) {
                stt->lambda = lam;
                stt->res2 = s0;
                stt->res_count = 0u;
            }
        }
        __syncthreads();
    }
}

// x[i] = uniform [0, 1) from a hash of (seed, i): the service's seeded start
// vectors (splitmix64 finaliser, as in the matrix generator).
__global__ void k_fill_uniform(double* __restrict__ x, int n, uint64_t seed) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9e3779b97f4a7c15ull * (uint64_t)(i + 1);
        z ^= z >> 30;
        z *= 0xbf58476d1ce4e5b9ull;
        z ^= z >> 27;
        z *= 0x94d049bb133111ebull;
        z ^= z >> 31;
        x[i] = (double)(z >> 11) * 0x1.0p-53;
    }
}

template <typename VT, typename XT, typename AT>
struct BatchKernels {
    static constexpr int SMEM = (kBatchNT / 32) * kBatchStages * WarpStage<VT, kMliIpt>::BYTES;
    template <bool KEYS>
    static int grid(int sm_count) {
        static int occ = -1;
        if (occ < 0) {
            auto k = k_batch_spmv<VT, XT, AT, kBatchNT, kMliIpt, KEYS>;
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
            int o = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, kBatchNT, SMEM);
            occ = o > 0 ? o : 1;
        }
        return occ * sm_count;
    }
    // keys: a key step (SpMV and fix-up fold the largest key, k_batch_keys
    // advances the state); else the norm row pass (with v_k . v_{k+1} when
    // want_dot).
    static cudaError_t step(const BatchTable* T, int want_dot, bool keys, int sm_count, cudaStream_t st) {
        if (keys) {
            k_batch_spmv<VT, XT, AT, kBatchNT, kMliIpt, true><<<grid<true>(sm_count), kBatchNT, SMEM, st>>>(T);
            k_batch_fixup<XT, AT, true><<<8 * sm_count, 256, 0, st>>>(T);
            k_batch_keys<<<sm_count, 256, 0, st>>>(T);
            return cudaGetLastError();
        }
        k_batch_spmv<VT, XT, AT, kBatchNT, kMliIpt><<<grid<false>(sm_count), kBatchNT, SMEM, st>>>(T);
        k_batch_fixup<XT, AT><<<8 * sm_count, 256, 0, st>>>(T);
        k_batch_norm<XT><<<3 * sm_count, 256, 0, st>>>(T, want_dot);
        return cudaGetLastError();
    }
};

}  // namespace

// Resident grid of a k_batch_sell instance: every warp's range of slice
// groups starts at once (a second wave would double the step).
template <typename VT, int SUM>
static int sell_batch_grid(int sm_count) {
    static int occ = 0;
    if (occ == 0) {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_batch_sell<VT, SUM>, 256, 0) != cudaSuccess || o < 1)
            o = 1;
        occ = o;
    }
    return occ * sm_count;
}

// A step of a SELL-32 class: a key step (the slots' largest keys, then the
// state advance), the step before a round's last (the group sums of squares
// and the per-slot totals), or the round's last step (which also needs
// v_k . v_{k+1}: the row pass).
template <typename VT>
static void launch_batch_sell(const BatchTable* T, int sum, int sm_count, cudaStream_t st) {
    if (sum == kSellKeys) {
        k_batch_sell<VT, kSellKeys><<<sell_batch_grid<VT, kSellKeys>(sm_count), 256, 0, st>>>(T);
        k_batch_keys<<<sm_count, 256, 0, st>>>(T);
    } else if (sum == kSellSquares) {
        k_batch_sell<VT, kSellSquares><<<sell_batch_grid<VT, kSellSquares>(sm_count), 256, 0, st>>>(T);
        k_batch_grp<<<sm_count, 256, 0, st>>>(T);
    } else {
        k_batch_sell<VT, kSellNone><<<sell_batch_grid<VT, kSellNone>(sm_count), 256, 0, st>>>(T);
        k_batch_norm<float><<<3 * sm_count, 256, 0, st>>>(T, 1);
    }
}

void batch_prepare(int sm_count) {
    BatchKernels<double, double, double>::grid<false>(sm_count);
    BatchKernels<double, double, double>::grid<true>(sm_count);
    BatchKernels<float, float, float>::grid<false>(sm_count);
    BatchKernels<float, float, float>::grid<true>(sm_count);
    BatchKernels<__nv_bfloat16, float, float>::grid<false>(sm_count);
    BatchKernels<__nv_bfloat16, float, float>::grid<true>(sm_count);
    sell_batch_grid<float, kSellNone>(sm_count);
    sell_batch_grid<float, kSellSquares>(sm_count);
    sell_batch_grid<float, kSellKeys>(sm_count);
    sell_batch_grid<__nv_bfloat16, kSellNone>(sm_count);
    sell_batch_grid<__nv_bfloat16, kSellSquares>(sm_count);
    sell_batch_grid<__nv_bfloat16, kSellKeys>(sm_count);
}

// A round of `steps` power steps: key steps, then the two steps whose norms
// the round's Rayleigh quotient and residual use (||v_{k-1}||^2, then
// ||v_k||^2 with v_{k-1} . v_k), then the residual.
cudaError_t launch_batch_round(int cfg, const BatchTable* T, int steps, int sm_count, cudaStream_t st, bool sell) {
    for (int it = 0; it < steps; ++it) {
        const int want_dot = it == steps - 1;
        const bool keys = it < steps - 2;
        cudaError_t e;
        if (sell) {
            const int sum = keys ? kSellKeys : want_dot ? kSellNone : kSellSquares;
            if (cfg == kCfgBF16) launch_batch_sell<__nv_bfloat16>(T, sum, sm_count, st);
            else launch_batch_sell<float>(T, sum, sm_count, st);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            continue;
        }
        switch (cfg) {
            case kCfgF32: e = BatchKernels<float, float, float>::step(T, want_dot, keys, sm_count, st); break;
            case kCfgBF16: e = BatchKernels<__nv_bfloat16, float, float>::step(T, want_dot, keys, sm_count, st); break;
            default: e = BatchKernels<double, double, double>::step(T, want_dot, keys, sm_count, st); break;
        }
        if (e != cudaSuccess) return e;
    }
    if (cfg == kCfgF64) k_batch_resid<double><<<4 * sm_count, 256, 0, st>>>(T);
    else k_batch_resid<float><<<4 * sm_count, 256, 0, st>>>(T);
    return cudaGetLastError();
}

cudaError_t launch_tile_slots(const BatchTable* T, int nslots, cudaStream_t st) {
    if (nslots <= 0) return cudaSuccess;
    k_tile_slots<<<nslots < 1024 ? nslots : 1024, 256, 0, st>>>(T);
    return cudaGetLastError();
}

cudaError_t launch_fill_uniform(double* x, int n, uint64_t seed, int sm_count, cudaStream_t st) {
    long long blocks = (n + 255) / 256;
    if (blocks > sm_count * 8) blocks = sm_count * 8;
    if (blocks < 1) blocks = 1;
    k_fill_uniform<<<(int)blocks, 256, 0, st>>>(x, n, seed);
    return cudaGetLastError();
}

}  // namespace pwmgpu
