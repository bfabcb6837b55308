// merge.cu -- merge-path SpMV, its fix-up pass and the power-method kernels.
//
// Kernels (reference analogue in brackets):
//   k_merge_partition  [CRS_Merge::searchPathOnDiag, CRS_Merge.hpp:42-62, for
//                       the diagonals of :96-107]
//   k_merge_spmv       [CRS_Merge::mv, :95-134]   persistent, TMA-staged tiles
//   k_merge_fixup      [CRS_Merge::mv carry fix-up, :136-140] + deterministic
//                       grid reduction of the power method's ||y||^2
//   k_power_finalize   [Util/VectorUtill.hpp:34-41 normalize of the last two iterates]
//   k_poisson_crs      [Util/Poisson.hpp:32-83 fillPoisson, one thread per row]
//   k_dot2 / k_resid   Rayleigh quotient and eigen-residual passes (not in the
//                       reference; used by the solve with a stopping test)
#include <cstdio>
#include <type_traits>

#include "internal.h"
#include "merge.cuh"

namespace pwmgpu {

// ---------------------------------------------------------------------------
// K1: merge-path partition
// ---------------------------------------------------------------------------
__global__ void k_merge_partition(const int32_t* __restrict__ row_start, int nor, int nnz, long long ipt,
                                  int parts, int2* __restrict__ out) {
    const int total = nor + nnz;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t <= parts; t += gridDim.x * blockDim.x) {
        long long d = ipt * t;
        int dd = d < total ? (int)d : total;
        out[t] = merge_search_global(dd, row_start + 1, nor, nnz);
    }
}

// ---------------------------------------------------------------------------
// Plan: lane-interleaved storage, row-end masks and per-sub-tile metadata.
// One warp per sub-tile (see merge.cuh for the layout).
//   rec[2s]   = {rw0, kw0, rw1, kw1}: the sub-tile's merge coordinates
//   rec[2s+1] = {fr: row holding the sub-tile's first nonzero (rw1 if none),
//                flags: kFlagGeneral if an empty row completes here,
//                       kFlagOpen0 if row fr began in an earlier sub-tile,
//                base: storage base of the sub-tile, nkw}
// ---------------------------------------------------------------------------
__global__ void k_mli_plan(const int32_t* __restrict__ row_start, const int32_t* __restrict__ col,
                           const double* __restrict__ val, const int2* __restrict__ subc, int nsub,
                           int32_t* __restrict__ colp, double* __restrict__ valp, uint16_t* __restrict__ masks,
                           int4* __restrict__ rec) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int s = blockIdx.x * wpb + (threadIdx.x >> 5); s < nsub; s += gridDim.x * wpb) {
        const int2 c0 = subc[s], c1 = subc[s + 1];
        const int rw0 = c0.x, kw0 = c0.y, rw1 = c1.x, kw1 = c1.y;
        const int nkw = kw1 - kw0;
        const int qm = nkw >> 5, rem = nkw & 31;
        const int cnt = qm + (lane < rem ? 1 : 0);
        const int b0 = kw0 + lane * qm + (lane < rem ? lane : rem);
        const long long base = mli_base(kw0, s);
        // an empty row whose end item lies in this sub-tile?
        bool empty_here = false;
        for (int r = rw0 + lane; r < rw1; r += 32) empty_here |= (row_start[r] == row_start[r + 1]);
        const bool general = __any_sync(0xffffffffu, empty_here);
        uint32_t m = 0;
        if (cnt > 0) {
            int a = row_of(row_start, b0, rw0, rw1);
            for (int j = 0; j < cnt; ++j) {
                const int b = b0 + j;
                while (a < rw1 && row_start[a + 1] <= b) ++a;  // past empty rows
                if (a < rw1 && b + 1 == row_start[a + 1]) m |= 1u << j;
                colp[base + mli_pos(lane, j, qm, lane_vec<int32_t>())] = col[b];
                valp[base + mli_pos(lane, j, qm, lane_vec<double>())] = val[b];
            }
        }
        masks[(long long)s * 32 + lane] = (uint16_t)m;
        if (lane == 0) {
            const int fr = nkw > 0 ? row_of(row_start, kw0, rw0, rw1) : rw1;
            int flags = general ? kFlagGeneral : 0;
            if (nkw > 0 && row_start[fr] < kw0) flags |= kFlagOpen0;
            rec[2LL * s] = make_int4(rw0, kw0, rw1, kw1);
            rec[2LL * s + 1] = make_int4(fr, flags, (int)base, nkw);
        }
    }
}

// Values in another precision / vector width: element (l, j) moves from
// mli_pos(l, j, qm, 2) (FP64) to mli_pos(l, j, qm, 16/sizeof(T)).
template <typename T>
__global__ void k_mli_convert(const double* __restrict__ valp, const int2* __restrict__ subc,
                              const int4* __restrict__ rec, int nsub, T* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    constexpr int V = lane_vec<T>();
    for (int s = blockIdx.x * wpb + (threadIdx.x >> 5); s < nsub; s += gridDim.x * wpb) {
        const int nkw = subc[s + 1].y - subc[s].y;
        const int qm = nkw >> 5, rem = nkw & 31;
        const int cnt = qm + (lane < rem ? 1 : 0);
        const long long base = rec[2LL * s + 1].z;
        for (int j = 0; j < cnt; ++j) out[base + mli_pos(lane, j, qm, V)] = (T)valp[base + mli_pos(lane, j, qm, lane_vec<double>())];
    }
}

// 16-bit columns.  Sub-tile s holds elements [base, base + nkw) of the
// lane-interleaved storage; when every sub-tile's columns span less than 2^16
// (banded and stencil matrices: the rows of a sub-tile are consecutive), the
// plan also keeps col - cbase(s) as uint16 with cbase(s) = the sub-tile's
// smallest column in rec0.w (rec0.w otherwise holds kw1, which no kernel
// reads).  Pass 1: cbase per sub-tile, flag[0] = 1 if some span is too wide.
__global__ void k_mli_colspan(const int32_t* __restrict__ colp, const int4* __restrict__ rec, int nsub,
                              int* __restrict__ cbase, int* __restrict__ flag) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int s = blockIdx.x * wpb + (threadIdx.x >> 5); s < nsub; s += gridDim.x * wpb) {
        const int4 r1 = rec[2LL * s + 1];
        const long long base = r1.z;
        const int nkw = r1.w;
        int lo = INT_MAX, hi = INT_MIN;
        for (int k = lane; k < nkw; k += 32) {
            const int c = colp[base + k];
            lo = min(lo, c);
            hi = max(hi, c);
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            cbase[s] = nkw > 0 ? lo : 0;
            if (nkw > 0 && (long long)hi - (long long)lo > 65535) atomicOr(flag, 1);
        }
    }
}

// Pass 2: the uint16 offsets and rec0.w = cbase.
__global__ void k_mli_col16(const int32_t* __restrict__ colp, int4* __restrict__ rec, int nsub,
                            const int* __restrict__ cbase, uint16_t* __restrict__ colp16) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int s = blockIdx.x * wpb + (threadIdx.x >> 5); s < nsub; s += gridDim.x * wpb) {
        const int4 r1 = rec[2LL * s + 1];
        const long long base = r1.z;
        const int nkw = r1.w, cb = cbase[s];
        for (int k = lane; k < nkw; k += 32) colp16[base + k] = (uint16_t)(colp[base + k] - cb);
        if (lane == 0) rec[2LL * s].w = cb;
    }
}

// Back to CRS order (for reading the matrix out).
__global__ void k_mli_unpermute(const int32_t* __restrict__ colp, const double* __restrict__ valp,
                                const int2* __restrict__ subc, const int4* __restrict__ rec, int nsub,
                                int32_t* __restrict__ col, double* __restrict__ val) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int s = blockIdx.x * wpb + (threadIdx.x >> 5); s < nsub; s += gridDim.x * wpb) {
        const int kw0 = subc[s].y, nkw = subc[s + 1].y - kw0;
        const int qm = nkw >> 5, rem = nkw & 31;
        const int cnt = qm + (lane < rem ? 1 : 0);
        const int b0 = kw0 + lane * qm + (lane < rem ? lane : rem);
        const long long base = rec[2LL * s + 1].z;
        for (int j = 0; j < cnt; ++j) {
            col[b0 + j] = colp[base + mli_pos(lane, j, qm, lane_vec<int32_t>())];
            val[b0 + j] = valp[base + mli_pos(lane, j, qm, lane_vec<double>())];
        }
    }
}

// ---------------------------------------------------------------------------
// K2: merge-path SpMV (plain or with the power-method epilogue).  Each warp
// takes sub-tiles s = global warp, + total warps, ... and double-buffers them
// through its own shared-memory stages (TMA bulk copies, mbarriers).
// ---------------------------------------------------------------------------
template <typename VT, typename XT, typename AT>
struct MergeArgs {
    const int32_t* row_start;
    const int32_t* colp;
    const VT* valp;
    const int4* rec;
    const uint16_t* masks;
    int nor, nsub;
    const XT* x;
    XT* y;
    AT* carries;           // one per sub-tile
    const double* nsq_in;  // MODE_POWER: ||x||^2 (source of the 2^e rescale), or null for e = 0
    int* status;
    int tile0 = 0;  // the pass covers sub-tiles [tile0, tile0 + nsub)
    const uint16_t* colp16 = nullptr;  // C16 kernels: 16-bit column offsets (base in rec0.w)
    double* npart = nullptr;  // MODE_POWER: per-CTA sums of the squares of the rows the CTA completes, or null
    // MODE_POWER / MODE_SCALE: the largest magnitude key of x (source of the
    // 2^e rescale instead of nsq_in), or null
    const unsigned int* mx_in = nullptr;
    unsigned int* mx_out = nullptr;  // MODE_SCALE: atomicMax target for the keys of y
};

// The 2^e rescale of a power step from its input's largest magnitude key or
// squared norm (neither: e = 0).
template <int MODE, typename XT>
__device__ __forceinline__ int step_exponent(const unsigned int* mx_in, const double* nsq_in) {
    if (MODE == MODE_SPMV) return 0;
    if (mx_in) return pow2_rescale_exponent_key<XT>(*mx_in);
    return nsq_in ? pow2_rescale_exponent(*nsq_in, rescale_window<XT>()) : 0;
}


constexpr int kMliStages = 2;

// One SpMV pass of this warp: its sub-tiles s = global warp, + total warps,
// double-buffered through its shared-memory stages.  `ticket` counts this
// warp's stage uses so far, so mbarrier phases carry across passes of a
// persistent kernel.  Returns false (warp-uniformly) after a timeout, once
// this warp's copies in flight have landed or a short bound ran out.
template <int MODE, typename VT, typename XT, typename AT, int NT, int IPT, bool XCOH, bool C16, bool CG = false>
// MODE_POWER: ss += the squares of the rows the warp completes (as stored;
// rows that a fix-up completes are left to the fix-up); MODE_SCALE: mx max=
// their magnitude keys.
__device__ __forceinline__ bool warp_pass(const MergeArgs<VT, XT, AT>& a, const XT* __restrict__ x,
                                          XT* __restrict__ y, unsigned char* stages, uint64_t* bars, int* crow,
                                          AT* cval, AT* hval, uint32_t& ticket, int e, uint64_t pol, double& ss,
                                          unsigned& mx) {
    using S = WarpStage<VT, IPT, C16>;
    constexpr int NS = kMliStages;
    constexpr int W = NT / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * W + w, tw = gridDim.x * W;
    const int n = gw < a.nsub ? (a.nsub - 1 - gw) / tw + 1 : 0;  // this warp's sub-tiles
    int4 pref = make_int4(0, 0, 0, 0);
    if (lane == 0) {
        for (int k = 0; k < NS && k < n; ++k) {
            const uint32_t u = ticket + k;
            const int s = a.tile0 + gw + k * tw;
            issue_subtile<VT, IPT, C16>(stages + (u % NS) * S::BYTES, &bars[u % NS], s, __ldg(a.rec + 2LL * s + 1),
                                        a.rec, a.masks, a.colp, a.colp16, a.valp, pol);
        }
        if (n > NS) pref = __ldg(a.rec + 2LL * (a.tile0 + gw + NS * tw) + 1);
    }
    __syncwarp();
    int i = 0;
    for (; i < n; ++i) {
        const uint32_t u = ticket + i;
        const int k = u % NS;
        const int s = a.tile0 + gw + i * tw;
        unsigned char* st = stages + k * S::BYTES;
        const bool ok = mbar_wait_bounded(&bars[k], (u / NS) & 1u, a.status);
        if (!__all_sync(0xffffffffu, ok)) break;  // warp-uniform exit on a timeout
        AT xv[IPT];
        gather_subtile<VT, XT, AT, IPT, XCOH, C16, CG>(st, x, xv);
        constexpr bool NORM = MODE == MODE_POWER;
        const bool general = reinterpret_cast<const int4*>(st)[1].y & kFlagGeneral;
        if constexpr (MODE == MODE_SCALE && !CG && !XCOH) {
            // a key-tracking step without a rescale (e == 0, nearly every
            // step) runs the instance without the rescale in its unrolled
            // loop: 4096^2 stencil power step 0.2209 -> 0.2171 ms.  (The
            // L1-bypass instances and the persistent kernel keep one
            // instance: the split made the irregular matrix's step 2 % and
            // the persistent kernel's iteration 6 % slower.)
            if (e != 0) {
                if (general)
                    finish_subtile<MODE, true, VT, XT, AT, IPT, C16, NORM, true>(s, st, xv, a.row_start, y, a.carries,
                                                                                 a.nor, e, crow, cval, hval, ss, &mx);
                else
                    finish_subtile<MODE, false, VT, XT, AT, IPT, C16, NORM, true>(s, st, xv, a.row_start, y, a.carries,
                                                                                  a.nor, e, crow, cval, hval, ss, &mx);
            } else if (general) {
                finish_subtile<MODE, true, VT, XT, AT, IPT, C16, NORM, false>(s, st, xv, a.row_start, y, a.carries,
                                                                              a.nor, e, crow, cval, hval, ss, &mx);
            } else {
                finish_subtile<MODE, false, VT, XT, AT, IPT, C16, NORM, false>(s, st, xv, a.row_start, y, a.carries,
                                                                               a.nor, e, crow, cval, hval, ss, &mx);
            }
        } else if (general) {
            finish_subtile<MODE, true, VT, XT, AT, IPT, C16, NORM>(s, st, xv, a.row_start, y, a.carries, a.nor, e,
                                                                   crow, cval, hval, ss, &mx);
        } else {
            finish_subtile<MODE, false, VT, XT, AT, IPT, C16, NORM>(s, st, xv, a.row_start, y, a.carries, a.nor, e,
                                                                    crow, cval, hval, ss, &mx);
        }
        // every lane is done with this stage (finish_subtile ends with a warp
        // barrier): refill it with the warp's sub-tile i + NS
        if (lane == 0 && i + NS < n) {
            fence_proxy_async();
            issue_subtile<VT, IPT, C16>(st, &bars[k], s + NS * tw, pref, a.rec, a.masks, a.colp, a.colp16, a.valp,
                                        pol);
            pref = (i + NS + 1 < n) ? __ldg(a.rec + 2LL * (s + (NS + 1) * tw) + 1) : make_int4(0, 0, 0, 0);
        }
    }
    if (i < n) {
        // Leaving early after a timeout: let this warp's copies in flight land
        // (short bounded waits) before the CTA's shared memory goes away.
        if (lane == 0)
            for (int t = i; t < n && t < i + NS; ++t) {
                const uint32_t u = ticket + t;
                mbar_wait_bounded(&bars[u % NS], (u / NS) & 1u, a.status, kWaitCycles / 8, false);
            }
        __syncwarp();
        return false;
    }
    ticket += (uint32_t)n;
    return true;
}

// L1: launch variant (0: shared-memory-heavy carveout, most resident CTAs;
// 1: a smaller carveout that leaves more L1 for the x gathers); the code is
// the same, the two instances carry different function attributes.
// C16: the plan's 16-bit column offsets are streamed instead of 32-bit columns.
// CG: the x gathers bypass L1 (FP64 instances only).
template <int MODE, typename VT, typename XT, typename AT, int NT, int IPT, int L1 = 0, bool C16 = false,
          bool CG = false>
__global__ void __launch_bounds__(NT) k_merge_spmv(MergeArgs<VT, XT, AT> a) {
    using S = WarpStage<VT, IPT, C16>;
    constexpr int W = NT / 32;
    constexpr int NS = kMliStages;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bars[W][NS];
    __shared__ int crow[NT];
    __shared__ AT cval[NT];
    __shared__ AT hval[NT];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        for (int k = 0; k < NS; ++k) mbar_init(&bars[w][k], 1);
        fence_mbar_init();
    }
    __syncwarp();
    // x, y, carries and ||x||^2 may belong to the kernel before on the stream
    pdl_wait();
    const int e = step_exponent<MODE, XT>(a.mx_in, a.nsq_in);
    uint32_t ticket = 0;
    unsigned char* stages = smem_raw + (size_t)w * NS * S::BYTES;
    double ss = 0.0;
    unsigned mx = 0u;
    warp_pass<MODE, VT, XT, AT, NT, IPT, false, C16, CG>(a, a.x, a.y, stages, bars[w], crow + 32 * w,
                                                         cval + 32 * w, hval + 32 * w, ticket, e,
                                                         policy_evict_first(), ss, mx);
    if (MODE == MODE_SCALE && a.mx_out) block_max_out<NT>(mx, a.mx_out);
    if (MODE == MODE_POWER && a.npart) {
        // this CTA's share of ||y||^2 (k_fix_runs adds the fixed-up rows and
        // sums the shares in a fixed order)
        __shared__ double red[NT / 32];
        const double t = block_sum<NT>(ss, red);
        if (threadIdx.x == 0) a.npart[blockIdx.x] = t;
    }
}

template <typename XT, typename AT>
struct FixArgs {
    const int32_t* row_start;
    const int2* tiles;
    int nor, num_tiles;
    XT* y;
    const AT* carries;
    const double* nsq_in;  // MODE_POWER: ||x||^2, source of the rescale exponent
    int t_lo = 0, t_hi = -1;  // first sub-tiles of the runs to fix: [t_lo, t_hi) (t_hi < 0: all)
};

// Stand-alone fix-up kernel (one thread per sub-tile).
template <int MODE, typename XT, typename AT>
__global__ void __launch_bounds__(256) k_merge_fixup(FixArgs<XT, AT> a) {
    const int e = (MODE == MODE_POWER && a.nsq_in) ? pow2_rescale_exponent(*a.nsq_in, rescale_window<XT>()) : 0;
    const int t0 = a.t_lo + blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const int t_end = a.t_hi < 0 ? a.num_tiles : a.t_hi;
    double no_ss = 0.0;
    fixup_pass<MODE, XT, AT>(a.row_start, a.tiles, a.nor, a.num_tiles, a.y, a.carries, e, t0, t_end, stride, no_ss);
}

// Fix-up runs, found once per matrix: sub-tile t starts a run when it leaves
// row r = subc[t+1].x unfinished and sub-tile t-1 did not; the run's
// sub-tiles t..n-1 all end in row r and sub-tile n completes it; the carries
// are real only if n started inside row r (as in fixup_pass).
__global__ void k_run_flags(const int32_t* __restrict__ row_start, const int2* __restrict__ subc, int nsub, int nor,
                            int* __restrict__ flag, int4* __restrict__ desc) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nsub; t += gridDim.x * blockDim.x) {
        const int r = subc[t + 1].x;
        int ok = r < nor && (t == 0 || subc[t].x != r);
        int n = t + 1;
        if (ok) {
            while (n < nsub && subc[n + 1].x == r) ++n;
            ok = subc[n].y > row_start[r];
        }
        flag[t] = ok;
        desc[t] = make_int4(t, n, r, 0);
    }
}

// pre[t] = runs whose first sub-tile is before t
__global__ void k_run_compact(const int* __restrict__ pre, const int4* __restrict__ desc, int nsub,
                              int4* __restrict__ runs) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nsub; t += gridDim.x * blockDim.x)
        if (pre[t + 1] != pre[t]) runs[pre[t]] = desc[t];
}

// ||y||^2 of a power step, summed inside its SpMV and fix-up kernels:
// npart[0, nspmv) hold the SpMV CTAs' shares; the fix-up CTAs add theirs
// after them and the last fix-up CTA sums all shares in order into *nsq_out.
struct FixNorm {
    double* npart = nullptr;  // null: no norm
    int nspmv = 0;
    unsigned int* counter = nullptr;  // zero between launches
    double* nsq_out = nullptr;
    const unsigned int* mx_in = nullptr;  // the step's rescale from its input's largest key (else nsq_in)
    unsigned int* mx_out = nullptr;       // MODE_SCALE: atomicMax target for the keys of the fixed rows
};

// One thread per run: y[r] += (carries[t] + ... + carries[n-1]) -- the sums of
// fixup_pass in the same order, without its search (one descriptor load, then
// the carries and y[r] together).
template <int MODE, typename XT, typename AT>
__global__ void __launch_bounds__(256) k_fix_runs(const int4* __restrict__ runs, int k0, int k1, XT* __restrict__ y,
                                                  const AT* __restrict__ carries, const double* nsq_in, FixNorm nrm) {
    const int kk = k0 + blockIdx.x * blockDim.x + threadIdx.x;
    const int4 d0 = kk < k1 ? runs[kk] : make_int4(0, 0, 0, 0);  // plan data: before the wait
    pdl_wait();  // carries and y come from the SpMV before on the stream
    const int e = step_exponent<MODE, XT>(nrm.mx_in, nsq_in);
    double ss = 0.0;
    unsigned mx = 0u;
    for (int k = kk; k < k1; k += gridDim.x * blockDim.x) {
        const int4 d = k == kk ? d0 : runs[k];
        AT sum = __ldcg(carries + d.x);
        for (int j = d.x + 1; j < d.y; ++j) sum += __ldcg(carries + j);
        const XT v = (XT)((AT)__ldcg(y + d.z) + (MODE != MODE_SPMV && e != 0 ? scale_pow2(sum, e) : sum));
        y[d.z] = v;
        if (MODE == MODE_POWER) ss = fma((double)v, (double)v, ss);
        if (MODE == MODE_SCALE) mx = max(mx, mag_key(v));
    }
    if (MODE == MODE_SCALE && nrm.mx_out) block_max_out<256>(mx, nrm.mx_out);
    if (MODE != MODE_POWER || !nrm.npart) return;
    __shared__ double red[8];
    __shared__ bool am_last;
    const double t = block_sum<256>(ss, red);
    if (threadIdx.x == 0) {
        nrm.npart[nrm.nspmv + blockIdx.x] = t;
        __threadfence();
        am_last = atomicAdd(nrm.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (am_last && threadIdx.x < 32) {
        __threadfence();
        const int n = nrm.nspmv + (int)gridDim.x;
        double s0 = 0.0;
        for (int i = threadIdx.x; i < n; i += 32) s0 += __ldcg(nrm.npart + i);
        for (int o = 16; o > 0; o >>= 1) s0 += __shfl_down_sync(0xffffffffu, s0, o);
        if (threadIdx.x == 0) {
            *nrm.nsq_out = s0;
            *nrm.counter = 0u;
        }
    }
}

// ||y||^2 (and x . y with DOT) with one deterministic reduction: per-CTA
// partials, then the last CTA sums them in order.  out[0] = sum y^2,
// out[1] = sum x y.
template <typename XT, bool DOT>
__global__ void __launch_bounds__(256) k_power_norm(const XT* __restrict__ y, const XT* __restrict__ x, int n,
                                                    double* partials, unsigned int* counter, double* out) {
    __shared__ double red[32];
    __shared__ bool am_last;
    double ss = 0.0, dd = 0.0;
    norm_rows<XT, DOT>(y, x, 0, n, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, ss, dd);
    ss = block_sum<256>(ss, red);
    if (DOT) dd = block_sum<256>(dd, red);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = ss;
        partials[2 * blockIdx.x + 1] = dd;
        __threadfence();
        am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (am_last && threadIdx.x < 32) {
        __threadfence();
        const int l = threadIdx.x;
        double s0 = 0.0, s1 = 0.0;
        for (int i = l; i < (int)gridDim.x; i += 32) {
            s0 += __ldcg(partials + 2 * i);
            s1 += __ldcg(partials + 2 * i + 1);
        }
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_down_sync(0xffffffffu, s0, o);
            s1 += __shfl_down_sync(0xffffffffu, s1, o);
        }
        if (l == 0) {
            out[0] = s0;
            if (DOT) out[1] = s1;
            *counter = 0u;
        }
    }
}

// ---------------------------------------------------------------------------
// Grid-wide barrier for a cooperative launch, with a bounded wait: after
// `budget` clock64 cycles (kWaitCycles unless a test shortens it), or once
// another CTA has recorded a failure, it records PWMGPU_ERR_TIMEOUT and
// returns false in every thread of the CTA.  The barrier opens when
// gridDim.x + extra CTAs have arrived (extra is 0 except in the timeout test,
// whose barrier therefore never opens).
// bar[0] counts arrivals, bar[1] is the generation; both start at zero.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned int atom_add_acq_rel_gpu(unsigned int* p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void red_add_release_gpu(unsigned int* p, unsigned int v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_gpu(unsigned int* p, unsigned int v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 of each CTA releases the CTA's writes (fence after the CTA
// barrier) and arrives with an acq_rel atomic; the last arrival resets the
// count and bumps the generation with a release; the others spin on the
// generation with acquire loads.  After the final CTA barrier every thread's
// ordinary loads see every CTA's writes from before the barrier.
__device__ __forceinline__ bool grid_sync(unsigned int* bar, int* status, long long budget, unsigned int extra) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int g = ld_acquire_gpu(bar + 1);
        __threadfence();
        const unsigned int arrived = atom_add_acq_rel_gpu(bar, 1u) + 1u;
        int ok = 1;
        if (arrived == gridDim.x + extra) {
            st_relaxed_gpu(bar, 0u);
            red_add_release_gpu(bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            unsigned int spins = 0;
            while (ld_acquire_gpu(bar + 1) == g) {
                if ((++spins & 1023u) == 0u) {
                    if (*(volatile int*)status != PWMGPU_OK) { ok = 0; break; }
                    if (clock64() - t0 > budget) {
                        atomicCAS(status, PWMGPU_OK, PWMGPU_ERR_TIMEOUT);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        __threadfence();
        ok_s = ok && (*(volatile int*)status == PWMGPU_OK);
    }
    __syncthreads();
    return ok_s != 0;
}

// ---------------------------------------------------------------------------
// K5: the power-method step fused into one persistent kernel (cooperative
// launch).  Iteration k (k0 <= k < k0 + nk):
//   v_{k+1} = 2^{e_k} A v_k         (SpMV pass; e_k from ||v_k||^2: an exact
//                                     rescale, applied only when the norm
//                                     leaves a wide window)
//   carries of v_{k+1}               (fix-up pass)
//   ||v_{k+1}||^2                    (squares in both passes; per-CTA shares
//                                     summed in a fixed order)
//   v_k . v_{k+1} and ||v_{k+1}||^2 in a row pass on the last iteration when
//   `result` is set, then the Rayleigh quotient lambda_k = 2^{-e_k} v_k.v_{k+1} /
//   ||v_k||^2 and the eigen-residual ||2^{-e_k} v_{k+1} - lambda_k v_k||^2
// Vectors ping-pong: iteration k reads X when k is even, Y when odd.  Two
// grid barriers per iteration (SpMV | fix-up | total): the squares of
// ||v_{k+1}||^2 are taken where the rows are stored -- the SpMV pass squares
// the rows it completes from its coalesced row buffer (about one FP64 FMA
// per 32 rows per warp instruction, beside one per nonzero: GB300's FP64
// pipe is 2 operations per clock per SM), the fix-up pass the rows it
// completes; the last iteration of a chunk with a result adds a row pass
// (and a barrier) for v_k . v_{k+1}.  The normalisation of
// the reference (y /= ||y||, Util/VectorUtill.hpp:34-41) is carried by the
// exponent and applied once at the end (k_power_finalize).  All reductions
// are FP64 and in a fixed order, whatever the vector type.
// ---------------------------------------------------------------------------
template <typename VT, typename XT, typename AT>
struct PowerArgs {
    MergeArgs<VT, XT, AT> m;
    const int2* subc;
    XT* X;
    XT* Y;
    int k0, nk;
    double* nsq;       // nsq[k] = ||v_k||^2; nsq[k0] read when k0 > 0; nsq[k0+1 .. k0+nk] written
    double* result;    // null, or (k = k0+nk-1 >= 1): {lambda_k, residual^2, ||v_k||^2, v_k.v_{k+1}, e_k}
    double* partials;  // 2 per CTA
    unsigned int* barrier;
    GridWait wait;     // grid barrier budget and extra arrivals
    // mxk[k]: largest magnitude key of v_k, zeroed (or null: every iteration
    // sums ||v||^2).  Iterations before the last two store only the keys.
    unsigned int* mxk;
    // The plan's fix-up runs (null: the fix-up pass searches the sub-tiles).
    const int4* runs;
    int nruns;
};

// The fix-up pass over the plan's run list: thread t0, t0 + stride, ... adds
// run k's carries to its row -- the sums of fixup_pass in the same order
// (k_fix_runs' loop, for the persistent kernel).
template <int MODE, typename XT, typename AT, bool NORM>
__device__ __forceinline__ void fix_runs_pass(const int4* __restrict__ runs, int nruns, XT* __restrict__ y,
                                              const AT* __restrict__ carries, int e, int t0, int stride, double& ss,
                                              unsigned* mx) {
    for (int k = t0; k < nruns; k += stride) {
        const int4 d = __ldg(runs + k);
        AT sum = __ldcg(carries + d.x);
        for (int j = d.x + 1; j < d.y; ++j) sum += __ldcg(carries + j);
        const XT v = (XT)((AT)__ldcg(y + d.z) + (e != 0 ? scale_pow2(sum, e) : sum));
        y[d.z] = v;
        if (NORM) ss = fma((double)v, (double)v, ss);
        if (MODE == MODE_SCALE) *mx = max(*mx, mag_key(v));
    }
}

// Sum two per-CTA partials over the grid in a fixed order (every CTA gets the
// same totals); call after a grid barrier.
template <int NT>
__device__ __forceinline__ void grid_total2(const double* partials, double* total) {
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < 32) {
        double s0 = 0.0, s1 = 0.0;
        for (int i = lane; i < (int)gridDim.x; i += 32) {
            s0 += __ldcg(partials + 2 * i);
            s1 += __ldcg(partials + 2 * i + 1);
        }
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_down_sync(0xffffffffu, s0, o);
            s1 += __shfl_down_sync(0xffffffffu, s1, o);
        }
        if (lane == 0) {
            total[0] = s0;
            total[1] = s1;
        }
    }
    __syncthreads();
}

// (at most 80 registers: 6 CTAs per SM fit beside the 16-bit-column stages)
template <typename VT, typename XT, typename AT, int NT, int IPT, int L1 = 0, bool C16 = false>
__global__ void __launch_bounds__(NT, 6) k_power_persistent(PowerArgs<VT, XT, AT> p) {
    using S = WarpStage<VT, IPT, C16>;
    constexpr int W = NT / 32;
    constexpr int NS = kMliStages;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bars[W][NS];
    __shared__ int crow[NT];
    __shared__ AT cval[NT];
    __shared__ AT hval[NT];
    __shared__ double red[32];
    __shared__ double total[2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const MergeArgs<VT, XT, AT>& a = p.m;
    if (lane == 0) {
        for (int k = 0; k < NS; ++k) mbar_init(&bars[w][k], 1);
        fence_mbar_init();
    }
    __syncwarp();
    const uint64_t pol = policy_evict_first();
    uint32_t ticket = 0;
    double nsq_cur = p.k0 > 0 ? p.nsq[p.k0] : 0.0;
    double nsq_last = 0.0;
    int e = 0;
    bool prev_keys = false;  // iteration k-1 stored only its magnitude keys (mxk[k])
    unsigned char* stages = smem_raw + (size_t)w * NS * S::BYTES;
    const int tid = blockIdx.x * NT + threadIdx.x, nthr = gridDim.x * NT;
    for (int k = p.k0; k < p.k0 + p.nk; ++k) {
        const XT* in = (k & 1) ? p.Y : p.X;
        XT* out = (k & 1) ? p.X : p.Y;
        e = k == 0 ? 0
            : prev_keys ? pow2_rescale_exponent_key<XT>(__ldcg(p.mxk + k))
                        : pow2_rescale_exponent(nsq_cur, rescale_window<XT>());
        if (p.mxk && k < p.k0 + p.nk - 2) {
            // only the rescale needs this iterate's size: the largest key,
            // folded into mxk[k+1] by every warp, read after the barrier
            double no_ss = 0.0;
            unsigned mx = 0u;
            warp_pass<MODE_SCALE, VT, XT, AT, NT, IPT, true, C16>(a, in, out, stages, bars[w], crow + 32 * w,
                                                                  cval + 32 * w, hval + 32 * w, ticket, e, pol,
                                                                  no_ss, mx);
            if (!grid_sync(p.barrier, a.status, p.wait.cycles, p.wait.extra)) return;
            if (p.runs)
                fix_runs_pass<MODE_SCALE, XT, AT, false>(p.runs, p.nruns, out, a.carries, e, tid, nthr, no_ss, &mx);
            else
                fixup_pass<MODE_SCALE, XT, AT, false>(a.row_start, p.subc, a.nor, a.nsub, out, a.carries, e, tid,
                                                      a.nsub, nthr, no_ss, &mx);
            block_max_out<NT>(mx, p.mxk + k + 1);
            if (!grid_sync(p.barrier, a.status, p.wait.cycles, p.wait.extra)) return;
            prev_keys = true;
            continue;
        }
        prev_keys = false;
        nsq_last = nsq_cur;
        const bool want_dot = p.result && k == p.k0 + p.nk - 1;
        double ss = 0.0, dd = 0.0;
        unsigned mx = 0u;
        warp_pass<MODE_POWER, VT, XT, AT, NT, IPT, true, C16>(a, in, out, stages, bars[w], crow + 32 * w,
                                                              cval + 32 * w, hval + 32 * w, ticket, e, pol, ss, mx);
        if (!grid_sync(p.barrier, a.status, p.wait.cycles, p.wait.extra)) return;
        if (p.runs)
            fix_runs_pass<MODE_POWER, XT, AT, true>(p.runs, p.nruns, out, a.carries, e, tid, nthr, ss, &mx);
        else
            fixup_pass<MODE_POWER, XT, AT, true>(a.row_start, p.subc, a.nor, a.nsub, out, a.carries, e, tid, a.nsub,
                                                 nthr, ss);
        if (want_dot) {
            // the Rayleigh dot needs v_k: a row pass for both sums
            if (!grid_sync(p.barrier, a.status, p.wait.cycles, p.wait.extra)) return;
            ss = 0.0;
            norm_rows<XT, true>(out, in, 0, a.nor, tid, nthr, ss, dd);
        }
        const double t_ss = block_sum<NT>(ss, red);
        const double t_dd = block_sum<NT>(dd, red);
        if (threadIdx.x == 0) {
            p.partials[2 * blockIdx.x] = t_ss;
            p.partials[2 * blockIdx.x + 1] = t_dd;
        }
        if (!grid_sync(p.barrier, a.status, p.wait.cycles, p.wait.extra)) return;
        grid_total2<NT>(p.partials, total);  // every CTA, same order
        nsq_cur = total[0];
        const double dot = total[1];
        if (blockIdx.x == 0 && threadIdx.x == 0) p.nsq[k + 1] = nsq_cur;
        __syncthreads();  // total[] is rewritten below
        if (want_dot) {
            // lambda_k and the eigen-residual of u = v_k / ||v_k||
            const double lam = scale_pow2(dot, -e) / nsq_last;
            double rr = 0.0;
            for (int i = blockIdx.x * NT + threadIdx.x; i < a.nor; i += gridDim.x * NT) {
                const double d = scale_pow2((double)__ldcg(out + i), -e) - lam * (double)__ldcg(in + i);
                rr = fma(d, d, rr);
            }
            const double t_rr = block_sum<NT>(rr, red);
            if (!grid_sync(p.barrier, a.status, p.wait.cycles, p.wait.extra)) return;  // everyone has read partials
            if (threadIdx.x == 0) {
                p.partials[2 * blockIdx.x] = t_rr;
                p.partials[2 * blockIdx.x + 1] = 0.0;
            }
            if (!grid_sync(p.barrier, a.status, p.wait.cycles, p.wait.extra)) return;
            grid_total2<NT>(p.partials, total);
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                p.result[0] = lam;
                p.result[1] = total[0];
                p.result[2] = nsq_last;
                p.result[3] = dot;
                p.result[4] = (double)e;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Normalise the last two iterates of the power method (VectorUtill.hpp:34-41):
// v_last /= sqrt(nsq_last); v_prev /= sqrt(nsq_prev) when prev is an iterate.
// The reference divides each element; here each element is multiplied by
// the FP64 reciprocal (within 1 ulp of the quotient; an FP64 divide per
// element would make this pass FP64-pipe bound on GB300).
// ---------------------------------------------------------------------------
template <typename XT>
__global__ void k_power_finalize(XT* __restrict__ last, const double* nsq_last, XT* __restrict__ prev,
                                 const double* nsq_prev, int n) {
    const double rl = 1.0 / sqrt(*nsq_last);
    const double rp = prev ? 1.0 / sqrt(*nsq_prev) : 1.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        last[i] = (XT)((double)last[i] * rl);
        if (prev) prev[i] = (XT)((double)prev[i] * rp);
    }
}

// ---------------------------------------------------------------------------
// Device Poisson generator (Util/Poisson.hpp:32-83 order, one thread per row;
// the row start is the closed form of the per-row counts).
// ---------------------------------------------------------------------------
__host__ __device__ inline long long poisson_row_start(long long row, long long m, long long n) {
    long long mn = m * n;
    long long below = row > m ? row - m : 0;               // rows >= m before `row`
    long long left = row - (row + m - 1) / m;              // row % m != 0
    long long right = row - row / m;                       // row % m != m-1
    long long above = row < mn - m ? row : (mn - m > 0 ? mn - m : 0);  // row < mn - m
    return below + left + row + right + above;
}

// Rows [r0, r1) of the m x n matrix (Poisson.hpp:33-83 with first_row /
// last_row): row starts counted from row r0, global columns.
__global__ void k_poisson_crs(int m, int n, int r0, int r1, int32_t* __restrict__ row_start,
                              int32_t* __restrict__ col, double* __restrict__ val) {
    const int N = m * n;
    const long long k0 = poisson_row_start(r0, m, n);
    for (int row = r0 + blockIdx.x * blockDim.x + threadIdx.x; row < r1; row += gridDim.x * blockDim.x) {
        long long k = poisson_row_start(row, m, n) - k0;
        if (row >= m) { col[k] = row - m; val[k] = -1.0; ++k; }
        if (row % m != 0) { col[k] = row - 1; val[k] = -1.0; ++k; }
        col[k] = row; val[k] = 4.0; ++k;
        if (row % m != m - 1) { col[k] = row + 1; val[k] = -1.0; ++k; }
        if (row < N - m) { col[k] = row + m; val[k] = -1.0; ++k; }
        row_start[row - r0 + 1] = (int32_t)k;
        if (row == r0) row_start[0] = 0;
    }
}

// ---------------------------------------------------------------------------
// Monitor passes for the solve: dot products with a deterministic reduction.
// k_dot2: out[0] = sum a*b, out[1] = sum b*b (a, b vectors of length n)
// k_resid: out[0] = sum (sb*b - sa*a)^2
// ---------------------------------------------------------------------------
template <typename XT>
__global__ void __launch_bounds__(256) k_dot2(const XT* __restrict__ va, const XT* __restrict__ vb, int n,
                                              double* partials, unsigned int* counter, double* out) {
    __shared__ double red[32];
    __shared__ bool am_last;
    double s_ab = 0.0, s_bb = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double x = (double)va[i], y = (double)vb[i];
        s_ab = fma(x, y, s_ab);
        s_bb = fma(y, y, s_bb);
    }
    double t0 = block_sum<256>(s_ab, red);
    double t1 = block_sum<256>(s_bb, red);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = t0;
        partials[2 * blockIdx.x + 1] = t1;
        __threadfence();
        am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (am_last && threadIdx.x < 32) {
        __threadfence();
        const int l = threadIdx.x;
        double a0 = 0.0, a1 = 0.0;
        for (int i = l; i < (int)gridDim.x; i += 32) {
            a0 += __ldcg(partials + 2 * i);
            a1 += __ldcg(partials + 2 * i + 1);
        }
        for (int o = 16; o > 0; o >>= 1) {
            a0 += __shfl_down_sync(0xffffffffu, a0, o);
            a1 += __shfl_down_sync(0xffffffffu, a1, o);
        }
        if (l == 0) {
            out[0] = a0;
            out[1] = a1;
            *counter = 0u;
        }
    }
}

// The result pass of a solve chunk run with separate kernels (the persistent
// kernel's `want_dot` pass): from ||v_k||^2 (nsq_k, k >= 1) and nd = {||v_{k+1}||^2,
// v_k . v_{k+1}} of the last norm pass, lambda_k = 2^{-e} dot / ||v_k||^2 and
// the eigen-residual ||2^{-e} v_{k+1} - lambda_k v_k||^2 (deterministic:
// per-CTA partials summed in order by the last CTA); result = {lambda,
// residual^2, ||v_k||^2, dot, e}, and nsq_next = ||v_{k+1}||^2.
template <typename XT>
__global__ void __launch_bounds__(256) k_solve_result(const XT* __restrict__ in, const XT* __restrict__ out, int n,
                                                      const double* nsq_k, const double* nd, double* nsq_next,
                                                      double* result, double* partials, unsigned int* counter) {
    __shared__ double red[32];
    __shared__ bool am_last;
    const double nsq_last = *nsq_k, dot = nd[1];
    const int e = pow2_rescale_exponent(nsq_last, rescale_window<XT>());
    const double lam = scale_pow2(dot, -e) / nsq_last;
    double rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double d = scale_pow2((double)__ldcg(out + i), -e) - lam * (double)__ldcg(in + i);
        rr = fma(d, d, rr);
    }
    const double t = block_sum<256>(rr, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = t;
        __threadfence();
        am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (am_last && threadIdx.x < 32) {
        __threadfence();
        const int l = threadIdx.x;
        double a0 = 0.0;
        for (int i = l; i < (int)gridDim.x; i += 32) a0 += __ldcg(partials + i);
        for (int o = 16; o > 0; o >>= 1) a0 += __shfl_down_sync(0xffffffffu, a0, o);
        if (l == 0) {
            result[0] = lam;
            result[1] = a0;
            result[2] = nsq_last;
            result[3] = dot;
            result[4] = (double)e;
            *nsq_next = nd[0];
            *counter = 0u;
        }
    }
}

template <typename XT>
__global__ void __launch_bounds__(256) k_resid(const XT* __restrict__ va, double sa, const XT* __restrict__ vb,
                                               double sb, int n, double* partials, unsigned int* counter,
                                               double* out) {
    __shared__ double red[32];
    __shared__ bool am_last;
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d = sb * (double)vb[i] - sa * (double)va[i];
        s = fma(d, d, s);
    }
    double t = block_sum<256>(s, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = t;
        __threadfence();
        am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (am_last && threadIdx.x < 32) {
        __threadfence();
        const int l = threadIdx.x;
        double a0 = 0.0;
        for (int i = l; i < (int)gridDim.x; i += 32) a0 += __ldcg(partials + i);
        for (int o = 16; o > 0; o >>= 1) a0 += __shfl_down_sync(0xffffffffu, a0, o);
        if (l == 0) {
            out[0] = a0;
            *counter = 0u;
        }
    }
}

template <typename SRC, typename DST>
__global__ void k_convert(const SRC* __restrict__ s, DST* __restrict__ d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = (DST)s[i];
}
template <>
__global__ void k_convert<double, __nv_bfloat16>(const double* __restrict__ s, __nv_bfloat16* __restrict__ d,
                                                 long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = __double2bfloat16(s[i]);
}

// flag[0] |= 1 if some value is not exactly representable in BF16 (the mixed
// solve then streams FP32 values instead)
__global__ void k_bf16_exact(const double* __restrict__ v, long long n, int* flag) {
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double d = v[i];
        bad |= (double)__bfloat162float(__double2bfloat16(d)) != d;
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// ===========================================================================
// Host launchers
// ===========================================================================

long long mli_storage_elems(long long nnz, long long nsub) { return mli_size(nnz, nsub); }

// Kernel configurations (threads per CTA, items per lane).
// Shared-memory carveout (percent of the maximum) of the L1-preferring launch
// variant: room for 4 CTAs' stages, the rest of the 256 KB as L1.
constexpr int kL1Carveout = 72;

// Launch variant v of the merge kernels: bit 0 = L1 (the smaller shared-memory
// carveout), bit 1 = C16 (16-bit column offsets; only for plans that have them).
template <typename VT, typename XT, typename AT, int NT, int IPT>
struct MergeKernels {
    static constexpr int smem(bool c16) {
        return (NT / 32) * kMliStages * (c16 ? WarpStage<VT, IPT, true>::BYTES : WarpStage<VT, IPT, false>::BYTES);
    }

    template <typename K>
    static int setup(K k, int l1, int bytes) {
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (l1) cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, kL1Carveout);
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, NT, bytes) != cudaSuccess) o = 0;
        return o;
    }

    static constexpr bool kHasCG = std::is_same<VT, double>::value;

    template <int L1, bool C16>
    static int setup_spmv() {
        setup(k_merge_spmv<MODE_POWER, VT, XT, AT, NT, IPT, L1, C16>, L1, smem(C16));
        setup(k_merge_spmv<MODE_SCALE, VT, XT, AT, NT, IPT, L1, C16>, L1, smem(C16));
        if constexpr (kHasCG) {
            setup(k_merge_spmv<MODE_POWER, VT, XT, AT, NT, IPT, L1, C16, true>, L1, smem(C16));
            setup(k_merge_spmv<MODE_SCALE, VT, XT, AT, NT, IPT, L1, C16, true>, L1, smem(C16));
            setup(k_merge_spmv<MODE_SPMV, VT, XT, AT, NT, IPT, L1, C16, true>, L1, smem(C16));
        }
        return setup(k_merge_spmv<MODE_SPMV, VT, XT, AT, NT, IPT, L1, C16>, L1, smem(C16));
    }

    static MergeGeom geom(int v = 0) {
        v &= 3;
        static int occ[4] = {-1, -1, -1, -1};
        if (occ[v] < 0) {
            int o;
            switch (v) {
                case 1: o = setup_spmv<1, false>(); break;
                case 2: o = setup_spmv<0, true>(); break;
                case 3: o = setup_spmv<1, true>(); break;
                default: o = setup_spmv<0, false>(); break;
            }
            occ[v] = o > 0 ? o : 1;
        }
        return MergeGeom{32 * IPT, NT / 32, smem(v & 2), occ[v], NT};
    }

    template <int L1, bool C16>
    static const void* power_kernel() {
        return (const void*)k_power_persistent<VT, XT, AT, NT, IPT, L1, C16>;
    }
    static const void* power_kernel(int v) {
        switch (v & 3) {
            case 1: return power_kernel<1, false>();
            case 2: return power_kernel<0, true>();
            case 3: return power_kernel<1, true>();
            default: return power_kernel<0, false>();
        }
    }

    // resident CTAs per SM of the persistent power kernel (0: cannot launch)
    static int power_occ(int v = 0) {
        v &= 3;
        static int occ[4] = {-1, -1, -1, -1};
        if (occ[v] < 0) {
            const void* k = power_kernel(v);
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem(v & 2));
            if (v & 1) cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, kL1Carveout);
            int o = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, NT, smem(v & 2)) != cudaSuccess) o = 0;
            occ[v] = o;
        }
        return occ[v];
    }

    static cudaError_t power(const DevMatrix& M, const void* valp, const MliPlan& P, int grid, void* X, void* Y,
                             void* carries, int k0, int nk, double* nsq, double* result, double* partials,
                             unsigned int* barrier, int* status, cudaStream_t st, int v, GridWait wait,
                             unsigned int* mxk) {
        if (!P.colp16) v &= ~2;
        v &= 3;
        power_occ(v);
        PowerArgs<VT, XT, AT> p{{M.row_start, P.colp, (const VT*)valp, P.rec, P.masks, M.nor, P.nsub, nullptr,
                                 nullptr, (AT*)carries, nullptr, status, 0, P.colp16},
                                P.subc, (XT*)X, (XT*)Y, k0, nk, nsq, result, partials, barrier, wait, mxk,
                                P.runs, P.nruns};
        cudaError_t e = cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned int), st);
        if (e != cudaSuccess) return e;
        void* args[] = {&p};
        // cooperative launch: fails instead of running if the grid cannot be
        // co-resident, so the grid barriers cannot wait on unscheduled CTAs
        return cudaLaunchCooperativeKernel(power_kernel(v), dim3(grid), dim3(NT), args, smem(v & 2), st);
    }

    template <int L1, bool C16, bool CG = false>
    static void launch_spmv(int mode, const MergeArgs<VT, XT, AT>& a, int grid, cudaStream_t st, bool pdl) {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(NT);
        cfg.dynamicSmemBytes = smem(C16);
        cfg.stream = st;
        cudaLaunchAttribute attr{};
        attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr.val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = pdl ? 1 : 0;
        if (mode == MODE_POWER)
            cudaLaunchKernelEx(&cfg, k_merge_spmv<MODE_POWER, VT, XT, AT, NT, IPT, L1, C16, CG>, a);
        else if (mode == MODE_SCALE)
            cudaLaunchKernelEx(&cfg, k_merge_spmv<MODE_SCALE, VT, XT, AT, NT, IPT, L1, C16, CG>, a);
        else
            cudaLaunchKernelEx(&cfg, k_merge_spmv<MODE_SPMV, VT, XT, AT, NT, IPT, L1, C16, CG>, a);
    }

    template <int L1, bool C16>
    static void launch_spmv_cg(bool cg, int mode, const MergeArgs<VT, XT, AT>& a, int grid, cudaStream_t st,
                               bool pdl) {
        if constexpr (kHasCG) {
            if (cg) {
                launch_spmv<L1, C16, true>(mode, a, grid, st, pdl);
                return;
            }
        }
        launch_spmv<L1, C16, false>(mode, a, grid, st, pdl);
    }

    static cudaError_t spmv(int mode, const DevMatrix& M, const void* valp, const MliPlan& P, int grid,
                            const void* x, void* y, void* carries, const double* nsq_in, int* status,
                            cudaStream_t st, int v, int tile0 = 0, int nsub = -1, bool pdl = true,
                            double* npart = nullptr, const unsigned int* mx_in = nullptr,
                            unsigned int* mx_out = nullptr) {
        if (!P.colp16) v &= ~2;
        geom(v);
        MergeArgs<VT, XT, AT> a{M.row_start, P.colp, (const VT*)valp, P.rec, P.masks, M.nor,
                                nsub < 0 ? P.nsub : nsub, (const XT*)x, (XT*)y, (AT*)carries, nsq_in, status,
                                tile0, P.colp16, npart, mx_in, mx_out};
        const bool cg = (v >> 2) & 1;
        switch (v & 3) {
            case 1: launch_spmv_cg<1, false>(cg, mode, a, grid, st, pdl); break;
            case 2: launch_spmv_cg<0, true>(cg, mode, a, grid, st, pdl); break;
            case 3: launch_spmv_cg<1, true>(cg, mode, a, grid, st, pdl); break;
            default: launch_spmv_cg<0, false>(cg, mode, a, grid, st, pdl); break;
        }
        return cudaGetLastError();
    }
};

// The configurations the library instantiates (ids are stable: the
// autotuner cache stores them).  All share IPT = 12 (the storage layout
// depends on the sub-tile size), and differ in value type.
using CfgF64 = MergeKernels<double, double, double, 128, kMliIpt>;
using CfgF32 = MergeKernels<float, float, float, 128, kMliIpt>;
using CfgBF16 = MergeKernels<__nv_bfloat16, float, float, 128, kMliIpt>;

MergeGeom merge_geometry(int cfg, int l1) {
    switch (cfg) {
        case kCfgF32: return CfgF32::geom(l1);
        case kCfgBF16: return CfgBF16::geom(l1);
        default: return CfgF64::geom(l1);
    }
}

void warm_launch_caches(int sm_count) {
    for (int cfg : {kCfgF64, kCfgF32, kCfgBF16})
        for (int v = 0; v < 4; ++v) {
            (void)merge_geometry(cfg, v);
            (void)power_persistent_grid(cfg, 1, sm_count, v);
        }
    (void)sell_grid(1, sm_count);
}

int merge_grid(int cfg, int nsub, int sm_count, int l1) {
    MergeGeom g = merge_geometry(cfg, l1);
    long long ctas = (nsub + g.w - 1) / g.w;
    long long grid = (long long)g.occ * sm_count;
    if (grid > ctas) grid = ctas;
    return grid > 0 ? (int)grid : 1;
}

int power_persistent_grid(int cfg, int nsub, int sm_count, int l1) {
    int occ;
    switch (cfg) {
        case kCfgF32: occ = CfgF32::power_occ(l1); break;
        case kCfgBF16: occ = CfgBF16::power_occ(l1); break;
        default: occ = CfgF64::power_occ(l1); break;
    }
    if (occ <= 0) return 0;
    const MergeGeom g = merge_geometry(cfg);
    long long ctas = (nsub + g.w - 1) / g.w;
    long long grid = (long long)occ * sm_count;
    if (grid > ctas) grid = ctas;
    return grid > 0 ? (int)grid : 1;
}

cudaError_t launch_power_persistent(int cfg, const DevMatrix& M, const void* valp, const MliPlan& P, int grid,
                                    void* X, void* Y, void* carries, int k0, int nk, double* nsq, double* result,
                                    double* partials, unsigned int* barrier, int* status, cudaStream_t st, int l1,
                                    GridWait wait, unsigned int* mxk) {
    if (nk <= 0) return cudaSuccess;
    switch (cfg) {
        case kCfgF32:
            return CfgF32::power(M, valp, P, grid, X, Y, carries, k0, nk, nsq, result, partials, barrier, status, st,
                                 l1, wait, mxk);
        case kCfgBF16:
            return CfgBF16::power(M, valp, P, grid, X, Y, carries, k0, nk, nsq, result, partials, barrier, status,
                                  st, l1, wait, mxk);
        default:
            return CfgF64::power(M, valp, P, grid, X, Y, carries, k0, nk, nsq, result, partials, barrier, status, st,
                                 l1, wait, mxk);
    }
}

cudaError_t launch_merge_partition(const int32_t* row_start, int nor, long long nnz, long long ipt, int parts,
                                   int2* out, cudaStream_t st) {
    int threads = 256;
    long long blocks = (parts + 1 + threads - 1) / threads;
    if (blocks > 65535) blocks = 65535;
    k_merge_partition<<<(int)blocks, threads, 0, st>>>(row_start, nor, (int)nnz, ipt, parts, out);
    return cudaGetLastError();
}

static int warp_grid(int nsub, int sm_count) {
    long long g = (nsub + 7) / 8;
    if (g > (long long)sm_count * 32) g = (long long)sm_count * 32;
    return g > 0 ? (int)g : 1;
}

cudaError_t launch_mli_plan(const int32_t* row_start, const int32_t* col, const double* val, const MliPlan& P,
                            int sm_count, cudaStream_t st) {
    if (P.nsub == 0) return cudaSuccess;
    k_mli_plan<<<warp_grid(P.nsub, sm_count), 256, 0, st>>>(row_start, col, val, P.subc, P.nsub, P.colp, P.valp,
                                                             P.masks, P.rec);
    return cudaGetLastError();
}

cudaError_t launch_mli_colspan(const MliPlan& P, int* cbase, int* flag, int sm_count, cudaStream_t st) {
    if (P.nsub == 0) return cudaSuccess;
    k_mli_colspan<<<warp_grid(P.nsub, sm_count), 256, 0, st>>>(P.colp, P.rec, P.nsub, cbase, flag);
    return cudaGetLastError();
}

cudaError_t launch_mli_col16(const MliPlan& P, const int* cbase, int sm_count, cudaStream_t st) {
    if (P.nsub == 0 || !P.colp16) return cudaSuccess;
    k_mli_col16<<<warp_grid(P.nsub, sm_count), 256, 0, st>>>(P.colp, P.rec, P.nsub, cbase, P.colp16);
    return cudaGetLastError();
}

cudaError_t launch_mli_convert(const MliPlan& P, int cfg, void* out, int sm_count, cudaStream_t st) {
    if (P.nsub == 0) return cudaSuccess;
    if (cfg == kCfgBF16)
        k_mli_convert<__nv_bfloat16><<<warp_grid(P.nsub, sm_count), 256, 0, st>>>(P.valp, P.subc, P.rec, P.nsub,
                                                                                   (__nv_bfloat16*)out);
    else
        k_mli_convert<float><<<warp_grid(P.nsub, sm_count), 256, 0, st>>>(P.valp, P.subc, P.rec, P.nsub,
                                                                           (float*)out);
    return cudaGetLastError();
}

cudaError_t launch_mli_unpermute(const MliPlan& P, int32_t* col, double* val, int sm_count, cudaStream_t st) {
    if (P.nsub == 0) return cudaSuccess;
    k_mli_unpermute<<<warp_grid(P.nsub, sm_count), 256, 0, st>>>(P.colp, P.valp, P.subc, P.rec, P.nsub, col, val);
    return cudaGetLastError();
}

cudaError_t launch_merge_spmv(int cfg, int mode, const DevMatrix& M, const void* valp, const MliPlan& P, int grid,
                              const void* x, void* y, void* carries, const double* nsq_in, int* status,
                              cudaStream_t st, int l1, double* npart, const unsigned int* mx_in,
                              unsigned int* mx_out) {
    if (P.nsub == 0) return cudaSuccess;
    switch (cfg) {
        case kCfgF32:
            return CfgF32::spmv(mode, M, valp, P, grid, x, y, carries, nsq_in, status, st, l1, 0, -1, true, npart,
                                mx_in, mx_out);
        case kCfgBF16:
            return CfgBF16::spmv(mode, M, valp, P, grid, x, y, carries, nsq_in, status, st, l1, 0, -1, true, npart,
                                 mx_in, mx_out);
        default:
            return CfgF64::spmv(mode, M, valp, P, grid, x, y, carries, nsq_in, status, st, l1, 0, -1, true, npart,
                                mx_in, mx_out);
    }
}

template <typename XT, typename AT>
static cudaError_t fixup_impl(int mode, const DevMatrix& M, const int2* tiles, int num_tiles, XT* y,
                              const AT* carries, const double* nsq_in, int fix_grid, cudaStream_t st) {
    FixArgs<XT, AT> a{M.row_start, tiles, M.nor, num_tiles, y, carries, nsq_in};
    if (mode == MODE_POWER) k_merge_fixup<MODE_POWER, XT, AT><<<fix_grid, 256, 0, st>>>(a);
    else k_merge_fixup<MODE_SPMV, XT, AT><<<fix_grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_merge_fixup_f64(int mode, const DevMatrix& M, const int2* tiles, int num_tiles, double* y,
                                   const double* carries, const double* nsq_in, int fix_grid, cudaStream_t st) {
    return fixup_impl<double, double>(mode, M, tiles, num_tiles, y, carries, nsq_in, fix_grid, st);
}

cudaError_t launch_merge_fixup_f32(int mode, const DevMatrix& M, const int2* tiles, int num_tiles, float* y,
                                   const float* carries, const double* nsq_in, int fix_grid, cudaStream_t st) {
    return fixup_impl<float, float>(mode, M, tiles, num_tiles, y, carries, nsq_in, fix_grid, st);
}

// Chunk records of the pipelined host-array SpMV: chunk c covers sub-tiles
// [c*nsub/K, (c+1)*nsub/K); out[c] = {first sub-tile, its first row, 1 if
// that row began in the previous chunk, largest column the chunk reads}.
// kPlanCtas CTAs per chunk share the column scan (atomicMax into out[c].w,
// which starts at -1).
constexpr int kPlanCtas = 32;
__global__ void __launch_bounds__(256) k_pipeline_plan(const int32_t* __restrict__ row_start,
                                                       const int2* __restrict__ subc, const int4* __restrict__ rec,
                                                       const int32_t* __restrict__ colp, int nsub, int K,
                                                       int4* __restrict__ out) {
    __shared__ int red[256];
    const int c = blockIdx.x / kPlanCtas, part = blockIdx.x % kPlanCtas;
    const int s0 = (int)((long long)nsub * c / K), s1 = (int)((long long)nsub * (c + 1) / K);
    // the chunk's storage is contiguous (gaps between sub-tiles hold 0)
    const int4 a1 = __ldg(rec + 2LL * s0 + 1), b1 = __ldg(rec + 2LL * (s1 - 1) + 1);
    const long long lo = a1.z, hi = (long long)b1.z + b1.w, len = hi - lo;
    const long long p0 = lo + len * part / kPlanCtas, p1 = lo + len * (part + 1) / kPlanCtas;
    int mx = -1;
    for (long long k = p0 + threadIdx.x; k < p1; k += blockDim.x) mx = max(mx, __ldg(colp + k));
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = max(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicMax(&out[c].w, red[0]);
        if (part == 0) {
            const int2 c0 = subc[s0];
            const int split = (s0 > 0 && c0.y > row_start[c0.x]) ? 1 : 0;
            out[c].x = s0;
            out[c].y = c0.x;
            out[c].z = split;
        }
    }
}

cudaError_t launch_pipeline_plan(const int32_t* row_start, const MliPlan& P, int K, int* out, cudaStream_t st) {
    if (K <= 0 || P.nsub <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(out, 0xFF, sizeof(int4) * (size_t)K, st);  // -1 everywhere
    if (e != cudaSuccess) return e;
    k_pipeline_plan<<<K * kPlanCtas, 256, 0, st>>>(row_start, P.subc, P.rec, P.colp, P.nsub, K,
                                                   reinterpret_cast<int4*>(out));
    return cudaGetLastError();
}

// SpMV over sub-tiles [t0, t1) (FP64) and the fix-up of the runs starting in
// [f0, f1).
cudaError_t launch_merge_spmv_range(const DevMatrix& M, const MliPlan& P, int t0, int t1, int grid, const double* x,
                                    double* y, double* carries, int* status, cudaStream_t st, int l1) {
    if (t1 <= t0) return cudaSuccess;
    // without programmatic overlap: CTAs waiting on the previous chunk would hold
    // the SMs the pageable-array copy kernels of the other streams need
    return CfgF64::spmv(MODE_SPMV, M, P.valp, P, grid, x, y, carries, nullptr, status, st, l1, t0, t1 - t0, false);
}

cudaError_t launch_merge_fixup_range(const DevMatrix& M, const int2* tiles, int num_tiles, int f0, int f1, double* y,
                                     const double* carries, cudaStream_t st, int sm_count) {
    if (f1 <= f0) return cudaSuccess;
    FixArgs<double, double> a{M.row_start, tiles, M.nor, num_tiles, y, carries, nullptr, f0, f1};
    k_merge_fixup<MODE_SPMV, double, double><<<fixup_grid(f1 - f0, sm_count), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_power_norm_f64(const double* y, const double* x, int n, double* partials, unsigned int* counter,
                                  double* out, int grid, cudaStream_t st) {
    if (x) k_power_norm<double, true><<<grid, 256, 0, st>>>(y, x, n, partials, counter, out);
    else k_power_norm<double, false><<<grid, 256, 0, st>>>(y, x, n, partials, counter, out);
    return cudaGetLastError();
}

// One thread per sub-tile: a fix-up is a short chain of dependent L2 loads,
// so its time is latency, not bandwidth -- every sub-tile in flight at once
// (a grid capped at one CTA per SM left ~7 sub-tiles per thread and cost
// ~24 us per SpMV on the 4096^2 Poisson matrix).
cudaError_t launch_power_norm_f32(const float* y, const float* x, int n, double* partials, unsigned int* counter,
                                  double* out, int grid, cudaStream_t st) {
    if (x) k_power_norm<float, true><<<grid, 256, 0, st>>>(y, x, n, partials, counter, out);
    else k_power_norm<float, false><<<grid, 256, 0, st>>>(y, x, n, partials, counter, out);
    return cudaGetLastError();
}

cudaError_t launch_solve_result(bool f32, const void* in, const void* out, int n, const double* nsq_k,
                                const double* nd, double* nsq_next, double* result, double* partials,
                                unsigned int* counter, int grid, cudaStream_t st) {
    if (f32)
        k_solve_result<float><<<grid, 256, 0, st>>>((const float*)in, (const float*)out, n, nsq_k, nd, nsq_next,
                                                     result, partials, counter);
    else
        k_solve_result<double><<<grid, 256, 0, st>>>((const double*)in, (const double*)out, n, nsq_k, nd, nsq_next,
                                                      result, partials, counter);
    return cudaGetLastError();
}

int build_fix_runs(MliPlan& P, const int32_t* row_start, int nor, int sm_count, cudaStream_t st) {
    (void)sm_count;
    P.nruns = 0;
    if (P.nsub <= 0) return 0;
    int* scan_scratch = nullptr;
    int4* desc = nullptr;
    int rc = 0;
    const int nb = (P.nsub + 255) / 256;
    do {
        if (cudaMalloc((void**)&desc, sizeof(int4) * (size_t)P.nsub) != cudaSuccess ||
            cudaMalloc((void**)&scan_scratch, sizeof(int) * (size_t)scan_scratch_elems(P.nsub + 1)) != cudaSuccess ||
            cudaMalloc((void**)&P.run_pre, sizeof(int) * ((size_t)P.nsub + 1)) != cudaSuccess) {
            rc = 1;
            break;
        }
        // run_pre[0] = 0, run_pre[t + 1] = flag[t]; the inclusive scan of
        // run_pre + 1 makes run_pre[t] the runs that start before t
        if (cudaMemsetAsync(P.run_pre, 0, sizeof(int), st) != cudaSuccess) { rc = 1; break; }
        k_run_flags<<<nb, 256, 0, st>>>(row_start, P.subc, P.nsub, nor, P.run_pre + 1, desc);
        if (launch_inclusive_scan(P.run_pre + 1, P.nsub, scan_scratch, st) != cudaSuccess) { rc = 1; break; }
        int total = 0;
        if (cudaMemcpyAsync(&total, P.run_pre + P.nsub, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = 1;
            break;
        }
        P.nruns = total;
        if (cudaMalloc((void**)&P.runs, sizeof(int4) * (size_t)(total > 0 ? total : 1)) != cudaSuccess) { rc = 1; break; }
        if (total > 0) k_run_compact<<<nb, 256, 0, st>>>(P.run_pre, desc, P.nsub, P.runs);
        if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = 1;
    } while (0);
    if (desc) dev_free(desc);
    if (scan_scratch) dev_free(scan_scratch);
    if (rc) {
        (void)cudaGetLastError();
        if (P.runs) dev_free(P.runs);
        if (P.run_pre) dev_free(P.run_pre);
        P.runs = nullptr;
        P.run_pre = nullptr;
        P.nruns = 0;
    }
    return rc;
}

template <typename XT, typename AT>
static cudaError_t fix_runs_impl(int mode, const MliPlan& P, int k0, int k1, XT* y, const AT* carries,
                                 const double* nsq_in, cudaStream_t st, const FixNorm& nrm = FixNorm{}) {
    if (k1 <= k0 && !nrm.npart) return cudaSuccess;  // (a MODE_SCALE step without runs has no keys to add)
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(k1 > k0 ? (k1 - k0 + 255) / 256 : 1);  // the norm's last CTA runs even without runs
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    const int4* runs = P.runs;
    if (mode == MODE_POWER)
        cudaLaunchKernelEx(&cfg, k_fix_runs<MODE_POWER, XT, AT>, runs, k0, k1, y, carries, nsq_in, nrm);
    else if (mode == MODE_SCALE)
        cudaLaunchKernelEx(&cfg, k_fix_runs<MODE_SCALE, XT, AT>, runs, k0, k1, y, carries, nsq_in, nrm);
    else
        cudaLaunchKernelEx(&cfg, k_fix_runs<MODE_SPMV, XT, AT>, runs, k0, k1, y, carries, nsq_in, FixNorm{});
    return cudaGetLastError();
}

cudaError_t launch_fix_runs_f64(int mode, const MliPlan& P, int k0, int k1, double* y, const double* carries,
                                const double* nsq_in, cudaStream_t st) {
    return fix_runs_impl<double, double>(mode, P, k0, k1, y, carries, nsq_in, st);
}

cudaError_t launch_fix_runs_f32(int mode, const MliPlan& P, int k0, int k1, float* y, const float* carries,
                                const double* nsq_in, cudaStream_t st) {
    return fix_runs_impl<float, float>(mode, P, k0, k1, y, carries, nsq_in, st);
}

int power_norm_parts(const MliPlan& P, int spmv_grid) {
    return spmv_grid + (P.nruns > 0 ? (P.nruns + 255) / 256 : 1);
}

cudaError_t launch_fix_runs_scale(bool f32, const MliPlan& P, void* y, const void* carries, const double* nsq_in,
                                  const unsigned int* mx_in, unsigned int* mx_out, cudaStream_t st) {
    FixNorm nrm;
    nrm.mx_in = mx_in;
    nrm.mx_out = mx_out;
    if (f32)
        return fix_runs_impl<float, float>(MODE_SCALE, P, 0, P.nruns, (float*)y, (const float*)carries, nsq_in, st,
                                           nrm);
    return fix_runs_impl<double, double>(MODE_SCALE, P, 0, P.nruns, (double*)y, (const double*)carries, nsq_in, st,
                                         nrm);
}

cudaError_t launch_fix_runs_norm(bool f32, const MliPlan& P, void* y, const void* carries, const double* nsq_in,
                                 double* npart, int spmv_grid, unsigned int* counter, double* nsq_out,
                                 cudaStream_t st, const unsigned int* mx_in) {
    FixNorm nrm;
    nrm.npart = npart;
    nrm.nspmv = spmv_grid;
    nrm.counter = counter;
    nrm.nsq_out = nsq_out;
    nrm.mx_in = mx_in;
    if (f32)
        return fix_runs_impl<float, float>(MODE_POWER, P, 0, P.nruns, (float*)y, (const float*)carries, nsq_in, st,
                                           nrm);
    return fix_runs_impl<double, double>(MODE_POWER, P, 0, P.nruns, (double*)y, (const double*)carries, nsq_in, st,
                                         nrm);
}

int fixup_grid(int num_tiles, int sm_count) {
    (void)sm_count;
    const long long g = (num_tiles + 255) / 256;
    return g > 0 ? (int)(g < (1LL << 30) ? g : (1LL << 30)) : 1;
}

cudaError_t launch_power_finalize_f64(double* last, const double* nsq_last, double* prev, const double* nsq_prev,
                                      int n, int sm_count, cudaStream_t st) {
    int blocks = (n + 255) / 256;
    if (blocks > sm_count * 8) blocks = sm_count * 8;
    if (blocks < 1) blocks = 1;
    k_power_finalize<double><<<blocks, 256, 0, st>>>(last, nsq_last, prev, nsq_prev, n);
    return cudaGetLastError();
}

cudaError_t launch_poisson_crs(int m, int n, int32_t* row_start, int32_t* col, double* val, int sm_count,
                               cudaStream_t st, int first_row, int last_row) {
    if (last_row < 0) last_row = m * n;
    long long rows = (long long)last_row - first_row;
    long long blocks = (rows + 255) / 256;
    if (blocks > sm_count * 16) blocks = sm_count * 16;
    if (blocks < 1) blocks = 1;
    k_poisson_crs<<<(int)blocks, 256, 0, st>>>(m, n, first_row, last_row, row_start, col, val);
    return cudaGetLastError();
}

long long poisson_rows_nnz(int m, int n, int first_row, int last_row) {
    return poisson_row_start(last_row, m, n) - poisson_row_start(first_row, m, n);
}

int dot_grid(long long n, int sm_count) {
    long long g = (n + 255) / 256;
    if (g > sm_count * 4) g = sm_count * 4;
    return g > 0 ? (int)g : 1;
}

template <typename XT>
static cudaError_t dot2_impl(const XT* a, const XT* b, int n, double* partials, unsigned int* counter, double* out,
                             int grid, cudaStream_t st) {
    k_dot2<XT><<<grid, 256, 0, st>>>(a, b, n, partials, counter, out);
    return cudaGetLastError();
}
cudaError_t launch_dot2_f64(const double* a, const double* b, int n, double* partials, unsigned int* counter,
                            double* out, int grid, cudaStream_t st) {
    return dot2_impl<double>(a, b, n, partials, counter, out, grid, st);
}
cudaError_t launch_dot2_f32(const float* a, const float* b, int n, double* partials, unsigned int* counter,
                            double* out, int grid, cudaStream_t st) {
    return dot2_impl<float>(a, b, n, partials, counter, out, grid, st);
}
cudaError_t launch_resid_f64(const double* a, double sa, const double* b, double sb, int n, double* partials,
                             unsigned int* counter, double* out, int grid, cudaStream_t st) {
    k_resid<double><<<grid, 256, 0, st>>>(a, sa, b, sb, n, partials, counter, out);
    return cudaGetLastError();
}
cudaError_t launch_resid_f32(const float* a, double sa, const float* b, double sb, int n, double* partials,
                             unsigned int* counter, double* out, int grid, cudaStream_t st) {
    k_resid<float><<<grid, 256, 0, st>>>(a, sa, b, sb, n, partials, counter, out);
    return cudaGetLastError();
}
cudaError_t launch_convert_f64_f32(const double* s, float* d, long long n, int sm_count, cudaStream_t st) {
    k_convert<double, float><<<sm_count * 8, 256, 0, st>>>(s, d, n);
    return cudaGetLastError();
}
cudaError_t launch_convert_f32_f64(const float* s, double* d, long long n, int sm_count, cudaStream_t st) {
    k_convert<float, double><<<sm_count * 8, 256, 0, st>>>(s, d, n);
    return cudaGetLastError();
}
cudaError_t launch_convert_f64_bf16(const double* s, void* d, long long n, int sm_count, cudaStream_t st) {
    k_convert<double, __nv_bfloat16><<<sm_count * 8, 256, 0, st>>>(s, (__nv_bfloat16*)d, n);
    return cudaGetLastError();
}

cudaError_t launch_bf16_exact(const double* v, long long n, int* flag, int sm_count, cudaStream_t st) {
    long long blocks = (n + 255) / 256;
    if (blocks > sm_count * 8) blocks = sm_count * 8;
    if (blocks < 1) blocks = 1;
    k_bf16_exact<<<(int)blocks, 256, 0, st>>>(v, n, flag);
    return cudaGetLastError();
}

}  // namespace pwmgpu
