// batch.cu -- one power-method step of many solves per launch (the serving
// loop's rounds; no counterpart in the reference, whose power iteration
// serves one matrix per call: CRS.hpp:118-130).
//
// Per step, for every slot j of a class table (see batch.h):
//   k_batch_spmv    v_{k+1} = 2^{e_k} A_j v_k over all slots' sub-tiles
//                   (merge-path sub-tiles, TMA-staged, the power epilogue of
//                   the single-matrix kernel) and per-sub-tile partial sums
//                   of ||v_{k+1}||^2 (and v_k . v_{k+1} on a round's last step)
//   k_batch_reduce  carries of each slot (fix-up), then per-slot sums over
//                   its sub-tiles in a fixed order; the slot's last CTA
//                   advances the slot state (k, ||v||^2)
// and once per round
//   k_batch_resid   lambda and ||A u - lambda u||^2 of u = v_{k-1}/||v_{k-1}||.
// Grids are fixed (graph-captured rounds); the kernels read the table's
// sizes from device memory, so one graph serves every composition.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "batch.h"
#include "internal.h"
#include "merge.cuh"

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
        const int key = FIELD == 0 ? __ldg(&slots[mid].tile0) : FIELD == 1 ? __ldg(&slots[mid].red0)
                                                                            : __ldg(&slots[mid].res0);
        if (key <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <typename VT, int IPT>
__device__ __forceinline__ void issue_global(unsigned char* st, uint64_t* bar, const BatchSlot* slots, int nslots,
                                             int g, uint64_t pol) {
    const int j = find_slot<0>(slots, nslots, g);
    const BatchSlot& d = slots[j];
    const int s = g - d.tile0;
    issue_subtile<VT, IPT>(st, bar, s, __ldg(d.rec + 2LL * s + 1), d.rec, d.masks, d.colp,
                           static_cast<const VT*>(d.valp), pol);
}

template <typename VT, typename XT, typename AT, int NT, int IPT>
__global__ void __launch_bounds__(NT) k_batch_spmv(const BatchTable* __restrict__ Tp, int want_dot) {
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
    if (lane == 0) {
        for (int k = 0; k < NS; ++k) mbar_init(&bars[w][k], 1);
        fence_mbar_init();
        for (int k = 0; k < NS && k < n; ++k)
            issue_global<VT, IPT>(stages + k * S::BYTES, &bars[w][k], T.slots, T.nslots, gw + k * tw, pol);
    }
    __syncwarp();
    int i = 0;
    for (; i < n; ++i) {
        const int k = i % NS;
        const int g = gw + i * tw;
        unsigned char* st = stages + k * S::BYTES;
        const bool ok = mbar_wait_bounded(&bars[w][k], (uint32_t)(i / NS) & 1u, T.status);
        if (!__all_sync(0xffffffffu, ok)) break;
        const int j = find_slot<0>(T.slots, T.nslots, g);
        const BatchSlot& d = T.slots[j];
        const SlotState& ss_ = T.states[d.state];
        const int kit = ss_.k;
        const int e = kit > 0 ? pow2_exponent_from_nsq(ss_.nsq) : 0;
        const XT* in = static_cast<const XT*>((kit & 1) ? d.Y : d.X);
        XT* out = static_cast<XT*>((kit & 1) ? d.X : d.Y);
        const int s = g - d.tile0;
        AT xv[IPT];
        gather_subtile<VT, XT, AT, IPT>(st, in, xv);
        double sq = 0.0, dd = 0.0;
        if (reinterpret_cast<const int4*>(st)[1].y & kFlagGeneral)
            finish_subtile<MODE_POWER, true, VT, XT, AT, IPT>(s, st, xv, d.row_start, out, static_cast<AT*>(d.carries),
                                                              d.nor, e, sq, crow, cval, hval, want_dot ? in : nullptr,
                                                              &dd);
        else
            finish_subtile<MODE_POWER, false, VT, XT, AT, IPT>(s, st, xv, d.row_start, out,
                                                               static_cast<AT*>(d.carries), d.nor, e, sq, crow, cval,
                                                               hval, want_dot ? in : nullptr, &dd);
        for (int o = 16; o > 0; o >>= 1) {
            sq += __shfl_down_sync(0xffffffffu, sq, o);
            dd += __shfl_down_sync(0xffffffffu, dd, o);
        }
        if (lane == 0) {
            T.tile_part[2LL * g] = sq;
            T.tile_part[2LL * g + 1] = dd;
            if (i + NS < n) {
                fence_proxy_async();
                issue_global<VT, IPT>(st, &bars[w][k], T.slots, T.nslots, g + NS * tw, pol);
            }
        }
        __syncwarp();
    }
    if (i < n) {  // timed out: let this warp's copies in flight land first
        if (lane == 0)
            for (int t = i; t < n && t < i + NS; ++t)
                mbar_wait_bounded(&bars[w][t % NS], (uint32_t)(t / NS) & 1u, T.status, kWaitCycles / 8, false);
        __syncwarp();
    }
}

template <typename XT, typename AT>
__global__ void __launch_bounds__(256) k_batch_reduce(const BatchTable* __restrict__ Tp, int want_dot) {
    __shared__ double red[32];
    __shared__ int last;
    const BatchTable T = *Tp;
    for (int c = blockIdx.x; c < T.nred; c += gridDim.x) {
        const int j = find_slot<1>(T.slots, T.nslots, c);
        const BatchSlot& d = T.slots[j];
        SlotState* stt = T.states + d.state;
        const int kit = stt->k;
        const int e = kit > 0 ? pow2_exponent_from_nsq(stt->nsq) : 0;
        const XT* in = static_cast<const XT*>((kit & 1) ? d.Y : d.X);
        XT* out = static_cast<XT*>((kit & 1) ? d.X : d.Y);
        const int lo = (c - d.red0) * kRedTiles;
        const int hi = min(d.nsub, lo + kRedTiles);
        double sq = 0.0, dd = 0.0;
        fixup_pass<MODE_POWER, XT, AT>(d.row_start, d.subc, d.nor, d.nsub, out, static_cast<const AT*>(d.carries), e,
                                       sq, want_dot ? in : nullptr, &dd, lo + threadIdx.x, hi, blockDim.x);
        for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) {
            sq += T.tile_part[2LL * (d.tile0 + t)];
            dd += T.tile_part[2LL * (d.tile0 + t) + 1];
        }
        sq = block_sum<256>(sq, red);
        dd = block_sum<256>(dd, red);
        if (threadIdx.x == 0) {
            T.red_part[2LL * c] = sq;
            T.red_part[2LL * c + 1] = dd;
            __threadfence();
            last = atomicAdd(&stt->red_count, 1u) == (unsigned)d.nred - 1u;
        }
        __syncthreads();
        if (last && threadIdx.x < 32) {
            __threadfence();
            double s0 = 0.0, s1 = 0.0;
            for (int q = threadIdx.x; q < d.nred; q += 32) {
                s0 += __ldcg(T.red_part + 2LL * (d.red0 + q));
                s1 += __ldcg(T.red_part + 2LL * (d.red0 + q) + 1);
            }
            for (int o = 16; o > 0; o >>= 1) {
                s0 += __shfl_down_sync(0xffffffffu, s0, o);
                s1 += __shfl_down_sync(0xffffffffu, s1, o);
            }
            if (threadIdx.x == 0) {
                stt->nsq_prev = stt->nsq;
                stt->nsq = s0;
                if (want_dot) stt->dot = s1;
                stt->k = kit + 1;
                stt->red_count = 0u;
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
    for (int c = blockIdx.x; c < T.nres; c += gridDim.x) {
        const int j = find_slot<2>(T.slots, T.nslots, c);
        const BatchSlot& d = T.slots[j];
        SlotState* stt = T.states + d.state;
        const int kit = stt->k;  // >= 2 after a round
        const double nsq_prev = stt->nsq_prev;
        const int e = kit - 1 > 0 ? pow2_exponent_from_nsq(nsq_prev) : 0;
        const double lam = scale_pow2(stt->dot, -e) / nsq_prev;
        const XT* cur = static_cast<const XT*>((kit & 1) ? d.Y : d.X);
        const XT* prev = static_cast<const XT*>((kit & 1) ? d.X : d.Y);
        const int lo = (c - d.res0) * kResRows;
        const int hi = min(d.nor, lo + kResRows);
        double rr = 0.0;
        for (int r = lo + threadIdx.x; r < hi; r += blockDim.x) {
            const double dl = scale_pow2((double)cur[r], -e) - lam * (double)prev[r];
            rr = fma(dl, dl, rr);
        }
        rr = block_sum<256>(rr, red);
        if (threadIdx.x == 0) {
            T.res_part[c] = rr;
            __threadfence();
            last = atomicAdd(&stt->res_count, 1u) == (unsigned)d.nres - 1u;
        }
        __syncthreads();
        if (last && threadIdx.x < 32) {
            __threadfence();
            double s0 = 0.0;
            for (int q = threadIdx.x; q < d.nres; q += 32) s0 += __ldcg(T.res_part + d.res0 + q);
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
    static int grid(int sm_count) {
        static int occ = -1;
        if (occ < 0) {
            auto k = k_batch_spmv<VT, XT, AT, kBatchNT, kMliIpt>;
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
            int o = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, kBatchNT, SMEM);
            occ = o > 0 ? o : 1;
        }
        return occ * sm_count;
    }
    static cudaError_t step(const BatchTable* T, int want_dot, int sm_count, cudaStream_t st) {
        k_batch_spmv<VT, XT, AT, kBatchNT, kMliIpt><<<grid(sm_count), kBatchNT, SMEM, st>>>(T, want_dot);
        k_batch_reduce<XT, AT><<<2 * sm_count, 256, 0, st>>>(T, want_dot);
        return cudaGetLastError();
    }
};

}  // namespace

void batch_prepare(int sm_count) {
    BatchKernels<double, double, double>::grid(sm_count);
    BatchKernels<float, float, float>::grid(sm_count);
    BatchKernels<__nv_bfloat16, float, float>::grid(sm_count);
}

cudaError_t launch_batch_round(int cfg, const BatchTable* T, int steps, int sm_count, cudaStream_t st) {
    for (int it = 0; it < steps; ++it) {
        const int want_dot = it == steps - 1;
        cudaError_t e;
        switch (cfg) {
            case kCfgF32: e = BatchKernels<float, float, float>::step(T, want_dot, sm_count, st); break;
            case kCfgBF16: e = BatchKernels<__nv_bfloat16, float, float>::step(T, want_dot, sm_count, st); break;
            default: e = BatchKernels<double, double, double>::step(T, want_dot, sm_count, st); break;
        }
        if (e != cudaSuccess) return e;
    }
    if (cfg == kCfgF64) k_batch_resid<double><<<2 * sm_count, 256, 0, st>>>(T);
    else k_batch_resid<float><<<2 * sm_count, 256, 0, st>>>(T);
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
