// sell.cu -- SELL-32 storage and SpMV for FP32 / BF16 values: the
// low-precision iterations of the power method on stencil and banded
// matrices.
//
// Slice s holds rows [32 s, 32 s + 32); its width w_s is its longest row.
// Element j of row 32 s + l sits at soff[s] + 32 j + l (column-major inside
// the slice: for each j a warp reads 32 consecutive elements), its column as
// a 16-bit offset from 32 s - 32768 (every column within 32768 rows of the
// slice fits: stencils, banded matrices), its value as FP32 or BF16.  Rows
// shorter than w_s are padded with the offset 0xFFFF (never a column: the
// largest offset stored is 65534) and value 0; the kernel skips it, so it
// needs no row lengths.  One lane computes one row: the row's products
// summed left to right in CRS order, as CRS::mv (Matrix/CRS.hpp:99-109)
// sums them -- no carries, no fix-up, and a fraction of the merge kernel's
// instructions per nonzero, which is what the low-precision iterations are
// bound by (the FP64 merge kernel is bound by HBM and the FP64 pipe
// instead, where this format gains nothing).  A warp keeps two slices in
// flight and issues a slice's column and value loads together.  A matrix
// gets the format when every column fits and the padding stays within a
// quarter of its nonzeros.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"
#include "merge.cuh"
#include "sell.cuh"

namespace pwmgpu {

namespace {

constexpr int kSellNT = 256;  // threads per CTA

// soff[s + 1] = 32 * longest row of slice s (scanned afterwards); *total +=
// the same in 64 bits (the padded size, checked before the 32-bit scan).
__global__ void k_sell_width(const int32_t* __restrict__ row_start, int nor, int nslices, int32_t* __restrict__ soff,
                             unsigned long long* total) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    unsigned long long sum = 0;
    for (int s = blockIdx.x * wpb + (threadIdx.x >> 5); s < nslices; s += gridDim.x * wpb) {
        const int r = s * 32 + lane;
        int len = r < nor ? row_start[r + 1] - row_start[r] : 0;
        for (int o = 16; o > 0; o >>= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
        if (lane == 0) soff[s + 1] = 32 * len;
        sum += 32ull * (unsigned long long)len;
    }
    if (lane == 0 && sum) atomicAdd(total, sum);
}

// Lane l of the warp of slice s writes row 32 s + l; *flag = 1 when a column
// does not fit the 16-bit offset (0 .. 65534 from 32 s - 32768).
template <typename VT>
__global__ void k_sell_fill(const int32_t* __restrict__ row_start, const int32_t* __restrict__ col,
                            const double* __restrict__ val, int nor, int nslices, const int32_t* __restrict__ soff,
                            uint16_t* __restrict__ col16, VT* __restrict__ sval, int* flag) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    bool bad = false;
    for (int s = blockIdx.x * wpb + (threadIdx.x >> 5); s < nslices; s += gridDim.x * wpb) {
        const int r = s * 32 + lane;
        const int rs = r < nor ? row_start[r] : 0;
        const int len = r < nor ? row_start[r + 1] - rs : 0;
        const int o0 = soff[s], w = (soff[s + 1] - o0) >> 5;
        const int cb = s * 32 - 32768;
        for (int j = 0; j < w; ++j) {
            const long long e = (long long)o0 + 32LL * j + lane;
            if (j < len) {
                const int off = col[rs + j] - cb;
                bad |= off < 0 || off >= (int)kSellPad;
                col16[e] = (uint16_t)off;
                sval[e] = (VT)val[rs + j];
            } else {
                col16[e] = kSellPad;
                sval[e] = (VT)0.0f;
            }
        }
    }
    if (bad) atomicOr(flag, 1);
}

template <typename VT>
struct SellArgs {
    const int32_t* soff;
    const uint16_t* col16;
    const VT* val;
    const int32_t* row_start;
    int nor, nslices;
    const float* x;
    float* y;
    const double* nsq_in;  // ||x||^2, source of the power method's 2^e rescale, or null (e = 0)
    double* npart;         // null, or per-CTA shares of ||y||^2 ...
    unsigned int* counter;  // ... summed in order by the last CTA (counter zero between launches)
    double* nsq_out;        // ... into *nsq_out
};

// y = 2^e A x, one lane per row; a warp takes slices s and s + (warps in the
// grid) together, then moves on by twice that.  With npart, also ||y||^2
// (FP64, widened on the integer pipes; deterministic for a fixed grid).
template <typename VT>
__global__ void __launch_bounds__(kSellNT) k_sell_spmv(SellArgs<VT> a) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, tw = (gridDim.x * blockDim.x) >> 5;
    pdl_wait();  // x and ||x||^2 come from the kernel before on the stream
    const int e = a.nsq_in ? pow2_rescale_exponent(*a.nsq_in, rescale_window<float>()) : 0;
    double ss = 0.0;
    for (int s = gw; s < a.nslices; s += 2 * tw) {
        const int s2 = s + tw;
        const bool two = s2 < a.nslices;
        const int oa = __ldg(a.soff + s), wa = (__ldg(a.soff + s + 1) - oa) >> 5;
        const int ob = two ? __ldg(a.soff + s2) : 0, wb = two ? (__ldg(a.soff + s2 + 1) - ob) >> 5 : 0;
        float ya, yb;
        sell_rows2(a.col16 + oa + lane, a.val + oa + lane, a.x, s * 32 - 32768, wa, a.col16 + ob + lane,
                   a.val + ob + lane, a.x, s2 * 32 - 32768, wb, ya, yb);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = (h ? s2 : s) * 32 + lane;
            float out = h ? yb : ya;
            if (e != 0) out = scale_pow2(out, e);
            const bool live = (h == 0 || two) && r < a.nor;
            if (live) a.y[r] = out;
            else out = 0.0f;
            if (a.npart) {
                const double wv = __any_sync(0xffffffffu, widen_special(out)) ? (double)out : widen_normal(out);
                ss = fma(wv, wv, ss);
            }
        }
    }
    if (!a.npart) return;
    __shared__ double red[kSellNT / 32];
    __shared__ bool am_last;
    const double t = block_sum<kSellNT>(ss, red);
    if (threadIdx.x == 0) {
        a.npart[blockIdx.x] = t;
        __threadfence();
        am_last = atomicAdd(a.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (am_last && threadIdx.x < 32) {
        __threadfence();
        double s0 = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) s0 += __ldcg(a.npart + i);
        for (int o = 16; o > 0; o >>= 1) s0 += __shfl_down_sync(0xffffffffu, s0, o);
        if (threadIdx.x == 0) {
            *a.nsq_out = s0;
            *a.counter = 0u;
        }
    }
}

template <typename VT>
cudaError_t sell_spmv_impl(const SellPlan& S, const void* val, const int32_t* row_start, int nor, const float* x,
                           float* y, const double* nsq_in, double* nsq_out, unsigned int* counter, int sm_count,
                           cudaStream_t st) {
    SellArgs<VT> a{S.soff, S.col16, (const VT*)val, row_start, nor, S.nslices, x, y, nsq_in,
                   nsq_out ? S.npart : nullptr, counter, nsq_out};
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(sell_grid(S.nslices, sm_count));
    cfg.blockDim = dim3(kSellNT);
    cfg.stream = st;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_sell_spmv<VT>, a);
    return cudaGetLastError();
}

}  // namespace

int sell_grid(int nslices, int sm_count) {
    static int occ = 0;
    if (occ == 0) {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_sell_spmv<float>, kSellNT, 0) != cudaSuccess || o < 1)
            o = 1;
        occ = o < 8 ? o : 8;  // the shares of ||y||^2 have room for 8 CTAs per SM
    }
    const long long ctas = ((long long)nslices + kSellNT / 32 - 1) / (kSellNT / 32);
    const long long cap = (long long)occ * sm_count;
    const long long g = ctas < cap ? ctas : cap;
    return g > 0 ? (int)g : 1;
}

void SellPlan::release() {
    dev_free(soff);
    dev_free(col16);
    dev_free(val32);
    dev_free(valbf);
    dev_free(npart);
    soff = nullptr;
    col16 = nullptr;
    val32 = nullptr;
    valbf = nullptr;
    npart = nullptr;
    nslices = 0;
    stored = 0;
    state = 0;
}

int sell_build(SellPlan& S, const int32_t* row_start, const int32_t* col, const double* val, int nor, long long nnz,
               bool bf16, int sm_count, cudaStream_t st) {
    if (S.state < 0) return 1;
    if (nor <= 0 || nnz <= 0) {
        S.state = -1;
        return 1;
    }
    const int ns = (nor + 31) / 32;
    const int blocks = (int)std::min<long long>(((long long)ns + 7) / 8, 32LL * sm_count);
    int* flag = nullptr;
    int32_t* scratch = nullptr;
    unsigned long long* total = nullptr;
    int rc = 0;
    do {
        if (S.state == 0) {
            if (cudaMalloc((void**)&S.soff, sizeof(int32_t) * ((size_t)ns + 1)) != cudaSuccess ||
                cudaMalloc((void**)&total, sizeof(unsigned long long)) != cudaSuccess) {
                rc = 2;
                break;
            }
            if (cudaMemsetAsync(S.soff, 0, sizeof(int32_t), st) != cudaSuccess ||
                cudaMemsetAsync(total, 0, sizeof(unsigned long long), st) != cudaSuccess) {
                rc = 2;
                break;
            }
            k_sell_width<<<blocks, 256, 0, st>>>(row_start, nor, ns, S.soff, total);
            unsigned long long h = 0;
            if (cudaMemcpyAsync(&h, total, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess) {
                rc = 2;
                break;
            }
            // padding within a quarter of the nonzeros, offsets within int32
            if ((double)h > 1.25 * (double)nnz || h >= (1ULL << 31) - 64) {
                rc = 1;
                break;
            }
            if (cudaMalloc((void**)&scratch, sizeof(int32_t) * (size_t)scan_scratch_elems(ns)) != cudaSuccess ||
                launch_inclusive_scan(S.soff + 1, ns, scratch, st) != cudaSuccess ||
                cudaMalloc((void**)&S.col16, sizeof(uint16_t) * ((size_t)h + 16)) != cudaSuccess ||
                cudaMalloc((void**)&S.npart, sizeof(double) * (8 * (size_t)sm_count + 64)) != cudaSuccess ||
                cudaMalloc((void**)&flag, sizeof(int)) != cudaSuccess || cudaMemsetAsync(flag, 0, sizeof(int), st) != cudaSuccess) {
                rc = 2;
                break;
            }
            S.nslices = ns;
            S.stored = (long long)h;
        }
        void** dst = bf16 ? &S.valbf : (void**)&S.val32;
        if (*dst == nullptr) {
            const size_t esz = bf16 ? sizeof(__nv_bfloat16) : sizeof(float);
            if (cudaMalloc(dst, esz * ((size_t)S.stored + 16)) != cudaSuccess) {
                rc = 2;
                break;
            }
            if (!flag && (cudaMalloc((void**)&flag, sizeof(int)) != cudaSuccess ||
                          cudaMemsetAsync(flag, 0, sizeof(int), st) != cudaSuccess)) {
                rc = 2;
                break;
            }
            // the columns are (re)written with every value array: same bits
            if (bf16)
                k_sell_fill<__nv_bfloat16><<<blocks, 256, 0, st>>>(row_start, col, val, nor, ns, S.soff, S.col16,
                                                                   (__nv_bfloat16*)S.valbf, flag);
            else
                k_sell_fill<float><<<blocks, 256, 0, st>>>(row_start, col, val, nor, ns, S.soff, S.col16, S.val32,
                                                           flag);
            int hf = 0;
            if (cudaMemcpyAsync(&hf, flag, sizeof hf, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
                rc = 2;
                break;
            }
            if (hf) {
                rc = 1;
                break;
            }
        }
        S.state = 1;
    } while (0);
    if (flag) dev_free(flag);
    if (scratch) dev_free(scratch);
    if (total) dev_free(total);
    if (rc) {
        (void)cudaGetLastError();
        S.release();
        S.state = rc == 1 ? -1 : 0;  // ineligible for good; out of memory: try again later
    }
    return rc;
}

cudaError_t launch_sell_spmv(const SellPlan& S, bool bf16, const int32_t* row_start, int nor, const float* x, float* y,
                             const double* nsq_in, double* nsq_out, unsigned int* counter, int sm_count,
                             cudaStream_t st) {
    if (bf16)
        return sell_spmv_impl<__nv_bfloat16>(S, S.valbf, row_start, nor, x, y, nsq_in, nsq_out, counter, sm_count,
                                             st);
    return sell_spmv_impl<float>(S, S.val32, row_start, nor, x, y, nsq_in, nsq_out, counter, sm_count, st);
}

}  // namespace pwmgpu
