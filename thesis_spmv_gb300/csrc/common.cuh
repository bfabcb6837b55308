// common.cuh -- device helpers shared by the pwmgpu kernels (sm_103a).
//
// * TMA 1D bulk copies (cp.async.bulk) completing on an mbarrier.
// * Bounded mbarrier waits: every wait gives up after a clock64 budget, sets
//   the launch's status word and lets the kernel return (no trap, no hang).
// * Exact power-of-two rescaling done on the exponent field (integer pipe),
//   so the power method never spends an FP64 multiply per row on scaling:
//   on GB300 the FP64 pipe (about 1.9 DFMA/clk/SM) is a co-bottleneck with HBM.
#pragma once
#include <cmath>
#include <cstring>
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "internal.h"
#include "pwmgpu.h"

namespace pwmgpu {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while its predecessor on the stream finishes;
// pdl_wait() blocks until the predecessor has completed and its writes are
// visible (a no-op without such a predecessor); pdl_trigger() lets this
// kernel's own dependent launch start early.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Arrive (count 1) and announce `bytes` of asynchronous transactions.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded wait on an mbarrier phase.  Returns false when the budget runs out
// (recording PWMGPU_ERR_TIMEOUT) or when another thread of the launch has
// already recorded a failure; the caller then leaves the kernel.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* status,
                                                  long long budget = kWaitCycles, bool watch_status = true) {
    if (mbar_try_wait(bar, parity)) return true;
    long long t0 = clock64();
    unsigned spins = 0;
    while (!mbar_try_wait(bar, parity)) {
        if ((++spins & 255u) == 0u) {
            if (watch_status && *(volatile int*)status != PWMGPU_OK) return false;
            if (clock64() - t0 > budget) {
                atomicCAS(status, PWMGPU_OK, PWMGPU_ERR_TIMEOUT);
                return false;
            }
        }
    }
    return true;
}

// L2 eviction policy for data read exactly once per pass (the matrix stream):
// evict-first keeps the gathered vector resident in L2 instead.
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// Default L2 policy (for data other CTAs read again, like x windows).
__device__ __forceinline__ uint64_t policy_evict_normal() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// 1D bulk copy global -> shared (TMA engine).  dst, src 16-byte aligned, bytes
// a non-zero multiple of 16.  Completion is signalled on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                         uint64_t policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// ---- exact scaling by 2^e ------------------------------------------------
// Multiplying by a power of two is exact unless the result leaves the normal
// range; the normal case is an integer add on the exponent field.  Zeros,
// subnormals, infinities, NaNs and out-of-range results take an FP multiply.
__device__ __forceinline__ double scale_pow2(double v, int e) {
    long long bits = __double_as_longlong(v);
    int ex = (int)((bits >> 52) & 0x7FF);
    int ne = ex + e;
    if (ex != 0 && ex != 0x7FF && ne > 0 && ne < 0x7FF) return __longlong_as_double(bits + ((long long)e << 52));
    return v * ldexp(1.0, e);
}

__device__ __forceinline__ float scale_pow2(float v, int e) {
    int bits = __float_as_int(v);
    int ex = (bits >> 23) & 0xFF;
    int ne = ex + e;
    if (ex != 0 && ex != 0xFF && ne > 0 && ne < 0xFF) return __int_as_float(bits + (e << 23));
    return v * ldexpf(1.0f, e);
}

// Exponent e that brings a vector with squared norm `nsq` to a norm in
// [1, 2) when scaled by 2^e, computed from the exponent field only
// (nsq = m * 2^q with m in [0.5, 1) gives e = -floor((q - 1) / 2)).  Zero,
// subnormal and non-finite inputs give 0: no rescaling.
__host__ __device__ __forceinline__ int pow2_exponent_from_nsq(double nsq) {
    long long bits;
#ifdef __CUDA_ARCH__
    bits = __double_as_longlong(nsq);
#else
    std::memcpy(&bits, &nsq, sizeof bits);
#endif
    int ex = (int)((bits >> 52) & 0x7FF);
    if (bits <= 0 || ex == 0 || ex == 0x7FF) return 0;
    int q = ex - 1022;  // frexp exponent of a normal positive double
    int h = q - 1;
    int fl = (h >= 0) ? h / 2 : -((-h + 1) / 2);  // floor(h / 2)
    return -fl;
}

// Exponent of the power method's rescale for an iterate with squared norm
// nsq: 0 (no rescale) while nsq stays within [2^-window, 2^window], else the
// exponent that brings the norm into [1, 2).  Rescaling by powers of two is
// exact, so the schedule does not change the normalised iterates; it only
// keeps them clear of overflow and underflow.  window: 256 for FP64 vectors,
// 32 for FP32 vectors.
__host__ __device__ __forceinline__ int pow2_rescale_exponent(double nsq, int window) {
    long long bits;
#ifdef __CUDA_ARCH__
    bits = __double_as_longlong(nsq);
#else
    std::memcpy(&bits, &nsq, sizeof bits);
#endif
    const int ex = (int)((bits >> 52) & 0x7FF) - 1023;  // unbiased exponent
    if (bits > 0 && ex >= -window && ex < window) return 0;
    return pow2_exponent_from_nsq(nsq);
}
template <typename XT>
__host__ __device__ __forceinline__ int rescale_window() {
    return sizeof(XT) == 4 ? 32 : 256;
}

// Magnitude key of a vector element: the sign-cleared top 32 bits of its
// IEEE-754 pattern (FP64: sign, exponent and 20 mantissa bits; FP32: the whole
// word).  For finite values the key orders like |v|, so the largest key of a
// vector (an integer max: no FP64 pipe) gives the exponent of its largest
// element.
__device__ __forceinline__ unsigned mag_key(double v) {
    return (unsigned)((unsigned long long)__double_as_longlong(v) >> 32) & 0x7FFFFFFFu;
}
__device__ __forceinline__ unsigned mag_key(float v) { return __float_as_uint(v) & 0x7FFFFFFFu; }

// Exponent e of the exact 2^e rescale from the largest magnitude key of a
// vector (instead of its squared norm): no rescale while the largest element
// 2^E satisfies 2E in [-window, window) -- then ||v||^2 lies within
// 2^[-window, window + 2 + log2 n), far from the range ends -- else e = -E,
// which brings the largest element into [1, 2).  A zero vector or a
// non-finite key gives 0; a subnormal largest element is scaled by 2^900.
template <typename XT>
__host__ __device__ __forceinline__ int pow2_rescale_exponent_key(unsigned key) {
    constexpr int kShift = sizeof(XT) == 4 ? 23 : 20;
    constexpr int kBias = sizeof(XT) == 4 ? 127 : 1023;
    constexpr unsigned kInf = sizeof(XT) == 4 ? 0x7F800000u : 0x7FF00000u;
    if (key == 0u || key >= kInf) return 0;
    const int field = (int)(key >> kShift);
    if (field == 0) return sizeof(XT) == 4 ? 100 : 900;
    const int ex = field - kBias;
    if (2 * ex >= -rescale_window<XT>() && 2 * ex < rescale_window<XT>()) return 0;
    return -ex;
}

// ---- value conversions ---------------------------------------------------
template <typename T> __device__ __forceinline__ double to_f64(T v);
template <> __device__ __forceinline__ double to_f64<double>(double v) { return v; }
template <> __device__ __forceinline__ double to_f64<float>(float v) { return (double)v; }
template <> __device__ __forceinline__ double to_f64<__nv_bfloat16>(__nv_bfloat16 v) { return (double)__bfloat162float(v); }

// FP32 -> FP64 widening on the integer pipes: for a normal float the IEEE-754
// fields move over (exponent rebiased by 1023 - 127 = 896, mantissa to the top
// of the 52-bit field), a zero keeps its sign.  Subnormals, infinities and
// NaNs (widen_special) are left to the conversion instruction.  On GB300 the
// FP64 pipe runs 2 operations per clock per SM, so row passes over FP32
// vectors keep it for their FMAs.
__device__ __forceinline__ bool widen_special(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xFFu;
    return ex == 0xFFu || (ex == 0u && (u & 0x7FFFFFu) != 0u);
}
__device__ __forceinline__ double widen_normal(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xFFu;
    const unsigned hi = (u & 0x80000000u) | (ex != 0u ? (ex + 896u) << 20 : 0u) | ((u & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}

template <typename T> __device__ __forceinline__ float to_f32(T v);
template <> __device__ __forceinline__ float to_f32<double>(double v) { return (float)v; }
template <> __device__ __forceinline__ float to_f32<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f32<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

}  // namespace pwmgpu
