// hostcopy.cu -- copies between pageable host memory and device memory done
// by SM loads / stores, for hosts whose GPU reaches pageable memory directly
// (cudaDevAttrPageableMemoryAccess = 1, e.g. coherent CPU-GPU links).  The
// copy engines stage pageable memory through a bounce buffer at about half
// the link's speed; loads and stores from the SMs move it at close to the
// pinned rate.  Used by pwmgpu_mv for caller arrays that are not pinned.
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace pwmgpu {

namespace {

constexpr int kCopyThreads = 256;
// 32 CTAs x 256 threads x 4 loads of 16 bytes: 512 KB in flight, enough for
// the link; more CTAs slowed the pipelined SpMV they run beside (measured:
// 1.92 ms at 4, 1.33 at 32, 1.68 at 128 CTAs for the 4096^2 Poisson call).
constexpr int kCopyCtas = 32;

// 16-byte elements; `tail` copies one trailing double (odd counts).
__global__ void __launch_bounds__(kCopyThreads) k_host_copy16(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                              long long n16, const double* tail_src,
                                                              double* tail_dst) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n16; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n16; i += stride) dst[i] = src[i];
    if (tail_src && blockIdx.x == 0 && threadIdx.x == 0) *tail_dst = *tail_src;
}

__global__ void __launch_bounds__(kCopyThreads) k_host_copy8(const double* __restrict__ src, double* __restrict__ dst,
                                                             long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        const double a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

int copy_grid(long long n) {
    const long long g = (n + kCopyThreads - 1) / kCopyThreads;
    return (int)(g < kCopyCtas ? (g > 0 ? g : 1) : kCopyCtas);
}

}  // namespace

cudaError_t launch_host_copy(const double* src, double* dst, long long n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const uintptr_t as = (uintptr_t)src % 16, ad = (uintptr_t)dst % 16;
    if (as != ad || as % 8 != 0) {  // different 16-byte phases: 8-byte elements
        k_host_copy8<<<copy_grid(n), kCopyThreads, 0, st>>>(src, dst, n);
        return cudaGetLastError();
    }
    long long head = as ? 1 : 0;  // both 8 bytes past a 16-byte boundary: peel one element
    if (head) {
        k_host_copy8<<<1, 32, 0, st>>>(src, dst, 1);
        src += 1;
        dst += 1;
        n -= 1;
        if (n == 0) return cudaGetLastError();
    }
    const long long n16 = n / 2;
    const bool odd = (n & 1) != 0;
    k_host_copy16<<<copy_grid(n16 > 0 ? n16 : 1), kCopyThreads, 0, st>>>(
        reinterpret_cast<const uint4*>(src), reinterpret_cast<uint4*>(dst), n16, odd ? src + n - 1 : nullptr,
        odd ? dst + n - 1 : nullptr);
    return cudaGetLastError();
}

}  // namespace pwmgpu
