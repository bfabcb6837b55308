// noalloc.cu -- y = A x on caller-owned device CRS arrays without allocating.
//
// Who needs this: callers that cannot allocate device memory at call time --
// a host runtime whose allocator owns all device memory after start-up (it
// hands out pre-sized buffers only), a latency-bound serving loop that must
// not hit cudaMalloc / cudaFree (both can synchronise the whole device), or
// a plug-in that is only given device pointers.  The handle-based API
// (pwmgpu_create / pwmgpu_load_csr) allocates its plan and scratch; this entry
// point instead keeps its scratch -- the merge-path sub-tile coordinates and
// the per-sub-tile carries -- in one file-scope __device__ array of fixed size
// that every GPU loading the library holds until the process exits.
//
// The kernels follow the merge-path SpMV of the library (CRS_Merge.hpp:95-141
// restated): k_merge_partition cuts the merge path into sub-tiles of
// kNoAllocWM items, k_noalloc_spmv processes one sub-tile per warp straight
// from the CRS arrays (lanes split the sub-tile's nonzeros, one FMA each; row
// ends found by walking row_start), and k_merge_fixup adds the carries.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "internal.h"
#include "merge.cuh"

namespace pwmgpu {

// Scratch size and the largest problem it serves: every sub-tile needs one
// int2 coordinate and one double carry (16 bytes).
constexpr int kNoAllocWM = 256;                         // merge items per sub-tile
constexpr size_t kNoAllocBytes = 8u << 20;              // 8 MiB
constexpr long long kNoAllocMaxSub = (long long)(kNoAllocBytes / 16) - 1;
constexpr long long kNoAllocMaxItems = kNoAllocMaxSub * kNoAllocWM;  // nor + nnz limit

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

constexpr int kNoAllocIpt = kNoAllocWM / 32;

// One warp per sub-tile, reading the CRS arrays directly.
__global__ void __launch_bounds__(256) k_noalloc_spmv(const int32_t* __restrict__ row_start,
                                                      const int32_t* __restrict__ col,
                                                      const double* __restrict__ val, const int2* __restrict__ subc,
                                                      int nsub, int nor, const double* __restrict__ x,
                                                      double* __restrict__ y, double* __restrict__ carries) {
    __shared__ int crow_s[256];
    __shared__ double cval_s[256];
    __shared__ double hval_s[256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int* crow = crow_s + 32 * w;
    double* cval = cval_s + 32 * w;
    double* hval = hval_s + 32 * w;
    for (int s = blockIdx.x * 8 + w; s < nsub; s += gridDim.x * 8) {
        const int2 c0 = subc[s], c1 = subc[s + 1];
        const int rw0 = c0.x, kw0 = c0.y, rw1 = c1.x, kw1 = c1.y;
        const int nkw = kw1 - kw0;
        const int qm = nkw >> 5, rem = nkw & 31;
        const int cnt = qm + (lane < rem ? 1 : 0);
        const int q = qm + (rem ? 1 : 0);
        const int b0 = kw0 + lane * qm + (lane < rem ? lane : rem);
        const int fr = nkw > 0 ? row_of(row_start, kw0, rw0, rw1) : rw1;
        for (int r = rw0 + lane; r < fr; r += 32) y[r] = 0.0;  // no nonzeros here
        int a = cnt > 0 ? row_of(row_start, b0, rw0, rw1) : rw1;
        const bool head_open = cnt > 0 && __ldg(row_start + a) < b0;
        int rend = (cnt > 0 && a < rw1) ? __ldg(row_start + a + 1) : INT_MAX;
        double xv[kNoAllocIpt], vv[kNoAllocIpt];
#pragma unroll
        for (int j = 0; j < kNoAllocIpt; ++j) {
            xv[j] = (j < cnt) ? __ldg(x + __ldg(col + b0 + j)) : 0.0;
            vv[j] = (j < cnt) ? __ldg(val + b0 + j) : 0.0;
        }
        double acc = 0.0;
        bool to_head = head_open && lane > 0;  // first completed row goes to hval
#pragma unroll
        for (int j = 0; j < kNoAllocIpt; ++j) {
            if (j < q) {
                acc = fma(vv[j], xv[j], acc);
                const int bn = b0 + j + 1;
                if (j < cnt && bn == rend) {
                    if (to_head) hval[lane] = acc;
                    else y[a] = acc;
                    to_head = false;
                    acc = 0.0;
                    ++a;
                    // empty rows that end here are written as 0
                    while (a < rw1 && __ldg(row_start + a + 1) == bn) {
                        y[a] = 0.0;
                        ++a;
                    }
                    rend = a < rw1 ? __ldg(row_start + a + 1) : INT_MAX;
                }
            }
        }
        if (cnt == 0) a = rw1;
        crow[lane] = a;
        cval[lane] = acc;
        __syncwarp();
        if (lane == 0 || crow[lane - 1] != a) {
            double sum = acc;
            int u = lane + 1;
            for (; u < 32 && crow[u] == a; ++u) sum += cval[u];
            // A row below rw1 ends inside this sub-tile, so some lane at or
            // after the leader completes it and the run stops before lane 32;
            // the u < 32 test keeps hval[u] inside this warp's slice anyway.
            if (a < rw1) {
                const int b0u = kw0 + u * qm + (u < rem ? u : rem);
                if (u < 32 && __ldg(row_start + a) < b0u) y[a] = hval[u] + sum;
            } else if (a < nor) {
                carries[s] = sum;
            }
        }
        __syncwarp();
    }
}

std::mutex g_mu;
void* g_scratch_addr[64] = {nullptr};  // per device ordinal
int g_sm_count[64] = {0};              // SM count of that device, read with the address

// Failures are reported through pwmgpu_last_error(), like every entry point.
int nfail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    record_error(buf);
    return code;
}

// Device address of the scratch array on the current device and that
// device's SM count, looked up once per device (the array's name is only a
// host-side stand-in).
int scratch_address(void** out, int* sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return nfail(PWMGPU_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return nfail(PWMGPU_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        int count = 0;
        e = cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess || count < 1)
            return nfail(PWMGPU_ERR_CUDA, "SM count of device %d: %s", dev, cudaGetErrorString(e));
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return nfail(PWMGPU_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed on device %d: %s", dev,
                         cudaGetErrorString(e));
        g_sm_count[dev] = count;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    *sms = g_sm_count[dev];
    return PWMGPU_OK;
}

}  // namespace

}  // namespace pwmgpu

using namespace pwmgpu;

extern "C" int pwmgpu_mv_csr_device_noalloc(int32_t nor, int32_t noc, int32_t nnz, const int32_t* row_start,
                                             const int32_t* col_ind, const double* vals, const double* x, double* y,
                                             void* stream) {
    if (nor < 0 || noc < 0 || nnz < 0) return nfail(PWMGPU_ERR_INVALID, "negative size");
    if ((long long)nor + nnz > kNoAllocMaxItems)
        return nfail(PWMGPU_ERR_INVALID,
                     "nor + nnz = %lld exceeds this entry point's fixed scratch (at most %lld merge items; use "
                     "pwmgpu_create / pwmgpu_load_csr for larger matrices)",
                     (long long)nor + nnz, kNoAllocMaxItems);
    if (nor == 0) return PWMGPU_OK;
    if (!row_start || !y || (nnz > 0 && (!col_ind || !vals || !x)))
        return nfail(PWMGPU_ERR_INVALID, "null device array");
    void* base = nullptr;
    int sms = 1;
    int rc = scratch_address(&base, &sms);
    if (rc != PWMGPU_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const long long total = (long long)nor + nnz;
    const int nsub = (int)((total + kNoAllocWM - 1) / kNoAllocWM);
    int2* subc = reinterpret_cast<int2*>(base);
    double* carries = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(base) + 8 * (kNoAllocMaxSub + 1));
    // Scratch keeps the previous call's contents: clear the carries used now.
    cudaError_t e = cudaMemsetAsync(carries, 0, sizeof(double) * (size_t)nsub, st);
    if (e == cudaSuccess) e = launch_merge_partition(row_start, nor, nnz, kNoAllocWM, nsub, subc, st);
    if (e == cudaSuccess) {
        long long blocks = (nsub + 7) / 8;
        if (blocks > (long long)sms * 8) blocks = (long long)sms * 8;
        k_noalloc_spmv<<<(int)blocks, 256, 0, st>>>(row_start, col_ind, vals, subc, nsub, nor, x, y, carries);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        DevMatrix M;
        M.nor = nor;
        M.noc = noc;
        M.nnz = nnz;
        M.row_start = const_cast<int32_t*>(row_start);
        e = launch_merge_fixup_f64(kModeSpmv, M, subc, nsub, y, carries, nullptr, fixup_grid(nsub, sms), st);
    }
    if (e != cudaSuccess) return nfail(PWMGPU_ERR_CUDA, "pwmgpu_mv_csr_device_noalloc: %s", cudaGetErrorString(e));
    return PWMGPU_OK;
}
