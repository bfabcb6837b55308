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
// K2: merge-path SpMV (plain or with the power-method epilogue)
// ---------------------------------------------------------------------------
template <typename VT, typename XT, typename AT>
struct MergeArgs {
    const int32_t* row_start;
    const int32_t* col;
    const VT* val;
    const int2* tiles;
    int nor, nnz, num_tiles;
    const XT* x;
    XT* y;
    AT* carries;
    const double* nsq_in;  // MODE_POWER: ||x||^2 (source of the 2^e rescale), or null for e = 0
    double* partials;      // MODE_POWER: per-CTA sum of squares
    int* status;
};

template <int MODE, typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
__global__ void __launch_bounds__(NT, 2) k_merge_spmv(MergeArgs<VT, XT, AT> a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    MergeSmem<VT, XT, AT, NT, IPT, STAGES> sm{smem_raw};
    const int tid = threadIdx.x;
    const int G = gridDim.x;
    const int my_tiles = blockIdx.x < a.num_tiles ? (a.num_tiles - 1 - blockIdx.x) / G + 1 : 0;
    const int e = (MODE == MODE_POWER && a.nsq_in) ? pow2_exponent_from_nsq(*a.nsq_in) : 0;
    const uint64_t pol = policy_evict_first();

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&sm.bar()[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0)
        for (int s = 0; s < STAGES && s < my_tiles; ++s)
            issue_tile(sm, s, blockIdx.x + s * G, a.tiles, a.row_start, a.col, a.val, a.nor, pol);

    double sumsq = 0.0;
    for (int i = 0; i < my_tiles; ++i) {
        const int s = i % STAGES;
        const uint32_t parity = (uint32_t)(i / STAGES) & 1u;
        // the stage of tile i-1 is free (the previous iteration ended with a barrier)
        if (tid == 0 && i >= 1 && i + STAGES - 1 < my_tiles)
            issue_tile(sm, (i + STAGES - 1) % STAGES, blockIdx.x + (i + STAGES - 1) * G, a.tiles, a.row_start,
                       a.col, a.val, a.nor, pol);
        if (!process_tile<MODE>(sm, s, parity, blockIdx.x + i * G, a.x, a.y, a.carries, a.nor, e, sumsq, a.status))
            return;
    }
    if (MODE == MODE_POWER) {
        double t = block_sum<NT>(sumsq, sm.red());
        if (tid == 0) a.partials[blockIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------
// Fix-up: add each tile's carry to the row that the tile left unfinished.
// One thread per tile; the first tile of a run of tiles ending in the same
// row adds the run in tile order (deterministic).  The run's row r is
// completed (and its partial written) by the first tile after the run; the
// carry is real only if that tile started inside row r.
// MODE_POWER also finishes ||y||^2: the sum of squares of the rows fixed
// here, then one deterministic reduction over all partials by the last CTA.
// ---------------------------------------------------------------------------
template <typename XT, typename AT>
struct FixArgs {
    const int32_t* row_start;
    const int2* tiles;
    int nor, num_tiles;
    XT* y;
    const AT* carries;
    const double* nsq_in;
    const double* spmv_partials;
    int n_spmv_partials;
    double* fix_partials;
    unsigned int* counter;
    double* nsq_out;
};

template <int MODE, typename XT, typename AT>
__global__ void __launch_bounds__(256) k_merge_fixup(FixArgs<XT, AT> a) {
    __shared__ double red[32];
    __shared__ bool am_last;
    const int e = (MODE == MODE_POWER && a.nsq_in) ? pow2_exponent_from_nsq(*a.nsq_in) : 0;
    double sumsq = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < a.num_tiles; t += gridDim.x * blockDim.x) {
        const int r = a.tiles[t + 1].x;
        if (r >= a.nor) continue;
        if (t > 0 && a.tiles[t].x == r) continue;  // not the first tile of the run
        AT sum = a.carries[t];
        int n = t + 1;
        while (n < a.num_tiles && a.tiles[n + 1].x == r) sum += a.carries[n++];
        // tile n starts at (r, tiles[n].y) and completes row r
        if (a.tiles[n].y > a.row_start[r]) {
            AT v;
            if (MODE == MODE_POWER) v = (AT)a.y[r] + scale_pow2(sum, e);
            else v = (AT)a.y[r] + sum;
            a.y[r] = (XT)v;
            if (MODE == MODE_POWER) sumsq = fma((double)v, (double)v, sumsq);
        }
    }
    if (MODE != MODE_POWER) return;
    double t = block_sum<256>(sumsq, red);
    if (threadIdx.x == 0) {
        a.fix_partials[blockIdx.x] = t;
        __threadfence();
        unsigned prev = atomicAdd(a.counter, 1u);
        am_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (am_last && threadIdx.x < 32) {
        __threadfence();
        // lane l sums partials l, l+32, ... in order; then a fixed shuffle tree
        const int l = threadIdx.x;
        double s = 0.0;
        for (int i = l; i < a.n_spmv_partials; i += 32) s += __ldcg(a.spmv_partials + i);
        for (int i = l; i < (int)gridDim.x; i += 32) s += __ldcg(a.fix_partials + i);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (l == 0) {
            *a.nsq_out = s;
            *a.counter = 0u;
        }
    }
}

// ---------------------------------------------------------------------------
// Normalise the last two iterates of the power method (VectorUtill.hpp:34-41):
// v_last /= sqrt(nsq_last); v_prev /= sqrt(nsq_prev) when prev is an iterate.
// ---------------------------------------------------------------------------
template <typename XT>
__global__ void k_power_finalize(XT* __restrict__ last, const double* nsq_last, XT* __restrict__ prev,
                                 const double* nsq_prev, int n) {
    const double nl = sqrt(*nsq_last);
    const double np = prev ? sqrt(*nsq_prev) : 1.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        last[i] = (XT)((double)last[i] / nl);
        if (prev) prev[i] = (XT)((double)prev[i] / np);
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

__global__ void k_poisson_crs(int m, int n, int32_t* __restrict__ row_start, int32_t* __restrict__ col,
                              double* __restrict__ val) {
    const int N = m * n;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < N; row += gridDim.x * blockDim.x) {
        long long k = poisson_row_start(row, m, n);
        if (row >= m) { col[k] = row - m; val[k] = -1.0; ++k; }
        if (row % m != 0) { col[k] = row - 1; val[k] = -1.0; ++k; }
        col[k] = row; val[k] = 4.0; ++k;
        if (row % m != m - 1) { col[k] = row + 1; val[k] = -1.0; ++k; }
        if (row < N - m) { col[k] = row + m; val[k] = -1.0; ++k; }
        row_start[row + 1] = (int32_t)k;
        if (row == 0) row_start[0] = 0;
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

// ===========================================================================
// Host launchers
// ===========================================================================

// Tile configurations (threads per CTA, items per thread, pipeline stages).
template <typename VT, typename XT, typename AT, int NT, int IPT, int STAGES>
struct MergeKernels {
    using L = MergeLayout<VT, XT, AT, NT, IPT, STAGES>;
    static constexpr int TM = L::TM;
    static constexpr int SMEM = L::BYTES;

    static int occupancy() {
        static int occ = -1;
        if (occ < 0) {
            auto k = k_merge_spmv<MODE_SPMV, VT, XT, AT, NT, IPT, STAGES>;
            auto kp = k_merge_spmv<MODE_POWER, VT, XT, AT, NT, IPT, STAGES>;
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
            cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
            int o = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, NT, SMEM);
            occ = o > 0 ? o : 1;
        }
        return occ;
    }

    static cudaError_t spmv(int mode, const DevMatrix& M, const VT* val, const int2* tiles, int num_tiles, int grid,
                            const XT* x, XT* y, AT* carries, const double* nsq_in, double* partials, int* status,
                            cudaStream_t st) {
        occupancy();
        MergeArgs<VT, XT, AT> a{M.row_start, M.col, val, tiles, M.nor, (int)M.nnz, num_tiles, x, y, carries,
                                nsq_in, partials, status};
        if (mode == MODE_POWER)
            k_merge_spmv<MODE_POWER, VT, XT, AT, NT, IPT, STAGES><<<grid, NT, SMEM, st>>>(a);
        else
            k_merge_spmv<MODE_SPMV, VT, XT, AT, NT, IPT, STAGES><<<grid, NT, SMEM, st>>>(a);
        return cudaGetLastError();
    }
};

// The configurations the library instantiates.  Config ids are stable
// numbers used by the autotuner cache.
using F64_256x7 = MergeKernels<double, double, double, 256, 7, 2>;
using F64_128x11 = MergeKernels<double, double, double, 128, 11, 3>;
using F32_256x7 = MergeKernels<float, float, float, 256, 7, 2>;
using BF16_256x7 = MergeKernels<__nv_bfloat16, float, float, 256, 7, 2>;

int merge_items_per_tile(int cfg) {
    switch (cfg) {
        case 1: return F64_128x11::TM;
        default: return F64_256x7::TM;
    }
}

int merge_grid(int cfg, int num_tiles, int sm_count) {
    int occ = (cfg == 1) ? F64_128x11::occupancy() : F64_256x7::occupancy();
    long long g = (long long)occ * sm_count;
    if (g > num_tiles) g = num_tiles;
    return g > 0 ? (int)g : 1;
}

int merge_grid_f32(int num_tiles, int sm_count, bool bf16) {
    int occ = bf16 ? BF16_256x7::occupancy() : F32_256x7::occupancy();
    long long g = (long long)occ * sm_count;
    if (g > num_tiles) g = num_tiles;
    return g > 0 ? (int)g : 1;
}

cudaError_t launch_merge_partition(const int32_t* row_start, int nor, long long nnz, long long ipt, int parts,
                                   int2* out, cudaStream_t st) {
    int threads = 256;
    long long blocks = (parts + 1 + threads - 1) / threads;
    if (blocks > 65535) blocks = 65535;
    k_merge_partition<<<(int)blocks, threads, 0, st>>>(row_start, nor, (int)nnz, ipt, parts, out);
    return cudaGetLastError();
}

cudaError_t launch_merge_spmv_f64(int cfg, int mode, const DevMatrix& M, const int2* tiles, int num_tiles, int grid,
                                  const double* x, double* y, double* carries, const double* nsq_in,
                                  double* partials, int* status, cudaStream_t st) {
    if (cfg == 1)
        return F64_128x11::spmv(mode, M, M.val, tiles, num_tiles, grid, x, y, carries, nsq_in, partials, status, st);
    return F64_256x7::spmv(mode, M, M.val, tiles, num_tiles, grid, x, y, carries, nsq_in, partials, status, st);
}

cudaError_t launch_merge_spmv_f32(int mode, const DevMatrix& M, const void* val, bool bf16, const int2* tiles,
                                  int num_tiles, int grid, const float* x, float* y, float* carries,
                                  const double* nsq_in, double* partials, int* status, cudaStream_t st) {
    if (bf16)
        return BF16_256x7::spmv(mode, M, (const __nv_bfloat16*)val, tiles, num_tiles, grid, x, y, carries, nsq_in,
                                partials, status, st);
    return F32_256x7::spmv(mode, M, (const float*)val, tiles, num_tiles, grid, x, y, carries, nsq_in, partials,
                           status, st);
}

int merge_items_per_tile_f32() { return F32_256x7::TM; }

template <typename XT, typename AT>
static cudaError_t fixup_impl(int mode, const DevMatrix& M, const int2* tiles, int num_tiles, XT* y,
                              const AT* carries, const double* nsq_in, const double* spmv_partials, int n_spmv,
                              double* fix_partials, int fix_grid, unsigned int* counter, double* nsq_out,
                              cudaStream_t st) {
    FixArgs<XT, AT> a{M.row_start, tiles, M.nor, num_tiles, y, carries, nsq_in, spmv_partials, n_spmv,
                      fix_partials, counter, nsq_out};
    if (mode == MODE_POWER) k_merge_fixup<MODE_POWER, XT, AT><<<fix_grid, 256, 0, st>>>(a);
    else k_merge_fixup<MODE_SPMV, XT, AT><<<fix_grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_merge_fixup_f64(int mode, const DevMatrix& M, const int2* tiles, int num_tiles, double* y,
                                   const double* carries, const double* nsq_in, const double* spmv_partials,
                                   int n_spmv, double* fix_partials, int fix_grid, unsigned int* counter,
                                   double* nsq_out, cudaStream_t st) {
    return fixup_impl<double, double>(mode, M, tiles, num_tiles, y, carries, nsq_in, spmv_partials, n_spmv,
                                      fix_partials, fix_grid, counter, nsq_out, st);
}

cudaError_t launch_merge_fixup_f32(int mode, const DevMatrix& M, const int2* tiles, int num_tiles, float* y,
                                   const float* carries, const double* nsq_in, const double* spmv_partials,
                                   int n_spmv, double* fix_partials, int fix_grid, unsigned int* counter,
                                   double* nsq_out, cudaStream_t st) {
    return fixup_impl<float, float>(mode, M, tiles, num_tiles, y, carries, nsq_in, spmv_partials, n_spmv,
                                    fix_partials, fix_grid, counter, nsq_out, st);
}

int fixup_grid(int num_tiles, int sm_count) {
    long long g = (num_tiles + 255) / 256;
    if (g > sm_count) g = sm_count;
    return g > 0 ? (int)g : 1;
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
                               cudaStream_t st) {
    long long N = (long long)m * n;
    long long blocks = (N + 255) / 256;
    if (blocks > sm_count * 16) blocks = sm_count * 16;
    if (blocks < 1) blocks = 1;
    k_poisson_crs<<<(int)blocks, 256, 0, st>>>(m, n, row_start, col, val);
    return cudaGetLastError();
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

}  // namespace pwmgpu
