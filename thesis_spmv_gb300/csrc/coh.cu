// coh.cu -- row-distributed Hilbert-blocked CO-H (SOA_Implementations/
// BlockCOH.hpp) on the GPU.
//
// Storage is the reference's: rows split into P partitions by nonzero count
// (:325-355); per partition beta = 2^min(15, 3 + ceil(log2 sqrt(max(rows_p,
// noc)))) (:119-132); blocks ordered along a Hilbert curve over the block
// grid (:103-114, :400-402); inside a block ICRS (TripletToCRS.hpp:402-452):
// 16-bit column jumps that overflow by +beta at a row change, 16-bit row
// jumps; between blocks BICRS (:404-445): int16 column jumps that overflow by
// +hb at a block-row change, int16 block-row jumps.  Built on the host here,
// bit for bit the reference's arrays.  The device copy of the column jumps
// and values starts every block on a multiple of 8 elements (zeros between
// blocks, never read as elements) so a lane loads its 8 elements with wide
// loads; the block table holds the padded offsets.
//
// The GPU kernel (k_coh_spmv) gives each partition to one warp (a partition
// owns its rows, as a thread does in BlockCOH::mv :479-510).  The warp walks
// the partition's blocks in Hilbert order (block positions decoded once at
// build time) and each block's elements in chunks of 32 x 8: lane l takes 8
// consecutive elements and decodes them with a warp prefix sum of the column
// jumps (running position S: column = S mod beta, row changes = S / beta;
// rows from a warp prefix sum of the row jumps, staged in shared memory).  A
// lane accumulates its runs of equal rows with one FMA per nonzero; a run
// that crosses lanes is summed by the lane where it starts (lane order) and
// one crossing the chunk end is carried.  A partition adds into its own rows
// of y (zeroed first; the read-modify-writes stay in L2).  The walk is
// latency-bound, so residency is what counts: 8 CTAs of 4 warps per SM
// (64 registers); an earlier shared-memory y window of 2048 rows per warp
// capped residency at 3 CTAs per SM and was 1.66x slower on the 4096^2
// stencil.  Rows are written by one lane at a time and blocks in order: no
// atomics, a fixed summation order (per row, Hilbert block order, as in the
// reference).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pwmgpu {

namespace {

constexpr int kCohK = 8;           // elements per lane per chunk (one 16-byte load of jumps)
static_assert(kCohK == 8, "a lane loads its column jumps as one uint4");
constexpr int kCohWarps = 4;       // warps per CTA
constexpr int kCohOcc = 8;         // resident CTAs per SM (64 registers): 32 warps

// BlockCOH.hpp:79-114 rowColToHilbert: index of cell (row, col) on the
// Hilbert curve over a size x size grid.
int hilbert_index(int size, int row, int col) {
    int index = 0;
    for (int s = size / 2; s > 0; s /= 2) {
        const int rr = (row & s) > 0;
        const int cr = (col & s) > 0;
        index += s * s * ((3 * cr) ^ rr);
        if (rr == 0) {
            if (cr == 1) {
                col = size - 1 - col;
                row = size - 1 - row;
            }
            std::swap(row, col);
        }
    }
    return index;
}

__global__ void __launch_bounds__(32 * kCohWarps, kCohOcc) k_coh_spmv(const int4* __restrict__ parts, int nparts,
                                                             const int4* __restrict__ blocks,
                                                             const uint16_t* __restrict__ row_jump,
                                                             const uint16_t* __restrict__ col_jump,
                                                             const double* __restrict__ data,
                                                             const double* __restrict__ x, double* __restrict__ y,
                                                             const double* nsq_in) {
    constexpr int K = kCohK;
    constexpr int CH = 32 * K;
    __shared__ int rbuf_s[kCohWarps][CH + 1];
    __shared__ int frow_s[kCohWarps][32];
    __shared__ int crow_s[kCohWarps][32];
    __shared__ double hval_s[kCohWarps][32];
    __shared__ double cval_s[kCohWarps][32];
    __shared__ int multi_s[kCohWarps][32];
    __shared__ int carry_row_s[kCohWarps];
    __shared__ double carry_s[kCohWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int* rbuf = rbuf_s[w];
    int* frow = frow_s[w];
    int* crow = crow_s[w];
    double* hval = hval_s[w];
    double* cval = cval_s[w];
    int* multi = multi_s[w];
    const int e = nsq_in ? pow2_rescale_exponent(*nsq_in, 256) : 0;
    if (lane == 0) carry_row_s[w] = -1;
    __syncwarp();
    for (int p = blockIdx.x * kCohWarps + w; p < nparts; p += gridDim.x * kCohWarps) {
        // parts[2p] = {first row, rows, block bits, first block}, parts[2p+1].x = blocks
        const int4 pa = __ldg(parts + 2 * p);
        const int nb = __ldg(&parts[2 * p + 1].x);
        const int trs = pa.x, nrows = pa.y, bits = pa.z, b0 = pa.w;
        const int beta = 1 << bits;
        double* yp = y + trs;  // the partition's rows (no other warp writes them)
        for (int r = lane; r < nrows; r += 32) yp[r] = 0.0;
        __syncwarp();
        for (int b = b0; b < b0 + nb; ++b) {
            // blocks[2b] = {block row, block col, first element, first row jump}, blocks[2b+1].x = nnz
            const int4 ba = __ldg(blocks + 2 * b);
            const int n = __ldg(&blocks[2 * b + 1].x);
            double* yb = yp + (long long)ba.x * beta;
            const double* xb = x + (long long)ba.y * beta;
            const long long eb = ba.z;
            const uint16_t* rj = row_jump + ba.w;
            int s_base = 0;          // position of the previous chunk's last element
            int ch_base = 0;         // its row-change count
            int r_base = __ldg(rj);  // its row (block-local)
            int carry_row = -1;      // run open across the chunk boundary
            double carry = 0.0;
            for (int cs = 0; cs < n; cs += CH) {
                // ---- positions: warp prefix sum of the column jumps
                const int i0 = cs + lane * K;
                int pos[K];
                double dv[K];
                int tot = 0;
                // the block starts on a multiple of 8 elements in the device
                // copy, padded past its end: one 16-byte load of jumps, four
                // of values
                uint4 cj = make_uint4(0u, 0u, 0u, 0u);
                double2 dd[K / 2];
#pragma unroll
                for (int t = 0; t < K / 2; ++t) dd[t] = make_double2(0.0, 0.0);
                if (i0 < n) {
                    cj = __ldg(reinterpret_cast<const uint4*>(col_jump + eb + i0));
#pragma unroll
                    for (int t = 0; t < K / 2; ++t) dd[t] = __ldg(reinterpret_cast<const double2*>(data + eb + i0) + t);
                }
                const uint32_t cw[4] = {cj.x, cj.y, cj.z, cj.w};
#pragma unroll
                for (int t = 0; t < K; ++t) {
                    const bool v = i0 + t < n;
                    const int jump = (int)((t & 1) ? (cw[t >> 1] >> 16) : (cw[t >> 1] & 0xFFFFu));
                    tot += v ? jump : 0;
                    dv[t] = v ? ((t & 1) ? dd[t >> 1].y : dd[t >> 1].x) : 0.0;
                    pos[t] = tot;
                }
                int incl = tot;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += u;
                }
                const int excl = s_base + incl - tot;
                const int s_last = s_base + __shfl_sync(0xffffffffu, incl, 31);
                // ---- rows reached in this chunk: R[ch_base + j] = rbuf[j]
                const int ch_last = s_last >> bits;
                const int nchg = ch_last - ch_base;
                int run = r_base;
                for (int c0 = 0; c0 < nchg; c0 += 32) {
                    const int c = c0 + lane;
                    int v = c < nchg ? (int)__ldg(rj + ch_base + 1 + c) : 0;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int u = __shfl_up_sync(0xffffffffu, v, o);
                        if (lane >= o) v += u;
                    }
                    if (c < nchg) rbuf[c + 1] = run + v;
                    run += __shfl_sync(0xffffffffu, v, 31);
                }
                if (lane == 0) rbuf[0] = r_base;
                __syncwarp();
                // ---- the lane's runs: middle runs are complete and written here
                const bool has = i0 < n;
                int first = INT_MAX, cur = INT_MAX;
                double acc = 0.0, head = 0.0;
                bool is_multi = false;
#pragma unroll
                for (int t = 0; t < K; ++t) {
                    if (i0 + t < n) {
                        const int S = excl + pos[t];
                        const int row = rbuf[(S >> bits) - ch_base];
                        const double xv = __ldg(xb + (S & (beta - 1)));
                        if (t == 0) {
                            first = cur = row;
                        } else if (row != cur) {
                            if (!is_multi) {
                                head = acc;
                                is_multi = true;
                            } else {
                                yb[cur] = yb[cur] + (e != 0 ? scale_pow2(acc, e) : acc);
                            }
                            acc = 0.0;
                            cur = row;
                        }
                        acc = fma(dv[t], xv, acc);
                    }
                }
                if (!is_multi) head = acc;
                // the run carried from the previous chunk continues in lane 0, or is complete
                if (lane == 0 && carry_row >= 0) {
                    if (has && first == carry_row) {
                        head += carry;
                        if (!is_multi) acc += carry;
                    } else {
                        yb[carry_row] = yb[carry_row] + (e != 0 ? scale_pow2(carry, e) : carry);
                    }
                }
                frow[lane] = has ? first : INT_MAX;
                crow[lane] = has ? cur : INT_MAX;
                hval[lane] = head;
                cval[lane] = acc;
                multi[lane] = is_multi ? 1 : 0;
                __syncwarp();
                if (has) {
                    const bool cont_in = lane > 0 && frow[lane] == crow[lane - 1];
                    // a first run that is not also the last run, starting here: complete
                    if (is_multi && !cont_in) yb[first] = yb[first] + (e != 0 ? scale_pow2(head, e) : head);
                    // the last run starts here (or the lane is one run not continuing): lead its chain
                    if (is_multi || !cont_in) {
                        double sum = acc;
                        int u = lane + 1;
                        bool ended = false;
                        while (u < 32 && frow[u] == cur) {
                            if (multi[u]) {
                                sum += hval[u];
                                ended = true;
                                break;
                            }
                            sum += cval[u];
                            ++u;
                        }
                        if (!ended && u == 32) {  // runs into the next chunk
                            carry_row_s[w] = cur;
                            carry_s[w] = sum;
                        } else {
                            yb[cur] = yb[cur] + (e != 0 ? scale_pow2(sum, e) : sum);
                        }
                    }
                }
                __syncwarp();
                // the carry for the next chunk: set by the chain that reached lane 31
                // (or -1); the block's last chunk flushes it below
                carry_row = carry_row_s[w];
                carry = carry_s[w];
                s_base = s_last;
                ch_base = ch_last;
                r_base = rbuf[nchg];
                __syncwarp();
                if (lane == 0) carry_row_s[w] = -1;
                __syncwarp();
            }
            if (lane == 0 && carry_row >= 0) yb[carry_row] = yb[carry_row] + (e != 0 ? scale_pow2(carry, e) : carry);
            __syncwarp();
        }
        __syncwarp();
    }
}

}  // namespace

// BlockCOH.hpp:119-132: block bits of a partition.
static int coh_bits(int rows_p, int noc) {
    const int mx = std::max(rows_p, noc);
    const int lg = (int)std::ceil(std::log2(std::sqrt((double)mx)));
    return std::min(15, 3 + lg);
}

int coh_build_host(int nor, int noc, long long nnz, const int32_t* row_start, const int32_t* col, const double* val,
                   int threads, std::vector<int32_t>& part_info, std::vector<uint16_t>& row_jump,
                   std::vector<uint16_t>& col_jump, std::vector<double>& data, std::vector<int32_t>& block_nnz,
                   std::vector<int16_t>& row_jump_block, std::vector<int16_t>& col_jump_block,
                   std::vector<int>& parts, std::vector<int>& blocks) {
    // :325-355 partition count and nonzero-balanced row split (partitions the
    // split never reaches are empty, at row nor)
    if (nor / std::max(threads, 1) < 8) threads = nor / 8;
    if (threads < 1) threads = 1;
    std::vector<int> prs((size_t)threads, nor), pn((size_t)threads, 0);
    prs[0] = 0;
    {
        int rsi = 1, pid = 0;
        long long row_sum = 0;
        const long long share = nnz / threads;
        for (int i = 0; i < nor; ++i) {
            const long long rn = row_start[i + 1] - row_start[i];
            row_sum += rn;
            if (row_sum > share && pid != threads - 1) {
                pn[(size_t)pid++] = (int)(row_sum - rn);
                prs[(size_t)rsi++] = i;
                row_sum = rn;
            }
        }
        pn[(size_t)pid] = (int)row_sum;
    }
    const int T = threads;
    // per-partition outputs, built in parallel, concatenated after
    struct PartOut {
        std::vector<uint16_t> rj, cj;
        std::vector<double> d;
        std::vector<int32_t> bn;
        std::vector<int16_t> rjb, cjb;
        std::vector<int> blk;  // 4 ints per block: block row, block col, local element start, local row-jump start
        int info[9];
    };
    std::vector<PartOut> out((size_t)T);
    auto work = [&](int p0, int p1) {
        std::vector<std::pair<uint64_t, int64_t>> keys;
        for (int p = p0; p < p1; ++p) {
            PartOut& o = out[(size_t)p];
            const int trs = prs[(size_t)p];
            const int rows_p = (p != T - 1) ? prs[(size_t)p + 1] - trs : nor - trs;
            const int bits = coh_bits(rows_p, noc);
            const int beta = 1 << bits;
            const int hb = (noc + beta - 1) / beta;
            const int vb = (rows_p + beta - 1) / beta;
            const int mx = std::max(rows_p, noc);
            const int hsize = (int)std::pow(2.0, std::ceil(std::log2((double)mx)));
            const int64_t e0 = trs < nor ? row_start[trs] : nnz;
            const int64_t e1 = (trs + rows_p) <= nor ? row_start[trs + rows_p] : nnz;
            const int np = (int)(e1 - e0);
            keys.clear();
            for (int r = trs; r < trs + rows_p; ++r)
                for (int64_t k = row_start[r]; k < row_start[r + 1]; ++k) {
                    const uint32_t br = (uint32_t)(r - trs) / (uint32_t)beta, bc = (uint32_t)col[k] / (uint32_t)beta;
                    const uint64_t h = (uint32_t)hilbert_index(hsize / beta, (int)br, (int)bc);
                    const uint32_t lr = (uint32_t)(r - trs) % (uint32_t)beta, lc = (uint32_t)col[k] % (uint32_t)beta;
                    keys.emplace_back((h << 32) | ((uint64_t)lr << 16) | lc, k);
                }
            std::sort(keys.begin(), keys.end());
            std::vector<int> rowof((size_t)np);
            for (int r = trs; r < trs + rows_p; ++r)
                for (int64_t k = row_start[r]; k < row_start[r + 1]; ++k) rowof[(size_t)(k - e0)] = r;
            o.cj.resize((size_t)np);
            o.d.resize((size_t)np);
            int16_t old_br = 0, old_bc = 0;
            int i = 0;
            while (i < np) {
                const int64_t k0 = keys[(size_t)i].second;
                const int br = (rowof[(size_t)(k0 - e0)] - trs) / beta, bc = col[k0] / beta;
                int j = i;
                while (j < np) {
                    const int64_t kj = keys[(size_t)j].second;
                    if ((rowof[(size_t)(kj - e0)] - trs) / beta != br || col[kj] / beta != bc) break;
                    ++j;
                }
                const int16_t nbr = (int16_t)br, nbc = (int16_t)bc;
                if (o.bn.empty()) {
                    o.rjb.push_back(nbr);
                    o.cjb.push_back(nbc);
                } else if (nbr == old_br) {
                    o.cjb.push_back((int16_t)(nbc - old_bc));
                } else {
                    o.rjb.push_back((int16_t)(nbr - old_br));
                    o.cjb.push_back((int16_t)(nbc - old_bc + hb));
                }
                old_br = nbr;
                old_bc = nbc;
                o.blk.insert(o.blk.end(), {br, bc, i, (int)o.rj.size()});
                o.bn.push_back(j - i);
                uint16_t prev_r = 0, prev_c = 0;
                for (int q = i; q < j; ++q) {
                    const int64_t k = keys[(size_t)q].second;
                    const uint16_t lr = (uint16_t)((rowof[(size_t)(k - e0)] - trs) % beta);
                    const uint16_t lc = (uint16_t)(col[k] % beta);
                    if (q == i) {
                        o.rj.push_back(lr);
                        o.cj[(size_t)q] = lc;
                    } else if (lr != prev_r) {
                        o.cj[(size_t)q] = (uint16_t)((lc + beta) - prev_c);
                        o.rj.push_back((uint16_t)(lr - prev_r));
                    } else {
                        o.cj[(size_t)q] = (uint16_t)(lc - prev_c);
                    }
                    o.d[(size_t)q] = val[k];
                    prev_r = lr;
                    prev_c = lc;
                }
                i = j;
            }
            const int info[9] = {trs, beta, bits, hb, vb, np, (int)o.bn.size(), (int)o.rj.size(), (int)o.rjb.size()};
            std::memcpy(o.info, info, sizeof info);
        }
    };
    const int nt = std::max(1, std::min(T, (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, (int)((long long)T * t / nt), (int)((long long)T * (t + 1) / nt));
    for (auto& t : th) t.join();
    part_info.assign((size_t)9 * T, 0);
    row_jump.clear();
    col_jump.clear();
    data.clear();
    block_nnz.clear();
    row_jump_block.clear();
    col_jump_block.clear();
    parts.assign((size_t)8 * T, 0);
    blocks.clear();
    long long eoff = 0, rjoff = 0, boff = 0;
    for (int p = 0; p < T; ++p) {
        PartOut& o = out[(size_t)p];
        std::memcpy(&part_info[(size_t)9 * p], o.info, sizeof o.info);
        const int rows_p = (p != T - 1) ? prs[(size_t)p + 1] - prs[(size_t)p] : nor - prs[(size_t)p];
        int* pp = &parts[(size_t)8 * p];
        pp[0] = prs[(size_t)p];
        pp[1] = rows_p;
        pp[2] = o.info[2];
        pp[3] = (int)boff;
        pp[4] = (int)o.bn.size();
        for (size_t b = 0; b < o.bn.size(); ++b) {
            blocks.insert(blocks.end(), {o.blk[4 * b], o.blk[4 * b + 1], (int)(eoff + o.blk[4 * b + 2]),
                                         (int)(rjoff + o.blk[4 * b + 3]), o.bn[b], 0, 0, 0});
        }
        row_jump.insert(row_jump.end(), o.rj.begin(), o.rj.end());
        col_jump.insert(col_jump.end(), o.cj.begin(), o.cj.end());
        data.insert(data.end(), o.d.begin(), o.d.end());
        block_nnz.insert(block_nnz.end(), o.bn.begin(), o.bn.end());
        row_jump_block.insert(row_jump_block.end(), o.rjb.begin(), o.rjb.end());
        col_jump_block.insert(col_jump_block.end(), o.cjb.begin(), o.cjb.end());
        eoff += (long long)o.cj.size();
        rjoff += (long long)o.rj.size();
        boff += (long long)o.bn.size();
    }
    return T;
}

cudaError_t launch_coh_spmv(const int* parts, int nparts, const int* blocks, const uint16_t* row_jump,
                            const uint16_t* col_jump, const double* data, const double* x, double* y,
                            const double* nsq_in, int sm_count, cudaStream_t st) {
    if (nparts <= 0) return cudaSuccess;
    long long grid = (nparts + kCohWarps - 1) / kCohWarps;
    if (grid > (long long)sm_count * kCohOcc) grid = (long long)sm_count * kCohOcc;
    k_coh_spmv<<<(int)grid, 32 * kCohWarps, 0, st>>>(reinterpret_cast<const int4*>(parts), nparts,
                                                    reinterpret_cast<const int4*>(blocks), row_jump, col_jump, data,
                                                    x, y, nsq_in);
    return cudaGetLastError();
}

}  // namespace pwmgpu
