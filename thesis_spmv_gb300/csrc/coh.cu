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
// bit for bit the reference's arrays (pwmgpu_get_coh returns them).
//
// The device executes the same blocks as tiles of the tile kernel
// (k_csb_spmv, csb.cu): rows are cut into windows of S rows (S <= 1024, a
// y window in shared memory per CTA), each CO-H block into the tiles its
// elements form in a window and an S-column x window; a window's tiles are
// taken partition by partition in the partition's Hilbert block order, a
// block's tiles by column window.  A tile of at least kTileDenseUnit
// elements stages its x window in shared memory with a TMA bulk copy and is
// read row-major (one FMA per element inside a lane's rows); the window's
// sparse tiles -- the blocks of a random matrix hold a handful of elements --
// are merged into one row-major unit that gathers x through L1 / L2.  The
// first GPU kernel walked a partition's blocks with one warp, decoding the
// jumps with warp prefix sums and adding into y in global memory: a chain of
// dependent loads per 256-element chunk that was latency-bound at 0.66 ms on
// the 4096^2 Poisson matrix (2021 GB/s of CRS bytes) and 5.7 ms on the
// 4.19M-row irregular matrix (156 GB/s).  Per row, the tile kernel adds the
// merged sparse unit first, then the dense tiles in the window's order; the
// per-row error bound holds for any order.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <thread>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pwmgpu {

namespace {

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

// The CO-H matrix as tile-kernel units (see the header comment).
void coh_tile_units(int nor, int noc, long long nnz, const int32_t* row_start, const int32_t* col, const double* val,
                    const std::vector<int>& parts, int S, std::vector<uint32_t>& ind, std::vector<double>& data,
                    std::vector<int>& win_ptr, std::vector<int>& unit_data) {
    struct Tile {
        int lo, hi, c0;
    };
    const int T = (int)(parts.size() / 8);
    const int nwin = (nor + S - 1) / S;
    ind.resize((size_t)nnz);
    data.resize((size_t)nnz);
    std::vector<std::vector<Tile>> tiles((size_t)nwin);
    std::vector<int> first((size_t)T), bits((size_t)T), hgrid((size_t)T);
    for (int p = 0; p < T; ++p) {
        first[(size_t)p] = parts[(size_t)8 * p];
        bits[(size_t)p] = parts[(size_t)8 * p + 2];
        const int rows_p = parts[(size_t)8 * p + 1];
        const int mx = std::max(std::max(rows_p, noc), 1);
        const int hsize = (int)std::pow(2.0, std::ceil(std::log2((double)mx)));  // as coh_build_host
        hgrid[(size_t)p] = std::max(hsize >> bits[(size_t)p], 1);
    }
    auto work = [&](int w0, int w1) {
        // (partition << 40 | Hilbert index of the block, column window,
        //  local row << 32 | column, CRS position)
        std::vector<std::tuple<uint64_t, uint32_t, uint64_t, int64_t>> key;
        for (int w = w0; w < w1; ++w) {
            const int r0 = w * S, r1 = std::min(nor, r0 + S);
            const int64_t e0 = row_start[r0];
            key.clear();
            int p = (int)(std::upper_bound(first.begin(), first.end(), r0) - first.begin()) - 1;
            for (int r = r0; r < r1; ++r) {
                while (p + 1 < T && first[(size_t)p + 1] <= r) ++p;
                const int b = bits[(size_t)p];
                const uint32_t br = (uint32_t)(r - first[(size_t)p]) >> b;
                for (int64_t k = row_start[r]; k < row_start[r + 1]; ++k) {
                    const uint32_t bc = (uint32_t)col[k] >> b;
                    const uint64_t h = (uint64_t)(uint32_t)hilbert_index(hgrid[(size_t)p], (int)br, (int)bc);
                    key.emplace_back(((uint64_t)p << 40) | h, (uint32_t)col[k] / (uint32_t)S,
                                     ((uint64_t)(r - r0) << 32) | (uint64_t)(uint32_t)col[k], k);
                }
            }
            std::sort(key.begin(), key.end());
            std::vector<Tile>& tl = tiles[(size_t)w];
            uint64_t cur_blk = ~0ull;
            uint32_t cur_c = ~0u;
            for (size_t q = 0; q < key.size(); ++q) {
                const int64_t k = std::get<3>(key[q]);
                const uint32_t cwin = std::get<1>(key[q]);
                const uint32_t lr = (uint32_t)(std::get<2>(key[q]) >> 32);
                const int dst = (int)(e0 + (int64_t)q);
                const int c0 = (int)cwin * S;
                ind[(size_t)dst] = (lr << 16) | (uint32_t)(col[k] - c0);
                data[(size_t)dst] = val[k];
                if (std::get<0>(key[q]) != cur_blk || cwin != cur_c) {
                    tl.push_back(Tile{dst, dst + 1, c0});
                    cur_blk = std::get<0>(key[q]);
                    cur_c = cwin;
                } else {
                    tl.back().hi = dst + 1;
                }
            }
        }
    };
    const int nt = std::max(1, std::min<int>(nwin, (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back(work, (int)((long long)nwin * t / nt), (int)((long long)nwin * (t + 1) / nt));
    for (auto& t : th) t.join();
    // per window: sparse tiles first, then dense ones (win_ptr holds both starts)
    win_ptr.assign(2 * (size_t)nwin + 1, 0);
    unit_data.clear();
    int o = 0;
    for (int w = 0; w < nwin; ++w) {
        win_ptr[2 * (size_t)w] = o;
        for (int dense = 0; dense < 2; ++dense) {
            if (dense) win_ptr[2 * (size_t)w + 1] = o;
            for (const Tile& u : tiles[(size_t)w]) {
                if ((u.hi - u.lo >= kTileDenseUnit) != (dense == 1)) continue;
                unit_data.insert(unit_data.end(), {u.lo, u.hi, u.c0, 0});
                ++o;
            }
        }
    }
    win_ptr[2 * (size_t)nwin] = o;
}

}  // namespace pwmgpu
