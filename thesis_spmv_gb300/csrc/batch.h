// batch.h -- device tables of the batched power iterations (the serving
// loop's rounds).  Shared by batch.cu (kernels) and service.cpp (host).
//
// A class table lists the live solves ("slots") that iterate with one value
// / vector type and one layout (merge path, or SELL-32 slices for the FP32 /
// BF16 iterations of stencil and banded matrices: then "sub-tiles" below are
// 32-row slices and there is no fix-up).  The sub-tiles of all its slots form one list: slot j owns
// global sub-tiles [tile0_j, tile0_j + nsub_j), cut from its own merge path,
// so the list is the merge path of the block-diagonal matrix of all slots,
// cut at the matrix boundaries.  One launch runs an SpMV step of every slot;
// sums over a slot run in a fixed order over its own sub-tiles, so a solve
// gives the same bits alone and in any mix.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pwmgpu {

constexpr int kFixTiles = 256;    // sub-tiles per fix-up chunk (one per thread: a fix-up is latency-bound)
constexpr int kSellGroup = 16;    // SELL-32 classes: slices per group of the in-kernel norm
constexpr int kRowChunk = 16384;  // rows per norm / residual chunk (a multiple of 4)

struct BatchSlot {
    const int32_t* row_start;
    const int32_t* colp;
    const void* valp;
    const int4* rec;
    const uint16_t* masks;
    const int2* subc;
    void* X;  // v_k for even k
    void* Y;  // v_k for odd k
    void* carries;
    const int32_t* soff;    // SELL-32 classes: slice offsets (nsub = slices, tile0 = first global slice)
    const uint16_t* col16;  // SELL-32 classes: 16-bit column offsets (values in valp)
    int nor, nsub;
    int tile0;       // first global sub-tile
    int fix0, nfix;  // fix-up chunks [fix0, fix0 + nfix) (kFixTiles sub-tiles each); SELL-32
                     // classes: slice groups (kSellGroup slices each) of the norm
    int row0, nrow;  // row chunks [row0, row0 + nrow) (kRowChunk rows each)
    int state;       // index into the state array
    int pad;
};

// Per-solve iteration state, advanced on the device.
struct SlotState {
    int k;              // steps done in the current phase: v_k is the newest iterate
    int exact_res;      // set by the host: the round's residual pass must run over the rows
    double nsq;         // ||v_k||^2 (k >= 1)
    double nsq_prev;    // ||v_{k-1}||^2
    double dot;         // v_{k-1} . v_k, from the last step of a round
    double lambda;      // Rayleigh quotient of u = v_{k-1} / ||v_{k-1}||
    double res2;        // ||A u - lambda u||^2 * ||v_{k-1}||^2
    unsigned int norm_count, res_count;  // last-CTA counters (zero between kernels)
    // Key steps (a round's steps before its last two): only the exponent of
    // the next exact 2^e rescale needs v_k's size, so those steps track the
    // largest magnitude key of the stored rows instead of ||v||^2.
    unsigned int mx;       // largest magnitude key of v_k (when keyed)
    unsigned int mx_next;  // atomic-max target of a key step (zero between steps)
    int keyed;             // v_k came from a key step: its rescale uses mx, nsq is stale
    int pad;
};

struct BatchTable {
    int nslots, ntiles, nfix, nrow;
    const BatchSlot* slots;
    SlotState* states;
    int* tile_slot;     // slot of each global sub-tile
    double* row_part;   // 2 per row chunk: sum of squares, dot
    double* res_part;   // 1 per row chunk
    double* grp_part;   // SELL-32 classes: 1 per slice group (sum of squares)
    int* status;
};

}  // namespace pwmgpu
