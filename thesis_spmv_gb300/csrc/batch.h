// batch.h -- device tables of the batched power iterations (the serving
// loop's rounds).  Shared by batch.cu (kernels) and service.cpp (host).
//
// A class table lists the live solves ("slots") that iterate with one value
// / vector type.  The sub-tiles of all its slots form one list: slot j owns
// global sub-tiles [tile0_j, tile0_j + nsub_j), cut from its own merge path,
// so the list is the merge path of the block-diagonal matrix of all slots,
// cut at the matrix boundaries.  One launch runs an SpMV step of every slot;
// sums over a slot run in a fixed order over its own sub-tiles, so a solve
// gives the same bits alone and in any mix.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pwmgpu {

constexpr int kRedTiles = 2048;   // sub-tiles per reduction chunk
constexpr int kResRows = 32768;   // rows per residual chunk

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
    int nor, nsub;
    int tile0;       // first global sub-tile
    int red0, nred;  // reduction chunks [red0, red0 + nred)
    int res0, nres;  // residual chunks [res0, res0 + nres)
    int state;       // index into the state array
    int pad;
};

// Per-solve iteration state, advanced on the device.
struct SlotState {
    int k;              // steps done in the current phase: v_k is the newest iterate
    int pad0;
    double nsq;         // ||v_k||^2 (k >= 1)
    double nsq_prev;    // ||v_{k-1}||^2
    double dot;         // v_{k-1} . v_k, from the last step of a round
    double lambda;      // Rayleigh quotient of u = v_{k-1} / ||v_{k-1}||
    double res2;        // ||A u - lambda u||^2 * ||v_{k-1}||^2
    unsigned int red_count, res_count;  // last-CTA counters (zero between kernels)
};

struct BatchTable {
    int nslots, ntiles, nred, nres;
    const BatchSlot* slots;
    SlotState* states;
    double* tile_part;  // 2 per global sub-tile: sum of squares, dot
    double* red_part;   // 2 per reduction chunk
    double* res_part;   // 1 per residual chunk
    int* status;
};

}  // namespace pwmgpu
