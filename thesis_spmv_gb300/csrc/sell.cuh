// sell.cuh -- the SELL-32 row routine shared by the single-matrix kernel
// (sell.cu) and the batched service's kernel (batch.cu).
//
// Element j of row 32 s + l of a slice at element offset o sits at
// o + 32 j + l; its column is cb + offset with cb = 32 s - 32768 and a
// 16-bit offset, kSellPad marking the padding after a row's last element.
#pragma once
#include <cstdint>

#include "common.cuh"

namespace pwmgpu {

constexpr int kSellJ = 8;  // elements per lane whose loads are issued together
constexpr uint16_t kSellPad = 0xFFFF;

// Rows of two slices at once, one per lane (widths wa, wb; wb = 0 for none):
// each row's products summed left to right in CRS order.  For J
// elements of both rows the column and value loads are issued together,
// then the x gathers, then the FMAs.  cp*, vp*: the lane's first element.
// The columns and values are read once per step: streaming loads
// (ld.global.cs, evict-first in L1 and L2), so the stream does not push the
// x rows a stencil's slices read again (rows r - m and r + m) out of L2.
template <typename VT, int J = kSellJ>
__device__ __forceinline__ void sell_rows2(const uint16_t* __restrict__ cpa, const VT* __restrict__ vpa,
                                           const float* __restrict__ xa, int cba, int wa,
                                           const uint16_t* __restrict__ cpb, const VT* __restrict__ vpb,
                                           const float* __restrict__ xb, int cbb, int wb, float& ya, float& yb) {
    float acca = 0.0f, accb = 0.0f;
    const int w = wa > wb ? wa : wb;
    for (int j = 0; j < w; j += J) {
        uint16_t ca[J], cb[J];
        float va[J], vb[J], ga[J], gb[J];
#pragma unroll
        for (int u = 0; u < J; ++u) {
            ca[u] = j + u < wa ? __ldcs(cpa + 32 * (j + u)) : kSellPad;
            cb[u] = j + u < wb ? __ldcs(cpb + 32 * (j + u)) : kSellPad;
            va[u] = j + u < wa ? to_f32(__ldcs(vpa + 32 * (j + u))) : 0.0f;
            vb[u] = j + u < wb ? to_f32(__ldcs(vpb + 32 * (j + u))) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < J; ++u) {
            ga[u] = ca[u] != kSellPad ? __ldg(xa + cba + (int)ca[u]) : 0.0f;
            gb[u] = cb[u] != kSellPad ? __ldg(xb + cbb + (int)cb[u]) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < J; ++u) {
            if (ca[u] != kSellPad) acca = fmaf(va[u], ga[u], acca);
            if (cb[u] != kSellPad) accb = fmaf(vb[u], gb[u], accb);
        }
    }
    ya = acca;
    yb = accb;
}

}  // namespace pwmgpu
