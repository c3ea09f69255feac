// Warp-tile evaluation of the per-shape culling network (tensor cores).
//
// A warp evaluates the network of one shape for up to 64 points (two per
// lane: point `lane` and `lane + 32`):
//   h0 = bf16(sin(W0 p + b0))                  CUDA cores, staged in shared memory
//   a1 = h0 W1^T + b1   (64 x 64 x 64)         mma.sync m16n8k16 BF16, FP32 accumulate
//   y  = relu(a1) . w2 + b2                    FP32, reduced across the quad
// The same function serves the contact pass and the margin calibration, so
// the culling decision at run time is exactly the calibrated function.
#pragma once
#include <cstdint>
#include "dem_device.cuh"

namespace sdg {

struct CullerLayout {  // offsets into one shape's FP32 parameter block
    static constexpr int W0 = 0, B0 = 192, W1 = 256, B1 = 256 + 4096, W2 = B1 + 64, B2 = W2 + 64;
};
static_assert(CullerLayout::B2 + 4 == CULLER_PARAMS, "culler parameter layout");

__device__ __forceinline__ uint32_t packBf16(float lo, float hi) {
    uint32_t a = __float_as_uint(lo), b = __float_as_uint(hi);
    // Round to nearest even to BF16.
    a = (a + 0x7FFFu + ((a >> 16) & 1u)) >> 16;
    b = (b + 0x7FFFu + ((b >> 16) & 1u)) >> 16;
    return (a & 0xFFFFu) | (b << 16);
}

__device__ __forceinline__ void mma16816(float c[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

constexpr int CULLER_ROW = 36;                       // u32 per staged row (32 + 4 bank padding)
constexpr int CULLER_TILE_WORDS = 64 * CULLER_ROW;   // per warp

// tile: this warp's 64 rows x CULLER_ROW u32 (BF16 pairs) of shared memory.
// Returns the prediction for the lane's two points (garbage for inactive).
__device__ __forceinline__ void cullerTile(const float* params, const uint32_t* w1, f3 p0, f3 p1, uint32_t* tile,
                                           float& y0, float& y1) {
    const uint32_t lane = threadIdx.x & 31u, g = lane >> 2, t = lane & 3u;
    // Features of the lane's two points into rows lane and lane + 32.
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        f3 q = half ? p1 : p0;
        uint32_t* row = tile + (lane + 32 * half) * CULLER_ROW;
        for (int j = 0; j < 64; j += 2) {
            const float* w = params + CullerLayout::W0 + 3 * j;
            float za = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w[0], q.x), __fmul_rn(w[1], q.y)), __fmul_rn(w[2], q.z)),
                                 params[CullerLayout::B0 + j]);
            float zb = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w[3], q.x), __fmul_rn(w[4], q.y)), __fmul_rn(w[5], q.z)),
                                 params[CullerLayout::B0 + j + 1]);
            row[j >> 1] = packBf16(__sinf(za), __sinf(zb));
        }
    }
    __syncwarp();
    float out[4][2];
#pragma unroll
    for (int mt = 0; mt < 4; ++mt) {
        float rowSum[2] = {0.f, 0.f};
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint32_t* ra = tile + (mt * 16 + g) * CULLER_ROW + kk * 8 + t;
                const uint32_t* rb = tile + (mt * 16 + g + 8) * CULLER_ROW + kk * 8 + t;
                const uint32_t* wb = w1 + (nt * 8 + g) * 32 + kk * 8 + t;
                mma16816(c, ra[0], rb[0], ra[4], rb[4], __ldg(wb), __ldg(wb + 4));
            }
            int j0 = nt * 8 + 2 * t;
            float b0 = params[CullerLayout::B1 + j0], b1 = params[CullerLayout::B1 + j0 + 1];
            float w0 = params[CullerLayout::W2 + j0], w1v = params[CullerLayout::W2 + j0 + 1];
            float h00 = fmaxf(__fadd_rn(c[0], b0), 0.f), h01 = fmaxf(__fadd_rn(c[1], b1), 0.f);
            float h10 = fmaxf(__fadd_rn(c[2], b0), 0.f), h11 = fmaxf(__fadd_rn(c[3], b1), 0.f);
            rowSum[0] = __fadd_rn(rowSum[0], __fadd_rn(__fmul_rn(h00, w0), __fmul_rn(h01, w1v)));
            rowSum[1] = __fadd_rn(rowSum[1], __fadd_rn(__fmul_rn(h10, w0), __fmul_rn(h11, w1v)));
        }
        // Reduce the four lanes of a quad (fixed butterfly order).
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            rowSum[r] = __fadd_rn(rowSum[r], __shfl_xor_sync(0xffffffffu, rowSum[r], 1));
            rowSum[r] = __fadd_rn(rowSum[r], __shfl_xor_sync(0xffffffffu, rowSum[r], 2));
            out[mt][r] = __fadd_rn(rowSum[r], params[CullerLayout::B2]);
        }
    }
    __syncwarp();
    // Point n = 16*mt + row; its value sits in lane 4*(row % 8), register row/8.
    auto fetch = [&](uint32_t n) {
        uint32_t mt = n >> 4, row = n & 15u;
        float v = 0.f;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            float a = __shfl_sync(0xffffffffu, out[m][0], (row & 7u) * 4);
            float b = __shfl_sync(0xffffffffu, out[m][1], (row & 7u) * 4);
            if (uint32_t(m) == mt) v = row < 8 ? a : b;
        }
        return v;
    };
    y0 = fetch(lane);
    y1 = fetch(lane + 32);
}

}  // namespace sdg
