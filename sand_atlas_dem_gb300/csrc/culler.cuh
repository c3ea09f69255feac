// Block-tile evaluation of the per-shape culling networks on the 5th-generation
// tensor cores (tcgen05, accumulator in tensor memory).
//
// A CTA of 128 threads evaluates 128 points (one row per thread) at a time:
//   h0 = bf16(sin(W0 p + b0))          CUDA cores, each row with its own shape's
//                                      W0, b0, written to shared memory as the
//                                      MMA's A operand (128 x 64 BF16)
//   a1 = h0 W1^T                       tcgen05.mma kind::f16, M = 128, N = 64,
//                                      K = 64 (four K = 16 steps), BF16 x BF16,
//                                      FP32 accumulator in 64 TMEM columns;
//                                      B = the shape's W1 (64 x 64 BF16)
//   y  = b2 + sum_n relu(a1[n] + b1[n]) w2[n]   FP32, per row in n order, from
//                                      the row's accumulators (tcgen05.ld)
// Rows are sorted by shape; a tile holding several shapes runs one MMA per
// shape (same A, that shape's B) and each row keeps its own shape's result.
// One thread issues the MMAs; their completion arrives on an mbarrier that
// every thread waits on (bounded).  Operands use the canonical K-major layout
// without swizzle: 8-row x 16-byte core matrices, 128 bytes apart along K
// (leading byte offset) and 1024 bytes apart along M/N (stride byte offset).
// The same block function serves the contact pass and the margin
// calibration, so the culling decision at run time is exactly the calibrated
// function.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include "dem_device.cuh"

namespace sdg {

struct CullerLayout {  // offsets into one shape's FP32 parameter block
    static constexpr int W0 = 0, B0 = 192, W1 = 256, B1 = 256 + 4096, W2 = B1 + 64, B2 = W2 + 64;
};
static_assert(CullerLayout::B2 + 4 == CULLER_PARAMS, "culler parameter layout");

constexpr uint32_t CULLER_ROWS = 128;     // rows (points) per tile: the MMA's M
// Margins: per shape one calibrated margin for the whole shape, then one per
// cell of an 8^3 grid over the shape's root box (the largest prediction at
// inside calibration points in the cell and its neighbours).
constexpr uint32_t CULLER_CELLS = 8;
constexpr uint32_t CULLER_MARGINS = 1 + CULLER_CELLS * CULLER_CELLS * CULLER_CELLS;
// The cell of a point of a shape's frame (clamped to the grid).
__device__ __forceinline__ uint32_t cullerCell(float4 low, float4 high, f3 p) {
    float q[3] = {__fdiv_rn(__fsub_rn(p.x, low.x), __fsub_rn(high.x, low.x)),
                  __fdiv_rn(__fsub_rn(p.y, low.y), __fsub_rn(high.y, low.y)),
                  __fdiv_rn(__fsub_rn(p.z, low.z), __fsub_rn(high.z, low.z))};
    uint32_t k[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float f = floorf(__fmul_rn(q[a], float(CULLER_CELLS)));
        k[a] = f <= 0.0f ? 0u : (f >= float(CULLER_CELLS - 1) ? CULLER_CELLS - 1 : uint32_t(f));
    }
    return (k[2] * CULLER_CELLS + k[1]) * CULLER_CELLS + k[0];
}
constexpr uint32_t CULLER_COLUMNS = 64;   // TMEM columns (FP32 accumulators, N)

struct CullerShared {
    alignas(1024) unsigned char a[CULLER_ROWS * 128];  // 128 x 64 BF16, K-major canonical
    alignas(1024) unsigned char b[64 * 128];           // 64 x 64 BF16 (W1 of one shape)
    alignas(8) uint64_t barrier;
    uint32_t tmem;                                     // TMEM address of the accumulators
    uint32_t nextShape[2];                             // the next shape to run (two slots)
    uint32_t failed;
};

__device__ __forceinline__ uint32_t cullerSmem(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// Byte offset of (row, 8-element K group) in the canonical layout.
__device__ __forceinline__ uint32_t cullerTileOffset(uint32_t row, uint32_t group) {
    return (row >> 3) * 1024u + group * 128u + (row & 7u) * 16u;
}
// Shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t cullerDescriptor(uint32_t address) {
    return uint64_t((address >> 4) & 0x3FFFu) | (uint64_t(128u >> 4) << 16) | (uint64_t(1024u >> 4) << 32) |
           (uint64_t(1) << 46);
}
// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 64, M = 128.
constexpr uint32_t CULLER_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ bool cullerWait(uint32_t bar, uint32_t parity) {
    for (uint32_t k = 0; k < (1u << 22); ++k) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Set-up by the whole CTA (128 threads): TMEM columns and the mbarrier.
__device__ __forceinline__ void cullerBegin(CullerShared& sh) {
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(cullerSmem(&sh.tmem)),
                     "r"(CULLER_COLUMNS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cullerSmem(&sh.barrier)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sh.failed = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Tear-down: after a wait that gave up, wait once more (bounded) for the MMA
// in flight, then free the TMEM columns.
__device__ __forceinline__ void cullerEnd(CullerShared& sh, uint32_t phase) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (sh.failed && threadIdx.x == 0) cullerWait(cullerSmem(&sh.barrier), phase ^ 1u);
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(sh.tmem), "r"(CULLER_COLUMNS)
                     : "memory");
}

// One tile: thread i evaluates row i (point p of shape `shape`, EMPTY for no
// row) and returns its prediction.  `phase` is the mbarrier parity, kept by
// the caller across tiles.  Returns false (every thread) if an MMA wait gave
// up; the predictions are then meaningless.
__device__ __forceinline__ bool cullerTile(CullerShared& sh, const float* params, const uint32_t* w1, uint32_t shape,
                                           f3 p, uint32_t& phase, float& y) {
    const uint32_t row = threadIdx.x, warp = row >> 5;
    __syncthreads();  // every thread is done with the previous tile's A, B and slots
    // Features of the row (zeros for no row) into A.
    {
        const float* q = params + size_t(shape == EMPTY ? 0u : shape) * CULLER_PARAMS;
#pragma unroll 1
        for (uint32_t group = 0; group < 8; ++group) {
            uint32_t packed[4];
#pragma unroll
            for (uint32_t e = 0; e < 4; ++e) {
                float v[2];
#pragma unroll
                for (uint32_t h = 0; h < 2; ++h) {
                    uint32_t j = group * 8 + 2 * e + h;
                    const float* w = q + CullerLayout::W0 + 3 * j;
                    float z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(__ldg(w), p.x), __fmul_rn(__ldg(w + 1), p.y)),
                                                  __fmul_rn(__ldg(w + 2), p.z)),
                                        __ldg(q + CullerLayout::B0 + j));
                    v[h] = shape == EMPTY ? 0.0f : __sinf(z);
                }
                __nv_bfloat162 pair = __floats2bfloat162_rn(v[0], v[1]);  // round to nearest even
                packed[e] = *reinterpret_cast<uint32_t*>(&pair);
            }
            *reinterpret_cast<uint4*>(sh.a + cullerTileOffset(row, group)) =
                make_uint4(packed[0], packed[1], packed[2], packed[3]);
        }
    }
    // The shapes among the rows, smallest first (rows are sorted, EMPTY
    // last): each round's minimum over the rows above the current shape goes
    // to one of two slots; a slot is reset a barrier after its last read.
    if (row == 0) sh.nextShape[0] = sh.nextShape[1] = EMPTY;
    __syncthreads();
    if (shape != EMPTY) atomicMin(&sh.nextShape[0], shape);
    __syncthreads();
    uint32_t current = sh.nextShape[0];
    bool ok = true;
    y = 0.0f;
    for (uint32_t round = 0; current != EMPTY; ++round) {
        // B: the shape's W1 (row n, K-major; 64 bytes a thread).
        {
            const uint4* from = reinterpret_cast<const uint4*>(w1 + size_t(current) * 2048);
            uint32_t n = row >> 1, half = row & 1u;
#pragma unroll
            for (uint32_t g = 0; g < 4; ++g) {
                uint32_t group = half * 4 + g;
                *reinterpret_cast<uint4*>(sh.b + cullerTileOffset(n, group)) = __ldg(from + n * 8 + group);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // This round's candidates go to slot (round + 1) & 1; slot round & 1,
        // last read before the barrier above, serves the round after.
        if (row == 0) {
            sh.nextShape[round & 1u] = EMPTY;
            uint32_t a = cullerSmem(sh.a), b = cullerSmem(sh.b);
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k) {
                uint64_t da = cullerDescriptor(a + 256u * k), db = cullerDescriptor(b + 256u * k);
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(sh.tmem),
                    "l"(da), "l"(db), "r"(CULLER_IDESC), "r"(k));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             cullerSmem(&sh.barrier))
                         : "memory");
        }
        if (!cullerWait(cullerSmem(&sh.barrier), phase)) sh.failed = 1;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        uint32_t acc[64];
        uint32_t address = sh.tmem + ((warp * 32u) << 16);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
            "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,"
            "%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
            : "=r"(acc[0]), "=r"(acc[1]), "=r"(acc[2]), "=r"(acc[3]), "=r"(acc[4]), "=r"(acc[5]), "=r"(acc[6]),
              "=r"(acc[7]), "=r"(acc[8]), "=r"(acc[9]), "=r"(acc[10]), "=r"(acc[11]), "=r"(acc[12]), "=r"(acc[13]),
              "=r"(acc[14]), "=r"(acc[15]), "=r"(acc[16]), "=r"(acc[17]), "=r"(acc[18]), "=r"(acc[19]),
              "=r"(acc[20]), "=r"(acc[21]), "=r"(acc[22]), "=r"(acc[23]), "=r"(acc[24]), "=r"(acc[25]),
              "=r"(acc[26]), "=r"(acc[27]), "=r"(acc[28]), "=r"(acc[29]), "=r"(acc[30]), "=r"(acc[31]),
              "=r"(acc[32]), "=r"(acc[33]), "=r"(acc[34]), "=r"(acc[35]), "=r"(acc[36]), "=r"(acc[37]),
              "=r"(acc[38]), "=r"(acc[39]), "=r"(acc[40]), "=r"(acc[41]), "=r"(acc[42]), "=r"(acc[43]),
              "=r"(acc[44]), "=r"(acc[45]), "=r"(acc[46]), "=r"(acc[47]), "=r"(acc[48]), "=r"(acc[49]),
              "=r"(acc[50]), "=r"(acc[51]), "=r"(acc[52]), "=r"(acc[53]), "=r"(acc[54]), "=r"(acc[55]),
              "=r"(acc[56]), "=r"(acc[57]), "=r"(acc[58]), "=r"(acc[59]), "=r"(acc[60]), "=r"(acc[61]),
              "=r"(acc[62]), "=r"(acc[63])
            : "r"(address));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (shape == current) {
            const float* q = params + size_t(current) * CULLER_PARAMS;
            float out = __ldg(q + CullerLayout::B2);
#pragma unroll
            for (uint32_t n = 0; n < 64; ++n) {
                float h = fmaxf(__fadd_rn(__uint_as_float(acc[n]), __ldg(q + CullerLayout::B1 + n)), 0.0f);
                out = __fadd_rn(out, __fmul_rn(h, __ldg(q + CullerLayout::W2 + n)));
            }
            y = out;
        } else if (shape != EMPTY && shape > current) {
            atomicMin(&sh.nextShape[(round + 1) & 1u], shape);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        ok = ok && !sh.failed;
        current = sh.nextShape[(round + 1) & 1u];
    }
    return ok;
}

}  // namespace sdg
