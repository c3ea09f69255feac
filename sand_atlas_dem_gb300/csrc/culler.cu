// Learned conservative culler: one small signed-distance network per shape.
//
// Network (per shape s, coordinates in the shape frame, normalized units):
//   h0 = sin(W0 p + b0)            64 Fourier features of the 3 coordinates
//   h1 = relu(W1 h0 + b1)          64 -> 64
//   y  = w2 . h1 + b2              predicted signed distance / shell width
// Training data: points uniform in the shell |phi| <= shell around each
// surface, labelled by the exact BVH distance (meshDistance, the same
// function the contact query uses).  Training: full-batch-per-step mini
// batches, mean squared error, Adam; FP32 master weights, every reduction in
// a fixed order (bit-reproducible).  The culler never produces a force: a node
// is skipped only when y exceeds a per-shape margin calibrated to be larger
// than y at every sampled point inside the shape; every other node goes to
// the exact query.
//
// All kernels are batched over shapes (blockIdx.y = shape).
#include <algorithm>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "culler.cuh"
#include "dem_device.cuh"
#include "launch.h"

namespace sdg {

constexpr int H = 64;  // features and hidden width

struct Net {  // per-shape parameter block, FP32, offsets in floats
    static constexpr int W0 = 0, B0 = W0 + 3 * H, W1 = B0 + H, B1 = W1 + H * H, W2 = B1 + H, B2 = W2 + H,
                         SIZE = B2 + 4;  // padded to 16 bytes
};

// Counter-based uniform in [0,1): a 32-bit mix of (seed, shape, index, axis).
__device__ __forceinline__ float uniformHash(uint32_t seed, uint32_t shape, uint32_t index, uint32_t axis) {
    uint32_t h = seed * 0x9E3779B9u ^ (shape * 0x85EBCA6Bu) ^ (index * 0xC2B2AE35u) ^ (axis * 0x27D4EB2Fu);
    h ^= h >> 16; h *= 0x7FEB352Du; h ^= h >> 15; h *= 0x846CA68Bu; h ^= h >> 16;
    return (h >> 8) * (1.0f / 16777216.0f);
}

// Candidate points uniform in the shape's root box grown by `shell`;
// out[k] = (x, y, z, phi), accept[k] = |phi| <= shell (or phi <= 0 when
// inside_only).  phi is the exact signed distance of the contact query.
__global__ void k_shellCandidates(const __grid_constant__ Params P, uint32_t count, uint32_t seed, float shell,
                                  uint32_t insideOnly, float4* out, uint32_t* accept) {
    const Res& r = P.r;
    uint32_t s = blockIdx.y;
    uint32_t root = r.meshRoots[s].x;
    // Inside points come from the shape's own box; shell points from the box
    // grown by the shell width.
    float pad = insideOnly ? 0.0f : shell;
    f3 lo = xyz(r.meshMin[root]) - mk(pad, pad, pad), hi = xyz(r.meshMax[root]) + mk(pad, pad, pad);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        f3 u = mk(uniformHash(seed, s, k, 0), uniformHash(seed, s, k, 1), uniformHash(seed, s, k, 2));
        f3 p = lo + u * (hi - lo);
        float4 f = meshDistance(r, s, p, false);
        size_t at = size_t(s) * count + k;
        out[at] = w4(p, f.w);
        accept[at] = insideOnly ? (f.w <= 0.0f) : (fabsf(f.w) <= shell);
    }
}
// Points on each shape's surface (uniform triangle, uniform barycentric
// point), label 0: the inside boundary, where a network's largest prediction
// over the inside of a shape is usually reached.  Shape s owns triangles
// [triStart[s], triStart[s + 1]) of the packed triangle array.
__global__ void k_surfacePoints(const float4* triangles, const uint32_t* triStart, uint32_t count, uint32_t seed,
                                float4* out) {
    uint32_t s = blockIdx.y;
    uint32_t first = triStart[s], n = triStart[s + 1] - first;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        uint32_t t = first + min(uint32_t(uniformHash(seed, s, k, 0) * float(n)), n - 1);
        float u = uniformHash(seed, s, k, 1), v = uniformHash(seed, s, k, 2);
        if (u + v > 1.0f) { u = 1.0f - u; v = 1.0f - v; }
        f3 a = xyz(triangles[3 * t]), b = xyz(triangles[3 * t + 1]), c = xyz(triangles[3 * t + 2]);
        out[size_t(s) * count + k] = w4(a + (b - a) * u + (c - a) * v, 0.0f);
    }
}
// Stream compaction of accepted candidates in index order (exclusive scan
// already in `offsets`), per shape, capped at `capacity` points.
__global__ void k_compact(const float4* in, const uint32_t* accept, const uint32_t* offsets, uint32_t count,
                          uint32_t capacity, float4* out) {
    uint32_t s = blockIdx.y;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        size_t at = size_t(s) * count + k;
        if (!accept[at]) continue;
        uint32_t slot = offsets[at] - offsets[size_t(s) * count];
        if (slot < capacity) out[size_t(s) * capacity + slot] = in[at];
    }
}

// ---------------------------------------------------------------- network
// Forward and backward of a batch: one thread per point, parameters of the
// shape in shared memory, activations in registers.  Per-point gradient
// contributions are written out; the parameter reductions are separate
// fixed-order kernels.
struct TrainArgs {
    const float* params;       // shapes x Net::SIZE
    const float4* points;      // shapes x pointsPerShape (x, y, z, phi)
    uint32_t pointsPerShape, batch, step, seed;
    float scale;               // target = phi / scale
    float over;                // weight of an over-prediction inside the shape (target <= 0)
    float* dA1;                // shapes x batch x H   (dL/da1)
    float* H0;                 // shapes x batch x H
    float* dZ0;                // shapes x batch x H   (dL/dz0)
    float* dY;                 // shapes x batch
    float* H1;                 // shapes x batch x H
    float* loss;               // shapes x batch       squared error per point
    uint32_t* index;           // shapes x batch       sampled point of each row
};

__device__ __forceinline__ uint32_t batchIndex(const TrainArgs& a, uint32_t s, uint32_t i) {
    uint32_t h = (a.step + 1) * 0x9E3779B9u ^ (i * 0x85EBCA6Bu) ^ (s * 0xC2B2AE35u) ^ a.seed;
    h ^= h >> 16; h *= 0x7FEB352Du; h ^= h >> 15; h *= 0x846CA68Bu; h ^= h >> 16;
    return h % a.pointsPerShape;
}

__global__ void __launch_bounds__(128) k_trainPoints(TrainArgs a) {
    __shared__ float p[Net::SIZE];
    uint32_t s = blockIdx.y;
    const float* params = a.params + size_t(s) * Net::SIZE;
    for (int k = threadIdx.x; k < Net::SIZE; k += blockDim.x) p[k] = params[k];
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.batch) return;
    uint32_t pick = batchIndex(a, s, i);
    float4 q = a.points[size_t(s) * a.pointsPerShape + pick];
    size_t row = size_t(s) * a.batch + i;
    a.index[row] = pick;
    float h0[H], c0[H], h1[H];
    for (int j = 0; j < H; ++j) {
        float z = p[Net::W0 + 3 * j] * q.x + p[Net::W0 + 3 * j + 1] * q.y + p[Net::W0 + 3 * j + 2] * q.z + p[Net::B0 + j];
        h0[j] = sinf(z);
        c0[j] = cosf(z);
    }
    float y = p[Net::B2];
    for (int j = 0; j < H; ++j) {
        float acc = p[Net::B1 + j];
        for (int k = 0; k < H; ++k) acc += p[Net::W1 + H * j + k] * h0[k];
        h1[j] = acc > 0.f ? acc : 0.f;
        y += p[Net::W2 + j] * h1[j];
    }
    float t = q.w / a.scale;
    float err = y - t;
    // Asymmetric squared error: an over-prediction at a point inside the
    // shape weighs `over` times as much (the calibrated margin is the largest
    // prediction inside, so it is what pushes the margin up).
    float weight = (t <= 0.f && err > 0.f) ? a.over : 1.f;
    a.loss[row] = weight * err * err;
    float dy = 2.f * weight * err / float(a.batch);
    a.dY[row] = dy;
    float dz[H];
    for (int k = 0; k < H; ++k) dz[k] = 0.f;
    for (int j = 0; j < H; ++j) {
        float da = h1[j] > 0.f ? dy * p[Net::W2 + j] : 0.f;
        a.dA1[row * H + j] = da;
        a.H1[row * H + j] = h1[j];
        for (int k = 0; k < H; ++k) dz[k] += da * p[Net::W1 + H * j + k];
    }
    for (int k = 0; k < H; ++k) {
        a.H0[row * H + k] = h0[k];
        a.dZ0[row * H + k] = dz[k] * c0[k];
    }
}

// Parameter gradients, one thread per parameter, sums over the batch in row
// order (deterministic).
__global__ void k_trainGrads(TrainArgs a, float* grads) {
    uint32_t s = blockIdx.y;
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Net::SIZE) return;
    size_t base = size_t(s) * a.batch;
    float g = 0.f;
    if (k < Net::B0) {  // W0[j][c]
        uint32_t j = k / 3, c = k % 3;
        for (uint32_t i = 0; i < a.batch; ++i) {
            float4 q = a.points[size_t(s) * a.pointsPerShape + a.index[base + i]];
            float coord = c == 0 ? q.x : (c == 1 ? q.y : q.z);
            g += a.dZ0[(base + i) * H + j] * coord;
        }
    } else if (k < Net::W1) {
        uint32_t j = k - Net::B0;
        for (uint32_t i = 0; i < a.batch; ++i) g += a.dZ0[(base + i) * H + j];
    } else if (k < Net::B1) {
        uint32_t j = (k - Net::W1) / H, c = (k - Net::W1) % H;
        for (uint32_t i = 0; i < a.batch; ++i) g += a.dA1[(base + i) * H + j] * a.H0[(base + i) * H + c];
    } else if (k < Net::W2) {
        uint32_t j = k - Net::B1;
        for (uint32_t i = 0; i < a.batch; ++i) g += a.dA1[(base + i) * H + j];
    } else if (k < Net::B2) {
        uint32_t j = k - Net::W2;
        for (uint32_t i = 0; i < a.batch; ++i) g += a.dY[base + i] * a.H1[(base + i) * H + j];
    } else if (k == Net::B2) {
        for (uint32_t i = 0; i < a.batch; ++i) g += a.dY[base + i];
    }
    grads[size_t(s) * Net::SIZE + k] = g;
}

// Adam (Kingma & Ba 2015) on every parameter of every shape.
__global__ void k_adam(float* params, const float* grads, float* m, float* v, uint32_t total, float lr,
                       float beta1, float beta2, float eps, uint32_t step) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= total) return;
    float g = grads[k];
    float mk1 = beta1 * m[k] + (1.f - beta1) * g;
    float vk1 = beta2 * v[k] + (1.f - beta2) * g * g;
    m[k] = mk1;
    v[k] = vk1;
    float mhat = mk1 / (1.f - powf(beta1, float(step)));
    float vhat = vk1 / (1.f - powf(beta2, float(step)));
    params[k] -= lr * mhat / (sqrtf(vhat) + eps);
}

// ------------------------------------------------------------- inference
// Evaluation with the inference weights (W1 and the output row rounded to
// BF16, FP32 accumulation): the exact function the culler applies in the
// contact pass, here for calibration and tests.
__device__ __forceinline__ float cullerEval(const float* p, const __nv_bfloat16* w1, float x, float y, float z) {
    float h0[H];
    for (int j = 0; j < H; ++j) {
        float zz = p[Net::W0 + 3 * j] * x + p[Net::W0 + 3 * j + 1] * y + p[Net::W0 + 3 * j + 2] * z + p[Net::B0 + j];
        h0[j] = __bfloat162float(__float2bfloat16(__sinf(zz)));
    }
    float out = p[Net::B2];
    for (int j = 0; j < H; ++j) {
        float acc = 0.f;
        for (int k = 0; k < H; ++k) acc += __bfloat162float(w1[H * j + k]) * h0[k];
        acc += p[Net::B1 + j];
        out += p[Net::W2 + j] * (acc > 0.f ? acc : 0.f);
    }
    return out;
}
__global__ void k_cullerEval(const float* params, const __nv_bfloat16* w1, const float4* points, uint32_t count,
                             float* out) {
    uint32_t s = blockIdx.y;
    const float* p = params + size_t(s) * Net::SIZE;
    const __nv_bfloat16* w = w1 + size_t(s) * H * H;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        float4 q = points[size_t(s) * count + k];
        out[size_t(s) * count + k] = cullerEval(p, w, q.x, q.y, q.z);
    }
}
__global__ void k_roundWeights(const float* params, __nv_bfloat16* w1, uint32_t shapes) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= shapes * H * H) return;
    uint32_t s = k / (H * H), e = k % (H * H);
    w1[k] = __float2bfloat16(params[size_t(s) * Net::SIZE + Net::W1 + e]);
}

// The run-time culling function (tensor-core tile, culler.cuh) on stored
// points: shape s owns points [s count, (s + 1) count); tiles of 128 rows of
// that shape-sorted list, one CTA of 128 threads per tile in turn.  A tile
// whose tensor-core wait gave up writes NaN predictions.
__global__ void __launch_bounds__(128) k_cullerPredict(const float* params, const uint32_t* w1, const float4* points,
                                                        uint32_t shapes, uint32_t count, float* out) {
    __shared__ CullerShared sh;
    cullerBegin(sh);
    uint32_t phase = 0, total = shapes * count, tiles = (total + CULLER_ROWS - 1) / CULLER_ROWS;
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        uint32_t i = t * CULLER_ROWS + threadIdx.x;
        float4 q = i < total ? points[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        float y;
        bool ok = cullerTile(sh, params, w1, i < total ? i / count : EMPTY, xyz(q), phase, y);
        if (i < total) out[i] = ok ? y : __int_as_float(0x7fc00000);
        if (!ok) break;
    }
    cullerEnd(sh, phase);
}
__device__ __forceinline__ uint32_t orderedKey(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
// Per shape: the largest prediction over points with phi <= 0 (inside).
__global__ void k_insideMax(const float4* points, const float* y, uint32_t count, uint32_t* keys) {
    uint32_t s = blockIdx.y;
    uint32_t best = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        size_t at = size_t(s) * count + k;
        if (points[at].w <= 0.0f) best = max(best, orderedKey(y[at]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31u) == 0 && best) atomicMax(&keys[s], best);
}

// Per (shape, cell of the 8^3 grid over the shape's root box): the largest
// prediction over points with phi <= 0, and how many there were.
__global__ void k_insideMaxCells(const float4* points, const float* y, uint32_t count, const uint4* roots,
                                 const float4* meshMin, const float4* meshMax, uint32_t* keys, uint32_t* counts) {
    uint32_t s = blockIdx.y;
    uint32_t root = roots[s].x;
    float4 low = meshMin[root], high = meshMax[root];
    const uint32_t cells = CULLER_MARGINS - 1;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        size_t at = size_t(s) * count + k;
        float4 q = points[at];
        if (q.w > 0.0f) continue;
        uint32_t cell = cullerCell(low, high, xyz(q));
        atomicMax(&keys[s * cells + cell], orderedKey(y[at]));
        atomicAdd(&counts[s * cells + cell], 1u);
    }
}

}  // namespace sdg

using namespace sdg;

extern "C" {

int sdg_culler_margin_cells(void) { return CULLER_MARGINS - 1; }

// Per (shape, cell): ordered-integer maximum of the predictions at inside
// points and their count (keys and counts zeroed first, shapes x
// sdg_culler_margin_cells() words each); roots, mesh_min, mesh_max: the
// packed library's meshRoots, meshMin, meshMax.
int sdg_culler_inside_max_cells(const void* points, const void* predictions, uint32_t shapes, uint32_t count,
                                const void* roots, const void* mesh_min, const void* mesh_max, void* keys,
                                void* counts, void* stream) {
    dim3 grid((count + 255) / 256 < 256 ? (count + 255) / 256 : 256, shapes);
    k_insideMaxCells<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float4*>(points), static_cast<const float*>(predictions), count,
        static_cast<const uint4*>(roots), static_cast<const float4*>(mesh_min), static_cast<const float4*>(mesh_max),
        static_cast<uint32_t*>(keys), static_cast<uint32_t*>(counts));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int sdg_culler_param_count(void) { return Net::SIZE; }

// Run-time culling predictions for stored points (shapes x count).
int sdg_culler_tile_eval(const void* params, const void* w1_bf16, const void* points, uint32_t shapes,
                         uint32_t count, void* out, void* stream) {
    uint32_t tiles = (shapes * count + CULLER_ROWS - 1) / CULLER_ROWS;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t grid = std::max(1u, std::min(tiles, 2u * uint32_t(sms)));
    if (tiles)
        k_cullerPredict<<<grid, CULLER_ROWS, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const float*>(params), static_cast<const uint32_t*>(w1_bf16),
            static_cast<const float4*>(points), shapes, count, static_cast<float*>(out));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Ordered-integer maximum of the predictions at inside points, per shape
// (keys must be zeroed first; decode: k & 0x80000000 ? k ^ 0x80000000 : ~k).
int sdg_culler_inside_max(const void* points, const void* predictions, uint32_t shapes, uint32_t count, void* keys,
                          void* stream) {
    dim3 grid((count + 255) / 256 < 256 ? (count + 255) / 256 : 256, shapes);
    k_insideMax<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float4*>(points), static_cast<const float*>(predictions), count,
        static_cast<uint32_t*>(keys));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int sdg_culler_sample(void* const* buffers, const uint64_t* bytes, const double* values, uint32_t nvalues,
                      uint32_t shapes, uint32_t count, uint32_t seed, float shell, uint32_t inside_only,
                      void* out_points, void* accept, void* stream) {
    Params P;
    if (int rc = unpack_params(buffers, bytes, values, nvalues, P)) return rc;
    dim3 grid((count + 255) / 256 < 512 ? (count + 255) / 256 : 512, shapes);
    k_shellCandidates<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        P, count, seed, shell, inside_only, static_cast<float4*>(out_points), static_cast<uint32_t*>(accept));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int sdg_culler_surface(const void* triangles, const void* tri_start, uint32_t shapes, uint32_t count, uint32_t seed,
                       void* out_points, void* stream) {
    if (!triangles || !tri_start || !out_points) return 1;
    dim3 grid((count + 255) / 256 < 512 ? (count + 255) / 256 : 512, shapes);
    k_surfacePoints<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float4*>(triangles), static_cast<const uint32_t*>(tri_start), count, seed,
        static_cast<float4*>(out_points));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int sdg_culler_compact(const void* points, const void* accept, const void* offsets, uint32_t shapes,
                       uint32_t count, uint32_t capacity, void* out, void* stream) {
    dim3 grid((count + 255) / 256 < 512 ? (count + 255) / 256 : 512, shapes);
    k_compact<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float4*>(points), static_cast<const uint32_t*>(accept),
        static_cast<const uint32_t*>(offsets), count, capacity, static_cast<float4*>(out));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// One Adam step of every shape's network on a batch drawn from its points.
// `scratch` holds 4*batch*64 + 3*batch floats per shape; `grads`, `m`, `v`
// are shapes*param_count floats.
int sdg_culler_train_step(void* params, const void* points, uint32_t shapes, uint32_t points_per_shape,
                          uint32_t batch, uint32_t step, uint32_t seed, float scale, float over, float lr,
                          void* grads, void* m, void* v, void* scratch, float* loss_out, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float* f = static_cast<float*>(scratch);
    size_t rows = size_t(shapes) * batch;
    TrainArgs a{static_cast<const float*>(params), static_cast<const float4*>(points), points_per_shape, batch,
                step, seed, scale, over, f, f + rows * H, f + 2 * rows * H, f + 4 * rows * H, f + 3 * rows * H,
                f + 4 * rows * H + rows, reinterpret_cast<uint32_t*>(f + 4 * rows * H + 2 * rows)};
    k_trainPoints<<<dim3((batch + 127) / 128, shapes), 128, 0, s>>>(a);
    k_trainGrads<<<dim3((Net::SIZE + 127) / 128, shapes), 128, 0, s>>>(a, static_cast<float*>(grads));
    k_adam<<<(shapes * Net::SIZE + 255) / 256, 256, 0, s>>>(static_cast<float*>(params), static_cast<float*>(grads),
                                                           static_cast<float*>(m), static_cast<float*>(v),
                                                           shapes * Net::SIZE, lr, 0.9f, 0.999f, 1e-8f, step + 1);
    if (loss_out) cudaMemcpyAsync(loss_out, a.loss, rows * sizeof(float), cudaMemcpyDeviceToDevice, s);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Forward and backward only (no update): per-parameter gradients of the mean
// squared error for the batch of `step` (the gradient check entry).
int sdg_culler_gradients(const void* params, const void* points, uint32_t shapes, uint32_t points_per_shape,
                         uint32_t batch, uint32_t step, uint32_t seed, float scale, float over, void* grads,
                         void* scratch, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float* f = static_cast<float*>(scratch);
    size_t rows = size_t(shapes) * batch;
    TrainArgs a{static_cast<const float*>(params), static_cast<const float4*>(points), points_per_shape, batch,
                step, seed, scale, over, f, f + rows * H, f + 2 * rows * H, f + 4 * rows * H, f + 3 * rows * H,
                f + 4 * rows * H + rows, reinterpret_cast<uint32_t*>(f + 4 * rows * H + 2 * rows)};
    k_trainPoints<<<dim3((batch + 127) / 128, shapes), 128, 0, s>>>(a);
    k_trainGrads<<<dim3((Net::SIZE + 127) / 128, shapes), 128, 0, s>>>(a, static_cast<float*>(grads));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int sdg_culler_round(const void* params, void* w1_bf16, uint32_t shapes, void* stream) {
    k_roundWeights<<<(shapes * H * H + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float*>(params), static_cast<__nv_bfloat16*>(w1_bf16), shapes);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int sdg_culler_eval(const void* params, const void* w1_bf16, const void* points, uint32_t shapes, uint32_t count,
                    void* out, void* stream) {
    dim3 grid((count + 255) / 256 < 512 ? (count + 255) / 256 : 512, shapes);
    k_cullerEval<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float*>(params), static_cast<const __nv_bfloat16*>(w1_bf16),
        static_cast<const float4*>(points), count, static_cast<float*>(out));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // extern "C"
