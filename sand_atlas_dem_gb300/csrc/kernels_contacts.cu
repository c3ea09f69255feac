// Neighbour build, mesh contact collection, friction-history merge, contact
// law and the deterministic force gather.
//
// Contact order is canonical and equal to the reference CPU collector's
// (cpu_scheduling.slang:53-91): pair index, then direction, then leaf cluster
// in preorder, then node in meshSampleIndices order.  The collector keeps it
// with no atomics on contact slots: a flat leaf cull per directed pair, an
// exclusive scan to (directed pair, leaf) work items, one warp per item for
// the exact node queries (two nodes per lane, ballot hit masks), an
// exclusive scan of hit counts, and an emit pass that recomputes only the
// hits.  The history merge and the gather then walk sorted runs instead of a
// hash table and linked lists, so every run is reproducible bit for bit.
#include <cuda_runtime.h>
#include "culler.cuh"
#include "dem_device.cuh"
#include "launch.h"

namespace sdg {

constexpr uint32_t WARP = 32;
__device__ __forceinline__ uint32_t laneId() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t warpGlobal() { return (blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ uint32_t warpStride() { return (gridDim.x * blockDim.x) >> 5; }
__device__ __forceinline__ uint32_t lanesBelow() { return (1u << laneId()) - 1u; }

// ------------------------------------------------------------------- scan
__device__ __forceinline__ uint32_t scanCount(const ScanCount& c) {
    if (!c.ptr) return c.constant;
    uint32_t v = *c.ptr;
    return (v < c.cap ? v : c.cap) * c.mul;
}
__device__ __forceinline__ uint32_t blockInclusive(uint32_t v, uint32_t* shared) {
    // 256 threads: warp scans, then a scan of the 8 warp totals.
    uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) shared[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (blockDim.x >> 5) ? shared[lane] : 0;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < (blockDim.x >> 5)) shared[lane] = w;
    }
    __syncthreads();
    uint32_t add = warp ? shared[warp - 1] : 0;
    __syncthreads();
    return v + add;
}
__global__ void k_scanReduce(const uint32_t* in, ScanCount count, const uint32_t* gate, uint32_t* partials) {
    __shared__ uint32_t shared[32];
    if (gate && *gate == 0) return;
    uint32_t n = scanCount(count);
    uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
    uint32_t begin = blockIdx.x * chunk, end = min(n, begin + chunk);
    uint32_t sum = 0;
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) sum += in[i];
    sum = blockInclusive(sum, shared);
    if (threadIdx.x == blockDim.x - 1) partials[blockIdx.x] = sum;
}
__global__ void k_scanTop(ScanCount count, uint32_t* out, bool writeEnd, uint32_t* totalDst, const uint32_t* gate,
                          uint32_t* partials, uint32_t blocks) {
    __shared__ uint32_t shared[32];
    if (gate && *gate == 0) return;
    // blocks <= 1024: one element per thread.
    uint32_t v = threadIdx.x < blocks ? partials[threadIdx.x] : 0;
    uint32_t inc = blockInclusive(v, shared);
    if (threadIdx.x < blocks) partials[blocks + threadIdx.x] = inc - v;
    if (threadIdx.x == blockDim.x - 1) {
        uint32_t n = scanCount(count);
        if (writeEnd) out[n] = inc;
        if (totalDst) *totalDst = inc;
    }
}
__global__ void k_scanApply(const uint32_t* in, uint32_t* out, ScanCount count, const uint32_t* gate,
                            const uint32_t* partials, uint32_t* list) {
    __shared__ uint32_t shared[32];
    __shared__ uint32_t tileTotal;
    if (gate && *gate == 0) return;
    uint32_t n = scanCount(count);
    uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
    uint32_t begin = blockIdx.x * chunk, end = min(n, begin + chunk);
    uint32_t carry = partials[gridDim.x + blockIdx.x];
    for (uint32_t base = begin; base < end; base += blockDim.x) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < end ? in[i] : 0;
        uint32_t inc = blockInclusive(v, shared);
        if (i < end) {
            out[i] = carry + inc - v;
            if (list && v) list[carry + inc - v] = i;
        }
        if (threadIdx.x == blockDim.x - 1) tileTotal = inc;
        __syncthreads();
        carry += tileTotal;
        __syncthreads();
    }
}

void launch_scan(const uint32_t* in, uint32_t* out, ScanCount count, bool writeEnd, uint32_t* totalDst,
                 const uint32_t* gate, uint32_t* partials, cudaStream_t s) {
    k_scanReduce<<<SCAN_BLOCKS, 256, 0, s>>>(in, count, gate, partials);
    k_scanTop<<<1, 1024, 0, s>>>(count, out, writeEnd, totalDst, gate, partials, SCAN_BLOCKS);
    k_scanApply<<<SCAN_BLOCKS, 256, 0, s>>>(in, out, count, gate, partials, nullptr);
}

// The step's scans (r.scanPartials); with `list`, the apply pass also lists
// each index whose value is nonzero at its scanned offset (stream compaction
// in index order).
void launch_step_scan(const Res& r, const uint32_t* in, uint32_t* out, ScanCount count, bool writeEnd,
                      uint32_t* totalDst, const uint32_t* gate, cudaStream_t s, uint32_t* list = nullptr) {
    k_scanReduce<<<SCAN_BLOCKS, 256, 0, s>>>(in, count, gate, r.scanPartials);
    k_scanTop<<<1, 1024, 0, s>>>(count, out, writeEnd, totalDst, gate, r.scanPartials, SCAN_BLOCKS);
    k_scanApply<<<SCAN_BLOCKS, 256, 0, s>>>(in, out, count, gate, r.scanPartials, list);
}

// ------------------------------------------------------------ neighbours
// solver.slang:184-186
// Bin grid of a specimen: sb = (bins x, y, z, first bin of the specimen).
__device__ __forceinline__ void binIndex(const Res& r, uint32_t i, uint4 sb, float4 box, uint32_t b[3]) {
    float4 p = r.position[i];
    uint32_t bins[3] = {sb.x, sb.y, sb.z};
    float g[3] = {floorf(__fmul_rn(__fdiv_rn(p.x, box.x), float(sb.x))),
                  floorf(__fmul_rn(__fdiv_rn(p.y, box.y), float(sb.y))),
                  floorf(__fmul_rn(__fdiv_rn(p.z, box.z), float(sb.z)))};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        uint32_t v = uint32_t(g[k]);
        b[k] = v < bins[k] - 1 ? v : bins[k] - 1;
    }
}
__device__ __forceinline__ uint32_t binFlat(uint4 sb, const uint32_t b[3]) {
    return sb.w + (b[0] * sb.y + b[1]) * sb.z + b[2];
}
__device__ __forceinline__ uint32_t modIndex(int a, uint32_t n) { return uint32_t((a % int(n) + int(n)) % int(n)); }

__global__ void k_binsClear(const __grid_constant__ Params P) {
    const Res& r = P.r;
    if (r.control[4] == 0) return;
    for (uint32_t b = gtid(); b < P.c.binCount; b += gstride()) r.binCounts[b] = 0;
}
// solver.slang:350-359
__global__ void k_binsFill(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t id = gtid();
    if (id >= c.N || r.control[4] == 0) return;
    f3 p = xyz(r.position[id]), pl = xyz(r.positionRemainder[id]);
    if (!finite3(p) || !finite3(pl)) { fail(r, F_NONFINITE); return; }
    uint32_t sp = specimenOf(r, id);
    float4 cell = r.cell[3 * sp];
    if (c.periodic == 0) {
        f3 box = xyz(cell);
        if (__fadd_rn(p.x, pl.x) < 0 || __fadd_rn(p.y, pl.y) < 0 || __fadd_rn(p.z, pl.z) < 0 ||
            __fadd_rn(__fsub_rn(p.x, box.x), pl.x) >= 0 || __fadd_rn(__fsub_rn(p.y, box.y), pl.y) >= 0 ||
            __fadd_rn(__fsub_rn(p.z, box.z), pl.z) >= 0) { fail(r, F_ESCAPE); return; }
    }
    uint32_t b[3];
    uint4 sb = r.specimenBins[sp];
    binIndex(r, id, sb, cell, b);
    uint32_t bin = binFlat(sb, b);
    uint32_t slot = atomicAdd(&r.binCounts[bin], 1u);
    if (slot < c.binCapacity) r.binParticles[bin * c.binCapacity + slot] = id;
    else fail(r, F_BIN);
}
// Order each bin's slots by grain id: the serial reference fills bins in id
// order, which fixes the pair order downstream.  Rank sort in shared memory.
__global__ void k_binsSort(const __grid_constant__ Params P) {
    extern __shared__ uint32_t ids[];
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[4] == 0) return;
    uint32_t cap = c.binCapacity;
    uint32_t* sorted = ids + cap;
    for (uint32_t bin = blockIdx.x; bin < c.binCount; bin += gridDim.x) {
        uint32_t occ = min(r.binCounts[bin], cap);
        for (uint32_t k = threadIdx.x; k < occ; k += blockDim.x) ids[k] = r.binParticles[bin * cap + k];
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < occ; k += blockDim.x) {
            uint32_t v = ids[k], rank = 0;
            for (uint32_t t = 0; t < occ; ++t) rank += ids[t] < v;
            sorted[rank] = v;
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < occ; k += blockDim.x) r.binParticles[bin * cap + k] = sorted[k];
        __syncthreads();
    }
}
// ---- radix-sorted cell list (solver.slang:345-359 fills the bins serially,
// in grain order; a stable sort of the grains by bin gives the same slots).
// Keys are the flat bin indices (a grain that fails the checks gets
// binCount, past every bin); an LSD radix sort of 8-bit digits (stable:
// each pass keeps the order of equal digits) orders (bin, grain) pairs, and
// each bin's run is then copied into the reference's fixed-capacity slots.
// The scratch lives in byJPairs (pair ids by second grain), which the
// neighbour build rewrites only after the pairs exist: keys and grains twice
// (ping-pong) and the per-(digit, tile) counts.
constexpr uint32_t RADIX = 256, RADIX_ITEMS = 8, RADIX_TILE = 256 * RADIX_ITEMS;
struct RadixScratch {
    uint32_t *keys[2], *vals[2], *counts;
    uint32_t tiles;
};
__host__ __device__ __forceinline__ uint32_t radixTiles(uint32_t n) { return (n + RADIX_TILE - 1) / RADIX_TILE; }
// Words of byJPairs the sort needs (the radix path runs only where they fit).
__host__ __device__ __forceinline__ uint64_t radixWords(uint32_t n) {
    return 4ull * n + uint64_t(RADIX) * radixTiles(n) + 1;
}
__host__ __device__ __forceinline__ RadixScratch radixScratch(const Res& r, const Config& c) {
    uint32_t* base = r.byJPairs;
    RadixScratch x;
    x.keys[0] = base;
    x.vals[0] = base + c.N;
    x.keys[1] = base + 2 * size_t(c.N);
    x.vals[1] = base + 3 * size_t(c.N);
    x.counts = base + 4 * size_t(c.N);
    x.tiles = radixTiles(c.N);
    return x;
}
// Keys: the same checks and bin as k_binsFill.
__global__ void k_binKeys(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t id = gtid();
    if (id >= c.N || r.control[4] == 0) return;
    RadixScratch x = radixScratch(r, c);
    uint32_t key = c.binCount;
    f3 p = xyz(r.position[id]), pl = xyz(r.positionRemainder[id]);
    uint32_t sp = specimenOf(r, id);
    float4 cell = r.cell[3 * sp];
    bool ok = finite3(p) && finite3(pl);
    if (!ok) fail(r, F_NONFINITE);
    if (ok && c.periodic == 0) {
        f3 box = xyz(cell);
        if (__fadd_rn(p.x, pl.x) < 0 || __fadd_rn(p.y, pl.y) < 0 || __fadd_rn(p.z, pl.z) < 0 ||
            __fadd_rn(__fsub_rn(p.x, box.x), pl.x) >= 0 || __fadd_rn(__fsub_rn(p.y, box.y), pl.y) >= 0 ||
            __fadd_rn(__fsub_rn(p.z, box.z), pl.z) >= 0) {
            fail(r, F_ESCAPE);
            ok = false;
        }
    }
    if (ok) {
        uint32_t b[3];
        uint4 sb = r.specimenBins[sp];
        binIndex(r, id, sb, cell, b);
        key = binFlat(sb, b);
    }
    x.keys[0][id] = key;
    x.vals[0][id] = id;
}
// Digit counts of each tile: counts[digit * tiles + tile].
__global__ void __launch_bounds__(256) k_radixCount(const __grid_constant__ Params P, uint32_t shift, uint32_t from) {
    __shared__ uint32_t hist[RADIX];
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[4] == 0) return;
    RadixScratch x = radixScratch(r, c);
    hist[threadIdx.x] = 0;
    __syncthreads();
    uint32_t base = blockIdx.x * RADIX_TILE;
    for (uint32_t k = threadIdx.x; k < RADIX_TILE && base + k < c.N; k += blockDim.x)
        atomicAdd(&hist[(x.keys[from][base + k] >> shift) & (RADIX - 1)], 1u);
    __syncthreads();
    x.counts[threadIdx.x * x.tiles + blockIdx.x] = hist[threadIdx.x];
}
// Stable scatter of a tile: its elements in index order, 256 at a time; an
// element's place is its digit's offset for the tile (the scanned counts),
// plus the tile's earlier elements with that digit (a running count), plus
// the earlier warps of the same 256 with it, plus the lower lanes of its
// warp with it (__match_any_sync).
__global__ void __launch_bounds__(256) k_radixScatter(const __grid_constant__ Params P, uint32_t shift, uint32_t from) {
    __shared__ uint32_t offset[RADIX], warpCount[8][RADIX];
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[4] == 0) return;
    RadixScratch x = radixScratch(r, c);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    offset[threadIdx.x] = x.counts[threadIdx.x * x.tiles + blockIdx.x];
#pragma unroll
    for (uint32_t w = 0; w < 8; ++w) warpCount[w][threadIdx.x] = 0;
    __syncthreads();
    uint32_t base = blockIdx.x * RADIX_TILE;
    for (uint32_t round = 0; round < RADIX_ITEMS; ++round) {
        uint32_t i = base + round * 256 + threadIdx.x;
        bool valid = i < c.N && round * 256 + threadIdx.x < RADIX_TILE;
        uint32_t key = valid ? x.keys[from][i] : 0u, val = valid ? x.vals[from][i] : 0u;
        uint32_t digit = valid ? (key >> shift) & (RADIX - 1) : RADIX;  // RADIX: no element
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t below = __popc(peers & lanesBelow());
        if (valid && below == 0) warpCount[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t place = offset[digit] + below;
            for (uint32_t w = 0; w < warp; ++w) place += warpCount[w][digit];
            x.keys[from ^ 1u][place] = key;
            x.vals[from ^ 1u][place] = val;
        }
        __syncthreads();
        // These 256 elements of each digit move its offset on.
        uint32_t total = 0;
#pragma unroll
        for (uint32_t w = 0; w < 8; ++w) {
            total += warpCount[w][threadIdx.x];
            warpCount[w][threadIdx.x] = 0;
        }
        offset[threadIdx.x] += total;
        __syncthreads();
    }
}
// Each bin's run of the sorted grains into its reference slots.
__global__ void k_binsFromSorted(const __grid_constant__ Params P, uint32_t from) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[4] == 0) return;
    RadixScratch x = radixScratch(r, c);
    for (uint32_t k = gtid(); k < c.N; k += gstride()) {
        uint32_t bin = x.keys[from][k];
        if (bin >= c.binCount || (k > 0 && x.keys[from][k - 1] == bin)) continue;  // not the start of a run
        uint32_t occ = 0;
        while (k + occ < c.N && x.keys[from][k + occ] == bin) {
            if (occ < c.binCapacity) r.binParticles[bin * c.binCapacity + occ] = x.vals[from][k + occ];
            ++occ;
        }
        r.binCounts[bin] = occ;
        if (occ > c.binCapacity) fail(r, F_BIN);
    }
}
// solver.slang:360-392: the pair search, a warp per grain with ballot
// compaction.  An FP32 minimum-image estimate rejects grains that are clearly
// beyond range before the exact FP64 branch decides.  The grain's
// stencil bins (the reference's x, y, z order) are taken 32 at a time, one
// per lane with its occupancy; their slots form one candidate sequence in
// the reference's order (bin, then slot), which the lanes test 32 at a time
// (the FP32 estimate, then the exact FP64 branch).  A ballot of the passing
// candidates counts them or, in the emit pass, gives each its place in
// order: the pair list is the serial search's, pair for pair.
template <bool Emit>
__device__ __forceinline__ void findPairsWarp(const Res& r, const Config& c, uint32_t id) {
    const uint32_t lane = laneId();
    uint32_t sp = specimenOf(r, id);
    uint4 sb = r.specimenBins[sp];
    uint32_t bins[3] = {sb.x, sb.y, sb.z};
    float4 cell = r.cell[3 * sp];
    uint32_t b[3];
    binIndex(r, id, sb, cell, b);
    float cutoff = r.referenceCell[2 * sp + 1].w;
    float box[3] = {cell.x, cell.y, cell.z};
    int reach[3], low[3];
    uint32_t width[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        reach[k] = int(ceilf(__fmul_rn(__fdiv_rn(cutoff, box[k]), float(bins[k]))));
        low[k] = max(int(b[k]) - reach[k], 0);
        int high = min(int(b[k]) + reach[k], int(bins[k]) - 1);
        uint32_t w = uint32_t(2 * reach[k] + 1);
        width[k] = c.periodic != 0 ? min(w, bins[k]) : uint32_t(high - low[k] + 1);
    }
    float4 pi = r.position[id], li = r.positionRemainder[id];
    float ri = r.body[id].z;
    uint32_t stencil = width[0] * width[1] * width[2];
    uint32_t count = 0, base = Emit ? r.pairOffsets[id] : 0u;
    for (uint32_t q0 = 0; q0 < stencil; q0 += 32) {
        // Lane q: stencil bin q0 + q (x slowest, z fastest) and its occupancy.
        uint32_t q = q0 + lane, bin = 0, occ = 0;
        if (q < stencil) {
            uint32_t z = q % width[2], y = (q / width[2]) % width[1], x = q / (width[2] * width[1]);
            uint32_t cc[3];
            if (c.periodic != 0) {
                cc[0] = modIndex(int(b[0]) - reach[0] + int(x), bins[0]);
                cc[1] = modIndex(int(b[1]) - reach[1] + int(y), bins[1]);
                cc[2] = modIndex(int(b[2]) - reach[2] + int(z), bins[2]);
            } else {
                cc[0] = uint32_t(low[0] + int(x));
                cc[1] = uint32_t(low[1] + int(y));
                cc[2] = uint32_t(low[2] + int(z));
            }
            bin = binFlat(sb, cc);
            occ = min(r.binCounts[bin], c.binCapacity);
        }
        uint32_t inclusive = occ;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, inclusive, o);
            if (lane >= o) inclusive += t;
        }
        uint32_t total = __shfl_sync(0xffffffffu, inclusive, 31);
        for (uint32_t c0 = 0; c0 < total; c0 += 32) {
            uint32_t k = c0 + lane;
            // The stencil bin holding candidate k: the first lane whose
            // inclusive count exceeds k (every lane searches, past the end
            // with the last candidate, so that each shuffle has the warp).
            uint32_t kk = min(k, total - 1), lo = 0, hi = 31;
#pragma unroll
            for (uint32_t step = 0; step < 5; ++step) {
                uint32_t mid = (lo + hi) >> 1;
                if (__shfl_sync(0xffffffffu, inclusive, mid) > kk) hi = mid; else lo = mid + 1;
            }
            uint32_t before = __shfl_sync(0xffffffffu, inclusive - occ, lo);
            uint32_t at = __shfl_sync(0xffffffffu, bin, lo);
            bool pass = false;
            uint32_t j = 0;
            if (k < total) {
                j = r.binParticles[at * c.binCapacity + (k - before)];
                if (j > id) {
                    float range = __fadd_rn(__fadd_rn(ri, r.body[j].z), c.skin);
                    float rr = __fmul_rn(range, range);
                    bool near = true;
                    if (c.sourceSurfaceNormal == 0) {
                        float4 pj = r.position[j], lj = r.positionRemainder[j];
                        float e[3] = {(pj.x - pi.x) + (lj.x - li.x), (pj.y - pi.y) + (lj.y - li.y),
                                      (pj.z - pi.z) + (lj.z - li.z)};
                        if (c.periodic != 0) {
#pragma unroll
                            for (int a = 0; a < 3; ++a) e[a] -= floorf(e[a] / box[a] + 0.5f) * box[a];
                        }
                        near = e[0] * e[0] + e[1] * e[1] + e[2] * e[2] <= 1.002f * rr;  // estimate: ~1e-6 relative
                    }
                    if (near) {
                        f3 d = centerBranch64(r, c, id, j);
                        float dd = dot(d, d);
                        if (c.sourceSurfaceNormal != 0 && dd < 1e-12f) fail(r, F_COINCIDENT);
                        else pass = dd <= rr;
                    }
                }
            }
            uint32_t ballot = __ballot_sync(0xffffffffu, pass);
            if (Emit && pass) {
                uint32_t index = base + count + __popc(ballot & lanesBelow());
                if (index < c.pairCapacity) r.pairs[index] = make_uint2(id, j);
                else fail(r, F_PAIR);
            }
            count += __popc(ballot);
        }
    }
    if (!Emit && lane == 0) r.pairCounts[id] = count;
}
__global__ void __launch_bounds__(256) k_pairsCountWarp(const __grid_constant__ Params P) {
    if (P.r.control[4] == 0) return;
    for (uint32_t id = warpGlobal(); id < P.c.N; id += warpStride()) findPairsWarp<false>(P.r, P.c, id);
}
// solver.slang:388-392 (the pair total is written by the scan)
__global__ void __launch_bounds__(256) k_pairsEmitWarp(const __grid_constant__ Params P) {
    const Res& r = P.r;
    if (r.control[4] == 0) return;
    if (gtid() == 0) r.work[W_REBUILDS] += 1u;
    for (uint32_t id = warpGlobal(); id < P.c.N; id += warpStride()) findPairsWarp<true>(r, P.c, id);
    for (uint32_t id = gtid(); id < P.c.N; id += gstride()) {
        r.referencePosition[id] = r.position[id];
        r.referencePositionRemainder[id] = r.positionRemainder[id];
        uint32_t sp = specimenOf(r, id);
        r.referenceCell[2 * sp] = r.cell[3 * sp];
    }
}
// Pairs grouped by their second grain, ascending pair id per grain.
__global__ void k_byJReset(const __grid_constant__ Params P) {
    const Res& r = P.r;
    if (r.control[4] == 0) return;
    for (uint32_t g = gtid(); g <= P.c.N; g += gstride()) {
        r.byJCounts[g] = 0;
        if (g < P.c.N) r.byJCursor[g] = 0;
    }
}
__global__ void k_byJCount(const __grid_constant__ Params P) {
    const Res& r = P.r;
    if (r.control[4] == 0) return;
    uint32_t n = activePairs(r, P.c);
    for (uint32_t p = gtid(); p < n; p += gstride()) atomicAdd(&r.byJCounts[r.pairs[p].y], 1u);
}
__global__ void k_byJFill(const __grid_constant__ Params P) {
    const Res& r = P.r;
    if (r.control[4] == 0) return;
    uint32_t n = activePairs(r, P.c);
    for (uint32_t p = gtid(); p < n; p += gstride()) {
        uint32_t j = r.pairs[p].y;
        uint32_t slot = atomicAdd(&r.byJCursor[j], 1u);
        r.byJPairs[r.byJOffsets[j] + slot] = p;
    }
}
__global__ void k_byJSort(const __grid_constant__ Params P) {
    const Res& r = P.r;
    uint32_t g = gtid();
    if (g >= P.c.N || r.control[4] == 0) return;
    uint32_t begin = r.byJOffsets[g], end = r.byJOffsets[g + 1];
    for (uint32_t a = begin + 1; a < end; ++a) {
        uint32_t v = r.byJPairs[a], k = a;
        while (k > begin && r.byJPairs[k - 1] > v) { r.byJPairs[k] = r.byJPairs[k - 1]; --k; }
        r.byJPairs[k] = v;
    }
}

// ------------------------------------------------------------ collection
// Per pair: FP64 branches of both directions, root cull mask and 3x4
// source-to-target transforms (prepareMeshPairs, solver.slang:468-489), and
// the pair table of the history side being written.
// Upper bound of |R(a) v - R(b) v| / |v| for the rotations of quaternions a
// and b: with 2 alpha the angle between them (or between a and -b), the chord
// 2 sin(2 alpha / 2) <= 4 sin(alpha / 2) = 2 |a -/+ b|.
__device__ __forceinline__ float rotationChord(float4 a, float4 b) {
    float4 d = make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
    float4 s = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
    float dd = d.x * d.x + d.y * d.y + d.z * d.z + d.w * d.w;
    float ss = s.x * s.x + s.y * s.y + s.z * s.z + s.w * s.w;
    return 2.0f * sqrtf(fminf(dd, ss));
}
// Whether the filter results stored for pair p no longer cover it.  They were
// built with every test grown by `margin` (target frame, unscaled).  A node x
// of grain i lies at local = R_j^T (R_i s_i x - b) / s_j in grain j's frame;
// between the build (0) and now (1), for any node that can touch j now
// (|R_i s_i x - b| <= r_j, the bounding radius),
//   s_j |local1 - local0| <= chord_i r_i + |b1 - b0| + chord_j r_j,
// and symmetrically for the other direction.  While that stays below
// margin x min(s_i, s_j), every node that passes the tests now passed the
// grown tests then, so the stored survivors contain every node the filters
// would keep now.  The factor 1.001 and the 1e-5 term cover the FP32
// rounding of the bound and of quaternions that are not exactly unit.
__device__ __forceinline__ bool filterStale(const Res& r, float margin, uint32_t p, uint2 ij, f3 branch) {
    uint2 ref = r.filterRefPairs[p];
    if (ref.x != ij.x || ref.y != ij.y) return true;
    float4 bi = r.body[ij.x], bj = r.body[ij.y];
    float drift = rotationChord(r.rotation[ij.x], r.filterRefRotation[ij.x]) * bi.z +
                  length(branch - xyz(r.filterRefBranch[p])) +
                  rotationChord(r.rotation[ij.y], r.filterRefRotation[ij.y]) * bj.z;
    float slack = 1e-5f * (1.0f + bi.z + bj.z + length(branch));
    return 1.001f * drift + slack > margin * fminf(bi.x, bj.x);
}
__global__ void k_pairSetup(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t n = activePairs(r, c);
    float margin = __uint_as_float(r.work[W_FILTER_MARGIN]);  // the margin the stored results were built with
    bool check = r.work[W_FILTER] == 0;
    for (uint32_t p = gtid(); p < n; p += gstride()) {
        uint2 ij = r.pairs[p];
        f3 branch[2] = {centerBranch64(r, c, ij.x, ij.y), centerBranch64(r, c, ij.y, ij.x)};
        r.dpairBranch[2 * p] = w4(branch[0], 0.f);
        r.dpairBranch[2 * p + 1] = w4(branch[1], 0.f);
        if (check && filterStale(r, margin, p, ij, branch[0])) atomicOr(&r.work[W_FILTER], 1u);
        r.sidePairB[p] = ij.y;
    }
    uint32_t grains = c.N;
    for (uint32_t g = gtid(); g <= grains; g += gstride())
        r.sidePairOffsets[g] = g < grains ? min(r.pairOffsets[g], n) : n;
}
// Root cull masks and source-to-target transforms of every directed pair
// (prepareMeshPairs, solver.slang:468-489), on steps that build the filter
// results, with the tests grown by the margin.
__global__ void k_pairMasks(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0 || r.work[W_FILTER] == 0) return;
    uint32_t n = activePairs(r, c);
    float margin = buildMargin(r, c);
    for (uint32_t p = gtid(); p < n; p += gstride()) {
        uint2 ij = r.pairs[p];
        f3 branch[2] = {xyz(r.dpairBranch[2 * p]), xyz(r.dpairBranch[2 * p + 1])};
        uint32_t mask = 0;
        if (meshClusterMayContact(r, ij.x, ij.y, r.meshClusterInfo[r.shapeId[ij.x]].x, branch[0], margin)) mask |= 1;
        if (meshClusterMayContact(r, ij.y, ij.x, r.meshClusterInfo[r.shapeId[ij.y]].x, branch[1], margin)) mask |= 2;
        for (uint32_t pass = 0; pass < 2; ++pass) {
            if ((mask & (1u << pass)) == 0) continue;
            uint32_t i = pass == 0 ? ij.x : ij.y, j = pass == 0 ? ij.y : ij.x;
            float4 qi = r.rotation[i], qj = r.rotation[j];
            float sj = r.body[j].x;
            float ratio = __fdiv_rn(r.body[i].x, sj);
            f3 a = qinv(qj, qrot(qi, mk(ratio, 0.f, 0.f)));
            f3 b = qinv(qj, qrot(qi, mk(0.f, ratio, 0.f)));
            f3 cz = qinv(qj, qrot(qi, mk(0.f, 0.f, ratio)));
            f3 offset = qinv(qj, -branch[pass]) / sj;
            uint32_t base = 4 * (2 * p + pass);
            r.meshPairTransform[base] = make_float4(a.x, b.x, cz.x, offset.x);
            r.meshPairTransform[base + 1] = make_float4(a.y, b.y, cz.y, offset.y);
            r.meshPairTransform[base + 2] = make_float4(a.z, b.z, cz.z, offset.z);
            r.meshPairTransform[base + 3] = make_float4(__fdiv_rn(length(branch[pass]), sj), 0.f, 0.f, 0.f);
        }
        r.meshPairMask[p] = mask;
    }
}
// resetMeshContacts (solver.slang:396-403)
// The stored filter results (items, survivor masks and list) serve this step
// if they are complete and were built under this configured margin on a
// pair list of the same length; k_pairSetup then checks each pair and how
// far its grains have moved, and asks for a build if any pair is no longer
// covered.  The margin adapts to the motion, between the configured margin m
// and 16 m: a build within 8 collector runs of the last one doubles it, a
// build after more than 64 halves it (a larger margin keeps a few more nodes
// in the stored lists; it never changes a result).
__global__ void k_resetContacts(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    r.control[2] = 0;
    r.control[6] = 0;
    bool on = c.filterMargin > 0.0f;
    uint32_t base = __float_as_uint(c.filterMargin);
    bool valid = r.work[W_FILTER_VALID] != 0 && r.work[W_FILTER_BASE] == base;
    bool build = !on || !valid || r.work[W_FILTER_PAIRS] != r.control[1];
    r.work[W_FILTER] = build ? 1u : 0u;
    r.work[W_FILTER_STEPS] += 1u;
    if (on) {
        uint32_t age = r.work[W_FILTER_AGE] + 1u;
        r.work[W_FILTER_AGE] = age;
        float current = __uint_as_float(r.work[W_FILTER_MARGIN]);
        float next = c.filterMargin;
        if (valid)
            next = age <= 8u ? fminf(2.0f * current, 16.0f * c.filterMargin)
                             : (age > 64u ? fmaxf(0.5f * current, c.filterMargin) : current);
        r.work[W_FILTER_NEXT] = __float_as_uint(next);
    }
    if (build) r.work[W_CANDIDATES] = 0;
}
// Flat leaf cull: one warp per directed pair; meshPairBounds (solver.slang:
// 404-417) + meshBoxMayContact (:274-288) on every leaf, gated by the root
// mask.  Equivalent in contacts to the reference's hierarchical walks since
// every test is conservative and each node's decision is exact.
// The enclosure plane test in the source grain's own frame.  With m the
// target-frame normal n rotated to the world, the plane value of a node at
// x (source shape frame, unscaled) is n.local + w = n'.x + w' with
// n' = (s_src/s_dst) qinv(q_src, m) and w' = w - m.branch/s_dst, so one
// 3-term dot per node replaces the two quaternion rotations.  A node (or a
// whole leaf box) is rejected only when n'.x + w' exceeds an upper bound of
// the reference pad 2^-17 (1 + max|local|) -- |local| <= (s_src |x| +
// |branch|) / s_dst -- plus a slack 1e-5 x the magnitudes involved, far
// above the FP32 rounding of either evaluation order.  Such a node would be
// rejected by the reference's own plane test: no contact changes.
struct SourcePlane {
    float4 plane;  // n', w'
    float4 scale;  // s_src/s_dst, |branch|_1/s_dst, |w|, |n'|_1
};
__device__ __forceinline__ SourcePlane sourcePlane(float4 plane, float4 qs, float4 qd, float ss, float sd, f3 branch) {
    SourcePlane sp;
    f3 m = qrot(qd, xyz(plane));
    float k = __fdiv_rn(ss, sd);
    f3 n = qinv(qs, m) * k;
    float w = __fsub_rn(plane.w, __fdiv_rn(dot(m, branch), sd));
    float bn = __fdiv_rn(__fadd_rn(__fadd_rn(fabsf(branch.x), fabsf(branch.y)), fabsf(branch.z)), sd);
    sp.plane = w4(n, w);
    sp.scale = make_float4(k, bn, fabsf(plane.w), __fadd_rn(__fadd_rn(fabsf(n.x), fabsf(n.y)), fabsf(n.z)));
    return sp;
}
// Rejection bound for points with |x|_1 <= extent.
__device__ __forceinline__ float sourcePlaneBound(const SourcePlane& sp, float extent) {
    float reach = __fadd_rn(__fmul_rn(sp.scale.x, extent), sp.scale.y);
    float pad = __fmul_rn(0.00000762939453125f, __fadd_rn(1.0f, reach));
    float slack = __fmul_rn(1e-5f, __fadd_rn(__fadd_rn(__fadd_rn(1.0f, sp.scale.z), reach),
                                            __fmul_rn(sp.scale.w, extent)));
    return __fadd_rn(pad, slack);
}
// `grow` widens a test for the stored filter results: the plane value moves
// by at most |n| = 1 times a node's displacement in the target frame, so
// `grow` = margin x 1.001 (FP32 unit normals) covers every placement within
// the margin.
__device__ __forceinline__ bool nodeBeyondSourcePlane(const SourcePlane& sp, f3 x, float grow = 0.0f) {
    float extent = __fadd_rn(__fadd_rn(fabsf(x.x), fabsf(x.y)), fabsf(x.z));
    return __fadd_rn(dot(xyz(sp.plane), x), sp.plane.w) > __fadd_rn(sourcePlaneBound(sp, extent), grow);
}
__device__ __forceinline__ bool leafBeyondSourcePlane(const SourcePlane& sp, f3 low, f3 high, float grow = 0.0f) {
    f3 c = 0.5f * (low + high), h = 0.5f * (high - low);
    float nearest = __fsub_rn(__fadd_rn(dot(xyz(sp.plane), c), sp.plane.w), dot(abs3(xyz(sp.plane)), h));
    float extent = __fadd_rn(__fadd_rn(__fadd_rn(fabsf(c.x), fabsf(c.y)), fabsf(c.z)),
                             __fadd_rn(__fadd_rn(h.x, h.y), h.z));
    return nearest > __fadd_rn(sourcePlaneBound(sp, extent), grow);
}
// Enclosure plane of the target most violated by the source centre
// (cpu_scheduling.slang:58-71): warp arg-max, lowest index on ties.  Every
// lane returns the plane.
__device__ __forceinline__ float4 enclosurePlane(const Res& r, uint32_t j, uint32_t targetShape, f3 branch) {
    f3 centre = (-qinv(r.rotation[j], branch)) / r.body[j].x;
    uint4 first = __ldg(&r.meshHullInfo[6 * targetShape]);
    uint4 last = __ldg(&r.meshHullInfo[6 * targetShape + 5]);
    uint32_t begin = first.x, end = last.x + last.y;
    float best = -1e30f;
    uint32_t bestIndex = EMPTY;
    for (uint32_t k = begin + laneId(); k < end; k += WARP) {
        float4 candidate = __ldg(&r.meshPlanes[k]);
        float violation = __fadd_rn(dot(xyz(candidate), centre), candidate.w);
        if (violation > best) { best = violation; bestIndex = k; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float ob = __shfl_xor_sync(0xffffffffu, best, o);
        uint32_t oi = __shfl_xor_sync(0xffffffffu, bestIndex, o);
        if (ob > best || (ob == best && oi < bestIndex)) { best = ob; bestIndex = oi; }
    }
    return bestIndex == EMPTY ? make_float4(0.f, 0.f, 0.f, 0.f) : __ldg(&r.meshPlanes[bestIndex]);
}
// Runs on steps that build the filter results: with a margin every test is
// grown by it and the pose the results are built at is recorded.
__global__ void k_leafCull(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.work[W_FILTER] == 0) return;
    uint32_t n = 2 * activePairs(r, c);
    bool live = r.control[0] == 0;
    float margin = buildMargin(r, c);
    float grow = __fmul_rn(1.001f, margin);
    if (margin > 0.0f) {
        for (uint32_t g = gtid(); g < c.N; g += gstride()) r.filterRefRotation[g] = r.rotation[g];
        if (storedKeep(c))
            for (uint32_t b = gtid(); b <= c.shapes * WALK_BUCKETS; b += gstride()) r.walkBucketCount[b] = 0;
        if (gtid() == 0) {
            r.work[W_FILTER_VALID] = 0;
            r.work[W_FILTER_PAIRS] = r.control[1];
            r.work[W_FILTER_MARGIN] = __float_as_uint(margin);
            r.work[W_FILTER_BASE] = __float_as_uint(c.filterMargin);
            r.work[W_FILTER_AGE] = 0;
            r.work[W_FILTER_BUILDS] += 1u;
        }
    }
    for (uint32_t d = warpGlobal(); d < n; d += warpStride()) {
        uint32_t p = d >> 1, pass = d & 1;
        uint2 ij = r.pairs[p];
        uint32_t i = pass ? ij.y : ij.x, j = pass ? ij.x : ij.y;
        if (margin > 0.0f && pass == 0 && laneId() == 0) {
            r.filterRefPairs[p] = ij;
            r.filterRefBranch[p] = r.dpairBranch[d];
        }
        uint32_t count = 0;
        if (live && ((r.meshPairMask[p] >> pass) & 1u)) {
            uint4 li = __ldg(&r.meshLeafInfo[r.shapeId[i]]);
            uint32_t targetShape = r.shapeId[j];
            float4 plane;
            SourcePlane source;
            {
                f3 branch = xyz(r.dpairBranch[d]);
                plane = enclosurePlane(r, j, targetShape, branch);
                source = sourcePlane(plane, r.rotation[i], r.rotation[j], r.body[i].x, r.body[j].x, branch);
                if (laneId() == 0) {
                    r.dpairPlane[d] = plane;
                    r.dpairSourcePlane[2 * d] = source.plane;
                    r.dpairSourcePlane[2 * d + 1] = source.scale;
                }
            }
            for (uint32_t k0 = 0; k0 < li.y; k0 += WARP) {
                // Lane per leaf: the cheap tests (target root box, source-frame
                // plane); then, for each leaf still in, the whole warp tests the
                // hull group's planes in parallel.  Every test is a conservative
                // "may contact", so their order does not matter.
                uint32_t k = k0 + laneId();
                bool open = false;
                f3 centre = mk(0.f, 0.f, 0.f), half = centre;
                uint32_t group = 0;
                if (k < li.y) {
                    uint32_t leaf = __ldg(&r.meshLeaves[li.x + k]);
                    f3 low, high;
                    meshPairBounds(r, d, leaf, low, high, margin);
                    open = meshBoxGroup(r, targetShape, low, high, centre, half, group) &&
                           !leafBeyondSourcePlane(source, xyz(__ldg(&r.meshClusterMin[leaf])),
                                                  xyz(__ldg(&r.meshClusterMax[leaf])), grow);
                }
                uint32_t pending = __ballot_sync(0xffffffffu, open), m = 0;
                while (pending) {
                    uint32_t lane = __ffs(pending) - 1;
                    pending &= pending - 1;
                    f3 cl = mk(__shfl_sync(0xffffffffu, centre.x, lane), __shfl_sync(0xffffffffu, centre.y, lane),
                               __shfl_sync(0xffffffffu, centre.z, lane));
                    f3 hl = mk(__shfl_sync(0xffffffffu, half.x, lane), __shfl_sync(0xffffffffu, half.y, lane),
                               __shfl_sync(0xffffffffu, half.z, lane));
                    uint4 info = __ldg(&r.meshHullInfo[6 * targetShape + __shfl_sync(0xffffffffu, group, lane)]);
                    bool outside = false;
                    for (uint32_t q = laneId(); q < info.y; q += WARP) {
                        float4 plane = __ldg(&r.meshPlanes[info.x + q]);
                        outside |= __fsub_rn(__fadd_rn(dot(xyz(plane), cl), plane.w), dot(abs3(xyz(plane)), hl)) > 0;
                    }
                    if (!__any_sync(0xffffffffu, outside)) m |= 1u << lane;
                }
                if (laneId() == 0) r.leafMask[size_t(d) * c.leafWords + k0 / WARP] = m;
                count += __popc(m);
            }
        }
        if (laneId() == 0) r.dpairLeafCount[d] = count;
    }
}
__global__ void k_leafEmit(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0 || r.work[W_FILTER] == 0) return;
    uint32_t n = 2 * activePairs(r, c);
    for (uint32_t d = warpGlobal(); d < n; d += warpStride()) {
        if (r.dpairLeafCount[d] == 0) continue;
        uint32_t p = d >> 1, pass = d & 1;
        uint2 ij = r.pairs[p];
        uint32_t i = pass ? ij.y : ij.x;
        uint4 li = __ldg(&r.meshLeafInfo[r.shapeId[i]]);
        uint32_t base = r.dpairCandOffset[d];
        for (uint32_t k0 = 0; k0 < li.y; k0 += WARP) {
            uint32_t m = r.leafMask[size_t(d) * c.leafWords + k0 / WARP];
            uint32_t k = k0 + laneId();
            if ((m >> laneId()) & 1u) {
                uint32_t slot = base + __popc(m & lanesBelow());
                if (slot < c.candidateCapacity) r.candidates[slot] = make_uint2(d, __ldg(&r.meshLeaves[li.x + k]));
            }
            base += __popc(m);
        }
    }
}
// Node query in stages.  The filter stage (one warp per (directed pair,
// leaf) item, two nodes per lane) applies the one-dot enclosure-plane test
// in the source frame and records each item's surviving nodes as a 64-bit
// mask.  A scan turns the survivor counts into offsets and the survivors are
// listed in canonical order.  A dense pass (one thread per survivor) places
// each in the target frame and applies the target-frame plane and the hull;
// with the learned culler on, a second pass evaluates the target's network
// for 64 survivors per warp on tensor cores.  A scan keeps the survivors no
// test ruled out and the exact stage runs one thread per kept survivor: full
// warps of BVH walks instead of warps in which most lanes were rejected and
// idle.  Each hit sets its bit in
// the item's hit mask (integer atomics: the result does not depend on their
// order) and keeps its record in the survivor's scratch slot; the emit pass
// copies hits to their canonical offsets.
__global__ void __launch_bounds__(256) k_nodeFilter(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t n = min(r.work[W_CANDIDATES], c.candidateCapacity);
    // Stored survivors serve this step (their hit masks were cleared by the
    // previous step's emit).
    if (r.work[W_FILTER] == 0) return;
    float grow = __fmul_rn(1.001f, buildMargin(r, c));
    // Two items per warp, one per half-warp, four node slots per lane
    // (slot = lane in half + 16 j): twice the loads in flight per instruction.
    uint32_t half = laneId() >> 4, hl = laneId() & 15u;
    for (uint32_t pair0 = 2 * warpGlobal(); pair0 < n; pair0 += 2 * warpStride()) {
        uint32_t item = pair0 + half;
        bool keep[4] = {false, false, false, false};
        if (item < n && r.control[0] == 0) {
            uint2 cd = r.candidates[item];
            uint32_t d = cd.x, p = d >> 1, pass = d & 1;
            uint2 ij = r.pairs[p];
            uint32_t src = pass ? ij.y : ij.x;
            SourcePlane source{r.dpairSourcePlane[2 * d], r.dpairSourcePlane[2 * d + 1]};
            uint4 range = __ldg(&r.meshClusterRanges[cd.y]);
            const float4* samples = r.sample + __ldg(&r.sampleInfo[r.shapeId[src]].x);
            // One dot per node against the source-frame plane; the exact
            // placement, target-frame plane and hull follow in a dense pass.
            float4 x[4];
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j) {
                uint32_t k = hl + 16 * j;
                x[j] = k < range.y ? __ldg(&samples[__ldg(&r.meshSampleIndices[range.x + k])])
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j)
                keep[j] = hl + 16 * j < range.y && !nodeBeyondSourcePlane(source, xyz(x[j]), grow);
        }
        uint32_t b[4];
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j) b[j] = __ballot_sync(0xffffffffu, keep[j]);
        if (hl == 0 && item < n) {
            uint32_t sh = 16 * half;
            uint32_t m0 = ((b[0] >> sh) & 0xFFFFu) | (((b[1] >> sh) & 0xFFFFu) << 16);
            uint32_t m1 = ((b[2] >> sh) & 0xFFFFu) | (((b[3] >> sh) & 0xFFFFu) << 16);
            r.candSurvMask[item] = make_uint2(m0, m1);
            r.candSurvCount[item] = __popc(m0) + __popc(m1);
            r.candHitMask[item] = make_uint2(0u, 0u);
            r.candHitCount[item] = 0;
        }
    }
}
// Source node, partner and target-frame position of survivor s (the same
// expressions as nodePrefilter: the same arm and local bits).
struct SurvivorNode {
    uint32_t item, slot, src, dst, node;
    f3 arm, local;
};
__device__ __forceinline__ SurvivorNode survivorNode(const Res& r, uint32_t s) {
    SurvivorNode v;
    uint2 sv = r.survivors[s];
    v.item = sv.x;
    v.slot = sv.y;
    uint2 cd = r.candidates[sv.x];
    uint32_t d = cd.x, p = d >> 1, pass = d & 1;
    uint2 ij = r.pairs[p];
    v.src = pass ? ij.y : ij.x;
    v.dst = pass ? ij.x : ij.y;
    v.node = __ldg(&r.meshSampleIndices[__ldg(&r.meshClusterRanges[cd.y]).x + sv.y]);
    float4 sp = __ldg(&r.sample[__ldg(&r.sampleInfo[r.shapeId[v.src]].x) + v.node]);
    v.arm = qrot(r.rotation[v.src], xyz(sp) * r.body[v.src].x);
    v.local = qinv(r.rotation[v.dst], v.arm - xyz(r.dpairBranch[d])) / r.body[v.dst].x;
    return v;
}
// Exact placement, target-frame enclosure plane and hull of every survivor
// of the one-dot test (nodePrefilter, one thread each): survKeep[s] = 1 for
// the nodes that go on to the exact query.
// When the exact-query list is stored with the filter results, this pass
// runs only on build steps, with the plane, hull and grid tests grown by the
// margin (a node the grid bounds farther than the margin from the surface
// cannot reach it while the results serve).
__global__ void __launch_bounds__(256) k_survivorPrefilter(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    bool stored = storedKeep(c);
    if (r.control[0] != 0 || (stored && r.work[W_FILTER] == 0)) return;
    float grow = stored ? __fmul_rn(1.001f, buildMargin(r, c)) : 0.0f;
    uint32_t n = min(r.work[W_SURVIVORS], c.survivorCapacity);
    for (uint32_t s = gtid(); s < n; s += gstride()) {
        uint2 sv = r.survivors[s];
        uint2 cd = r.candidates[sv.x];
        uint32_t d = cd.x, p = d >> 1, pass = d & 1;
        uint2 ij = r.pairs[p];
        uint32_t src = pass ? ij.y : ij.x, dst = pass ? ij.x : ij.y;
        uint32_t node = __ldg(&r.meshSampleIndices[__ldg(&r.meshClusterRanges[cd.y]).x + sv.y]);
        float4 plane = r.dpairPlane[d];
        f3 arm, local;
        bool keep = nodePrefilter(r, src, dst, node, xyz(r.dpairBranch[d]), &plane, arm, local, grow);
        // A node certified outside the target by the distance-bound grid
        // cannot be a contact (the exact query would find phi > 0).
        if (keep && c.distanceGridEnabled && distanceBound(r, r.shapeId[dst], local) > grow) keep = false;
        r.survKeep[s] = keep ? 1u : 0u;
        if (keep && stored) {
            uint32_t bucket = walkBucket(r, r.shapeId[dst], local);
            r.walkKey[s] = bucket;
            atomicAdd(&r.walkBucketCount[bucket], 1u);
        }
    }
}
// Distance-bound grid of every shape (built once per library): one thread per
// cell evaluates the exact signed distance at the cell centre (meshDistance,
// the query the contacts use) and stores phi - (half diagonal) x 1.001 -
// 1e-5 (1 + |centre|_1).  The grid spans the shape's root box with cubic
// cells of edge (largest box extent) / GRID.
__global__ void k_distanceGrid(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    const uint32_t cells = GRID * GRID * GRID;
    for (uint32_t t = gtid(); t < c.shapes * cells; t += gstride()) {
        uint32_t shape = t / cells, cell = t % cells;
        uint32_t root = __ldg(&r.meshRoots[shape].x);
        f3 low = xyz(__ldg(&r.meshMin[root])), high = xyz(__ldg(&r.meshMax[root]));
        f3 extent = high - low;
        float h = __fdiv_rn(mx(mx(extent.x, extent.y), extent.z), float(GRID));
        if (cell == 0) r.distanceGridInfo[shape] = w4(low, h);
        uint32_t gx = cell % GRID, gy = (cell / GRID) % GRID, gz = cell / (GRID * GRID);
        f3 centre = low + mk(__fmul_rn(float(gx) + 0.5f, h), __fmul_rn(float(gy) + 0.5f, h),
                             __fmul_rn(float(gz) + 0.5f, h));
        uint32_t nearest;
        float phi = meshDistance(r, shape, centre, false, 0xFFFFFFFFu, &nearest).w;
        r.distanceGridTriangle[t] = nearest;
        float reach = __fmul_rn(__fmul_rn(0.8660254f, h), 1.001f);
        float slack = __fmul_rn(1e-5f, __fadd_rn(1.0f, __fadd_rn(__fadd_rn(fabsf(centre.x), fabsf(centre.y)),
                                                                 fabsf(centre.z))));
        r.distanceGrid[t] = __fsub_rn(__fsub_rn(phi, reach), slack);
    }
}
// Learned culler over the kept survivors, on the tensor cores (culler.cuh).
// The survivors are first sorted by target shape (a counting sort into
// walkKey: per-shape counts, their scan, then placement -- the walk-bucket
// arrays and walkKey serve the stored exact-query list only, which the
// culler does not use), so that a 128-row tile holds one shape, or a few at
// its ends.  The culler clears keep[s] when the target's network places a
// kept survivor s beyond the shape's calibrated margin; the exact query
// decides every other one.  The order of the sorted list within a shape is
// immaterial: each row's prediction depends on its own point only.
__device__ __forceinline__ uint32_t survivorTargetShape(const Res& r, const Config& c, uint32_t s) {
    uint2 sv = r.survivors[s];
    uint32_t d = r.candidates[sv.x].x;
    uint2 ij = r.pairs[d >> 1];
    uint32_t shape = r.shapeId[(d & 1) ? ij.x : ij.y];
    return shape < c.shapes ? shape : EMPTY;
}
// Per-shape counts of the kept survivors (walkBucketCount[shape]; zero on
// entry: the placement below takes each back to zero).
__global__ void k_cullCount(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t n = min(r.work[W_SURVIVORS], c.survivorCapacity);
    for (uint32_t s = gtid(); s < n; s += gstride()) {
        uint32_t shape = r.survKeep[s] ? survivorTargetShape(r, c, s) : EMPTY;
        uint32_t same = __match_any_sync(__activemask(), shape);
        if (shape != EMPTY && laneId() == uint32_t(__ffs(same) - 1)) atomicAdd(&r.walkBucketCount[shape], __popc(same));
    }
}
// Placement in shape order (walkKey); each count returns to zero.
__global__ void k_cullPlace(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t n = min(r.work[W_SURVIVORS], c.survivorCapacity);
    for (uint32_t s = gtid(); s < n; s += gstride()) {
        uint32_t shape = r.survKeep[s] ? survivorTargetShape(r, c, s) : EMPTY;
        uint32_t same = __match_any_sync(__activemask(), shape);
        uint32_t leader = __ffs(same) - 1, base = 0;
        if (shape != EMPTY && laneId() == leader) base = atomicSub(&r.walkBucketCount[shape], __popc(same));
        base = __shfl_sync(same, base, leader);
        if (shape != EMPTY) {
            uint32_t rank = __popc(same & lanesBelow());
            r.walkKey[r.walkBucketOffset[shape] + base - 1 - rank] = s;
        }
    }
}
__global__ void __launch_bounds__(CULLER_ROWS) k_cullSurvivors(const __grid_constant__ Params P) {
    __shared__ CullerShared sh;
    __shared__ uint32_t live, tested, culled;
    const Res& r = P.r;
    const Config& c = P.c;
    if (threadIdx.x == 0) {
        live = r.control[0] == 0;
        tested = culled = 0;
    }
    cullerBegin(sh);  // synchronizes
    uint32_t phase = 0;
    uint32_t n = live ? min(r.work[W_CULL_ROWS], c.survivorCapacity) : 0u;
    uint32_t tiles = (n + CULLER_ROWS - 1) / CULLER_ROWS;
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        uint32_t i = t * CULLER_ROWS + threadIdx.x, s = EMPTY, shape = EMPTY;
        f3 local = mk(0.f, 0.f, 0.f);
        float margin = 0.0f;
        if (i < n) {
            s = r.walkKey[i];
            SurvivorNode v = survivorNode(r, s);
            local = v.local;
            shape = r.shapeId[v.dst];
            uint32_t root = __ldg(&r.meshRoots[shape].x);
            margin = r.cullerMargin[size_t(shape) * CULLER_MARGINS + 1 +
                                    cullerCell(__ldg(&r.meshMin[root]), __ldg(&r.meshMax[root]), local)];
        }
        float y;
        if (!cullerTile(sh, r.cullerParams, r.cullerW1, shape, local, phase, y)) {
            if (threadIdx.x == 0) fail(r, F_WAIT);
            break;
        }
        if (shape != EMPTY) {
            atomicAdd(&tested, 1u);
            if (y > margin) {
                r.survKeep[s] = 0u;
                atomicAdd(&culled, 1u);
            }
        }
    }
    cullerEnd(sh, phase);  // synchronizes
    if (threadIdx.x == 0 && tested) {
        atomicAdd(&r.cullerStats[0], tested);
        atomicAdd(&r.cullerStats[1], culled);
    }
}
// Survivors kept for the exact query (their survivor indices): in survivor
// order, or, when the list is stored with the filter results, grouped by
// walk bucket (each bucket filled from its end; the order within a bucket
// is immaterial: every walk is independent and its hit lands in its
// survivor's slot).
__global__ void k_walkList(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    bool stored = storedKeep(c);
    if (r.control[0] != 0 || (stored && r.work[W_FILTER] == 0)) return;
    uint32_t n = min(r.work[W_SURVIVORS], c.survivorCapacity);
    if (stored && gtid() == 0) r.work[W_DORMANT] = 0;  // a new list: no slot sleeps yet
    for (uint32_t s = gtid(); s < n; s += gstride()) {
        if (!r.survKeep[s]) continue;
        if (stored) {
            uint32_t bucket = r.walkKey[s];
            uint32_t slot = r.walkBucketOffset[bucket] + atomicSub(&r.walkBucketCount[bucket], 1u) - 1u;
            r.walkList[slot] = s;
            r.walkCertTriangle[slot] = make_uint2(EMPTY, EMPTY);
            // The slot's node record: what its exact query reads every step
            // (one load instead of the survivor -> item -> pair -> sample chain).
            uint2 sv = r.survivors[s];
            uint2 cd = r.candidates[sv.x];
            uint2 ij = r.pairs[cd.x >> 1];
            uint32_t src = (cd.x & 1) ? ij.y : ij.x, dst = (cd.x & 1) ? ij.x : ij.y;
            uint32_t node = __ldg(&r.meshSampleIndices[__ldg(&r.meshClusterRanges[cd.y]).x + sv.y]);
            r.walkNode[slot] = make_uint4(src, dst, cd.x, __ldg(&r.sampleInfo[r.shapeId[src]].x) + node);
            r.walkItem[slot] = sv;
        } else {
            r.walkList[r.keepOffset[s]] = s;
        }
    }
}
// Survivor list in canonical (item, node slot) order.
// On a build step with a margin, it also marks the stored results complete
// when no list overflowed.
__global__ void k_survivorList(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0 || r.work[W_FILTER] == 0) return;
    uint32_t n = min(r.work[W_CANDIDATES], c.candidateCapacity);
    if (gtid() == 0 && c.filterMargin > 0.0f)
        r.work[W_FILTER_VALID] = r.work[W_CANDIDATES] <= c.candidateCapacity && r.work[W_SURVIVORS] <= c.survivorCapacity;
    for (uint32_t item = warpGlobal(); item < n; item += warpStride()) {
        uint2 m = r.candSurvMask[item];
        if ((m.x | m.y) == 0) continue;
        uint32_t base = r.candSurvOffset[item];
#pragma unroll
        for (uint32_t half = 0; half < 2; ++half) {
            uint32_t word = half ? m.y : m.x;
            if (!((word >> laneId()) & 1u)) continue;
            uint32_t s = base + (half ? __popc(m.x) : 0) + __popc(word & lanesBelow());
            if (s < c.survivorCapacity) r.survivors[s] = make_uint2(item, laneId() + half * WARP);
            else fail(r, F_CONTACT);
        }
    }
}
// Exact query, one thread per kept survivor.
__device__ __forceinline__ void recordHitAt(const Res& r, uint32_t s, uint32_t item, uint32_t slot, float4 pd,
                                            float4 na) {
    r.hitScratch[2 * s] = pd;
    r.hitScratch[2 * s + 1] = na;
    atomicOr(slot < WARP ? &r.candHitMask[item].x : &r.candHitMask[item].y, 1u << (slot & 31u));
    atomicAdd(&r.candHitCount[item], 1u);
}
__device__ __forceinline__ void recordHit(const Res& r, uint32_t s, const SurvivorNode& v, float4 pd, float4 na) {
    recordHitAt(r, s, v.item, v.slot, pd, na);
}
// A stored walk slot's node, placed in the target frame from its record:
// the same expressions as survivorNode (the same arm and local bits).
struct WalkNode {
    uint4 rec;  // source, target, directed pair, packed sample
    float4 sp, bs, bd, qd;
    f3 arm, local;
};
__device__ __forceinline__ WalkNode walkNode(const Res& r, uint32_t t) {
    WalkNode w;
    w.rec = r.walkNode[t];
    w.sp = __ldg(&r.sample[w.rec.w]);
    w.bs = r.body[w.rec.x];
    w.bd = r.body[w.rec.y];
    w.qd = r.rotation[w.rec.y];
    float4 qs = r.rotation[w.rec.x];
    f3 branch = xyz(r.dpairBranch[w.rec.z]);
    w.arm = qrot(qs, xyz(w.sp) * w.bs.x);
    w.local = qinv(w.qd, w.arm - branch) / w.bd.x;
    return w;
}
// Exact queries of a list built every step (margin 0 or the learned culler):
// one seeded walk per node.
__global__ void __launch_bounds__(256) k_nodeWalk(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t n = min(r.work[W_KEPT], c.survivorCapacity);
    for (uint32_t t = gtid(); t < n; t += gstride()) {
        uint32_t s = r.walkList[t];
        SurvivorNode v = survivorNode(r, s);
        float4 pd, na;
        uint32_t shape = r.shapeId[v.dst];
        // Seed the walk with the triangle nearest to the node's grid cell.
        float4 f = meshDistance(r, shape, v.local, false, gridSeed(r, shape, v.local));
        if (nodeContactFrom(r, c, v.src, v.dst, v.node, v.arm, f, pd, na)) recordHit(r, s, v, pd, na);
    }
}
// Exact queries of a stored list.  A stored list keeps its slots from step
// to step, and each slot keeps a certificate: the nearest triangle T found by
// a certifying walk at the point p0, and a gap g below which no other
// triangle's distance lies above T's.  Distances are 1-Lipschitz in the
// point, so while 2 |p - p0| + slack < g, T is still the unique nearest
// triangle at p and the walk would record it with the values closestTriangle
// gives for it: the step evaluates T alone (with its partner or tie, where it
// has one).  The slack, 4e-6 (1 + |p|_1), covers the FP32 rounding of the
// distances: with e the largest difference between a computed triangle
// distance and the exact one (a few units in the last place of |p|, about
// 3e-7 (1 + |p|) here), the other triangles stay strictly farther while
// 2 |p - p0| + 4e = g; the slack is above 4e.  A dormant slot is skipped: its node cannot touch the target
// before the stored results are built again.  The other slots are flagged
// (survKeep, unused by a stored list while it is walked), listed in slot
// order -- the walk-bucket order, so that a warp's walks stay coherent -- and
// walked by k_nodeWalkSlow in full warps.
__global__ void __launch_bounds__(256) k_nodeWalkKnown(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t n = min(r.work[W_KEPT], c.survivorCapacity);
    for (uint32_t t = gtid(); t < n; t += gstride()) {
        uint2 cert = r.walkCertTriangle[t];
        uint32_t triangle = cert.x;
        bool known = false;
        if (triangle == DORMANT) {
            known = true;
        } else if (triangle != EMPTY) {
            // Every load below depends only on the slot: they issue together.
            uint32_t base = 3 * (triangle & 0x3FFFFFFFu);
            float4 ta = __ldg(&r.meshTriangles[base]), tb = __ldg(&r.meshTriangles[base + 1]),
                   tc = __ldg(&r.meshTriangles[base + 2]);
            float4 cp = r.walkCertPoint[t];
            WalkNode w = walkNode(r, t);
            float slack = __fmul_rn(4e-6f, __fadd_rn(1.0f, __fadd_rn(__fadd_rn(fabsf(w.local.x), fabsf(w.local.y)),
                                                                    fabsf(w.local.z))));
            known = __fadd_rn(__fmul_rn(2.002f, length(w.local - xyz(cp))), slack) < cp.w;
            if (known) {
                float4 pd, na;
                float4 f = meshDistanceAt(r, w.local, triangle, cert.y, ta, tb, tc, known);
                if (known && nodeContactWith(r, c, w.rec.x, w.sp, w.bs, w.bd, w.qd, w.arm, f, pd, na)) {
                    uint2 it = r.walkItem[t];
                    recordHitAt(r, r.walkList[t], it.x, it.y, pd, na);
                }
            }
        }
        r.survKeep[t] = known ? 0u : 1u;
    }
}
// Dormant slots.  Until the next build, the motion check of k_pairSetup
// bounds chord_i r_i + |d branch| + chord_j r_j by m s_j (chord: of a
// grain's rotation since the build; r: bounding radius; s: scale), so a node
// inside the target's bounding sphere -- as every node touching it is --
// lies within m (target frame, unscaled) of where it was at the build, and
// a node at distance |v| from the target's centre now lies within
// m max(1, |v| / r_j) of it.  A node farther outside than the sum (times
// 1.001, plus the distance rounding slack) cannot touch the target before
// the next build, and its slot sleeps.
// One slot's certifying walk (by its warp when `Warp`; lane 0 records).
template <bool Warp>
__device__ __forceinline__ void certifySlot(const Res& r, const Config& c, uint32_t t, float margin, float reach,
                                            const float4* children, uint32_t nodeBase, const float4* triangles,
                                            uint32_t triangleBase) {
    WalkNode w = walkNode(r, t);
    uint32_t shape = r.shapeId[w.rec.y], triangle, tie;
    float gap;
    float4 f = meshDistanceCertifiedT<Warp>(r, shape, w.local, gridSeed(r, shape, w.local), reach, triangle, tie, gap,
                                            children, nodeBase, triangles, triangleBase);
    if (Warp && laneId() != 0) return;
    float slack = __fmul_rn(2e-5f, __fadd_rn(1.0f, __fadd_rn(__fadd_rn(fabsf(w.local.x), fabsf(w.local.y)),
                                                             fabsf(w.local.z))));
    float reachNow = fmaxf(1.0f, __fdiv_rn(__fmul_rn(length(w.local), w.bd.x), w.bd.z));
    float sleep = __fmul_rn(__fmul_rn(1.001f, margin), __fadd_rn(1.0f, reachNow));
    bool dormant = triangle != EMPTY && f.w > __fadd_rn(sleep, slack);
    if (dormant) {
        // One count per group of lanes marking slots together.
        uint32_t group = __activemask();
        if (laneId() == uint32_t(__ffs(group) - 1)) atomicAdd(&r.work[W_DORMANT], uint32_t(__popc(group)));
    }
    r.walkCertTriangle[t] = dormant ? make_uint2(DORMANT, EMPTY) : make_uint2(triangle, tie);
    r.walkCertPoint[t] = w4(w.local, gap);
    float4 pd, na;
    if (nodeContactWith(r, c, w.rec.x, w.sp, w.bs, w.bd, w.qd, w.arm, f, pd, na)) {
        uint2 it = r.walkItem[t];
        recordHitAt(r, r.walkList[t], it.x, it.y, pd, na);
    }
}
// A certifying walk for each listed slot, recording its new certificate.
// Few walks (up to two per warp of the grid) run a warp each; more run a
// lane each, in 32-slot runs of the list (coherent walks) dealt to the
// blocks in turn, so that either way they spread over every SM.  Only a
// list longer than `above` is walked here (k_nodeWalkStaged takes the
// shorter ones; 0: every list).
__global__ void __launch_bounds__(256) k_nodeWalkSlow(const __grid_constant__ Params P, uint32_t above) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t n = min(r.work[W_SLOW], c.survivorCapacity);
    if (n <= above && above != 0) return;
    if (gtid() == 0) r.work[W_CERTIFIED] += min(r.work[W_KEPT], c.survivorCapacity) - n;
    float margin = __uint_as_float(r.work[W_FILTER_MARGIN]);
    float reach = __fadd_rn(__fmul_rn(2.01f, margin), 1e-4f);
    uint32_t warps = gridDim.x * (blockDim.x >> 5), warp = blockIdx.x + gridDim.x * (threadIdx.x >> 5);
    if (n <= 2 * warps) {
        for (uint32_t i = warp; i < n; i += warps)
            certifySlot<true>(r, c, r.walkKey[i], margin, reach, r.meshChildren, 0u, r.meshTriangles, 0u);
    } else {
        for (uint32_t i = 32 * warp + laneId(); i < n; i += 32 * warps)
            certifySlot<false>(r, c, r.walkKey[i], margin, reach, r.meshChildren, 0u, r.meshTriangles, 0u);
    }
}
// The same walks with each target shape's BVH node records staged in shared
// memory.  The slow list is in walk-bucket order, so each shape's walks form
// one run of it (from the scan of the flags at the shape's first bucket to
// the scan at the next shape's); the runs are cut into units of one shape,
// dealt to the CTAs in turn.  A CTA copies its unit's shape records (one
// 64-byte record per node, up to STAGE_BYTES) into shared memory by bulk
// asynchronous copies completing on an mbarrier -- once per change of shape
// -- and walks the unit: a warp per walk when the step has few walks, a lane
// per walk otherwise.  Internal node visits then read shared memory instead
// of L2; leaves read their triangles from the library as before.  A shape
// whose records exceed the stage is walked from the library by the same CTA.
constexpr uint32_t STAGE_THREADS = 512;
constexpr uint32_t STAGE_BYTES = 192u << 10;
constexpr uint32_t STAGE_MAX_SHAPES = 4096;
constexpr uint32_t STAGE_CHUNK = 16u << 10;
// The staged kernel runs one CTA per SM and takes lists of up to two walks
// per warp of its grid; longer lists go to k_nodeWalkSlow (a lane per walk,
// full occupancy), which hides the walks' load latency better there.
__device__ __forceinline__ uint32_t smemAddress(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ bool mbarrierWait(uint32_t bar, uint32_t parity) {
    // Bounded: about 2^22 polls (far beyond a 192 KB copy), then give up.
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
__global__ void __launch_bounds__(STAGE_THREADS, 1) k_nodeWalkStaged(const __grid_constant__ Params P) {
    extern __shared__ __align__(128) unsigned char stageMemory[];
    float4* stage = reinterpret_cast<float4*>(stageMemory);
    uint32_t* unitStart = reinterpret_cast<uint32_t*>(stageMemory + STAGE_BYTES);  // shapes + 1
    __shared__ __align__(8) uint64_t barrier;
    __shared__ uint32_t warpTotals[STAGE_THREADS / 32], carry, liveFlag, triangleFirst, triangleEnd;
    const Res& r = P.r;
    const Config& c = P.c;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warpId = tid >> 5, warps = STAGE_THREADS / 32;
    if (tid == 0) liveFlag = r.control[0] == 0 ? 1u : 0u;
    __syncthreads();
    if (!liveFlag) return;  // block-uniform
    uint32_t n = min(r.work[W_SLOW], c.survivorCapacity);
    if (n > 2u * gridDim.x * warps) return;  // a long list: k_nodeWalkSlow walks it
    if (blockIdx.x == 0 && tid == 0) r.work[W_CERTIFIED] += min(r.work[W_KEPT], c.survivorCapacity) - n;
    if (n == 0) return;
    float margin = __uint_as_float(r.work[W_FILTER_MARGIN]);
    float reach = __fadd_rn(__fmul_rn(2.01f, margin), 1e-4f);
    // Walks per unit: one or two per warp, so that the units spread over
    // every CTA.
    uint32_t per = n <= gridDim.x * warps ? warps : 2u * warps;
    // Units per shape, scanned into unitStart (exclusive; unitStart[shapes] = total).
    if (tid == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < c.shapes; base += STAGE_THREADS) {
        uint32_t s = base + tid, units = 0;
        if (s < c.shapes) {
            uint32_t lo = r.keepOffset[r.walkBucketOffset[s * WALK_BUCKETS]];
            uint32_t hi = r.keepOffset[r.walkBucketOffset[(s + 1) * WALK_BUCKETS]];
            units = (hi - lo + per - 1) / per;
        }
        uint32_t x = units;
#pragma unroll
        for (uint32_t d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) warpTotals[warpId] = x;
        __syncthreads();
        if (warpId == 0) {
            uint32_t t = lane < warps ? warpTotals[lane] : 0u;
#pragma unroll
            for (uint32_t d = 1; d < 32; d <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, t, d);
                if (lane >= d) t += y;
            }
            if (lane < warps) warpTotals[lane] = t;  // inclusive over warps
        }
        __syncthreads();
        uint32_t before = carry + (warpId ? warpTotals[warpId - 1] : 0u) + x - units;
        if (s < c.shapes) unitStart[s] = before;
        __syncthreads();
        if (tid == 0) carry += warpTotals[warps - 1];
        __syncthreads();
    }
    if (tid == 0) unitStart[c.shapes] = carry;
    uint32_t bar = smemAddress(&barrier);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    uint32_t total = unitStart[c.shapes], phase = 0, staged = EMPTY, stagedFirst = 0;
    bool stalled = false, trianglesStaged = false;  // the same on every thread
    for (uint32_t u = blockIdx.x; u < total && !stalled; u += gridDim.x) {
        // The unit's shape: the last s with unitStart[s] <= u.
        uint32_t lo = 0, hi = c.shapes;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (unitStart[mid] <= u) lo = mid; else hi = mid;
        }
        uint32_t shape = lo;
        uint32_t first = r.keepOffset[r.walkBucketOffset[shape * WALK_BUCKETS]] + (u - unitStart[shape]) * per;
        uint32_t last = min(first + per, r.keepOffset[r.walkBucketOffset[(shape + 1) * WALK_BUCKETS]]);
        uint4 nodes = __ldg(&r.meshRoots[shape]);
        uint32_t bytes = (nodes.y - nodes.x) * 64u;
        bool fits = bytes <= STAGE_BYTES;
        if (fits && staged != shape) {
            __syncthreads();  // every warp is done with the staged shape
            if (tid == 0) {
                triangleFirst = EMPTY;
                triangleEnd = 0;
                // The async proxy overwrites what the generic proxy read.
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
                const char* from = reinterpret_cast<const char*>(r.meshChildren + 4 * size_t(nodes.x));
                uint32_t to = smemAddress(stage);
                for (uint32_t off = 0; off < bytes; off += STAGE_CHUNK) {
                    uint32_t size = min(STAGE_CHUNK, bytes - off);
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                        ::"r"(to + off), "l"(from + off), "r"(size), "r"(bar)
                        : "memory");
                }
            }
            if (!mbarrierWait(bar, phase)) {
                fail(r, F_WAIT);
                stalled = true;  // block-uniform only if every thread timed out: re-checked below
            }
            phase ^= 1u;
            staged = shape;
            // Every thread leaves together if any thread gave up.
            stalled = __syncthreads_or(stalled);
            if (stalled) break;
            // The shape's triangles: the range its leaves reference (a
            // reduction over the staged records), staged after the records
            // when both fit.
            for (uint32_t k = tid; k < nodes.y - nodes.x; k += STAGE_THREADS) {
                float4 head = stage[4 * k];
                if (__float_as_uint(head.w) == LEAF_MARK) {
                    atomicMin(&triangleFirst, __float_as_uint(head.x));
                    atomicMax(&triangleEnd, __float_as_uint(head.x) + __float_as_uint(head.y));
                }
            }
            __syncthreads();
            stagedFirst = triangleFirst;
            uint32_t triangleBytes = triangleEnd > stagedFirst ? (triangleEnd - stagedFirst) * 48u : 0u;
            trianglesStaged = triangleBytes != 0 && bytes + triangleBytes <= STAGE_BYTES;
            if (trianglesStaged) {
                if (tid == 0) {
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(triangleBytes)
                                 : "memory");
                    const char* from = reinterpret_cast<const char*>(r.meshTriangles + 3 * size_t(stagedFirst));
                    uint32_t to = smemAddress(stage) + bytes;
                    for (uint32_t off = 0; off < triangleBytes; off += STAGE_CHUNK) {
                        uint32_t size = min(STAGE_CHUNK, triangleBytes - off);
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                            ::"r"(to + off), "l"(from + off), "r"(size), "r"(bar)
                            : "memory");
                    }
                }
                if (!mbarrierWait(bar, phase)) {
                    fail(r, F_WAIT);
                    stalled = true;
                }
                phase ^= 1u;
                stalled = __syncthreads_or(stalled);
                if (stalled) break;
            }
        }
        const float4* children = fits ? stage : r.meshChildren;
        uint32_t base = fits ? nodes.x : 0u;
        bool local = fits && trianglesStaged;
        const float4* triangles = local ? stage + 4 * size_t(nodes.y - nodes.x) : r.meshTriangles;
        uint32_t triangleBase = local ? stagedFirst : 0u;
        for (uint32_t i = first + warpId; i < last; i += warps)
            certifySlot<true>(r, c, r.walkKey[i], margin, reach, children, base, triangles, triangleBase);
    }
    if (stalled && tid == 0) {
        // A copy may still be landing: wait for it (bounded) before the
        // shared memory is released.
        mbarrierWait(bar, phase ^ 1u);
    }
}
// L2 prefetch, first in a step, of what the step's exact queries read
// through chains of dependent loads: the packed library (BVH node records,
// triangles, pseudonormals, node samples) and, with a stored exact-query
// list, its per-slot certificates and node records.  One bulk copy-engine
// prefetch (cp.async.bulk.prefetch.L2) per 16 KB, from two CTAs per SM: the
// lines arrive while the drift, neighbour and pair kernels run, instead of
// one latency at a time inside the walks (64 KB pieces from four CTAs took
// longer than the walks saved).  A hint only: nothing waits for it and no result
// depends on it.  Every range starts 16-byte aligned (float4/uint4/uint2
// arrays from the allocator) and is cut to a multiple of 16 bytes.
__global__ void k_prefetch(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    constexpr uint32_t CHUNK = 16u << 10;
    uint32_t kept = storedKeep(c) ? min(r.work[W_KEPT], c.survivorCapacity) : 0u;
    const void* base[9] = {r.meshChildren, r.meshTriangles, r.meshNormals, r.sample, r.walkCertTriangle,
                           r.walkCertPoint, r.walkNode, r.walkItem, r.walkList};
    uint64_t size[9] = {16ull * c.library16[0], 16ull * c.library16[1], 16ull * c.library16[2],
                        16ull * c.library16[3], 8ull * kept, 16ull * kept, 16ull * kept, 8ull * kept, 4ull * kept};
    uint32_t chunk = gtid();
    for (int k = 0; k < 9; ++k) {
        uint64_t bytes = size[k] & ~uint64_t(15);
        uint64_t chunks = (bytes + CHUNK - 1) / CHUNK;
        for (; chunk < chunks; chunk += gstride()) {
            uint64_t offset = uint64_t(chunk) * CHUNK;
            uint64_t left = bytes - offset;
            uint32_t n = left < CHUNK ? uint32_t(left) : CHUNK;
            const char* at = static_cast<const char*>(base[k]) + offset;
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(at), "r"(n) : "memory");
        }
        chunk -= uint32_t(chunks);
    }
}
// Emits one item's hits (the warp, lane per node slot of each 32-slot half).
__device__ __forceinline__ void emitItem(const Res& r, const Config& c, uint32_t item, uint2 m) {
    uint2 cd = r.candidates[item];
    uint32_t d = cd.x, p = d >> 1, pass = d & 1;
    uint2 ij = r.pairs[p];
    uint32_t src = pass ? ij.y : ij.x, dst = pass ? ij.x : ij.y;
    uint4 range = __ldg(&r.meshClusterRanges[cd.y]);
    uint2 sm = r.candSurvMask[item];
    uint32_t out = r.candHitOffset[item], in = r.candSurvOffset[item];
#pragma unroll
    for (uint32_t half = 0; half < 2; ++half) {
        uint32_t word = half ? m.y : m.x;
        if (!((word >> laneId()) & 1u)) continue;
        uint32_t rank = (half ? __popc(m.x) : 0) + __popc(word & lanesBelow());
        uint32_t survivorRank = (half ? __popc(sm.x) : 0) + __popc((half ? sm.y : sm.x) & lanesBelow());
        uint32_t slot = out + rank, from = in + survivorRank;
        if (slot >= c.contactCapacity || from >= c.survivorCapacity) { fail(r, F_CONTACT); continue; }
        uint32_t node = __ldg(&r.meshSampleIndices[range.x + laneId() + half * WARP]);
        r.meta[slot] = make_uint4(src, dst, node, 0);
        r.pointDepth[slot] = r.hitScratch[2 * from];
        r.normalArea[slot] = r.hitScratch[2 * from + 1];
        r.contactPair[slot] = p;
    }
}
// Copies the hits of each item from their survivor slots to their canonical
// offsets, and clears the item's hit mask and count for the next step (also
// on a failed step, whose walks may have set bits before the failure: the
// masks are all zero whenever a step starts, so a step that reuses the
// stored survivors needs no clearing pass).
__global__ void __launch_bounds__(256) k_nodeEmit(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    bool live = r.control[0] == 0;
    uint32_t n = min(r.work[W_CANDIDATES], c.candidateCapacity);
    // Lane per item: read and clear the masks of 32 items, then the warp
    // emits the items with hits one after the other.
    for (uint32_t first = WARP * warpGlobal(); first < n; first += WARP * warpStride()) {
        uint32_t mine = first + laneId();
        uint2 own = mine < n ? r.candHitMask[mine] : make_uint2(0u, 0u);
        bool any = (own.x | own.y) != 0;
        if (any) {
            r.candHitMask[mine] = make_uint2(0u, 0u);
            r.candHitCount[mine] = 0;
        }
        uint32_t pending = __ballot_sync(0xffffffffu, any);
        if (!live) continue;
        while (pending) {
            uint32_t lane = __ffs(pending) - 1;
            pending &= pending - 1;
            uint32_t item = first + lane;
            uint2 m = make_uint2(__shfl_sync(0xffffffffu, own.x, lane), __shfl_sync(0xffffffffu, own.y, lane));
            emitItem(r, c, item, m);
        }
    }
}
// The same contact records from a stored exact-query list, a thread per
// stored slot instead of a warp per item: a slot whose node hit (its bit in
// its item's hit mask) writes its record at its item's offset plus the
// number of the item's hits at lower node slots -- the canonical place
// k_nodeEmit gives it -- from the slot's own node record (source, target,
// directed pair, packed sample) and its hit scratch.  Dormant slots never
// hit.  The item masks are cleared by k_clearHits afterwards (a slot cannot
// clear its item's mask while the item's other hits still read it).
__global__ void k_clearHits(const __grid_constant__ Params P);
__global__ void __launch_bounds__(256) k_emitSlots(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t n = min(r.work[W_KEPT], c.survivorCapacity);
    for (uint32_t t = gtid(); t < n; t += gstride()) {
        if (r.walkCertTriangle[t].x == DORMANT) continue;
        uint2 it = r.walkItem[t];
        uint2 m = r.candHitMask[it.x];
        uint32_t word = it.y < WARP ? m.x : m.y, bit = 1u << (it.y & 31u);
        if (!(word & bit)) continue;
        uint32_t rank = (it.y < WARP ? 0u : __popc(m.x)) + __popc(word & (bit - 1u));
        uint32_t slot = r.candHitOffset[it.x] + rank, from = r.walkList[t];
        if (slot >= c.contactCapacity || from >= c.survivorCapacity) { fail(r, F_CONTACT); continue; }
        uint4 rec = r.walkNode[t];
        uint32_t node = rec.w - __ldg(&r.sampleInfo[r.shapeId[rec.x]].x);
        r.meta[slot] = make_uint4(rec.x, rec.y, node, 0);
        r.pointDepth[slot] = r.hitScratch[2 * from];
        r.normalArea[slot] = r.hitScratch[2 * from + 1];
        r.contactPair[slot] = rec.z >> 1;
    }
}
// Per pair: first contact of the pair on the side being written, and counts.
__device__ __forceinline__ void contactStart(const Params& P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t n = activePairs(r, c);
    uint32_t total = r.control[2];
    if (total > c.contactCapacity) fail(r, F_CONTACT);
    if (r.control[0] != 0) return;
    uint32_t items = min(r.work[W_CANDIDATES], c.candidateCapacity);
    for (uint32_t p = gtid(); p <= n; p += gstride()) {
        uint32_t first = r.dpairCandOffset[2 * p];
        uint32_t start = first < items ? r.candHitOffset[first] : total;
        r.sideContactStart[p] = start;
        if (p < n) {
            uint32_t next = r.dpairCandOffset[2 * p + 2];
            uint32_t end = next < items ? r.candHitOffset[next] : total;
            r.contactCounts[p] = end - start;
        }
    }
}
__global__ void k_contactStart(const __grid_constant__ Params P) { contactStart(P); }
// Hit masks and counts of every item back to zero for the next step (also
// after a failed step, whose walks may have set bits), and the per-pair
// contact starts (k_contactStart) in the same launch.
__global__ void k_clearHits(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t n = min(r.work[W_CANDIDATES], c.candidateCapacity);
    for (uint32_t i = gtid(); i < n; i += gstride()) {
        r.candHitMask[i] = make_uint2(0u, 0u);
        r.candHitCount[i] = 0;
    }
    contactStart(P);
}

// ------------------------------------------------------------ SDF geometry
// solver.slang:188-200: trilinear signed distance and gradient from the
// target shape's grid, in the FP32 order of the reference's generated CPU
// code (lerp(x, y, s) = x + (y - x) * s, products left to right).
__device__ __forceinline__ float4 sdfQuery(const Res& r, uint32_t shape, f3 p) {
    uint4 meta = __ldg(&r.grids[shape]);
    float4 o = __ldg(&r.gridOrigin[shape]);
    f3 g = (p - xyz(o)) / o.w;
    int ax = int(floorf(g.x)), ay = int(floorf(g.y)), az = int(floorf(g.z));
    if (ax < 0 || ay < 0 || az < 0 || ax >= int(meta.y) - 1 || ay >= int(meta.z) - 1 || az >= int(meta.w) - 1)
        return make_float4(0.f, 0.f, 0.f, 1.00000002004087734e+20f);
    f3 t = g - mk(float(ax), float(ay), float(az));
    f3 u = mk(1.f, 1.f, 1.f) - t;
    float value = 0.f;
    f3 grad = mk(0.f, 0.f, 0.f);
#pragma unroll
    for (uint32_t i = 0; i < 2; ++i)
#pragma unroll
        for (uint32_t j = 0; j < 2; ++j)
#pragma unroll
            for (uint32_t k = 0; k < 2; ++k) {
                f3 w = u + (t - u) * mk(float(i), float(j), float(k));
                float f = __ldg(&r.distance[meta.x + ((uint32_t(ax) + i) * meta.z + (uint32_t(ay) + j)) * meta.w +
                                            (uint32_t(az) + k)]);
                value = __fadd_rn(value, __fmul_rn(__fmul_rn(__fmul_rn(f, w.x), w.y), w.z));
                f3 v = mk(__fmul_rn(__fmul_rn(__fsub_rn(__fmul_rn(2.0f, float(i)), 1.0f), w.y), w.z),
                          __fmul_rn(__fmul_rn(__fsub_rn(__fmul_rn(2.0f, float(j)), 1.0f), w.x), w.z),
                          __fmul_rn(__fmul_rn(__fsub_rn(__fmul_rn(2.0f, float(k)), 1.0f), w.x), w.y));
                grad = grad + (f * v) / o.w;
            }
    return w4(grad, value);
}
// solver.slang:319-343 with the SDF geometry; the directed-pair branch is
// the FP64 one k_pairSetup stored (the same bits as the per-call reference).
__device__ __forceinline__ bool sdfNodeContact(const Res& r, const Config& c, uint32_t src, uint32_t dst,
                                               uint32_t node, f3 branch, float4& pd, float4& na) {
    uint32_t sid = r.shapeId[src];
    float4 sp = __ldg(&r.sample[__ldg(&r.sampleInfo[sid].x) + node]);
    float4 bs = r.body[src], bd = r.body[dst];
    f3 arm = qrot(r.rotation[src], xyz(sp) * bs.x);
    f3 local = qinv(r.rotation[dst], arm - branch) / bd.x;
    // Beyond the target's bounding radius by more than a grid-cell diagonal,
    // all eight grid values around the node are distances of points outside
    // the shape (positive), so the interpolated distance is positive: no
    // contact, as the full query would find; skip its grid loads.
    float reach = __fadd_rn(__fdiv_rn(bd.z, bd.x), __fmul_rn(1.7339f, __ldg(&r.gridOrigin[r.shapeId[dst]].w)));
    if (dot(local, local) > __fmul_rn(reach, reach)) return false;
    float4 f = sdfQuery(r, r.shapeId[dst], local);
    pd = w4(arm, __fmul_rn(-f.w, bd.x));
    if (pd.w <= 0.0f) return false;
    f3 grad = qrot(r.rotation[dst], xyz(f));
    float len = length(grad);
    if (len < 1.00000001168609742e-07f || !isfinite(pd.w)) { fail(r, F_DEGENERATE); return false; }
    na = w4(grad / len, __fmul_rn(__fmul_rn(sp.w, bs.x), bs.x));
    if (pd.w > __fmul_rn(c.maxOverlap, mn(bs.w, bd.w))) fail(r, F_PENETRATION);
    return true;
}
// The contacts of pair p on virtual lane v of the reference's 64-thread
// group (solver.slang:536-565): its nodes s = v, v + 64, ... over the first
// grain's nodes, then the second's.  With `emit`, they are written from
// `slot` on; returns how many there are.
__device__ __forceinline__ uint32_t sdfLane(const Res& r, const Config& c, uint32_t p, uint2 ij, uint32_t a,
                                            uint32_t total, uint32_t v, bool emit, uint32_t slot) {
    f3 b0 = xyz(r.dpairBranch[2 * p]), b1 = xyz(r.dpairBranch[2 * p + 1]);
    uint32_t count = 0;
    for (uint32_t s = v; s < total; s += 64) {
        bool first = s < a;
        uint32_t i = first ? ij.x : ij.y, j = first ? ij.y : ij.x, node = first ? s : s - a;
        float4 pd, na;
        if (!sdfNodeContact(r, c, i, j, node, first ? b0 : b1, pd, na)) continue;
        if (emit) {
            uint32_t out = slot + count;
            if (out >= c.contactCapacity) { fail(r, F_CONTACT); return count; }
            r.meta[out] = make_uint4(i, j, node, 0);
            r.pointDepth[out] = pd;
            r.normalArea[out] = na;
            r.contactPair[out] = p;
        }
        count++;
    }
    return count;
}
// countContacts (solver.slang:538-549): one warp per pair, each lane two of
// the 64 virtual lanes.
__global__ void k_sdfCount(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t n = activePairs(r, c);
    for (uint32_t p = warpGlobal(); p < n; p += warpStride()) {
        uint2 ij = r.pairs[p];
        uint32_t a = __ldg(&r.sampleInfo[r.shapeId[ij.x]].y), total = a + __ldg(&r.sampleInfo[r.shapeId[ij.y]].y);
        uint32_t low = sdfLane(r, c, p, ij, a, total, laneId(), false, 0);
        uint32_t high = sdfLane(r, c, p, ij, a, total, laneId() + WARP, false, 0);
        r.sdfLaneCounts[size_t(WARP) * p + laneId()] = low | (high << 16);  // at most 81 each
        uint32_t count = low + high;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
        if (laneId() == 0) r.contactCounts[p] = count;
    }
}
// emitContacts (solver.slang:551-565): each virtual lane writes its contacts
// after those of the lanes below it, so a pair's contacts are in the
// reference's order (lane, then node).  Also the per-pair contact starts of
// the history side being written.
__global__ void k_sdfEmit(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t n = activePairs(r, c);
    uint32_t total = r.control[2];
    if (total > c.contactCapacity) fail(r, F_CONTACT);
    if (r.control[0] != 0) return;
    for (uint32_t p = warpGlobal(); p < n; p += warpStride()) {
        uint2 ij = r.pairs[p];
        uint32_t a = __ldg(&r.sampleInfo[r.shapeId[ij.x]].y), nodes = a + __ldg(&r.sampleInfo[r.shapeId[ij.y]].y);
        uint32_t counts = r.sdfLaneCounts[size_t(WARP) * p + laneId()];  // from k_sdfCount
        uint32_t low = counts & 0xFFFFu, high = counts >> 16;
        uint32_t incLow = low, incHigh = high;
#pragma unroll
        for (uint32_t o = 1; o < WARP; o <<= 1) {
            uint32_t x = __shfl_up_sync(0xffffffffu, incLow, o), y = __shfl_up_sync(0xffffffffu, incHigh, o);
            if (laneId() >= o) { incLow += x; incHigh += y; }
        }
        uint32_t lowTotal = __shfl_sync(0xffffffffu, incLow, WARP - 1);
        uint32_t base = r.contactOffsets[p];
        sdfLane(r, c, p, ij, a, nodes, laneId(), true, base + incLow - low);
        sdfLane(r, c, p, ij, a, nodes, laneId() + WARP, true, base + lowTotal + incHigh - high);
    }
    for (uint32_t p = gtid(); p <= n; p += gstride()) r.sideContactStart[p] = p < n ? r.contactOffsets[p] : total;
}

// ---------------------------------------------------------------- friction
// solver.slang:691-696
__device__ __forceinline__ f3 transported(f3 x, f3 a, f3 b, float spin) {
    float cc = mn(mx(dot(a, b), -1.0f), 1.0f);
    if (cc < -0.999999f) return mk(0.f, 0.f, 0.f);
    f3 v = cross(a, b);
    f3 out = (x + cross(v, x)) + cross(v, cross(v, x)) / __fadd_rn(1.0f, cc);
    float cs = cosf(spin), sn = sinf(spin);
    out = (out * cs + cross(b, out) * sn) + (b * dot(b, out)) * __fsub_rn(1.0f, cs);
    return out - b * dot(out, b);
}
// normal.slang:2-11
__device__ __forceinline__ void normalResponse(float depth, float area, float vn, float stiffness, float viscosity,
                                               float weight, float& force, float& lossPower) {
    force = 0.f;
    lossPower = 0.f;
    if (depth <= 0) return;
    float elastic = __fmul_rn(__fmul_rn(__fmul_rn(weight, stiffness), area), depth);
    force = viscosity == 0 ? elastic
                           : mx(0.0f, __fsub_rn(elastic, __fmul_rn(__fmul_rn(__fmul_rn(weight, viscosity), area), vn)));
    lossPower = mx(0.0f, __fmul_rn(__fsub_rn(elastic, force), vn));
}
// History key within a pair: direction (source > target) then the node's
// position in its shape's cluster order; runs of one pair are sorted by it.
// With the SDF geometry a pair's contacts are in the reference emit order:
// s = node (first grain) or V_first + node (second grain), taken by virtual
// lane s mod 64, then s / 64.
__device__ __forceinline__ uint32_t pairKey(const Res& r, const Config& c, uint32_t src, uint32_t dst,
                                            uint32_t node) {
    if (c.meshGeometry == 0) {
        uint32_t s = src > dst ? __ldg(&r.sampleInfo[r.shapeId[dst]].y) + node : node;
        return ((s & 63u) << 24) | (s >> 6);
    }
    return (src > dst ? 0x80000000u : 0u) | __ldg(&r.meshSampleRank[__ldg(&r.sampleInfo[r.shapeId[src]].x) + node]);
}
// Slot of key (src, dst, node) among the committed contacts, or EMPTY.
// The committed side stores, per grain a, the run of its pairs (a, b) with
// b > a and, per pair, its contacts sorted by pairKey: a sorted merge done as
// a run lookup plus a binary search.
__device__ __forceinline__ uint32_t historySlot(const Res& r, const Config& c, uint32_t src, uint32_t dst,
                                                uint32_t node) {
    uint32_t a = min(src, dst), b = max(src, dst);
    uint32_t begin = r.oldPairOffsets[a], end = r.oldPairOffsets[a + 1];
    uint32_t q = EMPTY;
    for (uint32_t k = begin; k < end; ++k)
        if (r.oldPairB[k] == b) { q = k; break; }
    if (q == EMPTY) return EMPTY;
    uint32_t lo = r.oldContactStart[q], hi = r.oldContactStart[q + 1];
    uint32_t key = pairKey(r, c, src, dst, node);
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        uint4 m = r.oldMeta[mid];
        uint32_t mk2 = pairKey(r, c, m.x, m.y, m.z);
        if (mk2 < key) lo = mid + 1;
        else hi = mid;
    }
    if (lo < r.oldContactStart[q + 1]) {
        uint4 m = r.oldMeta[lo];
        if (m.x == src && m.y == dst && m.z == node) return lo;
    }
    return EMPTY;
}
// ------------------------------------------------------------------ planes
// Signed distance of a grain surface point (centre + arm) from the plane
// (solver.slang:605-610), from the centre's two-sum.
__device__ __forceinline__ float localWallDistance(const Res& r, uint32_t wall, Sum2 centre, f3 arm) {
    Sum2 sum = wallAddDot(centre, xyz(r.wallPlane[wall]), arm);
    sum = wallAddDot(sum, xyz(r.wallRemainder[wall]), arm);
    return __fadd_rn(sum.hi, sum.lo);
}
// The per-(wall, grain) terms of the cluster bound (solver.slang:613-624):
// the plane normal in the grain's scaled frame, the centre distance and the
// grain-independent part of the FP32 pad.
struct WallFrame {
    f3 normal;
    float normalLength, base, padBase;
};
__device__ __forceinline__ WallFrame wallFrame(const Res& r, uint32_t body, uint32_t wall, float base) {
    float4 plane = r.wallPlane[wall];
    WallFrame f;
    f.normal = qinv(r.rotation[body], xyz(plane)) * r.body[body].x;
    f.normalLength = length(f.normal);
    f.base = base;
    f.padBase = __fadd_rn(__fadd_rn(1.0f, fabsf(plane.w)), length(xyz(r.position[body])));
    return f;
}
// solver.slang:613-624: whether any node of a sample cluster can reach
// behind the plane (fixed-normal support bound with an FP32 pad).
__device__ __forceinline__ bool wallClusterMayContact(const Res& r, const WallFrame& f, uint32_t cluster) {
    f3 low = xyz(__ldg(&r.meshClusterMin[cluster])), high = xyz(__ldg(&r.meshClusterMax[cluster]));
    f3 center = 0.5f * (low + high), half = 0.5f * (high - low);
    float support = __fsub_rn(dot(f.normal, center), dot(abs3(f.normal), half));
    float pad = __fmul_rn(__fmul_rn(64.0f, 1.1920928955078125e-7f),
                          __fadd_rn(f.padBase, __fmul_rn(f.normalLength, __fadd_rn(length(center), length(half)))));
    return __fadd_rn(f.base, support) <= pad;
}
// solver.slang:625-638: node `node` of grain `body` behind the plane, with
// its record (arm and depth; plane normal and node area).  `flag` raises the
// non-finite and penetration flags (once per step: in the counting pass).
__device__ __forceinline__ bool wallNode(const Res& r, const Config& c, uint32_t body, uint32_t wall, Sum2 centre,
                                        uint32_t node, bool flag, float4& pd, float4& na) {
    float4 point = __ldg(&r.sample[__ldg(&r.sampleInfo[r.shapeId[body]].x) + node]);
    float4 b = r.body[body];
    f3 arm = qrot(r.rotation[body], xyz(point) * b.x);
    float phi = localWallDistance(r, wall, centre, arm);
    if (!isfinite(phi)) {
        if (flag) fail(r, F_NONFINITE);
        return false;
    }
    if (phi >= 0) return false;
    if (flag && -phi > __fmul_rn(c.maxOverlap, b.w)) fail(r, F_PENETRATION);
    pd = w4(arm, -phi);
    na = w4(xyz(r.wallPlane[wall]), __fmul_rn(__fmul_rn(point.w, b.x), b.x));
    return true;
}
// Whether grain `body` may reach behind plane `wall`: the centre-distance
// early-out of collectWallContacts (solver.slang:642-653), one lane per item.
__device__ __forceinline__ bool wallReach(const Res& r, uint32_t body, uint32_t wall, Sum2& centre) {
    float4 plane = r.wallPlane[wall];
    centre = wallCentreDistance(r, body, wall);
    float phi = __fadd_rn(centre.hi, centre.lo);
    float pad = __fmul_rn(__fmul_rn(64.0f, 1.1920928955078125e-7f),
                          __fadd_rn(__fadd_rn(1.0f, length(xyz(r.position[body]))), fabsf(plane.w)));
    return !(phi > __fadd_rn(r.body[body].z, pad));
}
// The plane contacts of one (wall, grain) item that passed the early-out, in
// the reference CPU collector's order (cpu_scheduling.slang:133-154): the
// grain's nodes in order (SDF geometry), or its sample clusters in preorder
// -- a cluster the plane cannot reach skips its subtree -- and each visited
// cluster's nodes in order (mesh geometry).  One warp: the 32 clusters from
// the walk's cursor are bounded at once (one per lane), then the walk
// advances through them with the lanes' results; nodes are tested 32 per
// round, order kept by ballot ranks.  Counted, or written from `slot` on.
// Returns the count.
__device__ uint32_t wallItem(const Res& r, const Config& c, uint32_t item, Sum2 centre, bool emit, uint32_t slot) {
    uint32_t body = item % c.N, wall = item / c.N, lane = laneId();
    float phi = __fadd_rn(centre.hi, centre.lo);
    uint32_t shape = r.shapeId[body], count = 0;
    auto visit = [&](bool valid, uint32_t node) {
        float4 pd, na;
        bool hit = valid && wallNode(r, c, body, wall, centre, node, !emit, pd, na);
        uint32_t mask = __ballot_sync(0xffffffffu, hit);
        if (emit && hit) {
            uint32_t out = slot + count + __popc(mask & ((1u << lane) - 1u));
            if (out >= c.contactCapacity) {
                fail(r, F_CONTACT);
            } else {
                r.meta[out] = make_uint4(body, c.N + wall, node, 1u);
                r.pointDepth[out] = pd;
                r.normalArea[out] = na;
            }
        }
        count += __popc(mask);
    };
    if (c.meshGeometry == 0) {
        uint32_t nodes = __ldg(&r.sampleInfo[shape].y);
        for (uint32_t base = 0; base < nodes; base += WARP) visit(base + lane < nodes, base + lane);
        return count;
    }
    WallFrame frame = wallFrame(r, body, wall, phi);
    uint4 info = __ldg(&r.meshClusterInfo[shape]);
    uint32_t end = info.x + info.y, cursor = info.x;
    // Every window moves the cursor forward (escape links point forward; a
    // link that does not ends the walk).
    for (uint32_t guard = 0; cursor < end && guard < info.y; ++guard) {
        uint32_t window = cursor, cl = window + lane;
        bool candidate = cl < end && wallClusterMayContact(r, frame, cl);
        uint4 range = cl < end ? __ldg(&r.meshClusterRanges[cl]) : make_uint4(0u, 0u, 0u, 0u);
        uint32_t mask = __ballot_sync(0xffffffffu, candidate);
        while (cursor < end && cursor - window < WARP) {
            uint32_t k = cursor - window;
            uint32_t x = __shfl_sync(0xffffffffu, range.x, int(k)), y = __shfl_sync(0xffffffffu, range.y, int(k));
            uint32_t z = __shfl_sync(0xffffffffu, range.z, int(k));
            if ((mask >> k) & 1u) {
                for (uint32_t base = 0; base < y; base += WARP) {
                    uint32_t n = base + lane;
                    visit(n < y, n < y ? __ldg(&r.meshSampleIndices[x + n]) : 0u);
                }
                ++cursor;
            } else {
                cursor = z > cursor ? z : end;
            }
        }
    }
    return count;
}
// Plane contacts per (wall, grain), wall-major: each lane runs the early-out
// of one item, then the warp collects its items that pass, one after the
// other.  A warp's 32 items are a grid of warps apart: the grains near a wall
// are runs of consecutive items, spread this way over many warps.  Records
// where the plane contacts start.
__global__ void k_wallCount(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    if (gtid() == 0) r.work[W_WALL_BASE] = r.control[2];
    uint32_t items = c.N * c.wallCount, lane = laneId(), stride = warpStride(), first = warpGlobal();
    for (uint32_t base = 0; base < items; base += stride * WARP) {
        uint32_t item = base + lane * stride + first;
        Sum2 centre{0.f, 0.f};
        bool reach = item < items && wallReach(r, item % c.N, item / c.N, centre);
        if (item < items && !reach) r.wallCounts[item] = 0;
        for (uint32_t mask = __ballot_sync(0xffffffffu, reach); mask; mask &= mask - 1u) {
            uint32_t k = __ffs(mask) - 1u, it = base + k * stride + first;
            Sum2 ck{__shfl_sync(0xffffffffu, centre.hi, int(k)), __shfl_sync(0xffffffffu, centre.lo, int(k))};
            uint32_t n = wallItem(r, c, it, ck, false, 0);
            if (lane == 0) r.wallCounts[it] = n;
        }
    }
}
// The plane contacts appended after the grain-grain ones (gpu.py:544-545),
// per-(wall, grain) starts and the new contact total.
__global__ void k_wallEmit(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t items = c.N * c.wallCount, base0 = r.work[W_WALL_BASE], lane = laneId();
    for (uint32_t i = gtid(); i <= items; i += gstride()) r.sideWallStart[i] = base0 + r.wallOffsets[i];
    if (gtid() == 0) {
        uint32_t total = base0 + r.wallOffsets[items];
        r.control[2] = total;
        if (total > c.contactCapacity) fail(r, F_CONTACT);
    }
    uint32_t stride = warpStride(), first = warpGlobal();
    for (uint32_t base = 0; base < items; base += stride * WARP) {
        uint32_t item = base + lane * stride + first;
        bool some = item < items && r.wallCounts[item] != 0;
        for (uint32_t mask = __ballot_sync(0xffffffffu, some); mask; mask &= mask - 1u) {
            uint32_t it = base + (__ffs(mask) - 1u) * stride + first;
            wallItem(r, c, it, wallCentreDistance(r, it % c.N, it / c.N), true, base0 + r.wallOffsets[it]);
        }
    }
}
// Within one (wall, grain) run, the order of a node's contact: its position in
// the grain's cluster order (mesh) or its index (SDF).
__device__ __forceinline__ uint32_t wallKey(const Res& r, const Config& c, uint32_t body, uint32_t node) {
    return c.meshGeometry == 0 ? node : __ldg(&r.meshSampleRank[__ldg(&r.sampleInfo[r.shapeId[body]].x) + node]);
}
// Slot of the committed plane contact (body, wall, node), or EMPTY: binary
// search of the committed (wall, grain) run.
__device__ __forceinline__ uint32_t wallHistorySlot(const Res& r, const Config& c, uint32_t body, uint32_t wall,
                                                    uint32_t node) {
    uint32_t item = wall * c.N + body;
    uint32_t lo = r.oldWallStart[item], end = r.oldWallStart[item + 1], hi = end;
    uint32_t key = wallKey(r, c, body, node);
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (wallKey(r, c, body, r.oldMeta[mid].z) < key) lo = mid + 1;
        else hi = mid;
    }
    if (lo < end) {
        uint4 m = r.oldMeta[lo];
        if (m.x == body && m.y == c.N + wall && m.z == node) return lo;
    }
    return EMPTY;
}
// solver.slang:702-733 with plane.slang:13-36: a plane contact.
__device__ __forceinline__ void resolveWall(const Res& r, const Config& c, uint32_t id, uint4 key) {
    uint32_t i = key.x, w = key.y - c.N;
    float4 m = r.wallMaterial[w];
    float viscosity = m.w;
    f3 nrm = xyz(r.normalArea[id]);
    f3 wi = viscosity > 0 ? xyz(r.forceOmega[i]) : omegaOf(r, i);
    f3 elastic = mk(0.f, 0.f, 0.f);
    if (c.historyStep != 0) {
        uint32_t old = wallHistorySlot(r, c, i, w, key.z);
        if (old != EMPTY)
            elastic = transported(xyz(r.oldSlip[old]), xyz(r.oldNormal[old]), nrm,
                                  __fmul_rn(__fmul_rn(0.5f, dot(wi + mk(0.f, 0.f, 0.f), nrm)), c.dt));
    }
    f3 arm = xyz(r.pointDepth[id]);
    f3 v = viscosity > 0 ? xyz(r.forceVelocity[i]) : xyz(r.velocity[i]) + xyz(r.velocityRemainder[i]);
    f3 rv = (v + cross(wi, arm)) - xyz(r.wallVelocity[w]);
    float4 forceEnergy = make_float4(0.f, 0.f, 0.f, 0.f), slipLoss = forceEnergy;
    float lossPower = 0.f;
    bool sliding = false;
    float signedDistance = -r.pointDepth[id].w, area = r.normalArea[id].w;
    if (signedDistance < 0) {
        float depth = -signedDistance;
        f3 tangent = rv - nrm * dot(rv, nrm);
        f3 trial = (elastic - nrm * dot(elastic, nrm)) + c.dt * tangent;
        f3 slip = trial;
        float fn;
        normalResponse(depth, area, dot(rv, nrm), m.x, viscosity, 1.0f, fn, lossPower);
        f3 ft = __fmul_rn(-m.y, area) * slip;
        float magnitude = length(ft);
        if (magnitude > __fmul_rn(m.z, fn) && magnitude > 0) {
            sliding = true;
            ft = ft * __fdiv_rn(__fmul_rn(m.z, fn), magnitude);
            slip = (-ft) / __fmul_rn(m.y, area);
        }
        forceEnergy = w4(fn * nrm + ft, __fmul_rn(__fmul_rn(0.5f, area), __fadd_rn(__fmul_rn(__fmul_rn(m.x, depth), depth),
                                                                               __fmul_rn(m.y, dot(slip, slip)))));
        slipLoss = w4(slip, mx(0.0f, -dot(ft, trial - slip)));
    }
    r.slip[id] = slipLoss;
    r.contactForce[id] = forceEnergy;
    r.normalLossPower[id] = lossPower;
    if (!isfinite(forceEnergy.x) || !isfinite(forceEnergy.y) || !isfinite(forceEnergy.z) || !isfinite(forceEnergy.w) ||
        !isfinite(lossPower)) {
        fail(r, F_NONFINITE);
        return;
    }
    if (sliding) atomicAdd(&r.control[6], 1u);
}
// solver.slang:834-856: per (wall, grain), the reaction, its moment about
// the origin and the wall power over the grain's contacts with that wall, in
// its linked-list order (descending contact id), and the accumulated work.
__global__ void k_gatherWallRows(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t items = c.N * c.wallCount;
    for (uint32_t item = gtid(); item < items; item += gstride()) {
        uint32_t body = item % c.N, wall = item / c.N;
        uint32_t lo = r.sideWallStart[item], hi = r.sideWallStart[item + 1];
        f3 centre = mk(0.f, 0.f, 0.f), velocity = centre;
        if (hi > lo) {
            centre = xyz(r.position[body]) + xyz(r.positionRemainder[body]);
            velocity = xyz(r.wallVelocity[wall]);
        }
        f3 reaction = mk(0.f, 0.f, 0.f), moment = reaction;
        float power = 0.f;
        for (uint32_t k = hi; k > lo; --k) {
            f3 force = xyz(r.contactForce[k - 1]);
            f3 point = centre + xyz(r.pointDepth[k - 1]);
            reaction = reaction - force;
            moment = moment - cross(point, force);
            power = __fadd_rn(power, dot(force, velocity));
        }
        float4 work = r.wallAccumulated[item];
        r.wallRows[3 * item] = w4(reaction, __uint_as_float(hi - lo));
        r.wallRows[3 * item + 1] = w4(moment, power);
        r.wallRows[3 * item + 2] = make_float4(__fadd_rn(work.x, work.y), 0.f, 0.f, 0.f);
    }
}

// solver.slang:702-733: the plane contacts, after the grain-grain ones.
__global__ void k_resolveWalls(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t n = activeContacts(r, c);
    for (uint32_t id = min(r.work[W_WALL_BASE], n) + gtid(); id < n; id += gstride()) resolveWall(r, c, id, r.meta[id]);
}
// solver.slang:702-749 (particle-particle contacts)
__global__ void k_resolve(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t n = activeContacts(r, c);
    // With planes, the grain-grain contacts end where the plane contacts
    // begin; those are resolved by k_resolveWalls.
    if (c.wallCount != 0) n = min(n, r.work[W_WALL_BASE]);
    for (uint32_t id = gtid(); id < n; id += gstride()) {
        uint4 key = r.meta[id];
        uint32_t i = key.x, j = key.y;
        f3 nrm = xyz(r.normalArea[id]);
        float viscosity = c.normalViscosity;
        f3 wi = viscosity > 0 ? xyz(r.forceOmega[i]) : omegaOf(r, i);
        f3 wj = viscosity > 0 ? xyz(r.forceOmega[j]) : omegaOf(r, j);
        f3 elastic = mk(0.f, 0.f, 0.f);
        if (c.historyStep != 0) {
            uint32_t old = historySlot(r, c, i, j, key.z);
            if (old != EMPTY)
                elastic = transported(xyz(r.oldSlip[old]), xyz(r.oldNormal[old]), nrm,
                                      __fmul_rn(__fmul_rn(0.5f, dot(wi + wj, nrm)), c.dt));
        }
        f3 arm = xyz(r.pointDepth[id]);
        uint32_t p = r.contactPair[id];
        f3 branch = xyz(r.dpairBranch[2 * p + (i > j ? 1 : 0)]);
        f3 translation = viscosity > 0 ? xyz(r.forceVelocity[i]) - xyz(r.forceVelocity[j])
                                       : xyz(r.velocity[i]) - xyz(r.velocity[j]);
        f3 rv = ((translation - xyz(r.cell[3 * specimenOf(r, i) + 1]) * branch) + cross(wi, arm)) - cross(wj, arm - branch);
        elastic = elastic + (rv - nrm * dot(rv, nrm)) * c.dt;
        f3 trial = elastic;
        float area = r.normalArea[id].w, depth = r.pointDepth[id].w;
        float fn, lossPower;
        normalResponse(depth, area, dot(rv, nrm), c.kn, viscosity, 0.5f, fn, lossPower);
        r.normalLossPower[id] = lossPower;
        float ktA = __fmul_rn(__fmul_rn(-0.5f, c.kt), area);
        f3 ft = ktA * elastic;
        float magnitude = length(ft);
        if (magnitude > __fmul_rn(c.mu, fn) && magnitude > 0) {
            ft = ft * __fdiv_rn(__fmul_rn(c.mu, fn), magnitude);
            elastic = (-ft) / __fmul_rn(__fmul_rn(0.5f, c.kt), area);
            atomicAdd(&r.control[6], 1u);
        }
        r.slip[id] = w4(elastic, mx(0.0f, -dot(ft, trial - elastic)));
        float4 cf = w4(fn * nrm + ft,
                       __fmul_rn(__fmul_rn(0.25f, area), __fadd_rn(__fmul_rn(__fmul_rn(c.kn, depth), depth),
                                                                   __fmul_rn(c.kt, dot(elastic, elastic)))));
        r.contactForce[id] = cf;
        if (!isfinite(cf.x) || !isfinite(cf.y) || !isfinite(cf.z) || !isfinite(cf.w) || !isfinite(lossPower))
            fail(r, F_NONFINITE);
    }
}

// -------------------------------------------------------------------- gather
// solver.slang:760-811, one warp per grain.  Contacts of grain g are taken in
// the order the reference's linked lists hold them (descending contact id):
// pairs where g is first (a contiguous run) and second (the byJ run) merged
// from the highest pair id down, each pair's contacts from the last.  Lanes
// load and evaluate 32 contacts at a time and store their terms in shared
// memory; every accumulator component is an independent sequential chain
// (the compensated force and torque sums are componentwise), so lane j then
// replays chain j over the 32 terms in that order: the sums are
// bit-identical to the serial loop, with 22 chains advancing in parallel.
struct GatherTerms {
    f3 force, torque, s0, s1, s2;
    float energy, denom, depth, dissipation, normalPower, stiffness, viscous;
};
// Accumulator chains: 0-2 force and 3-5 torque (compensated), 6-14 the three
// stress rows (subtracted), 15 energy, 16 denominator, 17 deepest overlap
// (maximum), 18 dissipation, 19 normal loss power, 20-21 timestep rates.
constexpr uint32_t GATHER_CHAINS = 22;
constexpr uint32_t GATHER_STRIDE = WARP + 1;  // padded rows: conflict-free on both sides
__device__ __forceinline__ f3 shfl3(f3 v, int lane) {
    return mk(__shfl_sync(0xffffffffu, v.x, lane), __shfl_sync(0xffffffffu, v.y, lane),
              __shfl_sync(0xffffffffu, v.z, lane));
}
// Lane `chain` replays its accumulator chain over the `count` terms of one
// round, in order (compensated sums, subtracted stress rows, maximum depth,
// plain sums; the timestep rates only under the active-contact policy).
__device__ __forceinline__ void replayChain(float (*terms)[GATHER_STRIDE], uint32_t count, uint32_t chain, bool rates,
                                            float& acc, float& accLow) {
    if (chain < 6) {
        for (uint32_t k = 0; k < count; ++k) {  // compensated3, one component
            float y = __fadd_rn(terms[chain][k], accLow);
            float nx = __fadd_rn(acc, y);
            accLow = __fsub_rn(y, __fsub_rn(nx, acc));
            acc = nx;
        }
    } else if (chain < 15) {
        for (uint32_t k = 0; k < count; ++k) acc = __fsub_rn(acc, terms[chain][k]);
    } else if (chain == 17) {
        for (uint32_t k = 0; k < count; ++k) acc = mx(acc, terms[chain][k]);
    } else if (chain < GATHER_CHAINS && (chain < 20 || rates)) {
        for (uint32_t k = 0; k < count; ++k) acc = __fadd_rn(acc, terms[chain][k]);
    }
}
__device__ __forceinline__ void storeTerms(float (*terms)[GATHER_STRIDE], uint32_t lane, const GatherTerms& g) {
    const float v[GATHER_CHAINS] = {g.force.x, g.force.y, g.force.z, g.torque.x, g.torque.y, g.torque.z,
                                    g.s0.x, g.s0.y, g.s0.z, g.s1.x, g.s1.y, g.s1.z,
                                    g.s2.x, g.s2.y, g.s2.z, g.energy, g.denom, g.depth,
                                    g.dissipation, g.normalPower, g.stiffness, g.viscous};
#pragma unroll
    for (uint32_t j = 0; j < GATHER_CHAINS; ++j) terms[j][lane] = v[j];
}
// solver.slang:773-791, the plane branch: full force, moment about the
// grain centre, virial with the arm, full energy and losses; the wall's own
// material in the timestep rates with coupling 1.
__device__ __forceinline__ GatherTerms wallTerms(const Res& r, const Config& c, uint32_t contact, uint32_t wall,
                                                 float mass, float bw, float inverseInertia) {
    GatherTerms g{};
    float4 cf = r.contactForce[contact], pdv = r.pointDepth[contact];
    f3 force = xyz(cf), arm = xyz(pdv);
    if (c.activeTimestep != 0) {
        float mobility = __fadd_rn(__fdiv_rn(1.0f, mass), __fmul_rn(dot(arm, arm), inverseInertia));
        float4 m = r.wallMaterial[wall];
        float area = __fmul_rn(1.0f, r.normalArea[contact].w);
        float friction = __fadd_rn(1.0f, m.z);
        g.stiffness = __fmul_rn(__fmul_rn(area, __fadd_rn(__fmul_rn(m.x, friction), m.y)), mobility);
        g.viscous = __fmul_rn(__fmul_rn(__fmul_rn(area, m.w), friction), mobility);
    }
    g.force = force;
    g.torque = cross(arm, force);
    g.s0 = force.x * arm;
    g.s1 = force.y * arm;
    g.s2 = force.z * arm;
    g.energy = cf.w;
    g.denom = length(force);
    g.depth = __fdiv_rn(pdv.w, bw);
    g.dissipation = r.slip[contact].w;
    g.normalPower = r.normalLossPower[contact];
    return g;
}
// Three CTAs of 256 per SM (at most 80 registers): measured faster than the
// unbounded 101-register build (two CTAs) and than four CTAs (spills).
__global__ void __launch_bounds__(256, 3) k_gather(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (r.control[0] != 0) return;
    uint32_t pairs = activePairs(r, c);
    __shared__ uint32_t window[8][4][WARP];  // per warp: B candidates, merged pairs, offsets, range ends
    __shared__ float termRows[8][GATHER_CHAINS][GATHER_STRIDE];
    uint32_t* wb = window[threadIdx.x >> 5][0];
    uint32_t* wp = window[threadIdx.x >> 5][1];
    uint32_t* wo = window[threadIdx.x >> 5][2];
    uint32_t* we = window[threadIdx.x >> 5][3];
    float (*terms)[GATHER_STRIDE] = termRows[threadIdx.x >> 5];
    const uint32_t chain = laneId();
    for (uint32_t id = warpGlobal(); id < c.N; id += warpStride()) {
        // This lane's chain: running value and compensation residual.
        float acc = 0.f, accLow = 0.f;
        f3 one = mk(1.f, 1.f, 1.f);
        float inverseInertia = mx(mx(dot(abs3(xyz(r.invI[3 * id])), one), dot(abs3(xyz(r.invI[3 * id + 1])), one)),
                                  dot(abs3(xyz(r.invI[3 * id + 2])), one));
        float m_ = r.body[id].y, bw = r.body[id].w;
        // Plane contacts come first in the grain's list: they were appended
        // last (highest wall first, each run from its last contact).
        for (uint32_t w = c.wallCount; w-- > 0;) {
            uint32_t lo = r.sideWallStart[w * c.N + id], hi = r.sideWallStart[w * c.N + id + 1];
            while (hi > lo) {
                uint32_t count = min(hi - lo, WARP);
                if (laneId() < count) storeTerms(terms, laneId(), wallTerms(r, c, hi - 1 - laneId(), w, m_, bw, inverseInertia));
                __syncwarp();
                replayChain(terms, count, chain, c.activeTimestep != 0, acc, accLow);
                __syncwarp();
                hi -= count;
            }
        }
        uint32_t aBegin = min(r.pairOffsets[id], pairs), aEnd = min(aBegin + r.pairCounts[id], pairs);
        uint32_t bBegin = r.byJOffsets[id], bEnd = r.byJOffsets[id + 1];
        // The grain's pairs in descending pair id (the first-grain run
        // aBegin..aEnd-1 and the second-grain run byJPairs[bBegin..bEnd),
        // both ascending, merged from the top), taken 32 at a time: each
        // window is merged by ranks, its pairs' contact ranges are scanned,
        // and its contacts -- each pair's from the last -- are processed 32
        // per round in that flattened order, the reference's LIFO order.
        uint32_t ia = aEnd, ib = bEnd;
        while (ia > aBegin || ib > bBegin) {
            uint32_t na = min(ia - aBegin, WARP), nb = min(ib - bBegin, WARP), lane = laneId();
            uint32_t bv = lane < nb ? r.byJPairs[ib - 1 - lane] : 0u;  // descending
            wb[lane] = bv;
            __syncwarp();
            // Rank of each candidate among the union of both windows.
            uint32_t av = ia - 1 - lane;                                // descending, valid for lane < na
            uint32_t rankA = WARP, rankB = WARP;
            if (lane < na) {
                uint32_t lo = 0, hi = nb;                               // B candidates greater than av
                while (lo < hi) { uint32_t mid = (lo + hi) >> 1; if (wb[mid] > av) lo = mid + 1; else hi = mid; }
                rankA = lane + lo;
            }
            if (lane < nb) {
                uint32_t greater = bv >= ia - 1 ? 0u : min(na, ia - 1 - bv);  // A candidates greater than bv
                rankB = lane + greater;
            }
            uint32_t takeA = __popc(__ballot_sync(0xffffffffu, rankA < WARP));
            uint32_t takeB = __popc(__ballot_sync(0xffffffffu, rankB < WARP));
            __syncwarp();
            if (rankA < WARP) wp[rankA] = av;
            if (rankB < WARP) wp[rankB] = bv;
            __syncwarp();
            uint32_t m = takeA + takeB, cnt = 0, pairId = 0, last = 0;
            if (lane < m) {
                pairId = wp[lane];
                uint32_t begin = r.sideContactStart[pairId];
                last = r.sideContactStart[pairId + 1];
                cnt = last - begin;
            }
            uint32_t incl = cnt;
#pragma unroll
            for (uint32_t o = 1; o < WARP; o <<= 1) {
                uint32_t t2 = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t2;
            }
            uint32_t total = __shfl_sync(0xffffffffu, incl, WARP - 1);
            wo[lane] = incl - cnt;
            we[lane] = last;
            __syncwarp();
            for (uint32_t q0 = 0; q0 < total; q0 += WARP) {
                uint32_t count = min(total - q0, WARP);
                GatherTerms g{};
                if (lane < count) {
                    uint32_t q = q0 + lane, lo = 0, hi = m;             // last window slot with offset <= q
                    while (hi - lo > 1) { uint32_t mid = (lo + hi) >> 1; if (wo[mid] <= q) lo = mid; else hi = mid; }
                    uint32_t p = wp[lo];
                    uint32_t contact = we[lo] - 1 - (q - wo[lo]);
                    uint4 key = r.meta[contact];
                    bool source = key.x == id;
                    float4 cf = r.contactForce[contact];
                    f3 force = xyz(cf);
                    float4 pdv = r.pointDepth[contact];
                    f3 arm = xyz(pdv);
                    f3 branch = xyz(r.dpairBranch[2 * p + (key.x > key.y ? 1u : 0u)]);
                    if (c.activeTimestep != 0) {
                        f3 localArm = source ? arm : arm - branch;
                        float mobility = __fadd_rn(__fdiv_rn(1.0f, m_), __fmul_rn(dot(localArm, localArm), inverseInertia));
                        float half = __fmul_rn(r.normalArea[contact].w, 0.5f);
                        g.stiffness = __fmul_rn(__fmul_rn(__fmul_rn(2.0f, half), __fadd_rn(__fmul_rn(c.kn, __fadd_rn(1.0f, c.mu)), c.kt)), mobility);
                        g.viscous = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(2.0f, half), c.normalViscosity), __fadd_rn(1.0f, c.mu)), mobility);
                    }
                    g.force = source ? force : -force;
                    g.torque = source ? cross(arm, force) : cross(arm - branch, -force);
                    g.s0 = __fmul_rn(0.5f, force.x) * branch;
                    g.s1 = __fmul_rn(0.5f, force.y) * branch;
                    g.s2 = __fmul_rn(0.5f, force.z) * branch;
                    g.energy = __fmul_rn(0.5f, cf.w);
                    g.denom = length(force);
                    uint32_t other = source ? key.y : key.x;
                    float wmin = source ? mn(bw, r.body[other].w) : mn(r.body[other].w, bw);
                    g.depth = __fdiv_rn(pdv.w, wmin);
                    g.dissipation = __fmul_rn(0.5f, r.slip[contact].w);
                    g.normalPower = __fmul_rn(0.5f, r.normalLossPower[contact]);
                    storeTerms(terms, lane, g);
                }
                __syncwarp();
                replayChain(terms, count, chain, c.activeTimestep != 0, acc, accLow);
                __syncwarp();
            }
            __syncwarp();
            ia -= takeA;
            ib -= takeB;
        }
        // Collect the chains on lane 0.
        float sums[GATHER_CHAINS], lows[6];
#pragma unroll
        for (uint32_t j = 0; j < GATHER_CHAINS; ++j) sums[j] = __shfl_sync(0xffffffffu, acc, int(j));
#pragma unroll
        for (uint32_t j = 0; j < 6; ++j) lows[j] = __shfl_sync(0xffffffffu, accLow, int(j));
        if (laneId() == 0) {
            f3 f = mk(sums[0], sums[1], sums[2]) + mk(lows[0], lows[1], lows[2]);
            f3 t = mk(sums[3], sums[4], sums[5]) + mk(lows[3], lows[4], lows[5]);
            f3 stress0 = mk(sums[6], sums[7], sums[8]), stress1 = mk(sums[9], sums[10], sums[11]),
               stress2 = mk(sums[12], sums[13], sums[14]);
            float energy = sums[15], denom = sums[16], maxDepth = sums[17], dissipation = sums[18],
                  normalPower = sums[19], stiffnessRate = sums[20], viscousRate = sums[21];
            r.timestepRows[id] = make_float4(stiffnessRate, viscousRate, 0.f, 0.f);
            float4 ns = r.normalDamping[id];
            ns.z = normalPower;
            r.normalDamping[id] = ns;
            r.force[id] = w4(f, maxDepth);
            r.torque[id] = w4(t, dissipation);
            r.particleStress[3 * id] = w4(stress0, 0.f);
            r.particleStress[3 * id + 1] = w4(stress1, 0.f);
            r.particleStress[3 * id + 2] = w4(stress2, 0.f);
            f3 v = xyz(r.velocity[id]);
            float kinetic = __fmul_rn(0.5f, __fadd_rn(__fmul_rn(m_, dot(v, v)), dot(xyz(r.momentum[id]), omegaOf(r, id))));
            r.particleDiagnostic[id] = make_float4(kinetic, energy, length(f), denom);
            float4 high = r.accumulated[id], low = r.accumulatedRemainder[id];
            compensated4(high, low, make_float4(dissipation, 0.f, 0.f, 0.f));
            r.accumulated[id] = high;
            r.accumulatedRemainder[id] = low;
        }
    }
}

// ---------------------------------------------------------------- launchers
static inline uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }
constexpr uint32_t PERSISTENT = 152 * 8;  // warps-per-item kernels: 8 CTAs of 256 per SM

// SMs of the current device (152 on GB300), read once.
static uint32_t smCount() {
    static uint32_t sms = 0;
    if (!sms) {
        int device = 0, count = 0;
        if (cudaGetDevice(&device) == cudaSuccess &&
            cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && count > 0)
            sms = uint32_t(count);
        else
            sms = 152;
    }
    return sms;
}
// Grid of `perSM` CTAs per SM (the tuned value, or `fallback` when 0).
static inline uint32_t grid(uint32_t perSM, uint32_t fallback) { return smCount() * (perSM ? perSM : fallback); }

// The neighbour build on rebuild steps (every kernel returns at once on the
// others): the cell list by radix sort (or, where byJPairs is too small to
// hold the sort's scratch, by atomic fill and a rank sort per bin), the pair
// search with a warp per grain, then the pairs grouped by second grain.
static void neighbours(const Params& P, cudaStream_t s) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t T = 256;
    k_binsClear<<<blocks(c.binCount, T), T, 0, s>>>(P);
    if (uint64_t(c.pairCapacity) >= radixWords(c.N)) {
        uint32_t tiles = radixTiles(c.N), from = 0, bits = 1;
        while (bits < 32 && (uint64_t(1) << bits) <= c.binCount) ++bits;  // keys 0 .. binCount
        k_binKeys<<<blocks(c.N, T), T, 0, s>>>(P);
        RadixScratch x = radixScratch(r, c);
        for (uint32_t shift = 0; shift < bits; shift += 8, from ^= 1u) {
            k_radixCount<<<tiles, T, 0, s>>>(P, shift, from);
            launch_step_scan(r, x.counts, x.counts, ScanCount{nullptr, 0, 0, RADIX * tiles}, false, nullptr,
                             r.control + 4, s);
            k_radixScatter<<<tiles, T, 0, s>>>(P, shift, from);
        }
        k_binsFromSorted<<<blocks(c.N, T), T, 0, s>>>(P, from);
    } else {
        k_binsFill<<<blocks(c.N, T), T, 0, s>>>(P);
        k_binsSort<<<min(c.binCount, 152u * 16u), 128, 2 * c.binCapacity * sizeof(uint32_t), s>>>(P);
    }
    k_pairsCountWarp<<<PERSISTENT, T, 0, s>>>(P);
    launch_step_scan(r, r.pairCounts, r.pairOffsets, ScanCount{nullptr, 0, 0, c.N}, false, r.control + 1, r.control + 4,
                s);
    k_pairsEmitWarp<<<PERSISTENT, T, 0, s>>>(P);
    k_byJReset<<<blocks(c.N + 1, T), T, 0, s>>>(P);
    k_byJCount<<<PERSISTENT, T, 0, s>>>(P);
    launch_step_scan(r, r.byJCounts, r.byJOffsets, ScanCount{nullptr, 0, 0, c.N}, true, nullptr, r.control + 4,
                s);
    k_byJFill<<<PERSISTENT, T, 0, s>>>(P);
    k_byJSort<<<blocks(c.N, T), T, 0, s>>>(P);
}

// Pair set-up (branches, the stored-filter motion check); with the SDF
// geometry also the contact counts and their scan.
static void collectHead(const Params& P, cudaStream_t s) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t T = 256;
    k_resetContacts<<<1, 1, 0, s>>>(P);
    k_pairSetup<<<grid(c.cullBlocksPerSM, 8), T, 0, s>>>(P);
    if (c.meshGeometry == 0) {
        k_sdfCount<<<grid(c.queryBlocksPerSM, 8), T, 0, s>>>(P);
        launch_step_scan(r, r.contactCounts, r.contactOffsets, ScanCount{r.control + 1, c.pairCapacity, 1, 0}, false,
                    r.control + 2, nullptr, s);
    }
}
// Root masks, leaf cull and the (directed pair, leaf) item list: steps that
// build the filter results (every kernel returns at once on the others).
static void cullBuild(const Params& P, cudaStream_t s) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (c.meshGeometry == 0) return;
    uint32_t T = 256, g = grid(c.cullBlocksPerSM, 8);
    k_pairMasks<<<g, T, 0, s>>>(P);
    k_leafCull<<<g, T, 0, s>>>(P);
    launch_step_scan(r, r.dpairLeafCount, r.dpairCandOffset, ScanCount{r.control + 1, c.pairCapacity, 2, 0}, true,
                r.work + W_CANDIDATES, r.work + W_FILTER, s);
    k_leafEmit<<<g, T, 0, s>>>(P);
}
// Pair set-up, leaf cull and the (directed pair, leaf) item list; with the
// SDF geometry, pair set-up, contact counts and their scan.
static void collectCull(const Params& P, cudaStream_t s) {
    collectHead(P, s);
    cullBuild(P, s);
}
// Node filter, survivor list and (with the learned culler) the kept list.
static void collectFilter(const Params& P, cudaStream_t s) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (c.meshGeometry == 0) return;
    uint32_t warps = c.queryWarps == 4 ? 4 : 8;
    k_nodeFilter<<<grid(c.queryBlocksPerSM, 8), 32 * warps, 0, s>>>(P);
    launch_step_scan(r, r.candSurvCount, r.candSurvOffset, ScanCount{r.work + W_CANDIDATES, c.candidateCapacity, 1, 0},
                true, r.work + W_SURVIVORS, r.work + W_FILTER, s);
    k_survivorList<<<grid(c.contactBlocksPerSM, 8), 256, 0, s>>>(P);
    k_survivorPrefilter<<<grid(c.walkBlocksPerSM, 8), 256, 0, s>>>(P);
    if (c.cullerEnabled) {
        uint32_t g = grid(c.contactBlocksPerSM, 8);
        k_cullCount<<<g, 256, 0, s>>>(P);
        launch_step_scan(r, r.walkBucketCount, r.walkBucketOffset, ScanCount{nullptr, 0, 0, c.shapes}, true,
                         r.work + W_CULL_ROWS, nullptr, s);
        k_cullPlace<<<g, 256, 0, s>>>(P);
        k_cullSurvivors<<<grid(0, 4), CULLER_ROWS, 0, s>>>(P);  // 4 x 64 TMEM columns per SM
    }
    if (c.filterMargin > 0.0f && c.cullerEnabled == 0)
        launch_step_scan(r, r.walkBucketCount, r.walkBucketOffset, ScanCount{nullptr, 0, 0, c.shapes * WALK_BUCKETS}, true,
                    r.work + W_KEPT, r.work + W_FILTER, s);
    else
        launch_step_scan(r, r.survKeep, r.keepOffset, ScanCount{r.work + W_SURVIVORS, c.survivorCapacity, 1, 0}, true,
                    r.work + W_KEPT, nullptr, s);
    k_walkList<<<grid(c.contactBlocksPerSM, 8), 256, 0, s>>>(P);
}
// The exact queries.
static void collectWalk(const Params& P, cudaStream_t s) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (c.meshGeometry == 0) {
        k_sdfEmit<<<grid(c.queryBlocksPerSM, 8), 256, 0, s>>>(P);
    } else if (c.filterMargin > 0.0f && c.cullerEnabled == 0) {
        uint32_t g = grid(c.walkBlocksPerSM, 8);
        k_nodeWalkKnown<<<g, 256, 0, s>>>(P);
        // The flags' scan also lists the flagged slots in slot order (the
        // walk-bucket order) into walkKey.
        launch_step_scan(r, r.survKeep, r.keepOffset, ScanCount{r.work + W_KEPT, c.survivorCapacity, 1, 0}, true,
                         r.work + W_SLOW, nullptr, s, r.walkKey);
        if (c.shapes <= STAGE_MAX_SHAPES) {
            size_t dynamic = STAGE_BYTES + 4 * (size_t(c.shapes) + 1);
            // The opt-in shared-memory limit, set once per device.
            static uint64_t attributed = 0;
            int device = 0;
            cudaGetDevice(&device);
            if (device < 64 && !((attributed >> device) & 1u)) {
                cudaFuncSetAttribute(k_nodeWalkStaged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(STAGE_BYTES + 4 * (STAGE_MAX_SHAPES + 1)));
                attributed |= uint64_t(1) << device;
            }
            k_nodeWalkStaged<<<smCount(), STAGE_THREADS, dynamic, s>>>(P);
            k_nodeWalkSlow<<<g, 256, 0, s>>>(P, 2u * smCount() * (STAGE_THREADS / 32));
        } else {
            k_nodeWalkSlow<<<g, 256, 0, s>>>(P, 0u);
        }
    } else {
        k_nodeWalk<<<grid(c.walkBlocksPerSM, 8), 256, 0, s>>>(P);
    }
}
static void collectQuery(const Params& P, cudaStream_t s) {
    collectFilter(P, s);
    collectWalk(P, s);
}
// Canonical offsets of the hits, the contact records and per-pair starts.
static void collectEmit(const Params& P, cudaStream_t s) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (c.meshGeometry == 0) return;
    launch_step_scan(r, r.candHitCount, r.candHitOffset, ScanCount{r.work + W_CANDIDATES, c.candidateCapacity, 1, 0}, true,
                r.control + 2, nullptr, s);
    uint32_t g = grid(c.contactBlocksPerSM, 8);
    if (storedKeep(c)) {
        k_emitSlots<<<g, 256, 0, s>>>(P);
        k_clearHits<<<g, 256, 0, s>>>(P);  // and the per-pair contact starts
    } else {
        k_nodeEmit<<<g, 256, 0, s>>>(P);
        k_contactStart<<<g, 256, 0, s>>>(P);
    }
}
// Plane contacts after the grain-grain ones: counts, their scan, records.
static void collectWalls(const Params& P, cudaStream_t s) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (c.wallCount == 0) return;
    uint32_t items = c.N * c.wallCount, g = min(blocks(items, 8), grid(0, 8));
    k_wallCount<<<g, 256, 0, s>>>(P);
    launch_step_scan(r, r.wallCounts, r.wallOffsets, ScanCount{nullptr, 0, 0, items}, true, nullptr, nullptr, s);
    k_wallEmit<<<g, 256, 0, s>>>(P);
}
static void contacts(const Params& P, cudaStream_t s) {
    collectCull(P, s);
    collectQuery(P, s);
    collectEmit(P, s);
    collectWalls(P, s);
}
// The exact queries, contact emit and plane contacts: the part of the
// collector every step runs once the filter results are in place.
static void collectTail(const Params& P, cudaStream_t s) {
    collectWalk(P, s);
    collectEmit(P, s);
    collectWalls(P, s);
}

int launch_contacts(const std::string_view& name, const Params& P, uint32_t count, cudaStream_t s) {
    const Config& c = P.c;
    uint32_t T = 256;
    if (name == "neighbours") neighbours(P, s);
    else if (name == "collect") contacts(P, s);
    else if (name == "collectCull") collectCull(P, s);
    else if (name == "collectHead") collectHead(P, s);
    else if (name == "prefetch") {
        if (c.meshGeometry != 0) k_prefetch<<<grid(0, 2), 64, 0, s>>>(P);
    }
    else if (name == "collectBuild") { cullBuild(P, s); collectFilter(P, s); }
    else if (name == "collectTail") collectTail(P, s);
    else if (name == "collectQuery") collectQuery(P, s);
    else if (name == "collectFilter") collectFilter(P, s);
    else if (name == "collectWalk") collectWalk(P, s);
    else if (name == "collectEmit") collectEmit(P, s);
    else if (name == "resolveContacts") {
        k_resolve<<<grid(c.contactBlocksPerSM, 8), T, 0, s>>>(P);
        if (c.wallCount) k_resolveWalls<<<grid(0, 2), T, 0, s>>>(P);
    }
    else if (name == "distanceGrid") {
        if (c.meshGeometry != 0) k_distanceGrid<<<grid(0, 8), T, 0, s>>>(P);
    }
    else if (name == "gather") k_gather<<<min(blocks(c.N, 8), max(1u, grid(c.gatherWarps, 64) / 8)), T, 0, s>>>(P);
    else if (name == "collectWalls") collectWalls(P, s);
    else if (name == "gatherWallRows") {
        if (c.wallCount) k_gatherWallRows<<<blocks(c.N * c.wallCount, T), T, 0, s>>>(P);
    }
    else return 1;
    (void)count;
    return 0;
}

}  // namespace sdg
