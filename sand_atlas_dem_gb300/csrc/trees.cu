// Median-split trees of the packed mesh layout, built on the device.
//
// The reference packs two trees per shape on the host, by recursion
// (src/sand_atlas_dem/mesh.py): the source-node cluster tree (`partition`,
// mesh.py:33-56; at most 64 nodes a leaf) and the triangle BVH (`build`,
// mesh.py:164-201; at most 4 triangles a leaf).  Both follow one rule: a node
// holding m items splits when m exceeds the leaf size, by a stable sort of
// its items along the axis of largest key extent (np.ptp(...).argmax(): the
// first axis on ties), the left child taking the first m/2.  Its bounds are
// the items' FP32 minimum and maximum moved one ulp outward (np.nextafter),
// and nodes are numbered in preorder with an escape link past the subtree.
//
// The shape of such a tree depends on the item count alone: the preorder
// index of a right child is its parent's + 1 + nodes(m/2), where nodes(m) is
// the node count of a tree over m items (treeNodes below).  Only the order of
// the items and the bounds depend on the coordinates.  So the build runs
// level by level over every shape at once instead of by recursion:
//
//   1. bounds and key extents of each node of the level: a warp per piece of
//      at most PIECE items, the pieces' partials folded per node (no atomics);
//   2. the node's record (escape link; first item and count for a leaf), its
//      bounds, its split axis, and its two children appended to the next
//      level's list;
//   3. the stable sort of each internal node's items by the split coordinate:
//      nodes of at most SMALL items by rank in shared memory (a warp a node),
//      larger ones by four 8-bit LSD radix passes whose digit offsets are
//      taken per node, so items never leave their node's range.
//
// The sort key maps an FP32 coordinate to an order-preserving uint32, with
// -0 read as +0: numpy compares the two equal, so a stable sort keeps their
// order.  Item coordinates must be finite (the host checks).
#include <algorithm>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "launch.h"

namespace sdg {
namespace trees {

constexpr uint32_t PIECE = 8192;  // items one warp reduces
constexpr uint32_t SMALL = 256;   // largest node sorted by rank in shared memory
constexpr uint32_t TILE = 2048;   // items of one radix block (256 threads x 8)
constexpr uint32_t RADIX = 256;
constexpr uint32_t MAX_LEVELS = 64;
constexpr uint32_t MAX_ITEMS = 1u << 30;

// One node of a level: preorder index, first item, item count, split axis.
struct Entry {
    uint32_t node, start, count, axis;
};

// Node count of the median-split tree over m items.  The sizes of one level
// are at most two consecutive integers k and k + 1 (children of k and k + 1
// are k/2 or k/2 + 1), so each level is two (size, multiplicity) pairs.
__host__ __device__ inline uint32_t treeNodes(uint32_t m, uint32_t leaf) {
    uint32_t size[2] = {m, 0}, mult[2] = {1, 0}, total = 0;
    while (mult[0] | mult[1]) {
        uint32_t ns[2] = {0, 0}, nm[2] = {0, 0};
        for (int e = 0; e < 2; ++e) {
            if (!mult[e]) continue;
            total += mult[e];
            if (size[e] <= leaf) continue;
            const uint32_t half[2] = {size[e] / 2, size[e] - size[e] / 2};
            for (int h = 0; h < 2; ++h) {
                const int slot = (nm[0] == 0 || ns[0] == half[h]) ? 0 : 1;
                ns[slot] = half[h];
                nm[slot] += mult[e];
            }
        }
        size[0] = ns[0]; size[1] = ns[1]; mult[0] = nm[0]; mult[1] = nm[1];
    }
    return total;
}

__device__ __forceinline__ float nextDown(float x) {
    const uint32_t u = __float_as_uint(x);
    if ((u & 0x7fffffffu) == 0) return __uint_as_float(0x80000001u);  // +-0 -> -smallest subnormal
    return __uint_as_float(u & 0x80000000u ? u + 1 : u - 1);
}

__device__ __forceinline__ float nextUp(float x) {
    const uint32_t u = __float_as_uint(x);
    if ((u & 0x7fffffffu) == 0) return __uint_as_float(0x00000001u);
    return __uint_as_float(u & 0x80000000u ? u - 1 : u + 1);
}

__device__ __forceinline__ uint32_t sortable(float x) {
    uint32_t u = __float_as_uint(x);
    if (u == 0x80000000u) u = 0;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float component(const float4& v, uint32_t axis) {
    return axis == 0 ? v.x : (axis == 1 ? v.y : v.z);
}

__global__ void k_treeIota(uint32_t* order, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) order[i] = i;
}

// Turns each position's item index into its row within its shape: the
// shape is the last whose first item is at or before the position (items
// never leave their shape).
__global__ void k_treeLocal(uint32_t* order, uint32_t n, const uint32_t* firsts, uint32_t shapes) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = shapes - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (firsts[mid] <= p) lo = mid; else hi = mid - 1;
        }
        order[p] -= firsts[lo];
    }
}

// Partial extents of one piece of one node: key minimum and maximum, box
// minimum and maximum (12 floats).  Warp w handles piece w % parts of entry
// w / parts.  `low`/`high` null: the boxes are the keys (single points).
__global__ void __launch_bounds__(256) k_treeReduce(const Entry* level, uint32_t entries, uint32_t parts,
                                                    const float4* keys, const float4* low, const float4* high,
                                                    const uint32_t* order, float* partial) {
    const uint64_t w = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (w >= uint64_t(entries) * parts) return;
    const Entry e = level[w / parts];
    const uint32_t piece = uint32_t(w % parts);
    if (uint64_t(piece) * PIECE >= e.count) return;
    const uint32_t begin = e.start + piece * PIECE;
    const uint32_t end = e.start + min(e.count, (piece + 1) * PIECE);
    float a[12];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        a[c] = a[6 + c] = INFINITY;
        a[3 + c] = a[9 + c] = -INFINITY;
    }
    // Four items a lane per round: their index loads, then their key (and
    // box) gathers, issued back to back.
    for (uint32_t base = begin + lane; base < end; base += 128) {
        uint32_t id[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) id[u] = base + 32 * u < end ? order[base + 32 * u] : 0xffffffffu;
        float4 k[4], l[4], h[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (id[u] == 0xffffffffu) continue;
            k[u] = keys[id[u]];
            l[u] = low ? low[id[u]] : k[u];
            h[u] = high ? high[id[u]] : k[u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (id[u] == 0xffffffffu) continue;
            a[0] = fminf(a[0], k[u].x); a[1] = fminf(a[1], k[u].y); a[2] = fminf(a[2], k[u].z);
            a[3] = fmaxf(a[3], k[u].x); a[4] = fmaxf(a[4], k[u].y); a[5] = fmaxf(a[5], k[u].z);
            a[6] = fminf(a[6], l[u].x); a[7] = fminf(a[7], l[u].y); a[8] = fminf(a[8], l[u].z);
            a[9] = fmaxf(a[9], h[u].x); a[10] = fmaxf(a[10], h[u].y); a[11] = fmaxf(a[11], h[u].z);
        }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
#pragma unroll
        for (int c = 0; c < 12; ++c) {
            const float o = __shfl_xor_sync(0xffffffffu, a[c], off);
            a[c] = (c % 6) < 3 ? fminf(a[c], o) : fmaxf(a[c], o);
        }
    }
    if (lane < 12) {
        float v = a[0];
#pragma unroll
        for (int c = 1; c < 12; ++c) v = lane == c ? a[c] : v;
        partial[w * 12 + lane] = v;
    }
}

// Folds a node's pieces; writes its record (escape, first item, count,
// depth; first and count zero for an internal node) and outward-rounded
// bounds; for an internal node picks the split axis, appends the two
// children to the next level and the node to the small or large sort list.
__global__ void __launch_bounds__(256) k_treeNodes(const Entry* level, uint32_t entries, uint32_t parts,
                                                   const float* partial, uint32_t leaf, uint32_t depth,
                                                   uint4* records, float4* nodeLow, float4* nodeHigh, Entry* next,
                                                   Entry* large, Entry* small, uint32_t* counters) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= entries) return;
    const Entry e = level[i];
    float a[12];
    const float* p = partial + uint64_t(i) * parts * 12;
#pragma unroll
    for (int c = 0; c < 12; ++c) a[c] = p[c];
    const uint32_t pieces = (e.count + PIECE - 1) / PIECE;
    for (uint32_t j = 1; j < pieces; ++j) {
#pragma unroll
        for (int c = 0; c < 12; ++c) {
            const float o = p[j * 12 + c];
            a[c] = (c % 6) < 3 ? fminf(a[c], o) : fmaxf(a[c], o);
        }
    }
    nodeLow[e.node] = make_float4(nextDown(a[6]), nextDown(a[7]), nextDown(a[8]), 0.f);
    nodeHigh[e.node] = make_float4(nextUp(a[9]), nextUp(a[10]), nextUp(a[11]), 0.f);
    const uint32_t escape = e.node + treeNodes(e.count, leaf);
    if (e.count <= leaf) {
        records[e.node] = make_uint4(escape, e.start, e.count, depth);
        return;
    }
    records[e.node] = make_uint4(escape, 0, 0, depth);
    const float extent[3] = {a[3] - a[0], a[4] - a[1], a[5] - a[2]};
    uint32_t axis = 0;
    if (extent[1] > extent[axis]) axis = 1;
    if (extent[2] > extent[axis]) axis = 2;
    const uint32_t half = e.count / 2;
    const uint32_t slot = atomicAdd(&counters[0], 2u);
    next[slot] = Entry{e.node + 1, e.start, half, 0};
    next[slot + 1] = Entry{e.node + 1 + treeNodes(half, leaf), e.start + half, e.count - half, 0};
    const Entry task{e.node, e.start, e.count, axis};
    if (e.count > SMALL)
        large[atomicAdd(&counters[1], 1u)] = task;
    else
        small[atomicAdd(&counters[2], 1u)] = task;
}

// Stable sort of a node of at most SMALL items, a warp per node: an item's
// place is the number of items with a smaller key, plus the earlier items
// with an equal one.
__global__ void __launch_bounds__(256) k_treeSmallSort(const Entry* small, uint32_t count, const float4* keys,
                                                       uint32_t* order) {
    __shared__ uint32_t key[8][SMALL], ids[8][SMALL];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t i = blockIdx.x * 8 + warp;
    if (i >= count) return;
    const Entry e = small[i];
    for (uint32_t t = lane; t < e.count; t += 32) {
        const uint32_t id = order[e.start + t];
        ids[warp][t] = id;
        key[warp][t] = sortable(component(keys[id], e.axis));
    }
    __syncwarp();
    for (uint32_t t = lane; t < e.count; t += 32) {
        const uint32_t k = key[warp][t];
        uint32_t rank = 0;
        for (uint32_t u = 0; u < e.count; ++u) {
            const uint32_t ku = key[warp][u];
            rank += (ku < k) | ((ku == k) & (u < t));
        }
        order[e.start + rank] = ids[warp][t];
    }
}

// Radix pass `pass` over the large nodes, block b = tile b % tiles of node
// b / tiles: the tile's digit histogram.  Pass 0 also writes the sort keys.
__global__ void __launch_bounds__(256) k_treeCount(const Entry* large, uint32_t tiles, uint32_t pass,
                                                   const float4* keys, const uint32_t* order, uint32_t* key0,
                                                   const uint32_t* keySrc, uint32_t* counts) {
    __shared__ uint32_t hist[RADIX];
    const Entry e = large[blockIdx.x / tiles];
    const uint32_t tile = blockIdx.x % tiles;
    if (uint64_t(tile) * TILE >= e.count) return;
    const uint32_t begin = e.start + tile * TILE, end = e.start + min(e.count, (tile + 1) * TILE);
    hist[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t shift = 8 * pass;
    // A thread's (at most) 8 items: loads first, then the histogram.
    uint32_t k[TILE / 256];
#pragma unroll
    for (int j = 0; j < int(TILE / 256); ++j) {
        const uint32_t p = begin + j * 256 + threadIdx.x;
        if (p >= end) continue;
        if (pass == 0) {
            k[j] = sortable(component(keys[order[p]], e.axis));
            key0[p] = k[j];
        } else {
            k[j] = keySrc[p];
        }
    }
#pragma unroll
    for (int j = 0; j < int(TILE / 256); ++j)
        if (begin + j * 256 + threadIdx.x < end) atomicAdd(&hist[(k[j] >> shift) & (RADIX - 1)], 1u);
    __syncthreads();
    counts[uint64_t(blockIdx.x) * RADIX + threadIdx.x] = hist[threadIdx.x];
}

// Per large node: replaces its tiles' digit counts by the places their first
// items take -- the node's first item, plus every item of a smaller digit,
// plus the earlier tiles' items of the same digit.
__global__ void __launch_bounds__(256) k_treeOffsets(const Entry* large, uint32_t tiles, uint32_t* counts) {
    __shared__ uint32_t warpTotal[8];
    const Entry e = large[blockIdx.x];
    const uint32_t used = (e.count + TILE - 1) / TILE;
    uint32_t* c = counts + uint64_t(blockIdx.x) * tiles * RADIX + threadIdx.x;
    uint32_t total = 0;
    for (uint32_t t = 0; t < used; ++t) total += c[uint64_t(t) * RADIX];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = total;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) warpTotal[warp] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; ++w) before += warpTotal[w];
    uint32_t running = e.start + before + incl - total;
    for (uint32_t t = 0; t < used; ++t) {
        const uint32_t n = c[uint64_t(t) * RADIX];
        c[uint64_t(t) * RADIX] = running;
        running += n;
    }
}

// Lanes of the warp whose digit equals this lane's: one ballot per digit
// bit, plus one on validity (invalid lanes match only each other).
__device__ __forceinline__ uint32_t sameDigit(uint32_t digit, bool valid) {
    uint32_t peers = __ballot_sync(0xffffffffu, valid);
    if (!valid) peers = ~peers;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const bool bit = (digit >> b) & 1u;
        const uint32_t set = __ballot_sync(0xffffffffu, bit);
        peers &= bit ? set : ~set;
    }
    return peers;
}

// Stable scatter of a tile.  Warp w holds the tile's items w*256 .. w*256+255
// (8 a lane, loaded first, kept in registers) and ranks them among its own
// items of the same digit: earlier sub-rounds through its shared histogram,
// lower lanes of the same sub-round through the digit match.  A prefix over
// the warps of each digit's count gives each warp its first rank per digit
// within the tile.  The items are then staged in shared memory in digit
// order and written out from there, so that consecutive threads write
// consecutive places of a digit's run (coalesced stores).
__global__ void __launch_bounds__(256) k_treeScatter(const Entry* large, uint32_t tiles, uint32_t pass,
                                                     const uint32_t* counts, const uint32_t* keySrc,
                                                     const uint32_t* orderSrc, uint32_t* keyDst, uint32_t* orderDst) {
    __shared__ uint32_t hist[8][RADIX];
    __shared__ uint32_t tileBase[RADIX], localBase[RADIX], warpTotal[8];
    __shared__ uint32_t stagedKey[TILE], stagedId[TILE];
    const Entry e = large[blockIdx.x / tiles];
    const uint32_t tile = blockIdx.x % tiles;
    if (uint64_t(tile) * TILE >= e.count) return;
    const uint32_t begin = e.start + tile * TILE, end = e.start + min(e.count, (tile + 1) * TILE);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t first = begin + warp * 256 + lane;
    uint32_t key[8], id[8], rank[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t p = first + j * 32;
        key[j] = p < end ? keySrc[p] : 0u;
        id[j] = p < end ? orderSrc[p] : 0u;
    }
#pragma unroll
    for (int w = 0; w < 8; ++w) hist[w][threadIdx.x] = 0;
    __syncthreads();
    const uint32_t shift = 8 * pass;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const bool valid = first + j * 32 < end;
        const uint32_t digit = (key[j] >> shift) & (RADIX - 1);
        const uint32_t peers = sameDigit(digit, valid);
        const uint32_t below = __popc(peers & ((1u << lane) - 1u));
        const uint32_t before = valid ? hist[warp][digit] : 0u;
        __syncwarp();
        if (valid && below == 0) hist[warp][digit] = before + __popc(peers);
        __syncwarp();
        rank[j] = before + below;
    }
    __syncthreads();
    // Thread d: the warps' first ranks for digit d, the tile's count of it,
    // and (block scan) where digit d starts among the tile's items.
    uint32_t total = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        const uint32_t c = hist[w][threadIdx.x];
        hist[w][threadIdx.x] = total;
        total += c;
    }
    uint32_t incl = total;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) warpTotal[warp] = incl;
    tileBase[threadIdx.x] = counts[uint64_t(blockIdx.x) * RADIX + threadIdx.x];
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; ++w) before += warpTotal[w];
    localBase[threadIdx.x] = before + incl - total;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (first + j * 32 < end) {
            const uint32_t digit = (key[j] >> shift) & (RADIX - 1);
            const uint32_t at = localBase[digit] + hist[warp][digit] + rank[j];
            stagedKey[at] = key[j];
            stagedId[at] = id[j];
        }
    }
    __syncthreads();
    const uint32_t n = end - begin;
    for (uint32_t q = threadIdx.x; q < n; q += 256) {
        const uint32_t k = stagedKey[q];
        const uint32_t digit = (k >> shift) & (RADIX - 1);
        const uint32_t place = tileBase[digit] + (q - localBase[digit]);
        keyDst[place] = k;
        orderDst[place] = stagedId[q];
    }
}

// Per-level sizes of every shape's tree, for launch shapes and scratch.
struct LevelPlan {
    uint64_t entries = 0, large = 0, small = 0;
    uint32_t maxCount = 0, maxLarge = 0;
};

static std::vector<LevelPlan> plan(const uint32_t* counts, uint32_t shapes, uint32_t leaf) {
    std::vector<LevelPlan> levels;
    for (uint32_t s = 0; s < shapes; ++s) {
        uint64_t size[2] = {counts[s], 0}, mult[2] = {1, 0};
        for (uint32_t d = 0; mult[0] | mult[1]; ++d) {
            if (levels.size() <= d) levels.resize(d + 1);
            LevelPlan& L = levels[d];
            uint64_t ns[2] = {0, 0}, nm[2] = {0, 0};
            for (int e = 0; e < 2; ++e) {
                if (!mult[e]) continue;
                L.entries += mult[e];
                L.maxCount = std::max<uint32_t>(L.maxCount, uint32_t(size[e]));
                if (size[e] <= leaf) continue;
                if (size[e] > SMALL) {
                    L.large += mult[e];
                    L.maxLarge = std::max<uint32_t>(L.maxLarge, uint32_t(size[e]));
                } else {
                    L.small += mult[e];
                }
                const uint64_t half[2] = {size[e] / 2, size[e] - size[e] / 2};
                for (int h = 0; h < 2; ++h) {
                    const int slot = (nm[0] == 0 || ns[0] == half[h]) ? 0 : 1;
                    ns[slot] = half[h];
                    nm[slot] += mult[e];
                }
            }
            size[0] = ns[0]; size[1] = ns[1]; mult[0] = nm[0]; mult[1] = nm[1];
        }
    }
    return levels;
}

struct Scratch {
    uint64_t lists, large, small, partial, counts, keys, order, counters, firsts, total;
};

static uint64_t align256(uint64_t x) { return (x + 255) & ~uint64_t(255); }

static Scratch layout(const std::vector<LevelPlan>& levels, uint64_t items, uint32_t shapes) {
    uint64_t entries = 1, large = 1, small = 1, partial = 1, counts = 1;
    for (const LevelPlan& L : levels) {
        entries = std::max(entries, L.entries);
        large = std::max(large, L.large);
        small = std::max(small, L.small);
        partial = std::max(partial, L.entries * ((L.maxCount + PIECE - 1) / PIECE));
        counts = std::max(counts, L.large * ((L.maxLarge + TILE - 1) / TILE));
    }
    Scratch s{};
    uint64_t at = 0;
    s.lists = at; at += align256(2 * entries * sizeof(Entry));
    s.large = at; at += align256(large * sizeof(Entry));
    s.small = at; at += align256(small * sizeof(Entry));
    s.partial = at; at += align256(partial * 12 * sizeof(float));
    s.counts = at; at += align256(counts * RADIX * sizeof(uint32_t));
    s.keys = at; at += align256(2 * items * sizeof(uint32_t));
    s.order = at; at += align256(items * sizeof(uint32_t));
    s.counters = at; at += align256(MAX_LEVELS * 4 * sizeof(uint32_t));
    s.firsts = at; at += align256(uint64_t(shapes) * sizeof(uint32_t));
    s.total = at;
    return s;
}

static int check(const uint32_t* counts, uint32_t shapes, uint32_t leaf, uint64_t& items, uint64_t& nodes) {
    if (!counts || shapes == 0 || leaf == 0) {
        set_last_error("median trees: need at least one shape and a leaf size of at least 1");
        return 1;
    }
    items = 0;
    nodes = 0;
    for (uint32_t s = 0; s < shapes; ++s) {
        if (counts[s] == 0) {
            set_last_error("median trees: shape " + std::to_string(s) + " has no items");
            return 1;
        }
        items += counts[s];
        if (items > MAX_ITEMS) {
            set_last_error("median trees: more than 2^30 items");
            return 1;
        }
        nodes += treeNodes(counts[s], leaf);
    }
    return 0;
}

}  // namespace trees
}  // namespace sdg

using namespace sdg;
using namespace sdg::trees;

extern "C" uint32_t sdg_median_tree_nodes(uint32_t items, uint32_t leaf) {
    return (items == 0 || leaf == 0) ? 0u : treeNodes(items, leaf);
}

extern "C" uint64_t sdg_median_trees_scratch(const uint32_t* counts, uint32_t shapes, uint32_t leaf) {
    uint64_t items, nodes;
    if (check(counts, shapes, leaf, items, nodes)) return 0;
    return layout(plan(counts, shapes, leaf), items, shapes).total;
}

extern "C" int sdg_median_trees(const float* keys, const float* low, const float* high, const uint32_t* counts,
                                uint32_t shapes, uint32_t leaf, uint32_t* order, uint32_t* records, float* nodeLow,
                                float* nodeHigh, void* scratch, uint64_t scratchBytes, void* stream) {
    uint64_t items, nodes;
    if (check(counts, shapes, leaf, items, nodes)) return 1;
    if (!keys || !order || !records || !nodeLow || !nodeHigh || !scratch || (!low) != (!high)) {
        set_last_error("median trees: null buffer (low and high must both be given or both be null)");
        return 1;
    }
    const std::vector<LevelPlan> levels = plan(counts, shapes, leaf);
    if (levels.size() > MAX_LEVELS) {
        set_last_error("median trees: more than 64 levels");
        return 1;
    }
    const Scratch sl = layout(levels, items, shapes);
    if (scratchBytes < sl.total) {
        set_last_error("median trees: scratch smaller than sdg_median_trees_scratch()");
        return 1;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char* base = static_cast<char*>(scratch);
    uint64_t maxEntries = 1;
    for (const LevelPlan& L : levels) maxEntries = std::max(maxEntries, L.entries);
    Entry* lists[2] = {reinterpret_cast<Entry*>(base + sl.lists), reinterpret_cast<Entry*>(base + sl.lists) + maxEntries};
    Entry* large = reinterpret_cast<Entry*>(base + sl.large);
    Entry* small = reinterpret_cast<Entry*>(base + sl.small);
    float* partial = reinterpret_cast<float*>(base + sl.partial);
    uint32_t* tileCounts = reinterpret_cast<uint32_t*>(base + sl.counts);
    uint32_t* keyBuf[2] = {reinterpret_cast<uint32_t*>(base + sl.keys), reinterpret_cast<uint32_t*>(base + sl.keys) + items};
    uint32_t* orderBuf[2] = {order, reinterpret_cast<uint32_t*>(base + sl.order)};
    uint32_t* counters = reinterpret_cast<uint32_t*>(base + sl.counters);
    uint32_t* firsts = reinterpret_cast<uint32_t*>(base + sl.firsts);
    const float4* k4 = reinterpret_cast<const float4*>(keys);
    const float4* l4 = reinterpret_cast<const float4*>(low);
    const float4* h4 = reinterpret_cast<const float4*>(high);

    // Level 0: each shape's root over its items, in item order.
    std::vector<Entry> roots(shapes);
    std::vector<uint32_t> first(shapes);
    uint32_t item = 0, node = 0;
    for (uint32_t sh = 0; sh < shapes; ++sh) {
        roots[sh] = Entry{node, item, counts[sh], 0};
        first[sh] = item;
        item += counts[sh];
        node += treeNodes(counts[sh], leaf);
    }
    cudaError_t err = cudaMemcpyAsync(lists[0], roots.data(), shapes * sizeof(Entry), cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(firsts, first.data(), shapes * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess) err = cudaMemsetAsync(counters, 0, MAX_LEVELS * 4 * sizeof(uint32_t), s);
    k_treeIota<<<uint32_t(std::min<uint64_t>((items + 255) / 256, 4096)), 256, 0, s>>>(order, uint32_t(items));
    if (err != cudaSuccess) {
        set_last_error(std::string("median trees: ") + cudaGetErrorString(err));
        return 2;
    }
    for (uint32_t d = 0; d < levels.size(); ++d) {
        const LevelPlan& L = levels[d];
        Entry* cur = lists[d & 1];
        Entry* next = lists[(d + 1) & 1];
        const uint32_t parts = (L.maxCount + PIECE - 1) / PIECE;
        const uint64_t warps = L.entries * parts;
        k_treeReduce<<<uint32_t((warps + 7) / 8), 256, 0, s>>>(cur, uint32_t(L.entries), parts, k4, l4, h4, order,
                                                               partial);
        k_treeNodes<<<uint32_t((L.entries + 255) / 256), 256, 0, s>>>(
            cur, uint32_t(L.entries), parts, partial, leaf, d, reinterpret_cast<uint4*>(records),
            reinterpret_cast<float4*>(nodeLow), reinterpret_cast<float4*>(nodeHigh), next, large, small,
            counters + 4 * d);
        if (L.small)
            k_treeSmallSort<<<uint32_t((L.small + 7) / 8), 256, 0, s>>>(small, uint32_t(L.small), k4, order);
        if (L.large) {
            const uint32_t tiles = (L.maxLarge + TILE - 1) / TILE;
            const uint32_t blocks = uint32_t(L.large * tiles);
            for (uint32_t pass = 0; pass < 4; ++pass) {
                const uint32_t src = pass & 1, dst = src ^ 1;
                k_treeCount<<<blocks, 256, 0, s>>>(large, tiles, pass, k4, order, keyBuf[0], keyBuf[src],
                                                   tileCounts);
                k_treeOffsets<<<uint32_t(L.large), 256, 0, s>>>(large, tiles, tileCounts);
                k_treeScatter<<<blocks, 256, 0, s>>>(large, tiles, pass, tileCounts, keyBuf[src], orderBuf[src],
                                                     keyBuf[dst], orderBuf[dst]);
            }
        }
    }
    k_treeLocal<<<uint32_t(std::min<uint64_t>((items + 255) / 256, 4096)), 256, 0, s>>>(order, uint32_t(items), firsts,
                                                                                      shapes);
    err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) {
        set_last_error(std::string("median trees: ") + cudaGetErrorString(err));
        return 2;
    }
    return 0;
}
