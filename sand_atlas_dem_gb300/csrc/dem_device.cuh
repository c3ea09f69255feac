// Device-side arithmetic and resource layout of the GB300 mesh-surface DEM step.
//
// Exactness contract: every FP32 expression that decides a pair, a contact
// key or a history slot is evaluated in the operation order of the reference
// CPU backend (the Slang-generated C++ of src/sand_atlas_dem/shaders/
// solver.slang): dot = ((0 + x0*y0) + x1*y1) + x2*y2, length = sqrt(dot),
// min/max as the ternaries a<b?a:b and a>b?a:b, float literals, no FMA
// contraction (this translation unit is built with --fmad=false and IEEE
// division/square root).  The minimum-image branch is FP64 as in
// shaders/cpu_scheduling.slang:10-15, evaluated once per directed pair.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sdg {

constexpr uint32_t EMPTY = 0xffffffffu;
// A stored walk slot whose node was found farther outside its target than
// any motion the stored filter results allow before their next build.
constexpr uint32_t DORMANT = 0xfffffffeu;
constexpr int RESOURCE_COUNT = 77;

// Solver flags (src/sand_atlas_dem/gpu.py:11-26) plus one for bounded waits.
enum Flag : uint32_t {
    F_DEGENERATE = 2, F_PENETRATION = 4, F_BIN = 8, F_PAIR = 16, F_CONTACT = 32, F_HASH = 64,
    F_CYCLE = 128, F_IMAGE = 256, F_NONFINITE = 512, F_STACK = 1024, F_ESCAPE = 2048,
    F_BOX = 4096, F_TIMESTEP = 8192, F_COINCIDENT = 16384, F_WAIT = 65536
};

struct Config {
    uint32_t activeTimestep, N, shapes, pairCapacity, contactCapacity, binCapacity, binCount;
    uint32_t bins[3];
    uint32_t hashSize;
    float dt, kn, kt, mu, normalViscosity, skin, drag, maxOverlap;
    uint32_t historyStep, meshGeometry, periodic, wallCount, wallBoxEnabled, sourceSurfaceNormal;
    // Backend extension values.
    uint32_t leafWords;          // 32-bit words per directed pair in the leaf mask
    uint32_t candidateCapacity;  // (directed pair, leaf cluster) work items
    uint32_t viscousCapture;     // fuse captureContactKinematics into beginStep
    uint32_t specimens;          // independent periodic specimens batched in one launch
    uint32_t cullerEnabled;      // learned culler in front of the exact node query
    // Launch shapes chosen by the autotuner (0 = built-in default).  They
    // change how work is spread over the SMs, never which work or its order
    // of accumulation, so every choice gives bit-identical results.
    uint32_t queryBlocksPerSM;   // node query CTAs per SM
    uint32_t queryWarps;         // node query warps per CTA (4 or 8)
    uint32_t cullBlocksPerSM;    // pair set-up, leaf cull and leaf emit CTAs per SM
    uint32_t contactBlocksPerSM; // node emit, contact starts and contact law CTAs per SM
    uint32_t gatherWarps;        // gather warps (grains in flight) per SM
    uint32_t walkBlocksPerSM;    // exact-query CTAs (256 threads, one node each) per SM
    uint32_t survivorCapacity;   // nodes that pass the conservative filters, per step
    uint32_t distanceGridEnabled;  // skip nodes the distance-bound grid certifies outside
    // Reach of the cached filter results, in the target shape's unscaled
    // frame: the leaf cull and node filter run with their tests grown by this
    // distance and their survivors are reused while no node has moved that far
    // relative to its partner (0 = run the filters every step).
    float filterMargin;
    // Sizes (16-byte units, from the caller's buffer sizes; 0 = unknown) of
    // the library arrays the exact queries read: meshChildren, meshTriangles,
    // meshNormals, sample.  The step prefetches them into L2.
    uint32_t library16[4];
};

// Buffers: the reference Resources block (solver.slang:20-100) in declaration
// order, then this backend's extension buffers.
struct Res {
    uint32_t* control; float4* cell; float4* position; float4* positionRemainder;
    float4* velocityRemainder; float4* momentumRemainder; float4* rotationRemainder;
    float4* referencePositionRemainder; float4* cellLog; float4* accumulatedRemainder;
    float4* velocity; float4* rotation; float4* momentum; float4* force; float4* torque;
    float4* referencePosition; float4* referenceCell; const uint32_t* shapeId; const float4* body;
    const float4* invI; const uint4* grids; const uint4* sampleInfo; const float4* gridOrigin;
    const float* distance; const float4* sample; const uint4* meshRoots; const uint4* meshHullInfo;
    const float4* meshPlanes; const float4* meshMin; const float4* meshMax; const uint4* meshLinks;
    const float4* meshTriangles; const float4* meshNormals; const uint4* meshFrontier;
    uint32_t* meshPairMask; float4* meshPairTransform; const uint4* meshClusterInfo;
    const uint4* meshClusterRanges; const float4* meshClusterMin; const float4* meshClusterMax;
    const uint32_t* meshSampleIndices; uint32_t* binCounts; uint32_t* binParticles;
    uint32_t* pairCounts; uint32_t* pairOffsets; uint2* pairs; uint32_t* contactCounts;
    uint32_t* contactOffsets; uint4* meta; float4* pointDepth; float4* normalArea; float4* slip;
    float4* contactForce; float* normalLossPower; float4* normalDamping; float4* forceVelocity;
    float4* forceOmega; const uint4* oldMeta; const float4* oldSlip; const float4* oldNormal;
    const uint32_t* oldHash; uint32_t* hash; uint32_t* heads; uint32_t* next;
    float4* particleStress; float4* timestepRows; float4* particleDiagnostic;
    float4* diagnosticRows; float4* accumulated; float4* fabricRows; float4* wallPlane;
    float4* wallRemainder; float4* wallVelocity; float4* wallMaterial; uint32_t* wallBoxIds;
    float4* wallRows; float4* wallAccumulated;
    // ---- extension (index 77 onward)
    const uint4* meshLeafInfo;        // per shape: first leaf slot, leaf count
    const uint32_t* meshLeaves;       // leaf cluster ids, preorder
    const uint32_t* meshSampleRank;   // per packed sample: position in meshSampleIndices
    uint32_t* byJCounts;              // N+1
    uint32_t* byJOffsets;             // N+1
    uint32_t* byJCursor;              // N
    uint32_t* byJPairs;               // pairCapacity: pair ids grouped by second grain
    float4* dpairBranch;              // 2*pairCapacity: FP64-exact branch per directed pair
    uint32_t* dpairLeafCount;         // 2*pairCapacity+1
    uint32_t* dpairCandOffset;        // 2*pairCapacity+1
    uint32_t* leafMask;               // 2*pairCapacity*leafWords
    uint2* candidates;                // candidateCapacity: (directed pair, leaf cluster)
    uint32_t* candHitCount;           // candidateCapacity+1
    uint32_t* candHitOffset;          // candidateCapacity+1
    uint2* candHitMask;               // candidateCapacity: 64-bit node hit mask
    uint32_t* contactPair;            // contactCapacity: pair of each contact
    uint32_t* sidePairOffsets;        // N+1   (history side being written)
    uint32_t* sidePairB;              // pairCapacity
    uint32_t* sideContactStart;       // pairCapacity+1
    const uint32_t* oldPairOffsets;   // N+1   (committed history side)
    const uint32_t* oldPairB;         // pairCapacity
    const uint32_t* oldContactStart;  // pairCapacity+1
    uint32_t* work;                   // 64 counters
    uint32_t* scanPartials;           // 2*SCAN_BLOCKS
    float4* hitScratch;               // 2*survivorCapacity: (point/depth, normal/area) per survivor
    uint32_t* candSurvCount;          // candidateCapacity+1: nodes of each item left for the exact query
    float4* dpairPlane;               // 2*pairCapacity: enclosure plane of the target facing the source
    const uint32_t* grainSpecimen;    // N: specimen of each grain
    const uint4* specimenBins;        // specimens: bin grid x, y, z and first bin
    const float* cullerParams;        // shapes x CULLER_PARAMS: FP32 network parameters
    const uint32_t* cullerW1;         // shapes x 64 x 64 BF16 hidden weights (packed in pairs)
    const float* cullerMargin;        // shapes x (1 + 8^3): skip a node when the prediction exceeds its cell's
    uint32_t* cullerStats;            // 2 counters: nodes evaluated, nodes culled
    uint2* candSurvMask;              // candidateCapacity: 64-bit mask of the item's surviving nodes
    uint32_t* candSurvOffset;         // candidateCapacity+1: first survivor of each item
    uint2* survivors;                 // survivorCapacity: (item, node slot) of each surviving node
    uint32_t* survKeep;               // survivorCapacity+1: 1 = the learned culler keeps the survivor
    uint32_t* keepOffset;             // survivorCapacity+1: exclusive scan of survKeep
    uint32_t* walkList;               // survivorCapacity: survivors left for the exact query
    float4* dpairSourcePlane;         // 4*pairCapacity: the enclosure plane in the source frame, and its bound terms
    const float4* meshChildren;       // 4 per BVH node: both children's bounds (internal) or the triangle range
    float* distanceGrid;              // shapes x GRID^3: certified lower bound of the signed distance per cell
    float4* distanceGridInfo;         // shapes: grid origin xyz, cell size
    uint32_t* distanceGridTriangle;   // shapes x GRID^3: triangle nearest to each cell centre
    float4* filterRefRotation;        // N: orientation when the filter results were built
    float4* filterRefBranch;          // pairCapacity: first-to-second branch when they were built
    uint2* filterRefPairs;            // pairCapacity: the pair list they were built on
    uint32_t* walkKey;                // survivorCapacity: bucket of each kept survivor (target shape, coarse cell)
    uint32_t* walkBucketCount;        // shapes x WALK_BUCKETS + 1: kept survivors per bucket
    uint32_t* walkBucketOffset;       // shapes x WALK_BUCKETS + 1: first walk-list slot of each bucket
    uint32_t* sdfLaneCounts;          // SDF geometry, 32 x pairCapacity: contacts of virtual lanes l and l + 32
    float4* walkCertPoint;            // survivorCapacity: per stored walk slot, where its certificate was taken, and the gap
    uint2* walkCertTriangle;          // survivorCapacity: x its certified nearest triangle (EMPTY: none; DORMANT:
                                      // cannot touch before the next build), y a triangle of another leaf tying it
                                      // with the same result (EMPTY: none)
    uint32_t* wallCounts;             // wallCount x N: plane contacts of each (wall, grain), wall-major
    uint32_t* wallOffsets;            // wallCount x N + 1: their exclusive scan
    uint32_t* sideWallStart;          // wallCount x N + 1: first contact of each (wall, grain), side being written
    const uint32_t* oldWallStart;     // wallCount x N + 1: the same on the committed side
    uint4* walkNode;                  // survivorCapacity: per stored walk slot (source, target, directed pair, packed sample)
    uint2* walkItem;                  // survivorCapacity: per stored walk slot (item, node slot)
};
constexpr int EXTENSION_COUNT = 59;
constexpr uint32_t WALK_CELLS = 24;  // coarse cells per axis of a shape's grid box for the walk order
constexpr uint32_t WALK_BUCKETS = WALK_CELLS * WALK_CELLS * WALK_CELLS;
constexpr uint32_t GRID = 48;  // cells per axis of each shape's distance-bound grid
constexpr int CULLER_PARAMS = 3 * 64 + 64 + 64 * 64 + 64 + 64 + 4;
constexpr int BUFFER_COUNT = RESOURCE_COUNT + EXTENSION_COUNT;
constexpr int CONFIG_VALUES = 25;
constexpr int VALUE_COUNT = CONFIG_VALUES + 14;
constexpr int SCAN_BLOCKS = 608;  // 4 per SM on a 152-SM GB300
// work[] slots
constexpr int W_CANDIDATES = 0;
constexpr int W_SURVIVORS = 2;
constexpr int W_KEPT = 3;
constexpr int W_FILTER = 5;         // 1 = build the filter results this step, 0 = reuse them
constexpr int W_FILTER_VALID = 6;   // 1 = the stored filter results are complete
constexpr int W_FILTER_PAIRS = 7;   // pair count they were built on
constexpr int W_FILTER_MARGIN = 8;  // margin they were built with (float bits)
constexpr int W_FILTER_BUILDS = 9;  // steps that built them (counter)
constexpr int W_FILTER_STEPS = 10;  // steps that ran the collector (counter)
constexpr int W_FILTER_AGE = 11;    // collector runs since they were built
constexpr int W_FILTER_NEXT = 12;   // margin a build of this step uses (float bits)
constexpr int W_FILTER_BASE = 13;   // configured margin they were built under (float bits)
constexpr int W_SLOW = 14;          // stored walk slots left for a full walk this step
constexpr int W_CERTIFIED = 15;     // exact queries answered by a certificate (counter)
constexpr int W_WALL_BASE = 16;     // first plane contact: the grain-grain contact total
constexpr int W_REBUILDS = 17;      // steps that rebuilt the neighbour list (counter)
constexpr int W_DORMANT = 18;       // dormant slots in the stored exact-query list
constexpr int W_CULL_ROWS = 19;     // kept survivors in the culler's shape-sorted list

struct Params {
    Config c;
    Res r;
};

// ------------------------------------------------------------------ vectors
struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 xyz(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ float4 w4(f3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 operator/(f3 a, f3 b) { return {__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y), __fdiv_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z)}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float4 add4(float4 a, float4 b) {
    return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ float4 sub4(float4 a, float4 b) {
    return make_float4(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __fsub_rn(a.w, b.w));
}
__device__ __forceinline__ float4 scale4(float4 a, float s) {
    return make_float4(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s));
}
__device__ __forceinline__ float mn(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float mx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ f3 mn3(f3 a, f3 b) { return {mn(a.x, b.x), mn(a.y, b.y), mn(a.z, b.z)}; }
__device__ __forceinline__ f3 mx3(f3 a, f3 b) { return {mx(a.x, b.x), mx(a.y, b.y), mx(a.z, b.z)}; }
__device__ __forceinline__ f3 abs3(f3 a) { return {fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
__device__ __forceinline__ float dot(f3 a, f3 b) {
    float r = __fadd_rn(0.0f, __fmul_rn(a.x, b.x));
    r = __fadd_rn(r, __fmul_rn(a.y, b.y));
    return __fadd_rn(r, __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float dot4(float4 a, float4 b) {
    float r = __fadd_rn(0.0f, __fmul_rn(a.x, b.x));
    r = __fadd_rn(r, __fmul_rn(a.y, b.y));
    r = __fadd_rn(r, __fmul_rn(a.z, b.z));
    return __fadd_rn(r, __fmul_rn(a.w, b.w));
}
__device__ __forceinline__ float length(f3 a) { return __fsqrt_rn(dot(a, a)); }
__device__ __forceinline__ f3 cross(f3 l, f3 r) {
    return {__fsub_rn(__fmul_rn(l.y, r.z), __fmul_rn(l.z, r.y)),
            __fsub_rn(__fmul_rn(l.z, r.x), __fmul_rn(l.x, r.z)),
            __fsub_rn(__fmul_rn(l.x, r.y), __fmul_rn(l.y, r.x))};
}
__device__ __forceinline__ float comp(f3 a, uint32_t i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ bool finite3(f3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }

// Quaternions xyzw, body to world (solver.slang:104-106).
__device__ __forceinline__ f3 qrot(float4 q, f3 v) {
    f3 u = xyz(q);
    return v + 2.0f * cross(u, cross(u, v) + q.w * v);
}
__device__ __forceinline__ f3 qinv(float4 q, f3 v) { return qrot(make_float4(-q.x, -q.y, -q.z, q.w), v); }
__device__ __forceinline__ float4 qmul(float4 a, float4 b) {
    f3 v = (a.w * xyz(b) + b.w * xyz(a)) + cross(xyz(a), xyz(b));
    return w4(v, __fsub_rn(__fmul_rn(a.w, b.w), dot(xyz(a), xyz(b))));
}
// normalize(x) = x * (1 / sqrt(dot(x, x))).
__device__ __forceinline__ float4 normalize4(float4 q) { return scale4(q, __fdiv_rn(1.0f, __fsqrt_rn(dot4(q, q)))); }

__device__ __forceinline__ void fail(const Res& r, uint32_t bit) { atomicOr(r.control, bit); }

// solver.slang:111-118
__device__ __forceinline__ void compensated3(f3& high, f3& low, f3 inc) {
    f3 y = inc + low;
    f3 nx = high + y;
    f3 moved = nx - high;
    low = y - moved;
    high = nx;
}
__device__ __forceinline__ void compensated4(float4& high, float4& low, float4 inc) {
    float4 y = add4(inc, low);
    float4 nx = add4(high, y);
    float4 moved = sub4(nx, high);
    low = sub4(y, moved);
    high = nx;
}
// solver.slang:119-123
__device__ __forceinline__ float expm1Stable(float x) {
    if (fabsf(x) < 0.01f) {
        float t = __fadd_rn(__fdiv_rn(1.0f, 24.0f), __fdiv_rn(x, 120.0f));
        t = __fadd_rn(__fdiv_rn(1.0f, 6.0f), __fmul_rn(x, t));
        t = __fadd_rn(0.5f, __fmul_rn(x, t));
        t = __fadd_rn(1.0f, __fmul_rn(x, t));
        return __fmul_rn(x, t);
    }
    return __fsub_rn(expf(x), 1.0f);
}
__device__ __forceinline__ f3 expm1Stable3(f3 x) { return {expm1Stable(x.x), expm1Stable(x.y), expm1Stable(x.z)}; }
__device__ __forceinline__ f3 exp3(f3 x) { return {expf(x.x), expf(x.y), expf(x.z)}; }
// solver.slang:124-129
__device__ __forceinline__ float4 rotationIncrement(f3 w, float dt, float4 q) {
    float half = __fmul_rn(__fmul_rn(0.5f, length(w)), dt);
    float coefficient = fabsf(half) < 0.001f
        ? __fmul_rn(__fmul_rn(0.5f, dt), __fsub_rn(1.0f, __fdiv_rn(__fmul_rn(half, half), 6.0f)))
        : __fdiv_rn(sinf(half), length(w));
    float s = sinf(__fmul_rn(0.5f, half));
    float cm1 = __fmul_rn(__fmul_rn(-2.0f, s), s);
    return qmul(w4(coefficient * w, cm1), q);
}

// Batched specimens: grain i belongs to specimen s = grainSpecimen[i]; the
// specimen's cell rows (lengths, imposed log rates, initial lengths; the
// reference cell buffer, gpu.py:223-226) start at cell[3s], its cellLog and
// referenceCell rows at [2s].  A single specimen is s = 0 throughout.
__device__ __forceinline__ uint32_t specimenOf(const Res& r, uint32_t i) { return r.grainSpecimen[i]; }

// The periodic image shift floor(d / box + 0.5) of a raw separation d.
// Where |d| <= 0.45 box it is 0 and where 0.55 box <= |d| <= 1.45 box it is
// +-1: d / box + 0.5 lies in [0.05, 0.95] or [1.05, 1.95] (mirrored for
// d < 0), whatever the rounding of the FP64 division.  An FP32 comparison
// (relative error 1e-7) cannot move |d| across those margins, so it picks the
// very value the FP64 expression takes; only near |d| = box / 2 (and beyond
// 1.45 box) is the FP64 expression evaluated.  That spares nearly every
// pair the FP64 division, a few dozen instructions on GB300's narrow FP64
// pipe.
__device__ __forceinline__ double imageShift(double d, double box) {
    float ad = fabsf(__double2float_rn(d)), fb = __double2float_rn(box);
    if (ad <= __fmul_rn(0.45f, fb)) return 0.0;
    if (ad >= __fmul_rn(0.55f, fb) && ad <= __fmul_rn(1.45f, fb)) return d > 0.0 ? 1.0 : -1.0;
    return floor(__dadd_rn(__ddiv_rn(d, box), 0.5));
}
// Minimum-image branch j - i in FP64, cast to FP32 (cpu_scheduling.slang:10-15).
__device__ __forceinline__ f3 centerBranch64(const Res& r, const Config& c, uint32_t i, uint32_t j) {
    float4 pi = r.position[i], pj = r.position[j], li = r.positionRemainder[i], lj = r.positionRemainder[j];
    float4 cell = r.cell[3 * specimenOf(r, i)];
    double dx = __dadd_rn(__dsub_rn((double)pj.x, (double)pi.x), __dsub_rn((double)lj.x, (double)li.x));
    double dy = __dadd_rn(__dsub_rn((double)pj.y, (double)pi.y), __dsub_rn((double)lj.y, (double)li.y));
    double dz = __dadd_rn(__dsub_rn((double)pj.z, (double)pi.z), __dsub_rn((double)lj.z, (double)li.z));
    if (c.periodic != 0) {
        double bx = cell.x, by = cell.y, bz = cell.z;
        dx = __dsub_rn(dx, __dmul_rn(imageShift(dx, bx), bx));
        dy = __dsub_rn(dy, __dmul_rn(imageShift(dy, by), by));
        dz = __dsub_rn(dz, __dmul_rn(imageShift(dz, bz), bz));
    }
    return {__double2float_rn(dx), __double2float_rn(dy), __double2float_rn(dz)};
}
// solver.slang:154-158
__device__ __forceinline__ f3 omega(const Res& r, uint32_t i, float4 q, f3 l) {
    f3 b = qinv(q, l);
    f3 w = {dot(xyz(r.invI[3 * i]), b), dot(xyz(r.invI[3 * i + 1]), b), dot(xyz(r.invI[3 * i + 2]), b)};
    return qrot(q, w);
}
__device__ __forceinline__ f3 omegaOf(const Res& r, uint32_t i) {
    return omega(r, i, r.rotation[i], xyz(r.momentum[i]) + xyz(r.momentumRemainder[i]));
}

// ------------------------------------------------------------ mesh queries
// solver.slang:203-219
__device__ __forceinline__ f3 closestTriangle(f3 p, f3 a, f3 b, f3 c, uint32_t& feature) {
    f3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    feature = 4;
    if (d1 <= 0 && d2 <= 0) return a;
    f3 bp = p - b;
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { feature = 5; return b; }
    float vc = __fsub_rn(__fmul_rn(d1, d4), __fmul_rn(d3, d2));
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { feature = 1; return a + __fdiv_rn(d1, __fsub_rn(d1, d3)) * ab; }
    f3 cp = p - c;
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) { feature = 6; return c; }
    float vb = __fsub_rn(__fmul_rn(d5, d2), __fmul_rn(d1, d6));
    if (vb <= 0 && d2 >= 0 && d6 <= 0) { feature = 3; return a + __fdiv_rn(d2, __fsub_rn(d2, d6)) * ac; }
    float va = __fsub_rn(__fmul_rn(d3, d6), __fmul_rn(d5, d4));
    float e43 = __fsub_rn(d4, d3), e56 = __fsub_rn(d5, d6);
    if (va <= 0 && e43 >= 0 && e56 >= 0) { feature = 2; return b + __fdiv_rn(e43, __fadd_rn(e43, e56)) * (c - b); }
    float inv = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(va, vb), vc));
    feature = 0;
    return (a + ab * __fmul_rn(vb, inv)) + ac * __fmul_rn(vc, inv);
}
// solver.slang:220-223
__device__ __forceinline__ float boxDistance(f3 low, f3 high, f3 p) {
    f3 d = mx3(mx3(low - p, p - high), mk(0.f, 0.f, 0.f));
    return dot(d, d);
}
__device__ __forceinline__ float meshBoxDistance(const Res& r, uint32_t node, f3 p) {
    return boxDistance(xyz(__ldg(&r.meshMin[node])), xyz(__ldg(&r.meshMax[node])), p);
}
constexpr uint32_t LEAF_MARK = 0xFFFFFFFFu;
// Signed distance and direction from the recorded nearest point (the end of
// solver.slang:224-252).
__device__ __forceinline__ float4 distanceResult(const Res& r, f3 p, float best, f3 nearest, uint32_t nearestNormal,
                                                 bool found, bool surfaceNormal) {
    f3 pseudo = found ? xyz(__ldg(&r.meshNormals[nearestNormal])) : mk(0.f, 0.f, 0.f);
    float distance = __fsqrt_rn(best);
    f3 off = p - nearest;
    float side = dot(off, pseudo) < 0 ? -1.0f : 1.0f;
    f3 normal = surfaceNormal ? pseudo : (distance > 1e-12f ? (side * off) / distance : pseudo);
    return w4(normal, __fmul_rn(side, distance));
}
// Nearest-first BVH walk with cached pushed box distances (the reference CPU
// variant, cpu_scheduling.slang:18-48, bit-identical to solver.slang:224-252).
// With `seed` (a triangle of the shape) the walk starts with its best just
// above that triangle's squared distance d, computed exactly as the walk
// computes it: d (1 + 2^-20), one float up.  That prunes only nodes whose
// box lies farther than every triangle the walk could still record, and
// changes nothing else: the surviving nodes are visited in the same order
// and the first nearest triangle reached is recorded as before.  The 2^-20
// keeps the nearest triangle's boxes in the walk even where FP32 rounding
// puts a box distance a few units in the last place above the triangle's
// own distance (an unseeded walk has no tighter bound than d there).
// `nearestTriangle`, when given, receives the recorded triangle.
__device__ __forceinline__ float4 meshDistance(const Res& r, uint32_t shape, f3 p, bool surfaceNormal,
                                               uint32_t seed = 0xFFFFFFFFu, uint32_t* nearestTriangle = nullptr) {
    uint32_t root = __ldg(&r.meshRoots[shape].x);
    uint32_t pending[32];
    float pendingDistance[32];
    uint32_t top = 1;
    pending[0] = root;
    pendingDistance[0] = meshBoxDistance(r, root, p);
    float best = 1e30f;
    if (seed != 0xFFFFFFFFu) {
        uint32_t feature;
        f3 q = closestTriangle(p, xyz(__ldg(&r.meshTriangles[3 * seed])), xyz(__ldg(&r.meshTriangles[3 * seed + 1])),
                               xyz(__ldg(&r.meshTriangles[3 * seed + 2])), feature);
        f3 dq = p - q;
        float d = dot(dq, dq);
        best = nextafterf(__fadd_rn(d, __fmul_rn(d, 9.5367431640625e-07f)), 1e30f);
    }
    f3 nearest = mk(0.f, 0.f, 0.f);
    uint32_t nearestNormal = 0;
    bool found = false;
    // Each node's record holds both children's bounds (the same floats as
    // meshMin/meshMax) and the escape link of the first child, so a step of
    // the walk is one round of independent loads instead of three dependent
    // ones; the visit order and every distance are unchanged.
    while (top > 0) {
        uint32_t slot = --top, node = pending[slot];
        if (pendingDistance[slot] > best) continue;
        const float4* record = r.meshChildren + 4 * size_t(node);
        float4 r0 = __ldg(record), r1 = __ldg(record + 1);
        if (__float_as_uint(r0.w) != LEAF_MARK) {
            float4 r2 = __ldg(record + 2), r3 = __ldg(record + 3);
            uint32_t a = node + 1, b = __float_as_uint(r0.w);
            float da = boxDistance(xyz(r0), xyz(r1), p), db = boxDistance(xyz(r2), xyz(r3), p);
            if (da < db) { uint32_t s = a; a = b; b = s; float ds = da; da = db; db = ds; }
            if (top + 2 > 32) { fail(r, F_STACK); return make_float4(0.f, 0.f, 0.f, 1e20f); }
            if (da <= best) { pending[top] = a; pendingDistance[top++] = da; }
            if (db <= best) { pending[top] = b; pendingDistance[top++] = db; }
            continue;
        }
        uint32_t first = __float_as_uint(r0.x), count = __float_as_uint(r0.y);
        for (uint32_t k = 0; k < count; ++k) {
            uint32_t triangle = first + k, feature;
            f3 q = closestTriangle(p, xyz(__ldg(&r.meshTriangles[3 * triangle])), xyz(__ldg(&r.meshTriangles[3 * triangle + 1])),
                                   xyz(__ldg(&r.meshTriangles[3 * triangle + 2])), feature);
            f3 dq = p - q;
            float distance = dot(dq, dq);
            if (distance < best) { best = distance; nearest = q; nearestNormal = 7 * triangle + feature; found = true; }
        }
    }
    if (nearestTriangle) *nearestTriangle = found ? nearestNormal / 7 : 0xFFFFFFFFu;
    return distanceResult(r, p, best, nearest, nearestNormal, found, surfaceNormal);
}
// The nearest triangle of the shape to p and the gap to every other one.
// The same nearest-first walk, keeping the two smallest squared distances and
// pruning by the second (times 1 + 2^-20, against FP32 box rounding), from
// the cap B = (sqrt(d_seed) + reach)^2: it records the triangle the walk
// records and returns, in `gap`, a lower bound of (distance to every other
// triangle) - (distance to it), or 0 when a triangle ties it.  Only gaps up
// to about `reach` are found.  `triangle` receives the recorded triangle; a
// triangle that ties it exactly in the same BVH leaf (two faces meeting at
// an edge) is not counted against the gap but returned as a partner, in the
// top two bits (its offset after it in the leaf): between the two, the walk
// records the partner only where it is strictly nearer.  A triangle of
// another leaf whose result ties it bit for bit -- the same squared
// distance, closest point and pseudonormal, as the two faces of an edge
// give when both compute the edge point from the same endpoints -- is not
// counted against the gap either but returned in `tie`: whichever of the two
// a walk records, its result is the same.
__device__ __forceinline__ bool sameResult(const Res& r, f3 q, uint32_t normal, f3 q2, uint32_t normal2) {
    float4 n = __ldg(&r.meshNormals[normal]), n2 = __ldg(&r.meshNormals[normal2]);
    return __float_as_uint(q.x) == __float_as_uint(q2.x) && __float_as_uint(q.y) == __float_as_uint(q2.y) &&
           __float_as_uint(q.z) == __float_as_uint(q2.z) && __float_as_uint(n.x) == __float_as_uint(n2.x) &&
           __float_as_uint(n.y) == __float_as_uint(n2.y) && __float_as_uint(n.z) == __float_as_uint(n2.z);
}
// `Warp`: the whole warp runs one walk (p, shape, seed and reach the same on
// every lane).  Every lane then holds the same stack and takes the same
// decisions; the lanes evaluate a leaf's triangles together and its results
// are taken in triangle order, so the walk and its result are the
// one-thread walk's.  A few walks fill a warp each, instead of one lane of a
// diverging warp each.
// `children`/`nodeBase`: where the walk reads node n's record --
// children + 4 (n - nodeBase): the library's meshChildren (base 0) or the
// shape's records staged in shared memory (base: its first node); and
// `triangles`/`triangleBase` likewise for triangle t's three vertices,
// triangles + 3 (t - triangleBase).
template <bool Warp>
__device__ __forceinline__ float4 meshDistanceCertifiedT(const Res& r, uint32_t shape, f3 p, uint32_t seed,
                                                         float reach, uint32_t& triangle, uint32_t& tie, float& gap,
                                                         const float4* children, uint32_t nodeBase,
                                                         const float4* triangles, uint32_t triangleBase) {
    uint32_t root = __ldg(&r.meshRoots[shape].x);
    auto vertex = [&](uint32_t t, uint32_t k) { return xyz(triangles[3 * (t - triangleBase) + k]); };
    uint32_t pending[32];
    float pendingDistance[32];
    uint32_t top = 1;
    pending[0] = root;
    pendingDistance[0] = meshBoxDistance(r, root, p);
    float cap = 1e30f;
    if (seed != 0xFFFFFFFFu) {
        uint32_t feature;
        f3 q = closestTriangle(p, vertex(seed, 0), vertex(seed, 1), vertex(seed, 2), feature);
        f3 dq = p - q;
        float root2 = __fadd_rn(__fsqrt_rn(dot(dq, dq)), reach);
        cap = nextafterf(__fmul_rn(__fmul_rn(root2, root2), 1.0000019073486328f), 1e30f);
    }
    float best = cap, second = cap;
    f3 nearest = mk(0.f, 0.f, 0.f);
    uint32_t nearestNormal = 0, bestNode = 0xFFFFFFFFu, partner = 0, tied = EMPTY;
    bool found = false;
    // One leaf triangle's result, in the walk's order.
    auto take = [&](uint32_t node, uint32_t t, f3 q, uint32_t feature, float distance) {
        if (distance < best) {
            second = best;
            best = distance; nearest = q; nearestNormal = 7 * t + feature; found = true;
            bestNode = node;
            partner = 0;
            tied = EMPTY;
        } else if (distance == best && found && node == bestNode && partner == 0) {
            partner = t - nearestNormal / 7;  // 1..3: later in the same leaf
        } else if (distance == best && found && node != bestNode && tied == EMPTY &&
                   sameResult(r, q, 7 * t + feature, nearest, nearestNormal)) {
            tied = t;
        } else if (distance < second) {
            second = distance;
        }
    };
    while (top > 0) {
        uint32_t slot = --top, node = pending[slot];
        float limit = __fmul_rn(second, 1.00000095367431640625f);
        if (pendingDistance[slot] > limit) continue;
        const float4* record = children + 4 * size_t(node - nodeBase);
        float4 r0 = record[0], r1 = record[1];
        if (__float_as_uint(r0.w) != LEAF_MARK) {
            float4 r2 = record[2], r3 = record[3];
            uint32_t a = node + 1, b = __float_as_uint(r0.w);
            float da = boxDistance(xyz(r0), xyz(r1), p), db = boxDistance(xyz(r2), xyz(r3), p);
            if (da < db) { uint32_t s = a; a = b; b = s; float ds = da; da = db; db = ds; }
            if (top + 2 > 32) {
                fail(r, F_STACK);
                triangle = tie = EMPTY;
                gap = 0.f;
                return make_float4(0.f, 0.f, 0.f, 1e20f);
            }
            if (da <= limit) { pending[top] = a; pendingDistance[top++] = da; }
            if (db <= limit) { pending[top] = b; pendingDistance[top++] = db; }
            continue;
        }
        uint32_t first = __float_as_uint(r0.x), count = __float_as_uint(r0.y);
        if constexpr (Warp) {
            const uint32_t lane = threadIdx.x & 31u;
            for (uint32_t k0 = 0; k0 < count; k0 += 32) {
                uint32_t t = first + k0 + lane, feature = 0;
                f3 q = mk(0.f, 0.f, 0.f);
                float distance = 0.f;
                if (k0 + lane < count) {
                    q = closestTriangle(p, vertex(t, 0), vertex(t, 1), vertex(t, 2), feature);
                    f3 dq = p - q;
                    distance = dot(dq, dq);
                }
                uint32_t m = min(32u, count - k0);
                for (uint32_t j = 0; j < m; ++j) {
                    f3 qj = mk(__shfl_sync(0xffffffffu, q.x, j), __shfl_sync(0xffffffffu, q.y, j),
                               __shfl_sync(0xffffffffu, q.z, j));
                    take(node, first + k0 + j, qj, __shfl_sync(0xffffffffu, feature, j),
                         __shfl_sync(0xffffffffu, distance, j));
                }
            }
        } else {
            for (uint32_t k = 0; k < count; ++k) {
                uint32_t t = first + k, feature;
                f3 q = closestTriangle(p, vertex(t, 0), vertex(t, 1), vertex(t, 2), feature);
                f3 dq = p - q;
                take(node, t, q, feature, dot(dq, dq));
            }
        }
    }
    triangle = found ? (nearestNormal / 7) | (partner << 30) : 0xFFFFFFFFu;
    tie = found ? tied : EMPTY;
    gap = found ? __fsub_rn(__fsqrt_rn(second), __fsqrt_rn(best)) : 0.f;
    return distanceResult(r, p, best, nearest, nearestNormal, found, false);
}
__device__ __forceinline__ float4 meshDistanceCertified(const Res& r, uint32_t shape, f3 p, uint32_t seed, float reach,
                                                        uint32_t& triangle, uint32_t& tie, float& gap) {
    return meshDistanceCertifiedT<false>(r, shape, p, seed, reach, triangle, tie, gap, r.meshChildren, 0u,
                                         r.meshTriangles, 0u);
}
// The walk's result when the certified triangle (and its same-leaf partner,
// encoded as by meshDistanceCertified, and its tie of another leaf) are
// known to be nearer than every other: the same closest point, squared
// distance and feature the walk records -- the partner's only where it is
// strictly nearer, as the leaf's triangles are taken in order.  With a tie
// (EMPTY: none) the result stands only where the tie gives the same result
// bit for bit (the walk may reach either leaf first); `same` is cleared
// otherwise, and the caller walks.
// `a`, `b`, `c` are the certified triangle's vertices (loaded by the caller).
__device__ __forceinline__ float4 meshDistanceAt(const Res& r, f3 p, uint32_t certified, uint32_t tie, float4 a,
                                                 float4 b, float4 c, bool& same) {
    uint32_t triangle = certified & 0x3FFFFFFFu, partner = certified >> 30, feature;
    f3 q = closestTriangle(p, xyz(a), xyz(b), xyz(c), feature);
    f3 dq = p - q;
    float best = dot(dq, dq);
    uint32_t normal = 7 * triangle + feature;
    if (partner != 0) {
        uint32_t other = triangle + partner, otherFeature;
        f3 q2 = closestTriangle(p, xyz(__ldg(&r.meshTriangles[3 * other])), xyz(__ldg(&r.meshTriangles[3 * other + 1])),
                                xyz(__ldg(&r.meshTriangles[3 * other + 2])), otherFeature);
        f3 dq2 = p - q2;
        float d2 = dot(dq2, dq2);
        if (d2 < best) { best = d2; q = q2; normal = 7 * other + otherFeature; }
    }
    same = true;
    if (tie != EMPTY) {
        uint32_t tieFeature;
        f3 q3 = closestTriangle(p, xyz(__ldg(&r.meshTriangles[3 * tie])), xyz(__ldg(&r.meshTriangles[3 * tie + 1])),
                                xyz(__ldg(&r.meshTriangles[3 * tie + 2])), tieFeature);
        f3 dq3 = p - q3;
        same = __float_as_uint(dot(dq3, dq3)) == __float_as_uint(best) && sameResult(r, q3, 7 * tie + tieFeature, q, normal);
    }
    return distanceResult(r, p, best, q, normal, true, false);
}
// solver.slang:259-272.  With `grow` > 0 the root box and every hull plane
// are moved out by that distance (unit normals): the test then admits every
// point within `grow` of one it admits unmoved.
__device__ __forceinline__ bool meshMayContain(const Res& r, uint32_t shape, f3 p, float grow = 0.0f) {
    uint32_t root = __ldg(&r.meshRoots[shape].x);
    f3 low = xyz(__ldg(&r.meshMin[root])), high = xyz(__ldg(&r.meshMax[root]));
    if (grow > 0.0f) {
        if (__fadd_rn(p.x, grow) < low.x || __fadd_rn(p.y, grow) < low.y || __fadd_rn(p.z, grow) < low.z ||
            __fsub_rn(p.x, grow) > high.x || __fsub_rn(p.y, grow) > high.y || __fsub_rn(p.z, grow) > high.z)
            return false;
    } else if (p.x < low.x || p.y < low.y || p.z < low.z || p.x > high.x || p.y > high.y || p.z > high.z) {
        return false;
    }
    f3 direction = (p - 0.5f * (low + high)) / (high - low);
    f3 a = abs3(direction);
    uint32_t axis = a.x >= a.y && a.x >= a.z ? 0 : (a.y >= a.z ? 1 : 2);
    uint32_t group = 2 * axis + (comp(direction, axis) >= 0 ? 1 : 0);
    uint4 info = __ldg(&r.meshHullInfo[6 * shape + group]);
    for (uint32_t i = 0; i < info.y; ++i) {
        float4 plane = __ldg(&r.meshPlanes[info.x + i]);
        if (__fadd_rn(dot(xyz(plane), p), plane.w) > grow) return false;
    }
    return true;
}
// solver.slang:274-288
__device__ __forceinline__ bool meshBoxMayContact(const Res& r, uint32_t shape, f3 low, f3 high) {
    uint32_t root = __ldg(&r.meshRoots[shape].x);
    f3 tl = xyz(__ldg(&r.meshMin[root])), th = xyz(__ldg(&r.meshMax[root]));
    if (high.x < tl.x || high.y < tl.y || high.z < tl.z || low.x > th.x || low.y > th.y || low.z > th.z) return false;
    f3 center = 0.5f * (low + high), half = 0.5f * (high - low);
    f3 direction = (center - 0.5f * (tl + th)) / (th - tl);
    f3 a = abs3(direction);
    uint32_t axis = a.x >= a.y && a.x >= a.z ? 0 : (a.y >= a.z ? 1 : 2);
    uint32_t group = 2 * axis + (comp(direction, axis) >= 0 ? 1 : 0);
    uint4 info = __ldg(&r.meshHullInfo[6 * shape + group]);
    for (uint32_t i = 0; i < info.y; ++i) {
        float4 plane = __ldg(&r.meshPlanes[info.x + i]);
        if (__fsub_rn(__fadd_rn(dot(xyz(plane), center), plane.w), dot(abs3(xyz(plane)), half)) > 0) return false;
    }
    return true;
}
// The first half of meshBoxMayContact: the target's root box test, and the
// centre, half extent and hull group its plane loop would use.
__device__ __forceinline__ bool meshBoxGroup(const Res& r, uint32_t shape, f3 low, f3 high, f3& center, f3& half,
                                             uint32_t& group) {
    uint32_t root = __ldg(&r.meshRoots[shape].x);
    f3 tl = xyz(__ldg(&r.meshMin[root])), th = xyz(__ldg(&r.meshMax[root]));
    if (high.x < tl.x || high.y < tl.y || high.z < tl.z || low.x > th.x || low.y > th.y || low.z > th.z) return false;
    center = 0.5f * (low + high);
    half = 0.5f * (high - low);
    f3 direction = (center - 0.5f * (tl + th)) / (th - tl);
    f3 a = abs3(direction);
    uint32_t axis = a.x >= a.y && a.x >= a.z ? 0 : (a.y >= a.z ? 1 : 2);
    group = 2 * axis + (comp(direction, axis) >= 0 ? 1 : 0);
    return true;
}
// solver.slang:290-305, with the directed-pair branch supplied.
// With `margin`, the box is grown by that distance (the test then holds for
// every placement within `margin` of this one).
__device__ __forceinline__ bool meshClusterMayContact(const Res& r, uint32_t src, uint32_t dst, uint32_t cluster, f3 branch,
                                                      float margin = 0.0f) {
    f3 sl = xyz(r.meshClusterMin[cluster]), sh = xyz(r.meshClusterMax[cluster]);
    f3 low = mk(1e30f, 1e30f, 1e30f), high = mk(-1e30f, -1e30f, -1e30f);
    float4 qs = r.rotation[src], qd = r.rotation[dst];
    float ss = r.body[src].x, sd = r.body[dst].x;
    for (uint32_t corner = 0; corner < 8; ++corner) {
        f3 p = mk((corner & 1) ? sh.x : sl.x, (corner & 2) ? sh.y : sl.y, (corner & 4) ? sh.z : sl.z);
        p = qinv(qd, qrot(qs, p * ss) - branch) / sd;
        low = mn3(low, p);
        high = mx3(high, p);
    }
    float pad = __fmul_rn(0.00000762939453125f,
        __fadd_rn(__fadd_rn(__fadd_rn(1.0f, mx(mx(fabsf(low.x), fabsf(low.y)), fabsf(low.z))),
                            mx(mx(fabsf(high.x), fabsf(high.y)), fabsf(high.z))), __fdiv_rn(length(branch), sd)));
    if (margin > 0.0f) pad = __fadd_rn(pad, margin);
    low = low - mk(pad, pad, pad);
    high = high + mk(pad, pad, pad);
    return meshBoxMayContact(r, r.shapeId[dst], low, high);
}
// solver.slang:404-417
// With `margin`, the bounds are grown by that distance.
__device__ __forceinline__ void meshPairBounds(const Res& r, uint32_t direction, uint32_t cluster, f3& low, f3& high,
                                               float margin = 0.0f) {
    f3 cmin = xyz(__ldg(&r.meshClusterMin[cluster])), cmax = xyz(__ldg(&r.meshClusterMax[cluster]));
    f3 center = 0.5f * (cmin + cmax);
    f3 half = 0.5f * (cmax - cmin);
    float cc[3], e[3];
#pragma unroll
    for (uint32_t axis = 0; axis < 3; ++axis) {
        float4 row = r.meshPairTransform[4 * direction + axis];
        cc[axis] = __fadd_rn(dot(xyz(row), center), row.w);
        e[axis] = dot(abs3(xyz(row)), half);
    }
    low = mk(cc[0], cc[1], cc[2]) - mk(e[0], e[1], e[2]);
    high = mk(cc[0], cc[1], cc[2]) + mk(e[0], e[1], e[2]);
    float pad = __fmul_rn(0.000030517578125f,
        __fadd_rn(__fadd_rn(__fadd_rn(1.0f, mx(mx(fabsf(low.x), fabsf(low.y)), fabsf(low.z))),
                            mx(mx(fabsf(high.x), fabsf(high.y)), fabsf(high.z))), r.meshPairTransform[4 * direction + 3].x));
    if (margin > 0.0f) pad = __fadd_rn(pad, margin);
    low = low - mk(pad, pad, pad);
    high = high + mk(pad, pad, pad);
}
// solver.slang:319-343; the directed-pair branch is precomputed (same bits).
// Split in two so that work can be filtered between the cheap conservative
// rejections and the exact query: nodePrefilter places the node in the
// target's frame and applies, with `plane`, the reference CPU backend's
// per-directed-pair enclosure-plane prefilter (cpu.py:56-76), then the hull
// cull; nodeExact is the exact distance query and the contact record.  Both
// rejections are conservative and change no contact.  `grow` > 0 widens both
// tests by that distance (for the stored filter results).
__device__ __forceinline__ bool nodeTests(const Res& r, uint32_t targetShape, const float4* plane, f3 local,
                                          float grow = 0.0f) {
    if (plane) {
        float pad = __fmul_rn(0.00000762939453125f,
                              __fadd_rn(1.0f, mx(mx(fabsf(local.x), fabsf(local.y)), fabsf(local.z))));
        if (grow > 0.0f) pad = __fadd_rn(pad, grow);
        if (__fadd_rn(dot(xyz(*plane), local), plane->w) > pad) return false;
    }
    return meshMayContain(r, targetShape, local, grow);
}
__device__ __forceinline__ bool nodePrefilter(const Res& r, uint32_t src, uint32_t dst, uint32_t node, f3 branch,
                                              const float4* plane, f3& arm, f3& local, float grow = 0.0f) {
    uint32_t sid = r.shapeId[src];
    float4 sp = __ldg(&r.sample[__ldg(&r.sampleInfo[sid].x) + node]);
    float4 qs = r.rotation[src], qd = r.rotation[dst];
    arm = qrot(qs, xyz(sp) * r.body[src].x);
    local = qinv(qd, arm - branch) / r.body[dst].x;
    return nodeTests(r, r.shapeId[dst], plane, local, grow);
}
// The contact record from the target's signed distance f at the node.
// The contact record of a node whose target-frame query gave f, from the
// node's sample `sp`, both grains' body rows and the target's rotation
// (loaded by the caller); `src` is read only for the source-surface normal.
__device__ __forceinline__ bool nodeContactWith(const Res& r, const Config& c, uint32_t src, float4 sp, float4 bs,
                                                float4 bd, float4 qd, f3 arm, float4 f, float4& pd, float4& na) {
    pd = w4(arm, __fmul_rn(-f.w, bd.x));
    if (pd.w <= 0.0f) return false;
    f3 grad = qrot(qd, xyz(f));
    float len = length(grad);
    if (c.sourceSurfaceNormal != 0) {
        float4 own = meshDistance(r, r.shapeId[src], xyz(sp), true);
        if (fabsf(own.w) > 0.00000999999974738f) { fail(r, F_DEGENERATE); return false; }
        grad = -qrot(r.rotation[src], xyz(own));
        len = length(grad);
    }
    if (len < 1.00000001168609742e-07f || !isfinite(pd.w)) { fail(r, F_DEGENERATE); return false; }
    na = w4(grad / len, __fmul_rn(__fmul_rn(sp.w, bs.x), bs.x));
    if (pd.w > __fmul_rn(c.maxOverlap, mn(bs.w, bd.w))) fail(r, F_PENETRATION);
    return true;
}
__device__ __forceinline__ bool nodeContactFrom(const Res& r, const Config& c, uint32_t src, uint32_t dst,
                                                uint32_t node, f3 arm, float4 f, float4& pd, float4& na) {
    uint32_t sid = r.shapeId[src];
    float4 sp = __ldg(&r.sample[__ldg(&r.sampleInfo[sid].x) + node]);
    return nodeContactWith(r, c, src, sp, r.body[src], r.body[dst], r.rotation[dst], arm, f, pd, na);
}
__device__ __forceinline__ bool nodeExact(const Res& r, const Config& c, uint32_t src, uint32_t dst, uint32_t node,
                                          f3 arm, f3 local, float4& pd, float4& na, uint32_t seed = 0xFFFFFFFFu) {
    float4 f = meshDistance(r, r.shapeId[dst], local, false, seed);
    return nodeContactFrom(r, c, src, dst, node, arm, f, pd, na);
}
__device__ __forceinline__ bool nodeContact(const Res& r, const Config& c, uint32_t src, uint32_t dst, uint32_t node,
                                            f3 branch, float4& pd, float4& na, const float4* plane = nullptr) {
    f3 arm, local;
    if (!nodePrefilter(r, src, dst, node, branch, plane, arm, local)) return false;
    return nodeExact(r, c, src, dst, node, arm, local, pd, na);
}

// Certified lower bound of the target shape's signed distance at `local`
// (shape frame, unscaled), from its cell of the distance-bound grid.  The
// signed distance to a closed mesh is 1-Lipschitz, so every point of a cell
// lies at least phi(centre) - (half diagonal) from the surface; the grid
// stores that bound less a slack above the FP32 error of the centre query.
// Points outside the grid (outside the shape's root box) get -inf.
// Index of the grid cell holding `local` in the shape's grid, or EMPTY
// outside it.
__device__ __forceinline__ uint32_t gridCell(const Res& r, uint32_t shape, f3 local) {
    float4 info = __ldg(&r.distanceGridInfo[shape]);
    float inv = __fdiv_rn(1.0f, info.w);
    float gx = floorf(__fmul_rn(__fsub_rn(local.x, info.x), inv));
    float gy = floorf(__fmul_rn(__fsub_rn(local.y, info.y), inv));
    float gz = floorf(__fmul_rn(__fsub_rn(local.z, info.z), inv));
    if (!(gx >= 0.f && gy >= 0.f && gz >= 0.f && gx < float(GRID) && gy < float(GRID) && gz < float(GRID)))
        return 0xFFFFFFFFu;
    return (uint32_t(gz) * GRID + uint32_t(gy)) * GRID + uint32_t(gx);
}
// Walk-order bucket of a node at `local` against `shape`: the shape, then
// the coarse cell (WALK_CELLS per axis over the grid box, clamped).  Nodes
// of one bucket take similar paths through the shape's BVH.
__device__ __forceinline__ uint32_t walkBucket(const Res& r, uint32_t shape, f3 local) {
    float4 info = __ldg(&r.distanceGridInfo[shape]);
    float inv = __fdiv_rn(float(WALK_CELLS), __fmul_rn(info.w, float(GRID)));
    float g[3] = {__fmul_rn(__fsub_rn(local.x, info.x), inv), __fmul_rn(__fsub_rn(local.y, info.y), inv),
                  __fmul_rn(__fsub_rn(local.z, info.z), inv)};
    uint32_t k[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        k[a] = g[a] >= float(WALK_CELLS - 1) ? WALK_CELLS - 1 : (g[a] >= 1.0f ? uint32_t(g[a]) : 0u);
    return shape * WALK_BUCKETS + (k[2] * WALK_CELLS + k[1]) * WALK_CELLS + k[0];
}
__device__ __forceinline__ float distanceBound(const Res& r, uint32_t shape, f3 local) {
    uint32_t cell = gridCell(r, shape, local);
    if (cell == 0xFFFFFFFFu) return -1e30f;
    return __ldg(&r.distanceGrid[size_t(shape) * GRID * GRID * GRID + cell]);
}
// The triangle nearest to the centre of the cell holding `local` (a seed
// for meshDistance), or EMPTY outside the grid.
__device__ __forceinline__ uint32_t gridSeed(const Res& r, uint32_t shape, f3 local) {
    uint32_t cell = gridCell(r, shape, local);
    if (cell == 0xFFFFFFFFu) return 0xFFFFFFFFu;
    return __ldg(&r.distanceGridTriangle[size_t(shape) * GRID * GRID * GRID + cell]);
}

// ---------------------------------------------------------------- helpers
// Whether the exact-query list itself is stored with the filter results
// (built with grown tests and ordered by target shape and coarse cell).  Not
// with the learned culler, whose calibrated decision is taken every step.
__host__ __device__ __forceinline__ bool storedKeep(const Config& c) { return c.filterMargin > 0.0f && c.cullerEnabled == 0; }
// Margin the filter results are built with on this step (0 without them).
__device__ __forceinline__ float buildMargin(const Res& r, const Config& c) {
    return c.filterMargin > 0.0f ? __uint_as_float(r.work[W_FILTER_NEXT]) : 0.0f;
}
__device__ __forceinline__ uint32_t activePairs(const Res& r, const Config& c) {
    uint32_t n = r.control[1];
    return n < c.pairCapacity ? n : c.pairCapacity;
}
__device__ __forceinline__ uint32_t activeContacts(const Res& r, const Config& c) {
    uint32_t n = r.control[2];
    return n < c.contactCapacity ? n : c.contactCapacity;
}
__device__ __forceinline__ uint32_t gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ uint32_t gstride() { return gridDim.x * blockDim.x; }

// ------------------------------------------------------------------ planes
// Error-free two-sums of the plane offsets (solver.slang:578-595; the
// materialisation mask is zero, so its rounding barriers are identities).
struct Sum2 { float hi, lo; };
__device__ __forceinline__ Sum2 wallTwoSum(float a, float b) {
    float high = __fadd_rn(a, b), v = __fsub_rn(high, a);
    return {high, __fadd_rn(__fsub_rn(a, __fsub_rn(high, v)), __fsub_rn(b, v))};
}
__device__ __forceinline__ Sum2 wallAdd(Sum2 a, float b) {
    Sum2 sum = wallTwoSum(a.hi, b);
    return wallTwoSum(sum.hi, __fadd_rn(sum.lo, a.lo));
}
__device__ __forceinline__ Sum2 wallAddDot(Sum2 sum, f3 a, f3 b) {
    float px = __fmul_rn(a.x, b.x), py = __fmul_rn(a.y, b.y), pz = __fmul_rn(a.z, b.z);
    sum = wallAdd(sum, px);
    sum = wallAdd(sum, __fmaf_rn(a.x, b.x, -px));
    sum = wallAdd(sum, py);
    sum = wallAdd(sum, __fmaf_rn(a.y, b.y, -py));
    sum = wallAdd(sum, pz);
    return wallAdd(sum, __fmaf_rn(a.z, b.z, -pz));
}
// Signed offset of the grain centre from the plane, never forming a
// world-space surface point (solver.slang:596-604).
__device__ __forceinline__ Sum2 wallCentreDistance(const Res& r, uint32_t body, uint32_t wall) {
    float4 plane = r.wallPlane[wall], low = r.wallRemainder[wall];
    f3 p = xyz(r.position[body]), pl = xyz(r.positionRemainder[body]);
    Sum2 sum{-plane.w, -low.w};
    sum = wallAddDot(sum, xyz(plane), p);
    sum = wallAddDot(sum, xyz(plane), pl);
    sum = wallAddDot(sum, xyz(low), p);
    return wallAddDot(sum, xyz(low), pl);
}
// Half-step work of every wall on grain id, added to its compensated
// per-(wall, grain) total (solver.slang:135-146).
__device__ __forceinline__ float wallStepWork(const Res& r, const Config& c, uint32_t id, float dt) {
    float total = 0.f;
    for (uint32_t w = 0; w < c.wallCount; ++w) {
        uint32_t index = w * c.N + id;
        float increment = __fmul_rn(dt, r.wallRows[3 * index + 1].w);
        float4 state = r.wallAccumulated[index];
        float y = __fadd_rn(increment, state.y);
        float high = __fadd_rn(state.x, y);
        float low = __fsub_rn(y, __fsub_rn(high, state.x));
        r.wallAccumulated[index] = make_float4(high, low, 0.f, 0.f);
        r.wallRows[3 * index + 2] = make_float4(__fadd_rn(high, low), 0.f, 0.f, 0.f);
        total = __fadd_rn(total, increment);
    }
    return total;
}

}  // namespace sdg
