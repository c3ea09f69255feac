// CPU ORACLE — test infrastructure only.  Nothing in the product links or
// calls this file; tests, the smoke check and the benchmark's CPU baseline
// use it as the checker.
//
// Serial C++ restatement of the reference CPU backend for one mesh-surface
// DEM step: the Slang kernels of src/sand_atlas_dem/shaders/solver.slang with
// the CPU substitutions of shaders/cpu_scheduling.slang (serial atomics
// :3-6, FP64 minimum image :10-15, cached-distance BVH walk :18-48,
// per-directed-pair enclosure plane + cluster walk :53-91) as the reference
// CPU backend assembles them (src/sand_atlas_dem/cpu.py:46-103).
//
// FP32 operation order follows the Slang-generated C++ of the reference
// (evidence/hostun424-cpu-pair-plane-counts-v1/.../instrumented-collector.cpp):
// dot = ((0 + x0*y0) + x1*y1) + x2*y2, length = sqrtf(dot), min/max are the
// ternaries a<b?a:b / a>b?a:b, literals are real.  Build with
// -O3 -fno-fast-math -ffp-contract=off (cpu.py:323-334).
//
// ABI (mirrors the reference cpu_dispatch, cpu.py:189-300):
//   oracle_dispatch(name, count, buffers, bytes, values, nvalues)
// buffers[0..76] are the reference Resources fields in declaration order
// (solver.slang:20-100), followed by entry-point uniform buffers; values are
// the 25 Config scalars (solver.slang:12-19) followed by entry-point uniform
// scalars.  Returns 0, or -1 for an unknown kernel name.  Solver failures go
// to control[0] exactly as on the device.

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <atomic>
#include <string_view>
#include <thread>
#include <vector>

// The arithmetic type: float (the restatement of the reference's FP32 step,
// libdem_oracle.so) or, built with -DORACLE_FP64=1, double (the FP64 drift
// oracle, libdem_oracle64.so: the same step with every float buffer and
// every FP32 operation in double precision).
#ifndef ORACLE_FP64
#define ORACLE_FP64 0
#endif
#if ORACLE_FP64
using real = double;
#else
using real = float;
#endif

namespace {

struct vec3 { real x, y, z; };
struct vec4 { real x, y, z, w; };
struct uint4 { uint32_t x, y, z, w; };
struct uint2 { uint32_t x, y; };
struct double3 { double x, y, z; };

inline vec3 f3(real x, real y, real z) { return {x, y, z}; }
inline vec3 xyz(const vec4& a) { return {a.x, a.y, a.z}; }
inline vec4 f4(const vec3& a, real w) { return {a.x, a.y, a.z, w}; }
inline vec3 operator+(vec3 a, vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(vec3 a, vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(vec3 a, vec3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator/(vec3 a, vec3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline vec3 operator*(real s, vec3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline vec3 operator*(vec3 a, real s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator/(vec3 a, real s) { return {a.x / s, a.y / s, a.z / s}; }
inline vec3 operator-(vec3 a) { return {-a.x, -a.y, -a.z}; }
inline vec4 operator+(vec4 a, vec4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline vec4 operator-(vec4 a, vec4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
inline vec4 operator*(vec4 a, real s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }

inline real mn(real a, real b) { return a < b ? a : b; }
inline real mx(real a, real b) { return a > b ? a : b; }
inline vec3 mn3(vec3 a, vec3 b) { return {mn(a.x, b.x), mn(a.y, b.y), mn(a.z, b.z)}; }
inline vec3 mx3(vec3 a, vec3 b) { return {mx(a.x, b.x), mx(a.y, b.y), mx(a.z, b.z)}; }
inline vec3 abs3(vec3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline real dot(vec3 a, vec3 b) {
    real r = 0.0f;
    r = r + a.x * b.x;
    r = r + a.y * b.y;
    r = r + a.z * b.z;
    return r;
}
inline real dot4(vec4 a, vec4 b) {
    real r = 0.0f;
    r = r + a.x * b.x;
    r = r + a.y * b.y;
    r = r + a.z * b.z;
    r = r + a.w * b.w;
    return r;
}
inline real length(vec3 a) { return std::sqrt(dot(a, a)); }
inline vec3 cross(vec3 l, vec3 r) {
    return {l.y * r.z - l.z * r.y, l.z * r.x - l.x * r.z, l.x * r.y - l.y * r.x};
}
inline real comp(vec3 a, uint32_t i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline bool finite3(vec3 a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }

// solver.slang:104-106
inline vec3 qrot(vec4 q, vec3 v) {
    vec3 u = xyz(q);
    return v + 2.0f * cross(u, cross(u, v) + q.w * v);
}
inline vec3 qinv(vec4 q, vec3 v) { return qrot(vec4{-q.x, -q.y, -q.z, q.w}, v); }
inline vec4 qmul(vec4 a, vec4 b) {
    vec3 v = (a.w * xyz(b) + b.w * xyz(a)) + cross(xyz(a), xyz(b));
    return f4(v, a.w * b.w - dot(xyz(a), xyz(b)));
}
// Slang normalize: x * rsqrt(dot(x, x)), rsqrt = 1 / sqrt.
inline vec4 normalize4(vec4 q) { return q * (1.0f / std::sqrt(dot4(q, q))); }

const uint32_t EMPTY = 0xffffffffu;

struct Config {
    uint32_t activeTimestep, N, shapes, pairCapacity, contactCapacity, binCapacity, binCount;
    uint32_t bins[3];
    uint32_t hashSize;
    real dt, kn, kt, mu, normalViscosity, skin, drag, maxOverlap;
    uint32_t historyStep, meshGeometry, periodic, wallCount, wallBoxEnabled, sourceSurfaceNormal;
};

struct R {
    Config c;
    uint32_t* control; vec4* cell; vec4* position; vec4* positionRemainder;
    vec4* velocityRemainder; vec4* momentumRemainder; vec4* rotationRemainder;
    vec4* referencePositionRemainder; vec4* cellLog; vec4* accumulatedRemainder;
    vec4* velocity; vec4* rotation; vec4* momentum; vec4* force; vec4* torque;
    vec4* referencePosition; vec4* referenceCell; uint32_t* shapeId; vec4* body; vec4* invI;
    uint4* grids; uint4* sampleInfo; vec4* gridOrigin; real* distance; vec4* sample;
    uint4* meshRoots; uint4* meshHullInfo; vec4* meshPlanes; vec4* meshMin; vec4* meshMax;
    uint4* meshLinks; vec4* meshTriangles; vec4* meshNormals; uint4* meshFrontier;
    uint32_t* meshPairMask; vec4* meshPairTransform; uint4* meshClusterInfo;
    uint4* meshClusterRanges; vec4* meshClusterMin; vec4* meshClusterMax;
    uint32_t* meshSampleIndices; uint32_t* binCounts; uint32_t* binParticles; uint32_t* pairCounts;
    uint32_t* pairOffsets; uint2* pairs; uint32_t* contactCounts; uint32_t* contactOffsets;
    uint4* meta; vec4* pointDepth; vec4* normalArea; vec4* slip; vec4* contactForce;
    real* normalLossPower; vec4* normalDamping; vec4* forceVelocity; vec4* forceOmega;
    uint4* oldMeta; vec4* oldSlip; vec4* oldNormal; uint32_t* oldHash; uint32_t* hash;
    uint32_t* heads; uint32_t* next; vec4* particleStress; vec4* timestepRows;
    vec4* particleDiagnostic; vec4* diagnosticRows; vec4* accumulated; vec4* fabricRows;
    vec4* wallPlane; vec4* wallRemainder; vec4* wallVelocity; vec4* wallMaterial;
    uint32_t* wallBoxIds; vec4* wallRows; vec4* wallAccumulated;
    void** extra;      // entry-point uniform buffers
    const double* uni; // entry-point uniform scalars
};

void bind(R& r, void** b, const double* v) {
    static_assert(sizeof(void*) * 77 == offsetof(R, extra) - offsetof(R, control), "pointer block");
    std::memcpy(static_cast<void*>(&r.control), b, 77 * sizeof(void*));
    r.extra = b + 77;
    Config& c = r.c;
    c.activeTimestep = uint32_t(v[0]); c.N = uint32_t(v[1]); c.shapes = uint32_t(v[2]);
    c.pairCapacity = uint32_t(v[3]); c.contactCapacity = uint32_t(v[4]);
    c.binCapacity = uint32_t(v[5]); c.binCount = uint32_t(v[6]);
    c.bins[0] = uint32_t(v[7]); c.bins[1] = uint32_t(v[8]); c.bins[2] = uint32_t(v[9]);
    c.hashSize = uint32_t(v[10]);
    c.dt = real(v[11]); c.kn = real(v[12]); c.kt = real(v[13]); c.mu = real(v[14]);
    c.normalViscosity = real(v[15]); c.skin = real(v[16]); c.drag = real(v[17]);
    c.maxOverlap = real(v[18]);
    c.historyStep = uint32_t(v[19]); c.meshGeometry = uint32_t(v[20]); c.periodic = uint32_t(v[21]);
    c.wallCount = uint32_t(v[22]); c.wallBoxEnabled = uint32_t(v[23]);
    c.sourceSurfaceNormal = uint32_t(v[24]);
    r.uni = v + 25;
}

inline void fail(R& r, uint32_t bit) { r.control[0] |= bit; }  // solver.slang:183, serial

// solver.slang:111-118 (rounded3/4 are identities while control[15] is zero)
inline void compensated3(vec3& high, vec3& low, vec3 inc) {
    vec3 y = inc + low;
    vec3 nx = high + y;
    vec3 moved = nx - high;
    low = y - moved;
    high = nx;
}
inline void compensated4(vec4& high, vec4& low, vec4 inc) {
    vec4 y = inc + low;
    vec4 nx = high + y;
    vec4 moved = nx - high;
    low = y - moved;
    high = nx;
}
// solver.slang:119-123
inline real expm1Stable(real x) {
    if (std::fabs(x) < 0.01f)
        return x * (1.0f + x * (0.5f + x * (1.0f / 6.0f + x * (1.0f / 24.0f + x / 120.0f))));
    return std::exp(x) - 1.0f;
}
inline vec3 expm1Stable3(vec3 x) { return {expm1Stable(x.x), expm1Stable(x.y), expm1Stable(x.z)}; }
// solver.slang:124-129
inline vec4 rotationIncrement(vec3 w, real dt, vec4 q) {
    real half = 0.5f * length(w) * dt;
    real coefficient = std::fabs(half) < 0.001f ? 0.5f * dt * (1.0f - half * half / 6.0f)
                                                 : std::sin(half) / length(w);
    real cm1 = -2.0f * std::sin(0.5f * half) * std::sin(0.5f * half);
    return qmul(f4(coefficient * w, cm1), q);
}
// solver.slang:130-134
inline void accumulate(R& r, uint32_t id, vec4 inc) {
    vec4 high = r.accumulated[id], low = r.accumulatedRemainder[id];
    compensated4(high, low, inc);
    r.accumulated[id] = high;
    r.accumulatedRemainder[id] = low;
}
// cpu_scheduling.slang:10-15 (FP64 branch, cast to FP32)
inline vec3 centerBranch(R& r, uint32_t i, uint32_t j) {
    double3 box{double(r.cell[0].x), double(r.cell[0].y), double(r.cell[0].z)};
    double3 pj{double(r.position[j].x), double(r.position[j].y), double(r.position[j].z)};
    double3 pi{double(r.position[i].x), double(r.position[i].y), double(r.position[i].z)};
    double3 lj{double(r.positionRemainder[j].x), double(r.positionRemainder[j].y), double(r.positionRemainder[j].z)};
    double3 li{double(r.positionRemainder[i].x), double(r.positionRemainder[i].y), double(r.positionRemainder[i].z)};
    double3 d{(pj.x - pi.x) + (lj.x - li.x), (pj.y - pi.y) + (lj.y - li.y), (pj.z - pi.z) + (lj.z - li.z)};
    if (r.c.periodic != 0) {
        d.x = d.x - std::floor(d.x / box.x + 0.5) * box.x;
        d.y = d.y - std::floor(d.y / box.y + 0.5) * box.y;
        d.z = d.z - std::floor(d.z / box.z + 0.5) * box.z;
    }
    return {real(d.x), real(d.y), real(d.z)};
}
// solver.slang:154-158
inline vec3 omega(R& r, uint32_t i) {
    vec3 b = qinv(r.rotation[i], xyz(r.momentum[i]) + xyz(r.momentumRemainder[i]));
    vec3 w{dot(xyz(r.invI[3 * i]), b), dot(xyz(r.invI[3 * i + 1]), b), dot(xyz(r.invI[3 * i + 2]), b)};
    return qrot(r.rotation[i], w);
}
// solver.slang:159-163
inline real rotationalEnergy(R& r, uint32_t i, vec3 l) {
    vec3 b = qinv(r.rotation[i], l);
    vec3 w{dot(xyz(r.invI[3 * i]), b), dot(xyz(r.invI[3 * i + 1]), b), dot(xyz(r.invI[3 * i + 2]), b)};
    return 0.5f * dot(b, w);
}
// solver.slang:164-169
inline void accumulateNormalLoss(R& r, uint32_t id, real dt) {
    vec4 value = r.normalDamping[id];
    vec3 high{value.x, 0, 0}, low{value.y, 0, 0};
    compensated3(high, low, f3(value.z * dt, 0, 0));
    value.x = high.x;
    value.y = low.x;
    r.normalDamping[id] = value;
}
// solver.slang:176-180
inline real cellPower(R& r, uint32_t i) {
    vec3 diagonal{r.particleStress[3 * i].x, r.particleStress[3 * i + 1].y, r.particleStress[3 * i + 2].z};
    vec3 v = xyz(r.velocity[i]);
    return -dot(diagonal + r.body[i].y * v * v, xyz(r.cell[1]));
}
inline real floorf_(real x) { return std::floor(x); }
// solver.slang:181-186
inline vec3 image(R& r, vec3 d) {
    vec3 box = xyz(r.cell[0]);
    if (r.c.periodic == 0) return d;
    return d - f3(floorf_(d.x / box.x + 0.5f), floorf_(d.y / box.y + 0.5f), floorf_(d.z / box.z + 0.5f)) * box;
}
inline void binIndex(R& r, uint32_t i, uint32_t b[3]) {
    vec3 p = xyz(r.position[i]), box = xyz(r.cell[0]);
    real g[3] = {floorf_(p.x / box.x * real(r.c.bins[0])), floorf_(p.y / box.y * real(r.c.bins[1])),
                  floorf_(p.z / box.z * real(r.c.bins[2]))};
    for (int k = 0; k < 3; ++k) {
        uint32_t v = uint32_t(g[k]);
        b[k] = v < r.c.bins[k] - 1 ? v : r.c.bins[k] - 1;
    }
}
inline uint32_t binFlat(R& r, const uint32_t b[3]) { return (b[0] * r.c.bins[1] + b[1]) * r.c.bins[2] + b[2]; }
inline uint32_t modIndex(int a, uint32_t n) { return uint32_t((a % int(n) + int(n)) % int(n)); }

// solver.slang:203-219
vec3 closestTriangle(vec3 p, vec3 a, vec3 b, vec3 c, uint32_t& feature) {
    vec3 ab = b - a, ac = c - a, ap = p - a;
    real d1 = dot(ab, ap), d2 = dot(ac, ap);
    feature = 4;
    if (d1 <= 0 && d2 <= 0) return a;
    vec3 bp = p - b;
    real d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { feature = 5; return b; }
    real vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { feature = 1; return a + (d1 / (d1 - d3)) * ab; }
    vec3 cp = p - c;
    real d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) { feature = 6; return c; }
    real vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) { feature = 3; return a + (d2 / (d2 - d6)) * ac; }
    real va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        feature = 2;
        return b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b);
    }
    real inv = 1.0f / (va + vb + vc);
    feature = 0;
    return a + ab * (vb * inv) + ac * (vc * inv);
}
// solver.slang:220-223
inline real meshBoxDistance(R& r, uint32_t node, vec3 p) {
    vec3 d = mx3(mx3(xyz(r.meshMin[node]) - p, p - xyz(r.meshMax[node])), f3(0, 0, 0));
    return dot(d, d);
}
// cpu_scheduling.slang:18-48 (cached pushed distances; same result as the
// original solver.slang:224-252 walk)
vec4 meshDistance(R& r, uint32_t shape, vec3 p, bool surfaceNormal) {
    uint32_t root = r.meshRoots[shape].x;
    uint32_t pending[32];
    real pendingDistance[32];
    uint32_t top = 1;
    pending[0] = root;
    pendingDistance[0] = meshBoxDistance(r, root, p);
    real best = 1e30f;
    vec3 nearest{0, 0, 0};
    uint32_t nearestNormal = 0;
    bool found = false;
    while (top > 0) {
        uint32_t slot = --top, node = pending[slot];
        if (pendingDistance[slot] > best) continue;
        uint4 link = r.meshLinks[node];
        if (link.z == 0) {
            uint32_t a = node + 1, b = r.meshLinks[a].x;
            real da = meshBoxDistance(r, a, p), db = meshBoxDistance(r, b, p);
            if (da < db) { uint32_t s = a; a = b; b = s; real ds = da; da = db; db = ds; }
            if (top + 2 > 32) { fail(r, 1024); return {0, 0, 0, 1e20f}; }
            if (da <= best) { pending[top] = a; pendingDistance[top++] = da; }
            if (db <= best) { pending[top] = b; pendingDistance[top++] = db; }
            continue;
        }
        for (uint32_t j = 0; j < link.z; ++j) {
            uint32_t triangle = link.y + j, feature;
            vec3 q = closestTriangle(p, xyz(r.meshTriangles[3 * triangle]), xyz(r.meshTriangles[3 * triangle + 1]),
                                       xyz(r.meshTriangles[3 * triangle + 2]), feature);
            real distance = dot(p - q, p - q);
            if (distance < best) { best = distance; nearest = q; nearestNormal = 7 * triangle + feature; found = true; }
        }
    }
    vec3 pseudo = found ? xyz(r.meshNormals[nearestNormal]) : f3(0, 0, 0);
    real distance = std::sqrt(best);
    real side = dot(p - nearest, pseudo) < 0 ? -1.0f : 1.0f;
    vec3 normal = surfaceNormal ? pseudo : (distance > 1e-12f ? (side * (p - nearest)) / distance : pseudo);
    return f4(normal, side * distance);
}
// solver.slang:259-272
bool meshMayContain(R& r, uint32_t shape, vec3 p) {
    uint32_t root = r.meshRoots[shape].x;
    vec3 low = xyz(r.meshMin[root]), high = xyz(r.meshMax[root]);
    if (p.x < low.x || p.y < low.y || p.z < low.z || p.x > high.x || p.y > high.y || p.z > high.z) return false;
    vec3 direction = (p - 0.5f * (low + high)) / (high - low);
    vec3 a = abs3(direction);
    uint32_t axis = a.x >= a.y && a.x >= a.z ? 0 : (a.y >= a.z ? 1 : 2);
    uint32_t group = 2 * axis + (comp(direction, axis) >= 0 ? 1 : 0);
    uint4 info = r.meshHullInfo[6 * shape + group];
    for (uint32_t i = 0; i < info.y; ++i) {
        vec4 plane = r.meshPlanes[info.x + i];
        if (dot(xyz(plane), p) + plane.w > 0) return false;
    }
    return true;
}
// solver.slang:274-288
bool meshBoxMayContact(R& r, uint32_t shape, vec3 low, vec3 high) {
    uint32_t root = r.meshRoots[shape].x;
    vec3 tl = xyz(r.meshMin[root]), th = xyz(r.meshMax[root]);
    if (high.x < tl.x || high.y < tl.y || high.z < tl.z || low.x > th.x || low.y > th.y || low.z > th.z) return false;
    vec3 center = 0.5f * (low + high), half = 0.5f * (high - low);
    vec3 direction = (center - 0.5f * (tl + th)) / (th - tl);
    vec3 a = abs3(direction);
    uint32_t axis = a.x >= a.y && a.x >= a.z ? 0 : (a.y >= a.z ? 1 : 2);
    uint32_t group = 2 * axis + (comp(direction, axis) >= 0 ? 1 : 0);
    uint4 info = r.meshHullInfo[6 * shape + group];
    for (uint32_t i = 0; i < info.y; ++i) {
        vec4 plane = r.meshPlanes[info.x + i];
        if (dot(xyz(plane), center) + plane.w - dot(abs3(xyz(plane)), half) > 0) return false;
    }
    return true;
}
// solver.slang:290-305
bool meshClusterMayContact(R& r, uint32_t src, uint32_t dst, uint32_t cluster) {
    vec3 sl = xyz(r.meshClusterMin[cluster]), sh = xyz(r.meshClusterMax[cluster]);
    vec3 branch = centerBranch(r, src, dst), low{1e30f, 1e30f, 1e30f}, high{-1e30f, -1e30f, -1e30f};
    for (uint32_t corner = 0; corner < 8; ++corner) {
        vec3 p{(corner & 1) ? sh.x : sl.x, (corner & 2) ? sh.y : sl.y, (corner & 4) ? sh.z : sl.z};
        p = qinv(r.rotation[dst], qrot(r.rotation[src], p * r.body[src].x) - branch) / r.body[dst].x;
        low = mn3(low, p);
        high = mx3(high, p);
    }
    real pad = 0.00000762939453125f *
                (1.0f + mx(mx(std::fabs(low.x), std::fabs(low.y)), std::fabs(low.z)) +
                 mx(mx(std::fabs(high.x), std::fabs(high.y)), std::fabs(high.z)) + length(branch) / r.body[dst].x);
    low = low - f3(pad, pad, pad);
    high = high + f3(pad, pad, pad);
    return meshBoxMayContact(r, r.shapeId[dst], low, high);
}
// solver.slang:404-417
void meshPairBounds(R& r, uint32_t direction, uint32_t cluster, vec3& low, vec3& high) {
    vec3 center = 0.5f * (xyz(r.meshClusterMin[cluster]) + xyz(r.meshClusterMax[cluster]));
    vec3 half = 0.5f * (xyz(r.meshClusterMax[cluster]) - xyz(r.meshClusterMin[cluster]));
    real c[3], e[3];
    for (uint32_t axis = 0; axis < 3; ++axis) {
        vec4 row = r.meshPairTransform[4 * direction + axis];
        c[axis] = dot(xyz(row), center) + row.w;
        e[axis] = dot(abs3(xyz(row)), half);
    }
    low = f3(c[0], c[1], c[2]) - f3(e[0], e[1], e[2]);
    high = f3(c[0], c[1], c[2]) + f3(e[0], e[1], e[2]);
    real pad = 0.000030517578125f *
                (1.0f + mx(mx(std::fabs(low.x), std::fabs(low.y)), std::fabs(low.z)) +
                 mx(mx(std::fabs(high.x), std::fabs(high.y)), std::fabs(high.z)) +
                 r.meshPairTransform[4 * direction + 3].x);
    low = low - f3(pad, pad, pad);
    high = high + f3(pad, pad, pad);
}
// solver.slang:319-343 with the CPU enclosure-plane prefilter (cpu.py:56-76)
bool nodeContact(R& r, uint32_t src, uint32_t dst, uint32_t node, vec4& pd, vec4& na, vec4 rejectionPlane) {
    uint32_t sid = r.shapeId[src];
    vec4 sp = r.sample[r.sampleInfo[sid].x + node];
    vec3 arm = qrot(r.rotation[src], xyz(sp) * r.body[src].x);
    vec3 branch = centerBranch(r, src, dst);
    vec3 local = qinv(r.rotation[dst], arm - branch) / r.body[dst].x;
    uint32_t targetShape = r.shapeId[dst];
    vec4 f;
    real planePad = 0.00000762939453125f *
                     (1.0f + mx(mx(std::fabs(local.x), std::fabs(local.y)), std::fabs(local.z)));
    if (dot(xyz(rejectionPlane), local) + rejectionPlane.w > planePad) { pd = {0, 0, 0, 0}; na = {0, 0, 0, 0}; return false; }
    if (!meshMayContain(r, targetShape, local)) { pd = {0, 0, 0, 0}; na = {0, 0, 0, 0}; return false; }
    f = meshDistance(r, targetShape, local, false);
    pd = f4(arm, -f.w * r.body[dst].x);
    na = {0, 0, 0, 0};
    if (pd.w <= 0.0f) return false;
    vec3 grad = qrot(r.rotation[dst], xyz(f));
    real len = length(grad);
    if (r.c.sourceSurfaceNormal != 0) {
        vec4 own = meshDistance(r, sid, xyz(sp), true);
        if (std::fabs(own.w) > 0.00000999999974738f) { fail(r, 2); return false; }
        grad = -qrot(r.rotation[src], xyz(own));
        len = length(grad);
    }
    if (len < 1.00000001168609742e-07f || !std::isfinite(pd.w)) { fail(r, 2); return false; }
    na = f4(grad / len, sp.w * r.body[src].x * r.body[src].x);
    if (pd.w > r.c.maxOverlap * mn(r.body[src].w, r.body[dst].w)) fail(r, 4);
    return true;
}

// solver.slang:188-200: trilinear signed distance and its gradient from the
// shape's grid (FP32 order of the archived generated C++: lerp(x, y, s) =
// x + (y - x) * s; products left to right).
vec4 sdf(R& r, uint32_t s, vec3 p) {
    uint4 meta = r.grids[s];
    vec4 o = r.gridOrigin[s];
    vec3 g = (p - xyz(o)) / o.w;
    int32_t a[3] = {int32_t(std::floor(g.x)), int32_t(std::floor(g.y)), int32_t(std::floor(g.z))};
    int32_t dims[3] = {int32_t(meta.y), int32_t(meta.z), int32_t(meta.w)};
    for (int k = 0; k < 3; ++k)
        if (a[k] < 0 || a[k] >= dims[k] - 1) return {0.0f, 0.0f, 0.0f, 1.00000002004087734e+20f};
    vec3 t = g - f3(real(a[0]), real(a[1]), real(a[2]));
    vec3 u = f3(1.0f, 1.0f, 1.0f) - t;
    real value = 0.0f;
    vec3 grad = f3(0.0f, 0.0f, 0.0f);
    for (uint32_t i = 0; i < 2; ++i)
        for (uint32_t j = 0; j < 2; ++j)
            for (uint32_t k = 0; k < 2; ++k) {
                vec3 b = f3(real(i), real(j), real(k));
                vec3 w = u + (t - u) * b;
                uint32_t ix = uint32_t(a[0]) + i, iy = uint32_t(a[1]) + j, iz = uint32_t(a[2]) + k;
                real f = r.distance[meta.x + (ix * meta.z + iy) * meta.w + iz];
                value = value + f * w.x * w.y * w.z;
                vec3 v = f3((2.0f * real(i) - 1.0f) * w.y * w.z, (2.0f * real(j) - 1.0f) * w.x * w.z,
                              (2.0f * real(k) - 1.0f) * w.x * w.y);
                grad = grad + (f * v) / o.w;
            }
    return f4(grad, value);
}
// solver.slang:319-343 with the SDF geometry (meshGeometry == 0).
bool nodeContactSdf(R& r, uint32_t src, uint32_t dst, uint32_t node, vec4& pd, vec4& na) {
    uint32_t sid = r.shapeId[src];
    vec4 sp = r.sample[r.sampleInfo[sid].x + node];
    vec3 arm = qrot(r.rotation[src], xyz(sp) * r.body[src].x);
    vec3 branch = centerBranch(r, src, dst);
    vec3 local = qinv(r.rotation[dst], arm - branch) / r.body[dst].x;
    vec4 f = sdf(r, r.shapeId[dst], local);
    pd = f4(arm, -f.w * r.body[dst].x);
    na = {0, 0, 0, 0};
    if (pd.w <= 0.0f) return false;
    vec3 grad = qrot(r.rotation[dst], xyz(f));
    real len = length(grad);
    if (len < 1.00000001168609742e-07f || !std::isfinite(pd.w)) { fail(r, 2); return false; }
    na = f4(grad / len, sp.w * r.body[src].x * r.body[src].x);
    if (pd.w > r.c.maxOverlap * mn(r.body[src].w, r.body[dst].w)) fail(r, 4);
    return true;
}

// ---------------------------------------------------------------- kernels

real wallStepWork(R& r, uint32_t id, real dt);
// solver.slang:858-888
void beginStep(R& r, uint32_t id) {
    if (id >= r.c.N || r.control[0] != 0) return;
    real dt = r.c.dt;
    vec3 rate = xyz(r.cell[1]);
    accumulateNormalLoss(r, id, 0.5f * dt);
    vec3 v = xyz(r.velocity[id]), vl = xyz(r.velocityRemainder[id]);
    vec3 l = xyz(r.momentum[id]), ll = xyz(r.momentumRemainder[id]);
    compensated3(v, vl, 0.5f * dt * xyz(r.force[id]) / r.body[id].y);
    compensated3(l, ll, 0.5f * dt * xyz(r.torque[id]));
    real loss = -expm1Stable(-r.c.drag * dt) *
                 (0.5f * r.body[id].y * dot(v + vl, v + vl) + rotationalEnergy(r, id, l + ll));
    real cp = 0.5f * dt * cellPower(r, id);
    accumulate(r, id, vec4{0, loss, cp, wallStepWork(r, id, 0.5f * dt)});
    real damping = expm1Stable(-0.5f * r.c.drag * dt);
    compensated3(v, vl, damping * (v + vl));
    compensated3(l, ll, damping * (l + ll));
    r.momentum[id] = f4(l, 0);
    r.momentumRemainder[id] = f4(ll, 0);
    vec4 q = r.rotation[id], ql = r.rotationRemainder[id];
    vec3 w = omega(r, id);
    r.rotation[id] = normalize4(q + rotationIncrement(w, 0.5f * dt, q));
    w = omega(r, id);
    compensated4(q, ql, rotationIncrement(w, dt, q));
    if (std::fabs(dot4(q, q) - 1.0f) > 2e-6f) { q = normalize4(q); ql = {0, 0, 0, 0}; }
    r.rotation[id] = q;
    r.rotationRemainder[id] = ql;
    vec3 logarithm = xyz(r.cellLog[0]), residual = xyz(r.cellLog[1]);
    compensated3(logarithm, residual, rate * dt);
    vec3 box = xyz(r.cell[2]) * f3(std::exp(logarithm.x), std::exp(logarithm.y), std::exp(logarithm.z));
    vec3 p = xyz(r.position[id]), pl = xyz(r.positionRemainder[id]);
    compensated3(p, pl, expm1Stable3(rate * dt) * (p + pl) + dt * (v + vl));
    if (!finite3(p) || !finite3(pl)) { fail(r, 512); return; }
    if (r.c.periodic != 0) p = p - f3(floorf_(p.x / box.x), floorf_(p.y / box.y), floorf_(p.z / box.z)) * box;
    else if (p.x + pl.x < 0 || p.y + pl.y < 0 || p.z + pl.z < 0 || (p.x - box.x) + pl.x >= 0 ||
             (p.y - box.y) + pl.y >= 0 || (p.z - box.z) + pl.z >= 0) { fail(r, 2048); return; }
    r.position[id] = f4(p, 0);
    r.positionRemainder[id] = f4(pl, 0);
    compensated3(v, vl, expm1Stable3(-rate * dt) * (v + vl));
    r.velocity[id] = f4(v, 0);
    r.velocityRemainder[id] = f4(vl, 0);
}
// solver.slang:889-897
void advanceCell(R& r) {
    if (r.control[0] != 0) return;
    vec3 logarithm = xyz(r.cellLog[0]), residual = xyz(r.cellLog[1]);
    compensated3(logarithm, residual, xyz(r.cell[1]) * r.c.dt);
    r.cellLog[0] = f4(logarithm, 0);
    r.cellLog[1] = f4(residual, 0);
    r.cell[0] = f4(xyz(r.cell[2]) * f3(std::exp(logarithm.x), std::exp(logarithm.y), std::exp(logarithm.z)), 0);
    r.control[4] = 0;
    if (r.c.periodic != 0 && r.referenceCell[1].w >= 0.5f * mn(r.cell[0].x, mn(r.cell[0].y, r.cell[0].z))) fail(r, 256);
}
// solver.slang:898-904
void checkRebuild(R& r, uint32_t id) {
    if (id >= r.c.N) return;
    vec3 d = image(r, (xyz(r.position[id]) - xyz(r.referencePosition[id])) +
                            (xyz(r.positionRemainder[id]) - xyz(r.referencePositionRemainder[id])));
    real deformation = length(xyz(r.cell[0]) - xyz(r.referenceCell[0]));
    if (length(d) + deformation > 0.5f * r.c.skin) r.control[4] |= 1;
}
// solver.slang:905-920
void finishStep(R& r, uint32_t id) {
    if (id >= r.c.N || r.control[0] != 0) return;
    accumulateNormalLoss(r, id, 0.5f * r.c.dt);
    vec3 v = xyz(r.velocity[id]), vl = xyz(r.velocityRemainder[id]);
    vec3 l = xyz(r.momentum[id]), ll = xyz(r.momentumRemainder[id]);
    compensated3(v, vl, 0.5f * r.c.dt * xyz(r.force[id]) / r.body[id].y);
    compensated3(l, ll, 0.5f * r.c.dt * xyz(r.torque[id]));
    real loss = -expm1Stable(-r.c.drag * r.c.dt) *
                 (0.5f * r.body[id].y * dot(v + vl, v + vl) + rotationalEnergy(r, id, l + ll));
    real cp = 0.5f * r.c.dt * cellPower(r, id);
    accumulate(r, id, vec4{0, loss, cp, wallStepWork(r, id, 0.5f * r.c.dt)});
    real damping = expm1Stable(-0.5f * r.c.drag * r.c.dt);
    compensated3(v, vl, damping * (v + vl));
    compensated3(l, ll, damping * (l + ll));
    if (!finite3(v) || !finite3(l)) { fail(r, 512); return; }
    r.velocity[id] = f4(v, 0);
    r.velocityRemainder[id] = f4(vl, 0);
    r.momentum[id] = f4(l, 0);
    r.momentumRemainder[id] = f4(ll, 0);
}
// solver.slang:170-175
void captureContactKinematics(R& r, uint32_t id) {
    if (id >= r.c.N || r.control[0] != 0) return;
    r.forceVelocity[id] = f4(xyz(r.velocity[id]) + xyz(r.velocityRemainder[id]), 0);
    r.forceOmega[id] = f4(omega(r, id), 0);
}
// solver.slang:345-359
void clearBins(R& r, uint32_t id) {
    if (r.control[4] == 0) return;
    if (id < r.c.binCount) r.binCounts[id] = 0;
}
void fillBins(R& r, uint32_t id) {
    if (id >= r.c.N || r.control[4] == 0) return;
    vec3 p = xyz(r.position[id]), pl = xyz(r.positionRemainder[id]);
    if (!finite3(p) || !finite3(pl)) { fail(r, 512); return; }
    vec3 box = xyz(r.cell[0]);
    if (r.c.periodic == 0 && (p.x + pl.x < 0 || p.y + pl.y < 0 || p.z + pl.z < 0 || (p.x - box.x) + pl.x >= 0 ||
                              (p.y - box.y) + pl.y >= 0 || (p.z - box.z) + pl.z >= 0)) { fail(r, 2048); return; }
    uint32_t b[3];
    binIndex(r, id, b);
    uint32_t bin = binFlat(r, b);
    uint32_t slot = r.binCounts[bin]++;
    if (slot < r.c.binCapacity) r.binParticles[bin * r.c.binCapacity + slot] = id;
    else fail(r, 8);
}
// solver.slang:360-384
uint32_t findPairs(R& r, uint32_t id, bool emit) {
    uint32_t b[3];
    binIndex(r, id, b);
    real cutoff = r.referenceCell[1].w;
    int reach[3], low[3], high[3];
    uint32_t width[3];
    real box[3] = {r.cell[0].x, r.cell[0].y, r.cell[0].z};
    for (int k = 0; k < 3; ++k) {
        reach[k] = int(std::ceil(cutoff / box[k] * real(r.c.bins[k])));
        low[k] = int(b[k]) - reach[k] > 0 ? int(b[k]) - reach[k] : 0;
        high[k] = int(b[k]) + reach[k] < int(r.c.bins[k]) - 1 ? int(b[k]) + reach[k] : int(r.c.bins[k]) - 1;
        uint32_t w = uint32_t(2 * reach[k] + 1);
        width[k] = r.c.periodic != 0 ? (w < r.c.bins[k] ? w : r.c.bins[k]) : uint32_t(high[k] - low[k] + 1);
    }
    uint32_t count = 0;
    for (uint32_t x = 0; x < width[0]; ++x)
        for (uint32_t y = 0; y < width[1]; ++y)
            for (uint32_t z = 0; z < width[2]; ++z) {
                uint32_t c[3] = {modIndex(int(b[0]) - reach[0] + int(x), r.c.bins[0]),
                                 modIndex(int(b[1]) - reach[1] + int(y), r.c.bins[1]),
                                 modIndex(int(b[2]) - reach[2] + int(z), r.c.bins[2])};
                if (r.c.periodic == 0) { c[0] = uint32_t(low[0] + int(x)); c[1] = uint32_t(low[1] + int(y)); c[2] = uint32_t(low[2] + int(z)); }
                uint32_t bi = binFlat(r, c);
                uint32_t occupancy = r.binCounts[bi] < r.c.binCapacity ? r.binCounts[bi] : r.c.binCapacity;
                for (uint32_t slot = 0; slot < occupancy; ++slot) {
                    uint32_t j = r.binParticles[bi * r.c.binCapacity + slot];
                    if (j <= id) continue;
                    vec3 d = centerBranch(r, id, j);
                    if (r.c.sourceSurfaceNormal != 0 && dot(d, d) < 1e-12f) { fail(r, 16384); continue; }
                    real range = r.body[id].z + r.body[j].z + r.c.skin;
                    if (dot(d, d) > range * range) continue;
                    if (emit) {
                        uint32_t index = r.pairOffsets[id] + count;
                        if (index < r.c.pairCapacity) r.pairs[index] = uint2{id, j};
                        else fail(r, 16);
                    }
                    count++;
                }
            }
    return count;
}
void countPairs(R& r, uint32_t id) {
    if (id < r.c.N && r.control[4] != 0) r.pairCounts[id] = findPairs(r, id, false);
}
// Exclusive scan of pairCounts (scan.slang / cpu.py:476-490, exact uint32).
void scanPairs(R& r) {
    if (r.control[4] == 0) return;
    uint32_t total = 0;
    for (uint32_t i = 0; i < r.c.N; ++i) { r.pairOffsets[i] = total; total += r.pairCounts[i]; }
}
void emitPairs(R& r, uint32_t id) {
    if (id >= r.c.N || r.control[4] == 0) return;
    findPairs(r, id, true);
    r.referencePosition[id] = r.position[id];
    r.referencePositionRemainder[id] = r.positionRemainder[id];
    if (id == 0) {
        r.control[1] = r.pairOffsets[r.c.N - 1] + r.pairCounts[r.c.N - 1];
        r.referenceCell[0] = r.cell[0];
    }
}
// SDF geometry collector (solver.slang:536-572), serial: 64 lanes per pair,
// lane l taking the pair's nodes l, l+64, ... (the first grain's nodes, then
// the second's); a pair's contacts are written lane by lane.
inline uint32_t sdfNodes(R& r, uint2 ij, uint32_t& a) {
    a = r.sampleInfo[r.shapeId[ij.x]].y;
    return a + r.sampleInfo[r.shapeId[ij.y]].y;
}
void countContacts(R& r, uint32_t pair) {
    if (pair >= r.c.pairCapacity) return;
    uint32_t count = 0;
    if (pair < r.control[1] && r.control[0] == 0) {
        uint2 ij = r.pairs[pair];
        uint32_t a, total = sdfNodes(r, ij, a);
        for (uint32_t s = 0; s < total; ++s) {
            vec4 pd, na;
            if (nodeContactSdf(r, s < a ? ij.x : ij.y, s < a ? ij.y : ij.x, s < a ? s : s - a, pd, na)) count++;
        }
    }
    r.contactCounts[pair] = count;
}
void scanContacts(R& r) {  // exclusive scan over the pair capacity (cpu.py:476-490)
    uint32_t sum = 0;
    for (uint32_t p = 0; p < r.c.pairCapacity; ++p) {
        r.contactOffsets[p] = sum;
        sum += r.contactCounts[p];
    }
}
void contactTotal(R& r) {
    uint32_t n = r.c.pairCapacity;
    r.control[2] = r.contactOffsets[n - 1] + r.contactCounts[n - 1];
    r.control[6] = 0;
    if (r.control[2] > r.c.contactCapacity) fail(r, 32);
}
void emitContacts(R& r, uint32_t pair) {
    uint32_t active = r.control[1] < r.c.pairCapacity ? r.control[1] : r.c.pairCapacity;
    if (pair >= active || r.control[0] != 0) return;
    uint2 ij = r.pairs[pair];
    uint32_t a, total = sdfNodes(r, ij, a);
    uint32_t offset = r.contactOffsets[pair];
    for (uint32_t lane = 0; lane < 64; ++lane)
        for (uint32_t s = lane; s < total; s += 64) {
            uint32_t i = s < a ? ij.x : ij.y, j = s < a ? ij.y : ij.x, node = s < a ? s : s - a;
            vec4 pd, na;
            if (nodeContactSdf(r, i, j, node, pd, na)) {
                if (offset >= r.c.contactCapacity) { fail(r, 32); break; }
                r.meta[offset] = uint4{i, j, node, 0};
                r.pointDepth[offset] = pd;
                r.normalArea[offset] = na;
                offset++;
            }
        }
}
// solver.slang:396-403
void resetMeshContacts(R& r, uint32_t id) {
    if (r.control[0] != 0) return;
    if (id < r.c.pairCapacity) r.contactCounts[id] = 0;
    if (id == 0) { r.control[2] = 0; r.control[6] = 0; }
}
inline uint32_t activePairs(R& r) { return r.control[1] < r.c.pairCapacity ? r.control[1] : r.c.pairCapacity; }
// solver.slang:468-489
void prepareMeshPairs(R& r, uint32_t id) {
    if (id >= activePairs(r) || r.control[0] != 0) return;
    uint2 ij = r.pairs[id];
    uint32_t mask = 0;
    if (meshClusterMayContact(r, ij.x, ij.y, r.meshClusterInfo[r.shapeId[ij.x]].x)) mask |= 1;
    if (meshClusterMayContact(r, ij.y, ij.x, r.meshClusterInfo[r.shapeId[ij.y]].x)) mask |= 2;
    for (uint32_t pass = 0; pass < 2; ++pass) {
        if ((mask & (1u << pass)) == 0) continue;
        uint32_t i = pass == 0 ? ij.x : ij.y, j = pass == 0 ? ij.y : ij.x;
        real ratio = r.body[i].x / r.body[j].x;
        vec3 a = qinv(r.rotation[j], qrot(r.rotation[i], f3(ratio, 0, 0)));
        vec3 b = qinv(r.rotation[j], qrot(r.rotation[i], f3(0, ratio, 0)));
        vec3 c = qinv(r.rotation[j], qrot(r.rotation[i], f3(0, 0, ratio)));
        vec3 branch = centerBranch(r, i, j), offset = qinv(r.rotation[j], -branch) / r.body[j].x;
        uint32_t base = 4 * (2 * id + pass);
        r.meshPairTransform[base] = vec4{a.x, b.x, c.x, offset.x};
        r.meshPairTransform[base + 1] = vec4{a.y, b.y, c.y, offset.y};
        r.meshPairTransform[base + 2] = vec4{a.z, b.z, c.z, offset.z};
        r.meshPairTransform[base + 3] = vec4{length(branch) / r.body[j].x, 0, 0, 0};
    }
    r.meshPairMask[id] = mask;
}
// cpu_scheduling.slang:53-91
void cpuCollectMesh(R& r, uint32_t pair) {
    if (pair >= activePairs(r) || r.control[0] != 0) return;
    uint2 ij = r.pairs[pair];
    for (uint32_t pass = 0; pass < 2; ++pass) {
        uint32_t i = pass == 0 ? ij.x : ij.y, j = pass == 0 ? ij.y : ij.x;
        vec3 sourceCentre = -qinv(r.rotation[j], centerBranch(r, i, j)) / r.body[j].x;
        vec4 rejectionPlane{0, 0, 0, 0};
        real largest = -1e30f;
        for (uint32_t group = 0; group < 6; ++group) {
            uint4 hull = r.meshHullInfo[6 * r.shapeId[j] + group];
            for (uint32_t plane = 0; plane < hull.y; ++plane) {
                vec4 enclosure = r.meshPlanes[hull.x + plane];
                real violation = dot(xyz(enclosure), sourceCentre) + enclosure.w;
                if (violation > largest) { largest = violation; rejectionPlane = enclosure; }
            }
        }
        uint4 info = r.meshClusterInfo[r.shapeId[i]];
        uint32_t cluster = info.x;
        while (cluster < info.x + info.y) {
            bool candidate = meshClusterMayContact(r, i, j, cluster);
            uint4 range = r.meshClusterRanges[cluster];
            if (candidate) {
                for (uint32_t lane = 0; lane < range.y; ++lane) {
                    uint32_t node = r.meshSampleIndices[range.x + lane];
                    vec4 pd, na;
                    if (nodeContact(r, i, j, node, pd, na, rejectionPlane)) {
                        uint32_t offset = r.control[2]++;
                        if (offset >= r.c.contactCapacity) { fail(r, 32); return; }
                        r.meta[offset] = uint4{i, j, node, 0};
                        r.pointDepth[offset] = pd;
                        r.normalArea[offset] = na;
                        r.contactCounts[pair]++;
                    }
                }
            }
            cluster = candidate ? cluster + 1 : range.z;
        }
    }
}
// Pair-parallel collector (the reference worker bridge, shaders/
// cpu_parallel.hpp:31-116): every pair collects with private control words
// into private storage, then contacts are concatenated in pair order, so the
// result equals the serial collector's; flags of all pairs are ORed.
void collectParallel(R& r, uint32_t pairs, uint32_t threads) {
    if (threads <= 1 || pairs <= 1 || r.control[0] != 0) {
        for (uint32_t p = 0; p < pairs; ++p) cpuCollectMesh(r, p);
        return;
    }
    std::vector<std::vector<uint4>> meta(pairs);
    std::vector<std::vector<vec4>> point(pairs), normal(pairs);
    std::vector<uint32_t> flags(pairs, 0), counts(pairs, 0);
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        R local = r;
        uint32_t control[16];
        std::vector<uint4> m;
        std::vector<vec4> pd, na;
        for (;;) {
            uint32_t pair = next.fetch_add(1, std::memory_order_relaxed);
            if (pair >= pairs) return;
            uint2 ij = r.pairs[pair];
            uint32_t capacity = r.sampleInfo[r.shapeId[ij.x]].y + r.sampleInfo[r.shapeId[ij.y]].y;
            m.resize(capacity);
            pd.resize(capacity);
            na.resize(capacity);
            std::memcpy(control, r.control, sizeof(control));
            control[0] = 0;
            control[2] = 0;
            local.control = control;
            local.c.contactCapacity = capacity;
            local.meta = m.data();
            local.pointDepth = pd.data();
            local.normalArea = na.data();
            local.contactCounts = counts.data();  // one writer per pair
            cpuCollectMesh(local, pair);
            flags[pair] = control[0];
            meta[pair].assign(m.begin(), m.begin() + control[2]);
            point[pair].assign(pd.begin(), pd.begin() + control[2]);
            normal[pair].assign(na.begin(), na.begin() + control[2]);
        }
    };
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < threads && t < pairs; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    uint64_t total = 0;
    uint32_t all = 0;
    for (uint32_t p = 0; p < pairs; ++p) { total += meta[p].size(); all |= flags[p]; }
    r.control[2] = uint32_t(total < 0xffffffffu ? total : 0xffffffffu);
    if (total > r.c.contactCapacity) all |= 32;
    r.control[0] |= all;
    if (all) return;
    size_t offset = 0;
    for (uint32_t p = 0; p < pairs; ++p) {
        size_t k = meta[p].size();
        if (k) {
            std::memcpy(r.meta + offset, meta[p].data(), k * sizeof(uint4));
            std::memcpy(r.pointDepth + offset, point[p].data(), k * sizeof(vec4));
            std::memcpy(r.normalArea + offset, normal[p].data(), k * sizeof(vec4));
        }
        r.contactCounts[p] = uint32_t(k);
        offset += k;
    }
}
// Exhaustive node set: cpu_scheduling.slang:104-131 + solver.slang:566-572
// (count, scan, total, emit); every node of both grains, no cull.
void exhaustiveContacts(R& r) {
    uint32_t pairs = activePairs(r);
    vec4 none{0, 0, 0, 0};
    std::vector<uint32_t> counts(r.c.pairCapacity, 0);
    if (r.control[0] == 0) {
        for (uint32_t pair = 0; pair < pairs; ++pair) {
            uint2 ij = r.pairs[pair];
            uint32_t a = r.sampleInfo[r.shapeId[ij.x]].y, total = a + r.sampleInfo[r.shapeId[ij.y]].y;
            for (uint32_t s = 0; s < total; ++s) {
                vec4 pd, na;
                if (nodeContact(r, s < a ? ij.x : ij.y, s < a ? ij.y : ij.x, s < a ? s : s - a, pd, na, none)) counts[pair]++;
            }
        }
    }
    uint32_t offset = 0;
    for (uint32_t p = 0; p < r.c.pairCapacity; ++p) { r.contactCounts[p] = counts[p]; r.contactOffsets[p] = offset; offset += counts[p]; }
    r.control[2] = offset;
    r.control[6] = 0;
    if (r.control[2] > r.c.contactCapacity) fail(r, 32);
    if (r.control[0] != 0) return;
    for (uint32_t pair = 0; pair < pairs; ++pair) {
        uint2 ij = r.pairs[pair];
        uint32_t a = r.sampleInfo[r.shapeId[ij.x]].y, total = a + r.sampleInfo[r.shapeId[ij.y]].y, o = r.contactOffsets[pair];
        for (uint32_t s = 0; s < total; ++s) {
            uint32_t i = s < a ? ij.x : ij.y, j = s < a ? ij.y : ij.x, node = s < a ? s : s - a;
            vec4 pd, na;
            if (nodeContact(r, i, j, node, pd, na, none)) {
                if (o >= r.c.contactCapacity) { fail(r, 32); break; }
                r.meta[o] = uint4{i, j, node, 0};
                r.pointDepth[o] = pd;
                r.normalArea[o] = na;
                o++;
            }
        }
    }
}
// ------------------------------------------------------------------ planes
// solver.slang:578-595: error-free two-sums (the materialisation mask
// rounded1 is the identity while control[15] is zero).
struct Sum2 { real hi, lo; };
inline Sum2 wallTwoSum(real a, real b) {
    real high = a + b, v = high - a;
    real low = (a - (high - v)) + (b - v);
    return {high, low};
}
inline Sum2 wallAdd(Sum2 a, real b) {
    Sum2 sum = wallTwoSum(a.hi, b);
    return wallTwoSum(sum.hi, sum.lo + a.lo);
}
inline Sum2 wallAddDot(Sum2 sum, vec3 a, vec3 b) {
    vec3 product = a * b;
    vec3 error{std::fma(a.x, b.x, -product.x), std::fma(a.y, b.y, -product.y), std::fma(a.z, b.z, -product.z)};
    for (uint32_t axis = 0; axis < 3; ++axis) {
        sum = wallAdd(sum, comp(product, axis));
        sum = wallAdd(sum, comp(error, axis));
    }
    return sum;
}
// solver.slang:596-604: the plane's signed offset at the grain centre.
Sum2 wallCentreDistance(R& r, uint32_t body, uint32_t wall) {
    vec4 plane = r.wallPlane[wall], low = r.wallRemainder[wall];
    vec3 p = xyz(r.position[body]), pl = xyz(r.positionRemainder[body]);
    Sum2 sum{-plane.w, -low.w};
    sum = wallAddDot(sum, xyz(plane), p);
    sum = wallAddDot(sum, xyz(plane), pl);
    sum = wallAddDot(sum, xyz(low), p);
    return wallAddDot(sum, xyz(low), pl);
}
// solver.slang:605-610
real localWallDistance(R& r, uint32_t body, uint32_t wall, vec3 arm) {
    Sum2 sum = wallCentreDistance(r, body, wall);
    sum = wallAddDot(sum, xyz(r.wallPlane[wall]), arm);
    sum = wallAddDot(sum, xyz(r.wallRemainder[wall]), arm);
    return sum.hi + sum.lo;
}
// solver.slang:613-624
bool wallClusterMayContact(R& r, uint32_t body, uint32_t wall, uint32_t cluster) {
    vec3 low = xyz(r.meshClusterMin[cluster]), high = xyz(r.meshClusterMax[cluster]);
    vec4 plane = r.wallPlane[wall];
    vec3 normal = qinv(r.rotation[body], xyz(plane)) * r.body[body].x;
    vec3 center = 0.5f * (low + high), half = 0.5f * (high - low);
    Sum2 centreDistance = wallCentreDistance(r, body, wall);
    real base = centreDistance.hi + centreDistance.lo;
    real support = dot(normal, center) - dot(abs3(normal), half);
    real pad = 64.0f * 1.1920928955078125e-7f *
                (((1.0f + std::fabs(plane.w)) + length(xyz(r.position[body]))) +
                 length(normal) * (length(center) + length(half)));
    return base + support <= pad;
}
// solver.slang:625-638 (serial append)
void appendWallContact(R& r, uint32_t body, uint32_t wall, uint32_t node) {
    vec4 point = r.sample[r.sampleInfo[r.shapeId[body]].x + node];
    vec3 arm = qrot(r.rotation[body], xyz(point) * r.body[body].x);
    vec4 plane = r.wallPlane[wall];
    real phi = localWallDistance(r, body, wall, arm);
    if (!std::isfinite(phi)) { fail(r, 512); return; }
    if (phi >= 0) return;
    if (-phi > r.c.maxOverlap * r.body[body].w) fail(r, 4);
    uint32_t offset = r.control[2]++;
    if (offset >= r.c.contactCapacity) { fail(r, 32); return; }
    r.meta[offset] = uint4{body, r.c.N + wall, node, 1};
    r.pointDepth[offset] = f4(arm, -phi);
    r.normalArea[offset] = f4(xyz(plane), point.w * r.body[body].x * r.body[body].x);
}
// cpu_scheduling.slang:133-154: one (wall, grain) per id, wall-major; nodes
// in order (SDF geometry) or the grain's sample clusters in preorder.
void collectWallContacts(R& r, uint32_t id) {
    uint32_t body = id % r.c.N, wall = id / r.c.N;
    if (wall >= r.c.wallCount || r.control[0] != 0) return;
    vec4 plane = r.wallPlane[wall];
    Sum2 centreDistance = wallCentreDistance(r, body, wall);
    real phi = centreDistance.hi + centreDistance.lo;
    real pad = 64.0f * 1.1920928955078125e-7f * ((1.0f + length(xyz(r.position[body]))) + std::fabs(plane.w));
    if (phi > r.body[body].z + pad) return;
    if (r.c.meshGeometry == 0) {
        uint32_t count = r.sampleInfo[r.shapeId[body]].y;
        for (uint32_t node = 0; node < count; ++node) appendWallContact(r, body, wall, node);
        return;
    }
    uint4 info = r.meshClusterInfo[r.shapeId[body]];
    uint32_t cluster = info.x;
    while (cluster < info.x + info.y) {
        bool candidate = wallClusterMayContact(r, body, wall, cluster);
        uint4 range = r.meshClusterRanges[cluster];
        if (candidate)
            for (uint32_t lane = 0; lane < range.y; ++lane)
                appendWallContact(r, body, wall, r.meshSampleIndices[range.x + lane]);
        cluster = candidate ? cluster + 1 : range.z;
    }
}
// solver.slang:669-687 (one thread)
void advanceWalls(R& r) {
    if (r.control[0] != 0) return;
    for (uint32_t w = 0; w < r.c.wallCount; ++w) {
        vec4 plane = r.wallPlane[w], residual = r.wallRemainder[w];
        vec3 high{plane.w, 0, 0}, low{residual.w, 0, 0};
        compensated3(high, low, f3(dot(xyz(plane), xyz(r.wallVelocity[w])) * r.c.dt, 0, 0));
        plane.w = high.x;
        residual.w = low.x;
        if (!std::isfinite(high.x) || !std::isfinite(low.x)) { fail(r, 512); return; }
        r.wallPlane[w] = plane;
        r.wallRemainder[w] = residual;
    }
    if (r.c.wallBoxEnabled != 0) {
        for (uint32_t axis = 0; axis < 3; ++axis) {
            uint32_t lo = r.wallBoxIds[2 * axis], hi = r.wallBoxIds[2 * axis + 1];
            real low = r.wallPlane[lo].w + r.wallRemainder[lo].w;
            real high = -(r.wallPlane[hi].w + r.wallRemainder[hi].w);
            if (low < 0 || high > comp(xyz(r.cell[0]), axis) || high <= low) fail(r, 4096);
        }
    }
}
// solver.slang:135-146: half-step wall work per (wall, grain) row.
real wallStepWork(R& r, uint32_t id, real dt) {
    real total = 0;
    for (uint32_t w = 0; w < r.c.wallCount; ++w) {
        uint32_t index = w * r.c.N + id;
        real increment = dt * r.wallRows[3 * index + 1].w;
        vec4 state = r.wallAccumulated[index];
        vec3 high{state.x, 0, 0}, low{state.y, 0, 0};
        compensated3(high, low, f3(increment, 0, 0));
        r.wallAccumulated[index] = vec4{high.x, low.x, 0, 0};
        r.wallRows[3 * index + 2] = vec4{high.x + low.x, 0, 0, 0};
        total = total + increment;
    }
    return total;
}
// solver.slang:834-856
void gatherWallRows(R& r, uint32_t index) {
    if (index >= r.c.N * r.c.wallCount || r.control[0] != 0) return;
    uint32_t body = index % r.c.N, wall = index / r.c.N, count = 0, visited = 0;
    vec3 reaction{0, 0, 0}, moment{0, 0, 0};
    real power = 0;
    uint32_t entry = r.heads[body];
    while (entry != EMPTY) {
        if (visited++ > 2 * r.c.contactCapacity) { fail(r, 128); return; }
        uint32_t contact = entry / 2;
        if (r.meta[contact].y == r.c.N + wall) {
            vec3 force = xyz(r.contactForce[contact]);
            vec3 point = (xyz(r.position[body]) + xyz(r.positionRemainder[body])) + xyz(r.pointDepth[contact]);
            reaction = reaction - force;
            moment = moment - cross(point, force);
            power = power + dot(force, xyz(r.wallVelocity[wall]));
            count++;
        }
        entry = r.next[entry];
    }
    vec4 work = r.wallAccumulated[index];
    // The contact count travels in the row's w as an integer bit pattern;
    // the FP64 build (a drift oracle without planes) stores its value.
#if ORACLE_FP64
    real bits = real(count);
#else
    real bits;
    std::memcpy(&bits, &count, 4);
#endif
    r.wallRows[3 * index] = f4(reaction, bits);
    r.wallRows[3 * index + 1] = f4(moment, power);
    r.wallRows[3 * index + 2] = vec4{work.x + work.y, 0, 0, 0};
}
// solver.slang:950-955
void refreshWallPower(R& r, uint32_t index) {
    if (index >= r.c.N * r.c.wallCount) return;
    vec4 value = r.wallRows[3 * index + 1];
    value.w = -dot(xyz(r.wallRows[3 * index]), xyz(r.wallVelocity[index / r.c.N]));
    r.wallRows[3 * index + 1] = value;
}

// solver.slang:689-696
inline uint32_t hashKey(R& r, uint4 key) {
    uint32_t h = key.x * 73856093u ^ key.y * 19349663u ^ key.z * 83492791u;
    h ^= h >> 16;
    return h & (r.c.hashSize - 1);
}
vec3 transported(vec3 x, vec3 a, vec3 b, real spin) {
    real c = mn(mx(dot(a, b), -1.0f), 1.0f);
    if (c < -0.999999f) return {0, 0, 0};
    vec3 v = cross(a, b);
    vec3 out = x + cross(v, x) + cross(v, cross(v, x)) / (1.0f + c);
    out = out * std::cos(spin) + cross(b, out) * std::sin(spin) + b * dot(b, out) * (1.0f - std::cos(spin));
    return out - b * dot(out, b);
}
// normal.slang:2-11
struct NormalResponse { real force, lossPower; };
NormalResponse normalResponse(real depth, real area, real normalVelocity, real stiffness, real viscosity, real weight) {
    NormalResponse value{0, 0};
    if (depth <= 0) return value;
    real elastic = weight * stiffness * area * depth;
    value.force = viscosity == 0 ? elastic : mx(0.0f, elastic - weight * viscosity * area * normalVelocity);
    value.lossPower = mx(0.0f, (elastic - value.force) * normalVelocity);
    return value;
}
// plane.slang:6-36: one-sided penalty plane with Coulomb slip.
struct PlaneResponse { vec4 forceEnergy, slipLoss; bool sliding; real normalLossPower; };
PlaneResponse planeViscousResponse(vec3 normal, real signedDistance, real area, vec3 relativeVelocity,
                                   vec3 oldSlip, real kn, real kt, real mu, real viscosity, real dt) {
    PlaneResponse value{{0, 0, 0, 0}, {0, 0, 0, 0}, false, 0};
    if (signedDistance >= 0) return value;
    real depth = -signedDistance;
    vec3 tangent = relativeVelocity - normal * dot(relativeVelocity, normal);
    vec3 trial = oldSlip - normal * dot(oldSlip, normal) + dt * tangent;
    vec3 slip = trial;
    NormalResponse response = normalResponse(depth, area, dot(relativeVelocity, normal), kn, viscosity, 1.0f);
    real fn = response.force;
    value.normalLossPower = response.lossPower;
    vec3 ft = -kt * area * slip;
    real magnitude = length(ft);
    if (magnitude > mu * fn && magnitude > 0) {
        value.sliding = true;
        ft = ft * (mu * fn / magnitude);
        slip = -ft / (kt * area);
    }
    value.forceEnergy = f4(fn * normal + ft, 0.5f * area * (kn * depth * depth + kt * dot(slip, slip)));
    value.slipLoss = f4(slip, mx(0.0f, -dot(ft, trial - slip)));
    return value;
}
// solver.slang:723-740: the grain-grain law of one directed node contact from
// its transported elastic slip: the trial slip over the step, the normal
// response (half weight: each pair contact is counted from both grains), the
// tangential traction and its Coulomb cap.
struct GrainLaw { vec4 slipLoss, forceEnergy; real normalLossPower; bool sliding; };
GrainLaw grainLaw(vec3 n, real depth, real area, vec3 rv, vec3 elastic, real kn, real kt, real mu, real viscosity,
                  real dt) {
    GrainLaw value{{0, 0, 0, 0}, {0, 0, 0, 0}, 0, false};
    elastic = elastic + (rv - n * dot(rv, n)) * dt;
    vec3 trial = elastic;
    NormalResponse response = normalResponse(depth, area, dot(rv, n), kn, viscosity, 0.5f);
    real fn = response.force;
    value.normalLossPower = response.lossPower;
    vec3 ft = -0.5f * kt * area * elastic;
    real magnitude = length(ft);
    if (magnitude > mu * fn && magnitude > 0) {
        ft = ft * (mu * fn / magnitude);
        elastic = -ft / (0.5f * kt * area);
        value.sliding = true;
    }
    value.slipLoss = f4(elastic, mx(0.0f, -dot(ft, trial - elastic)));
    value.forceEnergy = f4(fn * n + ft, 0.25f * area * (kn * depth * depth + kt * dot(elastic, elastic)));
    return value;
}
// solver.slang:697-701
void clearContactStorage(R& r, uint32_t id) {
    if (id < r.c.hashSize) r.hash[id] = EMPTY;
    if (id < r.c.N) r.heads[id] = EMPTY;
}
inline uint32_t activeContacts(R& r) { return r.control[2] < r.c.contactCapacity ? r.control[2] : r.c.contactCapacity; }
// solver.slang:702-749
void resolveContacts(R& r, uint32_t id) {
    if (id >= activeContacts(r) || r.control[0] != 0) return;
    uint4 key = r.meta[id];
    uint32_t i = key.x, j = key.y;
    vec3 n = xyz(r.normalArea[id]);
    bool wall = j >= r.c.N;
    real viscosity = r.c.normalViscosity;
    if (wall) viscosity = r.wallMaterial[j - r.c.N].w;
    vec3 wi = viscosity > 0 ? xyz(r.forceOmega[i]) : omega(r, i), wj{0, 0, 0};
    if (!wall) wj = viscosity > 0 ? xyz(r.forceOmega[j]) : omega(r, j);
    vec3 elastic{0, 0, 0};
    uint32_t slot = hashKey(r, key);
    if (r.c.historyStep != 0) {
        for (uint32_t probe = 0; probe < r.c.hashSize; ++probe) {
            uint32_t old = r.oldHash[slot];
            if (old == EMPTY) break;
            uint4 k2 = r.oldMeta[old];
            if (k2.x == key.x && k2.y == key.y && k2.z == key.z) {
                elastic = transported(xyz(r.oldSlip[old]), xyz(r.oldNormal[old]), n, 0.5f * dot(wi + wj, n) * r.c.dt);
                break;
            }
            slot = (slot + 1) & (r.c.hashSize - 1);
        }
    }
    vec3 arm = xyz(r.pointDepth[id]);
    if (wall) {
        uint32_t w = j - r.c.N;
        vec4 material = r.wallMaterial[w];
        vec3 v = viscosity > 0 ? xyz(r.forceVelocity[i]) : xyz(r.velocity[i]) + xyz(r.velocityRemainder[i]);
        vec3 rv = v + cross(wi, arm) - xyz(r.wallVelocity[w]);
        PlaneResponse response = planeViscousResponse(n, -r.pointDepth[id].w, r.normalArea[id].w, rv, elastic,
                                                      material.x, material.y, material.z, material.w, r.c.dt);
        r.slip[id] = response.slipLoss;
        r.contactForce[id] = response.forceEnergy;
        r.normalLossPower[id] = response.normalLossPower;
        vec4 fe = response.forceEnergy;
        if (!std::isfinite(fe.x) || !std::isfinite(fe.y) || !std::isfinite(fe.z) || !std::isfinite(fe.w) ||
            !std::isfinite(response.normalLossPower)) { fail(r, 512); return; }
        if (response.sliding) r.control[6]++;
        uint32_t oldHead = r.heads[i];
        r.heads[i] = 2 * id;
        r.next[2 * id] = oldHead;
        r.next[2 * id + 1] = EMPTY;
        return;
    }
    vec3 branch = centerBranch(r, i, j);
    vec3 translation = xyz(r.velocity[i]) - xyz(r.velocity[j]);
    if (viscosity > 0) translation = xyz(r.forceVelocity[i]) - xyz(r.forceVelocity[j]);
    vec3 rv = translation - xyz(r.cell[1]) * branch + cross(wi, arm) - cross(wj, arm - branch);
    real area = r.normalArea[id].w, depth = r.pointDepth[id].w;
    GrainLaw law = grainLaw(n, depth, area, rv, elastic, r.c.kn, r.c.kt, r.c.mu, viscosity, r.c.dt);
    r.normalLossPower[id] = law.normalLossPower;
    if (law.sliding) r.control[6]++;
    r.slip[id] = law.slipLoss;
    vec4 cf = law.forceEnergy;
    r.contactForce[id] = cf;
    if (!std::isfinite(cf.x) || !std::isfinite(cf.y) || !std::isfinite(cf.z) || !std::isfinite(cf.w) ||
        !std::isfinite(law.normalLossPower)) { fail(r, 512); return; }
    uint32_t oldHead = r.heads[i];
    r.heads[i] = 2 * id;
    r.next[2 * id] = oldHead;
    oldHead = r.heads[j];
    r.heads[j] = 2 * id + 1;
    r.next[2 * id + 1] = oldHead;
}
// solver.slang:750-759
void buildHistoryHash(R& r, uint32_t id) {
    if (id >= activeContacts(r) || r.control[0] != 0) return;
    uint32_t slot = hashKey(r, r.meta[id]);
    for (uint32_t probe = 0; probe < r.c.hashSize; ++probe) {
        if (r.hash[slot] == EMPTY) { r.hash[slot] = id; return; }
        slot = (slot + 1) & (r.c.hashSize - 1);
    }
    fail(r, 64);
}
// solver.slang:760-811
void gather(R& r, uint32_t id) {
    if (id >= r.c.N || r.control[0] != 0) return;
    vec3 f{0, 0, 0}, t{0, 0, 0}, fLow{0, 0, 0}, tLow{0, 0, 0};
    vec3 stress0{0, 0, 0}, stress1{0, 0, 0}, stress2{0, 0, 0};
    real energy = 0, denom = 0, maxDepth = 0, dissipation = 0, normalPower = 0;
    real stiffnessRate = 0, viscousRate = 0;
    vec3 one{1, 1, 1};
    real inverseInertia = mx(mx(dot(abs3(xyz(r.invI[3 * id])), one), dot(abs3(xyz(r.invI[3 * id + 1])), one)),
                              dot(abs3(xyz(r.invI[3 * id + 2])), one));
    uint32_t entry = r.heads[id], visited = 0;
    while (entry != EMPTY) {
        if (visited++ > 2 * r.c.contactCapacity) { fail(r, 128); return; }
        uint32_t contact = entry / 2;
        bool source = (entry & 1) == 0;
        uint4 key = r.meta[contact];
        vec3 force = xyz(r.contactForce[contact]);
        vec3 arm = xyz(r.pointDepth[contact]);
        if (r.c.activeTimestep != 0) {
            bool wall = key.y >= r.c.N;
            vec3 localArm = source ? arm : arm - centerBranch(r, key.x, key.y);
            real mobility = 1.0f / r.body[id].y + dot(localArm, localArm) * inverseInertia;
            vec4 material{r.c.kn, r.c.kt, r.c.mu, r.c.normalViscosity};
            if (wall) material = r.wallMaterial[key.y - r.c.N];
            real area = r.normalArea[contact].w * (wall ? 1.0f : 0.5f);
            real coupling = wall ? 1.0f : 2.0f;
            stiffnessRate = stiffnessRate + coupling * area * (material.x * (1.0f + material.z) + material.y) * mobility;
            viscousRate = viscousRate + coupling * area * material.w * (1.0f + material.z) * mobility;
        }
        if (key.y >= r.c.N) {
            compensated3(f, fLow, force);
            compensated3(t, tLow, cross(arm, force));
            stress0 = stress0 - force.x * arm;
            stress1 = stress1 - force.y * arm;
            stress2 = stress2 - force.z * arm;
            energy = energy + r.contactForce[contact].w;
            denom = denom + length(force);
            maxDepth = mx(maxDepth, r.pointDepth[contact].w / r.body[key.x].w);
            dissipation = dissipation + r.slip[contact].w;
            normalPower = normalPower + r.normalLossPower[contact];
            entry = r.next[entry];
            continue;
        }
        vec3 branch = centerBranch(r, key.x, key.y);
        compensated3(f, fLow, source ? force : -force);
        compensated3(t, tLow, source ? cross(arm, force) : cross(arm - branch, -force));
        stress0 = stress0 - 0.5f * force.x * branch;
        stress1 = stress1 - 0.5f * force.y * branch;
        stress2 = stress2 - 0.5f * force.z * branch;
        energy = energy + 0.5f * r.contactForce[contact].w;
        denom = denom + length(force);
        maxDepth = mx(maxDepth, r.pointDepth[contact].w / mn(r.body[key.x].w, r.body[key.y].w));
        dissipation = dissipation + 0.5f * r.slip[contact].w;
        normalPower = normalPower + 0.5f * r.normalLossPower[contact];
        entry = r.next[entry];
    }
    f = f + fLow;
    t = t + tLow;
    r.timestepRows[id] = vec4{stiffnessRate, viscousRate, 0, 0};
    vec4 normalState = r.normalDamping[id];
    normalState.z = normalPower;
    r.normalDamping[id] = normalState;
    r.force[id] = f4(f, maxDepth);
    r.torque[id] = f4(t, dissipation);
    r.particleStress[3 * id] = f4(stress0, 0);
    r.particleStress[3 * id + 1] = f4(stress1, 0);
    r.particleStress[3 * id + 2] = f4(stress2, 0);
    vec3 v = xyz(r.velocity[id]);
    real kinetic = 0.5f * (r.body[id].y * dot(v, v) + dot(xyz(r.momentum[id]), omega(r, id)));
    r.particleDiagnostic[id] = vec4{kinetic, energy, length(f), denom};
    accumulate(r, id, vec4{dissipation, 0, 0, 0});
}
// solver.slang:815-832
void checkContactTimestep(R& r, uint32_t id) {
    if (id >= r.c.N || r.control[0] != 0 || r.c.dt == 0) return;
    real dt = r.c.dt;
    real rx = r.timestepRows[id].x, ry = r.timestepRows[id].y;
    vec3 v = xyz(r.velocity[id]) + xyz(r.velocityRemainder[id]);
    real speed = length(v) + dt * length(xyz(r.force[id])) / r.body[id].y;
    vec3 one{1, 1, 1};
    real inverseInertia = mx(mx(dot(abs3(xyz(r.invI[3 * id])), one), dot(abs3(xyz(r.invI[3 * id + 1])), one)),
                              dot(abs3(xyz(r.invI[3 * id + 2])), one));
    real spin = inverseInertia * (length(xyz(r.momentum[id]) + xyz(r.momentumRemainder[id])) + dt * length(xyz(r.torque[id])));
    real wallSpeed = 0;
    for (uint32_t w = 0; w < r.c.wallCount; ++w) wallSpeed = mx(wallSpeed, length(xyz(r.wallVelocity[w])));
    real motion = dt * (speed + r.body[id].z * spin + wallSpeed);
    bool finite = std::isfinite(rx) && std::isfinite(ry) && std::isfinite(motion) && std::isfinite(spin);
    if (!finite) { fail(r, 512); return; }
    vec3 rate = abs3(xyz(r.cell[1]));
    if (dt * std::sqrt(rx) > 0.1f || dt * ry > 0.1f || dt * spin > 0.01f || motion > 0.25f * r.c.skin ||
        rate.x * dt > 0.01f || rate.y * dt > 0.01f || rate.z * dt > 0.01f) fail(r, 8192);
}
// solver.slang:922-936
void diagnosticRows(R& r, uint32_t id) {
    if (id >= r.c.N) return;
    vec3 v = xyz(r.velocity[id]);
    real m = r.body[id].y;
    real kinetic = 0.5f * (m * dot(v, v) + dot(xyz(r.momentum[id]), omega(r, id)));
    vec4* row = r.diagnosticRows + 8 * size_t(id);
    row[0] = f4(xyz(r.particleStress[3 * id]), kinetic);
    row[1] = f4(xyz(r.particleStress[3 * id + 1]), r.particleDiagnostic[id].y);
    row[2] = f4(xyz(r.particleStress[3 * id + 2]), length(xyz(r.force[id])));
    row[3] = f4(m * v.x * v, r.particleDiagnostic[id].w);
    row[4] = f4(m * v.y * v, r.force[id].w);
    row[5] = f4(m * v.z * v, r.torque[id].w);
    row[6] = r.accumulated[id];
    vec4 ns = r.normalDamping[id];
    row[7] = vec4{ns.x + ns.y, ns.z, 0, 0};
}
// solver.slang:938-947
void fabricRows(R& r, uint32_t id) {
    if (id >= r.c.pairCapacity) return;
    vec4 a{0, 0, 0, 0}, b{0, 0, 0, 0};
    if (id < r.control[1] && r.contactCounts[id] > 0) {
        uint2 ij = r.pairs[id];
        vec3 d = centerBranch(r, ij.x, ij.y);
        vec3 n = d * (1.0f / std::sqrt(dot(d, d)));
        a = vec4{n.x * n.x, n.y * n.y, n.z * n.z, n.x * n.y};
        b = vec4{n.x * n.z, n.y * n.z, 1, 0};
    }
    r.fabricRows[2 * id] = a;
    r.fabricRows[2 * id + 1] = b;
}

}  // namespace

extern "C" int oracle_dispatch(const char* name, uint32_t count, void** buffers, const uint64_t* bytes,
                               const double* values, uint32_t nvalues) {
    (void)bytes;
    R r;
    bind(r, buffers, values);
    std::string_view k(name);
    auto each = [&](auto fn) { for (uint32_t id = 0; id < count; ++id) fn(r, id); };
    if (k == "beginStep") each(beginStep);
    else if (k == "advanceCell") advanceCell(r);
    else if (k == "checkRebuild") each(checkRebuild);
    else if (k == "finishStep") each(finishStep);
    else if (k == "captureContactKinematics") each(captureContactKinematics);
    else if (k == "clearBins") each(clearBins);
    else if (k == "fillBins") each(fillBins);
    else if (k == "countPairs") each(countPairs);
    else if (k == "scanPairs") scanPairs(r);
    else if (k == "emitPairs") each(emitPairs);
    else if (k == "resetMeshContacts") each(resetMeshContacts);
    else if (k == "prepareMeshPairs") each(prepareMeshPairs);
    else if (k == "collectMeshFrontiers") collectParallel(r, count, nvalues > 25 ? uint32_t(r.uni[0]) : 1u);
    else if (k == "exhaustiveContacts") exhaustiveContacts(r);
    else if (k == "countContacts") each(countContacts);
    else if (k == "scanContacts") scanContacts(r);
    else if (k == "contactTotal") contactTotal(r);
    else if (k == "emitContacts") each(emitContacts);
    else if (k == "clearContactStorage") each(clearContactStorage);
    else if (k == "resolveContacts") each(resolveContacts);
    else if (k == "buildHistoryHash") each(buildHistoryHash);
    else if (k == "gather") each(gather);
    else if (k == "checkContactTimestep") each(checkContactTimestep);
    else if (k == "collectWallContacts") each(collectWallContacts);
    else if (k == "gatherWallRows") each(gatherWallRows);
    else if (k == "advanceWalls") advanceWalls(r);
    else if (k == "refreshWallPower") each(refreshWallPower);
    else if (k == "diagnosticRows") each(diagnosticRows);
    else if (k == "fabricRows") each(fabricRows);
    // Probes (entry-point uniforms after the Config scalars).
    else if (k == "meshProbe") {  // solver.slang:253-257: uniform shape; points, result
        uint32_t shape = uint32_t(r.uni[1]);
        vec4* points = static_cast<vec4*>(r.extra[0]);
        vec4* result = static_cast<vec4*>(r.extra[1]);
        for (uint32_t id = 0; id < count; ++id) result[id] = meshDistance(r, shape, xyz(points[id]), false);
    } else if (k == "meshCullProbe") {  // solver.slang:314-318
        uint32_t shape = uint32_t(r.uni[1]);
        vec4* points = static_cast<vec4*>(r.extra[0]);
        uint32_t* result = static_cast<uint32_t*>(r.extra[1]);
        for (uint32_t id = 0; id < count; ++id) result[id] = meshMayContain(r, shape, xyz(points[id])) ? 1 : 0;
    } else if (k == "meshClusterProbe") {  // solver.slang:306-313: src, dst
        uint32_t src = uint32_t(r.uni[1]), dst = uint32_t(r.uni[2]);
        uint32_t* result = static_cast<uint32_t*>(r.extra[0]);
        for (uint32_t id = 0; id < count; ++id)
            result[id] = meshClusterMayContact(r, src, dst, r.meshClusterInfo[r.shapeId[src]].x + id) ? 1 : 0;
    } else if (k == "meshPairBoundsProbe") {  // solver.slang:418-424: direction, first
        uint32_t direction = uint32_t(r.uni[1]), first = uint32_t(r.uni[2]);
        vec4* result = static_cast<vec4*>(r.extra[0]);
        for (uint32_t id = 0; id < count; ++id) {
            vec3 lo, hi;
            meshPairBounds(r, direction, first + id, lo, hi);
            result[2 * id] = f4(lo, 0);
            result[2 * id + 1] = f4(hi, 0);
        }
    } else if (k == "planeProbe") {  // plane.slang:44-64: N; normal; offset, kn, kt, mu, dt
        vec3 normal{real(r.uni[1]), real(r.uni[2]), real(r.uni[3])};
        real offset = real(r.uni[4]), kn = real(r.uni[5]), kt = real(r.uni[6]), mu = real(r.uni[7]);
        real dt = real(r.uni[8]);
        vec4* pointArea = static_cast<vec4*>(r.extra[0]);
        vec4* relativeVelocity = static_cast<vec4*>(r.extra[1]);
        vec4* oldSlipActive = static_cast<vec4*>(r.extra[2]);
        vec4* forceEnergy = static_cast<vec4*>(r.extra[3]);
        vec4* slipLoss = static_cast<vec4*>(r.extra[4]);
        vec4* torqueActive = static_cast<vec4*>(r.extra[5]);
        for (uint32_t id = 0; id < count; ++id) {
            vec4 point = pointArea[id];
            real phi = dot(normal, xyz(point)) - offset;
            vec3 old = oldSlipActive[id].w != 0 ? xyz(oldSlipActive[id]) : vec3{0, 0, 0};
            PlaneResponse value = planeViscousResponse(normal, phi, point.w, xyz(relativeVelocity[id]), old, kn, kt,
                                                       mu, 0.0f, dt);
            forceEnergy[id] = value.forceEnergy;
            slipLoss[id] = value.slipLoss;
            torqueActive[id] = f4(cross(xyz(point), xyz(value.forceEnergy)), phi < 0 ? 1.0f : 0.0f);
        }
    } else if (k == "grainLawProbe") {  // grainLaw per contact: N; kn, kt, mu, viscosity, dt
        real kn = real(r.uni[1]), kt = real(r.uni[2]), mu = real(r.uni[3]), viscosity = real(r.uni[4]);
        real dt = real(r.uni[5]);
        vec4* normalDepth = static_cast<vec4*>(r.extra[0]);
        vec4* slipArea = static_cast<vec4*>(r.extra[1]);
        vec4* velocity = static_cast<vec4*>(r.extra[2]);
        vec4* forceEnergy = static_cast<vec4*>(r.extra[3]);
        vec4* slipLoss = static_cast<vec4*>(r.extra[4]);
        for (uint32_t id = 0; id < count; ++id) {
            GrainLaw v = grainLaw(xyz(normalDepth[id]), normalDepth[id].w, slipArea[id].w, xyz(velocity[id]),
                                  xyz(slipArea[id]), kn, kt, mu, viscosity, dt);
            forceEnergy[id] = v.forceEnergy;
            slipLoss[id] = v.slipLoss;
        }
    } else if (k == "transportProbe") {  // transported per contact: slip and spin, old normal, new normal
        vec4* slipSpin = static_cast<vec4*>(r.extra[0]);
        vec4* oldNormal = static_cast<vec4*>(r.extra[1]);
        vec4* newNormal = static_cast<vec4*>(r.extra[2]);
        vec4* result = static_cast<vec4*>(r.extra[3]);
        for (uint32_t id = 0; id < count; ++id)
            result[id] = f4(transported(xyz(slipSpin[id]), xyz(oldNormal[id]), xyz(newNormal[id]), slipSpin[id].w), 0);
    } else if (k == "normalProbe") {  // normal.slang:166-174: stiffness, viscosity, weight
        real stiffness = real(r.uni[1]), viscosity = real(r.uni[2]), weight = real(r.uni[3]);
        vec4* input = static_cast<vec4*>(r.extra[0]);
        vec4* output = static_cast<vec4*>(r.extra[1]);
        for (uint32_t id = 0; id < count; ++id) {
            NormalResponse v = normalResponse(input[id].x, input[id].y, input[id].z, stiffness, viscosity, weight);
            output[id] = vec4{v.force, v.lossPower, 0, 0};
        }
    } else return -1;
    return 0;
}
