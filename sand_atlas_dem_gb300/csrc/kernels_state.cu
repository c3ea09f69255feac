// Per-grain state kernels: kick-drift-kick integrator with affine periodic
// cell streaming, cell update, Verlet rebuild trigger, timestep guard and the
// diagnostic rows with their fixed-order tree reduction.
//
// Each kernel is one thread per grain (HBM-bound: ~0.5 KB of float4 state per
// grain and step) and restates the arithmetic of the reference kernel named
// beside it, in the same FP32 operation order.
#include "dem_device.cuh"
#include "launch.h"

namespace sdg {

// solver.slang:159-163
__device__ __forceinline__ float rotationalEnergy(const Res& r, uint32_t i, float4 q, f3 l) {
    f3 b = qinv(q, l);
    f3 w = {dot(xyz(r.invI[3 * i]), b), dot(xyz(r.invI[3 * i + 1]), b), dot(xyz(r.invI[3 * i + 2]), b)};
    return __fmul_rn(0.5f, dot(b, w));
}
// solver.slang:164-169
__device__ __forceinline__ void accumulateNormalLoss(const Res& r, uint32_t id, float dt) {
    float4 value = r.normalDamping[id];
    f3 high = mk(value.x, 0.f, 0.f), low = mk(value.y, 0.f, 0.f);
    compensated3(high, low, mk(__fmul_rn(value.z, dt), 0.f, 0.f));
    value.x = high.x;
    value.y = low.x;
    r.normalDamping[id] = value;
}
// solver.slang:176-180 (reads the velocity buffer as stored)
__device__ __forceinline__ float cellPower(const Res& r, uint32_t i) {
    f3 diagonal = mk(r.particleStress[3 * i].x, r.particleStress[3 * i + 1].y, r.particleStress[3 * i + 2].z);
    f3 v = xyz(r.velocity[i]);
    return -dot(diagonal + (r.body[i].y * v) * v, xyz(r.cell[3 * specimenOf(r, i) + 1]));
}
// solver.slang:130-134
__device__ __forceinline__ void accumulate(const Res& r, uint32_t id, float4 inc) {
    float4 high = r.accumulated[id], low = r.accumulatedRemainder[id];
    compensated4(high, low, inc);
    r.accumulated[id] = high;
    r.accumulatedRemainder[id] = low;
}
// Half kick, drag and its losses, shared by beginStep and finishStep.
__device__ __forceinline__ void halfKick(const Res& r, const Config& c, uint32_t id, f3& v, f3& vl, f3& l, f3& ll) {
    float dt = c.dt, m = r.body[id].y;
    float hdt = __fmul_rn(0.5f, dt);
    accumulateNormalLoss(r, id, hdt);
    v = xyz(r.velocity[id]);
    vl = xyz(r.velocityRemainder[id]);
    l = xyz(r.momentum[id]);
    ll = xyz(r.momentumRemainder[id]);
    compensated3(v, vl, (hdt * xyz(r.force[id])) / m);
    compensated3(l, ll, hdt * xyz(r.torque[id]));
    f3 vs = v + vl;
    float loss = __fmul_rn(-expm1Stable(__fmul_rn(-c.drag, dt)),
                           __fadd_rn(__fmul_rn(__fmul_rn(0.5f, m), dot(vs, vs)),
                                     rotationalEnergy(r, id, r.rotation[id], l + ll)));
    float cp = __fmul_rn(hdt, cellPower(r, id));
    accumulate(r, id, make_float4(0.f, loss, cp, wallStepWork(r, c, id, hdt)));
    float damping = expm1Stable(__fmul_rn(__fmul_rn(-0.5f, c.drag), dt));
    compensated3(v, vl, damping * (v + vl));
    compensated3(l, ll, damping * (l + ll));
}

// solver.slang:858-888 (+ captureContactKinematics :170-175 when viscous)
__global__ void k_beginStep(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t id = gtid();
    if (id >= c.N || r.control[0] != 0) return;
    float dt = c.dt;
    uint32_t sp = specimenOf(r, id);
    f3 rate = xyz(r.cell[3 * sp + 1]);
    f3 v, vl, l, ll;
    halfKick(r, c, id, v, vl, l, ll);
    r.momentum[id] = w4(l, 0.f);
    r.momentumRemainder[id] = w4(ll, 0.f);
    float4 q = r.rotation[id], ql = r.rotationRemainder[id];
    f3 lt = l + ll;
    f3 w = omega(r, id, q, lt);
    float4 mid = normalize4(add4(q, rotationIncrement(w, __fmul_rn(0.5f, dt), q)));
    w = omega(r, id, mid, lt);
    compensated4(q, ql, rotationIncrement(w, dt, q));
    if (fabsf(__fsub_rn(dot4(q, q), 1.0f)) > 2e-6f) {
        q = normalize4(q);
        ql = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    r.rotation[id] = q;
    r.rotationRemainder[id] = ql;
    f3 logarithm = xyz(r.cellLog[2 * sp]), residual = xyz(r.cellLog[2 * sp + 1]);
    compensated3(logarithm, residual, rate * dt);
    f3 box = xyz(r.cell[3 * sp + 2]) * exp3(logarithm);
    f3 p = xyz(r.position[id]), pl = xyz(r.positionRemainder[id]);
    compensated3(p, pl, expm1Stable3(rate * dt) * (p + pl) + dt * (v + vl));
    if (!finite3(p) || !finite3(pl)) { fail(r, F_NONFINITE); return; }
    if (c.periodic != 0) {
        p = p - mk(floorf(__fdiv_rn(p.x, box.x)), floorf(__fdiv_rn(p.y, box.y)), floorf(__fdiv_rn(p.z, box.z))) * box;
    } else if (__fadd_rn(p.x, pl.x) < 0 || __fadd_rn(p.y, pl.y) < 0 || __fadd_rn(p.z, pl.z) < 0 ||
               __fadd_rn(__fsub_rn(p.x, box.x), pl.x) >= 0 || __fadd_rn(__fsub_rn(p.y, box.y), pl.y) >= 0 ||
               __fadd_rn(__fsub_rn(p.z, box.z), pl.z) >= 0) {
        fail(r, F_ESCAPE);
        return;
    }
    r.position[id] = w4(p, 0.f);
    r.positionRemainder[id] = w4(pl, 0.f);
    compensated3(v, vl, expm1Stable3((-rate) * dt) * (v + vl));
    r.velocity[id] = w4(v, 0.f);
    r.velocityRemainder[id] = w4(vl, 0.f);
    if (c.viscousCapture) {
        r.forceVelocity[id] = w4(v + vl, 0.f);
        r.forceOmega[id] = w4(omega(r, id, q, lt), 0.f);
    }
}

// solver.slang:170-175 (stand-alone form, used by initialize/restore paths)
__global__ void k_captureContactKinematics(const __grid_constant__ Params P) {
    const Res& r = P.r;
    uint32_t id = gtid();
    if (id >= P.c.N || r.control[0] != 0) return;
    r.forceVelocity[id] = w4(xyz(r.velocity[id]) + xyz(r.velocityRemainder[id]), 0.f);
    r.forceOmega[id] = w4(omegaOf(r, id), 0.f);
}

// solver.slang:889-897, one thread per specimen.
__global__ void k_advanceCell(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t sp = gtid();
    if (sp >= c.specimens || r.control[0] != 0) return;
    f3 logarithm = xyz(r.cellLog[2 * sp]), residual = xyz(r.cellLog[2 * sp + 1]);
    compensated3(logarithm, residual, xyz(r.cell[3 * sp + 1]) * c.dt);
    r.cellLog[2 * sp] = w4(logarithm, 0.f);
    r.cellLog[2 * sp + 1] = w4(residual, 0.f);
    float4 cell = w4(xyz(r.cell[3 * sp + 2]) * exp3(logarithm), 0.f);
    r.cell[3 * sp] = cell;
    if (sp == 0) r.control[4] = 0;
    if (c.periodic != 0 && r.referenceCell[2 * sp + 1].w >= __fmul_rn(0.5f, mn(cell.x, mn(cell.y, cell.z))))
        fail(r, F_IMAGE);
}

// solver.slang:898-904
__global__ void k_checkRebuild(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t id = gtid();
    if (id >= c.N) return;
    f3 d = (xyz(r.position[id]) - xyz(r.referencePosition[id])) +
           (xyz(r.positionRemainder[id]) - xyz(r.referencePositionRemainder[id]));
    uint32_t sp = specimenOf(r, id);
    if (c.periodic != 0) {
        f3 box = xyz(r.cell[3 * sp]);
        d = d - mk(floorf(__fadd_rn(__fdiv_rn(d.x, box.x), 0.5f)), floorf(__fadd_rn(__fdiv_rn(d.y, box.y), 0.5f)),
                   floorf(__fadd_rn(__fdiv_rn(d.z, box.z), 0.5f))) * box;
    }
    float deformation = length(xyz(r.cell[3 * sp]) - xyz(r.referenceCell[2 * sp]));
    if (__fadd_rn(length(d), deformation) > __fmul_rn(0.5f, c.skin)) atomicOr(&r.control[4], 1u);
}

// solver.slang:905-920
__global__ void k_finishStep(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t id = gtid();
    if (id >= c.N || r.control[0] != 0) return;
    f3 v, vl, l, ll;
    halfKick(r, c, id, v, vl, l, ll);
    if (!finite3(v) || !finite3(l)) { fail(r, F_NONFINITE); return; }
    r.velocity[id] = w4(v, 0.f);
    r.velocityRemainder[id] = w4(vl, 0.f);
    r.momentum[id] = w4(l, 0.f);
    r.momentumRemainder[id] = w4(ll, 0.f);
}

__device__ __forceinline__ float inverseInertiaBound(const Res& r, uint32_t id) {
    f3 one = mk(1.f, 1.f, 1.f);
    return mx(mx(dot(abs3(xyz(r.invI[3 * id])), one), dot(abs3(xyz(r.invI[3 * id + 1])), one)),
              dot(abs3(xyz(r.invI[3 * id + 2])), one));
}

// solver.slang:815-832
__global__ void k_checkContactTimestep(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t id = gtid();
    if (id >= c.N || r.control[0] != 0 || c.dt == 0) return;
    float dt = c.dt;
    float4 rates = r.timestepRows[id];
    f3 v = xyz(r.velocity[id]) + xyz(r.velocityRemainder[id]);
    float speed = __fadd_rn(length(v), __fdiv_rn(__fmul_rn(dt, length(xyz(r.force[id]))), r.body[id].y));
    float inverseInertia = inverseInertiaBound(r, id);
    float spin = __fmul_rn(inverseInertia, __fadd_rn(length(xyz(r.momentum[id]) + xyz(r.momentumRemainder[id])),
                                                     __fmul_rn(dt, length(xyz(r.torque[id])))));
    float wallSpeed = 0.f;
    for (uint32_t w = 0; w < c.wallCount; ++w) wallSpeed = mx(wallSpeed, length(xyz(r.wallVelocity[w])));
    float motion = __fmul_rn(dt, __fadd_rn(__fadd_rn(speed, __fmul_rn(r.body[id].z, spin)), wallSpeed));
    bool finite = isfinite(rates.x) && isfinite(rates.y) && isfinite(motion) && isfinite(spin);
    if (!finite) { fail(r, F_NONFINITE); return; }
    f3 rate = abs3(xyz(r.cell[3 * specimenOf(r, id) + 1]));
    if (__fmul_rn(dt, __fsqrt_rn(rates.x)) > 0.1f || __fmul_rn(dt, rates.y) > 0.1f || __fmul_rn(dt, spin) > 0.01f ||
        motion > __fmul_rn(0.25f, c.skin) || __fmul_rn(rate.x, dt) > 0.01f || __fmul_rn(rate.y, dt) > 0.01f ||
        __fmul_rn(rate.z, dt) > 0.01f)
        fail(r, F_TIMESTEP);
}

// solver.slang:922-936
__global__ void k_diagnosticRows(const __grid_constant__ Params P) {
    const Res& r = P.r;
    uint32_t id = gtid();
    if (id >= P.c.N) return;
    f3 v = xyz(r.velocity[id]);
    float m = r.body[id].y;
    float kinetic = __fmul_rn(0.5f, __fadd_rn(__fmul_rn(m, dot(v, v)), dot(xyz(r.momentum[id]), omegaOf(r, id))));
    float4* row = r.diagnosticRows + 8 * size_t(id);
    row[0] = w4(xyz(r.particleStress[3 * id]), kinetic);
    row[1] = w4(xyz(r.particleStress[3 * id + 1]), r.particleDiagnostic[id].y);
    row[2] = w4(xyz(r.particleStress[3 * id + 2]), length(xyz(r.force[id])));
    row[3] = w4(__fmul_rn(m, v.x) * v, r.particleDiagnostic[id].w);
    row[4] = w4(__fmul_rn(m, v.y) * v, r.force[id].w);
    row[5] = w4(__fmul_rn(m, v.z) * v, r.torque[id].w);
    row[6] = r.accumulated[id];
    float4 ns = r.normalDamping[id];
    row[7] = make_float4(__fadd_rn(ns.x, ns.y), ns.z, 0.f, 0.f);
}

// solver.slang:938-947
__global__ void k_fabricRows(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t id = gtid();
    if (id >= c.pairCapacity) return;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (id < r.control[1] && r.contactCounts[id] > 0) {
        uint2 ij = r.pairs[id];
        f3 d = centerBranch64(r, c, ij.x, ij.y);
        f3 n = d * __fdiv_rn(1.0f, __fsqrt_rn(dot(d, d)));
        a = make_float4(__fmul_rn(n.x, n.x), __fmul_rn(n.y, n.y), __fmul_rn(n.z, n.z), __fmul_rn(n.x, n.y));
        b = make_float4(__fmul_rn(n.x, n.z), __fmul_rn(n.y, n.z), 1.f, 0.f);
    }
    r.fabricRows[2 * id] = a;
    r.fabricRows[2 * id + 1] = b;
}

// diagnostic.slang:3-28: per 256-row group, values[lane] += values[lane+step]
// for step = 128..1; (maxRow, 3) reduces with max instead of sum.
__global__ void k_reduceRows(const float4* input, float4* output, uint32_t n, uint32_t rows, int maxRow) {
    __shared__ float4 values[256];
    uint32_t lane = threadIdx.x, id = blockIdx.x * 256 + lane;
    for (uint32_t row = 0; row < rows; ++row) {
        values[lane] = id < n ? input[size_t(id) * rows + row] : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        for (uint32_t step = 128; step > 0; step /= 2) {
            if (lane < step) {
                float4 a = values[lane], b = values[lane + step];
                float4 s = add4(a, b);
                if (int(row) == maxRow) s.w = mx(a.w, b.w);
                values[lane] = s;
            }
            __syncthreads();
        }
        if (lane == 0) output[size_t(blockIdx.x) * rows + row] = values[0];
        __syncthreads();
    }
}

// solver.slang:669-687: the planes advance along their normals by
// velocity . normal x dt (compensated offsets); with a boundary box, its six
// planes must keep a positive gap inside the domain.  One thread.
__global__ void k_advanceWalls(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    if (gtid() != 0 || r.control[0] != 0) return;
    for (uint32_t w = 0; w < c.wallCount; ++w) {
        float4 plane = r.wallPlane[w], residual = r.wallRemainder[w];
        float inc = __fmul_rn(dot(xyz(plane), xyz(r.wallVelocity[w])), c.dt);
        float y = __fadd_rn(inc, residual.w);
        float high = __fadd_rn(plane.w, y);
        float low = __fsub_rn(y, __fsub_rn(high, plane.w));
        plane.w = high;
        residual.w = low;
        if (!isfinite(high) || !isfinite(low)) { fail(r, F_NONFINITE); return; }
        r.wallPlane[w] = plane;
        r.wallRemainder[w] = residual;
    }
    if (c.wallBoxEnabled != 0) {
        float4 box = r.cell[0];
        for (uint32_t axis = 0; axis < 3; ++axis) {
            uint32_t lo = r.wallBoxIds[2 * axis], hi = r.wallBoxIds[2 * axis + 1];
            float low = __fadd_rn(r.wallPlane[lo].w, r.wallRemainder[lo].w);
            float high = -__fadd_rn(r.wallPlane[hi].w, r.wallRemainder[hi].w);
            float extent = axis == 0 ? box.x : axis == 1 ? box.y : box.z;
            if (low < 0 || high > extent || high <= low) fail(r, F_BOX);
        }
    }
}
// solver.slang:950-955: wall power of the committed rows at new wall
// velocities (no contact is re-resolved).
__global__ void k_refreshWallPower(const __grid_constant__ Params P) {
    const Res& r = P.r;
    const Config& c = P.c;
    uint32_t total = c.N * c.wallCount;
    for (uint32_t index = gtid(); index < total; index += gstride()) {
        float4 value = r.wallRows[3 * index + 1];
        value.w = -dot(xyz(r.wallRows[3 * index]), xyz(r.wallVelocity[index / c.N]));
        r.wallRows[3 * index + 1] = value;
    }
}
// diagnostic.slang:33-49: per wall, 256-row tree sums of the three
// (wall, grain) rows, the contact count (row 0, w) summed as an integer.
__global__ void k_reduceWallRows(const float4* input, float4* output, uint32_t n, uint32_t outputCount) {
    __shared__ float4 values[256];
    __shared__ uint32_t counts[256];
    uint32_t lane = threadIdx.x, id = blockIdx.x * 256 + lane, wall = blockIdx.y;
    for (uint32_t row = 0; row < 3; ++row) {
        float4 value = id < n ? input[3 * (size_t(wall) * n + id) + row] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (row == 0) {
            counts[lane] = __float_as_uint(value.w);
            value.w = 0.f;
        }
        values[lane] = value;
        __syncthreads();
        for (uint32_t step = 128; step > 0; step /= 2) {
            if (lane < step) {
                values[lane] = add4(values[lane], values[lane + step]);
                if (row == 0) counts[lane] += counts[lane + step];
            }
            __syncthreads();
        }
        if (lane == 0) {
            float4 total = values[0];
            if (row == 0) total.w = __uint_as_float(counts[0]);
            output[3 * (size_t(wall) * outputCount + blockIdx.x) + row] = total;
        }
        __syncthreads();
    }
}

static inline uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

int launch_state(const std::string_view& name, const Params& P, uint32_t count, cudaStream_t s) {
    const uint32_t T = 256;
    uint32_t n = count ? count : 1;
    if (name == "beginStep") k_beginStep<<<blocks(n, T), T, 0, s>>>(P);
    else if (name == "captureContactKinematics") k_captureContactKinematics<<<blocks(n, T), T, 0, s>>>(P);
    else if (name == "advanceCell") k_advanceCell<<<blocks(P.c.specimens, 64), 64, 0, s>>>(P);
    else if (name == "checkRebuild") k_checkRebuild<<<blocks(n, T), T, 0, s>>>(P);
    else if (name == "finishStep") k_finishStep<<<blocks(n, T), T, 0, s>>>(P);
    else if (name == "checkContactTimestep") k_checkContactTimestep<<<blocks(n, T), T, 0, s>>>(P);
    else if (name == "diagnosticRows") k_diagnosticRows<<<blocks(n, T), T, 0, s>>>(P);
    else if (name == "fabricRows") k_fabricRows<<<blocks(n, T), T, 0, s>>>(P);
    else if (name == "advanceWalls") k_advanceWalls<<<1, 32, 0, s>>>(P);
    else if (name == "refreshWallPower") k_refreshWallPower<<<blocks(max(1u, P.c.N * P.c.wallCount), T), T, 0, s>>>(P);
    else return 1;
    return 0;
}

void launch_reduce_rows(const float4* input, float4* output, uint32_t n, uint32_t rows, int maxRow, cudaStream_t s) {
    k_reduceRows<<<blocks(n, 256), 256, 0, s>>>(input, output, n, rows, maxRow);
}

void launch_reduce_wall_rows(const float4* input, float4* output, uint32_t n, uint32_t walls, cudaStream_t s) {
    uint32_t groups = blocks(n, 256);
    k_reduceWallRows<<<dim3(groups, walls), 256, 0, s>>>(input, output, n, groups);
}

}  // namespace sdg
