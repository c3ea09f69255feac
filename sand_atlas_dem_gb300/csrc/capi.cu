// C ABI of the GB300 mesh-surface DEM step (declared in include/sand_dem_gb300.h).
//
// Buffers follow the reference Resources order (solver.slang:20-100, the
// order the reference CPU backend binds in cpu_dispatch, cpu.py:189-300),
// then this backend's extension buffers; values are the reference Config
// scalars (solver.slang:12-19) then the extension values.  Plain pointers and
// sizes only.  Entry points return 0 on success, nonzero on a CUDA or argument
// error (text via sdg_last_error); solver failures are reported in control[0]
// exactly as the reference does.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <string_view>
#include <vector>
#include <cuda_runtime.h>
#include "dem_device.cuh"
#include "launch.h"

namespace sdg {

static thread_local std::string g_error;

void set_last_error(const std::string& what) { g_error = what; }

static int record(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return 0;
    g_error = std::string(where) + ": " + cudaGetErrorString(e);
    return 2;
}

static int unpack(void* const* buffers, const uint64_t* bytes, const double* values, uint32_t nvalues, Params& P) {
    if (!buffers || !values || nvalues < VALUE_COUNT) {
        g_error = "expected " + std::to_string(BUFFER_COUNT) + " buffers and " + std::to_string(VALUE_COUNT) + " values";
        return 1;
    }
    static_assert(sizeof(Res) == BUFFER_COUNT * sizeof(void*), "buffer block");
    std::memcpy(static_cast<void*>(&P.r), buffers, sizeof(Res));
    (void)bytes;
    Config& c = P.c;
    const double* v = values;
    c.activeTimestep = uint32_t(v[0]); c.N = uint32_t(v[1]); c.shapes = uint32_t(v[2]);
    c.pairCapacity = uint32_t(v[3]); c.contactCapacity = uint32_t(v[4]); c.binCapacity = uint32_t(v[5]);
    c.binCount = uint32_t(v[6]); c.bins[0] = uint32_t(v[7]); c.bins[1] = uint32_t(v[8]); c.bins[2] = uint32_t(v[9]);
    c.hashSize = uint32_t(v[10]);
    c.dt = float(v[11]); c.kn = float(v[12]); c.kt = float(v[13]); c.mu = float(v[14]);
    c.normalViscosity = float(v[15]); c.skin = float(v[16]); c.drag = float(v[17]); c.maxOverlap = float(v[18]);
    c.historyStep = uint32_t(v[19]); c.meshGeometry = uint32_t(v[20]); c.periodic = uint32_t(v[21]);
    c.wallCount = uint32_t(v[22]); c.wallBoxEnabled = uint32_t(v[23]); c.sourceSurfaceNormal = uint32_t(v[24]);
    c.leafWords = uint32_t(v[25]); c.candidateCapacity = uint32_t(v[26]); c.viscousCapture = uint32_t(v[27]);
    c.specimens = uint32_t(v[28]);
    c.cullerEnabled = uint32_t(v[29]);
    c.queryBlocksPerSM = uint32_t(v[30]); c.queryWarps = uint32_t(v[31]); c.cullBlocksPerSM = uint32_t(v[32]);
    c.contactBlocksPerSM = uint32_t(v[33]); c.gatherWarps = uint32_t(v[34]); c.walkBlocksPerSM = uint32_t(v[35]);
    c.survivorCapacity = uint32_t(v[36]);
    c.distanceGridEnabled = uint32_t(v[37]);
    c.filterMargin = float(v[38]);
    {
        // meshChildren, meshTriangles, meshNormals, sample (buffer order).
        const int library[4] = {77 + 40, 31, 32, 24};
        for (int k = 0; k < 4; ++k)
            c.library16[k] = bytes ? uint32_t(std::min<uint64_t>(bytes[library[k]] / 16, 0xFFFFFFFFu)) : 0u;
    }
    if (!(c.filterMargin >= 0.0f) || c.filterMargin > 1.0f) {
        g_error = "filter margin must lie in [0, 1] (target shape frame)";
        return 1;
    }
    if (c.queryBlocksPerSM > 32 || c.cullBlocksPerSM > 32 || c.contactBlocksPerSM > 32 || c.gatherWarps > 64 ||
        c.walkBlocksPerSM > 32 ||
        (c.queryWarps != 0 && c.queryWarps != 4 && c.queryWarps != 8)) {
        g_error = "launch shape out of range (CTAs per SM <= 32, query warps 4 or 8, gather warps per SM <= 64)";
        return 1;
    }
    if (c.specimens == 0) { g_error = "at least one specimen required"; return 1; }
    if (c.N == 0) {
        g_error = "the GB300 step needs N > 0";
        return 1;
    }
    if (c.wallCount != 0 && (c.specimens != 1 || c.periodic != 0)) {
        g_error = "planes bound a single nonperiodic specimen";
        return 1;
    }
    // The (wall, grain) items and their three rows are indexed in uint32
    // (item = wall * N + grain, row = 3 * item + k).
    if (uint64_t(c.wallCount) * c.N * 3 > uint64_t(UINT32_MAX)) {
        g_error = "3 x planes x grains must stay below 2^32 (the (wall, grain) row index is 32-bit)";
        return 1;
    }
    if (c.meshGeometry == 0 && c.sourceSurfaceNormal != 0) {
        g_error = "the source-surface normal needs the mesh contact geometry";
        return 1;
    }
    if (bytes) {
        // Capacity cross-checks against the buffer sizes the caller passed.
        if (bytes[48] < uint64_t(c.contactCapacity) * 16 || bytes[45] < uint64_t(c.pairCapacity) * 8 ||
            bytes[2] < uint64_t(c.N) * 16 || bytes[42] < uint64_t(c.binCount) * c.binCapacity * 4 ||
            bytes[77 + 11] < uint64_t(c.candidateCapacity) * 8 ||
            bytes[77 + 10] < uint64_t(2) * c.pairCapacity * c.leafWords * 4 ||
            bytes[77 + 24] < uint64_t(c.survivorCapacity) * 32 || bytes[77 + 35] < uint64_t(c.survivorCapacity) * 8 ||
            bytes[77 + 33] < uint64_t(c.candidateCapacity) * 8 ||
            bytes[77 + 34] < (uint64_t(c.candidateCapacity) + 1) * 4 ||
            bytes[77 + 25] < (uint64_t(c.candidateCapacity) + 1) * 4 ||
            bytes[77 + 36] < (uint64_t(c.survivorCapacity) + 1) * 4 ||
            bytes[77 + 37] < (uint64_t(c.survivorCapacity) + 1) * 4 || bytes[77 + 38] < uint64_t(c.survivorCapacity) * 4 ||
            bytes[77 + 39] < uint64_t(4) * c.pairCapacity * 16 ||
            bytes[77 + 41] < uint64_t(c.shapes) * GRID * GRID * GRID * 4 || bytes[77 + 42] < uint64_t(c.shapes) * 16 ||
            bytes[77 + 43] < uint64_t(c.shapes) * GRID * GRID * GRID * 4 || bytes[77 + 44] < uint64_t(c.N) * 16 ||
            bytes[77 + 45] < uint64_t(c.pairCapacity) * 16 || bytes[77 + 46] < uint64_t(c.pairCapacity) * 8 ||
            bytes[77 + 47] < uint64_t(c.survivorCapacity) * 4 ||
            bytes[77 + 48] < (uint64_t(c.shapes) * WALK_BUCKETS + 1) * 4 ||
            bytes[77 + 49] < (uint64_t(c.shapes) * WALK_BUCKETS + 1) * 4 ||
            (c.meshGeometry == 0 && bytes[77 + 50] < uint64_t(c.pairCapacity) * 32 * 4) ||
            bytes[77 + 51] < uint64_t(c.survivorCapacity) * 16 || bytes[77 + 52] < uint64_t(c.survivorCapacity) * 8 ||
            bytes[77 + 57] < uint64_t(c.survivorCapacity) * 16 || bytes[77 + 58] < uint64_t(c.survivorCapacity) * 8 ||
            (c.wallCount != 0 &&
             (bytes[70] < uint64_t(c.wallCount) * 16 || bytes[71] < uint64_t(c.wallCount) * 16 ||
              bytes[72] < uint64_t(c.wallCount) * 16 || bytes[73] < uint64_t(c.wallCount) * 16 ||
              (c.wallBoxEnabled != 0 && bytes[74] < 6 * 4) ||
              bytes[75] < uint64_t(c.wallCount) * c.N * 48 || bytes[76] < uint64_t(c.wallCount) * c.N * 16 ||
              bytes[77 + 53] < uint64_t(c.wallCount) * c.N * 4 ||
              bytes[77 + 54] < (uint64_t(c.wallCount) * c.N + 1) * 4 ||
              bytes[77 + 55] < (uint64_t(c.wallCount) * c.N + 1) * 4 ||
              bytes[77 + 56] < (uint64_t(c.wallCount) * c.N + 1) * 4))) {
            g_error = "a buffer is smaller than its configured capacity";
            return 1;
        }
    }
    return 0;
}

int unpack_params(void* const* buffers, const uint64_t* bytes, const double* values, uint32_t nvalues,
                  Params& P) {
    return unpack(buffers, bytes, values, nvalues, P);
}

void launch_forces(const Params& P, cudaStream_t s, bool captureKinematics) {
    const Config& c = P.c;
    if (c.normalViscosity > 0 && captureKinematics) launch_state("captureContactKinematics", P, c.N, s);
    launch_contacts("neighbours", P, c.N, s);
    launch_contacts("collect", P, 0, s);
    launch_contacts("resolveContacts", P, 0, s);
    launch_contacts("gather", P, c.N, s);
    launch_contacts("gatherWallRows", P, c.N, s);
    if (c.activeTimestep) launch_state("checkContactTimestep", P, c.N, s);
}

// Whether the filter results (items, survivor and exact-query lists) are
// stored and rebuilt only on the steps whose motion check asks for it.
static bool storedFilters(const Config& c) {
    return c.meshGeometry != 0 && c.filterMargin > 0.0f && c.cullerEnabled == 0;
}

// One step of Engine._advance_once (gpu.py:714-724); captureContactKinematics
// is fused into beginStep when the normal law is viscous.  The two parts that
// most steps skip -- the neighbour build (device flag control[4], set by
// checkRebuild) and the filter build (work[W_FILTER], set by the pair set-up's
// motion check) -- go through `branch(flag, body)`: plain launches run the
// body on s (its kernels return at once when the flag is clear); graph
// capture makes it the body of a conditional node keyed on the flag.
template <class Branch>
static void stepSequence(const Params& P, cudaStream_t s, Branch&& branch) {
    const Config& c = P.c;
    if (c.activeTimestep) launch_state("checkContactTimestep", P, c.N, s);
    launch_contacts("prefetch", P, 0, s);
    Params B = P;
    B.c.viscousCapture = c.normalViscosity > 0 ? 1u : 0u;
    launch_state("beginStep", B, c.N, s);
    launch_state("advanceCell", P, c.specimens, s);
    if (c.wallCount) launch_state("advanceWalls", P, 1, s);
    launch_state("checkRebuild", P, c.N, s);
    branch(P.r.control + 4, [&](cudaStream_t b) { launch_contacts("neighbours", P, c.N, b); });
    if (storedFilters(c)) {
        launch_contacts("collectHead", P, 0, s);
        branch(P.r.work + W_FILTER, [&](cudaStream_t b) { launch_contacts("collectBuild", P, 0, b); });
        launch_contacts("collectTail", P, 0, s);
    } else {
        launch_contacts("collect", P, 0, s);
    }
    launch_contacts("resolveContacts", P, 0, s);
    launch_contacts("gather", P, c.N, s);
    launch_contacts("gatherWallRows", P, c.N, s);
    if (c.activeTimestep) launch_state("checkContactTimestep", P, c.N, s);
    launch_state("finishStep", P, c.N, s);
}

void launch_step(const Params& P, cudaStream_t s) {
    stepSequence(P, s, [&](const uint32_t*, auto&& body) { body(s); });
}

// Sets a conditional node's value from a device flag (graph replay).
__global__ void k_setCondition(cudaGraphConditionalHandle handle, const uint32_t* flag) {
    cudaGraphSetConditional(handle, *flag != 0u ? 1u : 0u);
}

// Committed/new history sides swap every step (gpu.py:725).
static Params swapSides(const Params& P) {
    Params Q = P;
    Res& r = Q.r;
    std::swap(*reinterpret_cast<void**>(&r.meta), *reinterpret_cast<void**>(const_cast<uint4**>(&r.oldMeta)));
    std::swap(*reinterpret_cast<void**>(&r.slip), *reinterpret_cast<void**>(const_cast<float4**>(&r.oldSlip)));
    std::swap(*reinterpret_cast<void**>(&r.normalArea), *reinterpret_cast<void**>(const_cast<float4**>(&r.oldNormal)));
    std::swap(*reinterpret_cast<void**>(&r.hash), *reinterpret_cast<void**>(const_cast<uint32_t**>(&r.oldHash)));
    std::swap(*reinterpret_cast<void**>(&r.sidePairOffsets), *reinterpret_cast<void**>(const_cast<uint32_t**>(&r.oldPairOffsets)));
    std::swap(*reinterpret_cast<void**>(&r.sidePairB), *reinterpret_cast<void**>(const_cast<uint32_t**>(&r.oldPairB)));
    std::swap(*reinterpret_cast<void**>(&r.sideContactStart), *reinterpret_cast<void**>(const_cast<uint32_t**>(&r.oldContactStart)));
    std::swap(*reinterpret_cast<void**>(&r.sideWallStart), *reinterpret_cast<void**>(const_cast<uint32_t**>(&r.oldWallStart)));
    return Q;
}

// Kernel launches of a captured step: those every step runs, and those of
// the neighbour-build and filter-build bodies (run only on steps whose flag
// is set).
struct StepKernels {
    uint32_t always = 0, branch[2] = {0, 0};
};

// Captured one-step graphs for the two history-side orientations of a
// buffer/config set, keyed on the orientation-independent parameter pair.
struct Engine {
    std::vector<unsigned char> key;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    StepKernels kernels;
    cudaStream_t aux = nullptr;  // captures the conditional bodies
    ~Engine() {
        reset();
        if (aux) cudaStreamDestroy(aux);
    }
    void reset() {
        for (auto& e : exec)
            if (e) { cudaGraphExecDestroy(e); e = nullptr; }
        key.clear();
        kernels = StepKernels{};
    }
};

static uint32_t kernelNodes(cudaGraph_t graph) {
    size_t count = 0;
    cudaGraphGetNodes(graph, nullptr, &count);
    std::vector<cudaGraphNode_t> nodes(count);
    cudaGraphGetNodes(graph, nodes.data(), &count);
    uint32_t k = 0;
    for (auto n : nodes) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(n, &t);
        k += t == cudaGraphNodeTypeKernel;
    }
    return k;
}

// One step as a graph: the step sequence captured on s, each branch an IF
// node whose condition a one-thread kernel sets from the branch's device
// flag just before it (the condition defaults to 1 -- run -- on every
// launch), its body captured on aux into the node's body graph.
static int capture(const Params& P, cudaStream_t s, cudaStream_t aux, cudaGraphExec_t* out, StepKernels* kernels) {
    cudaGraph_t graph = nullptr;
    int rc = record(cudaGraphCreate(&graph, 0), "graph create");
    if (rc) return rc;
    rc = record(cudaStreamBeginCaptureToGraph(s, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                "begin capture");
    if (rc) { cudaGraphDestroy(graph); return rc; }
    StepKernels counted;
    int branches = 0;
    stepSequence(P, s, [&](const uint32_t* flag, auto&& body) {
        int index = branches++;
        if (rc) return;
        cudaGraphConditionalHandle handle;
        rc = record(cudaGraphConditionalHandleCreate(&handle, graph, 1u, cudaGraphCondAssignDefault),
                    "conditional handle");
        if (rc) return;
        k_setCondition<<<1, 1, 0, s>>>(handle, flag);
        cudaStreamCaptureStatus status;
        cudaGraph_t target = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        const cudaGraphEdgeData* edges = nullptr;
        size_t count = 0;
        rc = record(cudaStreamGetCaptureInfo(s, &status, nullptr, &target, &deps, &edges, &count), "capture info");
        if (rc) return;
        cudaGraphNodeParams params = {};
        params.type = cudaGraphNodeTypeConditional;
        params.conditional.handle = handle;
        params.conditional.type = cudaGraphCondTypeIf;
        params.conditional.size = 1;
        cudaGraphNode_t node;
        rc = record(cudaGraphAddNode(&node, target, deps, edges, count, &params), "conditional node");
        if (rc) return;
        cudaGraph_t bodyGraph = params.conditional.phGraph_out[0];
        rc = record(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
                    "capture dependencies");
        if (rc) return;
        rc = record(cudaStreamBeginCaptureToGraph(aux, bodyGraph, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal), "begin body capture");
        if (rc) return;
        body(aux);
        cudaGraph_t done = nullptr;
        rc = record(cudaStreamEndCapture(aux, &done), "end body capture");
        if (!rc && index < 2) counted.branch[index] = kernelNodes(bodyGraph);
    });
    cudaGraph_t captured = nullptr;
    int end = record(cudaStreamEndCapture(s, &captured), "end capture");
    rc = rc ? rc : end;
    if (!rc) {
        counted.always = kernelNodes(graph);
        rc = record(cudaGraphInstantiate(out, graph, 0), "instantiate");
    }
    cudaGraphDestroy(graph);
    if (!rc) *kernels = counted;
    return rc;
}

}  // namespace sdg

using namespace sdg;

extern "C" {

int sdg_abi_version(void) { return 1; }
int sdg_buffer_count(void) { return BUFFER_COUNT; }
int sdg_value_count(void) { return VALUE_COUNT; }
const char* sdg_last_error(void) { return g_error.c_str(); }

int sdg_dispatch(const char* kernel, uint32_t count, void* const* buffers, const uint64_t* bytes, const double* values,
                 uint32_t nvalues, void* stream) {
    Params P;
    if (int rc = unpack(buffers, bytes, values, nvalues, P)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::string_view k(kernel ? kernel : "");
    if (k == "step") launch_step(P, s);
    else if (k == "forces") launch_forces(P, s, true);
    else if (k == "forcesNoCapture") launch_forces(P, s, false);
    else if (launch_state(k, P, count, s) != 0 && launch_contacts(k, P, count, s) != 0) {
        g_error = "unknown kernel " + std::string(k);
        return 1;
    }
    return record(cudaGetLastError(), kernel);
}

// Phase timing of one step (events between the launch groups of
// launch_step; not graph-captured).  phase_ms receives SDG_PHASES values:
// drift (checkContactTimestep, beginStep, advanceCell, checkRebuild),
// neighbours, pair setup + leaf cull + item emit, node filter + survivor
// list, exact node queries, contact emit, friction history + contact law, force gather, final kick.
int sdg_engine_profile(void* engine, void* const* buffers, const uint64_t* bytes, const double* values,
                       uint32_t nvalues, float* phase_ms, void* stream) {
    if (!engine || !phase_ms) { g_error = "null argument"; return 1; }
    Params P;
    if (int rc = unpack(buffers, bytes, values, nvalues, P)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int phases = 9;
    cudaEvent_t ev[phases + 1];
    for (auto& e : ev)
        if (int rc = record(cudaEventCreate(&e), "event")) return rc;
    const Config& c = P.c;
    cudaEventRecord(ev[0], s);
    if (c.activeTimestep) launch_state("checkContactTimestep", P, c.N, s);
    Params B = P;
    B.c.viscousCapture = c.normalViscosity > 0 ? 1u : 0u;
    launch_state("beginStep", B, c.N, s);
    launch_state("advanceCell", P, c.specimens, s);
    if (c.wallCount) launch_state("advanceWalls", P, 1, s);
    launch_state("checkRebuild", P, c.N, s);
    cudaEventRecord(ev[1], s);
    launch_contacts("neighbours", P, c.N, s);
    cudaEventRecord(ev[2], s);
    launch_contacts("collectCull", P, 0, s);
    cudaEventRecord(ev[3], s);
    launch_contacts("collectFilter", P, 0, s);
    cudaEventRecord(ev[4], s);
    launch_contacts("collectWalk", P, 0, s);
    cudaEventRecord(ev[5], s);
    launch_contacts("collectEmit", P, 0, s);
    launch_contacts("collectWalls", P, 0, s);
    cudaEventRecord(ev[6], s);
    launch_contacts("resolveContacts", P, 0, s);
    cudaEventRecord(ev[7], s);
    launch_contacts("gather", P, c.N, s);
    launch_contacts("gatherWallRows", P, c.N, s);
    if (c.activeTimestep) launch_state("checkContactTimestep", P, c.N, s);
    cudaEventRecord(ev[8], s);
    launch_state("finishStep", P, c.N, s);
    cudaEventRecord(ev[9], s);
    int rc = record(cudaEventSynchronize(ev[phases]), "profile sync");
    for (int k = 0; k < phases && !rc; ++k) rc = record(cudaEventElapsedTime(&phase_ms[k], ev[k], ev[k + 1]), "elapsed");
    for (auto& e : ev) cudaEventDestroy(e);
    return rc ? rc : record(cudaGetLastError(), "profile");
}

// Engine.diagnostics in one call: the per-grain diagnostic rows and the
// per-pair fabric rows with their 256-wide tree reductions
// (diagnostic.slang:3-28; the same levels as sdg_reduce_rows), ping-ponged
// through two scratch buffers, then the final 8 + 2 rows, the first three
// cell rows and the 16 control words copied to `host` (pinned, 272 bytes:
// 8 rows, 2 rows, 3 rows, 16 words).  The caller waits on the stream.
static int reduceLevels(const float4* input, uint32_t n, uint32_t rows, int maxRow, float4* a, float4* b,
                        uint64_t scratchBytes, const float4** result, cudaStream_t s) {
    const float4* src = input;
    float4* out = a;
    while (n > 1) {
        uint32_t groups = (n + 255) / 256;
        if (uint64_t(groups) * rows * 16 > scratchBytes) { g_error = "diagnostics scratch too small"; return 1; }
        launch_reduce_rows(src, out, n, rows, maxRow, s);
        src = out;
        out = out == a ? b : a;
        n = groups;
    }
    *result = src;
    return 0;
}
int sdg_engine_diagnostics(void* const* buffers, const uint64_t* bytes, const double* values, uint32_t nvalues,
                           void* scratch_a, void* scratch_b, uint64_t scratch_bytes, void* host, void* stream) {
    if (!scratch_a || !scratch_b || !host) { g_error = "null diagnostics argument"; return 1; }
    Params P;
    if (int rc = unpack(buffers, bytes, values, nvalues, P)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const Config& c = P.c;
    auto* a = static_cast<float4*>(scratch_a);
    auto* b = static_cast<float4*>(scratch_b);
    char* out = static_cast<char*>(host);
    const float4* rows = nullptr;
    launch_state("diagnosticRows", P, c.N, s);
    if (int rc = reduceLevels(P.r.diagnosticRows, c.N, 8, 4, a, b, scratch_bytes, &rows, s)) return rc;
    cudaMemcpyAsync(out, rows, 8 * 16, cudaMemcpyDeviceToHost, s);
    launch_state("fabricRows", P, c.pairCapacity, s);
    if (int rc = reduceLevels(P.r.fabricRows, c.pairCapacity, 2, -1, a, b, scratch_bytes, &rows, s)) return rc;
    cudaMemcpyAsync(out + 128, rows, 2 * 16, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(out + 160, P.r.cell, 3 * 16, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(out + 208, P.r.control, 16 * 4, cudaMemcpyDeviceToHost, s);
    return record(cudaGetLastError(), "diagnostics");
}

int sdg_reduce_rows(const void* input, void* output, uint32_t n, uint32_t rows, int32_t max_row, void* stream) {
    if (!input || !output || rows == 0) { g_error = "bad reduction arguments"; return 1; }
    launch_reduce_rows(static_cast<const float4*>(input), static_cast<float4*>(output), n, rows, max_row,
                       static_cast<cudaStream_t>(stream));
    return record(cudaGetLastError(), "reduce rows");
}

// Per-wall tree sums of the (wall, grain) rows, one level (diagnostic.slang:33-49).
int sdg_reduce_wall_rows(const void* input, void* output, uint32_t n, uint32_t walls, void* stream) {
    if (!input || !output || walls == 0 || n == 0) { g_error = "bad wall reduction arguments"; return 1; }
    launch_reduce_wall_rows(static_cast<const float4*>(input), static_cast<float4*>(output), n, walls,
                            static_cast<cudaStream_t>(stream));
    return record(cudaGetLastError(), "reduce wall rows");
}

// Exclusive scan of n uint32 values (the reference's hierarchical Scan,
// gpu.py:65-91 / scan.slang): out[i] = sum of in[0..i); *total (device
// pointer, optional) receives the sum.  `partials` is caller-owned device
// scratch of SDG_SCAN_PARTIALS uint32 words.
int sdg_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, uint32_t* partials,
                       void* stream) {
    if ((!in || !out) && n) { g_error = "null scan buffer"; return 1; }
    if (!partials) { g_error = "null scan partials"; return 1; }
    launch_scan(in, out, ScanCount{nullptr, 0, 0, n}, false, total, nullptr, partials,
                static_cast<cudaStream_t>(stream));
    return record(cudaGetLastError(), "scan");
}

int sdg_scan_partials(void) { return 2 * SCAN_BLOCKS; }

// Device-to-device copies of n buffers on `stream` (the engine's
// transactional backup before a chunk and its restore): one kernel launch
// per 64 buffers instead of one copy call each.  Each (buffer, block-row)
// pair of the grid copies a strided share of its buffer, in 16-byte words
// where both ends are 16-byte aligned, else byte by byte.
struct CopyList {
    uint64_t dst[64], src[64], bytes[64];
    uint32_t n;
};
__global__ void k_copyBuffers(const __grid_constant__ CopyList L) {
    uint32_t k = blockIdx.y;
    if (k >= L.n) return;
    uint64_t bytes = L.bytes[k];
    char* d = reinterpret_cast<char*>(L.dst[k]);
    const char* s = reinterpret_cast<const char*>(L.src[k]);
    uint64_t stride = uint64_t(gridDim.x) * blockDim.x, t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    uint64_t words = ((L.dst[k] | L.src[k]) & 15u) == 0 ? bytes / 16 : 0;
    for (uint64_t i = t; i < words; i += stride)
        reinterpret_cast<uint4*>(d)[i] = reinterpret_cast<const uint4*>(s)[i];
    for (uint64_t i = 16 * words + t; i < bytes; i += stride) d[i] = s[i];
}
int sdg_copy_buffers(void* const* dst, void* const* src, const uint64_t* bytes, uint32_t n, void* stream) {
    if (n && (!dst || !src || !bytes)) { g_error = "null copy arguments"; return 1; }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (uint32_t k = 0; k < n;) {
        CopyList L = {};
        uint64_t largest = 0;
        for (; k < n && L.n < 64; ++k) {
            if (!bytes[k]) continue;
            if (!dst[k] || !src[k]) { g_error = "null copy arguments"; return 1; }
            L.dst[L.n] = reinterpret_cast<uint64_t>(dst[k]);
            L.src[L.n] = reinterpret_cast<uint64_t>(src[k]);
            L.bytes[L.n] = bytes[k];
            largest = std::max(largest, bytes[k]);
            ++L.n;
        }
        if (!L.n) continue;
        // Enough blocks per buffer for the largest one (16 KB each), up to 64.
        uint32_t rows = uint32_t(std::min<uint64_t>(64, std::max<uint64_t>(1, largest >> 14)));
        k_copyBuffers<<<dim3(rows, L.n), 256, 0, s>>>(L);
        if (int rc = record(cudaGetLastError(), "copy")) return rc;
    }
    return 0;
}

void* sdg_engine_create(void) { return new (std::nothrow) Engine(); }
void sdg_engine_destroy(void* engine) { delete static_cast<Engine*>(engine); }

// Advances `steps` steps starting from the history side the buffers describe,
// alternating sides; with use_graph, each side's step is a captured CUDA graph
// replayed (recaptured when buffers or values change).
int sdg_engine_advance(void* engine, void* const* buffers, const uint64_t* bytes, const double* values,
                       uint32_t nvalues, uint32_t steps, uint32_t use_graph, void* stream) {
    Engine* e = static_cast<Engine*>(engine);
    if (!e) { g_error = "null engine"; return 1; }
    Params P;
    if (int rc = unpack(buffers, bytes, values, nvalues, P)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Params side[2] = {P, swapSides(P)};
    if (!use_graph) {
        for (uint32_t k = 0; k < steps; ++k) launch_step(side[k & 1], s);
        return record(cudaGetLastError(), "advance");
    }
    // Orientation-independent key: the side whose buffers sort first is 0.
    bool flipped = std::memcmp(&side[0], &side[1], sizeof(Params)) > 0;
    const Params& first = side[flipped ? 1 : 0];
    const Params& second = side[flipped ? 0 : 1];
    std::vector<unsigned char> key(2 * sizeof(Params));
    std::memcpy(key.data(), &first, sizeof(Params));
    std::memcpy(key.data() + sizeof(Params), &second, sizeof(Params));
    if (key != e->key) {
        e->reset();
        if (!e->aux)
            if (int rc = record(cudaStreamCreateWithFlags(&e->aux, cudaStreamNonBlocking), "capture stream")) return rc;
        StepKernels kernels;
        if (int rc = capture(first, s, e->aux, &e->exec[0], &kernels)) { e->reset(); return rc; }
        if (int rc = capture(second, s, e->aux, &e->exec[1], &kernels)) { e->reset(); return rc; }
        e->kernels = kernels;
        e->key = key;
    }
    uint32_t start = flipped ? 1u : 0u;
    for (uint32_t k = 0; k < steps; ++k)
        if (int rc = record(cudaGraphLaunch(e->exec[(start + k) & 1], s), "graph launch")) return rc;
    return 0;
}

// Kernel launches of a captured step that skips both conditional bodies (0
// before the first graph capture).
int sdg_engine_kernels_per_step(void* engine) {
    Engine* e = static_cast<Engine*>(engine);
    return e ? int(e->kernels.always) : -1;
}

// Kernel launches inside conditional body `branch` of a captured step: 0 =
// the neighbour build (run on rebuild steps), 1 = the filter build (run on
// steps that build the stored filter results; absent without them).
int sdg_engine_branch_kernels(void* engine, int branch) {
    Engine* e = static_cast<Engine*>(engine);
    if (!e || branch < 0 || branch > 1) return -1;
    return int(e->kernels.branch[branch]);
}

}  // extern "C"
