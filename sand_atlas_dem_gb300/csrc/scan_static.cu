// Exclusive scan whose block partials live in a fixed device array of this
// library instead of caller-owned scratch (no counterpart in the reference).
//
// Who needs it: a host that reaches this library only through its C ABI and
// holds no device allocator of its own -- a cgo, JNI or ctypes stub that is
// handed the input and output buffers by someone else -- and a caller whose
// device-memory budget is fixed once its buffers are sized, so that a scan
// issued later may not grow it.  Both can hand over `in`, `out` and `total`
// but cannot produce the SDG_SCAN_PARTIALS words sdg_exclusive_scan wants.
//
// This entry point allocates nothing: no cudaMalloc/cudaFree and no library
// routine that allocates.  The partials are the file-scope array below
// (2 x SCAN_BLOCKS uint32 = 4,864 bytes per device).  Its device address is
// looked up once per device, with that device current, on the first call;
// that first call must come before any stream capture on the device.  The
// address belongs to the device's current context: after a device reset
// (cudaDeviceReset) the next call sees a context with a new ID and looks the
// address up again, so that call too must come before any stream capture.
//
// A CUDA error still pending from an earlier, unrelated call is left for its
// owner: the entry point reports it without launching and does not clear it.
//
// Nothing in the array has to start at zero: every word a call reads was
// written earlier in the same call (block sums by the first kernel, their
// exclusive prefix by the second).  Two calls in flight at once on the same
// device (two streams, or two host threads) share the array and race; the
// caller serialises them, for example by issuing them on one stream.
#include <mutex>
#include <string>
#include <cuda.h>
#include <cuda_runtime.h>
#include "dem_device.cuh"
#include "launch.h"

namespace sdg {

static __device__ __align__(256) uint32_t g_scanPartials[2 * SCAN_BLOCKS];

// Largest n accepted: keeps the per-block chunk arithmetic (n + blocks - 1
// and begin + chunk, in uint32) clear of overflow.
constexpr uint32_t STATIC_SCAN_MAX_N = 1u << 30;
constexpr int MAX_DEVICES = 64;

static std::mutex g_setupLock;
static uint32_t* g_partials[MAX_DEVICES] = {};
// ID of the context each cached address belongs to (cuCtxGetId: unique for
// the life of the process, never reused).
static unsigned long long g_contextId[MAX_DEVICES] = {};

using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);
static CtxGetCurrent g_ctxGetCurrent = nullptr;
static CtxGetId g_ctxGetId = nullptr;

static int fail(const std::string& what) {
    set_last_error(what);
    return 1;
}

// ID of the current context, through driver entry points the runtime hands
// out (no link against the driver library).  Called with g_setupLock held.
static int currentContextId(unsigned long long* id) {
    if (!g_ctxGetCurrent || !g_ctxGetId) {
        void* current = nullptr;
        void* getId = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &current, 12000, cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &getId, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !current || !getId)
            return fail("static scan: driver entry points cuCtxGetCurrent/cuCtxGetId unavailable");
        g_ctxGetCurrent = reinterpret_cast<CtxGetCurrent>(current);
        g_ctxGetId = reinterpret_cast<CtxGetId>(getId);
    }
    CUcontext ctx = nullptr;
    if (g_ctxGetCurrent(&ctx) != CUDA_SUCCESS || !ctx) return fail("static scan: no current context");
    if (g_ctxGetId(ctx, id) != CUDA_SUCCESS) return fail("static scan: cuCtxGetId failed");
    return 0;
}

// Device address of g_scanPartials on the current device (set-up on first
// use on the device, and again after its context was replaced).
static int partialsForCurrentDevice(uint32_t** out) {
    int device = -1;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail(std::string("static scan: cudaGetDevice: ") + cudaGetErrorString(e));
    if (device < 0 || device >= MAX_DEVICES) return fail("static scan: device ordinal out of range");
    // cudaFree(nullptr) would also make the primary context current, but it
    // is an allocator call; cudaSetDevice makes it current without one.
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(std::string("static scan: cudaSetDevice: ") + cudaGetErrorString(e));
    std::lock_guard<std::mutex> hold(g_setupLock);
    unsigned long long context = 0;
    if (int rc = currentContextId(&context)) return rc;
    if (!g_partials[device] || g_contextId[device] != context) {
        void* address = nullptr;
        e = cudaGetSymbolAddress(&address, g_scanPartials);
        if (e != cudaSuccess || !address)
            return fail(std::string("static scan: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_partials[device] = static_cast<uint32_t*>(address);
        g_contextId[device] = context;
    }
    *out = g_partials[device];
    return 0;
}

}  // namespace sdg

using namespace sdg;

extern "C" {

int sdg_exclusive_scan_static(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, void* stream) {
    if ((!in || !out) && n) return fail("static scan: null scan buffer");
    if (n > STATIC_SCAN_MAX_N)
        return fail("static scan: n = " + std::to_string(n) + " exceeds the limit of " +
                    std::to_string(STATIC_SCAN_MAX_N) + " values");
    // An error pending from an earlier call belongs to that call: report it
    // without consuming it, and launch nothing.
    cudaError_t prior = cudaPeekAtLastError();
    if (prior != cudaSuccess)
        return fail(std::string("static scan: an earlier CUDA error is pending (not cleared): ") +
                    cudaGetErrorString(prior));
    uint32_t* partials = nullptr;
    if (int rc = partialsForCurrentDevice(&partials)) return rc;
    launch_scan(in, out, ScanCount{nullptr, 0, 0, n}, false, total, nullptr, partials,
                static_cast<cudaStream_t>(stream));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(std::string("static scan: launch: ") + cudaGetErrorString(e));
    return 0;
}

}  // extern "C"
