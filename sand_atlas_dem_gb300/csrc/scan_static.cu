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
// that first call must come before any stream capture on the device.
//
// Nothing in the array has to start at zero: every word a call reads was
// written earlier in the same call (block sums by the first kernel, their
// exclusive prefix by the second).  Two calls in flight at once on the same
// device (two streams, or two host threads) share the array and race; the
// caller serialises them, for example by issuing them on one stream.
#include <mutex>
#include <string>
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

static int fail(const std::string& what) {
    set_last_error(what);
    return 1;
}

// Device address of g_scanPartials on the current device (set-up on first use).
static int partialsForCurrentDevice(uint32_t** out) {
    int device = -1;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail(std::string("static scan: cudaGetDevice: ") + cudaGetErrorString(e));
    if (device < 0 || device >= MAX_DEVICES) return fail("static scan: device ordinal out of range");
    std::lock_guard<std::mutex> hold(g_setupLock);
    if (!g_partials[device]) {
        void* address = nullptr;
        e = cudaGetSymbolAddress(&address, g_scanPartials);
        if (e != cudaSuccess || !address)
            return fail(std::string("static scan: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_partials[device] = static_cast<uint32_t*>(address);
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
    uint32_t* partials = nullptr;
    if (int rc = partialsForCurrentDevice(&partials)) return rc;
    launch_scan(in, out, ScanCount{nullptr, 0, 0, n}, false, total, nullptr, partials,
                static_cast<cudaStream_t>(stream));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(std::string("static scan: launch: ") + cudaGetErrorString(e));
    return 0;
}

}  // extern "C"
