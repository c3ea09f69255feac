// Host launchers shared by the kernel translation units and the C ABI.
#pragma once
#include <cstdint>
#include <string>
#include <string_view>
#include <cuda_runtime.h>
#include "dem_device.cuh"

namespace sdg {

// Buffer/value block to kernel parameters (capi.cu); 0 = ok.
int unpack_params(void* const* buffers, const uint64_t* bytes, const double* values, uint32_t nvalues,
                  Params& P);

// Sets the text sdg_last_error returns on this thread (capi.cu).
void set_last_error(const std::string& what);

// Launch a reference-named kernel; 0 = launched, 1 = unknown name.
int launch_state(const std::string_view& name, const Params& P, uint32_t count, cudaStream_t s);
int launch_contacts(const std::string_view& name, const Params& P, uint32_t count, cudaStream_t s);
void launch_reduce_rows(const float4* input, float4* output, uint32_t n, uint32_t rows, int maxRow, cudaStream_t s);
void launch_reduce_wall_rows(const float4* input, float4* output, uint32_t n, uint32_t walls, cudaStream_t s);

// Device-wide exclusive scan of n uint32 values, n = constant or
// min(*countPtr, cap) * mul read on the device.  Writes out[0..n), optionally
// out[n] = total and *totalDst = total.  Skipped when gate && *gate == 0.
struct ScanCount {
    const uint32_t* ptr;
    uint32_t cap, mul, constant;
};
void launch_scan(const uint32_t* in, uint32_t* out, ScanCount count, bool writeEnd, uint32_t* totalDst,
                 const uint32_t* gate, uint32_t* partials, cudaStream_t s);

// Launch one full step (all phases) on stream s.
void launch_step(const Params& P, cudaStream_t s);
// The force phases only (neighbours, contacts, friction, gather).
void launch_forces(const Params& P, cudaStream_t s, bool captureKinematics);

}  // namespace sdg
