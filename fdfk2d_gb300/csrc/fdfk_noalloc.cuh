// Single time step with all device buffers carved from a fixed static device
// array (fdfk_noalloc.cu).
#pragma once
#include "fdfk_gb300.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <string>

namespace fdfk {

// Size of the static device scratch: 16 Mi floats (64 MiB).
constexpr size_t kNoAllocFloats = size_t(1) << 24;
// Largest NX or NZ the fixed host damping tables hold.
constexpr int kNoAllocMaxDim = 1 << 16;

// Scratch floats one step of this geometry needs (every region rounded up to 256 bytes).
size_t noalloc_floats_needed(const fdfk_params& p);

// One step of updatedispl_ semantics on the static scratch; `p` already validated.
int step_noalloc(const fdfk_params& p, int it, const float* const strips[12], const float* c, float* ux, float* uz,
                 float* const bp[12], float* const bu[24], const float* stag, const float* coll, cudaStream_t st,
                 std::string& err, long long* launches);

}  // namespace fdfk
